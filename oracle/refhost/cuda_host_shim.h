// Host-CPU emulation of the small CUDA subset used by the reference FWI core
// (deps/CustomOps/FWI/Src/*.cu of FwiFlow.jl), so that the reference's own
// source files compile with g++ and run on a machine without a GPU.
//
// TEST INFRASTRUCTURE ONLY. This header is force-included (g++ -include) when
// oracle/Makefile.refhost compiles the reference sources into oracle/_ref/.
// Nothing in the product links it.
//
// What is emulated:
//  * kernel launches: `k<<<grid, block>>>(args)` is rewritten by the build
//    recipe (a sed pass piped straight into g++) to
//    `SHIM_LAUNCH(k, grid, block)(args)`, which runs every thread of every
//    block sequentially on the calling host thread;
//  * kernels that use __syncthreads (the one-block misfit reduction
//    `cuda_cal_objective`, utilities.cu:169-205) run one std::thread per CUDA
//    thread with a real barrier, so their shared-memory tree reduction keeps
//    its order of operations;
//  * atomicAdd is a plain read-add-write (execution is sequential);
//  * device memory is host memory; cudaMemcpy* is memcpy;
//  * cuFFT's 1-D R2C / C2R plans are an unnormalised O(n^2) DFT in double
//    precision (mathematical definition, used only by the optional band-pass
//    filter path, utilities.cu:872-923).
// Device math functions resolve to the host libm, so results agree with a GPU
// run of the same sources to within a few ulps per operation, not bit for bit.
#pragma once

#define __global__
#define __device__
#define __host__
#define __forceinline__ inline
#define __shared__ static
#define __constant__ static

#include <cuda_runtime.h>
#include <cuComplex.h>
#include <cufft.h>

#include <cassert>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>

namespace shim {

struct ThreadCtx {
  uint3 tid;
  uint3 bid;
  dim3 bdim;
  dim3 gdim;
};
extern thread_local ThreadCtx ctx;

bool kernel_needs_barrier(const char* name);
void run_block_threaded(dim3 g, uint3 bid, dim3 b, const std::function<void()>& body);
void syncthreads();

template <class Body>
void run_grid(const char* name, dim3 g, dim3 b, Body&& body) {
  if (kernel_needs_barrier(name)) {
    std::function<void()> f = body;
    for (unsigned bz = 0; bz < g.z; ++bz)
      for (unsigned by = 0; by < g.y; ++by)
        for (unsigned bx = 0; bx < g.x; ++bx) run_block_threaded(g, make_uint3(bx, by, bz), b, f);
    return;
  }
  ctx.gdim = g;
  ctx.bdim = b;
  for (unsigned bz = 0; bz < g.z; ++bz)
    for (unsigned by = 0; by < g.y; ++by)
      for (unsigned bx = 0; bx < g.x; ++bx) {
        ctx.bid = make_uint3(bx, by, bz);
        for (unsigned tz = 0; tz < b.z; ++tz)
          for (unsigned ty = 0; ty < b.y; ++ty)
            for (unsigned tx = 0; tx < b.x; ++tx) {
              ctx.tid = make_uint3(tx, ty, tz);
              body();
            }
      }
}

struct Launch {
  const char* name;
  dim3 g, b;
  Launch(const char* n, dim3 g_, dim3 b_, size_t = 0, cudaStream_t = nullptr) : name(n), g(g_), b(b_) {}
  template <class F>
  auto operator->*(F f) const {
    Launch self = *this;
    return [self, f](auto... a) { run_grid(self.name, self.g, self.b, [&]() { f(a...); }); };
  }
};

}  // namespace shim

#define threadIdx (shim::ctx.tid)
#define blockIdx (shim::ctx.bid)
#define blockDim (shim::ctx.bdim)
#define gridDim (shim::ctx.gdim)
#define __syncthreads() shim::syncthreads()

inline float atomicAdd(float* p, float v) {
  float old = *p;
  *p = old + v;
  return old;
}

#define SHIM_LAUNCH(k, ...) (shim::Launch(#k, __VA_ARGS__)->*[](auto... a) { k(a...); })
