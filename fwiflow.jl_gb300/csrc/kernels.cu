// GB300 (sm_103a) kernels of the elastic FWI operator: 4th-order staggered
// velocity-stress sweeps with CPML, the fused reverse-time / adjoint / imaging
// sweeps, the residual / misfit reduction and the model set-up.
//
// Per time step the reference launches el_stress, add_source, el_velocity,
// recording and five from_bnd kernels forward (libCUFD.cu:202-240) and twelve
// kernels backward (libCUFD.cu:374-445). Here a forward step is two sweeps and
// a backward step is two sweeps:
//   forward  F1: boundary-ring save + stress update + source + recording
//            F2: velocity update
//   backward B : source removal + reverse stress + lambda/mu imaging + stress
//                ring restore + velocity adjoint                 (step it)
//            C : residual injection + stress adjoint + source gradient (it-1)
//                + reverse velocity + rho imaging + velocity ring restore
// The reference scatters the mu and rho kernels with atomicAdd
// (el_stress.cu:113-124, el_velocity.cu:101-110); here every cell gathers the
// contributions of its neighbours, recomputing their derivative terms from the
// read-only fields of the same sweep, so there are no atomics and the sums are
// deterministic.
#include "fwigb_kernels.h"

#include <cudaTypedefs.h>

#include <cstdint>
#include <utility>

namespace fwigb {
namespace {

constexpr float C1 = 1.125f;          // 9/8  (el_stress.cu:42)
constexpr float C2 = 1.0f / 24.0f;    // 1/24 (el_stress.cu:43)
constexpr float kMega = 1.0e6f;       // MEGA (utilities.h:16)

// Bounded waits: a sweep that has waited this long (global timer) for its
// staged tiles gives up, raises its error word and returns instead of
// hanging. Each poll asks the hardware to suspend the thread until the
// barrier phase completes or kWaitHintNs pass, so a waiting warp issues a
// few instructions instead of spinning.
constexpr unsigned long long kWaitLimitNs = 2000000000ull;
constexpr unsigned kWaitHintNs = 1000000u;
// Polls (without a suspend hint) of the injected wait of the timeout test
// hook (stage_wait).
constexpr unsigned kInjectPolls = 256;

// ---- mbarrier / TMA (sm_90+ PTX; issued by one thread per block) ----
__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ bool mbar_try_wait_hint(uint64_t* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity), "r"(kWaitHintNs)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ unsigned long long global_timer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// Waits for phase `parity` of the barrier, at most kWaitLimitNs.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned parity) {
  if (mbar_try_wait_hint(bar, parity)) return true;
  const unsigned long long t0 = global_timer_ns();
  for (;;) {
    if (mbar_try_wait_hint(bar, parity)) return true;
    if (global_timer_ns() - t0 > kWaitLimitNs) return false;
  }
}
// Polls phase `parity` of the barrier `polls` times without a suspend hint.
__device__ __forceinline__ bool mbar_poll(uint64_t* bar, unsigned parity, unsigned polls) {
  for (unsigned n = 0; n < polls; ++n)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
__device__ __forceinline__ void tma_load_2d(float* dst, const CUtensorMap* tm, int c0, int c1, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(tm)), "r"(c0), "r"(c1), "r"(smem_u32(bar))
      : "memory");
}

// Starts staging NA arrays of the tile at (z0, x0) into shared memory: one
// 2-D TMA copy each of the box [z0-4, z0-4+BOXZ) x [x0-2, x0+TX+2), zero
// filled outside the grid. The leader initialises the mbarrier (fenced so the
// copies see it) and issues the copies after the block has met the barrier's
// initialisation; the caller then loads its own-cell operands (which overlap
// with the copies) and calls stage_wait.
template <int NA, int TX, int BOXZ>
__device__ __forceinline__ void stage_issue(const TileMaps& mp, float* sm, uint64_t* bar, int z0, int x0) {
  constexpr int N = BOXZ * (TX + 4);
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    mbar_expect_tx(bar, NA * N * static_cast<unsigned>(sizeof(float)));
#pragma unroll
    for (int a = 0; a < NA; ++a) tma_load_2d(sm + a * N, &mp.t[a], z0 - 4, x0 - 2, bar);
  }
}
__device__ __forceinline__ void stage_init(uint64_t* bar) {
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    mbar_init(bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
}
template <int NA, int TX, int BOXZ>
__device__ __forceinline__ void stage_begin(const TileMaps& mp, float* sm, uint64_t* bar, int z0, int x0) {
  stage_init(bar);
  stage_issue<NA, TX, BOXZ>(mp, sm, bar, z0, x0);
}

// Waits (bounded) for the staged tiles. On a timeout the error word is raised
// and the thread waits once more so that copies still in flight land before
// the block exits; the caller then returns without computing. Should that
// second wait run out too, copies may still land after the block has left:
// the host then reports FWIGB_ERR_TIMEOUT for the whole call and its outputs
// are undefined (the next run re-zeroes every field it uses).
// `inject` (the timeout test hook): once the tiles have landed, the thread
// also waits for the barrier's next phase, which nothing completes, so the
// bounded wait runs out with no copy in flight and the error word is raised.
__device__ __forceinline__ bool stage_wait(uint64_t* bar, unsigned* err, bool inject = false) {
  if (!mbar_wait_bounded(bar, 0)) {
    atomicOr(err, 1u);
    mbar_wait_bounded(bar, 0);
    return false;
  }
  if (inject && !mbar_poll(bar, 1, kInjectPolls)) {
    atomicOr(err, 1u);
    return false;
  }
  return true;
}

// Staggered 4th-order differences. Dm uses (i-2, i-1, i, i+1), Dp
// (i-1, i, i+1, i+2); `s` is the stride of the direction and r the
// reciprocal spacing. sdm / sdp read a staged tile (32-bit indices), gdm / gdp
// global memory.
__device__ __forceinline__ float sdm(const float* a, int i, int s, float r) {
  return (C1 * (a[i] - a[i - s]) - C2 * (a[i + s] - a[i - 2 * s])) * r;
}
__device__ __forceinline__ float sdp(const float* a, int i, int s, float r) {
  return (C1 * (a[i + s] - a[i]) - C2 * (a[i + 2 * s] - a[i - s])) * r;
}
__device__ __forceinline__ float gdm(const float* __restrict__ a, size_t i, size_t s, float r) {
  return (C1 * (a[i] - a[i - s]) - C2 * (a[i + s] - a[i - 2 * s])) * r;
}
__device__ __forceinline__ float gdp(const float* __restrict__ a, size_t i, size_t s, float r) {
  return (C1 * (a[i + s] - a[i]) - C2 * (a[i + 2 * s] - a[i - s])) * r;
}

// Index of cell (z, x) in the per-step boundary ring, or -1. Top and bottom
// bands are stored column by column (5 depths each), left and right bands
// column by column over their height, so a warp of consecutive depths writes
// consecutive words.
__device__ __forceinline__ int ring_index(const Geo& g, int z, int x) {
  if (z < g.rz0 || z > g.rz1 || x < g.rx0 || x > g.rx1) return -1;
  if (z <= g.rz0 + 4) return (x - g.rx0) * 5 + (z - g.rz0);
  if (z >= g.rz1 - 4) return 5 * g.ringW + (x - g.rx0) * 5 + (z - (g.rz1 - 4));
  if (x <= g.rx0 + 4) return 10 * g.ringW + (x - g.rx0) * g.ringH + (z - (g.rz0 + 5));
  if (x >= g.rx1 - 4) return 10 * g.ringW + 5 * g.ringH + (x - (g.rx1 - 4)) * g.ringH + (z - (g.rz0 + 5));
  return -1;
}

// from_bnd of step it for cell (z, x) when it lies in the ring: the stresses
// before the step's update and the velocities of the staged tile
// (Boundary.cu:55-76).
__device__ __forceinline__ void ring_save(const Geo& g, const StoreD& st, int it, int z, int x, float szz, float sxz,
                                          float sxx, float vz, float vx) {
  const int k = ring_index(g, z, x);
  if (k < 0) return;
  float* p = st.base + static_cast<size_t>(it) * 5 * g.ring_len + k;
  p[0] = szz;
  p[g.ring_len] = sxz;
  p[2 * g.ring_len] = sxx;
  p[3 * g.ring_len] = vz;
  p[4 * g.ring_len] = vx;
}

// a / K of the CPML formulas, with the division skipped where K == 1 (exact:
// a / 1 == a), i.e. everywhere outside the CPML.
__device__ __forceinline__ float kdiv(float a, float K) { return K == 1.0f ? a : a / K; }

__device__ __forceinline__ bool in_box(int z, int x, int z0, int z1, int x0, int x1) {
  return z >= z0 && z <= z1 && x >= x0 && x <= x1;
}

// Whether the tile of tz depths x tx columns at (z0, x0) meets the bounding
// box of the shot's receivers and source.
__device__ __forceinline__ bool tile_meets_shot_box(const ShotD& sh, int z0, int x0, int tz, int tx) {
  return !(z0 + tz - 1 < sh.rbz0 || z0 > sh.rbz1 || x0 + tx - 1 < sh.rbx0 || x0 > sh.rbx1);
}

// Receiver list of the 32 x 8 bin holding (z, x).
__device__ __forceinline__ int2 bin_range(const ShotD& sh, int z, int x) {
  const int b = (z / kBinZ) + (x / kBinX) * sh.nbin_z;
  return make_int2(sh.blk_off[b], sh.blk_off[b + 1]);
}

// Every sweep is one launch per time step for a pack of shots: blockIdx.z is
// the shot (its slot holds its sub-grid, fields, source, receivers and TMA
// maps), blockIdx.x / blockIdx.y the tile of TZ depths x TX columns. A tile
// inside the shot's fast rectangle runs the sweep's fast body (the interior
// form of the reference kernels); a tile inside the mid rectangle (no CPML
// cell) runs the fast body with per-cell ring, band and guard handling; any
// other tile runs its edge body (the full CPML / boundary-ring / band
// logic). The choice is uniform per block. Blocks past a narrower shot's grid
// leave before staging anything, and so do blocks whose tile lies wholly
// below row zact1 (the nPad rows, where no sweep reads or writes a cell of
// its own) unless it holds the shot's source or a receiver. Block
// (32, TX): lane threadIdx.x covers R adjacent depths (R = TZ / 32),
// threadIdx.y the column; `b` is the index of its first cell in a staged box
// (column stride BOXZ = TZ + 8).
// Programmatic dependent launch: a sweep lets the next sweep's blocks be
// scheduled as soon as all of its own blocks have started, and waits
// (pdl_wait) for the previous sweep to complete, and its writes to be
// visible, before it touches any field. The parameter reads, the tile
// classification, the staging-barrier set-up and, in fast tiles and backward
// edge tiles, the loads of the media (which no sweep writes) come before the
// wait and overlap the previous sweep's last blocks.
#define SWEEP_KERNEL_TILE(TZ_)                                                 \
  const int shot = K == 1 ? 0 : static_cast<int>(blockIdx.z);                  \
  const Geo& g0 = P.slots[shot].g;                                             \
  const int z0 = blockIdx.x * (TZ_), x0 = blockIdx.y * TX;                     \
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");              \
  if (z0 >= g0.nz || x0 >= g0.nx) return;                                      \
  if (z0 > g0.zact1 && !tile_meets_shot_box(P.slots[shot].sh, z0, x0, (TZ_), TX)) return; \
  const TileSplit ts = tile_split(g0, TX, (TZ_));                              \
  const bool fast = static_cast<int>(blockIdx.x) >= ts.ftz0 &&                 \
                    static_cast<int>(blockIdx.x) < ts.ftz1 &&                  \
                    static_cast<int>(blockIdx.y) >= ts.ftx0 &&                 \
                    static_cast<int>(blockIdx.y) < ts.ftx1;                    \
  const bool mid = !fast && static_cast<int>(blockIdx.x) >= ts.mtz0 &&         \
                   static_cast<int>(blockIdx.x) < ts.mtz1 &&                   \
                   static_cast<int>(blockIdx.y) >= ts.mtx0 &&                  \
                   static_cast<int>(blockIdx.y) < ts.mtx1;

#define SWEEP_BODY_SLOT()                                                      \
  const ShotSlot& S = P.slots[shot];                                           \
  const Geo& g = S.g;

// A fast tile lies wholly inside the grid. `special` marks the tiles that
// meet the bounding box of the shot's receivers and source.
#define SWEEP_FAST_SLOT(TZ_)                                                   \
  SWEEP_BODY_SLOT()                                                            \
  const ShotD& sh = S.sh;                                                      \
  const bool special = !(z0 + (TZ_) - 1 < sh.rbz0 || z0 > sh.rbz1 ||           \
                         x0 + TX - 1 < sh.rbx0 || x0 > sh.rbx1);

__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// Fast tiles: the thread's first cell (z, x), its global index i and its box
// index b (every cell of a fast tile is inside the grid).
#define SWEEP_CELL(BOXZ_, R_)                                                  \
  const Fields& f = S.f;                                                       \
  const MediaD& m = S.m;                                                       \
  const int z = z0 + (R_) * static_cast<int>(threadIdx.x), x = x0 + threadIdx.y; \
  const size_t ldz = static_cast<size_t>(g.ldz);                               \
  const size_t i = static_cast<size_t>(x) * ldz + z;                           \
  const int b = (threadIdx.y + 2) * (BOXZ_) + (R_) * threadIdx.x + 4;

// Fast tiles: the staging barrier is set up before the media loads and the
// tile copies are issued right after pdl_wait (SWEEP_TMA).
#define SWEEP_SMEM(BOXZ_)                                                      \
  constexpr int N = (BOXZ_) * (TX + 4);                                        \
  extern __shared__ __align__(128) float sm[];                                 \
  __shared__ __align__(8) uint64_t bar;                                        \
  stage_init(&bar);
#define SWEEP_TMA(NA, BOXZ_) stage_issue<NA, TX, (BOXZ_)>(P.maps[shot], sm, &bar, z0, x0);

// Edge tiles: the thread's first cell (z, x), its global index i, its box
// index b and whether the cell lies in the grid (`live`; a thread with no
// cell in the grid takes part in the staging set-up only, and the tile's
// first thread, which issues and awaits the copies, is always live).
#define SWEEP_EDGE_CELL(BOXZ_, R_)                                             \
  const Fields& f = S.f;                                                       \
  const MediaD& m = S.m;                                                       \
  const CpmlD& c = S.c;                                                        \
  const int z = z0 + (R_) * static_cast<int>(threadIdx.x), x = x0 + threadIdx.y; \
  const bool live = z < g.nz && x < g.nx;                                      \
  const int rows_in = live ? g.nz - z : 0;                                     \
  const size_t ldz = static_cast<size_t>(g.ldz);                               \
  const size_t i = static_cast<size_t>(x) * ldz + z;                           \
  const int b = (threadIdx.y + 2) * (BOXZ_) + (R_) * threadIdx.x + 4;           \
  (void)rows_in;

// Values of the thread's R depths that lie in the grid (rows_in of them);
// the others are left 0.
template <int R>
__device__ __forceinline__ void ldrows(const float* p, int rows_in, float (&v)[R]) {
#pragma unroll
  for (int r = 0; r < R; ++r) v[r] = r < rows_in ? p[r] : 0.0f;
}

// Paired loads / stores of two adjacent depths (8-byte aligned: even depth,
// ldz a multiple of 32, even box index).
__device__ __forceinline__ float2 ld2(const float* p) { return *reinterpret_cast<const float2*>(p); }
__device__ __forceinline__ void st2(float* p, float a, float b) { *reinterpret_cast<float2*>(p) = make_float2(a, b); }

// 4th-order staggered difference from its four samples: (C1 (p - q) -
// C2 (s - t)) r, the expression of sdm / sdp.
__device__ __forceinline__ float dd(float p, float q, float s, float t, float r) {
  return (C1 * (p - q) - C2 * (s - t)) * r;
}

// Register budgets (measured on GB300 over the tile widths; the sweeps wait
// on memory latency, so resident warps count for more than the bytes
// spilled): forward sweeps 32 registers (64 warps per SM; with two cells per
// thread 9 % faster than 40 registers on a 16-shot group). Backward sweeps:
// NT resident threads per SM, so 65536 / NT registers: with one cell per
// thread 2048 (32 registers, 52-96 bytes spilled; 4 % faster than 40 on the
// 64-shot workload) or 1536 (40 registers; 10 % faster on a lone 608 x 1600
// shot, whose arrays stay partly in L2), picked by the autotuner; with two
// cells 1024 (64 registers).
#define FWD_BOUNDS __launch_bounds__(32 * TX, 2048 / (32 * TX))
#define BWD_BOUNDS __launch_bounds__(32 * TX, (NT / (32 * TX)) > 0 ? (NT / (32 * TX)) : 1)

// ---------------------------------------------------------------------------
// F1: el_stress (el_stress.cu:50-88) + add_source (utilities.cu:521-541) +
// recording (utilities.cu:557-567) + from_bnd of the 5 fields (Boundary.cu:55-76).
// Staged: vz, vx. Edge body: the per-cell code for each of the thread's R
// depths (after the staged tiles have landed).
template <int TX, int K, int R>
__device__ __forceinline__ void fwd_stress_edge(const SweepPack<K>& P, int shot, int z0, int x0, int it, int save,
                                                bool inject, unsigned* err) {
  constexpr int BOXZ = 32 * R + 8;
  SWEEP_BODY_SLOT()
  SWEEP_EDGE_CELL(BOXZ, R)
  SWEEP_SMEM(BOXZ)
  pdl_wait();
  SWEEP_TMA(2, BOXZ)
  if (!live) return;
  const ShotD& sh = S.sh;
  const bool rec_tile = tile_meets_shot_box(sh, z0, x0, 32 * R, TX);
  const StoreD& st = S.st;
  if (!stage_wait(&bar, err, inject)) return;
  const float* s_vz = sm;
  const float* s_vx = sm + N;
  auto cell = [&](const int z, const size_t i, const int b) {
    float szz = f.szz[i], sxx = f.sxx[i];
    const float sxz = f.sxz[i];
    const float lam = m.lam[i], l2m = m.l2m[i], amu = m.aveMu[i];
    if (save) {
      const int k = ring_index(g, z, x);
      if (k >= 0) {
        float* p = st.base + static_cast<size_t>(it) * 5 * g.ring_len + k;
        p[0] = szz;
        p[g.ring_len] = sxz;
        p[2 * g.ring_len] = sxx;
        p[3 * g.ring_len] = s_vz[b];
        p[4 * g.ring_len] = s_vx[b];
      }
    }
    const bool dom = in_box(z, x, g.zs0, g.zs1, g.xs0, g.xs1);
    const bool src = (z == sh.src_z && x == sh.src_x);
    if (dom) {
      float dvz_dz = sdm(s_vz, b, 1, g.rdz);
      float dvx_dx = sdm(s_vx, b, BOXZ, g.rdx);
      float dvx_dz = sdp(s_vx, b, 1, g.rdz);
      float dvz_dx = sdp(s_vz, b, BOXZ, g.rdx);
      if ((z < g.nPml) || (z > g.zpml_hi)) {
        float mm = c.b_z[z] * f.m_dvz_dz[i] + c.a_z[z] * dvz_dz;
        f.m_dvz_dz[i] = mm;
        dvz_dz = dvz_dz / c.K_z[z] + mm;
        mm = c.b_zh[z] * f.m_dvx_dz[i] + c.a_zh[z] * dvx_dz;
        f.m_dvx_dz[i] = mm;
        dvx_dz = dvx_dz / c.K_zh[z] + mm;
      }
      if ((x < g.nPml) || (x > g.xpml_hi_s)) {
        float mm = c.b_x[x] * f.m_dvx_dx[i] + c.a_x[x] * dvx_dx;
        f.m_dvx_dx[i] = mm;
        dvx_dx = dvx_dx / c.K_x[x] + mm;
        mm = c.b_xh[x] * f.m_dvz_dx[i] + c.a_xh[x] * dvz_dx;
        f.m_dvz_dx[i] = mm;
        dvz_dx = dvz_dx / c.K_xh[x] + mm;
      }
      szz += (l2m * dvz_dz + lam * dvx_dx) * g.dt;
      sxx += (lam * dvz_dz + l2m * dvx_dx) * g.dt;
      f.sxz[i] = sxz + amu * (dvx_dz + dvz_dx) * g.dt;
    }
    if (src) {
      szz += sh.src_szz[it];
      sxx += sh.src_sxx[it];
    }
    if (dom || src) {
      f.szz[i] = szz;
      f.sxx[i] = sxx;
    }
    // The velocity sweep that follows does not change the stresses, so the
    // sample of step it+1 is taken here.
    if (rec_tile && z >= sh.rbz0 && z <= sh.rbz1) {
      const int2 rr = bin_range(sh, z, x);
      for (int k = rr.x; k < rr.y; ++k) {
        const int r = sh.blk_rec[k];
        if (sh.rec_z[r] == z && sh.rec_x[r] == x)
          sh.data[static_cast<size_t>(r) * sh.nSteps + it + 1] = szz + 3.0f * sxx;
      }
    }
  };
#pragma unroll
  for (int r = 0; r < R; ++r)
    if (z + r < g.nz) cell(z + r, i + r, b + r);
}

// F2: el_velocity, isFor = true (el_velocity.cu:45-82). Staged: szz, sxx, sxz.
template <int TX, int K, int R>
__device__ __forceinline__ void fwd_velocity_edge(const SweepPack<K>& P, int shot, int z0, int x0, unsigned* err) {
  constexpr int BOXZ = 32 * R + 8;
  SWEEP_BODY_SLOT()
  SWEEP_EDGE_CELL(BOXZ, R)
  SWEEP_SMEM(BOXZ)
  pdl_wait();
  SWEEP_TMA(3, BOXZ)
  if (!live) return;
  if (!stage_wait(&bar, err)) return;
  const float* s_szz = sm;
  const float* s_sxx = sm + N;
  const float* s_sxz = sm + 2 * N;
  auto cell = [&](const int z, const size_t i, const int b) {
    if (!in_box(z, x, g.zs0, g.zs1, g.xs0, g.xs1)) return;
    const float vz = f.vz[i], vx = f.vx[i], bA = m.bycA[i], bB = m.bycB[i];
    float dszz_dz = sdp(s_szz, b, 1, g.rdz);
    float dsxz_dx = sdm(s_sxz, b, BOXZ, g.rdx);
    float dsxz_dz = sdm(s_sxz, b, 1, g.rdz);
    float dsxx_dx = sdp(s_sxx, b, BOXZ, g.rdx);
    if ((z < g.nPml) || (z > g.zpml_hi)) {
      float mm = c.b_zh[z] * f.m_dszz_dz[i] + c.a_zh[z] * dszz_dz;
      f.m_dszz_dz[i] = mm;
      dszz_dz = dszz_dz / c.K_zh[z] + mm;
      mm = c.b_z[z] * f.m_dsxz_dz[i] + c.a_z[z] * dsxz_dz;
      f.m_dsxz_dz[i] = mm;
      dsxz_dz = dsxz_dz / c.K_z[z] + mm;
    }
    if ((x < g.nPml) || (x > g.xpml_hi_v)) {
      float mm = c.b_x[x] * f.m_dsxz_dx[i] + c.a_x[x] * dsxz_dx;
      f.m_dsxz_dx[i] = mm;
      dsxz_dx = dsxz_dx / c.K_x[x] + mm;
      mm = c.b_xh[x] * f.m_dsxx_dx[i] + c.a_xh[x] * dsxx_dx;
      f.m_dsxx_dx[i] = mm;
      dsxx_dx = dsxx_dx / c.K_xh[x] + mm;
    }
    const float nvz = vz + (dszz_dz + dsxz_dx) * bA * g.dt;
    const float nvx = vx + (dsxz_dz + dsxx_dx) * bB * g.dt;
    f.vz[i] = nvz;
    f.vx[i] = nvx;
    if (S.gr.illum) S.gr.illum[i] += nvz * nvz + nvx * nvx;
  };
#pragma unroll
  for (int r = 0; r < R; ++r)
    if (z + r < g.nz) cell(z + r, i + r, b + r);
}

// ---------------------------------------------------------------------------
// B: add_source(-) + el_stress(isFor=false) with the lambda / mu kernels +
// to_bnd(stress) + el_velocity_adj. Staged: vz, vx, szz_a, sxx_a, sxz_a.
template <int TX, int K, int R>
__device__ __forceinline__ void bwd_B_edge(const SweepPack<K>& P, int shot, int z0, int x0, int j, unsigned* err) {
  constexpr int BOXZ = 32 * R + 8;
  SWEEP_BODY_SLOT()
  SWEEP_EDGE_CELL(BOXZ, R)
  SWEEP_SMEM(BOXZ)
  const Grads& gr = S.gr;
  float p_lam[R], p_l2m[R], p_amu[R], p_w[R], p_h[R];
  float p_szz[R], p_sxx[R], p_sxz[R], p_gl[R], p_gm[R], p_vza[R], p_vxa[R];
  ldrows<R>(m.lam + i, rows_in, p_lam);
  ldrows<R>(m.l2m + i, rows_in, p_l2m);
  ldrows<R>(m.aveMu + i, rows_in, p_amu);
  ldrows<R>(m.muw + i, rows_in, p_w);
  ldrows<R>(m.hs + i, rows_in, p_h);
  pdl_wait();
  SWEEP_TMA(5, BOXZ)
  ldrows<R>(f.szz + i, rows_in, p_szz);
  ldrows<R>(f.sxx + i, rows_in, p_sxx);
  ldrows<R>(f.sxz + i, rows_in, p_sxz);
  ldrows<R>(gr.lam + i, rows_in, p_gl);
  ldrows<R>(gr.mu + i, rows_in, p_gm);
  ldrows<R>(f.vz_a + i, rows_in, p_vza);
  ldrows<R>(f.vx_a + i, rows_in, p_vxa);
  if (!live) return;
  const ShotD& sh = S.sh;
  const StoreD& st = S.st;
  const int it = S.nSteps - 2 - j;  // this shot's time step at backward iteration j
  const float dt = g.dt;
  if (!stage_wait(&bar, err)) return;
  const float* s_vz = sm;
  const float* s_vx = sm + N;
  const float* s_szz_a = sm + 2 * N;
  const float* s_sxx_a = sm + 3 * N;
  const float* s_sxz_a = sm + 4 * N;
  auto cell = [&](const int r, const int z, const size_t i, const int b) {
  float szz = p_szz[r], sxx = p_sxx[r], sxz = p_sxz[r];
  const float lam = p_lam[r], l2m = p_l2m[r], amu = p_amu[r];
  const float gl = p_gl[r], gm = p_gm[r], w = p_w[r], h = p_h[r];
  const float va_z = p_vza[r], va_x = p_vxa[r];
  const bool interior = in_box(z, x, g.zi0, g.zi1, g.xi0, g.xi1);
  const bool src = (z == sh.src_z && x == sh.src_x);
  const int k = ring_index(g, z, x);
  float e_own = 0.0f, gmu_own = 0.0f;
  if (interior || src || k >= 0) {
    if (src) {
      szz -= sh.src_szz_r[it];
      sxx -= sh.src_sxx_r[it];
    }
    if (interior) {
      const float dvz_dz = sdm(s_vz, b, 1, g.rdz);
      const float dvx_dx = sdm(s_vx, b, BOXZ, g.rdx);
      const float dvx_dz = sdp(s_vx, b, 1, g.rdz);
      const float dvz_dx = sdp(s_vz, b, BOXZ, g.rdx);
      szz -= (l2m * dvz_dz + lam * dvx_dx) * dt;
      sxx -= (lam * dvz_dz + l2m * dvx_dx) * dt;
      e_own = dvx_dz + dvz_dx;
      sxz -= amu * e_own * dt;
      const float sa = s_szz_a[b], xa = s_sxx_a[b];
      gr.lam[i] = gl + -(sa + xa) * (dvz_dz + dvx_dx) * dt * kMega;
      gmu_own = (-2.0f * sa * dvz_dz * dt - 2.0f * xa * dvx_dx * dt) * kMega;
    }
    if (k >= 0) {
      const float* p = st.base + static_cast<size_t>(it) * 5 * g.ring_len + k;
      szz = p[0];
      sxz = p[g.ring_len];
      sxx = p[2 * g.ring_len];
    }
    f.szz[i] = szz;
    f.sxx[i] = sxx;
    f.sxz[i] = sxz;
  }
  // mu kernel: own term plus the harmonic-average chain rule of the 2x2 blocks
  // whose top-left corner is (z,x), (z-1,x), (z,x-1), (z-1,x-1), with the
  // guards of el_stress.cu:118-123 (the x guard of :120 is always true).
  if (in_box(z, x, g.zi0, g.zi1, g.xi0, g.xi1 + 1)) {
    float acc = gm + gmu_own;
    const float* __restrict__ hs = m.hs;
    if (x <= g.xi1) {
      if (h != 0.0f) acc += w * (-s_sxz_a[b] * e_own * dt * h);
      if (z - 1 >= g.zi0) {
        const float hj = hs[i - 1];
        const int bj = b - 1;
        if (hj != 0.0f)
          acc += w * (-s_sxz_a[bj] * (sdp(s_vx, bj, 1, g.rdz) + sdp(s_vz, bj, BOXZ, g.rdx)) * dt * hj);
      }
    }
    if (x - 1 >= g.xi0) {
      const float hj = hs[i - ldz];
      const int bj = b - BOXZ;
      if (hj != 0.0f) acc += w * (-s_sxz_a[bj] * (sdp(s_vx, bj, 1, g.rdz) + sdp(s_vz, bj, BOXZ, g.rdx)) * dt * hj);
      if (z - 1 >= g.zi0 && x <= g.xi1) {
        const float h2 = hs[i - ldz - 1];
        const int b2 = b - BOXZ - 1;
        if (h2 != 0.0f)
          acc += w * (-s_sxz_a[b2] * (sdp(s_vx, b2, 1, g.rdz) + sdp(s_vz, b2, BOXZ, g.rdx)) * dt * h2);
      }
    }
    gr.mu[i] = acc;
  }
  // el_velocity_adj (el_velocity_adj.cu:57-102); the psi memory terms are
  // read only where their CPML coefficient is non-zero.
  if (!in_box(z, x, g.zs0, g.zs1, g.xs0, g.xs1)) return;
  const bool zp = (z < g.nPml) || (z > g.zpml_hi);
  const bool xp = (x < g.nPml) || (x > g.xpml_hi_s);
  {
    const float Kx = c.K_x[x], Kzh = c.K_zh[z];
    const float dszz_dx = -sdp(s_szz_a, b, BOXZ, g.rdx);
    const float dsxx_dx = -sdp(s_sxx_a, b, BOXZ, g.rdx);
    const float dsxz_dz = -sdm(s_sxz_a, b, 1, g.rdz);
    float t = kdiv(lam * dszz_dx, Kx) * dt + kdiv(l2m * dsxx_dx, Kx) * dt + kdiv(amu, Kzh) * dsxz_dz * dt;
    const float ax = c.a_x[x], azh = c.a_zh[z];
    if (ax != 0.0f) t += ax * (-gdp(f.m_dvx_dx, i, ldz, g.rdx));
    if (azh != 0.0f) t += azh * (-gdm(f.m_dvx_dz, i, 1, g.rdz));
    const float v = va_x + t;
    f.vx_a[i] = v;
    if (xp || zp) {
      const float bB = m.bycB[i];
      if (xp) f.m_dsxx_dx[i] = c.b_xh[x] * f.m_dsxx_dx[i] + bB * v * dt;
      if (zp) f.m_dsxz_dz[i] = c.b_z[z] * f.m_dsxz_dz[i] + bB * v * dt;
    }
  }
  {
    const float Kz = c.K_z[z], Kxh = c.K_xh[x];
    const float dszz_dz = -sdp(s_szz_a, b, 1, g.rdz);
    const float dsxx_dz = -sdp(s_sxx_a, b, 1, g.rdz);
    const float dsxz_dx = -sdm(s_sxz_a, b, BOXZ, g.rdx);
    float t = kdiv(l2m * dszz_dz, Kz) * dt + kdiv(lam * dsxx_dz, Kz) * dt + kdiv(amu, Kxh) * dsxz_dx * dt;
    const float az = c.a_z[z], axh = c.a_xh[x];
    if (az != 0.0f) t += az * (-gdp(f.m_dvz_dz, i, 1, g.rdz));
    if (axh != 0.0f) t += axh * (-gdm(f.m_dvz_dx, i, ldz, g.rdx));
    const float v = va_z + t;
    f.vz_a[i] = v;
    if (xp || zp) {
      const float bA = m.bycA[i];
      if (xp) f.m_dsxz_dx[i] = c.b_x[x] * f.m_dsxz_dx[i] + bA * v * dt;
      if (zp) f.m_dszz_dz[i] = c.b_zh[z] * f.m_dszz_dz[i] + bA * v * dt;
    }
  }
  };
#pragma unroll
  for (int r = 0; r < R; ++r)
    if (z + r < g.nz) cell(r, z + r, i + r, b + r);
}

// C: res_injection (utilities.cu:569-580) + el_stress_adj (el_stress_adj.cu:53-97)
//    + source_grad (utilities.cu:582-593) + el_velocity(isFor=false) with the
//    density kernel (el_velocity.cu:84-117) + to_bnd(velocity).
//    Staged: vz_a, vx_a, szz, sxx, sxz.
template <int TX, int K, int R>
__device__ __forceinline__ void bwd_C_edge(const SweepPack<K>& P, int shot, int z0, int x0, int j, unsigned* err) {
  constexpr int BOXZ = 32 * R + 8;
  SWEEP_BODY_SLOT()
  SWEEP_EDGE_CELL(BOXZ, R)
  SWEEP_SMEM(BOXZ)
  const Grads& gr = S.gr;
  const int rev = S.nSteps - 2 - j >= 1;
  float p_bA[R], p_bB[R], p_amu[R], p_lam[R], p_l2m[R], p_sa[R], p_xa[R], p_za[R], p_vz[R], p_vx[R], p_gd[R];
  ldrows<R>(m.bycA + i, rows_in, p_bA);
  ldrows<R>(m.bycB + i, rows_in, p_bB);
  ldrows<R>(m.aveMu + i, rows_in, p_amu);
  ldrows<R>(m.lam + i, rows_in, p_lam);
  ldrows<R>(m.l2m + i, rows_in, p_l2m);
  pdl_wait();
  SWEEP_TMA(5, BOXZ)
  ldrows<R>(f.szz_a + i, rows_in, p_sa);
  ldrows<R>(f.sxx_a + i, rows_in, p_xa);
  ldrows<R>(f.sxz_a + i, rows_in, p_za);
  ldrows<R>(f.vz + i, rev ? rows_in : 0, p_vz);
  ldrows<R>(f.vx + i, rev ? rows_in : 0, p_vx);
  ldrows<R>(gr.den + i, rev ? rows_in : 0, p_gd);
  if (!live) return;
  const ShotD& sh = S.sh;
  const StoreD& st = S.st;
  const bool rec_tile = tile_meets_shot_box(sh, z0, x0, 32 * R, TX);
  // Backward iteration j handles res_injection + el_stress_adj of step
  // it = nSteps - 2 - j (j = -1: the shot's last step) and the reverse
  // velocity of step it - 1.
  const int it = S.nSteps - 2 - j;
  const float dt = g.dt;
  if (!stage_wait(&bar, err)) return;
  const float* s_vz_a = sm;
  const float* s_vx_a = sm + N;
  const float* s_szz = sm + 2 * N;
  const float* s_sxx = sm + 3 * N;
  const float* s_sxz = sm + 4 * N;
  auto cell = [&](const int r, const int z, const size_t i, const int b) {
  float sa = p_sa[r], xa = p_xa[r], za = p_za[r];
  const float bA = p_bA[r], bB = p_bB[r], amu = p_amu[r], lam = p_lam[r], l2m = p_l2m[r];
  float vz = p_vz[r], vx = p_vx[r], gd = p_gd[r];
  const bool dom = in_box(z, x, g.zs0, g.zs1, g.xs0, g.xs1);
  bool injected = false;
  if (rec_tile && z >= sh.rbz0 && z <= sh.rbz1) {
    const int2 rr = bin_range(sh, z, x);
    for (int k = rr.x; k < rr.y; ++k) {
      const int r = sh.blk_rec[k];
      if (sh.rec_z[r] == z && sh.rec_x[r] == x) {
        const float rv = sh.res[static_cast<size_t>(r) * sh.nSteps + it];
        sa += rv;
        xa += 3.0f * rv;
        injected = true;
      }
    }
  }
  if (dom) {
    {
      const float dvz_dx = -sdp(s_vz_a, b, BOXZ, g.rdx);
      const float dvx_dz = -sdp(s_vx_a, b, 1, g.rdz);
      float t = kdiv(dvz_dx, c.K_x[x]) * bA * dt + kdiv(dvx_dz, c.K_z[z]) * bB * dt;
      const float ax = c.a_x[x], az = c.a_z[z];
      if (ax != 0.0f) t += ax * (-gdp(f.m_dsxz_dx, i, ldz, g.rdx));
      if (az != 0.0f) t += az * (-gdp(f.m_dsxz_dz, i, 1, g.rdz));
      za += t;
      f.sxz_a[i] = za;
    }
    const bool xb = (x <= g.xband_lo) || (x >= g.xband_hi);
    const bool zb = (z <= g.zband_lo) || (z >= g.zband_hi);
    if (xb) f.m_dvz_dx[i] = c.b_xh[x] * f.m_dvz_dx[i] + za * amu * dt;
    if (zb) f.m_dvx_dz[i] = c.b_zh[z] * f.m_dvx_dz[i] + za * amu * dt;
    {
      const float dvx_dx = -sdm(s_vx_a, b, BOXZ, g.rdx);
      const float dvz_dz = -sdm(s_vz_a, b, 1, g.rdz);
      float tx = kdiv(bB * dvx_dx, c.K_xh[x]) * dt;
      float tz = kdiv(bA * dvz_dz, c.K_zh[z]) * dt;
      const float axh = c.a_xh[x], azh = c.a_zh[z];
      if (axh != 0.0f) tx += axh * (-gdm(f.m_dsxx_dx, i, ldz, g.rdx));
      if (azh != 0.0f) tz += azh * (-gdm(f.m_dszz_dz, i, 1, g.rdz));
      xa += tx;
      sa += tz;
    }
    if (xb) f.m_dvx_dx[i] = c.b_x[x] * f.m_dvx_dx[i] + lam * sa * dt + l2m * xa * dt;
    if (zb) f.m_dvz_dz[i] = c.b_z[z] * f.m_dvz_dz[i] + l2m * sa * dt + lam * xa * dt;
  }
  if (dom || injected) {
    f.szz_a[i] = sa;
    f.sxx_a[i] = xa;
  }
  if (!rev) return;
  if (z == sh.src_z && x == sh.src_x) sh.gstf[it - 1] = -(sa + 3.0f * xa) * dt;
  const bool interior = in_box(z, x, g.zi0, g.zi1, g.xi0, g.xi1);
  float tA = 0.0f, tB = 0.0f;
  const int k = ring_index(g, z, x);
  if (interior) {
    const float ea = sdp(s_szz, b, 1, g.rdz) + sdm(s_sxz, b, BOXZ, g.rdx);  // dszz_dz + dsxz_dx
    const float eb = sdm(s_sxz, b, 1, g.rdz) + sdp(s_sxx, b, BOXZ, g.rdx);  // dsxz_dz + dsxx_dx
    vz -= ea * bA * dt;
    vx -= eb * bB * dt;
    tA = -s_vz_a[b] * ea * dt * (-bA * bA * 0.5f);
    tB = -s_vx_a[b] * eb * dt * (-bB * bB * 0.5f);
  }
  if (k >= 0) {
    const float* p = st.base + static_cast<size_t>(it - 1) * 5 * g.ring_len + k;
    vz = p[3 * g.ring_len];
    vx = p[4 * g.ring_len];
  }
  if (interior || k >= 0) {
    f.vz[i] = vz;
    f.vx[i] = vx;
  }
  // rho kernel gather: (z,x) receives A and B of itself, A of (z-1,x) and B of
  // (z,x-1) (el_velocity.cu:101-110; the x guard of :109 is always true).
  if (in_box(z, x, g.zi0, g.zi1, g.xi0, g.xi1 + 1)) {
    float acc = gd;
    if (x <= g.xi1) {
      acc += tA;
      acc += tB;
      if (z - 1 >= g.zi0) {
        const int bj = b - 1;
        const float bAj = m.bycA[i - 1];
        const float ea = sdp(s_szz, bj, 1, g.rdz) + sdm(s_sxz, bj, BOXZ, g.rdx);
        acc += -s_vz_a[bj] * ea * dt * (-bAj * bAj * 0.5f);
      }
    }
    if (x - 1 >= g.xi0) {
      const int bj = b - BOXZ;
      const float bBj = m.bycB[i - ldz];
      const float eb = sdm(s_sxz, bj, 1, g.rdz) + sdp(s_sxx, bj, BOXZ, g.rdx);
      acc += -s_vx_a[bj] * eb * dt * (-bBj * bBj * 0.5f);
    }
    gr.den[i] = acc;
  }
  };
#pragma unroll
  for (int r = 0; r < R; ++r)
    if (z + r < g.nz) cell(r, z + r, i + r, b + r);
}

// ---------------------------------------------------------------------------
// Fast-tile forms of the four sweeps. Every cell of a fast tile is in the
// stencil domain and the reverse-time interior, outside the CPML, the
// adjoint memory bands and the boundary ring, with K = 1 and a = 0: the
// reference's CPML divisions by K are exact there (x / 1 = x) and are left
// out, the memory-array updates and the ring are never reached, and the
// source / receiver terms are evaluated only in tiles that meet the bounding
// box of the shot's receivers and source. Operation order otherwise follows
// the edge kernels.

// Forward fast bodies, one depth per thread (32-row tiles).
// MID: the tile is a mid tile (no CPML cell; it may hold ring cells), and
// the boundary ring of step it is saved when `save` is set.
// The media arrays are read by every sweep and, in a batched launch, by every
// shot of the pack (their sub-grids are windows of the same model): their
// loads carry an L2 evict-last policy so that the streamed fields do not push
// them out of L2 (createpolicy / ld.global.L2::cache_hint).
__device__ __forceinline__ uint64_t media_policy() {
  uint64_t p;
  asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ float ldm(const float* a, uint64_t pol) {
  float v;
  asm("ld.global.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(v) : "l"(a), "l"(pol));
  return v;
}
__device__ __forceinline__ float2 ldm2(const float* a, uint64_t pol) {
  float2 v;
  asm("ld.global.L2::cache_hint.v2.f32 {%0, %1}, [%2], %3;" : "=f"(v.x), "=f"(v.y) : "l"(a), "l"(pol));
  return v;
}
template <int R>
__device__ __forceinline__ void ldrm(const float* p, float (&v)[R], uint64_t pol) {
  if constexpr (R == 2) {
    const float2 t = ldm2(p, pol);
    v[0] = t.x;
    v[1] = t.y;
  } else {
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = ldm(p + r, pol);
  }
}

template <int TX, int K, bool MID>
__device__ __forceinline__ void fwd_stress_fast1(const SweepPack<K>& P, int shot, int z0, int x0, int it, int save,
                                                 bool inject, unsigned* err) {
  SWEEP_FAST_SLOT(kTileZ)
  SWEEP_CELL(kBoxZ, 1)
  SWEEP_SMEM(kBoxZ)
  const uint64_t pol = media_policy();
  const float lam = ldm(m.lam + i, pol), l2m = ldm(m.l2m + i, pol), amu = ldm(m.aveMu + i, pol);
  pdl_wait();
  SWEEP_TMA(2, kBoxZ)
  float szz = f.szz[i], sxx = f.sxx[i];
  const float sxz = f.sxz[i];
  if (!stage_wait(&bar, err, inject)) return;
  const float* s_vz = sm;
  const float* s_vx = sm + N;
  if constexpr (MID) {
    if (save) ring_save(g, S.st, it, z, x, szz, sxz, sxx, s_vz[b], s_vx[b]);
  } else {
    (void)save;
  }
  const float dvz_dz = sdm(s_vz, b, 1, g.rdz);
  const float dvx_dx = sdm(s_vx, b, kBoxZ, g.rdx);
  const float dvx_dz = sdp(s_vx, b, 1, g.rdz);
  const float dvz_dx = sdp(s_vz, b, kBoxZ, g.rdx);
  szz += (l2m * dvz_dz + lam * dvx_dx) * g.dt;
  sxx += (lam * dvz_dz + l2m * dvx_dx) * g.dt;
  f.sxz[i] = sxz + amu * (dvx_dz + dvz_dx) * g.dt;
  if (special) {
    if (z == sh.src_z && x == sh.src_x) {
      szz += sh.src_szz[it];
      sxx += sh.src_sxx[it];
    }
    if (z >= sh.rbz0 && z <= sh.rbz1) {
      const int2 rr = bin_range(sh, z, x);
      for (int k = rr.x; k < rr.y; ++k) {
        const int r = sh.blk_rec[k];
        if (sh.rec_z[r] == z && sh.rec_x[r] == x)
          sh.data[static_cast<size_t>(r) * sh.nSteps + it + 1] = szz + 3.0f * sxx;
      }
    }
  }
  f.szz[i] = szz;
  f.sxx[i] = sxx;
}

template <int TX, int K>
__device__ __forceinline__ void fwd_velocity_fast1(const SweepPack<K>& P, int shot, int z0, int x0, unsigned* err) {
  SWEEP_FAST_SLOT(kTileZ)
  (void)special;
  SWEEP_CELL(kBoxZ, 1)
  SWEEP_SMEM(kBoxZ)
  const uint64_t pol = media_policy();
  const float bA = ldm(m.bycA + i, pol), bB = ldm(m.bycB + i, pol);
  pdl_wait();
  SWEEP_TMA(3, kBoxZ)
  const float vz = f.vz[i], vx = f.vx[i];
  if (!stage_wait(&bar, err)) return;
  const float* s_szz = sm;
  const float* s_sxx = sm + N;
  const float* s_sxz = sm + 2 * N;
  const float dszz_dz = sdp(s_szz, b, 1, g.rdz);
  const float dsxz_dx = sdm(s_sxz, b, kBoxZ, g.rdx);
  const float dsxz_dz = sdm(s_sxz, b, 1, g.rdz);
  const float dsxx_dx = sdp(s_sxx, b, kBoxZ, g.rdx);
  const float nvz = vz + (dszz_dz + dsxz_dx) * bA * g.dt;
  const float nvx = vx + (dsxz_dz + dsxx_dx) * bB * g.dt;
  f.vz[i] = nvz;
  f.vx[i] = nvx;
  if (S.gr.illum) S.gr.illum[i] += nvz * nvz + nvx * nvx;
}

// Forward fast bodies, two adjacent depths per thread (R = 2): own-cell
// operands and results move as float2, and the staged samples are read in
// pairs (b-2, b-1), (b, b+1), (b+2, b+3) along z and (b, b+1) at each
// column offset along x, which cover the stencils of both depths.
template <int TX, int K, int R, bool MID>
__device__ __forceinline__ void fwd_stress_fast2(const SweepPack<K>& P, int shot, int z0, int x0, int it, int save,
                                                 bool inject, unsigned* err) {
  static_assert(R == 2, "the forward fast bodies handle two depths per thread");
  constexpr int TZ = 32 * R, BOXZ = TZ + 8;
  SWEEP_FAST_SLOT(TZ)
  SWEEP_CELL(BOXZ, R)
  SWEEP_SMEM(BOXZ)
  const uint64_t pol = media_policy();
  const float2 lam = ldm2(m.lam + i, pol), l2m = ldm2(m.l2m + i, pol), amu = ldm2(m.aveMu + i, pol);
  pdl_wait();
  SWEEP_TMA(2, BOXZ)
  const float2 szz = ld2(f.szz + i), sxx = ld2(f.sxx + i), sxz = ld2(f.sxz + i);
  if (!stage_wait(&bar, err, inject)) return;
  const float* s_vz = sm;
  const float* s_vx = sm + N;
  if constexpr (MID) {
    if (save) {
      ring_save(g, S.st, it, z, x, szz.x, sxz.x, sxx.x, s_vz[b], s_vx[b]);
      ring_save(g, S.st, it, z + 1, x, szz.y, sxz.y, sxx.y, s_vz[b + 1], s_vx[b + 1]);
    }
  } else {
    (void)save;
  }
  const float rdz = g.rdz, rdx = g.rdx, dt = g.dt;
  const float2 zm = ld2(s_vz + b - 2), z0v = ld2(s_vz + b), zp = ld2(s_vz + b + 2);
  const float2 xm = ld2(s_vx + b - 2), x0v = ld2(s_vx + b), xp = ld2(s_vx + b + 2);
  const float2 zc1 = ld2(s_vz + b + BOXZ), zc2 = ld2(s_vz + b + 2 * BOXZ), zcm = ld2(s_vz + b - BOXZ);
  const float2 xc1 = ld2(s_vx + b + BOXZ), xcm = ld2(s_vx + b - BOXZ), xcm2 = ld2(s_vx + b - 2 * BOXZ);
  // depth z (.x): sdm_z(vz) = dd(a[b], a[b-1], a[b+1], a[b-2]); sdp_z(vx) = dd(a[b+1], a[b], a[b+2], a[b-1])
  const float dvz_dz0 = dd(z0v.x, zm.y, z0v.y, zm.x, rdz), dvz_dz1 = dd(z0v.y, z0v.x, zp.x, zm.y, rdz);
  const float dvx_dz0 = dd(x0v.y, x0v.x, xp.x, xm.y, rdz), dvx_dz1 = dd(xp.x, x0v.y, xp.y, x0v.x, rdz);
  // along x: sdm_x(vx) = dd(a[b], a[b-B], a[b+B], a[b-2B]); sdp_x(vz) = dd(a[b+B], a[b], a[b+2B], a[b-B])
  const float dvx_dx0 = dd(x0v.x, xcm.x, xc1.x, xcm2.x, rdx), dvx_dx1 = dd(x0v.y, xcm.y, xc1.y, xcm2.y, rdx);
  const float dvz_dx0 = dd(zc1.x, z0v.x, zc2.x, zcm.x, rdx), dvz_dx1 = dd(zc1.y, z0v.y, zc2.y, zcm.y, rdx);
  float szz0 = szz.x + (l2m.x * dvz_dz0 + lam.x * dvx_dx0) * dt;
  float szz1 = szz.y + (l2m.y * dvz_dz1 + lam.y * dvx_dx1) * dt;
  float sxx0 = sxx.x + (lam.x * dvz_dz0 + l2m.x * dvx_dx0) * dt;
  float sxx1 = sxx.y + (lam.y * dvz_dz1 + l2m.y * dvx_dx1) * dt;
  st2(f.sxz + i, sxz.x + amu.x * (dvx_dz0 + dvz_dx0) * dt, sxz.y + amu.y * (dvx_dz1 + dvz_dx1) * dt);
  if (special) {
    float* szr[2] = {&szz0, &szz1};
    float* sxr[2] = {&sxx0, &sxx1};
#pragma unroll
    for (int r = 0; r < 2; ++r) {
      const int zr = z + r;
      if (zr == sh.src_z && x == sh.src_x) {
        *szr[r] += sh.src_szz[it];
        *sxr[r] += sh.src_sxx[it];
      }
      if (zr < sh.rbz0 || zr > sh.rbz1) continue;
      const int2 rr = bin_range(sh, zr, x);
      for (int k = rr.x; k < rr.y; ++k) {
        const int q = sh.blk_rec[k];
        if (sh.rec_z[q] == zr && sh.rec_x[q] == x)
          sh.data[static_cast<size_t>(q) * sh.nSteps + it + 1] = *szr[r] + 3.0f * *sxr[r];
      }
    }
  }
  st2(f.szz + i, szz0, szz1);
  st2(f.sxx + i, sxx0, sxx1);
}

template <int TX, int K, int R>
__device__ __forceinline__ void fwd_velocity_fast2(const SweepPack<K>& P, int shot, int z0, int x0, unsigned* err) {
  static_assert(R == 2, "the forward fast bodies handle two depths per thread");
  constexpr int TZ = 32 * R, BOXZ = TZ + 8;
  SWEEP_FAST_SLOT(TZ)
  (void)special;
  SWEEP_CELL(BOXZ, R)
  SWEEP_SMEM(BOXZ)
  const uint64_t pol = media_policy();
  const float2 bA = ldm2(m.bycA + i, pol), bB = ldm2(m.bycB + i, pol);
  pdl_wait();
  SWEEP_TMA(3, BOXZ)
  const float2 vz = ld2(f.vz + i), vx = ld2(f.vx + i);
  if (!stage_wait(&bar, err)) return;
  const float* s_szz = sm;
  const float* s_sxx = sm + N;
  const float* s_sxz = sm + 2 * N;
  const float rdz = g.rdz, rdx = g.rdx, dt = g.dt;
  const float2 pm = ld2(s_szz + b - 2), p0 = ld2(s_szz + b), pp = ld2(s_szz + b + 2);
  const float2 qm = ld2(s_sxz + b - 2), q0 = ld2(s_sxz + b), qp = ld2(s_sxz + b + 2);
  const float2 qcm = ld2(s_sxz + b - BOXZ), qc1 = ld2(s_sxz + b + BOXZ), qcm2 = ld2(s_sxz + b - 2 * BOXZ);
  const float2 r0 = ld2(s_sxx + b), rc1 = ld2(s_sxx + b + BOXZ), rc2 = ld2(s_sxx + b + 2 * BOXZ),
               rcm = ld2(s_sxx + b - BOXZ);
  // sdp_z(szz) = dd(a[b+1], a[b], a[b+2], a[b-1]); sdm_x(sxz) = dd(a[b], a[b-B], a[b+B], a[b-2B]);
  // sdm_z(sxz) = dd(a[b], a[b-1], a[b+1], a[b-2]); sdp_x(sxx) = dd(a[b+B], a[b], a[b+2B], a[b-B])
  const float dszz_dz0 = dd(p0.y, p0.x, pp.x, pm.y, rdz), dszz_dz1 = dd(pp.x, p0.y, pp.y, p0.x, rdz);
  const float dsxz_dx0 = dd(q0.x, qcm.x, qc1.x, qcm2.x, rdx), dsxz_dx1 = dd(q0.y, qcm.y, qc1.y, qcm2.y, rdx);
  const float dsxz_dz0 = dd(q0.x, qm.y, q0.y, qm.x, rdz), dsxz_dz1 = dd(q0.y, q0.x, qp.x, qm.y, rdz);
  const float dsxx_dx0 = dd(rc1.x, r0.x, rc2.x, rcm.x, rdx), dsxx_dx1 = dd(rc1.y, r0.y, rc2.y, rcm.y, rdx);
  const float nvz0 = vz.x + (dszz_dz0 + dsxz_dx0) * bA.x * dt, nvz1 = vz.y + (dszz_dz1 + dsxz_dx1) * bA.y * dt;
  const float nvx0 = vx.x + (dsxz_dz0 + dsxx_dx0) * bB.x * dt, nvx1 = vx.y + (dsxz_dz1 + dsxx_dx1) * bB.y * dt;
  st2(f.vz + i, nvz0, nvz1);
  st2(f.vx + i, nvx0, nvx1);
  if (S.gr.illum) {
    const float2 e = ld2(S.gr.illum + i);
    st2(S.gr.illum + i, e.x + (nvz0 * nvz0 + nvx0 * nvx0), e.y + (nvz1 * nvz1 + nvx1 * nvx1));
  }
}

// Own-cell values of a thread's R adjacent depths (8-byte paired when R == 2:
// even depth, ldz a multiple of 32).
template <int R>
__device__ __forceinline__ void ldr(const float* p, float (&v)[R]) {
  if constexpr (R == 2) {
    const float2 t = ld2(p);
    v[0] = t.x;
    v[1] = t.y;
  } else {
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = p[r];
  }
}
template <int R>
__device__ __forceinline__ void str(float* p, const float (&v)[R]) {
  if constexpr (R == 2) {
    st2(p, v[0], v[1]);
  } else {
#pragma unroll
    for (int r = 0; r < R; ++r) p[r] = v[r];
  }
}

// Backward fast bodies, R adjacent depths per thread (tiles of 32 R rows):
// the own-cell operands of all R depths are loaded before the staged tiles
// are awaited; the depths are then computed in turn (the stencil samples
// two depths share are read once after unrolling).
// MID: a mid tile (no CPML cell): the reverse stress update and the lambda
// term only at cells of the reverse-time interior, the ring's stresses of
// step it restored, and the mu gathers with the guards of the edge form.
template <int TX, int K, int R, bool MID>
__device__ __forceinline__ void bwd_B_fast(const SweepPack<K>& P, int shot, int z0, int x0, int j, unsigned* err) {
  constexpr int TZ = 32 * R, BOXZ = TZ + 8;
  SWEEP_FAST_SLOT(TZ)
  SWEEP_CELL(BOXZ, R)
  SWEEP_SMEM(BOXZ)
  const Grads& gr = S.gr;
  const int it = S.nSteps - 2 - j;
  const float dt = g.dt;
  float szz[R], sxx[R], sxz[R], lam[R], l2m[R], amu[R], gl[R], gm[R], w[R], h[R], va_z[R], va_x[R], hx[R];
  const uint64_t pol = media_policy();
  ldrm<R>(m.lam + i, lam, pol);
  ldrm<R>(m.l2m + i, l2m, pol);
  ldrm<R>(m.aveMu + i, amu, pol);
  ldrm<R>(m.muw + i, w, pol);
  ldrm<R>(m.hs + i, h, pol);
  ldrm<R>(m.hs + i - ldz, hx, pol);
  const float hz0 = ldm(m.hs + i - 1, pol), hzx0 = ldm(m.hs + i - ldz - 1, pol);
  pdl_wait();
  SWEEP_TMA(5, BOXZ)
  ldr<R>(f.szz + i, szz);
  ldr<R>(f.sxx + i, sxx);
  ldr<R>(f.sxz + i, sxz);
  ldr<R>(gr.lam + i, gl);
  ldr<R>(gr.mu + i, gm);
  ldr<R>(f.vz_a + i, va_z);
  ldr<R>(f.vx_a + i, va_x);
  // Fast one-row tiles share the strain e = dvx_dz + dvz_dx of the mu
  // gathers: each thread computes its own cell's, warp 0 the tile's x0 - 1
  // column and z0 - 1 row, and the gathers read their neighbours' from
  // shared memory (s_e: columns x0 - 1 .. x0 + TX - 1, depths z0 - 1 ..
  // z0 + 31, stride 33) instead of recomputing them. Same operations per value.
  constexpr bool kShare = !MID && R == 1;
  const bool ok = stage_wait(&bar, err);
  if constexpr (kShare) {
    if (!__syncthreads_and(ok)) return;  // (a uniform exit: the block meets a barrier below)
  } else {
    if (!ok) return;
  }
  const float* s_vz = sm;
  const float* s_vx = sm + N;
  const float* s_szz_a = sm + 2 * N;
  const float* s_sxx_a = sm + 3 * N;
  const float* s_sxz_a = sm + 4 * N;
  float e_me = 0.0f, e_up = 0.0f, e_left = 0.0f, e_upleft = 0.0f;
  if constexpr (kShare) {
    float* s_e = sm + 5 * N;
    const int ty = threadIdx.y, tx = threadIdx.x;
    e_me = sdp(s_vx, b, 1, g.rdz) + sdp(s_vz, b, BOXZ, g.rdx);
    s_e[(ty + 1) * 33 + tx + 1] = e_me;
    if (ty == 0) {
      const int bl = b - BOXZ;  // (z, x0 - 1)
      s_e[tx + 1] = sdp(s_vx, bl, 1, g.rdz) + sdp(s_vz, bl, BOXZ, g.rdx);
      if (tx <= TX) {
        const int bu = (tx + 1) * BOXZ + 3;  // (z0 - 1, x0 - 1 + tx)
        s_e[tx * 33] = sdp(s_vx, bu, 1, g.rdz) + sdp(s_vz, bu, BOXZ, g.rdx);
      }
    }
    __syncthreads();
    e_up = s_e[(ty + 1) * 33 + tx];
    e_left = s_e[ty * 33 + tx + 1];
    e_upleft = s_e[ty * 33 + tx];
  }
  float o_gl[R], o_gm[R], o_szz[R], o_sxx[R], o_sxz[R], o_vza[R], o_vxa[R];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int bb = b + r;
    const int zr = z + r;
    const float hz = r == 0 ? hz0 : h[r - 1];     // hs at (z-1, x)
    const float hzx = r == 0 ? hzx0 : hx[r - 1];  // hs at (z-1, x-1)
    if (special && zr == sh.src_z && x == sh.src_x) {
      szz[r] -= sh.src_szz_r[it];
      sxx[r] -= sh.src_sxx_r[it];
    }
    const bool inter = !MID || in_box(zr, x, g.zi0, g.zi1, g.xi0, g.xi1);
    const float dvz_dz = sdm(s_vz, bb, 1, g.rdz);
    const float dvx_dx = sdm(s_vx, bb, BOXZ, g.rdx);
    float e_own = 0.0f, gmu_own = 0.0f;
    if (inter) {
      o_szz[r] = szz[r] - (l2m[r] * dvz_dz + lam[r] * dvx_dx) * dt;
      o_sxx[r] = sxx[r] - (lam[r] * dvz_dz + l2m[r] * dvx_dx) * dt;
      if constexpr (kShare)
        e_own = e_me;
      else
        e_own = sdp(s_vx, bb, 1, g.rdz) + sdp(s_vz, bb, BOXZ, g.rdx);  // dvx_dz + dvz_dx
      o_sxz[r] = sxz[r] - amu[r] * e_own * dt;
      const float sa = s_szz_a[bb], xa = s_sxx_a[bb];
      o_gl[r] = gl[r] + -(sa + xa) * (dvz_dz + dvx_dx) * dt * kMega;
      gmu_own = (-2.0f * sa * dvz_dz * dt - 2.0f * xa * dvx_dx * dt) * kMega;
    } else {
      o_szz[r] = szz[r];
      o_sxx[r] = sxx[r];
      o_sxz[r] = sxz[r];
      o_gl[r] = gl[r];
    }
    if constexpr (MID) {  // to_bnd of the stresses (the ring's values replace the update)
      const int k = ring_index(g, zr, x);
      if (k >= 0) {
        const float* p = S.st.base + static_cast<size_t>(it) * 5 * g.ring_len + k;
        o_szz[r] = p[0];
        o_sxz[r] = p[g.ring_len];
        o_sxx[r] = p[2 * g.ring_len];
      }
    }
    // mu kernel: own term and the three neighbouring 2x2 blocks; in a fast
    // tile all guards hold, in a mid tile they are those of el_stress.cu:118-123.
    if (!MID || in_box(zr, x, g.zi0, g.zi1, g.xi0, g.xi1 + 1)) {
      const bool own_col = !MID || x <= g.xi1;
      const bool up = !MID || zr - 1 >= g.zi0;
      const bool left = !MID || x - 1 >= g.xi0;
      float acc = gm[r] + gmu_own;
      if (own_col) {
        if (h[r] != 0.0f) acc += w[r] * (-s_sxz_a[bb] * e_own * dt * h[r]);
        if (up && hz != 0.0f) {
          const int bj = bb - 1;
          const float e = kShare ? e_up : sdp(s_vx, bj, 1, g.rdz) + sdp(s_vz, bj, BOXZ, g.rdx);
          acc += w[r] * (-s_sxz_a[bj] * e * dt * hz);
        }
      }
      if (left) {
        if (hx[r] != 0.0f) {
          const int bj = bb - BOXZ;
          const float e = kShare ? e_left : sdp(s_vx, bj, 1, g.rdz) + sdp(s_vz, bj, BOXZ, g.rdx);
          acc += w[r] * (-s_sxz_a[bj] * e * dt * hx[r]);
        }
        if (up && own_col && hzx != 0.0f) {
          const int b2 = bb - BOXZ - 1;
          const float e = kShare ? e_upleft : sdp(s_vx, b2, 1, g.rdz) + sdp(s_vz, b2, BOXZ, g.rdx);
          acc += w[r] * (-s_sxz_a[b2] * e * dt * hzx);
        }
      }
      o_gm[r] = acc;
    } else {
      o_gm[r] = gm[r];
    }
    // el_velocity_adj without the psi memory terms.
    {
      const float dszz_dx = -sdp(s_szz_a, bb, BOXZ, g.rdx);
      const float dsxx_dx = -sdp(s_sxx_a, bb, BOXZ, g.rdx);
      const float dsxz_dz = -sdm(s_sxz_a, bb, 1, g.rdz);
      o_vxa[r] = va_x[r] + (lam[r] * dszz_dx * dt + l2m[r] * dsxx_dx * dt + amu[r] * dsxz_dz * dt);
    }
    {
      const float dszz_dz = -sdp(s_szz_a, bb, 1, g.rdz);
      const float dsxx_dz = -sdp(s_sxx_a, bb, 1, g.rdz);
      const float dsxz_dx = -sdm(s_sxz_a, bb, BOXZ, g.rdx);
      o_vza[r] = va_z[r] + (l2m[r] * dszz_dz * dt + lam[r] * dsxx_dz * dt + amu[r] * dsxz_dx * dt);
    }
  }
  str<R>(gr.lam + i, o_gl);
  str<R>(f.szz + i, o_szz);
  str<R>(f.sxx + i, o_sxx);
  str<R>(f.sxz + i, o_sxz);
  str<R>(gr.mu + i, o_gm);
  str<R>(f.vx_a + i, o_vxa);
  str<R>(f.vz_a + i, o_vza);
}

// MID: a mid tile (no CPML cell): the adjoint memory arrays updated in their
// bands (el_stress_adj.cu:68-94, within 2 cells of the CPML), the reverse
// velocity update and its density terms only at cells of the reverse-time
// interior, the ring's velocities of step it-1 restored, and the density
// gathers with the guards of the edge form.
template <int TX, int K, int R, bool MID>
__device__ __forceinline__ void bwd_C_fast(const SweepPack<K>& P, int shot, int z0, int x0, int j, unsigned* err) {
  constexpr int TZ = 32 * R, BOXZ = TZ + 8;
  SWEEP_FAST_SLOT(TZ)
  SWEEP_CELL(BOXZ, R)
  SWEEP_SMEM(BOXZ)
  const Grads& gr = S.gr;
  const int it = S.nSteps - 2 - j;
  const int rev = it >= 1;
  const float dt = g.dt;
  float sa[R], xa[R], za[R], bA[R], bB[R], vz[R], vx[R], gd[R], bBj[R];
  const uint64_t pol = media_policy();
  ldrm<R>(m.bycA + i, bA, pol);
  ldrm<R>(m.bycB + i, bB, pol);
  pdl_wait();
  SWEEP_TMA(5, BOXZ)
  ldr<R>(f.szz_a + i, sa);
  ldr<R>(f.sxx_a + i, xa);
  ldr<R>(f.sxz_a + i, za);
  float bAj0 = 0.0f;
#pragma unroll
  for (int r = 0; r < R; ++r) vz[r] = vx[r] = gd[r] = bBj[r] = 0.0f;
  if (rev) {
    ldr<R>(f.vz + i, vz);
    ldr<R>(f.vx + i, vx);
    ldr<R>(gr.den + i, gd);
    ldrm<R>(m.bycB + i - ldz, bBj, pol);
    bAj0 = ldm(m.bycA + i - 1, pol);
  }
  if (!stage_wait(&bar, err)) return;
  const float* s_vz_a = sm;
  const float* s_vx_a = sm + N;
  const float* s_szz = sm + 2 * N;
  const float* s_sxx = sm + 3 * N;
  const float* s_sxz = sm + 4 * N;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int bb = b + r;
    if (special && z + r >= sh.rbz0 && z + r <= sh.rbz1) {
      const int2 rr = bin_range(sh, z + r, x);
      for (int k = rr.x; k < rr.y; ++k) {
        const int q = sh.blk_rec[k];
        if (sh.rec_z[q] == z + r && sh.rec_x[q] == x) {
          const float rv = sh.res[static_cast<size_t>(q) * sh.nSteps + it];
          sa[r] += rv;
          xa[r] += 3.0f * rv;
        }
      }
    }
    {
      const float dvz_dx = -sdp(s_vz_a, bb, BOXZ, g.rdx);
      const float dvx_dz = -sdp(s_vx_a, bb, 1, g.rdz);
      za[r] += dvz_dx * bA[r] * dt + dvx_dz * bB[r] * dt;
    }
    {
      const float dvx_dx = -sdm(s_vx_a, bb, BOXZ, g.rdx);
      const float dvz_dz = -sdm(s_vz_a, bb, 1, g.rdz);
      xa[r] += bB[r] * dvx_dx * dt;
      sa[r] += bA[r] * dvz_dz * dt;
    }
    if constexpr (MID) {
      const int zr = z + r;
      const bool xb = (x <= g.xband_lo) || (x >= g.xband_hi);
      const bool zb = (zr <= g.zband_lo) || (zr >= g.zband_hi);
      if (xb || zb) {
        const CpmlD& c = S.c;
        const size_t ir = i + r;
        const float amu = m.aveMu[ir], lam = m.lam[ir], l2m = m.l2m[ir];
        if (xb) f.m_dvz_dx[ir] = c.b_xh[x] * f.m_dvz_dx[ir] + za[r] * amu * dt;
        if (zb) f.m_dvx_dz[ir] = c.b_zh[zr] * f.m_dvx_dz[ir] + za[r] * amu * dt;
        if (xb) f.m_dvx_dx[ir] = c.b_x[x] * f.m_dvx_dx[ir] + lam * sa[r] * dt + l2m * xa[r] * dt;
        if (zb) f.m_dvz_dz[ir] = c.b_z[zr] * f.m_dvz_dz[ir] + l2m * sa[r] * dt + lam * xa[r] * dt;
      }
    }
  }
  str<R>(f.sxz_a + i, za);
  str<R>(f.szz_a + i, sa);
  str<R>(f.sxx_a + i, xa);
  if (!rev) return;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int bb = b + r;
    if (special && z + r == sh.src_z && x == sh.src_x) sh.gstf[it - 1] = -(sa[r] + 3.0f * xa[r]) * dt;
    const int zr = z + r;
    const bool inter = !MID || in_box(zr, x, g.zi0, g.zi1, g.xi0, g.xi1);
    const float ea = sdp(s_szz, bb, 1, g.rdz) + sdm(s_sxz, bb, BOXZ, g.rdx);  // dszz_dz + dsxz_dx
    const float eb = sdm(s_sxz, bb, 1, g.rdz) + sdp(s_sxx, bb, BOXZ, g.rdx);  // dsxz_dz + dsxx_dx
    if (inter) {
      vz[r] = vz[r] - ea * bA[r] * dt;
      vx[r] = vx[r] - eb * bB[r] * dt;
    }
    if constexpr (MID) {  // to_bnd of the velocities of step it - 1
      const int k = ring_index(g, zr, x);
      if (k >= 0) {
        const float* p = S.st.base + static_cast<size_t>(it - 1) * 5 * g.ring_len + k;
        vz[r] = p[3 * g.ring_len];
        vx[r] = p[4 * g.ring_len];
      }
    }
    // rho kernel gather: in a fast tile all guards hold, in a mid tile they
    // are those of el_velocity.cu:101-110.
    if (!MID || in_box(zr, x, g.zi0, g.zi1, g.xi0, g.xi1 + 1)) {
      const float bAj = r == 0 ? bAj0 : bA[r - 1];  // bycA at (z-1, x)
      float acc = gd[r];
      if (!MID || x <= g.xi1) {
        acc += -s_vz_a[bb] * ea * dt * (-bA[r] * bA[r] * 0.5f);
        acc += -s_vx_a[bb] * eb * dt * (-bB[r] * bB[r] * 0.5f);
        if (!MID || zr - 1 >= g.zi0) {
          const int bj = bb - 1;
          const float e = sdp(s_szz, bj, 1, g.rdz) + sdm(s_sxz, bj, BOXZ, g.rdx);
          acc += -s_vz_a[bj] * e * dt * (-bAj * bAj * 0.5f);
        }
      }
      if (!MID || x - 1 >= g.xi0) {
        const int bj = bb - BOXZ;
        const float e = sdm(s_sxz, bj, 1, g.rdz) + sdp(s_sxx, bj, BOXZ, g.rdx);
        acc += -s_vx_a[bj] * e * dt * (-bBj[r] * bBj[r] * 0.5f);
      }
      gd[r] = acc;
    }
  }
  str<R>(f.vz + i, vz);
  str<R>(f.vx + i, vx);
  str<R>(gr.den + i, gd);
}

// Backward fast bodies with two adjacent depths per thread, staged samples
// read in pairs (as the forward two-row bodies): with b even, the float2 at
// b + o (o even) holds the depths of both cells at offset o, so a z stencil
// of both depths takes the pairs at b - 2, b, b + 2 and an x stencil the
// pairs at b + k BOXZ. Operation order per cell is that of the one-row body.
template <int TX, int K>
__device__ __forceinline__ void bwd_B_fast2(const SweepPack<K>& P, int shot, int z0, int x0, int j, unsigned* err) {
  constexpr int TZ = 64, BOXZ = TZ + 8, R = 2;
  SWEEP_FAST_SLOT(TZ)
  SWEEP_CELL(BOXZ, R)
  SWEEP_SMEM(BOXZ)
  const Grads& gr = S.gr;
  const int it = S.nSteps - 2 - j;
  const float dt = g.dt;
  float szz[2], sxx[2], sxz[2], lam[2], l2m[2], amu[2], gl[2], gm[2], w[2], h[2], va_z[2], va_x[2], hx[2];
  const uint64_t pol = media_policy();
  ldrm<2>(m.lam + i, lam, pol);
  ldrm<2>(m.l2m + i, l2m, pol);
  ldrm<2>(m.aveMu + i, amu, pol);
  ldrm<2>(m.muw + i, w, pol);
  ldrm<2>(m.hs + i, h, pol);
  ldrm<2>(m.hs + i - ldz, hx, pol);
  const float hz0 = ldm(m.hs + i - 1, pol), hzx0 = ldm(m.hs + i - ldz - 1, pol);
  pdl_wait();
  SWEEP_TMA(5, BOXZ)
  ldr<2>(f.szz + i, szz);
  ldr<2>(f.sxx + i, sxx);
  ldr<2>(f.sxz + i, sxz);
  ldr<2>(gr.lam + i, gl);
  ldr<2>(gr.mu + i, gm);
  ldr<2>(f.vz_a + i, va_z);
  ldr<2>(f.vx_a + i, va_x);
  if (!stage_wait(&bar, err)) return;
  const float* s_vz = sm;
  const float* s_vx = sm + N;
  const float* s_sza = sm + 2 * N;
  const float* s_xxa = sm + 3 * N;
  const float* s_xza = sm + 4 * N;
  const float rdz = g.rdz, rdx = g.rdx;
  constexpr int B = BOXZ;
  // vz: z pairs and x pairs
  const float2 VZm = ld2(s_vz + b - 2), V0 = ld2(s_vz + b), VZp = ld2(s_vz + b + 2);
  const float2 Vp1 = ld2(s_vz + b + B), Vp2 = ld2(s_vz + b + 2 * B), Vm1 = ld2(s_vz + b - B),
               Vm2 = ld2(s_vz + b - 2 * B);
  // vx: z pairs at columns 0 and -1, x pairs
  const float2 UZm = ld2(s_vx + b - 2), U0 = ld2(s_vx + b), UZp = ld2(s_vx + b + 2);
  const float2 Um1 = ld2(s_vx + b - B), Up1 = ld2(s_vx + b + B), Um2 = ld2(s_vx + b - 2 * B);
  const float2 UmZm = ld2(s_vx + b - B - 2), UmZp = ld2(s_vx + b - B + 2);
  // depth b - 1 at columns +1, +2, -1, -2 (the mu gathers of the upper cell)
  const float vz_p1m = s_vz[b + B - 1], vz_p2m = s_vz[b + 2 * B - 1], vz_m1m = s_vz[b - B - 1],
              vz_m2m = s_vz[b - 2 * B - 1];
  // own-cell strains
  const float dvz_dz[2] = {dd(V0.x, VZm.y, V0.y, VZm.x, rdz), dd(V0.y, V0.x, VZp.x, VZm.y, rdz)};
  const float dvx_dx[2] = {dd(U0.x, Um1.x, Up1.x, Um2.x, rdx), dd(U0.y, Um1.y, Up1.y, Um2.y, rdx)};
  const float dvx_dz[2] = {dd(U0.y, U0.x, UZp.x, UZm.y, rdz), dd(UZp.x, U0.y, UZp.y, U0.x, rdz)};
  const float dvz_dx[2] = {dd(Vp1.x, V0.x, Vp2.x, Vm1.x, rdx), dd(Vp1.y, V0.y, Vp2.y, Vm1.y, rdx)};
  // e = dvx_dz + dvz_dx at (z, x), (z-1, x), (z, x-1), (z-1, x-1) for both depths
  const float e_own[2] = {dvx_dz[0] + dvz_dx[0], dvx_dz[1] + dvz_dx[1]};
  const float e_zm0 = dd(U0.x, UZm.y, U0.y, UZm.x, rdz) + dd(vz_p1m, VZm.y, vz_p2m, vz_m1m, rdx);
  const float e_xm[2] = {dd(Um1.y, Um1.x, UmZp.x, UmZm.y, rdz) + dd(V0.x, Vm1.x, Vp1.x, Vm2.x, rdx),
                         dd(UmZp.x, Um1.y, UmZp.y, Um1.x, rdz) + dd(V0.y, Vm1.y, Vp1.y, Vm2.y, rdx)};
  const float e_zxm0 = dd(Um1.x, UmZm.y, Um1.y, UmZm.x, rdz) + dd(VZm.y, vz_m1m, vz_p1m, vz_m2m, rdx);
  const float e_zm[2] = {e_zm0, e_own[0]};
  const float e_zxm[2] = {e_zxm0, e_xm[0]};
  // adjoint stresses
  const float2 SA0 = ld2(s_sza + b), SAZm = ld2(s_sza + b - 2), SAZp = ld2(s_sza + b + 2);
  const float2 SAp1 = ld2(s_sza + b + B), SAp2 = ld2(s_sza + b + 2 * B), SAm1 = ld2(s_sza + b - B);
  const float2 XA0 = ld2(s_xxa + b), XAZm = ld2(s_xxa + b - 2), XAZp = ld2(s_xxa + b + 2);
  const float2 XAp1 = ld2(s_xxa + b + B), XAp2 = ld2(s_xxa + b + 2 * B), XAm1 = ld2(s_xxa + b - B);
  const float2 ZA0 = ld2(s_xza + b), ZAZm = ld2(s_xza + b - 2), ZAZp = ld2(s_xza + b + 2);
  const float2 ZAm1 = ld2(s_xza + b - B), ZAp1 = ld2(s_xza + b + B), ZAm2 = ld2(s_xza + b - 2 * B);
  const float2 ZAmZm = ld2(s_xza + b - B - 2);
  const float sa_[2] = {SA0.x, SA0.y}, xa_[2] = {XA0.x, XA0.y};
  const float za_own[2] = {ZA0.x, ZA0.y}, za_zm[2] = {ZAZm.y, ZA0.x};
  const float za_xm[2] = {ZAm1.x, ZAm1.y}, za_zxm[2] = {ZAmZm.y, ZAm1.x};
  const float dszz_dx[2] = {-dd(SAp1.x, SA0.x, SAp2.x, SAm1.x, rdx), -dd(SAp1.y, SA0.y, SAp2.y, SAm1.y, rdx)};
  const float dsxx_dx[2] = {-dd(XAp1.x, XA0.x, XAp2.x, XAm1.x, rdx), -dd(XAp1.y, XA0.y, XAp2.y, XAm1.y, rdx)};
  const float dsxz_dz[2] = {-dd(ZA0.x, ZAZm.y, ZA0.y, ZAZm.x, rdz), -dd(ZA0.y, ZA0.x, ZAZp.x, ZAZm.y, rdz)};
  const float dszz_dz[2] = {-dd(SA0.y, SA0.x, SAZp.x, SAZm.y, rdz), -dd(SAZp.x, SA0.y, SAZp.y, SA0.x, rdz)};
  const float dsxx_dz[2] = {-dd(XA0.y, XA0.x, XAZp.x, XAZm.y, rdz), -dd(XAZp.x, XA0.y, XAZp.y, XA0.x, rdz)};
  const float dsxz_dx[2] = {-dd(ZA0.x, ZAm1.x, ZAp1.x, ZAm2.x, rdx), -dd(ZA0.y, ZAm1.y, ZAp1.y, ZAm2.y, rdx)};
  float o_gl[2], o_gm[2], o_szz[2], o_sxx[2], o_sxz[2], o_vza[2], o_vxa[2];
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    const float hz = r == 0 ? hz0 : h[0];
    const float hzx = r == 0 ? hzx0 : hx[0];
    if (special && z + r == sh.src_z && x == sh.src_x) {
      szz[r] -= sh.src_szz_r[it];
      sxx[r] -= sh.src_sxx_r[it];
    }
    o_szz[r] = szz[r] - (l2m[r] * dvz_dz[r] + lam[r] * dvx_dx[r]) * dt;
    o_sxx[r] = sxx[r] - (lam[r] * dvz_dz[r] + l2m[r] * dvx_dx[r]) * dt;
    o_sxz[r] = sxz[r] - amu[r] * e_own[r] * dt;
    o_gl[r] = gl[r] + -(sa_[r] + xa_[r]) * (dvz_dz[r] + dvx_dx[r]) * dt * kMega;
    const float gmu_own = (-2.0f * sa_[r] * dvz_dz[r] * dt - 2.0f * xa_[r] * dvx_dx[r] * dt) * kMega;
    float acc = gm[r] + gmu_own;
    if (h[r] != 0.0f) acc += w[r] * (-za_own[r] * e_own[r] * dt * h[r]);
    if (hz != 0.0f) acc += w[r] * (-za_zm[r] * e_zm[r] * dt * hz);
    if (hx[r] != 0.0f) acc += w[r] * (-za_xm[r] * e_xm[r] * dt * hx[r]);
    if (hzx != 0.0f) acc += w[r] * (-za_zxm[r] * e_zxm[r] * dt * hzx);
    o_gm[r] = acc;
    o_vxa[r] = va_x[r] + (lam[r] * dszz_dx[r] * dt + l2m[r] * dsxx_dx[r] * dt + amu[r] * dsxz_dz[r] * dt);
    o_vza[r] = va_z[r] + (l2m[r] * dszz_dz[r] * dt + lam[r] * dsxx_dz[r] * dt + amu[r] * dsxz_dx[r] * dt);
  }
  str<2>(gr.lam + i, o_gl);
  str<2>(f.szz + i, o_szz);
  str<2>(f.sxx + i, o_sxx);
  str<2>(f.sxz + i, o_sxz);
  str<2>(gr.mu + i, o_gm);
  str<2>(f.vx_a + i, o_vxa);
  str<2>(f.vz_a + i, o_vza);
}

template <int TX, int K>
__device__ __forceinline__ void bwd_C_fast2(const SweepPack<K>& P, int shot, int z0, int x0, int j, unsigned* err) {
  constexpr int TZ = 64, BOXZ = TZ + 8, R = 2;
  SWEEP_FAST_SLOT(TZ)
  SWEEP_CELL(BOXZ, R)
  SWEEP_SMEM(BOXZ)
  const Grads& gr = S.gr;
  const int it = S.nSteps - 2 - j;
  const int rev = it >= 1;
  const float dt = g.dt;
  float sa[2], xa[2], za[2], bA[2], bB[2], vz[2], vx[2], gd[2], bBj[2];
  const uint64_t pol = media_policy();
  ldrm<2>(m.bycA + i, bA, pol);
  ldrm<2>(m.bycB + i, bB, pol);
  pdl_wait();
  SWEEP_TMA(5, BOXZ)
  ldr<2>(f.szz_a + i, sa);
  ldr<2>(f.sxx_a + i, xa);
  ldr<2>(f.sxz_a + i, za);
  float bAj0 = 0.0f;
  vz[0] = vz[1] = vx[0] = vx[1] = gd[0] = gd[1] = bBj[0] = bBj[1] = 0.0f;
  if (rev) {
    ldr<2>(f.vz + i, vz);
    ldr<2>(f.vx + i, vx);
    ldr<2>(gr.den + i, gd);
    ldrm<2>(m.bycB + i - ldz, bBj, pol);
    bAj0 = ldm(m.bycA + i - 1, pol);
  }
  if (!stage_wait(&bar, err)) return;
  const float* s_vza = sm;
  const float* s_vxa = sm + N;
  const float* s_szz = sm + 2 * N;
  const float* s_sxx = sm + 3 * N;
  const float* s_sxz = sm + 4 * N;
  const float rdz = g.rdz, rdx = g.rdx;
  constexpr int B = BOXZ;
  const float2 VA0 = ld2(s_vza + b), VAZm = ld2(s_vza + b - 2), VAZp = ld2(s_vza + b + 2);
  const float2 VAp1 = ld2(s_vza + b + B), VAp2 = ld2(s_vza + b + 2 * B), VAm1 = ld2(s_vza + b - B);
  const float2 XA0 = ld2(s_vxa + b), XAZm = ld2(s_vxa + b - 2), XAZp = ld2(s_vxa + b + 2);
  const float2 XAm1 = ld2(s_vxa + b - B), XAp1 = ld2(s_vxa + b + B), XAm2 = ld2(s_vxa + b - 2 * B);
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    if (special && z + r >= sh.rbz0 && z + r <= sh.rbz1) {
      const int2 rr = bin_range(sh, z + r, x);
      for (int k = rr.x; k < rr.y; ++k) {
        const int q = sh.blk_rec[k];
        if (sh.rec_z[q] == z + r && sh.rec_x[q] == x) {
          const float rv = sh.res[static_cast<size_t>(q) * sh.nSteps + it];
          sa[r] += rv;
          xa[r] += 3.0f * rv;
        }
      }
    }
  }
  {
    const float dvz_dx[2] = {-dd(VAp1.x, VA0.x, VAp2.x, VAm1.x, rdx), -dd(VAp1.y, VA0.y, VAp2.y, VAm1.y, rdx)};
    const float dvx_dz[2] = {-dd(XA0.y, XA0.x, XAZp.x, XAZm.y, rdz), -dd(XAZp.x, XA0.y, XAZp.y, XA0.x, rdz)};
    const float dvx_dx[2] = {-dd(XA0.x, XAm1.x, XAp1.x, XAm2.x, rdx), -dd(XA0.y, XAm1.y, XAp1.y, XAm2.y, rdx)};
    const float dvz_dz[2] = {-dd(VA0.x, VAZm.y, VA0.y, VAZm.x, rdz), -dd(VA0.y, VA0.x, VAZp.x, VAZm.y, rdz)};
#pragma unroll
    for (int r = 0; r < 2; ++r) {
      za[r] += dvz_dx[r] * bA[r] * dt + dvx_dz[r] * bB[r] * dt;
      xa[r] += bB[r] * dvx_dx[r] * dt;
      sa[r] += bA[r] * dvz_dz[r] * dt;
    }
  }
  str<2>(f.sxz_a + i, za);
  str<2>(f.szz_a + i, sa);
  str<2>(f.sxx_a + i, xa);
  if (!rev) return;
  const float2 PZm = ld2(s_szz + b - 2), PZ0 = ld2(s_szz + b), PZp = ld2(s_szz + b + 2);
  const float2 Q0 = ld2(s_sxz + b), Qm1 = ld2(s_sxz + b - B), Qp1 = ld2(s_sxz + b + B), Qm2 = ld2(s_sxz + b - 2 * B);
  const float2 QZm = ld2(s_sxz + b - 2), QZp = ld2(s_sxz + b + 2);
  const float2 QmZm = ld2(s_sxz + b - B - 2), QmZp = ld2(s_sxz + b - B + 2);
  const float2 X0 = ld2(s_sxx + b), Xp1 = ld2(s_sxx + b + B), Xp2 = ld2(s_sxx + b + 2 * B), Xm1 = ld2(s_sxx + b - B),
               Xm2 = ld2(s_sxx + b - 2 * B);
  // sxz at depth b - 1, columns -1, +1, -2 (the upper cell's z-neighbour gather)
  const float q_m1m = s_sxz[b - B - 1], q_p1m = s_sxz[b + B - 1], q_m2m = s_sxz[b - 2 * B - 1];
  // ea = dszz_dz + dsxz_dx, eb = dsxz_dz + dsxx_dx at (z, x) for both depths
  const float ea[2] = {dd(PZ0.y, PZ0.x, PZp.x, PZm.y, rdz) + dd(Q0.x, Qm1.x, Qp1.x, Qm2.x, rdx),
                       dd(PZp.x, PZ0.y, PZp.y, PZ0.x, rdz) + dd(Q0.y, Qm1.y, Qp1.y, Qm2.y, rdx)};
  const float eb[2] = {dd(Q0.x, QZm.y, Q0.y, QZm.x, rdz) + dd(Xp1.x, X0.x, Xp2.x, Xm1.x, rdx),
                       dd(Q0.y, Q0.x, QZp.x, QZm.y, rdz) + dd(Xp1.y, X0.y, Xp2.y, Xm1.y, rdx)};
  // ea at (z-1, x): the upper cell's from depth b - 1, the lower cell's is ea[0]
  const float ea_zm0 = dd(PZ0.x, PZm.y, PZ0.y, PZm.x, rdz) + dd(QZm.y, q_m1m, q_p1m, q_m2m, rdx);
  // eb at (z, x-1)
  const float eb_xm[2] = {dd(Qm1.x, QmZm.y, Qm1.y, QmZm.x, rdz) + dd(X0.x, Xm1.x, Xp1.x, Xm2.x, rdx),
                          dd(Qm1.y, Qm1.x, QmZp.x, QmZm.y, rdz) + dd(X0.y, Xm1.y, Xp1.y, Xm2.y, rdx)};
  const float ea_zm[2] = {ea_zm0, ea[0]};
  const float va_own[2] = {VA0.x, VA0.y}, va_zm[2] = {VAZm.y, VA0.x};
  const float xa_own[2] = {XA0.x, XA0.y}, xa_xm[2] = {XAm1.x, XAm1.y};
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    if (special && z + r == sh.src_z && x == sh.src_x) sh.gstf[it - 1] = -(sa[r] + 3.0f * xa[r]) * dt;
    vz[r] = vz[r] - ea[r] * bA[r] * dt;
    vx[r] = vx[r] - eb[r] * bB[r] * dt;
    const float bAj = r == 0 ? bAj0 : bA[0];
    float acc = gd[r];
    acc += -va_own[r] * ea[r] * dt * (-bA[r] * bA[r] * 0.5f);
    acc += -xa_own[r] * eb[r] * dt * (-bB[r] * bB[r] * 0.5f);
    acc += -va_zm[r] * ea_zm[r] * dt * (-bAj * bAj * 0.5f);
    acc += -xa_xm[r] * eb_xm[r] * dt * (-bBj[r] * bBj[r] * 0.5f);
    gd[r] = acc;
  }
  str<2>(f.vz + i, vz);
  str<2>(f.vx + i, vx);
  str<2>(gr.den + i, gd);
}

// ---------------------------------------------------------------------------
// The sweep kernels: one launch per sweep and time step.

// Forward sweeps: R depths per thread (tiles of 32 R rows), R in {1, 2}
// picked per workload by the autotuner.
// flags: bit 0 saves the boundary ring, bit 1 is the timeout test hook
// (stage_wait's `inject`).
template <int TX, int K, int R>
__global__ void FWD_BOUNDS k_fwd_stress(const __grid_constant__ SweepPack<K> P, int it, int flags, unsigned* err) {
  SWEEP_KERNEL_TILE(32 * R)
  const bool inject = (flags & 2) != 0;
  if (fast) {
    if constexpr (R == 1)
      fwd_stress_fast1<TX, K, false>(P, shot, z0, x0, it, 0, inject, err);
    else
      fwd_stress_fast2<TX, K, R, false>(P, shot, z0, x0, it, 0, inject, err);
  } else if (mid) {
    if constexpr (R == 1)
      fwd_stress_fast1<TX, K, true>(P, shot, z0, x0, it, flags & 1, inject, err);
    else
      fwd_stress_fast2<TX, K, R, true>(P, shot, z0, x0, it, flags & 1, inject, err);
  } else {
    fwd_stress_edge<TX, K, R>(P, shot, z0, x0, it, flags & 1, inject, err);
  }
}

template <int TX, int K, int R>
__global__ void FWD_BOUNDS k_fwd_velocity(const __grid_constant__ SweepPack<K> P, unsigned* err) {
  SWEEP_KERNEL_TILE(32 * R)
  // A mid tile of this sweep has nothing beyond the fast form: no CPML cell,
  // every cell in the stencil domain, and no ring or band work.
  if (fast || mid) {
    if constexpr (R == 1)
      fwd_velocity_fast1<TX, K>(P, shot, z0, x0, err);
    else
      fwd_velocity_fast2<TX, K, R>(P, shot, z0, x0, err);
  } else {
    fwd_velocity_edge<TX, K, R>(P, shot, z0, x0, err);
  }
}

// Backward sweeps: R depths per thread (tiles of 32 R rows), R in {1, 2};
// NT resident threads per SM (the register budget, BWD_BOUNDS).
template <int TX, int K, int R, int NT>
__global__ void BWD_BOUNDS k_bwd_B(const __grid_constant__ SweepPack<K> P, int j, unsigned* err) {
  SWEEP_KERNEL_TILE(32 * R)
  if (fast) {
    if constexpr (R == 1)
      bwd_B_fast<TX, K, 1, false>(P, shot, z0, x0, j, err);
    else
      bwd_B_fast2<TX, K>(P, shot, z0, x0, j, err);
  } else if (mid) {
    bwd_B_fast<TX, K, R, true>(P, shot, z0, x0, j, err);
  } else {
    bwd_B_edge<TX, K, R>(P, shot, z0, x0, j, err);
  }
}

template <int TX, int K, int R, int NT>
__global__ void BWD_BOUNDS k_bwd_C(const __grid_constant__ SweepPack<K> P, int j, unsigned* err) {
  SWEEP_KERNEL_TILE(32 * R)
  if (fast) {
    if constexpr (R == 1)
      bwd_C_fast<TX, K, 1, false>(P, shot, z0, x0, j, err);
    else
      bwd_C_fast2<TX, K>(P, shot, z0, x0, j, err);
  } else if (mid) {
    bwd_C_fast<TX, K, R, true>(P, shot, z0, x0, j, err);
  } else {
    bwd_C_edge<TX, K, R>(P, shot, z0, x0, j, err);
  }
}

// ---------------------------------------------------------------------------
// Model set-up.
constexpr int kT = 32;

// Row-major double [nz][nx] (MPa) -> column-major float (Pa), through a
// shared-memory tile so both sides are coalesced (libCUFD.cu:67-78).
__global__ void k_media_from_rowmajor(int nz, int nx, int ldz, const double* __restrict__ L,
                                      const double* __restrict__ M, const double* __restrict__ D, float* lam,
                                      float* mu, float* den, unsigned* cpmax_bits) {
  __shared__ double tl[kT][kT + 1], tm[kT][kT + 1], td[kT][kT + 1];
  const int x0 = blockIdx.x * kT, z0 = blockIdx.y * kT;
  for (int r = threadIdx.y; r < kT; r += blockDim.y) {
    const int z = z0 + r, x = x0 + threadIdx.x;
    if (z < nz && x < nx) {
      const size_t s = static_cast<size_t>(z) * nx + x;
      tl[r][threadIdx.x] = L[s];
      tm[r][threadIdx.x] = M[s];
      td[r][threadIdx.x] = D[s];
    }
  }
  __syncthreads();
  float cpmax = 0.0f;
  for (int r = threadIdx.y; r < kT; r += blockDim.y) {
    const int x = x0 + r, z = z0 + threadIdx.x;
    if (z < nz && x < nx) {
      const size_t d = static_cast<size_t>(x) * ldz + z;
      const float l = static_cast<float>(tl[threadIdx.x][r] * 1e6);
      const float u = static_cast<float>(tm[threadIdx.x][r] * 1e6);
      const float rho = static_cast<float>(td[threadIdx.x][r]);
      lam[d] = l;
      mu[d] = u;
      den[d] = rho;
      const float cp = static_cast<float>(sqrt((l + 2.0 * u) / rho));  // velInit (utilities.cu:119-121)
      cpmax = fmaxf(cpmax, cp);
    }
  }
  // cp >= 0 (or NaN), so its bit pattern orders like an unsigned integer.
  atomicMax(cpmax_bits, __float_as_uint(cpmax));
}

// aveMuInit / aveBycInit (utilities.cu:125-152) plus the terms of the fused
// imaging sweeps.
__global__ void k_media_derived(int nz, int nx, int ldz, const float* __restrict__ lam,
                                const float* __restrict__ mu, const float* __restrict__ den, float* l2m,
                                float* aveMu, float* bycA, float* bycB, float* hs, float* muw) {
  const int z = blockIdx.x * blockDim.x + threadIdx.x;
  const int x = blockIdx.y * blockDim.y + threadIdx.y;
  if (z >= nz || x >= nx) return;
  const size_t i = static_cast<size_t>(x) * ldz + z;
  const float u = mu[i];
  l2m[i] = lam[i] + 2.0f * u;
  muw[i] = (u != 0.0f) ? static_cast<float>(1.0 / (static_cast<double>(u) * u)) : 0.0f;
  float am = 0.0f, ha = 0.0f, ba = 1.0f / 1000.0f, bb = 1.0f / 1000.0f;
  if (z >= 2 && z <= nz - 3 && x >= 2 && x <= nx - 3) {
    const float a = u, b = mu[i + 1], c = mu[i + ldz], d = mu[i + ldz + 1];
    if (!(a == 0.0f || b == 0.0f || c == 0.0f || d == 0.0f)) {
      const double s = 1.0 / a + 1.0 / b + 1.0 / c + 1.0 / d;
      am = static_cast<float>(4.0 / s);
      ha = static_cast<float>(am / s * 1e6);
    }
    ba = static_cast<float>(2.0 / (den[i + 1] + den[i]));
    bb = static_cast<float>(2.0 / (den[i + ldz] + den[i]));
  }
  aveMu[i] = am;
  hs[i] = ha;
  bycA[i] = ba;
  bycB[i] = bb;
}

// Column-major float -> row-major double (libCUFD.cu:480-486).
__global__ void k_to_rowmajor(int nz, int nx, int ldz, const float* __restrict__ src, double* dst, double scale) {
  __shared__ float t[kT][kT + 1];
  const int z0 = blockIdx.x * kT, x0 = blockIdx.y * kT;
  for (int r = threadIdx.y; r < kT; r += blockDim.y) {
    const int x = x0 + r, z = z0 + threadIdx.x;
    if (z < nz && x < nx) t[r][threadIdx.x] = src[static_cast<size_t>(x) * ldz + z];
  }
  __syncthreads();
  for (int r = threadIdx.y; r < kT; r += blockDim.y) {
    const int z = z0 + r, x = x0 + threadIdx.x;
    if (z < nz && x < nx) dst[static_cast<size_t>(z) * nx + x] = t[threadIdx.x][r] * scale;
  }
}

// ---------------------------------------------------------------------------
// Residual (libCUFD.cu:257-313): taper obs and syn, res = obs - syn with
// sample 0 zeroed (gpuMinus, utilities.cu:154-167), partial sums of res^2 in
// double, then the adjoint taper.
constexpr int kResThreads = 256;
constexpr int kResBlocks = 304;  // 2 x 152 SMs

__global__ void __launch_bounds__(kResThreads)
    k_residual(int nrec, int nSteps, const float* __restrict__ obs, float* syn, float* res,
               const float* __restrict__ taper_o, const float* __restrict__ taper_r, int per_trace,
               double* partials) {
  const size_t n = static_cast<size_t>(nrec) * nSteps;
  double acc = 0.0;
  for (size_t k = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; k < n;
       k += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const int t = static_cast<int>(k % nSteps);
    const float wo = taper_o ? (per_trace ? taper_o[k] : taper_o[t]) : 1.0f;
    const float wr = taper_r ? (per_trace ? taper_r[k] : taper_r[t]) : 1.0f;
    const float s = syn[k] * wo;
    const float o = obs[k] * wo;
    syn[k] = s;
    const float d = (t == 0) ? 0.0f : o - s;
    acc += static_cast<double>(d) * d;
    res[k] = d * wr;
  }
  __shared__ double sh[kResThreads / 32];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = (threadIdx.x < kResThreads / 32) ? sh[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) partials[blockIdx.x] = v;
  }
}

// out = in * taper (taper [nrec][nSteps] when per_trace, else [nSteps]); in
// may be out.
__global__ void k_apply_taper(int nrec, int nSteps, const float* in, float* out, const float* __restrict__ taper,
                              int per_trace) {
  const size_t n = static_cast<size_t>(nrec) * nSteps;
  for (size_t k = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; k < n;
       k += static_cast<size_t>(gridDim.x) * blockDim.x)
    out[k] = in[k] * (per_trace ? taper[k] : taper[k % nSteps]);
}

// Band-pass of every trace as a circular convolution with the filter's
// impulse response h (length 2 nt, see the engine): y[r][t] =
// sum_{s < nt} x[r][s] h[(t - s) mod 2 nt]. Block: trace blockIdx.y, outputs
// t0 .. t0 + 255; the samples and the 511 taps a chunk of 256 samples needs
// are staged in shared memory. x and y are distinct.
constexpr int kFilt = 256;
__global__ void __launch_bounds__(kFilt) k_trace_filter(int nt, const float* __restrict__ x, float* __restrict__ y,
                                                        const float* __restrict__ h) {
  __shared__ float xs[kFilt];
  __shared__ float hs[2 * kFilt];
  const int r = blockIdx.y, t0 = blockIdx.x * kFilt, tid = threadIdx.x, t = t0 + tid;
  const int n2 = 2 * nt;
  const float* xr = x + static_cast<size_t>(r) * nt;
  float acc = 0.0f;
  for (int s0 = 0; s0 < nt; s0 += kFilt) {
    xs[tid] = (s0 + tid < nt) ? xr[s0 + tid] : 0.0f;
    for (int j = tid; j < 2 * kFilt - 1; j += kFilt) {
      int m = (t0 - s0 - (kFilt - 1) + j) % n2;
      if (m < 0) m += n2;
      hs[j] = h[m];
    }
    __syncthreads();
#pragma unroll 8
    for (int u = 0; u < kFilt; ++u) acc += xs[u] * hs[tid - u + kFilt - 1];
    __syncthreads();
  }
  if (t < nt) y[static_cast<size_t>(r) * nt + t] = acc;
}

// Source-wavelet update (source_update, utilities.cu:927-1035). Traces are
// zero-padded to M = 2 nt and tapered by w2 (cuda_window over M, ratio 0.01;
// only its first nt values meet data); the spectra O_r(f), C_r(f) of observed
// and synthetic traces, f = 0 .. nt, are direct DFTs
//   X(f) = sum_{t < nt} w2[t] x[t] e^{-2 pi i f t / M},
// an FP32 GEMM of the twiddle table (cos, sin)(2 pi k / M), k = f t mod M,
// against the traces. Block: 64 frequencies x 32 traces, samples in chunks of
// 32 staged in shared memory; thread (fg, rg) = (tid & 15, tid >> 4) holds the
// four spectra (O, C; re, im) of frequencies f0 + fg + 16 i (i < 4) for traces
// r0 + rg + 16 j (j < 2). Each block writes its traces' partial sums of
//   num(f) = sum_r conj(C_r) O_r,  den(f) = sum_r |C_r|^2
// to part[(blockIdx.y * 3 + {0: Re num, 1: Im num, 2: den}) * (nt + 1) + f].
constexpr int kSpF = 64, kSpR = 32, kSpT = 32, kSpPad = kSpT + 4;
__global__ void __launch_bounds__(256) k_src_spectra(int nt, int nrec, const float* __restrict__ obs,
                                                     const float* __restrict__ syn, const float* __restrict__ w2,
                                                     const float2* __restrict__ tw, float* __restrict__ part) {
  __shared__ __align__(16) float sc[kSpF][kSpPad];
  __shared__ __align__(16) float ss[kSpF][kSpPad];
  __shared__ __align__(16) float so[kSpR][kSpPad];
  __shared__ __align__(16) float sd[kSpR][kSpPad];
  __shared__ float red[3][16][kSpF];
  const int tid = threadIdx.x, fg = tid & 15, rg = tid >> 4;
  const int f0 = blockIdx.x * kSpF, r0 = blockIdx.y * kSpR;
  const int nf = nt + 1;
  const unsigned M = 2u * static_cast<unsigned>(nt);
  float acc[4][2][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[i][j][q] = 0.0f;
  for (int t0 = 0; t0 < nt; t0 += kSpT) {
    for (int e = tid; e < kSpF * kSpT; e += 256) {
      const int fl = e / kSpT, tl = e % kSpT, f = f0 + fl, t = t0 + tl;
      float2 v = make_float2(0.0f, 0.0f);
      if (f < nf && t < nt) v = tw[(static_cast<unsigned>(f) * static_cast<unsigned>(t)) % M];
      sc[fl][tl] = v.x;
      ss[fl][tl] = v.y;
    }
    for (int e = tid; e < kSpR * kSpT; e += 256) {
      const int rl = e / kSpT, tl = e % kSpT, r = r0 + rl, t = t0 + tl;
      float o = 0.0f, d = 0.0f;
      if (r < nrec && t < nt) {
        const size_t q = static_cast<size_t>(r) * nt + t;
        const float w = w2[t];
        o = obs[q] * w;
        d = syn[q] * w;
      }
      so[rl][tl] = o;
      sd[rl][tl] = d;
    }
    __syncthreads();
#pragma unroll 2
    for (int tl = 0; tl < kSpT; tl += 4) {
      float4 c[4], sn[4], o[2], d[2];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        c[i] = *reinterpret_cast<const float4*>(&sc[fg + 16 * i][tl]);
        sn[i] = *reinterpret_cast<const float4*>(&ss[fg + 16 * i][tl]);
      }
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        o[j] = *reinterpret_cast<const float4*>(&so[rg + 16 * j][tl]);
        d[j] = *reinterpret_cast<const float4*>(&sd[rg + 16 * j][tl]);
      }
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) {
          float* a = acc[i][j];
          a[0] = fmaf(o[j].x, c[i].x, a[0]);
          a[1] = fmaf(-o[j].x, sn[i].x, a[1]);
          a[2] = fmaf(d[j].x, c[i].x, a[2]);
          a[3] = fmaf(-d[j].x, sn[i].x, a[3]);
          a[0] = fmaf(o[j].y, c[i].y, a[0]);
          a[1] = fmaf(-o[j].y, sn[i].y, a[1]);
          a[2] = fmaf(d[j].y, c[i].y, a[2]);
          a[3] = fmaf(-d[j].y, sn[i].y, a[3]);
          a[0] = fmaf(o[j].z, c[i].z, a[0]);
          a[1] = fmaf(-o[j].z, sn[i].z, a[1]);
          a[2] = fmaf(d[j].z, c[i].z, a[2]);
          a[3] = fmaf(-d[j].z, sn[i].z, a[3]);
          a[0] = fmaf(o[j].w, c[i].w, a[0]);
          a[1] = fmaf(-o[j].w, sn[i].w, a[1]);
          a[2] = fmaf(d[j].w, c[i].w, a[2]);
          a[3] = fmaf(-d[j].w, sn[i].w, a[3]);
        }
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    float nre = 0.0f, nim = 0.0f, den = 0.0f;
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const float Or = acc[i][j][0], Oi = acc[i][j][1], Cr = acc[i][j][2], Ci = acc[i][j][3];
      nre += Cr * Or + Ci * Oi;
      nim += Cr * Oi - Ci * Or;
      den += Cr * Cr + Ci * Ci;
    }
    red[0][rg][fg + 16 * i] = nre;
    red[1][rg][fg + 16 * i] = nim;
    red[2][rg][fg + 16 * i] = den;
  }
  __syncthreads();
  if (tid < 3 * kSpF) {
    const int q = tid / kSpF, fl = tid % kSpF, f = f0 + fl;
    float v = 0.0f;
    for (int u = 0; u < 16; ++u) v += red[q][u][fl];
    if (f < nf) part[(static_cast<size_t>(blockIdx.y) * 3 + q) * nf + f] = v;
  }
}

// coef(f) = num(f) / (den(f) + 1e-6) over the trace blocks' partial sums,
// added in block order (cuda_spectrum_update, utilities.cu:768-826).
__global__ void k_src_coef(int nf, int nblk, const float* __restrict__ part, float2* __restrict__ coef) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  float nre = 0.0f, nim = 0.0f, den = 0.0f;
  for (int b = 0; b < nblk; ++b) {
    nre += part[(static_cast<size_t>(b) * 3 + 0) * nf + f];
    nim += part[(static_cast<size_t>(b) * 3 + 1) * nf + f];
    den += part[(static_cast<size_t>(b) * 3 + 2) * nf + f];
  }
  den += 1e-6f;
  coef[f] = make_float2(nre / den, nim / den);
}

// Impulse response of the update, the length-M inverse transform of the
// Hermitian spectrum coef(0 .. nt) divided by M (the C2R + cuda_normalize
// pair): k[n] = (coef_0 + coef_nt (-1)^n + 2 sum_{f=1}^{nt-1} Re(coef_f
// e^{2 pi i f n / M})) / M, accumulated in double. Multiplying a padded
// trace's spectrum by coef and cropping is then y[t] = sum_{m < nt} x[m]
// k[(t - m) mod M] (k_trace_filter).
__global__ void k_src_response(int nt, const float2* __restrict__ coef, const float2* __restrict__ tw,
                               float* __restrict__ kresp) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  const int M = 2 * nt;
  if (n >= M) return;
  double acc = static_cast<double>(coef[0].x) + static_cast<double>(coef[nt].x) * ((n & 1) ? -1.0 : 1.0);
  int k = 0;
  for (int f = 1; f < nt; ++f) {
    k += n;
    if (k >= M) k -= M;
    const float2 c = coef[f], w = tw[k];
    acc += 2.0 * (static_cast<double>(c.x) * w.x - static_cast<double>(c.y) * w.y);
  }
  kresp[n] = static_cast<float>(acc / M);
}

// The updated wavelet's source terms for the reverse reconstruction, as the
// add_source arithmetic forms them (utilities.cu:528-555): 1500^2 amp dt in
// float, and 3 * 1500^2 * amp * dt in double rounded once.
__global__ void k_src_terms(int nt, float dt, const float* __restrict__ amp, float* __restrict__ szz,
                            float* __restrict__ sxx) {
  const int it = blockIdx.x * blockDim.x + threadIdx.x;
  if (it >= nt) return;
  const float scale = 2250000.0f;
  const float a = amp[it];
  szz[it] = __fmul_rn(__fmul_rn(scale, a), dt);
  sxx[it] = static_cast<float>(__dmul_rn(__dmul_rn(__dmul_rn(3.0, static_cast<double>(scale)), static_cast<double>(a)),
                                         static_cast<double>(dt)));
}

// Adds the per-shot gradients and / or illuminations of a shot group into
// the global ones, in group order (deterministic): shot k's sub-grid column j
// is global padded column x_off[k] + j.
__global__ void k_reduce_grads(int nz, int nx, int ldz, int nshots, const ShotSlot* __restrict__ slots, float* g_lam,
                               float* g_mu, float* g_den, float* g_illum) {
  const int z = blockIdx.x * blockDim.x + threadIdx.x;
  const int x = blockIdx.y * blockDim.y + threadIdx.y;
  if (z >= nz || x >= nx) return;
  const size_t i = static_cast<size_t>(x) * ldz + z;
  if (g_lam) {
    float a = g_lam[i], b = g_mu[i], c = g_den[i];
    for (int k = 0; k < nshots; ++k) {
      const int xs = x - slots[k].x_off;
      if (xs < 0 || xs >= slots[k].g.nx) continue;
      const size_t j = static_cast<size_t>(xs) * ldz + z;
      a += slots[k].gr.lam[j];
      b += slots[k].gr.mu[j];
      c += slots[k].gr.den[j];
    }
    g_lam[i] = a;
    g_mu[i] = b;
    g_den[i] = c;
  }
  if (g_illum) {
    float e = g_illum[i];
    for (int k = 0; k < nshots; ++k) {
      const int xs = x - slots[k].x_off;
      if (xs < 0 || xs >= slots[k].g.nx) continue;
      e += slots[k].gr.illum[static_cast<size_t>(xs) * ldz + z];
    }
    g_illum[i] = e;
  }
}

// Fixed-order sum of the block partials into *acc (one warp).
__global__ void k_sum_partials(const double* __restrict__ partials, int n, double* acc) {
  double v = 0.0;
  for (int k = threadIdx.x; k < n; k += 32) v += partials[k];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if (threadIdx.x == 0) *acc += v;
}

}  // namespace

// ---------------------------------------------------------------------------
namespace {

template <int TX, int BOXZ>
constexpr size_t smem_bytes(int na) {
  return static_cast<size_t>(na) * BOXZ * (TX + 4) * sizeof(float);
}
// Backward sweep B, one-row tiles: the five staged boxes, then the strains its
// fast bodies' mu gathers share ((TX + 1) columns x 33 depths).
template <int TX>
constexpr size_t bwd_B_smem_one_row() {
  return smem_bytes<TX, kBoxZ>(5) + static_cast<size_t>((TX + 1) * 33) * sizeof(float);
}

}  // namespace

#define FWIGB_DISPATCH_TX(tx, ...) \
  switch (tx) {                    \
    case 4: {                      \
      constexpr int TX = 4;        \
      __VA_ARGS__;                 \
      break;                       \
    }                              \
    case 8: {                      \
      constexpr int TX = 8;        \
      __VA_ARGS__;                 \
      break;                       \
    }                              \
    default: {                     \
      constexpr int TX = 16;       \
      __VA_ARGS__;                 \
      break;                       \
    }                              \
  }

// Launches a sweep with programmatic stream serialisation (see
// SWEEP_KERNEL_TILE); inside a stream capture this becomes a programmatic
// dependency edge of the graph.
template <typename... KArgs, typename... Args>
void launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

dim3 sweep_grid(int tx, int tz, const SweepGrid& gr, int nshots) {
  return dim3((gr.nz + tz - 1) / tz, (gr.nx + tx - 1) / tx, nshots);
}

template <int K>
int launch_fwd_stress(cudaStream_t s, int tx, int rows, const SweepPack<K>& p, int nshots, const SweepGrid& gr, int it,
                      int flags, unsigned* err) {
  const int sv = flags & 3;
  if (rows == 2)
    FWIGB_DISPATCH_TX(tx, launch_pdl(k_fwd_stress<TX, K, 2>, sweep_grid(TX, kTileZFwd, gr, nshots), dim3(32, TX),
                                     smem_bytes<TX, kBoxZFwd>(2), s, p, it, sv, err))
  else
    FWIGB_DISPATCH_TX(tx, launch_pdl(k_fwd_stress<TX, K, 1>, sweep_grid(TX, kTileZ, gr, nshots), dim3(32, TX),
                                     smem_bytes<TX, kBoxZ>(2), s, p, it, sv, err))
  return 1;
}

template <int K>
int launch_fwd_velocity(cudaStream_t s, int tx, int rows, const SweepPack<K>& p, int nshots, const SweepGrid& gr,
                        unsigned* err) {
  if (rows == 2)
    FWIGB_DISPATCH_TX(tx, launch_pdl(k_fwd_velocity<TX, K, 2>, sweep_grid(TX, kTileZFwd, gr, nshots), dim3(32, TX),
                                     smem_bytes<TX, kBoxZFwd>(3), s, p, err))
  else
    FWIGB_DISPATCH_TX(tx, launch_pdl(k_fwd_velocity<TX, K, 1>, sweep_grid(TX, kTileZ, gr, nshots), dim3(32, TX),
                                     smem_bytes<TX, kBoxZ>(3), s, p, err))
  return 1;
}

template <int K>
int launch_bwd_B(cudaStream_t s, int tx, int rows, int regs, const SweepPack<K>& p, int nshots,
                 const SweepGrid& gr, int j, unsigned* err) {
  if (rows == 2)
    FWIGB_DISPATCH_TX(tx, launch_pdl(k_bwd_B<TX, K, 2, 1024>, sweep_grid(TX, kTileZFwd, gr, nshots), dim3(32, TX),
                                     smem_bytes<TX, kBoxZFwd>(5), s, p, j, err))
  else if (regs > 32)
    FWIGB_DISPATCH_TX(tx, launch_pdl(k_bwd_B<TX, K, 1, 1536>, sweep_grid(TX, kTileZ, gr, nshots), dim3(32, TX),
                                     bwd_B_smem_one_row<TX>(), s, p, j, err))
  else
    FWIGB_DISPATCH_TX(tx, launch_pdl(k_bwd_B<TX, K, 1, 2048>, sweep_grid(TX, kTileZ, gr, nshots), dim3(32, TX),
                                     bwd_B_smem_one_row<TX>(), s, p, j, err))
  return 1;
}

template <int K>
int launch_bwd_C(cudaStream_t s, int tx, int rows, int regs, const SweepPack<K>& p, int nshots,
                 const SweepGrid& gr, int j, unsigned* err) {
  if (rows == 2)
    FWIGB_DISPATCH_TX(tx, launch_pdl(k_bwd_C<TX, K, 2, 1024>, sweep_grid(TX, kTileZFwd, gr, nshots), dim3(32, TX),
                                     smem_bytes<TX, kBoxZFwd>(5), s, p, j, err))
  else if (regs > 32)
    FWIGB_DISPATCH_TX(tx, launch_pdl(k_bwd_C<TX, K, 1, 1536>, sweep_grid(TX, kTileZ, gr, nshots), dim3(32, TX),
                                     smem_bytes<TX, kBoxZ>(5), s, p, j, err))
  else
    FWIGB_DISPATCH_TX(tx, launch_pdl(k_bwd_C<TX, K, 1, 2048>, sweep_grid(TX, kTileZ, gr, nshots), dim3(32, TX),
                                     smem_bytes<TX, kBoxZ>(5), s, p, j, err))
  return 1;
}

#define FWIGB_INSTANTIATE(K)                                                                                    \
  template int launch_fwd_stress<K>(cudaStream_t, int, int, const SweepPack<K>&, int, const SweepGrid&, int, int,  \
                                    unsigned*);                                                                  \
  template int launch_fwd_velocity<K>(cudaStream_t, int, int, const SweepPack<K>&, int, const SweepGrid&,        \
                                      unsigned*);                                                                \
  template int launch_bwd_B<K>(cudaStream_t, int, int, int, const SweepPack<K>&, int, const SweepGrid&, int,      \
                               unsigned*);                                                                       \
  template int launch_bwd_C<K>(cudaStream_t, int, int, int, const SweepPack<K>&, int, const SweepGrid&, int,      \
                               unsigned*);
FWIGB_INSTANTIATE(1)
FWIGB_INSTANTIATE(kPackShots)
#undef FWIGB_INSTANTIATE

// Tensor maps: one per staged array, a 2-D view (z inner, x outer; row stride
// ldz floats) with the box kBoxZ x (TX + 4), and kBoxZFwd x (TX + 4) for
// the two-row sweeps. cuTensorMapEncodeTiled checks the
// base (16-byte aligned: every array starts a multiple of ldz*nx floats into
// a 256-byte aligned allocation) and the stride (ldz*4, a multiple of 128);
// the x coordinate of every copy, z0 - 4 with z0 a multiple of 32, is a
// multiple of 4 floats.
bool encode_sweep_maps(const Geo& g, const Fields& f, int tx, SweepMaps& out, const char** err) {
  // g is the shot's sub-grid; f its fields.
  static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  if (!encode) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn) {
      *err = "cuTensorMapEncodeTiled unavailable";
      return false;
    }
    encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }
  if (g.ldz % 32 != 0) {
    *err = "column stride is not a multiple of 32 floats";
    return false;
  }
  auto one = [&](CUtensorMap* m, float* base, int boxz) {
    if (reinterpret_cast<uintptr_t>(base) % 16 != 0) return false;
    const cuuint64_t dims[2] = {static_cast<cuuint64_t>(g.nz), static_cast<cuuint64_t>(g.nx)};
    const cuuint64_t strides[1] = {static_cast<cuuint64_t>(g.ldz) * sizeof(float)};
    const cuuint32_t box[2] = {static_cast<cuuint32_t>(boxz), static_cast<cuuint32_t>(tx + 4)};
    const cuuint32_t estr[2] = {1, 1};
    return encode(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, base, dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
  };
  bool ok = true;
  const int F = kBoxZFwd, B = kBoxZ;
  ok = ok && one(&out.f1.t[0], f.vz, B) && one(&out.f1.t[1], f.vx, B);
  ok = ok && one(&out.f2.t[0], f.szz, B) && one(&out.f2.t[1], f.sxx, B) && one(&out.f2.t[2], f.sxz, B);
  ok = ok && one(&out.f1w.t[0], f.vz, F) && one(&out.f1w.t[1], f.vx, F);
  ok = ok && one(&out.f2w.t[0], f.szz, F) && one(&out.f2w.t[1], f.sxx, F) && one(&out.f2w.t[2], f.sxz, F);
  ok = ok && one(&out.b.t[0], f.vz, B) && one(&out.b.t[1], f.vx, B) && one(&out.b.t[2], f.szz_a, B) &&
       one(&out.b.t[3], f.sxx_a, B) && one(&out.b.t[4], f.sxz_a, B);
  ok = ok && one(&out.c.t[0], f.vz_a, B) && one(&out.c.t[1], f.vx_a, B) && one(&out.c.t[2], f.szz, B) &&
       one(&out.c.t[3], f.sxx, B) && one(&out.c.t[4], f.sxz, B);
  ok = ok && one(&out.bw.t[0], f.vz, F) && one(&out.bw.t[1], f.vx, F) && one(&out.bw.t[2], f.szz_a, F) &&
       one(&out.bw.t[3], f.sxx_a, F) && one(&out.bw.t[4], f.sxz_a, F);
  ok = ok && one(&out.cw.t[0], f.vz_a, F) && one(&out.cw.t[1], f.vx_a, F) && one(&out.cw.t[2], f.szz, F) &&
       one(&out.cw.t[3], f.sxx, F) && one(&out.cw.t[4], f.sxz, F);
  if (!ok) *err = "cuTensorMapEncodeTiled rejected a sweep tile";
  return ok;
}

void launch_media_from_rowmajor(cudaStream_t s, int nz, int nx, int ldz, const double* lam_mpa, const double* mu_mpa,
                                const double* den, float* lam, float* mu, float* den_f, unsigned* cpmax_bits) {
  dim3 grid((nx + kT - 1) / kT, (nz + kT - 1) / kT);
  k_media_from_rowmajor<<<grid, dim3(kT, 8), 0, s>>>(nz, nx, ldz, lam_mpa, mu_mpa, den, lam, mu, den_f, cpmax_bits);
}

void launch_media_derived(cudaStream_t s, int nz, int nx, int ldz, const float* lam, const float* mu,
                          const float* den, float* l2m, float* aveMu, float* bycA, float* bycB, float* hs,
                          float* muw) {
  dim3 grid((nz + 31) / 32, (nx + 7) / 8);
  k_media_derived<<<grid, dim3(32, 8), 0, s>>>(nz, nx, ldz, lam, mu, den, l2m, aveMu, bycA, bycB, hs, muw);
}

int residual_blocks(int n) {
  int b = (n + kResThreads - 1) / kResThreads;
  return b < kResBlocks ? (b < 1 ? 1 : b) : kResBlocks;
}

void launch_residual(cudaStream_t s, int nrec, int nSteps, const float* obs, float* syn, float* res,
                     const float* taper_o, const float* taper_r, int per_trace, double* partials) {
  const int nb = residual_blocks(nrec * nSteps);
  k_residual<<<nb, kResThreads, 0, s>>>(nrec, nSteps, obs, syn, res, taper_o, taper_r, per_trace, partials);
}

void launch_apply_taper(cudaStream_t s, int nrec, int nSteps, const float* in, float* out, const float* taper,
                        int per_trace) {
  k_apply_taper<<<residual_blocks(nrec * nSteps), kResThreads, 0, s>>>(nrec, nSteps, in, out, taper, per_trace);
}

int src_spectra_blocks(int nrec) { return (nrec + kSpR - 1) / kSpR; }

void launch_src_update_coef(cudaStream_t s, int nrec, int nt, const float* obs, const float* syn, const float* w2,
                            const float2* tw, float* part, float2* coef, float* kresp) {
  const int nf = nt + 1, nblk = src_spectra_blocks(nrec);
  k_src_spectra<<<dim3((nf + kSpF - 1) / kSpF, nblk), 256, 0, s>>>(nt, nrec, obs, syn, w2, tw, part);
  k_src_coef<<<(nf + 255) / 256, 256, 0, s>>>(nf, nblk, part, coef);
  k_src_response<<<(2 * nt + 63) / 64, 64, 0, s>>>(nt, coef, tw, kresp);
}

void launch_src_terms(cudaStream_t s, int nt, float dt, const float* amp, float* szz, float* sxx) {
  k_src_terms<<<(nt + 255) / 256, 256, 0, s>>>(nt, dt, amp, szz, sxx);
}

void launch_trace_filter(cudaStream_t s, int nrec, int nt, const float* x, float* y, const float* h) {
  k_trace_filter<<<dim3((nt + kFilt - 1) / kFilt, nrec), kFilt, 0, s>>>(nt, x, y, h);
}

void launch_sum_partials(cudaStream_t s, const double* partials, int n, double* acc) {
  k_sum_partials<<<1, 32, 0, s>>>(partials, n, acc);
}

void launch_reduce_grads(cudaStream_t s, int nz, int nx, int ldz, int nshots, const ShotSlot* slots, float* g_lam,
                         float* g_mu, float* g_den, float* g_illum) {
  dim3 grid((nz + 31) / 32, (nx + 7) / 8);
  k_reduce_grads<<<grid, dim3(32, 8), 0, s>>>(nz, nx, ldz, nshots, slots, g_lam, g_mu, g_den, g_illum);
}

void launch_to_rowmajor(cudaStream_t s, int nz, int nx, int ldz, const float* src, double* dst, double scale) {
  dim3 grid((nz + kT - 1) / kT, (nx + kT - 1) / kT);
  k_to_rowmajor<<<grid, dim3(kT, 8), 0, s>>>(nz, nx, ldz, src, dst, scale);
}

}  // namespace fwigb
