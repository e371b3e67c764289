// Learned gradient preconditioner: a small CNN (3x3 convolutions, GELU) in
// BF16 with FP32 accumulation on the tensor cores, hand-written for sm_103a
// with warp-level mma.sync.m16n8k16 (bf16 x bf16 -> f32) and ldmatrix. The
// network has no counterpart in the reference.
//
// Image layout: Hz x Wx pixels, x-major with z fastest (pixel p = x*Hz + z,
// the orientation of the wavefield arrays), channels innermost: element
// (p, c) at p*C + c. Hz must be a multiple of 32 (the padded grid heights of
// the FWI workloads are). Channel counts are padded to 16 or 32; padded
// channels carry zeros.
//
// Kernels:
//   k_conv3x3_tc   the 32-output-channel convolutions on the 5th-generation
//                  tensor cores: tcgen05.mma (kind::f16, BF16 in, FP32 out)
//                  with the accumulators in tensor memory, one 128-depth x
//                  4-column pixel tile per block (see its comment)
//   k_conv3x3      (one 32 z x 8 x pixel tile per block, warp-level
//                  mma.sync) y = epilogue(conv(x, W) + b): GELU with the pre-activation
//                  kept (forward), linear FP32 (last layer), or linear times
//                  GELU'(z) (backward data, where W is the flipped,
//                  transposed kernel: dX = conv(dZ, W'))
//   k_conv3x3_wgrad  per-block partial dW[tap][ci][co] = sum_p X(p+tap) dZ(p)
//   k_reduce_partials, k_bias_grad, k_adam, k_pack_weights, k_mse_grad
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <cstdint>
#include <mutex>

#include "fwiflow_gb300.h"

namespace fwigb_cnn {
namespace {

constexpr int kTz = 32;  // tile height (z)
constexpr int kTx = 8;   // tile width (x); one warp per column
constexpr int kHz = kTz + 2, kHx = kTx + 2;  // tile with its 1-pixel halo

__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void ldmatrix_x4(unsigned (&r)[4], const void* p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0, %1, %2, %3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(smem_u32(p)));
}

__device__ __forceinline__ void ldmatrix_x4_trans(unsigned (&r)[4], const void* p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0, %1, %2, %3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(smem_u32(p)));
}

// D = A(16x16, row) * B(16x8, col) + D, bf16 inputs, f32 accumulators.
__device__ __forceinline__ void mma_bf16(float (&d)[4], const unsigned (&a)[4], unsigned b0, unsigned b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
      "{%0, %1, %2, %3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float x) {
  return 0.5f * (1.0f + erff(x * 0.70710678118654752f)) + x * 0.39894228040143268f * expf(-0.5f * x * x);
}

__device__ __forceinline__ unsigned pack_bf16(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const unsigned*>(&v);
}

// Loads the (Tz+2) x (Tx+2) pixel tile with halo of a C-channel image into
// shared memory (row stride C + 8 bf16: conflict-free ldmatrix), zeros
// outside the image.
template <int C>
__device__ __forceinline__ void load_tile(const __nv_bfloat16* __restrict__ img, int Hz, int Wx, int z0, int x0,
                                          __nv_bfloat16* s) {
  constexpr int CS = C + 8, CH = C / 8;  // 16-byte chunks per pixel
  const int tid = threadIdx.x;
  for (int k = tid; k < kHz * kHx * CH; k += blockDim.x) {
    const int ch = k % CH, pix = k / CH;
    const int hz = pix % kHz, hx = pix / kHz;
    const int z = z0 + hz - 1, x = x0 + hx - 1;
    uint4 v = make_uint4(0u, 0u, 0u, 0u);
    if (z >= 0 && z < Hz && x >= 0 && x < Wx)
      v = *reinterpret_cast<const uint4*>(img + (static_cast<size_t>(x) * Hz + z) * C + ch * 8);
    *reinterpret_cast<uint4*>(s + (hx * kHz + hz) * CS + ch * 8) = v;
  }
}

enum Epilogue { kEpiGelu = 0, kEpiLinearF32 = 1, kEpiDGelu = 2 };

// One block: 32 z x 8 x pixels, 8 warps (warp w = column x0 + w, two m-tiles
// of 16 depths). CIN in {16, 32}, COUT in {16, 32}. wfrag holds the weights
// in mma B-fragment order: [tap][CIN/16][COUT/8][lane] of uint2.
template <int CIN, int COUT, int EPI>
__global__ void __launch_bounds__(256) k_conv3x3(const __nv_bfloat16* __restrict__ x_in, int Hz, int Wx,
                                                 const uint2* __restrict__ wfrag, const float* __restrict__ bias,
                                                 __nv_bfloat16* __restrict__ y_bf16, float* __restrict__ y_f32,
                                                 __nv_bfloat16* __restrict__ z_pre,
                                                 const __nv_bfloat16* __restrict__ z_prev) {
  constexpr int CS = CIN + 8;
  constexpr int KC = CIN / 16, NT = COUT / 8;
  constexpr int NFRAG = 9 * KC * NT * 32;
  __shared__ __align__(16) __nv_bfloat16 s_x[kHz * kHx * CS];
  __shared__ __align__(16) uint2 s_w[NFRAG];
  const int z0 = blockIdx.x * kTz, x0 = blockIdx.y * kTx;
  load_tile<CIN>(x_in, Hz, Wx, z0, x0, s_x);
  for (int k = threadIdx.x; k < NFRAG; k += blockDim.x) s_w[k] = wfrag[k];
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = lane >> 2, t = lane & 3;
  float acc[2][NT][4];
#pragma unroll
  for (int m = 0; m < 2; ++m)
#pragma unroll
    for (int n = 0; n < NT; ++n)
#pragma unroll
      for (int e = 0; e < 4; ++e) acc[m][n][e] = 0.0f;
  // ldmatrix row of this lane: depth (lane % 16) of the m-tile, channel
  // half (lane / 16) of the 16-channel k-chunk.
  const int lrow = lane & 15, lcol = (lane >> 4) * 8;
#pragma unroll
  for (int tap = 0; tap < 9; ++tap) {
    const int ky = tap / 3, kx = tap % 3;  // pixel offset (ky - 1, kx - 1); halo index +1
#pragma unroll
    for (int kc = 0; kc < KC; ++kc) {
      unsigned a[2][4];
#pragma unroll
      for (int m = 0; m < 2; ++m)
        ldmatrix_x4(a[m], s_x + ((warp + kx) * kHz + m * 16 + lrow + ky) * CS + kc * 16 + lcol);
#pragma unroll
      for (int n = 0; n < NT; ++n) {
        const uint2 b = s_w[((tap * KC + kc) * NT + n) * 32 + lane];
        mma_bf16(acc[0][n], a[0], b.x, b.y);
        mma_bf16(acc[1][n], a[1], b.x, b.y);
      }
    }
  }
  const int x = x0 + warp;
  if (x >= Wx) return;
#pragma unroll
  for (int m = 0; m < 2; ++m)
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      const int z = z0 + m * 16 + g + half * 8;
      const size_t p = static_cast<size_t>(x) * Hz + z;
#pragma unroll
      for (int n = 0; n < NT; ++n) {
        const int c = n * 8 + 2 * t;
        float v0 = acc[m][n][2 * half], v1 = acc[m][n][2 * half + 1];
        if (EPI == kEpiGelu) {
          v0 += bias[c];
          v1 += bias[c + 1];
          *reinterpret_cast<unsigned*>(z_pre + p * COUT + c) = pack_bf16(v0, v1);
          *reinterpret_cast<unsigned*>(y_bf16 + p * COUT + c) = pack_bf16(gelu(v0), gelu(v1));
        } else if (EPI == kEpiLinearF32) {
          y_f32[p * COUT + c] = v0 + bias[c];
          y_f32[p * COUT + c + 1] = v1 + bias[c + 1];
        } else {  // backward data through the previous layer's GELU
          const __nv_bfloat162 zp = *reinterpret_cast<const __nv_bfloat162*>(z_prev + p * COUT + c);
          v0 *= gelu_grad(__low2float(zp));
          v1 *= gelu_grad(__high2float(zp));
          *reinterpret_cast<unsigned*>(y_bf16 + p * COUT + c) = pack_bf16(v0, v1);
        }
      }
    }
}

// ---------------------------------------------------------------------------
// tcgen05 convolution (sm_100 family). The convolution is an implicit GEMM
// per output column: D[128 depths][32 couts] = sum over 9 taps of
// A_tap[128][CIN] * B_tap[CIN][32]. Both operands live in shared memory in the
// canonical no-swizzle K-major layout: 16-byte units of 8 consecutive
// channels, 8-row core matrices 128 bytes apart (SBO) and channel groups LBO
// apart. Rows of the input tile are consecutive depths of one column, so the
// operand of a tap (ky, kx) is the tile column x + kx started ky rows down: a
// descriptor offset of 16 ky bytes.
//
// Persistent and warp-specialised: one CTA per SM walks the image's tiles
// (128 depths x 4 columns each) with a stride of the grid.
//   warp 0 (one thread)  TMA producer: the input tile with its 1-pixel halo,
//                        130 depths x 6 columns x CIN channels, as CIN/8 3-D
//                        boxes (8 channels x 130 x 6, zero fill outside the
//                        image) into a kTcStages-deep ring of shared-memory
//                        stages; a box lands exactly in the K-major layout
//                        above (16-byte units, depth fastest, then column).
//   warp 1 (one thread)  MMA issuer: 4 columns x 9 taps x CIN/16 tcgen05.mma
//                        per tile into one of kTcAcc tensor-memory
//                        accumulators (4 columns x 32 couts = 128 TMEM
//                        columns each); tcgen05.commit frees the stage and
//                        publishes the accumulator.
//   warps 4..19          epilogue: warpgroup g reads column g of the
//                        accumulator with tcgen05.ld (warp w owns TMEM lanes
//                        32 (w % 4) .. +31, i.e. depths z0 + 32 (w % 4) +
//                        lane), applies the fused epilogue and stores BF16,
//                        then releases the accumulator.
// So the load of tile i+1, the MMAs of tile i+1 and the epilogue of tile i
// overlap. The weights (B operand) are loaded once per CTA. Every wait is
// bounded by the global timer: a role whose wait runs out raises bit 1 of
// *err and stops; the others then run out too, and the CTA frees its tensor
// memory and returns.
constexpr int kTcRows = 128, kTcCols = 4;  // pixels per tile: 128 depths x 4 columns
constexpr int kTcTileRows = kTcRows + 2, kTcTileCols = kTcCols + 2;
constexpr int kTcStages = 2, kTcAcc = 2;
constexpr int kTcThreads = 640;  // warps 0..3: producer, MMA, 2 idle; warps 4..19: 4 epilogue warpgroups
constexpr uint32_t kTcBox = kTcTileRows * kTcTileCols * 16;  // bytes of one 8-channel box
constexpr uint32_t kTcBoxStride = (kTcBox + 127) / 128 * 128;  // boxes 128-byte aligned in a stage
constexpr unsigned long long kTcWaitNs = 2000000000ull;

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void mbar_init_n(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ bool mbar_test(uint64_t* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity), "r"(1000000u)
      : "memory");
  return ok != 0;
}
// Bounded wait (global timer) for phase `parity` of an mbarrier.
__device__ __forceinline__ bool mbar_wait_ns(uint64_t* bar, unsigned parity) {
  if (mbar_test(bar, parity)) return true;
  const unsigned long long t0 = global_ns();
  for (;;) {
    if (mbar_test(bar, parity)) return true;
    if (global_ns() - t0 > kTcWaitNs) return false;
  }
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* tm, int c0, int c1, int c2, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::
          "r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(tm)), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// Shared-memory matrix descriptor: start, leading (K-direction) and stride
// (8-row-group) byte offsets, all >> 4; descriptor version 1; no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t start, uint32_t lbo, uint32_t sbo) {
  return static_cast<uint64_t>((start >> 4) & 0x3FFFu) | (static_cast<uint64_t>((lbo >> 4) & 0x3FFFu) << 16) |
         (static_cast<uint64_t>((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}
// Instruction descriptor of kind::f16: D FP32, A and B BF16, both K-major,
// N = 32, M = 128.
constexpr uint32_t kTcIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((32u >> 3) << 17) | ((128u >> 4) << 24);

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
          d_tmem),
      "l"(adesc), "l"(bdesc), "r"(kTcIdesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void tc_ld32(uint32_t taddr, float (&v)[32]) {
  unsigned r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int k = 0; k < 32; ++k) v[k] = __uint_as_float(r[k]);
}

// CIN in {16, 32} input channels, 32 output channels. EPI kEpiGelu (bias,
// pre-activation and GELU, BF16) or kEpiDGelu (times GELU'(z_prev), BF16).
// tmap: the input image as a 3-D tensor (channels, depths, columns), box
// 8 x 130 x 6. wpack: the B operand in its shared-memory layout, 16-byte
// units (q, n) at (q * 32 + n) for q = tap * CIN/8 + channel group
// (k_pack_weights_tc).
template <int CIN, int EPI>
__global__ void __launch_bounds__(kTcThreads, 1)
    k_conv3x3_tc(const __grid_constant__ CUtensorMap tmap, int Hz, int Wx, const uint4* __restrict__ wpack,
                 const float* __restrict__ bias, __nv_bfloat16* __restrict__ y, __nv_bfloat16* __restrict__ z_pre,
                 const __nv_bfloat16* __restrict__ z_prev, unsigned* err) {
  constexpr int QA = CIN / 8;                    // channel groups (boxes) of the input
  constexpr uint32_t STAGE = QA * kTcBoxStride;  // bytes of one input stage
  constexpr int QB = 9 * CIN / 8;                // channel groups of B over the taps
  extern __shared__ __align__(1024) uint8_t tc_smem[];
  uint8_t* sA = tc_smem;                            // kTcStages stages
  uint4* sB = reinterpret_cast<uint4*>(tc_smem + kTcStages * STAGE);
  __shared__ __align__(8) uint64_t full[kTcStages], empty[kTcStages], acc_full[kTcAcc], acc_empty[kTcAcc];
  __shared__ uint32_t tmem_slot;
  __shared__ int abort_flag;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int ntz = (Hz + kTcRows - 1) / kTcRows, ntx = (Wx + kTcCols - 1) / kTcCols, ntiles = ntz * ntx;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "r"(kTcAcc * 128)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  for (int u = tid; u < QB * 32; u += blockDim.x) sB[u] = wpack[u];
  if (tid == 0) {
    for (int k = 0; k < kTcStages; ++k) {
      mbar_init_n(&full[k], 1);
      mbar_init_n(&empty[k], 1);
    }
    for (int k = 0; k < kTcAcc; ++k) {
      mbar_init_n(&acc_full[k], 1);
      mbar_init_n(&acc_empty[k], 16 * 32);  // every epilogue thread
    }
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // weights visible to the tensor cores
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;
  if (warp == 0) {
    if (lane == 0) {  // TMA producer
      int i = 0;
      for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++i) {
        const int st = i % kTcStages;
        if (i >= kTcStages && !mbar_wait_ns(&empty[st], ((i / kTcStages) - 1) & 1)) {
          atomicOr(err, 2u);
          atomicExch(&abort_flag, 1);
          break;
        }
        if (*reinterpret_cast<volatile int*>(&abort_flag)) break;
        const int z0 = (t % ntz) * kTcRows, x0 = (t / ntz) * kTcCols;
        mbar_expect_tx(&full[st], QA * kTcBox);
#pragma unroll
        for (int q = 0; q < QA; ++q) tma_load_3d(sA + st * STAGE + q * kTcBoxStride, &tmap, q * 8, z0 - 1, x0 - 1, &full[st]);
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {  // MMA issuer
      const uint32_t b0 = smem_u32(sB);
      int i = 0;
      for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++i) {
        const int st = i % kTcStages, ac = i % kTcAcc;
        bool ok = mbar_wait_ns(&full[st], (i / kTcStages) & 1);
        if (ok && i >= kTcAcc) ok = mbar_wait_ns(&acc_empty[ac], ((i / kTcAcc) - 1) & 1);
        if (!ok || *reinterpret_cast<volatile int*>(&abort_flag)) {
          atomicOr(err, 2u);
          atomicExch(&abort_flag, 1);
          break;
        }
        tc_fence_after();
        const uint32_t a0 = smem_u32(sA + st * STAGE);
        const uint32_t d0 = tmem + ac * 128;
#pragma unroll 1
        for (int j = 0; j < kTcCols; ++j)
#pragma unroll 1
          for (int tap = 0; tap < 9; ++tap) {
            const int ky = tap / 3, kx = tap % 3;
#pragma unroll
            for (int s = 0; s < CIN / 16; ++s) {
              const uint32_t a = a0 + 2 * s * kTcBoxStride + ((j + kx) * kTcTileRows + ky) * 16;
              const uint32_t b = b0 + (tap * QA + 2 * s) * 32 * 16;
              tc_mma(d0 + j * 32, smem_desc(a, kTcBoxStride, 128), smem_desc(b, 32 * 16, 128), (tap | s) != 0);
            }
          }
        tc_commit(&empty[st]);    // the stage is free once these MMAs have read it
        tc_commit(&acc_full[ac]);  // and the accumulator is ready
      }
    }
  } else if (warp >= 4) {  // epilogue: warpgroup g takes pixel column g of each tile
    const int g = (warp - 4) >> 2, quarter = warp & 3;
    int i = 0;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++i) {
      const int ac = i % kTcAcc;
      const bool ok = __all_sync(0xffffffffu, mbar_wait_ns(&acc_full[ac], (i / kTcAcc) & 1));
      if (!ok) {
        if (lane == 0) {
          atomicOr(err, 2u);
          atomicExch(&abort_flag, 1);
        }
        break;
      }
      tc_fence_after();
      const int z0 = (t % ntz) * kTcRows, x0 = (t / ntz) * kTcCols;
      float v[32];
      tc_ld32(tmem + (static_cast<uint32_t>(quarter * 32) << 16) + ac * 128 + g * 32, v);
      tc_fence_before();
      mbar_arrive(&acc_empty[ac]);  // the accumulator's column is in registers
      const int z = z0 + quarter * 32 + lane, x = x0 + g;
      if (z < Hz && x < Wx) {
        const size_t p = (static_cast<size_t>(x) * Hz + z) * 32;
        unsigned o0[16], o1[16];
        if (EPI == kEpiGelu) {
#pragma unroll
          for (int c = 0; c < 16; ++c) {
            const float a = v[2 * c] + bias[2 * c], b = v[2 * c + 1] + bias[2 * c + 1];
            o0[c] = pack_bf16(a, b);
            o1[c] = pack_bf16(gelu(a), gelu(b));
          }
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            reinterpret_cast<uint4*>(z_pre + p)[k] = make_uint4(o0[4 * k], o0[4 * k + 1], o0[4 * k + 2], o0[4 * k + 3]);
            reinterpret_cast<uint4*>(y + p)[k] = make_uint4(o1[4 * k], o1[4 * k + 1], o1[4 * k + 2], o1[4 * k + 3]);
          }
        } else {
          const uint4* zp = reinterpret_cast<const uint4*>(z_prev + p);
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            const uint4 w = zp[k];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
              const unsigned h = e == 0 ? w.x : (e == 1 ? w.y : (e == 2 ? w.z : w.w));
              // BF16 -> FP32 is exact: the BF16 bits are the top half of the float.
              const float lo = __uint_as_float(h << 16), hi = __uint_as_float(h & 0xFFFF0000u);
              const int c = 4 * k + e;
              o0[c] = pack_bf16(v[2 * c] * gelu_grad(lo), v[2 * c + 1] * gelu_grad(hi));
            }
          }
#pragma unroll
          for (int k = 0; k < 4; ++k)
            reinterpret_cast<uint4*>(y + p)[k] = make_uint4(o0[4 * k], o0[4 * k + 1], o0[4 * k + 2], o0[4 * k + 3]);
        }
      }
    }
  }
  // Teardown: the epilogue has taken every accumulator the MMA thread
  // committed (or the CTA aborted on a timeout, after each role's own bounded
  // wait), so the tensor memory is free to go.
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTcAcc * 128)
                              : "memory");
}

// Packs W[9][cin][cout] (FP32) into the B operand of k_conv3x3_tc: unit
// (q, n) of 8 BF16 = B[n][k = 8q .. 8q+7] with B[n][tap*KIN + kk] =
// W[tap][kk][n] (forward, KIN = cin_pad) or W[8 - tap][n][kk] (transposed:
// the data gradient, KIN = cout_pad, n over cin_pad). N must be 32.
__global__ void k_pack_weights_tc(const float* __restrict__ w, int cin, int cout, int CIN, int COUT, int transposed,
                                  uint4* __restrict__ out) {
  const int KIN = transposed ? COUT : CIN;
  const int total = 9 * KIN / 8 * 32;
  const int u = blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= total) return;
  const int n = u % 32, q = u / 32;
  unsigned h[4];
  for (int e2 = 0; e2 < 4; ++e2) {
    float v[2];
    for (int t = 0; t < 2; ++t) {
      const int k = q * 8 + e2 * 2 + t, tap = k / KIN, kk = k % KIN;
      int ci, co, tp;
      if (transposed) {
        ci = n;
        co = kk;
        tp = 8 - tap;
      } else {
        ci = kk;
        co = n;
        tp = tap;
      }
      v[t] = (ci < cin && co < cout) ? w[(static_cast<size_t>(tp) * cin + ci) * cout + co] : 0.0f;
    }
    h[e2] = pack_bf16(v[0], v[1]);
  }
  out[u] = make_uint4(h[0], h[1], h[2], h[3]);
}

// Weight gradient partials. One block (9 warps, warp = tap) per 32 x 8 pixel
// tile: dW_tap[ci][co] += sum over the tile's pixels p of X(p + off_tap)[ci] *
// dZ(p)[co], as a GEMM with K = pixels: A = X_tap^T and B = dZ, both read
// pixel-major from shared memory with ldmatrix.trans. Writes the block's
// partial [9][CIN][COUT] (FP32) to part + block * 9*CIN*COUT.
template <int CIN, int COUT>
__global__ void __launch_bounds__(288) k_conv3x3_wgrad(const __nv_bfloat16* __restrict__ x_in,
                                                       const __nv_bfloat16* __restrict__ dz, int Hz, int Wx,
                                                       float* __restrict__ part) {
  constexpr int CSX = CIN + 8, CSZ = COUT + 8;
  constexpr int MT = CIN / 16, NT = COUT / 8;
  __shared__ __align__(16) __nv_bfloat16 s_x[kHz * kHx * CSX];
  __shared__ __align__(16) __nv_bfloat16 s_dz[kTz * kTx * CSZ];
  const int z0 = blockIdx.x * kTz, x0 = blockIdx.y * kTx;
  load_tile<CIN>(x_in, Hz, Wx, z0, x0, s_x);
  {
    constexpr int CH = COUT / 8;
    for (int k = threadIdx.x; k < kTz * kTx * CH; k += blockDim.x) {
      const int ch = k % CH, pix = k / CH;
      const int zz = pix % kTz, xx = pix / kTz;
      const int x = x0 + xx;
      uint4 v = make_uint4(0u, 0u, 0u, 0u);
      if (x < Wx) v = *reinterpret_cast<const uint4*>(dz + (static_cast<size_t>(x) * Hz + z0 + zz) * COUT + ch * 8);
      *reinterpret_cast<uint4*>(s_dz + pix * CSZ + ch * 8) = v;
    }
  }
  __syncthreads();
  const int tap = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ky = tap / 3, kx = tap % 3;
  const int g = lane >> 2, t = lane & 3, q = lane >> 3, r8 = lane & 7;
  float acc[MT][NT][4];
#pragma unroll
  for (int m = 0; m < MT; ++m)
#pragma unroll
    for (int n = 0; n < NT; ++n)
#pragma unroll
      for (int e = 0; e < 4; ++e) acc[m][n][e] = 0.0f;
  // A^T fragment rows: pixel (q >= 2 ? 8 : 0) + r8, channel offset (q & 1) * 8.
  const int a_px = (q >> 1) * 8 + r8, a_c = (q & 1) * 8;
  // B fragment rows: pixel (q & 1) * 8 + r8, channel offset (q >> 1) * 8.
  const int b_px = (q & 1) * 8 + r8, b_c = (q >> 1) * 8;
  for (int s = 0; s < kTz * kTx / 16; ++s) {  // 16 pixels per k-step: half a column
    const int xx = s >> 1, zz0 = (s & 1) * 16;
    unsigned a[MT][4];
#pragma unroll
    for (int m = 0; m < MT; ++m)
      ldmatrix_x4_trans(a[m], s_x + ((xx + kx) * kHz + zz0 + a_px + ky) * CSX + m * 16 + a_c);
#pragma unroll
    for (int nb = 0; nb < NT / 2; ++nb) {
      unsigned b[4];
      ldmatrix_x4_trans(b, s_dz + (xx * kTz + zz0 + b_px) * CSZ + nb * 16 + b_c);
#pragma unroll
      for (int m = 0; m < MT; ++m) {
        mma_bf16(acc[m][2 * nb], a[m], b[0], b[1]);
        mma_bf16(acc[m][2 * nb + 1], a[m], b[2], b[3]);
      }
    }
  }
  float* out = part + static_cast<size_t>(blockIdx.y * gridDim.x + blockIdx.x) * 9 * CIN * COUT +
               static_cast<size_t>(tap) * CIN * COUT;
#pragma unroll
  for (int m = 0; m < MT; ++m)
#pragma unroll
    for (int n = 0; n < NT; ++n) {
      const int ci = m * 16 + g, co = n * 8 + 2 * t;
      out[ci * COUT + co] = acc[m][n][0];
      out[ci * COUT + co + 1] = acc[m][n][1];
      out[(ci + 8) * COUT + co] = acc[m][n][2];
      out[(ci + 8) * COUT + co + 1] = acc[m][n][3];
    }
}

// out[i] = sum over b < nblocks of part[b * n + i], in block order.
__global__ void k_reduce_partials(const float* __restrict__ part, int nblocks, int n, float* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float s = 0.0f;
  for (int b = 0; b < nblocks; ++b) s += part[static_cast<size_t>(b) * n + i];
  out[i] = s;
}

// Per-block partial sums over pixels of dZ[p][co] (bias gradient): block b
// sums pixels [b*chunk, (b+1)*chunk) into part[b * C + co].
template <int C>
__global__ void k_bias_partials(const __nv_bfloat16* __restrict__ dz, long long npix, int chunk,
                                float* __restrict__ part) {
  __shared__ float s[256];
  const int co = threadIdx.x % C, lane_set = threadIdx.x / C, sets = blockDim.x / C;
  const long long p0 = static_cast<long long>(blockIdx.x) * chunk;
  float acc = 0.0f;
  for (long long p = p0 + lane_set; p < p0 + chunk && p < npix; p += sets) acc += __bfloat162float(dz[p * C + co]);
  s[threadIdx.x] = acc;
  __syncthreads();
  if (threadIdx.x < C) {
    float v = 0.0f;
    for (int k = 0; k < sets; ++k) v += s[k * C + threadIdx.x];
    part[static_cast<size_t>(blockIdx.x) * C + threadIdx.x] = v;
  }
}

// Adam on FP32 parameters (bias-corrected, no weight decay).
__global__ void k_adam(float* __restrict__ w, const float* __restrict__ gr, float* __restrict__ m1,
                       float* __restrict__ m2, int n, float lr, float b1, float b2, float eps, float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float g = gr[i];
  const float a = b1 * m1[i] + (1.0f - b1) * g;
  const float v = b2 * m2[i] + (1.0f - b2) * g * g;
  m1[i] = a;
  m2[i] = v;
  w[i] -= lr * (a / c1) / (sqrtf(v / c2) + eps);
}

// Packs FP32 weights W[tap][ci][co] (cin x cout real channels, ci / co
// padded to CIN / COUT with zeros) into B-fragment order for k_conv3x3:
// forward: frag[tap][kc][n][lane] = (W[tap][kc*16+2t, +1][n*8+g],
// W[tap][kc*16+2t+8, +9][n*8+g]); transposed (backward data): the same for
// W'[tap][co][ci] = W[8 - tap][ci][co] (CIN' = COUT, COUT' = CIN).
__global__ void k_pack_weights(const float* __restrict__ w, int cin, int cout, int CIN, int COUT, int transposed,
                               uint2* __restrict__ frag) {
  const int KIN = transposed ? COUT : CIN;   // k extent of the packed conv
  const int NOUT = transposed ? CIN : COUT;  // n extent
  const int KC = KIN / 16, NT = NOUT / 8;
  const int total = 9 * KC * NT * 32;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= total) return;
  const int lane = idx % 32, n = (idx / 32) % NT, kc = (idx / 32 / NT) % KC, tap = idx / 32 / NT / KC;
  const int g = lane >> 2, t = lane & 3;
  auto W = [&](int k, int o) -> float {  // element (k, o) of the packed conv's tap
    int ci, co, tp;
    if (transposed) {
      ci = o;
      co = k;
      tp = 8 - tap;
    } else {
      ci = k;
      co = o;
      tp = tap;
    }
    if (ci >= cin || co >= cout) return 0.0f;
    return w[(static_cast<size_t>(tp) * cin + ci) * cout + co];
  };
  const int o = n * 8 + g, k = kc * 16 + 2 * t;
  frag[idx] = make_uint2(pack_bf16(W(k, o), W(k + 1, o)), pack_bf16(W(k + 8, o), W(k + 9, o)));
}

// Masked mean-squared error of the first nc channels of y (FP32, C channels)
// against target (FP32, nc channels): per-block partial loss sums, and
// dy = 2 (y - target) mask / count as BF16 [p][C] (zero elsewhere).
template <int C>
__global__ void k_mse_grad(const float* __restrict__ y, const float* __restrict__ target,
                           const float* __restrict__ mask, long long npix, int nc, float inv_count,
                           __nv_bfloat16* __restrict__ dy, float* __restrict__ part) {
  __shared__ float s[256];
  const long long p = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  float l = 0.0f;
  if (p < npix) {
    const float mk = mask[p];
    for (int c = 0; c < C; ++c) {
      float d = 0.0f;
      if (c < nc) {
        const float e = (y[p * C + c] - target[p * nc + c]) * mk;
        l += e * e;
        d = 2.0f * e * inv_count;
      }
      dy[p * C + c] = __float2bfloat16_rn(d);
    }
  }
  s[threadIdx.x] = l;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = s[0];
}

template <int CIN, int COUT, int EPI>
cudaError_t conv(const void* x, int Hz, int Wx, const void* wfrag, const float* bias, void* y_bf16, float* y_f32,
                 void* z_pre, const void* z_prev, cudaStream_t s) {
  const dim3 grid(Hz / kTz, (Wx + kTx - 1) / kTx);
  k_conv3x3<CIN, COUT, EPI><<<grid, 256, 0, s>>>(
      static_cast<const __nv_bfloat16*>(x), Hz, Wx, static_cast<const uint2*>(wfrag), bias,
      static_cast<__nv_bfloat16*>(y_bf16), y_f32, static_cast<__nv_bfloat16*>(z_pre),
      static_cast<const __nv_bfloat16*>(z_prev));
  return cudaGetLastError();
}

// The input image of k_conv3x3_tc as a 3-D tensor map: dimensions (cin
// channels, Hz depths, Wx columns) of BF16, box 8 x 130 x 6, zero fill
// outside. cuTensorMapEncodeTiled checks the base (16-byte aligned) and the
// strides (cin * 2 and Hz * cin * 2 bytes, multiples of 16); every copy's
// channel coordinate is a multiple of 8 (16 bytes).
bool encode_input_map(CUtensorMap* m, const void* x, int Hz, int Wx, int cin) {
  static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  });
  if (!encode || reinterpret_cast<uintptr_t>(x) % 16 != 0) return false;
  const cuuint64_t dims[3] = {static_cast<cuuint64_t>(cin), static_cast<cuuint64_t>(Hz), static_cast<cuuint64_t>(Wx)};
  const cuuint64_t strides[2] = {static_cast<cuuint64_t>(cin) * 2, static_cast<cuuint64_t>(Hz) * cin * 2};
  const cuuint32_t box[3] = {8, static_cast<cuuint32_t>(kTcTileRows), static_cast<cuuint32_t>(kTcTileCols)};
  const cuuint32_t estr[3] = {1, 1, 1};
  return encode(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(x), dims, strides, box, estr,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace
}  // namespace fwigb_cnn

using namespace fwigb_cnn;

extern "C" {

int fwigb_cnn_conv3x3(const void* x, int Hz, int Wx, int cin_pad, int cout_pad, int epilogue, const void* wfrag,
                      const float* bias, void* y_bf16, float* y_f32, void* z_pre, const void* z_prev,
                      void* stream) {
  cudaGetLastError();  // drop a stale non-sticky error of an earlier, unrelated call
  if (!x || !wfrag || Hz <= 0 || Wx <= 0 || Hz % kTz != 0) return FWIGB_ERR_ARG;
  if (epilogue == kEpiGelu && (!bias || !y_bf16 || !z_pre)) return FWIGB_ERR_ARG;
  if (epilogue == kEpiLinearF32 && (!bias || !y_f32)) return FWIGB_ERR_ARG;
  if (epilogue == kEpiDGelu && (!y_bf16 || !z_prev)) return FWIGB_ERR_ARG;
  if (epilogue < 0 || epilogue > 2) return FWIGB_ERR_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaErrorInvalidValue;
#define FWIGB_CONV_CASE(CI, CO)                                                                           \
  if (cin_pad == CI && cout_pad == CO) {                                                                  \
    if (epilogue == kEpiGelu)                                                                             \
      e = conv<CI, CO, kEpiGelu>(x, Hz, Wx, wfrag, bias, y_bf16, y_f32, z_pre, z_prev, s);               \
    else if (epilogue == kEpiLinearF32)                                                                   \
      e = conv<CI, CO, kEpiLinearF32>(x, Hz, Wx, wfrag, bias, y_bf16, y_f32, z_pre, z_prev, s);          \
    else                                                                                                  \
      e = conv<CI, CO, kEpiDGelu>(x, Hz, Wx, wfrag, bias, y_bf16, y_f32, z_pre, z_prev, s);              \
  }
  FWIGB_CONV_CASE(16, 32)
  FWIGB_CONV_CASE(32, 32)
  FWIGB_CONV_CASE(32, 16)
#undef FWIGB_CONV_CASE
  if (e == cudaErrorInvalidValue) return FWIGB_ERR_UNSUPPORTED;
  return e == cudaSuccess ? FWIGB_OK : FWIGB_ERR_CUDA;
}

int fwigb_cnn_wgrad_partials(const void* x, const void* dz, int Hz, int Wx, int cin_pad, int cout_pad,
                             float* partials, void* stream) {
  cudaGetLastError();  // drop a stale non-sticky error of an earlier, unrelated call
  if (!x || !dz || !partials || Hz <= 0 || Wx <= 0 || Hz % kTz != 0) return FWIGB_ERR_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const dim3 grid(Hz / kTz, (Wx + kTx - 1) / kTx);
  const auto* xi = static_cast<const __nv_bfloat16*>(x);
  const auto* di = static_cast<const __nv_bfloat16*>(dz);
  if (cin_pad == 16 && cout_pad == 32)
    k_conv3x3_wgrad<16, 32><<<grid, 288, 0, s>>>(xi, di, Hz, Wx, partials);
  else if (cin_pad == 32 && cout_pad == 32)
    k_conv3x3_wgrad<32, 32><<<grid, 288, 0, s>>>(xi, di, Hz, Wx, partials);
  else if (cin_pad == 32 && cout_pad == 16)
    k_conv3x3_wgrad<32, 16><<<grid, 288, 0, s>>>(xi, di, Hz, Wx, partials);
  else
    return FWIGB_ERR_UNSUPPORTED;
  return cudaGetLastError() == cudaSuccess ? FWIGB_OK : FWIGB_ERR_CUDA;
}

int fwigb_cnn_tile_count(int Hz, int Wx) { return (Hz / kTz) * ((Wx + kTx - 1) / kTx); }

int fwigb_cnn_conv3x3_tc(const void* x, int Hz, int Wx, int cin_pad, int epilogue, const void* wpack,
                         const float* bias, void* y_bf16, void* z_pre, const void* z_prev, unsigned* err_word,
                         void* stream) {
  cudaGetLastError();  // drop a stale non-sticky error of an earlier, unrelated call
  if (!x || !wpack || !y_bf16 || !err_word || Hz <= 0 || Wx <= 0) return FWIGB_ERR_ARG;
  if (epilogue == kEpiGelu && (!bias || !z_pre)) return FWIGB_ERR_ARG;
  if (epilogue == kEpiDGelu && !z_prev) return FWIGB_ERR_ARG;
  if (epilogue != kEpiGelu && epilogue != kEpiDGelu) return FWIGB_ERR_UNSUPPORTED;
  if (cin_pad != 16 && cin_pad != 32) return FWIGB_ERR_UNSUPPORTED;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  CUtensorMap tmap;
  if (!encode_input_map(&tmap, x, Hz, Wx, cin_pad)) return FWIGB_ERR_CUDA;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return FWIGB_ERR_CUDA;
  const int ntiles = ((Hz + kTcRows - 1) / kTcRows) * ((Wx + kTcCols - 1) / kTcCols);
  const int grid = ntiles < sms ? ntiles : sms;  // persistent: at most one CTA per SM
  const auto* wp = static_cast<const uint4*>(wpack);
  auto* yo = static_cast<__nv_bfloat16*>(y_bf16);
  auto* zo = static_cast<__nv_bfloat16*>(z_pre);
  const auto* zi = static_cast<const __nv_bfloat16*>(z_prev);
  auto launch = [&](auto kernel, int cin) -> cudaError_t {
    const size_t smem = static_cast<size_t>(kTcStages) * (cin / 8) * kTcBoxStride + 9 * cin / 8 * 32 * 16;
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e != cudaSuccess) return e;
    kernel<<<grid, kTcThreads, smem, s>>>(tmap, Hz, Wx, wp, bias, yo, zo, zi, err_word);
    return cudaGetLastError();
  };
  cudaError_t e;
  if (cin_pad == 16)
    e = epilogue == kEpiGelu ? launch(k_conv3x3_tc<16, kEpiGelu>, 16) : launch(k_conv3x3_tc<16, kEpiDGelu>, 16);
  else
    e = epilogue == kEpiGelu ? launch(k_conv3x3_tc<32, kEpiGelu>, 32) : launch(k_conv3x3_tc<32, kEpiDGelu>, 32);
  return e == cudaSuccess ? FWIGB_OK : FWIGB_ERR_CUDA;
}

int fwigb_cnn_pack_weights_tc(const float* w, int cin, int cout, int cin_pad, int cout_pad, int transposed,
                              void* pack, void* stream) {
  cudaGetLastError();  // drop a stale non-sticky error of an earlier, unrelated call
  if (!w || !pack || cin <= 0 || cout <= 0 || cin > cin_pad || cout > cout_pad) return FWIGB_ERR_ARG;
  const int kin = transposed ? cout_pad : cin_pad, nout = transposed ? cin_pad : cout_pad;
  if ((kin != 16 && kin != 32) || nout != 32) return FWIGB_ERR_UNSUPPORTED;
  const int total = 9 * kin / 8 * 32;
  k_pack_weights_tc<<<(total + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(
      w, cin, cout, cin_pad, cout_pad, transposed, static_cast<uint4*>(pack));
  return cudaGetLastError() == cudaSuccess ? FWIGB_OK : FWIGB_ERR_CUDA;
}

int fwigb_cnn_reduce_partials(const float* partials, int nblocks, int n, float* out, void* stream) {
  cudaGetLastError();  // drop a stale non-sticky error of an earlier, unrelated call
  if (!partials || !out || nblocks <= 0 || n <= 0) return FWIGB_ERR_ARG;
  k_reduce_partials<<<(n + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(partials, nblocks, n, out);
  return cudaGetLastError() == cudaSuccess ? FWIGB_OK : FWIGB_ERR_CUDA;
}

int fwigb_cnn_bias_partials(const void* dz, long long npix, int c_pad, int chunk, float* partials, void* stream) {
  cudaGetLastError();  // drop a stale non-sticky error of an earlier, unrelated call
  if (!dz || !partials || npix <= 0 || chunk <= 0) return FWIGB_ERR_ARG;
  const int nb = static_cast<int>((npix + chunk - 1) / chunk);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const auto* d = static_cast<const __nv_bfloat16*>(dz);
  if (c_pad == 16)
    k_bias_partials<16><<<nb, 256, 0, s>>>(d, npix, chunk, partials);
  else if (c_pad == 32)
    k_bias_partials<32><<<nb, 256, 0, s>>>(d, npix, chunk, partials);
  else
    return FWIGB_ERR_UNSUPPORTED;
  return cudaGetLastError() == cudaSuccess ? FWIGB_OK : FWIGB_ERR_CUDA;
}

int fwigb_cnn_adam(float* w, const float* grad, float* m1, float* m2, int n, float lr, float beta1, float beta2,
                   float eps, int step, void* stream) {
  cudaGetLastError();  // drop a stale non-sticky error of an earlier, unrelated call
  if (!w || !grad || !m1 || !m2 || n <= 0 || step <= 0) return FWIGB_ERR_ARG;
  const float c1 = 1.0f - powf(beta1, static_cast<float>(step));
  const float c2 = 1.0f - powf(beta2, static_cast<float>(step));
  k_adam<<<(n + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(w, grad, m1, m2, n, lr, beta1, beta2, eps,
                                                                         c1, c2);
  return cudaGetLastError() == cudaSuccess ? FWIGB_OK : FWIGB_ERR_CUDA;
}

int fwigb_cnn_pack_weights(const float* w, int cin, int cout, int cin_pad, int cout_pad, int transposed, void* frag,
                           void* stream) {
  cudaGetLastError();  // drop a stale non-sticky error of an earlier, unrelated call
  if (!w || !frag || cin <= 0 || cout <= 0 || cin > cin_pad || cout > cout_pad) return FWIGB_ERR_ARG;
  const int kin = transposed ? cout_pad : cin_pad, nout = transposed ? cin_pad : cout_pad;
  if (kin % 16 != 0 || nout % 8 != 0) return FWIGB_ERR_ARG;
  const int total = 9 * (kin / 16) * (nout / 8) * 32;
  k_pack_weights<<<(total + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(
      w, cin, cout, cin_pad, cout_pad, transposed, static_cast<uint2*>(frag));
  return cudaGetLastError() == cudaSuccess ? FWIGB_OK : FWIGB_ERR_CUDA;
}

int fwigb_cnn_mse_grad(const float* y, const float* target, const float* mask, long long npix, int c_pad, int nc,
                       float inv_count, void* dy, float* partials, void* stream) {
  cudaGetLastError();  // drop a stale non-sticky error of an earlier, unrelated call
  if (!y || !target || !mask || !dy || !partials || npix <= 0 || nc > c_pad) return FWIGB_ERR_ARG;
  const int nb = static_cast<int>((npix + 255) / 256);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  auto* d = static_cast<__nv_bfloat16*>(dy);
  if (c_pad == 16)
    k_mse_grad<16><<<nb, 256, 0, s>>>(y, target, mask, npix, nc, inv_count, d, partials);
  else
    return FWIGB_ERR_UNSUPPORTED;
  return cudaGetLastError() == cudaSuccess ? FWIGB_OK : FWIGB_ERR_CUDA;
}

}  // extern "C"
