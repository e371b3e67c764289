// Device-side data structures of the GB300 elastic FWI engine and the host
// launch interface of its kernels (implemented in kernels.cu).
//
// Layout in HBM: every grid array is column-major [nx][ldz] float, z fastest,
// as in the reference (a(z,x) = a[x*nz + z], el_stress.cu:1-19) but with the
// column stride ldz = nz rounded up to 32, so every column starts on a
// 128-byte boundary: one warp reads 32 consecutive depths in one transaction
// and every TMA tile of the sweeps starts 16-byte aligned.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstddef>

namespace fwigb {

// Sweep tiles: backward sweeps 32 depths x TX columns, one cell per thread;
// forward sweeps 64 depths x TX columns, two adjacent depths per thread
// (block 32 x TX in both), TX in {4, 8, 16} chosen per sweep by the
// autotuner.
constexpr int kTileZ = 32;
constexpr int kRowsFwd = 2;
constexpr int kTileZFwd = kTileZ * kRowsFwd;
// Receivers are binned on a fixed 32 x 8 grid, independent of the sweep tile.
constexpr int kBinZ = 32;
constexpr int kBinX = 8;
// TMA box of one staged array: depths z0-4 .. z0+tile+3 (start aligned to
// 16 bytes), columns x0-2 .. x0+TX+1.
constexpr int kBoxZ = kTileZ + 8;
constexpr int kBoxZFwd = kTileZFwd + 8;
constexpr int kTileXs[3] = {4, 8, 16};

// Tensor maps of the (up to 5) arrays a sweep stages into shared memory.
struct TileMaps {  // 128-byte aligned (CUtensorMap)
  CUtensorMap t[5];
};

// Grid geometry and the index ranges of the reference kernels.
struct Geo {
  int nz, nx, nPml, nPad;
  int ldz;                 // column stride of every grid array (nz rounded up to 32)
  int zs0, zs1, xs0, xs1;  // stencil domain [2, nz-nPad-3] x [2, nx-3] (el_stress.cu:52)
  int zi0, zi1, xi0, xi1;  // reverse-time interior (el_stress.cu:93)
  int zpml_hi;             // z-PML: z < nPml || z > zpml_hi   (= nz-nPml-nPad-1)
  int xpml_hi_s;           // stress / adjoint x-PML: x > xpml_hi_s (= nx-nPml-1)
  int xpml_hi_v;           // forward velocity x-PML: x > xpml_hi_v (= nx-nPml, el_velocity.cu:56)
  int xband_lo, xband_hi;  // adjoint memory band in x: x <= xband_lo || x >= xband_hi
  int zband_lo, zband_hi;  // adjoint memory band in z
  // Boundary ring saved each forward step: box [rz0,rz1]x[rx0,rx1] minus its
  // inner box shrunk by 5 (the 5 layers around the interior, Boundary.cu:17-27).
  int rz0, rz1, rx0, rx1, ringW, ringH, ring_len;
  // Fast box (inclusive cell ranges): cells where every sweep reduces to its
  // interior form. Inside the stencil domain and the reverse-time interior
  // (with the z-1 / x-1 neighbours of the imaging gathers), outside the CPML,
  // the adjoint memory bands and the boundary ring, and with K = 1, a = 0 in
  // both CPML profiles. Empty when fz0 > fz1 or fx0 > fx1.
  int fz0, fz1, fx0, fx1;
  // Mid box: cells of the stencil domain outside the CPML (K = 1, a = 0 in
  // both profiles); it holds the fast box. Tiles inside it but not inside the
  // fast box (the ring, adjoint-memory band and interior-guard cells next to
  // the CPML) run the mid form of a sweep: the fast arithmetic with per-cell
  // ring, band and guard handling.
  int mz0, mz1, mx0, mx1;
  // Last row any sweep reads its own cells of or writes, apart from the
  // shot's source and receivers: max(zs1, rz1). Rows below it (the nPad rows
  // past the stencil domain) are only read as halo.
  int zact1;
  float dt, rdz, rdx;
};

// Split of a sub-grid's tiles (tz depths x tx columns, ntz x ntx in all)
// into the fast tiles, the rectangle [ftz0, ftz1) x [ftx0, ftx1) of tiles
// inside the fast box, the mid tiles, those of the rectangle [mtz0, mtz1) x
// [mtx0, mtx1) inside the mid box that are not fast, and the edge tiles
// around them.
struct TileSplit {
  int ntz, ntx, ftz0, ftz1, ftx0, ftx1, mtz0, mtz1, mtx0, mtx1;
};

__host__ __device__ inline TileSplit tile_split(const Geo& g, int tx, int tz) {
  TileSplit s;
  s.ntz = (g.nz + tz - 1) / tz;
  s.ntx = (g.nx + tx - 1) / tx;
  s.ftz0 = (g.fz0 + tz - 1) / tz;
  s.ftz1 = (g.fz1 + 1) / tz;
  s.ftx0 = (g.fx0 + tx - 1) / tx;
  s.ftx1 = (g.fx1 + 1) / tx;
  if (g.fz0 > g.fz1 || g.fx0 > g.fx1 || s.ftz1 <= s.ftz0 || s.ftx1 <= s.ftx0) s.ftz0 = s.ftz1 = s.ftx0 = s.ftx1 = 0;
  s.mtz0 = (g.mz0 + tz - 1) / tz;
  s.mtz1 = (g.mz1 + 1) / tz;
  s.mtx0 = (g.mx0 + tx - 1) / tx;
  s.mtx1 = (g.mx1 + 1) / tx;
  if (g.mz0 > g.mz1 || g.mx0 > g.mx1 || s.mtz1 <= s.mtz0 || s.mtx1 <= s.mtx0) s.mtz0 = s.mtz1 = s.mtx0 = s.mtx1 = 0;
  return s;
}

struct Fields {
  float *vz, *vx, *szz, *sxx, *sxz;
  float *vz_a, *vx_a, *szz_a, *sxx_a, *sxz_a;
  float *m_dvz_dz, *m_dvz_dx, *m_dvx_dz, *m_dvx_dx;    // forward CPML / adjoint psi memory
  float *m_dszz_dz, *m_dsxx_dx, *m_dsxz_dz, *m_dsxz_dx;  // forward CPML / adjoint phi memory
};

struct MediaD {
  const float* lam;    // lambda [Pa]
  const float* l2m;    // lambda + 2 mu [Pa]
  const float* aveMu;  // harmonic 2x2 average of mu (aveMuInit, utilities.cu:125-140)
  const float* bycA;   // 2 / (rho(z) + rho(z+1))  (aveBycInit, utilities.cu:142-152)
  const float* bycB;   // 2 / (rho(x) + rho(x+1))
  const float* hs;     // aveMu / sum(1/mu over the 2x2 block) * 1e6, 0 where aveMu == 0
  const float* muw;    // 1 / mu^2, 0 where mu == 0
};

struct CpmlD {
  const float *K_z, *a_z, *b_z, *K_zh, *a_zh, *b_zh;  // length nz
  const float *K_x, *a_x, *b_x, *K_xh, *a_xh, *b_xh;  // length nx
};

// Per-shot data for the sweeps.
struct ShotD {
  int src_z, src_x;       // source cell (padded-grid indices)
  const float* src_szz;   // per step: 1500^2 * amp * dt (add_source, utilities.cu:528-538)
  const float* src_sxx;   // per step: 3 * 1500^2 * amp * dt
  const float* src_szz_r; // the terms the reverse reconstruction subtracts: src_szz / src_sxx, or
  const float* src_sxx_r; // those of the updated wavelet under the source update (libCUFD.cu:326-328, 391-394)
  int nrec, nSteps;
  const int* rec_z;       // receiver cells
  const int* rec_x;
  const int* blk_off;     // receivers per 32 x 8 bin (CSR over the bins)
  const int* blk_rec;
  int nbin_z;             // bins along z
  int rbz0, rbz1, rbx0, rbx1;  // bounding box (cells) of the receivers and the source
  float* data;            // synthetic gathers [nrec][nSteps]
  const float* res;       // adjoint source [nrec][nSteps]
  float* gstf;            // source-time-function gradient [nSteps]
};

struct StoreD {
  float* base;  // [step][5 fields: szz, sxz, sxx, vz, vx][ring_len]
};

struct Grads {
  float* lam;
  float* mu;
  float* den;
  float* illum;  // source illumination sum_t (vz^2 + vx^2), or null when not accumulated
};

// Everything one shot's sweeps need, for a shot running on its own sub-grid
// (an aperture window of the model: padded columns x_off .. x_off + g.nx - 1)
// with its own record length. Media pointers are views of the global media
// shifted by x_off columns; CPML x profiles are those of the sub-grid width.
struct ShotSlot {
  Geo g;
  Fields f;
  MediaD m;
  CpmlD c;
  ShotD sh;
  StoreD st;
  Grads gr;  // this shot's gradient on its sub-grid
  int nSteps;
  int x_off;
};

// Tensor maps of the sweeps for one tile width: F1 stages vz, vx; F2 szz,
// sxx, sxz; B vz, vx, szz_a, sxx_a, sxz_a; C vz_a, vx_a, szz, sxx, sxz.
struct SweepMaps {
  TileMaps f1, f2, b, c;
  TileMaps f1w, f2w, bw, cw;  // the sweeps with two-row tiles (kBoxZFwd boxes)
};
// Launch variants of the sweeps: 0 F1, 1 F2, 2 B, 3 C (one row per thread),
// 4 F1, 5 F2, 6 B, 7 C (two rows per thread).
constexpr int kSweepVariants = 8;

// What one sweep launch reads for up to K shots, passed by value as a
// __grid_constant__ kernel parameter: the block of shot k reads its slot and
// tensor maps from the constant bank (no global-memory round trip before its
// first stencil load). K = 1 for a lone shot; kPackShots for a batch, which
// keeps the parameter block under the 32 KB kernel-parameter limit.
constexpr int kPackShots = 16;
template <int K>
struct SweepPack {
  TileMaps maps[K];
  ShotSlot slots[K];
};
static_assert(sizeof(SweepPack<kPackShots>) < 32000, "sweep pack exceeds the kernel parameter limit");

// Encodes the sweep tensor maps for tile width tx (host; needs the driver's
// cuTensorMapEncodeTiled). Returns false with a message on failure.
bool encode_sweep_maps(const Geo& g, const Fields& f, int tx, SweepMaps& out, const char** err);

// Launch extent of one sweep over the first shots of a pack: the widest
// sub-grid among them (nx), and the rows down to the last one any of them
// touches (nz: zact1 + 1, or further down to the lowest source or receiver).
// Blocks past a shot's own grid leave at once.
struct SweepGrid {
  int nz, nx;
};

// ---- launchers (kernels.cu). One launch covers the first `nshots` (<= K)
// shots of a pack. err is a device word that a sweep sets when a bounded
// wait for its staged tiles gives up. The backward sweeps take the backward
// iteration j; shot k works on its step nSteps_k - 2 - j. Instantiated for
// K = 1 and K = kPackShots. Each returns the number of kernels it launched.
// The forward launchers take the rows per thread (1 or 2; the pack's maps
// must be the matching variant). launch_fwd_stress flags: bit 0 saves the
// boundary ring of step it; bit 1 is the timeout test hook (the sweep's
// bounded wait runs out after its tiles have landed and raises err).
template <int K>
int launch_fwd_stress(cudaStream_t s, int tx, int rows, const SweepPack<K>& p, int nshots, const SweepGrid& gr,
                      int it, int flags, unsigned* err);
template <int K>
int launch_fwd_velocity(cudaStream_t s, int tx, int rows, const SweepPack<K>& p, int nshots, const SweepGrid& gr,
                        unsigned* err);
// The backward launchers also take the register budget of one-row tiles:
// 32 (64 warps per SM) or 40 (48 warps per SM); two-row tiles use 64.
template <int K>
int launch_bwd_B(cudaStream_t s, int tx, int rows, int regs, const SweepPack<K>& p, int nshots, const SweepGrid& gr,
                 int j, unsigned* err);
template <int K>
int launch_bwd_C(cudaStream_t s, int tx, int rows, int regs, const SweepPack<K>& p, int nshots, const SweepGrid& gr,
                 int j, unsigned* err);
// Adds the per-shot gradients (when g_lam is not null) and illuminations (when
// g_illum is not null) of the first nshots slots into the global ones.
void launch_reduce_grads(cudaStream_t s, int nz, int nx, int ldz, int nshots, const ShotSlot* slots, float* g_lam,
                         float* g_mu, float* g_den, float* g_illum);

// Model set-up: row-major double (lambda, mu in MPa) -> column-major float media.
// cpmax_bits receives atomicMax of the P velocity's float bits.
void launch_media_from_rowmajor(cudaStream_t s, int nz, int nx, int ldz, const double* lam_mpa, const double* mu_mpa,
                                const double* den, float* lam, float* mu, float* den_f, unsigned* cpmax_bits);
void launch_media_derived(cudaStream_t s, int nz, int nx, int ldz, const float* lam, const float* mu,
                          const float* den, float* l2m, float* aveMu, float* bycA, float* bycB, float* hs,
                          float* muw);

// Residual: res = taper_r * (taper_o * obs - taper_o * syn) with sample 0
// zeroed; syn is tapered in place. taper arrays are [nrec][nSteps] when
// per_trace, else [nSteps]. Block partial sums of res^2 (before the adjoint
// taper) go to partials[0..nblocks).
int residual_blocks(int n);
void launch_residual(cudaStream_t s, int nrec, int nSteps, const float* obs, float* syn, float* res,
                     const float* taper_o, const float* taper_r, int per_trace, double* partials);
void launch_sum_partials(cudaStream_t s, const double* partials, int n, double* acc);
// (taper_o / taper_r may be null: a weight of 1.)

// out = in * taper (per_trace: [nrec][nSteps], else [nSteps]).
void launch_apply_taper(cudaStream_t s, int nrec, int nSteps, const float* in, float* out, const float* taper,
                        int per_trace);
// Band-pass of nrec traces of nt samples: y = x circularly convolved with the
// impulse response h (2 nt floats); x and y distinct.
void launch_trace_filter(cudaStream_t s, int nrec, int nt, const float* x, float* y, const float* h);
// Source-wavelet update of one shot: spectra partial sums into part
// (src_spectra_blocks(nrec) x 3 x (nt + 1) floats), coef (nt + 1), and the
// update's impulse response kresp (2 nt floats). w2: the padded-length taper
// (nt floats); tw: the twiddle table (cos, sin)(2 pi k / 2 nt), 2 nt entries.
int src_spectra_blocks(int nrec);
void launch_src_update_coef(cudaStream_t s, int nrec, int nt, const float* obs, const float* syn, const float* w2,
                            const float2* tw, float* part, float2* coef, float* kresp);
void launch_src_terms(cudaStream_t s, int nt, float dt, const float* amp, float* szz, float* sxx);

// Column-major float grid (stride ldz) -> row-major double.
void launch_to_rowmajor(cudaStream_t s, int nz, int nx, int ldz, const float* src, double* dst, double scale);

}  // namespace fwigb
