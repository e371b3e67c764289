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

namespace fwigb {
namespace {

constexpr float C1 = 1.125f;          // 9/8  (el_stress.cu:42)
constexpr float C2 = 1.0f / 24.0f;    // 1/24 (el_stress.cu:43)
constexpr float kMega = 1.0e6f;       // MEGA (utilities.h:16)

// Staggered 4th-order differences; Dm uses (i-2, i-1, i, i+1), Dp (i-1, i, i+1, i+2).
__device__ __forceinline__ float dmz(const float* __restrict__ a, size_t i, float r) {
  return (C1 * (a[i] - a[i - 1]) - C2 * (a[i + 1] - a[i - 2])) * r;
}
__device__ __forceinline__ float dpz(const float* __restrict__ a, size_t i, float r) {
  return (C1 * (a[i + 1] - a[i]) - C2 * (a[i + 2] - a[i - 1])) * r;
}
__device__ __forceinline__ float dmx(const float* __restrict__ a, size_t i, int nz, float r) {
  return (C1 * (a[i] - a[i - nz]) - C2 * (a[i + nz] - a[i - 2 * nz])) * r;
}
__device__ __forceinline__ float dpx(const float* __restrict__ a, size_t i, int nz, float r) {
  return (C1 * (a[i + nz] - a[i]) - C2 * (a[i + 2 * nz] - a[i - nz])) * r;
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

__device__ __forceinline__ bool in_box(int z, int x, int z0, int z1, int x0, int x1) {
  return z >= z0 && z <= z1 && x >= x0 && x <= x1;
}

// ---------------------------------------------------------------------------
// F1: el_stress (el_stress.cu:50-88) + add_source (utilities.cu:521-541) +
// recording (utilities.cu:557-567) + from_bnd of the 5 fields (Boundary.cu:55-76).
__global__ void __launch_bounds__(kTileZ* kTileX)
    k_fwd_stress(Geo g, Fields f, MediaD m, CpmlD c, ShotD sh, StoreD st, int it, int save) {
  const int z = blockIdx.x * kTileZ + threadIdx.x;
  const int x = blockIdx.y * kTileX + threadIdx.y;
  if (z >= g.nz || x >= g.nx) return;
  const int nz = g.nz;
  const size_t i = static_cast<size_t>(x) * nz + z;
  if (save) {
    const int k = ring_index(g, z, x);
    if (k >= 0) {
      float* p = st.base + static_cast<size_t>(it) * 5 * g.ring_len + k;
      p[0] = f.szz[i];
      p[g.ring_len] = f.sxz[i];
      p[2 * g.ring_len] = f.sxx[i];
      p[3 * g.ring_len] = f.vz[i];
      p[4 * g.ring_len] = f.vx[i];
    }
  }
  const bool dom = in_box(z, x, g.zs0, g.zs1, g.xs0, g.xs1);
  const bool src = (z == sh.src_z && x == sh.src_x);
  float szz = f.szz[i], sxx = f.sxx[i];
  if (dom) {
    const float* __restrict__ vz = f.vz;
    const float* __restrict__ vx = f.vx;
    float dvz_dz = dmz(vz, i, g.rdz);
    float dvx_dx = dmx(vx, i, nz, g.rdx);
    float dvx_dz = dpz(vx, i, g.rdz);
    float dvz_dx = dpx(vz, i, nz, g.rdx);
    const bool zp = (z < g.nPml) || (z > g.zpml_hi);
    const bool xp = (x < g.nPml) || (x > g.xpml_hi_s);
    if (zp) {
      float mm = c.b_z[z] * f.m_dvz_dz[i] + c.a_z[z] * dvz_dz;
      f.m_dvz_dz[i] = mm;
      dvz_dz = dvz_dz / c.K_z[z] + mm;
      mm = c.b_zh[z] * f.m_dvx_dz[i] + c.a_zh[z] * dvx_dz;
      f.m_dvx_dz[i] = mm;
      dvx_dz = dvx_dz / c.K_zh[z] + mm;
    }
    if (xp) {
      float mm = c.b_x[x] * f.m_dvx_dx[i] + c.a_x[x] * dvx_dx;
      f.m_dvx_dx[i] = mm;
      dvx_dx = dvx_dx / c.K_x[x] + mm;
      mm = c.b_xh[x] * f.m_dvz_dx[i] + c.a_xh[x] * dvz_dx;
      f.m_dvz_dx[i] = mm;
      dvz_dx = dvz_dx / c.K_xh[x] + mm;
    }
    const float lam = m.lam[i], l2m = m.l2m[i];
    szz += (l2m * dvz_dz + lam * dvx_dx) * g.dt;
    sxx += (lam * dvz_dz + l2m * dvx_dx) * g.dt;
    f.sxz[i] = f.sxz[i] + m.aveMu[i] * (dvx_dz + dvz_dx) * g.dt;
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
  // sample of step it+1 can be taken here.
  const int b = blockIdx.x + blockIdx.y * gridDim.x;
  for (int k = sh.blk_off[b]; k < sh.blk_off[b + 1]; ++k) {
    const int r = sh.blk_rec[k];
    if (sh.rec_z[r] == z && sh.rec_x[r] == x) sh.data[static_cast<size_t>(r) * sh.nSteps + it + 1] = szz + 3.0f * sxx;
  }
}

// F2: el_velocity, isFor = true (el_velocity.cu:45-82).
__global__ void __launch_bounds__(kTileZ* kTileX) k_fwd_velocity(Geo g, Fields f, MediaD m, CpmlD c) {
  const int z = blockIdx.x * kTileZ + threadIdx.x;
  const int x = blockIdx.y * kTileX + threadIdx.y;
  if (!in_box(z, x, g.zs0, g.zs1, g.xs0, g.xs1)) return;
  const int nz = g.nz;
  const size_t i = static_cast<size_t>(x) * nz + z;
  const float* __restrict__ szz = f.szz;
  const float* __restrict__ sxx = f.sxx;
  const float* __restrict__ sxz = f.sxz;
  float dszz_dz = dpz(szz, i, g.rdz);
  float dsxz_dx = dmx(sxz, i, nz, g.rdx);
  float dsxz_dz = dmz(sxz, i, g.rdz);
  float dsxx_dx = dpx(sxx, i, nz, g.rdx);
  const bool zp = (z < g.nPml) || (z > g.zpml_hi);
  const bool xp = (x < g.nPml) || (x > g.xpml_hi_v);
  if (zp) {
    float mm = c.b_zh[z] * f.m_dszz_dz[i] + c.a_zh[z] * dszz_dz;
    f.m_dszz_dz[i] = mm;
    dszz_dz = dszz_dz / c.K_zh[z] + mm;
    mm = c.b_z[z] * f.m_dsxz_dz[i] + c.a_z[z] * dsxz_dz;
    f.m_dsxz_dz[i] = mm;
    dsxz_dz = dsxz_dz / c.K_z[z] + mm;
  }
  if (xp) {
    float mm = c.b_x[x] * f.m_dsxz_dx[i] + c.a_x[x] * dsxz_dx;
    f.m_dsxz_dx[i] = mm;
    dsxz_dx = dsxz_dx / c.K_x[x] + mm;
    mm = c.b_xh[x] * f.m_dsxx_dx[i] + c.a_xh[x] * dsxx_dx;
    f.m_dsxx_dx[i] = mm;
    dsxx_dx = dsxx_dx / c.K_xh[x] + mm;
  }
  f.vz[i] += (dszz_dz + dsxz_dx) * m.bycA[i] * g.dt;
  f.vx[i] += (dsxz_dz + dsxx_dx) * m.bycB[i] * g.dt;
}

// ---------------------------------------------------------------------------
// B: add_source(-) + el_stress(isFor=false) + to_bnd(stress) + el_velocity_adj.
__global__ void __launch_bounds__(kTileZ* kTileX)
    k_bwd_B(Geo g, Fields f, MediaD m, CpmlD c, ShotD sh, StoreD st, Grads gr, int it) {
  const int z = blockIdx.x * kTileZ + threadIdx.x;
  const int x = blockIdx.y * kTileX + threadIdx.y;
  if (z >= g.nz || x >= g.nx) return;
  const int nz = g.nz;
  const size_t i = static_cast<size_t>(x) * nz + z;
  const float dt = g.dt;
  const float* __restrict__ vz = f.vz;
  const float* __restrict__ vx = f.vx;
  const float* __restrict__ sxz_a = f.sxz_a;
  const bool interior = in_box(z, x, g.zi0, g.zi1, g.xi0, g.xi1);
  const bool src = (z == sh.src_z && x == sh.src_x);
  const int k = ring_index(g, z, x);
  float e_own = 0.0f, gmu_own = 0.0f;
  if (interior || src || k >= 0) {
    float szz = f.szz[i], sxx = f.sxx[i], sxz = f.sxz[i];
    if (src) {
      szz -= sh.src_szz[it];
      sxx -= sh.src_sxx[it];
    }
    if (interior) {
      const float dvz_dz = dmz(vz, i, g.rdz);
      const float dvx_dx = dmx(vx, i, nz, g.rdx);
      const float dvx_dz = dpz(vx, i, g.rdz);
      const float dvz_dx = dpx(vz, i, nz, g.rdx);
      const float lam = m.lam[i], l2m = m.l2m[i];
      szz -= (l2m * dvz_dz + lam * dvx_dx) * dt;
      sxx -= (lam * dvz_dz + l2m * dvx_dx) * dt;
      e_own = dvx_dz + dvz_dx;
      sxz -= m.aveMu[i] * e_own * dt;
      const float sa = f.szz_a[i], xa = f.sxx_a[i];
      gr.lam[i] += -(sa + xa) * (dvz_dz + dvx_dx) * dt * kMega;
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
    float acc = gr.mu[i] + gmu_own;
    const float w = m.muw[i];
    const float* __restrict__ hs = m.hs;
    if (x <= g.xi1) {
      const float h = hs[i];
      if (h != 0.0f) acc += w * (-sxz_a[i] * e_own * dt * h);
      if (z - 1 >= g.zi0) {
        const size_t j = i - 1;
        const float hj = hs[j];
        if (hj != 0.0f) acc += w * (-sxz_a[j] * (dpz(vx, j, g.rdz) + dpx(vz, j, nz, g.rdx)) * dt * hj);
      }
    }
    if (x - 1 >= g.xi0) {
      const size_t j = i - nz;
      const float hj = hs[j];
      if (hj != 0.0f) acc += w * (-sxz_a[j] * (dpz(vx, j, g.rdz) + dpx(vz, j, nz, g.rdx)) * dt * hj);
      if (z - 1 >= g.zi0 && x <= g.xi1) {
        const size_t j2 = i - nz - 1;
        const float h2 = hs[j2];
        if (h2 != 0.0f) acc += w * (-sxz_a[j2] * (dpz(vx, j2, g.rdz) + dpx(vz, j2, nz, g.rdx)) * dt * h2);
      }
    }
    gr.mu[i] = acc;
  }
  // el_velocity_adj (el_velocity_adj.cu:161-206).
  if (!in_box(z, x, g.zs0, g.zs1, g.xs0, g.xs1)) return;
  const float* __restrict__ szz_a = f.szz_a;
  const float* __restrict__ sxx_a = f.sxx_a;
  const float lam = m.lam[i], l2m = m.l2m[i], amu = m.aveMu[i];
  const bool zp = (z < g.nPml) || (z > g.zpml_hi);
  const bool xp = (x < g.nPml) || (x > g.xpml_hi_s);
  {
    const float Kx = c.K_x[x], Kzh = c.K_zh[z];
    const float dszz_dx = -dpx(szz_a, i, nz, g.rdx);
    const float dsxx_dx = -dpx(sxx_a, i, nz, g.rdx);
    const float dsxz_dz = -dmz(sxz_a, i, g.rdz);
    float t = lam * dszz_dx / Kx * dt + l2m * dsxx_dx / Kx * dt + amu / Kzh * dsxz_dz * dt;
    const float ax = c.a_x[x], azh = c.a_zh[z];
    if (ax != 0.0f) t += ax * (-dpx(f.m_dvx_dx, i, nz, g.rdx));
    if (azh != 0.0f) t += azh * (-dmz(f.m_dvx_dz, i, g.rdz));
    const float v = f.vx_a[i] + t;
    f.vx_a[i] = v;
    if (xp) f.m_dsxx_dx[i] = c.b_xh[x] * f.m_dsxx_dx[i] + m.bycB[i] * v * dt;
    if (zp) f.m_dsxz_dz[i] = c.b_z[z] * f.m_dsxz_dz[i] + m.bycB[i] * v * dt;
  }
  {
    const float Kz = c.K_z[z], Kxh = c.K_xh[x];
    const float dszz_dz = -dpz(szz_a, i, g.rdz);
    const float dsxx_dz = -dpz(sxx_a, i, g.rdz);
    const float dsxz_dx = -dmx(sxz_a, i, nz, g.rdx);
    float t = l2m * dszz_dz / Kz * dt + lam * dsxx_dz / Kz * dt + amu / Kxh * dsxz_dx * dt;
    const float az = c.a_z[z], axh = c.a_xh[x];
    if (az != 0.0f) t += az * (-dpz(f.m_dvz_dz, i, g.rdz));
    if (axh != 0.0f) t += axh * (-dmx(f.m_dvz_dx, i, nz, g.rdx));
    const float v = f.vz_a[i] + t;
    f.vz_a[i] = v;
    if (xp) f.m_dsxz_dx[i] = c.b_x[x] * f.m_dsxz_dx[i] + m.bycA[i] * v * dt;
    if (zp) f.m_dszz_dz[i] = c.b_zh[z] * f.m_dszz_dz[i] + m.bycA[i] * v * dt;
  }
}

// C: res_injection (utilities.cu:569-580) + el_stress_adj (el_stress_adj.cu:53-97)
//    + source_grad (utilities.cu:582-593) + el_velocity(isFor=false) with the
//    density kernel (el_velocity.cu:220-244) + to_bnd(velocity).
__global__ void __launch_bounds__(kTileZ* kTileX)
    k_bwd_C(Geo g, Fields f, MediaD m, CpmlD c, ShotD sh, StoreD st, Grads gr, int it, int rev) {
  const int z = blockIdx.x * kTileZ + threadIdx.x;
  const int x = blockIdx.y * kTileX + threadIdx.y;
  if (z >= g.nz || x >= g.nx) return;
  const int nz = g.nz;
  const size_t i = static_cast<size_t>(x) * nz + z;
  const float dt = g.dt;
  const bool dom = in_box(z, x, g.zs0, g.zs1, g.xs0, g.xs1);
  float sa = f.szz_a[i], xa = f.sxx_a[i];
  bool injected = false;
  const int b = blockIdx.x + blockIdx.y * gridDim.x;
  for (int k = sh.blk_off[b]; k < sh.blk_off[b + 1]; ++k) {
    const int r = sh.blk_rec[k];
    if (sh.rec_z[r] == z && sh.rec_x[r] == x) {
      const float rv = sh.res[static_cast<size_t>(r) * sh.nSteps + it];
      sa += rv;
      xa += 3.0f * rv;
      injected = true;
    }
  }
  if (dom) {
    const float* __restrict__ vz_a = f.vz_a;
    const float* __restrict__ vx_a = f.vx_a;
    const float bA = m.bycA[i], bB = m.bycB[i], amu = m.aveMu[i];
    // sxz
    float za = f.sxz_a[i];
    {
      const float dvz_dx = -dpx(vz_a, i, nz, g.rdx);
      const float dvx_dz = -dpz(vx_a, i, g.rdz);
      float t = dvz_dx / c.K_x[x] * bA * dt + dvx_dz / c.K_z[z] * bB * dt;
      const float ax = c.a_x[x], az = c.a_z[z];
      if (ax != 0.0f) t += ax * (-dpx(f.m_dsxz_dx, i, nz, g.rdx));
      if (az != 0.0f) t += az * (-dpz(f.m_dsxz_dz, i, g.rdz));
      za += t;
      f.sxz_a[i] = za;
    }
    const bool xb = (x <= g.xband_lo) || (x >= g.xband_hi);
    const bool zb = (z <= g.zband_lo) || (z >= g.zband_hi);
    if (xb) f.m_dvz_dx[i] = c.b_xh[x] * f.m_dvz_dx[i] + za * amu * dt;
    if (zb) f.m_dvx_dz[i] = c.b_zh[z] * f.m_dvx_dz[i] + za * amu * dt;
    {
      const float dvx_dx = -dmx(vx_a, i, nz, g.rdx);
      const float dvz_dz = -dmz(vz_a, i, g.rdz);
      float tx = bB * dvx_dx / c.K_xh[x] * dt;
      float tz = bA * dvz_dz / c.K_zh[z] * dt;
      const float axh = c.a_xh[x], azh = c.a_zh[z];
      if (axh != 0.0f) tx += axh * (-dmx(f.m_dsxx_dx, i, nz, g.rdx));
      if (azh != 0.0f) tz += azh * (-dmz(f.m_dszz_dz, i, g.rdz));
      xa += tx;
      sa += tz;
    }
    const float lam = m.lam[i], l2m = m.l2m[i];
    if (xb) f.m_dvx_dx[i] = c.b_x[x] * f.m_dvx_dx[i] + lam * sa * dt + l2m * xa * dt;
    if (zb) f.m_dvz_dz[i] = c.b_z[z] * f.m_dvz_dz[i] + l2m * sa * dt + lam * xa * dt;
  }
  if (dom || injected) {
    f.szz_a[i] = sa;
    f.sxx_a[i] = xa;
  }
  if (!rev) return;
  if (z == sh.src_z && x == sh.src_x) sh.gstf[it - 1] = -(sa + 3.0f * xa) * dt;

  const float* __restrict__ szz = f.szz;
  const float* __restrict__ sxx = f.sxx;
  const float* __restrict__ sxz = f.sxz;
  const float* __restrict__ vz_a = f.vz_a;
  const float* __restrict__ vx_a = f.vx_a;
  const bool interior = in_box(z, x, g.zi0, g.zi1, g.xi0, g.xi1);
  float tA = 0.0f, tB = 0.0f;
  if (interior) {
    const float ea = dpz(szz, i, g.rdz) + dmx(sxz, i, nz, g.rdx);  // dszz_dz + dsxz_dx
    const float eb = dmz(sxz, i, g.rdz) + dpx(sxx, i, nz, g.rdx);  // dsxz_dz + dsxx_dx
    const float bA = m.bycA[i], bB = m.bycB[i];
    f.vz[i] -= ea * bA * dt;
    f.vx[i] -= eb * bB * dt;
    tA = -vz_a[i] * ea * dt * (-bA * bA * 0.5f);
    tB = -vx_a[i] * eb * dt * (-bB * bB * 0.5f);
  }
  const int k = ring_index(g, z, x);
  if (k >= 0) {
    const float* p = st.base + static_cast<size_t>(it - 1) * 5 * g.ring_len + k;
    f.vz[i] = p[3 * g.ring_len];
    f.vx[i] = p[4 * g.ring_len];
  }
  // rho kernel gather: (z,x) receives A and B of itself, A of (z-1,x) and B of
  // (z,x-1) (el_velocity.cu:238-243; the x guard of :242 is always true).
  if (in_box(z, x, g.zi0, g.zi1, g.xi0, g.xi1 + 1)) {
    float acc = gr.den[i];
    if (x <= g.xi1) {
      acc += tA;
      acc += tB;
      if (z - 1 >= g.zi0) {
        const size_t j = i - 1;
        const float bA = m.bycA[j];
        const float ea = dpz(szz, j, g.rdz) + dmx(sxz, j, nz, g.rdx);
        acc += -vz_a[j] * ea * dt * (-bA * bA * 0.5f);
      }
    }
    if (x - 1 >= g.xi0) {
      const size_t j = i - nz;
      const float bB = m.bycB[j];
      const float eb = dmz(sxz, j, g.rdz) + dpx(sxx, j, nz, g.rdx);
      acc += -vx_a[j] * eb * dt * (-bB * bB * 0.5f);
    }
    gr.den[i] = acc;
  }
}

// ---------------------------------------------------------------------------
// Model set-up.
constexpr int kT = 32;

// Row-major double [nz][nx] (MPa) -> column-major float (Pa), through a
// shared-memory tile so both sides are coalesced (libCUFD.cu:67-78).
__global__ void k_media_from_rowmajor(int nz, int nx, const double* __restrict__ L, const double* __restrict__ M,
                                      const double* __restrict__ D, float* lam, float* mu, float* den,
                                      unsigned* cpmax_bits) {
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
      const size_t d = static_cast<size_t>(x) * nz + z;
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
__global__ void k_media_derived(int nz, int nx, const float* __restrict__ lam, const float* __restrict__ mu,
                                const float* __restrict__ den, float* l2m, float* aveMu, float* bycA, float* bycB,
                                float* hs, float* muw) {
  const int z = blockIdx.x * blockDim.x + threadIdx.x;
  const int x = blockIdx.y * blockDim.y + threadIdx.y;
  if (z >= nz || x >= nx) return;
  const size_t i = static_cast<size_t>(x) * nz + z;
  const float u = mu[i];
  l2m[i] = lam[i] + 2.0f * u;
  muw[i] = (u != 0.0f) ? static_cast<float>(1.0 / (static_cast<double>(u) * u)) : 0.0f;
  float am = 0.0f, ha = 0.0f, ba = 1.0f / 1000.0f, bb = 1.0f / 1000.0f;
  if (z >= 2 && z <= nz - 3 && x >= 2 && x <= nx - 3) {
    const float a = u, b = mu[i + 1], c = mu[i + nz], d = mu[i + nz + 1];
    if (!(a == 0.0f || b == 0.0f || c == 0.0f || d == 0.0f)) {
      const double s = 1.0 / a + 1.0 / b + 1.0 / c + 1.0 / d;
      am = static_cast<float>(4.0 / s);
      ha = static_cast<float>(am / s * 1e6);
    }
    ba = static_cast<float>(2.0 / (den[i + 1] + den[i]));
    bb = static_cast<float>(2.0 / (den[i + nz] + den[i]));
  }
  aveMu[i] = am;
  hs[i] = ha;
  bycA[i] = ba;
  bycB[i] = bb;
}

// Column-major float -> row-major double (libCUFD.cu:480-486).
__global__ void k_to_rowmajor(int nz, int nx, const float* __restrict__ src, double* dst, double scale) {
  __shared__ float t[kT][kT + 1];
  const int z0 = blockIdx.x * kT, x0 = blockIdx.y * kT;
  for (int r = threadIdx.y; r < kT; r += blockDim.y) {
    const int x = x0 + r, z = z0 + threadIdx.x;
    if (z < nz && x < nx) t[r][threadIdx.x] = src[static_cast<size_t>(x) * nz + z];
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
    const float wo = per_trace ? taper_o[k] : taper_o[t];
    const float wr = per_trace ? taper_r[k] : taper_r[t];
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

// Fixed-order sum of the block partials into *acc (one warp).
__global__ void k_sum_partials(const double* __restrict__ partials, int n, double* acc) {
  double v = 0.0;
  for (int k = threadIdx.x; k < n; k += 32) v += partials[k];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if (threadIdx.x == 0) *acc += v;
}

}  // namespace

// ---------------------------------------------------------------------------
static dim3 sweep_grid(const Geo& g) { return dim3((g.nz + kTileZ - 1) / kTileZ, (g.nx + kTileX - 1) / kTileX); }

void launch_fwd_stress(cudaStream_t s, const Geo& g, const Fields& f, const MediaD& m, const CpmlD& c,
                       const ShotD& sh, const StoreD& st, int it, bool save) {
  k_fwd_stress<<<sweep_grid(g), dim3(kTileZ, kTileX), 0, s>>>(g, f, m, c, sh, st, it, save ? 1 : 0);
}

void launch_fwd_velocity(cudaStream_t s, const Geo& g, const Fields& f, const MediaD& m, const CpmlD& c) {
  k_fwd_velocity<<<sweep_grid(g), dim3(kTileZ, kTileX), 0, s>>>(g, f, m, c);
}

void launch_bwd_B(cudaStream_t s, const Geo& g, const Fields& f, const MediaD& m, const CpmlD& c, const ShotD& sh,
                  const StoreD& st, const Grads& gr, int it) {
  k_bwd_B<<<sweep_grid(g), dim3(kTileZ, kTileX), 0, s>>>(g, f, m, c, sh, st, gr, it);
}

void launch_bwd_C(cudaStream_t s, const Geo& g, const Fields& f, const MediaD& m, const CpmlD& c, const ShotD& sh,
                  const StoreD& st, const Grads& gr, int it, bool rev) {
  k_bwd_C<<<sweep_grid(g), dim3(kTileZ, kTileX), 0, s>>>(g, f, m, c, sh, st, gr, it, rev ? 1 : 0);
}

void launch_media_from_rowmajor(cudaStream_t s, int nz, int nx, const double* lam_mpa, const double* mu_mpa,
                                const double* den, float* lam, float* mu, float* den_f, unsigned* cpmax_bits) {
  dim3 grid((nx + kT - 1) / kT, (nz + kT - 1) / kT);
  k_media_from_rowmajor<<<grid, dim3(kT, 8), 0, s>>>(nz, nx, lam_mpa, mu_mpa, den, lam, mu, den_f, cpmax_bits);
}

void launch_media_derived(cudaStream_t s, int nz, int nx, const float* lam, const float* mu, const float* den,
                          float* l2m, float* aveMu, float* bycA, float* bycB, float* hs, float* muw,
                          unsigned* /*cpmax_bits*/) {
  dim3 grid((nz + 31) / 32, (nx + 7) / 8);
  k_media_derived<<<grid, dim3(32, 8), 0, s>>>(nz, nx, lam, mu, den, l2m, aveMu, bycA, bycB, hs, muw);
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

void launch_sum_partials(cudaStream_t s, const double* partials, int n, double* acc) {
  k_sum_partials<<<1, 32, 0, s>>>(partials, n, acc);
}

void launch_to_rowmajor(cudaStream_t s, int nz, int nx, const float* src, double* dst, double scale) {
  dim3 grid((nz + kT - 1) / kT, (nx + kT - 1) / kT);
  k_to_rowmajor<<<grid, dim3(kT, 8), 0, s>>>(nz, nx, src, dst, scale);
}

}  // namespace fwigb
