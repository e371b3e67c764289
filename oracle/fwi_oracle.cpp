// CPU oracle for the elastic FWI operator of FwiFlow.jl (deps/CustomOps/FWI/Src).
//
// TEST INFRASTRUCTURE ONLY. This file is the parity checker for the GB300 CUDA
// path and the timed CPU baseline ("port") of bench.py. Only tests/,
// __graft_entry__.smoke() and bench.py's CPU-baseline / reference arm load it.
// The product library never links or calls it.
//
// It restates, loop for loop and in the same floating-point types, the
// reference driver `cufd` (libCUFD.cu:34-580) and the kernels it launches:
//   el_stress        (el_stress.cu:24-133)       forward + reverse/imaging
//   el_velocity      (el_velocity.cu:20-118)     forward + reverse/imaging
//   el_stress_adj    (el_stress_adj.cu:22-104)
//   el_velocity_adj  (el_velocity_adj.cu:22-107)
//   add_source, recording, res_injection, source_grad (utilities.cu:506-593)
//   from_bnd / to_bnd boundary strips (utilities.cu:361-424, Boundary.cu:5-102)
//   cuda_window (both overloads), gpuMinus, cuda_cal_objective (utilities.cu:154-205, 653-747)
//   media set-up aveMuInit / aveBycInit / velInit (utilities.cu:109-152, Model.cu:15-93)
//   cpmlInit (utilities.cu:242-358, Cpml.cu:7-117), compCourantNumber (utilities.cu:225-240)
// Where the reference promotes an expression to double (a `2.0`, `1e6` or
// `3.0` literal), the oracle does too. The reference's atomicAdd scatter of
// the mu and rho kernels is restated as the same per-cell contributions summed
// in a fixed order. Build with -ffp-contract=off so x86 and Arm agree.
//
// Parsing of the parameter / survey JSON files (Parameter.cpp, Src_Rec.cu) is
// restated in oracle/oracle.py, which hands the parsed geometry to this file.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// The reference promotes some products of its time loop to double (a double
// literal 2.0, MEGA or RSXXZZ in a float expression). prom_t is that type;
// building with -DORACLE_FP32 makes it float, which gives the same algorithm
// with FP32 arithmetic only: the tests use it to measure how far FP32 rounding
// alone moves a result from the reference's (the "FP32 floor" of a case).
#ifdef ORACLE_FP32
typedef float prom_t;
#else
typedef double prom_t;
#endif
constexpr double kPI = 3.141592653589793238462643383279502884197169;  // utilities.h:15
constexpr prom_t kMEGA = 1e6;                                          // utilities.h:16
constexpr prom_t kRSXXZZ = 3.0;                                        // utilities.h:21
constexpr prom_t kTwo = 2.0;
constexpr int kLayerStore = 5;                                         // Boundary.cu:24

struct Grid {
  int nz, nx, nPml, nPad, nSteps;
  float dz, dx, dt;
  size_t cells() const { return static_cast<size_t>(nz) * nx; }
  size_t at(int z, int x) const { return static_cast<size_t>(x) * nz + z; }
};

struct Cpml {
  std::vector<float> K_z, a_z, b_z, K_z_half, a_z_half, b_z_half;
  std::vector<float> K_x, a_x, b_x, K_x_half, a_x_half, b_x_half;
};

// cpmlInit, utilities.cu:242-358 (CpAve forced to 3000 at :259).
void cpml_profile(std::vector<float>& K, std::vector<float>& a, std::vector<float>& b, std::vector<float>& K_half,
                  std::vector<float>& a_half, std::vector<float>& b_half, int N, int nPml, float dh, float f0,
                  float dt) {
  const float Rcoef = 0.0008f;
  const float K_MAX_PML = 2.0f;
  const float ALPHA_MAX_PML = static_cast<float>(2.0 * kPI * (f0 / 2.0));
  const float NPOWER = 8.0f;
  const float c1 = 0.25f, c2 = 0.75f, c3 = 0.0f;
  const float thickness_PML = nPml * dh;
  const float CpAve = 3000.0f;
  const float d0_h = static_cast<float>(-(NPOWER + 1) * CpAve * std::log(Rcoef) / (2.0 * thickness_PML));
  std::vector<float> damp(N, 0.0f), damp_half(N, 0.0f), alpha(N, 0.0f), alpha_half(N, 0.0f);
  K.assign(N, 1.0f);
  K_half.assign(N, 1.0f);
  a.assign(N, 0.0f);
  a_half.assign(N, 0.0f);
  b.assign(N, 0.0f);
  b_half.assign(N, 0.0f);
  auto damping = [&](float xn) {
    return d0_h * (c1 * xn + c2 * std::pow(xn, NPOWER) + c3 * std::pow(xn, 2 * NPOWER));
  };
  for (int i = 0; i < N; ++i) {
    float depth = (nPml - i) * dh;  // left edge, integer points
    if (depth >= 0.0f) {
      const float xn = depth / thickness_PML;
      damp[i] = damping(xn);
      K[i] = static_cast<float>(1.0 + (K_MAX_PML - 1.0) * std::pow(xn, NPOWER));
      alpha[i] = static_cast<float>(ALPHA_MAX_PML * (1.0 - xn));
    }
    depth = static_cast<float>((nPml - i - 0.5) * dh);  // left edge, half points
    if (depth >= 0.0f) {
      const float xn = depth / thickness_PML;
      damp_half[i] = damping(xn);
      K_half[i] = static_cast<float>(1.0 + (K_MAX_PML - 1.0) * std::pow(xn, NPOWER));
      alpha_half[i] = static_cast<float>(ALPHA_MAX_PML * (1.0 - xn));
    }
    depth = (nPml - N + i) * dh;  // right edge, integer points
    if (depth >= 0.0f) {
      const float xn = depth / thickness_PML;
      damp[i] = damping(xn);
      K[i] = static_cast<float>(1.0 + (K_MAX_PML - 1.0) * std::pow(xn, NPOWER));
      alpha[i] = static_cast<float>(ALPHA_MAX_PML * (1.0 - xn));
    }
    depth = static_cast<float>((nPml - N + i + 0.5) * dh);  // right edge, half points
    if (depth >= 0.0f) {
      const float xn = depth / thickness_PML;
      damp_half[i] = damping(xn);
      K_half[i] = static_cast<float>(1.0 + (K_MAX_PML - 1.0) * std::pow(xn, NPOWER));
      alpha_half[i] = static_cast<float>(ALPHA_MAX_PML * (1.0 - xn));
    }
    if (alpha[i] < 0.0f) alpha[i] = 0.0f;
    if (alpha_half[i] < 0.0f) alpha_half[i] = 0.0f;
    b[i] = std::exp(-(damp[i] / K[i] + alpha[i]) * dt);
    b_half[i] = std::exp(-(damp_half[i] / K_half[i] + alpha_half[i]) * dt);
    if (std::fabs(damp[i]) > 1.0e-6)
      a[i] = static_cast<float>(damp[i] * (b[i] - 1.0) / (K[i] * (damp[i] + K[i] * alpha[i])));
    if (std::fabs(damp_half[i]) > 1.0e-6)
      a_half[i] = static_cast<float>(damp_half[i] * (b_half[i] - 1.0) /
                                     (K_half[i] * (damp_half[i] + K_half[i] * alpha_half[i])));
  }
}

struct Media {
  std::vector<float> lam, mu, den, aveMu, bycA, bycB;
};

struct Fields {
  std::vector<float> vz, vx, szz, sxx, sxz;
  std::vector<float> vz_a, vx_a, szz_a, sxx_a, sxz_a;
  std::vector<float> m_dvz_dz, m_dvz_dx, m_dvx_dz, m_dvx_dx;
  std::vector<float> m_dszz_dz, m_dsxx_dx, m_dsxz_dz, m_dsxz_dx;
  void alloc(size_t n) {
    for (auto* f : {&vz, &vx, &szz, &sxx, &sxz, &vz_a, &vx_a, &szz_a, &sxx_a, &sxz_a, &m_dvz_dz, &m_dvz_dx, &m_dvx_dz,
                    &m_dvx_dx, &m_dszz_dz, &m_dsxx_dx, &m_dsxz_dz, &m_dsxz_dx})
      f->assign(n, 0.0f);
  }
};

const float C1 = static_cast<float>(9.0 / 8.0);   // el_stress.cu:42
const float C2 = static_cast<float>(1.0 / 24.0);  // el_stress.cu:43

// ---------------------------------------------------------------------------
// el_stress, isFor = true (el_stress.cu:50-88).
void stress_forward(const Grid& g, const Media& m, const Cpml& c, Fields& f) {
  const int nz = g.nz, nx = g.nx, nPml = g.nPml, nPad = g.nPad;
  const float dz = g.dz, dx = g.dx, dt = g.dt;
#pragma omp parallel for schedule(static)
  for (int x = 2; x <= nx - 3; ++x) {
    for (int z = 2; z <= nz - nPad - 3; ++z) {
      const size_t i = g.at(z, x);
      const float* vz = f.vz.data();
      const float* vx = f.vx.data();
      float dvz_dz = (C1 * (vz[i] - vz[i - 1]) - C2 * (vz[i + 1] - vz[i - 2])) / dz;
      float dvx_dx = (C1 * (vx[i] - vx[i - nz]) - C2 * (vx[i + nz] - vx[i - 2 * nz])) / dx;
      const bool zpml = (z < nPml) || (z > nz - nPml - nPad - 1);
      const bool xpml = (x < nPml) || (x > nx - nPml - 1);
      if (zpml) {
        f.m_dvz_dz[i] = c.b_z[z] * f.m_dvz_dz[i] + c.a_z[z] * dvz_dz;
        dvz_dz = dvz_dz / c.K_z[z] + f.m_dvz_dz[i];
      }
      if (xpml) {
        f.m_dvx_dx[i] = c.b_x[x] * f.m_dvx_dx[i] + c.a_x[x] * dvx_dx;
        dvx_dx = dvx_dx / c.K_x[x] + f.m_dvx_dx[i];
      }
      const float lam = m.lam[i], mu = m.mu[i];
      f.szz[i] = static_cast<float>(f.szz[i] + ((lam + kTwo * mu) * dvz_dz + lam * dvx_dx) * dt);
      f.sxx[i] = static_cast<float>(f.sxx[i] + (lam * dvz_dz + (lam + kTwo * mu) * dvx_dx) * dt);
      float dvx_dz = (C1 * (vx[i + 1] - vx[i]) - C2 * (vx[i + 2] - vx[i - 1])) / dz;
      float dvz_dx = (C1 * (vz[i + nz] - vz[i]) - C2 * (vz[i + 2 * nz] - vz[i - nz])) / dx;
      if (zpml) {
        f.m_dvx_dz[i] = c.b_z_half[z] * f.m_dvx_dz[i] + c.a_z_half[z] * dvx_dz;
        dvx_dz = dvx_dz / c.K_z_half[z] + f.m_dvx_dz[i];
      }
      if (xpml) {
        f.m_dvz_dx[i] = c.b_x_half[x] * f.m_dvz_dx[i] + c.a_x_half[x] * dvz_dx;
        dvz_dx = dvz_dx / c.K_x_half[x] + f.m_dvz_dx[i];
      }
      f.sxz[i] = f.sxz[i] + m.aveMu[i] * (dvx_dz + dvz_dx) * dt;
    }
  }
}

// el_velocity, isFor = true (el_velocity.cu:45-82). The x-PML test is
// `x > nx - nPml`, one cell narrower than el_stress's (el_velocity.cu:56,71).
void velocity_forward(const Grid& g, const Media& m, const Cpml& c, Fields& f) {
  const int nz = g.nz, nx = g.nx, nPml = g.nPml, nPad = g.nPad;
  const float dz = g.dz, dx = g.dx, dt = g.dt;
#pragma omp parallel for schedule(static)
  for (int x = 2; x <= nx - 3; ++x) {
    for (int z = 2; z <= nz - nPad - 3; ++z) {
      const size_t i = g.at(z, x);
      const float* szz = f.szz.data();
      const float* sxx = f.sxx.data();
      const float* sxz = f.sxz.data();
      float dszz_dz = (C1 * (szz[i + 1] - szz[i]) - C2 * (szz[i + 2] - szz[i - 1])) / dz;
      float dsxz_dx = (C1 * (sxz[i] - sxz[i - nz]) - C2 * (sxz[i + nz] - sxz[i - 2 * nz])) / dx;
      const bool zpml = (z < nPml) || (z > nz - nPml - nPad - 1);
      const bool xpml = (x < nPml) || (x > nx - nPml);
      if (zpml) {
        f.m_dszz_dz[i] = c.b_z_half[z] * f.m_dszz_dz[i] + c.a_z_half[z] * dszz_dz;
        dszz_dz = dszz_dz / c.K_z_half[z] + f.m_dszz_dz[i];
      }
      if (xpml) {
        f.m_dsxz_dx[i] = c.b_x[x] * f.m_dsxz_dx[i] + c.a_x[x] * dsxz_dx;
        dsxz_dx = dsxz_dx / c.K_x[x] + f.m_dsxz_dx[i];
      }
      f.vz[i] += (dszz_dz + dsxz_dx) * m.bycA[i] * dt;
      float dsxz_dz = (C1 * (sxz[i] - sxz[i - 1]) - C2 * (sxz[i + 1] - sxz[i - 2])) / dz;
      float dsxx_dx = (C1 * (sxx[i + nz] - sxx[i]) - C2 * (sxx[i + 2 * nz] - sxx[i - nz])) / dx;
      if (zpml) {
        f.m_dsxz_dz[i] = c.b_z[z] * f.m_dsxz_dz[i] + c.a_z[z] * dsxz_dz;
        dsxz_dz = dsxz_dz / c.K_z[z] + f.m_dsxz_dz[i];
      }
      if (xpml) {
        f.m_dsxx_dx[i] = c.b_x_half[x] * f.m_dsxx_dx[i] + c.a_x_half[x] * dsxx_dx;
        dsxx_dx = dsxx_dx / c.K_x_half[x] + f.m_dsxx_dx[i];
      }
      f.vx[i] += (dsxz_dz + dsxx_dx) * m.bycB[i] * dt;
    }
  }
}

// el_velocity, isFor = false (el_velocity.cu:84-117): reverse reconstruction of
// v in the interior and the density kernel through the buoyancy averages.
// The reference scatters with atomicAdd; here each cell's two contributions are
// stored and gathered afterwards, including the always-true guard of
// el_velocity.cu:109 that also feeds column nx - nPml.
void velocity_reverse(const Grid& g, const Media& m, Fields& f, std::vector<float>& gDen, std::vector<float>& tA,
                      std::vector<float>& tB) {
  const int nz = g.nz, nx = g.nx, nPml = g.nPml, nPad = g.nPad;
  const float dz = g.dz, dx = g.dx, dt = g.dt;
  const int z0 = nPml, z1 = nz - nPad - 1 - nPml, x0 = nPml, x1 = nx - 1 - nPml;
#pragma omp parallel for schedule(static)
  for (int x = x0; x <= x1; ++x) {
    for (int z = z0; z <= z1; ++z) {
      const size_t i = g.at(z, x);
      const float* szz = f.szz.data();
      const float* sxx = f.sxx.data();
      const float* sxz = f.sxz.data();
      const float dszz_dz = (C1 * (szz[i + 1] - szz[i]) - C2 * (szz[i + 2] - szz[i - 1])) / dz;
      const float dsxz_dx = (C1 * (sxz[i] - sxz[i - nz]) - C2 * (sxz[i + nz] - sxz[i - 2 * nz])) / dx;
      f.vz[i] -= (dszz_dz + dsxz_dx) * m.bycA[i] * dt;
      const float dsxz_dz = (C1 * (sxz[i] - sxz[i - 1]) - C2 * (sxz[i + 1] - sxz[i - 2])) / dz;
      const float dsxx_dx = (C1 * (sxx[i + nz] - sxx[i]) - C2 * (sxx[i + 2 * nz] - sxx[i - nz])) / dx;
      f.vx[i] -= (dsxz_dz + dsxx_dx) * m.bycB[i] * dt;
      const float ba = m.bycA[i], bb = m.bycB[i];
      tA[i] = static_cast<float>(-f.vz_a[i] * (dszz_dz + dsxz_dx) * dt * (-(static_cast<prom_t>(ba) * ba) / kTwo));
      tB[i] = static_cast<float>(-f.vx_a[i] * (dsxz_dz + dsxx_dx) * dt * (-(static_cast<prom_t>(bb) * bb) / kTwo));
    }
  }
  // Gather: rho(z,x) receives A and B of (z,x), A of (z-1,x) when z <= z1, and
  // B of (z,x-1) for every interior (z,x-1).
#pragma omp parallel for schedule(static)
  for (int x = x0; x <= x1 + 1; ++x) {
    for (int z = z0; z <= z1; ++z) {
      const size_t i = g.at(z, x);
      float acc = gDen[i];
      if (x <= x1) {
        acc += tA[i];
        acc += tB[i];
        if (z - 1 >= z0) acc += tA[i - 1];
      }
      if (x - 1 >= x0) acc += tB[i - nz];
      gDen[i] = acc;
    }
  }
}

// el_stress, isFor = false (el_stress.cu:90-131): reverse reconstruction of the
// stresses in the interior plus the lambda and mu kernels. The mu kernel's
// harmonic-average chain rule (el_stress.cu:113-124) scatters to the 2x2 block;
// restated as stored per-cell scales gathered afterwards with the same guards.
void stress_reverse(const Grid& g, const Media& m, Fields& f, std::vector<float>& gLam, std::vector<float>& gMu,
                    std::vector<float>& tS) {
  const int nz = g.nz, nx = g.nx, nPml = g.nPml, nPad = g.nPad;
  const float dz = g.dz, dx = g.dx, dt = g.dt;
  const int z0 = nPml, z1 = nz - nPad - 1 - nPml, x0 = nPml, x1 = nx - 1 - nPml;
#pragma omp parallel for schedule(static)
  for (int x = x0; x <= x1; ++x) {
    for (int z = z0; z <= z1; ++z) {
      const size_t i = g.at(z, x);
      const float* vz = f.vz.data();
      const float* vx = f.vx.data();
      const float dvz_dz = (C1 * (vz[i] - vz[i - 1]) - C2 * (vz[i + 1] - vz[i - 2])) / dz;
      const float dvx_dx = (C1 * (vx[i] - vx[i - nz]) - C2 * (vx[i + nz] - vx[i - 2 * nz])) / dx;
      const float lam = m.lam[i], mu = m.mu[i];
      f.szz[i] = static_cast<float>(f.szz[i] - ((lam + kTwo * mu) * dvz_dz + lam * dvx_dx) * dt);
      f.sxx[i] = static_cast<float>(f.sxx[i] - (lam * dvz_dz + (lam + kTwo * mu) * dvx_dx) * dt);
      const float dvx_dz = (C1 * (vx[i + 1] - vx[i]) - C2 * (vx[i + 2] - vx[i - 1])) / dz;
      const float dvz_dx = (C1 * (vz[i + nz] - vz[i]) - C2 * (vz[i + 2 * nz] - vz[i - nz])) / dx;
      f.sxz[i] -= m.aveMu[i] * (dvx_dz + dvz_dx) * dt;
      gLam[i] = static_cast<float>(gLam[i] + -(f.szz_a[i] + f.sxx_a[i]) * (dvz_dz + dvx_dx) * dt * kMEGA);
      gMu[i] = static_cast<float>(gMu[i] + (-kTwo * f.szz_a[i] * dvz_dz * dt - kTwo * f.sxx_a[i] * dvx_dx * dt) * kMEGA);
      float scale = 0.0f;
      if (m.aveMu[i] != 0.0f) {
        const prom_t one = 1.0;
        const prom_t inv_sum = one / m.mu[i] + one / m.mu[i + 1] + one / m.mu[i + nz] + one / m.mu[i + nz + 1];
        scale = static_cast<float>(-f.sxz_a[i] * (dvx_dz + dvz_dx) * dt * m.aveMu[i] / inv_sum * kMEGA);
      }
      tS[i] = scale;
    }
  }
  // Gather of the 2x2 scatter: mu(z,x) gets w(z,x) * scale of (z,x), (z-1,x)
  // [if z <= z1], (z,x-1) [always], (z-1,x-1) [if z <= z1 and x <= x1];
  // w = 1 / mu(z,x)^2.
#pragma omp parallel for schedule(static)
  for (int x = x0; x <= x1 + 1; ++x) {
    for (int z = z0; z <= z1 + 1; ++z) {
      const size_t i = g.at(z, x);
      const prom_t w = prom_t(1.0) / (static_cast<prom_t>(m.mu[i]) * m.mu[i]);
      float acc = gMu[i];
      bool any = false;
      if (x <= x1 && z <= z1 && m.aveMu[i] != 0.0f) {
        acc += static_cast<float>(w * tS[i]);
        any = true;
      }
      if (z - 1 >= z0 && z <= z1 && x <= x1 && m.aveMu[i - 1] != 0.0f) {
        acc += static_cast<float>(w * tS[i - 1]);
        any = true;
      }
      if (x - 1 >= x0 && z <= z1 && m.aveMu[i - nz] != 0.0f) {
        acc += static_cast<float>(w * tS[i - nz]);
        any = true;
      }
      if (x - 1 >= x0 && z - 1 >= z0 && z <= z1 && x <= x1 && m.aveMu[i - nz - 1] != 0.0f) {
        acc += static_cast<float>(w * tS[i - nz - 1]);
        any = true;
      }
      if (any) gMu[i] = acc;
    }
  }
}

// el_velocity_adj (el_velocity_adj.cu:22-107): adjoint of the velocity/CPML step.
void velocity_adjoint(const Grid& g, const Media& m, const Cpml& c, Fields& f) {
  const int nz = g.nz, nx = g.nx, nPml = g.nPml, nPad = g.nPad;
  const float dz = g.dz, dx = g.dx, dt = g.dt;
#pragma omp parallel for schedule(static)
  for (int x = 2; x <= nx - 3; ++x) {
    for (int z = 2; z <= nz - nPad - 3; ++z) {
      const size_t i = g.at(z, x);
      const float lam = m.lam[i], mu = m.mu[i];
      const float* mvxx = f.m_dvx_dx.data();
      const float* mvxz = f.m_dvx_dz.data();
      const float* mvzz = f.m_dvz_dz.data();
      const float* mvzx = f.m_dvz_dx.data();
      const float* szz = f.szz_a.data();
      const float* sxx = f.sxx_a.data();
      const float* sxz = f.sxz_a.data();
      const bool zpml = (z < nPml) || (z > nz - nPml - nPad - 1);
      const bool xpml = (x < nPml) || (x > nx - nPml - 1);
      const float dpsixx_dx = (-C1 * (mvxx[i + nz] - mvxx[i]) + C2 * (mvxx[i + 2 * nz] - mvxx[i - nz])) / dx;
      const float dszz_dx = (-C1 * (szz[i + nz] - szz[i]) + C2 * (szz[i + 2 * nz] - szz[i - nz])) / dx;
      const float dsxx_dx = (-C1 * (sxx[i + nz] - sxx[i]) + C2 * (sxx[i + 2 * nz] - sxx[i - nz])) / dx;
      const float dpsixz_dz = (-C1 * (mvxz[i] - mvxz[i - 1]) + C2 * (mvxz[i + 1] - mvxz[i - 2])) / dz;
      const float dsxz_dz = (-C1 * (sxz[i] - sxz[i - 1]) + C2 * (sxz[i + 1] - sxz[i - 2])) / dz;
      {
        const float t1 = c.a_x[x] * dpsixx_dx + lam * dszz_dx / c.K_x[x] * dt;
        const prom_t t = t1 + (lam + kTwo * mu) * dsxx_dx / c.K_x[x] * dt + c.a_z_half[z] * dpsixz_dz +
                         m.aveMu[i] / c.K_z_half[z] * dsxz_dz * dt;
        f.vx_a[i] = static_cast<float>(f.vx_a[i] + t);
      }
      if (xpml) f.m_dsxx_dx[i] = c.b_x_half[x] * f.m_dsxx_dx[i] + m.bycB[i] * f.vx_a[i] * dt;
      if (zpml) f.m_dsxz_dz[i] = c.b_z[z] * f.m_dsxz_dz[i] + m.bycB[i] * f.vx_a[i] * dt;
      const float dpsizz_dz = (-C1 * (mvzz[i + 1] - mvzz[i]) + C2 * (mvzz[i + 2] - mvzz[i - 1])) / dz;
      const float dszz_dz = (-C1 * (szz[i + 1] - szz[i]) + C2 * (szz[i + 2] - szz[i - 1])) / dz;
      const float dsxx_dz = (-C1 * (sxx[i + 1] - sxx[i]) + C2 * (sxx[i + 2] - sxx[i - 1])) / dz;
      const float dpsizx_dx = (-C1 * (mvzx[i] - mvzx[i - nz]) + C2 * (mvzx[i + nz] - mvzx[i - 2 * nz])) / dx;
      const float dsxz_dx = (-C1 * (sxz[i] - sxz[i - nz]) + C2 * (sxz[i + nz] - sxz[i - 2 * nz])) / dx;
      {
        const prom_t t = c.a_z[z] * dpsizz_dz + (lam + kTwo * mu) * dszz_dz / c.K_z[z] * dt +
                         lam * dsxx_dz / c.K_z[z] * dt + c.a_x_half[x] * dpsizx_dx +
                         m.aveMu[i] / c.K_x_half[x] * dsxz_dx * dt;
        f.vz_a[i] = static_cast<float>(f.vz_a[i] + t);
      }
      if (xpml) f.m_dsxz_dx[i] = c.b_x[x] * f.m_dsxz_dx[i] + m.bycA[i] * f.vz_a[i] * dt;
      if (zpml) f.m_dszz_dz[i] = c.b_z_half[z] * f.m_dszz_dz[i] + m.bycA[i] * f.vz_a[i] * dt;
    }
  }
}

// el_stress_adj (el_stress_adj.cu:22-104): adjoint of the stress/CPML step; the
// four adjoint memory variables are updated over the whole stencil domain.
void stress_adjoint(const Grid& g, const Media& m, const Cpml& c, Fields& f) {
  const int nz = g.nz, nx = g.nx, nPad = g.nPad;
  const float dz = g.dz, dx = g.dx, dt = g.dt;
#pragma omp parallel for schedule(static)
  for (int x = 2; x <= nx - 3; ++x) {
    for (int z = 2; z <= nz - nPad - 3; ++z) {
      const size_t i = g.at(z, x);
      const float lam = m.lam[i], mu = m.mu[i];
      const float* msxzx = f.m_dsxz_dx.data();
      const float* msxzz = f.m_dsxz_dz.data();
      const float* msxxx = f.m_dsxx_dx.data();
      const float* mszzz = f.m_dszz_dz.data();
      const float* vz = f.vz_a.data();
      const float* vx = f.vx_a.data();
      const float dphi_xz_x_dx = (-C1 * (msxzx[i + nz] - msxzx[i]) + C2 * (msxzx[i + 2 * nz] - msxzx[i - nz])) / dx;
      const float dvz_dx = (-C1 * (vz[i + nz] - vz[i]) + C2 * (vz[i + 2 * nz] - vz[i - nz])) / dx;
      const float dphi_xz_z_dz = (-C1 * (msxzz[i + 1] - msxzz[i]) + C2 * (msxzz[i + 2] - msxzz[i - 1])) / dz;
      const float dvx_dz = (-C1 * (vx[i + 1] - vx[i]) + C2 * (vx[i + 2] - vx[i - 1])) / dz;
      f.sxz_a[i] += c.a_x[x] * dphi_xz_x_dx + dvz_dx / c.K_x[x] * m.bycA[i] * dt + c.a_z[z] * dphi_xz_z_dz +
                    dvx_dz / c.K_z[z] * m.bycB[i] * dt;
      f.m_dvz_dx[i] = c.b_x_half[x] * f.m_dvz_dx[i] + f.sxz_a[i] * m.aveMu[i] * dt;
      f.m_dvx_dz[i] = c.b_z_half[z] * f.m_dvx_dz[i] + f.sxz_a[i] * m.aveMu[i] * dt;
      const float dphi_xx_x_dx = (-C1 * (msxxx[i] - msxxx[i - nz]) + C2 * (msxxx[i + nz] - msxxx[i - 2 * nz])) / dx;
      const float dvx_dx = (-C1 * (vx[i] - vx[i - nz]) + C2 * (vx[i + nz] - vx[i - 2 * nz])) / dx;
      const float dphi_zz_z_dz = (-C1 * (mszzz[i] - mszzz[i - 1]) + C2 * (mszzz[i + 1] - mszzz[i - 2])) / dz;
      const float dvz_dz = (-C1 * (vz[i] - vz[i - 1]) + C2 * (vz[i + 1] - vz[i - 2])) / dz;
      f.sxx_a[i] += c.a_x_half[x] * dphi_xx_x_dx + m.bycB[i] * dvx_dx / c.K_x_half[x] * dt;
      f.szz_a[i] += c.a_z_half[z] * dphi_zz_z_dz + m.bycA[i] * dvz_dz / c.K_z_half[z] * dt;
      f.m_dvx_dx[i] = static_cast<float>(c.b_x[x] * f.m_dvx_dx[i] + lam * f.szz_a[i] * dt +
                                         (lam + kTwo * mu) * f.sxx_a[i] * dt);
      f.m_dvz_dz[i] = static_cast<float>(c.b_z[z] * f.m_dvz_dz[i] + (lam + kTwo * mu) * f.szz_a[i] * dt +
                                         lam * f.sxx_a[i] * dt);
    }
  }
}

// add_source (utilities.cu:521-555) with the 9x9 Gaussian of src_rec_gauss_amp
// (utilities.cu:506-519); isFor selects += or -=.
void add_source(const Grid& g, Fields& f, float amp, int zs, int xs, bool isFor, const float* gauss) {
  const float scale = static_cast<float>(std::pow(1500.0, 2));
  for (int gx = 0; gx < 9; ++gx)
    for (int gz = 0; gz < 9; ++gz) {
      const size_t i = g.at(zs + gz - 4, xs + gx - 4);
      const float ga = gauss[gz + gx * 9];
      const float t = scale * amp * g.dt * ga;
      const prom_t t3 = kRSXXZZ * scale * amp * g.dt * ga;
      if (isFor) {
        f.szz[i] += t;
        f.sxx[i] = static_cast<float>(f.sxx[i] + t3);
      } else {
        f.szz[i] -= t;
        f.sxx[i] = static_cast<float>(f.sxx[i] - t3);
      }
    }
}

// Boundary strip index map (utilities.cu:361-424): element k of the per-step
// store lives at field cell strip_cell[k].
std::vector<size_t> strip_cells(const Grid& g) {
  const int nzB = g.nz - 2 * g.nPml - g.nPad + 4, nxB = g.nx - 2 * g.nPml + 4, L = kLayerStore;
  const int len = 2 * (L * nzB + L * nxB);
  std::vector<size_t> cells(len);
  for (int k = 0; k < len; ++k) {
    int z, x;
    if (k < L * nzB) {
      const int j = k / nzB, r = k - j * nzB;
      z = r + g.nPml - 2;
      x = j + g.nPml - 2;
    } else if (k < 2 * L * nzB) {
      const int kk = k - L * nzB, j = kk / nzB, r = kk - j * nzB;
      z = r + g.nPml - 2;
      x = g.nx - g.nPml - j - 1 + 2;
    } else if (k < L * (2 * nzB + nxB)) {
      const int kk = k - 2 * L * nzB, r = kk / nxB, j = kk - r * nxB;
      z = r + g.nPml - 2;
      x = j + g.nPml - 2;
    } else {
      const int kk = k - L * (2 * nzB + nxB), r = kk / nxB, j = kk - r * nxB;
      z = g.nz - g.nPml - g.nPad - r - 1 + 2;
      x = j + g.nPml - 2;
    }
    cells[k] = g.at(z, x);
  }
  return cells;
}

// cuda_window without per-trace windows (utilities.cu:707-747).
bool taper(float* data, int nt, int nrec, float dt, float ratio) {
  const float t0 = 0.0f, t3 = nt * dt, offset = nt * dt * ratio;
  if (2.0 * offset >= t3 - t0) return false;
  const float t1 = t0 + offset, t2 = t3 - offset;
  std::vector<float> w(nt);
  for (int it = 0; it < nt; ++it) {
    const float t = it * dt;
    float amp;
    if (t >= t0 && t < t1)
      amp = static_cast<float>(std::sin(kPI / 2.0 * (t - t0) / (t1 - t0)));
    else if (t >= t1 && t < t2)
      amp = 1.0f;
    else if (t >= t2 && t < t3)
      amp = static_cast<float>(std::cos(kPI / 2.0 * (t - t2) / (t3 - t2)));
    else
      amp = 0.0f;
    w[it] = amp * amp;
  }
  for (int r = 0; r < nrec; ++r)
    for (int it = 0; it < nt; ++it) data[static_cast<size_t>(r) * nt + it] *= w[it];
  return true;
}

// cuda_window with per-trace windows and weights (utilities.cu:653-705).
void taper_windowed(float* data, int nt, int nrec, float dt, float ratio, const float* ws, const float* we,
                    const float* wt) {
  if (ratio > 0.5f) return;
  for (int r = 0; r < nrec; ++r) {
    float t0 = ws[r], t3 = we[r];
    const float t_max = nt * dt;
    if (t0 < 0.0f) t0 = 0.0f;
    if (t0 > t_max) t0 = t_max;
    if (t3 < 0.0f) t3 = 0.0f;
    if (t3 > t_max) t3 = t_max;
    const float offset = (t3 - t0) * ratio;
    if (offset <= 0.0f) continue;
    const float t1 = t0 + offset, t2 = t3 - offset;
    for (int it = 0; it < nt; ++it) {
      const float t = it * dt;
      float amp;
      if (t >= t0 && t < t1)
        amp = static_cast<float>(std::sin(kPI / 2.0 * (t - t0) / (t1 - t0)));
      else if (t >= t1 && t < t2)
        amp = 1.0f;
      else if (t >= t2 && t < t3)
        amp = static_cast<float>(std::cos(kPI / 2.0 * (t - t2) / (t3 - t2)));
      else
        amp = 0.0f;
      data[static_cast<size_t>(r) * nt + it] *= amp * amp * wt[r];
    }
  }
}

// cuda_cal_objective (utilities.cu:169-205): 512 strided partial sums, then a
// shared-memory tree; the order of additions is kept.
float objective(const float* err, int ng) {
  const int B = 512;
  float s[B];
  for (int tid = 0; tid < B; ++tid) {
    float acc = 0.0f;
    for (int k = 0; k < (ng + B - 1) / B; ++k) {
      const int id = k * B + tid;
      const float a = (id < ng) ? err[id] : 0.0f;
      acc += a * a;
    }
    s[tid] = acc;
  }
  for (int h = B / 2; h >= 1; h /= 2)
    for (int tid = 0; tid < h; ++tid) s[tid] += s[tid + h];
  return s[0];
}

}  // namespace

extern "C" {

struct oracle_para {
  int nz, nx, nSteps, nPml, nPad;
  float dz, dx, dt, f0;
  int if_win;
  int if_filter;     // "filter" key present (Parameter.cpp:155-167)
  float filter[4];   // band-pass corner frequencies f0 < f1 <= f2 < f3 [Hz]
  int if_src_update; // "if_src_update" (Parameter.cpp:170-174)
};

struct oracle_shot {
  int z_src, x_src;  // survey-file indices (nPml is added here, Src_Rec.cu:86,90)
  int nrec;
  const int* z_rec;  // survey-file indices (nPml is added here, Src_Rec.cu:105,113)
  const int* x_rec;
  const float* win_start;  // per receiver, only when if_win
  const float* win_end;
  const float* weights;
};

enum { ORACLE_OK = 0, ORACLE_BAD_ARG = 1, ORACLE_COURANT = 3 };

// Restates cufd (libCUFD.cu:34-580) for one call. calc_id 0: misfit,
// 1: gradients, 2: observed gathers. obs[i] is shot i's observed data
// [nrec][nSteps] (calc 0/1). syn_out[i] (optional) receives shot i's gathers as
// the reference keeps them: raw for calc 2, after the taper for calc 0/1.
// res_out[i] (optional) receives the adjoint source (tapered residual).
// Band-pass of bp_filter1d (utilities.cu:872-923, cuda_bp_filter1d :596-626)
// on each of nrec traces of nt samples: the trace zero-padded to 2 nt, its
// spectrum times amp(f)^2 with amp the sin / 1 / cos band-pass of the corner
// frequencies (bin frequencies k / (2 nt dt) in float, as the kernel computes
// them), back to time, cropped to nt and scaled by 1 / (2 nt). Restated as
// the equivalent circular convolution with the real, even impulse response
// h[m] = (a_0 + 2 sum_{k=1}^{nt-1} a_k cos(pi k m / nt) + a_nt cos(pi m)) / (2 nt),
// a_k = amp(f_k)^2, accumulated in double.
static void bp_filter(float* data, int nt, int nrec, float dt, const float* fc) {
  const int n2 = 2 * nt;
  const float df = static_cast<float>(1.0 / dt / n2);
  std::vector<double> a(nt + 1);
  const double kPi = 3.14159265358979323846;
  for (int k = 0; k <= nt; ++k) {
    const float freq = k * df;
    float amp;
    if (freq >= fc[0] && freq < fc[1])
      amp = static_cast<float>(std::sin(kPi / 2.0 * (freq - fc[0]) / (fc[1] - fc[0])));
    else if (freq >= fc[1] && freq < fc[2])
      amp = 1.0f;
    else if (freq >= fc[2] && freq < fc[3])
      amp = static_cast<float>(std::cos(kPi / 2.0 * (freq - fc[2]) / (fc[3] - fc[2])));
    else
      amp = 0.0f;
    a[k] = static_cast<double>(amp * amp);
  }
  std::vector<double> h(n2);
  for (int m = 0; m < n2; ++m) {
    double s = a[0] + a[nt] * ((m & 1) ? -1.0 : 1.0);
    for (int k = 1; k < nt; ++k) s += 2.0 * a[k] * std::cos(kPi * k * m / nt);
    h[m] = s / n2;
  }
  std::vector<float> y(nt);
  for (int r = 0; r < nrec; ++r) {
    float* x = data + static_cast<size_t>(r) * nt;
    for (int t = 0; t < nt; ++t) {
      double acc = 0.0;
      for (int s = 0; s < nt; ++s) acc += static_cast<double>(x[s]) * h[(t - s + n2) % n2];
      y[t] = static_cast<float>(acc);
    }
    std::copy(y.begin(), y.end(), x);
  }
}

// Source-wavelet update of one shot (source_update, utilities.cu:927-1035, with
// cuda_spectrum_update :768-840). The observed and synthetic traces o, d
// [nrec][nt] (already tapered / filtered) are zero-padded to M = 2 nt and
// tapered over the padded length (cuda_window, ratio 0.01); their spectra
// O_r, C_r (float, as cuFFT returns them) give per frequency f = 0 .. nt
//   coef[f] = sum_r conj(C_r) O_r / (sum_r |C_r|^2 + 1e-6)   (float).
// The padded, tapered synthetic and the (unpadded-tapered) wavelet become
// IFFT(spectrum * coef) cropped to nt and divided by M: restated as the
// circular convolution with k = IFFT(coef) / M, accumulated in double. d and
// src are replaced; k is returned for the adjoint (src_update_adj).
static std::vector<double> src_update(float* d, const float* o, float* src, int nt, int nrec, float dt) {
  const int M = 2 * nt;
  const double kTwoPi = 6.283185307179586476925286766559;
  std::vector<double> cs(M), sn(M);
  for (int k = 0; k < M; ++k) {
    cs[k] = std::cos(kTwoPi * k / M);
    sn[k] = std::sin(kTwoPi * k / M);
  }
  std::vector<float> op(static_cast<size_t>(nrec) * M, 0.0f), dp(static_cast<size_t>(nrec) * M, 0.0f);
  for (int r = 0; r < nrec; ++r)
    for (int t = 0; t < nt; ++t) {
      op[static_cast<size_t>(r) * M + t] = o[static_cast<size_t>(r) * nt + t];
      dp[static_cast<size_t>(r) * M + t] = d[static_cast<size_t>(r) * nt + t];
    }
  taper(op.data(), M, nrec, dt, 0.01f);
  taper(dp.data(), M, nrec, dt, 0.01f);
  std::vector<double> cre(nt + 1), cim(nt + 1);
  for (int f = 0; f <= nt; ++f) {
    double nre = 0.0, nim = 0.0, den = 0.0;
    for (int r = 0; r < nrec; ++r) {
      double ore = 0.0, oim = 0.0, dre = 0.0, dim = 0.0;
      const float* orow = op.data() + static_cast<size_t>(r) * M;
      const float* drow = dp.data() + static_cast<size_t>(r) * M;
      for (int t = 0; t < nt; ++t) {  // the padded half is zero
        const int k = static_cast<int>((static_cast<long long>(f) * t) % M);
        ore += orow[t] * cs[k];
        oim -= orow[t] * sn[k];
        dre += drow[t] * cs[k];
        dim -= drow[t] * sn[k];
      }
      const double Or = static_cast<float>(ore), Oi = static_cast<float>(oim);
      const double Cr = static_cast<float>(dre), Ci = static_cast<float>(dim);
      nre += Cr * Or + Ci * Oi;
      nim += Cr * Oi - Ci * Or;
      den += Cr * Cr + Ci * Ci;
    }
    const float denf = static_cast<float>(den) + 1e-6f;
    cre[f] = static_cast<float>(static_cast<float>(nre) / static_cast<double>(denf));
    cim[f] = static_cast<float>(static_cast<float>(nim) / static_cast<double>(denf));
  }
  // k[n] = (coef_0 + coef_nt (-1)^n + 2 sum_{f=1}^{nt-1} Re(coef_f e^{2 pi i f n / M})) / M
  std::vector<double> kr(M);
  for (int n = 0; n < M; ++n) {
    double acc = cre[0] + cre[nt] * ((n & 1) ? -1.0 : 1.0);
    for (int f = 1; f < nt; ++f) {
      const int k = static_cast<int>((static_cast<long long>(f) * n) % M);
      acc += 2.0 * (cre[f] * cs[k] - cim[f] * sn[k]);
    }
    kr[n] = acc / M;
  }
  auto conv = [&](const float* x, float* y) {
    for (int t = 0; t < nt; ++t) {
      double acc = 0.0;
      for (int m = 0; m < nt; ++m) acc += static_cast<double>(x[m]) * kr[(t - m + M) % M];
      y[t] = static_cast<float>(acc);
    }
  };
  for (int r = 0; r < nrec; ++r) conv(dp.data() + static_cast<size_t>(r) * M, d + static_cast<size_t>(r) * nt);
  std::vector<float> s0(src, src + nt);
  conv(s0.data(), src);
  return kr;
}

// source_update_adj (utilities.cu:1037-1080): residual traces zero-padded to
// 2 nt, tapered (ratio 0.01), times coef in frequency (not its conjugate), back,
// cropped and divided by 2 nt (amp_ratio is 1, libCUFD.cu:286): the circular
// convolution with the k of src_update.
static void src_update_adj(float* res, int nt, int nrec, float dt, const std::vector<double>& kr) {
  const int M = 2 * nt;
  std::vector<float> rp(M);
  for (int r = 0; r < nrec; ++r) {
    float* x = res + static_cast<size_t>(r) * nt;
    std::fill(rp.begin(), rp.end(), 0.0f);
    std::copy(x, x + nt, rp.begin());
    taper(rp.data(), M, 1, dt, 0.01f);
    for (int t = 0; t < nt; ++t) {
      double acc = 0.0;
      for (int m = 0; m < nt; ++m) acc += static_cast<double>(rp[m]) * kr[(t - m + M) % M];
      x[t] = static_cast<float>(acc);
    }
  }
}

static int cufd_impl(const oracle_para* p, const oracle_shot* shots, int group_size, const int* shot_ids,
                     const double* Lambda, const double* Mu, const double* Den, const double* stf, int calc_id,
                     const float* const* obs, float* const* syn_out, float* const* res_out, double* misfit,
                     double* grad_Lambda, double* grad_Mu, double* grad_Den, double* grad_stf, int nthreads,
                     double* illum, float* const* src_out) {
  if (calc_id < 0 || calc_id > 2 || !p) return ORACLE_BAD_ARG;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
  const bool if_res = (calc_id == 0 || calc_id == 1);  // Parameter.cpp:132-144
  const bool withAdj = (calc_id == 1);
  Grid g{p->nz, p->nx, p->nPml, p->nPad, p->nSteps, p->dz, p->dx, p->dt};
  const int nz = g.nz, nx = g.nx, nSteps = g.nSteps;
  const size_t n = g.cells();

  // Media (libCUFD.cu:67-79, Model.cu:15-93, utilities.cu:109-152).
  Media m;
  m.lam.resize(n);
  m.mu.resize(n);
  m.den.resize(n);
  for (int z = 0; z < nz; ++z)
    for (int x = 0; x < nx; ++x) {
      m.lam[g.at(z, x)] = static_cast<float>(Lambda[static_cast<size_t>(z) * nx + x] * 1e6);
      m.mu[g.at(z, x)] = static_cast<float>(Mu[static_cast<size_t>(z) * nx + x] * 1e6);
      m.den[g.at(z, x)] = static_cast<float>(Den[static_cast<size_t>(z) * nx + x]);
    }
  m.aveMu.assign(n, 0.0f);
  m.bycA.assign(n, static_cast<float>(1.0 / 1000.0));
  m.bycB.assign(n, static_cast<float>(1.0 / 1000.0));
  float cp_max = -1.0f;
  for (size_t i = 0; i < n; ++i) {
    const float cp = static_cast<float>(std::sqrt((m.lam[i] + 2.0 * m.mu[i]) / m.den[i]));
    if (i == 0 || cp > cp_max) cp_max = cp;
  }
  for (int x = 2; x <= nx - 3; ++x)
    for (int z = 2; z <= nz - 3; ++z) {
      const size_t i = g.at(z, x);
      const float a = m.mu[i], b = m.mu[i + 1], c = m.mu[i + nz], d = m.mu[i + nz + 1];
      if (a == 0.0f || b == 0.0f || c == 0.0f || d == 0.0f)
        m.aveMu[i] = 0.0f;
      else
        m.aveMu[i] = static_cast<float>(4.0 / (1.0 / a + 1.0 / b + 1.0 / c + 1.0 / d));
      m.bycA[i] = static_cast<float>(2.0 / (m.den[i + 1] + m.den[i]));
      m.bycB[i] = static_cast<float>(2.0 / (m.den[i + nz] + m.den[i]));
    }
  // compCourantNumber (utilities.cu:225-240); the reference exits, we report.
  {
    const float dh_min = (g.dz < g.dx) ? g.dz : g.dx;
    const float courant = static_cast<float>(cp_max * g.dt * std::sqrt(2.0f) * (1.0 / 24.0 + 9.0 / 8.0) / dh_min);
    if (courant > 1.0f) return ORACLE_COURANT;
  }
  Cpml c;
  cpml_profile(c.K_z, c.a_z, c.b_z, c.K_z_half, c.a_z_half, c.b_z_half, nz - g.nPad, g.nPml, g.dz, p->f0, g.dt);
  cpml_profile(c.K_x, c.a_x, c.b_x, c.K_x_half, c.a_x_half, c.b_x_half, nx, g.nPml, g.dx, p->f0, g.dt);

  float gauss[81];
  for (int gx = 0; gx < 9; ++gx)
    for (int gz = 0; gz < 9; ++gz) {
      const int idz = gz - 4, idx = gx - 4;
      gauss[gz + gx * 9] = std::exp(static_cast<float>(-1000.0 * (std::pow(float(idz), 2.0f) +
                                                                   std::pow(float(idx), 2.0f))));
    }

  std::vector<size_t> strip;
  int len = 0;
  std::vector<float> store;  // 5 fields x nSteps x len
  if (withAdj) {
    strip = strip_cells(g);
    len = static_cast<int>(strip.size());
    store.assign(static_cast<size_t>(5) * nSteps * len, 0.0f);
  }
  std::vector<float> gLam, gMu, gDen, tA, tB, tS;
  if (withAdj) {
    gLam.assign(n, 0.0f);
    gMu.assign(n, 0.0f);
    gDen.assign(n, 0.0f);
    tA.assign(n, 0.0f);
    tB.assign(n, 0.0f);
    tS.assign(n, 0.0f);
  }

  Fields f;
  f.alloc(n);
  float l2 = 0.0f;
  for (int is = 0; is < group_size; ++is) {
    const oracle_shot& sh = shots[is];
    const int zs = sh.z_src + g.nPml, xs = sh.x_src + g.nPml;
    const int nrec = sh.nrec;
    std::vector<size_t> rec(nrec);
    for (int r = 0; r < nrec; ++r) rec[r] = g.at(sh.z_rec[r] + g.nPml, sh.x_rec[r] + g.nPml);
    // Source wavelet: stf row of shot_ids[is], tapered with ratio 0.001 (Src_Rec.cu:133-140).
    std::vector<float> src(nSteps);
    for (int it = 0; it < nSteps; ++it) src[it] = static_cast<float>(stf[static_cast<size_t>(shot_ids[is]) * nSteps + it]);
    taper(src.data(), nSteps, 1, g.dt, 0.001f);

    f.alloc(n);
    std::vector<float> data(static_cast<size_t>(nrec) * nSteps, 0.0f);
    // Forward time loop (libCUFD.cu:202-240).
    for (int it = 0; it <= nSteps - 2; ++it) {
      if (withAdj) {
        const std::vector<float>* fl[5] = {&f.szz, &f.sxz, &f.sxx, &f.vz, &f.vx};
        for (int k = 0; k < 5; ++k) {
          float* dst = store.data() + (static_cast<size_t>(k) * nSteps + it) * len;
          for (int e = 0; e < len; ++e) dst[e] = (*fl[k])[strip[e]];
        }
      }
      stress_forward(g, m, c, f);
      add_source(g, f, src[it], zs, xs, true, gauss);
      velocity_forward(g, m, c, f);
      if (illum)  // source illumination: sum over forward steps of vz^2 + vx^2 (this package's definition)
        for (int z = 0; z < nz; ++z)
          for (int x = 0; x < nx; ++x) {
            const double a = f.vz[g.at(z, x)], b = f.vx[g.at(z, x)];
            illum[static_cast<size_t>(z) * nx + x] += a * a + b * b;
          }
      for (int r = 0; r < nrec; ++r)
        data[static_cast<size_t>(r) * nSteps + it + 1] = static_cast<float>(f.szz[rec[r]] + kRSXXZZ * f.sxx[rec[r]]);
    }
    if (!if_res) {
      if (syn_out && syn_out[is]) std::memcpy(syn_out[is], data.data(), data.size() * sizeof(float));
      continue;
    }
    // Residual and misfit (libCUFD.cu:254-330).
    std::vector<float> o(obs[is], obs[is] + data.size());
    if (p->if_win) {
      taper_windowed(o.data(), nSteps, nrec, g.dt, 0.005f, sh.win_start, sh.win_end, sh.weights);
      taper_windowed(data.data(), nSteps, nrec, g.dt, 0.005f, sh.win_start, sh.win_end, sh.weights);
    } else {
      taper(o.data(), nSteps, nrec, g.dt, 0.005f);
      taper(data.data(), nSteps, nrec, g.dt, 0.005f);
    }
    if (p->if_filter) {  // libCUFD.cu:273-277
      bp_filter(o.data(), nSteps, nrec, g.dt, p->filter);
      bp_filter(data.data(), nSteps, nrec, g.dt, p->filter);
    }
    // Source-wavelet update (libCUFD.cu:279-286): the synthetic and the
    // wavelet change; the reverse reconstruction below subtracts the updated
    // wavelet, as the reference copies it back into the host source it uses
    // there (libCUFD.cu:326-328, 391-394).
    std::vector<double> kr;
    if (p->if_src_update) kr = src_update(data.data(), o.data(), src.data(), nSteps, nrec, g.dt);
    if (src_out && src_out[is]) std::memcpy(src_out[is], src.data(), nSteps * sizeof(float));
    std::vector<float> res(data.size());
    for (int r = 0; r < nrec; ++r)
      for (int it = 0; it < nSteps; ++it) {
        const size_t k = static_cast<size_t>(r) * nSteps + it;
        res[k] = (it == 0) ? 0.0f : o[k] - data[k];
      }
    l2 += objective(res.data(), nrec * nSteps);
    if (p->if_src_update) src_update_adj(res.data(), nSteps, nrec, g.dt, kr);  // libCUFD.cu:296-299
    if (p->if_filter) bp_filter(res.data(), nSteps, nrec, g.dt, p->filter);  // libCUFD.cu:301-304
    if (p->if_win)
      taper_windowed(res.data(), nSteps, nrec, g.dt, 0.1f, sh.win_start, sh.win_end, sh.weights);
    else
      taper(res.data(), nSteps, nrec, g.dt, 0.005f);
    if (syn_out && syn_out[is]) std::memcpy(syn_out[is], data.data(), data.size() * sizeof(float));
    if (res_out && res_out[is]) std::memcpy(res_out[is], res.data(), res.size() * sizeof(float));
    if (!withAdj) continue;

    // Backward (libCUFD.cu:334-457).
    for (auto* a : {&f.vz_a, &f.vx_a, &f.szz_a, &f.sxx_a, &f.sxz_a, &f.m_dvz_dz, &f.m_dvz_dx, &f.m_dvx_dz, &f.m_dvx_dx,
                    &f.m_dszz_dz, &f.m_dsxz_dx, &f.m_dsxz_dz, &f.m_dsxx_dx})
      std::fill(a->begin(), a->end(), 0.0f);
    std::vector<float> gStf(nSteps, 0.0f);
    auto inject = [&](int it) {  // res_injection (utilities.cu:569-580)
      for (int r = 0; r < nrec; ++r) {
        const float v = res[static_cast<size_t>(r) * nSteps + it];
        f.szz_a[rec[r]] += v;
        f.sxx_a[rec[r]] = static_cast<float>(f.sxx_a[rec[r]] + kRSXXZZ * v);
      }
    };
    auto restore = [&](int it, bool stress) {  // to_bnd
      const std::vector<float>* fl[5] = {&f.szz, &f.sxz, &f.sxx, &f.vz, &f.vx};
      for (int k = stress ? 0 : 3; k < (stress ? 3 : 5); ++k) {
        const float* src_ = store.data() + (static_cast<size_t>(k) * nSteps + it) * len;
        float* dst = const_cast<float*>(fl[k]->data());
        for (int e = 0; e < len; ++e) dst[strip[e]] = src_[e];
      }
    };
    velocity_adjoint(g, m, c, f);
    inject(nSteps - 1);
    stress_adjoint(g, m, c, f);
    for (int it = nSteps - 2; it >= 0; --it) {
      gStf[it] = static_cast<float>(-(f.szz_a[g.at(zs, xs)] + kRSXXZZ * f.sxx_a[g.at(zs, xs)]) * g.dt);
      velocity_reverse(g, m, f, gDen, tA, tB);
      restore(it, false);
      add_source(g, f, src[it], zs, xs, false, gauss);
      stress_reverse(g, m, f, gLam, gMu, tS);
      restore(it, true);
      velocity_adjoint(g, m, c, f);
      inject(it);
      stress_adjoint(g, m, c, f);
    }
    if (grad_stf)
      for (int it = 0; it < nSteps; ++it) grad_stf[static_cast<size_t>(is) * nSteps + it] = gStf[it];
  }
  if (withAdj) {
    for (int z = 0; z < nz; ++z)
      for (int x = 0; x < nx; ++x) {
        grad_Lambda[static_cast<size_t>(z) * nx + x] = gLam[g.at(z, x)];
        grad_Mu[static_cast<size_t>(z) * nx + x] = gMu[g.at(z, x)];
        grad_Den[static_cast<size_t>(z) * nx + x] = gDen[g.at(z, x)];
      }
  }
  if (if_res && !withAdj && misfit) *misfit = 0.5f * l2;  // libCUFD.cu:528-536 (float accumulator)
  return ORACLE_OK;
}

int oracle_cufd(const oracle_para* p, const oracle_shot* shots, int group_size, const int* shot_ids,
                const double* Lambda, const double* Mu, const double* Den, const double* stf, int calc_id,
                const float* const* obs, float* const* syn_out, float* const* res_out, double* misfit,
                double* grad_Lambda, double* grad_Mu, double* grad_Den, double* grad_stf, int nthreads) {
  return cufd_impl(p, shots, group_size, shot_ids, Lambda, Mu, Den, stf, calc_id, obs, syn_out, res_out, misfit,
                   grad_Lambda, grad_Mu, grad_Den, grad_stf, nthreads, nullptr, nullptr);
}

// oracle_cufd that also adds the source illumination of every shot, row-major
// [nz][nx] double, into illum (the caller zeroes it).
int oracle_cufd_illum(const oracle_para* p, const oracle_shot* shots, int group_size, const int* shot_ids,
                      const double* Lambda, const double* Mu, const double* Den, const double* stf, int calc_id,
                      const float* const* obs, float* const* syn_out, float* const* res_out, double* misfit,
                      double* grad_Lambda, double* grad_Mu, double* grad_Den, double* grad_stf, int nthreads,
                      double* illum) {
  return cufd_impl(p, shots, group_size, shot_ids, Lambda, Mu, Den, stf, calc_id, obs, syn_out, res_out, misfit,
                   grad_Lambda, grad_Mu, grad_Den, grad_stf, nthreads, illum, nullptr);
}

// oracle_cufd_illum that also returns each shot's source wavelet as the
// residual path leaves it (the updated wavelet under if_src_update, else the
// tapered one) in src_out[i] (nSteps floats, optional).
int oracle_cufd_full(const oracle_para* p, const oracle_shot* shots, int group_size, const int* shot_ids,
                     const double* Lambda, const double* Mu, const double* Den, const double* stf, int calc_id,
                     const float* const* obs, float* const* syn_out, float* const* res_out, double* misfit,
                     double* grad_Lambda, double* grad_Mu, double* grad_Den, double* grad_stf, int nthreads,
                     double* illum, float* const* src_out) {
  return cufd_impl(p, shots, group_size, shot_ids, Lambda, Mu, Den, stf, calc_id, obs, syn_out, res_out, misfit,
                   grad_Lambda, grad_Mu, grad_Den, grad_stf, nthreads, illum, src_out);
}

}  // extern "C"
