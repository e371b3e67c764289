// Host side of the GB300 elastic FWI operator: parameter / survey parsing,
// CPML profiles, device buffers, the per-shot forward / residual / adjoint
// schedule and the C ABI declared in include/fwiflow_gb300.h.
//
// Follows the reference driver cufd (deps/CustomOps/FWI/Src/libCUFD.cu:34-580)
// step for step, with these differences of mechanism (not of result):
//  * one forward sweep per gradient: the misfit comes out of the same forward
//    pass that saves the boundary ring (the reference's FwiOpGrad re-runs the
//    forward, FwiOp.cpp:130-223);
//  * device buffers live in a context and are reused across calls;
//  * failures return a status and a message instead of exit().
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "fwiflow_gb300.h"
#include "fwigb_kernels.h"
#include "json_lite.h"

namespace fwigb {

constexpr double kPI = 3.141592653589793238462643383279502884197169;

struct Params {
  int nz = 0, nx = 0, nSteps = 0, nPml = 0, nPad = 0;
  float dz = 0, dx = 0, dt = 0, f0 = 0;
  std::string survey_fname, data_dir_name, scratch_dir_name;
  bool if_save_scratch = false, if_win = false, if_filter = false, if_src_update = false;
  float filter[4] = {0, 0, 0, 0};
  bool operator==(const Params& o) const {
    return nz == o.nz && nx == o.nx && nSteps == o.nSteps && nPml == o.nPml && nPad == o.nPad && dz == o.dz &&
           dx == o.dx && dt == o.dt && f0 == o.f0 && survey_fname == o.survey_fname &&
           data_dir_name == o.data_dir_name && scratch_dir_name == o.scratch_dir_name && if_win == o.if_win &&
           if_filter == o.if_filter && if_src_update == o.if_src_update;
  }
};

struct ShotGeom {
  bool present = false;
  int z_src = 0, x_src = 0;  // padded-grid cell (survey index + nPml, Src_Rec.cu:86,90)
  std::vector<int> z_rec, x_rec;
  std::vector<float> win_start, win_end, weights;
};

// Parameter.cpp:16-178. Integer keys must be integers; dt, dz, dx, f0 any number.
static bool load_params(const std::string& path, Params& p, std::string& err) {
  JValue j;
  if (!json_read_first_line(path, j, err)) return false;
  if (j.kind != JValue::Object) {
    err = path + ": not a JSON object";
    return false;
  }
  auto need_int = [&](const char* k, int& v) {
    const JValue* x = j.get(k);
    if (!x || x->kind != JValue::Number || !x->is_integer) {
      err = path + ": missing or non-integer key " + k;
      return false;
    }
    v = static_cast<int>(x->num);
    return true;
  };
  auto need_num = [&](const char* k, float& v) {
    const JValue* x = j.get(k);
    if (!x || x->kind != JValue::Number) {
      err = path + ": missing or non-numeric key " + k;
      return false;
    }
    v = static_cast<float>(x->num);
    return true;
  };
  auto need_str = [&](const char* k, std::string& v) {
    const JValue* x = j.get(k);
    if (!x || x->kind != JValue::String) {
      err = path + ": missing or non-string key " + k;
      return false;
    }
    v = x->str;
    return true;
  };
  if (!need_int("nz", p.nz) || !need_int("nx", p.nx) || !need_num("dz", p.dz) || !need_num("dx", p.dx) ||
      !need_int("nSteps", p.nSteps) || !need_int("nPoints_pml", p.nPml) || !need_int("nPad", p.nPad) ||
      !need_num("dt", p.dt) || !need_num("f0", p.f0) || !need_str("survey_fname", p.survey_fname) ||
      !need_str("data_dir_name", p.data_dir_name))
    return false;
  if (const JValue* s = j.get("scratch_dir_name")) {
    if (s->kind != JValue::String) {
      err = path + ": scratch_dir_name must be a string";
      return false;
    }
    p.if_save_scratch = true;
    p.scratch_dir_name = s->str;
  }
  if (const JValue* w = j.get("if_win")) p.if_win = (w->kind == JValue::Bool) && w->b;
  if (const JValue* fl = j.get("filter")) {
    if (fl->kind != JValue::Array || fl->arr.size() < 4) {
      err = path + ": filter must be an array of 4 frequencies";
      return false;
    }
    p.if_filter = true;
    for (int k = 0; k < 4; ++k) p.filter[k] = static_cast<float>(fl->arr[k].num);
  }
  if (const JValue* su = j.get("if_src_update")) p.if_src_update = (su->kind == JValue::Bool) && su->b;
  if (p.nz < 8 || p.nx < 8 || p.nSteps < 1 || p.nPml < 3 || p.nPad < 0 || p.dz <= 0 || p.dx <= 0 || p.dt <= 0) {
    err = path + ": grid sizes or steps out of range";
    return false;
  }
  if (p.nz - 2 * p.nPml - p.nPad < 6 || p.nx - 2 * p.nPml < 6) {
    err = path + ": interior smaller than the 5-layer boundary ring";
    return false;
  }
  return true;
}

// Src_Rec.cu:19-245 for every shot of the survey file.
static bool load_survey(const Params& p, std::vector<ShotGeom>& shots, int& nrec_max, std::string& err) {
  JValue j;
  if (!json_read_first_line(p.survey_fname, j, err)) return false;
  const JValue* ns = j.get("nShots");
  if (!ns || ns->kind != JValue::Number) {
    err = p.survey_fname + ": missing nShots";
    return false;
  }
  const int nShots = static_cast<int>(ns->num);
  shots.assign(std::max(nShots, 0), ShotGeom());
  nrec_max = 0;
  for (int s = 0; s < nShots; ++s) {
    const JValue* d = j.get("shot" + std::to_string(s));
    if (!d) continue;  // a survey may list fewer shots; using a missing one is an error at staging time
    ShotGeom& g = shots[s];
    const JValue* zs = d->get("z_src");
    const JValue* xs = d->get("x_src");
    const JValue* nr = d->get("nrec");
    const JValue* zr = d->get("z_rec");
    const JValue* xr = d->get("x_rec");
    if (!zs || !xs || !nr || !zr || !xr || zr->kind != JValue::Array || xr->kind != JValue::Array) {
      err = p.survey_fname + ": shot" + std::to_string(s) + " lacks z_src/x_src/nrec/z_rec/x_rec";
      return false;
    }
    const int nrec = static_cast<int>(nr->num);
    if (nrec < 1 || static_cast<int>(zr->arr.size()) < nrec || static_cast<int>(xr->arr.size()) < nrec) {
      err = p.survey_fname + ": shot" + std::to_string(s) + " receiver arrays shorter than nrec";
      return false;
    }
    g.present = true;
    g.z_src = static_cast<int>(zs->num) + p.nPml;
    g.x_src = static_cast<int>(xs->num) + p.nPml;
    g.z_rec.resize(nrec);
    g.x_rec.resize(nrec);
    for (int r = 0; r < nrec; ++r) {
      g.z_rec[r] = static_cast<int>(zr->arr[r].num) + p.nPml;
      g.x_rec[r] = static_cast<int>(xr->arr[r].num) + p.nPml;
      if (g.z_rec[r] < 0 || g.z_rec[r] >= p.nz || g.x_rec[r] < 0 || g.x_rec[r] >= p.nx) {
        err = p.survey_fname + ": shot" + std::to_string(s) + " receiver outside the grid";
        return false;
      }
    }
    // The reference's 9x9 source stencil (utilities.cu:530-538) must stay on the grid.
    if (g.z_src < 4 || g.z_src >= p.nz - 4 || g.x_src < 4 || g.x_src >= p.nx - 4) {
      err = p.survey_fname + ": shot" + std::to_string(s) + " source too close to the grid edge";
      return false;
    }
    if (p.if_win) {
      const JValue* a = d->get("win_start");
      const JValue* b = d->get("win_end");
      const JValue* c = d->get("weights");
      if (!a || !b || !c || a->kind != JValue::Array || b->kind != JValue::Array || c->kind != JValue::Array ||
          static_cast<int>(a->arr.size()) < nrec || static_cast<int>(b->arr.size()) < nrec ||
          static_cast<int>(c->arr.size()) < nrec) {
        err = p.survey_fname + ": shot" + std::to_string(s) + " lacks win_start/win_end/weights";
        return false;
      }
      g.win_start.resize(nrec);
      g.win_end.resize(nrec);
      g.weights.resize(nrec);
      for (int r = 0; r < nrec; ++r) {
        g.win_start[r] = static_cast<float>(a->arr[r].num);
        g.win_end[r] = static_cast<float>(b->arr[r].num);
        g.weights[r] = static_cast<float>(c->arr[r].num);
      }
    }
    nrec_max = std::max(nrec_max, nrec);
  }
  return true;
}

// CPML profiles of cpmlInit (utilities.cu:242-358; CpAve fixed to 3000 at
// :259, K_max 2, alpha_max pi f0, R 0.0008, damping d0 (x/4 + 3x^8/4)), kept
// in the reference's float / double arithmetic. N is the profile length
// (nz - nPad for z, Cpml.cu:46-48), out arrays are padded to `len`.
static void cpml_profile(int N, int len, int nPml, float dh, float f0, float dt, float* K, float* a, float* b,
                         float* Kh, float* ah, float* bh) {
  const float R = 0.0008f, Kmax = 2.0f, npow = 8.0f, cpave = 3000.0f;
  const float amax = static_cast<float>(2.0 * kPI * (f0 / 2.0));
  const float thick = nPml * dh;
  const float d0 = static_cast<float>(-(npow + 1) * cpave * std::log(R) / (2.0 * thick));
  auto damp_of = [&](float xn) { return d0 * (0.25f * xn + 0.75f * std::pow(xn, npow) + 0.0f * std::pow(xn, 2 * npow)); };
  for (int i = 0; i < len; ++i) {
    K[i] = Kh[i] = 1.0f;
    a[i] = ah[i] = 0.0f;
    b[i] = bh[i] = 1.0f;
  }
  for (int i = 0; i < N; ++i) {
    float dmp = 0, dmph = 0, al = 0, alh = 0, k = 1, kh = 1;
    auto edge = [&](float depth, float& dd, float& kk, float& aa) {
      if (depth >= 0.0f) {
        const float xn = depth / thick;
        dd = damp_of(xn);
        kk = static_cast<float>(1.0 + (Kmax - 1.0) * std::pow(xn, npow));
        aa = static_cast<float>(amax * (1.0 - xn));
      }
    };
    edge((nPml - i) * dh, dmp, k, al);
    edge(static_cast<float>((nPml - i - 0.5) * dh), dmph, kh, alh);
    edge((nPml - N + i) * dh, dmp, k, al);
    edge(static_cast<float>((nPml - N + i + 0.5) * dh), dmph, kh, alh);
    if (al < 0.0f) al = 0.0f;
    if (alh < 0.0f) alh = 0.0f;
    const float bb = std::exp(-(dmp / k + al) * dt);
    const float bbh = std::exp(-(dmph / kh + alh) * dt);
    K[i] = k;
    Kh[i] = kh;
    b[i] = bb;
    bh[i] = bbh;
    a[i] = (std::fabs(dmp) > 1.0e-6) ? static_cast<float>(dmp * (bb - 1.0) / (k * (dmp + k * al))) : 0.0f;
    ah[i] = (std::fabs(dmph) > 1.0e-6) ? static_cast<float>(dmph * (bbh - 1.0) / (kh * (dmph + kh * alh))) : 0.0f;
  }
}

// sin^2 / cos^2 taper weights of cuda_window without windows (utilities.cu:707-747).
static bool taper_weights(int nt, float dt, float ratio, float* w) {
  const float t0 = 0.0f, t3 = nt * dt, off = nt * dt * ratio;
  if (2.0 * off >= t3 - t0) return false;
  const float t1 = t0 + off, t2 = t3 - off;
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
  return true;
}

// Per-trace windows and weights of cuda_window (utilities.cu:653-705). A trace
// whose window is empty is left unchanged (weight 1), as the reference returns
// before scaling it.
static void taper_weights_windowed(int nt, float dt, float ratio, float ws, float we, float wt, float* w) {
  for (int it = 0; it < nt; ++it) w[it] = 1.0f;
  if (ratio > 0.5f) return;
  float t0 = ws, t3 = we;
  const float tmax = nt * dt;
  t0 = std::min(std::max(t0, 0.0f), tmax);
  t3 = std::min(std::max(t3, 0.0f), tmax);
  const float off = (t3 - t0) * ratio;
  if (off <= 0.0f) return;
  const float t1 = t0 + off, t2 = t3 - off;
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
    w[it] = amp * amp * wt;
  }
}

// Grow-only device buffer.
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  cudaError_t ensure(size_t n) {
    if (n <= bytes) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    cudaError_t e = cudaMalloc(&p, n);
    if (e == cudaSuccess) bytes = n;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  template <class T>
  T* as(size_t offset_elems = 0) const {
    return static_cast<T*>(p) + offset_elems;
  }
};

struct StagedShot {
  int id;
  int nrec;
  ShotGeom* geom;
};

}  // namespace fwigb

using namespace fwigb;

struct fwigb_ctx {
  std::mutex mu;
  std::string err;
  std::string para_fname;
  int device = 0;
  Params p;
  std::vector<ShotGeom> survey;
  int nrec_max = 0;
  Geo geo{};
  cudaStream_t stream = nullptr;
  size_t cells = 0;   // allocated cells per grid array (ldz * nx)
  size_t ncell = 0;   // logical cells (nz * nx), the size of host arrays
  SweepMaps maps[3];  // tensor maps for tile widths 4, 8, 16
  int tx[4] = {8, 8, 8, 8};  // tile width per sweep (F1, F2, B, C)
  bool tuned_fwd = false, tuned_bwd = false;
  bool autotune = true;
  // device buffers
  DevBuf media, stage, cpml, fields, grads, store, scal, partials;
  DevBuf shot_src, shot_rec, shot_blk, shot_data, shot_taper, shot_gstf;
  // staged shots
  std::vector<StagedShot> staged;
  bool with_obs = false;
  bool per_trace_taper = false;
  int nblk = 0;  // receiver bins (32 x 8 cells)
  int nbin_z = 0;
  bool model_set = false;
  int last_calc = -1;
  long long launches = 0;
  // per-kernel event timing
  bool timing = false;
  std::vector<cudaEvent_t> ev_pool;
  std::vector<int> ev_kind;  // kind of the i-th event pair of the last run
};

namespace {

thread_local std::string g_err;

#define TRY_RC(call)                  \
  do {                                \
    int rc_ = (call);                 \
    if (rc_ != FWIGB_OK) return rc_;  \
  } while (0)

#define CK(call)                                                                                   \
  do {                                                                                             \
    cudaError_t e_ = (call);                                                                       \
    if (e_ != cudaSuccess) {                                                                       \
      ctx->err = std::string(#call) + ": " + cudaGetErrorString(e_);                               \
      return (e_ == cudaErrorMemoryAllocation) ? FWIGB_ERR_OOM : FWIGB_ERR_CUDA;                   \
    }                                                                                              \
  } while (0)

int tx_slot(int tx) { return tx == 4 ? 0 : (tx == 8 ? 1 : 2); }

Fields fields_of(fwigb_ctx* ctx) {
  float* b = ctx->fields.as<float>();
  const size_t n = ctx->cells;
  Fields f;
  float** slots[18] = {&f.vz,       &f.vx,       &f.szz,      &f.sxx,      &f.sxz,       &f.vz_a,
                       &f.vx_a,     &f.szz_a,    &f.sxx_a,    &f.sxz_a,    &f.m_dvz_dz,  &f.m_dvz_dx,
                       &f.m_dvx_dz, &f.m_dvx_dx, &f.m_dszz_dz, &f.m_dsxx_dx, &f.m_dsxz_dz, &f.m_dsxz_dx};
  for (int k = 0; k < 18; ++k) *slots[k] = b + k * n;
  return f;
}

// media: lam, mu, den, l2m, aveMu, bycA, bycB, hs, muw
MediaD media_of(fwigb_ctx* ctx) {
  float* b = ctx->media.as<float>();
  const size_t n = ctx->cells;
  MediaD m;
  m.lam = b;
  m.l2m = b + 3 * n;
  m.aveMu = b + 4 * n;
  m.bycA = b + 5 * n;
  m.bycB = b + 6 * n;
  m.hs = b + 7 * n;
  m.muw = b + 8 * n;
  return m;
}

CpmlD cpml_of(fwigb_ctx* ctx) {
  const float* b = ctx->cpml.as<float>();
  const int nz = ctx->p.nz, nx = ctx->p.nx;
  CpmlD c;
  c.K_z = b;
  c.a_z = b + nz;
  c.b_z = b + 2 * nz;
  c.K_zh = b + 3 * nz;
  c.a_zh = b + 4 * nz;
  c.b_zh = b + 5 * nz;
  const float* x = b + 6 * nz;
  c.K_x = x;
  c.a_x = x + nx;
  c.b_x = x + 2 * nx;
  c.K_xh = x + 3 * nx;
  c.a_xh = x + 4 * nx;
  c.b_xh = x + 5 * nx;
  return c;
}

int setup_geometry(fwigb_ctx* ctx) {
  const Params& p = ctx->p;
  Geo& g = ctx->geo;
  g.nz = p.nz;
  g.nx = p.nx;
  g.ldz = (p.nz + 31) / 32 * 32;
  g.nPml = p.nPml;
  g.nPad = p.nPad;
  g.zs0 = 2;
  g.zs1 = p.nz - p.nPad - 3;
  g.xs0 = 2;
  g.xs1 = p.nx - 3;
  g.zi0 = p.nPml;
  g.zi1 = p.nz - p.nPad - 1 - p.nPml;
  g.xi0 = p.nPml;
  g.xi1 = p.nx - 1 - p.nPml;
  g.zpml_hi = p.nz - p.nPml - p.nPad - 1;
  g.xpml_hi_s = p.nx - p.nPml - 1;
  g.xpml_hi_v = p.nx - p.nPml;
  g.rz0 = p.nPml - 2;
  g.rz1 = p.nz - p.nPml - p.nPad + 1;
  g.rx0 = p.nPml - 2;
  g.rx1 = p.nx - p.nPml + 1;
  g.ringW = g.rx1 - g.rx0 + 1;
  g.ringH = g.rz1 - g.rz0 + 1 - 10;
  g.ring_len = 10 * g.ringW + 10 * g.ringH;
  g.dt = p.dt;
  g.rdz = 1.0f / p.dz;
  g.rdx = 1.0f / p.dx;
  ctx->cells = static_cast<size_t>(g.ldz) * p.nx;
  ctx->ncell = static_cast<size_t>(p.nz) * p.nx;

  // CPML profiles (host) and the adjoint-memory bands derived from them.
  std::vector<float> h(6 * p.nz + 6 * p.nx);
  float* z = h.data();
  float* x = h.data() + 6 * p.nz;
  cpml_profile(p.nz - p.nPad, p.nz, p.nPml, p.dz, p.f0, p.dt, z, z + p.nz, z + 2 * p.nz, z + 3 * p.nz, z + 4 * p.nz,
               z + 5 * p.nz);
  cpml_profile(p.nx, p.nx, p.nPml, p.dx, p.f0, p.dt, x, x + p.nx, x + 2 * p.nx, x + 3 * p.nx, x + 4 * p.nx,
               x + 5 * p.nx);
  // An adjoint psi memory cell matters only within 2 cells of a cell whose
  // CPML coefficient a (or a_half) is non-zero; elsewhere the reference's
  // updates (el_stress_adj.cu:68-94) are multiplied by a == 0.
  auto band = [](const float* a, const float* ah, int n, int& lo, int& hi) {
    lo = -1000000;
    hi = 1000000;
    for (int i = 0; i < n / 2; ++i)
      if (a[i] != 0.0f || ah[i] != 0.0f) lo = i + 2;
    for (int i = n - 1; i >= n / 2; --i)
      if (a[i] != 0.0f || ah[i] != 0.0f) hi = i - 2;
  };
  band(z + p.nz, z + 4 * p.nz, p.nz - p.nPad, g.zband_lo, g.zband_hi);
  band(x + p.nx, x + 4 * p.nx, p.nx, g.xband_lo, g.xband_hi);
  CK(ctx->cpml.ensure(h.size() * sizeof(float)));
  CK(cudaMemcpy(ctx->cpml.p, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice));
  CK(ctx->media.ensure(9 * ctx->cells * sizeof(float)));
  CK(ctx->stage.ensure(3 * ctx->ncell * sizeof(double)));
  CK(ctx->fields.ensure(18 * ctx->cells * sizeof(float)));
  CK(ctx->grads.ensure(3 * ctx->cells * sizeof(float)));
  // [0]: misfit accumulator (double), [8]: cp max bits, [16]: sweep error word
  CK(ctx->scal.ensure(64));
  CK(cudaMemset(ctx->scal.p, 0, 64));
  // Padding rows (ldz > nz) and every field start at zero.
  CK(cudaMemset(ctx->media.p, 0, 9 * ctx->cells * sizeof(float)));
  CK(cudaMemset(ctx->fields.p, 0, 18 * ctx->cells * sizeof(float)));
  CK(ctx->partials.ensure(1024 * sizeof(double)));
  ctx->nbin_z = (p.nz + kBinZ - 1) / kBinZ;
  ctx->nblk = ctx->nbin_z * ((p.nx + kBinX - 1) / kBinX);
  const Fields f = fields_of(ctx);
  for (int k = 0; k < 3; ++k) {
    const char* why = nullptr;
    if (!encode_sweep_maps(g, f, kTileXs[k], ctx->maps[k], &why)) {
      ctx->err = why;
      return FWIGB_ERR_CUDA;
    }
  }
  return FWIGB_OK;
}

int open_ctx(const char* para_fname, int device, fwigb_ctx* ctx) {
  ctx->para_fname = para_fname;
  ctx->device = device;
  std::string err;
  if (!load_params(para_fname, ctx->p, err)) {
    ctx->err = err;
    return FWIGB_ERR_PARAM;
  }
  if (!load_survey(ctx->p, ctx->survey, ctx->nrec_max, err)) {
    ctx->err = err;
    return FWIGB_ERR_PARAM;
  }
  CK(cudaSetDevice(device));
  CK(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
  return setup_geometry(ctx);
}

int set_model(fwigb_ctx* ctx, const double* lam, const double* mu, const double* den) {
  if (!lam || !mu || !den) {
    ctx->err = "null model array";
    return FWIGB_ERR_ARG;
  }
  CK(cudaSetDevice(ctx->device));
  const size_t nh = ctx->ncell, n = ctx->cells;
  const int ldz = ctx->geo.ldz;
  double* st = ctx->stage.as<double>();
  CK(cudaMemcpyAsync(st, lam, nh * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(st + nh, mu, nh * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(st + 2 * nh, den, nh * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  unsigned* cpbits = reinterpret_cast<unsigned*>(ctx->scal.as<char>() + 8);
  CK(cudaMemsetAsync(cpbits, 0, sizeof(unsigned), ctx->stream));
  float* b = ctx->media.as<float>();
  launch_media_from_rowmajor(ctx->stream, ctx->p.nz, ctx->p.nx, ldz, st, st + nh, st + 2 * nh, b, b + n, b + 2 * n,
                             cpbits);
  launch_media_derived(ctx->stream, ctx->p.nz, ctx->p.nx, ldz, b, b + n, b + 2 * n, b + 3 * n, b + 4 * n, b + 5 * n,
                       b + 6 * n, b + 7 * n, b + 8 * n);
  CK(cudaGetLastError());
  unsigned bits = 0;
  CK(cudaMemcpyAsync(&bits, cpbits, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  float cpmax;
  std::memcpy(&cpmax, &bits, sizeof(float));
  // compCourantNumber (utilities.cu:225-240).
  const float dh = std::min(ctx->p.dz, ctx->p.dx);
  const float courant = static_cast<float>(cpmax * ctx->p.dt * std::sqrt(2.0f) * (1.0 / 24.0 + 9.0 / 8.0) / dh);
  if (!(courant <= 1.0f)) {
    char buf[160];
    std::snprintf(buf, sizeof(buf), "Courant number %.4f > 1 (max P velocity %.1f m/s)", courant, cpmax);
    ctx->err = buf;
    ctx->model_set = false;
    return FWIGB_ERR_COURANT;
  }
  ctx->model_set = true;
  return FWIGB_OK;
}

int stage_shots(fwigb_ctx* ctx, const double* stf, int n_stf_rows, const int* shot_ids, int n_shots, bool with_obs,
                const float* obs) {
  const Params& p = ctx->p;
  if (!stf || !shot_ids || n_shots < 1 || n_stf_rows < 1) {
    ctx->err = "stf / shot_ids missing";
    return FWIGB_ERR_ARG;
  }
  if (p.if_filter || p.if_src_update) {
    ctx->err = "parameter file asks for the band-pass filter or source update, which this build does not implement";
    return FWIGB_ERR_UNSUPPORTED;
  }
  CK(cudaSetDevice(ctx->device));
  const int nt = p.nSteps, nrm = ctx->nrec_max;
  ctx->staged.clear();
  for (int i = 0; i < n_shots; ++i) {
    const int id = shot_ids[i];
    if (id < 0 || id >= static_cast<int>(ctx->survey.size()) || !ctx->survey[id].present) {
      ctx->err = "shot id " + std::to_string(id) + " not in the survey file";
      return FWIGB_ERR_ARG;
    }
    if (id >= n_stf_rows) {
      ctx->err = "shot id " + std::to_string(id) + " has no stf row";
      return FWIGB_ERR_ARG;
    }
    ctx->staged.push_back({id, static_cast<int>(ctx->survey[id].z_rec.size()), &ctx->survey[id]});
  }
  const size_t ns = ctx->staged.size();
  // Sources: taper 0.001 (Src_Rec.cu:140) and the add_source scale (utilities.cu:528-538).
  std::vector<float> hsrc(2 * ns * nt);
  std::vector<float> w(nt);
  if (!taper_weights(nt, p.dt, 0.001f, w.data())) {
    ctx->err = "nSteps too small for the source taper";
    return FWIGB_ERR_ARG;
  }
  const float scale = 2250000.0f;  // pow(1500.0, 2)
  for (size_t s = 0; s < ns; ++s) {
    const double* row = stf + static_cast<size_t>(ctx->staged[s].id) * nt;
    for (int it = 0; it < nt; ++it) {
      const float amp = static_cast<float>(row[it]) * w[it];
      hsrc[(2 * s) * nt + it] = scale * amp * p.dt;
      hsrc[(2 * s + 1) * nt + it] = static_cast<float>(3.0 * scale * amp * p.dt);
    }
  }
  CK(ctx->shot_src.ensure(hsrc.size() * sizeof(float)));
  CK(cudaMemcpyAsync(ctx->shot_src.p, hsrc.data(), hsrc.size() * sizeof(float), cudaMemcpyHostToDevice,
                     ctx->stream));
  // Receivers and their per-block lists (CSR over the sweep grid).
  const int nbz = ctx->nbin_z;
  const int nblk = ctx->nblk;
  std::vector<int> hrec(2 * ns * nrm, 0), hblk(ns * (nblk + 1 + nrm), 0);
  for (size_t s = 0; s < ns; ++s) {
    const ShotGeom& g = *ctx->staged[s].geom;
    const int nrec = ctx->staged[s].nrec;
    int* rz = hrec.data() + 2 * s * nrm;
    int* rx = rz + nrm;
    int* off = hblk.data() + s * (nblk + 1 + nrm);
    int* lst = off + nblk + 1;
    std::vector<int> cnt(nblk + 1, 0);
    for (int r = 0; r < nrec; ++r) {
      rz[r] = g.z_rec[r];
      rx[r] = g.x_rec[r];
      cnt[(g.z_rec[r] / kBinZ) + (g.x_rec[r] / kBinX) * nbz + 1]++;
    }
    for (int b = 0; b < nblk; ++b) cnt[b + 1] += cnt[b];
    for (int b = 0; b <= nblk; ++b) off[b] = cnt[b];
    std::vector<int> pos(cnt.begin(), cnt.end() - 1);
    for (int r = 0; r < nrec; ++r) lst[pos[(g.z_rec[r] / kBinZ) + (g.x_rec[r] / kBinX) * nbz]++] = r;
  }
  CK(ctx->shot_rec.ensure(hrec.size() * sizeof(int)));
  CK(ctx->shot_blk.ensure(hblk.size() * sizeof(int)));
  CK(cudaMemcpyAsync(ctx->shot_rec.p, hrec.data(), hrec.size() * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->shot_blk.p, hblk.data(), hblk.size() * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  // Data buffers: obs | syn | res, each [ns][nrec_max][nSteps].
  const size_t per = static_cast<size_t>(nrm) * nt;
  CK(ctx->shot_data.ensure(3 * ns * per * sizeof(float)));
  ctx->with_obs = with_obs;
  if (with_obs) {
    float* d_obs = ctx->shot_data.as<float>();
    if (obs) {
      CK(cudaMemcpyAsync(d_obs, obs, ns * per * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
    } else {
      // libCUFD.cu:189-200: data_dir_name/Shot<id>.bin, [nrec][nSteps] float.
      std::vector<float> buf(per);
      for (size_t s = 0; s < ns; ++s) {
        const std::string fn = p.data_dir_name + "/Shot" + std::to_string(ctx->staged[s].id) + ".bin";
        std::FILE* fp = std::fopen(fn.c_str(), "rb");
        if (!fp) {
          ctx->err = "cannot read " + fn;
          return FWIGB_ERR_IO;
        }
        const size_t want = static_cast<size_t>(ctx->staged[s].nrec) * nt;
        const size_t got = std::fread(buf.data(), sizeof(float), want, fp);
        std::fclose(fp);
        if (got != want) {
          ctx->err = fn + " is shorter than nrec*nSteps";
          return FWIGB_ERR_IO;
        }
        CK(cudaMemcpy(d_obs + s * per, buf.data(), want * sizeof(float), cudaMemcpyHostToDevice));
      }
    }
  }
  // Taper weights: [2][nt] shared, or per trace [ns][2][nrec_max][nt] with windows.
  ctx->per_trace_taper = p.if_win;
  std::vector<float> ht;
  if (!p.if_win) {
    ht.resize(2 * nt);
    if (!taper_weights(nt, p.dt, 0.005f, ht.data())) {
      ctx->err = "nSteps too small for the data taper";
      return FWIGB_ERR_ARG;
    }
    std::copy(ht.begin(), ht.begin() + nt, ht.begin() + nt);
  } else {
    ht.assign(ns * 2 * per, 1.0f);
    for (size_t s = 0; s < ns; ++s) {
      const ShotGeom& g = *ctx->staged[s].geom;
      for (int r = 0; r < ctx->staged[s].nrec; ++r) {
        taper_weights_windowed(nt, p.dt, 0.005f, g.win_start[r], g.win_end[r], g.weights[r],
                               ht.data() + (2 * s) * per + static_cast<size_t>(r) * nt);
        taper_weights_windowed(nt, p.dt, 0.1f, g.win_start[r], g.win_end[r], g.weights[r],
                               ht.data() + (2 * s + 1) * per + static_cast<size_t>(r) * nt);
      }
    }
  }
  CK(ctx->shot_taper.ensure(ht.size() * sizeof(float)));
  CK(cudaMemcpyAsync(ctx->shot_taper.p, ht.data(), ht.size() * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
  CK(ctx->shot_gstf.ensure(ns * nt * sizeof(float)));
  CK(cudaStreamSynchronize(ctx->stream));  // host staging vectors go out of scope
  return FWIGB_OK;
}

// Tile-width autotuner: times every width of each sweep on this context's grid
// (a few launches each on the live buffers, which the run then resets) and
// keeps the fastest. Forward sweeps are tuned on the first run, backward sweeps
// on the first run with the adjoint.
int autotune(fwigb_ctx* ctx, const ShotD& sh, bool adj) {
  cudaStream_t s = ctx->stream;
  const Geo& g = ctx->geo;
  Fields f = fields_of(ctx);
  MediaD m = media_of(ctx);
  CpmlD c = cpml_of(ctx);
  StoreD st{ctx->store.as<float>()};
  float* gb = ctx->grads.as<float>();
  Grads gr{gb, gb + ctx->cells, gb + 2 * ctx->cells};
  unsigned* d_err = reinterpret_cast<unsigned*>(ctx->scal.as<char>() + 16);
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  const int kinds_end = (adj && ctx->p.nSteps >= 2) ? 4 : 2;
  for (int kind = ctx->tuned_fwd ? 2 : 0; kind < kinds_end; ++kind) {
    float best = 1e30f;
    for (int slot = 0; slot < 3; ++slot) {
      const int tx = kTileXs[slot];
      const SweepMaps& mp = ctx->maps[slot];
      auto launch = [&]() {
        switch (kind) {
          case 0: launch_fwd_stress(s, tx, mp.f1, g, f, m, c, sh, st, 0, false, d_err); break;
          case 1: launch_fwd_velocity(s, tx, mp.f2, g, f, m, c, d_err); break;
          case 2: launch_bwd_B(s, tx, mp.b, g, f, m, c, sh, st, gr, 0, d_err); break;
          default: launch_bwd_C(s, tx, mp.c, g, f, m, c, sh, st, gr, 1, true, d_err); break;
        }
      };
      for (int w = 0; w < 2; ++w) launch();
      CK(cudaEventRecord(e0, s));
      for (int r = 0; r < 10; ++r) launch();
      CK(cudaEventRecord(e1, s));
      CK(cudaEventSynchronize(e1));
      float ms = 0.0f;
      CK(cudaEventElapsedTime(&ms, e0, e1));
      if (ms < best) {
        best = ms;
        ctx->tx[kind] = tx;
      }
    }
  }
  CK(cudaGetLastError());
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  ctx->tuned_fwd = true;
  if (kinds_end == 4) ctx->tuned_bwd = true;
  return FWIGB_OK;
}

int run(fwigb_ctx* ctx, int calc_id) {
  if (calc_id < 0 || calc_id > 2) {
    ctx->err = "calc_id must be 0, 1 or 2";
    return FWIGB_ERR_ARG;
  }
  if (!ctx->model_set) {
    ctx->err = "no model set";
    return FWIGB_ERR_ARG;
  }
  if (ctx->staged.empty()) {
    ctx->err = "no shots staged";
    return FWIGB_ERR_ARG;
  }
  const bool if_res = calc_id != 2, adj = calc_id == 1;
  if (if_res && !ctx->with_obs) {
    ctx->err = "misfit needs observed data";
    return FWIGB_ERR_ARG;
  }
  CK(cudaSetDevice(ctx->device));
  const Params& p = ctx->p;
  const Geo& g = ctx->geo;
  const int nt = p.nSteps, nrm = ctx->nrec_max;
  const size_t ns = ctx->staged.size();
  const size_t per = static_cast<size_t>(nrm) * nt;
  cudaStream_t s = ctx->stream;
  if (adj) {
    const size_t store_bytes = static_cast<size_t>(nt) * 5 * g.ring_len * sizeof(float);
    CK(ctx->store.ensure(store_bytes));
  }
  if (ctx->autotune && (!ctx->tuned_fwd || (adj && !ctx->tuned_bwd))) {
    const StagedShot& S0 = ctx->staged[0];
    ShotD sh{};
    sh.src_z = S0.geom->z_src;
    sh.src_x = S0.geom->x_src;
    sh.src_szz = ctx->shot_src.as<float>(0);
    sh.src_sxx = ctx->shot_src.as<float>(nt);
    sh.nrec = S0.nrec;
    sh.nSteps = nt;
    sh.rec_z = ctx->shot_rec.as<int>(0);
    sh.rec_x = sh.rec_z + nrm;
    sh.blk_off = ctx->shot_blk.as<int>(0);
    sh.blk_rec = sh.blk_off + ctx->nblk + 1;
    sh.nbin_z = ctx->nbin_z;
    sh.data = ctx->shot_data.as<float>(ns * per);
    sh.res = ctx->shot_data.as<float>(2 * ns * per);
    sh.gstf = ctx->shot_gstf.as<float>(0);
    TRY_RC(autotune(ctx, sh, adj));
  }
  if (adj) {
    CK(cudaMemsetAsync(ctx->grads.p, 0, 3 * ctx->cells * sizeof(float), s));
    CK(cudaMemsetAsync(ctx->shot_gstf.p, 0, ns * nt * sizeof(float), s));
  }
  double* d_misfit = ctx->scal.as<double>();
  CK(cudaMemsetAsync(d_misfit, 0, sizeof(double), s));
  Fields f = fields_of(ctx);
  MediaD m = media_of(ctx);
  CpmlD c = cpml_of(ctx);
  StoreD st{ctx->store.as<float>()};
  float* gb = ctx->grads.as<float>();
  Grads gr{gb, gb + ctx->cells, gb + 2 * ctx->cells};
  unsigned* d_err = reinterpret_cast<unsigned*>(ctx->scal.as<char>() + 16);
  auto mp = [&](int kind) -> const SweepMaps& { return ctx->maps[tx_slot(ctx->tx[kind])]; };
  long long launches = 0;
  ctx->ev_kind.clear();
  size_t ev_used = 0;
  // Brackets a sweep launch with an event pair when per-kernel timing is on.
#define TIMED(kind, launch)                                              \
  do {                                                                   \
    if (ctx->timing) {                                                   \
      if (ev_used + 2 > ctx->ev_pool.size()) {                           \
        cudaEvent_t e0, e1;                                              \
        CK(cudaEventCreate(&e0));                                        \
        CK(cudaEventCreate(&e1));                                        \
        ctx->ev_pool.push_back(e0);                                      \
        ctx->ev_pool.push_back(e1);                                      \
      }                                                                  \
      CK(cudaEventRecord(ctx->ev_pool[ev_used], s));                     \
      launch;                                                            \
      CK(cudaEventRecord(ctx->ev_pool[ev_used + 1], s));                 \
      ev_used += 2;                                                      \
      ctx->ev_kind.push_back(kind);                                      \
    } else {                                                             \
      launch;                                                            \
    }                                                                    \
  } while (0)
  for (size_t is = 0; is < ns; ++is) {
    const StagedShot& S = ctx->staged[is];
    ShotD sh{};
    sh.src_z = S.geom->z_src;
    sh.src_x = S.geom->x_src;
    sh.src_szz = ctx->shot_src.as<float>((2 * is) * nt);
    sh.src_sxx = ctx->shot_src.as<float>((2 * is + 1) * nt);
    sh.nrec = S.nrec;
    sh.nSteps = nt;
    sh.rec_z = ctx->shot_rec.as<int>(2 * is * nrm);
    sh.rec_x = sh.rec_z + nrm;
    sh.blk_off = ctx->shot_blk.as<int>(is * (ctx->nblk + 1 + nrm));
    sh.blk_rec = sh.blk_off + ctx->nblk + 1;
    sh.nbin_z = ctx->nbin_z;
    float* d_obs = ctx->shot_data.as<float>(is * per);
    float* d_syn = ctx->shot_data.as<float>((ns + is) * per);
    float* d_res = ctx->shot_data.as<float>((2 * ns + is) * per);
    sh.data = d_syn;
    sh.res = d_res;
    sh.gstf = ctx->shot_gstf.as<float>(is * nt);
    // Fresh wavefields for each shot (libCUFD.cu:163-182) and an empty gather.
    CK(cudaMemsetAsync(ctx->fields.p, 0, 18 * ctx->cells * sizeof(float), s));
    CK(cudaMemsetAsync(d_syn, 0, per * sizeof(float), s));
    for (int it = 0; it <= nt - 2; ++it) {
      TIMED(0, launch_fwd_stress(s, ctx->tx[0], mp(0).f1, g, f, m, c, sh, st, it, adj, d_err));
      TIMED(1, launch_fwd_velocity(s, ctx->tx[1], mp(1).f2, g, f, m, c, d_err));
      launches += 2;
    }
    if (if_res) {
      const float* tw = ctx->shot_taper.as<float>();
      const float* to = ctx->per_trace_taper ? tw + (2 * is) * per : tw;
      const float* tr = ctx->per_trace_taper ? tw + (2 * is + 1) * per : tw + nt;
      const int nb = residual_blocks(S.nrec * nt);
      launch_residual(s, S.nrec, nt, d_obs, d_syn, d_res, to, tr, ctx->per_trace_taper ? 1 : 0,
                      ctx->partials.as<double>());
      launch_sum_partials(s, ctx->partials.as<double>(), nb, d_misfit);
      launches += 2;
    }
    if (adj) {
      // Zero the adjoint fields and the 8 memory arrays (libCUFD.cu:337-351).
      CK(cudaMemsetAsync(f.vz_a, 0, 13 * ctx->cells * sizeof(float), s));
      // The reference's first el_velocity_adj acts on all-zero fields (no-op);
      // then res_injection(nSteps-1) + el_stress_adj, source_grad(nSteps-2),
      // reverse velocity of step nSteps-2 ... (libCUFD.cu:353-445).
      TIMED(3, launch_bwd_C(s, ctx->tx[3], mp(3).c, g, f, m, c, sh, st, gr, nt - 1, nt - 1 >= 1, d_err));
      ++launches;
      for (int it = nt - 2; it >= 0; --it) {
        TIMED(2, launch_bwd_B(s, ctx->tx[2], mp(2).b, g, f, m, c, sh, st, gr, it, d_err));
        TIMED(3, launch_bwd_C(s, ctx->tx[3], mp(3).c, g, f, m, c, sh, st, gr, it, it >= 1, d_err));
        launches += 2;
      }
    }
  }
#undef TIMED
  CK(cudaGetLastError());
  ctx->launches = launches;
  ctx->last_calc = calc_id;
  return FWIGB_OK;
}

int kernel_times(fwigb_ctx* ctx, double* total_ms, long long* counts) {
  CK(cudaStreamSynchronize(ctx->stream));
  for (int k = 0; k < 4; ++k) {
    total_ms[k] = 0.0;
    counts[k] = 0;
  }
  for (size_t i = 0; i < ctx->ev_kind.size(); ++i) {
    float ms = 0.0f;
    CK(cudaEventElapsedTime(&ms, ctx->ev_pool[2 * i], ctx->ev_pool[2 * i + 1]));
    const int k = ctx->ev_kind[i];
    total_ms[k] += ms;
    counts[k] += 1;
  }
  return FWIGB_OK;
}

int fetch(fwigb_ctx* ctx, double* misfit, double* g_lam, double* g_mu, double* g_den, double* g_stf, float* gathers) {
  CK(cudaSetDevice(ctx->device));
  cudaStream_t s = ctx->stream;
  const Params& p = ctx->p;
  const size_t n = ctx->cells;
  const size_t ns = ctx->staged.size();
  const int nt = p.nSteps;
  const size_t per = static_cast<size_t>(ctx->nrec_max) * nt;
  {
    unsigned e = 0;
    CK(cudaMemcpyAsync(&e, ctx->scal.as<char>() + 16, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (e) {
      CK(cudaMemsetAsync(ctx->scal.as<char>() + 16, 0, sizeof(unsigned), s));
      ctx->err = "a sweep gave up waiting for its staged tiles (bounded wait); results are invalid";
      return FWIGB_ERR_TIMEOUT;
    }
  }
  if (misfit) {
    double acc = 0.0;
    CK(cudaMemcpyAsync(&acc, ctx->scal.p, sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    *misfit = 0.5 * acc;
  }
  if (g_lam || g_mu || g_den) {
    if (ctx->last_calc != 1) {
      ctx->err = "gradients requested from a run without adjoint";
      return FWIGB_ERR_ARG;
    }
    double* out[3] = {g_lam, g_mu, g_den};
    double* st = ctx->stage.as<double>();
    const size_t nh = ctx->ncell;
    for (int k = 0; k < 3; ++k) {
      if (!out[k]) continue;
      launch_to_rowmajor(s, p.nz, p.nx, ctx->geo.ldz, ctx->grads.as<float>(k * n), st + k * nh, 1.0);
      CK(cudaMemcpyAsync(out[k], st + k * nh, nh * sizeof(double), cudaMemcpyDeviceToHost, s));
    }
  }
  if (g_stf) {
    std::vector<float> h(ns * nt);
    CK(cudaMemcpyAsync(h.data(), ctx->shot_gstf.p, h.size() * sizeof(float), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    for (size_t k = 0; k < h.size(); ++k) g_stf[k] = h[k];
  }
  if (gathers) {
    CK(cudaMemcpyAsync(gathers, ctx->shot_data.as<float>(ns * per), ns * per * sizeof(float),
                       cudaMemcpyDeviceToHost, s));
  }
  CK(cudaStreamSynchronize(s));
  return FWIGB_OK;
}

int write_gathers(fwigb_ctx* ctx, const float* gathers) {
  // libCUFD.cu:514-521.
  const int nt = ctx->p.nSteps;
  const size_t per = static_cast<size_t>(ctx->nrec_max) * nt;
  for (size_t s = 0; s < ctx->staged.size(); ++s) {
    const std::string fn = ctx->p.data_dir_name + "/Shot" + std::to_string(ctx->staged[s].id) + ".bin";
    std::FILE* fp = std::fopen(fn.c_str(), "wb");
    if (!fp) {
      ctx->err = "cannot write " + fn;
      return FWIGB_ERR_IO;
    }
    const size_t want = static_cast<size_t>(ctx->staged[s].nrec) * nt;
    const size_t put = std::fwrite(gathers + s * per, sizeof(float), want, fp);
    std::fclose(fp);
    if (put != want) {
      ctx->err = "short write to " + fn;
      return FWIGB_ERR_IO;
    }
  }
  return FWIGB_OK;
}

#define TRY(call)            \
  do {                       \
    int rc_ = (call);        \
    if (rc_ != FWIGB_OK) return rc_; \
  } while (0)

}  // namespace

// ---------------------------------------------------------------------------
// C ABI
extern "C" {

int fwigb_create(const char* para_fname, int device, fwigb_ctx** out) {
  if (!para_fname || !out) {
    g_err = "null argument";
    return FWIGB_ERR_ARG;
  }
  auto* ctx = new (std::nothrow) fwigb_ctx();
  if (!ctx) {
    g_err = "out of host memory";
    return FWIGB_ERR_OOM;
  }
  int rc = open_ctx(para_fname, device, ctx);
  if (rc != FWIGB_OK) {
    g_err = ctx->err;
    fwigb_destroy(ctx);
    *out = nullptr;
    return rc;
  }
  *out = ctx;
  return FWIGB_OK;
}

int fwigb_destroy(fwigb_ctx* ctx) {
  if (!ctx) return FWIGB_OK;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  for (DevBuf* b : {&ctx->media, &ctx->stage, &ctx->cpml, &ctx->fields, &ctx->grads, &ctx->store, &ctx->scal,
                    &ctx->partials, &ctx->shot_src, &ctx->shot_rec, &ctx->shot_blk, &ctx->shot_data,
                    &ctx->shot_taper, &ctx->shot_gstf})
    b->release();
  for (cudaEvent_t e : ctx->ev_pool) cudaEventDestroy(e);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return FWIGB_OK;
}

const char* fwigb_last_error(const fwigb_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

const char* fwigb_last_global_error(void) { return g_err.c_str(); }

int fwigb_geometry(const fwigb_ctx* ctx, int* nz, int* nx, int* nSteps, int* n_survey_shots, int* nrec_max) {
  if (!ctx) return FWIGB_ERR_ARG;
  if (nz) *nz = ctx->p.nz;
  if (nx) *nx = ctx->p.nx;
  if (nSteps) *nSteps = ctx->p.nSteps;
  if (n_survey_shots) *n_survey_shots = static_cast<int>(ctx->survey.size());
  if (nrec_max) *nrec_max = ctx->nrec_max;
  return FWIGB_OK;
}

int fwigb_shot_nrec(const fwigb_ctx* ctx, int shot_id, int* nrec) {
  if (!ctx || !nrec || shot_id < 0 || shot_id >= static_cast<int>(ctx->survey.size()) ||
      !ctx->survey[shot_id].present)
    return FWIGB_ERR_ARG;
  *nrec = static_cast<int>(ctx->survey[shot_id].z_rec.size());
  return FWIGB_OK;
}

int fwigb_set_model(fwigb_ctx* ctx, const double* lambda, const double* mu, const double* den) {
  if (!ctx) return FWIGB_ERR_ARG;
  std::lock_guard<std::mutex> lk(ctx->mu);
  return set_model(ctx, lambda, mu, den);
}

int fwigb_stage_shots(fwigb_ctx* ctx, const double* stf, int n_stf_rows, const int* shot_ids, int n_shots,
                      int with_obs, const float* obs) {
  if (!ctx) return FWIGB_ERR_ARG;
  std::lock_guard<std::mutex> lk(ctx->mu);
  return stage_shots(ctx, stf, n_stf_rows, shot_ids, n_shots, with_obs != 0, obs);
}

int fwigb_run(fwigb_ctx* ctx, int calc_id) {
  if (!ctx) return FWIGB_ERR_ARG;
  std::lock_guard<std::mutex> lk(ctx->mu);
  return run(ctx, calc_id);
}

int fwigb_fetch(fwigb_ctx* ctx, double* misfit, double* g_lambda, double* g_mu, double* g_den, double* g_stf,
                float* gathers) {
  if (!ctx) return FWIGB_ERR_ARG;
  std::lock_guard<std::mutex> lk(ctx->mu);
  return fetch(ctx, misfit, g_lambda, g_mu, g_den, g_stf, gathers);
}

int fwigb_synchronize(fwigb_ctx* ctx) {
  if (!ctx) return FWIGB_ERR_ARG;
  CK(cudaStreamSynchronize(ctx->stream));
  return FWIGB_OK;
}

void* fwigb_stream(fwigb_ctx* ctx) { return ctx ? static_cast<void*>(ctx->stream) : nullptr; }

long long fwigb_last_launch_count(const fwigb_ctx* ctx) { return ctx ? ctx->launches : -1; }

int fwigb_tile_config(const fwigb_ctx* ctx, int* tile_x) {
  if (!ctx || !tile_x) return FWIGB_ERR_ARG;
  for (int k = 0; k < 4; ++k) tile_x[k] = ctx->tx[k];
  return FWIGB_OK;
}

int fwigb_set_tile_config(fwigb_ctx* ctx, const int* tile_x) {
  if (!ctx) return FWIGB_ERR_ARG;
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (!tile_x) {
    ctx->autotune = true;
    ctx->tuned_fwd = ctx->tuned_bwd = false;
    return FWIGB_OK;
  }
  for (int k = 0; k < 4; ++k)
    if (tile_x[k] != 4 && tile_x[k] != 8 && tile_x[k] != 16) {
      ctx->err = "tile widths must be 4, 8 or 16";
      return FWIGB_ERR_ARG;
    }
  for (int k = 0; k < 4; ++k) ctx->tx[k] = tile_x[k];
  ctx->autotune = false;
  return FWIGB_OK;
}

int fwigb_set_kernel_timing(fwigb_ctx* ctx, int enable) {
  if (!ctx) return FWIGB_ERR_ARG;
  std::lock_guard<std::mutex> lk(ctx->mu);
  ctx->timing = enable != 0;
  return FWIGB_OK;
}

int fwigb_kernel_times(fwigb_ctx* ctx, double* total_ms, long long* launches) {
  if (!ctx || !total_ms || !launches) return FWIGB_ERR_ARG;
  std::lock_guard<std::mutex> lk(ctx->mu);
  return kernel_times(ctx, total_ms, launches);
}

int fwigb_misfit(fwigb_ctx* ctx, const double* lambda, const double* mu, const double* den, const double* stf,
                 int n_stf_rows, const int* shot_ids, int n_shots, double* misfit) {
  if (!ctx || !misfit) return FWIGB_ERR_ARG;
  std::lock_guard<std::mutex> lk(ctx->mu);
  TRY(set_model(ctx, lambda, mu, den));
  TRY(stage_shots(ctx, stf, n_stf_rows, shot_ids, n_shots, true, nullptr));
  TRY(run(ctx, 0));
  return fetch(ctx, misfit, nullptr, nullptr, nullptr, nullptr, nullptr);
}

int fwigb_misfit_grad(fwigb_ctx* ctx, const double* lambda, const double* mu, const double* den, const double* stf,
                      int n_stf_rows, const int* shot_ids, int n_shots, double* misfit, double* g_lambda,
                      double* g_mu, double* g_den, double* g_stf) {
  if (!ctx) return FWIGB_ERR_ARG;
  std::lock_guard<std::mutex> lk(ctx->mu);
  TRY(set_model(ctx, lambda, mu, den));
  TRY(stage_shots(ctx, stf, n_stf_rows, shot_ids, n_shots, true, nullptr));
  TRY(run(ctx, 1));
  return fetch(ctx, misfit, g_lambda, g_mu, g_den, g_stf, nullptr);
}

int fwigb_misfit_grad_obs(fwigb_ctx* ctx, const double* lambda, const double* mu, const double* den,
                          const double* stf, int n_stf_rows, const int* shot_ids, int n_shots, const float* obs,
                          double* misfit, double* g_lambda, double* g_mu, double* g_den, double* g_stf) {
  if (!ctx || !obs) return FWIGB_ERR_ARG;
  std::lock_guard<std::mutex> lk(ctx->mu);
  TRY(set_model(ctx, lambda, mu, den));
  TRY(stage_shots(ctx, stf, n_stf_rows, shot_ids, n_shots, true, obs));
  const bool grad = g_lambda || g_mu || g_den || g_stf;
  TRY(run(ctx, grad ? 1 : 0));
  return fetch(ctx, misfit, g_lambda, g_mu, g_den, g_stf, nullptr);
}

int fwigb_obs(fwigb_ctx* ctx, const double* lambda, const double* mu, const double* den, const double* stf,
              int n_stf_rows, const int* shot_ids, int n_shots, float* gathers, int write_files) {
  if (!ctx) return FWIGB_ERR_ARG;
  std::lock_guard<std::mutex> lk(ctx->mu);
  TRY(set_model(ctx, lambda, mu, den));
  TRY(stage_shots(ctx, stf, n_stf_rows, shot_ids, n_shots, false, nullptr));
  TRY(run(ctx, 2));
  std::vector<float> tmp;
  float* out = gathers;
  if (!out && write_files) {
    tmp.resize(ctx->staged.size() * static_cast<size_t>(ctx->nrec_max) * ctx->p.nSteps);
    out = tmp.data();
  }
  if (out) TRY(fetch(ctx, nullptr, nullptr, nullptr, nullptr, nullptr, out));
  if (write_files) TRY(write_gathers(ctx, out));
  return FWIGB_OK;
}

int fwigb_cufd(double* misfit, double* grad_Lambda, double* grad_Mu, double* grad_Den, double* grad_stf,
               const double* Lambda, const double* Mu, const double* Den, const double* stf, int calc_id, int gpu_id,
               int group_size, const int* shot_ids, const char* para_fname) {
  if (!para_fname || calc_id < 0 || calc_id > 2) {
    g_err = "bad arguments";
    return FWIGB_ERR_ARG;
  }
  // One cached context per (parameter file, device); rebuilt when the file's
  // contents change (the reference re-reads it on every call).
  static std::mutex cache_mu;
  static std::map<std::pair<std::string, int>, fwigb_ctx*> cache;
  fwigb_ctx* ctx = nullptr;
  {
    std::lock_guard<std::mutex> lk(cache_mu);
    auto key = std::make_pair(std::string(para_fname), gpu_id);
    auto it = cache.find(key);
    Params fresh;
    std::string err;
    if (!load_params(para_fname, fresh, err)) {
      g_err = err;
      return FWIGB_ERR_PARAM;
    }
    if (it != cache.end() && !(it->second->p == fresh)) {
      fwigb_destroy(it->second);
      cache.erase(it);
      it = cache.end();
    }
    if (it == cache.end()) {
      int rc = fwigb_create(para_fname, gpu_id, &ctx);
      if (rc != FWIGB_OK) return rc;
      cache[key] = ctx;
    } else {
      ctx = it->second;
      // The survey may have changed on disk; re-read it (cheap next to a run).
      std::lock_guard<std::mutex> lk2(ctx->mu);
      if (!load_survey(ctx->p, ctx->survey, ctx->nrec_max, err)) {
        g_err = err;
        return FWIGB_ERR_PARAM;
      }
    }
  }
  // The stf input has one row per survey shot in the reference's callers; the
  // rows actually read are shot_ids[i].
  int max_id = 0;
  for (int i = 0; i < group_size; ++i) max_id = std::max(max_id, shot_ids[i]);
  const int n_rows = max_id + 1;
  int rc;
  if (calc_id == 0) {
    rc = fwigb_misfit(ctx, Lambda, Mu, Den, stf, n_rows, shot_ids, group_size, misfit);
  } else if (calc_id == 1) {
    rc = fwigb_misfit_grad(ctx, Lambda, Mu, Den, stf, n_rows, shot_ids, group_size, nullptr, grad_Lambda, grad_Mu,
                           grad_Den, grad_stf);
  } else {
    rc = fwigb_obs(ctx, Lambda, Mu, Den, stf, n_rows, shot_ids, group_size, nullptr, 1);
  }
  if (rc != FWIGB_OK) g_err = ctx->err;
  return rc;
}

}  // extern "C"
