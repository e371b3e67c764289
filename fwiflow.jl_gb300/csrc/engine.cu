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
  // Optional per-shot keys of this package (the reference's parser ignores
  // them): record length "nSteps" (<= the parameter file's) and an aperture
  // window "win_x0" .. "win_x1" of interior columns. The shot then runs on
  // the sub-grid of padded columns win_x0 .. win_x1 + 2 nPml.
  int nSteps = 0;
  int x_off = 0;   // first padded column of the shot's sub-grid
  int nx = 0;      // sub-grid width
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
    g.nSteps = p.nSteps;
    if (const JValue* v = d->get("nSteps")) {
      g.nSteps = static_cast<int>(v->num);
      if (v->kind != JValue::Number || g.nSteps < 2 || g.nSteps > p.nSteps) {
        err = p.survey_fname + ": shot" + std::to_string(s) + " nSteps must be in [2, " + std::to_string(p.nSteps) +
              "]";
        return false;
      }
    }
    g.x_off = 0;
    g.nx = p.nx;
    {
      const JValue* a = d->get("win_x0");
      const JValue* b = d->get("win_x1");
      if ((a != nullptr) != (b != nullptr)) {
        err = p.survey_fname + ": shot" + std::to_string(s) + " needs both win_x0 and win_x1";
        return false;
      }
      if (a) {
        const int w0 = static_cast<int>(a->num), w1 = static_cast<int>(b->num);
        const int nxi = p.nx - 2 * p.nPml;
        if (w0 < 0 || w1 >= nxi || w1 - w0 + 1 < 6) {
          err = p.survey_fname + ": shot" + std::to_string(s) + " aperture window outside the interior or too narrow";
          return false;
        }
        g.x_off = w0;
        g.nx = w1 - w0 + 1 + 2 * p.nPml;
      }
    }
    // Source and receivers must lie inside the shot's sub-grid (away from
    // its edge by the reference's 9x9 source stencil).
    if (g.x_src - g.x_off < 4 || g.x_src - g.x_off >= g.nx - 4) {
      err = p.survey_fname + ": shot" + std::to_string(s) + " source outside its aperture window";
      return false;
    }
    for (int r = 0; r < nrec; ++r)
      if (g.x_rec[r] - g.x_off < 0 || g.x_rec[r] - g.x_off >= g.nx) {
        err = p.survey_fname + ": shot" + std::to_string(s) + " receiver outside its aperture window";
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

// Impulse response of bp_filter1d (utilities.cu:872-923 with the gains of
// cuda_bp_filter1d, :596-626) for traces of nt samples: zero padding to 2 nt,
// spectrum times amp(f)^2 (amp the sin / 1 / cos band-pass of the corners, bin
// frequencies k / (2 nt dt) in float as the kernel computes them), inverse
// transform and the 1 / (2 nt) normalisation make the filter a circular
// convolution with h[m] = (a_0 + 2 sum_{0<k<nt} a_k cos(pi k m / nt) +
// a_nt cos(pi m)) / (2 nt), a_k = amp(f_k)^2; only bins inside the band
// contribute.
static std::vector<float> bandpass_response(int nt, float dt, const float* fc) {
  const int n2 = 2 * nt;
  const float df = static_cast<float>(1.0 / dt / n2);
  std::vector<std::pair<int, double>> a;
  for (int k = 0; k <= nt; ++k) {
    const float freq = k * df;
    float amp;
    if (freq >= fc[0] && freq < fc[1])
      amp = static_cast<float>(std::sin(kPI / 2.0 * (freq - fc[0]) / (fc[1] - fc[0])));
    else if (freq >= fc[1] && freq < fc[2])
      amp = 1.0f;
    else if (freq >= fc[2] && freq < fc[3])
      amp = static_cast<float>(std::cos(kPI / 2.0 * (freq - fc[2]) / (fc[3] - fc[2])));
    else
      amp = 0.0f;
    if (amp != 0.0f) a.emplace_back(k, static_cast<double>(amp * amp));
  }
  std::vector<float> h(n2, 0.0f);
  for (int m = 0; m < n2; ++m) {
    double v = 0.0;
    for (const auto& [k, ak] : a) {
      const double w = (k == 0 || k == nt) ? 1.0 : 2.0;
      v += w * ak * std::cos(kPI * static_cast<double>(k) * m / nt);
    }
    h[m] = static_cast<float>(v / n2);
  }
  return h;
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
    if (e == cudaSuccess)
      bytes = n;
    else
      cudaGetLastError();  // a failed allocation is reported here, not by the next launch check
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



// A staged shot: its survey geometry, its sub-grid and where its data sit in
// the per-shot pools (offsets in elements).
struct ShotPlan {
  int id = 0;
  const ShotGeom* geom = nullptr;
  int nSteps = 0, nrec = 0, nx = 0, x_off = 0;
  Geo g{};              // geometry of the shot's sub-grid
  int nbin_z = 0, nbin = 0;
  size_t src_off = 0;   // floats: 2 * nSteps (szz and sxx source terms)
  size_t rec_off = 0;   // ints: 2 * nrec (sub-grid z, then x)
  size_t blk_off = 0;   // ints: nbin + 1 + nrec (receiver bins, CSR)
  size_t data_off = 0;  // floats: obs | syn | res, each nrec * nSteps
  size_t taper_off = 0; // floats: 2 * nSteps, or 2 * nrec * nSteps with per-trace windows
  size_t filt_off = 0;  // floats: the band-pass impulse response (2 * nSteps), when filtering
  size_t supd_off = 0;  // floats: source update block (supd_floats), when if_src_update
  std::vector<float> src_amp;  // tapered source wavelet (host; kept for the scratch outputs)
  size_t gstf_off = 0;  // floats: nSteps
  size_t cpmlx_off = 0; // floats: 6 * nx (CPML x profiles of the sub-grid)
  int rbz0 = 0, rbz1 = 0, rbx0 = 0, rbx1 = 0;  // receivers + source bounding box
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
  Geo geo{};  // full grid
  cudaStream_t stream = nullptr;
  size_t cells = 0;  // allocated cells of a full-grid array (ldz * nx)
  size_t ncell = 0;  // logical cells (nz * nx), the size of host arrays
  // Full-grid buffers: media, staging, CPML z profiles + full-width x
  // profiles, global gradients, scalars, reduction partials.
  DevBuf media, stage, cpml, grads, scal, partials;
  // Staged shots and their data.
  std::vector<ShotPlan> plans;
  DevBuf shot_src, shot_rec, shot_blk, shot_data, shot_taper, shot_gstf, shot_cpmlx;
  DevBuf shot_filt, filt_tmp;  // band-pass impulse responses; two trace-block scratch buffers
  DevBuf scratch_tmp;          // conditioned observed data of the scratch outputs
  // Source-wavelet update: per-shot blocks (taper, wavelet, twiddles, updated
  // wavelet and its reverse source terms) and per-call spectra partial sums,
  // coefficients and impulse response (reused shot after shot).
  DevBuf shot_supd, supd_part, supd_coef, supd_k;
  size_t filt_tmp_floats = 0;
  bool with_obs = false;
  bool per_trace_taper = false;
  int nSteps_max = 0;  // longest staged record
  // Shot groups run concurrently; group state is per member slot.
  int max_batch = 0;      // cap on shots per group (0: memory budget only)
  size_t mem_budget = 0;  // bytes for group state (0: 90% of free device memory)
  size_t fields_stride = 0, store_stride = 0, grads_stride = 0;  // floats per member
  DevBuf g_fields, g_store, g_grads, g_slots;
  int group_cap = 0;
  // Launch parameter packs of the current group: for a lone shot one
  // SweepPack<1> per (sweep variant, tile width); else one
  // SweepPack<kPackShots> per (sweep variant, tile width, pack of consecutive
  // members), index (variant * 3 + tile slot) * npacks + pack. pack_nx[q] is
  // the widest member sub-grid of pack q.
  int group_size = 0, npacks = 0;
  std::vector<SweepPack<1>> pack1;
  std::vector<SweepPack<kPackShots>> packs;
  std::vector<int> pack_nx;
  // Launch extents per pack.
  std::vector<SweepGrid> pack_grid;
  int last_groups = 0;
  // CUDA graph of a single-group call's whole launch sequence, replayed while
  // everything it was captured from is unchanged (graph_key).
  bool use_graphs = true;
  cudaGraphExec_t graph_exec = nullptr;
  std::vector<uint64_t> graph_key;
  long long graph_launches = 0;
  bool illum = false;       // accumulate the source illumination in the runs
  bool illum_valid = false; // the last run accumulated it
  bool model_set = false;
  int last_calc = -1;
  long long launches = 0;
  int tx[4] = {8, 8, 8, 8};    // tile width per sweep (F1, F2, B, C)
  int rows[4] = {2, 2, 1, 1};  // depths per thread per sweep (1 or 2)
  int regs[4] = {32, 32, 32, 32};  // register budget of the backward sweeps' one-row tiles (32 or 40)
  bool tuned_fwd = false, tuned_bwd = false;
  bool autotune = true;
  // Timeout test hook: the first forward sweep of every run lets its bounded
  // wait run out (after its tiles have landed), so the run ends in
  // FWIGB_ERR_TIMEOUT.
  bool inject_timeout = false;
  // per-kernel event timing
  bool timing = false;
  std::vector<cudaEvent_t> ev_pool;
  std::vector<int> ev_kind;
};

namespace {

thread_local std::string g_err;

#define CK(call)                                                                                   \
  do {                                                                                             \
    cudaError_t e_ = (call);                                                                       \
    if (e_ != cudaSuccess) {                                                                       \
      ctx->err = std::string(#call) + ": " + cudaGetErrorString(e_);                               \
      return (e_ == cudaErrorMemoryAllocation) ? FWIGB_ERR_OOM : FWIGB_ERR_CUDA;                   \
    }                                                                                              \
  } while (0)

#define TRY_RC(call)                 \
  do {                               \
    int rc_ = (call);                \
    if (rc_ != FWIGB_OK) return rc_; \
  } while (0)

int tx_slot(int tx) { return tx == 4 ? 0 : (tx == 8 ? 1 : 2); }

// Media slots: lam, mu, den, l2m, aveMu, bycA, bycB, hs, muw (full grid).
MediaD media_view(fwigb_ctx* ctx, int x_off) {
  float* b = ctx->media.as<float>() + static_cast<size_t>(x_off) * ctx->geo.ldz;
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

// Geometry of a grid of width nx (the full grid or a shot's sub-grid) with
// the CPML profiles az/azh (z) and ax/axh (x) of that grid.
// Geometry of a (sub-)grid of width nx. zprof / xprof are the CPML profile
// blocks (K, a, b, K_half, a_half, b_half; nz resp. nx floats each).
Geo make_geo(const Params& p, int nx, const float* zprof, const float* xprof) {
  const float* az = zprof + p.nz;
  const float* azh = zprof + 4 * p.nz;
  const float* ax = xprof + nx;
  const float* axh = xprof + 4 * nx;
  Geo g{};
  g.nz = p.nz;
  g.nx = nx;
  g.ldz = (p.nz + 31) / 32 * 32;
  g.nPml = p.nPml;
  g.nPad = p.nPad;
  g.zs0 = 2;
  g.zs1 = p.nz - p.nPad - 3;
  g.xs0 = 2;
  g.xs1 = nx - 3;
  g.zi0 = p.nPml;
  g.zi1 = p.nz - p.nPad - 1 - p.nPml;
  g.xi0 = p.nPml;
  g.xi1 = nx - 1 - p.nPml;
  g.zpml_hi = p.nz - p.nPml - p.nPad - 1;
  g.xpml_hi_s = nx - p.nPml - 1;
  g.xpml_hi_v = nx - p.nPml;
  g.rz0 = p.nPml - 2;
  g.rz1 = p.nz - p.nPml - p.nPad + 1;
  g.rx0 = p.nPml - 2;
  g.rx1 = nx - p.nPml + 1;
  g.ringW = g.rx1 - g.rx0 + 1;
  g.ringH = g.rz1 - g.rz0 + 1 - 10;
  g.ring_len = 10 * g.ringW + 10 * g.ringH;
  g.dt = p.dt;
  g.rdz = 1.0f / p.dz;
  g.rdx = 1.0f / p.dx;
  g.zact1 = std::max(g.zs1, g.rz1);
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
  band(az, azh, p.nz - p.nPad, g.zband_lo, g.zband_hi);
  band(ax, axh, nx, g.xband_lo, g.xband_hi);
  // Fast box: the longest run of indices where every condition of the fast
  // sweeps holds (an empty box when none does).
  auto run = [](int n, auto ok, int& lo, int& hi) {
    lo = 1;
    hi = 0;
    int best = 0;
    for (int i = 0; i < n;) {
      if (!ok(i)) {
        ++i;
        continue;
      }
      int j = i;
      while (j + 1 < n && ok(j + 1)) ++j;
      if (j - i + 1 > best) {
        best = j - i + 1;
        lo = i;
        hi = j;
      }
      i = j + 1;
    }
  };
  const float* Kz = zprof;
  const float* Kzh = zprof + 3 * p.nz;
  const float* Kx = xprof;
  const float* Kxh = xprof + 3 * nx;
  run(p.nz, [&](int z) {
    return z >= g.zs0 && z <= g.zs1 && z >= g.nPml && z <= g.zpml_hi && z > g.zband_lo && z < g.zband_hi &&
           z >= g.zi0 + 1 && z <= g.zi1 && z >= g.rz0 + 5 && z <= g.rz1 - 5 && Kz[z] == 1.0f && Kzh[z] == 1.0f &&
           az[z] == 0.0f && azh[z] == 0.0f;
  }, g.fz0, g.fz1);
  run(nx, [&](int x) {
    return x >= g.xs0 && x <= g.xs1 && x >= g.nPml && x <= g.xpml_hi_s && x <= g.xpml_hi_v && x > g.xband_lo &&
           x < g.xband_hi && x >= g.xi0 + 1 && x <= g.xi1 && x >= g.rx0 + 5 && x <= g.rx1 - 5 && Kx[x] == 1.0f &&
           Kxh[x] == 1.0f && ax[x] == 0.0f && axh[x] == 0.0f;
  }, g.fx0, g.fx1);
  // Mid box: stencil domain without any CPML cell (K = 1, a = 0); it holds
  // the fast box plus the ring, band and interior-guard cells next to it.
  run(p.nz, [&](int z) {
    return z >= g.zs0 && z <= g.zs1 && z >= g.nPml && z <= g.zpml_hi && Kz[z] == 1.0f && Kzh[z] == 1.0f &&
           az[z] == 0.0f && azh[z] == 0.0f;
  }, g.mz0, g.mz1);
  run(nx, [&](int x) {
    return x >= g.xs0 && x <= g.xs1 && x >= g.nPml && x <= g.xpml_hi_s && x <= g.xpml_hi_v && Kx[x] == 1.0f &&
           Kxh[x] == 1.0f && ax[x] == 0.0f && axh[x] == 0.0f;
  }, g.mx0, g.mx1);
  if (g.fz0 <= g.fz1 && g.fx0 <= g.fx1 &&
      !(g.mz0 <= g.fz0 && g.fz1 <= g.mz1 && g.mx0 <= g.fx0 && g.fx1 <= g.mx1)) {
    g.mz0 = g.fz0;  // (never on the reference's grids) no mid tiles
    g.mz1 = g.fz1;
    g.mx0 = g.fx0;
    g.mx1 = g.fx1;
  }
  return g;
}

int setup_geometry(fwigb_ctx* ctx) {
  const Params& p = ctx->p;
  // CPML profiles: z (length nz, profile over nz - nPad, Cpml.cu:46-48) and x
  // of the full width; shots with an aperture window get their own x profiles.
  std::vector<float> h(6 * p.nz + 6 * p.nx);
  float* z = h.data();
  float* x = h.data() + 6 * p.nz;
  cpml_profile(p.nz - p.nPad, p.nz, p.nPml, p.dz, p.f0, p.dt, z, z + p.nz, z + 2 * p.nz, z + 3 * p.nz, z + 4 * p.nz,
               z + 5 * p.nz);
  cpml_profile(p.nx, p.nx, p.nPml, p.dx, p.f0, p.dt, x, x + p.nx, x + 2 * p.nx, x + 3 * p.nx, x + 4 * p.nx,
               x + 5 * p.nx);
  ctx->geo = make_geo(p, p.nx, z, x);
  ctx->cells = static_cast<size_t>(ctx->geo.ldz) * p.nx;
  ctx->ncell = static_cast<size_t>(p.nz) * p.nx;
  CK(ctx->cpml.ensure(h.size() * sizeof(float)));
  CK(cudaMemcpy(ctx->cpml.p, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice));
  CK(ctx->media.ensure(9 * ctx->cells * sizeof(float)));
  CK(cudaMemset(ctx->media.p, 0, 9 * ctx->cells * sizeof(float)));
  CK(ctx->stage.ensure(3 * ctx->ncell * sizeof(double)));
  CK(ctx->grads.ensure(4 * ctx->cells * sizeof(float)));  // lambda, mu, den, illumination
  // [0]: misfit accumulator (double), [8]: cp max bits, [16]: sweep error word
  CK(ctx->scal.ensure(64));
  CK(cudaMemset(ctx->scal.p, 0, 64));
  CK(ctx->partials.ensure(1024 * sizeof(double)));
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

// Drops a non-sticky error that an earlier, unrelated CUDA call of this host
// thread left behind (a failed allocation, say), so that this call's own
// launch checks report only this call's failures. Sticky errors (a corrupted
// context) persist and are still reported by the next call that fails.
void clear_stale_error() { cudaGetLastError(); }

int set_model(fwigb_ctx* ctx, const double* lam, const double* mu, const double* den) {
  if (!lam || !mu || !den) {
    ctx->err = "null model array";
    return FWIGB_ERR_ARG;
  }
  CK(cudaSetDevice(ctx->device));
  clear_stale_error();
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

// Per-shot block of the source-wavelet update (floats, 16-byte multiple):
// [w2: nt][wavelet: nt][twiddles (cos, sin)(2 pi k / 2 nt): 2 * 2 nt]
// [updated wavelet: nt][its szz terms: nt][its sxx terms: nt].
struct SupdLayout {
  size_t w2, amp, tw, upd, szz, sxx, size;
  explicit SupdLayout(int nt) {
    const size_t n = static_cast<size_t>(nt);
    w2 = 0;
    amp = n;
    tw = 2 * n;
    upd = 6 * n;
    szz = 7 * n;
    sxx = 8 * n;
    size = (9 * n + 3) / 4 * 4;
  }
};

int stage_shots(fwigb_ctx* ctx, const double* stf, int n_stf_rows, const int* shot_ids, int n_shots, bool with_obs,
                const float* obs) {
  const Params& p = ctx->p;
  if (!stf || !shot_ids || n_shots < 1 || n_stf_rows < 1) {
    ctx->err = "stf / shot_ids missing";
    return FWIGB_ERR_ARG;
  }
  CK(cudaSetDevice(ctx->device));
  const int nt_max = p.nSteps, nrm = ctx->nrec_max;
  ctx->plans.clear();
  size_t n_src = 0, n_rec = 0, n_blk = 0, n_data = 0, n_taper = 0, n_gstf = 0, n_cpmlx = 0, n_supd = 0;
  for (int k = 0; k < n_shots; ++k) {
    const int id = shot_ids[k];
    if (id < 0 || id >= static_cast<int>(ctx->survey.size()) || !ctx->survey[id].present) {
      ctx->err = "shot id " + std::to_string(id) + " not in the survey file";
      return FWIGB_ERR_ARG;
    }
    if (id >= n_stf_rows) {
      ctx->err = "shot id " + std::to_string(id) + " has no stf row";
      return FWIGB_ERR_ARG;
    }
    const ShotGeom& sg = ctx->survey[id];
    ShotPlan pl;
    pl.id = id;
    pl.geom = &sg;
    pl.nSteps = sg.nSteps;
    pl.nrec = static_cast<int>(sg.z_rec.size());
    pl.nx = sg.nx;
    pl.x_off = sg.x_off;
    pl.nbin_z = (p.nz + kBinZ - 1) / kBinZ;
    pl.nbin = pl.nbin_z * ((pl.nx + kBinX - 1) / kBinX);
    pl.src_off = n_src;
    n_src += 2 * static_cast<size_t>(pl.nSteps);
    pl.rec_off = n_rec;
    n_rec += 2 * static_cast<size_t>(pl.nrec);
    pl.blk_off = n_blk;
    n_blk += static_cast<size_t>(pl.nbin) + 1 + pl.nrec;
    pl.data_off = n_data;
    n_data += 3 * static_cast<size_t>(pl.nrec) * pl.nSteps;
    pl.taper_off = n_taper;
    n_taper += 2 * static_cast<size_t>(pl.nSteps) * (p.if_win ? pl.nrec : 1);
    pl.gstf_off = n_gstf;
    n_gstf += static_cast<size_t>(pl.nSteps);
    if (p.if_src_update) {
      if (pl.nSteps > 32768) {  // f * t of the spectra stays below 2^32
        ctx->err = "the source update takes records of at most 32768 steps";
        return FWIGB_ERR_ARG;
      }
      pl.supd_off = n_supd;
      n_supd += SupdLayout(pl.nSteps).size;
    }
    pl.cpmlx_off = n_cpmlx;
    n_cpmlx += 6 * static_cast<size_t>(pl.nx);
    ctx->plans.push_back(pl);
  }
  // Band-pass impulse responses, one per distinct record length.
  std::vector<float> hfilt;
  size_t tmp_need = 0;
  if (p.if_filter || p.if_src_update)
    for (const ShotPlan& pl : ctx->plans) tmp_need = std::max(tmp_need, static_cast<size_t>(pl.nrec) * pl.nSteps);
  if (p.if_filter) {
    std::map<int, size_t> at;
    for (ShotPlan& pl : ctx->plans) {
      auto it = at.find(pl.nSteps);
      if (it == at.end()) {
        it = at.emplace(pl.nSteps, hfilt.size()).first;
        const std::vector<float> h = bandpass_response(pl.nSteps, p.dt, p.filter);
        hfilt.insert(hfilt.end(), h.begin(), h.end());
      }
      pl.filt_off = it->second;
    }
  }
  std::vector<float> hsrc(n_src), htaper(n_taper, 1.0f), hcpml(n_cpmlx), hsupd(n_supd, 0.0f);
  std::vector<int> hrec(n_rec), hblk(n_blk, 0);
  const float* zprof = nullptr;
  std::vector<float> zh(6 * p.nz);
  cpml_profile(p.nz - p.nPad, p.nz, p.nPml, p.dz, p.f0, p.dt, zh.data(), zh.data() + p.nz, zh.data() + 2 * p.nz,
               zh.data() + 3 * p.nz, zh.data() + 4 * p.nz, zh.data() + 5 * p.nz);
  zprof = zh.data();
  const float scale = 2250000.0f;  // pow(1500.0, 2) (utilities.cu:528)
  ctx->nSteps_max = 0;
  for (ShotPlan& pl : ctx->plans) {
    const int nt = pl.nSteps;
    ctx->nSteps_max = std::max(ctx->nSteps_max, nt);
    // CPML x profiles of the sub-grid and its geometry.
    float* x = hcpml.data() + pl.cpmlx_off;
    cpml_profile(pl.nx, pl.nx, p.nPml, p.dx, p.f0, p.dt, x, x + pl.nx, x + 2 * pl.nx, x + 3 * pl.nx, x + 4 * pl.nx,
                 x + 5 * pl.nx);
    pl.g = make_geo(p, pl.nx, zprof, x);
    // Source: taper 0.001 (Src_Rec.cu:140) and the add_source scale (utilities.cu:528-538).
    std::vector<float> w(nt);
    if (!taper_weights(nt, p.dt, 0.001f, w.data())) {
      ctx->err = "nSteps too small for the source taper";
      return FWIGB_ERR_ARG;
    }
    const double* row = stf + static_cast<size_t>(pl.id) * nt_max;
    pl.src_amp.assign(nt, 0.0f);
    for (int it = 0; it < nt; ++it) {
      const float amp = static_cast<float>(row[it]) * w[it];
      pl.src_amp[it] = amp;
      hsrc[pl.src_off + it] = scale * amp * p.dt;
      hsrc[pl.src_off + nt + it] = static_cast<float>(3.0 * scale * amp * p.dt);
    }
    if (p.if_src_update) {
      // Taper of the padded traces (cuda_window over 2 nt, ratio 0.01,
      // utilities.cu:955-958), the wavelet and the transform's twiddles.
      const SupdLayout L(nt);
      float* b = hsupd.data() + pl.supd_off;
      std::vector<float> w2(2 * static_cast<size_t>(nt));
      taper_weights(2 * nt, p.dt, 0.01f, w2.data());
      std::copy(w2.begin(), w2.begin() + nt, b + L.w2);
      std::copy(pl.src_amp.begin(), pl.src_amp.end(), b + L.amp);
      const double two_pi = 6.283185307179586476925286766559;
      for (int k = 0; k < 2 * nt; ++k) {
        b[L.tw + 2 * k] = static_cast<float>(std::cos(two_pi * k / (2.0 * nt)));
        b[L.tw + 2 * k + 1] = static_cast<float>(std::sin(two_pi * k / (2.0 * nt)));
      }
    }
    // Receivers (sub-grid coordinates) and their 32 x 8 bins.
    const ShotGeom& g = *pl.geom;
    int* rz = hrec.data() + pl.rec_off;
    int* rx = rz + pl.nrec;
    int* off = hblk.data() + pl.blk_off;
    int* lst = off + pl.nbin + 1;
    std::vector<int> cnt(pl.nbin + 1, 0);
    // Bounding box of the receivers and the source (sub-grid cells).
    pl.rbz0 = pl.rbz1 = g.z_src;
    pl.rbx0 = pl.rbx1 = g.x_src - pl.x_off;
    for (int r = 0; r < pl.nrec; ++r) {
      rz[r] = g.z_rec[r];
      rx[r] = g.x_rec[r] - pl.x_off;
      cnt[(rz[r] / kBinZ) + (rx[r] / kBinX) * pl.nbin_z + 1]++;
      pl.rbz0 = std::min(pl.rbz0, rz[r]);
      pl.rbz1 = std::max(pl.rbz1, rz[r]);
      pl.rbx0 = std::min(pl.rbx0, rx[r]);
      pl.rbx1 = std::max(pl.rbx1, rx[r]);
    }
    for (int b = 0; b < pl.nbin; ++b) cnt[b + 1] += cnt[b];
    for (int b = 0; b <= pl.nbin; ++b) off[b] = cnt[b];
    std::vector<int> pos(cnt.begin(), cnt.end() - 1);
    for (int r = 0; r < pl.nrec; ++r) lst[pos[(rz[r] / kBinZ) + (rx[r] / kBinX) * pl.nbin_z]++] = r;
    // Taper weights of the data and of the adjoint source.
    float* tw = htaper.data() + pl.taper_off;
    if (!p.if_win) {
      if (!taper_weights(nt, p.dt, 0.005f, tw)) {
        ctx->err = "nSteps too small for the data taper";
        return FWIGB_ERR_ARG;
      }
      std::copy(tw, tw + nt, tw + nt);
    } else {
      const size_t per = static_cast<size_t>(pl.nrec) * nt;
      for (int r = 0; r < pl.nrec; ++r) {
        taper_weights_windowed(nt, p.dt, 0.005f, g.win_start[r], g.win_end[r], g.weights[r], tw + r * nt);
        taper_weights_windowed(nt, p.dt, 0.1f, g.win_start[r], g.win_end[r], g.weights[r], tw + per + r * nt);
      }
    }
  }
  ctx->per_trace_taper = p.if_win;
  CK(ctx->shot_src.ensure(std::max<size_t>(n_src, 1) * sizeof(float)));
  CK(ctx->shot_rec.ensure(std::max<size_t>(n_rec, 1) * sizeof(int)));
  CK(ctx->shot_blk.ensure(std::max<size_t>(n_blk, 1) * sizeof(int)));
  CK(ctx->shot_data.ensure(std::max<size_t>(n_data, 1) * sizeof(float)));
  CK(ctx->shot_taper.ensure(std::max<size_t>(n_taper, 1) * sizeof(float)));
  CK(ctx->shot_gstf.ensure(std::max<size_t>(n_gstf, 1) * sizeof(float)));
  CK(ctx->shot_cpmlx.ensure(std::max<size_t>(n_cpmlx, 1) * sizeof(float)));
  cudaStream_t s = ctx->stream;
  CK(cudaMemcpyAsync(ctx->shot_src.p, hsrc.data(), n_src * sizeof(float), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(ctx->shot_rec.p, hrec.data(), n_rec * sizeof(int), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(ctx->shot_blk.p, hblk.data(), n_blk * sizeof(int), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(ctx->shot_taper.p, htaper.data(), n_taper * sizeof(float), cudaMemcpyHostToDevice, s));
  if (p.if_filter) {
    CK(ctx->shot_filt.ensure(hfilt.size() * sizeof(float)));
    CK(cudaMemcpyAsync(ctx->shot_filt.p, hfilt.data(), hfilt.size() * sizeof(float), cudaMemcpyHostToDevice, s));
  }
  if (p.if_filter || p.if_src_update) {
    CK(ctx->filt_tmp.ensure(2 * tmp_need * sizeof(float)));
    ctx->filt_tmp_floats = tmp_need;
  }
  if (p.if_src_update) {
    int nt_big = 1, nb_big = 1;
    for (const ShotPlan& pl : ctx->plans) {
      nt_big = std::max(nt_big, pl.nSteps);
      nb_big = std::max(nb_big, src_spectra_blocks(pl.nrec));
    }
    CK(ctx->shot_supd.ensure(n_supd * sizeof(float)));
    CK(cudaMemcpyAsync(ctx->shot_supd.p, hsupd.data(), n_supd * sizeof(float), cudaMemcpyHostToDevice, s));
    CK(ctx->supd_part.ensure(static_cast<size_t>(nb_big) * 3 * (nt_big + 1) * sizeof(float)));
    CK(ctx->supd_coef.ensure(static_cast<size_t>(nt_big + 1) * sizeof(float2)));
    CK(ctx->supd_k.ensure(2 * static_cast<size_t>(nt_big) * sizeof(float)));
  }
  CK(cudaMemcpyAsync(ctx->shot_cpmlx.p, hcpml.data(), n_cpmlx * sizeof(float), cudaMemcpyHostToDevice, s));
  ctx->with_obs = with_obs;
  if (with_obs) {
    // Observed data: from memory ([n_shots][nrec_max][nSteps] with shot k's
    // [nrec][nSteps_k] block in its top-left corner) or from
    // data_dir_name/Shot<id>.bin ([nrec][nSteps_k] float, libCUFD.cu:189-200).
    std::vector<float> buf;
    for (size_t k = 0; k < ctx->plans.size(); ++k) {
      const ShotPlan& pl = ctx->plans[k];
      float* d_obs = ctx->shot_data.as<float>(pl.data_off);
      if (obs) {
        CK(cudaMemcpy2DAsync(d_obs, pl.nSteps * sizeof(float), obs + k * static_cast<size_t>(nrm) * nt_max,
                             nt_max * sizeof(float), pl.nSteps * sizeof(float), pl.nrec, cudaMemcpyHostToDevice, s));
      } else {
        const std::string fn = p.data_dir_name + "/Shot" + std::to_string(pl.id) + ".bin";
        std::FILE* fp = std::fopen(fn.c_str(), "rb");
        if (!fp) {
          ctx->err = "cannot read " + fn;
          return FWIGB_ERR_IO;
        }
        const size_t want = static_cast<size_t>(pl.nrec) * pl.nSteps;
        buf.resize(want);
        const size_t got = std::fread(buf.data(), sizeof(float), want, fp);
        std::fclose(fp);
        if (got != want) {
          ctx->err = fn + " is shorter than nrec*nSteps";
          return FWIGB_ERR_IO;
        }
        CK(cudaMemcpy(d_obs, buf.data(), want * sizeof(float), cudaMemcpyHostToDevice));
      }
    }
  }
  CK(cudaStreamSynchronize(s));  // host staging vectors go out of scope
  return FWIGB_OK;
}

// Shot groups for one run: shots sorted by record length (longest first) and
// cut into groups of at most group_cap members, which run concurrently.
// group_cap follows the device-memory budget of the group state (fields,
// gradients and, with the adjoint, the boundary store of every member).
int plan_groups(fwigb_ctx* ctx, bool adj, std::vector<std::vector<int>>& groups) {
  const Params& p = ctx->p;
  int nx_max = 0, ring_max = 0;
  for (const ShotPlan& pl : ctx->plans) {
    nx_max = std::max(nx_max, pl.nx);
    ring_max = std::max(ring_max, pl.g.ring_len);
  }
  const size_t ldz = ctx->geo.ldz;
  ctx->fields_stride = 18 * ldz * nx_max;
  ctx->grads_stride = (ctx->illum ? 4 : 3) * ldz * nx_max;
  ctx->store_stride = adj ? static_cast<size_t>(ctx->nSteps_max) * 5 * ring_max : 0;
  const size_t per_member = (ctx->fields_stride + ctx->grads_stride + ctx->store_stride) * sizeof(float);
  size_t budget = ctx->mem_budget;
  if (!budget) {
    size_t free_b = 0, total_b = 0;
    CK(cudaMemGetInfo(&free_b, &total_b));
    // Memory the group state already holds is reusable.
    free_b += ctx->g_fields.bytes + ctx->g_grads.bytes + ctx->g_store.bytes;
    budget = static_cast<size_t>(0.9 * static_cast<double>(free_b));
  }
  int cap = static_cast<int>(std::min<size_t>(budget / std::max<size_t>(per_member, 1), 1u << 16));
  if (ctx->max_batch > 0) cap = std::min(cap, ctx->max_batch);
  cap = std::min(cap, static_cast<int>(ctx->plans.size()));
  if (cap < 1) {
    ctx->err = "one shot's wavefields and boundary store do not fit in device memory";
    return FWIGB_ERR_OOM;
  }
  std::vector<int> order(ctx->plans.size());
  for (size_t k = 0; k < order.size(); ++k) order[k] = static_cast<int>(k);
  std::stable_sort(order.begin(), order.end(),
                   [&](int a, int b) { return ctx->plans[a].nSteps > ctx->plans[b].nSteps; });
  groups.clear();
  for (size_t k = 0; k < order.size(); k += cap)
    groups.emplace_back(order.begin() + k, order.begin() + std::min(order.size(), k + cap));
  ctx->group_cap = cap;
  (void)p;
  CK(ctx->g_fields.ensure(static_cast<size_t>(cap) * ctx->fields_stride * sizeof(float)));
  CK(ctx->g_grads.ensure(static_cast<size_t>(cap) * ctx->grads_stride * sizeof(float)));
  if (adj) CK(ctx->g_store.ensure(static_cast<size_t>(cap) * ctx->store_stride * sizeof(float)));
  CK(ctx->g_slots.ensure(static_cast<size_t>(cap) * sizeof(ShotSlot)));
  return FWIGB_OK;
}

// Launches sweep `w` (0 F1, 1 F2, 2 B, 3 C) with `rows` depths per thread
// (forward sweeps: 1 or 2) over the first `a` members of the current group at
// tile width tx, one launch per parameter pack; `arg` is the step (F1) or the
// backward iteration (B, C); `flags` those of launch_fwd_stress (F1 only).
// Returns the number of launches.
int launch_sweep(fwigb_ctx* ctx, int w, int tx, int rows, int a, int arg, int flags, unsigned* d_err) {
  cudaStream_t s = ctx->stream;
  const int variant = rows == 2 ? w + 4 : w;
  const size_t base = static_cast<size_t>(variant * 3 + tx_slot(tx));
  auto go = [&](const auto& pk, int n, const SweepGrid& gr) {
    switch (w) {
      case 0: return launch_fwd_stress(s, tx, rows, pk, n, gr, arg, flags, d_err);
      case 1: return launch_fwd_velocity(s, tx, rows, pk, n, gr, d_err);
      case 2: return launch_bwd_B(s, tx, rows, ctx->regs[2], pk, n, gr, arg, d_err);
      default: return launch_bwd_C(s, tx, rows, ctx->regs[3], pk, n, gr, arg, d_err);
    }
  };
  if (a <= 0) return 0;
  const SweepGrid* grids = ctx->pack_grid.data();
  if (ctx->group_size == 1) return go(ctx->pack1[base], 1, grids[0]);
  int n = 0;
  for (int q = 0; q * kPackShots < a; ++q)
    n += go(ctx->packs[base * ctx->npacks + q], std::min(kPackShots, a - q * kPackShots), grids[q]);
  return n;
}

// Builds and uploads the slots and tensor maps of a group's members.
int build_group(fwigb_ctx* ctx, const std::vector<int>& members, int& nx_max) {
  const size_t ldz = ctx->geo.ldz;
  std::vector<ShotSlot> slots(members.size());
  std::vector<TileMaps> maps(static_cast<size_t>(kSweepVariants * 3) * ctx->group_cap);
  const int nrm = 0;
  (void)nrm;
  nx_max = 0;
  const float* cz = ctx->cpml.as<float>();
  const int nz = ctx->p.nz;
  for (size_t k = 0; k < members.size(); ++k) {
    const ShotPlan& pl = ctx->plans[members[k]];
    nx_max = std::max(nx_max, pl.nx);
    ShotSlot& sl = slots[k];
    sl.g = pl.g;
    const size_t n = ldz * pl.nx;
    float* fb = ctx->g_fields.as<float>(k * ctx->fields_stride);
    float** f[18] = {&sl.f.vz,       &sl.f.vx,       &sl.f.szz,       &sl.f.sxx,       &sl.f.sxz,
                     &sl.f.vz_a,     &sl.f.vx_a,     &sl.f.szz_a,     &sl.f.sxx_a,     &sl.f.sxz_a,
                     &sl.f.m_dvz_dz, &sl.f.m_dvz_dx, &sl.f.m_dvx_dz,  &sl.f.m_dvx_dx,  &sl.f.m_dszz_dz,
                     &sl.f.m_dsxx_dx, &sl.f.m_dsxz_dz, &sl.f.m_dsxz_dx};
    for (int q = 0; q < 18; ++q) *f[q] = fb + q * n;
    sl.m = media_view(ctx, pl.x_off);
    const float* cx = ctx->shot_cpmlx.as<float>(pl.cpmlx_off);
    sl.c = CpmlD{cz,      cz + nz,      cz + 2 * nz,      cz + 3 * nz,      cz + 4 * nz,      cz + 5 * nz,
                 cx,      cx + pl.nx,   cx + 2 * pl.nx,   cx + 3 * pl.nx,   cx + 4 * pl.nx,   cx + 5 * pl.nx};
    ShotD& sh = sl.sh;
    sh.src_z = pl.geom->z_src;
    sh.src_x = pl.geom->x_src - pl.x_off;
    sh.src_szz = ctx->shot_src.as<float>(pl.src_off);
    sh.src_sxx = sh.src_szz + pl.nSteps;
    if (ctx->p.if_src_update) {
      const SupdLayout L(pl.nSteps);
      sh.src_szz_r = ctx->shot_supd.as<float>(pl.supd_off + L.szz);
      sh.src_sxx_r = ctx->shot_supd.as<float>(pl.supd_off + L.sxx);
    } else {
      sh.src_szz_r = sh.src_szz;
      sh.src_sxx_r = sh.src_sxx;
    }
    sh.nrec = pl.nrec;
    sh.nSteps = pl.nSteps;
    sh.rec_z = ctx->shot_rec.as<int>(pl.rec_off);
    sh.rec_x = sh.rec_z + pl.nrec;
    sh.blk_off = ctx->shot_blk.as<int>(pl.blk_off);
    sh.blk_rec = sh.blk_off + pl.nbin + 1;
    sh.nbin_z = pl.nbin_z;
    sh.rbz0 = pl.rbz0;
    sh.rbz1 = pl.rbz1;
    sh.rbx0 = pl.rbx0;
    sh.rbx1 = pl.rbx1;
    const size_t per = static_cast<size_t>(pl.nrec) * pl.nSteps;
    sh.data = ctx->shot_data.as<float>(pl.data_off + per);
    sh.res = ctx->shot_data.as<float>(pl.data_off + 2 * per);
    sh.gstf = ctx->shot_gstf.as<float>(pl.gstf_off);
    sl.st = StoreD{ctx->store_stride ? ctx->g_store.as<float>(k * ctx->store_stride) : nullptr};
    float* gb = ctx->g_grads.as<float>(k * ctx->grads_stride);
    sl.gr = Grads{gb, gb + n, gb + 2 * n, ctx->illum ? gb + 3 * n : nullptr};
    sl.nSteps = pl.nSteps;
    sl.x_off = pl.x_off;
    for (int t = 0; t < 3; ++t) {
      SweepMaps sm{};
      const char* why = nullptr;
      if (!encode_sweep_maps(pl.g, sl.f, kTileXs[t], sm, &why)) {
        ctx->err = why;
        return FWIGB_ERR_CUDA;
      }
      const TileMaps* per_sweep[kSweepVariants] = {&sm.f1, &sm.f2, &sm.b, &sm.c, &sm.f1w, &sm.f2w, &sm.bw, &sm.cw};
      for (int w = 0; w < kSweepVariants; ++w)
        maps[static_cast<size_t>(w * 3 + t) * ctx->group_cap + k] = *per_sweep[w];
    }
  }
  // Parameter packs (host; passed by value at every launch).
  const int G = static_cast<int>(members.size());
  ctx->group_size = G;
  ctx->npacks = (G + kPackShots - 1) / kPackShots;
  ctx->pack_nx.assign(ctx->npacks, 0);
  for (int k = 0; k < G; ++k) ctx->pack_nx[k / kPackShots] = std::max(ctx->pack_nx[k / kPackShots], slots[k].g.nx);
  // Launch extents: the widest member sub-grid, and rows down to the last
  // one a sweep touches (zact1, or the lowest source / receiver row).
  ctx->pack_grid.assign(ctx->npacks, SweepGrid{0, 0});
  for (int q = 0; q < ctx->npacks; ++q) ctx->pack_grid[q].nx = ctx->pack_nx[q];
  for (int k = 0; k < G; ++k) {
    const int rows = std::min(slots[k].g.nz, std::max(slots[k].g.zact1, slots[k].sh.rbz1) + 1);
    ctx->pack_grid[k / kPackShots].nz = std::max(ctx->pack_grid[k / kPackShots].nz, rows);
  }
  if (G == 1) {
    ctx->pack1.assign(kSweepVariants * 3, SweepPack<1>{});
    for (int w = 0; w < kSweepVariants * 3; ++w) {
      ctx->pack1[w].maps[0] = maps[static_cast<size_t>(w) * ctx->group_cap];
      ctx->pack1[w].slots[0] = slots[0];
    }
  } else {
    ctx->packs.assign(static_cast<size_t>(kSweepVariants * 3) * ctx->npacks, SweepPack<kPackShots>{});
    for (int w = 0; w < kSweepVariants * 3; ++w)
      for (int k = 0; k < G; ++k) {
        SweepPack<kPackShots>& pk = ctx->packs[static_cast<size_t>(w) * ctx->npacks + k / kPackShots];
        pk.maps[k % kPackShots] = maps[static_cast<size_t>(w) * ctx->group_cap + k];
        pk.slots[k % kPackShots] = slots[k];
      }
  }
  // Device copy of the slots for the gradient reduction.
  CK(cudaMemcpyAsync(ctx->g_slots.p, slots.data(), slots.size() * sizeof(ShotSlot), cudaMemcpyHostToDevice,
                     ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return FWIGB_OK;
}

// Tile autotuner: times every candidate tile of each sweep on the first
// group of the first run (on its live buffers, which the run then resets) and
// keeps the fastest: widths 4, 8, 16 for every sweep, times 1 or 2 depths per
// thread, and for the backward sweeps' one-row tiles 32 or 40 registers. The candidates are timed interleaved over
// several rounds and each keeps its best time, so a transient on the GPU does
// not decide the choice. The backward sweeps are tuned on the first run with
// the adjoint.
int autotune(fwigb_ctx* ctx, int nshots, int nx_max, bool adj) {
  cudaStream_t s = ctx->stream;
  unsigned* d_err = reinterpret_cast<unsigned*>(ctx->scal.as<char>() + 16);
  (void)nx_max;
  constexpr int kRounds = 4, kReps = 5, kMaxCand = 9;
  std::vector<cudaEvent_t> ev(2 * kRounds * kMaxCand);
  for (cudaEvent_t& e : ev) CK(cudaEventCreate(&e));
  const int kinds_end = (adj && ctx->nSteps_max >= 2) ? 4 : 2;
  for (int kind = ctx->tuned_fwd ? 2 : 0; kind < kinds_end; ++kind) {
    // (width, rows) candidates; the backward sweeps add one-row tiles at 40
    // registers (ctx->regs, read by launch_sweep, is set per candidate).
    const int ncand = kind >= 2 ? 9 : 6;
    auto cand = [&](int q, int& tx, int& rows) {
      tx = kTileXs[q % 3];
      rows = (q / 3) == 1 ? 2 : 1;
      ctx->regs[kind] = (q / 3) == 2 ? 40 : 32;
    };
    for (int q = 0; q < ncand; ++q) {  // warm-up
      int tx, rows;
      cand(q, tx, rows);
      launch_sweep(ctx, kind, tx, rows, nshots, 0, 0, d_err);
    }
    for (int r = 0; r < kRounds; ++r)
      for (int q = 0; q < ncand; ++q) {
        int tx, rows;
        cand(q, tx, rows);
        CK(cudaEventRecord(ev[2 * (r * kMaxCand + q)], s));
        for (int k = 0; k < kReps; ++k) launch_sweep(ctx, kind, tx, rows, nshots, 0, 0, d_err);
        CK(cudaEventRecord(ev[2 * (r * kMaxCand + q) + 1], s));
      }
    CK(cudaStreamSynchronize(s));
    float best = 1e30f;
    int qbest = 0;
    for (int q = 0; q < ncand; ++q) {
      float t = 1e30f;
      for (int r = 0; r < kRounds; ++r) {
        float ms = 0.0f;
        CK(cudaEventElapsedTime(&ms, ev[2 * (r * kMaxCand + q)], ev[2 * (r * kMaxCand + q) + 1]));
        t = std::min(t, ms);
      }
      if (t < best) {
        best = t;
        qbest = q;
      }
    }
    cand(qbest, ctx->tx[kind], ctx->rows[kind]);
  }
  CK(cudaGetLastError());
  for (cudaEvent_t e : ev) cudaEventDestroy(e);
  ctx->tuned_fwd = true;
  if (kinds_end == 4) ctx->tuned_bwd = true;
  return FWIGB_OK;
}

// Scratch outputs of a gradient call (libCUFD.cu:493-511), when the
// parameter file names scratch_dir_name: per shot, the injected residual
// (Residual_Shot<id>.bin), the processed synthetic (Syn_Shot<id>.bin), the
// conditioned observed data -- tapered and, with a filter, band-passed --
// (CondObs_Shot<id>.bin), each [nrec][nSteps] float, and the source wavelet
// used (src_updated<id>.bin, nSteps floats).
int write_scratch(fwigb_ctx* ctx) {
  const Params& p = ctx->p;
  cudaStream_t s = ctx->stream;
  size_t need = 0;
  for (const ShotPlan& pl : ctx->plans) need = std::max(need, static_cast<size_t>(pl.nrec) * pl.nSteps);
  CK(ctx->scratch_tmp.ensure(2 * need * sizeof(float)));
  float* ta = ctx->scratch_tmp.as<float>();
  float* tb = ctx->scratch_tmp.as<float>(need);
  std::vector<float> h;
  auto write = [&](const std::string& name, const float* data, size_t n) -> int {
    const std::string fn = p.scratch_dir_name + "/" + name;
    std::FILE* fp = std::fopen(fn.c_str(), "wb");
    if (!fp || std::fwrite(data, sizeof(float), n, fp) != n) {
      if (fp) std::fclose(fp);
      ctx->err = "cannot write " + fn;
      return FWIGB_ERR_IO;
    }
    std::fclose(fp);
    return FWIGB_OK;
  };
  for (const ShotPlan& pl : ctx->plans) {
    const int nt = pl.nSteps;
    const size_t per = static_cast<size_t>(pl.nrec) * nt;
    const float* tw = ctx->shot_taper.as<float>(pl.taper_off);
    launch_apply_taper(s, pl.nrec, nt, ctx->shot_data.as<float>(pl.data_off), ta, tw, ctx->per_trace_taper ? 1 : 0);
    const float* cond = ta;
    if (p.if_filter) {
      launch_trace_filter(s, pl.nrec, nt, ta, tb, ctx->shot_filt.as<float>(pl.filt_off));
      cond = tb;
    }
    h.resize(3 * per);
    CK(cudaMemcpyAsync(h.data(), ctx->shot_data.as<float>(pl.data_off + 2 * per), per * sizeof(float),
                       cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(h.data() + per, ctx->shot_data.as<float>(pl.data_off + per), per * sizeof(float),
                       cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(h.data() + 2 * per, cond, per * sizeof(float), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    const std::string id = std::to_string(pl.id);
    TRY_RC(write("Residual_Shot" + id + ".bin", h.data(), per));
    TRY_RC(write("Syn_Shot" + id + ".bin", h.data() + per, per));
    TRY_RC(write("CondObs_Shot" + id + ".bin", h.data() + 2 * per, per));
    if (p.if_src_update) {
      std::vector<float> upd(nt);
      CK(cudaMemcpyAsync(upd.data(), ctx->shot_supd.as<float>(pl.supd_off + SupdLayout(nt).upd), nt * sizeof(float),
                         cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
      TRY_RC(write("src_updated" + id + ".bin", upd.data(), nt));
    } else {
      TRY_RC(write("src_updated" + id + ".bin", pl.src_amp.data(), nt));
    }
  }
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
  if (ctx->plans.empty()) {
    ctx->err = "no shots staged";
    return FWIGB_ERR_ARG;
  }
  const bool if_res = calc_id != 2, adj = calc_id == 1;
  if (if_res && !ctx->with_obs) {
    ctx->err = "misfit needs observed data";
    return FWIGB_ERR_ARG;
  }
  CK(cudaSetDevice(ctx->device));
  clear_stale_error();
  std::vector<std::vector<int>> groups;
  TRY_RC(plan_groups(ctx, adj, groups));
  cudaStream_t s = ctx->stream;
  const int nz = ctx->p.nz;
  unsigned* d_err = reinterpret_cast<unsigned*>(ctx->scal.as<char>() + 16);
  double* d_misfit = ctx->scal.as<double>();
  CK(cudaMemsetAsync(d_misfit, 0, sizeof(double), s));
  if (adj) CK(cudaMemsetAsync(ctx->grads.p, 0, 3 * ctx->cells * sizeof(float), s));
  if (ctx->illum) CK(cudaMemsetAsync(ctx->grads.as<float>(3 * ctx->cells), 0, ctx->cells * sizeof(float), s));
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
  for (size_t gi = 0; gi < groups.size(); ++gi) {
    const std::vector<int>& mem = groups[gi];
    const int G = static_cast<int>(mem.size());
    int nx_max = 0;
    TRY_RC(build_group(ctx, mem, nx_max));
    if (ctx->autotune && (!ctx->tuned_fwd || (adj && !ctx->tuned_bwd))) TRY_RC(autotune(ctx, G, nx_max, adj));
    const ShotSlot* slots = ctx->g_slots.as<ShotSlot>();
    (void)nx_max;
    std::vector<int> nst(G);
    for (int k = 0; k < G; ++k) nst[k] = ctx->plans[mem[k]].nSteps;  // descending
    auto active = [&](int step) {  // members whose record reaches `step`
      int a = G;
      while (a > 0 && nst[a - 1] - 2 < step) --a;
      return a;
    };
    long long group_launches = 0;
    // The group's launch sequence (eager, or recorded into a CUDA graph).
    auto enqueue = [&]() -> int {
      // Fresh wavefields and gathers for every member (libCUFD.cu:163-187).
      CK(cudaMemsetAsync(ctx->g_fields.p, 0, static_cast<size_t>(G) * ctx->fields_stride * sizeof(float), s));
      for (int k = 0; k < G; ++k) {
        const ShotPlan& pl = ctx->plans[mem[k]];
        const size_t per = static_cast<size_t>(pl.nrec) * pl.nSteps;
        CK(cudaMemsetAsync(ctx->shot_data.as<float>(pl.data_off + per), 0, per * sizeof(float), s));
        if (adj) CK(cudaMemsetAsync(ctx->shot_gstf.as<float>(pl.gstf_off), 0, pl.nSteps * sizeof(float), s));
      }
      if (adj || ctx->illum)
        CK(cudaMemsetAsync(ctx->g_grads.p, 0, static_cast<size_t>(G) * ctx->grads_stride * sizeof(float), s));
      const int ntop = nst[0];
      for (int it = 0; it <= ntop - 2; ++it) {
        const int a = active(it);
        const int f1_flags = (adj ? 1 : 0) | (ctx->inject_timeout && it == 0 ? 2 : 0);
        TIMED(0, group_launches += launch_sweep(ctx, 0, ctx->tx[0], ctx->rows[0], a, it, f1_flags, d_err));
        TIMED(1, group_launches += launch_sweep(ctx, 1, ctx->tx[1], ctx->rows[1], a, 0, 0, d_err));
      }
      if (if_res) {
        for (int k = 0; k < G; ++k) {
          const ShotPlan& pl = ctx->plans[mem[k]];
          const int nt = pl.nSteps;
          const size_t per = static_cast<size_t>(pl.nrec) * nt;
          const float* tw = ctx->shot_taper.as<float>(pl.taper_off);
          const float* to = tw;
          const float* tr = ctx->per_trace_taper ? tw + per : tw + nt;
          const int nb = residual_blocks(pl.nrec * nt);
          const int pt = ctx->per_trace_taper ? 1 : 0;
          float* obs = ctx->shot_data.as<float>(pl.data_off);
          float* syn = ctx->shot_data.as<float>(pl.data_off + per);
          float* res = ctx->shot_data.as<float>(pl.data_off + 2 * per);
          if (!ctx->p.if_filter && !ctx->p.if_src_update) {
            launch_residual(s, pl.nrec, nt, obs, syn, res, to, tr, pt, ctx->partials.as<double>());
            launch_sum_partials(s, ctx->partials.as<double>(), nb, d_misfit);
            group_launches += 2;
          } else {
            // Taper; band-pass obs and syn; source-wavelet update of syn and
            // the wavelet; residual and misfit; adjoint update and band-pass
            // of the residual; adjoint taper (libCUFD.cu:256-310). The
            // processed synthetic replaces the gathers, as in the reference.
            float* ta = ctx->filt_tmp.as<float>();
            float* tb = ctx->filt_tmp.as<float>(ctx->filt_tmp_floats);
            const float* h = ctx->p.if_filter ? ctx->shot_filt.as<float>(pl.filt_off) : nullptr;
            launch_apply_taper(s, pl.nrec, nt, obs, ta, to, pt);
            launch_apply_taper(s, pl.nrec, nt, syn, syn, to, pt);
            group_launches += 2;
            const float* ob = ta;  // conditioned observed data
            float* spare = tb;     // free trace block
            if (h) {
              launch_trace_filter(s, pl.nrec, nt, ta, tb, h);
              launch_trace_filter(s, pl.nrec, nt, syn, ta, h);
              CK(cudaMemcpyAsync(syn, ta, per * sizeof(float), cudaMemcpyDeviceToDevice, s));
              ob = tb;
              spare = ta;
              group_launches += 2;
            }
            float* kresp = ctx->supd_k.as<float>();
            const float* w2 = nullptr;
            if (ctx->p.if_src_update) {
              // source_update (utilities.cu:927-1035): coef from the padded,
              // tapered spectra; syn and the wavelet through the response.
              const SupdLayout L(nt);
              float* b = ctx->shot_supd.as<float>(pl.supd_off);
              w2 = b + L.w2;
              launch_src_update_coef(s, pl.nrec, nt, ob, syn, w2, reinterpret_cast<const float2*>(b + L.tw),
                                     ctx->supd_part.as<float>(), ctx->supd_coef.as<float2>(), kresp);
              launch_apply_taper(s, pl.nrec, nt, syn, spare, w2, 0);
              launch_trace_filter(s, pl.nrec, nt, spare, syn, kresp);
              launch_trace_filter(s, 1, nt, b + L.amp, b + L.upd, kresp);
              launch_src_terms(s, nt, ctx->p.dt, b + L.upd, b + L.szz, b + L.sxx);
              group_launches += 7;
            }
            launch_residual(s, pl.nrec, nt, ob, syn, res, nullptr, nullptr, 0, ctx->partials.as<double>());
            launch_sum_partials(s, ctx->partials.as<double>(), nb, d_misfit);
            group_launches += 2;
            // The conditioned obs is no longer needed: both blocks are free.
            if (w2) {  // source_update_adj (utilities.cu:1037-1080), amp_ratio 1
              launch_apply_taper(s, pl.nrec, nt, res, ta, w2, 0);
              launch_trace_filter(s, pl.nrec, nt, ta, res, kresp);
              group_launches += 2;
            }
            const float* last = res;
            if (h) {
              launch_trace_filter(s, pl.nrec, nt, res, ta, h);
              last = ta;
              ++group_launches;
            }
            launch_apply_taper(s, pl.nrec, nt, last, res, tr, pt);
            ++group_launches;
          }
        }
      }
      if (adj) {
        // Zero the adjoint fields and the 8 memory arrays (libCUFD.cu:337-351):
        // field slots 5..17 of every member.
        for (int k = 0; k < G; ++k) {
          const size_t n = static_cast<size_t>(ctx->geo.ldz) * ctx->plans[mem[k]].nx;
          CK(cudaMemsetAsync(ctx->g_fields.as<float>(k * ctx->fields_stride + 5 * n), 0, 13 * n * sizeof(float), s));
        }
        // The reference's first el_velocity_adj acts on all-zero fields (no-op);
        // then res_injection(nSteps-1) + el_stress_adj, source_grad(nSteps-2),
        // reverse velocity of step nSteps-2 ... (libCUFD.cu:353-445), with
        // backward iteration j meaning step nSteps_k - 2 - j of member k.
        TIMED(3, group_launches += launch_sweep(ctx, 3, ctx->tx[3], ctx->rows[3], G, -1, 0, d_err));
        for (int j = 0; j <= ntop - 2; ++j) {
          const int a = active(j);
          TIMED(2, group_launches += launch_sweep(ctx, 2, ctx->tx[2], ctx->rows[2], a, j, 0, d_err));
          TIMED(3, group_launches += launch_sweep(ctx, 3, ctx->tx[3], ctx->rows[3], a, j, 0, d_err));
        }
      }
      if (adj || ctx->illum) {
        float* gb = ctx->grads.as<float>();
        launch_reduce_grads(s, nz, ctx->p.nx, ctx->geo.ldz, G, slots, adj ? gb : nullptr, gb + ctx->cells,
                            gb + 2 * ctx->cells, ctx->illum ? gb + 3 * ctx->cells : nullptr);
        ++group_launches;
      }
      return FWIGB_OK;
    };
    if (ctx->use_graphs && !ctx->timing && groups.size() == 1) {
      // A call of one group (a lone shot, or a batched group of any size) is
      // replayed from a CUDA graph captured on first use: per time step one
      // launch per sweep and parameter pack, plus the residual path. A call of
      // several groups would record a graph per group and call, so it runs
      // eagerly. The key holds every value the captured launches depend on:
      // the parameter packs (pointers, geometry, TMA maps) and launch extents,
      // tile choices, flags, the members' data offsets and the buffers of the
      // memsets / residual.
      std::vector<uint64_t> key = {static_cast<uint64_t>(calc_id), static_cast<uint64_t>(ctx->illum),
                                   static_cast<uint64_t>(ctx->per_trace_taper),
                                   static_cast<uint64_t>(ctx->inject_timeout), static_cast<uint64_t>(G)};
      for (int k = 0; k < 4; ++k)
        key.push_back((static_cast<uint64_t>(ctx->regs[k]) << 16) | (static_cast<uint64_t>(ctx->tx[k]) << 8) |
                      ctx->rows[k]);
      for (int k = 0; k < G; ++k) {
        const ShotPlan& pl = ctx->plans[mem[k]];
        for (uint64_t v : {static_cast<uint64_t>(pl.nrec), static_cast<uint64_t>(pl.nSteps),
                           static_cast<uint64_t>(pl.nx), static_cast<uint64_t>(pl.data_off),
                           static_cast<uint64_t>(pl.gstf_off), static_cast<uint64_t>(pl.taper_off),
                           static_cast<uint64_t>(pl.filt_off), static_cast<uint64_t>(pl.supd_off)})
          key.push_back(v);
      }
      for (uint64_t v : {static_cast<uint64_t>(ctx->fields_stride), static_cast<uint64_t>(ctx->grads_stride),
                         reinterpret_cast<uint64_t>(ctx->g_fields.p), reinterpret_cast<uint64_t>(ctx->g_grads.p),
                         reinterpret_cast<uint64_t>(ctx->shot_data.p), reinterpret_cast<uint64_t>(ctx->shot_gstf.p),
                         reinterpret_cast<uint64_t>(ctx->shot_taper.p), reinterpret_cast<uint64_t>(ctx->partials.p),
                         reinterpret_cast<uint64_t>(ctx->grads.p), reinterpret_cast<uint64_t>(ctx->scal.p),
                         reinterpret_cast<uint64_t>(ctx->g_slots.p), reinterpret_cast<uint64_t>(ctx->shot_filt.p),
                         reinterpret_cast<uint64_t>(ctx->filt_tmp.p), static_cast<uint64_t>(ctx->filt_tmp_floats),
                         static_cast<uint64_t>(ctx->p.if_src_update), reinterpret_cast<uint64_t>(ctx->shot_supd.p),
                         reinterpret_cast<uint64_t>(ctx->supd_part.p), reinterpret_cast<uint64_t>(ctx->supd_coef.p),
                         reinterpret_cast<uint64_t>(ctx->supd_k.p)})
        key.push_back(v);
      auto add_words = [&key](const void* p, size_t bytes) {
        const uint64_t* w = static_cast<const uint64_t*>(p);
        key.insert(key.end(), w, w + bytes / sizeof(uint64_t));
      };
      static_assert(sizeof(SweepPack<1>) % 8 == 0 && sizeof(SweepPack<kPackShots>) % 8 == 0,
                    "launch parameters are compared as 64-bit words");
      if (G == 1)
        add_words(ctx->pack1.data(), ctx->pack1.size() * sizeof(SweepPack<1>));
      else
        add_words(ctx->packs.data(), ctx->packs.size() * sizeof(SweepPack<kPackShots>));
      for (const SweepGrid& gr : ctx->pack_grid) key.push_back((static_cast<uint64_t>(gr.nz) << 32) | gr.nx);
      if (!ctx->graph_exec || key != ctx->graph_key) {
        if (ctx->graph_exec) {
          cudaGraphExecDestroy(ctx->graph_exec);
          ctx->graph_exec = nullptr;
        }
        CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        const int rc = enqueue();
        cudaGraph_t graph = nullptr;
        const cudaError_t ec = cudaStreamEndCapture(s, &graph);
        if (rc != FWIGB_OK) {
          if (graph) cudaGraphDestroy(graph);
          return rc;
        }
        CK(ec);
        const cudaError_t ei = cudaGraphInstantiate(&ctx->graph_exec, graph, 0);
        cudaGraphDestroy(graph);
        CK(ei);
        ctx->graph_key = std::move(key);
        ctx->graph_launches = group_launches;
      }
      group_launches = ctx->graph_launches;
      CK(cudaGraphLaunch(ctx->graph_exec, s));
    } else {
      TRY_RC(enqueue());
    }
    launches += group_launches;
    // The next group reuses the slots and maps; wait for this one.
    if (gi + 1 < groups.size()) CK(cudaStreamSynchronize(s));
  }
#undef TIMED
  CK(cudaGetLastError());
  ctx->launches = launches;
  ctx->last_calc = calc_id;
  ctx->last_groups = static_cast<int>(groups.size());
  ctx->illum_valid = ctx->illum;
  if (adj && ctx->p.if_save_scratch) TRY_RC(write_scratch(ctx));
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
  const int nt_max = p.nSteps;
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
    // Row k: shot k's source gradient, zero past its record length.
    size_t tot = 0;
    for (const ShotPlan& pl : ctx->plans) tot += pl.nSteps;
    std::vector<float> h(tot);
    CK(cudaMemcpyAsync(h.data(), ctx->shot_gstf.p, tot * sizeof(float), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    for (size_t k = 0; k < ctx->plans.size(); ++k) {
      const ShotPlan& pl = ctx->plans[k];
      for (int it = 0; it < nt_max; ++it)
        g_stf[k * nt_max + it] = it < pl.nSteps ? static_cast<double>(h[pl.gstf_off + it]) : 0.0;
    }
  }
  if (gathers) {
    // Shot k at offset k * nrec_max * nSteps as [nrec][nSteps], its
    // [nrec_k][nSteps_k] block in the top-left corner.
    const size_t blk = static_cast<size_t>(ctx->nrec_max) * nt_max;
    std::memset(gathers, 0, ctx->plans.size() * blk * sizeof(float));
    for (size_t k = 0; k < ctx->plans.size(); ++k) {
      const ShotPlan& pl = ctx->plans[k];
      const size_t per = static_cast<size_t>(pl.nrec) * pl.nSteps;
      CK(cudaMemcpy2DAsync(gathers + k * blk, nt_max * sizeof(float), ctx->shot_data.as<float>(pl.data_off + per),
                           pl.nSteps * sizeof(float), pl.nSteps * sizeof(float), pl.nrec, cudaMemcpyDeviceToHost, s));
    }
  }
  CK(cudaStreamSynchronize(s));
  return FWIGB_OK;
}

int write_gathers(fwigb_ctx* ctx, const float* gathers) {
  // libCUFD.cu:514-521, [nrec][nSteps_k] float per shot.
  const int nt_max = ctx->p.nSteps;
  const size_t blk = static_cast<size_t>(ctx->nrec_max) * nt_max;
  std::vector<float> row;
  for (size_t k = 0; k < ctx->plans.size(); ++k) {
    const ShotPlan& pl = ctx->plans[k];
    const std::string fn = ctx->p.data_dir_name + "/Shot" + std::to_string(pl.id) + ".bin";
    std::FILE* fp = std::fopen(fn.c_str(), "wb");
    if (!fp) {
      ctx->err = "cannot write " + fn;
      return FWIGB_ERR_IO;
    }
    bool ok = true;
    for (int r = 0; r < pl.nrec && ok; ++r)
      ok = std::fwrite(gathers + k * blk + static_cast<size_t>(r) * nt_max, sizeof(float), pl.nSteps, fp) ==
           static_cast<size_t>(pl.nSteps);
    std::fclose(fp);
    if (!ok) {
      ctx->err = "short write to " + fn;
      return FWIGB_ERR_IO;
    }
  }
  return FWIGB_OK;
}

#define TRY(call)                    \
  do {                               \
    int rc_ = (call);                \
    if (rc_ != FWIGB_OK) return rc_; \
  } while (0)

}  // namespace

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
  for (DevBuf* b : {&ctx->media, &ctx->stage, &ctx->cpml, &ctx->grads, &ctx->scal, &ctx->partials,
                    &ctx->shot_src, &ctx->shot_rec, &ctx->shot_blk, &ctx->shot_data, &ctx->shot_taper,
                    &ctx->shot_gstf, &ctx->shot_cpmlx, &ctx->shot_filt, &ctx->filt_tmp, &ctx->scratch_tmp,
                    &ctx->shot_supd, &ctx->supd_part, &ctx->supd_coef, &ctx->supd_k,
                    &ctx->g_fields,
                    &ctx->g_store, &ctx->g_grads,
                    &ctx->g_slots})
    b->release();
  for (cudaEvent_t e : ctx->ev_pool) cudaEventDestroy(e);
  if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
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

int fwigb_shot_info(const fwigb_ctx* ctx, int shot_id, int* nrec, int* nSteps, int* x_off, int* nx) {
  if (!ctx || shot_id < 0 || shot_id >= static_cast<int>(ctx->survey.size()) || !ctx->survey[shot_id].present)
    return FWIGB_ERR_ARG;
  const ShotGeom& g = ctx->survey[shot_id];
  if (nrec) *nrec = static_cast<int>(g.z_rec.size());
  if (nSteps) *nSteps = g.nSteps;
  if (x_off) *x_off = g.x_off;
  if (nx) *nx = g.nx;
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

int fwigb_sweep_time(fwigb_ctx* ctx, int kind, int reps, double* us_per_launch) {
  if (!ctx || !us_per_launch || kind < 0 || kind > 3 || reps < 1) return FWIGB_ERR_ARG;
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (ctx->group_size < 1) {
    ctx->err = "no group has run yet";
    return FWIGB_ERR_ARG;
  }
  cudaStream_t s = ctx->stream;
  unsigned* d_err = reinterpret_cast<unsigned*>(ctx->scal.as<char>() + 16);
  const int rows = ctx->rows[kind];
  CK(cudaStreamSynchronize(s));
  CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  for (int r = 0; r < reps; ++r) launch_sweep(ctx, kind, ctx->tx[kind], rows, ctx->group_size, 0, 0, d_err);
  cudaGraph_t graph = nullptr;
  CK(cudaStreamEndCapture(s, &graph));
  cudaGraphExec_t exec = nullptr;
  const cudaError_t ei = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  CK(ei);
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  CK(cudaGraphLaunch(exec, s));  // warm-up
  CK(cudaEventRecord(e0, s));
  CK(cudaGraphLaunch(exec, s));
  CK(cudaEventRecord(e1, s));
  CK(cudaEventSynchronize(e1));
  float ms = 0.0f;
  CK(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaGraphExecDestroy(exec);
  *us_per_launch = 1e3 * ms / reps;
  return FWIGB_OK;
}

int fwigb_set_graphs(fwigb_ctx* ctx, int enable) {
  if (!ctx) return FWIGB_ERR_ARG;
  std::lock_guard<std::mutex> lk(ctx->mu);
  ctx->use_graphs = enable != 0;
  if (!ctx->use_graphs && ctx->graph_exec) {
    cudaGraphExecDestroy(ctx->graph_exec);
    ctx->graph_exec = nullptr;
    ctx->graph_key.clear();
  }
  return FWIGB_OK;
}

int fwigb_tile_rows(const fwigb_ctx* ctx, int* rows) {
  if (!ctx || !rows) return FWIGB_ERR_ARG;
  for (int k = 0; k < 4; ++k) rows[k] = ctx->rows[k];
  return FWIGB_OK;
}

int fwigb_tile_registers(const fwigb_ctx* ctx, int* regs) {
  if (!ctx || !regs) return FWIGB_ERR_ARG;
  for (int k = 0; k < 4; ++k) regs[k] = k >= 2 && ctx->rows[k] == 1 ? ctx->regs[k] : (k >= 2 ? 64 : 32);
  return FWIGB_OK;
}

int fwigb_set_tile_registers(fwigb_ctx* ctx, const int* regs) {
  if (!ctx || !regs) return FWIGB_ERR_ARG;
  std::lock_guard<std::mutex> lk(ctx->mu);
  for (int k = 2; k < 4; ++k)
    if (regs[k] != 32 && regs[k] != 40) {
      ctx->err = "backward one-row tiles run at 32 or 40 registers";
      return FWIGB_ERR_ARG;
    }
  ctx->regs[2] = regs[2];
  ctx->regs[3] = regs[3];
  ctx->autotune = false;
  return FWIGB_OK;
}

int fwigb_set_tile_rows(fwigb_ctx* ctx, const int* rows) {
  if (!ctx || !rows) return FWIGB_ERR_ARG;
  std::lock_guard<std::mutex> lk(ctx->mu);
  for (int k = 0; k < 4; ++k)
    if (rows[k] != 1 && rows[k] != 2) {
      ctx->err = "depths per thread must be 1 or 2";
      return FWIGB_ERR_ARG;
    }
  for (int k = 0; k < 4; ++k) ctx->rows[k] = rows[k];
  ctx->autotune = false;
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

int fwigb_set_batching(fwigb_ctx* ctx, int max_shots, unsigned long long mem_budget_bytes) {
  if (!ctx || max_shots < 0) return FWIGB_ERR_ARG;
  std::lock_guard<std::mutex> lk(ctx->mu);
  ctx->max_batch = max_shots;
  ctx->mem_budget = static_cast<size_t>(mem_budget_bytes);
  return FWIGB_OK;
}

int fwigb_last_group_count(const fwigb_ctx* ctx) { return ctx ? ctx->last_groups : -1; }

int fwigb_test_inject_wait_timeout(fwigb_ctx* ctx, int enable) {
  if (!ctx) return FWIGB_ERR_ARG;
  std::lock_guard<std::mutex> lk(ctx->mu);
  ctx->inject_timeout = enable != 0;
  return FWIGB_OK;
}

int fwigb_set_illumination(fwigb_ctx* ctx, int enable) {
  if (!ctx) return FWIGB_ERR_ARG;
  std::lock_guard<std::mutex> lk(ctx->mu);
  ctx->illum = enable != 0;
  return FWIGB_OK;
}

int fwigb_fetch_illumination(fwigb_ctx* ctx, double* illum) {
  if (!ctx || !illum) return FWIGB_ERR_ARG;
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (!ctx->illum_valid) {
    ctx->err = "the last run did not accumulate the illumination (fwigb_set_illumination)";
    return FWIGB_ERR_ARG;
  }
  cudaStream_t s = ctx->stream;
  double* st = ctx->stage.as<double>();
  launch_to_rowmajor(s, ctx->p.nz, ctx->p.nx, ctx->geo.ldz, ctx->grads.as<float>(3 * ctx->cells), st, 1.0);
  CK(cudaMemcpyAsync(illum, st, ctx->ncell * sizeof(double), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
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
    tmp.resize(ctx->plans.size() * static_cast<size_t>(ctx->nrec_max) * ctx->p.nSteps);
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
