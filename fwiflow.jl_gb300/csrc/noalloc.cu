// Allocation-free misfit of one shot's gathers.
//
// Some callers cannot call cudaMalloc: an operator running inside another
// framework that owns the device memory pool (TensorFlow's BFC allocator, as
// for FwiFlow's own TF op, or an XLA / JAX runtime that has reserved most of
// the GPU) would either fail to allocate or fragment that pool, and a
// long-running service with a fixed device-memory budget must not allocate per
// request. fwigb_misfit_gathers_noalloc serves them: the caller passes device
// buffers for the inputs and outputs, and the only scratch it needs, one
// double per receiver trace plus the total, lives in the file-scope device
// array below. Its address is looked up once per device, by the first call
// made with that device current, so make that first call before any stream
// capture on that device. Each call synchronises its stream to return the
// misfit to the host.
//
// It reproduces the plain residual path of fwigb_misfit only: the fixed 0.005
// data taper, without per-trace windows, band-pass filter or source-wavelet
// update.
//
// The array holds kNoAllocMaxTraces + 1 doubles (512 KiB + 8 B). Every GPU that
// loads the library keeps it until the process exits. All calls share it:
// two calls whose kernels overlap on the GPU (different streams, or different
// host threads on the same device) race on it, so serialise such calls.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>

#include "fwiflow_gb300.h"

namespace {

constexpr int kNoAllocMaxTraces = 65536;
constexpr int kMaxDevices = 64;
constexpr double kPi = 3.141592653589793238462643383279502884197169;

// Per-trace sums of squared residuals [0, nrec) and the total at [kNoAllocMaxTraces].
static __device__ __align__(256) double g_trace_partials[kNoAllocMaxTraces + 1];

thread_local const char* t_noalloc_err = "";

// Weight amp^2 of the sin^2 / cos^2 taper of the reference's cuda_window
// without windows (deps/CustomOps/FWI/Src/utilities.cu:707-747), ratio 0.005.
__device__ float taper_weight(int it, int nt, float dt) {
  const float ratio = 0.005f;
  const float t0 = 0.0f, t3 = nt * dt, off = nt * dt * ratio;
  const float t1 = t0 + off, t2 = t3 - off;
  const float t = it * dt;
  float amp;
  if (t >= t0 && t < t1)
    amp = static_cast<float>(sin(kPi / 2.0 * (t - t0) / (t1 - t0)));
  else if (t >= t1 && t < t2)
    amp = 1.0f;
  else if (t >= t2 && t < t3)
    amp = static_cast<float>(cos(kPi / 2.0 * (t - t2) / (t3 - t2)));
  else
    amp = 0.0f;
  return amp * amp;
}

// One block per receiver trace: taper obs and syn (syn in place), residual
// with sample 0 zeroed, the trace's sum of squares into partials[r], and the
// adjoint-tapered residual into res.
__global__ void __launch_bounds__(256) k_trace_residual(const float* __restrict__ obs, float* syn, float* res,
                                                        int nSteps, float dt, double* partials) {
  const int r = blockIdx.x;
  const size_t base = static_cast<size_t>(r) * nSteps;
  double acc = 0.0;
  for (int t = threadIdx.x; t < nSteps; t += blockDim.x) {
    const float w = taper_weight(t, nSteps, dt);
    const float s = syn[base + t] * w;
    const float o = obs[base + t] * w;
    syn[base + t] = s;
    const float d = (t == 0) ? 0.0f : o - s;
    acc += static_cast<double>(d) * d;
    res[base + t] = d * w;
  }
  __shared__ double sh[8];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = (threadIdx.x < (blockDim.x >> 5)) ? sh[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) partials[r] = v;
  }
}

// Fixed-order sum of the trace partials; writes 0.5 * sum to partials[total_slot].
__global__ void k_sum_traces(double* partials, int nrec, int total_slot) {
  double v = 0.0;
  for (int k = threadIdx.x; k < nrec; k += 32) v += partials[k];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if (threadIdx.x == 0) partials[total_slot] = 0.5 * v;
}

// Device address of g_trace_partials, looked up once per device. Host code
// must not hand the symbol itself to a kernel: on the host it names a
// host-side stand-in, not device memory.
double* scratch_for_current_device(int* status) {
  static std::mutex mu;
  static double* addr[kMaxDevices] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    t_noalloc_err = "cannot query the current CUDA device";
    *status = FWIGB_ERR_CUDA;
    return nullptr;
  }
  std::lock_guard<std::mutex> lk(mu);
  if (!addr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_trace_partials);
    if (e != cudaSuccess || !p) {
      t_noalloc_err = "cudaGetSymbolAddress of the misfit scratch failed";
      *status = FWIGB_ERR_CUDA;
      return nullptr;
    }
    addr[dev] = static_cast<double*>(p);
  }
  *status = FWIGB_OK;
  return addr[dev];
}

}  // namespace

extern "C" {

int fwigb_misfit_gathers_noalloc(const float* d_obs, float* d_syn, float* d_res, int nrec, int nSteps, float dt,
                                 double* misfit, void* stream) {
  if (!d_obs || !d_syn || !d_res || !misfit || nSteps < 2 || !(dt > 0.0f)) {
    t_noalloc_err = "null buffer, nSteps < 2 or dt <= 0";
    return FWIGB_ERR_ARG;
  }
  if (nrec < 1 || nrec > kNoAllocMaxTraces) {
    t_noalloc_err = "nrec must be between 1 and 65536 (the size of the static misfit scratch)";
    return FWIGB_ERR_ARG;
  }
  // The taper's ramps span nSteps * dt * 0.005 seconds at each end of the
  // record; a zero (underflowed) or non-finite span would divide by zero.
  const float record = static_cast<float>(nSteps) * dt;
  if (!std::isfinite(record) || !(record * 0.005f > 0.0f)) {
    t_noalloc_err = "nSteps * dt gives no usable data taper (its ramp nSteps * dt * 0.005 must be positive and finite)";
    return FWIGB_ERR_ARG;
  }
  int st = FWIGB_OK;
  double* scratch = scratch_for_current_device(&st);
  if (!scratch) return st;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaGetLastError();  // drop a stale non-sticky error of an earlier, unrelated call of this thread
  k_trace_residual<<<nrec, 256, 0, s>>>(d_obs, d_syn, d_res, nSteps, dt, scratch);
  k_sum_traces<<<1, 32, 0, s>>>(scratch, nrec, kNoAllocMaxTraces);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(misfit, scratch + kNoAllocMaxTraces, sizeof(double),
                                            cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    t_noalloc_err = cudaGetErrorString(e);
    return FWIGB_ERR_CUDA;
  }
  return FWIGB_OK;
}

const char* fwigb_noalloc_last_error(void) { return t_noalloc_err; }

}  // extern "C"
