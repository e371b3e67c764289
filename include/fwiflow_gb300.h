/*
 * fwiflow_gb300.h — C ABI of the GB300 (sm_103a) elastic FWI operator.
 *
 * Drop-in for the FWI operator of FwiFlow.jl: the same inputs, units, layouts
 * and outputs as the reference driver
 *
 *   void cufd(double *misfit, double *grad_Lambda, double *grad_Mu,
 *             double *grad_Den, double *grad_stf, const double *Lambda,
 *             const double *Mu, const double *Den, const double *stf,
 *             int calc_id, const int gpu_id, int group_size,
 *             const int *shot_ids, const std::string para_fname);
 *   (deps/CustomOps/FWI/Src/libCUFD.cu:34-38)
 *
 * and of the TensorFlow ops built on it, FwiOp / FwiOpGrad / FwiObsOp
 * (deps/CustomOps/FWI/FwiOp.cpp:15-319, FwiOp.h:14-34), which the Julia
 * functions fwi_op / fwi_obs_op bind (src/Core.jl:20-53).
 *
 * Conventions (all as in the reference):
 *  - lambda, mu in MPa and den in kg/m^3 are row-major double [nz][nx] on the
 *    padded grid of the parameter file (nz, nx there include the PML and nPad);
 *  - stf is row-major double [n_stf_rows][nSteps]; row shot_ids[i] drives
 *    shot i; shot_ids are 0-based and name `shot<k>` entries of the survey file;
 *  - gradients are w.r.t. lambda and mu in MPa and den, accumulated over all
 *    shots of the call; g_stf row i belongs to the i-th shot of the call;
 *  - misfit = 0.5 * sum over shots, receivers and samples 1..nSteps-1 of the
 *    squared tapered residual;
 *  - observed data come from data_dir_name/Shot<id>.bin ([nrec][nSteps] f32)
 *    unless passed in memory.
 * Every call returns an fwigb_status; nothing calls exit(). The library
 * allocates its device buffers itself and keeps them in the context.
 */
#ifndef FWIFLOW_GB300_H_
#define FWIFLOW_GB300_H_

#ifdef __cplusplus
extern "C" {
#endif

typedef enum fwigb_status {
  FWIGB_OK = 0,
  FWIGB_ERR_ARG = 1,        /* bad argument (null pointer, size mismatch, bad calc_id) */
  FWIGB_ERR_PARAM = 2,      /* parameter or survey file unreadable / missing key */
  FWIGB_ERR_COURANT = 3,    /* Courant number > 1 (the reference exits, utilities.cu:239) */
  FWIGB_ERR_CUDA = 4,       /* CUDA runtime error */
  FWIGB_ERR_OOM = 5,        /* device allocation failed */
  FWIGB_ERR_IO = 6,         /* observed-data or output file I/O failed */
  FWIGB_ERR_TIMEOUT = 7,    /* a bounded device wait gave up: the call's outputs are undefined */
  FWIGB_ERR_UNSUPPORTED = 8 /* option of the parameter file the library does not implement */
} fwigb_status;

typedef struct fwigb_ctx fwigb_ctx;

/* Opens a context for one parameter file on one CUDA device. Replaces the
 * per-call set-up of cufd (libCUFD.cu:42-93: cudaSetDevice, Parameter, Model,
 * Cpml, Bnd, Src_Rec); the context keeps parsed geometry and device buffers
 * across calls. */
int fwigb_create(const char *para_fname, int device, fwigb_ctx **out);

/* Releases a context and its device memory. */
int fwigb_destroy(fwigb_ctx *ctx);

/* Message of the last failure on this context (never NULL). */
const char *fwigb_last_error(const fwigb_ctx *ctx);

/* Message of the last failure of fwigb_create / fwigb_cufd (thread-local). */
const char *fwigb_last_global_error(void);

/* FwiOp forward: misfit only (cufd calc_id 0; FwiOp.cpp:47-103). */
int fwigb_misfit(fwigb_ctx *ctx, const double *lambda, const double *mu, const double *den, const double *stf,
                 int n_stf_rows, const int *shot_ids, int n_shots, double *misfit);

/* FwiOpGrad (cufd calc_id 1; FwiOp.cpp:130-223), computed with a single
 * forward sweep: misfit (may be NULL) and the four gradients. g_stf has
 * n_shots rows of nSteps (the reference writes only the first group rows of
 * its [n_stf_rows][nSteps] output, libCUFD.cu:452-456). */
int fwigb_misfit_grad(fwigb_ctx *ctx, const double *lambda, const double *mu, const double *den, const double *stf,
                      int n_stf_rows, const int *shot_ids, int n_shots, double *misfit, double *g_lambda,
                      double *g_mu, double *g_den, double *g_stf);

/* FwiObsOp (cufd calc_id 2; FwiOp.cpp:260-317): forward modelling only.
 * gathers (may be NULL) receives shot i at offset i*nrec_max*nSteps as
 * [nrec][nSteps] float; write_files != 0 also writes data_dir_name/Shot<id>.bin
 * exactly as libCUFD.cu:514-521. */
int fwigb_obs(fwigb_ctx *ctx, const double *lambda, const double *mu, const double *den, const double *stf,
              int n_stf_rows, const int *shot_ids, int n_shots, float *gathers, int write_files);

/* Variant of fwigb_misfit / fwigb_misfit_grad taking observed data from
 * memory: obs holds shot i at offset i*nrec_max*nSteps as [nrec][nSteps]. */
int fwigb_misfit_grad_obs(fwigb_ctx *ctx, const double *lambda, const double *mu, const double *den,
                          const double *stf, int n_stf_rows, const int *shot_ids, int n_shots, const float *obs,
                          double *misfit, double *g_lambda, double *g_mu, double *g_den, double *g_stf);

/* Geometry of the context: nz, nx, nSteps, number of shots in the survey and
 * the largest receiver count of any shot. */
int fwigb_geometry(const fwigb_ctx *ctx, int *nz, int *nx, int *nSteps, int *n_survey_shots, int *nrec_max);

/* Number of receivers of survey shot `shot_id`. */
int fwigb_shot_nrec(const fwigb_ctx *ctx, int shot_id, int *nrec);

/* Receivers, record length, first padded column and width of the sub-grid of
 * survey shot `shot_id` (any pointer may be NULL). */
int fwigb_shot_info(const fwigb_ctx *ctx, int shot_id, int *nrec, int *nSteps, int *x_off, int *nx);

/* One-call drop-in for cufd itself (libCUFD.cu:34-38) with a C string for the
 * parameter file. calc_id 0 writes misfit, 1 writes the gradients (g_stf has
 * group_size rows), 2 writes Data/Shot<id>.bin. A context per (para_fname,
 * gpu_id) is cached and reused by later calls. */
int fwigb_cufd(double *misfit, double *grad_Lambda, double *grad_Mu, double *grad_Den, double *grad_stf,
               const double *Lambda, const double *Mu, const double *Den, const double *stf, int calc_id,
               int gpu_id, int group_size, const int *shot_ids, const char *para_fname);

/* ---- Staged interface: the calls above are set_model + stage_shots + run +
 * fetch. Keeping the model and the shots resident lets a caller (and the
 * benchmark) run the device part alone. ---- */

/* Uploads lambda, mu [MPa] and den (row-major double [nz][nx]), derives the
 * staggered media and checks the Courant number (libCUFD.cu:67-96). */
int fwigb_set_model(fwigb_ctx *ctx, const double *lambda, const double *mu, const double *den);

/* Stages the shots of a call: source rows of stf, receivers, and (when
 * with_obs) observed data, from `obs` ([n_shots][nrec_max][nSteps] float, may
 * be NULL) or else from data_dir_name/Shot<id>.bin. */
int fwigb_stage_shots(fwigb_ctx *ctx, const double *stf, int n_stf_rows, const int *shot_ids, int n_shots,
                      int with_obs, const float *obs);

/* Runs the staged shots on the device, asynchronously on the context's
 * stream. calc_id 0: misfit, 1: misfit and gradients, 2: gathers only. */
int fwigb_run(fwigb_ctx *ctx, int calc_id);

/* Copies results of the last run to the host (synchronises). Any pointer may
 * be NULL. g_stf has n_shots rows of nSteps. gathers as in fwigb_obs. */
int fwigb_fetch(fwigb_ctx *ctx, double *misfit, double *g_lambda, double *g_mu, double *g_den, double *g_stf,
                float *gathers);

/* Waits for the context's stream. */
int fwigb_synchronize(fwigb_ctx *ctx);

/* The context's CUDA stream (a cudaStream_t), for callers that time it. */
void *fwigb_stream(fwigb_ctx *ctx);

/* Number of kernel launches the last fwigb_run issued (host-side count). */
long long fwigb_last_launch_count(const fwigb_ctx *ctx);

/* Concurrent shots. The shots of a call run in groups, all members of a group
 * in the same launches (one per sweep and time step). A group holds at most
 * max_shots shots (0: no cap) and its state (wavefields, gradients, boundary
 * stores) at most mem_budget_bytes (0: 90% of the free device memory). Shots
 * may carry their own record length ("nSteps") and aperture window
 * ("win_x0", "win_x1", interior columns) as extra keys of the survey file;
 * the reference's parser ignores those keys. */
int fwigb_set_batching(fwigb_ctx *ctx, int max_shots, unsigned long long mem_budget_bytes);

/* Number of shot groups the last fwigb_run used. */
int fwigb_last_group_count(const fwigb_ctx *ctx);

/* Source illumination (no counterpart in the reference): with enable != 0 the
 * following runs also accumulate, over all their shots and forward steps, the
 * energy vz^2 + vx^2 of the forward velocity after each step (the diagonal
 * pseudo-Hessian proxy used to precondition the gradient).
 * fwigb_fetch_illumination copies the last run's sum as row-major double
 * [nz][nx]; it fails if that run did not accumulate it. */
int fwigb_set_illumination(fwigb_ctx *ctx, int enable);
int fwigb_fetch_illumination(fwigb_ctx *ctx, double *illum);

/* Test hook of the failure path (no counterpart in the reference, which has
 * no bounded waits): with enable != 0, the first forward sweep of every
 * following run waits, once its staged tiles have landed, for a barrier
 * phase that nothing completes; its bounded wait runs out, the run returns
 * FWIGB_ERR_TIMEOUT, and the context stays usable. No copy is in flight when
 * the wait gives up. Off by default. */
int fwigb_test_inject_wait_timeout(fwigb_ctx *ctx, int enable);

/* Tile widths (columns per thread block: 4, 8 or 16) of the four sweeps
 * (forward stress, forward velocity, backward B, backward C). By default an
 * autotuner times every width and 1 or 2 depths per thread on the context's
 * grid at the first run and keeps the fastest; fwigb_set_tile_config fixes
 * the widths (NULL re-enables tuning), fwigb_set_tile_rows the depths per
 * thread (1 or 2 each; it also stops the tuning).
 * fwigb_tile_rows gives the depths per thread of the four sweeps. */
int fwigb_tile_config(const fwigb_ctx *ctx, int *tile_x);
int fwigb_set_tile_config(fwigb_ctx *ctx, const int *tile_x);
int fwigb_tile_rows(const fwigb_ctx *ctx, int *rows);

/* Registers per thread of the four sweeps' tiles: the forward sweeps run at
 * 32, the backward sweeps' two-row tiles at 64 and their one-row tiles at 32
 * or 40, which the autotuner picks with the widths (32 until it has run).
 * fwigb_set_tile_registers fixes the backward one-row budget (entries 2 and 3:
 * 32 or 40; entries 0 and 1 are ignored) and stops the tuning. */
int fwigb_tile_registers(const fwigb_ctx *ctx, int *regs);
int fwigb_set_tile_registers(fwigb_ctx *ctx, const int *regs);
int fwigb_set_tile_rows(fwigb_ctx *ctx, const int *rows);

/* CUDA graphs (on by default): a run whose shots form a single group (one
 * shot, or a batched group) records its whole launch sequence (per time step
 * one launch per sweep and pack of up to 16 shots: about 4 for a lone shot)
 * into a CUDA graph the first time and replays it while the staged shots, the
 * model and data buffers and the tile choices are unchanged; per-kernel
 * timing runs eagerly. enable = 0 runs every call eagerly. */
int fwigb_set_graphs(fwigb_ctx *ctx, int enable);

/* Average duration of one launch of sweep `kind` (0 forward stress, 1 forward
 * velocity, 2 backward B, 3 backward C) over the last run's (last) group, at
 * its tuned tile: `reps` back-to-back launches recorded in a CUDA graph and
 * timed with events around the graph (no per-launch event overhead). The
 * launches work on the live wavefields, which the next run resets. */
int fwigb_sweep_time(fwigb_ctx *ctx, int kind, int reps, double *us_per_launch);

/* Per-kernel timing of fwigb_run: when enabled, a CUDA event pair on the
 * context's stream brackets every sweep launch. Kinds: 0 forward stress,
 * 1 forward velocity, 2 backward sweep B, 3 backward sweep C. */
int fwigb_set_kernel_timing(fwigb_ctx *ctx, int enable);

/* Totals of the timed launches of the last fwigb_run (synchronises):
 * total_ms[4] and launches[4], indexed by kind. */
int fwigb_kernel_times(fwigb_ctx *ctx, double *total_ms, long long *launches);

/* ---- Allocation-free misfit (no counterpart in the reference) ----
 * For callers that cannot call cudaMalloc: an operator inside a framework that
 * owns the device memory pool (TensorFlow's allocator, as for FwiFlow's own TF
 * op; an XLA / JAX runtime that reserved the GPU), or a service with a fixed
 * device-memory budget. For one shot whose gathers the caller already holds on
 * the device, computes the misfit and the adjoint source of fwigb_misfit's
 * plain residual path: the fixed 0.005 data taper, with no per-trace windows
 * (if_win), no band-pass filter and no source-wavelet update; with any of
 * those options on, fwigb_misfit's results differ from this call's.
 * d_obs, d_syn and d_res are device buffers [nrec][nSteps] float with
 * 1 <= nrec <= 65536; d_syn is tapered in place, d_res receives the adjoint
 * source, *misfit (host) the misfit.
 * The only scratch is a static device array of 65537 doubles that every GPU
 * loading the library keeps until exit; all calls share it, so calls that
 * overlap on the GPU race. The first call on a device (with that device
 * current) looks up the array's address: make that first call before any
 * stream capture on the device. Each call synchronises `stream` (a
 * cudaStream_t; NULL for the legacy default stream) to return the misfit.
 * Allocates nothing. */
int fwigb_misfit_gathers_noalloc(const float *d_obs, float *d_syn, float *d_res, int nrec, int nSteps, float dt,
                                 double *misfit, void *stream);

/* Message of the last failure of fwigb_misfit_gathers_noalloc (thread-local). */
const char *fwigb_noalloc_last_error(void);

/* ---- Learned gradient preconditioner: BF16 tensor-core 3x3 convolutions
 * (csrc/cnn.cu; no counterpart in the reference). Images are Hz x Wx pixels
 * (Hz a multiple of 32), x-major with z fastest, channels innermost and
 * padded to 16 or 32; BF16 activations, FP32 accumulation, weights packed in
 * tensor-core fragment order by fwigb_cnn_pack_weights. All calls enqueue on
 * `stream` (a cudaStream_t) and allocate nothing. ---- */

/* y = epilogue(conv3x3(x, W) + b), zero padding. (cin_pad, cout_pad) in
 * {(16,32), (32,32), (32,16)}. epilogue 0: GELU, writes the pre-activation to
 * z_pre and GELU of it to y_bf16; 1: linear, y_f32 (FP32); 2: no bias,
 * y_bf16 = conv(x, W) * GELU'(z_prev) (the data gradient through the previous
 * layer's GELU, with W packed transposed). */
int fwigb_cnn_conv3x3(const void *x, int Hz, int Wx, int cin_pad, int cout_pad, int epilogue, const void *wfrag,
                      const float *bias, void *y_bf16, float *y_f32, void *z_pre, const void *z_prev,
                      void *stream);
/* The convolutions with 32 outputs on the 5th-generation tensor cores
 * (tcgen05.mma, accumulators in tensor memory; 128 x 4 pixels per block):
 * cin_pad in {16, 32}, epilogue 0 (GELU, with z_pre) or 2 (times GELU'(z_prev)),
 * wpack from fwigb_cnn_pack_weights_tc. A block whose bounded wait for its
 * MMAs gives up sets bit 1 of *err_word (device memory) and writes nothing.
 * Any Hz > 0. */
int fwigb_cnn_conv3x3_tc(const void *x, int Hz, int Wx, int cin_pad, int epilogue, const void *wpack,
                         const float *bias, void *y_bf16, void *z_pre, const void *z_prev, unsigned *err_word,
                         void *stream);
/* Packs FP32 weights W[9][cin][cout] into the tcgen05 B operand of a
 * convolution with 32 outputs (cout_pad = 32), or (transposed != 0) of its
 * data gradient (cin_pad = 32 outputs, cout_pad in {16, 32} inputs). */
int fwigb_cnn_pack_weights_tc(const float *w, int cin, int cout, int cin_pad, int cout_pad, int transposed,
                              void *pack, void *stream);
/* Number of 32 x 8 pixel tiles (blocks) of an Hz x Wx image. */
int fwigb_cnn_tile_count(int Hz, int Wx);
/* Per-tile partial weight gradients [tiles][9][cin_pad][cout_pad] (FP32) of
 * dL/dW[tap][ci][co] = sum_p x(p + tap offset)[ci] dz(p)[co]. */
int fwigb_cnn_wgrad_partials(const void *x, const void *dz, int Hz, int Wx, int cin_pad, int cout_pad,
                             float *partials, void *stream);
/* out[i] = sum over blocks b (in order) of partials[b * n + i]. */
int fwigb_cnn_reduce_partials(const float *partials, int nblocks, int n, float *out, void *stream);
/* Per-chunk partial sums over pixels of dz[p][c] (bias gradient):
 * partials[ceil(npix / chunk)][c_pad]. */
int fwigb_cnn_bias_partials(const void *dz, long long npix, int c_pad, int chunk, float *partials, void *stream);
/* Adam step (bias-corrected) on n FP32 parameters; step counts from 1. */
int fwigb_cnn_adam(float *w, const float *grad, float *m1, float *m2, int n, float lr, float beta1, float beta2,
                   float eps, int step, void *stream);
/* Packs FP32 weights W[9][cin][cout] into fragment order for a convolution
 * with cin_pad inputs / cout_pad outputs, or (transposed != 0) for its data
 * gradient: W'[tap][co][ci] = W[8 - tap][ci][co]. */
int fwigb_cnn_pack_weights(const float *w, int cin, int cout, int cin_pad, int cout_pad, int transposed, void *frag,
                           void *stream);
/* Masked MSE of the first nc channels of y (FP32 [npix][c_pad]) against
 * target (FP32 [npix][nc]): per-256-pixel partial loss sums, and
 * dy = 2 (y - target) mask * inv_count as BF16 [npix][c_pad]. c_pad = 16. */
int fwigb_cnn_mse_grad(const float *y, const float *target, const float *mask, long long npix, int c_pad, int nc,
                       float inv_count, void *dy, float *partials, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* FWIFLOW_GB300_H_ */
