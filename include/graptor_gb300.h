/*
 * graptor_gb300.h -- C ABI of the GB300 primal-dual TGV/TV reconstruction library.
 *
 * The library replaces the device side of Graptor's solver: the OpenCL program
 * and the enqueue loop of tgv_radon (radon_tgv_primal_dual_3d.py:96-848,
 * :1135-1292; radon_tgv_primal_dual_2d.py:95-463, :710-851).  Python (or any
 * FFI) keeps the reference's entry points Reconstructionapproach2d/3d and calls
 * the functions below; graptor_gb300/radon_tgv_primal_dual_{2d,3d}.py are those
 * adapters.
 *
 * Conventions
 *  - Every function returns an int status: GT_OK or one of GT_ERR_*; no C++
 *    exception crosses this boundary.  gt_last_error() gives the message of the
 *    calling thread's last failure.
 *  - Host arrays are caller-owned and copied; device memory is library-owned.
 *  - A problem handle is bound to one CUDA device and one stream and is not
 *    thread-safe; distinct handles may be used from distinct threads.
 *  - Array layouts on the host side are the reference solver's, per channel c and
 *    slice z with s = c*Nz + z (the reference's Nz*Number_Channels axis):
 *        image  float32[S][N][N]     index (s*N + y)*N + x
 *        sino   float32[S][nang][nd] index (s*nang + j)*nd + i
 *    vector fields carry a leading component axis ([K][S][N][N]).
 */
#ifndef GRAPTOR_GB300_H
#define GRAPTOR_GB300_H

#include <stddef.h>

#if defined(__GNUC__)
#define GT_API __attribute__((visibility("default")))
#else
#define GT_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* status codes (Reconstruction_coupled.py:509-536 maps OOM to a smaller chunk) */
enum {
  GT_OK = 0,
  GT_ERR_OOM = 1,       /* device allocation failed  (reference: pyopencl.MemoryError) */
  GT_ERR_ARG = 2,       /* invalid argument / unsupported configuration */
  GT_ERR_TIMEOUT = 3,   /* a bounded device wait ran out */
  GT_ERR_CUDA = 4,      /* any other CUDA failure      (reference: pyopencl.Error) */
  GT_ERR_STATE = 5      /* call out of order (e.g. run before data) */
};

enum { GT_KL = 0, GT_L2 = 1 };               /* discrepancy,   radon_tgv_primal_dual_3d.py:1053-1068 */
enum { GT_TV = 0, GT_TGV = 1 };              /* regularisation, :1040-1051 */
enum { GT_UNCORR = 0, GT_FROB = 1, GT_NUCL = 2 }; /* coupling, :1079-1130 */

/* state fields for gt_get_state / gt_set_state (the reference's U, U_, P, P_, V, W, Lamb) */
enum { GT_U = 0, GT_UBAR = 1, GT_P = 2, GT_PBAR = 3, GT_V = 4, GT_W = 5, GT_LAMBDA = 6, GT_KU = 7, GT_DATA = 8,
       GT_ULO = 9 /* low part of u in the precise primal mode (gt_set_precise_primal) */ };

/* Problem description.  Mirrors the argument surface of Reconstructionapproach2d/3d
 * (radon_tgv_primal_dual_2d.py:69, radon_tgv_primal_dual_3d.py:69). */
typedef struct gt_desc {
  int dim;              /* 2: slice-wise 2-D (Nz independent slices), 3: volumetric */
  int N;                /* image side; the reference always uses N = nd (3-D :1316) */
  int Nz;               /* slices per channel */
  int C;                /* channels */
  int nd;               /* detector bins */
  int nang;             /* projection angles */
  const double *angles; /* radians, caller-shifted by +pi/2 as Reconstruction_coupled.py:233/:448 */
  float stepsize;       /* slice step (3-D z-derivative divisor), Stepsize argument */
  double alpha0;        /* second-order TGV weight, Parameter[0] */
  double alpha1;        /* first-order weight,      Parameter[1] */
  const double *mu;     /* [C] channel weights */
  int discrepancy;      /* GT_KL / GT_L2 */
  int regularisation;   /* GT_TV / GT_TGV */
  int coupling;         /* GT_UNCORR / GT_FROB / GT_NUCL */
  double normest;       /* > 0: use this operator-norm estimate; <= 0: FP64 power iteration on device */
  int device;           /* CUDA device ordinal */
  void *stream;         /* cudaStream_t to run on, or NULL for a library-owned stream */
  int autotune;         /* != 0: time the projector launch shapes at gt_set_data and keep the fastest */
} gt_desc;

typedef struct gt_problem gt_problem;

/* Allocate device state for one problem (replaces tgv_radon's buffer setup,
 * radon_tgv_primal_dual_3d.py:1147-1176, and radon_struct :947-979). */
GT_API int gt_problem_create(const gt_desc *desc, gt_problem **out);
GT_API void gt_problem_destroy(gt_problem *p);

/* Upload the sinogram data f (host, [S][nang][nd]) and reset the iterates to zero.
 * make_feasible != 0 applies Make_function_feasible (3-D :860-870).  This is also
 * where the operator norm is estimated when desc.normest <= 0 (3-D :1018-1030). */
GT_API int gt_set_data(gt_problem *p, const float *f_host, int make_feasible);

/* Run iters primal-dual iterations (the loop body of 3-D :1194-1221), graph-captured,
 * asynchronous on the problem's stream. */
GT_API int gt_run(gt_problem *p, int iters);
/* Wait for the problem's stream; GT_ERR_TIMEOUT if a kernel gave up a bounded wait
 * since the last call (the iterate is then invalid; the flag is cleared). */
GT_API int gt_synchronize(gt_problem *p);

/* Copy one state field to / from host memory in the layout described above.
 * GT_U after gt_run is the reference's returned Solution, GT_KU its Sinogram. */
GT_API int gt_get_state(gt_problem *p, int field, float *host);
/* The 3-D entry point's return values in float64, converted and reordered on the
 * device: GT_U as Solution [C][x][y][z] and GT_KU as Sinogram [C][nang][Nz][nd]
 * (radon_tgv_primal_dual_3d.py:1277-1318, the arrays Reconstructionapproach3d
 * returns).  host holds C N N Nz, resp. C nang Nz nd doubles.  Host-synchronous. */
GT_API int gt_get_output_f64(gt_problem *p, int field, double *host);
GT_API int gt_set_state(gt_problem *p, int field, const float *host);

/* Launch shapes the autotuner chose: [0] forward projector, [1] back projector
 * (indices into the configurations listed at launch_fwd / launch_bp). */
GT_API int gt_get_tuning(gt_problem *p, int out[2]);
/* Force the projector launch shapes (for tests and measurements); the values
 * range over the configurations listed at launch_fwd / launch_bp. */
GT_API int gt_set_tuning(gt_problem *p, int fwd_cfg, int bp_cfg);
/* Launch shape of the dual kernel: 0 = one slice per thread (every case),
 * 1 = two slices per thread with float2 accesses (3-D TGV, Frobenius or
 * uncorrelated coupling, C <= 4, Nz even), 2 = shape 0 with registers capped
 * for 5 resident blocks per SM (C <= 4), 3-5 = every operand loaded ahead of the
 * arithmetic (C <= 4; one channel ahead in blocks of 128 threads, all loads
 * first in blocks of 128 or 64 threads), 6 = one thread per voxel-channel and
 * 7 = per channel and slice pair (Frobenius or uncorrelated coupling, C <= 4;
 * 7 needs 3-D and Nz even), 8, 9 = shapes 6, 7 in blocks of 128 threads.  All
 * give bit-identical iterates; the autotuner picks the fastest.
 * gt_get_dual_shape returns the current one. */
GT_API int gt_set_dual_shape(gt_problem *p, int cfg);
GT_API int gt_get_dual_shape(gt_problem *p);
/* Iteration schedule.  1: the p / pbar half of the primal update (update_p +
 * its extrapolation, radon_tgv_primal_dual_3d.py:734-757, :1217-1221) runs right
 * after the dual update, beside the projector chain, and only the u / ubar half
 * (update_u, :706-729) waits for the back projection; 0: the whole primal update
 * runs after the back projection; 2 (3-D TGV, Frobenius or uncorrelated coupling,
 * C <= 4, Nz even): the p / pbar half of each iteration is computed inside the
 * next iteration's dual kernel (pbar at a voxel and its three predecessors from p,
 * v, w), which writes p, v, w to a second buffer set (12 floats per voxel-channel,
 * allocated by this call or the autotuner); the sets alternate within a run of
 * gt_run and every gt_run ends on the problem's own set with the state of plain
 * iterations.  The reference enqueues update_u then update_p after radon_ad
 * (:1194-1221); all schedules give bit-identical iterates.  The autotuner
 * (gt_set_data) times them as graph-captured iterations and keeps the fastest,
 * unless gt_set_schedule chose one; gt_get_schedule returns the current. */
GT_API int gt_set_schedule(gt_problem *p, int schedule);
/* Precise primal mode (no counterpart in the reference, off by default).  The
 * reference stores u in float32, so a primal step smaller than half an ulp of u
 * is lost; near convergence that stalls the relative primal-dual gap at a few
 * 1e-4 on volumes of 64^2 x 16 and more (an FP64 run of the same iteration keeps
 * falling).  With on = 1, u is held as two floats (u and a low part, 4 more bytes
 * per voxel-channel, allocated here and reset with the iterate): each step is
 * added to the low part and the pair renormalised (TwoSum), ubar is rounded from
 * the pair; everything else is unchanged.  gt_get_state(GT_U) returns the high
 * part and GT_ULO the low part (field of the image's size; GT_ERR_ARG when the
 * mode is off); setting u (gt_set_state, gt_set_state_device) clears the low
 * part, so a checkpoint restores u first, then GT_ULO. */
GT_API int gt_set_precise_primal(gt_problem *p, int on);
GT_API int gt_get_precise_primal(gt_problem *p);
GT_API int gt_get_schedule(gt_problem *p);

/* Time-to-gap building blocks (restarted primal-dual iterations).  No
 * counterpart in the reference, which always runs a fixed iteration count with
 * sigma = tau = 1/sqrt(Lsqr) (radon_tgv_primal_dual_3d.py:1180-1184).
 * gt_set_primal_weight: sigma = w/sqrt(Lsqr), tau = 1/(w sqrt(Lsqr)) (sigma tau
 * Lsqr stays 1, so the iteration still converges); w = 1 is the reference's step
 * pair and the default; kept across gt_set_data.  gt_restart: ubar = u, pbar = p
 * (the extrapolation restarts from the current point).  gt_snapshot copies
 * (u, p, v, w, lambda) aside (allocated on first use); gt_movement writes the L2
 * distance of the primal (u, p) and dual (v, w, lambda) parts from that copy to
 * out[0], out[1] (host-synchronous). */
GT_API int gt_set_primal_weight(gt_problem *p, double w);
GT_API double gt_get_primal_weight(gt_problem *p);
GT_API int gt_restart(gt_problem *p);
GT_API int gt_snapshot(gt_problem *p);
GT_API int gt_movement(gt_problem *p, double out[2]);

/* Test hook of the TMA-staged back projection (back-projection shapes 14, 15):
 * its next launches never issue the copy of `angle` (a wait nothing completes)
 * and poll at most `wait_limit` times per wait, so every block gives up, flags
 * the error and returns; gt_synchronize then reports GT_ERR_TIMEOUT.  angle < 0
 * restores normal operation (wait_limit 4194304 is the default). */
GT_API int gt_test_bp_stall(gt_problem *p, int angle, unsigned wait_limit);

/* Scalars the run uses: [0] normest, [1] sigma, [2] tau, [3] iterations run. */
GT_API int gt_get_scalars(gt_problem *p, double out[4]);

/* FP64 primal-dual gap of the current iterate (the reference has none; draft
 * at 3-D :882-927).  Problem solved by the loop (ne = operator-norm estimate,
 * K = R/ne, a~ = alpha/ne^2):
 *   P(u,p) = a1~ sum |grad u - p| + a0~ sum |E p|_W* + D(u),  u in [0, U]
 *   D_KL = (1/ne) sum mu (R u - f + f log(f/R u)),  D_L2 = sum mu/(2 ne^2) |R u - f|^2
 * Dual from the current (v, w, lambda): v~ = E^T w rescaled by theta into its
 * ball, dual value -F~*(lambda) + U sum min(0, K^T lambda + grad^T v~).
 * out: [0] primal, [1] dual, [2] P - D, [3] relative gap (P - D)/|P|;
 * U = 2 max(u). */
GT_API int gt_gap(gt_problem *p, double out[4]);

/* gt_gap with the box bound U given (U <= 0: 2 max(u)); out additionally
 * [4] theta, [5] U, [6] data term, [7] F~*(lambda). */
GT_API int gt_gap_ex(gt_problem *p, double U, double out[8]);

/* Standalone projectors on device memory in the library's device layout
 * (image [N*N][S], sinogram [nang*nd][S]); for tests and data generation.
 * Kernels `radon` (3-D :773-816) and `radon_ad` (3-D :818-844). */
GT_API int gt_radon(const float *img_dev, float *sino_dev, const double *angles, int N, int nd, int nang, int S,
             void *stream);
GT_API int gt_radon_ad(const float *sino_dev, float *img_dev, const double *angles, int N, int nd, int nang, int S,
                void *stream);

/* Run reps iterations kernel by kernel (not graph-captured, no overlap), timing
 * each kernel with CUDA events on the problem stream; ms_out[0..3] receive the
 * mean duration of k_dual, k_fwd, k_bp and k_update (n >= 4); with n >= 6 the
 * update runs as its two halves, ms_out[4] and ms_out[5] receive the u / ubar and
 * the p / pbar half and ms_out[3] their sum.  The iterations are real: the state
 * advances by reps iterations.  With n >= 7, ms_out[6] receives the fused dual
 * kernel of schedule 2 (timed afterwards on the state, into the second buffer set
 * only; 0 when schedule 2 is not set or does not apply). */
GT_API int gt_time_kernels(gt_problem *p, int reps, float *ms_out, int n);

/* Allocation-free operator-norm estimate.  No counterpart in the reference (which
 * estimates the norm inside tgv_radon with freshly allocated buffers).
 *
 * For callers that cannot allocate device memory while they run -- code inside a
 * host framework that owns the device memory (its pool or caching allocator), or
 * latency-sensitive code that cannot afford cudaFree's device-wide
 * synchronisation.  It runs the FP64 power iteration of gt_set_data (normest <= 0)
 * for the geometry (angles, N, nd, nang) on `device` / `stream` and writes the
 * estimate to *out, without cudaMalloc, cudaFree or any other allocation: its
 * scratch is a fixed 8 MiB device array inside the library (kept by every GPU
 * that loads the library until the process exits).
 * Limit: 4*nang + N*N + nd*nang + 256 <= 1048576 (doubles); larger geometries
 * return GT_ERR_ARG.  Every call is host-synchronous: it synchronises `stream`
 * and copies the estimate to the host before returning, so it blocks the calling
 * thread and must never be made on a stream that is being captured.  Calls share
 * the scratch: calls from concurrent host threads for one device race on it, so
 * serialise them.  Each call looks up the scratch's device address afresh (valid
 * after cudaDeviceReset too); the first call on a device also loads the library's
 * device code there.  The caller's current device is unchanged on return, on
 * success and on error. */
GT_API int gt_normest_noalloc(const double *angles, int N, int nd, int nang, int device, void *stream, double *out);

/* Batches of independent problems (uneven sizes, channels, angle sets,
 * discrepancies) on one device.  Each problem keeps its own buffers and tuned
 * launch shapes; gt_batch_run captures a chunk of iterations of all problems
 * into one CUDA graph as parallel branches and launches it, so one launch
 * advances the whole batch.  Data and results go through the member problems
 * (gt_batch_problem + gt_set_data / gt_get_state / gt_gap).  After changing a
 * member's data call gt_batch_invalidate before the next gt_batch_run.
 * (The reference solves problems one at a time: Reconstruction_coupled.py:188, :414.) */
typedef struct gt_batch gt_batch;
GT_API int gt_batch_create(int n, const gt_desc *descs, gt_batch **out);
GT_API void gt_batch_destroy(gt_batch *b);
GT_API int gt_batch_size(const gt_batch *b);
GT_API int gt_batch_problem(gt_batch *b, int k, gt_problem **out);
GT_API int gt_batch_run(gt_batch *b, int iters);
GT_API int gt_batch_synchronize(gt_batch *b);
GT_API int gt_batch_invalidate(gt_batch *b);
/* Run the batch's problems on `chains` concurrent chains (problem k on chain
 * k mod chains, one after another within a chain); default 8. */
GT_API int gt_batch_set_concurrency(gt_batch *b, int chains);
/* Leave problem k out of (active = 0) or bring it back into (1) the following
 * gt_batch_run calls, e.g. once it has reached its gap tolerance; its state is
 * kept.  All problems are active after gt_batch_create. */
GT_API int gt_batch_set_active(gt_batch *b, int k, int active);
/* How gt_batch_run advances the batch.  Mode 0 (default): one graph of the
 * members' own iterations (their tuned launch shapes and schedules) on
 * concurrent chains.  Mode 1 (fused): per iteration four launches, each over the
 * work units of every active member (dual update, forward projection + data
 * prox, back projection, primal update), every member with one fixed launch
 * shape; for many small problems, where per-member launches leave the GPU
 * underfilled.  Mode 1 needs every member to share the dimension, the
 * regularisation and the coupling (Frobenius or uncorrelated, <= 8 channels);
 * it returns GT_ERR_ARG otherwise.  Iterates are identical in both modes. */
GT_API int gt_batch_set_mode(gt_batch *b, int mode);
GT_API int gt_batch_get_mode(const gt_batch *b);

/* Kernels of the learned warm start (a small 3-D U-Net whose output initialises
 * the solver's image).  No counterpart in the reference, which always starts
 * from zero (radon_tgv_primal_dual_3d.py:1147-1176).  All pointers are device
 * pointers; tensors are [B][C][D][H][W] with W fastest; dtype codes are
 * 0 = float32, 1 = bfloat16.  Weights are bfloat16 [Co][Ci][k][k][k] (k = 1 or 3),
 * biases float32; every sum accumulates in float32.  Calls are asynchronous on
 * `stream`.
 *
 * A tensor argument is a channel-offset view: channels [off, off+C) of a tensor
 * with Ctot channels (x: Cx / x_off, y: Cy / co_off, dy: Cdy / dy_off), so the
 * U-Net's skip concatenations need no copies.
 *
 * gt_nn_conv3d: y view = conv(x view, w) + bias, optionally ReLU'd (relu = 1)
 *   and added to y first (accumulate = 1); W % 4 == 0.  With the weights of
 *   gt_nn_flip_weights, no bias and dy as x, it gives the data gradient.
 * gt_nn_flip_weights: wf[ci][co][t] = w[co][ci][k^3-1-t].
 * gt_nn_conv3d_wgrad: g[co][ci][t] (+)= sum over batch and voxels of
 *   dy[co] * x[ci] shifted by tap t; `part` holds ceil(B*D*H*W / kchunk)*Co*Ci*k^3
 *   floats of partial sums, reduced in a fixed order (deterministic).
 * gt_nn_bias_grad: db[co] (+)= sum of dy[:, co].
 * gt_nn_scale: y[b][c] = x[b][c] * scale[b*C + c] (scale on the device),
 *   floored at zero when floor0 = 1; also converts between dtypes.
 * gt_nn_relu_bwd: dy = 0 where y is not > 0 (dy and y: the same view).
 * gt_nn_pool2 / gt_nn_pool2_bwd: 2x2x2 average pooling of channels
 *   [off, off+C) of a wider tensor, and its gradient (added into dx).
 * gt_nn_up2 / gt_nn_up2_bwd: nearest 2x upsampling into channels [off, off+C)
 *   of a wider tensor, and its gradient.
 * gt_nn_mse: dp = 2 (p - q) / n and per-256-block partial sums of (p - q)^2
 *   (ceil(n/256) floats in part).
 * gt_nn_adam: Adam step (bias-corrected, step >= 1) on float32 master weights,
 *   refreshing the bfloat16 copy when w_bf16 is not NULL.
 * gt_nn_cast: float32 <-> bfloat16 (src_dtype 0: f32 -> bf16, 1: bf16 -> f32).
 * gt_nn_set_tensor_cores: 1 (default) runs gt_nn_conv3d with bfloat16 input,
 *   Ci % 16 == 0, Co % 16 == 0 and Co <= 256 on the tensor cores (tcgen05 MMA, FP32
 *   accumulator in tensor memory): 3x3x3 convolutions with Co <= 128 whose
 *   128-voxel blocks lie in one plane and cover whole rows (H W % 128 == 0 and W
 *   dividing 128 or a multiple of it) by the kernel that stages each 16-channel
 *   chunk's input halo and weights in shared memory once, the others by the kernel
 *   that gathers every tap's operands from global memory; 2 uses the gathering
 *   kernel for all of them; 0 keeps every convolution on the CUDA cores.
 * gt_nn_check: GT_ERR_TIMEOUT if a tensor-core convolution block gave up a bounded
 *   wait since the last call (its output is then not written; the flag is cleared);
 *   call it after synchronising the stream the convolutions ran on. */
GT_API int gt_nn_set_tensor_cores(int on);
GT_API int gt_nn_check(void);
GT_API int gt_nn_conv3d(const void *x, int x_dtype, int Ci, int Cx, int x_off, const void *w_bf16, const float *bias,
                        void *y, int y_dtype, int Co, int Cy, int co_off, int B, int D, int H, int W, int ksize,
                        int relu, int accumulate, void *stream);
GT_API int gt_nn_flip_weights(const void *w_bf16, void *wf_bf16, int Co, int Ci, int ksize, void *stream);
GT_API int gt_nn_conv3d_wgrad(const float *dy, int Co, int Cdy, int dy_off, const void *x, int x_dtype, int Ci, int Cx,
                              int x_off, int B, int D, int H, int W, int ksize, long long kchunk, float *part,
                              float *g, int accumulate, void *stream);
GT_API int gt_nn_bias_grad(const float *dy, int Co, int Cdy, int dy_off, int B, long long vol, float *db,
                           int accumulate, void *stream);
GT_API int gt_nn_scale(const void *x, int x_dtype, void *y, int y_dtype, int C, int B, long long vol,
                       const float *scale, int floor0, void *stream);
GT_API int gt_nn_relu_bwd(float *dy, const void *y, int y_dtype, int C, int Cy, int co_off, int B, long long vol,
                          void *stream);
GT_API int gt_nn_pool2(const void *x_bf16, int Cs, int src_off, void *y_bf16, int C, int B, int Do, int Ho, int Wo,
                       void *stream);
GT_API int gt_nn_pool2_bwd(const float *dy, float *dx, int C, int Cd, int dst_off, int B, int D, int H, int W,
                           void *stream);
GT_API int gt_nn_up2(const void *x_bf16, void *y_bf16, int C, int Cd, int dst_off, int B, int D, int H, int W,
                     void *stream);
GT_API int gt_nn_up2_bwd(const float *dy, int Cs, int src_off, float *dx, int C, int B, int Di, int Hi, int Wi,
                         void *stream);
GT_API int gt_nn_mse(const float *p, const float *q, long long n, float *dp, float *part, void *stream);
GT_API int gt_nn_adam(float *w_master, void *w_bf16, const float *g, float *m, float *v, long long n, float lr,
                      float b1, float b2, float eps, int step, void *stream);
GT_API int gt_nn_cast(const void *src, int src_dtype, void *dst, long long n, void *stream);

/* Device-side state access (for the warm start): like gt_get_state /
 * gt_set_state, in the same [comps][S][X] order, but to / from a device buffer,
 * asynchronous on the problem's stream (no host synchronisation). */
GT_API int gt_get_state_device(gt_problem *p, int field, float *dev);
GT_API int gt_set_state_device(gt_problem *p, int field, const float *dev);
/* Set the data dual lambda to the value consistent with the current u: the fixed
 * point of the reference's lambda update for K u (KL: mu (1 - f / K u), kept
 * where f > 10 K u, K u = 0 included; L2: mu (K u - f)).  For warm starts (set u, then this).  No
 * counterpart in the reference, which starts lambda at zero. */
GT_API int gt_dual_from_primal(gt_problem *p);
/* gt_dual_from_primal with options.  empty_weight in [0, 1]: on bins without data
 * (f = 0) lambda moves that fraction of the way to its fixed point (KL: mu,
 * where K u > 0; L2: mu K u); 1 is gt_dual_from_primal, 0 leaves those bins.
 * GT_DUAL_CAP10 / GT_DUAL_CAP100: where f > 10 K u (K u = 0 included) set
 * lambda = mu (1 - cap) with cap 10 / 100 instead of keeping it, a bounded strong
 * push on rays that the image misses.  GT_DUAL_REPAIR (KL): first lift u and ubar
 * along every ray with data (f > 0) that the image misses (K u = 0) by a back
 * projection of f / N on those bins, so that the primal value is finite;
 * GT_DUAL_REPAIR | GT_DUAL_NO_RESET does only that lift and leaves lambda. */
enum { GT_DUAL_CAP10 = 2, GT_DUAL_CAP100 = 4, GT_DUAL_REPAIR = 8, GT_DUAL_NO_RESET = 16 };
GT_API int gt_dual_from_primal_ex(gt_problem *p, int flags, float empty_weight);
/* The problem's CUDA stream (the one gt_desc.stream named, or its own). */
GT_API void *gt_problem_stream(gt_problem *p);

/* Two-resolution subsampling: Reconstructionapproach3dsubsmapling
 * (radon_tgv_primal_dual_3dsubsample.py:51).  Channels [0, C0) have sinograms on
 * the image's own detector (N bins, Nz slices, tilt series angles0); channels
 * [C0, C0+C1) have sinograms on a coarser grid (nd1 bins, Nz1 slices, tilt series
 * angles1) related to the fine grid by the reference's area-weighting matrix
 * (Create_sparse_matrix :631-651) built from pixel_ratio, refold, refnew and
 * stepsize.  The TGV regulariser couples all channels on the fine grid. */
typedef struct gt_subs gt_subs;
typedef struct gt_subs_desc {
  int N, Nz;            /* fine image N x N x Nz (detectors N) */
  int C0, C1;           /* channels with fine / coarse data (C0 + C1 <= 8, C1 >= 1) */
  int nang0, nang1;     /* angles of the two tilt series */
  int nd1, Nz1;         /* coarse detector bins and slices */
  const double *angles0, *angles1; /* radians, +pi/2 as the reference's callers pass them */
  float stepsize;
  double alpha0, alpha1;
  const double *mu;     /* [C0 + C1] */
  int discrepancy, regularisation, coupling;  /* coupling: GT_FROB or GT_UNCORR */
  double pixel_ratio;   /* coarse pixel size / fine pixel size (Topology p) */
  double refold[2];     /* reference point on the coarse grid (x, z) */
  double refnew[2];     /* the same point on the fine grid (x, z) */
  double normest;       /* > 0 used as given, else a power iteration from the all-ones image */
  int device;
  void *stream;
} gt_subs_desc;
enum { GT_SUBS_U = 0, GT_SUBS_KU0 = 1, GT_SUBS_KU1 = 2, GT_SUBS_KULO = 3 };
GT_API int gt_subs_create(const gt_subs_desc *d, gt_subs **out);
GT_API void gt_subs_destroy(gt_subs *s);
/* f0 [C0*Nz][nang0][N], f1 [C1*Nz1][nang1][nd1] (s = c*Nz + z); resets the iterates */
GT_API int gt_subs_set_data(gt_subs *s, const float *f0, const float *f1, int make_feasible);
GT_API int gt_subs_run(gt_subs *s, int iters);
/* GT_SUBS_U [(C0+C1)*Nz][N][N]; GT_SUBS_KU0 [C0*Nz][nang0][N]; GT_SUBS_KU1 [C1*Nz][nang1][N];
 * GT_SUBS_KULO [C1*Nz1][nang1][nd1] (the last iteration's projections) */
GT_API int gt_subs_get(gt_subs *s, int which, float *host);
GT_API double gt_subs_normest(const gt_subs *s);
/* the inner fine-grid problem (for gt_get_state / gt_set_state of the iterates) */
GT_API gt_problem *gt_subs_problem(gt_subs *s);

/* Number of kernel launches one iteration issues (for launch accounting). */
GT_API int gt_launches_per_iteration(const gt_problem *p);

/* Detection of unsuitable projections: the array stages of Find_Bad_projections
 * (find_bad_ele.py:139-230), whose host steps (loading, subsampling, combining the
 * neighbour errors, ranking) stay with the caller.  Stacks are [na][nz][nx] with nx
 * fastest; all pointers are device pointers; calls are asynchronous on `stream`.
 *
 * gt_badproj_smooth: out [na][nz-2s][nx-2s] (float32) = the (2s+1)^2 box sum of data
 *   (float64, summed in float64 row by row) / (4 s^2)       (reduce_noise, :69-75; s >= 1)
 * gt_badproj_wgrad: w [na][nz-2][nx-2] = max over the 8 neighbours of |c - nb|
 *   (diagonals divided by sqrt 2) times min |nb|, in float32   (weighted_gradient, :103-136)
 * gt_badproj_blocks: number of partial sums gt_badproj_compare writes per pair for this
 *   image size and radius; 0 when the radius leaves no interior pixel.
 * gt_badproj_compare: for every pair q = 0 .. na-offset-1 of projections (q, q+offset),
 *   err[q] = sum over the interior [r, nz-r) x [r, nx-r) of
 *   max(min_shift |U - V shifted|, min_shift |V - U shifted|), shifts |dz|, |dx| <= r,
 *   differences in float32, sums in float64 (compare_shift_twosided, :55-100, with the
 *   pairs of :177-190).  part holds gt_badproj_blocks(nz, nx, r) * (na - offset)
 *   doubles; e_out, when not NULL, receives the per-pixel maxima [na-offset][nz-2r][nx-2r].
 *   GT_ERR_ARG when the radius leaves no interior pixel. */
GT_API int gt_badproj_smooth(const double *data, int na, int nz, int nx, int steps, float *out, void *stream);
GT_API int gt_badproj_wgrad(const float *u, int na, int nz, int nx, float *w, void *stream);
GT_API int gt_badproj_blocks(int nz, int nx, int radius);
GT_API int gt_badproj_compare(const float *w, int na, int nz, int nx, int offset, int radius, double *part,
                              double *err, float *e_out, void *stream);

GT_API const char *gt_last_error(void);
GT_API const char *gt_version(void);

#ifdef __cplusplus
}
#endif
#endif /* GRAPTOR_GB300_H */
