// C ABI of the GB300 primal-dual TGV/TV reconstruction (declared in
// include/graptor_gb300.h): problem handles, host<->device layout changes,
// step-size setup and the graph-captured iteration loop.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <map>
#include <mutex>
#include <tuple>
#include <cstdio>
#include <cstdlib>
#include <algorithm>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "graptor_gb300.h"
#include "gt_common.cuh"

namespace gt {
cudaError_t launch_dual(const IterParams &P, int tgv, int cpl, cudaStream_t st);
bool dual_fused_ok(const IterParams &P, int tgv, int cpl);
cudaError_t launch_dual_fused(const IterParams &P, int tgv, int cpl, cudaStream_t st);
cudaError_t prepare_dual_fused(const IterParams &P, int cpl);
cudaError_t prepare_bp_tma();
cudaError_t launch_fwd(const IterParams &P, int disc, cudaStream_t st);
cudaError_t launch_bp(const IterParams &P, cudaStream_t st);
cudaError_t launch_update(const IterParams &P, int tgv, cudaStream_t st, int part);
cudaError_t launch_radon(const float *img, float *sino, const float4 *ofs, int N, int nd, int nang, int S,
                         cudaStream_t st);
cudaError_t launch_radon_ad(const float *sino, float *img, const float4 *ofs, int N, int nd, int nang, int S,
                            cudaStream_t st);
cudaError_t launch_transpose(const float *in, float *out, int rows, int cols, cudaStream_t st);
cudaError_t launch_output_f64(const float *in, double *out, int A, int B, int C, int Nz, int mode, cudaStream_t st);
cudaError_t launch_feasible(float *f, const float *r1, int nbin1, int S, cudaStream_t st);
cudaError_t launch_lambda_fixed(float *lam, const float *ku, const float *f, const double *mu, long long nbin, int S,
                                int Nz, int disc, float empty_weight, float cap, cudaStream_t st);
cudaError_t launch_missed_rays(const float *ku, const float *f, float *r, long long n, int N, cudaStream_t st);
cudaError_t launch_gather_slices(const float *src, int S, int s0, float *dst, int Sg, long long X, cudaStream_t st);
cudaError_t launch_scatter_slices(const float *src, int Sg, float *dst, int S, int s0, long long X, cudaStream_t st);
cudaError_t launch_csr_planes(const float *in, float *out, const int *start, const int *idx, const float *val,
                              int nang, int C, int nx_o, int nz_o, int nx_i, int nz_i, cudaStream_t st);
cudaError_t launch_lambda_update(float *lam, const float *ku, const float *f, const float *mu, float sigma,
                                 long long n, int S, int Nz, int disc, cudaStream_t st);
cudaError_t launch_sumsq(const float *x, long long n, double *part, int nb, cudaStream_t st);
cudaError_t launch_sqdiff(const float *a, const float *b, long long n, double *part, int nb, cudaStream_t st);
long long batch_blocks(const Dims &d, int ph);
int batch_shape(const Dims &d);
cudaError_t launch_batch_phase(const BatchTab &T, int ph, long long blocks, int dim, int tgv, int cpl, int cmax,
                               cudaStream_t st);
cudaError_t launch_scale_f32(float *x, long long n, float s, cudaStream_t st);
cudaError_t launch_add2(float *a, float *b, const float *d, long long n, cudaStream_t st);
cudaError_t normest64(const dvec4 *ofs, int N, int nd, int nang, int rounds, double *d_img, double *d_sino,
                      double *d_part, double *out, cudaStream_t st);
cudaError_t fill_f64(double *x, size_t n, double v, cudaStream_t st);
cudaError_t fill_f32(float *x, size_t n, float v, cudaStream_t st);
cudaError_t launch_ray_count(const float4 *ofs, int N, int nd, int nang, int *count, cudaStream_t st);
cudaError_t launch_ray_fill(const float4 *ofs, int N, int nd, int nang, const long long *start, int2 *ent,
                            cudaStream_t st);
cudaError_t launch_bp_table(const float4 *ofs, int N, int nd, int nang, int2 *tab, cudaStream_t st);
cudaError_t launch_run_count(const float4 *ofs, int N, int nd, int nang, int *count, cudaStream_t st);
size_t row_table_bytes(int N, int nang);
cudaError_t launch_row_fill(const float4 *ofs, int N, int nd, int nang, int4 *tab, int *bad, cudaStream_t st);
cudaError_t launch_run_fill(const float4 *ofs, int N, int nd, int nang, const long long *start, int4 *ent,
                            cudaStream_t st);
int num_proj_configs(int S, int which);
bool dual_z2_ok(const IterParams &P, int tgv, int cpl);
int num_dual_configs(const IterParams &P);
bool dual_cl_ok(const IterParams &P, int cpl);
bool dual_cl2_ok(const IterParams &P, int cpl);
int gap_blocks(const IterParams &P);
cudaError_t launch_gap_pass1(const IterParams &P, int disc, int tgv, int cpl, float *vt, double *part, int nb,
                             cudaStream_t st);
cudaError_t launch_gap_pass2(const IterParams &P, const float *vt, double theta, double U, double *part, int nb,
                             cudaStream_t st);
}  // namespace gt

namespace {

thread_local std::string g_err;

int set_err(int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

int cuda_err(cudaError_t e, const char *what, int line) {
  cudaGetLastError();  // clear a sticky-free error so the next call starts clean
  const int code = (e == cudaErrorMemoryAllocation) ? GT_ERR_OOM : GT_ERR_CUDA;
  return set_err(code, "%s failed (line %d): %s", what, line, cudaGetErrorString(e));
}

#define CK(call)                                                         \
  do {                                                                   \
    cudaError_t e_ = (call);                                             \
    if (e_ != cudaSuccess) return cuda_err(e_, #call, __LINE__);         \
  } while (0)

// Angle table of radon_struct (radon_tgv_primal_dual_3d.py:947-979): per angle
// (X, Y, offset, Xinv) = (cos, sin, centring offset, 1/cos) in double, with
// near-vertical rays (|1/cos| > 10 nd) made exactly vertical.  Detector width 1,
// shift 0 (the reference's defaults, which its callers never change).
void angle_table(const double *angles, int N, int nd, int nang, std::vector<double> &t64) {
  t64.assign((size_t)nang * 4, 0.0);
  const double mid_dom = (N - 1) / 2.0, mid_det = (nd - 1.0) / 2.0;
  for (int j = 0; j < nang; ++j) {
    double X = std::cos(angles[j]), Y = std::sin(angles[j]), Xinv = 1.0 / X;
    if (std::fabs(Xinv) > 10.0 * nd) {
      X = 0.0;
      Y = std::nearbyint(std::sin(angles[j]));  // NumPy round(): half to even
      Xinv = 0.0;
    }
    t64[4 * j + 0] = X;
    t64[4 * j + 1] = Y;
    t64[4 * j + 2] = mid_det - X * mid_dom - Y * mid_dom;
    t64[4 * j + 3] = Xinv;
  }
}

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

// cuTensorMapEncodeTiled from the driver (through the runtime's entry-point query,
// so the library needs no link against libcuda)
using EncodeTiledFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                   const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn encode_tiled() {
  static std::once_flag once;
  static EncodeTiledFn fn = nullptr;
  std::call_once(once, [] {
    void *ptr = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(ptr);
    cudaGetLastError();
  });
  return fn;
}

// TMA descriptor of lambda [nang][nd][S] for k_bp_tma: boxes of 16 bins x
// `slices` slices of one angle, zero fill outside.  False where S % 4 != 0 or the driver
// declines; the back projection then keeps its other shapes.
bool encode_lambda_map(CUtensorMap *map, float *lam, int S, int nd, int nang, unsigned slices) {
  EncodeTiledFn fn = encode_tiled();
  if (!fn || S % 4 != 0 || reinterpret_cast<uintptr_t>(lam) % 16 != 0) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)S, (cuuint64_t)nd, (cuuint64_t)nang};
  const cuuint64_t strides[2] = {(cuuint64_t)S * sizeof(float), (cuuint64_t)nd * S * sizeof(float)};
  const cuuint32_t box[3] = {slices, 16, 1};
  const cuuint32_t estride[3] = {1, 1, 1};
  return fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, lam, dims, strides, box, estride, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

struct gt_problem {
  gt::Dims d{};
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t side = nullptr;            // second stream: k_fwd runs beside k_dual
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  bool own_stream = false;
  int disc = GT_KL, reg = GT_TGV, cpl = GT_FROB;
  int K = 3, KW = 6;
  float stepsize = 1.f;
  double alpha0 = 4, alpha1 = 1, ne_in = 0, ne = 0, sigma = 0, tau = 0;
  std::vector<double> mu, ofs64h;
  void *block = nullptr;
  float4 *ofs = nullptr;
  dvec4 *ofs64 = nullptr;
  float *mu_eff = nullptr;
  float *u = nullptr, *ubar = nullptr, *p = nullptr, *pbar = nullptr, *v = nullptr, *w = nullptr;
  float *lam = nullptr, *f = nullptr, *ku = nullptr, *stage = nullptr, *kstar = nullptr;
  void *rays = nullptr;        // ray table (offsets + entries), built at creation
  void *runs = nullptr;        // 3-bin run table (offsets + entries), built at creation
  void *tiles = nullptr;       // row-tile table of k_bp_row, built at creation
  size_t ray_bytes = 0;
  void *gap_ws = nullptr;      // gap workspace (v~ planes + FP64 block partials), allocated on first gt_gap
  float *snap = nullptr;       // copy of (u, p, v, w, lambda) for gt_movement, allocated on first gt_snapshot
  float *fused = nullptr;      // second (p, v, w) of schedule 2, allocated when that schedule is timed or set
  float *ulo = nullptr;        // low parts of u in the precise primal mode (gt_set_precise_primal), or null
  double pweight = 1.0;        // primal weight: sigma = w / sqrt(Lsqr), tau = 1 / (w sqrt(Lsqr)); 1 = reference
  double *mu64 = nullptr;
  gt::IterParams P{};
  bool autotune = true;
  cudaGraphExec_t g_one = nullptr, g_chunk = nullptr;
  int chunk = 16;
  int schedule = 1;            // 1: p / pbar half of the primal update beside the projectors; 0: one update after
                               // them; 2: the p / pbar half fused into the next iteration's dual kernel
  bool schedule_set = false;   // chosen by gt_set_schedule (the autotuner leaves it)
  long long iters = 0;
  bool has_data = false;
  double lsqr = 0;             // > 0: step-size constant of a variant (two-resolution solver: 36)
  int *flags = nullptr;        // device error flags (P.err)
  CUtensorMap bp_tmap{};       // TMA descriptors of lambda for k_bp_tma, boxes of 128 and 256
  CUtensorMap bp_tmap_wide{};  // slices (valid when P.bp_tmap / P.bp_tmap_wide are set)
};

namespace {

// One iteration as a fork/join.  The projector chain k_fwd -> k_bp (issue- and
// cache-bound) needs only ubar and lambda; k_dual (DRAM-bound) needs ubar, pbar,
// v, w; they write disjoint fields, so they run on two streams and overlap.
// The p / pbar half of the primal update (update_p and its extrapolation) needs
// only k_dual's v and w, so it follows k_dual on the main stream, beside the
// projectors; the u / ubar half needs K* lambda and waits for both streams.
// Schedule 0 runs the whole primal update after the join.  Both schedules compute
// every value by the same operations (bit-identical iterates).
int enqueue_iteration(gt_problem *p) {
  const int tgv = p->reg == GT_TGV;
  CK(cudaEventRecord(p->ev_fork, p->stream));
  CK(cudaStreamWaitEvent(p->side, p->ev_fork, 0));
  CK(gt::launch_fwd(p->P, p->disc, p->side));
  CK(gt::launch_bp(p->P, p->side));
  CK(gt::launch_dual(p->P, tgv, p->cpl, p->stream));
  if (p->schedule == 1) CK(gt::launch_update(p->P, tgv, p->stream, 2));
  CK(cudaEventRecord(p->ev_join, p->side));
  CK(cudaStreamWaitEvent(p->stream, p->ev_join, 0));
  CK(gt::launch_update(p->P, tgv, p->stream, p->schedule == 1 ? 1 : 0));
  return GT_OK;
}

// Schedule 2: m iterations (m odd, >= 3) software-pipelined.  The p / pbar half of
// iteration k's primal update runs inside iteration k + 1's dual kernel (the fused
// form of k_dual_cl2), beside that iteration's projectors, and only the u / ubar
// half follows the join.  The fused kernel reads p, v, w of one buffer set and
// writes the next p, v, w to the other, so the sets alternate: iteration 0 runs the
// plain dual kernel on the problem's own set, iterations 1 .. m - 1 alternate
// between the sets (an even number of them, so the last writes the problem's own
// set), and a last launch of the p half completes iteration m - 1 there, pbar
// included.  Outside the pipeline the state is the same as after m plain
// iterations, value for value (the fused kernel computes p and the dual update by
// the same operations).
int enqueue_pipelined(gt_problem *p, int m) {
  gt::IterParams A = p->P;
  A.p2 = p->fused;
  A.v2 = p->fused + (size_t)p->K * p->d.vol;
  A.w2 = A.v2 + (size_t)p->K * p->d.vol;
  gt::IterParams B = A;
  std::swap(B.p, B.p2);
  std::swap(B.v, B.v2);
  std::swap(B.w, B.w2);
  for (int k = 0; k < m; ++k) {
    const gt::IterParams &X = (k % 2 == 1) ? A : B;  // fused kernel input set
    CK(cudaEventRecord(p->ev_fork, p->stream));
    CK(cudaStreamWaitEvent(p->side, p->ev_fork, 0));
    CK(gt::launch_fwd(p->P, p->disc, p->side));
    CK(gt::launch_bp(p->P, p->side));
    if (k == 0) CK(gt::launch_dual(p->P, 1, p->cpl, p->stream));
    else CK(gt::launch_dual_fused(X, 1, p->cpl, p->stream));
    CK(cudaEventRecord(p->ev_join, p->side));
    CK(cudaStreamWaitEvent(p->stream, p->ev_join, 0));
    gt::IterParams Q = p->P;  // the u half reads the v just written
    if (k > 0) Q.v = X.v2;
    CK(gt::launch_update(Q, 1, p->stream, 1));
  }
  CK(gt::launch_update(p->P, 1, p->stream, 2));
  return GT_OK;
}

bool fused_available(const gt_problem *p) { return gt::dual_fused_ok(p->P, p->reg == GT_TGV, p->cpl); }

// the second (p, v, w) set of schedule 2
int ensure_fused(gt_problem *p) {
  if (p->fused) return GT_OK;
  const size_t n = (size_t)(2 * p->K + p->KW) * p->d.vol;
  cudaError_t e = gt::prepare_dual_fused(p->P, p->cpl);
  if (e != cudaSuccess) return cuda_err(e, "cudaFuncSetAttribute (fused dual kernel)", __LINE__);
  e = cudaMalloc(&p->fused, sizeof(float) * n);
  if (e != cudaSuccess) {
    cudaGetLastError();
    p->fused = nullptr;
    return cuda_err(e, "cudaMalloc (schedule 2 buffers)", __LINE__);
  }
  return GT_OK;
}

void free_fused(gt_problem *p) {
  if (p->fused) cudaFree(p->fused);
  p->fused = nullptr;
}

int chunk_len(const gt_problem *p) { return p->schedule == 2 ? 32 : p->chunk; }

int capture(gt_problem *p, int n, cudaGraphExec_t *out) {
  cudaGraph_t g = nullptr;
  CK(cudaStreamBeginCapture(p->stream, cudaStreamCaptureModeThreadLocal));
  int rc = GT_OK;
  int k = 0;
  if (p->schedule == 2 && n >= 3 && p->fused) {
    const int m = n % 2 ? n : n - 1;
    rc = enqueue_pipelined(p, m);
    k = m;
  }
  for (; k < n && rc == GT_OK; ++k) rc = enqueue_iteration(p);
  cudaError_t e = cudaStreamEndCapture(p->stream, &g);
  if (rc != GT_OK) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return cuda_err(e, "cudaStreamEndCapture", __LINE__);
  e = cudaGraphInstantiate(out, g, cudaGraphInstantiateFlagUseNodePriority);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return cuda_err(e, "cudaGraphInstantiate", __LINE__);
  return GT_OK;
}

// device field -> (pointer, components, per-component X extent)
int field_info(gt_problem *p, int field, float **ptr, int *comps, size_t *X) {
  const size_t img = (size_t)p->d.N * p->d.N, sino = (size_t)p->d.nd * p->d.nang;
  switch (field) {
    case GT_U: *ptr = p->u; *comps = 1; *X = img; break;
    case GT_UBAR: *ptr = p->ubar; *comps = 1; *X = img; break;
    case GT_P: *ptr = p->p; *comps = p->K; *X = img; break;
    case GT_PBAR: *ptr = p->pbar; *comps = p->K; *X = img; break;
    case GT_V: *ptr = p->v; *comps = p->K; *X = img; break;
    case GT_W: *ptr = p->w; *comps = p->KW; *X = img; break;
    case GT_LAMBDA: *ptr = p->lam; *comps = 1; *X = sino; break;
    case GT_KU: *ptr = p->ku; *comps = 1; *X = sino; break;
    case GT_DATA: *ptr = p->f; *comps = 1; *X = sino; break;
    case GT_ULO: *ptr = p->ulo; *comps = 1; *X = img; break;
    default: return set_err(GT_ERR_ARG, "unknown state field %d", field);
  }
  if (!*ptr) return set_err(GT_ERR_ARG, "state field %d does not exist for this problem (regularisation, mode)", field);
  return GT_OK;
}

void set_scalars(gt_problem *p) {
  // tgv_radon :1178-1189 (3-D) / :753-762 (2-D)
  const double Lsqr = p->lsqr > 0 ? p->lsqr : (p->d.dim == 3 ? 17.0 : 0.5 * (18.0 + std::sqrt(33.0)));
  // sigma tau Lsqr = 1 for every primal weight; weight 1 is the reference's sigma = tau
  p->sigma = p->pweight / std::sqrt(Lsqr);
  p->tau = 1.0 / (p->pweight * std::sqrt(Lsqr));
  const double ne2 = p->ne * p->ne;
  const double a0 = p->alpha0 / ne2, a1 = p->alpha1 / ne2;
  p->P.sigma = (float)p->sigma;
  p->P.tau = (float)p->tau;
  p->P.sigma_data = (float)(p->sigma / p->ne);
  p->P.norming = (float)(1.0 / p->ne);
  p->P.ainv0 = (float)(1.0 / a0);
  p->P.ainv1 = (float)(1.0 / a1);
  p->P.stepsize = p->stepsize;
}

// channel weights of the data-term prox: KL mu, L2 mu/(sigma+mu) (3-D :1186-1189)
int upload_mu_eff(gt_problem *p) {
  std::vector<float> me(p->d.C);
  for (int c = 0; c < p->d.C; ++c)
    me[c] = (float)(p->disc == GT_KL ? p->mu[c] : p->mu[c] / (p->sigma + p->mu[c]));
  CK(cudaMemcpyAsync(p->mu_eff, me.data(), sizeof(float) * p->d.C, cudaMemcpyHostToDevice, p->stream));
  CK(cudaStreamSynchronize(p->stream));  // me is a host buffer
  return GT_OK;
}

// ---------------------------------------------------------------------------
// Autotuner: times every launch shape of k_fwd and k_bp (gt_kernels.cu,
// launch_fwd / launch_bp) with CUDA events on the problem's own buffers and keeps
// the fastest; choices are cached per problem shape for the process lifetime.
// It runs inside gt_set_data before the iterates are reset, so the extra
// launches never touch the solve.
using TuneKey = std::tuple<int, int, int, int, int, int, int, int, int, int>;
std::mutex g_tune_mu;
std::map<TuneKey, std::tuple<int, int, int, int>> g_tune;

int autotune(gt_problem *p) {
  const bool tgv = p->reg == GT_TGV;
  // every dual shape is tuned: at 256^2 x 60 x 4 the order of the shapes timed
  // alone is their order inside the overlapped iteration
  // back-projection shapes 14 and 15 (TMA-staged sinogram rows) are bit-identical
  // but slower on every measured workload (256^2 x 60 x 4: 0.43 / 0.45 against
  // 0.36 ms); they stay selectable by gt_set_tuning and are not tuned
  constexpr int kMaxCfg = 32;
  const int nc[3] = {std::min(kMaxCfg, gt::num_proj_configs(p->d.S, 0)),
                     std::min(kMaxCfg, gt::num_proj_configs(p->d.S, 1)),
                     std::min(kMaxCfg, gt::num_dual_configs(p->P))};
  // Shapes left out of the tuning (all stay selectable by gt_set_tuning), to bound
  // its time on batches of many distinct problems: the TMA back projector (above);
  // the multi-bin / multi-pixel run shapes (forward 5-8, back 9-12) once S >= 32,
  // 2-4x slower than the best shape on every measured workload there; the
  // chunk-outermost shapes (forward 9, back 13), which only pay when the image
  // exceeds L2, below 64 MB of image; one slice per thread (forward 4, back 8)
  // once S >= 128.
  const int S = p->d.S;
  const long long img_bytes = (long long)p->d.N * p->d.N * S * 4;
  auto skipped = [&](int which, int c) {
    if (which == 1 && (c == 14 || c == 15)) return true;
    if (S >= 32 && ((which == 0 && c >= 5 && c <= 8) || (which == 1 && c >= 9 && c <= 12))) return true;
    if (img_bytes < (64ll << 20) && ((which == 0 && c == 9) || (which == 1 && c == 13))) return true;
    if (S >= 128 && ((which == 0 && c == 4) || (which == 1 && c == 8))) return true;
    return false;
  };
  p->P.fwd_cfg = 0;
  p->P.bp_cfg = 0;
  p->P.dual_cfg = 0;
  if ((nc[0] <= 1 && nc[1] <= 1 && nc[2] <= 1) || !p->autotune) return GT_OK;
  const TuneKey key{p->d.dim, p->d.N, p->d.S, p->d.nd, p->d.nang, p->disc, p->d.C, p->d.Nz, p->reg, p->cpl};
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(key);
    if (it != g_tune.end()) {
      int sched = 0;
      std::tie(p->P.fwd_cfg, p->P.bp_cfg, p->P.dual_cfg, sched) = it->second;
      // sched < 0: the schedule was chosen by gt_set_schedule when the shapes were
      // tuned, not timed; 0 is the measured choice at 8M voxel-channels and above
      if (!p->schedule_set) p->schedule = sched >= 0 ? sched : (p->d.vol >= (8u << 20) ? 0 : 1);
      if (p->schedule == 2 && ensure_fused(p) != GT_OK) p->schedule = 0;  // no room for the second set
      return GT_OK;
    }
  }
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  // configurations interleaved over several rounds; each keeps its fastest round
  float ms_cfg[3][kMaxCfg];
  for (auto &r : ms_cfg) for (float &v : r) v = 1e30f;
  int rc = GT_OK;
  const bool log = std::getenv("GRAPTOR_TUNE_LOG") != nullptr;
  for (int round = 0; round < 4 && rc == GT_OK; ++round) {
    for (int which = 0; which < 3 && rc == GT_OK; ++which) {
      if (nc[which] <= 1) continue;
      float best_ms = 1e30f;
      for (int c = 0; c < nc[which]; ++c) best_ms = std::min(best_ms, ms_cfg[which][c]);
      for (int c = 0; c < nc[which] && rc == GT_OK; ++c) {
        if (skipped(which, c)) continue;
        // after the first round only configurations within 15 % of the best are timed again
        if (round > 0 && ms_cfg[which][c] > 1.15f * best_ms) continue;
        gt::IterParams Q = p->P;
        if (which == 0) Q.fwd_cfg = c; else if (which == 1) Q.bp_cfg = c; else Q.dual_cfg = c;
        auto launch = [&]() {
          if (which == 0) return gt::launch_fwd(Q, p->disc, p->stream);
          if (which == 1) return gt::launch_bp(Q, p->stream);
          return gt::launch_dual(Q, tgv, p->cpl, p->stream);
        };
        // the first round screens every shape with one timed launch, later rounds
        // time the contenders twice
        const int reps = round == 0 ? 1 : 2;
        cudaError_t e = launch();  // warm-up
        if (e == cudaSuccess) e = cudaEventRecord(e0, p->stream);
        for (int r = 0; r < reps && e == cudaSuccess; ++r) e = launch();
        if (e == cudaSuccess) e = cudaEventRecord(e1, p->stream);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        float ms = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        if (e != cudaSuccess) { rc = cuda_err(e, "autotune", __LINE__); break; }
        ms_cfg[which][c] = std::min(ms_cfg[which][c], ms / reps);
      }
    }
  }
  int best[3] = {0, 0, 0};
  static const char *names[3] = {"k_fwd", "k_bp", "k_dual"};
  for (int which = 0; which < 3; ++which)
    for (int c = 1; c < nc[which]; ++c)
      if (ms_cfg[which][c] < ms_cfg[which][best[which]]) best[which] = c;
  if (log && rc == GT_OK)
    for (int which = 0; which < 3; ++which)
      for (int c = 0; c < nc[which] && nc[which] > 1; ++c)
        fprintf(stderr, "graptor autotune %s cfg %d: %.4f ms%s\n", names[which], c, ms_cfg[which][c],
                c == best[which] ? " *" : "");
  if (rc) {
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
  }
  p->P.fwd_cfg = best[0];
  p->P.bp_cfg = best[1];
  p->P.dual_cfg = best[2];
  // the schedule (TGV only: TV has no p / pbar half): graph-captured iterations of
  // each, the faster kept; concurrency between the kernels decides, not their times
  // alone.  Problems below 8M voxel-channels keep schedule 1 (the two schedules are
  // within a few per cent there, e.g. 0.135 / 0.132 ms at 128^2 x 32 x 2).
  // Schedule 2 (the p half fused into the next dual kernel) is not timed: its
  // fused kernel is slower than the dual kernel and the p half together on every
  // measured workload (256^2 x 60 x 4: 1.07 ms against 0.25 + 0.16 ms), so it
  // stays a choice of gt_set_schedule.  The graphs are timed over 16 iterations.
  if (tgv && !p->schedule_set && p->d.vol < (8u << 20)) p->schedule = 1;
  if (tgv && !p->schedule_set && p->d.vol >= (8u << 20)) {
    const int nsched = 2;
    float ms_s[3] = {1e30f, 1e30f, 1e30f};
    for (int round = 0; round < 2 && rc == GT_OK; ++round) {
      for (int sched = 0; sched < nsched && rc == GT_OK; ++sched) {
        p->schedule = sched;
        cudaGraphExec_t g = nullptr;
        rc = capture(p, 16, &g);
        if (rc) break;
        cudaError_t e = cudaGraphLaunch(g, p->stream);
        if (e == cudaSuccess) e = cudaEventRecord(e0, p->stream);
        for (int r = 0; r < 2 && e == cudaSuccess; ++r) e = cudaGraphLaunch(g, p->stream);
        if (e == cudaSuccess) e = cudaEventRecord(e1, p->stream);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        float ms = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        cudaGraphExecDestroy(g);
        if (e != cudaSuccess) { rc = cuda_err(e, "autotune (schedule)", __LINE__); break; }
        ms_s[sched] = std::min(ms_s[sched], ms / 32);
      }
    }
    int bs = 0;
    for (int sched = 1; sched < nsched; ++sched)
      if (ms_s[sched] < ms_s[bs]) bs = sched;
    p->schedule = bs;
    if (bs != 2) free_fused(p);
    if (log && rc == GT_OK)
      fprintf(stderr, "graptor autotune schedule 0: %.4f ms, 1: %.4f ms, 2: %.4f ms per iteration\n", ms_s[0],
              ms_s[1], ms_s[2]);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune[key] = std::make_tuple(best[0], best[1], best[2], p->schedule_set ? -1 : p->schedule);
  return GT_OK;
}

}  // namespace

// error reporting for the library's other translation units
namespace gt {
int set_error(int code, const char *msg) { return set_err(code, "%s", msg); }
int cuda_error(cudaError_t e, const char *what, int line) { return cuda_err(e, what, line); }
}  // namespace gt

extern "C" {

const char *gt_last_error(void) { return g_err.c_str(); }
const char *gt_version(void) { return "graptor_gb300 0.1 (sm_103a)"; }

int gt_launches_per_iteration(const gt_problem *p) {
  if (!p) return 0;
  return 3 + (p->d.C > 8 ? (p->d.C + 7) / 8 : 1) + (p->schedule == 1 && p->reg == GT_TGV ? 1 : 0);
}

int gt_set_schedule(gt_problem *p, int schedule) {
  if (!p) return set_err(GT_ERR_ARG, "null argument");
  if (schedule < 0 || schedule > 2) return set_err(GT_ERR_ARG, "schedule must be 0, 1 or 2 (got %d)", schedule);
  if (schedule == 2 && !fused_available(p))
    return set_err(GT_ERR_ARG, "schedule 2 needs 3-D TGV, Frobenius or uncorrelated coupling, C <= 4 and Nz even");
  CK(cudaSetDevice(p->device));
  CK(cudaStreamSynchronize(p->stream));
  if (schedule == 2) {
    const int rc = ensure_fused(p);
    if (rc) return rc;
  } else {
    free_fused(p);
  }
  p->schedule = schedule;
  p->schedule_set = true;
  if (p->g_one) { cudaGraphExecDestroy(p->g_one); p->g_one = nullptr; }
  if (p->g_chunk) { cudaGraphExecDestroy(p->g_chunk); p->g_chunk = nullptr; }
  return GT_OK;
}

int gt_problem_create(const gt_desc *desc, gt_problem **out) {
  if (!desc || !out) return set_err(GT_ERR_ARG, "null argument");
  *out = nullptr;
  const gt_desc &D = *desc;
  if (D.dim != 2 && D.dim != 3) return set_err(GT_ERR_ARG, "dim must be 2 or 3 (got %d)", D.dim);
  if (D.N < 1 || D.Nz < 1 || D.C < 1 || D.nd < 1 || D.nang < 1)
    return set_err(GT_ERR_ARG, "sizes must be positive (N=%d Nz=%d C=%d nd=%d nang=%d)", D.N, D.Nz, D.C, D.nd, D.nang);
  if (D.coupling != GT_UNCORR && D.C > 8)
    return set_err(GT_ERR_ARG, "coupled regularisation supports at most 8 channels (got %d)", D.C);
  if (D.discrepancy != GT_KL && D.discrepancy != GT_L2) return set_err(GT_ERR_ARG, "bad discrepancy");
  if (D.regularisation != GT_TV && D.regularisation != GT_TGV) return set_err(GT_ERR_ARG, "bad regularisation");
  if (D.coupling < GT_UNCORR || D.coupling > GT_NUCL) return set_err(GT_ERR_ARG, "bad coupling");
  if (!D.angles || !D.mu) return set_err(GT_ERR_ARG, "angles and mu are required");
  if (!(D.stepsize > 0.f)) return set_err(GT_ERR_ARG, "stepsize must be positive");
  if (D.regularisation == GT_TGV && !(D.alpha0 > 0 && D.alpha1 > 0)) return set_err(GT_ERR_ARG, "alpha must be positive");
  if (D.regularisation == GT_TV && !(D.alpha1 > 0)) return set_err(GT_ERR_ARG, "alpha1 must be positive");
  const long long S = (long long)D.Nz * D.C;
  const long long vol = (long long)D.N * D.N * S, nbin = (long long)D.nd * D.nang * S;
  if ((long long)D.N * D.N > (1LL << 30) || S > (1LL << 20) || (long long)D.nd * D.nang > (1LL << 30))
    return set_err(GT_ERR_ARG, "problem too large for 32-bit pixel / bin indices");

  gt_problem *p = new (std::nothrow) gt_problem();
  if (!p) return set_err(GT_ERR_OOM, "host allocation failed");
  p->device = D.device;
  p->d.dim = D.dim; p->d.N = D.N; p->d.Nz = D.Nz; p->d.C = D.C; p->d.S = (int)S;
  p->d.nd = D.nd; p->d.nang = D.nang; p->d.vol = (size_t)vol; p->d.nbin = (size_t)nbin;
  p->disc = D.discrepancy; p->reg = D.regularisation; p->cpl = D.coupling;
  p->K = D.dim; p->KW = D.dim == 3 ? 6 : 3;
  p->stepsize = D.stepsize;
  p->alpha0 = D.alpha0; p->alpha1 = D.alpha1; p->ne_in = D.normest;
  p->autotune = D.autotune != 0;
  p->mu.assign(D.mu, D.mu + D.C);
  angle_table(D.angles, D.N, D.nd, D.nang, p->ofs64h);

  auto fail = [&](int rc) { gt_problem_destroy(p); return rc; };
  if (cudaSetDevice(D.device) != cudaSuccess) return fail(cuda_err(cudaGetLastError(), "cudaSetDevice", __LINE__));
  if (D.stream) {
    p->stream = (cudaStream_t)D.stream;
  } else {
    cudaError_t e = cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return fail(cuda_err(e, "cudaStreamCreate", __LINE__));
    p->own_stream = true;
  }
  {
    // The projector chain is the iteration's critical path (k_fwd -> k_bp ->
    // k_update) while k_dual beside it has slack, so the side stream gets the
    // highest priority: its blocks are scheduled first when both compete for SMs.
    // GRAPTOR_SIDE_PRIORITY=0 keeps the default priority.
    int lo = 0, hi = 0;
    cudaDeviceGetStreamPriorityRange(&lo, &hi);
    const char *env = std::getenv("GRAPTOR_SIDE_PRIORITY");
    const int prio = (env && env[0] == '0') ? lo : hi;
    cudaError_t e1 = cudaStreamCreateWithPriority(&p->side, cudaStreamNonBlocking, prio);
    if (e1 == cudaSuccess) e1 = cudaEventCreateWithFlags(&p->ev_fork, cudaEventDisableTiming);
    if (e1 == cudaSuccess) e1 = cudaEventCreateWithFlags(&p->ev_join, cudaEventDisableTiming);
    if (e1 != cudaSuccess) return fail(cuda_err(e1, "stream/event setup", __LINE__));
  }
  const bool tgv = D.regularisation == GT_TGV;
  const size_t fv = sizeof(float) * (size_t)vol, fb = sizeof(float) * (size_t)nbin;
  size_t off[16], total = 0;
  size_t sizes[] = {
      align256(sizeof(float4) * D.nang), align256(sizeof(dvec4) * D.nang), align256(sizeof(float) * D.C),
      align256(fv), align256(fv),                                   // u, ubar
      tgv ? align256(fv * p->K) : 0, tgv ? align256(fv * p->K) : 0, // p, pbar
      align256(fv * p->K),                                          // v
      tgv ? align256(fv * p->KW) : 0,                               // w
      align256(fb), align256(fb), align256(fb),                     // lam, f, ku
      align256(std::max(fv, fb)),                                   // stage
      align256(fv),                                                 // kstar
      align256(sizeof(double) * D.C),                               // mu (double)
      align256(sizeof(int) * 4)};                                   // error flags
  const int nsz = (int)(sizeof(sizes) / sizeof(sizes[0]));
  for (int k = 0; k < nsz; ++k) { off[k] = total; total += sizes[k]; }
  cudaError_t e = cudaMalloc(&p->block, total);
  if (e != cudaSuccess) {
    cudaGetLastError();
    gt_problem_destroy(p);
    return set_err(GT_ERR_OOM, "device allocation of %.3f GB failed: %s", total / 1e9, cudaGetErrorString(e));
  }
  char *b = (char *)p->block;
  p->ofs = (float4 *)(b + off[0]);
  p->ofs64 = (dvec4 *)(b + off[1]);
  p->mu_eff = (float *)(b + off[2]);
  p->u = (float *)(b + off[3]);
  p->ubar = (float *)(b + off[4]);
  p->p = tgv ? (float *)(b + off[5]) : nullptr;
  p->pbar = tgv ? (float *)(b + off[6]) : nullptr;
  p->v = (float *)(b + off[7]);
  p->w = tgv ? (float *)(b + off[8]) : nullptr;
  p->lam = (float *)(b + off[9]);
  p->f = (float *)(b + off[10]);
  p->ku = (float *)(b + off[11]);
  p->stage = (float *)(b + off[12]);
  p->kstar = (float *)(b + off[13]);
  p->mu64 = (double *)(b + off[14]);
  p->flags = (int *)(b + off[15]);

  std::vector<float> t32((size_t)D.nang * 4);
  for (size_t k = 0; k < t32.size(); ++k) t32[k] = (float)p->ofs64h[k];
  // zero the whole block first, then upload the angle tables into it
  if ((e = cudaMemsetAsync(p->block, 0, total, p->stream)) != cudaSuccess ||
      (e = cudaMemcpyAsync(p->ofs, t32.data(), sizeof(float) * t32.size(), cudaMemcpyHostToDevice, p->stream)) !=
          cudaSuccess ||
      (e = cudaMemcpyAsync(p->ofs64, p->ofs64h.data(), sizeof(double) * p->ofs64h.size(), cudaMemcpyHostToDevice,
                           p->stream)) != cudaSuccess ||
      (e = cudaStreamSynchronize(p->stream)) != cudaSuccess)
    return fail(cuda_err(e, "problem setup", __LINE__));

  // ray table of the forward projector (entries of all rays, see k_ray_fill)
  {
    const int nr = D.nd * D.nang;
    std::vector<int> cnt(nr);
    std::vector<long long> start(nr + 1, 0);
    int *d_cnt = (int *)p->stage;  // stage is free scratch now (>= nr floats)
    if ((e = gt::launch_ray_count(p->ofs, D.N, D.nd, D.nang, d_cnt, p->stream)) != cudaSuccess ||
        (e = cudaMemcpyAsync(cnt.data(), d_cnt, sizeof(int) * nr, cudaMemcpyDeviceToHost, p->stream)) != cudaSuccess ||
        (e = cudaStreamSynchronize(p->stream)) != cudaSuccess)
      return fail(cuda_err(e, "ray table count", __LINE__));
    for (int r = 0; r < nr; ++r) start[r + 1] = start[r] + cnt[r];
    const size_t off_b = align256(sizeof(long long) * (nr + 1));
    const size_t off_bp = off_b + align256(sizeof(int2) * (size_t)start[nr]);
    p->ray_bytes = off_bp + sizeof(int2) * (size_t)D.N * D.N * D.nang;
    if ((e = cudaMalloc(&p->rays, p->ray_bytes)) != cudaSuccess) {
      cudaGetLastError();
      gt_problem_destroy(p);
      return set_err(GT_ERR_OOM, "ray table allocation of %.3f GB failed", p->ray_bytes / 1e9);
    }
    long long *d_start = (long long *)p->rays;
    int2 *d_ent = (int2 *)((char *)p->rays + off_b);
    if ((e = cudaMemcpyAsync(d_start, start.data(), sizeof(long long) * (nr + 1), cudaMemcpyHostToDevice,
                             p->stream)) != cudaSuccess ||
        (e = gt::launch_ray_fill(p->ofs, D.N, D.nd, D.nang, d_start, d_ent, p->stream)) != cudaSuccess ||
        (e = gt::launch_bp_table(p->ofs, D.N, D.nd, D.nang, (int2 *)((char *)p->rays + off_bp), p->stream)) !=
            cudaSuccess ||
        (e = cudaStreamSynchronize(p->stream)) != cudaSuccess)
      return fail(cuda_err(e, "ray table fill", __LINE__));
    p->P.ray_start = d_start;
    p->P.ray_ent = d_ent;
    p->P.bp_tab = (const int2 *)((char *)p->rays + off_bp);
  }

  // 3-bin run table of the forward projector (k_fwd_rt); optional: without it
  // (no memory) the run shapes fall back to the ray table
  {
    const int nr = ((D.nd + 2) / 3) * D.nang;
    std::vector<int> cnt(nr);
    std::vector<long long> start(nr + 1, 0);
    int *d_cnt = (int *)p->stage;
    if ((e = gt::launch_run_count(p->ofs, D.N, D.nd, D.nang, d_cnt, p->stream)) != cudaSuccess ||
        (e = cudaMemcpyAsync(cnt.data(), d_cnt, sizeof(int) * nr, cudaMemcpyDeviceToHost, p->stream)) != cudaSuccess ||
        (e = cudaStreamSynchronize(p->stream)) != cudaSuccess)
      return fail(cuda_err(e, "run table count", __LINE__));
    for (int r = 0; r < nr; ++r) start[r + 1] = start[r] + cnt[r];
    const size_t off_e = align256(sizeof(long long) * (nr + 1));
    const size_t bytes = off_e + sizeof(int4) * (size_t)start[nr];
    if (cudaMalloc(&p->runs, bytes) != cudaSuccess) {
      cudaGetLastError();
      p->runs = nullptr;
    } else {
      long long *d_start = (long long *)p->runs;
      int4 *d_ent = (int4 *)((char *)p->runs + off_e);
      if ((e = cudaMemcpyAsync(d_start, start.data(), sizeof(long long) * (nr + 1), cudaMemcpyHostToDevice,
                               p->stream)) != cudaSuccess ||
          (e = gt::launch_run_fill(p->ofs, D.N, D.nd, D.nang, d_start, d_ent, p->stream)) != cudaSuccess ||
          (e = cudaStreamSynchronize(p->stream)) != cudaSuccess)
        return fail(cuda_err(e, "run table fill", __LINE__));
      p->P.run_start = d_start;
      p->P.run_ent = d_ent;
    }
  }

  // row-tile table of the register-blocked back projector (k_bp_row); optional:
  // without it (no memory, nd < 2, a geometry the table cannot describe) those
  // launch shapes fall back to the others
  if (D.nd >= 2) {
    const size_t tbytes = gt::row_table_bytes(D.N, D.nang);
    if (cudaMalloc(&p->tiles, align256(tbytes) + 256) == cudaSuccess) {
      int *d_bad = (int *)((char *)p->tiles + align256(tbytes));
      int bad = 0;
      if ((e = cudaMemsetAsync(d_bad, 0, sizeof(int), p->stream)) != cudaSuccess ||
          (e = gt::launch_row_fill(p->ofs, D.N, D.nd, D.nang, (int4 *)p->tiles, d_bad, p->stream)) != cudaSuccess ||
          (e = cudaMemcpyAsync(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, p->stream)) != cudaSuccess ||
          (e = cudaStreamSynchronize(p->stream)) != cudaSuccess)
        return fail(cuda_err(e, "row table fill", __LINE__));
      if (!bad) {
        p->P.row_ent = (const int4 *)p->tiles;
      } else {  // some lower bins do not step by 0 / 1 along a row: not used
        cudaFree(p->tiles);
        p->tiles = nullptr;
      }
    } else {
      cudaGetLastError();
      p->tiles = nullptr;
    }
  }

  gt::IterParams &P = p->P;
  P.d = p->d;
  P.ofs = p->ofs; P.mu = p->mu_eff;
  P.u = p->u; P.ubar = p->ubar; P.p = p->p; P.pbar = p->pbar; P.v = p->v; P.w = p->w;
  P.lam = p->lam; P.f = p->f; P.ku = p->ku; P.kstar = p->kstar; P.mu64 = p->mu64;
  P.err = p->flags;
  P.bp_skip_angle = -1;
  P.bp_wait_limit = 1u << 22;
  P.bp_tmap = encode_lambda_map(&p->bp_tmap, p->lam, p->d.S, p->d.nd, p->d.nang, 128) ? &p->bp_tmap : nullptr;
  P.bp_tmap_wide =
      encode_lambda_map(&p->bp_tmap_wide, p->lam, p->d.S, p->d.nd, p->d.nang, 256) ? &p->bp_tmap_wide : nullptr;
  if (P.bp_tmap_wide && gt::prepare_bp_tma() != cudaSuccess) {
    cudaGetLastError();
    P.bp_tmap_wide = nullptr;
  }
  *out = p;
  return GT_OK;
}

void gt_problem_destroy(gt_problem *p) {
  if (!p) return;
  cudaSetDevice(p->device);
  if (p->stream) cudaStreamSynchronize(p->stream);
  if (p->g_one) cudaGraphExecDestroy(p->g_one);
  if (p->g_chunk) cudaGraphExecDestroy(p->g_chunk);
  if (p->block) cudaFree(p->block);
  if (p->rays) cudaFree(p->rays);
  if (p->runs) cudaFree(p->runs);
  if (p->tiles) cudaFree(p->tiles);
  if (p->gap_ws) cudaFree(p->gap_ws);
  if (p->snap) cudaFree(p->snap);
  if (p->fused) cudaFree(p->fused);
  if (p->ulo) cudaFree(p->ulo);
  if (p->ev_fork) cudaEventDestroy(p->ev_fork);
  if (p->ev_join) cudaEventDestroy(p->ev_join);
  if (p->side) cudaStreamDestroy(p->side);
  if (p->own_stream && p->stream) cudaStreamDestroy(p->stream);
  delete p;
}

int gt_set_data(gt_problem *p, const float *f_host, int make_feasible) {
  if (!p || !f_host) return set_err(GT_ERR_ARG, "null argument");
  CK(cudaSetDevice(p->device));
  const gt::Dims &d = p->d;
  const int nb1 = d.nd * d.nang;
  CK(cudaMemcpyAsync(p->stage, f_host, sizeof(float) * d.nbin, cudaMemcpyHostToDevice, p->stream));
  CK(gt::launch_transpose(p->stage, p->f, d.S, nb1, p->stream));
  if (make_feasible) {
    // Make_function_feasible (3-D :860-870): bins the all-ones slice does not reach
    // (R 1 <= 0) are zeroed in every slice.  ku is free scratch here.
    float *ones = p->stage, *r1 = p->ku;
    CK(gt::fill_f32(ones, (size_t)d.N * d.N, 1.f, p->stream));
    CK(gt::launch_radon(ones, r1, p->ofs, d.N, d.nd, d.nang, 1, p->stream));
    CK(gt::launch_feasible(p->f, r1, nb1, d.S, p->stream));
  }
  // operator norm (radon_normest, 3-D :1018-1030): injected, or FP64 power iteration
  if (p->ne_in > 0) {
    p->ne = p->ne_in;
  } else {
    const size_t n = (size_t)d.N * d.N;
    double *scratch = nullptr;
    const size_t bytes = sizeof(double) * (n + (size_t)nb1 + 256);
    cudaError_t e = cudaMalloc(&scratch, bytes);
    if (e != cudaSuccess) return cuda_err(e, "cudaMalloc (normest scratch)", __LINE__);
    double ne = 0;
    e = gt::fill_f64(scratch, n, 1.0, p->stream);
    if (e == cudaSuccess)
      e = gt::normest64(p->ofs64, d.N, d.nd, d.nang, 30, scratch, scratch + n, scratch + n + nb1, &ne, p->stream);
    cudaFree(scratch);
    if (e != cudaSuccess) return cuda_err(e, "normest64", __LINE__);
    if (!(ne > 0) || !std::isfinite(ne)) return set_err(GT_ERR_CUDA, "operator norm estimate failed (%g)", ne);
    p->ne = ne;
  }
  set_scalars(p);
  {
    const int rc = upload_mu_eff(p);
    if (rc) return rc;
  }
  CK(cudaMemcpyAsync(p->mu64, p->mu.data(), sizeof(double) * d.C, cudaMemcpyHostToDevice, p->stream));
  p->P.ne64 = p->ne;
  // pick the projector launch shapes (uses lambda / ku / kstar as scratch: they are reset below)
  {
    const int rc = autotune(p);
    if (rc) return rc;
  }
  // zero iterates (tgv_radon :1160-1176)
  const size_t fv = sizeof(float) * d.vol;
  CK(cudaMemsetAsync(p->u, 0, fv, p->stream));
  CK(cudaMemsetAsync(p->ubar, 0, fv, p->stream));
  if (p->ulo) CK(cudaMemsetAsync(p->ulo, 0, fv, p->stream));
  if (p->p) CK(cudaMemsetAsync(p->p, 0, fv * p->K, p->stream));
  if (p->pbar) CK(cudaMemsetAsync(p->pbar, 0, fv * p->K, p->stream));
  CK(cudaMemsetAsync(p->v, 0, fv * p->K, p->stream));
  if (p->w) CK(cudaMemsetAsync(p->w, 0, fv * p->KW, p->stream));
  CK(cudaMemsetAsync(p->lam, 0, sizeof(float) * d.nbin, p->stream));
  CK(cudaMemsetAsync(p->ku, 0, sizeof(float) * d.nbin, p->stream));
  CK(cudaStreamSynchronize(p->stream));
  // the step scalars are baked into the captured graphs: recapture
  if (p->g_one) { cudaGraphExecDestroy(p->g_one); p->g_one = nullptr; }
  if (p->g_chunk) { cudaGraphExecDestroy(p->g_chunk); p->g_chunk = nullptr; }
  p->iters = 0;
  p->has_data = true;
  return GT_OK;
}

int gt_run(gt_problem *p, int iters) {
  if (!p) return set_err(GT_ERR_ARG, "null problem");
  if (!p->has_data) return set_err(GT_ERR_STATE, "gt_run before gt_set_data");
  if (iters < 0) return set_err(GT_ERR_ARG, "negative iteration count");
  if (iters == 0) return GT_OK;
  CK(cudaSetDevice(p->device));
  int rc;
  const int chunk = chunk_len(p);
  if (iters >= chunk && !p->g_chunk && (rc = capture(p, chunk, &p->g_chunk)) != GT_OK) return rc;
  if (!p->g_one && (rc = capture(p, 1, &p->g_one)) != GT_OK) return rc;
  int left = iters;
  while (left >= chunk) { CK(cudaGraphLaunch(p->g_chunk, p->stream)); left -= chunk; }
  if (p->schedule == 2 && p->fused && left >= 3) {  // the rest pipelined too, launched directly
    const int m = left % 2 ? left : left - 1;
    if ((rc = enqueue_pipelined(p, m)) != GT_OK) return rc;
    left -= m;
  }
  while (left > 0) { CK(cudaGraphLaunch(p->g_one, p->stream)); --left; }
  p->iters += iters;
  return GT_OK;
}

int gt_synchronize(gt_problem *p) {
  if (!p) return set_err(GT_ERR_ARG, "null problem");
  CK(cudaSetDevice(p->device));
  CK(cudaStreamSynchronize(p->stream));
  int flag = 0;
  CK(cudaMemcpy(&flag, p->flags, sizeof(int), cudaMemcpyDeviceToHost));
  if (flag) {
    CK(cudaMemset(p->flags, 0, sizeof(int)));
    return set_err(GT_ERR_TIMEOUT, "a back-projection block gave up waiting for its TMA copies; the iterate is invalid");
  }
  return GT_OK;
}

int gt_get_state(gt_problem *p, int field, float *host) {
  if (!p || !host) return set_err(GT_ERR_ARG, "null argument");
  float *ptr; int comps; size_t X;
  int rc = field_info(p, field, &ptr, &comps, &X);
  if (rc) return rc;
  CK(cudaSetDevice(p->device));
  const size_t S = p->d.S;
  for (int k = 0; k < comps; ++k) {
    const size_t plane = (field == GT_LAMBDA || field == GT_KU || field == GT_DATA) ? p->d.nbin : p->d.vol;
    CK(gt::launch_transpose(ptr + k * plane, p->stage, (int)X, (int)S, p->stream));
    CK(cudaMemcpyAsync(host + k * X * S, p->stage, sizeof(float) * X * S, cudaMemcpyDeviceToHost, p->stream));
  }
  CK(cudaStreamSynchronize(p->stream));
  return GT_OK;
}

int gt_get_output_f64(gt_problem *p, int field, double *host) {
  if (!p || !host) return set_err(GT_ERR_ARG, "null argument");
  if (p->d.dim != 3 || (field != GT_U && field != GT_KU))
    return set_err(GT_ERR_ARG, "gt_get_output_f64: the image (GT_U) or K u (GT_KU) of a 3-D problem");
  CK(cudaSetDevice(p->device));
  const bool img = field == GT_U;
  const int A = img ? p->d.N : p->d.nang, B = img ? p->d.N : p->d.nd;
  const size_t n = (size_t)A * B * p->d.S;
  double *tmp = nullptr;
  CK(cudaMallocAsync(&tmp, sizeof(double) * n, p->stream));
  cudaError_t e = gt::launch_output_f64(img ? p->u : p->ku, tmp, A, B, p->d.C, p->d.Nz, img ? 0 : 1, p->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(host, tmp, sizeof(double) * n, cudaMemcpyDeviceToHost, p->stream);
  const cudaError_t ef = cudaFreeAsync(tmp, p->stream);
  if (e == cudaSuccess) e = ef;
  if (e == cudaSuccess) e = cudaStreamSynchronize(p->stream);
  if (e != cudaSuccess) return cuda_err(e, "gt_get_output_f64", __LINE__);
  return GT_OK;
}

int gt_set_state(gt_problem *p, int field, const float *host) {
  if (!p || !host) return set_err(GT_ERR_ARG, "null argument");
  float *ptr; int comps; size_t X;
  int rc = field_info(p, field, &ptr, &comps, &X);
  if (rc) return rc;
  CK(cudaSetDevice(p->device));
  const size_t S = p->d.S;
  for (int k = 0; k < comps; ++k) {
    const size_t plane = (field == GT_LAMBDA || field == GT_KU || field == GT_DATA) ? p->d.nbin : p->d.vol;
    CK(cudaMemcpyAsync(p->stage, host + k * X * S, sizeof(float) * X * S, cudaMemcpyHostToDevice, p->stream));
    CK(gt::launch_transpose(p->stage, ptr + k * plane, (int)S, (int)X, p->stream));
  }
  if (field == GT_U && p->ulo) CK(cudaMemsetAsync(p->ulo, 0, sizeof(float) * p->d.vol, p->stream));
  CK(cudaStreamSynchronize(p->stream));
  return GT_OK;
}

int gt_get_state_device(gt_problem *p, int field, float *dev) {
  if (!p || !dev) return set_err(GT_ERR_ARG, "null argument");
  float *ptr; int comps; size_t X;
  int rc = field_info(p, field, &ptr, &comps, &X);
  if (rc) return rc;
  CK(cudaSetDevice(p->device));
  const size_t S = p->d.S;
  for (int k = 0; k < comps; ++k) {
    const size_t plane = (field == GT_LAMBDA || field == GT_KU || field == GT_DATA) ? p->d.nbin : p->d.vol;
    CK(gt::launch_transpose(ptr + k * plane, dev + k * X * S, (int)X, (int)S, p->stream));
  }
  return GT_OK;
}

int gt_set_state_device(gt_problem *p, int field, const float *dev) {
  if (!p || !dev) return set_err(GT_ERR_ARG, "null argument");
  float *ptr; int comps; size_t X;
  int rc = field_info(p, field, &ptr, &comps, &X);
  if (rc) return rc;
  CK(cudaSetDevice(p->device));
  const size_t S = p->d.S;
  for (int k = 0; k < comps; ++k) {
    const size_t plane = (field == GT_LAMBDA || field == GT_KU || field == GT_DATA) ? p->d.nbin : p->d.vol;
    CK(gt::launch_transpose(dev + k * X * S, ptr + k * plane, (int)S, (int)X, p->stream));
  }
  if (field == GT_U && p->ulo) CK(cudaMemsetAsync(p->ulo, 0, sizeof(float) * p->d.vol, p->stream));
  return GT_OK;
}

int gt_dual_from_primal_ex(gt_problem *p, int flags, float empty_weight) {
  if (!p) return set_err(GT_ERR_ARG, "null argument");
  if (!p->has_data) return set_err(GT_ERR_STATE, "gt_dual_from_primal before gt_set_data");
  if (flags & ~(GT_DUAL_CAP10 | GT_DUAL_CAP100 | GT_DUAL_REPAIR | GT_DUAL_NO_RESET))
    return set_err(GT_ERR_ARG, "unknown flags %d", flags);
  if (!(empty_weight >= 0.f && empty_weight <= 1.f)) return set_err(GT_ERR_ARG, "empty_weight must lie in [0, 1]");
  const float cap = (flags & GT_DUAL_CAP100) ? 100.f : ((flags & GT_DUAL_CAP10) ? 10.f : 0.f);
  CK(cudaSetDevice(p->device));
  // K u into the ku buffer (the next iteration's forward projection overwrites it)
  CK(gt::launch_radon(p->u, p->ku, p->ofs, p->d.N, p->d.nd, p->d.nang, p->d.S, p->stream));
  if ((flags & GT_DUAL_REPAIR) && p->disc == GT_KL) {
    // lift u along rays with data that the image misses: u, ubar += R^T r (stage holds
    // the image-sized correction), then project again
    CK(gt::launch_missed_rays(p->ku, p->f, p->ku, (long long)p->d.nbin, p->d.N, p->stream));
    CK(gt::launch_radon_ad(p->ku, p->stage, p->ofs, p->d.N, p->d.nd, p->d.nang, p->d.S, p->stream));
    CK(gt::launch_add2(p->u, p->ubar, p->stage, (long long)p->d.vol, p->stream));
    CK(gt::launch_radon(p->u, p->ku, p->ofs, p->d.N, p->d.nd, p->d.nang, p->d.S, p->stream));
  }
  if (flags & GT_DUAL_NO_RESET) return GT_OK;  // only the lift
  CK(gt::launch_lambda_fixed(p->lam, p->ku, p->f, p->mu64, (long long)p->d.nd * p->d.nang, p->d.S, p->d.Nz, p->disc,
                             empty_weight, cap, p->stream));
  return GT_OK;
}

int gt_dual_from_primal(gt_problem *p) { return gt_dual_from_primal_ex(p, 0, 1.f); }

void *gt_problem_stream(gt_problem *p) { return p ? (void *)p->stream : nullptr; }

int gt_set_tuning(gt_problem *p, int fwd_cfg, int bp_cfg) {
  if (!p) return set_err(GT_ERR_ARG, "null argument");
  if (fwd_cfg < 0 || fwd_cfg >= gt::num_proj_configs(p->d.S, 0) || bp_cfg < 0 ||
      bp_cfg >= gt::num_proj_configs(p->d.S, 1))
    return set_err(GT_ERR_ARG, "launch configuration out of range (%d forward, %d back-projection configurations)",
                   gt::num_proj_configs(p->d.S, 0), gt::num_proj_configs(p->d.S, 1));
  CK(cudaSetDevice(p->device));
  CK(cudaStreamSynchronize(p->stream));
  p->P.fwd_cfg = fwd_cfg;
  p->P.bp_cfg = bp_cfg;
  // the captured graphs hold the old launch shapes
  if (p->g_one) { cudaGraphExecDestroy(p->g_one); p->g_one = nullptr; }
  if (p->g_chunk) { cudaGraphExecDestroy(p->g_chunk); p->g_chunk = nullptr; }
  return GT_OK;
}

int gt_set_dual_shape(gt_problem *p, int cfg) {
  if (!p) return set_err(GT_ERR_ARG, "null argument");
  const int n = gt::num_dual_configs(p->P);
  if (cfg < 0 || cfg >= n || (cfg == 1 && !gt::dual_z2_ok(p->P, p->reg == GT_TGV, p->cpl)) ||
      ((cfg == 6 || cfg == 8) && !gt::dual_cl_ok(p->P, p->cpl)) ||
      ((cfg == 7 || cfg == 9) && !gt::dual_cl2_ok(p->P, p->cpl)))
    return set_err(GT_ERR_ARG, "dual launch shape %d not available here", cfg);
  CK(cudaSetDevice(p->device));
  CK(cudaStreamSynchronize(p->stream));
  p->P.dual_cfg = cfg;
  if (p->g_one) { cudaGraphExecDestroy(p->g_one); p->g_one = nullptr; }
  if (p->g_chunk) { cudaGraphExecDestroy(p->g_chunk); p->g_chunk = nullptr; }
  return GT_OK;
}

int gt_get_dual_shape(gt_problem *p) { return p ? p->P.dual_cfg : -1; }

int gt_get_schedule(gt_problem *p) { return p ? p->schedule : -1; }

int gt_set_precise_primal(gt_problem *p, int on) {
  if (!p) return set_err(GT_ERR_ARG, "null argument");
  CK(cudaSetDevice(p->device));
  CK(cudaStreamSynchronize(p->stream));
  if (on && !p->ulo) {
    cudaError_t e = cudaMalloc(&p->ulo, sizeof(float) * p->d.vol);
    if (e != cudaSuccess) {
      cudaGetLastError();
      p->ulo = nullptr;
      return set_err(GT_ERR_OOM, "precise primal mode: allocation of %.3f GB failed", 4e-9 * p->d.vol);
    }
    CK(cudaMemset(p->ulo, 0, sizeof(float) * p->d.vol));  // u = u + 0: the current iterate
  } else if (!on && p->ulo) {
    CK(cudaFree(p->ulo));
    p->ulo = nullptr;
  }
  p->P.ulo = p->ulo;
  // the captured graphs hold the old parameters
  if (p->g_one) { cudaGraphExecDestroy(p->g_one); p->g_one = nullptr; }
  if (p->g_chunk) { cudaGraphExecDestroy(p->g_chunk); p->g_chunk = nullptr; }
  return GT_OK;
}

int gt_get_precise_primal(gt_problem *p) { return p && p->ulo ? 1 : 0; }

int gt_set_primal_weight(gt_problem *p, double w) {
  if (!p || !(w > 0) || !std::isfinite(w)) return set_err(GT_ERR_ARG, "primal weight must be positive and finite");
  if (!p->has_data) return set_err(GT_ERR_STATE, "gt_set_primal_weight before gt_set_data");
  CK(cudaSetDevice(p->device));
  CK(cudaStreamSynchronize(p->stream));
  p->pweight = w;
  set_scalars(p);
  const int rc = upload_mu_eff(p);
  if (rc) return rc;
  // the captured graphs hold the old step sizes
  if (p->g_one) { cudaGraphExecDestroy(p->g_one); p->g_one = nullptr; }
  if (p->g_chunk) { cudaGraphExecDestroy(p->g_chunk); p->g_chunk = nullptr; }
  return GT_OK;
}

double gt_get_primal_weight(gt_problem *p) { return p ? p->pweight : 0.0; }

int gt_restart(gt_problem *p) {
  if (!p) return set_err(GT_ERR_ARG, "null argument");
  if (!p->has_data) return set_err(GT_ERR_STATE, "gt_restart before gt_set_data");
  CK(cudaSetDevice(p->device));
  const size_t fv = sizeof(float) * p->d.vol;
  CK(cudaMemcpyAsync(p->ubar, p->u, fv, cudaMemcpyDeviceToDevice, p->stream));
  if (p->reg == GT_TGV) CK(cudaMemcpyAsync(p->pbar, p->p, fv * p->K, cudaMemcpyDeviceToDevice, p->stream));
  return GT_OK;
}

namespace {
constexpr int kMoveBlocks = 1024;  // FP64 partial sums per field of gt_movement

// (pointer, element count) of the fields of a restart: primal u, p; dual v, w, lambda
void restart_fields(gt_problem *p, float *fld[5], size_t n[5]) {
  const size_t vol = p->d.vol;
  const bool tgv = p->reg == GT_TGV;
  fld[0] = p->u; n[0] = vol;
  fld[1] = p->p; n[1] = tgv ? vol * p->K : 0;
  fld[2] = p->v; n[2] = vol * p->K;
  fld[3] = p->w; n[3] = tgv ? vol * p->KW : 0;
  fld[4] = p->lam; n[4] = p->d.nbin;
}
}  // namespace

int gt_snapshot(gt_problem *p) {
  if (!p) return set_err(GT_ERR_ARG, "null argument");
  if (!p->has_data) return set_err(GT_ERR_STATE, "gt_snapshot before gt_set_data");
  CK(cudaSetDevice(p->device));
  float *fld[5];
  size_t n[5], total = 0;
  restart_fields(p, fld, n);
  for (size_t k : n) total += k;
  if (!p->snap) {  // the fields, then the FP64 block partials of gt_movement
    cudaError_t e = cudaMalloc(&p->snap, align256(sizeof(float) * total) + sizeof(double) * kMoveBlocks * 5);
    if (e != cudaSuccess) { p->snap = nullptr; return cuda_err(e, "cudaMalloc (snapshot)", __LINE__); }
  }
  size_t off = 0;
  for (int k = 0; k < 5; ++k) {
    if (n[k]) CK(cudaMemcpyAsync(p->snap + off, fld[k], sizeof(float) * n[k], cudaMemcpyDeviceToDevice, p->stream));
    off += n[k];
  }
  return GT_OK;
}

int gt_movement(gt_problem *p, double out[2]) {
  if (!p || !out) return set_err(GT_ERR_ARG, "null argument");
  if (!p->snap) return set_err(GT_ERR_STATE, "gt_movement before gt_snapshot");
  CK(cudaSetDevice(p->device));
  constexpr int nb = kMoveBlocks;
  float *fld[5];
  size_t n[5], total = 0;
  restart_fields(p, fld, n);
  for (size_t k : n) total += k;
  double *part = (double *)((char *)p->snap + align256(sizeof(float) * total));
  size_t off = 0;
  int rc = GT_OK;
  for (int k = 0; k < 5 && rc == GT_OK; ++k) {
    cudaError_t e = n[k] ? gt::launch_sqdiff(fld[k], p->snap + off, (long long)n[k], part + nb * k, nb, p->stream)
                         : cudaMemsetAsync(part + nb * k, 0, sizeof(double) * nb, p->stream);
    if (e != cudaSuccess) rc = cuda_err(e, "movement", __LINE__);
    off += n[k];
  }
  std::vector<double> h(nb * 5);
  if (rc == GT_OK) {
    cudaError_t e = cudaMemcpyAsync(h.data(), part, sizeof(double) * nb * 5, cudaMemcpyDeviceToHost, p->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(p->stream);
    if (e != cudaSuccess) rc = cuda_err(e, "movement", __LINE__);
  }
  if (rc) return rc;
  double s[5] = {0, 0, 0, 0, 0};
  for (int k = 0; k < 5; ++k)
    for (int b = 0; b < nb; ++b) s[k] += h[(size_t)nb * k + b];
  out[0] = std::sqrt(s[0] + s[1]);
  out[1] = std::sqrt(s[2] + s[3] + s[4]);
  return GT_OK;
}

int gt_test_bp_stall(gt_problem *p, int angle, unsigned wait_limit) {
  if (!p || wait_limit == 0) return set_err(GT_ERR_ARG, "invalid argument");
  CK(cudaSetDevice(p->device));
  CK(cudaStreamSynchronize(p->stream));
  p->P.bp_skip_angle = angle < 0 ? -1 : angle;
  p->P.bp_wait_limit = wait_limit;
  if (p->g_one) { cudaGraphExecDestroy(p->g_one); p->g_one = nullptr; }
  if (p->g_chunk) { cudaGraphExecDestroy(p->g_chunk); p->g_chunk = nullptr; }
  return GT_OK;
}

int gt_get_tuning(gt_problem *p, int out[2]) {
  if (!p || !out) return set_err(GT_ERR_ARG, "null argument");
  out[0] = p->P.fwd_cfg;
  out[1] = p->P.bp_cfg;
  return GT_OK;
}

int gt_get_scalars(gt_problem *p, double out[4]) {
  if (!p || !out) return set_err(GT_ERR_ARG, "null argument");
  out[0] = p->ne; out[1] = p->sigma; out[2] = p->tau; out[3] = (double)p->iters;
  return GT_OK;
}

int gt_gap_ex(gt_problem *p, double U, double out[8]) {
  if (!p || !out) return set_err(GT_ERR_ARG, "null argument");
  if (!p->has_data) return set_err(GT_ERR_STATE, "gt_gap before gt_set_data");
  CK(cudaSetDevice(p->device));
  const bool tgv = p->reg == GT_TGV;
  const int nb = gt::gap_blocks(p->P);
  const size_t vt_bytes = tgv ? align256(sizeof(float) * p->d.vol * p->K) : 0;
  if (!p->gap_ws) {
    cudaError_t e = cudaMalloc(&p->gap_ws, vt_bytes + sizeof(double) * 7 * (size_t)nb);
    if (e != cudaSuccess) { p->gap_ws = nullptr; return cuda_err(e, "cudaMalloc (gap workspace)", __LINE__); }
  }
  float *vt = tgv ? (float *)p->gap_ws : p->v;
  double *part = (double *)((char *)p->gap_ws + vt_bytes);
  std::vector<double> h(7 * (size_t)nb);
  // K* lambda of the current lambda (k_bp writes only that buffer); the passes
  // write only their own blocks' partials, so the buffer starts at zero
  CK(gt::launch_bp(p->P, p->stream));
  CK(cudaMemsetAsync(part, 0, sizeof(double) * 7 * (size_t)nb, p->stream));
  CK(gt::launch_gap_pass1(p->P, p->disc, tgv, p->cpl, vt, part, nb, p->stream));
  CK(cudaMemcpyAsync(h.data(), part, sizeof(double) * 6 * nb, cudaMemcpyDeviceToHost, p->stream));
  CK(cudaStreamSynchronize(p->stream));
  auto sum = [&](int q) { double a = 0; for (int k = 0; k < nb; ++k) a += h[(size_t)q * nb + k]; return a; };
  auto mx = [&](int q) { double a = 0; for (int k = 0; k < nb; ++k) a = std::max(a, h[(size_t)q * nb + k]); return a; };
  const double ne = p->ne, a0 = p->alpha0 / (ne * ne), a1 = p->alpha1 / (ne * ne);
  const double data = sum(0) / (p->disc == GT_KL ? ne : ne * ne), fstar = sum(1) / (p->disc == GT_KL ? ne : 1.0);
  const double reg1 = sum(2), reg0 = tgv ? sum(3) : 0.0, maxv = mx(4), maxu = mx(5);
  const double theta = maxv > 0 ? std::min(1.0, a1 / maxv) : 1.0;
  if (!(U > 0)) U = maxu > 0 ? 2.0 * maxu : 1.0;
  CK(gt::launch_gap_pass2(p->P, vt, theta, U, part, nb, p->stream));
  CK(cudaMemcpyAsync(h.data() + 6 * (size_t)nb, part + 6 * (size_t)nb, sizeof(double) * nb, cudaMemcpyDeviceToHost,
                     p->stream));
  CK(cudaStreamSynchronize(p->stream));
  const double box = sum(6);
  const double P = a1 * reg1 + a0 * reg0 + data, Dv = -fstar + box;
  out[0] = P; out[1] = Dv; out[2] = P - Dv; out[3] = (P - Dv) / std::fabs(P);
  out[4] = theta; out[5] = U; out[6] = data; out[7] = fstar;
  return GT_OK;
}

int gt_gap(gt_problem *p, double out[4]) {
  double o[8];
  const int rc = gt_gap_ex(p, 0.0, o);
  if (rc) return rc;
  for (int k = 0; k < 4; ++k) out[k] = o[k];
  return GT_OK;
}

int gt_time_kernels(gt_problem *p, int reps, float *ms_out, int n) {
  if (!p || !ms_out || reps < 1 || n < 4) return set_err(GT_ERR_ARG, "bad argument");
  if (!p->has_data) return set_err(GT_ERR_STATE, "gt_time_kernels before gt_set_data");
  CK(cudaSetDevice(p->device));
  // n >= 6: the primal update as its two halves (u / ubar, then p / pbar), timed
  // separately into ms_out[4], ms_out[5], and ms_out[3] = their sum
  const bool halves = n >= 6;
  cudaEvent_t ev[6];
  for (auto &e : ev) CK(cudaEventCreate(&e));
  float acc[5] = {0, 0, 0, 0, 0};
  int rc = GT_OK;
  const bool tgv = p->reg == GT_TGV;
  for (int r = 0; r < reps && rc == GT_OK; ++r) {
    cudaError_t e = cudaEventRecord(ev[0], p->stream);
    if (e == cudaSuccess) e = gt::launch_dual(p->P, tgv, p->cpl, p->stream);
    if (e == cudaSuccess) e = cudaEventRecord(ev[1], p->stream);
    if (e == cudaSuccess) e = gt::launch_fwd(p->P, p->disc, p->stream);
    if (e == cudaSuccess) e = cudaEventRecord(ev[2], p->stream);
    if (e == cudaSuccess) e = gt::launch_bp(p->P, p->stream);
    if (e == cudaSuccess) e = cudaEventRecord(ev[3], p->stream);
    if (e == cudaSuccess) e = gt::launch_update(p->P, tgv, p->stream, halves ? 1 : 0);
    if (e == cudaSuccess) e = cudaEventRecord(ev[4], p->stream);
    if (halves && e == cudaSuccess) e = gt::launch_update(p->P, tgv, p->stream, 2);
    if (e == cudaSuccess) e = cudaEventRecord(ev[5], p->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(ev[5]);
    if (e != cudaSuccess) { rc = cuda_err(e, "kernel timing", __LINE__); break; }
    for (int k = 0; k < 5; ++k) {
      float ms = 0;
      cudaEventElapsedTime(&ms, ev[k], ev[k + 1]);
      acc[k] += ms;
    }
    p->iters += 1;
  }
  // n >= 7: the fused dual kernel of schedule 2 into ms_out[6] (0 where it does not
  // apply or its second buffer set does not exist).  It reads the state and writes
  // only that second set, so the state does not change.
  if (n >= 7) {
    ms_out[6] = 0.f;
    if (rc == GT_OK && p->fused && fused_available(p)) {
      gt::IterParams Q = p->P;
      Q.p2 = p->fused;
      Q.v2 = p->fused + (size_t)p->K * p->d.vol;
      Q.w2 = Q.v2 + (size_t)p->K * p->d.vol;
      float tot = 0.f;
      for (int r = 0; r < reps && rc == GT_OK; ++r) {
        cudaError_t e = cudaEventRecord(ev[0], p->stream);
        if (e == cudaSuccess) e = gt::launch_dual_fused(Q, 1, p->cpl, p->stream);
        if (e == cudaSuccess) e = cudaEventRecord(ev[1], p->stream);
        if (e == cudaSuccess) e = cudaEventSynchronize(ev[1]);
        float ms = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, ev[0], ev[1]);
        if (e != cudaSuccess) { rc = cuda_err(e, "kernel timing (fused dual)", __LINE__); break; }
        tot += ms;
      }
      ms_out[6] = tot / reps;
    }
  }
  for (auto &e : ev) cudaEventDestroy(e);
  if (rc) return rc;
  for (int k = 0; k < 3; ++k) ms_out[k] = acc[k] / reps;
  ms_out[3] = (acc[3] + acc[4]) / reps;
  if (halves) {
    ms_out[4] = acc[3] / reps;
    ms_out[5] = acc[4] / reps;
  }
  return GT_OK;
}

static int run_projector(bool forward, const float *in, float *out, const double *angles, int N, int nd, int nang,
                         int S, void *stream) {
  if (!in || !out || !angles) return set_err(GT_ERR_ARG, "null argument");
  if (N < 1 || nd < 1 || nang < 1 || S < 1) return set_err(GT_ERR_ARG, "sizes must be positive");
  std::vector<double> t64;
  angle_table(angles, N, nd, nang, t64);
  std::vector<float> t32(t64.size());
  for (size_t k = 0; k < t64.size(); ++k) t32[k] = (float)t64[k];
  cudaStream_t st = (cudaStream_t)stream;
  float4 *ofs = nullptr;
  CK(cudaMalloc(&ofs, sizeof(float4) * nang));
  cudaError_t e = cudaMemcpyAsync(ofs, t32.data(), sizeof(float4) * nang, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = forward ? gt::launch_radon(in, out, ofs, N, nd, nang, S, st) : gt::launch_radon_ad(in, out, ofs, N, nd, nang, S, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(ofs);
  if (e != cudaSuccess) return cuda_err(e, forward ? "radon" : "radon_ad", __LINE__);
  return GT_OK;
}

int gt_radon(const float *img_dev, float *sino_dev, const double *angles, int N, int nd, int nang, int S,
             void *stream) {
  return run_projector(true, img_dev, sino_dev, angles, N, nd, nang, S, stream);
}

int gt_radon_ad(const float *sino_dev, float *img_dev, const double *angles, int N, int nd, int nang, int S,
                void *stream) {
  return run_projector(false, sino_dev, img_dev, angles, N, nd, nang, S, stream);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Batches: many independent problems (uneven sizes, channels, angle sets,
// discrepancies) advanced together.  Each problem keeps its buffers and tuned
// launch shapes; a chunk of iterations of all problems is captured into one
// CUDA graph as parallel branches (fork from a batch stream, join back), so one
// graph launch drives the whole batch and the GPU overlaps the problems' kernels.
// ---------------------------------------------------------------------------
struct gt_batch {
  std::vector<gt_problem *> probs;
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t fork = nullptr;
  std::vector<cudaEvent_t> joins;
  cudaGraphExec_t g_chunk = nullptr, g_one = nullptr;
  int chunk = 8;
  int chains = 8;  // problems are spread over this many concurrent chains
  long long iters = 0;
  std::vector<char> active;  // problems advanced by gt_batch_run
  int mode = 0;              // 0: a graph of per-problem chains; 1: fused launches over all members
  void *tab = nullptr;       // mode 1: device tables (members' IterParams, per-phase block starts, data terms)
  size_t tab_bytes = 0;
};

// One iteration of every problem: problem k runs on chain k % chains; chains run
// concurrently, problems of one chain one after another.
// Fused mode: per phase, one launch over the blocks of every active member.
// The tables are rebuilt (synchronously, before the capture) from the members'
// current parameters.
static int batch_capture_fused(gt_batch *b, int n, cudaGraphExec_t *out) {
  std::vector<gt_problem *> act;
  for (size_t k = 0; k < b->probs.size(); ++k)
    if (b->active[k]) act.push_back(b->probs[k]);
  const int na = (int)act.size();
  gt_problem *p0 = act[0];
  int cmax = 4;
  for (auto p : act) if (p->d.C > 4) cmax = 8;
  std::vector<gt::IterParams> P(na);
  std::vector<int> disc(2 * (size_t)na), start(4 * (size_t)(na + 1));  // data terms, then shapes
  long long total[4] = {0, 0, 0, 0};
  for (int ph = 0; ph < 4; ++ph) {
    for (int k = 0; k < na; ++k) {
      start[(size_t)ph * (na + 1) + k] = (int)total[ph];
      total[ph] += gt::batch_blocks(act[k]->d, ph);
    }
    start[(size_t)ph * (na + 1) + na] = (int)total[ph];
    if (total[ph] >= (1ll << 31)) return set_err(GT_ERR_ARG, "fused batch: more than 2^31 blocks in one launch");
  }
  for (int k = 0; k < na; ++k) {
    P[k] = act[k]->P;
    P[k].cbase = 0;
    disc[k] = act[k]->disc == GT_KL ? gt::KL : gt::L2;
    disc[na + k] = gt::batch_shape(act[k]->d);
  }
  const size_t offP = 0, offS = align256(sizeof(gt::IterParams) * na), offD = offS + align256(sizeof(int) * start.size());
  const size_t bytes = offD + sizeof(int) * 2 * na;
  if (bytes > b->tab_bytes) {
    if (b->tab) cudaFree(b->tab);
    b->tab = nullptr;
    b->tab_bytes = 0;
    CK(cudaMalloc(&b->tab, bytes));
    b->tab_bytes = bytes;
  }
  char *t = (char *)b->tab;
  CK(cudaMemcpyAsync(t + offP, P.data(), sizeof(gt::IterParams) * na, cudaMemcpyHostToDevice, b->stream));
  CK(cudaMemcpyAsync(t + offS, start.data(), sizeof(int) * start.size(), cudaMemcpyHostToDevice, b->stream));
  CK(cudaMemcpyAsync(t + offD, disc.data(), sizeof(int) * 2 * na, cudaMemcpyHostToDevice, b->stream));
  CK(cudaStreamSynchronize(b->stream));
  cudaGraph_t g = nullptr;
  CK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  cudaError_t e = cudaSuccess;
  const int tgv = p0->reg == GT_TGV, cpl = p0->cpl == GT_FROB ? gt::FROB : gt::UNCORR;
  for (int it = 0; it < n && e == cudaSuccess; ++it) {
    for (int ph = 0; ph < 4 && e == cudaSuccess; ++ph) {
      gt::BatchTab T{(const gt::IterParams *)(t + offP), (const int *)(t + offS) + (size_t)ph * (na + 1),
                     (const int *)(t + offD), (const int *)(t + offD) + na, na};
      e = gt::launch_batch_phase(T, ph, total[ph], p0->d.dim, tgv, cpl, cmax, b->stream);
    }
  }
  cudaError_t e2 = cudaStreamEndCapture(b->stream, &g);
  if (e != cudaSuccess || e2 != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return cuda_err(e != cudaSuccess ? e : e2, "fused batch capture", __LINE__);
  }
  e = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return cuda_err(e, "cudaGraphInstantiate (fused batch)", __LINE__);
  return GT_OK;
}

static int batch_capture(gt_batch *b, int n, cudaGraphExec_t *out) {
  if (b->mode == 1) return batch_capture_fused(b, n, out);
  cudaGraph_t g = nullptr;
  CK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  int rc = GT_OK;
  cudaError_t e = cudaSuccess;
  std::vector<size_t> act;  // the active problems, in order
  for (size_t k = 0; k < b->probs.size(); ++k)
    if (b->active[k]) act.push_back(k);
  const size_t np = act.size();
  const size_t chains = std::max<size_t>(1, std::min<size_t>(np, (size_t)b->chains));
  for (int it = 0; it < n && rc == GT_OK && e == cudaSuccess; ++it) {
    e = cudaEventRecord(b->fork, b->stream);
    for (size_t k = 0; k < np && rc == GT_OK && e == cudaSuccess; ++k) {
      gt_problem *p = b->probs[act[k]];
      // first problem of a chain waits for the fork, the others for their predecessor
      e = cudaStreamWaitEvent(p->stream, k < chains ? b->fork : b->joins[act[k - chains]], 0);
      if (e == cudaSuccess) rc = enqueue_iteration(p);
      if (rc == GT_OK && e == cudaSuccess) e = cudaEventRecord(b->joins[act[k]], p->stream);
    }
    for (size_t k = np - std::min(np, chains); k < np && rc == GT_OK && e == cudaSuccess; ++k)
      e = cudaStreamWaitEvent(b->stream, b->joins[act[k]], 0);
  }
  cudaError_t e2 = cudaStreamEndCapture(b->stream, &g);
  if (rc != GT_OK || e != cudaSuccess || e2 != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    if (rc) return rc;
    return cuda_err(e != cudaSuccess ? e : e2, "batch capture", __LINE__);
  }
  e = cudaGraphInstantiate(out, g, cudaGraphInstantiateFlagUseNodePriority);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return cuda_err(e, "cudaGraphInstantiate (batch)", __LINE__);
  return GT_OK;
}

extern "C" {

void gt_batch_destroy(gt_batch *b) {
  if (!b) return;
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->g_chunk) cudaGraphExecDestroy(b->g_chunk);
  if (b->g_one) cudaGraphExecDestroy(b->g_one);
  for (auto e : b->joins) if (e) cudaEventDestroy(e);
  if (b->fork) cudaEventDestroy(b->fork);
  for (auto p : b->probs) gt_problem_destroy(p);
  if (b->tab) cudaFree(b->tab);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

int gt_batch_set_mode(gt_batch *b, int mode) {
  if (!b || (mode != 0 && mode != 1)) return set_err(GT_ERR_ARG, "gt_batch_set_mode: mode must be 0 or 1");
  if (mode == 1) {
    const gt_problem *p0 = b->probs[0];
    for (auto p : b->probs) {
      if (p->d.dim != p0->d.dim || p->reg != p0->reg || p->cpl != p0->cpl)
        return set_err(GT_ERR_ARG, "fused batch: every member needs the same dimension, regularisation and coupling");
      if (p->cpl == GT_NUCL) return set_err(GT_ERR_ARG, "fused batch: nuclear coupling is not supported");
      if (p->d.C > 8) return set_err(GT_ERR_ARG, "fused batch: at most 8 channels per member");
      if (p->lsqr > 0) return set_err(GT_ERR_ARG, "fused batch: members of the two-resolution solver are not supported");
    }
  }
  CK(cudaSetDevice(b->device));
  CK(cudaStreamSynchronize(b->stream));
  b->mode = mode;
  return gt_batch_invalidate(b);
}

int gt_batch_get_mode(const gt_batch *b) { return b ? b->mode : -1; }

int gt_batch_create(int n, const gt_desc *descs, gt_batch **out) {
  if (!descs || !out || n < 1) return set_err(GT_ERR_ARG, "gt_batch_create: need n >= 1 descriptions");
  *out = nullptr;
  for (int k = 1; k < n; ++k)
    if (descs[k].device != descs[0].device) return set_err(GT_ERR_ARG, "gt_batch_create: one device per batch");
  gt_batch *b = new (std::nothrow) gt_batch();
  if (!b) return set_err(GT_ERR_OOM, "host allocation failed");
  b->device = descs[0].device;
  cudaError_t e = cudaSetDevice(b->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
  if (e != cudaSuccess) { gt_batch_destroy(b); return cuda_err(e, "batch setup", __LINE__); }
  for (int k = 0; k < n; ++k) {
    gt_desc d = descs[k];
    d.stream = nullptr;  // every problem runs on its own stream
    gt_problem *p = nullptr;
    const int rc = gt_problem_create(&d, &p);
    if (rc) { gt_batch_destroy(b); return rc; }
    b->probs.push_back(p);
    cudaEvent_t ev = nullptr;
    if ((e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming)) != cudaSuccess) {
      gt_batch_destroy(b);
      return cuda_err(e, "batch events", __LINE__);
    }
    b->joins.push_back(ev);
    b->active.push_back(1);
  }
  *out = b;
  return GT_OK;
}

int gt_batch_set_active(gt_batch *b, int k, int active) {
  if (!b || k < 0 || k >= (int)b->probs.size()) return set_err(GT_ERR_ARG, "gt_batch_set_active: bad index");
  if ((b->active[k] != 0) == (active != 0)) return GT_OK;
  CK(cudaSetDevice(b->device));
  CK(cudaStreamSynchronize(b->stream));
  b->active[k] = active ? 1 : 0;
  // the captured graphs hold the old member set
  if (b->g_chunk) { cudaGraphExecDestroy(b->g_chunk); b->g_chunk = nullptr; }
  if (b->g_one) { cudaGraphExecDestroy(b->g_one); b->g_one = nullptr; }
  return GT_OK;
}

int gt_batch_size(const gt_batch *b) { return b ? (int)b->probs.size() : 0; }

int gt_batch_problem(gt_batch *b, int k, gt_problem **out) {
  if (!b || !out || k < 0 || k >= (int)b->probs.size()) return set_err(GT_ERR_ARG, "gt_batch_problem: bad index");
  *out = b->probs[k];
  return GT_OK;
}

int gt_batch_run(gt_batch *b, int iters) {
  if (!b) return set_err(GT_ERR_ARG, "null batch");
  if (iters < 0) return set_err(GT_ERR_ARG, "negative iteration count");
  for (auto p : b->probs)
    if (!p->has_data) return set_err(GT_ERR_STATE, "gt_batch_run before every problem has data");
  if (iters == 0) return GT_OK;
  if (std::find(b->active.begin(), b->active.end(), 1) == b->active.end()) return GT_OK;  // nothing active
  CK(cudaSetDevice(b->device));
  // problems' own streams may still carry set-up work: the batch stream waits for it
  for (size_t k = 0; k < b->probs.size(); ++k) {
    CK(cudaEventRecord(b->joins[k], b->probs[k]->stream));
    CK(cudaStreamWaitEvent(b->stream, b->joins[k], 0));
  }
  int rc;
  if (iters >= b->chunk && !b->g_chunk && (rc = batch_capture(b, b->chunk, &b->g_chunk)) != GT_OK) return rc;
  if (!b->g_one && (rc = batch_capture(b, 1, &b->g_one)) != GT_OK) return rc;
  int left = iters;
  while (left >= b->chunk) { CK(cudaGraphLaunch(b->g_chunk, b->stream)); left -= b->chunk; }
  while (left > 0) { CK(cudaGraphLaunch(b->g_one, b->stream)); --left; }
  for (size_t k = 0; k < b->probs.size(); ++k)
    if (b->active[k]) b->probs[k]->iters += iters;
  b->iters += iters;
  return GT_OK;
}

int gt_batch_synchronize(gt_batch *b) {
  if (!b) return set_err(GT_ERR_ARG, "null batch");
  CK(cudaSetDevice(b->device));
  CK(cudaStreamSynchronize(b->stream));
  return GT_OK;
}

int gt_batch_set_concurrency(gt_batch *b, int chains) {
  if (!b || chains < 1) return set_err(GT_ERR_ARG, "gt_batch_set_concurrency: chains must be >= 1");
  b->chains = chains;
  return gt_batch_invalidate(b);
}

int gt_batch_invalidate(gt_batch *b) {
  if (!b) return set_err(GT_ERR_ARG, "null batch");
  if (b->g_chunk) { cudaGraphExecDestroy(b->g_chunk); b->g_chunk = nullptr; }
  if (b->g_one) { cudaGraphExecDestroy(b->g_one); b->g_one = nullptr; }
  return GT_OK;
}

}  // extern "C"

// ===========================================================================
// Two-resolution subsampling (radon_tgv_primal_dual_3dsubsample.py:51-1240).
// Channels [0, C0) have data at the image resolution (tilt series angles0);
// channels [C0, C0+C1) have data of a coarser detector and slice grid (nd1 x Nz1,
// tilt series angles1), related to the fine grid by an area-weighting matrix M
// per angle and channel: their forward operator is M R1 and its adjoint R1^T M^T.
// The regulariser couples all channels on the fine grid (k_dual / k_update of
// the inner problem); step constant Lsqr = 36 (:1033-1036).
// ===========================================================================
namespace {

// Create_Matrix_Line (3dsubsample :587-610): box of size a centred at (x, y) on
// the fine grid, area weights a*b / (4 r0 r1), indices clipped to the grid.
void matrix_line(const double a[2], double x, double y, int Nx, int Ny, std::vector<float> &A, std::vector<int> &I) {
  const double r0 = a[0] / 2., r1 = a[1] / 2.;
  const double xlower = x - r0, ylower = y - r1, xupper = x + r0, yupper = y + r1;
  const int xli = (int)std::ceil(x - r0 - 0.499999), yli = (int)std::ceil(y - r1 - 0.499999);
  const int xui = (int)std::floor(x + r0 + 0.499999), yui = (int)std::floor(y + r1 + 0.499999);
  for (int j = yli; j <= yui; ++j)
    for (int i = xli; i <= xui; ++i) {
      const double a1 = std::max(std::min(xupper - i, 0.5), -0.5), a2 = std::max(std::min(i - xlower, 0.5), -0.5);
      const double b1 = std::max(std::min(yupper - j, 0.5), -0.5), b2 = std::max(std::min(j - ylower, 0.5), -0.5);
      const double v = (a1 + a2) * (b1 + b2) / (4. * r0 * r1);
      const int ii = std::min(std::max(i, 0), Nx - 1), jj = std::min(std::max(j, 0), Ny - 1);
      A.push_back((float)v);
      I.push_back(ii + Nx * jj);
    }
}

}  // namespace

struct gt_subs {
  gt_problem *p = nullptr;   // all channels on the fine grid
  int C0 = 0, C1 = 0, Nz = 0, Nz1 = 0, nd1 = 0, nang0 = 0, nang1 = 0, N = 0;
  int S0 = 0, S1 = 0, S1lo = 0;
  int disc = GT_KL;
  void *block = nullptr;
  float4 *ofs0 = nullptr, *ofs1 = nullptr;
  float *ub0 = nullptr, *ub1 = nullptr, *ks0 = nullptr, *ks1 = nullptr;
  float *ku0 = nullptr, *ku1 = nullptr, *kulo = nullptr, *lamT = nullptr;
  float *f0 = nullptr, *f1 = nullptr, *lam0 = nullptr, *lam1 = nullptr, *mu0 = nullptr, *mu1 = nullptr;
  int *m_start = nullptr, *m_idx = nullptr, *mt_start = nullptr, *mt_idx = nullptr;
  float *m_val = nullptr, *mt_val = nullptr;
  double *part = nullptr;
  cudaGraphExec_t g_one = nullptr, g_chunk = nullptr;
  double normest = 0;
  float sigma_data = 0;
  bool has_data = false;
};

namespace {

// the projector side of one iteration on the side stream: both data groups
int subs_projections(gt_subs *s, cudaStream_t st) {
  gt_problem *p = s->p;
  const long long NN = (long long)s->N * s->N;
  const int nd0 = s->N;
  if (s->C0) {
    CK(gt::launch_gather_slices(p->ubar, p->d.S, 0, s->ub0, s->S0, NN, st));
    CK(gt::launch_radon(s->ub0, s->ku0, s->ofs0, s->N, nd0, s->nang0, s->S0, st));
    CK(gt::launch_lambda_update(s->lam0, s->ku0, s->f0, s->mu0, s->sigma_data, (long long)s->nang0 * nd0 * s->S0,
                                s->S0, s->Nz, s->disc, st));
    CK(gt::launch_radon_ad(s->lam0, s->ks0, s->ofs0, s->N, nd0, s->nang0, s->S0, st));
    CK(gt::launch_scatter_slices(s->ks0, s->S0, p->kstar, p->d.S, 0, NN, st));
  }
  CK(gt::launch_gather_slices(p->ubar, p->d.S, s->S0, s->ub1, s->S1, NN, st));
  CK(gt::launch_radon(s->ub1, s->ku1, s->ofs1, s->N, nd0, s->nang1, s->S1, st));
  CK(gt::launch_csr_planes(s->ku1, s->kulo, s->m_start, s->m_idx, s->m_val, s->nang1, s->C1, s->nd1, s->Nz1, nd0,
                           s->Nz, st));
  CK(gt::launch_lambda_update(s->lam1, s->kulo, s->f1, s->mu1, s->sigma_data, (long long)s->nang1 * s->nd1 * s->S1lo,
                              s->S1lo, s->Nz1, s->disc, st));
  CK(gt::launch_csr_planes(s->lam1, s->lamT, s->mt_start, s->mt_idx, s->mt_val, s->nang1, s->C1, nd0, s->Nz, s->nd1,
                           s->Nz1, st));
  CK(gt::launch_radon_ad(s->lamT, s->ks1, s->ofs1, s->N, nd0, s->nang1, s->S1, st));
  CK(gt::launch_scatter_slices(s->ks1, s->S1, p->kstar, p->d.S, s->S0, NN, st));
  return GT_OK;
}

int subs_iteration(gt_subs *s) {
  gt_problem *p = s->p;
  CK(cudaEventRecord(p->ev_fork, p->stream));
  CK(cudaStreamWaitEvent(p->side, p->ev_fork, 0));
  int rc = subs_projections(s, p->side);
  if (rc) return rc;
  const int tgv = p->reg == GT_TGV;
  CK(gt::launch_dual(p->P, tgv, p->cpl, p->stream));
  if (p->schedule == 1) CK(gt::launch_update(p->P, tgv, p->stream, 2));
  CK(cudaEventRecord(p->ev_join, p->side));
  CK(cudaStreamWaitEvent(p->stream, p->ev_join, 0));
  CK(gt::launch_update(p->P, tgv, p->stream, p->schedule == 1 ? 1 : 0));
  return GT_OK;
}

int subs_capture(gt_subs *s, int n, cudaGraphExec_t *out) {
  gt_problem *p = s->p;
  cudaGraph_t g = nullptr;
  CK(cudaStreamBeginCapture(p->stream, cudaStreamCaptureModeThreadLocal));
  int rc = GT_OK;
  for (int k = 0; k < n && rc == GT_OK; ++k) rc = subs_iteration(s);
  cudaError_t e = cudaStreamEndCapture(p->stream, &g);
  if (rc != GT_OK) { if (g) cudaGraphDestroy(g); return rc; }
  if (e != cudaSuccess) return cuda_err(e, "cudaStreamEndCapture", __LINE__);
  e = cudaGraphInstantiate(out, g, cudaGraphInstantiateFlagUseNodePriority);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return cuda_err(e, "cudaGraphInstantiate", __LINE__);
  return GT_OK;
}

}  // namespace

extern "C" {

void gt_subs_destroy(gt_subs *s) {
  if (!s) return;
  if (s->p) {
    cudaSetDevice(s->p->device);
    cudaStreamSynchronize(s->p->stream);
  }
  if (s->g_one) cudaGraphExecDestroy(s->g_one);
  if (s->g_chunk) cudaGraphExecDestroy(s->g_chunk);
  if (s->block) cudaFree(s->block);
  if (s->p) gt_problem_destroy(s->p);
  delete s;
}

int gt_subs_create(const gt_subs_desc *D, gt_subs **out) {
  if (!D || !out) return set_err(GT_ERR_ARG, "null argument");
  *out = nullptr;
  if (D->N < 1 || D->Nz < 1 || D->C0 < 0 || D->C1 < 1 || D->C0 + D->C1 > 8 || D->nang0 < (D->C0 ? 1 : 0) ||
      D->nang1 < 1 || D->nd1 < 1 || D->Nz1 < 1 || !(D->pixel_ratio > 0) || !D->angles1 || (D->C0 && !D->angles0) ||
      !D->mu || (D->coupling != GT_FROB && D->coupling != GT_UNCORR))
    return set_err(GT_ERR_ARG, "gt_subs_create: invalid description");
  gt_subs *s = new (std::nothrow) gt_subs();
  if (!s) return set_err(GT_ERR_OOM, "host allocation failed");
  s->C0 = D->C0; s->C1 = D->C1; s->Nz = D->Nz; s->Nz1 = D->Nz1; s->nd1 = D->nd1; s->N = D->N;
  s->nang0 = D->nang0; s->nang1 = D->nang1; s->disc = D->discrepancy;
  s->S0 = D->C0 * D->Nz; s->S1 = D->C1 * D->Nz; s->S1lo = D->C1 * D->Nz1;
  // inner problem: the fine grid for every channel, regulariser and primal update
  gt_desc d{};
  d.dim = 3; d.N = D->N; d.Nz = D->Nz; d.C = D->C0 + D->C1; d.nd = D->N;
  d.nang = D->C0 ? D->nang0 : D->nang1;
  d.angles = D->C0 ? D->angles0 : D->angles1;
  d.stepsize = D->stepsize; d.alpha0 = D->alpha0; d.alpha1 = D->alpha1; d.mu = D->mu;
  d.discrepancy = D->discrepancy; d.regularisation = D->regularisation; d.coupling = D->coupling;
  d.normest = 1.0; d.device = D->device; d.stream = D->stream; d.autotune = 0;
  int rc = gt_problem_create(&d, &s->p);
  if (rc) { delete s; return rc; }
  s->p->lsqr = 36.0;
  gt_problem *p = s->p;
  cudaError_t e;
  // interpolation matrix (Create_sparse_matrix :631-651 and its adjoint :612-629)
  const int nd0 = D->N;
  const double ratio[2] = {D->pixel_ratio, D->pixel_ratio / D->stepsize};
  const double refnew1 = D->refnew[1] / D->stepsize;  // :945 (divides the caller's list in place there)
  std::vector<int> start(1, 0), idx;
  std::vector<float> val;
  for (int j = 0; j < D->Nz1; ++j)
    for (int i = 0; i < D->nd1; ++i) {
      const double x = ratio[0] * (i - D->refold[0]) + D->refnew[0];
      const double y = ratio[1] * (j - D->refold[1]) + refnew1;
      matrix_line(ratio, x, y, nd0, D->Nz, val, idx);
      start.push_back((int)idx.size());
    }
  // adjoint: for every fine node, the rows that reference it, in row order (one
  // entry per reference, duplicates from clipping included)
  const int nfine = nd0 * D->Nz, nrow = D->nd1 * D->Nz1;
  std::vector<std::vector<int>> conn(nfine);
  for (int r = 0; r < nrow; ++r)
    for (int e2 = start[r]; e2 < start[r + 1]; ++e2) conn[idx[e2]].push_back(r);
  std::vector<int> tstart(1, 0), tidx;
  std::vector<float> tval;
  {
    std::vector<int> used(idx.size(), 0);
    for (int i = 0; i < nfine; ++i) {
      for (int r : conn[i]) {
        for (int e2 = start[r]; e2 < start[r + 1]; ++e2)
          if (idx[e2] == i && !used[e2]) { used[e2] = 1; tval.push_back(val[e2]); tidx.push_back(r); break; }
      }
      tstart.push_back((int)tidx.size());
    }
  }
  // device block
  const size_t NN = (size_t)D->N * D->N;
  const size_t nb0 = (size_t)D->nang0 * nd0 * s->S0, nb1 = (size_t)D->nang1 * nd0 * s->S1,
               nblo = (size_t)D->nang1 * D->nd1 * s->S1lo;
  size_t off = 0;
  auto take = [&](size_t bytes) { const size_t o = off; off += align256(std::max<size_t>(bytes, 4)); return o; };
  const size_t o_ofs0 = take(16 * (size_t)std::max(D->nang0, 1)), o_ofs1 = take(16 * (size_t)D->nang1);
  const size_t o_ub0 = take(4 * NN * s->S0), o_ub1 = take(4 * NN * s->S1);
  const size_t o_ks0 = take(4 * NN * s->S0), o_ks1 = take(4 * NN * s->S1);
  const size_t o_ku0 = take(4 * nb0), o_ku1 = take(4 * nb1), o_kulo = take(4 * nblo), o_lamT = take(4 * nb1);
  const size_t o_f0 = take(4 * nb0), o_f1 = take(4 * nblo), o_lam0 = take(4 * nb0), o_lam1 = take(4 * nblo);
  const size_t o_mu0 = take(4 * 8), o_mu1 = take(4 * 8);
  const size_t o_ms = take(4 * start.size()), o_mi = take(4 * idx.size()), o_mv = take(4 * val.size());
  const size_t o_ts = take(4 * tstart.size()), o_ti = take(4 * tidx.size()), o_tv = take(4 * tval.size());
  const size_t o_part = take(8 * 256);
  if ((e = cudaMalloc(&s->block, off)) != cudaSuccess) {
    cudaGetLastError();
    gt_subs_destroy(s);
    return set_err(GT_ERR_OOM, "two-resolution buffers (%.3f GB)", off / 1e9);
  }
  char *b = (char *)s->block;
  s->ofs0 = (float4 *)(b + o_ofs0); s->ofs1 = (float4 *)(b + o_ofs1);
  s->ub0 = (float *)(b + o_ub0); s->ub1 = (float *)(b + o_ub1); s->ks0 = (float *)(b + o_ks0);
  s->ks1 = (float *)(b + o_ks1); s->ku0 = (float *)(b + o_ku0); s->ku1 = (float *)(b + o_ku1);
  s->kulo = (float *)(b + o_kulo); s->lamT = (float *)(b + o_lamT); s->f0 = (float *)(b + o_f0);
  s->f1 = (float *)(b + o_f1); s->lam0 = (float *)(b + o_lam0); s->lam1 = (float *)(b + o_lam1);
  s->mu0 = (float *)(b + o_mu0); s->mu1 = (float *)(b + o_mu1);
  s->m_start = (int *)(b + o_ms); s->m_idx = (int *)(b + o_mi); s->m_val = (float *)(b + o_mv);
  s->mt_start = (int *)(b + o_ts); s->mt_idx = (int *)(b + o_ti); s->mt_val = (float *)(b + o_tv);
  s->part = (double *)(b + o_part);
  // angle tables: both series on the fine detector (radon_struct with n_detectors = Nx0, :926-931)
  auto table = [&](const double *ang, int nang, float4 *dst) -> int {
    std::vector<double> t64;
    angle_table(ang, D->N, nd0, nang, t64);
    std::vector<float> t32(t64.size());
    for (size_t k = 0; k < t64.size(); ++k) t32[k] = (float)t64[k];
    CK(cudaMemcpyAsync(dst, t32.data(), 4 * t32.size(), cudaMemcpyHostToDevice, p->stream));
    CK(cudaStreamSynchronize(p->stream));
    return GT_OK;
  };
  // zero the buffers first, then upload the tables into the block
  if ((e = cudaMemsetAsync(s->block, 0, o_ms, p->stream)) != cudaSuccess) {
    gt_subs_destroy(s);
    return cuda_err(e, "two-resolution set-up", __LINE__);
  }
  if (D->C0 && (rc = table(D->angles0, D->nang0, s->ofs0)) != GT_OK) { gt_subs_destroy(s); return rc; }
  if ((rc = table(D->angles1, D->nang1, s->ofs1)) != GT_OK) { gt_subs_destroy(s); return rc; }
  if ((e = cudaMemcpyAsync(s->m_start, start.data(), 4 * start.size(), cudaMemcpyHostToDevice, p->stream)) != cudaSuccess ||
      (e = cudaMemcpyAsync(s->m_idx, idx.data(), 4 * idx.size(), cudaMemcpyHostToDevice, p->stream)) != cudaSuccess ||
      (e = cudaMemcpyAsync(s->m_val, val.data(), 4 * val.size(), cudaMemcpyHostToDevice, p->stream)) != cudaSuccess ||
      (e = cudaMemcpyAsync(s->mt_start, tstart.data(), 4 * tstart.size(), cudaMemcpyHostToDevice, p->stream)) != cudaSuccess ||
      (e = cudaMemcpyAsync(s->mt_idx, tidx.data(), 4 * tidx.size(), cudaMemcpyHostToDevice, p->stream)) != cudaSuccess ||
      (e = cudaMemcpyAsync(s->mt_val, tval.data(), 4 * tval.size(), cudaMemcpyHostToDevice, p->stream)) != cudaSuccess ||
      (e = cudaStreamSynchronize(p->stream)) != cudaSuccess) {
    gt_subs_destroy(s);
    return cuda_err(e, "two-resolution set-up", __LINE__);
  }
  s->normest = D->normest;
  *out = s;
  return GT_OK;
}

// f0: [C0*Nz][nang0][N], f1: [C1*Nz1][nang1][nd1] (s = c*Nz + z); resets the iterates
int gt_subs_set_data(gt_subs *s, const float *f0, const float *f1, int make_feasible) {
  if (!s || (!f0 && s->C0) || !f1) return set_err(GT_ERR_ARG, "null argument");
  gt_problem *p = s->p;
  CK(cudaSetDevice(p->device));
  const int nd0 = s->N;
  const size_t nb0 = (size_t)s->nang0 * nd0 * s->S0, nblo = (size_t)s->nang1 * s->nd1 * s->S1lo;
  // host layout [S][bins] -> device [bins][S]
  if (s->C0) {
    CK(cudaMemcpyAsync(p->stage, f0, 4 * nb0, cudaMemcpyHostToDevice, p->stream));
    CK(gt::launch_transpose(p->stage, s->f0, s->S0, s->nang0 * nd0, p->stream));
  }
  CK(cudaMemcpyAsync(p->stage, f1, 4 * nblo, cudaMemcpyHostToDevice, p->stream));
  CK(gt::launch_transpose(p->stage, s->f1, s->S1lo, s->nang1 * s->nd1, p->stream));
  if (make_feasible) {
    // Make_function_feasible (3dsubsample :466-476): bins where the projection of the
    // all-ones slice is <= 0 are zeroed (the low-resolution data uses the mask of the
    // fine detector, restricted to its own bins)
    float *ones = p->stage, *r1 = p->ku;
    CK(gt::fill_f32(ones, (size_t)s->N * s->N, 1.f, p->stream));
    if (s->C0) {
      CK(gt::launch_radon(ones, r1, s->ofs0, s->N, nd0, s->nang0, 1, p->stream));
      CK(gt::launch_feasible(s->f0, r1, s->nang0 * nd0, s->S0, p->stream));
    }
    CK(gt::launch_radon(ones, r1, s->ofs1, s->N, nd0, s->nang1, 1, p->stream));
    std::vector<float> mask((size_t)s->nang1 * nd0);
    CK(cudaMemcpyAsync(mask.data(), r1, 4 * mask.size(), cudaMemcpyDeviceToHost, p->stream));
    CK(cudaStreamSynchronize(p->stream));
    std::vector<float> m1((size_t)s->nang1 * s->nd1, 1.f);
    for (int j = 0; j < s->nang1; ++j)
      for (int i = 0; i < std::min(nd0, s->nd1); ++i)
        if (mask[(size_t)j * nd0 + i] <= 0.f) m1[(size_t)j * s->nd1 + i] = 0.f;
    CK(cudaMemcpyAsync(r1, m1.data(), 4 * m1.size(), cudaMemcpyHostToDevice, p->stream));
    CK(gt::launch_feasible(s->f1, r1, s->nang1 * s->nd1, s->S1lo, p->stream));
  }
  // operator norm: injected, or a power iteration of K^T K from the all-ones image
  if (!(s->normest > 0)) {
    const long long n = (long long)p->d.vol;
    float *x = p->u;
    CK(gt::fill_f32(x, (size_t)n, 1.f, p->stream));
    double nrm = 0;
    std::vector<double> h(256);
    gt_problem *pp = p;
    for (int r = 0; r < 30; ++r) {
      CK(gt::launch_sumsq(x, n, s->part, 256, pp->stream));
      CK(cudaMemcpyAsync(h.data(), s->part, 8 * 256, cudaMemcpyDeviceToHost, pp->stream));
      CK(cudaStreamSynchronize(pp->stream));
      double a = 0;
      for (double v : h) a += v;
      nrm = std::sqrt(a);
      if (!(nrm > 0)) return set_err(GT_ERR_CUDA, "two-resolution operator norm estimate failed");
      CK(gt::launch_scale_f32(x, n, (float)(1.0 / nrm), pp->stream));
      // x <- K^T K x, per group (ubar is the projections' input)
      CK(cudaMemcpyAsync(p->ubar, x, 4 * (size_t)n, cudaMemcpyDeviceToDevice, pp->stream));
      const long long NN = (long long)s->N * s->N;
      if (s->C0) {
        CK(gt::launch_gather_slices(p->ubar, p->d.S, 0, s->ub0, s->S0, NN, pp->stream));
        CK(gt::launch_radon(s->ub0, s->ku0, s->ofs0, s->N, nd0, s->nang0, s->S0, pp->stream));
        CK(gt::launch_radon_ad(s->ku0, s->ks0, s->ofs0, s->N, nd0, s->nang0, s->S0, pp->stream));
        CK(gt::launch_scatter_slices(s->ks0, s->S0, x, p->d.S, 0, NN, pp->stream));
      }
      CK(gt::launch_gather_slices(p->ubar, p->d.S, s->S0, s->ub1, s->S1, NN, pp->stream));
      CK(gt::launch_radon(s->ub1, s->ku1, s->ofs1, s->N, nd0, s->nang1, s->S1, pp->stream));
      CK(gt::launch_csr_planes(s->ku1, s->kulo, s->m_start, s->m_idx, s->m_val, s->nang1, s->C1, s->nd1, s->Nz1, nd0,
                               s->Nz, pp->stream));
      CK(gt::launch_csr_planes(s->kulo, s->lamT, s->mt_start, s->mt_idx, s->mt_val, s->nang1, s->C1, nd0, s->Nz,
                               s->nd1, s->Nz1, pp->stream));
      CK(gt::launch_radon_ad(s->lamT, s->ks1, s->ofs1, s->N, nd0, s->nang1, s->S1, pp->stream));
      CK(gt::launch_scatter_slices(s->ks1, s->S1, x, p->d.S, s->S0, NN, pp->stream));
    }
    s->normest = std::sqrt(nrm);
  }
  p->ne = s->normest;
  set_scalars(p);
  s->sigma_data = p->P.sigma_data;
  // channel weights: KL mu, L2 mu/(sigma+mu) (:1038-1045)
  std::vector<float> me(8, 0.f);
  const int C = s->C0 + s->C1;
  for (int c = 0; c < C; ++c)
    me[c] = (float)(s->disc == GT_KL ? p->mu[c] : p->mu[c] / (p->sigma + p->mu[c]));
  CK(cudaMemcpyAsync(s->mu0, me.data(), 4 * 8, cudaMemcpyHostToDevice, p->stream));
  CK(cudaMemcpyAsync(s->mu1, me.data() + s->C0, 4 * (8 - s->C0), cudaMemcpyHostToDevice, p->stream));
  CK(cudaMemcpyAsync(p->mu_eff, me.data(), 4 * C, cudaMemcpyHostToDevice, p->stream));
  p->P.ne64 = p->ne;
  // zero the iterates (:1057-1075)
  const size_t fv = 4 * p->d.vol;
  CK(cudaMemsetAsync(p->u, 0, fv, p->stream));
  CK(cudaMemsetAsync(p->ubar, 0, fv, p->stream));
  if (p->p) CK(cudaMemsetAsync(p->p, 0, fv * p->K, p->stream));
  if (p->pbar) CK(cudaMemsetAsync(p->pbar, 0, fv * p->K, p->stream));
  CK(cudaMemsetAsync(p->v, 0, fv * p->K, p->stream));
  if (p->w) CK(cudaMemsetAsync(p->w, 0, fv * p->KW, p->stream));
  if (s->C0) CK(cudaMemsetAsync(s->lam0, 0, 4 * nb0, p->stream));
  CK(cudaMemsetAsync(s->lam1, 0, 4 * nblo, p->stream));
  CK(cudaStreamSynchronize(p->stream));
  if (s->g_one) { cudaGraphExecDestroy(s->g_one); s->g_one = nullptr; }
  if (s->g_chunk) { cudaGraphExecDestroy(s->g_chunk); s->g_chunk = nullptr; }
  p->iters = 0;
  p->has_data = true;
  s->has_data = true;
  return GT_OK;
}

int gt_subs_run(gt_subs *s, int iters) {
  if (!s) return set_err(GT_ERR_ARG, "null argument");
  if (!s->has_data) return set_err(GT_ERR_STATE, "gt_subs_run before gt_subs_set_data");
  if (iters <= 0) return iters == 0 ? GT_OK : set_err(GT_ERR_ARG, "negative iteration count");
  gt_problem *p = s->p;
  CK(cudaSetDevice(p->device));
  int rc;
  const int chunk = 16;
  if (iters >= chunk && !s->g_chunk && (rc = subs_capture(s, chunk, &s->g_chunk)) != GT_OK) return rc;
  if (!s->g_one && (rc = subs_capture(s, 1, &s->g_one)) != GT_OK) return rc;
  int left = iters;
  while (left >= chunk) { CK(cudaGraphLaunch(s->g_chunk, p->stream)); left -= chunk; }
  while (left > 0) { CK(cudaGraphLaunch(s->g_one, p->stream)); --left; }
  p->iters += iters;
  return GT_OK;
}

// which: GT_SUBS_U [C*Nz][N][N]; GT_SUBS_KU0 [C0*Nz][nang0][N]; GT_SUBS_KU1 [C1*Nz][nang1][N]
// (fine grid); GT_SUBS_KULO [C1*Nz1][nang1][nd1]
int gt_subs_get(gt_subs *s, int which, float *host) {
  if (!s || !host) return set_err(GT_ERR_ARG, "null argument");
  gt_problem *p = s->p;
  CK(cudaSetDevice(p->device));
  CK(cudaStreamSynchronize(p->stream));
  const int nd0 = s->N;
  const float *src; int rows, cols;
  switch (which) {
    case GT_SUBS_U: return gt_get_state(p, GT_U, host);
    case GT_SUBS_KU0: src = s->ku0; rows = s->nang0 * nd0; cols = s->S0; break;
    case GT_SUBS_KU1: src = s->ku1; rows = s->nang1 * nd0; cols = s->S1; break;
    case GT_SUBS_KULO: src = s->kulo; rows = s->nang1 * s->nd1; cols = s->S1lo; break;
    default: return set_err(GT_ERR_ARG, "unknown field %d", which);
  }
  if (cols == 0) return GT_OK;
  CK(gt::launch_transpose(src, p->stage, rows, cols, p->stream));
  CK(cudaMemcpyAsync(host, p->stage, 4 * (size_t)rows * cols, cudaMemcpyDeviceToHost, p->stream));
  CK(cudaStreamSynchronize(p->stream));
  return GT_OK;
}

double gt_subs_normest(const gt_subs *s) { return s ? s->normest : 0.0; }

gt_problem *gt_subs_problem(gt_subs *s) { return s ? s->p : nullptr; }

}  // extern "C"
