// Allocation-free operator-norm estimate (gt_normest_noalloc).
//
// Some callers cannot allocate device memory while they run: a host framework
// that owns the device memory (its own pool or caching allocator, where an
// outside cudaMalloc fragments the pool and may fail once the pool holds the
// memory), or latency-sensitive code that cannot afford cudaFree's implicit
// synchronisation of the whole device.  For them this entry point runs the same
// FP64 power iteration that gt_set_data runs when no estimate is supplied, but
// its scratch -- the angle table, one image slice, one sinogram slice and the
// partial sums -- lives in a fixed file-scope device array instead of a
// cudaMalloc'd buffer.  It calls no cudaMalloc, cudaFree or other allocating
// routine.
//
// The array is GT_NOALLOC_SCRATCH_DOUBLES doubles (8 MiB).  Every GPU that loads
// this library keeps it for the life of the process.  All calls share it and it
// keeps the last call's contents (every call rewrites what it reads before
// reading it).
//
// Every call is host-synchronous: it ends by synchronising `stream` and copying
// the estimate to the host, so it blocks until its GPU work is done and must
// never be made on a stream that is being captured into a CUDA graph.  Two calls
// therefore overlap on the GPU only when host threads call concurrently for the
// same device (or other work on that device touches the array); they then race on
// the scratch, so such threads must serialise their calls.
//
// Each call looks up the array's device address on the device it runs on
// (cudaGetSymbolAddress, with that device current) and passes that address to the
// kernels; it does not cache it, so a call made after cudaDeviceReset uses the
// array of the new context.  The first call on a device also loads the library's
// device code there.  The caller's current device is restored before returning.
#include <cuda_runtime.h>

#include <cmath>

#include "graptor_gb300.h"
#include "gt_common.cuh"

namespace gt {
cudaError_t normest64(const dvec4 *ofs, int N, int nd, int nang, int rounds, double *d_img, double *d_sino,
                      double *d_part, double *out, cudaStream_t st);
cudaError_t fill_f64(double *x, size_t n, double v, cudaStream_t st);
int set_error(int code, const char *msg);
int cuda_error(cudaError_t e, const char *what, int line);
}  // namespace gt

#define GT_NOALLOC_SCRATCH_DOUBLES (1u << 20)
#define GT_NOALLOC_PARTIALS 256

// In host code this name is only a host-side handle: its device address comes
// from cudaGetSymbolAddress below.
static __device__ __align__(256) double g_noalloc_scratch[GT_NOALLOC_SCRATCH_DOUBLES];

namespace {

// device address of the scratch array on the current device
int scratch_here(double **out) {
  void *ptr = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
  if (e != cudaSuccess) return gt::cuda_error(e, "cudaGetSymbolAddress(g_noalloc_scratch)", __LINE__);
  *out = static_cast<double *>(ptr);
  return GT_OK;
}

// the estimate on the current device (the entry point below selects it)
int normest_here(const double *angles, int N, int nd, int nang, void *stream, double *out) {
  double *base = nullptr;
  int rc = scratch_here(&base);
  if (rc) return rc;
  cudaError_t e;
  cudaStream_t st = (cudaStream_t)stream;
  dvec4 *ofs = reinterpret_cast<dvec4 *>(base);
  double *img = base + 4 * (size_t)nang, *sino = img + (size_t)N * N, *part = sino + (size_t)nd * nang;

  // angle table of radon_struct (radon_tgv_primal_dual_3d.py:947-979) in chunks
  // through a stack buffer (no host allocation either)
  const double mid_dom = (N - 1) / 2.0, mid_det = (nd - 1.0) / 2.0;
  dvec4 chunk[128];
  for (int j0 = 0; j0 < nang; j0 += 128) {
    const int m = nang - j0 < 128 ? nang - j0 : 128;
    for (int k = 0; k < m; ++k) {
      const double a = angles[j0 + k];
      double X = std::cos(a), Y = std::sin(a), Xinv = 1.0 / X;
      if (std::fabs(Xinv) > 10.0 * nd) {
        X = 0.0;
        Y = std::nearbyint(std::sin(a));
        Xinv = 0.0;
      }
      chunk[k] = dvec4{X, Y, mid_det - X * mid_dom - Y * mid_dom, Xinv};
    }
    // pageable source: the copy is staged before cudaMemcpyAsync returns, so the
    // stack chunk may be refilled right after
    e = cudaMemcpyAsync(ofs + j0, chunk, sizeof(dvec4) * m, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return gt::cuda_error(e, "cudaMemcpyAsync (angle table)", __LINE__);
  }
  // the power iteration starts from the all-ones image: overwrite the previous call's contents
  if ((e = gt::fill_f64(img, (size_t)N * N, 1.0, st)) != cudaSuccess) return gt::cuda_error(e, "fill", __LINE__);
  double ne = 0.0;
  if ((e = gt::normest64(ofs, N, nd, nang, 30, img, sino, part, &ne, st)) != cudaSuccess)
    return gt::cuda_error(e, "normest64", __LINE__);
  if (!(ne > 0) || !std::isfinite(ne)) return gt::set_error(GT_ERR_CUDA, "gt_normest_noalloc: estimate failed");
  *out = ne;
  return GT_OK;
}

}  // namespace

extern "C" int gt_normest_noalloc(const double *angles, int N, int nd, int nang, int device, void *stream,
                                  double *out) {
  if (!angles || !out) return gt::set_error(GT_ERR_ARG, "gt_normest_noalloc: null argument");
  if (N < 1 || nd < 1 || nang < 1) return gt::set_error(GT_ERR_ARG, "gt_normest_noalloc: sizes must be positive");
  const size_t need = 4 * (size_t)nang + (size_t)N * N + (size_t)nd * nang + GT_NOALLOC_PARTIALS;
  if (need > GT_NOALLOC_SCRATCH_DOUBLES)
    return gt::set_error(GT_ERR_ARG,
                         "gt_normest_noalloc: 4*nang + N*N + nd*nang + 256 must not exceed 1048576 doubles "
                         "(the fixed 8 MiB scratch); use gt_problem_create/gt_set_data for larger geometries");
  int caller = 0;
  cudaError_t e = cudaGetDevice(&caller);
  if (e != cudaSuccess) return gt::cuda_error(e, "cudaGetDevice", __LINE__);
  if (caller != device && (e = cudaSetDevice(device)) != cudaSuccess) {
    const int rc = gt::cuda_error(e, "cudaSetDevice", __LINE__);
    cudaSetDevice(caller);
    return rc;
  }
  const int rc = normest_here(angles, N, nd, nang, stream, out);
  // the caller's current device is left as it was, on success and on error alike
  if (caller != device && (e = cudaSetDevice(caller)) != cudaSuccess && rc == GT_OK)
    return gt::cuda_error(e, "cudaSetDevice (restoring the caller's device)", __LINE__);
  return rc;
}
