// Detection of unsuitable projections on the GPU: the three array stages of
// Find_Bad_projections (find_bad_ele.py:139-230) for a whole projection stack.
//
//   gt_badproj_smooth   box sum over a (2s+1)^2 window / (4 s^2)        (reduce_noise, :69-75)
//                       summed in FP64 in the reference's order, stored as FP32 (:152-155)
//   gt_badproj_wgrad    largest neighbour difference (diagonals / sqrt 2) times the
//                       smallest neighbour magnitude                    (weighted_gradient, :103-136)
//                       in FP32 as the reference computes it on its FP32 stack, so
//                       every value is bit-identical
//   gt_badproj_compare  for projection pairs (i, i + offset): per interior pixel the
//                       smallest |U - V shifted| over shifts within the radius, both
//                       ways, their maximum, summed per pair        (compare_shift(_twosided),
//                       :55-100, called at :177-190)
//
// The comparison dominates (radius^2 work per pixel).  A block covers 32 columns x
// 32 rows of one pair; a thread owns one column and eight consecutive rows, so every
// value loaded from the shifted window serves up to eight pixels (a sliding column
// window) and the loop is bound by FP32 issue, not by loads.  The per-pixel minima
// are exact in FP32 (rounding is monotone, so the minimum of rounded differences is
// the rounded minimum, which is what the reference's FP32 subtraction yields); the
// pair sums are FP64, per block in a fixed order and then over blocks in a fixed
// order, so results are deterministic.
#include <cuda_runtime.h>

#include "graptor_gb300.h"

namespace {

constexpr int CMP_TX = 32;          // columns per block (one warp wide)
constexpr int CMP_TY = 4;           // warps per block
constexpr int CMP_ROWS = 8;         // rows per thread
constexpr int CMP_TILE_Y = CMP_TY * CMP_ROWS;

inline unsigned nblk(long long n, int t) { return (unsigned)((n + t - 1) / t); }

__global__ void k_smooth(const double *__restrict__ d, int na, int nz, int nx, int s, float *__restrict__ out) {
  const int oz = nz - 2 * s, ox = nx - 2 * s;
  const long long n = (long long)na * oz * ox;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int x = (int)(i % ox);
  const int y = (int)((i / ox) % oz);
  const int a = (int)(i / ((long long)ox * oz));
  const double *p = d + ((size_t)a * nz + y) * nx + x;  // window corner (y + s - s, x + s - s)
  double acc = 0.0;
  for (int k = 0; k <= 2 * s; ++k)
    for (int l = 0; l <= 2 * s; ++l) acc += __ldg(p + (size_t)k * nx + l);
  out[i] = __double2float_rn(acc / (double)(4 * s * s));
}

__global__ void k_wgrad(const float *__restrict__ u, int na, int nz, int nx, float *__restrict__ w) {
  const int oz = nz - 2, ox = nx - 2;
  const long long n = (long long)na * oz * ox;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int x = (int)(i % ox) + 1;
  const int y = (int)((i / ox) % oz) + 1;
  const int a = (int)(i / ((long long)ox * oz));
  const float *p = u + ((size_t)a * nz + y) * nx + x;
  const float c = __ldg(p);
  const float rs2 = (float)1.4142135623730951;  // the reference's (1 + 1) ** 0.5, rounded to FP32
  float e = 0.f, m = 0.f;
  bool first = true;
#pragma unroll
  for (int di = -1; di <= 1; ++di)
#pragma unroll
    for (int dj = -1; dj <= 1; ++dj) {
      if (di == 0 && dj == 0) continue;
      const float nb = __ldg(p + di * nx + dj);
      float g = fabsf(c - nb);
      if (di != 0 && dj != 0) g = g / rs2;  // IEEE division, as NumPy's FP32 divide
      const float an = fabsf(nb);
      e = first ? g : fmaxf(e, g);
      m = first ? an : fminf(m, an);
      first = false;
    }
  w[i] = e * m;  // FP32 product = the FP64 product (exact) rounded to FP32
}

// the pixels j in [j0, j1] take the window values a (from V) and b (from U)
__device__ __forceinline__ void cmp_upd(float (&m1)[CMP_ROWS], float (&m2)[CMP_ROWS], const float (&u)[CMP_ROWS],
                                        const float (&v)[CMP_ROWS], float a, float b, int j0, int j1) {
#pragma unroll
  for (int j = 0; j < CMP_ROWS; ++j)
    if (j >= j0 && j <= j1) {
      m1[j] = fminf(m1[j], fabsf(u[j] - a));
      m2[j] = fminf(m2[j], fabsf(v[j] - b));
    }
}

// grid (tiles per pair, pairs), block (32, 4).  Pair q compares projection q (U)
// with q + offset (V) on the interior [r, nz - r) x [r, nx - r).  Column x of the
// interior, rows y0 .. y0 + 7; row t of the sliding window is image row y0 + t,
// t in [0, 2r + 7]; interior row y0 + j (image row y0 + j + r) uses t in [j, j + 2r].
// With 2r >= 7 the window splits into a head (t < 7: rows j <= t), a middle
// (every row) and a tail (t > 2r: rows j >= t - 2r), all with compile-time row sets.
__global__ void __launch_bounds__(CMP_TX *CMP_TY) k_compare(const float *__restrict__ W, int nz, int nx, int offset,
                                                            int r, int tiles_x, int tiles, double *__restrict__ part,
                                                            float *__restrict__ e_out) {
  const int mz = nz - 2 * r, mx = nx - 2 * r;
  const int pair = blockIdx.y, tile = blockIdx.x;
  const int xi = (tile % tiles_x) * CMP_TX + threadIdx.x;
  const int y0 = (tile / tiles_x) * CMP_TILE_Y + threadIdx.y * CMP_ROWS;
  const bool colok = xi < mx;
  const int x = r + min(xi, mx - 1);  // clamped into the interior: loads stay in the image
  const float *U = W + (size_t)pair * nz * nx;
  const float *V = W + (size_t)(pair + offset) * nz * nx;

  float u[CMP_ROWS], v[CMP_ROWS], m1[CMP_ROWS], m2[CMP_ROWS];
#pragma unroll
  for (int j = 0; j < CMP_ROWS; ++j) {
    const int y = r + min(y0 + j, mz - 1);
    u[j] = __ldg(U + (size_t)y * nx + x);
    v[j] = __ldg(V + (size_t)y * nx + x);
    m1[j] = __int_as_float(0x7f800000);
    m2[j] = __int_as_float(0x7f800000);
  }
  // every window row in the image (all warps but the bottom edge's) and the head
  // and tail apart: no clamping, no run-time row tests
  const bool fast = 2 * r >= CMP_ROWS - 1 && y0 + 2 * r + CMP_ROWS - 1 <= nz - 1;
  for (int l = -r; l <= r; ++l) {
    const float *pv = V + x + l;
    const float *pu = U + x + l;
    if (fast) {
      pv += (size_t)y0 * nx;
      pu += (size_t)y0 * nx;
#pragma unroll
      for (int t = 0; t < CMP_ROWS - 1; ++t)
        cmp_upd(m1, m2, u, v, __ldg(pv + t * nx), __ldg(pu + t * nx), 0, t);
      pv += (CMP_ROWS - 1) * nx;
      pu += (CMP_ROWS - 1) * nx;
#pragma unroll 2
      for (int t = CMP_ROWS - 1; t <= 2 * r; ++t) {
        cmp_upd(m1, m2, u, v, __ldg(pv), __ldg(pu), 0, CMP_ROWS - 1);
        pv += nx;
        pu += nx;
      }
#pragma unroll
      for (int t = 1; t < CMP_ROWS; ++t)
        cmp_upd(m1, m2, u, v, __ldg(pv + (t - 1) * nx), __ldg(pu + (t - 1) * nx), t, CMP_ROWS - 1);
    } else {
      for (int t = 0; t <= 2 * r + CMP_ROWS - 1; ++t) {
        const size_t row = (size_t)min(y0 + t, nz - 1);  // rows past the image serve only rows past the interior
        const float a = __ldg(pv + row * nx), b = __ldg(pu + row * nx);
#pragma unroll
        for (int j = 0; j < CMP_ROWS; ++j)
          if (t >= j && t - j <= 2 * r) {
            m1[j] = fminf(m1[j], fabsf(u[j] - a));
            m2[j] = fminf(m2[j], fabsf(v[j] - b));
          }
      }
    }
  }

  double s = 0.0;
#pragma unroll
  for (int j = 0; j < CMP_ROWS; ++j)
    if (colok && y0 + j < mz) {
      const float e = fmaxf(m1[j], m2[j]);
      s += (double)e;
      if (e_out) e_out[((size_t)pair * mz + (y0 + j)) * mx + xi] = e;
    }
#pragma unroll
  for (int o = 16; o; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  __shared__ double ws[CMP_TY];
  if (threadIdx.x == 0) ws[threadIdx.y] = s;
  __syncthreads();
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    double t = 0.0;
#pragma unroll
    for (int k = 0; k < CMP_TY; ++k) t += ws[k];
    part[(size_t)pair * tiles + tile] = t;
  }
}

__global__ void k_pair_sums(const double *__restrict__ part, int npairs, int tiles, double *__restrict__ err) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= npairs) return;
  double t = 0.0;
  for (int k = 0; k < tiles; ++k) t += part[(size_t)q * tiles + k];
  err[q] = t;
}

}  // namespace

namespace gt {
int set_error(int code, const char *msg);
int cuda_error(cudaError_t e, const char *what, int line);
}  // namespace gt

#define BAD_CK(expr, what)                                             \
  do {                                                                 \
    cudaError_t e_ = (expr);                                           \
    if (e_ != cudaSuccess) return gt::cuda_error(e_, what, __LINE__);   \
  } while (0)

extern "C" {

int gt_badproj_smooth(const double *data, int na, int nz, int nx, int steps, float *out, void *stream) {
  if (!data || !out || na < 1 || steps < 1 || nz <= 2 * steps || nx <= 2 * steps)
    return gt::set_error(GT_ERR_ARG, "gt_badproj_smooth: need steps >= 1 and nz, nx > 2 steps");
  const long long n = (long long)na * (nz - 2 * steps) * (nx - 2 * steps);
  k_smooth<<<nblk(n, 256), 256, 0, (cudaStream_t)stream>>>(data, na, nz, nx, steps, out);
  BAD_CK(cudaGetLastError(), "gt_badproj_smooth");
  return GT_OK;
}

int gt_badproj_wgrad(const float *u, int na, int nz, int nx, float *w, void *stream) {
  if (!u || !w || na < 1 || nz < 3 || nx < 3) return gt::set_error(GT_ERR_ARG, "gt_badproj_wgrad: need nz, nx >= 3");
  const long long n = (long long)na * (nz - 2) * (nx - 2);
  k_wgrad<<<nblk(n, 256), 256, 0, (cudaStream_t)stream>>>(u, na, nz, nx, w);
  BAD_CK(cudaGetLastError(), "gt_badproj_wgrad");
  return GT_OK;
}

int gt_badproj_blocks(int nz, int nx, int radius) {
  if (radius < 0 || nz - 2 * radius < 1 || nx - 2 * radius < 1) return 0;
  return ((nx - 2 * radius + CMP_TX - 1) / CMP_TX) * ((nz - 2 * radius + CMP_TILE_Y - 1) / CMP_TILE_Y);
}

int gt_badproj_compare(const float *w, int na, int nz, int nx, int offset, int radius, double *part, double *err,
                       float *e_out, void *stream) {
  if (!w || !part || !err || offset < 1 || na < 1)
    return gt::set_error(GT_ERR_ARG, "gt_badproj_compare: bad argument");
  const int tiles = gt_badproj_blocks(nz, nx, radius);
  if (tiles == 0) return gt::set_error(GT_ERR_ARG, "gt_badproj_compare: radius leaves no interior pixel");
  const int npairs = na - offset;
  if (npairs <= 0) return GT_OK;
  if (npairs > 65535) return gt::set_error(GT_ERR_ARG, "gt_badproj_compare: more than 65535 pairs");
  const int tiles_x = (nx - 2 * radius + CMP_TX - 1) / CMP_TX;
  k_compare<<<dim3(tiles, npairs), dim3(CMP_TX, CMP_TY), 0, (cudaStream_t)stream>>>(w, nz, nx, offset, radius, tiles_x,
                                                                                    tiles, part, e_out);
  BAD_CK(cudaGetLastError(), "gt_badproj_compare");
  k_pair_sums<<<nblk(npairs, 128), 128, 0, (cudaStream_t)stream>>>(part, npairs, tiles, err);
  BAD_CK(cudaGetLastError(), "gt_badproj_compare (sums)");
  return GT_OK;
}

}  // extern "C"
