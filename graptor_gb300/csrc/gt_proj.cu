// Register-blocked back projector of the solver iteration (sm_103a).
//
// The back-projection kernels of gt_kernels.cu give each warp one pixel and S
// slice values per lane group; both interpolation taps of every (pixel, angle)
// pair are loaded from L1 for that pixel alone, one load per two multiply-adds.
// Here (k_bp_row, back projection `radon_ad`, radon_tgv_primal_dual_3d.py:818-844)
// a warp owns 4 adjacent pixels of a row: per angle their taps lie on at most 5
// consecutive detector bins, loaded once and shared, so the L1 traffic halves.
//
// The geometry is fixed for a solve, so it is computed once per problem into a
// table with the reference's arithmetic.  Which accumulator a product goes to must
// be known at compile time (registers cannot be indexed at run time): the lower
// bins of 4 adjacent pixels of a row step by 0 or 1 (the detector coordinate
// moves by |cos| <= 1 per pixel), one of 8 step patterns per direction, and the
// kernel branches once per angle on the pattern.  Every pixel adds its two taps
// in the reference's order with the reference's weights (fused multiply-add, as
// the solver's other projector shapes); where a tap falls outside the detector
// the entry pairs the pixel with a zero weight on a bin inside it, and a zero
// product leaves a sum unchanged, so the iterates are identical to those of the
// other back-projection shapes.
#include <cuda_runtime.h>

#include <climits>

#include "gt_common.cuh"
#include "gt_geom.cuh"

namespace gt {

namespace {

constexpr int ROW_P = 4;            // pixels per back-projection row tile
constexpr int ROW_NB = ROW_P + 1;   // most consecutive bins their taps span
constexpr int ROW_WORDS = 3;        // int4 per (row tile, angle) entry

inline unsigned blocks(long long threads, int bs) { return (unsigned)((threads + bs - 1) / bs); }

// ---------------------------------------------------------------------------
// row-tile table
// ---------------------------------------------------------------------------
// Entry of the row tile (x0 .. x0 + 3, y) and angle o, ROW_WORDS int4:
// (b0, nb, pattern, 0), the lower-tap weights of its 4 pixels, the upper-tap
// weights.  Per pixel radon_ad's detector coordinate t = x X + y Y + off, lower
// bin floor(t) and fraction p (:832-839); taps (floor(t), 1 - p), (floor(t) + 1, p).
// The reference drops the lower tap at bin -1 and the upper tap at bin nd; the
// entry pairs the remaining tap with a zero-weight tap on the detector instead
// ((0, p; 1, 0) and (nd - 2, 0; nd - 1, 1 - p)), so every tap lies in [0, nd - 1].
// A pixel outside (-1, nd) or outside the image adds nothing: it takes the lower
// bin of its nearest pixel that does (t is monotone along the row, so such pixels
// are at the ends) with zero weights.  The lower bins lo_0..lo_3 then step by 0
// or 1 in one direction: pattern = dir * 8 + steps (bit r: step between pixels r
// and r + 1, dir 0: lo_r non-decreasing from lo_0 = b0, dir 1: non-increasing to
// lo_3 = b0).  Returns nb (taps b0 .. b0 + nb - 1), or -1 when the steps are not
// of that form (the tile kernel is then not used).
__device__ int row_entry(const float4 o, int x0, int y, int N, int nd, int4 *out) {
  int lo[ROW_P];
  float wl[ROW_P], wh[ROW_P];
  bool in[ROW_P];
  int first = -1, last = -1;
#pragma unroll
  for (int r = 0; r < ROW_P; ++r) {
    const int x = x0 + r;
    in[r] = false;
    lo[r] = 0;
    wl[r] = wh[r] = 0.f;
    if (x >= N || y >= N) continue;
    const float tt = __fadd_rn(__fadd_rn(__fmul_rn((float)x, o.x), __fmul_rn((float)y, o.y)), o.z);
    if (!(tt > -1.f && tt < (float)nd)) continue;
    const float fl = floorf(tt);
    const float p = fminf(__fsub_rn(tt, fl), 0x1.fffffep-1f);
    const float q = __fsub_rn(1.0f, p);
    int il = (int)fl;
    float a = q, b = p;
    if (il < 0) { il = 0; a = p; b = 0.f; }                  // only the upper tap, at bin 0
    else if (il > nd - 2) { il = nd - 2; a = 0.f; b = q; }   // only the lower tap, at bin nd - 1
    in[r] = true;
    lo[r] = il;
    wl[r] = a;
    wh[r] = b;
    if (first < 0) first = r;
    last = r;
  }
  int nb = 0, b0 = 0, pattern = 0;
  if (first >= 0) {
    for (int r = first - 1; r >= 0; --r) lo[r] = lo[r + 1];
    for (int r = last + 1; r < ROW_P; ++r) lo[r] = lo[r - 1];
    for (int r = first + 1; r <= last; ++r)
      if (!in[r]) return -1;  // not expected: t is monotone along the row
    bool up = true, down = true;
#pragma unroll
    for (int r = 0; r + 1 < ROW_P; ++r) {
      const int dlt = lo[r + 1] - lo[r];
      up = up && (dlt == 0 || dlt == 1);
      down = down && (dlt == 0 || dlt == -1);
    }
    if (!up && !down) return -1;
    const int dir = up ? 0 : 1;
#pragma unroll
    for (int r = 0; r + 1 < ROW_P; ++r) pattern |= (lo[r + 1] != lo[r]) << r;
    pattern |= dir << 3;
    b0 = up ? lo[0] : lo[ROW_P - 1];
    nb = (up ? lo[ROW_P - 1] : lo[0]) + 2 - b0;
  }
  out[0] = make_int4(b0, nb, pattern, 0);
  out[1] = make_int4(__float_as_int(wl[0]), __float_as_int(wl[1]), __float_as_int(wl[2]), __float_as_int(wl[3]));
  out[2] = make_int4(__float_as_int(wh[0]), __float_as_int(wh[1]), __float_as_int(wh[2]), __float_as_int(wh[3]));
  return nb;
}

// one thread per (row tile, angle); *bad is set when an entry cannot be formed
__global__ void k_row_fill(const float4 *__restrict__ ofs, int N, int nd, int nang, int4 *__restrict__ tab,
                           int *__restrict__ bad) {
  const int ntx = (N + ROW_P - 1) / ROW_P;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)ntx * N * nang) return;
  const long long tile = t / nang;
  const int j = (int)(t - tile * nang);
  const int y = (int)(tile / ntx), tx = (int)(tile - (long long)y * ntx);
  if (row_entry(__ldg(ofs + j), tx * ROW_P, y, N, nd, tab + t * ROW_WORDS) < 0) atomicExch(bad, 1);
}

// ---------------------------------------------------------------------------
// slice block of a lane: VW consecutive slices from s0 (VW = 4: one float4,
// VW = 2: one float2)
// ---------------------------------------------------------------------------
template <int VW>
__device__ __forceinline__ void st_slices(float *p, const float (&r)[VW]) {
  if (VW == 4) *reinterpret_cast<float4 *>(p) = make_float4(r[0], r[1 % VW], r[2 % VW], r[3 % VW]);
  else *reinterpret_cast<float2 *>(p) = make_float2(r[0], r[1 % VW]);
}

template <int VW>
__device__ __forceinline__ void fma2(float (&acc)[VW], float w, const float (&v)[VW]) {
#pragma unroll
  for (int s = 0; s < VW; ++s) acc[s] = __fmaf_rn(w, v[s], acc[s]);
}

// unpredicated load of VW slices (the caller clamps the address into the field)
template <int VW>
__device__ __forceinline__ void ld_any(const float *p, float (&r)[VW]) {
  if (VW == 4) {
    const float4 a = __ldg(reinterpret_cast<const float4 *>(p));
    r[0] = a.x; r[1 % VW] = a.y; r[2 % VW] = a.z; r[3 % VW] = a.w;
  } else {
    const float2 a = __ldg(reinterpret_cast<const float2 *>(p));
    r[0] = a.x; r[1 % VW] = a.y;
  }
}

// ---------------------------------------------------------------------------
// k_bp_row: a block's 8 warps own 2 x 4 row tiles of one slice block (an 8 x 4
// pixel region), so the taps they load for an angle overlap in L1.
// ---------------------------------------------------------------------------
// pixel r's lower tap for pattern PAT (see row_entry)
template <int PAT, int R>
struct RowTap {
  static constexpr int step(int r) { return (PAT >> r) & 1; }
  static constexpr int up_k(int r) { return r == 0 ? 0 : up_k(r - 1) + step(r - 1); }
  static constexpr int down_k(int r) { return r == ROW_P - 1 ? 0 : down_k(r + 1) + step(r); }
  static constexpr int k = (PAT & 8) ? down_k(R) : up_k(R);
};

template <int PAT, int VW>
__device__ __forceinline__ void row_apply(float (&acc)[ROW_P][VW], const float (&T)[ROW_NB][VW],
                                          const float (&wl)[ROW_P], const float (&wh)[ROW_P]) {
  fma2<VW>(acc[0], wl[0], T[RowTap<PAT, 0>::k]);
  fma2<VW>(acc[0], wh[0], T[RowTap<PAT, 0>::k + 1]);
  fma2<VW>(acc[1], wl[1], T[RowTap<PAT, 1>::k]);
  fma2<VW>(acc[1], wh[1], T[RowTap<PAT, 1>::k + 1]);
  fma2<VW>(acc[2], wl[2], T[RowTap<PAT, 2>::k]);
  fma2<VW>(acc[2], wh[2], T[RowTap<PAT, 2>::k + 1]);
  fma2<VW>(acc[3], wl[3], T[RowTap<PAT, 3>::k]);
  fma2<VW>(acc[3], wh[3], T[RowTap<PAT, 3>::k + 1]);
}

template <int VW>
__global__ void __launch_bounds__(256) k_bp_row(const IterParams P) {
  static_assert(ROW_P == 4, "row_apply handles 4 pixels");
  const Dims d = P.d;
  const int ntx = (d.N + ROW_P - 1) / ROW_P;
  const int warp = threadIdx.x >> 5;
  const int tx = blockIdx.x * 2 + (warp & 1), y = blockIdx.y * 4 + (warp >> 1);
  if (tx >= ntx || y >= d.N) return;
  const int s0 = blockIdx.z * 32 * VW + (int)(threadIdx.x & 31) * VW;
  const size_t S = d.S;
  const size_t jstride = (size_t)d.nd * S;
  const int4 *__restrict__ ent = P.row_ent + ((size_t)y * ntx + tx) * d.nang * ROW_WORDS;
  // lanes past S read the last slices (their sums are not stored)
  const float *__restrict__ lam = P.lam + min(s0, d.S - VW);

  float acc[ROW_P][VW];
#pragma unroll
  for (int r = 0; r < ROW_P; ++r)
#pragma unroll
    for (int s = 0; s < VW; ++s) acc[r][s] = 0.f;

  for (int j = 0; j < d.nang; ++j, ent += ROW_WORDS) {
    const int4 h = __ldg(ent);
    const int nb = h.y;
    if (nb == 0) continue;
    const int4 la = __ldg(ent + 1), ha = __ldg(ent + 2);
    const float wl[ROW_P] = {__int_as_float(la.x), __int_as_float(la.y), __int_as_float(la.z), __int_as_float(la.w)};
    const float wh[ROW_P] = {__int_as_float(ha.x), __int_as_float(ha.y), __int_as_float(ha.z), __int_as_float(ha.w)};
    const float *lj = lam + (size_t)j * jstride + (size_t)h.x * S;
    // taps past the tile's last bin re-read that bin (never used by the pattern)
    float T[ROW_NB][VW];
#pragma unroll
    for (int m = 0; m < ROW_NB; ++m) ld_any<VW>(lj + (size_t)min(m, nb - 1) * S, T[m]);
    switch (h.z) {
#define GT_ROW_CASE(c) \
  case c: row_apply<c, VW>(acc, T, wl, wh); break;
      GT_ROW_CASE(0) GT_ROW_CASE(1) GT_ROW_CASE(2) GT_ROW_CASE(3) GT_ROW_CASE(4) GT_ROW_CASE(5)
      GT_ROW_CASE(6) GT_ROW_CASE(7) GT_ROW_CASE(8) GT_ROW_CASE(9) GT_ROW_CASE(10) GT_ROW_CASE(11)
      GT_ROW_CASE(12) GT_ROW_CASE(13) GT_ROW_CASE(14) GT_ROW_CASE(15)
#undef GT_ROW_CASE
      default: break;
    }
  }
  if (s0 >= d.S) return;
#pragma unroll
  for (int r = 0; r < ROW_P; ++r) {
    const int x = tx * ROW_P + r;
    if (x < d.N) st_slices<VW>(P.kstar + ((size_t)y * d.N + x) * S + s0, acc[r]);
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
size_t row_table_bytes(int N, int nang) {
  return sizeof(int4) * ROW_WORDS * (size_t)((N + ROW_P - 1) / ROW_P) * N * nang;
}

cudaError_t launch_row_fill(const float4 *ofs, int N, int nd, int nang, int4 *tab, int *bad, cudaStream_t st) {
  const long long n = (long long)((N + ROW_P - 1) / ROW_P) * N * nang;
  k_row_fill<<<blocks(n, 128), 128, 0, st>>>(ofs, N, nd, nang, tab, bad);
  return cudaGetLastError();
}

// shape 0: 4 slices per lane; 1: 2 slices per lane
cudaError_t launch_bp_row(const IterParams &P, int shape, cudaStream_t st) {
  const int ntx = (P.d.N + ROW_P - 1) / ROW_P;
  const int vw = shape == 1 ? 2 : 4;
  const dim3 grid((ntx + 1) / 2, (P.d.N + 3) / 4, (P.d.S + 32 * vw - 1) / (32 * vw));
  if (vw == 4) k_bp_row<4><<<grid, 256, 0, st>>>(P);
  else k_bp_row<2><<<grid, 256, 0, st>>>(P);
  return cudaGetLastError();
}

}  // namespace gt
