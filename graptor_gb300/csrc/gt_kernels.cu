// GB300 kernels of the primal-dual TGV/TV reconstruction (sm_103a).
//
// One iteration of the reference loop (radon_tgv_primal_dual_3d.py:1194-1221:
// update_v, update_w, NormV, NormW, radon, update_lambda, radon_ad, update_u,
// update_p, two extrapolations) runs here as four kernels:
//
//   k_dual    update_v + update_w + the coupled ball projections of v and w
//             (one pass over ubar, pbar, v, w; writes v, w)
//   k_fwd     forward projection `radon` of ubar fused with the data-term prox
//             update_lambda (reads ubar, f, lambda; writes lambda and K ubar)
//   k_bp      back projection `radon_ad` of lambda (writes K* lambda)
//   k_update  update_u, update_p and both extrapolations (reads u, p, v, w,
//             K* lambda; writes u, ubar, p, pbar)
//
// k_dual and the chain k_fwd -> k_bp read only what the previous k_update wrote
// and write disjoint fields, so they run concurrently.
#include <cuda_runtime.h>
#include <algorithm>
#include <climits>
#include <type_traits>
#include <math.h>
#include <cmath>

#include "gt_common.cuh"
#include "gt_geom.cuh"
#include "gt_tma.cuh"

namespace gt {

// ===========================================================================
// ball projections
// ===========================================================================

// The nuclear-norm projections evaluate eigenvectors by formulas that cancel
// catastrophically when the off-diagonal entry is small, so their results depend
// on rounding: they are written with explicitly rounded operations (no fused
// multiply-add), in the reference's order, and with hypot / atan / cos / cube
// evaluated in double and rounded once (as the host C library's float versions
// are, to within their last bit).
__device__ __forceinline__ float fm(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fa(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fs(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float hyp(float a, float b) { return (float)sqrt((double)a * a + (double)b * b); }

// nuclear 2-D (update_NormV_Nucl, radon_tgv_primal_dual_2d.py:124-204): spectral
// projection of the C x 2 matrix A of one pixel via the 2x2 matrix A^T A = [a b; b c].
__device__ __forceinline__ void nucl2d_matrix(float a, float b, float c, float ainv, float M[3]) {
  const float eps = 0.00001f;
  float s1, s2, S1, S2;
  const float o = c < a ? c : a;
  if (fm(b, b) / fm(o, o) > eps && fm(o, o) > 0.f) {
    const float dd = fa(a, c), e = fs(a, c);
    float f = fa(fm(fm(4.f, b), b), fm(e, e));
    f = f < 0.f ? 0.f : sqrtf(f);
    s2 = (fs(dd, f) > 0.f) ? sqrtf(fm(fs(dd, f), 0.5f)) : 0.f;
    s1 = (fa(dd, f) > 0.f) ? sqrtf(fm(fa(dd, f), 0.5f)) : 0.f;
    const float g = fm(fa(e, f), 0.5f), h = fm(fs(e, f), 0.5f);
    float q0 = fa(fm(g, a), fm(b, b)), q1 = fa(fm(g, b), fm(c, b));
    float q2 = fa(fm(h, a), fm(b, b)), q3 = fa(fm(h, b), fm(b, c));
    const float n1 = hyp(q0, q1), n2 = hyp(q2, q3);
    if (n1 > 0.f) { q0 = q0 / n1; q1 = q1 / n1; }
    if (n2 > 0.f) { q2 = q2 / n2; q3 = q3 / n2; }
    S1 = (fm(s1, ainv) > 1.f) ? 1.f / fm(s1, ainv) : 1.f;
    S2 = (fm(s2, ainv) > 1.f) ? 1.f / fm(s2, ainv) : 1.f;
    M[0] = fa(fm(fm(q0, q0), S1), fm(fm(q2, q2), S2));
    M[2] = fa(fm(fm(q1, q1), S1), fm(fm(q3, q3), S2));
    M[1] = fa(fm(fm(S1, q0), q1), fm(fm(S2, q2), q3));
  } else {
    s1 = sqrtf(a);
    s2 = sqrtf(c);
    S1 = (fm(ainv, s1) > 1.f) ? 1.f / fm(ainv, s1) : 1.f;
    S2 = (fm(ainv, s2) > 1.f) ? 1.f / fm(ainv, s2) : 1.f;
    M[0] = S1; M[2] = S2; M[1] = 0.f;
  }
}

// nuclear 3-D helpers (radon_tgv_primal_dual_3d.py:190-284), results by value
__device__ __forceinline__ void diag2d(float a, float b, float c, float X[6]) {
  const float eps = 0.001f;
  const float o = c < a ? c : a;
  if (fm(b, b) / fm(o, o) > eps && fm(o, o) > 0.f) {
    const float dd = fa(a, c), e = fs(a, c);
    float f = fa(fm(fm(4.f, b), b), fm(e, e));
    f = f < 0.f ? 0.f : sqrtf(f);
    X[1] = (fs(dd, f) > 0.f) ? fm(fs(dd, f), 0.5f) : 0.f;
    X[0] = (fa(dd, f) > 0.f) ? fm(fa(dd, f), 0.5f) : 0.f;
    const float h = fm(fs(e, f), 0.5f);
    float v0 = 1.f, v1 = -h / b;
    const float n1 = hyp(v0, v1);
    v0 = v0 / n1; v1 = v1 / n1;
    X[2] = v0; X[3] = v1; X[4] = v1; X[5] = -v0;
  } else {
    X[0] = a; X[1] = c; X[2] = 1.f; X[3] = 0.f; X[4] = 0.f; X[5] = -1.f;
  }
}

__device__ __forceinline__ void eig3d(float a, float b, float c, float d, float e, float f, float out[3]) {
  const float pi = (float)3.14159265359;
  float c2 = -fa(fa(a, b), c);
  const float c1 = fs(fs(fs(fa(fa(fm(a, b), fm(a, c)), fm(b, c)), fm(d, d)), fm(e, e)), fm(f, f));
  const float c0 = fs(fs(fa(fa(fm(fm(a, f), f), fm(fm(b, e), e)), fm(fm(c, d), d)), fm(fm(a, b), c)),
                      fm(fm(fm(2.f, d), e), f));
  float p = (float)((double)fm(c2, c2) - 3.0 * (double)c1);
  const float cube = (float)((double)c2 * c2 * c2);
  const float q = fa(fs(fm(-13.5f, c0), cube), fm(fm(4.5f, c2), c1));
  const float inner = fm(27.f, fa(fm(fm(fm(0.25f, c1), c1), fs(p, c1)), fm(c0, fa(q, fm(6.75f, c0)))));
  float phi = fm(1.f / 3.f, (float)atan((double)(sqrtf(inner) / q)));
  if (q < 0.f) phi = fa(phi, pi / 3.f);
  const float x1 = fm(2.f, (float)cos((double)phi));
  const float x2 = fm(2.f, (float)cos((double)fa(phi, fm(2.f, pi) / 3.f)));
  const float x3 = fm(2.f, (float)cos((double)fs(phi, fm(2.f, pi) / 3.f)));
  p = sqrtf(p) / 3.f;
  c2 = c2 / 3.f;
  out[0] = fs(fm(p, x1), c2); out[1] = fs(fm(p, x2), c2); out[2] = fs(fm(p, x3), c2);
}

__device__ __forceinline__ void cross3(float a1, float a2, float a3, float b1, float b2, float b3, float o[3]) {
  o[0] = fs(fm(a2, b3), fm(a3, b2));
  o[1] = fs(fm(b1, a3), fm(a1, b3));
  o[2] = fs(fm(a1, b2), fm(a2, b1));
}

__device__ __forceinline__ float norm3(const float v[3]) { return sqrtf(fa(fa(fm(v[0], v[0]), fm(v[1], v[1])), fm(v[2], v[2]))); }

// nuclear 3-D (update_NormV_Nucl, radon_tgv_primal_dual_3d.py:290-520): returns the
// symmetric 3x3 projection matrix M (xx, yy, zz, xy, xz, yz) applied to every channel,
// for A^T A = [a r t; r b d; t d c].
__device__ void nucl3d_matrix(float a, float b, float c, float r, float t, float d, float ainv, float M[6]) {
  const float epsdt = 0.0001f, epsr = 0.0001f, epsoo = 0.0001f / ainv;
  const float ndt = fa(fm(d, d), fm(t, t));
  float oo = b < a ? b : a;
  float sig[3], v0[3], v1[3], v2[3], X[6], u1 = 1.f, u2 = 0.f;
  if (ndt < fm(fm(epsdt, oo), oo) && oo > epsoo) {
    diag2d(a, r, b, X);
    sig[0] = X[0]; sig[1] = X[1];
    sig[2] = (fm(c, c) < ndt) ? 1.f / epsdt : c;
    v0[0] = X[2]; v0[1] = X[3]; v0[2] = 0.f;
    v1[0] = X[4]; v1[1] = X[5]; v1[2] = 0.f;
    v2[0] = 0.f; v2[1] = 0.f; v2[2] = 1.f;
  } else if (oo < epsoo) {
    if (a >= b) {
      sig[0] = b; v0[0] = 0.f; v0[1] = 1.f; v0[2] = 0.f;
      diag2d(a, t, c, X);
      sig[1] = X[0]; sig[2] = X[1];
      v1[0] = X[2]; v1[1] = 0.f; v1[2] = X[3];
      v2[0] = X[4]; v2[1] = 0.f; v2[2] = X[5];
    } else {
      sig[0] = a; v0[0] = 1.f; v0[1] = 0.f; v0[2] = 0.f;
      diag2d(b, d, c, X);
      sig[1] = X[0]; sig[2] = X[1];
      v1[0] = 0.f; v1[1] = X[2]; v1[2] = X[3];
      v2[0] = 0.f; v2[1] = X[4]; v2[2] = X[5];
    }
  } else {
    // rotate about z so that the (x, z) entry vanishes (3-D :434-452)
    const float t1 = fs(fm(b, t), fm(d, r)), t2 = fs(fm(a, d), fm(t, r));
    u1 = d / sqrtf(ndt);
    u2 = t / sqrtf(ndt);
    const float bn = fa(fm(d, fa(fm(b, d), fm(r, t))), fm(t, fa(fm(a, t), fm(d, r)))) / ndt;
    const float an = fa(fm(t, t1), fm(d, t2)) / ndt;
    const float rn = fa(fm(-d, t1), fm(t, t2)) / ndt;
    const float dn = sqrtf(ndt);
    oo = bn < c ? bn : c;
    if (fabsf(rn) < fm(epsr, oo)) {
      diag2d(bn, dn, c, X);
      sig[0] = an; sig[1] = X[0]; sig[2] = X[1];
      v0[0] = 1.f; v0[1] = 0.f; v0[2] = 0.f;
      v1[0] = 0.f; v1[1] = X[2]; v1[2] = X[3];
      v2[0] = 0.f; v2[1] = X[4]; v2[2] = X[5];
    } else {
      eig3d(an, bn, c, rn, 0.f, dn, sig);
      cross3(fs(an, sig[0]), rn, 0.f, rn, fs(bn, sig[0]), dn, v0);
      float n = norm3(v0);
      v0[0] /= n; v0[1] /= n; v0[2] /= n;
      cross3(v0[0], v0[1], v0[2], 0.f, dn, fs(c, sig[1]), v1);
      n = norm3(v1);
      v1[0] /= n; v1[1] /= n; v1[2] /= n;
      cross3(v0[0], v0[1], v0[2], v1[0], v1[1], v1[2], v2);
      n = norm3(v2);
      v2[0] /= n; v2[1] /= n; v2[2] /= n;
    }
  }
  // eigenvectors back in the original frame (:476-479)
  float w[3][3];
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    const float *vv = m == 0 ? v0 : (m == 1 ? v1 : v2);
    w[m][0] = fa(fm(u1, vv[0]), fm(u2, vv[1]));
    w[m][1] = fa(fm(-u2, vv[0]), fm(u1, vv[1]));
    w[m][2] = vv[2];
  }
  float S[3];
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    const float sg = sig[m] > 0.f ? sqrtf(sig[m]) : 0.f;
    S[m] = (fm(sg, ainv) > 1.f) ? 1.f / fm(ainv, sg) : 1.f;
  }
  // M = W diag(S) W^T (:500-507)
  const int ii[6] = {0, 1, 2, 0, 0, 1}, jj[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
  for (int q = 0; q < 6; ++q)
    M[q] = fa(fa(fm(fm(S[0], w[0][ii[q]]), w[0][jj[q]]), fm(fm(S[1], w[1][ii[q]]), w[1][jj[q]])),
              fm(fm(S[2], w[2][ii[q]]), w[2][jj[q]]));
}

// squared norm of one channel's w in the reference's weighting:
//  3-D Frobenius  w0^2+w1^2+w2^2+(1.4142 w3)^2+1.4142^2 (w4^2+w5^2)   (3-D :583)
//  3-D uncorr.    w0^2+w1^2+w2^2+(1.4142 w3)^2+(1.4142 w4)^2+w5^2      (3-D :603)
//  2-D Frobenius  w0^2+w1^2+(2 w2)^2                                    (2-D :232)
//  2-D uncorr.    w0^2+w1^2+(1.4142 w2)^2                               (2-D :254)
template <int DIM, int CPL>
__device__ __forceinline__ float wnorm2(const float *w) {
  if (DIM == 3) {
    const float q3 = 1.4142f * w[3], q4 = 1.4142f * w[4];
    const float q5 = (CPL == UNCORR) ? w[5] : 1.4142f * w[5];
    return w[0] * w[0] + w[1] * w[1] + w[2] * w[2] + q3 * q3 + q4 * q4 + q5 * q5;
  } else {
    const float q2 = (CPL == UNCORR) ? 1.4142f * w[2] : 2.f * w[2];
    return w[0] * w[0] + w[1] * w[1] + q2 * q2;
  }
}

// One component of update_p (3-D :734-757) at one voxel-slice: the divergence of
// the symmetric tensor w by forward differences (wa, wb, wc the row's entries at the
// voxel, wan, wbn, wcn at its x / y / z successor; fx, fy, fz: first pixel / row /
// slice, hx, hy, hz: a successor exists), then p + tau (v + div w).  k_update and the
// fused dual kernel both compute p through this function, by the same operations.
__device__ __forceinline__ float p_step3(float po, float vk, float wa, float wan, float wb, float wbn, float wc,
                                         float wcn, bool fx, bool hx, bool fy, bool hy, bool fz, bool hz, float tau,
                                         float stepsize) {
  float A = -wa, B = -wb, Cz = -wc;
  if (fx) A = 0.f;
  if (hx) A += wan;
  if (fy) B = 0.f;
  if (hy) B += wbn;
  if (fz) Cz = 0.f;
  if (hz) Cz += wcn;
  Cz /= stepsize;
  return po + tau * (vk + A + B + Cz);
}

// projections of the dual variables onto the norm balls (NormV / NormW of the
// coupling): vv, ww of the nC channels of one voxel, in place.
template <int DIM, bool TGV, int CPL, int CMAX>
__device__ __forceinline__ void dual_project(const IterParams &P, const int nC, float (&vv)[CMAX][DIM],
                                             float (&ww)[CMAX][DIM == 3 ? 6 : 3]) {
  constexpr int K = DIM, KW = DIM == 3 ? 6 : 3;
  if (CPL == UNCORR) {
#pragma unroll
    for (int c = 0; c < CMAX; ++c) {
      if (c >= nC) break;
      float n2 = 0.f;
#pragma unroll
      for (int k = 0; k < K; ++k) n2 += vv[c][k] * vv[c][k];
      const float nv = sqrtf(n2) * P.ainv1;
      if (nv > 1.f) {
#pragma unroll
        for (int k = 0; k < K; ++k) vv[c][k] = vv[c][k] / nv;
      }
      if (TGV) {
        const float nw = sqrtf(wnorm2<DIM, UNCORR>(ww[c])) * P.ainv0;
        if (nw > 1.f) {
#pragma unroll
          for (int k = 0; k < KW; ++k) ww[c][k] = ww[c][k] / nw;
        }
      }
    }
  } else {
    if (CPL == FROB) {
      float n2 = 0.f;
#pragma unroll
      for (int c = 0; c < CMAX; ++c) {
        if (c >= nC) break;
#pragma unroll
        for (int k = 0; k < K; ++k) n2 += vv[c][k] * vv[c][k];
      }
      const float nv = sqrtf(n2) * P.ainv1;
      if (nv > 1.f) {
#pragma unroll
        for (int c = 0; c < CMAX; ++c) {
          if (c >= nC) break;
#pragma unroll
          for (int k = 0; k < K; ++k) vv[c][k] = vv[c][k] / nv;
        }
      }
    } else {  // NUCL: spectral projection of the C x K matrix
      if (DIM == 2) {
        float a = 0.f, b = 0.f, cc = 0.f;
#pragma unroll
        for (int c = 0; c < CMAX; ++c) {
          if (c >= nC) break;
          a = fa(a, fm(vv[c][0], vv[c][0])); b = fa(b, fm(vv[c][0], vv[c][1])); cc = fa(cc, fm(vv[c][1], vv[c][1]));
        }
        float M[3];
        nucl2d_matrix(a, b, cc, P.ainv1, M);
#pragma unroll
        for (int c = 0; c < CMAX; ++c) {
          if (c >= nC) break;
          const float v0 = vv[c][0], v1 = vv[c][1];
          vv[c][0] = fa(fm(v0, M[0]), fm(v1, M[1]));
          vv[c][1] = fa(fm(v0, M[1]), fm(v1, M[2]));
        }
      } else {
        float a = 0.f, b = 0.f, cc = 0.f, r = 0.f, tt = 0.f, dd = 0.f;
#pragma unroll
        for (int c = 0; c < CMAX; ++c) {
          if (c >= nC) break;
          const float X = vv[c][0], Y = vv[c][1], Z = vv[c][DIM - 1];
          a = fa(a, fm(X, X)); b = fa(b, fm(Y, Y)); cc = fa(cc, fm(Z, Z));
          r = fa(r, fm(X, Y)); tt = fa(tt, fm(X, Z)); dd = fa(dd, fm(Y, Z));
        }
        float M[6];
        nucl3d_matrix(a, b, cc, r, tt, dd, P.ainv1, M);
#pragma unroll
        for (int c = 0; c < CMAX; ++c) {
          if (c >= nC) break;
          const float A = vv[c][0], B = vv[c][1], Cc = vv[c][DIM - 1];
          vv[c][0] = fa(fa(fm(A, M[0]), fm(B, M[3])), fm(Cc, M[4]));
          vv[c][1] = fa(fa(fm(A, M[3]), fm(B, M[1])), fm(Cc, M[5]));
          vv[c][DIM - 1] = fa(fa(fm(A, M[4]), fm(B, M[5])), fm(Cc, M[2]));
        }
      }
    }
    if (TGV) {  // w: Frobenius coupling for both FROB and NUCL (3-D :1118-1124)
      float n2 = 0.f;
#pragma unroll
      for (int c = 0; c < CMAX; ++c) {
        if (c >= nC) break;
        n2 += wnorm2<DIM, FROB>(ww[c]);
      }
      const float nw = sqrtf(n2) * P.ainv0;
      if (nw > 1.f) {
#pragma unroll
        for (int c = 0; c < CMAX; ++c) {
          if (c >= nC) break;
#pragma unroll
          for (int k = 0; k < KW; ++k) ww[c][k] = ww[c][k] / nw;
        }
      }
    }
  }

}

// ===========================================================================
// k_dual: update_v (3-D :615-634, 2-D :265-284), update_w (3-D :637-660,
// 2-D :286-304), NormV / NormW (3-D :290-610, 2-D :98-258)
// thread = one (pixel, z); it owns all C channels of that voxel.
// ===========================================================================
template <int DIM, bool TGV, int CPL, int CMAX>
__device__ __forceinline__ void dual_body(const IterParams &P, long long bid) {
  constexpr int K = DIM, KW = DIM == 3 ? 6 : 3;
  const Dims d = P.d;
  const long long t = bid * blockDim.x + threadIdx.x;
  if (t >= (long long)d.N * d.N * d.Nz) return;
  const int pix = (int)(t / d.Nz);
  const int z = (int)(t - (long long)pix * d.Nz);
  const int y = pix / d.N, x = pix - y * d.N;
  const size_t vol = d.vol, S = d.S, rowS = (size_t)d.N * S;
  const float sigma = P.sigma;
  const float *__restrict__ ub = P.ubar;
  const float *__restrict__ pb = P.pbar;
  const int nC = min(CMAX, d.C - P.cbase);  // channels of this launch (channel groups for uncorrelated C > 8)

  float vv[CMAX][K], ww[CMAX][KW];
#pragma unroll
  for (int c = 0; c < CMAX; ++c) {
    if (c >= nC) break;
    const size_t i = (size_t)pix * S + (size_t)(P.cbase + c) * d.Nz + z;
    // gradient of ubar: forward differences, zero at the last index
    const float mu = -ub[i];
    float g[3];
    g[0] = (x < d.N - 1) ? mu + ub[i + S] : 0.f;
    g[1] = (y < d.N - 1) ? mu + ub[i + rowS] : 0.f;
    if (DIM == 3) g[2] = ((z < d.Nz - 1) ? mu + ub[i + 1] : 0.f) / P.stepsize;
    float pc[3];
#pragma unroll
    for (int k = 0; k < K; ++k) {
      pc[k] = TGV ? pb[k * vol + i] : 0.f;
      vv[c][k] = P.v[k * vol + i] + sigma * (g[k] - pc[k]);
    }
    if (TGV) {
      // symmetrised gradient of pbar: backward differences, zero at index 0
      float a[3], b[3], cz[3];
#pragma unroll
      for (int k = 0; k < K; ++k) {
        a[k] = x > 0 ? pc[k] - pb[k * vol + i - S] : 0.f;
        b[k] = y > 0 ? pc[k] - pb[k * vol + i - rowS] : 0.f;
        if (DIM == 3) cz[k] = (z > 0 ? pc[k] - pb[k * vol + i - 1] : 0.f) / P.stepsize;
      }
      float e[6];
      if (DIM == 3) {
        e[0] = a[0]; e[1] = b[1]; e[2] = cz[2];
        e[3] = 0.5f * (a[1] + b[0]);
        e[4] = 0.5f * (a[2] + cz[0]);
        e[5] = 0.5f * (b[2] + cz[1]);
      } else {
        e[0] = a[0]; e[1] = b[1];
        e[2] = 0.5f * (a[1] + b[0]);
      }
#pragma unroll
      for (int k = 0; k < KW; ++k) ww[c][k] = P.w[k * vol + i] + sigma * e[k];
    }
  }

  dual_project<DIM, TGV, CPL, CMAX>(P, nC, vv, ww);

  // ---- store
#pragma unroll
  for (int c = 0; c < CMAX; ++c) {
    if (c >= nC) break;
    const size_t i = (size_t)pix * S + (size_t)(P.cbase + c) * d.Nz + z;
#pragma unroll
    for (int k = 0; k < K; ++k) P.v[k * vol + i] = vv[c][k];
    if (TGV) {
#pragma unroll
      for (int k = 0; k < KW; ++k) P.w[k * vol + i] = ww[c][k];
    }
  }
}

template <int DIM, bool TGV, int CPL, int CMAX, int MINB = 1>
__global__ void __launch_bounds__(256, MINB) k_dual(const IterParams P) {
  dual_body<DIM, TGV, CPL, CMAX>(P, blockIdx.x);
}

// k_dual_pf: k_dual for a launch whose channel count is exactly CN (no channel
// guard), the operands of a channel -- ubar at the voxel and its three forward
// neighbours, pbar at the voxel and its three backward neighbours, v and w --
// loaded LA channels ahead of their arithmetic (LA = CN: every load before any
// arithmetic).  k_dual interleaves each channel's loads with its arithmetic and
// keeps few loads in flight (it is DRAM-latency bound); here a thread has up to
// 25 LA loads in flight.  The arithmetic is k_dual's, operation by operation, so
// the iterates are bit-identical.
template <int DIM, bool TGV, int CPL, int CN, int MINB = 1, int NT = 256, int LA = CN>
__global__ void __launch_bounds__(NT, MINB) k_dual_pf(const IterParams P) {
  constexpr int K = DIM, KW = DIM == 3 ? 6 : 3;
  const Dims d = P.d;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)d.N * d.N * d.Nz) return;
  const int pix = (int)(t / d.Nz);
  const int z = (int)(t - (long long)pix * d.Nz);
  const int y = pix / d.N, x = pix - y * d.N;
  const size_t vol = d.vol, S = d.S, rowS = (size_t)d.N * S;
  const bool hx = x < d.N - 1, hy = y < d.N - 1, hz = z < d.Nz - 1;  // forward neighbours exist
  const bool lx = x > 0, ly = y > 0, lz = z > 0;                      // backward neighbours exist
  const float *__restrict__ ub = P.ubar;
  const float *__restrict__ pb = P.pbar;
  const size_t i0 = (size_t)pix * S + (size_t)P.cbase * d.Nz + z;
  const float sigma = P.sigma;

  float u0[CN], ux[CN], uy[CN], uz[CN];
  float p0[CN][K], px[CN][K], py[CN][K], pz[CN][K];
  float vo[CN][K], wo[CN][KW];
  float vv[CN][K], ww[CN][KW];
  auto load = [&](const int c) {
    const size_t i = i0 + (size_t)c * d.Nz;
    u0[c] = ub[i];
    ux[c] = hx ? ub[i + S] : 0.f;
    uy[c] = hy ? ub[i + rowS] : 0.f;
    if (DIM == 3) uz[c] = hz ? ub[i + 1] : 0.f;
#pragma unroll
    for (int k = 0; k < K; ++k) {
      vo[c][k] = P.v[k * vol + i];
      if (TGV) {
        p0[c][k] = pb[k * vol + i];
        px[c][k] = lx ? pb[k * vol + i - S] : 0.f;
        py[c][k] = ly ? pb[k * vol + i - rowS] : 0.f;
        if (DIM == 3) pz[c][k] = lz ? pb[k * vol + i - 1] : 0.f;
      }
    }
    if (TGV) {
#pragma unroll
      for (int k = 0; k < KW; ++k) wo[c][k] = P.w[k * vol + i];
    }
  };
  auto compute = [&](const int c) {
    const float mu = -u0[c];
    float g[3];
    g[0] = hx ? mu + ux[c] : 0.f;
    g[1] = hy ? mu + uy[c] : 0.f;
    if (DIM == 3) g[2] = (hz ? mu + uz[c] : 0.f) / P.stepsize;
    float pc[3];
#pragma unroll
    for (int k = 0; k < K; ++k) {
      pc[k] = TGV ? p0[c][k] : 0.f;
      vv[c][k] = vo[c][k] + sigma * (g[k] - pc[k]);
    }
    if (TGV) {
      float a[3], b[3], cz[3];
#pragma unroll
      for (int k = 0; k < K; ++k) {
        a[k] = lx ? pc[k] - px[c][k] : 0.f;
        b[k] = ly ? pc[k] - py[c][k] : 0.f;
        if (DIM == 3) cz[k] = (lz ? pc[k] - pz[c][k] : 0.f) / P.stepsize;
      }
      float e[6];
      if (DIM == 3) {
        e[0] = a[0]; e[1] = b[1]; e[2] = cz[2];
        e[3] = 0.5f * (a[1] + b[0]);
        e[4] = 0.5f * (a[2] + cz[0]);
        e[5] = 0.5f * (b[2] + cz[1]);
      } else {
        e[0] = a[0]; e[1] = b[1];
        e[2] = 0.5f * (a[1] + b[0]);
      }
#pragma unroll
      for (int k = 0; k < KW; ++k) ww[c][k] = wo[c][k] + sigma * e[k];
    }
  };
#pragma unroll
  for (int c = 0; c < LA && c < CN; ++c) load(c);
#pragma unroll
  for (int c = 0; c < CN; ++c) {
    if (c + LA < CN) load(c + LA);
    compute(c);
  }

  dual_project<DIM, TGV, CPL, CN>(P, CN, vv, ww);

#pragma unroll
  for (int c = 0; c < CN; ++c) {
    const size_t i = i0 + (size_t)c * d.Nz;
#pragma unroll
    for (int k = 0; k < K; ++k) P.v[k * vol + i] = vv[c][k];
    if (TGV) {
#pragma unroll
      for (int k = 0; k < KW; ++k) P.w[k * vol + i] = ww[c][k];
    }
  }
}

// k_dual_cl: k_dual with one thread per voxel-channel (Frobenius or uncorrelated
// coupling, C <= CP channels).  The CP lanes of a voxel are consecutive lanes of a
// warp (channel fastest); each loads and updates its own channel (25 loads, all
// issued before the arithmetic) and the coupled norms gather the other channels'
// terms by shuffles and add them in k_dual's order (channels ascending, then
// components), so the iterates are bit-identical to k_dual's.  A thread holds one
// channel instead of all C, so the kernel runs at several times k_dual's
// occupancy with every load in flight.
template <int DIM, bool TGV, int CPL, int CP>
__global__ void __launch_bounds__(256) k_dual_cl(const IterParams P) {
  constexpr int K = DIM, KW = DIM == 3 ? 6 : 3;
  const Dims d = P.d;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long vt = t / CP;  // voxel (pixel, z)
  const int c = (int)(t - vt * CP);
  const bool valid = vt < (long long)d.N * d.N * d.Nz;
  const bool own = valid && c < d.C;  // lanes c >= C of a voxel only take part in the shuffles
  const int pix = valid ? (int)(vt / d.Nz) : 0;
  const int z = valid ? (int)(vt - (long long)pix * d.Nz) : 0;
  const int y = pix / d.N, x = pix - y * d.N;
  const size_t vol = d.vol, S = d.S, rowS = (size_t)d.N * S;
  const bool hx = x < d.N - 1, hy = y < d.N - 1, hz = z < d.Nz - 1;
  const bool lx = x > 0, ly = y > 0, lz = z > 0;
  const float *__restrict__ ub = P.ubar;
  const float *__restrict__ pb = P.pbar;
  const size_t i = (size_t)pix * S + (size_t)c * d.Nz + z;
  const unsigned lane0 = (threadIdx.x & 31) & ~(unsigned)(CP - 1);  // first lane of this voxel's group

  float u0 = 0.f, ux = 0.f, uy = 0.f, uz = 0.f;
  float p0[K], px[K], py[K], pz[K], vo[K], wo[KW];
#pragma unroll
  for (int k = 0; k < K; ++k) { p0[k] = px[k] = py[k] = pz[k] = vo[k] = 0.f; }
#pragma unroll
  for (int k = 0; k < KW; ++k) wo[k] = 0.f;
  if (own) {
    u0 = ub[i];
    if (hx) ux = ub[i + S];
    if (hy) uy = ub[i + rowS];
    if (DIM == 3 && hz) uz = ub[i + 1];
#pragma unroll
    for (int k = 0; k < K; ++k) {
      vo[k] = P.v[k * vol + i];
      if (TGV) {
        p0[k] = pb[k * vol + i];
        if (lx) px[k] = pb[k * vol + i - S];
        if (ly) py[k] = pb[k * vol + i - rowS];
        if (DIM == 3 && lz) pz[k] = pb[k * vol + i - 1];
      }
    }
    if (TGV) {
#pragma unroll
      for (int k = 0; k < KW; ++k) wo[k] = P.w[k * vol + i];
    }
  }

  const float sigma = P.sigma;
  float vv[K], ww[KW];
  {
    const float mu = -u0;
    float g[3];
    g[0] = hx ? mu + ux : 0.f;
    g[1] = hy ? mu + uy : 0.f;
    if (DIM == 3) g[2] = (hz ? mu + uz : 0.f) / P.stepsize;
    float pc[3];
#pragma unroll
    for (int k = 0; k < K; ++k) {
      pc[k] = TGV ? p0[k] : 0.f;
      vv[k] = vo[k] + sigma * (g[k] - pc[k]);
    }
    if (TGV) {
      float a[3], b[3], cz[3];
#pragma unroll
      for (int k = 0; k < K; ++k) {
        a[k] = lx ? pc[k] - px[k] : 0.f;
        b[k] = ly ? pc[k] - py[k] : 0.f;
        if (DIM == 3) cz[k] = (lz ? pc[k] - pz[k] : 0.f) / P.stepsize;
      }
      float e[6];
      if (DIM == 3) {
        e[0] = a[0]; e[1] = b[1]; e[2] = cz[2];
        e[3] = 0.5f * (a[1] + b[0]);
        e[4] = 0.5f * (a[2] + cz[0]);
        e[5] = 0.5f * (b[2] + cz[1]);
      } else {
        e[0] = a[0]; e[1] = b[1];
        e[2] = 0.5f * (a[1] + b[0]);
      }
#pragma unroll
      for (int k = 0; k < KW; ++k) ww[k] = wo[k] + sigma * e[k];
    }
  }

  if (CPL == UNCORR) {
    float n2 = 0.f;
#pragma unroll
    for (int k = 0; k < K; ++k) n2 += vv[k] * vv[k];
    const float nv = sqrtf(n2) * P.ainv1;
    if (nv > 1.f) {
#pragma unroll
      for (int k = 0; k < K; ++k) vv[k] = vv[k] / nv;
    }
    if (TGV) {
      const float nw = sqrtf(wnorm2<DIM, UNCORR>(ww)) * P.ainv0;
      if (nw > 1.f) {
#pragma unroll
        for (int k = 0; k < KW; ++k) ww[k] = ww[k] / nw;
      }
    }
  } else {  // FROB: the norms over the voxel's channels, summed in k_dual's order
    const int nC = d.C;
    float sq[K];
#pragma unroll
    for (int k = 0; k < K; ++k) sq[k] = vv[k] * vv[k];
    float n2 = 0.f;
#pragma unroll
    for (int cc = 0; cc < CP; ++cc) {
#pragma unroll
      for (int k = 0; k < K; ++k) {
        const float s = __shfl_sync(0xffffffffu, sq[k], lane0 + cc);
        if (cc < nC) n2 += s;
      }
    }
    const float nv = sqrtf(n2) * P.ainv1;
    if (nv > 1.f) {
#pragma unroll
      for (int k = 0; k < K; ++k) vv[k] = vv[k] / nv;
    }
    if (TGV) {
      const float wn = wnorm2<DIM, FROB>(ww);
      float m2 = 0.f;
#pragma unroll
      for (int cc = 0; cc < CP; ++cc) {
        const float s = __shfl_sync(0xffffffffu, wn, lane0 + cc);
        if (cc < nC) m2 += s;
      }
      const float nw = sqrtf(m2) * P.ainv0;
      if (nw > 1.f) {
#pragma unroll
        for (int k = 0; k < KW; ++k) ww[k] = ww[k] / nw;
      }
    }
  }

  if (own) {
#pragma unroll
    for (int k = 0; k < K; ++k) P.v[k * vol + i] = vv[k];
    if (TGV) {
#pragma unroll
      for (int k = 0; k < KW; ++k) P.w[k * vol + i] = ww[k];
    }
  }
}

__device__ __forceinline__ float2 ld2(const float *p) { return *reinterpret_cast<const float2 *>(p); }
__device__ __forceinline__ void st2(float *p, float a, float b) { *reinterpret_cast<float2 *>(p) = make_float2(a, b); }

// pbar and p of the slice pair (z0, z0 + 1) at offset j, pixel (xj, yj): update_p
// (3-D :734-757) and its extrapolation (:1217-1221) through p_step3.  po, vj, wj:
// p, v and w at j; wx: rows (w0 w3 w4) of w at the x successor (read where
// xj < N - 1); wy: rows (w3 w1 w5) at the y successor (yj < N - 1); wz: rows
// (w4 w5 w2) at slice z0 + 2 (z0 + 1 < Nz - 1).
__device__ __forceinline__ void pair_pstep(const IterParams &P, int xj, int yj, int z0, const float2 (&po)[3],
                                           const float2 (&wj)[6], const float2 (&vj)[3], const float2 (&wx)[3],
                                           const float2 (&wy)[3], const float (&wz)[3], float2 (&pn)[3],
                                           float2 (&pbr)[3]) {
  const Dims d = P.d;
  const int rx[3] = {0, 3, 4}, ry[3] = {3, 1, 5}, rz[3] = {4, 5, 2};
  const bool fx = xj == 0, hx = xj < d.N - 1, fy = yj == 0, hy = yj < d.N - 1;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float r0 = p_step3(po[k].x, vj[k].x, wj[rx[k]].x, wx[k].x, wj[ry[k]].x, wy[k].x, wj[rz[k]].x,
                             wj[rz[k]].y, fx, hx, fy, hy, z0 == 0, true, P.tau, P.stepsize);
    const float r1 = p_step3(po[k].y, vj[k].y, wj[rx[k]].y, wx[k].y, wj[ry[k]].y, wy[k].y, wj[rz[k]].y, wz[k], fx,
                             hx, fy, hy, false, z0 + 1 < d.Nz - 1, P.tau, P.stepsize);
    pn[k] = make_float2(r0, r1);
    pbr[k] = make_float2(2.0f * r0 - po[k].x, 2.0f * r1 - po[k].y);
  }
}

// The dual update of one channel's slice pair (z0, z0 + 1) of one voxel column,
// k_dual_cl's arithmetic and shuffle order per slice: v + sigma (grad ubar - pbar)
// and w + sigma E(pbar) (update_v :546-571, update_w :573-600), projected onto the
// coupling's balls (NormV / NormW).  The CP lanes of a voxel (from lane0) hold its
// channels; every lane of the warp must call this (shuffles).  Inputs: ubar at
// the pair (u0), its x / y successors (ux, uy) and slice z0 + 2 (uz1); pbar at the
// pair (p0), its x / y predecessors (px, py) and slice z0 - 1 (pzm); v, w at the pair.
// STEP1: the slice step size is 1, so the divisions by it (x / 1 = x exactly in IEEE
// arithmetic) are left out; the results are the same bits.
template <bool TGV, int CPL, int CP, bool STEP1 = false>
__device__ __forceinline__ void dual_pair_math(const IterParams &P, unsigned lane0, float2 u0, float2 ux, float2 uy,
                                               float uz1, const float2 (&p0)[3], const float2 (&px)[3],
                                               const float2 (&py)[3], const float (&pzm)[3], const float2 (&vo)[3],
                                               const float2 (&wo)[6], bool hx, bool hy, bool lx, bool ly, int z0,
                                               float (&vv)[2][3], float (&ww)[2][6]) {
  constexpr int K = 3, KW = 6;
  const bool hz[2] = {true, z0 + 1 < P.d.Nz - 1}, lz[2] = {z0 > 0, true};
  const float sigma = P.sigma;
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const float uc = h ? u0.y : u0.x, uxn = h ? ux.y : ux.x, uyn = h ? uy.y : uy.x;
    const float uzn = h ? uz1 : u0.y;
    const float mu = -uc;
    float g[3];
    g[0] = hx ? mu + uxn : 0.f;
    g[1] = hy ? mu + uyn : 0.f;
    g[2] = hz[h] ? mu + uzn : 0.f;
    if (!STEP1) g[2] /= P.stepsize;
    float pc[3];
#pragma unroll
    for (int k = 0; k < K; ++k) {
      pc[k] = TGV ? (h ? p0[k].y : p0[k].x) : 0.f;
      vv[h][k] = (h ? vo[k].y : vo[k].x) + sigma * (g[k] - pc[k]);
    }
    if (TGV) {
      float a[3], b[3], cz[3];
#pragma unroll
      for (int k = 0; k < K; ++k) {
        a[k] = lx ? pc[k] - (h ? px[k].y : px[k].x) : 0.f;
        b[k] = ly ? pc[k] - (h ? py[k].y : py[k].x) : 0.f;
        cz[k] = lz[h] ? pc[k] - (h ? p0[k].x : pzm[k]) : 0.f;
        if (!STEP1) cz[k] /= P.stepsize;
      }
      float e[6];
      e[0] = a[0]; e[1] = b[1]; e[2] = cz[2];
      e[3] = 0.5f * (a[1] + b[0]);
      e[4] = 0.5f * (a[2] + cz[0]);
      e[5] = 0.5f * (b[2] + cz[1]);
#pragma unroll
      for (int k = 0; k < KW; ++k) ww[h][k] = (h ? wo[k].y : wo[k].x) + sigma * e[k];
    }
  }

#pragma unroll
  for (int h = 0; h < 2; ++h) {
    if (CPL == UNCORR) {
      float n2 = 0.f;
#pragma unroll
      for (int k = 0; k < K; ++k) n2 += vv[h][k] * vv[h][k];
      const float nv = sqrtf(n2) * P.ainv1;
      if (nv > 1.f) {
#pragma unroll
        for (int k = 0; k < K; ++k) vv[h][k] = vv[h][k] / nv;
      }
      if (TGV) {
        const float nw = sqrtf(wnorm2<3, UNCORR>(ww[h])) * P.ainv0;
        if (nw > 1.f) {
#pragma unroll
          for (int k = 0; k < KW; ++k) ww[h][k] = ww[h][k] / nw;
        }
      }
    } else {
      const int nC = P.d.C;
      float sq[K];
#pragma unroll
      for (int k = 0; k < K; ++k) sq[k] = vv[h][k] * vv[h][k];
      float n2 = 0.f;
#pragma unroll
      for (int cc = 0; cc < CP; ++cc) {
#pragma unroll
        for (int k = 0; k < K; ++k) {
          const float s = __shfl_sync(0xffffffffu, sq[k], lane0 + cc);
          if (cc < nC) n2 += s;
        }
      }
      const float nv = sqrtf(n2) * P.ainv1;
      if (nv > 1.f) {
#pragma unroll
        for (int k = 0; k < K; ++k) vv[h][k] = vv[h][k] / nv;
      }
      if (TGV) {
        const float wn = wnorm2<3, FROB>(ww[h]);
        float m2 = 0.f;
#pragma unroll
        for (int cc = 0; cc < CP; ++cc) {
          const float s = __shfl_sync(0xffffffffu, wn, lane0 + cc);
          if (cc < nC) m2 += s;
        }
        const float nw = sqrtf(m2) * P.ainv0;
        if (nw > 1.f) {
#pragma unroll
          for (int k = 0; k < KW; ++k) ww[h][k] = ww[h][k] / nw;
        }
      }
    }
  }
}

// k_dual_cl2: k_dual_cl for two consecutive slices z0, z0 + 1 of one channel per
// thread (3-D, Nz even): the fields of both slices move as one float2, the slice
// neighbours outside the pair as one float each.  Per slice the arithmetic and the
// shuffle order are k_dual_cl's, so the iterates are bit-identical to k_dual's.
template <bool TGV, int CPL, int CP, bool STEP1 = false>
__global__ void __launch_bounds__(256) k_dual_cl2(const IterParams P) {
  constexpr int K = 3, KW = 6;
  const Dims d = P.d;
  const int nz2 = d.Nz >> 1;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long vt = t / CP;  // (pixel, slice pair)
  const int c = (int)(t - vt * CP);
  const bool valid = vt < (long long)d.N * d.N * nz2;
  const bool own = valid && c < d.C;
  const int pix = valid ? (int)(vt / nz2) : 0;
  const int z0 = valid ? 2 * (int)(vt - (long long)pix * nz2) : 0;
  const int y = pix / d.N, x = pix - y * d.N;
  const size_t vol = d.vol, S = d.S, rowS = (size_t)d.N * S;
  const bool hx = x < d.N - 1, hy = y < d.N - 1;
  const bool lx = x > 0, ly = y > 0;
  const float *__restrict__ ub = P.ubar;
  const float *__restrict__ pb = P.pbar;
  const size_t i = (size_t)pix * S + (size_t)c * d.Nz + z0;
  const unsigned lane0 = (threadIdx.x & 31) & ~(unsigned)(CP - 1);

  float2 u0 = make_float2(0.f, 0.f), ux = u0, uy = u0;
  float uz1 = 0.f;  // ubar at z0 + 2
  float2 p0[K], px[K], py[K], vo[K], wo[KW];
  float pzm[K];  // pbar at z0 - 1
#pragma unroll
  for (int k = 0; k < K; ++k) { p0[k] = px[k] = py[k] = vo[k] = u0; pzm[k] = 0.f; }
#pragma unroll
  for (int k = 0; k < KW; ++k) wo[k] = u0;
  if (own) {
    u0 = ld2(ub + i);
    if (hx) ux = ld2(ub + i + S);
    if (hy) uy = ld2(ub + i + rowS);
    if (z0 + 1 < d.Nz - 1) uz1 = ub[i + 2];
#pragma unroll
    for (int k = 0; k < K; ++k) {
      vo[k] = ld2(P.v + k * vol + i);
      if (TGV) {
        p0[k] = ld2(pb + k * vol + i);
        if (lx) px[k] = ld2(pb + k * vol + i - S);
        if (ly) py[k] = ld2(pb + k * vol + i - rowS);
        if (z0 > 0) pzm[k] = pb[k * vol + i - 1];
      }
    }
    if (TGV) {
#pragma unroll
      for (int k = 0; k < KW; ++k) wo[k] = ld2(P.w + k * vol + i);
    }
  }

  float vv[2][K], ww[2][KW];
  dual_pair_math<TGV, CPL, CP, STEP1>(P, lane0, u0, ux, uy, uz1, p0, px, py, pzm, vo, wo, hx, hy, lx, ly, z0, vv,
                                      ww);

  if (own) {
#pragma unroll
    for (int k = 0; k < K; ++k) st2(P.v + k * vol + i, vv[0][k], vv[1][k]);
    if (TGV) {
#pragma unroll
      for (int k = 0; k < KW; ++k) st2(P.w + k * vol + i, ww[0][k], ww[1][k]);
    }
  }
}

// k_dual_walk: the dual update of schedule 2 with the p / pbar half of the previous
// iteration's primal update fused in (3-D TGV, Frobenius or uncorrelated coupling,
// Nz even).  p, v, w are read from P.p, P.v, P.w and the new p, v, w written to
// P.p2, P.v2, P.w2 (another buffer set: the neighbours' old values must stay while
// other blocks read them); the pbar buffer is not used.
//
// The dual update at a voxel needs pbar there and at its x, y and z predecessors.
// A block covers NCOL pixel columns (the first a halo that only computes pbar)
// times ZC + 1 slice pairs of every channel (the first pair a halo likewise), and
// walks down R rows from y0, with a first step at row y0 - 1 for pbar only.  Per
// row each thread computes pbar of its own pair (update_p through pair_pstep) and
// publishes it in shared memory: the x predecessor's pbar comes from the column to
// the left, the z predecessor's from the pair below, the y predecessor's is the
// thread's own pbar of the previous row (registers).  A row's operands (w, v, p,
// the w rows and ubar of the next row, and at the block's last column / pair the
// operands beyond it) are copied into shared memory by cp.async one row ahead, so
// the next row's loads are in flight while a row is computed; the neighbours' w
// rows and ubar are read from those copies.  So every field is read from HBM about
// once, plus the halo column and pair.
// Thread layout: t = (column * (ZC + 1) + pair) * CP + channel lane, so the CP
// lanes of a voxel are adjacent (the coupling's shuffles).  Every value is
// computed by the same operations as k_update and k_dual_cl2: identical iterates.
namespace walk {
// float2 slots of a row buffer, each [T]: w0..w5, v0..v2, p0..p2, rows (w3 w1 w5)
// of the next row, ubar, ubar of the next row, rows (w0 w3 w4) and ubar of the x
// successor (last column), then float slots: rows (w4 w5 w2) and ubar at slice
// z0 + 2 (last pair)
constexpr int W = 0, V = 6, PO = 9, WY = 12, U0 = 15, UY = 16, WXE = 17, UXE = 20, NF2 = 21;
constexpr int WZE = 0, UZE = 3, NF1 = 4;
constexpr size_t bytes_per_thread = 2 * (NF2 * 8 + NF1 * 4) + 3 * 8;  // two row buffers + pbar exchange
}  // namespace walk

__device__ __forceinline__ void cp_async8(void *dst, const float *src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"((unsigned)__cvta_generic_to_shared(dst)), "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async4(void *dst, const float *src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"((unsigned)__cvta_generic_to_shared(dst)), "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

template <int CPL, int CP>
__global__ void __launch_bounds__(512, 1) k_dual_walk(const IterParams P, int ZC, int NCOL, int R) {
  using namespace walk;
  constexpr int K = 3, KW = 6;
  extern __shared__ float smem[];
  const Dims d = P.d;
  const int T = blockDim.x;
  const int colT = (ZC + 1) * CP;
  const int t = threadIdx.x;
  const int col = t / colT, rr = t - col * colT;
  const int pl = rr / CP, c = rr - pl * CP;
  const int x = (int)blockIdx.x * (NCOL - 1) - 1 + col;
  const int z0 = (int)blockIdx.z * 2 * ZC + 2 * (pl - 1);
  const int y0 = (int)blockIdx.y * R;
  const bool pthr = col < NCOL && x >= 0 && x < d.N && z0 >= 0 && z0 < d.Nz && c < d.C;
  const bool dthr = pthr && col >= 1 && pl >= 1;
  const bool nbx = col + 1 < NCOL;  // the x successor is in the block
  const bool nbz = pl < ZC;         // the pair above is in the block
  const size_t vol = d.vol, S = d.S, rowS = (size_t)d.N * S;
  const bool hx = x < d.N - 1, lx = x > 0, hz1 = z0 + 1 < d.Nz - 1;
  const unsigned lane0 = (threadIdx.x & 31) & ~(unsigned)(CP - 1);
  const int rx[3] = {0, 3, 4}, ry[3] = {3, 1, 5}, rz[3] = {4, 5, 2};
  const float *__restrict__ ub = P.ubar;
  const float *__restrict__ w = P.w;
  const float2 zero = make_float2(0.f, 0.f);
  float2 *const f2base = reinterpret_cast<float2 *>(smem);                // [2][NF2][T]
  float *const f1base = reinterpret_cast<float *>(f2base + 2 * NF2 * T);  // [2][NF1][T]
  float2 *const spb = reinterpret_cast<float2 *>(f1base + 2 * NF1 * T);   // [3][T]

  // copies of row y's operands into buffer b (threads that compute there)
  auto issue = [&](int y, int b) {
    if (pthr && y >= 0 && y < d.N) {
      const size_t i = ((size_t)y * d.N + x) * S + (size_t)c * d.Nz + z0;
      float2 *f2 = f2base + b * NF2 * T;
      float *f1 = f1base + b * NF1 * T;
#pragma unroll
      for (int k = 0; k < KW; ++k) cp_async8(f2 + (W + k) * T + t, w + k * vol + i);
#pragma unroll
      for (int k = 0; k < K; ++k) {
        cp_async8(f2 + (V + k) * T + t, P.v + k * vol + i);
        cp_async8(f2 + (PO + k) * T + t, P.p + k * vol + i);
        if (y < d.N - 1) cp_async8(f2 + (WY + k) * T + t, w + ry[k] * vol + i + rowS);
      }
      if (dthr) {
        cp_async8(f2 + U0 * T + t, ub + i);
        if (y < d.N - 1) cp_async8(f2 + UY * T + t, ub + i + rowS);
      }
      if (!nbx && hx) {
#pragma unroll
        for (int k = 0; k < K; ++k) cp_async8(f2 + (WXE + k) * T + t, w + rx[k] * vol + i + S);
        if (dthr) cp_async8(f2 + UXE * T + t, ub + i + S);
      }
      if (!nbz && hz1) {
#pragma unroll
        for (int k = 0; k < K; ++k) cp_async4(f1 + (WZE + k) * T + t, w + rz[k] * vol + i + 2);
        if (dthr) cp_async4(f1 + UZE * T + t, ub + i + 2);
      }
    }
    cp_async_commit();
  };

  float2 pprev[K];  // pbar of the previous row
#pragma unroll
  for (int k = 0; k < K; ++k) pprev[k] = zero;
  issue(y0 - 1, 0);
  for (int s = 0; s <= R; ++s) {
    const int y = y0 - 1 + s;
    const int b = s & 1;
    const bool act = pthr && y >= 0 && y < d.N;
    const bool hy = y < d.N - 1, ly = y > 0;
    if (s < R) {
      issue(y + 1, b ^ 1);
      cp_async_wait<1>();  // this row's copies (the next row's stay in flight)
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
    const float2 *f2 = f2base + b * NF2 * T;
    const float *f1 = f1base + b * NF1 * T;
    float2 wo[KW], vo[K], po[K], wy[K], pn[K], pbr[K];
#pragma unroll
    for (int k = 0; k < KW; ++k) wo[k] = zero;
#pragma unroll
    for (int k = 0; k < K; ++k) vo[k] = po[k] = wy[k] = pn[k] = pbr[k] = zero;
    if (act) {
#pragma unroll
      for (int k = 0; k < KW; ++k) wo[k] = f2[(W + k) * T + t];
      float2 wx[K];
      float wz[K];
#pragma unroll
      for (int k = 0; k < K; ++k) {
        vo[k] = f2[(V + k) * T + t];
        po[k] = f2[(PO + k) * T + t];
        if (hy) wy[k] = f2[(WY + k) * T + t];
        wx[k] = !hx ? zero : (nbx ? f2[(W + rx[k]) * T + t + colT] : f2[(WXE + k) * T + t]);
        wz[k] = !hz1 ? 0.f : (nbz ? f2[(W + rz[k]) * T + t + CP].x : f1[(WZE + k) * T + t]);
      }
      pair_pstep(P, x, y, z0, po, wo, vo, wx, wy, wz, pn, pbr);
    }
#pragma unroll
    for (int k = 0; k < K; ++k) spb[k * T + t] = pbr[k];
    __syncthreads();
    if (s >= 1) {  // the dual update of row y (uniform over the block: every lane shuffles)
      const bool dact = dthr && act;
      float2 u0 = zero, ux = zero, uy = zero, px[K], pyv[K];
      float uz1 = 0.f, pzm[K];
#pragma unroll
      for (int k = 0; k < K; ++k) { px[k] = pyv[k] = zero; pzm[k] = 0.f; }
      if (dact) {
        u0 = f2[U0 * T + t];
        if (hx) ux = nbx ? f2[U0 * T + t + colT] : f2[UXE * T + t];
        if (hy) uy = f2[UY * T + t];
        if (hz1) uz1 = nbz ? f2[U0 * T + t + CP].x : f1[UZE * T + t];
#pragma unroll
        for (int k = 0; k < K; ++k) {
          px[k] = spb[k * T + t - colT];
          pyv[k] = pprev[k];
          pzm[k] = spb[k * T + t - CP].y;
        }
      }
      float vv[2][K], ww[2][KW];
      dual_pair_math<true, CPL, CP>(P, lane0, u0, ux, uy, uz1, pbr, px, pyv, pzm, vo, wo, hx, hy, lx, ly, z0, vv,
                                    ww);
      if (dact) {
        const size_t i = ((size_t)y * d.N + x) * S + (size_t)c * d.Nz + z0;
#pragma unroll
        for (int k = 0; k < K; ++k) st2(P.v2 + k * vol + i, vv[0][k], vv[1][k]);
#pragma unroll
        for (int k = 0; k < KW; ++k) st2(P.w2 + k * vol + i, ww[0][k], ww[1][k]);
#pragma unroll
        for (int k = 0; k < K; ++k) st2(P.p2 + k * vol + i, pn[k].x, pn[k].y);
      }
    }
#pragma unroll
    for (int k = 0; k < K; ++k) pprev[k] = pbr[k];
    __syncthreads();  // the row buffer and the pbar exchange are free for the next row
  }
}

// k_dual_z2: k_dual for 3-D TGV with Frobenius or uncorrelated coupling, a thread
// per (pixel, pair of consecutive slices z0, z0+1): every field is read and
// written as float2 (half the load instructions of k_dual), in two phases (v,
// then w) to bound the registers.  Every value is computed by the same
// operations as in k_dual, so the iterates are bit-identical.  Needs Nz even.

template <int CPL, int CMAX>
__global__ void __launch_bounds__(256) k_dual_z2(const IterParams P) {
  const Dims d = P.d;
  const int nzq = d.Nz >> 1;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)d.N * d.N * nzq) return;
  const int pix = (int)(t / nzq);
  const int z0 = 2 * (int)(t - (long long)pix * nzq);
  const int y = pix / d.N, x = pix - y * d.N;
  const size_t vol = d.vol, S = d.S, rowS = (size_t)d.N * S;
  const float sigma = P.sigma;
  const float *__restrict__ ub = P.ubar;
  const float *__restrict__ pb = P.pbar;
  const int nC = min(CMAX, d.C);
  const bool hx = x < d.N - 1, hy = y < d.N - 1, hz = z0 + 1 < d.Nz - 1;  // forward neighbours
  const bool lx = x > 0, ly = y > 0, lz = z0 > 0;                          // backward neighbours

  // ---- v: gradient of ubar minus pbar, ball projection, store
  {
    float vv[CMAX][3][2];
#pragma unroll
    for (int c = 0; c < CMAX; ++c) {
      if (c >= nC) break;
      const size_t i = (size_t)pix * S + (size_t)c * d.Nz + z0;
      const float2 u = ld2(ub + i);
      float g[3][2];
      const float mu0 = -u.x, mu1 = -u.y;
      if (hx) { const float2 n = ld2(ub + i + S); g[0][0] = mu0 + n.x; g[0][1] = mu1 + n.y; } else { g[0][0] = g[0][1] = 0.f; }
      if (hy) { const float2 n = ld2(ub + i + rowS); g[1][0] = mu0 + n.x; g[1][1] = mu1 + n.y; } else { g[1][0] = g[1][1] = 0.f; }
      g[2][0] = (mu0 + u.y) / P.stepsize;
      g[2][1] = (hz ? mu1 + ub[i + 2] : 0.f) / P.stepsize;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const float2 pc = ld2(pb + k * vol + i), v = ld2(P.v + k * vol + i);
        vv[c][k][0] = v.x + sigma * (g[k][0] - pc.x);
        vv[c][k][1] = v.y + sigma * (g[k][1] - pc.y);
      }
    }
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      if (CPL == FROB) {
        float n2 = 0.f;
#pragma unroll
        for (int c = 0; c < CMAX; ++c) {
          if (c >= nC) break;
#pragma unroll
          for (int k = 0; k < 3; ++k) n2 += vv[c][k][q] * vv[c][k][q];
        }
        const float nv = sqrtf(n2) * P.ainv1;
        if (nv > 1.f) {
#pragma unroll
          for (int c = 0; c < CMAX; ++c) {
            if (c >= nC) break;
#pragma unroll
            for (int k = 0; k < 3; ++k) vv[c][k][q] = vv[c][k][q] / nv;
          }
        }
      } else {
#pragma unroll
        for (int c = 0; c < CMAX; ++c) {
          if (c >= nC) break;
          float n2 = 0.f;
#pragma unroll
          for (int k = 0; k < 3; ++k) n2 += vv[c][k][q] * vv[c][k][q];
          const float nv = sqrtf(n2) * P.ainv1;
          if (nv > 1.f) {
#pragma unroll
            for (int k = 0; k < 3; ++k) vv[c][k][q] = vv[c][k][q] / nv;
          }
        }
      }
    }
#pragma unroll
    for (int c = 0; c < CMAX; ++c) {
      if (c >= nC) break;
      const size_t i = (size_t)pix * S + (size_t)c * d.Nz + z0;
#pragma unroll
      for (int k = 0; k < 3; ++k) st2(P.v + k * vol + i, vv[c][k][0], vv[c][k][1]);
    }
  }

  // ---- w: symmetrised gradient of pbar, ball projection, store
  float ww[CMAX][6][2];
#pragma unroll
  for (int c = 0; c < CMAX; ++c) {
    if (c >= nC) break;
    const size_t i = (size_t)pix * S + (size_t)c * d.Nz + z0;
    float a[3][2], b[3][2], cz[3][2];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const float2 pc = ld2(pb + k * vol + i);
      if (lx) { const float2 n = ld2(pb + k * vol + i - S); a[k][0] = pc.x - n.x; a[k][1] = pc.y - n.y; } else { a[k][0] = a[k][1] = 0.f; }
      if (ly) { const float2 n = ld2(pb + k * vol + i - rowS); b[k][0] = pc.x - n.x; b[k][1] = pc.y - n.y; } else { b[k][0] = b[k][1] = 0.f; }
      cz[k][0] = (lz ? pc.x - pb[k * vol + i - 1] : 0.f) / P.stepsize;
      cz[k][1] = (pc.y - pc.x) / P.stepsize;
    }
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      float e[6];
      e[0] = a[0][q]; e[1] = b[1][q]; e[2] = cz[2][q];
      e[3] = 0.5f * (a[1][q] + b[0][q]);
      e[4] = 0.5f * (a[2][q] + cz[0][q]);
      e[5] = 0.5f * (b[2][q] + cz[1][q]);
#pragma unroll
      for (int k = 0; k < 6; ++k) ww[c][k][q] = e[k];
    }
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      const float2 w = ld2(P.w + k * vol + i);
      ww[c][k][0] = w.x + sigma * ww[c][k][0];
      ww[c][k][1] = w.y + sigma * ww[c][k][1];
    }
  }
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    if (CPL == FROB) {
      float n2 = 0.f;
#pragma unroll
      for (int c = 0; c < CMAX; ++c) {
        if (c >= nC) break;
        float wc[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) wc[k] = ww[c][k][q];
        n2 += wnorm2<3, FROB>(wc);
      }
      const float nw = sqrtf(n2) * P.ainv0;
      if (nw > 1.f) {
#pragma unroll
        for (int c = 0; c < CMAX; ++c) {
          if (c >= nC) break;
#pragma unroll
          for (int k = 0; k < 6; ++k) ww[c][k][q] = ww[c][k][q] / nw;
        }
      }
    } else {
#pragma unroll
      for (int c = 0; c < CMAX; ++c) {
        if (c >= nC) break;
        float wc[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) wc[k] = ww[c][k][q];
        const float nw = sqrtf(wnorm2<3, UNCORR>(wc)) * P.ainv0;
        if (nw > 1.f) {
#pragma unroll
          for (int k = 0; k < 6; ++k) ww[c][k][q] = ww[c][k][q] / nw;
        }
      }
    }
  }
#pragma unroll
  for (int c = 0; c < CMAX; ++c) {
    if (c >= nC) break;
    const size_t i = (size_t)pix * S + (size_t)c * d.Nz + z0;
#pragma unroll
    for (int k = 0; k < 6; ++k) st2(P.w + k * vol + i, ww[c][k][0], ww[c][k][1]);
  }
}

// coherent vector loads / stores of UW consecutive slices (fields a kernel also writes)
template <int VW> __device__ __forceinline__ void ldw(const float *p, float (&r)[VW]) {
  if (VW == 4) {
    const float4 q = *reinterpret_cast<const float4 *>(p);
    r[0] = q.x; r[1 % VW] = q.y; r[2 % VW] = q.z; r[3 % VW] = q.w;
  } else if (VW == 2) {
    const float2 q = *reinterpret_cast<const float2 *>(p);
    r[0] = q.x; r[1 % VW] = q.y;
  } else {
    r[0] = p[0];
  }
}
template <int VW> __device__ __forceinline__ void stv(float *p, const float (&r)[VW]) {
  if (VW == 4) *reinterpret_cast<float4 *>(p) = make_float4(r[0], r[1 % VW], r[2 % VW], r[3 % VW]);
  else if (VW == 2) *reinterpret_cast<float2 *>(p) = make_float2(r[0], r[1 % VW]);
  else p[0] = r[0];
}

// ===========================================================================
// slice sets: a lane owns VW slices and the per-pixel geometry of the
// projectors is computed once for them; every per-slice operation keeps the
// reference's order.
//   VW = 8: two float4 chunks, slices 4l..4l+3 and 128+4l..128+4l+3 of the warp's
//           256-slice block (l = lane), so each load instruction of the warp
//           reads 512 contiguous bytes; a warp never straddles pixels or bins.
//   VW = 4: one float4 chunk, slices 4l..4l+3 of the warp's 128-slice block
//           (twice the warps of VW = 8, half the registers).
//   VW = 2, 1: VW consecutive slices per thread (S not a multiple of 4).
// ===========================================================================
template <int VW>
struct Slices {
  int s0;         // first slice of chunk a (VW = 8: chunk b starts at s0 + 128)
  bool va, vb;    // chunk a / b inside [0, S)
  __device__ __forceinline__ void load(const float *base, float (&r)[VW]) const {
    if (VW == 8) {
      float4 a = make_float4(0.f, 0.f, 0.f, 0.f), b = a;
      if (va) a = __ldg(reinterpret_cast<const float4 *>(base + s0));
      if (vb) b = __ldg(reinterpret_cast<const float4 *>(base + s0 + 128));
      r[0] = a.x; r[1 % VW] = a.y; r[2 % VW] = a.z; r[3 % VW] = a.w;
      r[4 % VW] = b.x; r[5 % VW] = b.y; r[6 % VW] = b.z; r[7 % VW] = b.w;
    } else if (VW == 4) {
      float4 a = make_float4(0.f, 0.f, 0.f, 0.f);
      if (va) a = __ldg(reinterpret_cast<const float4 *>(base + s0));
      r[0] = a.x; r[1 % VW] = a.y; r[2 % VW] = a.z; r[3 % VW] = a.w;
    } else if (VW == 2) {
      const float2 a = __ldg(reinterpret_cast<const float2 *>(base + s0));
      r[0] = a.x; r[1 % VW] = a.y;
    } else {
      r[0] = __ldg(base + s0);
    }
  }
  // coherent load (fields this kernel also writes)
  __device__ __forceinline__ void loadw(const float *base, float (&r)[VW]) const {
    if (VW == 8) {
      float4 a = make_float4(0.f, 0.f, 0.f, 0.f), b = a;
      if (va) a = *reinterpret_cast<const float4 *>(base + s0);
      if (vb) b = *reinterpret_cast<const float4 *>(base + s0 + 128);
      r[0] = a.x; r[1 % VW] = a.y; r[2 % VW] = a.z; r[3 % VW] = a.w;
      r[4 % VW] = b.x; r[5 % VW] = b.y; r[6 % VW] = b.z; r[7 % VW] = b.w;
    } else if (VW == 4) {
      float4 a = make_float4(0.f, 0.f, 0.f, 0.f);
      if (va) a = *reinterpret_cast<const float4 *>(base + s0);
      r[0] = a.x; r[1 % VW] = a.y; r[2 % VW] = a.z; r[3 % VW] = a.w;
    } else if (VW == 2) {
      const float2 a = *reinterpret_cast<const float2 *>(base + s0);
      r[0] = a.x; r[1 % VW] = a.y;
    } else {
      r[0] = base[s0];
    }
  }
  __device__ __forceinline__ void store(float *base, const float (&r)[VW]) const {
    if (VW == 8) {
      if (va) *reinterpret_cast<float4 *>(base + s0) = make_float4(r[0], r[1 % VW], r[2 % VW], r[3 % VW]);
      if (vb) *reinterpret_cast<float4 *>(base + s0 + 128) = make_float4(r[4 % VW], r[5 % VW], r[6 % VW], r[7 % VW]);
    } else if (VW == 4) {
      if (va) *reinterpret_cast<float4 *>(base + s0) = make_float4(r[0], r[1 % VW], r[2 % VW], r[3 % VW]);
    } else if (VW == 2) {
      *reinterpret_cast<float2 *>(base + s0) = make_float2(r[0], r[1 % VW]);
    } else {
      base[s0] = r[0];
    }
  }
  __device__ __forceinline__ int slice(int k) const { return VW == 8 ? s0 + (k < 4 ? k : 124 + k) : s0 + k; }
  __device__ __forceinline__ bool valid(int k) const { return VW == 8 ? (k < 4 ? va : vb) : (VW == 4 ? va : true); }
};

// Map a thread to (unit, slice set).  VW = 8: one warp per (unit, 256-slice block);
// otherwise one thread per (unit, VW slices).  Returns false past the end.
template <int VW>
__device__ __forceinline__ bool map_thread(long long bid, long long units, int S, long long &unit, Slices<VW> &sl) {
  const long long t = bid * blockDim.x + threadIdx.x;
  if (VW == 8 || VW == 4) {
    const int span = VW * 32;
    const int nblk = (S + span - 1) / span;
    const long long w = t >> 5;
    if (w >= units * nblk) return false;
    unit = w / nblk;
    const int blk = (int)(w - unit * nblk);
    sl.s0 = blk * span + (int)(threadIdx.x & 31) * 4;
    sl.va = sl.s0 < S;
    sl.vb = VW == 8 && sl.s0 + 128 < S;
  } else {
    const int nsg = S / VW;
    if (t >= units * nsg) return false;
    unit = t / nsg;
    sl.s0 = (int)(t - unit * nsg) * VW;
    sl.va = sl.vb = true;
  }
  return true;
}

template <int VW>
__device__ __forceinline__ bool map_thread(long long units, int S, long long &unit, Slices<VW> &sl) {
  return map_thread<VW>((long long)blockIdx.x, units, S, unit, sl);
}

template <int VW>
static inline long long threads_for(long long units, int S) {
  return (VW == 8 || VW == 4) ? units * ((S + VW * 32 - 1) / (VW * 32)) * 32 : units * (S / VW);
}

// One slice per lane, a warp over 32 consecutive slices, the slice chunk outermost:
// the warps running at a time all work on the same 32 slices of every pixel or
// bin, so a projector's working set is one 32-slice chunk of the image or
// sinogram (e.g. 768^2 x 32 x 4 B = 75 MB, inside L2) instead of all S slices.
struct SlicesWL {
  int s0;
  bool va;
  __device__ __forceinline__ void load(const float *base, float (&r)[1]) const { r[0] = va ? __ldg(base + s0) : 0.f; }
  __device__ __forceinline__ void loadw(const float *base, float (&r)[1]) const { r[0] = va ? base[s0] : 0.f; }
  __device__ __forceinline__ void store(float *base, const float (&r)[1]) const { if (va) base[s0] = r[0]; }
  __device__ __forceinline__ int slice(int) const { return s0; }
  __device__ __forceinline__ bool valid(int) const { return va; }
};

__device__ __forceinline__ bool map_thread_wl(long long units, int S, long long &unit, SlicesWL &sl) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long w = t >> 5;
  const int nblk = (S + 31) / 32;
  if (w >= units * nblk) return false;
  const int blk = (int)(w / units);
  unit = w - (long long)blk * units;
  sl.s0 = blk * 32 + (int)(threadIdx.x & 31);
  sl.va = sl.s0 < S;
  return true;
}

static inline long long threads_for_wl(long long units, int S) { return units * ((S + 31) / 32) * 32; }

// ===========================================================================
// forward projection: kernel `radon` (3-D :773-816).  Ray (i, j) of slice s:
// acc = sum over rows y and x in [x_low, x_high] of (1 - |x X + y Y + off - i|)+ img.
// The arithmetic is the reference's, in its order and without contraction.
// ===========================================================================
template <int VW>
__device__ __forceinline__ void radon_ray(const float *__restrict__ img, size_t S, int N, const float4 o, int i,
                                          const Slices<VW> &sl, float (&acc)[VW]) {
  int ylo, yhi;
  ray_rows(o, i, N, ylo, yhi);
  const float fi = (float)i, fim = (float)(i - 1), fip = (float)(i + 1);
#pragma unroll
  for (int k = 0; k < VW; ++k) acc[k] = 0.f;
  for (int y = ylo; y <= yhi; ++y) {
    const float d = __fadd_rn(__fmul_rn((float)y, o.y), o.z);
    int xl, xh;
    if (o.x == 0.f) {
      if (d > fim && d < fip) { xl = 0; xh = N - 1; } else continue;
    } else if (o.x > 0.f) {
      xl = __float2int_rz(__fmul_rn(__fsub_rn(fim, d), o.w));
      xh = __float2int_rz(__fmul_rn(__fsub_rn(fip, d), o.w));
    } else {
      xl = __float2int_rz(__fmul_rn(__fsub_rn(fip, d), o.w));
      xh = __float2int_rz(__fmul_rn(__fsub_rn(fim, d), o.w));
    }
    xl = max(xl, 0);
    xh = min(xh, N - 1);
    const float *row = img + (size_t)y * N * S;
    for (int x = xl; x <= xh; ++x) {
      const float wgt = 1.0f - fabsf(__fsub_rn(__fadd_rn(__fmul_rn((float)x, o.x), d), fi));
      if (wgt > 0.f) {
        float val[VW];
        sl.load(row + (size_t)x * S, val);
#pragma unroll
        for (int k = 0; k < VW; ++k) acc[k] = __fadd_rn(acc[k], __fmul_rn(wgt, val[k]));
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Ray tables.  The geometry is fixed for a solve, so the (pixel, weight) list of
// every ray -- the reference's own row bounds and hat weights, in its row-major
// order -- is built once per problem (ray_count / ray_fill) and the iteration's
// forward projection streams it (radon_table): same sums in the same order,
// without the per-row bound computation.  Entry = (pixel index, weight).
// ---------------------------------------------------------------------------
template <bool FILL>
__device__ __forceinline__ int ray_walk(const float4 o, int i, int N, int2 *out) {
  int ylo, yhi;
  ray_rows(o, i, N, ylo, yhi);
  const float fi = (float)i, fim = (float)(i - 1), fip = (float)(i + 1);
  int n = 0;
  for (int y = ylo; y <= yhi; ++y) {
    const float d = __fadd_rn(__fmul_rn((float)y, o.y), o.z);
    int xl, xh;
    if (o.x == 0.f) {
      if (d > fim && d < fip) { xl = 0; xh = N - 1; } else continue;
    } else if (o.x > 0.f) {
      xl = __float2int_rz(__fmul_rn(__fsub_rn(fim, d), o.w));
      xh = __float2int_rz(__fmul_rn(__fsub_rn(fip, d), o.w));
    } else {
      xl = __float2int_rz(__fmul_rn(__fsub_rn(fip, d), o.w));
      xh = __float2int_rz(__fmul_rn(__fsub_rn(fim, d), o.w));
    }
    xl = max(xl, 0);
    xh = min(xh, N - 1);
    for (int x = xl; x <= xh; ++x) {
      const float wgt = 1.0f - fabsf(__fsub_rn(__fadd_rn(__fmul_rn((float)x, o.x), d), fi));
      if (wgt > 0.f) {
        if (FILL) out[n] = make_int2(y * N + x, __float_as_int(wgt));
        ++n;
      }
    }
  }
  return n;
}

__global__ void k_ray_count(const float4 *__restrict__ ofs, int N, int nd, int nang, int *__restrict__ count) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nd * nang) return;
  const int j = t / nd, i = t - j * nd;
  count[t] = ray_walk<false>(__ldg(ofs + j), i, N, nullptr);
}

__global__ void k_ray_fill(const float4 *__restrict__ ofs, int N, int nd, int nang, const long long *__restrict__ start,
                           int2 *__restrict__ ent) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nd * nang) return;
  const int j = t / nd, i = t - j * nd;
  ray_walk<true>(__ldg(ofs + j), i, N, ent + start[t]);
}

// Run table: the rays of three adjacent bins i0, i0+1, i0+2 of one angle walked
// together.  Per row the union of their x ranges is listed once, each pixel with
// its three weights (zero where the bin's hat does not cover it), in the rows-
// then-x order of the reference; a pixel is loaded once for the three bins.
// Every weight is the one ray_walk computes for that bin, and a zero weight adds
// an exact zero, so each bin's sum is the ray table's, term for term.
template <bool FILL>
__device__ __forceinline__ int run_walk(const float4 o, int i0, int N, int nd, int4 *out) {
  int ylo, yhi, ylo2, yhi2;
  ray_rows(o, i0, N, ylo, yhi);
  ray_rows(o, min(i0 + 2, nd - 1), N, ylo2, yhi2);
  ylo = min(ylo, ylo2);
  yhi = max(yhi, yhi2);
  int n = 0;
  for (int y = ylo; y <= yhi; ++y) {
    const float d = __fadd_rn(__fmul_rn((float)y, o.y), o.z);
    int xl[3], xh[3];
    int xmin = N, xmax = -1;
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      const int i = i0 + r;
      const float fim = (float)(i - 1), fip = (float)(i + 1);
      int a, b;
      if (o.x == 0.f) {
        if (d > fim && d < fip) { a = 0; b = N - 1; } else { a = N; b = -1; }
      } else if (o.x > 0.f) {
        a = __float2int_rz(__fmul_rn(__fsub_rn(fim, d), o.w));
        b = __float2int_rz(__fmul_rn(__fsub_rn(fip, d), o.w));
      } else {
        a = __float2int_rz(__fmul_rn(__fsub_rn(fip, d), o.w));
        b = __float2int_rz(__fmul_rn(__fsub_rn(fim, d), o.w));
      }
      a = max(a, 0);
      b = min(b, N - 1);
      if (i >= nd) { a = N; b = -1; }
      xl[r] = a;
      xh[r] = b;
      if (a <= b) { xmin = min(xmin, a); xmax = max(xmax, b); }
    }
    for (int x = xmin; x <= xmax; ++x) {
      const float tx = __fadd_rn(__fmul_rn((float)x, o.x), d);
      float w[3];
      bool any = false;
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        const float wr = 1.0f - fabsf(__fsub_rn(tx, (float)(i0 + r)));
        w[r] = (x >= xl[r] && x <= xh[r] && wr > 0.f) ? wr : 0.f;
        any = any || w[r] > 0.f;
      }
      if (any) {
        if (FILL) out[n] = make_int4(y * N + x, __float_as_int(w[0]), __float_as_int(w[1]), __float_as_int(w[2]));
        ++n;
      }
    }
  }
  return n;
}

__global__ void k_run_count(const float4 *__restrict__ ofs, int N, int nd, int nang, int *__restrict__ count) {
  const int nq = (nd + 2) / 3;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nq * nang) return;
  const int j = t / nq, q = t - j * nq;
  count[t] = run_walk<false>(__ldg(ofs + j), 3 * q, N, nd, nullptr);
}

__global__ void k_run_fill(const float4 *__restrict__ ofs, int N, int nd, int nang, const long long *__restrict__ start,
                           int4 *__restrict__ ent) {
  const int nq = (nd + 2) / 3;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nq * nang) return;
  const int j = t / nq, q = t - j * nq;
  run_walk<true>(__ldg(ofs + j), 3 * q, N, nd, ent + start[t]);
}

// acc += w * v per slice: the reference's separately rounded product and sum
// (EXACT), or one fused multiply-add (the solver's hot loops)
template <bool EXACT>
__device__ __forceinline__ float mac(float acc, float w, float v) {
  return EXACT ? __fadd_rn(acc, __fmul_rn(w, v)) : __fmaf_rn(w, v, acc);
}

template <int VW, bool EXACT, int UNR, class SL>
__device__ __forceinline__ void radon_table(const float *__restrict__ img, size_t S, const int2 *__restrict__ ent,
                                            int n, const SL &sl, float (&acc)[VW]) {
#pragma unroll
  for (int k = 0; k < VW; ++k) acc[k] = 0.f;
  // groups of UNR entries; the next group's entries are fetched while the current
  // group's pixel loads are in flight (the entry -> pixel dependency is hidden)
  int2 nx[UNR];
#pragma unroll
  for (int u = 0; u < UNR; ++u) nx[u] = u < n ? __ldg(ent + u) : make_int2(0, 0);
  int e = 0;
  for (; e + UNR <= n; e += UNR) {
    int2 en[UNR];
#pragma unroll
    for (int u = 0; u < UNR; ++u) en[u] = nx[u];
    float v[UNR][VW];
#pragma unroll
    for (int u = 0; u < UNR; ++u) sl.load(img + (size_t)en[u].x * S, v[u]);
#pragma unroll
    for (int u = 0; u < UNR; ++u) nx[u] = (e + UNR + u < n) ? __ldg(ent + e + UNR + u) : make_int2(0, 0);
#pragma unroll
    for (int u = 0; u < UNR; ++u) {
      const float w = __int_as_float(en[u].y);
#pragma unroll
      for (int k = 0; k < VW; ++k) acc[k] = mac<EXACT>(acc[k], w, v[u][k]);
    }
  }
  // remainder: its entries are already in nx
#pragma unroll
  for (int u = 0; u < UNR - 1; ++u) {
    if (e + u < n) {
      float va[VW];
      sl.load(img + (size_t)nx[u].x * S, va);
      const float wa = __int_as_float(nx[u].y);
#pragma unroll
      for (int k = 0; k < VW; ++k) acc[k] = mac<EXACT>(acc[k], wa, va[k]);
    }
  }
}

// k_fwd: radon of ubar fused with update_lambda_KL (3-D :690-704) or _L2 (:677-688).
template <int DISC, int VW, int UNR, bool WL = false>
__device__ __forceinline__ void fwd_body(const IterParams &P, long long bid) {
  const Dims d = P.d;
  long long unit;
  typename std::conditional<WL, SlicesWL, Slices<VW>>::type sl;
  if constexpr (WL) {
    static_assert(VW == 1, "one slice per lane");
    if (!map_thread_wl((long long)d.nd * d.nang, d.S, unit, sl)) return;
  } else {
    if (!map_thread<VW>(bid, (long long)d.nd * d.nang, d.S, unit, sl)) return;
  }
  const int b = (int)unit;
  const int j = b / d.nd, i = b - j * d.nd;
  float acc[VW];
  if (P.ray_start) {
    const long long r0 = __ldg(P.ray_start + b), r1 = __ldg(P.ray_start + b + 1);
    radon_table<VW, false, UNR>(P.ubar, d.S, P.ray_ent + r0, (int)(r1 - r0), sl, acc);
  } else if constexpr (!WL) {
    radon_ray<VW>(P.ubar, d.S, d.N, __ldg(P.ofs + j), i, sl, acc);
  } else {
    acc[0] = 0.f;  // not reached: the launcher offers the WL shape only with the ray table
  }
  const size_t q = (size_t)b * d.S;
  sl.store(P.ku + q, acc);
  float lam[VW], f[VW];
  sl.loadw(P.lam + q, lam);
  sl.load(P.f + q, f);
  const float sd = P.sigma_data;
#pragma unroll
  for (int k = 0; k < VW; ++k) {
    const float m = sl.valid(k) ? __ldg(P.mu + sl.slice(k) / d.Nz) : 0.f;
    if (DISC == KL) {
      const float sv = lam[k] + sd * acc[k];
      const float wv = sv - m;
      const float dv = wv * wv + 4.f * sd * f[k] * m;
      lam[k] = sv - 0.5f * (wv + sqrtf(dv));
    } else {
      lam[k] = (lam[k] + sd * (acc[k] - f[k])) * m;
    }
  }
  sl.store(P.lam + q, lam);
}

template <int DISC, int VW, int UNR, bool WL = false, int MINB = 1>
__global__ void __launch_bounds__(256, MINB) k_fwd(const IterParams P) {
  fwd_body<DISC, VW, UNR, WL>(P, blockIdx.x);
}

// ===========================================================================
// back projection: kernel `radon_ad` (3-D :818-844): linear interpolation
// between detector bins floor(t) and floor(t)+1 at t = dot((x, y, 1, 0), ofs[j]).
// ===========================================================================
template <int VW, bool EXACT = true, int AU = 1, class SL = Slices<VW>, int UA = 2>
__device__ __forceinline__ void radon_ad_pixel(const float *__restrict__ lam, size_t S, int nd, int nang,
                                               const float4 *__restrict__ ofs, float xf, float yf,
                                               const SL &sl, float (&acc)[VW]) {
#pragma unroll
  for (int k = 0; k < VW; ++k) acc[k] = 0.f;
  const float fnd = (float)nd;
  int j = 0;
  if constexpr (AU == 1) {
    // one angle at a time, taps accumulated as they arrive (the compiler overlaps
    // consecutive angles)
#pragma unroll UA
    for (; j < nang; ++j) {
      const float4 o = __ldg(ofs + j);
      const float tt = __fadd_rn(__fadd_rn(__fmul_rn(xf, o.x), __fmul_rn(yf, o.y)), o.z);
      if (tt > -1.f && tt < fnd) {
        const float fl = floorf(tt);
        const float p = fminf(__fsub_rn(tt, fl), 0x1.fffffep-1f);
        const float q = __fsub_rn(1.0f, p);
        const int il = (int)fl;
        const float *lj = lam + (size_t)j * nd * S;
        float a[VW], b[VW];
        if (il >= 0) {
          sl.load(lj + (size_t)il * S, a);
#pragma unroll
          for (int k = 0; k < VW; ++k) acc[k] = EXACT ? __fadd_rn(acc[k], __fmul_rn(q, a[k])) : __fmaf_rn(q, a[k], acc[k]);
        }
        if (il <= nd - 2) {
          sl.load(lj + (size_t)(il + 1) * S, b);
#pragma unroll
          for (int k = 0; k < VW; ++k) acc[k] = EXACT ? __fadd_rn(acc[k], __fmul_rn(p, b[k])) : __fmaf_rn(p, b[k], acc[k]);
        }
      }
    }
  } else {
  // AU angles per step: their taps are loaded together, then accumulated in angle order
  for (; j + AU <= nang; j += AU) {
    int il[AU];
    float p[AU];
    bool ta[AU], tb[AU];
    float a[AU][VW], b[AU][VW];
#pragma unroll
    for (int u = 0; u < AU; ++u) {
      const float4 o = __ldg(ofs + j + u);
      const float tt = __fadd_rn(__fadd_rn(__fmul_rn(xf, o.x), __fmul_rn(yf, o.y)), o.z);
      const bool in = tt > -1.f && tt < fnd;
      const float fl = floorf(tt);
      p[u] = fminf(__fsub_rn(tt, fl), 0x1.fffffep-1f);
      il[u] = (int)fl;
      ta[u] = in && il[u] >= 0;
      tb[u] = in && il[u] <= nd - 2;
      const float *lj = lam + (size_t)(j + u) * nd * S;
      if (ta[u]) sl.load(lj + (size_t)il[u] * S, a[u]);
      if (tb[u]) sl.load(lj + (size_t)(il[u] + 1) * S, b[u]);
    }
#pragma unroll
    for (int u = 0; u < AU; ++u) {
      const float q = __fsub_rn(1.0f, p[u]);
      if (ta[u]) {
#pragma unroll
        for (int k = 0; k < VW; ++k) acc[k] = EXACT ? __fadd_rn(acc[k], __fmul_rn(q, a[u][k])) : __fmaf_rn(q, a[u][k], acc[k]);
      }
      if (tb[u]) {
#pragma unroll
        for (int k = 0; k < VW; ++k) acc[k] = EXACT ? __fadd_rn(acc[k], __fmul_rn(p[u], b[u][k])) : __fmaf_rn(p[u], b[u][k], acc[k]);
      }
    }
  }
  for (; j < nang; ++j) {
    const float4 o = __ldg(ofs + j);
    const float tt = __fadd_rn(__fadd_rn(__fmul_rn(xf, o.x), __fmul_rn(yf, o.y)), o.z);
    if (tt > -1.f && tt < fnd) {
      const float fl = floorf(tt);
      const float p = fminf(__fsub_rn(tt, fl), 0x1.fffffep-1f);
      const float q = __fsub_rn(1.0f, p);
      const int il = (int)fl;
      const float *lj = lam + (size_t)j * nd * S;
      float a[VW], b[VW];
      if (il >= 0) {
        sl.load(lj + (size_t)il * S, a);
#pragma unroll
        for (int k = 0; k < VW; ++k) acc[k] = EXACT ? __fadd_rn(acc[k], __fmul_rn(q, a[k])) : __fmaf_rn(q, a[k], acc[k]);
      }
      if (il <= nd - 2) {
        sl.load(lj + (size_t)(il + 1) * S, b);
#pragma unroll
        for (int k = 0; k < VW; ++k) acc[k] = EXACT ? __fadd_rn(acc[k], __fmul_rn(p, b[k])) : __fmaf_rn(p, b[k], acc[k]);
      }
    }
  }
  }
}

// Back-projection table: per (pixel, angle) the detector bin floor(t) and the
// interpolation fraction p of radon_ad (3-D :832-839), computed once per problem
// with the reference's arithmetic; il = INT_MIN marks t outside (-1, nd).
__global__ void k_bp_table(const float4 *__restrict__ ofs, int N, int nd, int nang, int2 *__restrict__ tab) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)N * N * nang) return;
  const int pix = (int)(t / nang), j = (int)(t - (long long)pix * nang);
  const int y = pix / N, x = pix - y * N;
  const float4 o = __ldg(ofs + j);
  const float tt = __fadd_rn(__fadd_rn(__fmul_rn((float)x, o.x), __fmul_rn((float)y, o.y)), o.z);
  int2 e = make_int2(INT_MIN, 0);
  if (tt > -1.f && tt < (float)nd) {
    const float fl = floorf(tt);
    e = make_int2((int)fl, __float_as_int(fminf(__fsub_rn(tt, fl), 0x1.fffffep-1f)));
  }
  tab[t] = e;
}

template <int VW, bool EXACT>
__device__ __forceinline__ void bp_tap(float (&acc)[VW], float w, const float (&v)[VW]) {
#pragma unroll
  for (int k = 0; k < VW; ++k) acc[k] = mac<EXACT>(acc[k], w, v[k]);
}

template <int VW, bool EXACT, int AU, class SL>
__device__ __forceinline__ void radon_ad_table(const float *__restrict__ lam, size_t S, int nd, int nang,
                                               const int2 *__restrict__ tab, const SL &sl,
                                               float (&acc)[VW]) {
#pragma unroll
  for (int k = 0; k < VW; ++k) acc[k] = 0.f;
  const size_t jstride = (size_t)nd * S;
  int j = 0;
  if (AU == 2) {
    for (; j + 2 <= nang; j += 2) {  // two angles (four taps) in flight, accumulated in order
      const int2 e0 = __ldg(tab + j), e1 = __ldg(tab + j + 1);
      float a0[VW], b0[VW], a1[VW], b1[VW];
      const float *l0 = lam + (size_t)j * jstride, *l1 = l0 + jstride;
      const bool in0 = e0.x != INT_MIN, in1 = e1.x != INT_MIN;
      const bool ta0 = in0 && e0.x >= 0, tb0 = in0 && e0.x <= nd - 2;
      const bool ta1 = in1 && e1.x >= 0, tb1 = in1 && e1.x <= nd - 2;
      if (ta0) sl.load(l0 + (size_t)e0.x * S, a0);
      if (tb0) sl.load(l0 + (size_t)(e0.x + 1) * S, b0);
      if (ta1) sl.load(l1 + (size_t)e1.x * S, a1);
      if (tb1) sl.load(l1 + (size_t)(e1.x + 1) * S, b1);
      const float p0 = __int_as_float(e0.y), p1 = __int_as_float(e1.y);
      if (ta0) bp_tap<VW, EXACT>(acc, __fsub_rn(1.0f, p0), a0);
      if (tb0) bp_tap<VW, EXACT>(acc, p0, b0);
      if (ta1) bp_tap<VW, EXACT>(acc, __fsub_rn(1.0f, p1), a1);
      if (tb1) bp_tap<VW, EXACT>(acc, p1, b1);
    }
  }
  for (; AU > 2 && j + AU <= nang; j += AU) {  // AU angles (2 AU taps) in flight, accumulated in order
    int2 e[AU];
#pragma unroll
    for (int u = 0; u < AU; ++u) e[u] = __ldg(tab + j + u);
    float a[AU][VW], b[AU][VW];
    bool ta[AU], tb[AU];
#pragma unroll
    for (int u = 0; u < AU; ++u) {
      const bool in = e[u].x != INT_MIN;
      ta[u] = in && e[u].x >= 0;
      tb[u] = in && e[u].x <= nd - 2;
      const float *l = lam + (size_t)(j + u) * jstride;
      if (ta[u]) sl.load(l + (size_t)e[u].x * S, a[u]);
      if (tb[u]) sl.load(l + (size_t)(e[u].x + 1) * S, b[u]);
    }
#pragma unroll
    for (int u = 0; u < AU; ++u) {
      const float p = __int_as_float(e[u].y);
      if (ta[u]) bp_tap<VW, EXACT>(acc, __fsub_rn(1.0f, p), a[u]);
      if (tb[u]) bp_tap<VW, EXACT>(acc, p, b[u]);
    }
  }
  for (; j < nang; ++j) {
    const int2 e0 = __ldg(tab + j);
    if (e0.x != INT_MIN) {
      const float *l0 = lam + (size_t)j * jstride;
      const float p0 = __int_as_float(e0.y);
      float a0[VW], b0[VW];
      if (e0.x >= 0) { sl.load(l0 + (size_t)e0.x * S, a0); bp_tap<VW, EXACT>(acc, __fsub_rn(1.0f, p0), a0); }
      if (e0.x <= nd - 2) { sl.load(l0 + (size_t)(e0.x + 1) * S, b0); bp_tap<VW, EXACT>(acc, p0, b0); }
    }
  }
}

// update_u (3-D :706-729, 2-D :340-357) + update_p (3-D :734-757, 2-D :359-376) +
// extrapolation and swap (:1217-1221) for UW consecutive slices from s0.
// PART selects the halves: PART_U the u / ubar half (needs K* lambda), PART_P the
// p / pbar half (needs only the dual kernel's v and w), PART_ALL both.  Each half
// computes its values by the same operations whichever way it is launched.
enum { PART_ALL = 0, PART_U = 1, PART_P = 2 };
template <int DIM, bool TGV, int UW, int PART = PART_ALL>
__device__ __forceinline__ void primal_update(const IterParams &P, int x, int y, int s0, const float (&kstar)[UW]) {
  const Dims d = P.d;
  const size_t S = d.S, rowS = (size_t)d.N * S, vol = d.vol, i = ((size_t)y * d.N + x) * S + s0;
  int z[UW];
#pragma unroll
  for (int k = 0; k < UW; ++k) z[k] = (DIM == 3) ? (s0 + k) % d.Nz : 0;
  const float *__restrict__ v = P.v;

  if (PART != PART_P) {
  // divergence of v: backward differences (adjoint of the forward gradient)
  float a[UW], b[UW], am[UW], bm[UW], uo[UW], un[UW], ub[UW];
  ldw<UW>(v + i, a);
  ldw<UW>(v + vol + i, b);
  if (x > 0) ldw<UW>(v + i - S, am);
  if (y > 0) ldw<UW>(v + vol + i - rowS, bm);
  ldw<UW>(P.u + i, uo);
  float c[UW], cprev = 0.f;
  if (DIM == 3) {
    ldw<UW>(v + 2 * vol + i, c);
    if (z[0] > 0) cprev = v[2 * vol + i - 1];
  }
  float lo[UW], lon[UW];  // the low parts of u (precise primal mode, P.ulo set)
  if (P.ulo) ldw<UW>(P.ulo + i, lo);
#pragma unroll
  for (int k = 0; k < UW; ++k) {
    float ak = a[k], bk = b[k];
    if (x == d.N - 1) ak = 0.f;
    if (x > 0) ak -= am[k];
    if (y == d.N - 1) bk = 0.f;
    if (y > 0) bk -= bm[k];
    float sum;
    if (DIM == 3) {
      float ck = c[k];
      if (z[k] == d.Nz - 1) ck = 0.f;
      if (z[k] > 0) ck -= (k > 0 ? c[k - 1] : cprev);
      ck /= P.stepsize;
      sum = ak + bk + ck - P.norming * kstar[k];
    } else {
      sum = ak + bk - P.norming * kstar[k];
    }
    if (!P.ulo) {  // the reference's update (one rounding of u + tau sum)
      float r = uo[k] + P.tau * sum;
      if (r < 0.f) r = 0.f;
      un[k] = r;
      ub[k] = 2.0f * r - uo[k];
    } else {
      // u held as uo + lo (two floats): the step is added to the low part and
      // the pair renormalised by TwoSum (Knuth), so steps below half an ulp of u
      // are kept instead of absorbed
      const float t = lo[k] + P.tau * sum;
      const float r = __fadd_rn(uo[k], t);
      const float bv = __fsub_rn(r, uo[k]);
      const float e = __fadd_rn(__fsub_rn(uo[k], __fsub_rn(r, bv)), __fsub_rn(t, bv));
      const bool neg = r < 0.f || (r == 0.f && e < 0.f);
      un[k] = neg ? 0.f : r;
      lon[k] = neg ? 0.f : e;
      ub[k] = (2.0f * un[k] - uo[k]) + (2.0f * lon[k] - lo[k]);
    }
  }
  stv<UW>(P.ubar + i, ub);
  stv<UW>(P.u + i, un);
  if (P.ulo) stv<UW>(P.ulo + i, lon);
  }

  if (TGV && PART != PART_U) {
    const float *__restrict__ w = P.w;
    constexpr int K = DIM;
    // rows of the symmetric tensor: 3-D (w0 w3 w4), (w3 w1 w5), (w4 w5 w2); 2-D (w0 w2), (w2 w1)
    const int rx[3] = {0, DIM == 3 ? 3 : 2, 4}, ry[3] = {DIM == 3 ? 3 : 2, 1, 5}, rz[3] = {4, 5, 2};
#pragma unroll
    for (int k = 0; k < K; ++k) {
      float wa[UW], wan[UW], wb[UW], wbn[UW], po[UW], vk[UW], pn[UW], pb[UW];
      ldw<UW>(w + rx[k] * vol + i, wa);
      ldw<UW>(w + ry[k] * vol + i, wb);
      if (x < d.N - 1) ldw<UW>(w + rx[k] * vol + i + S, wan);
      if (y < d.N - 1) ldw<UW>(w + ry[k] * vol + i + rowS, wbn);
      ldw<UW>(P.p + k * vol + i, po);
      ldw<UW>(v + k * vol + i, vk);
      float wc[UW], wcnext = 0.f;
      if (DIM == 3) {
        ldw<UW>(w + rz[k] * vol + i, wc);
        if (z[UW - 1] < d.Nz - 1) wcnext = w[rz[k] * vol + i + UW];
      }
#pragma unroll
      for (int e = 0; e < UW; ++e) {
        float A = -wa[e], B = -wb[e];
        if (x == 0) A = 0.f;
        if (x < d.N - 1) A += wan[e];
        if (y == 0) B = 0.f;
        if (y < d.N - 1) B += wbn[e];
        float r;
        if (DIM == 3) {
          r = p_step3(po[e], vk[e], wa[e], wan[e], wb[e], wbn[e], wc[e], e < UW - 1 ? wc[e + 1] : wcnext, x == 0,
                      x < d.N - 1, y == 0, y < d.N - 1, z[e] == 0, z[e] < d.Nz - 1, P.tau, P.stepsize);
        } else {
          r = po[e] + P.tau * (vk[e] + A + B);
        }
        pn[e] = r;
        pb[e] = 2.0f * r - po[e];
      }
      stv<UW>(P.pbar + k * vol + i, pb);
      stv<UW>(P.p + k * vol + i, pn);
    }
  }
}

// Back projection of R consecutive pixels of one row at once.  Along a row the
// detector coordinate moves by X = cos(angle) per pixel (|X| <= 1), so the R
// pixels' taps span about R|X| + 2 bins: the pixels are visited in the order in
// which their bins increase and the two current taps slide along, each bin loaded
// once per angle.  Every pixel adds its taps in the reference's order (angles
// ascending, lower tap then upper tap) with the reference's interpolation weights.
template <int VW, int R, bool REV>
__device__ __forceinline__ void bp_run_angle(const float *__restrict__ lj, size_t S, int nd, float fnd, const float4 o,
                                             int x0, float yf, int N, const Slices<VW> &sl, float (&acc)[R][VW]) {
  int cur = -3;  // bins held: A = cur, B = cur + 1
  float A[VW], Bv[VW];
#pragma unroll
  for (int k = 0; k < VW; ++k) { A[k] = 0.f; Bv[k] = 0.f; }
#pragma unroll
  for (int rr = 0; rr < R; ++rr) {
    const int r = REV ? R - 1 - rr : rr;
    if (x0 + r >= N) continue;
    const float xf = (float)(x0 + r);
    const float tt = __fadd_rn(__fadd_rn(__fmul_rn(xf, o.x), __fmul_rn(yf, o.y)), o.z);
    if (!(tt > -1.f && tt < fnd)) continue;
    const float fl = floorf(tt);
    const float p = fminf(__fsub_rn(tt, fl), 0x1.fffffep-1f);
    const float q = __fsub_rn(1.0f, p);
    const int il = (int)fl;
    if (il != cur) {
      if (il == cur + 1) {
#pragma unroll
        for (int k = 0; k < VW; ++k) A[k] = Bv[k];
      } else if (il >= 0) {
        sl.load(lj + (size_t)il * S, A);
      }
      if (il <= nd - 2) sl.load(lj + (size_t)(il + 1) * S, Bv);
      cur = il;
    }
    if (il >= 0) {
#pragma unroll
      for (int k = 0; k < VW; ++k) acc[r][k] = __fmaf_rn(q, A[k], acc[r][k]);
    }
    if (il <= nd - 2) {
#pragma unroll
      for (int k = 0; k < VW; ++k) acc[r][k] = __fmaf_rn(p, Bv[k], acc[r][k]);
    }
  }
}

template <int VW, int R>
__global__ void __launch_bounds__(256) k_bp_run(const IterParams P) {
  const Dims d = P.d;
  const int nrun = (d.N + R - 1) / R;
  long long unit;
  Slices<VW> sl;
  if (!map_thread<VW>((long long)d.N * nrun, d.S, unit, sl)) return;
  const int y = (int)(unit / nrun), x0 = (int)(unit - (long long)y * nrun) * R;
  float acc[R][VW];
#pragma unroll
  for (int r = 0; r < R; ++r)
#pragma unroll
    for (int k = 0; k < VW; ++k) acc[r][k] = 0.f;
  const float fnd = (float)d.nd, yf = (float)y;
  for (int j = 0; j < d.nang; ++j) {
    const float4 o = __ldg(P.ofs + j);
    const float *lj = P.lam + (size_t)j * d.nd * d.S;
    if (o.x < 0.f) bp_run_angle<VW, R, true>(lj, d.S, d.nd, fnd, o, x0, yf, d.N, sl, acc);
    else bp_run_angle<VW, R, false>(lj, d.S, d.nd, fnd, o, x0, yf, d.N, sl, acc);
  }
#pragma unroll
  for (int r = 0; r < R; ++r)
    if (x0 + r < d.N) sl.store(P.kstar + ((size_t)y * d.N + x0 + r) * d.S, acc[r]);
}

// k_bp: back projection K* lambda of every (pixel, slice) into P.kstar; it only
// needs lambda, so it runs beside k_dual.
template <int VW, int AU, bool TAB, bool WL = false, int UA = 2>
__device__ __forceinline__ void bp_body(const IterParams &P, long long bid) {
  const Dims d = P.d;
  long long unit;
  typename std::conditional<WL, SlicesWL, Slices<VW>>::type sl;
  if constexpr (WL) {
    static_assert(VW == 1 && !TAB, "one slice per lane, geometry on the fly");
    if (!map_thread_wl((long long)d.N * d.N, d.S, unit, sl)) return;
  } else {
    if (!map_thread<VW>(bid, (long long)d.N * d.N, d.S, unit, sl)) return;
  }
  const int pix = (int)unit;
  float acc[VW];
  if (TAB && P.bp_tab) {
    radon_ad_table<VW, false, AU>(P.lam, d.S, d.nd, d.nang, P.bp_tab + (size_t)pix * d.nang, sl, acc);
  } else {
    const int y = pix / d.N, x = pix - y * d.N;
    radon_ad_pixel<VW, false, AU, decltype(sl), UA>(P.lam, d.S, d.nd, d.nang, P.ofs, (float)x, (float)y, sl, acc);
  }
  sl.store(P.kstar + (size_t)pix * d.S, acc);
}

template <int VW, int AU, bool TAB, bool WL = false, int UA = 2>
__global__ void __launch_bounds__(256) k_bp(const IterParams P) {
  bp_body<VW, AU, TAB, WL, UA>(P, blockIdx.x);
}

// k_bp_tma: back projection with the sinogram rows a pixel tile needs staged in
// shared memory by TMA.  A block owns an 8 x 8 pixel tile and 128 slices (one
// float4 per lane); per angle the tile's taps fall on at most 13 consecutive
// bins (the detector coordinate moves by |cos| + |sin| <= 1.4143 per pixel step),
// so one 16-bin x 128-slice box of lambda is copied per angle into a 4-stage ring
// while the previous angles are summed.  Warp w owns row y0 + w; lanes 0..7
// compute the geometry of the row's 8 pixels and broadcast it by shuffles, so
// the geometry is computed once per pixel and angle instead of once per slice
// group.  Every pixel adds its taps in the reference's order (angles ascending,
// lower tap then upper tap) with radon_ad's weights (3-D :832-839), as k_bp does,
// so the iterates are bit-identical.  Every wait on a copy is bounded: a block
// that gives up sets P.err, waits (bounded) for its copies in flight and leaves
// without storing.
constexpr int BPT_ST = 4, BPT_BINS = 16, BPT_TILE = 8;

// lowest bin the taps of the tile at (x0, y0) can touch for angle o: the floor of
// the smallest detector coordinate of the tile's corners, minus one for the
// rounding of interior pixels
__device__ __forceinline__ int bp_tile_lo(const float4 o, int x0, int y0) {
  float m = 3.0e38f;
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const float cx = (float)(x0 + (c & 1) * (BPT_TILE - 1)), cy = (float)(y0 + (c >> 1) * (BPT_TILE - 1));
    m = fminf(m, __fadd_rn(__fadd_rn(__fmul_rn(cx, o.x), __fmul_rn(cy, o.y)), o.z));
  }
  return (int)floorf(m) - 1;
}

template <int VW>
__device__ __forceinline__ void bpt_tap(float (&acc)[VW], float w, float4 a, float4 b) {
  acc[0] = __fmaf_rn(w, a.x, acc[0]); acc[1] = __fmaf_rn(w, a.y, acc[1]);
  acc[2] = __fmaf_rn(w, a.z, acc[2]); acc[3] = __fmaf_rn(w, a.w, acc[3]);
  if (VW == 8) {
    acc[4 % VW] = __fmaf_rn(w, b.x, acc[4 % VW]); acc[5 % VW] = __fmaf_rn(w, b.y, acc[5 % VW]);
    acc[6 % VW] = __fmaf_rn(w, b.z, acc[6 % VW]); acc[7 % VW] = __fmaf_rn(w, b.w, acc[7 % VW]);
  }
}

// VW = 4: a block covers 128 slices (one float4 per lane); VW = 8: 256 slices (two
// float4 per lane, slices 4l.. and 128+4l.., as Slices<8>)
template <int VW>
__global__ void __launch_bounds__(256) k_bp_tma(const IterParams P, const __grid_constant__ CUtensorMap tm) {
  constexpr int SC = 32 * VW;
  extern __shared__ __align__(128) float stage[];  // [BPT_ST][BPT_BINS][SC]
  __shared__ __align__(8) uint64_t full[BPT_ST];
  const Dims d = P.d;
  const int ntx = (d.N + BPT_TILE - 1) / BPT_TILE;
  const int bid = blockIdx.x;
  const int tx = bid % ntx, ty = (bid / ntx) % ntx, ch = bid / (ntx * ntx);
  const int x0 = BPT_TILE * tx, y0 = BPT_TILE * ty, sb = ch * SC;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int y = y0 + warp;
  const int sa = sb + 4 * lane, sbb = sa + 128;  // this lane's float4 chunks (the second for VW = 8)
  const int nang = d.nang, nd = d.nd;
  const float fnd = (float)nd;
  constexpr uint32_t BOX = BPT_BINS * SC * sizeof(float);
  if (threadIdx.x == 0) {
    for (int k = 0; k < BPT_ST; ++k) mbar_init(&full[k], 1);
    mbar_init_fence();
  }
  __syncthreads();
  const uint32_t limit = P.bp_wait_limit;
  auto issue = [&](int j) {
    if (j == P.bp_skip_angle) return;  // test hook: a copy nothing completes
    const int st = j % BPT_ST;
    mbar_arrive_expect_tx(&full[st], BOX);
    tma_load_3d(stage + (size_t)st * BPT_BINS * SC, &tm, &full[st], sb, bp_tile_lo(__ldg(P.ofs + j), x0, y0), j);
  };
  if (threadIdx.x == 0)
    for (int j = 0; j < BPT_ST && j < nang; ++j) issue(j);

  float acc[BPT_TILE][VW];
#pragma unroll
  for (int r = 0; r < BPT_TILE; ++r)
#pragma unroll
    for (int k = 0; k < VW; ++k) acc[r][k] = 0.f;
  bool tmo = nang > 0 && !mbar_wait_bounded(&full[0], 0, limit);
  int j = 0;
  for (; j < nang; ++j) {
    // every thread has waited for angle j's copy; all have finished angle j - 1
    if (__syncthreads_or(tmo)) break;
    if (threadIdx.x == 0 && j >= 1 && j - 1 + BPT_ST < nang) issue(j - 1 + BPT_ST);  // into the freed stage
    const int st = j % BPT_ST;
    const float4 o = __ldg(P.ofs + j);
    const int lo = bp_tile_lo(o, x0, y0);
    const int xr = x0 + (lane & (BPT_TILE - 1));
    const float tt = __fadd_rn(__fadd_rn(__fmul_rn((float)xr, o.x), __fmul_rn((float)y, o.y)), o.z);
    const bool in = xr < d.N && y < d.N && tt > -1.f && tt < fnd;
    const float fl = floorf(tt);
    const float pw = fminf(__fsub_rn(tt, fl), 0x1.fffffep-1f);
    const int rel = in ? (int)fl - lo : INT_MIN;
    const float *srow = stage + (size_t)st * BPT_BINS * SC + 4 * lane;
#pragma unroll
    for (int r = 0; r < BPT_TILE; ++r) {
      const int rr = __shfl_sync(0xffffffffu, rel, r);
      const float p = __shfl_sync(0xffffffffu, pw, r);
      if (rr == INT_MIN) continue;  // pixel outside the image or the detector for this angle
      const float q = __fsub_rn(1.0f, p);
      const int il = rr + lo;
      const bool tlo = il >= 0, thi = il <= nd - 2;
      float4 a0 = make_float4(0.f, 0.f, 0.f, 0.f), a1 = a0, b0 = a0, b1 = a0;
      if (rr >= 0 && rr <= BPT_BINS - 2) {
        const float *ra = srow + rr * SC;
        if (tlo) {
          a0 = *reinterpret_cast<const float4 *>(ra);
          if (VW == 8) a1 = *reinterpret_cast<const float4 *>(ra + 128);
        }
        if (thi) {
          b0 = *reinterpret_cast<const float4 *>(ra + SC);
          if (VW == 8) b1 = *reinterpret_cast<const float4 *>(ra + SC + 128);
        }
      } else {  // outside the staged bins (not reached): read lambda directly
        const float *lj = P.lam + (size_t)j * nd * d.S;
        if (tlo && sa < d.S) a0 = *reinterpret_cast<const float4 *>(lj + (size_t)il * d.S + sa);
        if (tlo && VW == 8 && sbb < d.S) a1 = *reinterpret_cast<const float4 *>(lj + (size_t)il * d.S + sbb);
        if (thi && sa < d.S) b0 = *reinterpret_cast<const float4 *>(lj + (size_t)(il + 1) * d.S + sa);
        if (thi && VW == 8 && sbb < d.S) b1 = *reinterpret_cast<const float4 *>(lj + (size_t)(il + 1) * d.S + sbb);
      }
      if (tlo) bpt_tap<VW>(acc[r], q, a0, a1);
      if (thi) bpt_tap<VW>(acc[r], p, b0, b1);
    }
    if (j + 1 < nang) tmo = !mbar_wait_bounded(&full[(j + 1) % BPT_ST], ((j + 1) / BPT_ST) & 1, limit);
  }
  if (j < nang) {
    // gave up waiting for angle j: flag it, let the copies in flight (angles j ..
    // the last issued) land, leave without storing
    if (threadIdx.x == 0) {
      atomicExch(P.err, 1);
      const int last = min(nang - 1, j >= 2 ? j - 2 + BPT_ST : BPT_ST - 1);
      for (int a = j; a <= last; ++a) mbar_wait_bounded(&full[a % BPT_ST], (a / BPT_ST) & 1, limit);
    }
    return;
  }
  if (y < d.N) {
#pragma unroll
    for (int r = 0; r < BPT_TILE; ++r) {
      if (x0 + r >= d.N) continue;
      float *o = P.kstar + ((size_t)y * d.N + x0 + r) * d.S;
      if (sa < d.S) *reinterpret_cast<float4 *>(o + sa) = make_float4(acc[r][0], acc[r][1], acc[r][2], acc[r][3]);
      if (VW == 8 && sbb < d.S)
        *reinterpret_cast<float4 *>(o + sbb) =
            make_float4(acc[r][4 % VW], acc[r][5 % VW], acc[r][6 % VW], acc[r][7 % VW]);
    }
  }
}

template <int VW>
static void bp_tma(const IterParams &P, cudaStream_t st) {
  constexpr int SC = 32 * VW;
  const int ntx = (P.d.N + BPT_TILE - 1) / BPT_TILE;
  const unsigned g = (unsigned)ntx * ntx * ((P.d.S + SC - 1) / SC);
  const size_t smem = (size_t)BPT_ST * BPT_BINS * SC * sizeof(float);
  k_bp_tma<VW><<<g, 256, smem, st>>>(P, *static_cast<const CUtensorMap *>(VW == 8 ? P.bp_tmap_wide : P.bp_tmap));
}

// shared-memory limits of the TMA back projection (64 KB of stages for 256-slice
// boxes), set once per problem on its device before any launch or capture
cudaError_t prepare_bp_tma() {
  return cudaFuncSetAttribute(k_bp_tma<8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)((size_t)BPT_ST * BPT_BINS * 256 * sizeof(float)));
}

// k_update: update_u + update_p + extrapolation for UW consecutive slices (PART:
// both halves, or one of them, see primal_update).
template <int DIM, bool TGV, int UW, int PART = PART_ALL>
__device__ __forceinline__ void update_body(const IterParams &P, long long bid) {
  const Dims d = P.d;
  const int nsg = d.S / UW;
  const long long t = bid * blockDim.x + threadIdx.x;
  if (t >= (long long)d.N * d.N * nsg) return;
  const int pix = (int)(t / nsg);
  const int s0 = (int)(t - (long long)pix * nsg) * UW;
  const int y = pix / d.N, x = pix - y * d.N;
  float ks[UW];
  if (PART != PART_P) ldw<UW>(P.kstar + (size_t)pix * d.S + s0, ks);
  primal_update<DIM, TGV, UW, PART>(P, x, y, s0, ks);
}

template <int DIM, bool TGV, int UW, int PART = PART_ALL>
__global__ void __launch_bounds__(256) k_update(const IterParams P) {
  update_body<DIM, TGV, UW, PART>(P, blockIdx.x);
}

// ===========================================================================
// standalone projectors
// ===========================================================================
template <int VW>
__global__ void k_radon(const float *__restrict__ img, float *__restrict__ sino, const float4 *__restrict__ ofs,
                        int N, int nd, int nang, int S) {
  long long unit;
  Slices<VW> sl;
  if (!map_thread<VW>((long long)nd * nang, S, unit, sl)) return;
  const int b = (int)unit, j = b / nd, i = b - j * nd;
  float acc[VW];
  radon_ray<VW>(img, S, N, __ldg(ofs + j), i, sl, acc);
  sl.store(sino + (size_t)b * S, acc);
}

template <int VW>
__global__ void k_radon_ad(const float *__restrict__ sino, float *__restrict__ img, const float4 *__restrict__ ofs,
                           int N, int nd, int nang, int S) {
  long long unit;
  Slices<VW> sl;
  if (!map_thread<VW>((long long)N * N, S, unit, sl)) return;
  const int pix = (int)unit, y = pix / N, x = pix - y * N;
  float acc[VW];
  radon_ad_pixel<VW>(sino, S, nd, nang, ofs, (float)x, (float)y, sl, acc);
  sl.store(img + (size_t)pix * S, acc);
}

// out[c][r] = in[r][c]: host layout [S][X] <-> device layout [X][S], 32x32 tiles,
// one block per tile (1-D grid, so neither extent is limited to 65535 tiles)
__global__ void k_transpose(const float *__restrict__ in, float *__restrict__ out, int rows, int cols) {
  __shared__ float tile[32][33];
  const int tiles_c = (cols + 31) / 32;
  const int tr = blockIdx.x / tiles_c, tc = blockIdx.x - tr * tiles_c;
  const int bx = tc * 32, by = tr * 32;
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int r = by + k, c = bx + threadIdx.x;
    if (r < rows && c < cols) tile[k][threadIdx.x] = in[(size_t)r * cols + c];
  }
  __syncthreads();
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int r = bx + k, c = by + threadIdx.x;
    if (r < cols && c < rows) out[(size_t)r * rows + c] = tile[threadIdx.x][k];
  }
}

// Make_function_feasible (3-D :860-870): zero data where R 1 <= 0 (slice 0 mask)
__global__ void k_feasible(float *__restrict__ f, const float *__restrict__ r1, int nbin1, int S) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)nbin1 * S) return;
  if (r1[t / S] <= 0.f) f[t] = 0.f;
}

// Data dual consistent with a primal image: lambda at the fixed point of the
// lambda update for the given K u.  KL (update_lambda_KL, 3-D :690-704): the
// fixed point of lam = s - (s - mu + sqrt((s - mu)^2 + 4 sigma f mu)) / 2 with
// s = lam + sigma ku is lam = mu (1 - f / ku).  Where K u is zero or far below
// the data (f > 10 K u: the image misses counts there) that value is unbounded
// below and would throw the next primal step far off, so lambda is kept.
// L2 (update_lambda_L2, :677-688, weight m = mu / (sigma + mu)): lam = mu (ku - f).
__global__ void k_lambda_fixed(float *__restrict__ lam, const float *__restrict__ ku, const float *__restrict__ f,
                               const double *__restrict__ mu, long long nbin, int S, int Nz, int disc,
                               float empty_weight, float cap) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nbin * S) return;
  const int s = (int)(t % S);
  const float m = (float)mu[s / Nz], k = ku[t], fv = f[t];
  if (fv == 0.f && empty_weight < 1.f) {  // bins without data move only part of the way to mu
    if (disc == 0 && k > 0.f) lam[t] = lam[t] + empty_weight * (m - lam[t]);
    if (disc != 0) lam[t] = lam[t] + empty_weight * (m * k - lam[t]);
    return;
  }
  if (disc == 0) {
    if (k > 0.f && fv <= 10.f * k) lam[t] = m * (1.0f - fv / k);
    else if (cap > 0.f && fv > 0.f) lam[t] = m * (1.0f - cap);  // f / K u capped: a strong push up the ray
  } else {
    lam[t] = m * (k - fv);
  }
}

// Rays the image misses: r = f / N where the data has counts (f > 0) but K u = 0,
// else 0.  Back-projected and added to u, it makes K u > 0 on those bins (about
// f / 2 there) so that the KL data term, and with it the primal value, is finite.
__global__ void k_missed_rays(const float *__restrict__ ku, const float *__restrict__ f, float *__restrict__ r,
                              long long n, float inv_n) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  r[t] = (f[t] > 0.f && !(ku[t] > 0.f)) ? f[t] * inv_n : 0.f;
}

__global__ void k_add2(float *__restrict__ a, float *__restrict__ b, const float *__restrict__ d, long long n) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  a[t] += d[t];
  b[t] += d[t];
}

cudaError_t launch_missed_rays(const float *ku, const float *f, float *r, long long n, int N, cudaStream_t st) {
  k_missed_rays<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(ku, f, r, n, 1.f / (float)N);
  return cudaGetLastError();
}

cudaError_t launch_add2(float *a, float *b, const float *d, long long n, cudaStream_t st) {
  k_add2<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(a, b, d, n);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// two-resolution subsampling (radon_tgv_primal_dual_3dsubsample.py)
// ---------------------------------------------------------------------------
// slices [s0, s0 + Sg) of a [X][S] field <-> a contiguous [X][Sg] field
__global__ void k_gather_slices(const float *__restrict__ src, int S, int s0, float *__restrict__ dst, int Sg,
                                long long X) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= X * Sg) return;
  const long long x = t / Sg;
  dst[t] = src[x * S + s0 + (t - x * Sg)];
}

__global__ void k_scatter_slices(const float *__restrict__ src, int Sg, float *__restrict__ dst, int S, int s0,
                                 long long X) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= X * Sg) return;
  const long long x = t / Sg;
  dst[x * S + s0 + (t - x * Sg)] = src[t];
}

// Sparsemultiplication (3dsubsample :403-428): for every angle j and channel c,
// out(x_o, z_o) = sum over the row (x_o + nx_o z_o) of the interpolation matrix of
// val * in(x_i, z_i), the column index being x_i + nx_i z_i; separately rounded
// products summed in entry order.  Layouts [(j nx + x)][c nz + z].
__global__ void k_csr_planes(const float *__restrict__ in, float *__restrict__ out, const int *__restrict__ start,
                             const int *__restrict__ idx, const float *__restrict__ val, int nang, int C, int nx_o,
                             int nz_o, int nx_i, int nz_i) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int So = C * nz_o, Si = C * nz_i;
  if (t >= (long long)nang * nx_o * So) return;
  const int s = (int)(t % So);
  const long long jx = t / So;
  const int x = (int)(jx % nx_o), j = (int)(jx / nx_o);
  const int c = s / nz_o, z = s - c * nz_o;
  const int row = x + nx_o * z;
  float sum = 0.f;
  for (int e = start[row]; e < start[row + 1]; ++e) {
    const int k1 = idx[e];
    const int zi = k1 / nx_i, xi = k1 - zi * nx_i;
    sum = __fadd_rn(sum, __fmul_rn(val[e], in[((size_t)j * nx_i + xi) * Si + c * nz_i + zi]));
  }
  out[t] = sum;
}

// update_lambda_KL / _L2 (3-D :677-704) on a sinogram [bins][S], channel s / Nz
__global__ void k_lambda_update(float *__restrict__ lam, const float *__restrict__ ku, const float *__restrict__ f,
                                const float *__restrict__ mu, float sigma, long long n, int S, int Nz, int disc) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const float m = mu[(int)(t % S) / Nz];
  if (disc == 0) {
    const float sv = lam[t] + sigma * ku[t];
    const float wv = sv - m;
    const float dv = wv * wv + 4 * sigma * f[t] * m;
    lam[t] = sv - 0.5f * (wv + sqrtf(dv));
  } else {
    lam[t] = (lam[t] + sigma * (ku[t] - f[t])) * m;
  }
}

// sum of squares in FP64, block partials
__global__ void k_sumsq_partial(const float *__restrict__ x, long long n, double *__restrict__ part) {
  __shared__ double sh[256];
  double a = 0.0;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const double v = x[k];
    a += v * v;
  }
  sh[threadIdx.x] = a;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

// sum of (a - b)^2 in FP64, block partials (restarted iterations: distance moved)
__global__ void k_sqdiff_partial(const float *__restrict__ a, const float *__restrict__ b, long long n,
                                 double *__restrict__ part) {
  __shared__ double sh[256];
  double acc = 0.0;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const double v = (double)a[k] - (double)b[k];
    acc += v * v;
  }
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

__global__ void k_scale_f32(float *__restrict__ x, long long n, float s) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) x[t] *= s;
}

cudaError_t launch_gather_slices(const float *src, int S, int s0, float *dst, int Sg, long long X, cudaStream_t st) {
  k_gather_slices<<<(unsigned)((X * Sg + 255) / 256), 256, 0, st>>>(src, S, s0, dst, Sg, X);
  return cudaGetLastError();
}
cudaError_t launch_scatter_slices(const float *src, int Sg, float *dst, int S, int s0, long long X, cudaStream_t st) {
  k_scatter_slices<<<(unsigned)((X * Sg + 255) / 256), 256, 0, st>>>(src, Sg, dst, S, s0, X);
  return cudaGetLastError();
}
cudaError_t launch_csr_planes(const float *in, float *out, const int *start, const int *idx, const float *val,
                              int nang, int C, int nx_o, int nz_o, int nx_i, int nz_i, cudaStream_t st) {
  k_csr_planes<<<(unsigned)(((long long)nang * nx_o * C * nz_o + 255) / 256), 256, 0, st>>>(in, out, start, idx, val, nang, C,
                                                                                  nx_o, nz_o, nx_i, nz_i);
  return cudaGetLastError();
}
cudaError_t launch_lambda_update(float *lam, const float *ku, const float *f, const float *mu, float sigma,
                                 long long n, int S, int Nz, int disc, cudaStream_t st) {
  k_lambda_update<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(lam, ku, f, mu, sigma, n, S, Nz, disc);
  return cudaGetLastError();
}
cudaError_t launch_sqdiff(const float *a, const float *b, long long n, double *part, int nb, cudaStream_t st) {
  k_sqdiff_partial<<<nb, 256, 0, st>>>(a, b, n, part);
  return cudaGetLastError();
}

cudaError_t launch_sumsq(const float *x, long long n, double *part, int nb, cudaStream_t st) {
  k_sumsq_partial<<<nb, 256, 0, st>>>(x, n, part);
  return cudaGetLastError();
}
cudaError_t launch_scale_f32(float *x, long long n, float s, cudaStream_t st) {
  k_scale_f32<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(x, n, s);
  return cudaGetLastError();
}

cudaError_t launch_lambda_fixed(float *lam, const float *ku, const float *f, const double *mu, long long nbin, int S,
                                int Nz, int disc, float empty_weight, float cap, cudaStream_t st) {
  k_lambda_fixed<<<(unsigned)((nbin * S + 255) / 256), 256, 0, st>>>(lam, ku, f, mu, nbin, S, Nz, disc, empty_weight,
                                                                      cap);
  return cudaGetLastError();
}

template <class T>
__global__ void k_fill(T *__restrict__ x, size_t n, T v) {
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) x[k] = v;
}

// ===========================================================================
// FP64 operator-norm power iteration (radon_normest, 3-D :1018-1030), one slice
// ===========================================================================
// FP64 forward projection of one slice, a warp per ray: lane l sums rows l, l+32,
// ..., then a fixed butterfly adds the 32 partial sums (deterministic).  Weights
// and bounds as the float projector, in double (the x range is widened by one
// pixel and the weight test decides).
__global__ void k_radon64_warp(const double *__restrict__ img, double *__restrict__ sino,
                               const dvec4 *__restrict__ ofs, int N, int nd, int nang) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long ray = t >> 5;
  const int lane = threadIdx.x & 31;
  if (ray >= (long long)nd * nang) return;  // whole warps leave together
  const int j = (int)(ray / nd), i = (int)(ray - (long long)j * nd);
  const dvec4 o = ofs[j];
  double acc = 0.0;
  for (int y = lane; y < N; y += 32) {
    const double dd = y * o.y + o.z;
    int xl, xh;
    if (o.x == 0.0) {
      if (dd > i - 1 && dd < i + 1) { xl = 0; xh = N - 1; } else continue;
    } else if (o.x > 0.0) {
      xl = (int)((i - 1 - dd) * o.w); xh = (int)((i + 1 - dd) * o.w);
    } else {
      xl = (int)((i + 1 - dd) * o.w); xh = (int)((i - 1 - dd) * o.w);
    }
    xl = max(xl - 1, 0); xh = min(xh + 1, N - 1);
    for (int x = xl; x <= xh; ++x) {
      const double wgt = 1.0 - fabs(x * o.x + dd - i);
      if (wgt > 0.0) acc += wgt * img[(size_t)y * N + x];
    }
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
  if (lane == 0) sino[ray] = acc;
}

__global__ void k_radon_ad64(const double *__restrict__ sino, double *__restrict__ img, const dvec4 *__restrict__ ofs,
                             int N, int nd, int nang) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= N * N) return;
  const int y = t / N, x = t - y * N;
  double acc = 0.0;
  for (int j = 0; j < nang; ++j) {
    const dvec4 o = ofs[j];
    const double tt = x * o.x + y * o.y + o.z;
    if (tt > -1.0 && tt < nd) {
      const double fl = floor(tt), p = tt - fl;
      const int il = (int)fl;
      if (il >= 0) acc += (1.0 - p) * sino[(size_t)j * nd + il];
      if (il <= nd - 2) acc += p * sino[(size_t)j * nd + il + 1];
    }
  }
  img[t] = acc;
}

// deterministic two-level sum: block partials then one block
__global__ void k_sum64_partial(const double *__restrict__ x, size_t n, double *__restrict__ part) {
  __shared__ double sh[256];
  double a = 0.0;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) a += x[k];
  sh[threadIdx.x] = a;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

__global__ void k_scale64(double *__restrict__ x, size_t n, const double *__restrict__ sum) {
  const double inv = 1.0 / sum[0];
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
    x[k] *= inv;
}

// ===========================================================================
// FP64 primal-dual gap of the current iterate (no counterpart in the reference's
// loop; its draft energy code is radon_tgv_primal_dual_3d.py:882-927).  Problem:
//   P = a1~ sum_x |grad u - p|_V + a0~ sum_x |E p|_W* + D(u),  u in [0, U]
//   D = -F~*(lam) + U sum min(0, K^T lam - theta div v~),  v~ = -div_sym w
// Per-block FP64 partial sums / maxima; the host reduces the blocks in order.
// ===========================================================================
enum { GQ_DATA = 0, GQ_FSTAR, GQ_REG1, GQ_REG0, GQ_MAXV, GQ_MAXU, GQ_BOX, GQ_N };

__device__ __forceinline__ void block_reduce_store(double v, bool is_max, double *out) {
  __shared__ double sh[32];
  for (int o = 16; o > 0; o >>= 1) {
    const double t = __shfl_down_sync(0xffffffffu, v, o);
    v = is_max ? fmax(v, t) : v + t;
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  if (wid == 0) {
    v = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : (is_max ? -1e300 : 0.0);
    for (int o = 16; o > 0; o >>= 1) {
      const double t = __shfl_down_sync(0xffffffffu, v, o);
      v = is_max ? fmax(v, t) : v + t;
    }
    if (lane == 0) out[blockIdx.x] = v;
  }
}

// data term and conjugate per bin: R u from the ray table (FP32 sum), terms in FP64
template <int DISC>
__global__ void __launch_bounds__(256) k_gap_data(const IterParams P, double *part_data, double *part_fstar) {
  const Dims d = P.d;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double data = 0.0, fs = 0.0;
  if (t < (long long)d.nbin) {
    const int b = (int)(t / d.S), s = (int)(t - (long long)b * d.S);
    const long long r0 = P.ray_start[b], r1 = P.ray_start[b + 1];
    float acc = 0.f;
    for (long long e = r0; e < r1; ++e) {
      const int2 en = P.ray_ent[e];
      acc = __fmaf_rn(__int_as_float(en.y), P.u[(size_t)en.x * d.S + s], acc);
    }
    const double Ru = acc, f = P.f[t], lam = P.lam[t];
    const double m = P.mu64[s / d.Nz];
    if (DISC == KL) {
      if (f > 0.0) {
        data = m * (Ru - f + f * log(f / Ru));  // +inf where R u = 0 < f
        fs = -m * f * log1p(-lam / m);
      } else {
        data = m * Ru;
      }
    } else {
      data = 0.5 * m * (Ru - f) * (Ru - f);   // the host divides by ne^2
      fs = lam * f / P.ne64 + 0.5 * lam * lam / m;
    }
  }
  block_reduce_store(data, false, part_data);
  block_reduce_store(fs, false, part_fstar);
}

// support of the ball {sum b w^2 <= 1} under <w, e> = sum m w e  -> weights m^2/b
template <int DIM, int CPL>
__device__ __forceinline__ double wsupport_weight(int k) {
  const double q = 1.4142 * 1.4142;
  if (DIM == 3) {
    if (k < 3) return 1.0;
    if (CPL == UNCORR && k == 5) return 4.0;
    return 4.0 / q;
  }
  if (k < 2) return 1.0;
  return CPL == UNCORR ? 4.0 / q : 1.0;
}

// singular values of the C x K matrix with Gram matrix G (K = 2 or 3), via the
// eigenvalues of G: 2x2 closed form, 3x3 trigonometric form for symmetric matrices
__device__ __forceinline__ void gram_singular(int K, const double G[6], double sv[3]) {
  if (K == 2) {
    const double a = G[0], b = G[1], c = G[2];
    const double tr = a + c, dt = sqrt(fmax(0.0, 0.25 * (a - c) * (a - c) + b * b));
    sv[0] = sqrt(fmax(0.0, 0.5 * tr + dt));
    sv[1] = sqrt(fmax(0.0, 0.5 * tr - dt));
    sv[2] = 0.0;
    return;
  }
  // G = [a d e; d b f; e f c] stored (a, b, c, d, e, f)
  const double a = G[0], b = G[1], c = G[2], dd = G[3], e = G[4], f = G[5];
  const double p1 = dd * dd + e * e + f * f;
  const double q = (a + b + c) / 3.0;
  const double p2 = (a - q) * (a - q) + (b - q) * (b - q) + (c - q) * (c - q) + 2.0 * p1;
  double l0, l1, l2;
  if (p2 <= 1e-300) {
    l0 = l1 = l2 = q;
  } else {
    const double pp = sqrt(p2 / 6.0);
    const double B0 = (a - q) / pp, B1 = (b - q) / pp, B2 = (c - q) / pp, B3 = dd / pp, B4 = e / pp, B5 = f / pp;
    const double detB = B0 * (B1 * B2 - B5 * B5) - B3 * (B3 * B2 - B5 * B4) + B4 * (B3 * B5 - B1 * B4);
    const double r = fmin(1.0, fmax(-1.0, 0.5 * detB));
    const double phi = acos(r) / 3.0;
    l0 = q + 2.0 * pp * cos(phi);
    l2 = q + 2.0 * pp * cos(phi + 2.0943951023931957);
    l1 = 3.0 * q - l0 - l2;
  }
  sv[0] = sqrt(fmax(0.0, l0));
  sv[1] = sqrt(fmax(0.0, l1));
  sv[2] = sqrt(fmax(0.0, l2));
}

// per (pixel, z), all channels: regulariser supports, v~ = -div_sym w (stored), max |v~|, max u
template <int DIM, bool TGV, int CPL, int CMAX>
__global__ void __launch_bounds__(256) k_gap_vox(const IterParams P, float *vt, double *part_reg1, double *part_reg0,
                                                 double *part_maxv, double *part_maxu) {
  constexpr int K = DIM, KW = DIM == 3 ? 6 : 3;
  const Dims d = P.d;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double reg1 = 0.0, reg0 = 0.0, maxv = 0.0, maxu = 0.0;
  if (t < (long long)d.N * d.N * d.Nz) {
    const int pix = (int)(t / d.Nz), z = (int)(t - (long long)pix * d.Nz);
    const int y = pix / d.N, x = pix - y * d.N;
    const size_t vol = d.vol, S = d.S, rowS = (size_t)d.N * S;
    const double st = P.stepsize;
    double G1[6] = {0, 0, 0, 0, 0, 0}, Gv[6] = {0, 0, 0, 0, 0, 0};
    double n1 = 0.0, n0 = 0.0, nv = 0.0;
    for (int c = 0; c < d.C; ++c) {
      const size_t i = (size_t)pix * S + (size_t)c * d.Nz + z;
      const double u0 = P.u[i];
      maxu = fmax(maxu, u0);
      double g[3], pc[3] = {0, 0, 0};
      g[0] = (x < d.N - 1) ? (double)P.u[i + S] - u0 : 0.0;
      g[1] = (y < d.N - 1) ? (double)P.u[i + rowS] - u0 : 0.0;
      if (DIM == 3) g[2] = (z < d.Nz - 1) ? ((double)P.u[i + 1] - u0) / st : 0.0;
      if (TGV)
        for (int k = 0; k < K; ++k) { pc[k] = P.p[k * vol + i]; g[k] -= pc[k]; }
      double sq = 0.0;
      for (int k = 0; k < K; ++k) sq += g[k] * g[k];
      if (CPL == UNCORR) reg1 += sqrt(sq); else n1 += sq;
      if (CPL == NUCL) {
        G1[0] += g[0] * g[0]; G1[1] += g[1] * g[1]; G1[3] += g[0] * g[1];
        if (DIM == 3) { G1[2] += g[2] * g[2]; G1[4] += g[0] * g[2]; G1[5] += g[1] * g[2]; }
      }
      double v3[3];
      if (TGV) {
        // E p (backward differences, zero at index 0) and its support
        double a[3], bb[3], cz[3] = {0, 0, 0};
        for (int k = 0; k < K; ++k) {
          a[k] = x > 0 ? pc[k] - (double)P.p[k * vol + i - S] : 0.0;
          bb[k] = y > 0 ? pc[k] - (double)P.p[k * vol + i - rowS] : 0.0;
          if (DIM == 3) cz[k] = z > 0 ? (pc[k] - (double)P.p[k * vol + i - 1]) / st : 0.0;
        }
        double e[6];
        if (DIM == 3) {
          e[0] = a[0]; e[1] = bb[1]; e[2] = cz[2];
          e[3] = 0.5 * (a[1] + bb[0]); e[4] = 0.5 * (a[2] + cz[0]); e[5] = 0.5 * (bb[2] + cz[1]);
        } else {
          e[0] = a[0]; e[1] = bb[1]; e[2] = 0.5 * (a[1] + bb[0]);
        }
        double se = 0.0;
        for (int k = 0; k < KW; ++k) se += wsupport_weight<DIM, CPL == NUCL ? FROB : CPL>(k) * e[k] * e[k];
        if (CPL == UNCORR) reg0 += sqrt(se); else n0 += se;
        // v~ = -div_sym w = E^T w (update_p's divergence with opposite sign)
        const int rx[3] = {0, DIM == 3 ? 3 : 2, 4}, ry[3] = {DIM == 3 ? 3 : 2, 1, 5}, rz[3] = {4, 5, 2};
        for (int k = 0; k < K; ++k) {
          double A = -(double)P.w[rx[k] * vol + i], B = -(double)P.w[ry[k] * vol + i], Cz = 0.0;
          if (x == 0) A = 0.0;
          if (x < d.N - 1) A += P.w[rx[k] * vol + i + S];
          if (y == 0) B = 0.0;
          if (y < d.N - 1) B += P.w[ry[k] * vol + i + rowS];
          if (DIM == 3) {
            Cz = -(double)P.w[rz[k] * vol + i];
            if (z == 0) Cz = 0.0;
            if (z < d.Nz - 1) Cz += P.w[rz[k] * vol + i + 1];
            Cz /= st;
          }
          v3[k] = -(A + B + Cz);
          vt[k * vol + i] = (float)v3[k];
        }
      } else {
        for (int k = 0; k < K; ++k) v3[k] = P.v[k * vol + i];
      }
      double sv = 0.0;
      for (int k = 0; k < K; ++k) sv += v3[k] * v3[k];
      if (CPL == UNCORR) maxv = fmax(maxv, sqrt(sv)); else nv += sv;
      if (CPL == NUCL) {
        Gv[0] += v3[0] * v3[0]; Gv[1] += v3[1] * v3[1]; Gv[3] += v3[0] * v3[1];
        if (DIM == 3) { Gv[2] += v3[2] * v3[2]; Gv[4] += v3[0] * v3[2]; Gv[5] += v3[1] * v3[2]; }
      }
    }
    if (CPL == FROB) {
      reg1 += sqrt(n1); reg0 += sqrt(n0); maxv = fmax(maxv, sqrt(nv));
    } else if (CPL == NUCL) {
      double s1[3], s2[3];
      double g1[6] = {G1[0], G1[1], G1[2], G1[3], G1[4], G1[5]}, gv[6] = {Gv[0], Gv[1], Gv[2], Gv[3], Gv[4], Gv[5]};
      if (DIM == 2) { g1[1] = G1[3]; g1[2] = G1[1]; gv[1] = Gv[3]; gv[2] = Gv[1]; }
      gram_singular(K, g1, s1);
      gram_singular(K, gv, s2);
      reg1 += s1[0] + s1[1] + s1[2];
      reg0 += sqrt(n0);
      maxv = fmax(maxv, fmax(s2[0], fmax(s2[1], s2[2])));
    }
  }
  block_reduce_store(reg1, false, part_reg1);
  block_reduce_store(reg0, false, part_reg0);
  block_reduce_store(maxv, true, part_maxv);
  block_reduce_store(maxu, true, part_maxu);
}

// dual box term per (pixel, s): U * min(0, K^T lam - theta div v~)
template <int DIM>
__global__ void __launch_bounds__(256) k_gap_box(const IterParams P, const float *vt, double theta, double U,
                                                 double *part_box) {
  const Dims d = P.d;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double box = 0.0;
  if (t < (long long)d.vol) {
    const int pix = (int)(t / d.S), s = (int)(t - (long long)pix * d.S);
    const int y = pix / d.N, x = pix - y * d.N, z = s % d.Nz;
    const size_t vol = d.vol, S = d.S, rowS = (size_t)d.N * S, i = (size_t)t;
    double a = vt[i], b = vt[vol + i];
    if (x == d.N - 1) a = 0.0;
    if (x > 0) a -= vt[i - S];
    if (y == d.N - 1) b = 0.0;
    if (y > 0) b -= vt[vol + i - rowS];
    double dv = a + b;
    if (DIM == 3) {
      double c = vt[2 * vol + i];
      if (z == d.Nz - 1) c = 0.0;
      if (z > 0) c -= vt[2 * vol + i - 1];
      dv += c / (double)P.stepsize;
    }
    const double g = (double)P.kstar[i] / P.ne64 - theta * dv;
    box = U * fmin(0.0, g);
  }
  block_reduce_store(box, false, part_box);
}

// ===========================================================================
// host-side launchers
// ===========================================================================
static inline unsigned blocks_for(long long n, int bs) { return (unsigned)((n + bs - 1) / bs); }

// k_dual_z2 applies: 3-D TGV, Frobenius or uncorrelated coupling, C <= 4, Nz even
bool dual_z2_ok(const IterParams &P, int tgv, int cpl) {
  return P.d.dim == 3 && tgv && (cpl == FROB || cpl == UNCORR) && P.d.C <= 4 && P.d.Nz % 2 == 0;
}

// dual launch shapes: 0 k_dual, 1 k_dual_z2 (where dual_z2_ok; else the same as 0),
// 2 k_dual with registers capped for 5 resident blocks (C <= 4; else as 0),
// 3-5 k_dual_pf: loads one channel ahead in 128-thread blocks (3), all loads first
// in 128-thread (4) or 64-thread (5) blocks (C <= 4; else as 0),
// 6 k_dual_cl: one thread per voxel-channel (Frobenius / uncorrelated, C <= 4; else as 0),
// 7 k_dual_cl2: one thread per channel and slice pair (3-D, Nz even; else as 6),
// 8, 9: shapes 6, 7 in blocks of 128 threads
int num_dual_configs(const IterParams &P) { return P.d.C <= 4 ? 10 : 1; }
bool dual_cl_ok(const IterParams &P, int cpl) { return cpl != NUCL && P.d.C <= 4; }
bool dual_cl2_ok(const IterParams &P, int cpl) { return dual_cl_ok(P, cpl) && P.d.dim == 3 && P.d.Nz % 2 == 0; }
// shape 7 or 9 where it is not available falls back to 6 or 8 (one slice per thread)

template <int CPL>
static void launch_dual_z2(const IterParams &P, cudaStream_t st) {
  const unsigned g = blocks_for((long long)P.d.N * P.d.N * (P.d.Nz / 2), 256);
  const int C = P.d.C;
  if (C <= 1) k_dual_z2<CPL, 1><<<g, 256, 0, st>>>(P);
  else if (C <= 2) k_dual_z2<CPL, 2><<<g, 256, 0, st>>>(P);
  else k_dual_z2<CPL, 4><<<g, 256, 0, st>>>(P);
}

template <int DIM, bool TGV, int CPL, int MINB, int NT, int LA = 4>
static void launch_dual_pf(const IterParams &P, cudaStream_t st) {
  const unsigned g = blocks_for((long long)P.d.N * P.d.N * P.d.Nz, NT);
  const int C = P.d.C;
  if (C == 1) k_dual_pf<DIM, TGV, CPL, 1, MINB, NT, 1><<<g, NT, 0, st>>>(P);
  else if (C == 2) k_dual_pf<DIM, TGV, CPL, 2, MINB, NT, LA < 2 ? LA : 2><<<g, NT, 0, st>>>(P);
  else if (C == 3) k_dual_pf<DIM, TGV, CPL, 3, MINB, NT, LA < 3 ? LA : 3><<<g, NT, 0, st>>>(P);
  else k_dual_pf<DIM, TGV, CPL, 4, MINB, NT, LA><<<g, NT, 0, st>>>(P);
}

template <int DIM, bool TGV, int CPL>
static cudaError_t launch_dual_c(const IterParams &P, cudaStream_t st) {
  const long long n = (long long)P.d.N * P.d.N * P.d.Nz;
  const unsigned g = blocks_for(n, 256);
  const int C = P.d.C;
  if (DIM == 3 && TGV && CPL != NUCL && P.dual_cfg == 1 && C <= 4 && P.d.Nz % 2 == 0) {
    launch_dual_z2<CPL == NUCL ? FROB : CPL>(P, st);
    return cudaGetLastError();
  }
  if (DIM == 3 && P.dual_cfg == 7 && C <= 4 && CPL != NUCL && P.d.Nz % 2 == 0) {  // ... and slice pair
    constexpr int Q = CPL == NUCL ? FROB : CPL;
    const long long cp = C <= 1 ? 1 : (C <= 2 ? 2 : 4);
    const unsigned gc = blocks_for((long long)P.d.N * P.d.N * (P.d.Nz / 2) * cp, 256);
    if (cp == 1) k_dual_cl2<TGV, Q, 1><<<gc, 256, 0, st>>>(P);
    else if (cp == 2) k_dual_cl2<TGV, Q, 2><<<gc, 256, 0, st>>>(P);
    else k_dual_cl2<TGV, Q, 4><<<gc, 256, 0, st>>>(P);
    return cudaGetLastError();
  }
  if (DIM == 3 && P.dual_cfg == 9 && C <= 4 && CPL != NUCL && P.d.Nz % 2 == 0) {
    constexpr int Q = CPL == NUCL ? FROB : CPL;
    const long long cp = C <= 1 ? 1 : (C <= 2 ? 2 : 4);
    const unsigned gc = blocks_for((long long)P.d.N * P.d.N * (P.d.Nz / 2) * cp, 128);
    const bool one = P.stepsize == 1.0f;  // the divisions by the step size are left out
    if (cp == 1) one ? k_dual_cl2<TGV, Q, 1, true><<<gc, 128, 0, st>>>(P) : k_dual_cl2<TGV, Q, 1><<<gc, 128, 0, st>>>(P);
    else if (cp == 2) one ? k_dual_cl2<TGV, Q, 2, true><<<gc, 128, 0, st>>>(P) : k_dual_cl2<TGV, Q, 2><<<gc, 128, 0, st>>>(P);
    else one ? k_dual_cl2<TGV, Q, 4, true><<<gc, 128, 0, st>>>(P) : k_dual_cl2<TGV, Q, 4><<<gc, 128, 0, st>>>(P);
    return cudaGetLastError();
  }
  if (P.dual_cfg >= 6 && C <= 4 && CPL != NUCL) {  // one thread per voxel-channel
    constexpr int Q = CPL == NUCL ? FROB : CPL;
    const long long cp = C <= 1 ? 1 : (C <= 2 ? 2 : 4);
    const int nt = (P.dual_cfg == 8 || P.dual_cfg == 9) ? 128 : 256;
    const unsigned gc = blocks_for(n * cp, nt);
    if (cp == 1) k_dual_cl<DIM, TGV, Q, 1><<<gc, nt, 0, st>>>(P);
    else if (cp == 2) k_dual_cl<DIM, TGV, Q, 2><<<gc, nt, 0, st>>>(P);
    else k_dual_cl<DIM, TGV, Q, 4><<<gc, nt, 0, st>>>(P);
    return cudaGetLastError();
  }
  if (P.dual_cfg >= 3 && P.dual_cfg <= 5 && C <= 4) {  // operands loaded ahead of the arithmetic
    if (P.dual_cfg == 3) launch_dual_pf<DIM, TGV, CPL, 5, 128, 1>(P, st);  // one channel ahead, 96 registers
    else if (P.dual_cfg == 4) launch_dual_pf<DIM, TGV, CPL, 4, 128>(P, st);  // all channels, 128 registers
    else launch_dual_pf<DIM, TGV, CPL, 8, 64>(P, st);                        // as 4 in 64-thread blocks
    return cudaGetLastError();
  }
  if (P.dual_cfg == 2 && C <= 4) {  // registers capped for 5 resident blocks
    if (C <= 1) k_dual<DIM, TGV, CPL, 1, 5><<<g, 256, 0, st>>>(P);
    else if (C <= 2) k_dual<DIM, TGV, CPL, 2, 5><<<g, 256, 0, st>>>(P);
    else k_dual<DIM, TGV, CPL, 4, 5><<<g, 256, 0, st>>>(P);
    return cudaGetLastError();
  }
  if (C <= 1) k_dual<DIM, TGV, CPL, 1><<<g, 256, 0, st>>>(P);
  else if (C <= 2) k_dual<DIM, TGV, CPL, 2><<<g, 256, 0, st>>>(P);
  else if (C <= 4) k_dual<DIM, TGV, CPL, 4><<<g, 256, 0, st>>>(P);
  else {
    // coupled: C <= 8 (checked at problem creation); uncorrelated: groups of 8 channels
    for (int cb = 0; cb < C; cb += 8) {
      IterParams Q = P;
      Q.cbase = cb;
      k_dual<DIM, TGV, CPL, 8><<<g, 256, 0, st>>>(Q);
    }
  }
  return cudaGetLastError();
}

template <int DIM, bool TGV>
static cudaError_t launch_dual_t(const IterParams &P, int cpl, cudaStream_t st) {
  if (cpl == UNCORR) return launch_dual_c<DIM, TGV, UNCORR>(P, st);
  if (cpl == FROB) return launch_dual_c<DIM, TGV, FROB>(P, st);
  return launch_dual_c<DIM, TGV, NUCL>(P, st);
}

cudaError_t launch_dual(const IterParams &P, int tgv, int cpl, cudaStream_t st) {
  if (P.d.dim == 3) return tgv ? launch_dual_t<3, true>(P, cpl, st) : launch_dual_t<3, false>(P, cpl, st);
  return tgv ? launch_dual_t<2, true>(P, cpl, st) : launch_dual_t<2, false>(P, cpl, st);
}

// the fused dual kernel (k_dual_cl2<..., FUSED>): 3-D TGV, Frobenius or
// uncorrelated coupling, C <= 4, Nz even
bool dual_fused_ok(const IterParams &P, int tgv, int cpl) { return tgv && dual_cl2_ok(P, cpl); }

// k_dual_walk geometry: channel lanes CP, pairs per z-chunk ZC (at most 15, the
// chunks as even as possible), columns per block NCOL (at most 512 threads), rows
// per block R
struct WalkShape {
  int cp, zc, ncol, rows, nch, threads;
  size_t smem;
};

static WalkShape walk_shape(const Dims &d) {
  WalkShape w;
  w.cp = d.C <= 1 ? 1 : (d.C <= 2 ? 2 : 4);
  const int nz2 = d.Nz / 2;
  w.nch = (nz2 + 14) / 15;
  w.zc = (nz2 + w.nch - 1) / w.nch;
  const int colT = (w.zc + 1) * w.cp;
  w.ncol = 512 / colT;
  w.rows = 32;
  w.threads = (w.ncol * colT + 31) / 32 * 32;
  w.smem = walk::bytes_per_thread * (size_t)w.threads;
  return w;
}

template <int CPL, int CP>
static cudaError_t walk_attr(size_t smem) {
  return cudaFuncSetAttribute(k_dual_walk<CPL, CP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

// the shared-memory limit of the fused kernel (outside stream capture)
cudaError_t prepare_dual_fused(const IterParams &P, int cpl) {
  const WalkShape ws = walk_shape(P.d);
  if (cpl == UNCORR) {
    if (ws.cp == 1) return walk_attr<UNCORR, 1>(ws.smem);
    if (ws.cp == 2) return walk_attr<UNCORR, 2>(ws.smem);
    return walk_attr<UNCORR, 4>(ws.smem);
  }
  if (ws.cp == 1) return walk_attr<FROB, 1>(ws.smem);
  if (ws.cp == 2) return walk_attr<FROB, 2>(ws.smem);
  return walk_attr<FROB, 4>(ws.smem);
}

cudaError_t launch_dual_fused(const IterParams &P, int tgv, int cpl, cudaStream_t st) {
  if (!dual_fused_ok(P, tgv, cpl) || !P.p2 || !P.v2 || !P.w2) return cudaErrorInvalidValue;
  const WalkShape ws = walk_shape(P.d);
  const dim3 grid((P.d.N + ws.ncol - 2) / (ws.ncol - 1), (P.d.N + ws.rows - 1) / ws.rows, ws.nch);
  const unsigned nt = ws.threads;
  if (cpl == UNCORR) {
    if (ws.cp == 1) k_dual_walk<UNCORR, 1><<<grid, nt, ws.smem, st>>>(P, ws.zc, ws.ncol, ws.rows);
    else if (ws.cp == 2) k_dual_walk<UNCORR, 2><<<grid, nt, ws.smem, st>>>(P, ws.zc, ws.ncol, ws.rows);
    else k_dual_walk<UNCORR, 4><<<grid, nt, ws.smem, st>>>(P, ws.zc, ws.ncol, ws.rows);
  } else {
    if (ws.cp == 1) k_dual_walk<FROB, 1><<<grid, nt, ws.smem, st>>>(P, ws.zc, ws.ncol, ws.rows);
    else if (ws.cp == 2) k_dual_walk<FROB, 2><<<grid, nt, ws.smem, st>>>(P, ws.zc, ws.ncol, ws.rows);
    else k_dual_walk<FROB, 4><<<grid, nt, ws.smem, st>>>(P, ws.zc, ws.ncol, ws.rows);
  }
  return cudaGetLastError();
}

// Forward projection of R adjacent bins of one angle at once.  For every row the
// union of the R bins' x ranges is read once and each pixel feeds every bin whose
// hat covers it, so a pixel loaded for bin i also serves bin i+1 (about (R+1)/2R
// of the loads of one bin at a time).  Each bin still sums its terms in the
// reference's order (rows ascending, x ascending) with the reference's bounds and
// weights.
template <int VW, int R, bool EXACT>
__device__ __forceinline__ void radon_run(const float *__restrict__ img, size_t S, int N, int nd, const float4 o,
                                          int i0, const Slices<VW> &sl, float (&acc)[R][VW]) {
#pragma unroll
  for (int r = 0; r < R; ++r)
#pragma unroll
    for (int k = 0; k < VW; ++k) acc[r][k] = 0.f;
  int ylo, yhi, ylo2, yhi2;
  ray_rows(o, i0, N, ylo, yhi);
  ray_rows(o, min(i0 + R - 1, nd - 1), N, ylo2, yhi2);
  ylo = min(ylo, ylo2);
  yhi = max(yhi, yhi2);
  for (int y = ylo; y <= yhi; ++y) {
    const float d = __fadd_rn(__fmul_rn((float)y, o.y), o.z);
    int xl[R], xh[R];
    int xmin = N, xmax = -1;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int i = i0 + r;
      const float fim = (float)(i - 1), fip = (float)(i + 1);
      int a, b;
      if (o.x == 0.f) {
        if (d > fim && d < fip) { a = 0; b = N - 1; } else { a = N; b = -1; }
      } else if (o.x > 0.f) {
        a = __float2int_rz(__fmul_rn(__fsub_rn(fim, d), o.w));
        b = __float2int_rz(__fmul_rn(__fsub_rn(fip, d), o.w));
      } else {
        a = __float2int_rz(__fmul_rn(__fsub_rn(fip, d), o.w));
        b = __float2int_rz(__fmul_rn(__fsub_rn(fim, d), o.w));
      }
      a = max(a, 0);
      b = min(b, N - 1);
      if (i >= nd) { a = N; b = -1; }
      xl[r] = a;
      xh[r] = b;
      if (a <= b) { xmin = min(xmin, a); xmax = max(xmax, b); }
    }
    const float *row = img + (size_t)y * N * S;
    // groups of G pixels: their loads are issued together, then consumed in x order
    constexpr int G = 4;
    for (int xg = xmin; xg <= xmax; xg += G) {
      float val[G][VW];
#pragma unroll
      for (int g = 0; g < G; ++g)
        if (xg + g <= xmax) sl.load(row + (size_t)(xg + g) * S, val[g]);
#pragma unroll
      for (int g = 0; g < G; ++g) {
        const int x = xg + g;
        if (x > xmax) break;
        const float tx = __fadd_rn(__fmul_rn((float)x, o.x), d);
#pragma unroll
        for (int r = 0; r < R; ++r) {
          const float wgt = 1.0f - fabsf(__fsub_rn(tx, (float)(i0 + r)));
          if (x >= xl[r] && x <= xh[r] && wgt > 0.f) {
#pragma unroll
            for (int k = 0; k < VW; ++k) acc[r][k] = mac<EXACT>(acc[r][k], wgt, val[g][k]);
          }
        }
      }
    }
  }
}

// k_fwd_run: k_fwd for runs of R bins (radon_run), same fused data-term prox.
template <int DISC, int VW, int R>
__global__ void __launch_bounds__(256) k_fwd_run(const IterParams P) {
  const Dims d = P.d;
  const int nrun = (d.nd + R - 1) / R;
  long long unit;
  Slices<VW> sl;
  if (!map_thread<VW>((long long)nrun * d.nang, d.S, unit, sl)) return;
  const int j = (int)(unit / nrun), i0 = (int)(unit - (long long)j * nrun) * R;
  float acc[R][VW];
  radon_run<VW, R, false>(P.ubar, d.S, d.N, d.nd, __ldg(P.ofs + j), i0, sl, acc);
  const float sd = P.sigma_data;
  float m[VW];
#pragma unroll
  for (int k = 0; k < VW; ++k) m[k] = sl.valid(k) ? __ldg(P.mu + sl.slice(k) / d.Nz) : 0.f;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    if (i0 + r >= d.nd) break;
    const size_t q = ((size_t)j * d.nd + i0 + r) * d.S;
    sl.store(P.ku + q, acc[r]);
    float lam[VW], f[VW];
    sl.loadw(P.lam + q, lam);
    sl.load(P.f + q, f);
#pragma unroll
    for (int k = 0; k < VW; ++k) {
      if (DISC == KL) {
        const float sv = lam[k] + sd * acc[r][k];
        const float wv = sv - m[k];
        const float dv = wv * wv + 4.f * sd * f[k] * m[k];
        lam[k] = sv - 0.5f * (wv + sqrtf(dv));
      } else {
        lam[k] = (lam[k] + sd * (acc[r][k] - f[k])) * m[k];
      }
    }
    sl.store(P.lam + q, lam);
  }
}

// k_fwd_rt: k_fwd over 3-bin runs from the run table (each pixel loaded once for
// three bins), same fused data-term prox per bin.
template <int DISC, int VW, int UNR>
__global__ void __launch_bounds__(256) k_fwd_rt(const IterParams P) {
  const Dims d = P.d;
  const int nq = (d.nd + 2) / 3;
  long long unit;
  Slices<VW> sl;
  if (!map_thread<VW>((long long)nq * d.nang, d.S, unit, sl)) return;
  const int j = (int)(unit / nq), i0 = 3 * (int)(unit - (long long)j * nq);
  float acc[3][VW];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int k = 0; k < VW; ++k) acc[r][k] = 0.f;
  const long long e0 = __ldg(P.run_start + unit), e1 = __ldg(P.run_start + unit + 1);
  const int4 *ent = P.run_ent + e0;
  const int n = (int)(e1 - e0);
  int e = 0;
  for (; e + UNR <= n; e += UNR) {
    int4 en[UNR];
    float v[UNR][VW];
#pragma unroll
    for (int u = 0; u < UNR; ++u) en[u] = __ldg(ent + e + u);
#pragma unroll
    for (int u = 0; u < UNR; ++u) sl.load(P.ubar + (size_t)en[u].x * d.S, v[u]);
#pragma unroll
    for (int u = 0; u < UNR; ++u) {
      const float w0 = __int_as_float(en[u].y), w1 = __int_as_float(en[u].z), w2 = __int_as_float(en[u].w);
#pragma unroll
      for (int k = 0; k < VW; ++k) {
        acc[0][k] = __fmaf_rn(w0, v[u][k], acc[0][k]);
        acc[1][k] = __fmaf_rn(w1, v[u][k], acc[1][k]);
        acc[2][k] = __fmaf_rn(w2, v[u][k], acc[2][k]);
      }
    }
  }
  for (; e < n; ++e) {
    const int4 en = __ldg(ent + e);
    float v[VW];
    sl.load(P.ubar + (size_t)en.x * d.S, v);
    const float w0 = __int_as_float(en.y), w1 = __int_as_float(en.z), w2 = __int_as_float(en.w);
#pragma unroll
    for (int k = 0; k < VW; ++k) {
      acc[0][k] = __fmaf_rn(w0, v[k], acc[0][k]);
      acc[1][k] = __fmaf_rn(w1, v[k], acc[1][k]);
      acc[2][k] = __fmaf_rn(w2, v[k], acc[2][k]);
    }
  }
  const float sd = P.sigma_data;
  float m[VW];
#pragma unroll
  for (int k = 0; k < VW; ++k) m[k] = sl.valid(k) ? __ldg(P.mu + sl.slice(k) / d.Nz) : 0.f;
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    if (i0 + r >= d.nd) break;
    const size_t q = ((size_t)j * d.nd + i0 + r) * d.S;
    sl.store(P.ku + q, acc[r]);
    float lam[VW], f[VW];
    sl.loadw(P.lam + q, lam);
    sl.load(P.f + q, f);
#pragma unroll
    for (int k = 0; k < VW; ++k) {
      if (DISC == KL) {
        const float sv = lam[k] + sd * acc[r][k];
        const float wv = sv - m[k];
        const float dv = wv * wv + 4.f * sd * f[k] * m[k];
        lam[k] = sv - 0.5f * (wv + sqrtf(dv));
      } else {
        lam[k] = (lam[k] + sd * (acc[r][k] - f[k])) * m[k];
      }
    }
    sl.store(P.lam + q, lam);
  }
}

// slices per lane: 8 (two float4 chunks) when S is a multiple of 4, else 2, else 1
static inline int vec_width(int S) { return (S % 4 == 0) ? 8 : (S % 2 == 0 ? 2 : 1); }

// Tunable launch shapes of the projector kernels (chosen per problem shape by
// the autotuner in gt_api.cu).  S a multiple of 4: k_fwd configs 0..3 =
// (slices per lane, ray-table entries in flight) = (8, 4), (8, 8), (4, 4), (4, 8),
// configs 5..8 = (slices per lane, bins per run) of k_fwd_run = (8, 2), (8, 4),
// (4, 4), (4, 8);
// k_bp configs 0..7 = (slices per lane, angles per step, geometry) = (8, 2, table),
// (8, 4, table), (4, 2, table), (4, 4, table), (8, 1, on the fly), (4, 1, on the fly),
// (8, 2, on the fly), (4, 2, on the fly); configs 9..12 = (slices per lane,
// pixels per run) of k_bp_run = (8, 4), (4, 8), (8, 8), (4, 4).  k_fwd config 9 and
// k_bp config 13: one slice per lane with the 32-slice chunk outermost (SlicesWL),
// for images and sinograms larger than L2.  k_fwd configs 10, 11: the 3-bin run
// table (k_fwd_rt) with (slices per lane, entries in flight) = (8, 4), (4, 8);
// configs 12, 13: (8, 8) and (8, 4) with registers capped for 5 / 6 resident blocks.
// k_bp configs 18, 19: the register-blocked row-tile kernel (gt_proj.cu) with 4 or
// 2 slices per lane.
// Otherwise one fixed shape with 2 or 1 slices per thread.
// One more candidate each: one slice per thread (k_fwd config 4, k_bp config 8),
// which keeps all lanes busy when S is small.
int num_proj_configs(int S, int which) {
  if (S % 4 != 0) return 1;
  return which == 0 ? 20 : 20;  // configs 4 / 8 (one slice per thread) stay candidates for every S
}

template <int VW, int UNR>
static void fwd_vw(const IterParams &P, int disc, cudaStream_t st) {
  const unsigned g = blocks_for(threads_for<VW>((long long)P.d.nd * P.d.nang, P.d.S), 256);
  if (disc == KL) k_fwd<KL, VW, UNR><<<g, 256, 0, st>>>(P);
  else k_fwd<L2, VW, UNR><<<g, 256, 0, st>>>(P);
}

// the same with a register cap for MINB resident blocks of 256 per SM (occupancy)
template <int VW, int UNR, int MINB>
static void fwd_vw_occ(const IterParams &P, int disc, cudaStream_t st) {
  const unsigned g = blocks_for(threads_for<VW>((long long)P.d.nd * P.d.nang, P.d.S), 256);
  if (disc == KL) k_fwd<KL, VW, UNR, false, MINB><<<g, 256, 0, st>>>(P);
  else k_fwd<L2, VW, UNR, false, MINB><<<g, 256, 0, st>>>(P);
}

template <int VW, int UNR>
static void fwd_rt(const IterParams &P, int disc, cudaStream_t st) {
  const long long units = (long long)((P.d.nd + 2) / 3) * P.d.nang;
  const unsigned g = blocks_for(threads_for<VW>(units, P.d.S), 256);
  if (disc == KL) k_fwd_rt<KL, VW, UNR><<<g, 256, 0, st>>>(P);
  else k_fwd_rt<L2, VW, UNR><<<g, 256, 0, st>>>(P);
}

static void fwd_wl(const IterParams &P, int disc, cudaStream_t st) {
  const unsigned g = blocks_for(threads_for_wl((long long)P.d.nd * P.d.nang, P.d.S), 256);
  if (disc == KL) k_fwd<KL, 1, 8, true><<<g, 256, 0, st>>>(P);
  else k_fwd<L2, 1, 8, true><<<g, 256, 0, st>>>(P);
}

template <int VW, int R>
static void fwd_run(const IterParams &P, int disc, cudaStream_t st) {
  const long long units = (long long)((P.d.nd + R - 1) / R) * P.d.nang;
  const unsigned g = blocks_for(threads_for<VW>(units, P.d.S), 256);
  if (disc == KL) k_fwd_run<KL, VW, R><<<g, 256, 0, st>>>(P);
  else k_fwd_run<L2, VW, R><<<g, 256, 0, st>>>(P);
}

cudaError_t launch_bp_row(const IterParams &P, int shape, cudaStream_t st);

cudaError_t launch_fwd(const IterParams &P, int disc, cudaStream_t st) {
  const int S = P.d.S;
  if (S % 4 == 0) {
    switch (P.fwd_cfg) {
      case 1: fwd_vw<8, 8>(P, disc, st); break;
      case 2: fwd_vw<4, 4>(P, disc, st); break;
      case 3: fwd_vw<4, 8>(P, disc, st); break;
      case 4: fwd_vw<1, 4>(P, disc, st); break;
      case 5: fwd_run<8, 2>(P, disc, st); break;
      case 6: fwd_run<8, 4>(P, disc, st); break;
      case 7: fwd_run<4, 4>(P, disc, st); break;
      case 8: fwd_run<4, 8>(P, disc, st); break;
      case 9:
        if (P.ray_start) fwd_wl(P, disc, st); else fwd_vw<8, 4>(P, disc, st);  // WL streams the ray table
        break;
      case 10:
        if (P.run_start) fwd_rt<8, 4>(P, disc, st); else fwd_vw<8, 4>(P, disc, st);
        break;
      case 11:
        if (P.run_start) fwd_rt<4, 8>(P, disc, st); else fwd_vw<8, 4>(P, disc, st);
        break;
      case 12: fwd_vw_occ<8, 8, 5>(P, disc, st); break;
      case 13: fwd_vw_occ<8, 4, 6>(P, disc, st); break;
      case 14: fwd_vw_occ<8, 4, 4>(P, disc, st); break;
      case 15: fwd_vw_occ<8, 8, 4>(P, disc, st); break;
      case 16: fwd_vw_occ<4, 8, 4>(P, disc, st); break;
      case 17: fwd_vw_occ<8, 2, 4>(P, disc, st); break;
      case 18: fwd_vw_occ<8, 2, 5>(P, disc, st); break;
      case 19: fwd_vw_occ<8, 4, 5>(P, disc, st); break;
      default: fwd_vw<8, 4>(P, disc, st); break;
    }
  } else if (S % 2 == 0) {
    fwd_vw<2, 4>(P, disc, st);
  } else {
    fwd_vw<1, 4>(P, disc, st);
  }
  return cudaGetLastError();
}

template <int VW, int AU, bool TAB = true>
static void bp_vw(const IterParams &P, cudaStream_t st) {
  k_bp<VW, AU, TAB><<<blocks_for(threads_for<VW>((long long)P.d.N * P.d.N, P.d.S), 256), 256, 0, st>>>(P);
}

template <int UA>
static void bp_ua(const IterParams &P, cudaStream_t st) {
  k_bp<8, 1, false, false, UA><<<blocks_for(threads_for<8>((long long)P.d.N * P.d.N, P.d.S), 256), 256, 0, st>>>(P);
}

static void bp_wl(const IterParams &P, cudaStream_t st) {
  k_bp<1, 1, false, true><<<blocks_for(threads_for_wl((long long)P.d.N * P.d.N, P.d.S), 256), 256, 0, st>>>(P);
}

template <int VW, int R>
static void bp_run(const IterParams &P, cudaStream_t st) {
  const long long units = (long long)P.d.N * ((P.d.N + R - 1) / R);
  k_bp_run<VW, R><<<blocks_for(threads_for<VW>(units, P.d.S), 256), 256, 0, st>>>(P);
}

cudaError_t launch_bp(const IterParams &P, cudaStream_t st) {
  const int S = P.d.S;
  if (S % 4 == 0 && (P.bp_cfg == 18 || P.bp_cfg == 19)) {
    // register-blocked row-tile kernel (gt_proj.cu); without its table the one-angle shape
    if (P.row_ent) return launch_bp_row(P, P.bp_cfg - 18, st);
    bp_vw<8, 1, false>(P, st);
    return cudaGetLastError();
  }
  if (S % 4 == 0) {
    switch (P.bp_cfg) {
      case 1: bp_vw<8, 4>(P, st); break;
      case 2: bp_vw<4, 2>(P, st); break;
      case 3: bp_vw<4, 4>(P, st); break;
      case 4: bp_vw<8, 1, false>(P, st); break;
      case 5: bp_vw<4, 1, false>(P, st); break;
      case 6: bp_vw<8, 2, false>(P, st); break;
      case 7: bp_vw<4, 2, false>(P, st); break;
      case 8: bp_vw<1, 1, false>(P, st); break;
      case 9: bp_run<8, 4>(P, st); break;
      case 10: bp_run<4, 8>(P, st); break;
      case 11: bp_run<8, 8>(P, st); break;
      case 12: bp_run<4, 4>(P, st); break;
      case 13: bp_wl(P, st); break;
      case 14:  // no descriptor: the one-angle shape (identical sums)
        if (P.bp_tmap) bp_tma<4>(P, st); else bp_vw<8, 1, false>(P, st);
        break;
      case 15:
        if (P.bp_tmap_wide) bp_tma<8>(P, st); else bp_vw<8, 1, false>(P, st);
        break;
      case 16: bp_ua<4>(P, st); break;  // the one-angle shape (4) with its angle loop unrolled 4x
      case 17: bp_ua<1>(P, st); break;  // ... not unrolled (fewer instructions in flight, faster)
      default: bp_vw<8, 2>(P, st); break;
    }
  } else if (S % 2 == 0) {
    bp_vw<2, 2>(P, st);
  } else {
    bp_vw<1, 2>(P, st);
  }
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// fused batch launches: the work units of every member in one launch per phase.
// Every member runs the same kernel body as in its own launch with a shape fixed
// by its slice count (batch_shape: dual k_dual, thread per voxel with all
// channels; forward the ray table; back projection geometry on the fly; update
// 4, 2 or 1 slices per thread as launch_update), so the iterates are identical to
// solving each member alone (all launch shapes give identical iterates).
// ---------------------------------------------------------------------------
__device__ __forceinline__ int batch_member(const int *__restrict__ start, int n, long long b) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(start + mid) <= b) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

template <int DIM, bool TGV, int CPL, int CMAX>
__global__ void __launch_bounds__(256) k_dual_batch(const BatchTab T) {
  const int k = batch_member(T.start, T.n, blockIdx.x);
  const IterParams P = T.P[k];
  dual_body<DIM, TGV, CPL, CMAX>(P, (long long)blockIdx.x - __ldg(T.start + k));
}

__global__ void __launch_bounds__(256) k_fwd_batch(const BatchTab T) {
  const int k = batch_member(T.start, T.n, blockIdx.x);
  const IterParams P = T.P[k];
  const long long bid = (long long)blockIdx.x - __ldg(T.start + k);
  const int sh = __ldg(T.shape + k);
  if (__ldg(T.disc + k) == KL) {
    if (sh == 2) fwd_body<KL, 8, 4>(P, bid);
    else if (sh == 1) fwd_body<KL, 4, 4>(P, bid);
    else fwd_body<KL, 1, 4>(P, bid);
  } else {
    if (sh == 2) fwd_body<L2, 8, 4>(P, bid);
    else if (sh == 1) fwd_body<L2, 4, 4>(P, bid);
    else fwd_body<L2, 1, 4>(P, bid);
  }
}

__global__ void __launch_bounds__(256) k_bp_batch(const BatchTab T) {
  const int k = batch_member(T.start, T.n, blockIdx.x);
  const IterParams P = T.P[k];
  const long long bid = (long long)blockIdx.x - __ldg(T.start + k);
  const int sh = __ldg(T.shape + k);
  if (sh == 2) bp_body<8, 1, false, false, 1>(P, bid);
  else if (sh == 1) bp_body<4, 1, false, false, 1>(P, bid);
  else bp_body<1, 1, false>(P, bid);
}

template <int DIM, bool TGV>
__global__ void __launch_bounds__(256) k_update_batch(const BatchTab T) {
  const int k = batch_member(T.start, T.n, blockIdx.x);
  const IterParams P = T.P[k];
  const long long bid = (long long)blockIdx.x - __ldg(T.start + k);
  if (P.d.S % 4 == 0) update_body<DIM, TGV, 4, PART_ALL>(P, bid);
  else if (P.d.S % 2 == 0) update_body<DIM, TGV, 2, PART_ALL>(P, bid);
  else update_body<DIM, TGV, 1, PART_ALL>(P, bid);
}

// slices per thread of a member's projector bodies in a fused batch: eight (two
// float4 chunks 128 apart) for S >= 192, four for 64 <= S < 192, else one (S a
// multiple of 4 for the vector shapes; small S keeps every lane busy with one)
int batch_shape(const Dims &d) {
  if (d.S % 4 != 0 || d.S < 64) return 0;
  return d.S >= 192 ? 2 : 1;
}

// blocks of one member in phase ph (0 dual, 1 forward, 2 back projection, 3 update)
long long batch_blocks(const Dims &d, int ph) {
  const int sh = batch_shape(d);
  auto proj = [&](long long units) {
    return blocks_for(sh == 2 ? threads_for<8>(units, d.S) : sh == 1 ? threads_for<4>(units, d.S)
                                                                     : threads_for<1>(units, d.S), 256);
  };
  switch (ph) {
    case 0: return blocks_for((long long)d.N * d.N * d.Nz, 256);
    case 1: return proj((long long)d.nd * d.nang);
    case 2: return proj((long long)d.N * d.N);
    default: {
      const int uw = d.S % 4 == 0 ? 4 : (d.S % 2 == 0 ? 2 : 1);
      return blocks_for((long long)d.N * d.N * (d.S / uw), 256);
    }
  }
}

// one phase of a fused batch iteration over `blocks` blocks; cmax = 4 or 8 (the
// dual kernel's channel registers, >= every member's C)
cudaError_t launch_batch_phase(const BatchTab &T, int ph, long long blocks, int dim, int tgv, int cpl, int cmax,
                               cudaStream_t st) {
  if (blocks <= 0) return cudaSuccess;
  const unsigned g = (unsigned)blocks;
  switch (ph) {
    case 0:
#define GT_DB(D, TG, CP, CM) k_dual_batch<D, TG, CP, CM><<<g, 256, 0, st>>>(T)
      if (dim == 3) {
        if (tgv) {
          if (cpl == FROB) { if (cmax == 4) GT_DB(3, true, FROB, 4); else GT_DB(3, true, FROB, 8); }
          else { if (cmax == 4) GT_DB(3, true, UNCORR, 4); else GT_DB(3, true, UNCORR, 8); }
        } else {
          if (cpl == FROB) { if (cmax == 4) GT_DB(3, false, FROB, 4); else GT_DB(3, false, FROB, 8); }
          else { if (cmax == 4) GT_DB(3, false, UNCORR, 4); else GT_DB(3, false, UNCORR, 8); }
        }
      } else {
        if (tgv) {
          if (cpl == FROB) { if (cmax == 4) GT_DB(2, true, FROB, 4); else GT_DB(2, true, FROB, 8); }
          else { if (cmax == 4) GT_DB(2, true, UNCORR, 4); else GT_DB(2, true, UNCORR, 8); }
        } else {
          if (cpl == FROB) { if (cmax == 4) GT_DB(2, false, FROB, 4); else GT_DB(2, false, FROB, 8); }
          else { if (cmax == 4) GT_DB(2, false, UNCORR, 4); else GT_DB(2, false, UNCORR, 8); }
        }
      }
#undef GT_DB
      break;
    case 1: k_fwd_batch<<<g, 256, 0, st>>>(T); break;
    case 2: k_bp_batch<<<g, 256, 0, st>>>(T); break;
    default:
      if (dim == 3) { if (tgv) k_update_batch<3, true><<<g, 256, 0, st>>>(T); else k_update_batch<3, false><<<g, 256, 0, st>>>(T); }
      else { if (tgv) k_update_batch<2, true><<<g, 256, 0, st>>>(T); else k_update_batch<2, false><<<g, 256, 0, st>>>(T); }
      break;
  }
  return cudaGetLastError();
}

template <int UW, int PART>
static void update_uw(const IterParams &P, int tgv, cudaStream_t st) {
  const unsigned g = blocks_for((long long)P.d.N * P.d.N * (P.d.S / UW), 256);
  if (P.d.dim == 3) {
    if (tgv) k_update<3, true, UW, PART><<<g, 256, 0, st>>>(P);
    else k_update<3, false, UW, PART_ALL><<<g, 256, 0, st>>>(P);
  } else {
    if (tgv) k_update<2, true, UW, PART><<<g, 256, 0, st>>>(P);
    else k_update<2, false, UW, PART_ALL><<<g, 256, 0, st>>>(P);
  }
}

template <int PART>
static void update_part(const IterParams &P, int tgv, cudaStream_t st) {
  const int S = P.d.S;
  if (S % 4 == 0) update_uw<4, PART>(P, tgv, st);
  else if (S % 2 == 0) update_uw<2, PART>(P, tgv, st);
  else update_uw<1, PART>(P, tgv, st);
}

// part: 0 both halves in one launch, 1 the u / ubar half, 2 the p / pbar half
// (TV has no p: part 1 is the whole update and part 2 launches nothing)
cudaError_t launch_update(const IterParams &P, int tgv, cudaStream_t st, int part) {
  if (part == 2 && !tgv) return cudaSuccess;
  if (part == 1) update_part<PART_U>(P, tgv, st);
  else if (part == 2) update_part<PART_P>(P, tgv, st);
  else update_part<PART_ALL>(P, tgv, st);
  return cudaGetLastError();
}

static inline bool aligned(const void *p, int bytes) { return ((uintptr_t)p % bytes) == 0; }

static int proj_width(const void *a, const void *b, int S) {
  int vw = vec_width(S);
  if (vw == 8 && !(aligned(a, 16) && aligned(b, 16))) vw = (S % 2 == 0) ? 2 : 1;
  if (vw == 2 && !(aligned(a, 8) && aligned(b, 8))) vw = 1;
  return vw;
}

cudaError_t launch_radon(const float *img, float *sino, const float4 *ofs, int N, int nd, int nang, int S,
                         cudaStream_t st) {
  const long long units = (long long)nd * nang;
  const int vw = proj_width(img, sino, S);
  if (vw == 8) k_radon<8><<<blocks_for(threads_for<8>(units, S), 256), 256, 0, st>>>(img, sino, ofs, N, nd, nang, S);
  else if (vw == 2) k_radon<2><<<blocks_for(threads_for<2>(units, S), 256), 256, 0, st>>>(img, sino, ofs, N, nd, nang, S);
  else k_radon<1><<<blocks_for(threads_for<1>(units, S), 256), 256, 0, st>>>(img, sino, ofs, N, nd, nang, S);
  return cudaGetLastError();
}

cudaError_t launch_radon_ad(const float *sino, float *img, const float4 *ofs, int N, int nd, int nang, int S,
                            cudaStream_t st) {
  const long long units = (long long)N * N;
  const int vw = proj_width(img, sino, S);
  if (vw == 8) k_radon_ad<8><<<blocks_for(threads_for<8>(units, S), 256), 256, 0, st>>>(sino, img, ofs, N, nd, nang, S);
  else if (vw == 2) k_radon_ad<2><<<blocks_for(threads_for<2>(units, S), 256), 256, 0, st>>>(sino, img, ofs, N, nd, nang, S);
  else k_radon_ad<1><<<blocks_for(threads_for<1>(units, S), 256), 256, 0, st>>>(sino, img, ofs, N, nd, nang, S);
  return cudaGetLastError();
}

cudaError_t launch_run_count(const float4 *ofs, int N, int nd, int nang, int *count, cudaStream_t st) {
  k_run_count<<<blocks_for((long long)((nd + 2) / 3) * nang, 128), 128, 0, st>>>(ofs, N, nd, nang, count);
  return cudaGetLastError();
}

cudaError_t launch_run_fill(const float4 *ofs, int N, int nd, int nang, const long long *start, int4 *ent,
                            cudaStream_t st) {
  k_run_fill<<<blocks_for((long long)((nd + 2) / 3) * nang, 128), 128, 0, st>>>(ofs, N, nd, nang, start, ent);
  return cudaGetLastError();
}

cudaError_t launch_ray_count(const float4 *ofs, int N, int nd, int nang, int *count, cudaStream_t st) {
  k_ray_count<<<blocks_for((long long)nd * nang, 128), 128, 0, st>>>(ofs, N, nd, nang, count);
  return cudaGetLastError();
}

cudaError_t launch_ray_fill(const float4 *ofs, int N, int nd, int nang, const long long *start, int2 *ent,
                            cudaStream_t st) {
  k_ray_fill<<<blocks_for((long long)nd * nang, 128), 128, 0, st>>>(ofs, N, nd, nang, start, ent);
  return cudaGetLastError();
}

// gap: returns per-quantity block partials in `part` ([GQ_N][nblk_max]); host reduces
int gap_blocks(const IterParams &P) {
  const long long a = (long long)P.d.nbin, b = (long long)P.d.N * P.d.N * P.d.Nz, c = (long long)P.d.vol;
  return (int)blocks_for(std::max(a, std::max(b, c)), 256);
}

template <int DIM, bool TGV, int CPL>
static void gap_vox_c(const IterParams &P, float *vt, double *part, int nb, cudaStream_t st) {
  const unsigned g = blocks_for((long long)P.d.N * P.d.N * P.d.Nz, 256);
  k_gap_vox<DIM, TGV, CPL, 8><<<g, 256, 0, st>>>(P, vt, part + GQ_REG1 * nb, part + GQ_REG0 * nb,
                                                 part + GQ_MAXV * nb, part + GQ_MAXU * nb);
}

template <int DIM, bool TGV>
static void gap_vox_t(const IterParams &P, int cpl, float *vt, double *part, int nb, cudaStream_t st) {
  if (cpl == UNCORR) gap_vox_c<DIM, TGV, UNCORR>(P, vt, part, nb, st);
  else if (cpl == FROB) gap_vox_c<DIM, TGV, FROB>(P, vt, part, nb, st);
  else gap_vox_c<DIM, TGV, NUCL>(P, vt, part, nb, st);
}

cudaError_t launch_gap_pass1(const IterParams &P, int disc, int tgv, int cpl, float *vt, double *part, int nb,
                             cudaStream_t st) {
  const unsigned gd = blocks_for((long long)P.d.nbin, 256);
  if (disc == KL) k_gap_data<KL><<<gd, 256, 0, st>>>(P, part + GQ_DATA * nb, part + GQ_FSTAR * nb);
  else k_gap_data<L2><<<gd, 256, 0, st>>>(P, part + GQ_DATA * nb, part + GQ_FSTAR * nb);
  if (P.d.dim == 3) {
    if (tgv) gap_vox_t<3, true>(P, cpl, vt, part, nb, st); else gap_vox_t<3, false>(P, cpl, vt, part, nb, st);
  } else {
    if (tgv) gap_vox_t<2, true>(P, cpl, vt, part, nb, st); else gap_vox_t<2, false>(P, cpl, vt, part, nb, st);
  }
  return cudaGetLastError();
}

cudaError_t launch_gap_pass2(const IterParams &P, const float *vt, double theta, double U, double *part, int nb,
                             cudaStream_t st) {
  const unsigned g = blocks_for((long long)P.d.vol, 256);
  if (P.d.dim == 3) k_gap_box<3><<<g, 256, 0, st>>>(P, vt, theta, U, part + GQ_BOX * nb);
  else k_gap_box<2><<<g, 256, 0, st>>>(P, vt, theta, U, part + GQ_BOX * nb);
  return cudaGetLastError();
}

cudaError_t launch_bp_table(const float4 *ofs, int N, int nd, int nang, int2 *tab, cudaStream_t st) {
  k_bp_table<<<blocks_for((long long)N * N * nang, 256), 256, 0, st>>>(ofs, N, nd, nang, tab);
  return cudaGetLastError();
}

// A state field in the device layout in[(a B + b) S + c Nz + z] to float64 in the
// reference's output layout: mode 0 (the image, a = y, b = x) out[c][b][a][z]
// (Solution [C][x][y][z]); mode 1 (the sinogram, a = angle, b = bin)
// out[c][a][z][b] (Sinogram [C][nang][Nz][nd]).  Mode 0 runs over (a, b, s) with
// s fastest, mode 1 over (a, s, b) with b fastest, so the float64 writes are
// contiguous (runs of Nz, resp. B).
__global__ void k_output_f64(const float *__restrict__ in, double *__restrict__ out, int A, int B, int C, int Nz,
                             int mode) {
  const long long S = (long long)C * Nz;
  const long long n = (long long)A * B * S;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    long long a, b, s;
    if (mode == 0) {
      s = t % S;
      const long long ab = t / S;
      b = ab % B;
      a = ab / B;
    } else {
      b = t % B;
      const long long as = t / B;
      s = as % S;
      a = as / S;
    }
    const long long c = s / Nz, z = s - c * Nz;
    const float v = __ldg(in + (a * B + b) * S + s);
    const long long o = mode == 0 ? ((c * B + b) * A + a) * Nz + z : ((c * A + a) * Nz + z) * B + b;
    out[o] = (double)v;
  }
}

cudaError_t launch_output_f64(const float *in, double *out, int A, int B, int C, int Nz, int mode, cudaStream_t st) {
  const long long n = (long long)A * B * C * Nz;
  const unsigned g = (unsigned)std::min<long long>((n + 255) / 256, 152LL * 16);
  k_output_f64<<<g, 256, 0, st>>>(in, out, A, B, C, Nz, mode);
  return cudaGetLastError();
}

cudaError_t launch_transpose(const float *in, float *out, int rows, int cols, cudaStream_t st) {
  const long long tiles = (long long)((rows + 31) / 32) * ((cols + 31) / 32);
  k_transpose<<<(unsigned)tiles, dim3(32, 8), 0, st>>>(in, out, rows, cols);
  return cudaGetLastError();
}

cudaError_t launch_feasible(float *f, const float *r1, int nbin1, int S, cudaStream_t st) {
  k_feasible<<<blocks_for((long long)nbin1 * S, 256), 256, 0, st>>>(f, r1, nbin1, S);
  return cudaGetLastError();
}

cudaError_t fill_f64(double *x, size_t n, double v, cudaStream_t st) {
  k_fill<double><<<256, 256, 0, st>>>(x, n, v);
  return cudaGetLastError();
}

cudaError_t fill_f32(float *x, size_t n, float v, cudaStream_t st) {
  k_fill<float><<<1024, 256, 0, st>>>(x, n, v);
  return cudaGetLastError();
}

// power iteration: up to `rounds` rounds of  s = sum(img); img /= s; img = R^T R img
// from the all-ones image, stopping once two consecutive sums agree to 1e-10;
// returns sqrt(s) (the reference's 10 rounds from randn, in FP32).
cudaError_t normest64(const dvec4 *ofs, int N, int nd, int nang, int rounds, double *d_img, double *d_sino,
                      double *d_part, double *out, cudaStream_t st) {
  const size_t n = (size_t)N * N;
  const int nb = 64;
  cudaError_t e;
  double prev = 0.0;
  for (int r = 0; r < rounds; ++r) {
    k_sum64_partial<<<nb, 256, 0, st>>>(d_img, n, d_part);
    k_sum64_partial<<<1, 256, 0, st>>>(d_part, nb, d_part + nb);
    if (r >= 4) {  // converged (consecutive sums within 1e-8, the estimate then within ~1e-10): stop early
      double s = 0.0;
      if ((e = cudaMemcpyAsync(&s, d_part + nb, sizeof(double), cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
      if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
      if (std::fabs(s - prev) <= 1e-8 * std::fabs(s)) {
        *out = sqrt(s);
        return cudaSuccess;
      }
      prev = s;
    }
    k_scale64<<<64, 256, 0, st>>>(d_img, n, d_part + nb);
    k_radon64_warp<<<blocks_for(32LL * nd * nang, 256), 256, 0, st>>>(d_img, d_sino, ofs, N, nd, nang);
    k_radon_ad64<<<blocks_for((long long)n, 128), 128, 0, st>>>(d_sino, d_img, ofs, N, nd, nang);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  k_sum64_partial<<<nb, 256, 0, st>>>(d_img, n, d_part);
  k_sum64_partial<<<1, 256, 0, st>>>(d_part, nb, d_part + nb);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  double s = 0.0;
  if ((e = cudaMemcpyAsync(&s, d_part + nb, sizeof(double), cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
  *out = sqrt(s);
  return cudaSuccess;
}

}  // namespace gt
