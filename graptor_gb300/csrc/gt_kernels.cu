// GB300 kernels of the primal-dual TGV/TV reconstruction (sm_103a).
//
// One iteration of the reference loop (radon_tgv_primal_dual_3d.py:1194-1221:
// update_v, update_w, NormV, NormW, radon, update_lambda, radon_ad, update_u,
// update_p, two extrapolations) runs here as three kernels:
//
//   k_dual    update_v + update_w + the coupled ball projections of v and w
//             (one pass over ubar, pbar, v, w; writes v, w)
//   k_fwd     forward projection `radon` of ubar fused with the data-term prox
//             update_lambda (reads ubar, f, lambda; writes lambda and K ubar)
//   k_primal  back projection `radon_ad` of lambda fused with update_u, update_p
//             and both extrapolations (reads u, p, v, w, lambda; writes u, ubar, p, pbar)
//
// k_dual and k_fwd only read what the previous k_primal wrote and write disjoint
// fields, so they need no ordering between them.
#include <cuda_runtime.h>
#include <math.h>

#include "gt_common.cuh"

namespace gt {

// ===========================================================================
// ball projections
// ===========================================================================

// nuclear 2-D (update_NormV_Nucl, radon_tgv_primal_dual_2d.py:124-204): spectral
// projection of the C x 2 matrix A of one pixel via the 2x2 matrix A^T A.
__device__ __forceinline__ void nucl2d_matrix(float a, float b, float c, float ainv, float M[3]) {
  const float eps = 0.00001f;
  float s1, s2, S1, S2;
  const float o = fminf(a, c);
  if ((b * b) / (o * o) > eps && o * o > 0.f) {
    const float dd = a + c, e = a - c;
    float f = 4.f * b * b + e * e;
    f = f < 0.f ? 0.f : sqrtf(f);
    s2 = (dd - f > 0.f) ? sqrtf((dd - f) * 0.5f) : 0.f;
    s1 = (dd + f > 0.f) ? sqrtf((dd + f) * 0.5f) : 0.f;
    const float g = (e + f) * 0.5f, h = (e - f) * 0.5f;
    float q0 = g * a + b * b, q1 = g * b + c * b, q2 = h * a + b * b, q3 = h * b + b * c;
    const float n1 = hypotf(q0, q1), n2 = hypotf(q2, q3);
    if (n1 > 0.f) { q0 = q0 / n1; q1 = q1 / n1; }
    if (n2 > 0.f) { q2 = q2 / n2; q3 = q3 / n2; }
    S1 = (s1 * ainv > 1.f) ? 1.f / (s1 * ainv) : 1.f;
    S2 = (s2 * ainv > 1.f) ? 1.f / (s2 * ainv) : 1.f;
    M[0] = q0 * q0 * S1 + q2 * q2 * S2;
    M[2] = q1 * q1 * S1 + q3 * q3 * S2;
    M[1] = S1 * q0 * q1 + S2 * q2 * q3;
  } else {
    s1 = sqrtf(a);
    s2 = sqrtf(c);
    S1 = (ainv * s1 > 1.f) ? 1.f / (ainv * s1) : 1.f;
    S2 = (ainv * s2 > 1.f) ? 1.f / (ainv * s2) : 1.f;
    M[0] = S1; M[2] = S2; M[1] = 0.f;
  }
}

// nuclear 3-D helpers (radon_tgv_primal_dual_3d.py:190-284), results by value
__device__ __forceinline__ void diag2d(float a, float b, float c, float X[6]) {
  const float eps = 0.001f;
  const float o = fminf(a, c);
  if ((b * b) / (o * o) > eps && o * o > 0.f) {
    const float dd = a + c, e = a - c;
    float f = 4.f * b * b + e * e;
    f = f < 0.f ? 0.f : sqrtf(f);
    X[1] = (dd - f > 0.f) ? (dd - f) * 0.5f : 0.f;
    X[0] = (dd + f > 0.f) ? (dd + f) * 0.5f : 0.f;
    const float h = (e - f) * 0.5f;
    float v0 = 1.f, v1 = -h / b;
    const float n1 = hypotf(v0, v1);
    v0 = v0 / n1; v1 = v1 / n1;
    X[2] = v0; X[3] = v1; X[4] = v1; X[5] = -v0;
  } else {
    X[0] = a; X[1] = c; X[2] = 1.f; X[3] = 0.f; X[4] = 0.f; X[5] = -1.f;
  }
}

__device__ __forceinline__ void eig3d(float a, float b, float c, float d, float e, float f, float out[3]) {
  const float pi = 3.14159265359f;
  float c2 = -(a + b + c);
  const float c1 = a * b + a * c + b * c - d * d - e * e - f * f;
  const float c0 = a * f * f + b * e * e + c * d * d - a * b * c - 2.f * d * e * f;
  float p = (float)((double)(c2 * c2) - 3.0 * (double)c1);
  const float q = -13.5f * c0 - c2 * c2 * c2 + 4.5f * c2 * c1;
  float phi = (1.f / 3.f) * atanf(sqrtf(27.f * (0.25f * c1 * c1 * (p - c1) + c0 * (q + 6.75f * c0))) / q);
  if (q < 0.f) phi += pi / 3.f;
  const float x1 = 2.f * cosf(phi), x2 = 2.f * cosf(phi + 2.f * pi / 3.f), x3 = 2.f * cosf(phi - 2.f * pi / 3.f);
  p = sqrtf(p) / 3.f;
  c2 = c2 / 3.f;
  out[0] = p * x1 - c2; out[1] = p * x2 - c2; out[2] = p * x3 - c2;
}

__device__ __forceinline__ void cross3(float a1, float a2, float a3, float b1, float b2, float b3, float o[3]) {
  o[0] = a2 * b3 - a3 * b2;
  o[1] = b1 * a3 - a1 * b3;
  o[2] = a1 * b2 - a2 * b1;
}

// nuclear 3-D (update_NormV_Nucl, radon_tgv_primal_dual_3d.py:290-520): returns the
// symmetric 3x3 projection matrix M (xx, yy, zz, xy, xz, yz) applied to every channel.
__device__ void nucl3d_matrix(float a, float b, float c, float r, float t, float d, float ainv, float M[6]) {
  const float epsdt = 0.0001f, epsr = 0.0001f, epsoo = 0.0001f / ainv;
  const float ndt = d * d + t * t;
  float oo = fminf(a, b);
  float sig[3], v0[3], v1[3], v2[3], X[6], u1 = 1.f, u2 = 0.f;
  if (ndt < epsdt * oo * oo && oo > epsoo) {
    diag2d(a, r, b, X);
    sig[0] = X[0]; sig[1] = X[1];
    sig[2] = (c * c < ndt) ? 1.f / epsdt : c;
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
    const float t1 = b * t - d * r, t2 = a * d - t * r;
    const float rs = sqrtf(ndt);
    u1 = d / rs;
    u2 = t / rs;
    const float bn = (d * (b * d + r * t) + t * (a * t + d * r)) / ndt;
    const float an = (t * t1 + d * t2) / ndt;
    const float rn = (-d * t1 + t * t2) / ndt;
    const float dn = rs;
    oo = fminf(c, bn);
    if (fabsf(rn) < epsr * oo) {
      diag2d(bn, dn, c, X);
      sig[0] = an; sig[1] = X[0]; sig[2] = X[1];
      v0[0] = 1.f; v0[1] = 0.f; v0[2] = 0.f;
      v1[0] = 0.f; v1[1] = X[2]; v1[2] = X[3];
      v2[0] = 0.f; v2[1] = X[4]; v2[2] = X[5];
    } else {
      eig3d(an, bn, c, rn, 0.f, dn, sig);
      cross3(an - sig[0], rn, 0.f, rn, bn - sig[0], dn, v0);
      float n = sqrtf(v0[0] * v0[0] + v0[1] * v0[1] + v0[2] * v0[2]);
      v0[0] /= n; v0[1] /= n; v0[2] /= n;
      cross3(v0[0], v0[1], v0[2], 0.f, dn, c - sig[1], v1);
      n = sqrtf(v1[0] * v1[0] + v1[1] * v1[1] + v1[2] * v1[2]);
      v1[0] /= n; v1[1] /= n; v1[2] /= n;
      cross3(v0[0], v0[1], v0[2], v1[0], v1[1], v1[2], v2);
      n = sqrtf(v2[0] * v2[0] + v2[1] * v2[1] + v2[2] * v2[2]);
      v2[0] /= n; v2[1] /= n; v2[2] /= n;
    }
  }
  float w[3][3];
  const float *vv[3] = {v0, v1, v2};
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    w[m][0] = u1 * vv[m][0] + u2 * vv[m][1];
    w[m][1] = -u2 * vv[m][0] + u1 * vv[m][1];
    w[m][2] = vv[m][2];
  }
  float S[3];
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    const float sg = sig[m] > 0.f ? sqrtf(sig[m]) : 0.f;
    S[m] = (sg * ainv > 1.f) ? 1.f / (ainv * sg) : 1.f;
  }
  M[0] = S[0] * w[0][0] * w[0][0] + S[1] * w[1][0] * w[1][0] + S[2] * w[2][0] * w[2][0];
  M[1] = S[0] * w[0][1] * w[0][1] + S[1] * w[1][1] * w[1][1] + S[2] * w[2][1] * w[2][1];
  M[2] = S[0] * w[0][2] * w[0][2] + S[1] * w[1][2] * w[1][2] + S[2] * w[2][2] * w[2][2];
  M[3] = S[0] * w[0][0] * w[0][1] + S[1] * w[1][0] * w[1][1] + S[2] * w[2][0] * w[2][1];
  M[4] = S[0] * w[0][0] * w[0][2] + S[1] * w[1][0] * w[1][2] + S[2] * w[2][0] * w[2][2];
  M[5] = S[0] * w[0][1] * w[0][2] + S[1] * w[1][1] * w[1][2] + S[2] * w[2][1] * w[2][2];
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

// ===========================================================================
// k_dual: update_v (3-D :615-634, 2-D :265-284), update_w (3-D :637-660,
// 2-D :286-304), NormV / NormW (3-D :290-610, 2-D :98-258)
// thread = one (pixel, z); it owns all C channels of that voxel.
// ===========================================================================
template <int DIM, bool TGV, int CPL, int CMAX>
__global__ void __launch_bounds__(256) k_dual(const IterParams P) {
  constexpr int K = DIM, KW = DIM == 3 ? 6 : 3;
  const Dims d = P.d;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
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

  // ---- projections
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
          a += vv[c][0] * vv[c][0]; b += vv[c][0] * vv[c][1]; cc += vv[c][1] * vv[c][1];
        }
        float M[3];
        nucl2d_matrix(a, b, cc, P.ainv1, M);
#pragma unroll
        for (int c = 0; c < CMAX; ++c) {
          if (c >= nC) break;
          const float v0 = vv[c][0], v1 = vv[c][1];
          vv[c][0] = v0 * M[0] + v1 * M[1];
          vv[c][1] = v0 * M[1] + v1 * M[2];
        }
      } else {
        float a = 0.f, b = 0.f, cc = 0.f, r = 0.f, tt = 0.f, dd = 0.f;
#pragma unroll
        for (int c = 0; c < CMAX; ++c) {
          if (c >= nC) break;
          const float X = vv[c][0], Y = vv[c][1], Z = vv[c][DIM - 1];
          a += X * X; b += Y * Y; cc += Z * Z; r += X * Y; tt += X * Z; dd += Y * Z;
        }
        float M[6];
        nucl3d_matrix(a, b, cc, r, tt, dd, P.ainv1, M);
#pragma unroll
        for (int c = 0; c < CMAX; ++c) {
          if (c >= nC) break;
          const float A = vv[c][0], B = vv[c][1], Cc = vv[c][DIM - 1];
          vv[c][0] = A * M[0] + B * M[3] + Cc * M[4];
          vv[c][1] = A * M[3] + B * M[1] + Cc * M[5];
          vv[c][DIM - 1] = A * M[4] + B * M[5] + Cc * M[2];
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

// ===========================================================================
// forward projection: kernel `radon` (3-D :773-816).  Ray (i, j) of slice s:
// acc = sum over rows y and x in [x_low, x_high] of (1 - |x X + y Y + off - i|)+ img.
// The arithmetic is the reference's, in its order and without contraction.
// ===========================================================================
__device__ __forceinline__ void ray_rows(const float4 o, int i, int N, int &ylo, int &yhi) {
  // rows whose x-extent [0, N-1] can reach detector coordinate (i-1, i+1); a
  // conservative superset (the per-row bounds below decide exactly).
  ylo = 0; yhi = N - 1;
  if (fabsf(o.y) < 1e-3f) return;
  const float tx = (float)(N - 1) * o.x;
  const float tmin = fminf(0.f, tx), tmax = fmaxf(0.f, tx);
  float ya, yb;
  if (o.y > 0.f) {
    ya = ((float)(i - 1) - o.z - tmax) / o.y;
    yb = ((float)(i + 1) - o.z - tmin) / o.y;
  } else {
    ya = ((float)(i + 1) - o.z - tmin) / o.y;
    yb = ((float)(i - 1) - o.z - tmax) / o.y;
  }
  ya = fminf(fmaxf(ya, -2.f), (float)N + 1.f);
  yb = fminf(fmaxf(yb, -2.f), (float)N + 1.f);
  ylo = max(0, (int)floorf(ya) - 1);
  yhi = min(N - 1, (int)ceilf(yb) + 1);
}

__device__ __forceinline__ float radon_ray(const float *__restrict__ img, size_t S, int N, const float4 o, int i) {
  int ylo, yhi;
  ray_rows(o, i, N, ylo, yhi);
  const float fi = (float)i, fim = (float)(i - 1), fip = (float)(i + 1);
  float acc = 0.f;
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
      if (wgt > 0.f) acc = __fadd_rn(acc, __fmul_rn(wgt, __ldg(row + (size_t)x * S)));
    }
  }
  return acc;
}

// k_fwd: radon of ubar fused with update_lambda_KL (3-D :690-704) or _L2 (:677-688).
template <int DISC>
__global__ void __launch_bounds__(256) k_fwd(const IterParams P) {
  const Dims d = P.d;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)d.nbin) return;
  const int b = (int)(t / d.S);
  const int s = (int)(t - (long long)b * d.S);
  const int j = b / d.nd, i = b - j * d.nd;
  const float4 o = __ldg(P.ofs + j);
  const float acc = radon_ray(P.ubar + s, d.S, d.N, o, i);
  const size_t q = (size_t)t;
  P.ku[q] = acc;
  const float m = __ldg(P.mu + s / d.Nz);
  const float sd = P.sigma_data;
  float lam = P.lam[q];
  if (DISC == KL) {
    const float sv = lam + sd * acc;
    const float wv = sv - m;
    const float dv = wv * wv + 4.f * sd * P.f[q] * m;
    lam = sv - 0.5f * (wv + sqrtf(dv));
  } else {
    lam = (lam + sd * (acc - P.f[q])) * m;
  }
  P.lam[q] = lam;
}

// ===========================================================================
// back projection: kernel `radon_ad` (3-D :818-844): linear interpolation
// between detector bins floor(t) and floor(t)+1 at t = dot((x, y, 1, 0), ofs[j]).
// ===========================================================================
__device__ __forceinline__ float radon_ad_pixel(const float *__restrict__ lam, size_t S, int nd, int nang,
                                                const float4 *__restrict__ ofs, float xf, float yf) {
  float acc = 0.f;
  const float fnd = (float)nd;
  for (int j = 0; j < nang; ++j) {
    const float4 o = __ldg(ofs + j);
    const float tt = __fadd_rn(__fadd_rn(__fmul_rn(xf, o.x), __fmul_rn(yf, o.y)), o.z);
    if (tt > -1.f && tt < fnd) {
      const float fl = floorf(tt);
      const float p = fminf(__fsub_rn(tt, fl), 0x1.fffffep-1f);
      const int il = (int)fl;
      const float *lj = lam + (size_t)j * nd * S;
      if (il >= 0) acc = __fadd_rn(acc, __fmul_rn(__fsub_rn(1.0f, p), __ldg(lj + (size_t)il * S)));
      if (il <= nd - 2) acc = __fadd_rn(acc, __fmul_rn(p, __ldg(lj + (size_t)(il + 1) * S)));
    }
  }
  return acc;
}

// k_primal: radon_ad of lambda + update_u (3-D :706-729, 2-D :340-357) +
// update_p (3-D :734-757, 2-D :359-376) + extrapolation and swap (:1217-1221).
// thread = one (pixel, s).
template <int DIM, bool TGV>
__global__ void __launch_bounds__(256) k_primal(const IterParams P) {
  const Dims d = P.d;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)d.vol) return;
  const int pix = (int)(t / d.S);
  const int s = (int)(t - (long long)pix * d.S);
  const int y = pix / d.N, x = pix - y * d.N;
  const int z = (DIM == 3) ? s % d.Nz : 0;
  const size_t S = d.S, rowS = (size_t)d.N * S, vol = d.vol, i = (size_t)t;

  const float kstar = radon_ad_pixel(P.lam + s, S, d.nd, d.nang, P.ofs, (float)x, (float)y);

  // divergence of v: backward differences (adjoint of the forward gradient)
  const float *__restrict__ v = P.v;
  float a = v[i], b = v[vol + i];
  if (x == d.N - 1) a = 0.f;
  if (x > 0) a -= v[i - S];
  if (y == d.N - 1) b = 0.f;
  if (y > 0) b -= v[vol + i - rowS];
  const float uo = P.u[i];
  float un;
  if (DIM == 3) {
    float c = v[2 * vol + i];
    if (z == d.Nz - 1) c = 0.f;
    if (z > 0) c -= v[2 * vol + i - 1];
    c /= P.stepsize;
    un = uo + P.tau * (a + b + c - P.norming * kstar);
  } else {
    un = uo + P.tau * (a + b - P.norming * kstar);
  }
  if (un < 0.f) un = 0.f;
  P.ubar[i] = 2.0f * un - uo;
  P.u[i] = un;

  if (TGV) {
    const float *__restrict__ w = P.w;
    if (DIM == 3) {
      // rows of the symmetric tensor: (w0 w3 w4), (w3 w1 w5), (w4 w5 w2)
      const int rx[3] = {0, 3, 4}, ry[3] = {3, 1, 5}, rz[3] = {4, 5, 2};
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        float A = -w[rx[k] * vol + i], B = -w[ry[k] * vol + i], Cz = -w[rz[k] * vol + i];
        if (x == 0) A = 0.f;
        if (x < d.N - 1) A += w[rx[k] * vol + i + S];
        if (y == 0) B = 0.f;
        if (y < d.N - 1) B += w[ry[k] * vol + i + rowS];
        if (z == 0) Cz = 0.f;
        if (z < d.Nz - 1) Cz += w[rz[k] * vol + i + 1];
        Cz /= P.stepsize;
        const float po = P.p[k * vol + i];
        const float pn = po + P.tau * (v[k * vol + i] + A + B + Cz);
        P.pbar[k * vol + i] = 2.0f * pn - po;
        P.p[k * vol + i] = pn;
      }
    } else {
      const int rx[2] = {0, 2}, ry[2] = {2, 1};
#pragma unroll
      for (int k = 0; k < 2; ++k) {
        float A = -w[rx[k] * vol + i], B = -w[ry[k] * vol + i];
        if (x == 0) A = 0.f;
        if (x < d.N - 1) A += w[rx[k] * vol + i + S];
        if (y == 0) B = 0.f;
        if (y < d.N - 1) B += w[ry[k] * vol + i + rowS];
        const float po = P.p[k * vol + i];
        const float pn = po + P.tau * (v[k * vol + i] + A + B);
        P.pbar[k * vol + i] = 2.0f * pn - po;
        P.p[k * vol + i] = pn;
      }
    }
  }
}

// ===========================================================================
// standalone projectors and layout transposes
// ===========================================================================
__global__ void k_radon(const float *__restrict__ img, float *__restrict__ sino, const float4 *__restrict__ ofs,
                        int N, int nd, int nang, int S) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)nd * nang * S) return;
  const int b = (int)(t / S), s = (int)(t - (long long)b * S);
  const int j = b / nd, i = b - j * nd;
  sino[t] = radon_ray(img + s, S, N, __ldg(ofs + j), i);
}

__global__ void k_radon_ad(const float *__restrict__ sino, float *__restrict__ img, const float4 *__restrict__ ofs,
                           int N, int nd, int nang, int S) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)N * N * S) return;
  const int pix = (int)(t / S), s = (int)(t - (long long)pix * S);
  const int y = pix / N, x = pix - y * N;
  img[t] = radon_ad_pixel(sino + s, S, nd, nang, ofs, (float)x, (float)y);
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

template <class T>
__global__ void k_fill(T *__restrict__ x, size_t n, T v) {
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) x[k] = v;
}

// ===========================================================================
// FP64 operator-norm power iteration (radon_normest, 3-D :1018-1030), one slice
// ===========================================================================
__global__ void k_radon64(const double *__restrict__ img, double *__restrict__ sino, const dvec4 *__restrict__ ofs,
                          int N, int nd, int nang) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nd * nang) return;
  const int j = t / nd, i = t - j * nd;
  const dvec4 o = ofs[j];
  double acc = 0.0;
  for (int y = 0; y < N; ++y) {
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
  sino[t] = acc;
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
// host-side launchers
// ===========================================================================
static inline unsigned blocks_for(long long n, int bs) { return (unsigned)((n + bs - 1) / bs); }

template <int DIM, bool TGV, int CPL>
static cudaError_t launch_dual_c(const IterParams &P, cudaStream_t st) {
  const long long n = (long long)P.d.N * P.d.N * P.d.Nz;
  const unsigned g = blocks_for(n, 256);
  const int C = P.d.C;
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

cudaError_t launch_fwd(const IterParams &P, int disc, cudaStream_t st) {
  const unsigned g = blocks_for((long long)P.d.nbin, 256);
  if (disc == KL) k_fwd<KL><<<g, 256, 0, st>>>(P);
  else k_fwd<L2><<<g, 256, 0, st>>>(P);
  return cudaGetLastError();
}

cudaError_t launch_primal(const IterParams &P, int tgv, cudaStream_t st) {
  const unsigned g = blocks_for((long long)P.d.vol, 256);
  if (P.d.dim == 3) {
    if (tgv) k_primal<3, true><<<g, 256, 0, st>>>(P);
    else k_primal<3, false><<<g, 256, 0, st>>>(P);
  } else {
    if (tgv) k_primal<2, true><<<g, 256, 0, st>>>(P);
    else k_primal<2, false><<<g, 256, 0, st>>>(P);
  }
  return cudaGetLastError();
}

cudaError_t launch_radon(const float *img, float *sino, const float4 *ofs, int N, int nd, int nang, int S,
                         cudaStream_t st) {
  k_radon<<<blocks_for((long long)nd * nang * S, 256), 256, 0, st>>>(img, sino, ofs, N, nd, nang, S);
  return cudaGetLastError();
}

cudaError_t launch_radon_ad(const float *sino, float *img, const float4 *ofs, int N, int nd, int nang, int S,
                            cudaStream_t st) {
  k_radon_ad<<<blocks_for((long long)N * N * S, 256), 256, 0, st>>>(sino, img, ofs, N, nd, nang, S);
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

// power iteration: 30 rounds of  s = sum(img); img /= s; img = R^T R img  from the
// all-ones image; returns sqrt(s) (the reference's 10 rounds from randn, in FP32).
cudaError_t normest64(const dvec4 *ofs, int N, int nd, int nang, int rounds, double *d_img, double *d_sino,
                      double *d_part, double *out, cudaStream_t st) {
  const size_t n = (size_t)N * N;
  const int nb = 64;
  cudaError_t e;
  for (int r = 0; r < rounds; ++r) {
    k_sum64_partial<<<nb, 256, 0, st>>>(d_img, n, d_part);
    k_sum64_partial<<<1, 256, 0, st>>>(d_part, nb, d_part + nb);
    k_scale64<<<64, 256, 0, st>>>(d_img, n, d_part + nb);
    k_radon64<<<blocks_for((long long)nd * nang, 128), 128, 0, st>>>(d_img, d_sino, ofs, N, nd, nang);
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
