/*
 * tgv_oracle.c -- CPU restatement of Graptor's primal-dual TGV/TV reconstruction.
 *
 * TEST INFRASTRUCTURE (the oracle).  Only tests/, the package's smoke check and
 * bench.py's CPU-baseline leg load this file's library, and only as the checker
 * or the timed CPU baseline; the product never calls it.
 *
 * Every function restates one piece of the reference's algorithm with the same
 * FP32 operation order, citing the reference line it follows
 * (radon_tgv_primal_dual_{2d,3d}.py).  Compiled with -ffp-contract=off so that
 * no multiply-add is fused, which is how the reference's kernels evaluate when
 * run through the oracle harness (oracle/refshim).
 *
 * Layout (C order, x fastest):
 *   image-domain scalar  u[s][y][x]            s = c*Nz + z  (channel-major, like
 *                                              the reference's Nz*Number_Channels axis)
 *   vector fields        p[k][s][y][x]         k = component (2-D: 2, 3-D: 3)
 *   symmetric tensor     w[k][s][y][x]         3-D: (xx, yy, zz, xy, xz, yz); 2-D: (xx, yy, xy)
 *   sinogram             f[s][j][i]            j = angle, i = detector
 * The reference stores vectors interleaved and padded (float3 = 16 B, W as float8);
 * the arithmetic does not depend on that.
 */
#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define EXPORT __attribute__((visibility("default")))

typedef struct {
  int dim;          /* 2 or 3 */
  int N;            /* image side (= detector count in the reference) */
  int Nz;           /* slices per channel (2-D: number of independent slices) */
  int C;            /* channels */
  int nd, nang;     /* detectors, angles */
  int discrepancy;  /* 0 = KL, 1 = L2 */
  int regularisation; /* 0 = TV, 1 = TGV */
  int coupling;     /* 0 = uncorrelated, 1 = Frobenius, 2 = nuclear */
  float stepsize;   /* slice step (3-D z-derivative divisor) */
} or_desc;

/* ------------------------------------------------------------------------- */
/* geometry: radon_struct, radon_tgv_primal_dual_3d.py:947-979                  */
/* ofs[j] = (X, Y, offset, Xinv) per angle, computed in double, stored float.  */
EXPORT void or_radon_struct(int N, int nd, int nang, const double *angles, float *ofs) {
  const double mid_dom = (N - 1) / 2.0, mid_det = (nd - 1.0) / 2.0;
  for (int j = 0; j < nang; ++j) {
    double X = cos(angles[j]), Y = sin(angles[j]), Xinv = 1.0 / X;
    if (fabs(Xinv) > 10.0 * nd) { /* near-vertical rays made vertical (:962-966) */
      X = 0.0;
      Y = nearbyint(sin(angles[j])); /* numpy round: half to even */
      Xinv = 0.0;
    }
    double off = mid_det - X * mid_dom - Y * mid_dom;
    ofs[4 * j + 0] = (float)X;
    ofs[4 * j + 1] = (float)Y;
    ofs[4 * j + 2] = (float)off;
    ofs[4 * j + 3] = (float)Xinv;
  }
}

/* ------------------------------------------------------------------------- */
/* forward projection: kernel `radon`, radon_tgv_primal_dual_3d.py:773-816       */
EXPORT void or_radon(float *sino, const float *img, const float *ofs, int N, int nd, int nang, int S) {
  const int X = N, Y = N;
#pragma omp parallel for collapse(2) schedule(static)
  for (int s = 0; s < S; ++s)
    for (int j = 0; j < nang; ++j) {
      const float ox = ofs[4 * j], oy = ofs[4 * j + 1], oz = ofs[4 * j + 2], ow = ofs[4 * j + 3];
      for (int i = 0; i < nd; ++i) {
        const float *row = img + (size_t)s * X * Y;
        float acc = 0.0f;
        for (int y = 0; y < Y; ++y, row += X) {
          int xl, xh;
          const float d = (float)y * oy + oz;
          if (ox == 0.0f) {
            if (d > (float)(i - 1) && d < (float)(i + 1)) { xl = 0; xh = X - 1; }
            else continue;
          } else if (ox > 0.0f) {
            xl = (int)(((float)(i - 1) - d) * ow);
            xh = (int)(((float)(i + 1) - d) * ow);
          } else {
            xl = (int)(((float)(i + 1) - d) * ow);
            xh = (int)(((float)(i - 1) - d) * ow);
          }
          if (xl < 0) xl = 0;
          if (xh > X - 1) xh = X - 1;
          for (int x = xl; x <= xh; ++x) {
            const float wgt = 1.0f - fabsf((float)x * ox + d - (float)i);
            if (wgt > 0.0f) acc += wgt * row[x];
          }
        }
        sino[((size_t)s * nang + j) * nd + i] = acc;
      }
    }
}

/* back projection: kernel `radon_ad`, radon_tgv_primal_dual_3d.py:818-844      */
EXPORT void or_radon_ad(float *img, const float *sino, const float *ofs, int N, int nd, int nang, int S) {
  const int X = N, Y = N, I = nd;
#pragma omp parallel for collapse(2) schedule(static)
  for (int s = 0; s < S; ++s)
    for (int y = 0; y < Y; ++y)
      for (int x = 0; x < X; ++x) {
        const float *sn = sino + (size_t)s * nang * nd;
        float acc = 0.0f;
        for (int j = 0; j < nang; ++j, sn += I) {
          /* dot((x, y, 1, 0), ofs[j]) */
          const float t = (float)x * ofs[4 * j] + (float)y * ofs[4 * j + 1] + 1.0f * ofs[4 * j + 2] +
                          0.0f * ofs[4 * j + 3];
          if (t > -1.0f && t < (float)I) {
            const float fl = floorf(t);
            float p = t - fl; /* OpenCL fract */
            if (p > 0x1.fffffep-1f) p = 0x1.fffffep-1f;
            if (fl >= 0.0f) acc += (1.0f - p) * sn[(int)fl];
            if (fl <= (float)(I - 2)) acc += p * sn[(int)(fl + 1.0f)];
          }
        }
        img[((size_t)s * Y + y) * X + x] = acc;
      }
}

/* ------------------------------------------------------------------------- */
/* dual step on v: update_v, 3-D :615-634, 2-D :265-284                         */
EXPORT void or_update_v(const or_desc *d, float *v, const float *ubar, const float *pbar, float sigma) {
  const int N = d->N, Nz = d->dim == 3 ? d->Nz : 1, K = d->dim;
  const int S = d->Nz * d->C;
  const size_t plane = (size_t)N * N, vol = plane * S;
#pragma omp parallel for collapse(2) schedule(static)
  for (int s = 0; s < S; ++s)
    for (int y = 0; y < N; ++y)
      for (int x = 0; x < N; ++x) {
        const int z = s % Nz;
        const size_t i = (size_t)s * plane + (size_t)y * N + x;
        const float mu = -ubar[i];
        float g[3];
        g[0] = (x < N - 1) ? mu + ubar[i + 1] : 0.0f;
        g[1] = (y < N - 1) ? mu + ubar[i + N] : 0.0f;
        if (K == 3) {
          g[2] = (z < Nz - 1) ? mu + ubar[i + plane] : 0.0f;
          g[2] = g[2] / d->stepsize;
        }
        for (int k = 0; k < K; ++k) v[k * vol + i] = v[k * vol + i] + sigma * (g[k] - pbar[k * vol + i]);
      }
}

/* dual step on w: update_w, 3-D :637-660, 2-D :286-304 (TV: update_w_empty)     */
EXPORT void or_update_w(const or_desc *d, float *w, const float *pbar, float sigma) {
  const int N = d->N, Nz = d->dim == 3 ? d->Nz : 1;
  const int S = d->Nz * d->C, KW = d->dim == 3 ? 6 : 3;
  const size_t plane = (size_t)N * N, vol = plane * S;
  if (!d->regularisation) { memset(w, 0, sizeof(float) * KW * vol); return; }
#pragma omp parallel for collapse(2) schedule(static)
  for (int s = 0; s < S; ++s)
    for (int y = 0; y < N; ++y)
      for (int x = 0; x < N; ++x) {
        const int z = s % Nz;
        const size_t i = (size_t)s * plane + (size_t)y * N + x;
        float a[3], b[3], c[3], e[6];
        const int K = d->dim;
        for (int k = 0; k < K; ++k) {
          const float pk = pbar[k * vol + i];
          a[k] = x > 0 ? pk - pbar[k * vol + i - 1] : 0.0f;  /* backward, zero at index 0 */
          b[k] = y > 0 ? pk - pbar[k * vol + i - N] : 0.0f;
          if (K == 3) c[k] = (z > 0 ? pk - pbar[k * vol + i - plane] : 0.0f) / d->stepsize;
        }
        if (K == 3) {
          e[0] = a[0]; e[1] = b[1]; e[2] = c[2];
          e[3] = 0.5f * (a[1] + b[0]);
          e[4] = 0.5f * (a[2] + c[0]);
          e[5] = 0.5f * (b[2] + c[1]);
        } else {
          e[0] = a[0]; e[1] = b[1];
          e[2] = 0.5f * (a[1] + b[0]);
        }
        for (int k = 0; k < KW; ++k) w[k * vol + i] = w[k * vol + i] + sigma * e[k];
      }
}

/* ball projections of v: update_NormV_{frob,unchor}, 3-D :529-565, 2-D :98-119, :208-220;
 * nuclear 2-D: update_NormV_Nucl :124-204                                         */
static void nucl2d_pixel(float *v, size_t vol, size_t i, size_t cstride, int C, float alphainv) {
  float a = 0, b = 0, c = 0;
  for (int ch = 0; ch < C; ++ch) {
    const float v0 = v[i + ch * cstride], v1 = v[vol + i + ch * cstride];
    a += v0 * v0; b += v0 * v1; c += v1 * v1;
  }
  const float eps = 0.00001f;
  float sigma1, sigma2, S1, S2, M0, M1, M2;
  const float o = a < c ? a : c;
  if ((b * b) / (o * o) > eps && o * o > 0) {
    const float dd = a + c, e = a - c;
    float f = 4 * b * b + e * e;
    if (f < 0) f = 0; else f = powf(f, 0.5f);
    sigma2 = (dd - f > 0) ? sqrtf((dd - f) * 0.5f) : 0.0f;
    sigma1 = (dd + f > 0) ? sqrtf((dd + f) * 0.5f) : 0.0f;
    const float g = (e + f) * 0.5f, h = (e - f) * 0.5f;
    float q0 = g * a + b * b, q1 = g * b + c * b;
    float q2 = h * a + b * b, q3 = h * b + b * c;
    const float n1 = hypotf(q0, q1), n2 = hypotf(q2, q3);
    if (n1 > 0) { q0 = q0 / n1; q1 = q1 / n1; }
    if (n2 > 0) { q2 = q2 / n2; q3 = q3 / n2; }
    S1 = ((sigma1 * alphainv) > 1) ? 1 / (sigma1 * alphainv) : 1.0f;
    S2 = ((sigma2 * alphainv) > 1) ? 1 / (sigma2 * alphainv) : 1.0f;
    M0 = q0 * q0 * S1 + q2 * q2 * S2;
    M2 = q1 * q1 * S1 + q3 * q3 * S2;
    M1 = S1 * q0 * q1 + S2 * q2 * q3;
  } else {
    sigma1 = powf(a, 0.5f);
    sigma2 = powf(c, 0.5f);
    S1 = ((alphainv * sigma1) > 1) ? 1 / (alphainv * sigma1) : 1.0f;
    S2 = ((alphainv * sigma2) > 1) ? 1 / (alphainv * sigma2) : 1.0f;
    M0 = S1; M2 = S2; M1 = 0.0f;
  }
  for (int ch = 0; ch < C; ++ch) {
    const float v0 = v[i + ch * cstride], v1 = v[vol + i + ch * cstride];
    v[i + ch * cstride] = v0 * M0 + v1 * M1;
    v[vol + i + ch * cstride] = v0 * M1 + v1 * M2;
  }
}

/* nuclear 3-D: update_NormV_Nucl with its helpers diagonalization2d, eigenvalues3d,
 * crossproduct, radon_tgv_primal_dual_3d.py:190-520.  The helpers return their
 * results through an output array (the original returns pointers to locals).     */
static float omin(float x, float y) { return y < x ? y : x; } /* OpenCL min */

static void diag2d(float a, float b, float c, float out[6]) { /* :222-284 */
  const float eps = 0.001f;
  float sigma1, sigma2, v0, v1, v2, v3;
  const float o = omin(a, c);
  if ((b * b) / (o * o) > eps && o * o > 0) {
    const float dd = a + c, e = a - c;
    float f = 4 * b * b + e * e;
    if (f < 0) f = 0; else f = sqrtf(f);
    sigma2 = (dd - f > 0) ? (dd - f) * 0.5f : 0;
    sigma1 = (dd + f > 0) ? (dd + f) * 0.5f : 0;
    const float h = (e - f) * 0.5f;
    v0 = 1; v1 = -h / b;
    const float n1 = hypotf(v0, v1);
    v0 = v0 / n1; v1 = v1 / n1;
    v2 = v1; v3 = -v0;
  } else {
    sigma1 = a; sigma2 = c; v0 = 1; v1 = 0; v2 = 0; v3 = -1;
  }
  out[0] = sigma1; out[1] = sigma2; out[2] = v0; out[3] = v1; out[4] = v2; out[5] = v3;
}

static void eig3d(float a, float b, float c, float d, float e, float f, float out[3]) { /* :190-221 */
  const float pi = (float)3.14159265359;
  float c2 = -(a + b + c);
  const float c1 = a * b + a * c + b * c - d * d - e * e - f * f;
  const float c0 = a * f * f + b * e * e + c * d * d - a * b * c - 2 * d * e * f;
  float p = (float)((double)(c2 * c2) - 3. * (double)c1);
  const float q = -27.f / 2.f * c0 - powf(c2, 3) + 9.f / 2.f * c2 * c1;
  float phi = 1.f / 3.f * atanf(sqrtf(27.f * (1.f / 4.f * c1 * c1 * (p - c1) + c0 * (q + 27.f / 4.f * c0))) / q);
  if (q < 0) phi += pi / 3.f;
  const float x1 = 2 * cosf(phi), x2 = 2 * cosf(phi + 2 * pi / 3.f), x3 = 2 * cosf(phi - 2 * pi / 3.f);
  p = sqrtf(p) / 3.f;
  c2 = c2 / 3.f;
  out[0] = p * x1 - c2; out[1] = p * x2 - c2; out[2] = p * x3 - c2;
}

static void cross3(float a1, float a2, float a3, float b1, float b2, float b3, float o[3]) { /* :224-231 */
  o[0] = a2 * b3 - a3 * b2;
  o[1] = b1 * a3 - a1 * b3;
  o[2] = a1 * b2 - a2 * b1;
}

static void nucl3d_voxel(float *V, size_t vol, size_t i, size_t cstride, int C, float alphainv) {
  float a = 0, b = 0, c = 0, r = 0, t = 0, d = 0;
  for (int ch = 0; ch < C; ++ch) {
    const size_t k = i + ch * cstride;
    const float x = V[k], y = V[vol + k], z = V[2 * vol + k];
    a += x * x; b += y * y; c += z * z; r += x * y; t += x * z; d += y * z;
  }
  const float epsdt = 0.0001f, epsr = 0.0001f, epsoo = 0.0001f / alphainv;
  float ndt = d * d + t * t, oo = omin(a, b);
  float sig[3], v0[3], v1[3], v2[3], X[6], u1, u2;
  if (ndt < epsdt * oo * oo && oo > epsoo) {
    diag2d(a, r, b, X);
    sig[0] = X[0]; sig[1] = X[1];
    sig[2] = (c * c < ndt) ? 1 / epsdt : c;
    v0[0] = X[2]; v0[1] = X[3]; v0[2] = 0.f;
    v1[0] = X[4]; v1[1] = X[5]; v1[2] = 0.f;
    v2[0] = 0.f; v2[1] = 0.f; v2[2] = 1.f;
    u1 = 1.f; u2 = 0.f;
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
    u1 = 1.f; u2 = 0.f;
  } else {
    /* rotate about z so that t vanishes (:434-452) */
    const float t1 = b * t - d * r, t2 = a * d - t * r;
    u1 = d / sqrtf(ndt);
    u2 = t / sqrtf(ndt);
    b = (d * (b * d + r * t) + t * (a * t + d * r)) / ndt;
    a = (t * t1 + d * t2) / ndt;
    r = (-d * t1 + t * t2) / ndt;
    d = sqrtf(ndt);
    oo = omin(c, b);
    if (fabsf(r) < epsr * oo) {
      diag2d(b, d, c, X);
      sig[0] = a; sig[1] = X[0]; sig[2] = X[1];
      v0[0] = 1.f; v0[1] = 0.f; v0[2] = 0.f;
      v1[0] = 0.f; v1[1] = X[2]; v1[2] = X[3];
      v2[0] = 0.f; v2[1] = X[4]; v2[2] = X[5];
    } else {
      float ev[3];
      eig3d(a, b, c, r, 0, d, ev);
      sig[0] = ev[0]; sig[1] = ev[1]; sig[2] = ev[2];
      cross3(a - sig[0], r, 0, r, b - sig[0], d, v0);
      const float n1 = sqrtf(v0[0] * v0[0] + v0[1] * v0[1] + v0[2] * v0[2]);
      for (int k = 0; k < 3; ++k) v0[k] /= n1;
      cross3(v0[0], v0[1], v0[2], 0, d, c - sig[1], v1);
      const float n2 = sqrtf(v1[0] * v1[0] + v1[1] * v1[1] + v1[2] * v1[2]);
      for (int k = 0; k < 3; ++k) v1[k] /= n2;
      cross3(v0[0], v0[1], v0[2], v1[0], v1[1], v1[2], v2);
      const float n3 = sqrtf(v2[0] * v2[0] + v2[1] * v2[1] + v2[2] * v2[2]);
      for (int k = 0; k < 3; ++k) v2[k] /= n3;
    }
  }
  /* eigenvectors back in the original frame (:476-479) */
  float w[3][3];
  const float *vv[3] = {v0, v1, v2};
  for (int m = 0; m < 3; ++m) {
    w[m][0] = u1 * vv[m][0] + u2 * vv[m][1];
    w[m][1] = -u2 * vv[m][0] + u1 * vv[m][1];
    w[m][2] = vv[m][2];
  }
  float S[3];
  for (int m = 0; m < 3; ++m) {
    sig[m] = sig[m] > 0 ? sqrtf(sig[m]) : 0;
    S[m] = (sig[m] * alphainv > 1) ? 1.f / (alphainv * sig[m]) : 1.f;
  }
  /* projection matrix M = W diag(S) W^T (:500-507) */
  float M[6];
  M[0] = S[0] * w[0][0] * w[0][0] + S[1] * w[1][0] * w[1][0] + S[2] * w[2][0] * w[2][0];
  M[1] = S[0] * w[0][1] * w[0][1] + S[1] * w[1][1] * w[1][1] + S[2] * w[2][1] * w[2][1];
  M[2] = S[0] * w[0][2] * w[0][2] + S[1] * w[1][2] * w[1][2] + S[2] * w[2][2] * w[2][2];
  M[3] = S[0] * w[0][0] * w[0][1] + S[1] * w[1][0] * w[1][1] + S[2] * w[2][0] * w[2][1];
  M[4] = S[0] * w[0][0] * w[0][2] + S[1] * w[1][0] * w[1][2] + S[2] * w[2][0] * w[2][2];
  M[5] = S[0] * w[0][1] * w[0][2] + S[1] * w[1][1] * w[1][2] + S[2] * w[2][1] * w[2][2];
  for (int ch = 0; ch < C; ++ch) {
    const size_t k = i + ch * cstride;
    const float A = V[k], B = V[vol + k], Cc = V[2 * vol + k];
    V[k] = A * M[0] + B * M[3] + Cc * M[4];
    V[vol + k] = A * M[3] + B * M[1] + Cc * M[5];
    V[2 * vol + k] = A * M[4] + B * M[5] + Cc * M[2];
  }
}

EXPORT void or_norm_v(const or_desc *d, float *v, float alphainv) {
  const int N = d->N, Nz = d->Nz, C = d->C, K = d->dim;
  const size_t plane = (size_t)N * N, vol = plane * Nz * C, cstride = plane * Nz;
#pragma omp parallel for collapse(2) schedule(static)
  for (int z = 0; z < Nz; ++z)
    for (int y = 0; y < N; ++y)
      for (int x = 0; x < N; ++x) {
        const size_t i = (size_t)z * plane + (size_t)y * N + x;
        if (d->coupling == 1) {
          float norm = 0.0f;
          for (int ch = 0; ch < C; ++ch) {
            const size_t k = i + ch * cstride;
            norm = K == 3 ? hypotf(hypotf(hypotf(v[k], v[vol + k]), v[2 * vol + k]), norm)
                          : hypotf(hypotf(v[k], v[vol + k]), norm);
          }
          norm = norm * alphainv;
          if (norm > 1.0f)
            for (int ch = 0; ch < C; ++ch)
              for (int c = 0; c < K; ++c) v[c * vol + i + ch * cstride] = v[c * vol + i + ch * cstride] / norm;
        } else if (d->coupling == 0) {
          for (int ch = 0; ch < C; ++ch) {
            const size_t k = i + ch * cstride;
            const float norm = (K == 3 ? hypotf(hypotf(v[k], v[vol + k]), v[2 * vol + k])
                                       : hypotf(v[k], v[vol + k])) * alphainv;
            if (norm > 1.0f)
              for (int c = 0; c < K; ++c) v[c * vol + k] /= norm;
          }
        } else if (K == 2) {
          nucl2d_pixel(v, vol, i, cstride, C, alphainv);
        } else {
          nucl3d_voxel(v, vol, i, cstride, C, alphainv);
        }
      }
}

/* ball projections of w: update_NormW_{frob,unchor}, 3-D :573-610, 2-D :223-258
 * (nuclear coupling uses the Frobenius projection for w, 3-D :1118-1124)          */
EXPORT void or_norm_w(const or_desc *d, float *w, float alphainv) {
  if (!d->regularisation) return; /* update_NormW_empty */
  const int N = d->N, Nz = d->Nz, C = d->C, K = d->dim, KW = K == 3 ? 6 : 3;
  const size_t plane = (size_t)N * N, vol = plane * Nz * C, cstride = plane * Nz;
#pragma omp parallel for collapse(2) schedule(static)
  for (int z = 0; z < Nz; ++z)
    for (int y = 0; y < N; ++y)
      for (int x = 0; x < N; ++x) {
        const size_t i = (size_t)z * plane + (size_t)y * N + x;
#define W_(c, k) w[(size_t)(c) * vol + (k)]
        if (d->coupling != 0) {
          float norm = 0.0f;
          for (int ch = 0; ch < C; ++ch) {
            const size_t k = i + ch * cstride;
            if (K == 3)
              norm = hypotf(hypotf(hypotf(W_(0, k), W_(1, k)), hypotf(W_(2, k), 1.4142f * W_(3, k))),
                            hypotf(1.4142f * hypotf(W_(4, k), W_(5, k)), norm));
            else
              norm = hypotf(hypotf(W_(0, k), W_(1, k)), hypotf(2.f * W_(2, k), norm)); /* factor 2: 2-D :232 */
          }
          norm = alphainv * norm;
          if (norm > 1.0f)
            for (int ch = 0; ch < C; ++ch)
              for (int c = 0; c < KW; ++c) W_(c, i + ch * cstride) = W_(c, i + ch * cstride) / norm;
        } else {
          for (int ch = 0; ch < C; ++ch) {
            const size_t k = i + ch * cstride;
            float norm;
            if (K == 3) /* 1.4142 scales w4 only, not w5 (3-D :603) */
              norm = hypotf(hypotf(hypotf(W_(0, k), W_(1, k)), hypotf(W_(2, k), 1.4142f * W_(3, k))),
                            hypotf(1.4142f * W_(4, k), W_(5, k))) * alphainv;
            else
              norm = hypotf(hypotf(W_(0, k), W_(1, k)), 1.4142f * W_(2, k)) * alphainv;
            if (norm > 1.0f)
              for (int c = 0; c < KW; ++c) W_(c, k) = W_(c, k) / norm;
          }
        }
#undef W_
      }
}

/* data-term dual prox: update_lambda_KL :690-704 / update_lambda_L2 :677-688      */
EXPORT void or_update_lambda(const or_desc *d, float *lam, const float *ku, const float *f, float sigma,
                             const float *mu) {
  const int S = d->Nz * d->C;
  const size_t per = (size_t)d->nd * d->nang;
#pragma omp parallel for schedule(static)
  for (int s = 0; s < S; ++s) {
    const float m = mu[s / d->Nz];
    for (size_t q = 0; q < per; ++q) {
      const size_t i = (size_t)s * per + q;
      if (d->discrepancy == 0) {
        const float sv = lam[i] + sigma * ku[i];
        const float wv = sv - m;
        const float dv = wv * wv + 4 * sigma * f[i] * m;
        lam[i] = sv - 0.5f * (wv + sqrtf(dv));
      } else {
        lam[i] = (lam[i] + sigma * (ku[i] - f[i])) * m;
      }
    }
  }
}

/* primal step on u: update_u, 3-D :706-729, 2-D :340-357                        */
EXPORT void or_update_u(const or_desc *d, float *unew, const float *u, const float *v, const float *kstar,
                        float tau, float norming) {
  const int N = d->N, Nz = d->dim == 3 ? d->Nz : 1, K = d->dim;
  const int S = d->Nz * d->C;
  const size_t plane = (size_t)N * N, vol = plane * S;
#pragma omp parallel for collapse(2) schedule(static)
  for (int s = 0; s < S; ++s)
    for (int y = 0; y < N; ++y)
      for (int x = 0; x < N; ++x) {
        const int z = s % Nz;
        const size_t i = (size_t)s * plane + (size_t)y * N + x;
        float a = v[i], b = v[vol + i], c = 0.0f;
        if (x == N - 1) a = 0.0f;
        if (x > 0) a -= v[i - 1];
        if (y == N - 1) b = 0.0f;
        if (y > 0) b -= v[vol + i - N];
        float r;
        if (K == 3) {
          c = v[2 * vol + i];
          if (z == Nz - 1) c = 0.0f;
          if (z > 0) c -= v[2 * vol + i - plane];
          c /= d->stepsize;
          r = u[i] + tau * (a + b + c - norming * kstar[i]);
        } else {
          r = u[i] + tau * (a + b - norming * kstar[i]);
        }
        if (r < 0) r = 0;
        unew[i] = r;
      }
}

/* primal step on p: update_p, 3-D :734-757, 2-D :359-376 (TV: update_p_empty)     */
EXPORT void or_update_p(const or_desc *d, float *pnew, const float *p, const float *v, const float *w, float tau) {
  const int N = d->N, Nz = d->dim == 3 ? d->Nz : 1, K = d->dim;
  const int S = d->Nz * d->C;
  const size_t plane = (size_t)N * N, vol = plane * S;
  if (!d->regularisation) { memset(pnew, 0, sizeof(float) * K * vol); return; }
#pragma omp parallel for collapse(2) schedule(static)
  for (int s = 0; s < S; ++s)
    for (int y = 0; y < N; ++y)
      for (int x = 0; x < N; ++x) {
        const int z = s % Nz;
        const size_t i = (size_t)s * plane + (size_t)y * N + x;
#define W_(c, k) w[(size_t)(c) * vol + (k)]
        if (K == 3) {
          /* rows of the symmetric tensor: (w0 w3 w4), (w3 w1 w5), (w4 w5 w2) */
          static const int rx[3] = {0, 3, 4}, ry[3] = {3, 1, 5}, rz[3] = {4, 5, 2};
          for (int k = 0; k < 3; ++k) {
            float A = -W_(rx[k], i), B = -W_(ry[k], i), Cz = -W_(rz[k], i);
            if (x == 0) A = 0.0f;
            if (x < N - 1) A += W_(rx[k], i + 1);
            if (y == 0) B = 0.0f;
            if (y < N - 1) B += W_(ry[k], i + N);
            if (z == 0) Cz = 0.0f;
            if (z < Nz - 1) Cz += W_(rz[k], i + plane);
            Cz /= d->stepsize;
            pnew[k * vol + i] = p[k * vol + i] + tau * (v[k * vol + i] + A + B + Cz);
          }
        } else {
          /* rows (w0 w2), (w2 w1) */
          static const int rx[2] = {0, 2}, ry[2] = {2, 1};
          for (int k = 0; k < 2; ++k) {
            float A = -W_(rx[k], i), B = -W_(ry[k], i);
            if (x == 0) A = 0.0f;
            if (x < N - 1) A += W_(rx[k], i + 1);
            if (y == 0) B = 0.0f;
            if (y < N - 1) B += W_(ry[k], i + N);
            pnew[k * vol + i] = p[k * vol + i] + tau * (v[k * vol + i] + A + B);
          }
        }
#undef W_
      }
}

/* extrapolation + swap: ElementwiseKernel U = 2 U_ - U (radon_tgv_primal_dual_3d.py:1075-1076,
 * :1217-1221) followed by the swap (U, U_) = (U_, U):  ubar <- 2 unew - u,  u <- unew.   */
EXPORT void or_extrapolate(float *u, float *ubar, const float *unew, size_t n) {
#pragma omp parallel for schedule(static)
  for (size_t i = 0; i < n; ++i) {
    ubar[i] = 2.0f * unew[i] - u[i];
    u[i] = unew[i];
  }
}

/* feasibility mask: Make_function_feasible, radon_tgv_primal_dual_3d.py:860-870:
 * bins that the all-ones image does not reach (R1 <= 0, slice 0) are zeroed in
 * every slice.                                                                   */
EXPORT void or_make_feasible(float *f, const float *ofs, int N, int nd, int nang, int S) {
  float *ones = (float *)malloc(sizeof(float) * N * N);
  float *r1 = (float *)malloc(sizeof(float) * nd * nang);
  for (int k = 0; k < N * N; ++k) ones[k] = 1.0f;
  or_radon(r1, ones, ofs, N, nd, nang, 1);
  for (int s = 0; s < S; ++s)
    for (int q = 0; q < nd * nang; ++q)
      if (r1[q] <= 0.0f) f[(size_t)s * nd * nang + q] = 0.0f;
  free(ones);
  free(r1);
}

/* ------------------------------------------------------------------------- */
/* the primal-dual loop: tgv_radon, radon_tgv_primal_dual_3d.py:1194-1221          */
typedef struct {
  float *u, *ubar;   /* U and U_ of the reference (after its swap: U = u, U_ = extrapolated) */
  float *p, *pbar;   /* P and P_ */
  float *v, *w, *lam;
} or_state;

/* Runs `iters` iterations in place. sigma, tau, alpha~ = alpha/ne^2 and mu' (KL: mu,
 * L2: mu/(sigma+mu)) are passed in already derived (tgv_radon :1180-1189).
 * ku_out (may be NULL) receives the last forward projection K u_ (the reference's
 * returned sinogram, :1278-1292).                                                  */
EXPORT int or_iterate(const or_desc *d, const float *ofs, const float *f, or_state *st, int iters, float sigma,
                      float tau, float sigma_data, float norming, float alphainv0, float alphainv1,
                      const float *mu_eff, float *ku_out) {
  const int S = d->Nz * d->C, K = d->dim;
  const size_t vol = (size_t)d->N * d->N * S, sz = (size_t)d->nd * d->nang * S;
  float *ku = (float *)malloc(sizeof(float) * sz);
  float *kstar = (float *)malloc(sizeof(float) * vol);
  float *unew = (float *)malloc(sizeof(float) * vol);
  float *pnew = (float *)malloc(sizeof(float) * K * vol);
  if (!ku || !kstar || !unew || !pnew) { free(ku); free(kstar); free(unew); free(pnew); return 1; }
  for (int it = 0; it < iters; ++it) {
    or_update_v(d, st->v, st->ubar, st->pbar, sigma);
    or_update_w(d, st->w, st->pbar, sigma);
    or_norm_v(d, st->v, alphainv1);
    or_norm_w(d, st->w, alphainv0);
    or_radon(ku, st->ubar, ofs, d->N, d->nd, d->nang, S);
    or_update_lambda(d, st->lam, ku, f, sigma_data, mu_eff);
    or_radon_ad(kstar, st->lam, ofs, d->N, d->nd, d->nang, S);
    or_update_u(d, unew, st->u, st->v, kstar, tau, norming);
    or_update_p(d, pnew, st->p, st->v, st->w, tau);
    or_extrapolate(st->u, st->ubar, unew, vol);
    or_extrapolate(st->p, st->pbar, pnew, (size_t)K * vol);
  }
  if (ku_out) memcpy(ku_out, ku, sizeof(float) * sz);
  free(ku); free(kstar); free(unew); free(pnew);
  return 0;
}
