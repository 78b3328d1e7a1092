// Ray geometry shared by the projector translation units.
#pragma once
#include <cuda_runtime.h>

namespace gt {

// Rows whose x-extent [0, N-1] can reach detector coordinate (i-1, i+1) for the
// angle o = (X, Y, offset, 1/X) of the forward projection `radon`
// (radon_tgv_primal_dual_3d.py:773-816): a conservative superset (the per-row
// bounds of the reference decide exactly).
__device__ __forceinline__ void ray_rows(const float4 o, int i, int N, int &ylo, int &yhi) {
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


// The reference's per-row x bounds of ray i (radon, :789-803): [xl, xh] after
// clamping to the image; false when the row does not meet the ray (X == 0 and
// the row's coordinate is outside (i-1, i+1)).
__device__ __forceinline__ bool row_bounds(const float4 o, float d, int i, int N, int &xl, int &xh) {
  const float fim = (float)(i - 1), fip = (float)(i + 1);
  if (o.x == 0.f) {
    if (d > fim && d < fip) { xl = 0; xh = N - 1; } else return false;
  } else if (o.x > 0.f) {
    xl = __float2int_rz(__fmul_rn(__fsub_rn(fim, d), o.w));
    xh = __float2int_rz(__fmul_rn(__fsub_rn(fip, d), o.w));
  } else {
    xl = __float2int_rz(__fmul_rn(__fsub_rn(fip, d), o.w));
    xh = __float2int_rz(__fmul_rn(__fsub_rn(fim, d), o.w));
  }
  xl = max(xl, 0);
  xh = min(xh, N - 1);
  return true;
}

}  // namespace gt
