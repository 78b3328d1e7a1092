// Kernels of the warm-start network: a small 3-D U-Net trained and run with
// BF16 weights and activations and FP32 accumulation.  No counterpart in the
// reference (it has no learned component).
//
// Tensors are [B][C][D][H][W] (W fastest).  Convolutions are 3x3x3 or 1x1x1,
// stride 1, zero padding (k-1)/2.  Outputs can be written at a channel offset of
// a wider tensor (the U-Net's skip concatenation is free) and can accumulate.
//
//   gt_nn_conv3d        forward (and, with transformed weights, the data gradient); BF16
//                       inputs with 16k in and out channels run on the tensor cores
//                       (k_conv3d_tc: tcgen05 MMA, accumulator in tensor memory)
//   gt_nn_flip_weights  w[co][ci][t] -> w'[ci][co][K3-1-t]   (data-gradient weights)
//   gt_nn_conv3d_wgrad  weight gradient as a split-K GEMM  dW = dY * im2col(X)^T
//   gt_nn_bias_grad, gt_nn_relu_bwd, gt_nn_pool2 / _bwd, gt_nn_up2 / _bwd,
//   gt_nn_mse, gt_nn_adam, gt_nn_cast
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "graptor_gb300.h"
#include "gt_tc.cuh"

namespace {

template <class T> __device__ __forceinline__ float ld(const T *p) { return (float)*p; }
template <> __device__ __forceinline__ float ld<__nv_bfloat16>(const __nv_bfloat16 *p) { return __bfloat162float(*p); }
template <class T> __device__ __forceinline__ void st(T *p, float v) { *p = (T)v; }
template <> __device__ __forceinline__ void st<__nv_bfloat16>(__nv_bfloat16 *p, float v) { *p = __float2bfloat16_rn(v); }

struct Shape {
  int B, D, H, W;
};

// ---------------------------------------------------------------------------
// forward convolution: a thread computes CO_T output channels for VX voxels
// along W; the block stages the weights of its channel tile, CI_CH input
// channels at a time, in shared memory (converted to FP32).
// ---------------------------------------------------------------------------
constexpr int CI_CH = 8;

template <class TI, class TO, int KS, int CO_T, int VX>
__global__ void __launch_bounds__(128) k_conv3d(const TI *__restrict__ x, int Ci, int Cx, int x_off,
                                                const __nv_bfloat16 *__restrict__ w,
                                                const float *__restrict__ bias, TO *__restrict__ y, int Co, int Cy,
                                                int co_off, Shape s, int relu, int accumulate) {
  constexpr int K3 = KS * KS * KS, R = KS / 2;
  __shared__ float sw[CO_T * CI_CH * K3];
  const int co0 = blockIdx.y * CO_T;
  const long long nvox = (long long)s.B * s.D * s.H * (s.W / VX);
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = t < nvox;
  int b = 0, d = 0, h = 0, w0 = 0;
  if (active) {
    long long r = t;
    const int wq = (int)(r % (s.W / VX)); r /= (s.W / VX);
    h = (int)(r % s.H); r /= s.H;
    d = (int)(r % s.D); b = (int)(r / s.D);
    w0 = wq * VX;
  }
  const size_t plane = (size_t)s.H * s.W, vol = plane * s.D;
  float acc[CO_T][VX];
#pragma unroll
  for (int c = 0; c < CO_T; ++c) {
    const float bv = (bias && co0 + c < Co) ? bias[co0 + c] : 0.f;
#pragma unroll
    for (int v = 0; v < VX; ++v) acc[c][v] = bv;
  }
  for (int ci0 = 0; ci0 < Ci; ci0 += CI_CH) {
    __syncthreads();
    for (int k = threadIdx.x; k < CO_T * CI_CH * K3; k += blockDim.x) {
      const int c = k / (CI_CH * K3), rem = k - c * CI_CH * K3, ci = rem / K3, tp = rem - ci * K3;
      sw[k] = (co0 + c < Co && ci0 + ci < Ci) ? __bfloat162float(w[((size_t)(co0 + c) * Ci + ci0 + ci) * K3 + tp]) : 0.f;
    }
    __syncthreads();
    if (!active) continue;
    const int cmax = min(CI_CH, Ci - ci0);
    for (int ci = 0; ci < cmax; ++ci) {
      const TI *xc = x + ((size_t)b * Cx + x_off + ci0 + ci) * vol;
#pragma unroll
      for (int kd = 0; kd < KS; ++kd) {
        const int dd = d + kd - R;
        if (dd < 0 || dd >= s.D) continue;
#pragma unroll
        for (int kh = 0; kh < KS; ++kh) {
          const int hh = h + kh - R;
          if (hh < 0 || hh >= s.H) continue;
          const TI *row = xc + (size_t)dd * plane + (size_t)hh * s.W;
          float xv[VX + KS - 1];
#pragma unroll
          for (int q = 0; q < VX + KS - 1; ++q) {
            const int ww = w0 + q - R;
            xv[q] = (ww >= 0 && ww < s.W) ? ld<TI>(row + ww) : 0.f;
          }
#pragma unroll
          for (int kw = 0; kw < KS; ++kw) {
            const int tp = (kd * KS + kh) * KS + kw;
#pragma unroll
            for (int c = 0; c < CO_T; ++c) {
              const float wv = sw[(c * CI_CH + ci) * K3 + tp];
#pragma unroll
              for (int v = 0; v < VX; ++v) acc[c][v] = fmaf(wv, xv[v + kw], acc[c][v]);
            }
          }
        }
      }
    }
  }
  if (!active) return;
#pragma unroll
  for (int c = 0; c < CO_T; ++c) {
    if (co0 + c >= Co) break;
    TO *yo = y + ((size_t)b * Cy + co_off + co0 + c) * vol + (size_t)d * plane + (size_t)h * s.W + w0;
#pragma unroll
    for (int v = 0; v < VX; ++v) {
      float r = acc[c][v];
      if (accumulate) r += ld<TO>(yo + v);
      if (relu) r = fmaxf(r, 0.f);
      st<TO>(yo + v, r);
    }
  }
}

// ---------------------------------------------------------------------------
// forward convolution on the tensor cores: implicit GEMM Y[voxel][co] =
// sum over (tap, ci) of X[voxel + tap][ci] W[co][ci][tap].  A block owns 128
// consecutive voxels (M = 128, one TMEM lane each) and all Co output channels
// (N = Co, one FP32 TMEM column each).  K runs over taps x 16-channel chunks;
// per chunk the 128 x 16 BF16 slice of im2col(X) (each thread gathers its voxel's
// 16 channels) and the Co x 16 BF16 weights are written to shared memory as
// 8-row x 16-byte core matrices, double-buffered, and one thread issues one
// tcgen05.mma (K = 16) and commits it to the stage's mbarrier; a stage is
// rewritten only after the MMA that read it has completed.  The epilogue reads
// the accumulator from tensor memory (tcgen05.ld, warp w = lanes 32w..32w+31),
// adds bias, the existing output (accumulate) and applies ReLU.  Waits are
// bounded: a block that gives up flags g_nn_err, never leaves tensor memory
// allocated, and stores nothing.
// ---------------------------------------------------------------------------
__device__ int g_nn_err;
constexpr uint32_t TC_WAIT_LIMIT = 1u << 20;

__device__ __forceinline__ uint32_t bf16_pair(__nv_bfloat16 lo, __nv_bfloat16 hi) {
  return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

template <class TO, int KS>
__global__ void __launch_bounds__(128) k_conv3d_tc(const __nv_bfloat16 *__restrict__ x, int Ci, int Cx, int x_off,
                                                   const __nv_bfloat16 *__restrict__ w,
                                                   const float *__restrict__ bias, TO *__restrict__ y, int Co, int Cy,
                                                   int co_off, Shape s, int relu, int accumulate) {
  constexpr int K3 = KS * KS * KS, R = KS / 2;
  constexpr int ABYTES = 128 * 16 * 2, BBYTES = 256 * 16 * 2;
  __shared__ __align__(1024) uint8_t sA[2][ABYTES];
  __shared__ __align__(1024) uint8_t sB[2][BBYTES];
  __shared__ __align__(8) uint64_t bar[2];
  __shared__ uint32_t tslot;
  const int tid = threadIdx.x, warp = tid >> 5;
  const long long nvox = (long long)s.B * s.D * s.H * s.W;
  const long long vox = (long long)blockIdx.x * 128 + tid;
  const bool active = vox < nvox;
  int b = 0, d = 0, h = 0, wx = 0;
  if (active) {
    long long r = vox;
    wx = (int)(r % s.W); r /= s.W;
    h = (int)(r % s.H); r /= s.H;
    d = (int)(r % s.D); b = (int)(r / s.D);
  }
  const size_t plane = (size_t)s.H * s.W, vol = plane * s.D;
  const uint32_t ncols = Co <= 32 ? 32u : (Co <= 64 ? 64u : (Co <= 128 ? 128u : 256u));
  if (warp == 0) gt::tmem_alloc(&tslot, ncols);
  if (tid == 0) {
    gt::mbar_init(&bar[0], 1);
    gt::mbar_init(&bar[1], 1);
    gt::mbar_init_fence();
  }
  gt::tc_fence_before();
  __syncthreads();
  gt::tc_fence_after();
  const uint32_t tmem = tslot;
  const int nci = Ci / 16, nk = K3 * nci;
  const uint32_t idesc = gt::tc_idesc_bf16_f32(128, Co);
  bool ok = true;
  int issued = 0;  // MMAs issued (their commits complete the stages' phases in order)
  for (int q = 0; q < nk; ++q) {
    const int st = q & 1;
    if (q >= 2) {  // the MMA that read this stage (chunk q - 2) must have completed
      const bool done = gt::mbar_wait_bounded(&bar[st], ((q - 2) >> 1) & 1, TC_WAIT_LIMIT);
      if (__syncthreads_or(!done)) { ok = false; break; }
    }
    const int t = q / nci, ci0 = (q - t * nci) * 16;
    {  // A: this thread's voxel, channels ci0 .. ci0 + 15 at tap t
      const int kd = t / (KS * KS), kh = (t / KS) % KS, kw = t % KS;
      const int dd = d + kd - R, hh = h + kh - R, w2 = wx + kw - R;
      const bool in = active && dd >= 0 && dd < s.D && hh >= 0 && hh < s.H && w2 >= 0 && w2 < s.W;
      uint32_t pk[8];
      if (in) {
        const __nv_bfloat16 *xp = x + ((size_t)b * Cx + x_off + ci0) * vol + (size_t)dd * plane + (size_t)hh * s.W + w2;
#pragma unroll
        for (int j = 0; j < 8; ++j) pk[j] = bf16_pair(xp[(size_t)(2 * j) * vol], xp[(size_t)(2 * j + 1) * vol]);
      } else {
#pragma unroll
        for (int j = 0; j < 8; ++j) pk[j] = 0u;
      }
      uint8_t *row = sA[st] + (tid >> 3) * 256 + (tid & 7) * 16;
      *reinterpret_cast<uint4 *>(row) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
      *reinterpret_cast<uint4 *>(row + 128) = make_uint4(pk[4], pk[5], pk[6], pk[7]);
    }
    for (int rr = tid; rr < Co * 2; rr += 128) {  // B: weights of tap t, Co rows x 16 channels
      const int co = rr >> 1, kc = rr & 1;
      const __nv_bfloat16 *wp = w + ((size_t)co * Ci + ci0 + kc * 8) * K3 + t;
      uint32_t pk[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) pk[j] = bf16_pair(wp[(size_t)(2 * j) * K3], wp[(size_t)(2 * j + 1) * K3]);
      *reinterpret_cast<uint4 *>(sB[st] + (co >> 3) * 256 + kc * 128 + (co & 7) * 16) =
          make_uint4(pk[0], pk[1], pk[2], pk[3]);
    }
    gt::fence_async_shared();
    __syncthreads();
    if (tid == 0) {
      gt::tc_fence_after();
      gt::tc_mma_bf16(tmem, gt::tc_smem_desc(sA[st], 128, 256), gt::tc_smem_desc(sB[st], 128, 256), idesc, q > 0);
      gt::tc_commit(&bar[st]);
    }
    issued = q + 1;
  }
  // the last issued MMA's commit covers every earlier one
  if (issued > 0) {
    const int ql = issued - 1;
    const bool done = gt::mbar_wait_bounded(&bar[ql & 1], (ql >> 1) & 1, TC_WAIT_LIMIT);
    ok = ok && done;
  }
  ok = !__syncthreads_or(!ok);
  gt::tc_fence_after();
  if (ok) {
    for (int c0 = 0; c0 < Co; c0 += 16) {
      float v[16];
      gt::tc_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
      if (active) {
        TO *yo = y + ((size_t)b * Cy + co_off + c0) * vol + (size_t)d * plane + (size_t)h * s.W + wx;
#pragma unroll
        for (int k = 0; k < 16; ++k) {
          float r = v[k] + (bias ? bias[c0 + k] : 0.f);
          if (accumulate) r += ld<TO>(yo + (size_t)k * vol);
          if (relu) r = fmaxf(r, 0.f);
          st<TO>(yo + (size_t)k * vol, r);
        }
      }
    }
  } else if (tid == 0) {
    atomicExch(&g_nn_err, 1);
  }
  gt::tc_fence_before();
  __syncthreads();
  // On the error path (a bounded wait gave up) the block does not know that the
  // MMA it waited for has finished when it frees the tensor memory below; the
  // wait limit is far above any MMA's duration, so this path is not expected to
  // occur, and the error flag makes the host discard the whole launch's output.
  if (warp == 0) gt::tmem_dealloc(tmem, ncols);
}

// ---------------------------------------------------------------------------
// 3x3x3 forward convolution on the tensor cores with the block's input halo and
// weights staged once per 16-channel chunk (k_conv3d_tc gathers every tap's
// operands from global memory).  The weights arrive as one bulk copy per chunk of
// their shared-memory image (k_conv_wimage, built once per call).  A block owns 128 consecutive voxels of one
// (b, d) plane: R = 128 / W rows of width W (W <= 128), or 128 voxels of one row
// (W a multiple of 128).  Per chunk of 16 input channels:
//   halo     the 3 x (R + 2) x (Wb + 2) input positions the block's 27 taps read,
//            channels 0-7 and 8-15 as two planes of 16-byte rows (zero outside
//            the volume);
//   weights  all 27 taps' Co x 16 weights as 8-row x 16-byte core matrices.
// A tap's B operand is then a descriptor into the weights.  Its A operand: for
// W >= 128 the 128 rows are 128 consecutive halo positions, so the descriptor
// points into the halo itself and the 27 MMAs of a chunk are issued back to back
// without any copy; for W < 128 the rows of the tap's shifted window are copied
// from the halo into a double-buffered A tile (two 16-byte shared-memory moves per
// thread) before each MMA.  Every wait is bounded (g_nn_err on timeout).
// ---------------------------------------------------------------------------
constexpr int TC2_A_BYTES = 128 * 16 * 2;

__host__ __device__ inline int tc2_rows(int W) { return W >= 128 ? 1 : 128 / W; }
__host__ __device__ inline int tc2_width(int W) { return W >= 128 ? 128 : W; }
__host__ __device__ inline int tc2_halo(int W) { return 3 * (tc2_rows(W) + 2) * (tc2_width(W) + 2); }
__host__ __device__ inline size_t tc2_align(size_t b) { return (b + 1023) & ~(size_t)1023; }
// dynamic shared memory: two halo planes, the weights, two A tiles (+ alignment slack)
inline size_t tc2_smem(int W, int Co) {
  return tc2_align((size_t)tc2_halo(W) * 32) + tc2_align((size_t)27 * Co * 32) + 2 * TC2_A_BYTES + 1024;
}

// The weights of every 16-channel chunk as the shared-memory image the MMAs read:
// per chunk, per tap t, Co rows x 16 channels as 8-row x 16-byte core matrices
// (tap t at t * Co * 32 bytes, row co at (co / 8) * 256 + (co % 8) * 16, channels
// 8-15 at + 128).  One thread per 16 bytes.
__global__ void k_conv_wimage(const __nv_bfloat16 *__restrict__ w, int Ci, int Co, uint4 *__restrict__ img) {
  const long long u = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long per_chunk = 27ll * Co * 2;
  if (u >= per_chunk * (Ci / 16)) return;
  const int ch = (int)(u / per_chunk);
  const int rem = (int)(u - ch * per_chunk);
  const int t = rem / (Co * 2), r2 = rem - t * Co * 2;
  const int cg = r2 >> 4, g = (r2 >> 3) & 1, cr = r2 & 7;  // core-matrix group, channel half, row
  const int co = cg * 8 + cr;
  const __nv_bfloat16 *wp = w + ((size_t)co * Ci + ch * 16 + 8 * g) * 27 + t;
  uint32_t pk[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) pk[j] = bf16_pair(wp[(size_t)(2 * j) * 27], wp[(size_t)(2 * j + 1) * 27]);
  img[u] = make_uint4(pk[0], pk[1], pk[2], pk[3]);
}

template <class TO>
__global__ void __launch_bounds__(128) k_conv3d_tc2(const __nv_bfloat16 *__restrict__ x, int Ci, int Cx, int x_off,
                                                    const uint4 *__restrict__ wimg,
                                                    const float *__restrict__ bias, TO *__restrict__ y, int Co,
                                                    int Cy, int co_off, Shape s, int relu, int accumulate) {
  extern __shared__ uint8_t dsm_raw[];
  uint8_t *dsm = (uint8_t *)(((uintptr_t)dsm_raw + 1023) & ~(uintptr_t)1023);
  __shared__ __align__(8) uint64_t bar[4];  // A stages 0 / 1, chunk completion, weight copy
  __shared__ uint32_t tslot;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int R = tc2_rows(s.W), Wb = tc2_width(s.W), HP = R + 2, WP = Wb + 2;
  const int P = 3 * HP * WP;
  const size_t plane_bytes = (size_t)P * 16;
  uint8_t *sH = dsm;                                   // halo: plane g at sH + g * plane_bytes
  uint8_t *sW = dsm + tc2_align(plane_bytes * 2);      // weights: tap t at sW + t * Co * 32
  uint8_t *sA = sW + tc2_align((size_t)27 * Co * 32);  // A tiles (W < 128)
  const bool direct = s.W >= 128;

  // the block's plane and first row / column
  const long long v0 = (long long)blockIdx.x * 128;
  const long long plane_vox = (long long)s.H * s.W;
  const int bd = (int)(v0 / plane_vox);
  const int b = bd / s.D, d = bd - b * s.D;
  const long long in_plane = v0 - (long long)bd * plane_vox;
  const int h0 = (int)(in_plane / s.W), w0 = (int)(in_plane - (long long)h0 * s.W);
  const size_t plane = (size_t)s.H * s.W, vol = plane * s.D;
  // this thread's voxel: row r, column c of the block
  const int r = direct ? 0 : tid / Wb, c = direct ? tid : tid - (tid / Wb) * Wb;

  const uint32_t ncols = Co <= 32 ? 32u : (Co <= 64 ? 64u : 128u);
  if (warp == 0) gt::tmem_alloc(&tslot, ncols);
  if (tid == 0) {
    gt::mbar_init(&bar[0], 1);
    gt::mbar_init(&bar[1], 1);
    gt::mbar_init(&bar[2], 1);
    gt::mbar_init(&bar[3], 1);
    gt::mbar_init_fence();
  }
  gt::tc_fence_before();
  __syncthreads();
  gt::tc_fence_after();
  const uint32_t tmem = tslot;
  const uint32_t idesc = gt::tc_idesc_bf16_f32(128, Co);
  const int nci = Ci / 16;
  bool ok = true;
  int q = 0;           // MMAs issued so far (A-tile path: their commits complete the stages in order)
  int wpending = -1;   // thread 0: parity of a weight copy not yet seen complete
  for (int ch = 0; ch < nci && ok; ++ch) {
    const int ci0 = ch * 16;
    if (ch > 0) {  // every MMA of the previous chunk must be done before its operands are rewritten
      const bool done = gt::mbar_wait_bounded(&bar[2], (ch - 1) & 1, TC_WAIT_LIMIT);
      if (__syncthreads_or(!done)) { ok = false; break; }
    }
    // weights of the chunk: one bulk copy of its image (only the MMA thread waits for it)
    const uint32_t wbytes = 27u * Co * 32u;
    if (tid == 0) {
      gt::mbar_arrive_expect_tx(&bar[3], wbytes);
      gt::bulk_load(sW, wimg + (size_t)ch * (wbytes / 16), wbytes, &bar[3]);
      wpending = ch & 1;
    }
    // halo: items of 4 adjacent columns x 16 channels (one 8-byte load per channel;
    // W and w0 are multiples of 4, so a group is wholly inside or outside the
    // volume), groups covering columns w0 - 4 .. w0 + Wb + 3, of which the halo keeps
    // w0 - 1 .. w0 + Wb; zero outside the volume
    {
      const __nv_bfloat16 *xc = x + ((size_t)b * Cx + x_off + ci0) * vol;
      const int ng = Wb / 4 + 2, items = 3 * HP * ng;
      for (int it = tid; it < items; it += 128) {
        const int row = it / ng, gq = it - row * ng;
        const int dd = row / HP, hh = row - dd * HP;
        const int dg = d - 1 + dd, hg = h0 - 1 + hh, wg4 = w0 - 4 + 4 * gq;
        uint2 v[16];
        if (dg >= 0 && dg < s.D && hg >= 0 && hg < s.H && wg4 >= 0 && wg4 < s.W) {
          const __nv_bfloat16 *xp = xc + (size_t)dg * plane + (size_t)hg * s.W + wg4;
#pragma unroll
          for (int j = 0; j < 16; ++j) v[j] = *reinterpret_cast<const uint2 *>(xp + (size_t)j * vol);
        } else {
#pragma unroll
          for (int j = 0; j < 16; ++j) v[j] = make_uint2(0u, 0u);
        }
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int ww = 4 * gq - 3 + e;  // halo column of element e (column w0 - 1 is halo column 0)
          if (ww < 0 || ww >= WP) continue;
          uint32_t pk[8];
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            // element e of channels 2j and 2j + 1: 16-bit half e & 1 of word e >> 1
            const uint32_t a = (e >> 1) ? v[2 * j].y : v[2 * j].x, c = (e >> 1) ? v[2 * j + 1].y : v[2 * j + 1].x;
            pk[j] = (e & 1) ? ((a >> 16) | (c & 0xffff0000u)) : ((a & 0xffffu) | (c << 16));
          }
          const size_t pos = (size_t)row * WP + ww;
          *reinterpret_cast<uint4 *>(sH + pos * 16) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
          *reinterpret_cast<uint4 *>(sH + plane_bytes + pos * 16) = make_uint4(pk[4], pk[5], pk[6], pk[7]);
        }
      }
    }
    gt::fence_async_shared();
    __syncthreads();
    if (tid == 0) {
      if (gt::mbar_wait_bounded(&bar[3], ch & 1, TC_WAIT_LIMIT)) wpending = -1;
      else ok = false;
    }
    if (__syncthreads_or(!ok)) { ok = false; break; }
    if (direct) {
      if (tid == 0) {
        gt::tc_fence_after();
        for (int t = 0; t < 27; ++t) {
          const int kd = t / 9, kh = (t / 3) % 3, kw = t % 3;
          const int p0 = (kd * HP + kh) * WP + kw;
          gt::tc_mma_bf16(tmem, gt::tc_smem_desc(sH + (size_t)p0 * 16, (uint32_t)plane_bytes, 128),
                          gt::tc_smem_desc(sW + (size_t)t * Co * 32, 128, 256), idesc, (ch > 0 || t > 0) ? 1 : 0);
        }
        gt::tc_commit(&bar[2]);
      }
    } else {
      for (int t = 0; t < 27 && ok; ++t, ++q) {
        const int st = q & 1;
        if (q >= 2) {  // the MMA that read this A tile (number q - 2) must have completed
          const bool done = gt::mbar_wait_bounded(&bar[st], ((q - 2) >> 1) & 1, TC_WAIT_LIMIT);
          if (__syncthreads_or(!done)) { ok = false; break; }
        }
        const int kd = t / 9, kh = (t / 3) % 3, kw = t % 3;
        const int pos = (kd * HP + r + kh) * WP + c + kw;
        const uint4 lo = *reinterpret_cast<const uint4 *>(sH + (size_t)pos * 16);
        const uint4 hi = *reinterpret_cast<const uint4 *>(sH + plane_bytes + (size_t)pos * 16);
        uint8_t *row = sA + st * TC2_A_BYTES + (tid >> 3) * 256 + (tid & 7) * 16;
        *reinterpret_cast<uint4 *>(row) = lo;
        *reinterpret_cast<uint4 *>(row + 128) = hi;
        gt::fence_async_shared();
        __syncthreads();
        if (tid == 0) {
          gt::tc_fence_after();
          gt::tc_mma_bf16(tmem, gt::tc_smem_desc(sA + st * TC2_A_BYTES, 128, 256),
                          gt::tc_smem_desc(sW + (size_t)t * Co * 32, 128, 256), idesc, (ch > 0 || t > 0) ? 1 : 0);
          gt::tc_commit(&bar[st]);
          if (t == 26) gt::tc_commit(&bar[2]);  // the chunk's last MMA: its operands may be rewritten after it
        }
      }
    }
  }
  // the last chunk's completion covers every MMA
  if (ok) ok = gt::mbar_wait_bounded(&bar[2], (nci - 1) & 1, TC_WAIT_LIMIT);
  ok = !__syncthreads_or(!ok);
  gt::tc_fence_after();
  const int h = h0 + r, wx = w0 + c;
  if (ok) {
    for (int c0 = 0; c0 < Co; c0 += 16) {
      float v[16];
      gt::tc_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
      TO *yo = y + ((size_t)b * Cy + co_off + c0) * vol + (size_t)d * plane + (size_t)h * s.W + wx;
#pragma unroll
      for (int k = 0; k < 16; ++k) {
        float o = v[k] + (bias ? bias[c0 + k] : 0.f);
        if (accumulate) o += ld<TO>(yo + (size_t)k * vol);
        if (relu) o = fmaxf(o, 0.f);
        st<TO>(yo + (size_t)k * vol, o);
      }
    }
  } else if (tid == 0) {
    atomicExch(&g_nn_err, 1);
    // a weight copy still in flight lands in this block's shared memory: wait for
    // it (bounded) before the block ends
    if (wpending >= 0) gt::mbar_wait_bounded(&bar[3], (uint32_t)wpending, TC_WAIT_LIMIT);
  }
  gt::tc_fence_before();
  __syncthreads();
  // as in k_conv3d_tc: on the timeout path the block cannot know that the MMA it
  // waited for has finished when it frees the tensor memory; the error flag makes
  // the host discard the launch's output
  if (warp == 0) gt::tmem_dealloc(tmem, ncols);
}

// the staged kernel applies: 3x3x3, 16k channels in and out, Co <= 128, blocks
// inside one (b, d) plane and whole rows (or 128-wide row pieces)
inline bool tc2_ok(int Ci, int Co, const Shape &s) {
  return Ci % 16 == 0 && Co % 16 == 0 && Co <= 128 && ((long long)s.H * s.W) % 128 == 0 &&
         (s.W % 128 == 0 || 128 % s.W == 0) && tc2_smem(s.W, Co) <= 227 * 1024;
}

int g_tc2_mode = 1;  // 1: the staged 3x3x3 tensor-core kernel where it applies

int g_tc_mode = 1;  // 1: tensor-core path where it applies, 0: CUDA cores only

// w[co][ci][t] -> w'[ci][co][K3-1-t]: convolving dY with w' gives dX (stride 1, same padding)
__global__ void k_flip(const __nv_bfloat16 *__restrict__ w, __nv_bfloat16 *__restrict__ wf, int Co, int Ci, int K3) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)Co * Ci * K3) return;
  const int tp = (int)(t % K3);
  const long long r = t / K3;
  const int ci = (int)(r % Ci), co = (int)(r / Ci);
  wf[((size_t)ci * Co + co) * K3 + (K3 - 1 - tp)] = w[t];
}

// ---------------------------------------------------------------------------
// weight gradient: dW[co][ci*K3 + t] = sum_{b, voxel} dY[b][co][v] X[b][ci][v + off(t)]
// GEMM M = Co, N = Ci*K3, K = voxels; a block computes a 16 x 64 tile over one
// K-chunk and writes it to part[chunk]; k_wgrad_reduce sums the chunks in order.
// ---------------------------------------------------------------------------
constexpr int WG_M = 16, WG_N = 64, WG_K = 32;

template <class TX, int KS>
__global__ void __launch_bounds__(256) k_wgrad(const float *__restrict__ dy, int Co, int Cdy, int dy_off,
                                               const TX *__restrict__ x, int Ci, int Cx, int x_off, Shape s,
                                               long long kchunk, float *__restrict__ part) {
  constexpr int K3 = KS * KS * KS, R = KS / 2;
  __shared__ float sa[WG_M][WG_K + 1];
  __shared__ float sb[WG_K][WG_N + 1];
  const int m0 = blockIdx.y * WG_M, n0 = blockIdx.x * WG_N, N = Ci * K3;
  const long long nvox = (long long)s.B * s.D * s.H * s.W;
  const long long k0 = (long long)blockIdx.z * kchunk, k1 = min(nvox, k0 + kchunk);
  const size_t plane = (size_t)s.H * s.W, vol = plane * s.D;
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;  // 16 x 16 threads, 4 columns each
  float acc[4] = {0, 0, 0, 0};
  for (long long kb = k0; kb < k1; kb += WG_K) {
    __syncthreads();
    for (int q = threadIdx.x; q < WG_M * WG_K; q += blockDim.x) {
      const int m = q / WG_K, kk = q - m * WG_K;
      const long long v = kb + kk;
      float val = 0.f;
      if (m0 + m < Co && v < k1) {
        const long long bb = v / vol, rv = v - bb * vol;
        val = dy[((size_t)bb * Cdy + dy_off + m0 + m) * vol + rv];
      }
      sa[m][kk] = val;
    }
    for (int q = threadIdx.x; q < WG_K * WG_N; q += blockDim.x) {
      const int kk = q / WG_N, n = q - kk * WG_N;
      const long long v = kb + kk;
      float val = 0.f;
      if (n0 + n < N && v < k1) {
        const int ci = (n0 + n) / K3, tp = (n0 + n) - ci * K3;
        const int kd = tp / (KS * KS), kh = (tp / KS) % KS, kw = tp % KS;
        long long r = v;
        const int ww = (int)(r % s.W); r /= s.W;
        const int hh = (int)(r % s.H); r /= s.H;
        const int dd = (int)(r % s.D); const int bb = (int)(r / s.D);
        const int zd = dd + kd - R, zh = hh + kh - R, zw = ww + kw - R;
        if (zd >= 0 && zd < s.D && zh >= 0 && zh < s.H && zw >= 0 && zw < s.W)
          val = ld<TX>(x + ((size_t)bb * Cx + x_off + ci) * vol + (size_t)zd * plane + (size_t)zh * s.W + zw);
      }
      sb[kk][n] = val;
    }
    __syncthreads();
#pragma unroll 8
    for (int kk = 0; kk < WG_K; ++kk) {
      const float a = sa[ty][kk];
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[j] = fmaf(a, sb[kk][tx + 16 * j], acc[j]);
    }
  }
  const int m = m0 + ty;
  if (m >= Co) return;
  for (int j = 0; j < 4; ++j) {
    const int n = n0 + tx + 16 * j;
    if (n < N) part[((size_t)blockIdx.z * Co + m) * N + n] = acc[j];
  }
}

__global__ void k_wgrad_reduce(const float *__restrict__ part, int nchunk, long long n, float *__restrict__ g,
                               int accumulate) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  float a = 0.f;
  for (int c = 0; c < nchunk; ++c) a += part[(size_t)c * n + t];
  g[t] = accumulate ? g[t] + a : a;
}

// db[co] (+)= sum over batch and voxels of dY (channel-offset view; one block per
// channel, fixed summation order)
__global__ void k_bias_grad(const float *__restrict__ dy, int Co, int Cdy, int dy_off, long long vol, int B,
                            float *__restrict__ db, int accumulate) {
  __shared__ float sh[256];
  const int co = blockIdx.x;
  float a = 0.f;
  for (int b = 0; b < B; ++b)
    for (long long v = threadIdx.x; v < vol; v += blockDim.x) a += dy[((size_t)b * Cdy + dy_off + co) * vol + v];
  sh[threadIdx.x] = a;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) db[co] = accumulate ? db[co] + sh[0] : sh[0];
}

// dY *= (Y > 0) for a ReLU output Y; dY and Y are the same channel-offset view
// (channels [co_off, co_off+C) of Cy-channel tensors)
template <class TY>
__global__ void k_relu_bwd(float *__restrict__ dy, const TY *__restrict__ y, int C, int Cy, int co_off, long long vol,
                           int B) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)B * C * vol) return;
  const long long v = t % vol, bc = t / vol;
  const int c = (int)(bc % C), b = (int)(bc / C);
  const size_t i = ((size_t)b * Cy + co_off + c) * vol + v;
  if (!(ld<TY>(y + i) > 0.f)) dy[i] = 0.f;
}

// y[b][c] = x[b][c] * scale[b*C + c], optionally floored at zero
template <class TI, class TO>
__global__ void k_scale(const TI *__restrict__ x, TO *__restrict__ y, int C, long long vol, int B,
                        const float *__restrict__ scale, int floor0) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)B * C * vol) return;
  float r = ld<TI>(x + t) * scale[t / vol];
  if (floor0) r = fmaxf(r, 0.f);
  st<TO>(y + t, r);
}

// 2x2x2 average pooling of channels [src_off, src_off+C) of a Cs-channel tensor
__global__ void k_pool2(const __nv_bfloat16 *__restrict__ x, int Cs, int src_off, __nv_bfloat16 *__restrict__ y, int C,
                        Shape so) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long n = (long long)so.B * C * so.D * so.H * so.W;
  if (t >= n) return;
  long long r = t;
  const int w = (int)(r % so.W); r /= so.W;
  const int h = (int)(r % so.H); r /= so.H;
  const int d = (int)(r % so.D); r /= so.D;
  const int c = (int)(r % C), b = (int)(r / C);
  const int W = so.W * 2, H = so.H * 2, D = so.D * 2;
  const __nv_bfloat16 *xc = x + ((size_t)b * Cs + src_off + c) * D * H * W;
  float a = 0.f;
  for (int k = 0; k < 8; ++k)
    a += __bfloat162float(xc[((size_t)(2 * d + (k >> 2)) * H + 2 * h + ((k >> 1) & 1)) * W + 2 * w + (k & 1)]);
  y[t] = __float2bfloat16_rn(0.125f * a);
}

// gradient of k_pool2: dX (channels [dst_off, dst_off+C) of a Cd-channel tensor) += dY / 8
__global__ void k_pool2_bwd(const float *__restrict__ dy, float *__restrict__ dx, int C, int Cd, int dst_off, Shape si) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long n = (long long)si.B * C * si.D * si.H * si.W;
  if (t >= n) return;
  long long r = t;
  const int w = (int)(r % si.W); r /= si.W;
  const int h = (int)(r % si.H); r /= si.H;
  const int d = (int)(r % si.D); r /= si.D;
  const int c = (int)(r % C), b = (int)(r / C);
  const int Wo = si.W / 2, Ho = si.H / 2, Do = si.D / 2;
  const float g = 0.125f * dy[((((size_t)b * C + c) * Do + d / 2) * Ho + h / 2) * Wo + w / 2];
  dx[((((size_t)b * Cd + dst_off + c) * si.D + d) * si.H + h) * si.W + w] += g;
}

// nearest 2x upsampling into channels [dst_off, dst_off+C) of a Cd-channel tensor
__global__ void k_up2(const __nv_bfloat16 *__restrict__ x, __nv_bfloat16 *__restrict__ y, int C, int Cd, int dst_off,
                      Shape so) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long n = (long long)so.B * C * so.D * so.H * so.W;
  if (t >= n) return;
  long long r = t;
  const int w = (int)(r % so.W); r /= so.W;
  const int h = (int)(r % so.H); r /= so.H;
  const int d = (int)(r % so.D); r /= so.D;
  const int c = (int)(r % C), b = (int)(r / C);
  const int Wi = so.W / 2, Hi = so.H / 2, Di = so.D / 2;
  y[((((size_t)b * Cd + dst_off + c) * so.D + d) * so.H + h) * so.W + w] =
      x[((((size_t)b * C + c) * Di + d / 2) * Hi + h / 2) * Wi + w / 2];
}

// gradient of k_up2: dX = sum of the 8 children of channels [src_off, src_off+C) of dY (Cs channels)
__global__ void k_up2_bwd(const float *__restrict__ dy, int Cs, int src_off, float *__restrict__ dx, int C, Shape si) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long n = (long long)si.B * C * si.D * si.H * si.W;
  if (t >= n) return;
  long long r = t;
  const int w = (int)(r % si.W); r /= si.W;
  const int h = (int)(r % si.H); r /= si.H;
  const int d = (int)(r % si.D); r /= si.D;
  const int c = (int)(r % C), b = (int)(r / C);
  const int W = si.W * 2, H = si.H * 2, D = si.D * 2;
  const float *g = dy + ((size_t)b * Cs + src_off + c) * D * H * W;
  float a = 0.f;
  for (int k = 0; k < 8; ++k) a += g[((size_t)(2 * d + (k >> 2)) * H + 2 * h + ((k >> 1) & 1)) * W + 2 * w + (k & 1)];
  dx[t] = a;
}

// mean squared error: per-block partial sums of (p - q)^2 and dP = 2 (p - q) / n
__global__ void k_mse(const float *__restrict__ p, const float *__restrict__ q, long long n, float *__restrict__ dp,
                      float *__restrict__ part) {
  __shared__ float sh[256];
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  float e = 0.f;
  if (t < n) {
    const float r = p[t] - q[t];
    e = r * r;
    dp[t] = 2.f * r / (float)n;
  }
  sh[threadIdx.x] = e;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

// Adam on FP32 master weights; the BF16 working copy is refreshed
__global__ void k_adam(float *__restrict__ wm, __nv_bfloat16 *__restrict__ wb, const float *__restrict__ g,
                       float *__restrict__ m, float *__restrict__ v, long long n, float lr, float b1, float b2,
                       float eps, float c1, float c2) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const float gt = g[t];
  const float mt = b1 * m[t] + (1.f - b1) * gt;
  const float vt = b2 * v[t] + (1.f - b2) * gt * gt;
  m[t] = mt;
  v[t] = vt;
  const float w = wm[t] - lr * (mt / c1) / (sqrtf(vt / c2) + eps);
  wm[t] = w;
  if (wb) wb[t] = __float2bfloat16_rn(w);
}

__global__ void k_cast_f2b(const float *__restrict__ a, __nv_bfloat16 *__restrict__ b, long long n) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) b[t] = __float2bfloat16_rn(a[t]);
}

__global__ void k_cast_b2f(const __nv_bfloat16 *__restrict__ a, float *__restrict__ b, long long n) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) b[t] = __bfloat162float(a[t]);
}

inline unsigned nblk(long long n, int bs) { return (unsigned)((n + bs - 1) / bs); }

template <class TI, class TO, int KS, int CO_T>
cudaError_t conv_t(const void *x, int Ci, int Cx, int x_off, const void *w, const float *bias, void *y, int Co, int Cy,
                   int co_off, Shape s, int relu, int accumulate, cudaStream_t st) {
  constexpr int VX = 4;
  if (s.W % VX != 0) return cudaErrorInvalidValue;
  dim3 g(nblk((long long)s.B * s.D * s.H * (s.W / VX), 128), (Co + CO_T - 1) / CO_T);
  k_conv3d<TI, TO, KS, CO_T, VX><<<g, 128, 0, st>>>((const TI *)x, Ci, Cx, x_off, (const __nv_bfloat16 *)w, bias,
                                                     (TO *)y, Co, Cy, co_off, s, relu, accumulate);
  return cudaGetLastError();
}

template <class TI, class TO>
cudaError_t conv_k(int ks, const void *x, int Ci, int Cx, int x_off, const void *w, const float *bias, void *y, int Co,
                   int Cy, int co_off, Shape s, int relu, int accumulate, cudaStream_t st) {
  if (ks == 3) return conv_t<TI, TO, 3, 8>(x, Ci, Cx, x_off, w, bias, y, Co, Cy, co_off, s, relu, accumulate, st);
  if (ks == 1) return conv_t<TI, TO, 1, 8>(x, Ci, Cx, x_off, w, bias, y, Co, Cy, co_off, s, relu, accumulate, st);
  return cudaErrorInvalidValue;
}

}  // namespace

namespace gt {
int set_error(int code, const char *msg);
int cuda_error(cudaError_t e, const char *what, int line);
}  // namespace gt

#define NN_CK(expr, what)                                              \
  do {                                                                 \
    cudaError_t e_ = (expr);                                           \
    if (e_ != cudaSuccess) return gt::cuda_error(e_, what, __LINE__);   \
  } while (0)

extern "C" {

// dtype codes: 0 = float32, 1 = bfloat16
int gt_nn_conv3d(const void *x, int x_dtype, int Ci, int Cx, int x_off, const void *w_bf16, const float *bias, void *y,
                 int y_dtype, int Co, int Cy, int co_off, int B, int D, int H, int W, int ksize, int relu,
                 int accumulate, void *stream) {
  if (!x || !w_bf16 || !y || Ci < 1 || Co < 1 || co_off < 0 || co_off + Co > Cy || x_off < 0 || x_off + Ci > Cx)
    return gt::set_error(GT_ERR_ARG, "gt_nn_conv3d: bad argument");
  if (B < 1 || D < 1 || H < 1 || W < 4 || W % 4 != 0 || (ksize != 1 && ksize != 3))
    return gt::set_error(GT_ERR_ARG, "gt_nn_conv3d: shape must be positive with W % 4 == 0, ksize 1 or 3");
  const Shape s{B, D, H, W};
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e;
  if (g_tc_mode && g_tc2_mode && x_dtype == 1 && ksize == 3 && tc2_ok(Ci, Co, s)) {
    const unsigned g = (unsigned)(((long long)B * D * H * W) / 128);
    const __nv_bfloat16 *xb = (const __nv_bfloat16 *)x, *wb = (const __nv_bfloat16 *)w_bf16;
    const size_t smem = tc2_smem(W, Co);
    // the weights' shared-memory image, in stream-ordered scratch freed after the launch
    const long long units = 27ll * Co * 2 * (Ci / 16);
    uint4 *img = nullptr;
    cudaError_t ea = cudaMallocAsync((void **)&img, sizeof(uint4) * units, st);
    if (ea == cudaSuccess) {
      k_conv_wimage<<<(unsigned)((units + 255) / 256), 256, 0, st>>>(wb, Ci, Co, img);
      ea = cudaGetLastError();
    }
    if (ea == cudaSuccess) {
      if (y_dtype == 1) {
        ea = cudaFuncSetAttribute(k_conv3d_tc2<__nv_bfloat16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (ea == cudaSuccess)
          k_conv3d_tc2<__nv_bfloat16><<<g, 128, smem, st>>>(xb, Ci, Cx, x_off, img, bias, (__nv_bfloat16 *)y, Co,
                                                            Cy, co_off, s, relu, accumulate);
      } else {
        ea = cudaFuncSetAttribute(k_conv3d_tc2<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (ea == cudaSuccess)
          k_conv3d_tc2<float><<<g, 128, smem, st>>>(xb, Ci, Cx, x_off, img, bias, (float *)y, Co, Cy, co_off, s,
                                                    relu, accumulate);
      }
      if (ea == cudaSuccess) ea = cudaGetLastError();
    }
    if (img) cudaFreeAsync(img, st);
    NN_CK(ea, "gt_nn_conv3d (staged tensor-core kernel)");
    return GT_OK;
  }
  if (g_tc_mode && x_dtype == 1 && Ci % 16 == 0 && Co % 16 == 0 && Co <= 256) {
    const unsigned g = (unsigned)(((long long)B * D * H * W + 127) / 128);
    const __nv_bfloat16 *xb = (const __nv_bfloat16 *)x, *wb = (const __nv_bfloat16 *)w_bf16;
    if (ksize == 3 && y_dtype == 1)
      k_conv3d_tc<__nv_bfloat16, 3><<<g, 128, 0, st>>>(xb, Ci, Cx, x_off, wb, bias, (__nv_bfloat16 *)y, Co, Cy, co_off, s, relu, accumulate);
    else if (ksize == 3)
      k_conv3d_tc<float, 3><<<g, 128, 0, st>>>(xb, Ci, Cx, x_off, wb, bias, (float *)y, Co, Cy, co_off, s, relu, accumulate);
    else if (y_dtype == 1)
      k_conv3d_tc<__nv_bfloat16, 1><<<g, 128, 0, st>>>(xb, Ci, Cx, x_off, wb, bias, (__nv_bfloat16 *)y, Co, Cy, co_off, s, relu, accumulate);
    else
      k_conv3d_tc<float, 1><<<g, 128, 0, st>>>(xb, Ci, Cx, x_off, wb, bias, (float *)y, Co, Cy, co_off, s, relu, accumulate);
    NN_CK(cudaGetLastError(), "gt_nn_conv3d (tensor cores)");
    return GT_OK;
  }
  if (x_dtype == 1 && y_dtype == 1)
    e = conv_k<__nv_bfloat16, __nv_bfloat16>(ksize, x, Ci, Cx, x_off, w_bf16, bias, y, Co, Cy, co_off, s, relu, accumulate, st);
  else if (x_dtype == 1 && y_dtype == 0)
    e = conv_k<__nv_bfloat16, float>(ksize, x, Ci, Cx, x_off, w_bf16, bias, y, Co, Cy, co_off, s, relu, accumulate, st);
  else if (x_dtype == 0 && y_dtype == 0)
    e = conv_k<float, float>(ksize, x, Ci, Cx, x_off, w_bf16, bias, y, Co, Cy, co_off, s, relu, accumulate, st);
  else if (x_dtype == 0 && y_dtype == 1)
    e = conv_k<float, __nv_bfloat16>(ksize, x, Ci, Cx, x_off, w_bf16, bias, y, Co, Cy, co_off, s, relu, accumulate, st);
  else
    return gt::set_error(GT_ERR_ARG, "gt_nn_conv3d: dtype must be 0 (f32) or 1 (bf16)");
  NN_CK(e, "gt_nn_conv3d");
  return GT_OK;
}

int gt_nn_set_tensor_cores(int on) {
  if (on < 0 || on > 2) return gt::set_error(GT_ERR_ARG, "gt_nn_set_tensor_cores: 0, 1 or 2");
  g_tc_mode = on ? 1 : 0;
  g_tc2_mode = on == 1 ? 1 : 0;
  return GT_OK;
}

int gt_nn_check(void) {
  int flag = 0;
  NN_CK(cudaMemcpyFromSymbol(&flag, g_nn_err, sizeof(int)), "gt_nn_check");
  if (flag) {
    const int zero = 0;
    NN_CK(cudaMemcpyToSymbol(g_nn_err, &zero, sizeof(int)), "gt_nn_check");
    return gt::set_error(GT_ERR_TIMEOUT, "a tensor-core convolution block gave up waiting for its MMA");
  }
  return GT_OK;
}

int gt_nn_flip_weights(const void *w_bf16, void *wf_bf16, int Co, int Ci, int ksize, void *stream) {
  const int K3 = ksize * ksize * ksize;
  k_flip<<<nblk((long long)Co * Ci * K3, 256), 256, 0, (cudaStream_t)stream>>>(
      (const __nv_bfloat16 *)w_bf16, (__nv_bfloat16 *)wf_bf16, Co, Ci, K3);
  NN_CK(cudaGetLastError(), "gt_nn_flip_weights");
  return GT_OK;
}

// part must hold nchunk * Co * Ci * K3 floats; nchunk = ceil(voxels / kchunk)
int gt_nn_conv3d_wgrad(const float *dy, int Co, int Cdy, int dy_off, const void *x, int x_dtype, int Ci, int Cx,
                       int x_off, int B, int D, int H, int W, int ksize, long long kchunk, float *part, float *g,
                       int accumulate, void *stream) {
  if (!dy || !x || !part || !g || kchunk < 1 || dy_off < 0 || dy_off + Co > Cdy || x_off < 0 || x_off + Ci > Cx)
    return gt::set_error(GT_ERR_ARG, "gt_nn_conv3d_wgrad: bad argument");
  const int K3 = ksize * ksize * ksize, N = Ci * K3;
  const long long nvox = (long long)B * D * H * W;
  const long long nchunk = (nvox + kchunk - 1) / kchunk;
  if (nchunk > 65535) return gt::set_error(GT_ERR_ARG, "gt_nn_conv3d_wgrad: kchunk too small (more than 65535 chunks)");
  const Shape s{B, D, H, W};
  cudaStream_t st = (cudaStream_t)stream;
  dim3 grid(nblk(N, WG_N), nblk(Co, WG_M), (unsigned)nchunk);
  if (ksize == 3 && x_dtype == 1)
    k_wgrad<__nv_bfloat16, 3><<<grid, 256, 0, st>>>(dy, Co, Cdy, dy_off, (const __nv_bfloat16 *)x, Ci, Cx, x_off, s, kchunk, part);
  else if (ksize == 1 && x_dtype == 1)
    k_wgrad<__nv_bfloat16, 1><<<grid, 256, 0, st>>>(dy, Co, Cdy, dy_off, (const __nv_bfloat16 *)x, Ci, Cx, x_off, s, kchunk, part);
  else if (ksize == 3 && x_dtype == 0)
    k_wgrad<float, 3><<<grid, 256, 0, st>>>(dy, Co, Cdy, dy_off, (const float *)x, Ci, Cx, x_off, s, kchunk, part);
  else if (ksize == 1 && x_dtype == 0)
    k_wgrad<float, 1><<<grid, 256, 0, st>>>(dy, Co, Cdy, dy_off, (const float *)x, Ci, Cx, x_off, s, kchunk, part);
  else
    return gt::set_error(GT_ERR_ARG, "gt_nn_conv3d_wgrad: ksize 1 or 3, dtype 0 or 1");
  const long long n = (long long)Co * N;
  k_wgrad_reduce<<<nblk(n, 256), 256, 0, st>>>(part, (int)nchunk, n, g, accumulate);
  NN_CK(cudaGetLastError(), "gt_nn_conv3d_wgrad");
  return GT_OK;
}

int gt_nn_bias_grad(const float *dy, int Co, int Cdy, int dy_off, int B, long long vol, float *db, int accumulate,
                    void *stream) {
  if (!dy || !db || Co < 1 || dy_off < 0 || dy_off + Co > Cdy) return gt::set_error(GT_ERR_ARG, "gt_nn_bias_grad: bad argument");
  k_bias_grad<<<Co, 256, 0, (cudaStream_t)stream>>>(dy, Co, Cdy, dy_off, vol, B, db, accumulate);
  NN_CK(cudaGetLastError(), "gt_nn_bias_grad");
  return GT_OK;
}

int gt_nn_scale(const void *x, int x_dtype, void *y, int y_dtype, int C, int B, long long vol, const float *scale,
                int floor0, void *stream) {
  if (!x || !y || !scale || C < 1 || B < 1 || vol < 1) return gt::set_error(GT_ERR_ARG, "gt_nn_scale: bad argument");
  const long long n = (long long)B * C * vol;
  cudaStream_t st = (cudaStream_t)stream;
  if (x_dtype == 0 && y_dtype == 0) k_scale<float, float><<<nblk(n, 256), 256, 0, st>>>((const float *)x, (float *)y, C, vol, B, scale, floor0);
  else if (x_dtype == 0 && y_dtype == 1) k_scale<float, __nv_bfloat16><<<nblk(n, 256), 256, 0, st>>>((const float *)x, (__nv_bfloat16 *)y, C, vol, B, scale, floor0);
  else if (x_dtype == 1 && y_dtype == 0) k_scale<__nv_bfloat16, float><<<nblk(n, 256), 256, 0, st>>>((const __nv_bfloat16 *)x, (float *)y, C, vol, B, scale, floor0);
  else if (x_dtype == 1 && y_dtype == 1) k_scale<__nv_bfloat16, __nv_bfloat16><<<nblk(n, 256), 256, 0, st>>>((const __nv_bfloat16 *)x, (__nv_bfloat16 *)y, C, vol, B, scale, floor0);
  else return gt::set_error(GT_ERR_ARG, "gt_nn_scale: dtype must be 0 (f32) or 1 (bf16)");
  NN_CK(cudaGetLastError(), "gt_nn_scale");
  return GT_OK;
}

int gt_nn_relu_bwd(float *dy, const void *y, int y_dtype, int C, int Cy, int co_off, int B, long long vol,
                   void *stream) {
  const long long n = (long long)B * C * vol;
  if (y_dtype == 1) k_relu_bwd<__nv_bfloat16><<<nblk(n, 256), 256, 0, (cudaStream_t)stream>>>(dy, (const __nv_bfloat16 *)y, C, Cy, co_off, vol, B);
  else k_relu_bwd<float><<<nblk(n, 256), 256, 0, (cudaStream_t)stream>>>(dy, (const float *)y, C, Cy, co_off, vol, B);
  NN_CK(cudaGetLastError(), "gt_nn_relu_bwd");
  return GT_OK;
}

int gt_nn_pool2(const void *x_bf16, int Cs, int src_off, void *y_bf16, int C, int B, int Do, int Ho, int Wo,
                void *stream) {
  const Shape so{B, Do, Ho, Wo};
  k_pool2<<<nblk((long long)B * C * Do * Ho * Wo, 256), 256, 0, (cudaStream_t)stream>>>(
      (const __nv_bfloat16 *)x_bf16, Cs, src_off, (__nv_bfloat16 *)y_bf16, C, so);
  NN_CK(cudaGetLastError(), "gt_nn_pool2");
  return GT_OK;
}

int gt_nn_pool2_bwd(const float *dy, float *dx, int C, int Cd, int dst_off, int B, int D, int H, int W, void *stream) {
  const Shape si{B, D, H, W};
  k_pool2_bwd<<<nblk((long long)B * C * D * H * W, 256), 256, 0, (cudaStream_t)stream>>>(dy, dx, C, Cd, dst_off, si);
  NN_CK(cudaGetLastError(), "gt_nn_pool2_bwd");
  return GT_OK;
}

int gt_nn_up2(const void *x_bf16, void *y_bf16, int C, int Cd, int dst_off, int B, int D, int H, int W, void *stream) {
  const Shape so{B, D, H, W};
  k_up2<<<nblk((long long)B * C * D * H * W, 256), 256, 0, (cudaStream_t)stream>>>(
      (const __nv_bfloat16 *)x_bf16, (__nv_bfloat16 *)y_bf16, C, Cd, dst_off, so);
  NN_CK(cudaGetLastError(), "gt_nn_up2");
  return GT_OK;
}

int gt_nn_up2_bwd(const float *dy, int Cs, int src_off, float *dx, int C, int B, int Di, int Hi, int Wi,
                  void *stream) {
  const Shape si{B, Di, Hi, Wi};
  k_up2_bwd<<<nblk((long long)B * C * Di * Hi * Wi, 256), 256, 0, (cudaStream_t)stream>>>(dy, Cs, src_off, dx, C, si);
  NN_CK(cudaGetLastError(), "gt_nn_up2_bwd");
  return GT_OK;
}

// part must hold ceil(n/256) floats
int gt_nn_mse(const float *p, const float *q, long long n, float *dp, float *part, void *stream) {
  k_mse<<<nblk(n, 256), 256, 0, (cudaStream_t)stream>>>(p, q, n, dp, part);
  NN_CK(cudaGetLastError(), "gt_nn_mse");
  return GT_OK;
}

int gt_nn_adam(float *w_master, void *w_bf16, const float *g, float *m, float *v, long long n, float lr, float b1,
               float b2, float eps, int step, void *stream) {
  const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
  k_adam<<<nblk(n, 256), 256, 0, (cudaStream_t)stream>>>(w_master, (__nv_bfloat16 *)w_bf16, g, m, v, n, lr, b1, b2,
                                                         eps, c1, c2);
  NN_CK(cudaGetLastError(), "gt_nn_adam");
  return GT_OK;
}

int gt_nn_cast(const void *src, int src_dtype, void *dst, long long n, void *stream) {
  if (src_dtype == 0) k_cast_f2b<<<nblk(n, 256), 256, 0, (cudaStream_t)stream>>>((const float *)src, (__nv_bfloat16 *)dst, n);
  else k_cast_b2f<<<nblk(n, 256), 256, 0, (cudaStream_t)stream>>>((const __nv_bfloat16 *)src, (float *)dst, n);
  NN_CK(cudaGetLastError(), "gt_nn_cast");
  return GT_OK;
}

}  // extern "C"
