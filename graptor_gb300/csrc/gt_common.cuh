// Shared definitions of the GB300 TGV/TV primal-dual solver kernels.
//
// Device layout ("slice-fastest"): for every image-domain field the S = C*Nz
// slice-channel values of one pixel are contiguous,
//     image field   f[(y*N + x)*S + s]            s = c*Nz + z
//     sinogram      g[(j*nd + i)*S + s]           j = angle, i = detector bin
//     vector / tensor fields: one such plane per component, planes `vol` apart.
// With s fastest, the per-pixel geometry of the projectors (detector coordinate,
// interpolation weights, loop bounds) is the same for every lane of a warp, and
// every global access of a warp is one contiguous run of slice values.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

// 4 doubles, 32-byte aligned (the FP64 angle table entry)
struct __align__(32) dvec4 {
  double x, y, z, w;
};

namespace gt {

enum { KL = 0, L2 = 1 };
enum { UNCORR = 0, FROB = 1, NUCL = 2 };

struct Dims {
  int dim;     // 2 or 3
  int N, Nz, C, S;
  int nd, nang;
  size_t vol;  // N*N*S
  size_t nbin; // nd*nang*S
};

// parameters of one iteration (the float32 kernel arguments of tgv_radon,
// radon_tgv_primal_dual_3d.py:1178-1221)
struct IterParams {
  Dims d;
  float sigma, tau;      // primal/dual steps 1/sqrt(Lsqr)
  float sigma_data;      // sigma / normest (update_lambda argument)
  float norming;         // 1 / normest     (update_u argument)
  float ainv0, ainv1;    // 1 / (alpha / normest^2)
  float stepsize;
  int cbase;             // first channel handled by a k_dual launch (0 unless C > 8)
  int fwd_cfg, bp_cfg;   // projector launch shapes (see launch_fwd / launch_bp)
  int dual_cfg;          // 0: k_dual, 1: k_dual_z2 (where dual_z2_ok)
  const float4 *ofs;     // [nang] (X, Y, offset, Xinv)
  const long long *ray_start;  // [nd*nang + 1] ray table offsets (null: walk rays on the fly)
  const int2 *ray_ent;         // (pixel, weight bits) entries of all rays
  const long long *run_start;  // [nang*ceil(nd/3) + 1] offsets of the 3-bin run table (null: none)
  const int4 *run_ent;         // (pixel, weight bits of bins i0, i0+1, i0+2) entries of all runs
  const int2 *bp_tab;          // [N*N][nang] (floor bin, fraction bits) of the back projection (or null)
  const int4 *row_ent;           // [N][ceil(N/4)][nang][3] back-projection row-tile entries (or null)
  const float *mu;       // [C] mu (KL) or mu/(sigma+mu) (L2)
  float *u, *ubar;       // [vol]
  float *p, *pbar, *v;   // [K][vol]
  float *w;              // [KW][vol]
  float *lam, *f, *ku;   // [nbin]
  float *kstar;          // [vol] back projection K* lambda
  float *p2, *v2, *w2;   // outputs of k_dual_cl2's fused form (p, v, w of the next iterate), or null
  float *ulo;            // [vol] low parts of u in the precise primal mode (u = u + ulo), or null
  const double *mu64;    // [C] mu (KL) or mu (L2) in double, for the gap
  double ne64;           // operator-norm estimate, for the gap
  const void *bp_tmap;   // host copies of the TMA descriptors of lambda for k_bp_tma with
  const void *bp_tmap_wide;  // 128- and 256-slice boxes, or null
  int *err;              // device flag: a kernel gave up a bounded wait (read by gt_synchronize)
  int bp_skip_angle;     // test hook of k_bp_tma: the copy of this angle is never issued (-1: none)
  unsigned bp_wait_limit;  // polls of one bounded wait in k_bp_tma
};

// Members of a fused batch launch (gt_batch mode 1): one launch covers the work
// units of every member; block b belongs to the member k with start[k] <= b <
// start[k + 1] and runs that member's kernel body as its block b - start[k].
struct BatchTab {
  const IterParams *P;   // [n] the members' iteration parameters (device copy)
  const int *start;      // [n + 1] first block of each member in this launch
  const int *disc;       // [n] data term of each member (KL / L2)
  const int *shape;      // [n] slices per thread of the member's projector / update bodies: 0 one, 1 four, 2 eight
  int n;
};

}  // namespace gt
