"""FP64 NumPy oracle of the primal-dual iteration, and the primal-dual gap.

Test infrastructure only (the checker for the FP64-accuracy figures and for the
device gap).  The iteration follows the reference loop
(radon_tgv_primal_dual_3d.py:1194-1221, 2-D :767-799) in double precision, with
the Radon operator as an exact sparse matrix of the reference's hat weights
(radon :773-816 without the float bound truncation) and the ball projections in
closed form (Frobenius / uncorrelated; the nuclear projection by SVD).

The problem the loop solves (with ne the operator-norm estimate, K = R/ne,
alpha~ = alpha/ne^2):

  min_{u >= 0, p}  a1~ sum_x ||grad u - p||_V  +  a0~ sum_x ||E p||_W*  +  D(u)

  D_KL(u) = (1/ne) sum_c mu_c sum_bins (R u - f + f log(f / R u))
  D_L2(u) = sum_c mu_c / (2 ne^2) ||R u_c - f_c||^2

||.||_W* is the support function of the reference's w-ball (NormW) under the
w inner product <w, e> = sum diag + 2 sum off-diag that update_p's adjoint
implies.  The gap bounds u to the box [0, U] so that the dual is finite:

  D(v~, w~, lam) = -F~*(lam) + U sum min(0, K^T lam + grad^T v~)
  v~ = theta E^T w,  w~ = theta w,  theta = min(1, a1~ / max ||E^T w||_V)

  relative gap = (P - D) / |P|
"""
from __future__ import annotations

import math

import numpy as np
import scipy.sparse as sp


# ----------------------------------------------------------------------- operator
def angle_table64(angles, N, nd):
    ang = np.asarray(angles, np.float64)
    X, Y = np.cos(ang), np.sin(ang)
    with np.errstate(divide="ignore"):
        Xinv = 1.0 / X
    m = np.abs(Xinv) > 10 * nd
    X[m] = 0.0
    Y[m] = np.round(np.sin(ang[m]))
    off = (nd - 1) / 2.0 - X * (N - 1) / 2.0 - Y * (N - 1) / 2.0
    return X, Y, off


def radon_matrix(angles, N, nd):
    """Sparse R: (nang*nd) x (N*N), rows j*nd + i, columns y*N + x; weight (1 - |t - i|)+."""
    X, Y, off = angle_table64(angles, N, nd)
    yy, xx = np.mgrid[0:N, 0:N]
    xx = xx.ravel().astype(np.float64)
    yy = yy.ravel().astype(np.float64)
    pix = np.arange(N * N)
    rows, cols, vals = [], [], []
    for j in range(len(X)):
        t = xx * X[j] + yy * Y[j] + off[j]
        fl = np.floor(t)
        p = t - fl
        for k, w in ((fl, 1.0 - p), (fl + 1, p)):
            ok = (k >= 0) & (k < nd) & (w > 0)
            rows.append(j * nd + k[ok].astype(np.int64))
            cols.append(pix[ok])
            vals.append(w[ok])
    return sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                         shape=(len(X) * nd, N * N))


# ----------------------------------------------------------------------- stencils
# fields: scalar u[S, N, N] ([s, y, x]); vectors [K, S, N, N]; s = c*Nz + z
def grad(u, dim, Nz, step):
    S, N, _ = u.shape
    g = np.zeros((dim,) + u.shape)
    g[0, :, :, :-1] = u[:, :, 1:] - u[:, :, :-1]
    g[1, :, :-1, :] = u[:, 1:, :] - u[:, :-1, :]
    if dim == 3:
        v = u.reshape(-1, Nz, N, N)
        gz = np.zeros_like(v)
        gz[:, :-1] = (v[:, 1:] - v[:, :-1]) / step
        g[2] = gz.reshape(u.shape)
    return g


def div(v, dim, Nz, step):
    """-grad^T: backward differences (update_u :716-725)."""
    S, N = v.shape[1], v.shape[2]
    d = np.zeros(v.shape[1:])
    a = v[0].copy(); a[:, :, -1] = 0; a[:, :, 1:] -= v[0][:, :, :-1]
    b = v[1].copy(); b[:, -1, :] = 0; b[:, 1:, :] -= v[1][:, :-1, :]
    d = a + b
    if dim == 3:
        c = v[2].reshape(-1, Nz, N, N).copy()
        src = v[2].reshape(-1, Nz, N, N)
        c[:, -1] = 0
        c[:, 1:] -= src[:, :-1]
        d = d + (c / step).reshape(d.shape)
    return d


def sym_grad(p, dim, Nz, step):
    """E p, backward differences, zero at index 0 (update_w :648-656)."""
    S, N = p.shape[1], p.shape[2]

    def bx(f):
        o = np.zeros_like(f); o[:, :, 1:] = f[:, :, 1:] - f[:, :, :-1]; return o

    def by(f):
        o = np.zeros_like(f); o[:, 1:, :] = f[:, 1:, :] - f[:, :-1, :]; return o

    def bz(f):
        v = f.reshape(-1, Nz, N, N); o = np.zeros_like(v); o[:, 1:] = (v[:, 1:] - v[:, :-1]) / step
        return o.reshape(f.shape)

    if dim == 3:
        a = [bx(p[k]) for k in range(3)]
        b = [by(p[k]) for k in range(3)]
        c = [bz(p[k]) for k in range(3)]
        return np.stack([a[0], b[1], c[2], 0.5 * (a[1] + b[0]), 0.5 * (a[2] + c[0]), 0.5 * (b[2] + c[1])])
    a = [bx(p[k]) for k in range(2)]
    b = [by(p[k]) for k in range(2)]
    return np.stack([a[0], b[1], 0.5 * (a[1] + b[0])])


def div_sym(w, dim, Nz, step):
    """-E^T under the w inner product (update_p :744-755)."""
    S, N = w.shape[1], w.shape[2]

    def fx(f):  # forward difference of the reference: -f + f(x+1), zero-handling at ends
        o = -f.copy(); o[:, :, 0] = 0; o[:, :, :-1] += f[:, :, 1:]; return o

    def fy(f):
        o = -f.copy(); o[:, 0, :] = 0; o[:, :-1, :] += f[:, 1:, :]; return o

    def fz(f):
        v = f.reshape(-1, Nz, N, N); o = -v.copy(); o[:, 0] = 0; o[:, :-1] += v[:, 1:]
        return (o / step).reshape(f.shape)

    if dim == 3:
        rows = [(0, 3, 4), (3, 1, 5), (4, 5, 2)]
        return np.stack([fx(w[a]) + fy(w[b]) + fz(w[c]) for a, b, c in rows])
    rows = [(0, 2), (2, 1)]
    return np.stack([fx(w[a]) + fy(w[b]) for a, b in rows])


# ----------------------------------------------------------------------- ball geometry
def w_weights(dim, coupling):
    """(ball weights b, pairing weights m) of the w space: the reference's NormW
    norm^2 = sum b_k w_k^2 (3-D :583/:603, 2-D :232/:254), and <w, e> = sum m_k w_k e_k."""
    q = 1.4142 ** 2
    if dim == 3:
        b = [1, 1, 1, q, q, 1.0] if coupling == "UNCORR" else [1, 1, 1, q, q, q]
        return np.array(b, np.float64), np.array([1, 1, 1, 2, 2, 2], np.float64)
    b = [1, 1, q] if coupling == "UNCORR" else [1, 1, 4.0]
    return np.array(b, np.float64), np.array([1, 1, 2.0])


def _group_norm(x, C, Nz, coupling):
    """per-voxel norms of x[K, S, N, N]: coupled over channels (FROB) or per channel."""
    K, S, N, _ = x.shape
    sq = (x ** 2).sum(0).reshape(C, Nz, N, N)
    if coupling == "UNCORR":
        return np.sqrt(sq).reshape(S, N, N)
    return np.broadcast_to(np.sqrt(sq.sum(0)), (C, Nz, N, N)).reshape(S, N, N)


def project(x, alpha, C, Nz, coupling, weights=None):
    """Projection onto {||x||_b <= alpha} per voxel (nuclear: singular values clipped)."""
    K = x.shape[0]
    b = np.ones(K) if weights is None else weights
    if coupling == "NUCL":
        S, N = x.shape[1], x.shape[2]
        A = x.reshape(K, C, Nz, N, N).transpose(2, 3, 4, 1, 0)  # [Nz, N, N, C, K]
        U, s, Vt = np.linalg.svd(A, full_matrices=False)
        s = np.minimum(s, alpha)
        A = (U * s[..., None, :]) @ Vt
        return A.transpose(4, 3, 0, 1, 2).reshape(x.shape)
    n = _group_norm(x * np.sqrt(b)[:, None, None, None], C, Nz, coupling) / alpha
    return x / np.maximum(n, 1.0)[None]


def support(e, C, Nz, coupling, b, m):
    """sum over voxels of the support function of the ball {sum b w^2 <= 1} under <w,e> = sum m w e."""
    if coupling == "NUCL":
        K, S, N, _ = e.shape
        A = e.reshape(K, C, Nz, N, N).transpose(2, 3, 4, 1, 0)
        return float(np.linalg.svd(A, compute_uv=False).sum())
    scaled = e * (m / np.sqrt(b))[:, None, None, None]
    n = _group_norm(scaled, C, Nz, coupling)
    if coupling == "UNCORR":
        return float(n.sum())
    S, N = e.shape[1], e.shape[2]
    return float(n.reshape(C, Nz, N, N)[0].sum())


# ----------------------------------------------------------------------- solver
class Solver64:
    def __init__(self, dim, N, Nz, C, nd, angles, f, alpha, mu, ne, discrepancy="KL", regularisation="TGV",
                 coupling="FROB", stepsize=1.0, feasible=True):
        self.dim, self.N, self.Nz, self.C, self.nd = dim, N, Nz, C, nd
        self.S = Nz * C
        self.R = radon_matrix(angles, N, nd)
        self.nang = len(angles)
        f = np.asarray(f, np.float64).reshape(self.S, self.nang, nd)
        if feasible:
            r1 = self.R @ np.ones(N * N)
            f = f * (r1.reshape(self.nang, nd) > 0)[None]
        self.f = f
        self.disc, self.reg, self.cpl, self.step = discrepancy, regularisation.upper(), coupling, float(stepsize)
        self.ne = float(ne)
        lsqr = 17.0 if dim == 3 else 0.5 * (18 + math.sqrt(33))
        self.sigma = self.tau = 1.0 / math.sqrt(lsqr)
        self.a0, self.a1 = alpha[0] / ne ** 2, alpha[1] / ne ** 2
        self.mu = np.asarray(mu, np.float64)
        self.wb, self.wm = w_weights(dim, coupling)
        z = lambda *sh: np.zeros(sh)  # noqa: E731
        S = self.S
        self.u, self.ubar = z(S, N, N), z(S, N, N)
        self.p, self.pbar, self.v = z(dim, S, N, N), z(dim, S, N, N), z(dim, S, N, N)
        self.w = z(6 if dim == 3 else 3, S, N, N)
        self.lam = z(S, self.nang, nd)

    def K(self, u):
        return (self.R @ u.reshape(self.S, -1).T).T.reshape(self.S, self.nang, self.nd) / self.ne

    def KT(self, lam):
        return (self.R.T @ lam.reshape(self.S, -1).T).T.reshape(self.S, self.N, self.N) / self.ne

    def mu_s(self):
        return np.repeat(self.mu, self.Nz)[:, None, None]

    def run(self, iters):
        d, Nz, st = self.dim, self.Nz, self.step
        sg, tau = self.sigma, self.tau
        for _ in range(iters):
            self.v = self.v + sg * (grad(self.ubar, d, Nz, st) - self.pbar)
            self.v = project(self.v, self.a1, self.C, Nz, self.cpl)
            if self.reg == "TGV":
                self.w = self.w + sg * sym_grad(self.pbar, d, Nz, st)
                self.w = project(self.w, self.a0, self.C, Nz, "FROB" if self.cpl == "NUCL" else self.cpl, self.wb)
            s = self.lam + sg * self.K(self.ubar)
            m = self.mu_s()
            if self.disc == "KL":
                wv = s - m
                self.lam = s - 0.5 * (wv + np.sqrt(wv * wv + 4 * (sg / self.ne) * self.f * m))
            else:
                self.lam = (s - (sg / self.ne) * self.f) * (m / (sg + m))
            un = np.maximum(0.0, self.u + tau * (div(self.v, d, Nz, st) - self.KT(self.lam)))
            self.ubar, self.u = 2 * un - self.u, un
            if self.reg == "TGV":
                pn = self.p + tau * (self.v + div_sym(self.w, d, Nz, st))
                self.pbar, self.p = 2 * pn - self.p, pn
        return self

    # ------------------------------------------------------------------- gap
    def energies(self, u, p, v, w, lam, U=None):
        """(primal, dual, gap, relative gap) of the scaled problem on the box u in [0, U]."""
        d, Nz, st, C = self.dim, self.Nz, self.step, self.C
        ne, m = self.ne, self.mu_s()
        Ru = self.K(u) * ne
        f = self.f
        if self.disc == "KL":
            with np.errstate(divide="ignore", invalid="ignore"):
                t = np.where(f > 0, f * np.log(f / np.maximum(Ru, 1e-300)), 0.0)
            data = float((m * (Ru - f + t)).sum() / ne)
            with np.errstate(divide="ignore", invalid="ignore"):
                # F*(lam) = -mu f log(1 - lam/mu) for f > 0; 0 for f = 0 (lam <= mu there)
                fstar = float(np.where(f > 0, -(m * f) * np.log1p(-lam / m), 0.0).sum() / ne)
        else:
            data = float((m / (2 * ne ** 2) * (Ru - f) ** 2).sum())
            fstar = float((lam * f / ne).sum() + (lam ** 2 / (2 * m)).sum())
        pv = p if self.reg == "TGV" else np.zeros_like(p)
        reg1 = self.a1 * support(grad(u, d, Nz, st) - pv, C, Nz, self.cpl, np.ones(d), np.ones(d))
        reg0 = 0.0
        if self.reg == "TGV":
            wc = "FROB" if self.cpl == "NUCL" else self.cpl
            reg0 = self.a0 * support(sym_grad(pv, d, Nz, st), C, Nz, wc, self.wb, self.wm)
        P = reg1 + reg0 + data
        # dual: v~ = E^T w (TGV) or v (TV), scaled into its ball
        vt = -div_sym(w, d, Nz, st) if self.reg == "TGV" else v
        nv = _group_norm(vt, C, Nz, "UNCORR" if self.cpl == "UNCORR" else "FROB").max() if self.cpl != "NUCL" \
            else np.linalg.svd(vt.reshape(d, C, Nz, self.N, self.N).transpose(2, 3, 4, 1, 0), compute_uv=False).max()
        theta = min(1.0, self.a1 / nv) if nv > 0 else 1.0
        if U is None:
            U = 2.0 * max(float(u.max()), 1e-30)
        g = self.KT(lam) - theta * div(vt, d, Nz, st)
        D = -fstar + U * float(np.minimum(g, 0.0).sum())
        return {"primal": P, "dual": D, "gap": P - D, "relative": (P - D) / abs(P), "theta": theta, "U": U}

    def gap(self, U=None):
        return self.energies(self.u, self.p, self.v, self.w, self.lam, U)
