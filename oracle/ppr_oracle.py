"""FP64 restatement of personalised PageRank and its adjoint.

TEST INFRASTRUCTURE, NOT PRODUCT CODE. Imported only by tests/ and
bench.py's CPU-baseline leg, as the checker or the timed CPU baseline.

The reference has no personalised or differentiable PageRank, so this
oracle is not pinned by the reference ("parity unpinned by the reference").
It is pinned instead by (1) a dense FP64 linear solve of the fixed point,
(2) FP64 central finite differences of the loss, checked here against
brute-force perturbed solves, and (3) the recurrence it shares with the
reference's pull PageRank (01_host/src/algorithms/openmp/pageRank.c:245-368:
pull over in-edges, dangling mass dropped).

Model, with forward CSR (offsets, dest) and per-edge weights w:
    P[v,u] = w_e / s_u for e = (u -> v), s_u = sum of u's out-weights
    R = (1-d) T + d P R,  L = <W, R>
    Lam = W + d P^T Lam,  dL/dT = (1-d) Lam
    g_e = d <Lam[v], R[u]>,  dL/dw_e = (g_e - sum_{e' of u} g_e' P_e') / s_u
"""
from __future__ import annotations

import numpy as np
import scipy.linalg as sla
import scipy.sparse as sp


def sources(offsets) -> np.ndarray:
    offsets = np.asarray(offsets, np.int64)
    return np.repeat(np.arange(len(offsets) - 1, dtype=np.int64), np.diff(offsets))


def normalised(offsets, w):
    """(P_e, s_u) in FP64."""
    src = sources(offsets)
    w = np.asarray(w, np.float64)
    s = np.bincount(src, weights=w, minlength=len(offsets) - 1)
    with np.errstate(divide="ignore", invalid="ignore"):
        p = np.where(s[src] > 0, w / s[src], 0.0)
    return p, s


def matrix(offsets, dest, w) -> sp.csr_matrix:
    """Sparse P (V x V, FP64): P[v, u] = w_e / s_u; repeated edges add up."""
    V = len(offsets) - 1
    p, _ = normalised(offsets, w)
    return sp.csr_matrix((p, (np.asarray(dest, np.int64), sources(offsets))), shape=(V, V))


def forward_iter(offsets, dest, w, T, d=0.85, tol=1e-7, max_iterations=1000, iterations=None):
    """Power iteration from R0 = (1-d) T; stops when the largest per-column L1
    change is below tol (or after exactly `iterations` sweeps when given).
    Returns (R, sweeps, last residual)."""
    P = matrix(offsets, dest, w)
    T = np.asarray(T, np.float64)
    R = (1 - d) * T
    n = iterations if iterations is not None else max_iterations
    res = np.inf
    it = 0
    for it in range(1, n + 1):
        Rn = (1 - d) * T + d * (P @ R)
        res = float(np.abs(Rn - R).sum(axis=0).max())
        R = Rn
        if iterations is None and res < tol:
            break
    return R, it, res


def _system(offsets, dest, w, d):
    V = len(offsets) - 1
    return np.eye(V) - d * matrix(offsets, dest, w).toarray()


def forward_dense(offsets, dest, w, T, d=0.85):
    """Exact fixed point R = (1-d) (I - dP)^-1 T by a dense FP64 solve."""
    A = _system(offsets, dest, w, d)
    return np.linalg.solve(A, (1 - d) * np.asarray(T, np.float64))


def loss(offsets, dest, w, T, W, d=0.85) -> float:
    return float(np.sum(np.asarray(W, np.float64) * forward_dense(offsets, dest, w, T, d)))


def adjoint_dense(offsets, dest, w, T, W, d=0.85):
    """Gradients by dense FP64 solves: (grad_w[E], grad_T[V,K], loss, R, Lam)."""
    A = _system(offsets, dest, w, d)
    W = np.asarray(W, np.float64)
    R = np.linalg.solve(A, (1 - d) * np.asarray(T, np.float64))
    Lam = np.linalg.solve(A.T, W)
    src = sources(offsets)
    dest = np.asarray(dest, np.int64)
    p, s = normalised(offsets, w)
    g = d * np.einsum("ek,ek->e", Lam[dest], R[src])
    wsum = np.bincount(src, weights=g * p, minlength=len(s))
    with np.errstate(divide="ignore", invalid="ignore"):
        gw = np.where(s[src] > 0, (g - wsum[src]) / s[src], 0.0)
    return gw, (1 - d) * Lam, float(np.sum(W * R)), R, Lam


class FiniteDifference:
    """Exact FP64 losses at perturbed weights w + t*e_i, for central
    differences (L(w+h e_i) - L(w-h e_i)) / 2h.

    Perturbing one weight of source u changes only column u of P, so the
    perturbed system A' = A - c e_u^T (c = d * (P'[:,u] - P[:,u])) is a
    rank-one update of A = I - dP, and Sherman-Morrison gives
    L' - L = (1-d) (c . Lt) R~[u] / (1 - (A^-1 c)[u]) with Lt = A^-T W,
    R~ = A^-1 T, from one LU factorisation of A."""

    def __init__(self, offsets, dest, w, T, W, d=0.85):
        self.off = np.asarray(offsets, np.int64)
        self.dest = np.asarray(dest, np.int64)
        self.w = np.asarray(w, np.float64)
        self.d = d
        A = _system(offsets, dest, w, d)
        self.lu = sla.lu_factor(A)
        self.Rt = sla.lu_solve(self.lu, np.asarray(T, np.float64))
        self.Lt = sla.lu_solve(self.lu, np.asarray(W, np.float64), trans=1)
        self.src = sources(offsets)

    def delta_loss(self, e: int, t: float) -> float:
        u = int(self.src[e])
        b, en = int(self.off[u]), int(self.off[u + 1])
        wu = self.w[b:en].copy()
        s0 = wu.sum()
        p0 = wu / s0
        wu[e - b] += t
        p1 = wu / wu.sum()
        c = np.zeros(len(self.off) - 1)
        np.add.at(c, self.dest[b:en], self.d * (p1 - p0))
        z = sla.lu_solve(self.lu, c)
        return float((1 - self.d) * (c @ self.Lt) @ self.Rt[u] / (1.0 - z[u]))

    def central(self, e: int, h: float = 1e-4) -> float:
        return (self.delta_loss(e, h) - self.delta_loss(e, -h)) / (2 * h)


def seeds_teleport(V, K, seeds_per_column=32, rng=None):
    """T[:, k] uniform over `seeds_per_column` distinct random vertices."""
    rng = rng or np.random.default_rng(0)
    T = np.zeros((V, K), np.float32)
    for k in range(K):
        idx = rng.choice(V, size=min(seeds_per_column, V), replace=False)
        T[idx, k] = 1.0 / len(idx)
    return T
