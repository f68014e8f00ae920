"""ORACLE / TEST INFRASTRUCTURE ONLY -- numpy restatement of the aggregation
multigrid that preconditions the flexible CG of the p' systems (the library's
p' option precond 4, CSR method 5, sysu_gnn_set_multigrid).  It has no
counterpart in the reference, whose p' solve is CG + SSOR
(navier_pressure.cpp:29) with the stopping test ||b - A x|| / ||b|| < eps
(tools.cpp:56-64), which this form keeps.  Never imported by the product.

The algorithm, restated from the library's description of it:

* hierarchy: greedy aggregation by strength of connection (Vanek, Mandel and
  Brezina, "Algebraic multigrid by smoothed aggregation", Computing 56, 1996,
  the unsmoothed form): strong(i) = {j != i : -a_ij sgn(a_ii) >= theta max_k
  -a_ik sgn(a_ii)}; pass 1 seeds, pass 2 attaches leftovers to the strongest
  aggregated strong neighbour, pass 3 singletons; Galerkin coarse operator
  A_c = P^T A P with piecewise-constant P, rows with the diagonal first and the
  other columns in order of first appearance; levels until <= dense_max rows;
* cycle: V(1,1) with weighted Jacobi (omega / a_ii) on every level, prolonged
  corrections scaled by gamma (over-correction), the coarsest level solved
  exactly (a singular one, rows summing to zero, through A + alpha 1 1^T with
  alpha = mean(a_ii) / n);
* Krylov: flexible CG (Notay, "Flexible conjugate gradients", SIAM J. Sci.
  Comput. 22, 2000), beta = z.q_{k-1} / p_{k-1}.q_{k-1}.

Rows of the input CSR are taken with the diagonal first and the other entries
in their given order, as the library stores them.
"""
from __future__ import annotations

import numpy as np


class Level:
    def __init__(self, rowptr, col, val):
        self.rp = np.asarray(rowptr, np.int64)
        self.col = np.asarray(col, np.int64)
        self.val = np.asarray(val, np.float64)
        self.n = len(self.rp) - 1
        self.diag = self.val[self.rp[:-1]]  # diagonal first
        self.rows = np.repeat(np.arange(self.n), np.diff(self.rp))
        self.agg = None
        self.nc = 0

    def matvec(self, x):
        y = np.zeros(self.n)
        np.add.at(y, self.rows, self.val * x[self.col])
        return y


def diag_first(rowptr, col, val):
    """CSR rows with the diagonal (summed duplicates) first, other entries in order."""
    n = len(rowptr) - 1
    rp, cl, vl = [0], [], []
    for i in range(n):
        ks = range(rowptr[i], rowptr[i + 1])
        d = sum(val[k] for k in ks if col[k] == i)
        cl.append(i)
        vl.append(d)
        for k in ks:
            if col[k] != i:
                cl.append(col[k])
                vl.append(val[k])
        rp.append(len(cl))
    return np.array(rp), np.array(cl), np.array(vl, np.float64)


def aggregate(L: Level, theta: float):
    n = L.n
    strong, sval = [], []
    for i in range(n):
        a, b = L.rp[i], L.rp[i + 1]
        sg = -1.0 if L.val[a] < 0 else 1.0
        js, cs = [], []
        cmax = 0.0
        for k in range(a + 1, b):
            if L.col[k] != i:
                cmax = max(cmax, -L.val[k] * sg)
        if cmax > 0.0:
            for k in range(a + 1, b):
                j = L.col[k]
                if j == i:
                    continue
                c = -L.val[k] * sg
                if c >= theta * cmax:
                    js.append(j)
                    cs.append(c)
        strong.append(js)
        sval.append(cs)
    agg = -np.ones(n, np.int64)
    na = 0
    for i in range(n):
        if agg[i] >= 0 or any(agg[j] >= 0 for j in strong[i]):
            continue
        agg[i] = na
        for j in strong[i]:
            agg[j] = na
        na += 1
    for i in range(n):
        if agg[i] >= 0:
            continue
        best, bc = -1, -1.0
        for j, c in zip(strong[i], sval[i]):
            if agg[j] >= 0 and c > bc:
                bc, best = c, agg[j]
        if best >= 0:
            agg[i] = best
    for i in range(n):
        if agg[i] < 0:
            agg[i] = na
            na += 1
    return agg, na


def galerkin(L: Level, agg, na):
    members = [[] for _ in range(na)]
    for i in range(L.n):
        members[agg[i]].append(i)
    rp, cl, vl = [0], [], []
    for I in range(na):
        slot = {I: len(cl)}
        cl.append(I)
        vl.append(0.0)
        for i in members[I]:
            for k in range(L.rp[i], L.rp[i + 1]):
                J = int(agg[L.col[k]])
                if J not in slot:
                    slot[J] = len(cl)
                    cl.append(J)
                    vl.append(0.0)
                vl[slot[J]] += L.val[k]
        rp.append(len(cl))
    return Level(rp, cl, vl)


def hierarchy(rowptr, col, val, theta=0.25, dense_max=200, max_levels=16):
    levels = [Level(*diag_first(rowptr, col, val))]
    while len(levels) < max_levels and levels[-1].n > dense_max:
        L = levels[-1]
        agg, na = aggregate(L, theta)
        if na >= L.n:
            break
        L.agg, L.nc = agg, na
        levels.append(galerkin(L, agg, na))
    return levels


def coarsest_inverse(L: Level):
    A = np.zeros((L.n, L.n))
    np.add.at(A, (L.rows, L.col), L.val)
    rowsum = np.abs(A.sum(axis=1)).max()
    if rowsum <= 1e-9 * np.abs(np.diag(A)).max():
        A = A + np.diag(A).mean() / L.n
    return np.linalg.inv(A)


def _coarsest(L: Level, r, omega, dense_max):
    if L.n <= dense_max:
        return coarsest_inverse(L) @ r
    # too large for the dense inverse: three Jacobi steps from zero
    w = omega / L.diag
    z = w * r
    for _ in range(2):
        z = z + w * (r - L.matvec(z))
    return z


def _prolonged(levels, l, r, omega, gamma, dense_max, post=None):
    """Level l's correction before its post-smoothing step: w r + gamma P z_{l+1}.
    post: {level: f(r, zp) -> z} replaces that coarse level's post-smoothing step
    (the learned form's network on a coarse level)."""
    L = levels[l]
    w = omega / L.diag
    t = r - L.matvec(w * r)
    rc = np.zeros(L.nc)
    np.add.at(rc, L.agg, t)
    if l + 1 == len(levels) - 1:
        zc = _coarsest(levels[l + 1], rc, omega, dense_max)
    else:
        C = levels[l + 1]
        zc = _prolonged(levels, l + 1, rc, omega, gamma, dense_max, post)
        if post and (l + 1) in post:
            zc = post[l + 1](rc, zc)
        else:
            zc = zc + omega / C.diag * (rc - C.matvec(zc))
    return w * r + gamma * zc[L.agg]


def cycle_fixed(levels, r, omega=0.8, gamma=1.8, dense_max=200, post=None):
    """Pre-smoothing and coarse correction at the finest level: z2, and t = r - A z2."""
    L0 = levels[0]
    if len(levels) == 1:
        z2 = omega / L0.diag * r
    else:
        z2 = _prolonged(levels, 0, r, omega, gamma, dense_max, post)
    return z2, r - L0.matvec(z2)


def vcycle(levels, r, omega=0.8, gamma=1.8, dense_max=200, post=None):
    """z = M r with the Jacobi post-smoother at the finest level."""
    z2, t = cycle_fixed(levels, r, omega, gamma, dense_max, post)
    return z2 + omega / levels[0].diag * t


def neumann_3d(nx, ny, nz, seed):
    """Test matrix: pure-Neumann 7-point Laplacian (rows sum to zero, so it is
    singular with the constant null vector, like the closed-cavity p' systems),
    negative diagonal, random face coefficients 1 +- 0.3, natural row order."""
    from gnn_np import laplacian_3d
    rp, cl, vl = laplacian_3d(nx, ny, nz, seed=seed, negative=True)
    n = len(rp) - 1
    rows = np.repeat(np.arange(n), np.diff(rp))
    off = np.zeros(n)
    np.add.at(off, rows[cl != rows], vl[cl != rows])
    vl = vl.copy()
    vl[cl == rows] = -off[rows[cl == rows]]
    return rp, cl, vl


def fcg(levels, b, M, eps=1e-8, maxit=500):
    """Flexible CG; returns x, iterations, relative residual."""
    A = levels[0]
    x = np.zeros_like(b)
    r = b.copy()
    bn = np.linalg.norm(b) or 1.0
    p_prev = q_prev = None
    res = np.linalg.norm(r) / bn
    it = 0
    while not (res < eps) and it < maxit:
        it += 1
        z = M(r)
        p = z if p_prev is None else z - (z @ q_prev) / (p_prev @ q_prev) * p_prev
        q = A.matvec(p)
        alpha = (p @ r) / (p @ q)
        x = x + alpha * p
        r = r - alpha * q
        res = np.linalg.norm(r) / bn
        p_prev, q_prev = p, q
    return x, it, res
