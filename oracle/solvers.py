"""NumPy restatement of the reference's eigensolver layer (test infrastructure only).

  src/solvers.jl:44-50      Dense
  src/solvers.jl:65-75      the shared true-residual check and roundoff floor
  src/solvers.jl:85-106     Lanczos (KrylovKit eigsolve; here scipy's ARPACK eigsh as the cross-check)
  src/lobpcg.jl:18-301      LOBPCG policy: preconditioners (fixed / per-Ritz Jacobi), product seed
                            perturbed by sqrt(eps), guard columns, n_conv_check = m + g, one random
                            retry, acceptance on the residual norms
  src/chebyshev.jl:1-406    Chebyshev-filtered subspace iteration, line for line

The LOBPCG core itself lives in an unvendored package (LOBPCGEigensolver 0.1.4); its iterates
are not pinned.  The core here is the block LOBPCG this repository runs on the GPU (hard
locking of a converged prefix, residuals orthogonalized against X, SVQB of [W P], Rayleigh-Ritz
on [X_active W P]); the boundary (eigenvalues vs Dense, true residuals) is what is compared.

Random streams: the reference seeds MersenneTwister(0x4b46) / (0x4346); this restatement uses
numpy's Philox bit generator keyed by the same constants.
"""
from __future__ import annotations

import math

import numpy as np

EPS = np.finfo(np.float64).eps


def dense_solve(H, m):
    M = H.to_matrix()
    M = (M + M.conj().T) / 2
    w, V = np.linalg.eigh(M)
    return (w[:m], V[:, :m]) if 0 < m < len(w) else (w, V)


def colnorms(A):
    return np.sqrt(np.sum(np.abs(A) ** 2, axis=0))


def worst_true_residual(H, E, V):
    """(worst, j): the largest ||H v_j - E_j v_j|| (src/solvers.jl:65-69)."""
    R = H.matvec(V) - V * E[None, :]
    r = colnorms(R)
    j = int(np.argmax(r))
    return float(r[j]), j


def residual_floor(hbound, E1):
    """10 eps max(|gershgorin|, |E_1|) (src/solvers.jl:75)."""
    return 10 * EPS * max(abs(hbound), abs(E1))


def _rng(key):
    return np.random.Generator(np.random.Philox(key))


# ---------------------------------------------------------------------------------------------
# LOBPCG


def perturbed_seed(X0, key=0x4B46):
    """Each column plus a vector of norm sqrt(eps)*||c|| along a fixed random direction (src/lobpcg.jl:167-177)."""
    X = np.array(X0, dtype=np.float64, copy=True)
    rng = _rng(key)
    d = math.sqrt(EPS)
    for j in range(X.shape[1]):
        r = rng.standard_normal(X.shape[0])
        X[:, j] += (d * np.linalg.norm(X[:, j]) / np.linalg.norm(r)) * r
    return X


def _blas():
    from scipy.linalg import blas
    return blas


def _gemm(A, B, trans_a=False, alpha=1.0, beta=0.0, C=None):
    """alpha op(A) B + beta C on F-ordered blocks; returns an F array.  Tall-skinny products (A'B and
    X C with many rows) go to the threaded C helpers (oracle/kf_apply_ref.c), the rest to BLAS
    dgemm.  A column slice of an F-ordered block is passed without a copy."""
    from . import capply
    tall = A.shape[0] >= 4096 and A.shape[1] <= 256 and B.shape[1] <= 256 and capply._fcols(A)
    if tall and trans_a and capply._fcols(B):
        G = capply.gram(A, B)
        if C is None:
            return G if alpha == 1.0 else alpha * G
        C *= beta
        C += alpha * G
        return C
    if tall and not trans_a and (C is None or (capply._fcols(C) and not np.shares_memory(C, A))):
        return capply.update(A, B, alpha, beta, C)
    blas = _blas()
    A = A if A.flags.f_contiguous else np.asfortranarray(A)
    B = B if B.flags.f_contiguous else np.asfortranarray(B)
    if C is None:
        return blas.dgemm(alpha, A, B, trans_a=int(trans_a))
    return blas.dgemm(alpha, A, B, beta=beta, c=C, trans_a=int(trans_a), overwrite_c=True)


def _fblock(N, k):
    return np.empty((N, k), order="F")


def svqb(M, cutoff):
    """Orthonormal basis of range(M) by the unit-diagonal Gram eigen-decomposition; drops small directions."""
    if M.shape[1] == 0:
        return M
    G = _gemm(M, M, trans_a=True)
    d = 1.0 / np.sqrt(np.maximum(np.diag(G), np.finfo(float).tiny))
    lam, U = np.linalg.eigh(d[:, None] * G * d[None, :])
    top = lam[-1]
    keep = lam > cutoff * top if top > 0 else np.zeros_like(lam, dtype=bool)
    T = (d[:, None] * U[:, keep]) / np.sqrt(lam[keep])[None, :]
    return _gemm(M, np.asfortranarray(T))


class SeparablePrecond:
    """The separable (fast-diagonalization) preconditioner on the host, restating the library's
    LOBPCG option: the reference's per-axis eigenbases of the single-axis terms
    (separable_eigenbases, src/apply.jl:606-642) give
        W_j = U diag(1 / hypot(S(p) - theta_j, eta_s)) U' R_j,   U = (x)_a U_a,
    S(p) the sum of the per-axis eigenvalues, eta_s = max(eta, 1e-3 ||H||)."""

    def __init__(self, H, eta, hbound):
        self.dims = list(H.dims)
        self.U, lam = H.separable_eigenbases()
        S = lam[0]
        for a in range(1, len(self.dims)):
            S = (S[:, None] + lam[a][None, :]).reshape(-1, order="F")
        self.S = np.ascontiguousarray(S)
        self.eta = max(eta, 1e-3 * abs(hbound))
        self.Ut = [None if u is None else np.ascontiguousarray(u.T) for u in self.U]
        self.Uc = [None if u is None else np.ascontiguousarray(u) for u in self.U]

    def _mode(self, X, a, A):
        """Y[l, i, r] = sum_j A[i, j] X[l, j, r] along axis a of the F-ordered (N, k) block X."""
        N, k = X.shape
        n = self.dims[a]
        L = int(np.prod(self.dims[:a]))
        R = N * k // (L * n)
        Xc = X.reshape(-1, order="F")
        if L == 1:
            Y = _gemm(A, Xc.reshape(n, R, order="F"))
            return Y.reshape(N, k, order="F")
        v = Xc.reshape(R, n, L)                       # C-order view of the F-ordered block
        Y = np.matmul(A, v)                           # batched over R, each an n x n by n x L product
        return np.asfortranarray(Y.reshape(-1).reshape(N, k, order="F"))

    def __call__(self, Rb, thp):
        from . import capply
        Y = Rb if Rb.flags.f_contiguous else np.asfortranarray(Rb)
        for a, ut in enumerate(self.Ut):
            if ut is not None:
                Y = self._mode(Y, a, ut)
        if Y is Rb:
            Y = Y.copy(order="F")
        capply.scale(Y, self.S, thp, self.eta, 0, Y)
        for a, u in enumerate(self.Uc):
            if u is not None:
                Y = self._mode(Y, a, u)
        return Y


def lobpcg_core(H, X, D, tol, maxiter, precond="ritz", eta=0.01, n_conv_check=None, cutoff=1e-12, sep=None,
                trace=None):
    """Block LOBPCG for the lowest columns of X's width.  Returns dict(lam, X, resid, iters, n_matvec).

    Every block is F-ordered and every tall product goes through BLAS; the residuals and the
    per-Ritz Jacobi scaling run in the C helpers (threaded).  `sep` is a SeparablePrecond for
    precond="separable".  Raises RuntimeError on breakdown (an empty [W P] basis with unconverged
    columns).
    """
    from . import capply
    N, w = X.shape
    n_conv_check = w if n_conv_check is None else n_conv_check
    X = svqb(np.asfortranarray(X), cutoff)
    if X.shape[1] < w:
        raise RuntimeError("LOBPCG: the initial block is rank deficient")
    X = svqb(X, cutoff)
    HX = np.asfortranarray(H.matvec(X))
    nmv = w
    lam, Q = np.linalg.eigh(_sym(_gemm(X, HX, trans_a=True)))
    Q = np.asfortranarray(Q)
    X, HX = _gemm(X, Q), _gemm(HX, Q)
    theta_prec = (np.sum(D[:, None] * X ** 2, axis=0) / np.sum(X ** 2, axis=0))
    P = _fblock(N, 0)
    Rb = _fblock(N, w)
    nl = 0
    res = np.full(w, np.inf)
    it = 0
    while True:
        act = slice(nl, w)
        R = Rb[:, :w - nl]
        res[act] = np.sqrt(capply.resid(X[:, act], HX[:, act], lam[act], R))
        if trace is not None:
            trace(it, res.copy())
        newly = 0
        while nl + newly < w and res[nl + newly] <= tol:
            newly += 1
        if nl + newly >= n_conv_check:
            nl += newly
            break
        if it >= maxiter:
            break
        it += 1
        # precondition the residuals of the still-active columns
        R = R[:, newly:]
        thp = theta_prec[newly:] if it == 1 else lam[nl + newly:w]
        na = w - nl - newly
        np_ = P.shape[1] - newly if P.shape[1] else 0
        Z = _fblock(N, na + np_)
        if precond == "ritz":
            capply.scale(R, D, thp, eta, 0, Z[:, :na])
        elif precond == "jacobi":
            capply.scale(R, D, np.array([D.min() - 1]), eta, 1, Z[:, :na])
        elif precond == "separable":
            Z[:, :na] = sep(R, thp)
        else:
            Z[:, :na] = R
        if np_:
            Z[:, na:] = P[:, newly:]
        nl += newly
        # orthogonalize [W P] against every column of X (one projection), then against itself (SVQB), twice
        for _ in range(2):
            Cx = _gemm(X, Z, trans_a=True)
            Z = _gemm(X, Cx, alpha=-1.0, beta=1.0, C=Z)
            Z = svqb(Z, cutoff)
        if Z.shape[1] == 0:
            raise RuntimeError("LOBPCG: the search directions vanished")
        HZ = np.asfortranarray(H.matvec(Z))
        nmv += Z.shape[1]
        Xa, HXa = X[:, nl:], HX[:, nl:]
        nz = Z.shape[1]
        A = np.empty((na + nz, na + nz))
        A[:na, :na] = _gemm(Xa, HXa, trans_a=True)
        A[:na, na:] = _gemm(Xa, HZ, trans_a=True)
        A[na:, :na] = A[:na, na:].T
        A[na:, na:] = _gemm(Z, HZ, trans_a=True)
        th, Cm = np.linalg.eigh(_sym(A))
        Cx = np.asfortranarray(Cm[:na, :na])
        Cz = np.asfortranarray(Cm[na:, :na])
        Xn = _gemm(Z, Cz, C=_gemm(Xa, Cx), beta=1.0)
        HXn = _gemm(HZ, Cz, C=_gemm(HXa, Cx), beta=1.0)
        X[:, nl:] = Xn
        HX[:, nl:] = HXn
        lam[nl:] = th[:na]
        P = _gemm(Z, Cz)
    order = np.argsort(lam, kind="stable")
    return {"lam": lam[order], "X": X[:, order], "resid": res[order], "iters": it, "n_matvec": nmv}


def _fast(H):
    """H with its matvec through the C restatement of mul! (oracle/kf_apply_ref.c) when H is a real
    `kfref.KronFreeOperator`, else H itself."""
    from . import capply, kfref
    if not isinstance(H, kfref.KronFreeOperator) or H.dtype != np.float64:
        return H
    CA = capply.CApply(H)

    class _F:
        N, dtype = H.N, H.dtype

        def matvec(self, X):
            return CA.matvec(X)

    return _F()


def _sym(A):
    return (A + A.T) / 2


class LOBPCG:
    """Option record mirroring src/tree.jl:66-87."""

    def __init__(self, tol=1e-8, maxiter=1000, preconditioner="ritz", eta=0.01, guard=4, seed="product"):
        if not (tol > 0 and math.isfinite(tol)):
            raise ValueError("LOBPCG: tol must be positive and finite")
        if maxiter < 1:
            raise ValueError("LOBPCG: maxiter must be at least 1")
        if preconditioner not in ("ritz", "jacobi", "none", "separable"):
            raise ValueError("LOBPCG: preconditioner must be ritz, jacobi, none or separable")
        if guard < 0:
            raise ValueError("LOBPCG: guard must be nonnegative")
        self.tol, self.maxiter, self.preconditioner, self.eta = tol, maxiter, preconditioner, eta
        self.guard, self.seed = guard, seed


class NotConverged(RuntimeError):
    """A solve that ran out of maxiter; `res` is the last iterate's record (lam, X, resid, iters)."""

    def __init__(self, msg, res):
        super().__init__(msg)
        self.res = res


def lobpcg_solve(s, H, m, X0=None):
    """The reference's lobpcg_solve policy (src/lobpcg.jl:217-301) around `lobpcg_core`."""
    N = H.N
    if m < 1:
        raise ValueError(f"LOBPCG requires m >= 1, got {m}")
    if N < 3 * m + 5:
        raise ValueError(f"LOBPCG needs N >= 3m + 5, got N = {N} for m = {m}")
    if X0 is not None:
        X0 = np.asarray(X0, dtype=np.float64)
        if X0.shape != (N, m):
            raise ValueError("LOBPCG: X0 has the wrong size")
        if not np.all(np.isfinite(X0)):
            raise ValueError("LOBPCG: X0 has non-finite entries")
        for j in range(m):
            if not np.any(X0[:, j]):
                raise ValueError(f"LOBPCG: column {j + 1} of X0 is zero")
    g = min(s.guard, (N - 5) // 3 - m)
    w = m + g
    pseed = H.product_seed(w) if s.seed == "product" else None
    D = H.full_diagonal()
    rng = _rng(0x5EED)
    sep = SeparablePrecond(H, s.eta, H.gershgorin_bound()) if s.preconditioner == "separable" else None
    Hm = _fast(H)

    def attempt(first, guards):
        X = np.empty((N, w), order="F")
        X[:, :m] = first
        X[:, m:] = rng.standard_normal((N, g)) if guards is None else guards
        return lobpcg_core(Hm, X, D, s.tol, s.maxiter, s.preconditioner, s.eta, n_conv_check=w, sep=sep)

    if X0 is not None:
        first = perturbed_seed(X0)
        guards = None if pseed is None else perturbed_seed(pseed[:, m:])
    elif pseed is not None:
        Q = perturbed_seed(pseed)
        first, guards = Q[:, :m], Q[:, m:]
    else:
        first, guards = rng.standard_normal((N, m)), None
    try:
        res = attempt(first, guards)
    except RuntimeError:
        if X0 is None and s.seed != "product":
            raise
        res = attempt(rng.standard_normal((N, m)), None)
    resid = res["resid"]
    bad = int(np.sum(~(resid[:m] <= s.tol)))
    if bad:
        raise NotConverged(f"LOBPCG: {bad} of {m} eigenpairs did not converge within {s.maxiter} iterations", res)
    return res["lam"][:m], res["X"][:, :m], res


# ---------------------------------------------------------------------------------------------
# Chebyshev-filtered subspace iteration (src/chebyshev.jl)

SVQB_CUTOFF = 1e-12
LOCK_FRACTION = 0.5
SEED_ADMIXTURE = 1e-2
CHEBYSHEV_GUARDS = 4
GUARD_GAIN_FRACTION = 0.1


class ChebyshevFilter:
    """Option record mirroring src/tree.jl:293-321."""

    def __init__(self, tol=1e-8, degree=100, extra=40, maxiter=50, rescale_every=20, ortho="svqb",
                 bound="gershgorin", seed="product"):
        if not (tol > 0 and math.isfinite(tol)):
            raise ValueError("ChebyshevFilter: tol must be positive and finite")
        if not 1 <= degree <= 200:
            raise ValueError("ChebyshevFilter: degree must lie in 1:200")
        if extra < 2:
            raise ValueError("ChebyshevFilter: extra must be at least 2")
        if maxiter < 1 or rescale_every < 1:
            raise ValueError("ChebyshevFilter: maxiter and rescale_every must be at least 1")
        if ortho not in ("svqb", "cholqr"):
            raise ValueError("ChebyshevFilter: ortho must be svqb or cholqr")
        self.tol, self.degree, self.extra, self.maxiter = tol, degree, extra, maxiter
        self.rescale_every, self.ortho, self.bound, self.seed = rescale_every, ortho, bound, seed


def _normalize_columns(Z):
    Z /= np.maximum(colnorms(Z), np.finfo(float).tiny)[None, :]
    return Z


def chebyshev_filter(H, X, lcut, lmax, degree, rescale_every):
    """T_degree((H - c)/e) X up to per-column scales (src/chebyshev.jl:38-54)."""
    c, e = (lmax + lcut) / 2, (lmax - lcut) / 2
    A = X.copy()
    B = (H.matvec(A) - c * A) / e
    for k in range(2, degree + 1):
        C = (2 / e) * (H.matvec(B) - c * B) - A
        A, B = B, C
        if k % rescale_every == 0:
            sc = np.maximum(colnorms(B), np.finfo(float).tiny)
            A = A / sc
            B = B / sc
    return B


def _project_out(Z, L):
    if L.shape[1] == 0:
        return Z
    for _ in range(2):
        Z = Z - L @ (L.T @ Z)
    return Z


def _svqb_pass(Z):
    if Z.shape[1] == 0:
        return Z[:, :0]
    G = _sym(Z.T @ Z)
    d = 1 / np.sqrt(np.maximum(np.diag(G), np.finfo(float).tiny))
    lam, U = np.linalg.eigh(d[:, None] * G * d[None, :])
    top = lam.max()
    keep = np.nonzero(lam > SVQB_CUTOFF * top)[0] if top > 0 else np.array([], dtype=int)
    if len(keep) == 0:
        return Z[:, :0]
    M = (d[:, None] * U[:, keep]) / np.sqrt(lam[keep])[None, :]
    return Z @ M


def _svqb(Z, L, rng):
    """src/chebyshev.jl:88-116."""
    N, na = Z.shape
    Z = _project_out(Z, L)
    W = _svqb_pass(_svqb_pass(Z))
    refills = 0
    while W.shape[1] < na:
        refills += 1
        if refills > 10:
            raise RuntimeError("ChebyshevFilter: SVQB could not refill the dropped directions")
        r = na - W.shape[1]
        Rr = rng.standard_normal((N, r))
        before = colnorms(Rr)
        Rr = _project_out(_project_out(Rr, L), W)
        after = colnorms(Rr)
        room = after > math.sqrt(EPS) * before
        Rr = Rr * room[None, :]
        Rr = _normalize_columns(Rr)
        S = _svqb_pass(Rr)
        if S.shape[1] == 0:
            continue
        S = _project_out(S, W)
        W = np.hstack([W, _svqb_pass(S)])
    return _project_out(W, L)


def _cholqr(Z, L):
    """src/chebyshev.jl:119-131."""
    Z = _project_out(Z, L)
    src = Z
    for _ in range(2):
        G = _sym(src.T @ src)
        try:
            U = np.linalg.cholesky(G).T
        except np.linalg.LinAlgError:
            raise RuntimeError("ChebyshevFilter: Cholesky-QR failed, the filtered block is numerically rank deficient")
        src = src @ np.linalg.inv(U)
    return _project_out(src, L)


def _chebyshev_degree(degree, t1, lcut, lmax):
    x = abs((t1 - (lmax + lcut) / 2) / ((lmax - lcut) / 2))
    if not x > 1:
        return degree
    cap = math.acosh(1 / math.sqrt(EPS)) / math.acosh(x)
    return degree if cap >= degree else max(int(math.floor(cap)), 1)


def _log_gain(t, lcut, lmax):
    x = abs((t - (lmax + lcut) / 2) / ((lmax - lcut) / 2))
    return math.acosh(x) if x > 1 else 0.0


def _counted_guards(theta, m, g, lcut, lmax, deg):
    if not (deg > 0 and math.isfinite(lcut)):
        return g
    ref = _log_gain(np.partition(theta, m - 1)[m - 1], lcut, lmax)
    if not ref > 0:
        return g
    k = 0
    for j in range(m, m + g):
        if _log_gain(theta[j], lcut, lmax) < GUARD_GAIN_FRACTION * ref:
            break
        k += 1
    return k


def _chebyshev_done(theta, nlock, m, need):
    if nlock < need:
        return False
    if nlock == len(theta):
        return True
    return theta[nlock] >= np.partition(theta[:nlock], m - 1)[m - 1]


def _admixed_seed(P):
    X = np.array(P, dtype=np.float64, copy=True)
    rng = _rng(0x4346)
    for j in range(X.shape[1]):
        r = rng.standard_normal(X.shape[0])
        X[:, j] += (SEED_ADMIXTURE * np.linalg.norm(X[:, j]) / np.linalg.norm(r)) * r
    return X


def _rayleigh_ritz(W, HW):
    th, Q = np.linalg.eigh(_sym(W.T @ HW))
    return th, W @ Q, HW @ Q


def chebyshev_solve(s, H, m, callback=None):
    """solve(::ChebyshevFilter, H, m) (src/chebyshev.jl:310-406).  Returns (E, V, info)."""
    N = H.N
    if m < 1 or m > N:
        raise ValueError("ChebyshevFilter: bad m")
    nb = min(m + s.extra, N)
    rng = _rng(0xC4EB)
    hbound = H.gershgorin_bound()
    lmax = hbound if s.bound == "gershgorin" else float(s.bound)
    X0 = _admixed_seed(H.product_seed(nb)) if s.seed == "product" else rng.standard_normal((N, nb))
    g = max(min(min(s.extra - 1, CHEBYSHEV_GUARDS), nb - 1 - m), 0)
    orth = (lambda Z, L: _svqb(Z, L, rng)) if s.ortho == "svqb" else _cholqr
    W = orth(_normalize_columns(X0.copy()), np.zeros((N, 0)))
    theta, X, HX = _rayleigh_ritz(W, H.matvec(W))
    nmv = nb
    _check_bound(theta, lmax)
    res = np.full(nb, np.inf)
    nlock, it, lcut, deg = 0, 0, float("nan"), 0
    while True:
        act = slice(nlock, nb)
        res[act] = colnorms(HX[:, act] - X[:, act] * theta[None, act])
        filtered = it >= 1 or nb == N
        floor = residual_floor(hbound, theta.min())
        while filtered and nlock < nb and res[nlock] <= LOCK_FRACTION * max(s.tol, floor):
            nlock += 1
        if callback is not None:
            callback(dict(iteration=it, lam=theta.copy(), residuals=res.copy(), n_locked=nlock, lcut=lcut, deg=deg))
        need = m + _counted_guards(theta, m, g, lcut, lmax, deg)
        if _chebyshev_done(theta, nlock, m, need):
            break
        if it >= s.maxiter:
            raise RuntimeError(f"ChebyshevFilter: within maxiter = {s.maxiter} iterations only {nlock} converged")
        it += 1
        act = slice(nlock, nb)
        lcut = theta[nb - 1]
        if not lcut < lmax:
            raise RuntimeError("ChebyshevFilter: the block's largest Ritz value reaches lambda_max")
        deg = _chebyshev_degree(s.degree, theta.min(), lcut, lmax)
        Z = chebyshev_filter(H, X[:, act], lcut, lmax, deg, s.rescale_every)
        nmv += deg * (nb - nlock)
        if not np.all(np.isfinite(Z)):
            raise RuntimeError("ChebyshevFilter: the filtered block is not finite")
        Z = _normalize_columns(Z)
        Wv = orth(Z, X[:, :nlock])
        HZ = H.matvec(Wv)
        nmv += Wv.shape[1]
        th, Xa, HXa = _rayleigh_ritz(Wv, HZ)
        X[:, act], HX[:, act], theta[act] = Xa, HXa, th
        _check_bound(theta[act], lmax)
    idx = np.argsort(theta[:nlock], kind="stable")[:m]
    E, V = theta[idx], X[:, idx]
    worst, jw = worst_true_residual(H, E, V)
    floor = residual_floor(hbound, E[0])
    if not worst <= max(s.tol, floor):
        raise RuntimeError(f"ChebyshevFilter: the true residual {worst} of pair {jw} exceeds the threshold")
    return E, V, dict(iters=it, n_matvec=nmv, worst=worst)


def _check_bound(theta, lmax):
    slack = math.sqrt(EPS) * max(abs(lmax), 1.0)
    if theta.max() > lmax + slack:
        raise RuntimeError("ChebyshevFilter: a Ritz value exceeds the upper end of the filter interval")


# ---------------------------------------------------------------------------------------------
# Lanczos (src/solvers.jl:85-106), cross-checked through ARPACK


def lanczos_solve(H, m, tol=1e-10, krylovdim=0, maxiter=1000):
    from scipy.sparse.linalg import LinearOperator, eigsh
    N = H.N
    if m < 1 or m > N:
        raise ValueError("Lanczos: bad m")
    op = LinearOperator((N, N), matvec=lambda v: H.matvec(v), dtype=H.dtype)
    ncv = min(N, max(2 * m + 10, krylovdim))
    w, V = eigsh(op, k=m, which="SA", tol=tol, ncv=ncv, maxiter=maxiter * N)
    p = np.argsort(w)
    return w[p], V[:, p]
