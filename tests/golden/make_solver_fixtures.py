"""Generate the eigenvalue fixtures of the full-size workloads with the CPU oracle.

  leaf3     the three-mode leaf (41 x 256 x 64 = 671,744 states), lowest 12 eigenvalues of the
            seeded theta draws the benchmark cycles through (numpy default_rng(20261205), 64 draws):
            the oracle's FP64 LOBPCG (oracle/solvers.py, C restatement of mul!, separable
            preconditioner, product seed) to ||H x - lambda x|| <= 1e-10 ||H||.
  xcheck    for a few of those draws, an independent solve: SciPy's LOBPCG from a random 20-column
            start with the same operator and preconditioner, to 1e-9 ||H||; its lowest 12 are
            recorded beside the oracle's so the fixture shows two unrelated iterations agree (no
            state skipped by the product seed or by locking).
  dense48   the dense parent (48^3 = 110,592 states, three dense pairwise port couplings, drawn
            from default_rng(20261210)), lowest 30 eigenvalues by SciPy's ARPACK Lanczos (eigsh),
            cross-checked by the oracle's LOBPCG (per-Ritz Jacobi).

  batch     the batched sweep (numpy default_rng(20261207)): 512 fluxonium leaves with
            n ~ U{200..1600} points plus 64 chains of 2-4 leaves, drawn in the benchmark's order; the
            lowest 10 eigenvalues of every leaf by LAPACK on the oracle's matrix, and the lowest 20
            of every chain parent (diag of the leaves' energies + g n_i n_{i+1} in the leaves' kept
            bases, built from the oracle's own leaf eigenvectors) by LAPACK or ARPACK.
  warm      the learned warm start's first 32 held-out theta (two transmons on the flat 61 x 61
            space, seed 20261209 draws of the parameter box), lowest 12 by LAPACK on the oracle's
            operator built from the reference's two-transmon spec.

Usage (results are merged into the JSON files next to this script, draw by draw):
  python tests/golden/make_solver_fixtures.py leaf3 --draws 5-24
  python tests/golden/make_solver_fixtures.py xcheck --draws 5,6
  python tests/golden/make_solver_fixtures.py dense48
Set OMP_NUM_THREADS to bound the threads the C oracle uses.
"""
from __future__ import annotations

import os

os.environ.setdefault("OMP_WAIT_POLICY", "PASSIVE")      # the C oracle's threads and BLAS's share the cores
os.environ.setdefault("OPENBLAS_THREAD_TIMEOUT", "4")

import argparse
import json
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import capply, circuits as oc, solvers as osol  # noqa: E402

LEAF3 = os.path.join(HERE, "leaf3_eigs.json")
DENSE48 = os.path.join(HERE, "dense48_eigs.json")
LEAF3_SEED = 20261205
LEAF3_DRAWS = 64
DENSE48_SEED = 20261210
BATCH = os.path.join(HERE, "batch_eigs.json")
BATCH_SEED = 20261207
WARM = os.path.join(HERE, "warm_eigs.json")
WARM_SEED = 20261209


def _load(path):
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f)
    return {}


def _save(path, d):
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(d, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def leaf3_thetas():
    rng = np.random.default_rng(LEAF3_SEED)
    return [oc.three_mode_theta(rng) for _ in range(LEAF3_DRAWS)]


def _resid(CA, E, V):
    V = np.asfortranarray(V)
    R = CA.matvec(V) - V * E[None, :]
    return np.sqrt(np.sum(R ** 2, axis=0))


def run_leaf3(draws, xcheck=False):
    out = _load(LEAF3)
    out.setdefault("seed", LEAF3_SEED)
    out.setdefault("workload", "three-mode leaf 41x256x64 (N=671,744), lowest 12")
    out.setdefault("draws", {})
    out.setdefault("xcheck", {})
    ths = leaf3_thetas()
    for d in draws:
        th = ths[d]
        H = oc.three_mode_operator(th)
        CA = capply.CApply(H)
        hb = H.gershgorin_bound()
        t0 = time.perf_counter()
        if not xcheck:
            E, V, r = osol.lobpcg_solve(osol.LOBPCG(tol=1e-10 * hb, preconditioner="separable", maxiter=2000), H, 12)
            res = _resid(CA, E, V)
            out["draws"][str(d)] = {"theta": th, "E": [float(x) for x in E], "hnorm": hb,
                                    "max_resid_rel": float(res.max() / hb), "iterations": int(r["iters"]),
                                    "method": "oracle LOBPCG, separable preconditioner, product seed, FP64, "
                                              "tol 1e-10 ||H||", "seconds": time.perf_counter() - t0}
            print(f"leaf3 draw {d}: {r['iters']} it, max res {res.max() / hb:.2e} ||H||, "
                  f"{time.perf_counter() - t0:.0f} s", flush=True)
        else:
            import scipy.sparse.linalg as sla
            N = H.N
            sep = osol.SeparablePrecond(H, 0.01, hb)
            shift = float(np.min(sep.S))

            def mm(X):
                return CA.matvec(np.asfortranarray(X.reshape(N, -1)))

            def prec(X):
                X = np.asfortranarray(X.reshape(N, -1))
                return sep(X, np.full(X.shape[1], shift))

            A = sla.LinearOperator((N, N), matvec=lambda x: mm(x).reshape(x.shape), matmat=mm, dtype=np.float64)
            M = sla.LinearOperator((N, N), matvec=lambda x: prec(x).reshape(x.shape), matmat=prec, dtype=np.float64)
            X0 = np.random.default_rng(1000 + d).standard_normal((N, 20))
            w, V = sla.lobpcg(A, X0, M=M, tol=1e-9 * hb, maxiter=600, largest=False)
            o = np.argsort(w)
            w, V = w[o][:12], V[:, o][:, :12]
            res = _resid(CA, w, V)
            out["xcheck"][str(d)] = {"E": [float(x) for x in w], "max_resid_rel": float(res.max() / hb),
                                     "method": "scipy.sparse.linalg.lobpcg, random 20-column start, separable "
                                               "preconditioner at a fixed shift, FP64, tol 1e-9 ||H||",
                                     "seconds": time.perf_counter() - t0}
            ref = out["draws"].get(str(d))
            if ref:
                dE = np.max(np.abs(w - np.array(ref["E"])) / np.abs(np.array(ref["E"])))
                out["xcheck"][str(d)]["max_rel_diff_vs_oracle_lobpcg"] = float(dE)
                print(f"xcheck draw {d}: max rel diff {dE:.2e}, max res {res.max() / hb:.2e}", flush=True)
        _save(LEAF3, out)


def run_dense48():
    import scipy.sparse.linalg as sla
    out = _load(DENSE48)
    H = oc.dense_parent_operator(np.random.default_rng(DENSE48_SEED), d=48)
    CA = capply.CApply(H)
    hb = H.gershgorin_bound()
    N = H.N
    t0 = time.perf_counter()
    A = sla.LinearOperator((N, N), matvec=lambda x: CA.matvec(x), dtype=np.float64)
    w, V = sla.eigsh(A, k=30, which="SA", tol=1e-13, ncv=90, v0=np.random.default_rng(7).standard_normal(N))
    o = np.argsort(w)
    w, V = w[o], V[:, o]
    res = _resid(CA, w, V)
    t1 = time.perf_counter()
    E2, V2, r = osol.lobpcg_solve(osol.LOBPCG(tol=1e-10 * hb, guard=2, maxiter=2000), H, 30)
    out.update({"seed": DENSE48_SEED, "workload": "dense parent 48^3 (N=110,592), lowest 30", "hnorm": hb,
                "E": [float(x) for x in w], "max_resid_rel": float(res.max() / hb),
                "method": "scipy.sparse.linalg.eigsh (ARPACK Lanczos, which=SA, tol 1e-13), FP64",
                "seconds": t1 - t0,
                "xcheck": {"E": [float(x) for x in E2], "iterations": int(r["iters"]),
                           "method": "oracle LOBPCG, per-Ritz Jacobi, product seed, FP64, tol 1e-10 ||H||",
                           "max_rel_diff": float(np.max(np.abs(E2 - w) / np.abs(w)))}})
    print(f"dense48: res {res.max() / hb:.2e} ||H||, lobpcg diff {out['xcheck']['max_rel_diff']:.2e}", flush=True)
    _save(DENSE48, out)


def batch_draws():
    """The batched sweep's leaves and chains, drawn in the benchmark's order."""
    rng = np.random.default_rng(BATCH_SEED)
    leaves = []
    for _ in range(512):
        th = oc.fluxonium_theta(rng)
        leaves.append((th, int(rng.integers(200, 1601))))
    chains = []
    for _ in range(64):
        k = int(rng.integers(2, 5))
        chains.append(([(oc.fluxonium_theta(rng), int(rng.integers(200, 1601))) for _ in range(k)],
                       [float(rng.uniform(0.01, 0.1)) for _ in range(k - 1)]))
    return leaves, chains


def run_batch():
    import scipy.sparse.linalg as sla
    from oracle import kfref
    leaves, chains = batch_draws()
    t0 = time.perf_counter()
    allv = leaves + [lf for c, _ in chains for lf in c]
    Es, Vs = [], []
    for th, n in allv:
        w, V = np.linalg.eigh(oc.fluxonium_operator(th, n).to_matrix())
        Es.append(w[:10])
        Vs.append(V[:, :10])
    k0 = len(leaves)
    parents = []
    for c, gs in chains:
        idx = list(range(k0, k0 + len(c)))
        k0 += len(c)
        ports = []
        for i in idx:
            n = allv[i][1]
            A = np.imag(kfref.localop(kfref.PhaseGrid(-5 * np.pi, 5 * np.pi, n, 4), "n").dense())   # n = i A
            ports.append(Vs[i].T @ A @ Vs[i])
        terms = [(1.0, [(a, kfref.DiagonalOp(Es[i]))]) for a, i in enumerate(idx)]
        for a in range(len(c) - 1):
            terms.append((-gs[a], [(a, kfref.DenseOp(ports[a])), (a + 1, kfref.DenseOp(ports[a + 1]))]))
        H = kfref.KronFreeOperator([10] * len(c), terms)
        if H.N <= 1000:
            w = np.linalg.eigvalsh(H.to_matrix())[:20]
        else:
            A = sla.LinearOperator((H.N, H.N), matvec=lambda x: H.matvec(x), dtype=np.float64)
            w = np.sort(sla.eigsh(A, k=20, which="SA", tol=1e-14, ncv=80,
                                  v0=np.random.default_rng(5).standard_normal(H.N))[0])
        parents.append([float(x) for x in w])
    _save(BATCH, {"seed": BATCH_SEED, "workload": "512 fluxonium leaves + 64 chains of 2-4 leaves",
                  "leaf_E": [[float(x) for x in e] for e in Es], "parent_E": parents,
                  "method": "LAPACK eigh on the oracle's leaf matrices; parents by LAPACK (<= 1000 states) or "
                            "ARPACK eigsh (tol 1e-14) on the oracle's parent operator",
                  "seconds": time.perf_counter() - t0})
    print(f"batch: {len(Es)} leaves, {len(parents)} parents, {time.perf_counter() - t0:.0f} s", flush=True)


def run_warm(count=32):
    from oracle import kfref
    sys.path.insert(0, os.path.join(ROOT, "kronfreecircuits.jl_gb300"))
    from kfgpu.warmstart import THETA_RANGES
    with open(os.path.join(HERE, "reference_goldens.json")) as f:
        spec = json.load(f)["specs"]["two_transmons"]
    rng = np.random.default_rng(WARM_SEED)
    ths = [{k: float(rng.uniform(*THETA_RANGES[k])) for k in THETA_RANGES} for _ in range(count)]
    t0 = time.perf_counter()
    out = []
    bases = {"varphi_1": kfref.ChargeBasis(30), "varphi_2": kfref.ChargeBasis(30)}
    for th in ths:
        H = kfref.KronFreeOperator([61, 61], kfref.leaf_terms(spec, th, bases, real=True),
                                   constant=kfref.constant_term(spec, th))
        out.append([float(x) for x in np.linalg.eigvalsh(H.to_matrix())[:12]])
    _save(WARM, {"seed": WARM_SEED, "theta": ths, "E": out,
                 "workload": "two transmons flat 61x61 (N=3,721), the first held-out theta",
                 "method": "LAPACK eigh on the oracle's operator from the reference's spec",
                 "seconds": time.perf_counter() - t0})
    print(f"warm: {count} theta, {time.perf_counter() - t0:.0f} s", flush=True)


def _parse(spec):
    out = []
    for part in spec.split(","):
        if "-" in part:
            a, b = part.split("-")
            out += list(range(int(a), int(b) + 1))
        else:
            out.append(int(part))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("what", choices=["leaf3", "xcheck", "dense48", "batch", "warm"])
    ap.add_argument("--draws", default="5-24")
    a = ap.parse_args()
    if a.what == "dense48":
        run_dense48()
    elif a.what == "batch":
        run_batch()
    elif a.what == "warm":
        run_warm()
    else:
        run_leaf3(_parse(a.draws), xcheck=a.what == "xcheck")


if __name__ == "__main__":
    main()
