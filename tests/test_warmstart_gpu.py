"""The learned warm start on the two-transmon circuit (flat 61 x 61 = 3,721 states, m = 12).

A network trained by the library's own kernels on the plain solver's eigenvectors proposes the
initial LOBPCG block for held-out theta.  Checked: the warm-started solves reach the same
eigenvalues as random starts (1e-9 relative), need fewer iterations on average (what the network
gains), and an untrained network's block is judged after 3 iterations and replaced by a random
start without harming the result (the plain method stays the fallback and the reference).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def trained(cuda):
    from kfgpu import warmstart as W
    train = W.sample_thetas(512, seed=11)
    Vs, _ = W.label(train)
    POD = W.pod_basis(Vs, k=128)
    ws = W.WarmStart(POD, 12, hidden=256, seed=1)
    losses = ws.fit(train, W.targets(Vs, POD), epochs=300, batch=128, lr=1e-3)
    return W, ws, losses


def test_network_trains(trained):
    W, ws, losses = trained
    assert losses[-1] < 0.2 * losses[0]


def test_warm_start_beats_random_start(trained):
    W, ws, _ = trained
    rows = W.evaluate(ws, W.sample_thetas(12, seed=99))
    for r in rows:
        assert r["max_dE"] < 1e-9 * np.max(np.abs(r["E"]))
    warm = np.mean([r["warm_iters"] for r in rows])
    rand = np.mean([r["random_iters"] for r in rows])
    assert warm < rand, (warm, rand)


def test_warm_start_against_the_product_seed(trained):
    """The solver's default start, the product seed, is the other baseline: on this weakly coupled
    circuit its product states are already close to the eigenvectors (3-5 iterations), closer
    than the network's block, so the learned start does not beat it; pinned here: the same
    eigenvalues, and the learned start within one and a half iterations of the product seed on
    average."""
    W, ws, _ = trained
    rows = W.evaluate(ws, W.sample_thetas(24, seed=98), product_arm=True)
    warm = np.mean([r["warm_iters"] for r in rows])
    prod = np.mean([r["product_iters"] for r in rows])
    assert warm <= prod + 1.5, (warm, prod)
    for r in rows:
        assert np.max(np.abs(r["E_warm"] - r["E_product"])) < 1e-9 * np.max(np.abs(r["E"]))


def test_untrained_network_is_judged_and_replaced(cuda):
    from kfgpu import warmstart as W
    th = W.sample_thetas(4, seed=5)
    rng = np.random.default_rng(0)
    POD = np.linalg.qr(rng.standard_normal((3721, 128)))[0]
    ws = W.WarmStart(POD, 12, seed=3)                       # random weights: a poor block
    ws.net.set_scaling(np.zeros(7), np.ones(7), np.zeros(128 * 12), np.ones(128 * 12))
    rows = W.evaluate(ws, th, fallback_resid=1e-6)
    assert all(r["fell_back"] == 1 for r in rows)
    for r in rows:
        assert r["max_dE"] < 1e-9 * np.max(np.abs(r["E"]))
