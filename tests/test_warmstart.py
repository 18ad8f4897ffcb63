"""The learned warm start: target / start-population conversions (CPU), and
what the trained network gains over the iteration without it (GPU)."""
import time

import numpy as np
import pytest

from portal_gb300 import synth
from portal_gb300.warmstart import start_pops, targets


def test_targets_and_start_pops_round_trip():
    rng = np.random.default_rng(0)
    j = np.arange(6)
    x = rng.dirichlet(np.ones(6), size=50)
    rho0 = x / np.sqrt(2 * j + 1)
    pp = np.zeros((50, 12))
    pp[:, 0::2] = rho0
    pp[:, 1::2] = rho0 * rng.uniform(-0.05, 0.05, size=(50, 6))
    Y = targets(pp, j)
    back = start_pops(Y, j)
    np.testing.assert_allclose(back, pp, rtol=1e-5, atol=1e-12)
    # the normalisation sum sqrt(2J+1) rho^0_0 = 1 of the SE solution
    np.testing.assert_allclose((back[:, 0::2] * np.sqrt(2 * j + 1)).sum(1), 1.0, rtol=1e-12)


@pytest.mark.gpu
def test_trained_network_reduces_passes_to_the_same_fixed_point(built_lib):
    """Train on five seeded turbulent cubes (8,192 points, 10-level rotor),
    then iterate a held-out cube from LTE and from the network's prediction,
    plain and accelerated (local operator + Ng)."""
    import portal_gb300 as pg
    from portal_gb300.warmstart import WarmStart

    mol = synth.linear_rotor(10)
    rc = synth.RunConfig(nth=12, nph=12, nvel=16, kmax=2, gvec=synth.gauge_vector(4))
    with WarmStart(mol.j_lev, seed=1) as ws, pg.Context(0) as ctx:
        ctx.set_molecule(mol)
        Xs, Ys = [], []
        for i in range(5):
            cl = synth.turbulent_cube(8192, 200 + i, mol, grid=32)
            ctx.set_cloud(cl)
            X, Y, _ = ws.collect(ctx, rc, cl.ab_all, cl.bulk_node_num)
            Xs.append(X)
            Ys.append(Y)
        losses = ws.fit(np.concatenate(Xs), np.concatenate(Ys), epochs=60)
        assert losses[-1] < 0.8 * losses[0]
        cl = synth.turbulent_cube(8192, 300, mol, grid=32)
        runs = {}
        for name, warm, ng, lo in (("plain", False, 0, False), ("warm", True, 0, False),
                                   ("acc", False, 4, True), ("warm+acc", True, 4, True)):
            ctx.set_cloud(cl)
            t0 = time.perf_counter()
            if warm:
                pp, _, n, res, _ = ws.solve(ctx, rc, tol=1e-6, max_iter=2000, ng_period=ng, local_operator=lo)
            else:
                pp, _, n, res, _ = ctx.lambda_iterate(rc, tol=1e-6, max_iter=2000, ng_period=ng,
                                                      local_operator=lo)
            runs[name] = (n, time.perf_counter() - t0, pp, res)
    for name, (n, _, _, res) in runs.items():
        assert res[-1] < 1e-6, name
    ref = runs["plain"][2][:, 0::2]
    for name in ("warm", "acc", "warm+acc"):
        got = runs[name][2][:, 0::2]
        assert np.abs(got - ref).max() <= 5e-5 * np.abs(ref).max(), name
    # the network's gain: fewer passes from its prediction than from LTE,
    # with and without the accelerations (the feature pass counts as one)
    assert runs["warm"][0] + 1 < 0.85 * runs["plain"][0]
    assert runs["warm+acc"][0] + 1 <= runs["acc"][0]
    # the accelerated, warm-started iteration against the plain method
    assert runs["plain"][1] > 3.0 * runs["warm+acc"][1]
