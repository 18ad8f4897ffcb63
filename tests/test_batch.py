"""Many models in one launch: the batch's results equal each model's own
node loop bit for bit (GPU)."""
import numpy as np
import pytest

from portal_gb300 import synth


def _models():
    out = []
    for i, (n, nlev) in enumerate([(3000, 4), (1500, 7), (5000, 5), (800, 9), (2200, 3)]):
        mol = synth.linear_rotor(nlev)
        cl = synth.power_law_sphere(n, 40 + i, mol, density_exp=1.0 + 0.2 * i, n0_cm3=10.0 ** (4 + 0.6 * i),
                                    b_dir=(0.6, 0.0, 0.8))
        out.append((cl, mol))
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("autotune,nvel", [(True, 12), (False, 12), (True, 16)])
def test_batch_matches_single_models(built_lib, autotune, nvel):
    """nvel 12: 25 channels in one padded slot; nvel 16: 33 channels, one
    full slot plus the remainder channel integrated lanes-over-lines."""
    import portal_gb300 as pg

    rc = synth.RunConfig(nth=8, nph=8, nvel=nvel, kmax=2, gvec=synth.gauge_vector(3))
    models = _models()
    ctxs = []
    for cl, mol in models:
        c = pg.Context(0)
        c.set_molecule(mol)
        c.set_cloud(cl)
        ctxs.append(c)
    seg_single, want = 0, []
    for c in ctxs:
        J0, J2, st, nseg = c.radiation_field(rc)
        pp, _ = c.solve_se(rc.kmax)
        want.append((J0, J2, pp))
        seg_single += nseg
    with pg.Batch(0) as b:
        for c in ctxs:
            b.add(c)
        b.prepare(rc, autotune=autotune)
        cfg, tune = b.config()
        assert cfg[0] in (5, 10) and cfg[1] >= 1 and cfg[2] in (2, 4, 8)
        if autotune:
            assert len(tune) >= 4 and (tune[:, 2] > 0).all()
        for use_graph in (True, False, True):
            nseg, ms = b.run(use_graph=use_graph)
            assert nseg == seg_single and ms > 0
            for c, (J0, J2, pp) in zip(ctxs, want):
                gJ0, gJ2, gpp = c.results()
                np.testing.assert_array_equal(gJ0, J0)
                np.testing.assert_array_equal(gJ2, J2)
                np.testing.assert_array_equal(gpp, pp)
    for c in ctxs:
        c.close()
