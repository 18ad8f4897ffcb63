"""The warm start's MLP: the FP64 oracle pinned by finite differences (CPU),
the library's BF16 forward / backward kernels against the oracle, training
and inference (GPU)."""
import numpy as np
import pytest

from oracle import mlp as om

SHAPE = (8, 64, 3, 40)   # n_in, width, depth, n_out: the warm start's layout at a test width


def _params(shapes, seed):
    rng = np.random.default_rng(seed)
    parts = []
    for fo, fi in shapes:
        parts.append(rng.uniform(-1, 1, fo * fi) * np.sqrt(6.0 / fi))
        parts.append(rng.normal(0, 0.1, fo))
    return np.concatenate(parts).astype(np.float32)


def test_bf16_rounding_known_values():
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: ties to even -> 1
    # 1 + 3*2^-8 is a tie between 1 + 2^-7 and 1 + 2^-6: ties to even -> 1 + 2^-6
    vals = np.array([1.0, 1 + 2 ** -8, 1 + 3 * 2 ** -8, 1 + 2 ** -8 + 2 ** -20, -2.5, 3.0e38], dtype=np.float32)
    want = np.array([1.0, 1.0, 1 + 2 ** -6, 1 + 2 ** -7, -2.5, 1.765625 * 2.0 ** 127])
    got = om.bf16_round(vals)
    assert np.array_equal(got[:5], want[:5])
    assert got[5] == want[5]


def test_oracle_backprop_matches_finite_differences():
    shapes = om.layer_shapes(5, 16, 2, 3)
    p = _params(shapes, 1).astype(np.float64)
    rng = np.random.default_rng(2)
    X, T = rng.normal(size=(12, 5)), rng.normal(size=(12, 3))
    _, g = om.loss_and_grad(p, shapes, X, T, bf16=False)
    idx = np.random.default_rng(3).choice(p.size, 60, replace=False)
    fd = om.finite_difference(p, shapes, X, T, idx)
    assert np.allclose(g[idx], fd, rtol=1e-6, atol=1e-9)


def test_oracle_bf16_close_to_exact():
    shapes = om.layer_shapes(*SHAPE)
    p = _params(shapes, 4)
    rng = np.random.default_rng(5)
    X, T = rng.normal(size=(64, 8)), rng.normal(size=(64, 40))
    l0, g0 = om.loss_and_grad(p, shapes, X, T, bf16=False)
    l1, g1 = om.loss_and_grad(p, shapes, X, T, bf16=True)
    assert abs(l1 - l0) < 2e-2 * l0
    assert np.linalg.norm(g1 - g0) < 3e-2 * np.linalg.norm(g0)


@pytest.mark.gpu
@pytest.mark.parametrize("B", [64, 200])
def test_gradients_match_oracle(built_lib, B):
    import portal_gb300 as pg

    shapes = om.layer_shapes(*SHAPE)
    p = _params(shapes, 6)
    rng = np.random.default_rng(7 + B)
    X = rng.normal(size=(B, 8)).astype(np.float32)
    T = rng.normal(size=(B, 40)).astype(np.float32)
    with pg.MLP(*SHAPE, seed=1) as m:
        assert m.num_params == p.size
        m.set_params(p)
        loss, g = m.gradients(X, T)
    lref, gref = om.loss_and_grad(p, shapes, X, T, bf16=True)
    _, gex = om.loss_and_grad(p, shapes, X, T, bf16=False)
    # same rounding points: FP32 accumulation vs FP64 and the rare BF16
    # rounding flips of FP32 intermediates are all that differ
    assert abs(loss - lref) <= 1e-5 * lref
    o = 0
    for fo, fi in shapes:
        for n in (fo * fi, fo):
            a, r = g[o:o + n].astype(np.float64), gref[o:o + n]
            scale = np.abs(r).max()
            assert np.abs(a - r).max() <= 2e-3 * scale, (o, n)
            assert np.linalg.norm(a - r) <= 2e-4 * np.linalg.norm(r) + 1e-12, (o, n)
            o += n
    # and against the exact FP64 gradient: the BF16 operand error only
    assert np.linalg.norm(g - gex) <= 3e-2 * np.linalg.norm(gex)


@pytest.mark.gpu
def test_training_fits_and_predict_matches_oracle(built_lib):
    import portal_gb300 as pg

    rng = np.random.default_rng(11)
    M = 8192
    X = rng.uniform(-2, 2, size=(M, 8)).astype(np.float32)
    W = rng.normal(size=(8, 6))
    Y = np.tanh(X @ W * 0.5) + 0.1 * np.sin(3 * X[:, :6])
    Y = (Y * 3 + 10).astype(np.float32)    # raw units away from zero mean / unit scale
    with pg.MLP(8, 64, 3, 6, seed=3) as m:
        losses = m.train(X, Y, epochs=30, batch=256, lr=2e-3, seed=5)
        assert losses[-1] < 0.05 * losses[0]
        assert losses[-1] < 0.02
        Xt = rng.uniform(-2, 2, size=(3000, 8)).astype(np.float32)
        Yp = m.predict(Xt)
        p, st = m.get_params()
    # standardisation statistics of the training set
    assert np.allclose(st, om.standardise(X, Y), rtol=1e-5, atol=1e-6)
    shapes = om.layer_shapes(8, 64, 3, 6)
    Yo = om.predict(p, st, shapes, Xt, bf16=True)
    assert np.abs(Yp - Yo).max() <= 2e-3 * np.abs(Yo).max()
