"""Learned warm start of the Lambda iteration (no reference counterpart).

The reference makes one pass of the node loop from LIME's populations.  The
Lambda iteration (``Context.lambda_iterate``) repeats that pass to
convergence; this module starts it closer to the answer.  A small MLP
(``portal_gb300.MLP``, trained and evaluated by the library's own BF16
kernels) maps eight local features of a node -- the cloud's conditions and
the first radiation field, ``Context.warmstart_features`` -- to that node's
converged level populations and alignment.  The iteration then starts from
the prediction; it alone decides convergence, so the fixed point it stops at
is the one it reaches without the network.

Targets per node (2 nlev values): log10 x_J, the fractional population of
level J (x_J = sqrt(2J+1) rho^0_0, floored at 1e-30), then 100 rho^2_0 /
rho^0_0 per level.  The start populations are the normalised 10^prediction,
made safe first: every predicted value is clipped to the range of its
training targets, and the populations per statistical weight are made
non-increasing along the level list (LAMDA lists levels by energy), so a
start is never a maser.  A start with an inversion amplifies along a ray
without bound (negative opacity) and leaves non-finite radiation fields; a
network evaluated outside its training data predicts such starts.  Neither
rule moves the fixed point, only the first pass.
"""
from __future__ import annotations

import numpy as np

from . import MLP

N_FEATURES = 8
X_FLOOR = 1e-30


def targets(pol_pops, j_lev) -> np.ndarray:
    """(N, 2 nlev) training targets from pol_pops (N, 2 nlev)."""
    pp = np.asarray(pol_pops, dtype=np.float64)
    sq = np.sqrt(2.0 * np.asarray(j_lev) + 1.0)
    rho0 = pp[:, 0::2]
    lx = np.log10(np.maximum(rho0 * sq[None, :], X_FLOOR))
    safe = np.where(rho0 != 0.0, rho0, 1.0)
    al = np.where(rho0 != 0.0, 100.0 * pp[:, 1::2] / safe, 0.0)
    return np.concatenate([lx, al], axis=1).astype(np.float32)


def start_pops(Y, j_lev, y_range=None) -> np.ndarray:
    """pol_pops (N, 2 nlev) from predicted targets: each column clipped to
    y_range (lo, hi) when given, x_J / (2J+1) made non-increasing along the
    levels, x_J normalised to sum 1, rho^0_0 = x_J / sqrt(2J+1), rho^2_0 from
    the predicted ratio."""
    Y = np.asarray(Y, dtype=np.float64)
    if y_range is not None:
        Y = np.clip(Y, y_range[0], y_range[1])
    nlev = Y.shape[1] // 2
    g = 2.0 * np.asarray(j_lev) + 1.0
    sq = np.sqrt(g)
    lx = np.clip(Y[:, :nlev], np.log10(X_FLOOR), 0.0)
    # no inversion: log10(x_J / g_J) non-increasing along the level list
    lx = np.minimum.accumulate(lx - np.log10(g)[None, :], axis=1) + np.log10(g)[None, :]
    x = 10.0 ** lx
    x /= x.sum(axis=1, keepdims=True)
    pp = np.zeros((Y.shape[0], 2 * nlev))
    pp[:, 0::2] = x / sq[None, :]
    pp[:, 1::2] = pp[:, 0::2] * Y[:, nlev:] / 100.0
    return pp


class WarmStart:
    """The network and the pipeline around it.

    ``collect`` turns one cloud into training rows (features after the first
    radiation field, converged targets), ``fit`` trains on the rows of many
    clouds, ``solve`` runs a warm-started Lambda iteration."""

    def __init__(self, j_lev, width: int = 256, depth: int = 3, seed: int = 0, device: int = 0):
        self.j_lev = np.asarray(j_lev, dtype=np.int64)
        self.nlev = len(self.j_lev)
        self.mlp = MLP(N_FEATURES, width, depth, 2 * self.nlev, seed=seed, device=device)
        self.y_range = None  # per-target (lo, hi) of the training rows

    def close(self):
        self.mlp.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @staticmethod
    def _live(ctx_cloud_ab, bulk):
        return np.asarray(ctx_cloud_ab[:bulk]) > 0.0

    def collect(self, ctx, rc, ab, bulk, *, tol=1e-6, max_iter=1000, ng_period=4, local_operator=True):
        """Training rows of the context's cloud, which must hold the starting
        populations: (features, targets, passes) of its live bulk nodes
        (ab > 0).  The targets come from an (accelerated) iteration to tol."""
        ctx.radiation_field(rc, fetch=False)
        X = ctx.warmstart_features()
        pp, _, n, res, _ = ctx.lambda_iterate(rc, tol=tol, max_iter=max_iter, ng_period=ng_period,
                                              local_operator=local_operator)
        if not res[-1] < tol:
            raise RuntimeError(f"training cloud did not converge in {max_iter} passes")
        live = self._live(ab, bulk)
        Y = targets(pp, self.j_lev)
        keep = live & np.all(np.isfinite(X[:bulk]), axis=1) & np.all(np.isfinite(Y[:bulk]), axis=1)
        return X[:bulk][keep], Y[:bulk][keep], n

    def fit(self, X, Y, epochs: int = 60, batch: int = 512, lr: float = 1e-3, seed: int = 0):
        """Train on stacked rows; returns the mean standardised loss per epoch."""
        Y = np.asarray(Y, dtype=np.float32)
        self.y_range = (Y.min(axis=0).astype(np.float64), Y.max(axis=0).astype(np.float64))
        return self.mlp.train(X, Y, epochs=epochs, batch=batch, lr=lr, seed=seed)

    def start(self, ctx, rc) -> np.ndarray:
        """Predicted start populations (N, 2 nlev) for the context's cloud
        (one radiation-field pass over its current populations)."""
        ctx.radiation_field(rc, fetch=False)
        X = ctx.warmstart_features()
        X = np.where(np.isfinite(X), X, 0.0).astype(np.float32)
        return start_pops(self.mlp.predict(X), self.j_lev, self.y_range)

    def solve(self, ctx, rc, *, tol=1e-6, max_iter=1000, ng_period=0, local_operator=False, fetch=True):
        """Warm-started Lambda iteration; returns lambda_iterate's tuple.
        The feature pass is one extra radiation field (not counted in the
        returned passes)."""
        sp = self.start(ctx, rc)
        return ctx.lambda_iterate(rc, tol=tol, max_iter=max_iter, start_pops=sp, fetch=fetch,
                                  ng_period=ng_period, local_operator=local_operator)

    def save(self, path: str):
        p, st = self.mlp.get_params()
        lo, hi = self.y_range if self.y_range is not None else (np.full(2 * self.nlev, -np.inf),
                                                                np.full(2 * self.nlev, np.inf))
        np.savez(path, params=p, stats=st, j_lev=self.j_lev, y_lo=lo, y_hi=hi,
                 shape=np.array([N_FEATURES, self.mlp.width, self.mlp.depth, 2 * self.nlev]))

    @classmethod
    def load(cls, path: str, device: int = 0) -> "WarmStart":
        z = np.load(path)
        n_in, width, depth, n_out = (int(v) for v in z["shape"])
        ws = cls(z["j_lev"], width=width, depth=depth, device=device)
        ws.mlp.set_params(z["params"], z["stats"])
        if "y_lo" in z and np.isfinite(z["y_lo"]).all():
            ws.y_range = (z["y_lo"], z["y_hi"])
        return ws
