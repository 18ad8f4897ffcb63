"""Small fixed workloads for profiling single kernels with ncu.

    python -m portal_gb300.profile_cases mlp_forward   # k_gemm_tc: 3 predicts of
                                                       # 65,536 rows through 8 -> 256 x 3 -> 40

Each case is seeded and finishes in seconds, so a capture of a few launches
ends by itself.
"""
from __future__ import annotations

import sys

import numpy as np


def mlp_forward(rows: int = 65536, reps: int = 3):
    import portal_gb300 as pg
    X = np.random.default_rng(0).normal(size=(rows, 8)).astype(np.float32)
    with pg.MLP(8, 256, 3, 40, seed=1) as m:
        for _ in range(reps):
            Y = m.predict(X)
    print("mlp_forward ok", float(np.abs(Y).mean()))


CASES = {"mlp_forward": mlp_forward}

if __name__ == "__main__":
    name = sys.argv[1] if len(sys.argv) > 1 else "mlp_forward"
    CASES[name]()
