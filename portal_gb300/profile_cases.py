"""Small fixed workloads for profiling single kernels with ncu.

    python -m portal_gb300.profile_cases mlp_forward   # k_gemm_tc: 3 predicts of
                                                       # 65,536 rows through 8 -> 256 x 3 -> 40
    python -m portal_gb300.profile_cases image         # k_image: 2 images, 257 x 257 pixels
                                                       # x 129 channels of a 32,768-point sphere

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


def image(points: int = 32768, im_pix: int = 128, nvel: int = 64, reps: int = 2):
    """The Stokes image of the benchmark sphere's recipe (seed 1, 10 levels)
    on fewer points, line 1-0 at 45 degrees, from the cloud's own
    populations (the image kernels need no converged solution)."""
    import portal_gb300 as pg
    from portal_gb300 import synth
    cloud, mol, rc = synth.config_cloud("sphere262k", n_points=points)
    g = np.sqrt(2.0 * mol.j_lev + 1.0)
    pp = np.zeros((cloud.node_num, 2 * mol.nlev))
    pp[:, 0::2] = cloud.lev_p / np.maximum(cloud.lev_p.sum(axis=1, keepdims=True), 1e-300) / g
    pp[:, 1::2] = 1e-3 * pp[:, 0::2]
    with pg.Context(0) as ctx:
        ctx.set_molecule(mol)
        ctx.set_cloud(cloud)
        for _ in range(reps):
            # n_depth_rt 1024: 0.6 GB of march scratch instead of 6 GB
            cube, st = ctx.image([1], [2], 0.78539816339, 0.0, nvel, 50.0, 0.0, im_pix, 0.7, pol_pops=pp,
                                 quantities=4, n_depth_rt=1024)
        kt = ctx.kernel_times()
    print("image ok", int(st.sum()), float(np.nanmax(cube[0])), {k: v for k, v in kt.items() if v[1]})


CASES = {"mlp_forward": mlp_forward, "image": image}

if __name__ == "__main__":
    name = sys.argv[1] if len(sys.argv) > 1 else "mlp_forward"
    CASES[name]()
