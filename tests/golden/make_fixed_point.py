"""Generate the FP64 fixed point of the iterated node loop (run from the repo
root: ``python tests/golden/make_fixed_point.py``), a fixture for the GPU
test of the Lambda iteration's limits (tests/test_accel.py).

The oracle (FP64 restatement of inverse_rt.f90 and get_rhovec, the node loop
of main_para.f90:210-257) is iterated like portal_lambda_iterate's plain
passes -- n_J = n_mol sqrt(2J+1) rho^0_0 between passes -- with the numpy Ng
step of oracle/accel.py every fourth pass, until a pass changes rho^0_0 by
less than 1e-13 (relative, over nodes and levels).  The case is a 1,024-point
turbulent cube (seed 300, grid 32) with a 10-level rotor, 8x8 directions,
17 channels, kmax 2.  The fixture holds the cloud itself (positions,
fields, neighbour lists: no triangulation on the machine that reads it),
the run configuration and the fixed point's pol_pops.
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

OUT = os.path.join(HERE, "fixed_point_cube1k.npz")
CASE = dict(n_points=1024, seed=300, grid=32, nlev=10, nth=8, nph=8, nvel=8, kmax=2, gauge_seed=4)


def case_cloud():
    from portal_gb300 import synth
    mol = synth.linear_rotor(CASE["nlev"])
    cloud = synth.turbulent_cube(CASE["n_points"], CASE["seed"], mol, grid=CASE["grid"])
    rc = synth.RunConfig(nth=CASE["nth"], nph=CASE["nph"], nvel=CASE["nvel"], kmax=CASE["kmax"],
                         gvec=synth.gauge_vector(CASE["gauge_seed"]))
    return cloud, mol, rc


def oracle_fixed_point(cloud, mol, rc, tol=1e-13, max_passes=2000, verbose=True):
    import oracle
    from oracle.accel import ng_populations
    P = oracle.OracleProblem(cloud, mol)
    n_mol = cloud.lev_p.sum(axis=1)
    g = np.sqrt(2 * mol.j_lev + 1.0)
    hist, t0 = [], time.time()
    for it in range(max_passes):
        J0, J2, _, _, nf = P.radiation_field(rc)
        assert nf == 0
        pp, _, _ = P.solve_se(rc.kmax, J0, J2)
        rho = pp[:, 0::2]
        old = P.lev_p / (n_mol[:, None] * g[None, :])
        res = float(np.max(np.abs(rho - old) / np.maximum(np.abs(rho), 1e-300)))
        if verbose and it % 10 == 0:
            print("pass %d change %.3e (%.0f s)" % (it, res, time.time() - t0), flush=True)
        if res < tol:
            return pp, it + 1, res
        hist.append(rho.copy())
        if len(hist) >= 4 and it % 4 == 3:
            rho, _ = ng_populations(hist[-4], hist[-3], hist[-2], hist[-1], g)
            hist.append(rho.copy())
        P.lev_p[:] = n_mol[:, None] * g[None, :] * rho
    raise RuntimeError("no fixed point to %g in %d passes" % (tol, max_passes))


def main():
    cloud, mol, rc = case_cloud()
    pp, passes, res = oracle_fixed_point(cloud, mol, rc)
    np.savez_compressed(
        OUT, xyz=cloud.xyz, vel=cloud.vel, b_all=cloud.b_all, t_kin=cloud.t_kin, t_dust=cloud.t_dust,
        dust_p=cloud.dust_p, h2_dens=cloud.h2_dens, ab_all=cloud.ab_all, lev_p=cloud.lev_p, bvec=cloud.bvec,
        nb_off=cloud.nb_off, nb_idx=cloud.nb_idx, tx=cloud.tx, bulk_node_num=cloud.bulk_node_num,
        case=np.array([CASE[k] for k in ("n_points", "seed", "grid", "nlev", "nth", "nph", "nvel", "kmax",
                                         "gauge_seed")]),
        gvec=np.asarray(rc.gvec), pol_pops=pp, passes=passes, last_change=res)
    print("wrote %s: %d passes, last change %.2e" % (OUT, passes, res))


if __name__ == "__main__":
    main()
