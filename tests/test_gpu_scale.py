"""Parity at the sizes the benchmark and the named workloads run, not on
down-scaled stand-ins: the CUDA path over the whole cloud, the FP64 oracle on
a stratified sample of its nodes (the oracle restates main_portal.x's node
loop, inverse_rt.f90:77-134 and main_sub.f90:93-137, and finish_portal.x's
pixel loop, para_finish.f90:352-449, node by node and pixel by pixel, so a
sample is the reference's own result at those nodes).

  sphere262k  262,144-point power-law sphere (seed 1), 10-level rotor, 24x24
              directions, 129 channels, kmax 6: the cloud bench.py times.
              256 nodes spread over radius (the 200 AU core, every radius
              rank, the surface): J^0_0 / J^2_0, segments per node, the SE
              from the same J, the chained populations.
  sphere4k    4,096-point sphere (seed 0), 5-level rotor: the full
              129 x 129 x 65 Stokes IQUV cube at 45 degrees against the
              oracle's image of the same populations, and the image of the
              GPU's own populations against the oracle's chain.
  cube1m      1,048,576-point turbulent cube (seed 4), 20-level rotor, 32x32
              directions, 129 channels, kmax 2: 48 nodes spread over density
              and radius.

Tolerances are those of test_gpu_parity (FP32 ray integration, FP32 LU with
FP64 refinement); each test prints what it measured.
"""
import numpy as np
import pytest

from test_gpu_parity import J0_MAX, J0_MED, J0_P99, J2_MAX, _check_J

pytestmark = pytest.mark.gpu


def _report(name, **vals):
    print("PARITY %s: %s" % (name, " ".join("%s=%.3g" % kv for kv in vals.items())), flush=True)


def _j_errors(J0, J2, oJ0, oJ2):
    r0 = np.abs(J0 - oJ0) / np.abs(oJ0)
    r2 = np.abs(J2 - oJ2) / np.abs(oJ0)
    return dict(j0_max=r0.max(), j0_p99=np.quantile(r0, 0.99), j0_med=np.median(r0), j2_max=r2.max())


def radius_sample(cloud, n_core=8, n_surface=8, n_spread=240, seed=0):
    """0-based bulk node ids: the innermost n_core nodes (inside the 200 AU
    core of the sphere), the outermost n_surface, and n_spread more, one drawn
    from each of n_spread equal slices of the radius ranking."""
    nb = cloud.bulk_node_num
    live = np.flatnonzero(cloud.ab_all[:nb] > 0)
    order = live[np.argsort(np.linalg.norm(cloud.xyz[live], axis=1), kind="stable")]
    rng = np.random.default_rng(seed)
    mid = order[n_core:len(order) - n_surface]
    edges = np.linspace(0, len(mid), n_spread + 1).astype(np.int64)
    spread = [mid[rng.integers(edges[i], edges[i + 1])] for i in range(n_spread)]
    return np.unique(np.concatenate([order[:n_core], order[len(order) - n_surface:], spread]))


def _se_checks(name, ctx, P, cloud, mol, kmax, J0, J2, oJ0, oJ2, nodes, pops_gpu, significant=None):
    """The SE of the sample from the oracle's J on both sides (1e-10), and
    the chained populations (GPU J -> GPU SE against oracle J -> oracle SE)."""
    J0m, J2m = J0.copy(), J2.copy()
    J0m[nodes], J2m[nodes] = oJ0[nodes], oJ2[nodes]
    pp_same, _ = ctx.solve_se(kmax, J0m, J2m)
    opp, ost = P.solve_se_nodes(kmax, oJ0, oJ2, nodes)
    assert not ost.any()
    o, g, c = opp[nodes, 0::2], pp_same[nodes, 0::2], pops_gpu[nodes, 0::2]
    sig = np.ones_like(o, dtype=bool) if significant is None else (
        np.abs(o) >= significant * np.abs(o).max(axis=1, keepdims=True))
    scale = np.abs(o).max(axis=1, keepdims=True)
    same0 = (np.abs(g - o) / np.abs(o))[sig].max()
    same2 = (np.abs(pp_same[nodes, 1::2] - opp[nodes, 1::2]) / scale).max()
    chain0 = (np.abs(c - o) / np.abs(o))[sig].max()
    chain2 = (np.abs(pops_gpu[nodes, 1::2] - opp[nodes, 1::2]) / scale).max()
    _report(name + " se", same_rho00=same0, same_rho20=same2, chain_rho00=chain0, chain_rho20=chain2)
    assert same0 < 1e-10 and same2 < 1e-10
    assert chain0 < 2e-4 and chain2 < 2e-5


@pytest.fixture(scope="module")
def sphere262k():
    from portal_gb300 import synth
    return synth.config_cloud("sphere262k", keep_raw=True)


def _check_device_neighbours(name, ctx, cloud):
    """portal_adj_list (adj_list_no_delaunay + SortUnique on the device)
    against the host construction of the same lists, bit for bit, with both
    times reported."""
    import time
    from portal_gb300 import synth
    t0 = time.perf_counter()
    off, idx = synth.neighbours_from_tets(cloud.tets, cloud.node_num)
    t_host = time.perf_counter() - t0
    t0 = time.perf_counter()
    dne, num, ms = ctx.adj_list(cloud.node_num, cloud.tets)
    t_call = time.perf_counter() - t0
    np.testing.assert_array_equal(num, np.diff(off))
    np.testing.assert_array_equal(dne, cloud.del_ne())
    np.testing.assert_array_equal(off, cloud.nb_off)
    np.testing.assert_array_equal(idx, cloud.nb_idx)
    _report(name + " neighbours", tets=cloud.tets.shape[0], device_ms=ms, call_s=t_call, host_numpy_s=t_host,
            max_ne=dne.shape[0])


def test_sphere262k_full_cloud_stratified_sample(built_lib, sphere262k):
    """The benchmark cloud itself: the whole node loop on the GPU, 256
    stratified nodes against the oracle."""
    import oracle
    import portal_gb300 as pg
    cloud, mol, rc = sphere262k
    nodes = radius_sample(cloud)
    r = np.linalg.norm(cloud.xyz[nodes], axis=1)
    assert len(nodes) == 256 and (r < 0.02).sum() >= 8 and r.max() > 0.99
    with pg.Context(0) as ctx:
        ctx.set_molecule(mol)
        ctx.set_cloud(cloud)
        J0, J2, st, nseg = ctx.radiation_field(rc)
        seg = ctx.node_segments()
        pops, st2 = ctx.solve_se(rc.kmax)
        assert not st.any() and not (st2 & pg.NODE_SINGULAR).any()
        assert seg.sum() == nseg
        P = oracle.OracleProblem(cloud, mol)
        oJ0, oJ2, ost, oseg = P.radiation_field_nodes(rc, nodes)
        assert not ost.any()
        e = _j_errors(J0[nodes], J2[nodes], oJ0[nodes], oJ2[nodes])
        dseg = np.abs(seg[nodes].astype(np.int64) - oseg)
        _report("sphere262k field", nodes=len(nodes), segments=int(oseg.sum()), seg_diff=int(dseg.sum()),
                **e)
        _check_J(J0[nodes], J2[nodes], oJ0[nodes], oJ2[nodes])
        assert dseg.sum() <= 1e-4 * oseg.sum()
        # the core nodes, where the walks are longest, by themselves
        core = nodes[r < 0.02]
        _check_J(J0[core], J2[core], oJ0[core], oJ2[core])
        _se_checks("sphere262k", ctx, P, cloud, mol, rc.kmax, J0, J2, oJ0, oJ2, nodes, pops)
        _check_device_neighbours("sphere262k", ctx, cloud)


def test_sphere4k_full_image_cube(built_lib, sphere4k, sphere4k_oracle):
    """The 4,096-point workload's output: one 129 x 129 x 65 Stokes IQUV
    cube at 45 degrees (im_pix 64, nvel 32, 100 m/s channels), pixel for
    pixel against the oracle's finish_portal loop on the same populations
    (I, tau within 1e-4 of the peak, Q/I and U/I within 1e-4).  Then the
    cube of the GPU's own node loop against the oracle's chain."""
    cloud, mol, rc = sphere4k
    import portal_gb300 as pg
    P = sphere4k_oracle["P"]
    opp = sphere4k_oracle["pops"]
    im = dict(th_inc=0.78539816339, ph_az=0.0, nvel=32, dvel=100.0, v0=0.0, im_pix=64, im_size=0.7)
    npx, nch = 2 * im["im_pix"] + 1, 2 * im["nvel"] + 1
    ocube, ost, nf = P.image([1], [2], opp, im["th_inc"], im["ph_az"], im["nvel"], im["dvel"], im["v0"],
                             im["im_pix"], im["im_size"])
    assert nf == 0
    o = ocube.reshape(8, npx, npx, 1, nch).transpose(0, 3, 4, 2, 1)
    with pg.Context(0) as ctx:
        ctx.set_molecule(mol)
        ctx.set_cloud(cloud)
        cube, st = ctx.image([1], [2], im["th_inc"], im["ph_az"], im["nvel"], im["dvel"], im["v0"],
                             im["im_pix"], im["im_size"], pol_pops=opp)
        assert not st.any() and cube.shape == (8, 1, nch, npx, npx)
        ctx.radiation_field(rc, fetch=False)
        ctx.solve_se(rc.kmax, fetch=False)
        chain, _ = ctx.image([1], [2], im["th_inc"], im["ph_az"], im["nvel"], im["dvel"], im["v0"],
                             im["im_pix"], im["im_size"])

    def errs(c):
        I, Q, U, tau = c[0, 0], c[1, 0], c[2, 0], c[3, 0]
        oI, oQ, oU, otau = o[0, 0], o[1, 0], o[2, 0], o[3, 0]
        Ipk = np.abs(oI).max()
        den = np.maximum(np.abs(oI), 1e-3 * Ipk)
        return dict(I=np.abs(I - oI).max() / Ipk, tau=np.abs(tau - otau).max() / np.abs(otau).max(),
                    QI=(np.abs(Q - oQ) / den).max(), UI=(np.abs(U - oU) / den).max(),
                    pol_frac=np.nanmax(np.hypot(oQ, oU) / den))

    e = errs(cube)
    ec = errs(chain)
    _report("sphere4k image", **e)
    _report("sphere4k image chain", **ec)
    assert np.isfinite(cube[:4]).all()
    assert not np.array_equal(chain[:4], cube[:4])   # the chain images other populations
    assert e["I"] < 1e-4 and e["tau"] < 1e-4 and e["QI"] < 1e-4 and e["UI"] < 1e-4
    assert ec["I"] < 1e-3 and ec["QI"] < 1e-4 and ec["UI"] < 1e-4


def density_sample(cloud, n=48, seed=0):
    """0-based bulk node ids of the turbulent cube: n/3 across the density
    ranking, n/3 across the radius ranking (centre to the corners of the
    cube, |X| -> 1), n/3 at random."""
    nb = cloud.bulk_node_num
    rng = np.random.default_rng(seed)
    k = n // 3
    by_n = np.argsort(cloud.h2_dens[:nb], kind="stable")
    by_r = np.argsort(np.linalg.norm(cloud.xyz[:nb], axis=1), kind="stable")
    pick = [by_n[int(q)] for q in np.linspace(0, nb - 1, k)]
    pick += [by_r[int(q)] for q in np.linspace(0, nb - 1, k)]
    pick += list(rng.choice(nb, n - 2 * k, replace=False))
    out = np.unique(np.asarray(pick, dtype=np.int64))
    return out


def test_cube1m_full_cloud_sample(built_lib):
    """The 1,048,576-point turbulent cube: the full node loop on the GPU
    (one pass, about a minute), 48 nodes across density and radius against
    the oracle.  20 levels at 20 K span ~60 decades, so the populations are
    compared on the levels above 1e-8 of each node's largest."""
    import oracle
    import portal_gb300 as pg
    from portal_gb300 import synth
    cloud, mol, rc = synth.config_cloud("cube1m", keep_raw=True)
    assert cloud.node_num == 1048576 and mol.nlev == 20
    nodes = density_sample(cloud)
    with pg.Context(0) as ctx:
        ctx.set_molecule(mol)
        ctx.set_cloud(cloud)
        J0, J2, st, nseg = ctx.radiation_field(rc)
        seg = ctx.node_segments()
        pops, st2 = ctx.solve_se(rc.kmax)
        assert not st.any() and not (st2 & pg.NODE_SINGULAR).any()
        P = oracle.OracleProblem(cloud, mol)
        oJ0, oJ2, ost, oseg = P.radiation_field_nodes(rc, nodes)
        assert not ost.any()
        e = _j_errors(J0[nodes], J2[nodes], oJ0[nodes], oJ2[nodes])
        dseg = np.abs(seg[nodes].astype(np.int64) - oseg)
        _report("cube1m field", nodes=len(nodes), segments=int(oseg.sum()), seg_diff=int(dseg.sum()),
                total_segments=nseg, **e)
        _check_J(J0[nodes], J2[nodes], oJ0[nodes], oJ2[nodes])
        assert dseg.sum() <= 1e-4 * oseg.sum()
        _se_checks("cube1m", ctx, P, cloud, mol, rc.kmax, J0, J2, oJ0, oJ2, nodes, pops, significant=1e-8)
        _check_device_neighbours("cube1m", ctx, cloud)
