"""CUDA path (through the C ABI) against the FP64 oracle on the same seeded
inputs.

Stated tolerances (FP32 ray integration with an FP32 Voronoi walk, FP32 LU +
FP64 refinement for the SE):
  J^0_0       per (node, line) relative error: max 2e-4, 99th pct 2e-5,
              median 2e-7 (the weak, optically thin high-J lines carry the
              largest FP32 error)
  J^2_0       per (node, line) |dJ^2_0| / J^0_0: max 5e-5
  rho (same J) relative 1e-10 (FP64 solve quality)
  rho (chain)  rho^0_0 relative 2e-4, |d rho^2_0| / rho^0_0 2e-5
  segments    equal to 1e-4 (near-degenerate Voronoi crossings may differ)
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

J0_MAX, J0_P99, J0_MED, J2_MAX = 2e-4, 2e-5, 2e-7, 5e-5


@pytest.fixture(scope="module")
def ctx(built_lib):
    import portal_gb300 as pg
    c = pg.Context(0)
    yield c
    c.close()


def _rf(ctx, cloud, mol, rc):
    ctx.set_molecule(mol)
    ctx.set_cloud(cloud)
    return ctx.radiation_field(rc)


def _check_J(J0, J2, oJ0, oJ2, mask=None):
    if mask is not None:
        J0, J2, oJ0, oJ2 = J0[mask], J2[mask], oJ0[mask], oJ2[mask]
    r0 = np.abs(J0 - oJ0) / np.abs(oJ0)
    r2 = np.abs(J2 - oJ2) / np.abs(oJ0)
    assert np.isfinite(J0).all() and np.isfinite(J2).all()
    assert r0.max() < J0_MAX, r0.max()
    assert np.quantile(r0, 0.99) < J0_P99, np.quantile(r0, 0.99)
    assert np.median(r0) < J0_MED, np.median(r0)
    assert r2.max() < J2_MAX, r2.max()


def test_radiation_field_sphere4k(ctx, sphere4k, sphere4k_oracle):
    cloud, mol, rc = sphere4k
    J0, J2, st, nseg = _rf(ctx, cloud, mol, rc)
    assert not st.any()
    assert abs(nseg - sphere4k_oracle["nseg"]) <= 1e-4 * sphere4k_oracle["nseg"]
    _check_J(J0, J2, sphere4k_oracle["J0"], sphere4k_oracle["J2"])


def test_solve_se_same_J_sphere4k(ctx, sphere4k, sphere4k_oracle):
    import portal_gb300 as pg
    cloud, mol, rc = sphere4k
    ctx.set_molecule(mol)
    ctx.set_cloud(cloud)
    pops, st = ctx.solve_se(rc.kmax, sphere4k_oracle["J0"], sphere4k_oracle["J2"])
    assert not (st & pg.NODE_SINGULAR).any()
    opp = sphere4k_oracle["P"].solve_se(rc.kmax, sphere4k_oracle["J0"], sphere4k_oracle["J2"])[0]
    scale = np.abs(opp[:, 0::2]).max(axis=1, keepdims=True)
    assert (np.abs(pops[:, 0::2] - opp[:, 0::2]) / np.abs(opp[:, 0::2])).max() < 1e-10
    assert (np.abs(pops[:, 1::2] - opp[:, 1::2]) / scale).max() < 1e-10
    g = np.sqrt(2 * mol.j_lev + 1)
    np.testing.assert_allclose((pops[:, 0::2] * g).sum(1), 1.0, rtol=1e-12)


def test_extra_info_rates_sphere4k(ctx, sphere4k, sphere4k_oracle):
    """The extra_info rates (spontaneous, radiative, collisional per
    component, em_coefs.f90:188-198 packed like the populations) and
    J2/J0 from the same J as the oracle."""
    cloud, mol, rc = sphere4k
    ctx.set_molecule(mol)
    ctx.set_cloud(cloud)
    for kmax in (2, rc.kmax):
        pops, st, jj, rt = ctx.solve_se(kmax, sphere4k_oracle["J0"], sphere4k_oracle["J2"], jj20=True, rates=True)
        _, _, _, ort = sphere4k_oracle["P"].solve_se(kmax, sphere4k_oracle["J0"], sphere4k_oracle["J2"], rates=True)
        bulk = cloud.bulk_node_num
        scale = np.abs(ort[:bulk]).max(axis=2, keepdims=True) + 1e-300
        assert (np.abs(rt[:bulk] - ort[:bulk]) / scale).max() < 1e-10
        assert np.abs(ort[:bulk]).max() > 0
        assert not rt[bulk:].any()
        with np.errstate(invalid="ignore", divide="ignore"):
            want = sphere4k_oracle["J2"] / sphere4k_oracle["J0"]
        live = cloud.ab_all[:bulk] > 0
        np.testing.assert_allclose(jj[:bulk][live], want[:bulk][live], rtol=1e-15)


def test_node_loop_chain_sphere4k(ctx, sphere4k, sphere4k_oracle):
    """Device-resident chain radiation field -> SE against oracle -> oracle."""
    cloud, mol, rc = sphere4k
    ctx.set_molecule(mol)
    ctx.set_cloud(cloud)
    ctx.radiation_field(rc, fetch=False)
    pops, st = ctx.solve_se(rc.kmax)
    opp = sphere4k_oracle["pops"]
    assert (np.abs(pops[:, 0::2] - opp[:, 0::2]) / np.abs(opp[:, 0::2])).max() < 2e-4
    scale = np.abs(opp[:, 0::2]).max(axis=1, keepdims=True)
    assert (np.abs(pops[:, 1::2] - opp[:, 1::2]) / scale).max() < 2e-5


def test_field_moments_hold_j20_in_every_frame(ctx, sphere4k):
    """The second moment M = sum w Ibar n n of line 1 (the warm start's J^2_0
    axis): its trace is J^0_0 and, along the node's field b, (3 b.M.b -
    tr M) / (2 sqrt 2) is the field-frame J^2_0 of inverse_rt.f90:128-129."""
    cloud, mol, rc = sphere4k
    J0, J2, st, _ = _rf(ctx, cloud, mol, rc)
    M = ctx.field_moments()
    b = cloud.bvec
    bMb = (M[:, 0] * b[:, 0] ** 2 + M[:, 1] * b[:, 1] ** 2 + M[:, 2] * b[:, 2] ** 2 +
           2.0 * (M[:, 3] * b[:, 0] * b[:, 1] + M[:, 4] * b[:, 0] * b[:, 2] + M[:, 5] * b[:, 1] * b[:, 2]))
    tr = M[:, 0] + M[:, 1] + M[:, 2]
    live = cloud.ab_all > 0
    live[cloud.bulk_node_num:] = False
    j0 = J0[live, 0]
    assert (np.abs(tr[live] - j0) / j0).max() < 1e-4
    j20 = (3.0 * bMb - tr) / (2.0 * np.sqrt(2.0))
    assert (np.abs(j20[live] - J2[live, 0]) / j0).max() < 1e-4
    assert np.abs(J2[live, 0]).max() > 1e-3 * j0.max()   # an anisotropic field to test against
    assert not M[~live].any()


def test_deterministic(ctx, sphere4k):
    cloud, mol, rc = sphere4k
    a = _rf(ctx, cloud, mol, rc)
    b = ctx.radiation_field(rc)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]) and a[3] == b[3]


def _small(n=2048, nlev=5, seed=5, **kw):
    from portal_gb300 import synth
    mol = synth.linear_rotor(nlev)
    cloud = synth.power_law_sphere(n, seed, mol, **kw)
    rc = synth.RunConfig(nth=8, nph=8, nvel=16, kmax=6, gvec=synth.gauge_vector(seed))
    return cloud, mol, rc


def test_two_collision_partners(ctx):
    """c_par = 2 (para and ortho H2 in LAMDA files such as the reference's
    CO_coro_v2.dat): rates mixed 25 % / 75 % after the temperature
    interpolation (miscellaneous.f90:331-360); the populations of the same J
    equal the oracle's to 1e-10."""
    import dataclasses
    import oracle
    cloud, mol, rc = _small(1024, t_law="loglinear")
    T = mol.col_temps[None, :]
    C2 = np.concatenate([0.5 * mol.C * (1.0 + T / 50.0), 2.0 * mol.C * (1.0 + T / 200.0)], axis=0)
    mol2 = dataclasses.replace(mol, C=C2)
    assert mol2.c_par == 2
    P = oracle.OracleProblem(cloud, mol2)
    oJ0, oJ2, _, _, _ = P.radiation_field(rc)
    opp, _, _ = P.solve_se(rc.kmax, oJ0, oJ2)
    ctx.set_molecule(mol2)
    ctx.set_cloud(cloud)
    pops, st = ctx.solve_se(rc.kmax, oJ0, oJ2)
    bulk = cloud.bulk_node_num
    scale = np.abs(opp[:bulk, 0::2]).max(axis=1, keepdims=True)
    assert (np.abs(pops[:bulk, 0::2] - opp[:bulk, 0::2]) / scale).max() < 1e-10
    assert (np.abs(pops[:bulk, 1::2] - opp[:bulk, 1::2]) / scale).max() < 1e-10
    # the second partner matters: the one-partner molecule gives other populations
    P1 = oracle.OracleProblem(cloud, mol)
    opp1, _, _ = P1.solve_se(rc.kmax, oJ0, oJ2)
    assert np.abs(opp1[:bulk, 0::2] - opp[:bulk, 0::2]).max() > 1e-3 * np.abs(opp[:bulk, 0::2]).max()


@pytest.mark.parametrize("mode", [1, 2])
def test_depolarising_collisions_against_oracle(ctx, mode):
    """Depolarising collisions (depol.f90:242-360 into setup_stateq's
    col_dep, pop_eqs.f90:642-648), which the reference leaves off
    (main_sub.f90:96): the populations and alignment of the same J as the
    oracle's with the same mode, 1e-10; the extra_info rates likewise; and
    the switch back to mode 0 restores the plain SE."""
    import oracle
    cloud, mol, rc = _small(1024, nlev=6, t_law="loglinear")
    P = oracle.OracleProblem(cloud, mol, depol=mode)
    oJ0, oJ2, _, _, _ = P.radiation_field(rc, 1, 128)
    opp, ost, _, ort = P.solve_se(rc.kmax, oJ0, oJ2, 1, 128, rates=True)
    plain = oracle.OracleProblem(cloud, mol).solve_se(rc.kmax, oJ0, oJ2, 1, 128)[0]
    ctx.set_molecule(mol)
    ctx.set_cloud(cloud)
    try:
        ctx.set_depolarization(mode)
        pops, st, rt = ctx.solve_se(rc.kmax, oJ0, oJ2, rates=True)
    finally:
        ctx.set_depolarization(0)
    scale = np.abs(opp[:128, 0::2]).max(axis=1, keepdims=True)
    assert (np.abs(pops[:128, 0::2] - opp[:128, 0::2]) / scale).max() < 1e-10
    assert (np.abs(pops[:128, 1::2] - opp[:128, 1::2]) / scale).max() < 1e-10
    rscale = np.abs(ort[:128]).max(axis=2, keepdims=True) + 1e-300
    assert (np.abs(rt[:128] - ort[:128]) / rscale).max() < 1e-10
    # the depolarisation is there: the alignment moved
    assert np.abs(opp[:128, 1::2] - plain[:128, 1::2]).max() > 1e-3 * np.abs(plain[:128, 1::2]).max()
    back, _ = ctx.solve_se(rc.kmax, oJ0, oJ2)
    np.testing.assert_allclose(back[:128], plain[:128], rtol=1e-10, atol=1e-14 * np.abs(plain).max())


def _se74():
    """A 2,048-point sphere with a 20-level rotor at kmax 6 (74 x 74 SE
    systems), LTE populations and the local Planck field with a small
    anisotropy."""
    import dataclasses
    from portal_gb300 import synth
    cloud, mol, rc = _small(2048, nlev=20, t_law="loglinear")
    frac = synth.lte_fractions(mol, np.maximum(cloud.t_kin, 1.0))
    cloud = dataclasses.replace(cloud, lev_p=np.ascontiguousarray(frac * (cloud.ab_all * cloud.h2_dens)[:, None]))
    nu = np.asarray(mol.nu)
    J0 = 1.4744995e-50 * nu ** 3 / np.expm1(4.79924e-11 * nu / np.maximum(cloud.t_kin, 1.0)[:, None])
    J2 = 1e-3 * J0 * np.cos(np.arange(cloud.node_num))[:, None]
    return cloud, mol, rc, J0, J2


def _against_oracle_se(pops, cloud, mol, rc, J0, J2, nodes=64, tol=1e-10):
    import oracle
    opp = oracle.OracleProblem(cloud, mol).solve_se(rc.kmax, J0, J2, 1, nodes)[0]
    scale = np.abs(opp[:nodes, 0::2]).max(axis=1, keepdims=True)
    assert (np.abs(pops[:nodes, 0::2] - opp[:nodes, 0::2]) / scale).max() < tol
    assert (np.abs(pops[:nodes, 1::2] - opp[:nodes, 1::2]) / scale).max() < tol


@pytest.mark.parametrize("team", [4])
def test_se_team_of_warps_matches_one_warp_and_oracle(ctx, monkeypatch, team):
    """74 x 74 systems (20-level rotor, kmax 6) solved by a team of warps per
    node (the default above 48 unknowns) and by one warp: the factorisation
    sees the same operations per element, so populations, alignment, rates
    and status are identical; against the oracle (get_rhovec,
    em_coefs.f90:115-201) on 64 nodes to 1e-10 from the same J."""
    import portal_gb300 as pg
    cloud, mol, rc, J0, J2 = _se74()
    ctx.set_molecule(mol)
    ctx.set_cloud(cloud)
    monkeypatch.setenv("PORTAL_SE_TEAM", "1")
    p1, s1, r1 = ctx.solve_se(rc.kmax, J0, J2, rates=True)
    monkeypatch.setenv("PORTAL_SE_TEAM", str(team))
    pt, st, rt = ctx.solve_se(rc.kmax, J0, J2, rates=True)
    assert np.array_equal(p1, pt) and np.array_equal(s1, st) and np.array_equal(r1, rt)
    assert not (st & pg.NODE_SINGULAR).any()
    _against_oracle_se(pt, cloud, mol, rc, J0, J2)


def test_se_fp64_mode_one_warp_and_team(ctx, monkeypatch):
    """PORTAL_SE_FP64=1 factorises every system in FP64 on the device -- the
    path the refinement falls back to when it stalls (the team's
    factorisation and the register triangular solves in FP64), which the
    well-conditioned workloads never reach otherwise.  Every live node is
    flagged PORTAL_NODE_REFINE; one warp and a team of four give identical
    results; both match the oracle to 1e-10 and the FP32-refined solve to
    1e-10."""
    import portal_gb300 as pg
    cloud, mol, rc, J0, J2 = _se74()
    ctx.set_molecule(mol)
    ctx.set_cloud(cloud)
    monkeypatch.setenv("PORTAL_SE_FP64", "0")
    p32, s32 = ctx.solve_se(rc.kmax, J0, J2)
    monkeypatch.setenv("PORTAL_SE_FP64", "1")
    res = {}
    for team in (1, 4):
        monkeypatch.setenv("PORTAL_SE_TEAM", str(team))
        res[team] = ctx.solve_se(rc.kmax, J0, J2)
    (p1, s1), (p4, s4) = res[1], res[4]
    assert np.array_equal(p1, p4) and np.array_equal(s1, s4)
    live = cloud.ab_all[: cloud.bulk_node_num] > 0
    assert ((s4[: cloud.bulk_node_num][live] & pg.NODE_REFINE) != 0).all()
    assert not (s4 & pg.NODE_SINGULAR).any()
    _against_oracle_se(p4, cloud, mol, rc, J0, J2)
    scale = np.abs(p32[:, 0::2]).max(axis=1, keepdims=True) + 1e-300
    assert (np.abs(p4[:, 0::2] - p32[:, 0::2]) / scale).max() < 1e-10
    assert (np.abs(p4[:, 1::2] - p32[:, 1::2]) / scale).max() < 1e-10


def test_n_depth_overflow_is_reported(ctx):
    import portal_gb300 as pg
    cloud, mol, rc = _small()
    rc.n_depth = 3
    ctx.set_molecule(mol)
    ctx.set_cloud(cloud)
    with pytest.raises(pg.PortalError) as e:
        ctx.radiation_field(rc)
    assert e.value.code == -4
    # the iterated node loop stops on it too (no pass runs on zeroed fields)
    ctx.set_cloud(cloud)
    with pytest.raises(pg.PortalError) as e:
        ctx.lambda_iterate(rc, tol=1e-6, max_iter=3)
    assert e.value.code == -4


def test_star_rays_beyond_nth_nph_are_reported(ctx):
    """A node so close to the star that star_all needs more than nth*nph
    rays stops the reference (miscellaneous.f90:1203-1206): an error here,
    with status bit PORTAL_NODE_STAR on that node."""
    import portal_gb300 as pg
    cloud, mol, rc = _small()
    R = 0.05
    r = np.linalg.norm(cloud.xyz[:cloud.bulk_node_num], axis=1)
    assert ((r > R) & (r < 1.06 * R)).any()   # 8 x 8 directions cannot hold these nodes' rays
    ctx.set_molecule(mol)
    ctx.set_cloud(cloud)
    ctx.set_star((2500.0, R * cloud.tx, (0.0, 0.0, 0.0)))
    try:
        with pytest.raises(pg.PortalError) as e:
            ctx.radiation_field(rc)
        assert e.value.code == -2 and "star" in str(e.value)
    finally:
        ctx.set_star(None)


def test_skipped_and_surface_nodes(ctx):
    """ab_all <= 0 nodes (main_para.f90:213) and nodes beyond bulk_node_num
    get J = 0 and pol_pops = 0, as in the reference."""
    import oracle
    cloud, mol, rc = _small()
    cloud.ab_all[[3, 10, 77]] = 0.0
    cloud.bulk_node_num = cloud.node_num - 100
    J0, J2, st, _ = _rf(ctx, cloud, mol, rc)
    pops, _ = ctx.solve_se(rc.kmax)
    for n in (3, 10, 77):
        assert (J0[n] == 0).all() and (pops[n] == 0).all()
    assert (J0[cloud.bulk_node_num:] == 0).all() and (pops[cloud.bulk_node_num:] == 0).all()
    P = oracle.OracleProblem(cloud, mol)
    oJ0, oJ2, _, _, _ = P.radiation_field(rc, 1, 200)
    m = np.ones(200, bool); m[[3, 10, 77]] = False
    _check_J(J0[:200], J2[:200], oJ0[:200], oJ2[:200], mask=m)


def test_star_mode_against_oracle(ctx):
    """star_mod = 1 (a 2,500 K star of 0.05 r_max at the centre): nodes inside
    the star are skipped (J and populations 0); every other node integrates
    over its own star_all ray set, the star rays ending on the star and
    starting from B(T_star).  J within the stated tolerances of the oracle's
    star-mode node loop, then the populations of the same J to 1e-10.  12 x
    12 directions: with 8 x 8 the nodes nearest the star would need more
    rays than nth*nph, where the reference stops."""
    import oracle
    cloud, mol, rc = _small()
    rc.nth = rc.nph = 12
    star = (2500.0, 0.05 * cloud.tx, (0.0, 0.0, 0.0))
    inside = np.linalg.norm(cloud.xyz, axis=1) <= 0.05
    assert 10 < inside[:cloud.bulk_node_num].sum() < cloud.bulk_node_num // 2
    ctx.set_molecule(mol)
    ctx.set_cloud(cloud)
    ctx.set_star(star)
    try:
        J0, J2, st, nseg = ctx.radiation_field(rc)
        pops, _ = ctx.solve_se(rc.kmax)
    finally:
        ctx.set_star(None)
    P = oracle.OracleProblem(cloud, mol, star=star)
    oJ0, oJ2, ost, onseg, nf = P.radiation_field(rc)
    assert nf == 0 and not st.any() and not ost.any()
    bulk = cloud.bulk_node_num
    assert (J0[:bulk][inside[:bulk]] == 0).all() and (pops[:bulk][inside[:bulk]] == 0).all()
    live = ~inside[:bulk] & (cloud.ab_all[:bulk] > 0)
    _check_J(J0[:bulk], J2[:bulk], oJ0[:bulk], oJ2[:bulk], mask=live)
    assert abs(nseg - onseg) <= 1e-4 * onseg
    # the star shows in the field of the nodes next to it
    J0n, _, _, _ = _rf(ctx, cloud, mol, rc)
    near = live & (np.linalg.norm(cloud.xyz[:bulk], axis=1) < 0.1)
    assert near.any() and np.abs(J0 - J0n)[:bulk][near].max() > 1e-3 * J0n[:bulk][near].max()
    opp, _, _ = P.solve_se(rc.kmax, J0, J2)
    assert (opp[:bulk][inside[:bulk]] == 0).all()
    np.testing.assert_allclose(pops[:bulk][live], opp[:bulk][live], rtol=1e-10, atol=1e-14)


def test_image_star_against_oracle(ctx):
    """Star mode in the image: pixels on the star's disc start at its front
    from B(T_star) (raytrace.f90:103-115); I, Q, U, tau against the oracle
    with the pixel-mode tolerances, NaN where the oracle's are."""
    import oracle
    cloud, mol, rc, im = _image_case(n=2048, im_pix=8)
    star = (2500.0, 0.1 * cloud.tx, (0.0, 0.0, 0.0))
    P = oracle.OracleProblem(cloud, mol)
    oJ0, oJ2, _, _, _ = P.radiation_field(rc)
    opp, _, _ = P.solve_se(rc.kmax, oJ0, oJ2)
    Ps = oracle.OracleProblem(cloud, mol, star=star)
    ctx.set_molecule(mol)
    ctx.set_cloud(cloud)
    ctx.set_star(star)
    try:
        cube, st = ctx.image(im["l1"], im["l2"], im["th_inc"], im["ph_az"], im["nvel"], im["dvel"], im["v0"],
                             im["im_pix"], im["im_size"], pol_pops=opp)
    finally:
        ctx.set_star(None)
    ocube, ost, nf = Ps.image(im["l1"], im["l2"], opp, im["th_inc"], im["ph_az"], im["nvel"], im["dvel"],
                              im["v0"], im["im_pix"], im["im_size"])
    assert nf == 0 and not st.any()
    npx, nch = 2 * im["im_pix"] + 1, 2 * im["nvel"] + 1
    o = ocube.reshape(8, npx, npx, 1, nch).transpose(0, 3, 4, 2, 1)
    _stokes_close(cube, o, [0])
    # the disc's rays start at the star's front: less optical depth than the star-less rays
    plain, _ = ctx.image(im["l1"], im["l2"], im["th_inc"], im["ph_az"], im["nvel"], im["dvel"], im["v0"],
                         im["im_pix"], im["im_size"], pol_pops=opp)
    c = im["im_pix"]
    assert (cube[3, 0, :, c, c] < plain[3, 0, :, c, c]).all()


def test_neighbour_lists_longer_than_a_warp(ctx):
    """Padding every neighbour list with non-adjacent nodes (beyond 32
    entries) leaves the Voronoi walk unchanged: the padded faces are never the
    nearest exit.  Checked against the oracle on the same padded lists."""
    import oracle
    cloud, mol, rc = _small(1024)
    N = cloud.node_num
    rng = np.random.default_rng(1)
    off, idx = cloud.nb_off, cloud.nb_idx
    new_off, new_idx = [0], []
    for i in range(N):
        own = set(idx[off[i]:off[i + 1]].tolist()) | {i}
        extra = [int(x) for x in rng.choice(N, 40, replace=False) if int(x) not in own][:24]
        lst = sorted(set(idx[off[i]:off[i + 1]].tolist()) | set(extra))
        new_idx += lst
        new_off.append(len(new_idx))
    cloud.nb_off = np.array(new_off, dtype=np.int64)
    cloud.nb_idx = np.array(new_idx, dtype=np.int32)
    assert np.diff(cloud.nb_off).max() > 32
    J0, J2, st, nseg = _rf(ctx, cloud, mol, rc)
    P = oracle.OracleProblem(cloud, mol)
    oJ0, oJ2, _, onseg, _ = P.radiation_field(rc, 1, 128)
    _check_J(J0[:128], J2[:128], oJ0[:128], oJ2[:128])


def test_dust_path(ctx):
    """Dust on (gas-to-dust ratio set): the dust branch of ray_in
    (inverse_rt.f90:298-311) against the oracle."""
    import oracle
    from portal_gb300 import synth
    cloud, mol, rc = _small(1024)
    cloud.dust_p[:] = cloud.h2_dens * synth.F4(2.32e-27) / 100.0
    J0, J2, st, _ = _rf(ctx, cloud, mol, rc)
    P = oracle.OracleProblem(cloud, mol)
    oJ0, oJ2, _, _, _ = P.radiation_field(rc, 1, 128)
    _check_J(J0[:128], J2[:128], oJ0[:128], oJ2[:128])


def test_sphere262k_shape_subset():
    """The 10-level / 24x24 / 129-channel shape on a 16,384-point cloud:
    first 64 nodes against the oracle."""
    import oracle
    import portal_gb300 as pg
    from portal_gb300 import synth
    cloud, mol, rc = synth.config_cloud("sphere262k", n_points=16384)
    with pg.Context(0) as c:
        c.set_molecule(mol)
        c.set_cloud(cloud)
        J0, J2, st, nseg = c.radiation_field(rc)
        pops, st2 = c.solve_se(rc.kmax)
    assert not st.any()
    P = oracle.OracleProblem(cloud, mol)
    oJ0, oJ2, _, _, _ = P.radiation_field(rc, 1, 64)
    _check_J(J0[:64], J2[:64], oJ0[:64], oJ2[:64])
    opp, _, _ = P.solve_se(rc.kmax, oJ0, oJ2, 1, 64)
    assert (np.abs(pops[:64, 0::2] - opp[:64, 0::2]) / np.abs(opp[:64, 0::2])).max() < 2e-4


def test_cube1m_shape_subset():
    """The turbulent-cube shape (20-level rotor, 32x32 directions, 129
    channels, kmax 2) on a 32,768-point cube: the full node loop on the
    device, first 24 nodes against the oracle, and the split of the
    accelerated iteration."""
    import oracle
    import portal_gb300 as pg
    from portal_gb300 import synth
    cloud, mol, rc = synth.config_cloud("cube1m", n_points=32768)
    with pg.Context(0) as c:
        c.set_molecule(mol)
        c.set_cloud(cloud)
        J0, J2, JE, LS, st = c.radiation_field_split(rc)
    assert not st.any()
    P = oracle.OracleProblem(cloud, mol)
    oJ0, oJ2, oJE, oLS, _ = P.radiation_field_split(rc, 1, 24)
    _check_J(J0[:24], J2[:24], oJ0[:24], oJ2[:24])
    assert (np.abs(JE[:24] - oJE[:24]) / oJE[:24]).max() < 2e-4
    assert np.abs(LS[:24] - oLS[:24]).max() < 2e-6
    # the plain node loop (setup_stateq's equations) against the oracle
    with pg.Context(0) as c:
        c.set_molecule(mol)
        c.set_cloud(cloud)
        c.radiation_field(rc, fetch=False)
        pops, _ = c.solve_se(rc.kmax)
    opp, _, _ = P.solve_se(rc.kmax, oJ0, oJ2, 1, 24)
    # 20 levels at 20 K span ~60 decades: compare the levels above 1e-8 of a
    # node's largest (the SE's refinement converges normwise)
    r, o = pops[:24, 0::2], opp[:24, 0::2]
    sig = np.abs(o) >= 1e-8 * np.abs(o).max(axis=1, keepdims=True)
    assert (np.abs(r - o) / np.abs(o))[sig].max() < 2e-4


# ---- Stokes image (finish_portal.x pixel mode) ----------------------------

def _image_case(n=4096, im_pix=16, nvel=8):
    from portal_gb300 import synth
    cloud, mol, rc = synth.config_cloud("sphere4k", n_points=n)
    return cloud, mol, rc, dict(l1=[1], l2=[2], th_inc=0.78539816339, ph_az=0.0, nvel=nvel, dvel=50.0,
                                v0=0.0, im_pix=im_pix, im_size=0.7)


def test_image_against_oracle(ctx):
    """I, Q, U, tau against the oracle's finish_portal pixel loop on the same
    pol_pops.  Tolerances: I and tau relative 1e-4 of the cube's peak, Q and U
    absolute 1e-4 of I per pixel-channel (Q/I within 1e-4)."""
    import oracle
    cloud, mol, rc, im = _image_case()
    P = oracle.OracleProblem(cloud, mol)
    oJ0, oJ2, _, _, _ = P.radiation_field(rc)
    opp, _, _ = P.solve_se(rc.kmax, oJ0, oJ2)
    ctx.set_molecule(mol)
    ctx.set_cloud(cloud)
    cube, st = ctx.image(im["l1"], im["l2"], im["th_inc"], im["ph_az"], im["nvel"], im["dvel"], im["v0"],
                         im["im_pix"], im["im_size"], pol_pops=opp)
    assert not st.any()
    ocube, ost, nf = P.image(im["l1"], im["l2"], opp, im["th_inc"], im["ph_az"], im["nvel"], im["dvel"],
                             im["v0"], im["im_pix"], im["im_size"])
    assert nf == 0
    npx = 2 * im["im_pix"] + 1
    nch = 2 * im["nvel"] + 1
    # oracle (8, n_rt, nlines, nch) with pixel p = a*npx + b  ->  (8, nlines, nch, b, a)
    o = ocube.reshape(8, npx, npx, 1, nch).transpose(0, 3, 4, 2, 1)
    I, Q, U, tau = cube[0], cube[1], cube[2], cube[3]
    oI, oQ, oU, otau = o[0], o[1], o[2], o[3]
    Ipk = np.abs(oI).max()
    assert np.abs(I - oI).max() < 1e-4 * Ipk, np.abs(I - oI).max() / Ipk
    assert np.abs(tau - otau).max() < 1e-4 * np.abs(otau).max()
    denom = np.maximum(np.abs(oI), 1e-3 * Ipk)
    assert (np.abs(Q - oQ) / denom).max() < 1e-4
    assert (np.abs(U - oU) / denom).max() < 1e-4
    # dust is off in this cloud: the dust maps are zero in both
    assert np.abs(cube[4:]).max() == 0.0 and np.abs(o[4:]).max() == 0.0


def _reversed_transitions(mol):
    """The same molecule with its radiative transitions listed in reverse
    order (a LAMDA file may list them in any order)."""
    import dataclasses
    return dataclasses.replace(mol, r_trans=mol.r_trans[::-1].copy(), A=mol.A[::-1].copy(),
                               freq_ghz=mol.freq_ghz[::-1].copy(), nu=mol.nu[::-1].copy(),
                               Bij=mol.Bij[::-1].copy(), kd_v=mol.kd_v[::-1].copy())


def _stokes_close(cube, ocube_t, lines):
    """I, Q, U, tau of (8, nl, nch, rays) against the oracle's, NaN where the
    oracle's are NaN; tolerances of the pixel-mode test."""
    for j in lines:
        I, Q, U, tau = (cube[q, j] for q in range(4))
        oI, oQ, oU, otau = (ocube_t[q, j] for q in range(4))
        for a, b in ((I, oI), (Q, oQ), (U, oU), (tau, otau)):
            np.testing.assert_array_equal(np.isnan(a), np.isnan(b))
        assert np.abs(tau - otau).max() < 1e-4 * np.abs(otau).max()
        ok = ~np.isnan(oI)
        if not ok.any():
            continue
        Ipk = np.abs(oI[ok]).max()
        assert Ipk > 0.0
        assert np.abs(I - oI)[ok].max() < 1e-4 * Ipk, (j, np.abs(I - oI)[ok].max() / Ipk)
        denom = np.maximum(np.abs(oI), 1e-3 * Ipk)[ok]
        assert (np.abs(Q - oQ)[ok] / denom).max() < 1e-4
        assert (np.abs(U - oU)[ok] / denom).max() < 1e-4


def test_image_nodes_against_oracle(ctx):
    """pix_mod = 0 (one ray per bulk node from its rotated sky position)
    against the oracle's per-node loop on the same pol_pops.  The molecule
    lists its transitions in reverse, so the per-node mode's t_Aji(l1) is
    another transition's A than the pixel mode's matched one; the second
    line (1, 3) has vanishing w^(2) on both levels, eta_Q = 0 and NaN I, Q,
    U in both (polarize_prop divides 0 by 0).  The xy rows are equal to the
    last bit; I, Q, U, tau within the pixel mode's tolerances."""
    import oracle
    cloud, mol, rc, im = _image_case(n=2048)
    P = oracle.OracleProblem(cloud, mol)
    oJ0, oJ2, _, _, _ = P.radiation_field(rc)
    opp, _, _ = P.solve_se(rc.kmax, oJ0, oJ2)
    rmol = _reversed_transitions(mol)
    Pr = oracle.OracleProblem(cloud, rmol)
    ctx.set_molecule(rmol)
    ctx.set_cloud(cloud)
    l1, l2 = [1, 1], [2, 3]
    cube, xy, st = ctx.image_nodes(l1, l2, 0.6, 0.3, im["nvel"], im["dvel"], im["v0"], pol_pops=opp)
    ocube, oxy, ost, nf = Pr.image_nodes(l1, l2, opp, 0.6, 0.3, im["nvel"], im["dvel"], im["v0"])
    assert nf == 0 and not st.any()
    np.testing.assert_array_equal(xy, oxy)
    o = ocube.transpose(0, 2, 3, 1)  # (8, nb, nl, nch) -> (8, nl, nch, nb)
    assert not np.isnan(o[0, 0]).any() and np.isnan(o[0, 1]).all()
    _stokes_close(cube, o, [0, 1])
    # t_Aji(1) of the reversed list is the top transition's A, not A(1 -> 2)
    with_matched = Pr.image(l1[:1], l2[:1], opp, 0.6, 0.3, im["nvel"], im["dvel"], im["v0"], 2, 0.5)[0]
    assert rmol.A[0] != mol.A[0] and np.isfinite(with_matched).all()


def test_image_face_on_field_is_nan_like_the_reference(ctx):
    """A field along the line of sight (B along z, th_inc = 0): sin(theta) =
    0 gives eta_Q = 0 and an undefined Stokes rotation, so the reference's I,
    Q, U are NaN wherever a line cell is crossed; the GPU image has the same
    NaN pattern and the same tau."""
    import oracle
    cloud, mol, rc, im = _image_case(n=2048, im_pix=6)
    P = oracle.OracleProblem(cloud, mol)
    oJ0, oJ2, _, _, _ = P.radiation_field(rc)
    opp, _, _ = P.solve_se(rc.kmax, oJ0, oJ2)
    ctx.set_molecule(mol)
    ctx.set_cloud(cloud)
    cube, st = ctx.image([1], [2], 0.0, 0.0, im["nvel"], im["dvel"], im["v0"], im["im_pix"], im["im_size"],
                         pol_pops=opp)
    ocube, ost, nf = P.image([1], [2], opp, 0.0, 0.0, im["nvel"], im["dvel"], im["v0"], im["im_pix"],
                             im["im_size"])
    npx, nch = 2 * im["im_pix"] + 1, 2 * im["nvel"] + 1
    o = ocube.reshape(8, npx, npx, 1, nch).transpose(0, 3, 4, 2, 1)
    assert np.isnan(o[0]).any()
    for q in range(3):
        np.testing.assert_array_equal(np.isnan(cube[q]), np.isnan(o[q]))
    assert np.abs(cube[3] - o[3]).max() < 1e-4 * np.abs(o[3]).max()


# ---- Lambda iteration -------------------------------------------------------

def test_lambda_iteration_against_oracle(ctx):
    """Three passes of the iterated node loop against the oracle iterated the
    same way (n_J = n_mol sqrt(2J+1) rho^0_0 between passes)."""
    import oracle
    cloud, mol, rc = _small(1024, nlev=5, t_uniform=20.0)
    n_mol = cloud.lev_p.sum(axis=1)
    g = np.sqrt(2 * mol.j_lev + 1.0)
    P = oracle.OracleProblem(cloud, mol)
    res_o = []
    for it in range(3):
        oJ0, oJ2, _, _, _ = P.radiation_field(rc)
        opp, _, _ = P.solve_se(rc.kmax, oJ0, oJ2)
        new = n_mol[:, None] * g[None, :] * opp[:, 0::2]
        old_rho = P.lev_p / (n_mol[:, None] * g[None, :])
        res_o.append(np.max(np.abs(opp[:, 0::2] - old_rho) / np.abs(opp[:, 0::2])))
        P.lev_p[:] = new          # the oracle struct points at this array
    ctx.set_molecule(mol)
    ctx.set_cloud(cloud)
    pops, lev, n, res, nseg = ctx.lambda_iterate(rc, tol=1e-30, max_iter=3)
    assert n == 3
    np.testing.assert_allclose(lev, P.lev_p, rtol=2e-4)
    np.testing.assert_allclose(res, res_o, rtol=0.05, atol=1e-6)
    # a warm start at the result of the passes continues from it
    pops2, lev2, n2, res2, _ = ctx.lambda_iterate(rc, tol=1e-30, max_iter=1, start_pops=pops)
    assert res2[0] < res[-1] * 1.5 + 1e-7
