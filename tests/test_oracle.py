"""The oracle against the golden fixtures and analytic limits (CPU only)."""
import ctypes as C
import json
import math
import os

import numpy as np
import pytest

import oracle
from portal_gb300 import synth

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _load(name):
    with open(os.path.join(GOLD, name)) as f:
        return json.load(f)


def test_wigner_3j_6j_against_sympy():
    g = _load("wigner.json")
    worst = 0.0
    for row in g["w3j"]:
        *a, v = row
        ex = float(v)
        got = oracle.wigner3j(*[2 * x for x in a])
        worst = max(worst, abs(got - ex) / max(abs(ex), 1e-300) if ex != 0 else abs(got))
    for row in g["w6j"]:
        *a, v = row
        ex = float(v)
        got = oracle.wigner6j(*[2 * x for x in a])
        worst = max(worst, abs(got - ex) / max(abs(ex), 1e-300) if ex != 0 else abs(got))
    assert worst < 1e-14, worst
    assert len(g["w3j"]) >= 600 and len(g["w6j"]) >= 300


def test_gauss_legendre_against_numpy_and_mpmath():
    g = _load("leggauss.json")
    for n, rule in g["rules"].items():
        x, w = oracle.gauss_legendre(int(n))
        ex = g["exact"][n]
        np.testing.assert_allclose(x, [float(v) for v in ex["x"]], rtol=0, atol=4e-16)
        np.testing.assert_allclose(w, [float(v) for v in ex["w"]], rtol=4e-15, atol=0)
        # numpy's leggauss itself carries ~1e-12 in the weights at n = 64
        np.testing.assert_allclose(x, rule["x"], rtol=0, atol=2e-15)
        np.testing.assert_allclose(w, rule["w"], rtol=5e-12, atol=0)


@pytest.mark.parametrize("n,expect", [(16, 178), (24, 388), (32, 678)])
def test_legendre_all_direction_count(n, expect):
    g = _load("leggauss.json")
    xth = oracle.legendre_all(n, n)
    assert len(xth) == expect == g["n_sphere"][str(n)]
    assert abs(xth[:, 2].sum() - 1.0) < 1e-13          # weights / 4 pi sum to 1
    # sum w P2(mu) = 0 for an exact rule
    assert abs((xth[:, 2] * (3 * xth[:, 0] ** 2 - 1) / 2).sum()) < 1e-13


def test_se_solution_against_lapack():
    g = _load("lapack.json")
    for case in g["cases"]:
        A = np.array(case["A"])
        rho = np.array(case["rho"])
        # oracle's LU-solve of the same system
        from scipy.linalg import solve
        x = solve(A, np.eye(A.shape[0])[:, 0])
        np.testing.assert_allclose(x, rho, rtol=1e-9, atol=1e-12 * np.abs(rho).max())


def test_se_oracle_matches_lapack_pipeline(sphere4k):
    """orc_solve_se (assembly + LU solve + packing) against the fixture's
    dgetri column for the same J."""
    cloud, mol, rc = sphere4k
    g = _load("lapack.json")
    P = oracle.OracleProblem(cloud, mol)
    N, R = cloud.node_num, mol.r_num
    for case in g["cases"]:
        node = case["node"]
        J0 = np.zeros((N, R)); J2 = np.zeros((N, R))
        J0[node - 1] = case["J0"]; J2[node - 1] = case["J2"]
        A = P.node_matrix(rc.kmax, node, J0, J2)
        A0 = np.array(case["A"])
        # rows 2.. of the oracle's matrix are the fixture's (row 1 replaced)
        np.testing.assert_allclose(A[1:], A0[1:], rtol=1e-12, atol=1e-300)
        pp, st, nf = P.solve_se(rc.kmax, J0, J2, node, node)
        rho = np.array(case["rho"])
        ca, c = [], 0
        for j in mol.j_lev:
            ca.append(c); c += len(range(0, min(2 * int(j), rc.kmax) + 1, 2))
        for i, j in enumerate(mol.j_lev):
            assert abs(pp[node - 1, 2 * i] - rho[ca[i]]) <= 1e-10 * abs(rho[ca[i]])
            if j:
                assert abs(pp[node - 1, 2 * i + 1] - rho[ca[i] + 1]) <= 1e-9 * abs(rho[ca[i]])


def _tiny_problem(n=512, seed=3, nlev=5, **kw):
    mol = synth.linear_rotor(nlev)
    cloud = synth.power_law_sphere(n, seed, mol, **kw)
    return cloud, mol


def test_se_limits_isotropic_and_collisional():
    """J^2 = 0 => rho^2_0 = 0; huge density => Boltzmann populations at T_kin;
    normalisation sum sqrt(2J+1) rho^0_0 = 1 (em_coefs.f90:158-164)."""
    cloud, mol = _tiny_problem(64, t_uniform=20.0)
    P = oracle.OracleProblem(cloud, mol)
    N, R = cloud.node_num, mol.r_num
    nu = mol.nu
    bb = np.array([oracle.black_body(2.73, v) for v in nu])
    J0 = np.tile(bb, (N, 1)); J2 = np.zeros((N, R))
    pp, st, nf = P.solve_se(6, J0, J2)
    g = 2 * mol.j_lev + 1
    np.testing.assert_allclose((pp[:, 0::2] * np.sqrt(g)).sum(1), 1.0, rtol=1e-12)
    assert np.abs(pp[:, 1::2]).max() <= 1e-12 * np.abs(pp[:, 0::2]).max()
    # collision dominated: n_H2 -> 1e14 cm^-3
    cloud.h2_dens[:] = 1e20
    P2 = oracle.OracleProblem(cloud, mol)
    pp2, _, _ = P2.solve_se(6, J0, J2)
    N_J = pp2[:, 0::2] * np.sqrt(g)
    ek = mol.e_levs * 4.79924e-11                         # h nu / k in K, the reference constant
    boltz = g * np.exp(-ek / 20.0)
    boltz /= boltz.sum()
    np.testing.assert_allclose(N_J, np.tile(boltz, (N, 1)), rtol=1e-6)


def test_optically_thin_limit_gives_cmb():
    """Vanishing populations: every ray returns the CMB, and J^0_0 equals
    B_nu(2.73 K) times the channel quadrature of the profile (inverse_rt.f90:
    275-339 sums phi dv over +-2 b, ~erf(2)); J^2_0 vanishes."""
    cloud, mol = _tiny_problem(256)
    cloud.lev_p *= 1e-30
    rc = synth.RunConfig(nth=8, nph=8, nvel=8, kmax=6, gvec=synth.gauge_vector(0))
    P = oracle.OracleProblem(cloud, mol)
    J0, J2, st, nseg, nf = P.radiation_field(rc, 1, 32)
    q = 2.0 * np.arange(-rc.nvel, rc.nvel + 1) / rc.nvel
    quad = (np.exp(-q * q) * 2.0 / (math.sqrt(math.pi) * rc.nvel)).sum()
    bb = np.array([oracle.black_body(2.73, v) for v in mol.nu])
    np.testing.assert_allclose(J0[:32], np.tile(bb * quad, (32, 1)), rtol=1e-9)
    assert np.abs(J2[:32]).max() < 1e-12 * J0[:32].max()


def test_walk_covers_ray_to_sphere():
    """Every walk ends on the unit sphere: the cumulative steps equal the
    exit distance / dx (to the rounding of each segment)."""
    import ctypes as C
    cloud, mol = _tiny_problem(2048)
    P = oracle.OracleProblem(cloud, mol)
    L = oracle.lib()
    dl = np.zeros(2 * 20001, dtype=np.int32)
    nc = C.c_int(0)
    rng = np.random.default_rng(0)
    dx = synth.F4(1e-6)
    for node in rng.integers(1, cloud.node_num + 1, size=50):
        d = rng.normal(size=3); d /= np.linalg.norm(d)
        st = L.orc_trace_out(C.byref(P.c), int(node), d.ctypes.data_as(oracle.P_D), C.c_double(dx), 20000,
                             dl.ctypes.data_as(oracle.P_I), C.byref(nc))
        assert st == 0
        n = nc.value
        X = cloud.xyz[node - 1]
        b = X @ d; cq = X @ X - 1.0
        s_exit = -b + math.sqrt(b * b - cq)
        assert abs(dl[2 * (n - 1) + 1] * dx - s_exit) <= (n + 1) * 0.5 * dx + 1e-12
        assert dl[2 * n] == 0 and all(dl[2 * i] > 0 for i in range(n))


def test_polarize_prop_against_rk4():
    """polarize_prop (raytrace.f90:1-56) against an RK4 integration of
    dI/ds = -eta_I I - eta_Q Q + eps_I, dQ/ds = -eta_Q I - eta_I Q + eps_Q."""
    import ctypes as C
    L = oracle.lib()
    L.orc_polarize_prop.restype = None
    L.orc_polarize_prop.argtypes = [C.c_double] * 5 + [oracle.P_D] * 3
    for (eI, eQ, sI, sQ, ds) in [(2.0, 0.5, 1.0, 0.1, 0.7), (0.3, -0.2, 0.5, 0.05, 3.0), (5.0, 1.0, 2.0, -0.3, 0.2)]:
        I, Q, U = C.c_double(0.4), C.c_double(-0.1), C.c_double(0.2)
        L.orc_polarize_prop(eI, eQ, sI, sQ, ds, C.byref(I), C.byref(Q), C.byref(U))
        y = np.array([0.4, -0.1]); h = ds / 4000
        f = lambda v: np.array([-eI * v[0] - eQ * v[1] + sI, -eQ * v[0] - eI * v[1] + sQ])
        for _ in range(4000):
            k1 = f(y); k2 = f(y + h / 2 * k1); k3 = f(y + h / 2 * k2); k4 = f(y + h * k3)
            y = y + h / 6 * (k1 + 2 * k2 + 2 * k3 + k4)
        np.testing.assert_allclose([I.value, Q.value], y, rtol=1e-9)
        assert abs(U.value - 0.2 * math.exp(-eI * ds)) < 1e-14


def test_node_maps_start_points_and_einstein_a():
    """The per-node mode (pix_mod = 0, para_finish.f90:245-350): the xy rows
    are tx times the rotated positions R_z(ph_az) R_x(th_inc) X of the bulk
    nodes; with the transitions listed in reverse, line (1, 2) radiates with
    t_Aji(1) = the top transition's A (:303), so its intensities differ from
    the same molecule listed in order; a line (1, 3), whose w^(2) vanish on
    both levels, has eta_Q = 0 and NaN I, Q, U (polarize_prop's 0/0) but a
    finite tau, while the pixel mode gives it A = 0 and zeros."""
    import dataclasses
    cloud, mol = _tiny_problem(512)
    rmol = dataclasses.replace(mol, r_trans=mol.r_trans[::-1].copy(), A=mol.A[::-1].copy(),
                               freq_ghz=mol.freq_ghz[::-1].copy(), nu=mol.nu[::-1].copy(),
                               Bij=mol.Bij[::-1].copy(), kd_v=mol.kd_v[::-1].copy())
    pp = np.zeros((cloud.node_num, 2 * mol.nlev))
    g = np.sqrt(2.0 * mol.j_lev + 1.0)
    pp[:, 0::2] = cloud.lev_p / cloud.lev_p.sum(axis=1, keepdims=True) / g
    pp[:, 1::2] = 1e-3 * pp[:, 0::2]
    th, ph = 0.6, 0.3
    outs = {}
    for name, m in (("ordered", mol), ("reversed", rmol)):
        P = oracle.OracleProblem(cloud, m)
        out, xy, st, nf = P.image_nodes([1, 1], [2, 3], pp, th, ph, 4, 80.0, 0.0, node_lo=0, node_hi=63)
        assert nf == 0 and not st[:64].any()
        outs[name] = out[:, :64]
    ct, sn = math.cos(th), math.sin(th)
    Rx = np.array([[1, 0, 0], [0, ct, -sn], [0, sn, ct]])
    cp, sp = math.cos(ph), math.sin(ph)
    Rz = np.array([[cp, -sp, 0], [sp, cp, 0], [0, 0, 1]])
    X = cloud.xyz[:cloud.bulk_node_num] @ (Rz @ Rx).T
    np.testing.assert_allclose(xy, cloud.tx * X[:, :2], rtol=0, atol=1e-14 * cloud.tx)
    a, b = outs["ordered"][0, :, 0], outs["reversed"][0, :, 0]
    assert np.isfinite(a).all() and np.isfinite(b).all()
    assert np.abs(a - b).max() > 1e-3 * np.abs(a).max()
    line13 = outs["reversed"][:, :, 1]
    assert np.isnan(line13[:3]).all() and np.isfinite(line13[3]).all() and line13[3].max() > 0.0
    P = oracle.OracleProblem(cloud, mol)
    pix, _, _ = P.image([1, 1], [2, 3], pp, th, ph, 4, 80.0, 0.0, 2, 0.5)
    assert np.abs(pix[0, :, 1]).max() == 0.0 and np.abs(pix[0, :, 0]).max() > 0.0


@pytest.mark.parametrize("nth,nph,dist", [(8, 8, 3.0), (16, 16, 1.5), (12, 12, 40.0), (16, 16, 1.05), (6, 6, 8.0)])
def test_star_all_ray_sets(nth, nph, dist):
    """star_all (miscellaneous.f90:1139-1226): the weights of a node's rays
    sum to one, the star's cone carries dOm / 4 pi with dOm = pi (R / d)^2,
    and the cone's rays point within th_star of the star (one ray: the
    reference's cos(1) stand-in, 1 rad off); the count stays within nth*nph."""
    rng = np.random.default_rng(nth + nph)
    b = rng.normal(size=3); b /= np.linalg.norm(b)
    k = rng.normal(size=3); k /= np.linalg.norm(k)
    g = np.asarray(synth.gauge_vector(3), dtype=np.float64)
    dOm = math.pi / dist ** 2
    xth, n_star = oracle.star_all(nth, nph, k, g, b, dOm)
    assert 1 <= n_star < len(xth) <= nth * nph
    np.testing.assert_allclose(xth[:, 2].sum(), 1.0, rtol=1e-13)
    np.testing.assert_allclose(xth[:n_star, 2].sum(), dOm / (4 * math.pi), rtol=1e-13)
    th_star = math.acos(1 - dOm / (2 * math.pi))
    d = np.zeros(3)
    L = oracle.lib()
    for mu, ph, _ in xth[:n_star]:
        L.orc_find_dir(b.ctypes.data_as(oracle.P_D), g.ctypes.data_as(oracle.P_D), C.c_double(math.acos(mu)),
                       C.c_double(ph), d.ctypes.data_as(oracle.P_D))
        ang = math.acos(min(1.0, float(d @ k)))
        if n_star == 1:
            assert abs(ang - 1.0) < 1e-9
        else:
            assert ang <= th_star + 1e-9


def test_star_mode_node_loop_skips_the_star_and_ends_rays_on_it():
    """Star mode in the oracle's node loop (main_para.f90:216-246): nodes
    inside the star get J = 0 and no populations; the star rays of a node
    just outside end on the star, so its walk is shorter than without the
    star, and B(T_star) raises its field."""
    cloud, mol = _tiny_problem(512)
    rc = synth.RunConfig(nth=8, nph=8, nvel=8, kmax=2, gvec=synth.gauge_vector(1))
    R = 0.08
    P0 = oracle.OracleProblem(cloud, mol)
    Ps = oracle.OracleProblem(cloud, mol, star=(3000.0, R * cloud.tx, (0.0, 0.0, 0.0)))
    r = np.linalg.norm(cloud.xyz, axis=1)
    inside = np.where(r[:64] <= R)[0]
    near = np.where((r[:64] > R) & (r[:64] < 2 * R))[0]
    assert len(inside) and len(near)
    J0, J2, st, nseg, nf = Ps.radiation_field(rc, 1, 64)
    J0n, _, _, nseg_n, _ = P0.radiation_field(rc, 1, 64)
    assert nf == 0 and not st[:64].any()
    assert (J0[inside] == 0).all() and (J2[inside] == 0).all()
    pp, _, _ = Ps.solve_se(rc.kmax, J0, J2, 1, 64)
    assert (pp[inside] == 0).all() and (pp[near] != 0).any()
    assert (J0[near, 0] > J0n[near, 0]).all()


def test_star_mode_image_starts_on_the_disc():
    """raytrace.f90:103-115: pixels within R_star of the star's sky position
    start at its front (less optical depth behind them, B(T_star) as the
    input); every other pixel is the star-less image exactly."""
    cloud, mol = _tiny_problem(512)
    pp = np.zeros((cloud.node_num, 2 * mol.nlev))
    g = np.sqrt(2.0 * mol.j_lev + 1.0)
    pp[:, 0::2] = cloud.lev_p / cloud.lev_p.sum(axis=1, keepdims=True) / g
    pp[:, 1::2] = 1e-3 * pp[:, 0::2]
    R = 0.15
    P0 = oracle.OracleProblem(cloud, mol)
    Ps = oracle.OracleProblem(cloud, mol, star=(3000.0, R * cloud.tx, (0.0, 0.0, 0.0)))
    im_pix, size = 4, 0.6
    a, _, nf0 = P0.image([1], [2], pp, 0.4, 0.2, 3, 80.0, 0.0, im_pix, size)
    b, _, nf1 = Ps.image([1], [2], pp, 0.4, 0.2, 3, 80.0, 0.0, im_pix, size)
    assert nf0 == 0 and nf1 == 0
    npx = 2 * im_pix + 1
    ij = np.array([(i - im_pix, j - im_pix) for i in range(npx) for j in range(npx)]) * size / im_pix
    on = np.hypot(ij[:, 0], ij[:, 1]) < R
    assert on.sum() == 1 and (~on).sum() == npx * npx - 1
    np.testing.assert_array_equal(a[:, ~on], b[:, ~on])
    assert (b[3, on] < a[3, on]).all()          # tau: the ray starts at the star's front


def _rodrigues(n, th):
    """rotmat (miscellaneous.f90:146-181): rotation by th about the unit n."""
    c, s = math.cos(th), math.sin(th)
    x, y, z = n
    return np.array([[c + (1 - c) * x * x, x * y * (1 - c) - z * s, x * z * (1 - c) + y * s],
                     [y * x * (1 - c) + z * s, c + (1 - c) * y * y, y * z * (1 - c) - x * s],
                     [z * x * (1 - c) - y * s, z * y * (1 - c) + x * s, c + (1 - c) * z * z]])


@pytest.mark.parametrize("dust", [False, True])
def test_node_field_against_an_independent_numpy_restatement(dust):
    """J^0_0 and J^2_0 of a few nodes from the oracle's inverse_rt against a
    separate numpy restatement written from inverse_rt.f90:1-137 and ray_in
    :217-344 (find_dir by explicit rotation matrices, the channel loop
    vectorised), with and without dust, on the oracle's own walks: the two
    agree to 1e-12."""
    import ctypes as C
    cloud, mol = _tiny_problem(384, t_law="loglinear", b_random=0.3)
    if dust:
        cloud.dust_p = cloud.h2_dens * synth.F4(2.32e-27) / 100.0
        cloud.t_dust = cloud.t_kin * 0.8
    rc = synth.RunConfig(nth=6, nph=6, nvel=6, kmax=2, gvec=synth.gauge_vector(2))
    P = oracle.OracleProblem(cloud, mol)
    J0, J2, st, _, nf = P.radiation_field(rc, 1, 12)
    assert nf == 0
    L = oracle.lib()
    xth = oracle.legendre_all(rc.nth, rc.nph)
    g = np.asarray(rc.gvec, dtype=np.float64)
    dx = rc.dx
    tdx = cloud.tx * dx
    dl = np.zeros(2 * (rc.n_depth + 2), dtype=np.int32)
    nc = C.c_int(0)
    spi = math.sqrt(math.pi)
    nvel = rc.nvel
    for node in range(1, 13):
        if not cloud.ab_all[node - 1] > 0:
            continue
        b = cloud.bvec[node - 1]
        xv = np.cross(b, g)
        xv /= np.linalg.norm(xv)
        j0 = np.zeros(mol.r_num)
        j2 = np.zeros(mol.r_num)
        for mu, ph, w in xth:
            d = _rodrigues(b, ph) @ (_rodrigues(xv, math.acos(mu)) @ b)
            stt = L.orc_trace_out(C.byref(P.c), node, d.ctypes.data_as(oracle.P_D), C.c_double(dx), rc.n_depth,
                                  dl.ctypes.data_as(oracle.P_I), C.byref(nc))
            assert stt == 0
            n = nc.value
            cells = dl[0:2 * n:2] - 1
            steps = dl[1:2 * n:2].astype(np.float64)
            v_ray = cloud.vel[cells] @ d
            v_node = cloud.vel[node - 1] @ d
            c_in = (3.0 * mu * mu - 1.0) / 2.0
            for k in range(mol.r_num):
                lo, up = mol.r_trans[k] - 1
                g1, g2 = 2 * mol.j_lev[lo] + 1, 2 * mol.j_lev[up] + 1
                nu0 = mol.nu[k]
                c1, c2, cnu = 2.2102191e-42 * nu0, 5.272859e-35 * nu0, 299792458.0 / nu0
                kv = c1 * mol.Bij[k] * (cloud.lev_p[cells, lo] - g1 * cloud.lev_p[cells, up] / g2)
                ev = c2 * mol.A[k] * cloud.lev_p[cells, up]
                bn = cloud.b_all[node - 1]
                nv = np.arange(-nvel, nvel + 1)
                v0 = 2.0 * bn * nv / nvel
                phi0 = np.exp(-(v0 / bn) ** 2) / (spi * bn)
                v0 = v0 + v_node
                I = np.full(nv.shape, oracle.black_body(2.73, nu0))
                al = mol.kd_v[k] * cloud.dust_p[cells]                     # dust opacity
                jd = al * np.array([oracle.black_body(cloud.t_dust[c], nu0) for c in cells])
                for i in range(n - 1, 0, -1):          # cells node_count .. 2
                    bi = cloud.b_all[cells[i]]
                    phi = cnu * np.exp(-((v0 - v_ray[i]) / bi) ** 2) / (spi * bi)
                    tau = (kv[i] * phi + al[i]) * tdx * (steps[i] - steps[i - 1])
                    upd = tau > 1e-30
                    with np.errstate(divide="ignore", invalid="ignore"):
                        S = (ev[i] * phi + jd[i]) / (kv[i] * phi + al[i])
                    I = np.where(upd, I * np.exp(-tau) + S * (1.0 - np.exp(-tau)), I)
                phin = phi0 * cnu
                taun = (kv[0] * phin + al[0]) * tdx * steps[0]
                Sn = (ev[0] * phin + jd[0]) / (kv[0] * phin + al[0])
                Iout = I * np.exp(-taun) + Sn * (1.0 - np.exp(-taun))
                Ibar = np.sum(phi0 * Iout * (2.0 * bn / nvel))
                j0[k] += Ibar * w
                j2[k] += Ibar * w * c_in / math.sqrt(2.0)
        np.testing.assert_allclose(j0, J0[node - 1], rtol=1e-12)
        np.testing.assert_allclose(j2, J2[node - 1], rtol=1e-9, atol=1e-12 * np.abs(j0).max())


def test_image_pixels_against_an_independent_numpy_restatement():
    """I, Q, U, tau of image pixels from the oracle's finish_portal loop
    against a second, numpy restatement written from para_finish.f90:222-240
    (population read-back), rotate_all_save, comp_emcoefs (em_coefs.f90:1-113),
    ray_in_raytrace (raytrace.f90:179-323) with rot_stokes / rot_stokes_back
    and polarize_prop, on the oracle's marches: equal to 1e-11 of the peak."""
    import ctypes as C
    cloud, mol = _tiny_problem(512, t_law="loglinear", b_random=0.4)
    N, nlev = cloud.node_num, mol.nlev
    rng = np.random.default_rng(3)
    g = np.sqrt(2.0 * mol.j_lev + 1.0)
    pp_in = np.zeros((N, 2 * nlev))
    pp_in[:, 0::2] = cloud.lev_p / cloud.lev_p.sum(axis=1, keepdims=True) / g
    pp_in[:, 1::2] = pp_in[:, 0::2] * rng.uniform(-0.02, 0.02, size=(N, nlev))
    P = oracle.OracleProblem(cloud, mol)
    th_inc, ph_az, nvel, dvel, v0, im_pix, size = 0.7, 0.4, 4, 90.0, 10.0, 3, 0.6
    out, st, nf = P.image([1], [2], pp_in, th_inc, ph_az, nvel, dvel, v0, im_pix, size)
    assert nf == 0
    # rotate_all_save miscellaneous.f90:844-907: x' = R_z(ph) R_x(th) x
    R = _rodrigues((0.0, 0.0, 1.0), ph_az) @ _rodrigues((1.0, 0.0, 0.0), th_inc)
    X, V, B = cloud.xyz @ R.T, cloud.vel @ R.T, cloud.bvec @ R.T
    # read-back para_finish.f90:226-239
    pp = pp_in.copy()
    pp[:, 0] = cloud.lev_p[:, 0] / g[0]
    for i in range(1, nlev):
        rat = pp_in[:, 2 * i + 1] / pp_in[:, 2 * i]
        pp[:, 2 * i + 1] = rat * cloud.lev_p[:, i] / g[i]
        pp[:, 2 * i] = cloud.lev_p[:, i] / g[i]
    # comp_emcoefs of line (1, 2) for the bulk nodes with pp(:,1) != 0
    j1, j2 = int(mol.j_lev[0]), int(mol.j_lev[1])
    nu0 = mol.e_levs[1] - mol.e_levs[0]
    Aji = mol.A[0]
    fas = (-1.0) ** (1 + j1 + j2)
    w1 = fas * math.sqrt(3.0 * (2 * j1 + 1)) * oracle.wigner6j(2, 2, 4, 2 * j1, 2 * j1, 2 * j2)
    w2 = fas * math.sqrt(3.0 * (2 * j2 + 1)) * oracle.wigner6j(2, 2, 4, 2 * j2, 2 * j2, 2 * j1)
    g1, g2 = 2.0 * j1 + 1, 2.0 * j2 + 1
    coef = np.zeros((N, 4))
    for n in range(cloud.bulk_node_num):
        if pp[n, 0] == 0.0:
            continue
        th = math.acos(B[n, 2])
        tki = (3.0 * math.cos(th) ** 2 - 1.0) / (2.0 * math.sqrt(2.0))
        tkq = -3.0 * math.sin(th) ** 2 / (2.0 * math.sqrt(2.0))
        r10, r20, r12, r22 = pp[n, 0], pp[n, 2], pp[n, 1], pp[n, 3]
        naI, naQ = 1.0 + w1 * (r12 / r10) * tki, w1 * (r12 / r10) * tkq
        nsI, nsQ = 1.0 + w2 * (r22 / r20) * tki, w2 * (r22 / r20) * tkq
        Bji = Aji / (nu0 ** 3 / 6.781962e49)
        hv = 5.273e-35 * nu0
        coef[n] = [hv * (g2 / g1) * Bji * (math.sqrt(g1) * r10 * naI - math.sqrt(g2) * r20 * nsI * g1 / g2),
                   hv * (g2 / g1) * Bji * (math.sqrt(g1) * r10 * naQ - math.sqrt(g2) * r20 * nsQ * g1 / g2),
                   hv * Aji * nsI * math.sqrt(g2) * r20, hv * Aji * nsQ * math.sqrt(g2) * r20]
    L = oracle.lib()
    L.orc_trace_out_raytrace.restype = C.c_int
    dx = synth.F4(1e-4)
    Xf = np.ascontiguousarray(X, dtype=np.float64)
    dl = np.zeros(2 * 10002, dtype=np.int32)
    nc = C.c_int(0)
    cnu = synth.F4(2.99792e8) / nu0
    I_cmb = oracle.black_body(2.73, nu0)
    npx = 2 * im_pix + 1
    peak = np.abs(out[0]).max()
    for p in (0, 5, 17, 24, 40):
        a, b2 = p // npx - im_pix, p % npx - im_pix
        x, y = a * size / im_pix, b2 * size / im_pix
        assert L.orc_trace_out_raytrace(C.c_double(x), C.c_double(y), N, Xf.ctypes.data_as(oracle.P_D),
                                        P.c.del_ne, P.c.del_num_ne, P.c.maxne, C.c_double(dx), 10000,
                                        dl.ctypes.data_as(oracle.P_I), C.byref(nc)) == 0
        n = nc.value
        cells, steps = dl[0:2 * n:2] - 1, dl[1:2 * n:2]
        vobs = np.arange(-nvel, nvel + 1) * dvel + v0
        I = np.full(vobs.shape, I_cmb)
        Qi, Ui, tau = np.zeros_like(I), np.zeros_like(I), np.zeros_like(I)
        for i in range(n - 1):
            c = cells[i]
            vc = np.exp(-((vobs - V[c, 2]) ** 2) / cloud.b_all[c] ** 2) / (cloud.b_all[c] * math.sqrt(math.pi))
            ch = np.array([B[c, 0], B[c, 1]]) / math.hypot(B[c, 0], B[c, 1])
            al = math.acos(ch[1]) * (-1.0 if ch[0] > 0.0 else 1.0)
            c2a, s2a = math.cos(2 * al), math.sin(2 * al)
            Q, U = Qi * c2a + Ui * s2a, Ui * c2a - Qi * s2a          # rot_stokes
            eI, eQ, sI, sQ = (cnu * vc * coef[c, q] for q in range(4))
            ds = cloud.tx * dx * (steps[i + 1] - steps[i])
            go = ds * eI > 1e-30
            shQ, chQ, et = np.sinh(eQ * ds), np.cosh(eQ * ds), np.exp(-eI * ds)
            with np.errstate(divide="ignore", invalid="ignore"):
                fac = 1.0 / (eI ** 2 - eQ ** 2)
                o11 = fac * eI * (1.0 - (chQ + (eQ / eI) * shQ) * et)
                o12 = -fac * eQ * (1.0 - (chQ + (eI / eQ) * shQ) * et)
            In = o11 * sI + o12 * sQ + et * (chQ * I - shQ * Q)
            Qn = o12 * sI + o11 * sQ + et * (-shQ * I + chQ * Q)
            I, Q, U = np.where(go, In, I), np.where(go, Qn, Q), np.where(go, U * et, U)
            tau = np.where(go, tau + eI * ds, tau)
            Qi, Ui = Q * c2a - U * s2a, U * c2a + Q * s2a              # rot_stokes_back
        got = out[:4, p, 0]
        for q, want in enumerate((I - I_cmb, Qi, Ui)):
            np.testing.assert_allclose(got[q], want, rtol=0, atol=1e-11 * peak)
        np.testing.assert_allclose(got[3], tau, rtol=1e-12, atol=1e-300)


@pytest.mark.parametrize("kmax", [0, 6])
def test_se_without_anisotropy_is_the_scalar_rate_equations(kmax):
    """With J^2_0 = 0 the polarized SE (setup_stateq pop_eqs.f90:361-653 on
    make_AC's rates) must give the textbook statistical equilibrium: level
    populations n_J = sqrt(2J+1) rho^0_0 from A_ul + B_ul J, B_lu J
    (B_lu = g_u/g_l B_ul, B_ul = 6.781962e49 A / nu^3) and collisions C_ul,
    C_lu = C_ul g_u/g_l exp(-h nu / k T), the rate table interpolated
    linearly in T; rho^2_0 = 0.  An independent numpy build of that scalar
    system, solved by numpy, equals the oracle to 1e-13.  (With kmax = 0 the
    alignment columns of the packing, rhovec(count_array(i) + 2) in
    main_sub.f90:116-135, hold the next level's rho^0_0, as in the
    reference, so they are checked for kmax >= 2 only.)"""
    mol = synth.linear_rotor(6)
    cloud = synth.power_law_sphere(64, 3, mol, t_law="loglinear")
    P = oracle.OracleProblem(cloud, mol)
    N, R = cloud.node_num, mol.r_num
    rng = np.random.default_rng(kmax)
    bb = np.array([oracle.black_body(30.0, v) for v in mol.nu])
    J0 = np.tile(bb, (N, 1)) * rng.uniform(0.01, 2.0, size=(N, R))
    pp, st, nf = P.solve_se(kmax, J0, np.zeros((N, R)))
    assert nf == 0
    g = 2 * mol.j_lev + 1
    ct = mol.col_temps
    for node in range(0, cloud.bulk_node_num, 7):
        T, nH2 = cloud.t_kin[node], cloud.h2_dens[node]
        Rm = np.zeros((mol.nlev, mol.nlev))          # Rm[i, j]: rate from level i to level j
        for k in range(R):
            lo, up = mol.r_trans[k] - 1
            nu = mol.e_levs[up] - mol.e_levs[lo]
            B21 = 6.781962e49 * mol.A[k] / nu ** 3
            Rm[up, lo] += mol.A[k] + B21 * J0[node, k]
            Rm[lo, up] += g[up] / g[lo] * B21 * J0[node, k]
        for k in range(mol.c_num):
            lo, up = mol.c_trans[k] - 1
            nu = mol.e_levs[up] - mol.e_levs[lo]
            C21 = float(np.interp(T, ct, mol.C[0, k])) * nH2 * 1e-6
            Rm[up, lo] += C21
            Rm[lo, up] += C21 * g[up] / g[lo] * math.exp(-4.79924e-11 * nu / T)
        M = Rm.T - np.diag(Rm.sum(axis=1))
        M[0, :] = 1.0
        rhs = np.zeros(mol.nlev)
        rhs[0] = 1.0
        n = np.linalg.solve(M, rhs)
        np.testing.assert_allclose(pp[node, 0::2] * np.sqrt(g), n, rtol=1e-13, atol=1e-16)
        if kmax >= 2:
            assert np.abs(pp[node, 1::2]).max() < 1e-14 * np.abs(pp[node, 0::2]).max()
        else:
            np.testing.assert_array_equal(pp[node, 3:-2:2], pp[node, 4::2])   # J >= 1 but the last
            assert pp[node, 1] == 0.0 and pp[node, -1] == 0.0


def test_image_dust_maps_against_an_independent_numpy_restatement():
    """The dust branch of ray_in_raytrace (raytrace.f90:268-290, :308-317:
    dust intensity, the sigma_0 / sigma_2 sums and the Q, U of aligned
    grains with alpha = 0.15, para_finish.f90:78) against a numpy
    restatement on the oracle's marches, for a cloud with dust (gas-to-dust
    100): the dust I, Q, U, tau to 1e-12 of their peaks."""
    import ctypes as C
    cloud, mol = _tiny_problem(384, t_law="loglinear", b_random=0.5)
    cloud.dust_p = cloud.h2_dens * synth.F4(2.32e-27) / 100.0
    cloud.t_dust = cloud.t_kin * 0.8
    N, nlev = cloud.node_num, mol.nlev
    g = np.sqrt(2.0 * mol.j_lev + 1.0)
    pp = np.zeros((N, 2 * nlev))
    pp[:, 0::2] = cloud.lev_p / np.maximum(cloud.lev_p.sum(axis=1, keepdims=True), 1e-300) / g
    pp[:, 1::2] = 1e-3 * pp[:, 0::2]
    P = oracle.OracleProblem(cloud, mol)
    th_inc, ph_az, nvel, im_pix, size, alpha = 0.9, 0.3, 2, 3, 0.6, 0.15
    out, st, nf = P.image([1], [2], pp, th_inc, ph_az, nvel, 80.0, 0.0, im_pix, size, alpha=alpha)
    assert nf == 0 and np.abs(out[4]).max() > 0.0 and np.abs(out[5]).max() > 0.0
    R = _rodrigues((0.0, 0.0, 1.0), ph_az) @ _rodrigues((1.0, 0.0, 0.0), th_inc)
    X, B = cloud.xyz @ R.T, cloud.bvec @ R.T
    nu0 = mol.e_levs[1] - mol.e_levs[0]
    kd = mol.kd_v[0]
    L = oracle.lib()
    dx = synth.F4(1e-4)
    Xf = np.ascontiguousarray(X, dtype=np.float64)
    dl = np.zeros(2 * 10002, dtype=np.int32)
    nc = C.c_int(0)
    I_cmb = oracle.black_body(2.73, nu0)
    npx = 2 * im_pix + 1
    peaks = [np.abs(out[q]).max() for q in range(4, 8)]
    for p in (0, 10, 24, 31, 48):
        a, b2 = p // npx - im_pix, p % npx - im_pix
        assert L.orc_trace_out_raytrace(C.c_double(a * size / im_pix), C.c_double(b2 * size / im_pix), N,
                                        Xf.ctypes.data_as(oracle.P_D), P.c.del_ne, P.c.del_num_ne, P.c.maxne,
                                        C.c_double(dx), 10000, dl.ctypes.data_as(oracle.P_I), C.byref(nc)) == 0
        n = nc.value
        cells, steps = dl[0:2 * n:2] - 1, dl[1:2 * n:2]
        Id, s0, s2, Qd, Ud, td = I_cmb, 0.0, 0.0, 0.0, 0.0, 0.0
        for i in range(n - 1):
            c = cells[i]
            tau_d = kd * cloud.dust_p[c] * cloud.tx * dx * (steps[i + 1] - steps[i])
            if tau_d > 1e-30:
                Ibb = oracle.black_body(cloud.t_dust[c], nu0)
                e = math.exp(-tau_d)
                mu2 = 1.0 - B[c, 2] * B[c, 2]
                sI, sQ = 0.5 * alpha * (mu2 - 2.0 / 3.0), alpha * mu2
                Id = Id * e + Ibb * (1 - e)
                s0 = s0 * e + Ibb * (1 - e)
                s2 = s2 * e + sI * Ibb * (1 - e)
                phi = math.acos(B[c, 1] / math.sqrt(B[c, 0] ** 2 + B[c, 1] ** 2))
                if B[c, 0] < 0.0:
                    phi = -phi
                Qd = Qd * e + sQ * Ibb * (1 - e) * math.cos(2 * phi)
                Ud = Ud * e + sQ * Ibb * (1 - e) * math.sin(2 * phi)
                td += tau_d
        Id -= I_cmb
        want = (Id, Id * Qd / (s0 - s2), Id * Ud / (s0 - s2), td) if Id != 0.0 else (0.0, 0.0, 0.0, 0.0)
        for q in range(4):
            np.testing.assert_allclose(out[4 + q, p, 0], want[q], rtol=0, atol=1e-12 * peaks[q])


def test_walks_against_an_independent_restatement():
    """trace_out / check_neigh_fast / pos_quadratic (inverse_rt.f90:139-214,
    miscellaneous.f90:1017-1098) restated in plain Python floats (the same
    IEEE operations in the same order: norm2 squared, left-to-right dot
    products, the REAL*4 1E-10 threshold, nint): the (cell, cumulative step)
    lists equal the oracle's bit for bit on 200 random rays."""
    import ctypes as C
    cloud, mol = _tiny_problem(1024)
    P = oracle.OracleProblem(cloud, mol)
    L = oracle.lib()
    X = [tuple(float(v) for v in row) for row in cloud.xyz]
    dne, dnn = cloud.del_ne(), cloud.del_num_ne()          # (maxne, N) and (N)
    thr = synth.F4(1e-10)
    dx = synth.F4(1e-6)
    rng = np.random.default_rng(7)
    dl = np.zeros(2 * 20002, dtype=np.int32)
    nc = C.c_int(0)

    def norm2(a, b, c):
        return math.sqrt(a * a + b * b + c * c)

    for _ in range(200):
        node = int(rng.integers(1, cloud.bulk_node_num + 1))
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        d = (float(d[0]), float(d[1]), float(d[2]))
        darr = np.array(d)
        assert L.orc_trace_out(C.byref(P.c), node, darr.ctypes.data_as(oracle.P_D), C.c_double(dx), 20000,
                               dl.ctypes.data_as(oracle.P_I), C.byref(nc)) == 0
        n = nc.value
        want = [(int(dl[2 * i]), int(dl[2 * i + 1])) for i in range(n)]
        # the restatement
        p = list(X[node - 1])
        cur, delta, out = node, 0.0, []
        while True:
            nd = norm2(*d)
            npn = norm2(*p)
            a_, b_, c_ = nd * nd, 2.0 * (p[0] * d[0] + p[1] * d[1] + p[2] * d[2]), npn * npn - 1.0
            dis = b_ * b_ - 4.0 * a_ * c_
            if dis > 0:
                r1 = (-b_ + math.sqrt(dis)) / (2.0 * a_)
                r2 = (-b_ - math.sqrt(dis)) / (2.0 * a_)
                delta = r2 if r2 > 0 else r1
            nxt = 0
            xc = X[cur - 1]
            e0 = (xc[0] - p[0], xc[1] - p[1], xc[2] - p[2])
            n4 = norm2(*e0)
            q4 = n4 * n4
            q5 = e0[0] * d[0] + e0[1] * d[1] + e0[2] * d[2]
            for s in range(int(dnn[cur - 1])):
                nb = int(dne[s, cur - 1])
                xn = X[nb - 1]
                e1 = (xn[0] - p[0], xn[1] - p[1], xn[2] - p[2])
                n1 = norm2(*e1)
                q1 = n1 * n1
                q2 = e1[0] * d[0] + e1[1] * d[1] + e1[2] * d[2]
                new_x = 0.5 * (q1 - q4) / (q2 - q5)
                if new_x > delta or new_x <= thr:
                    continue
                delta, nxt = new_x, nb
            p = [p[k] + delta * d[k] for k in range(3)]
            out.append([cur, int(math.floor(delta / dx + 0.5))])
            cur = nxt
            if nxt == 0:
                break
        for i in range(1, len(out)):
            out[i][1] += out[i - 1][1]
        assert [tuple(o) for o in out] == want


def test_image_marches_against_an_independent_restatement():
    """trace_out_raytrace (raytrace.f90:58-177) with check_neigh
    (miscellaneous.f90:1-46) restated in plain Python floats: the start
    node by the O(N) scan (strict <), then one 1e-4 step at a time, the exit
    at |P| > 1 and the nearest of the node and its neighbours (strict <, list
    order) after every step; the (node, step) lists equal the oracle's bit
    for bit."""
    import ctypes as C
    cloud, mol = _tiny_problem(512)
    P = oracle.OracleProblem(cloud, mol)
    L = oracle.lib()
    L.orc_trace_out_raytrace.restype = C.c_int
    X = [tuple(float(v) for v in row) for row in cloud.xyz]
    dne, dnn = cloud.del_ne(), cloud.del_num_ne()
    dx = synth.F4(1e-4)
    dl = np.zeros(2 * 10002, dtype=np.int32)
    nc = C.c_int(0)
    Xf = np.ascontiguousarray(cloud.xyz, dtype=np.float64)
    for x, y in ((0.0, 0.0), (0.31, -0.2), (-0.55, 0.4), (0.05, 0.66)):
        assert L.orc_trace_out_raytrace(C.c_double(x), C.c_double(y), cloud.node_num, Xf.ctypes.data_as(oracle.P_D),
                                        P.c.del_ne, P.c.del_num_ne, P.c.maxne, C.c_double(dx), 10000,
                                        dl.ctypes.data_as(oracle.P_I), C.byref(nc)) == 0
        want = [(int(dl[2 * i]), int(dl[2 * i + 1])) for i in range(nc.value)]
        z = -1.0 * math.sqrt(1.0 - x * x - y * y)
        rsave, node = 10.0, 0
        for i, c in enumerate(X):
            r = math.sqrt((x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2)
            if r < rsave:
                rsave, node = r, i + 1
        out, k = [], 0
        while True:
            z = z + dx
            k += 1
            done = math.sqrt(x * x + y * y + z * z) > 1.0
            if done:
                out.append((node, k))
            c = X[node - 1]
            d0 = (x - c[0]) * (x - c[0]) + (y - c[1]) * (y - c[1]) + (z - c[2]) * (z - c[2])
            new = node
            for s in range(int(dnn[node - 1])):
                nb = int(dne[s, node - 1])
                n_ = X[nb - 1]
                dd = (x - n_[0]) * (x - n_[0]) + (y - n_[1]) * (y - n_[1]) + (z - n_[2]) * (z - n_[2])
                if dd < d0:
                    d0, new = dd, nb
            if new != node:
                out.append((new, k))
                node = new
            if done:
                break
        assert out == want, (x, y)


@pytest.mark.parametrize("anis", [0.1, -0.3, 0.5])
def test_se_two_level_alignment_limit(anis):
    """The polarized SE in the two-level limit of Landi Degl'Innocenti &
    Landolfi (2004): a J = 0 -> 1 transition, collisions negligible and the
    radiation weak (B J / A = 1e-6, so stimulated emission is negligible)
    gives the upper level the alignment sigma^2_0 = rho^2_0 / rho^0_0 =
    w^(2)_{10} J^2_0 / J^0_0 with w^(2)_{10} = 1 (the unpolarized J = 0 lower
    level), to the O(B J / A) of stimulated emission."""
    import dataclasses
    mol = synth.linear_rotor(2)
    mol = dataclasses.replace(mol, C=mol.C * 1e-25)
    cloud = synth.power_law_sphere(64, 3, mol)
    P = oracle.OracleProblem(cloud, mol)
    N, R = cloud.node_num, mol.r_num
    nu, A = mol.nu[0], mol.A[0]
    B21 = 6.781962e49 * A / nu ** 3
    J0 = np.full((N, R), 1e-6 * A / B21)
    pp, st, nf = P.solve_se(2, J0, anis * J0)
    assert nf == 0
    w = 3.0 * oracle.wigner6j(2, 2, 4, 2, 2, 0)          # (-1)^2 sqrt(3) sqrt(3) {1 1 2; 1 1 0}
    assert w == pytest.approx(1.0, rel=1e-14)
    sig = pp[:cloud.bulk_node_num, 3] / pp[:cloud.bulk_node_num, 2]
    np.testing.assert_allclose(sig, w * anis, rtol=1e-5)


# ---- depolarising collisions (depol.f90:242-360) ---------------------------

def _depol_restated(mol, kmax):
    """de_polarization restated with sympy's exact Wigner symbols: D0_all
    [K/2 - 1, level, temperature], the rate out of level 1 to level m read
    where the reference reads it (C_j0(:, m), m = 1..2J; 0 for m = 1 and for
    m beyond the levels)."""
    wig = pytest.importorskip("sympy.physics.wigner")
    nlev, nT = mol.nlev, mol.c_temp
    Cj0 = np.zeros((nT, nlev + 1))
    for q in range(mol.c_num):
        lo, up = mol.c_trans[q]
        if lo == 1:
            Cj0[:, up] = mol.C[0, q]
    out = np.zeros((kmax // 2, nlev, nT))
    for i in range(2, nlev + 1):
        j = i - 1
        for k in range(2, min(2 * j, kmax) + 1, 2):
            for m in range(1, 2 * j + 1):
                w1 = float(wig.wigner_3j(j, j, m, 0, 0, 0))
                w2 = float(wig.wigner_6j(j, j, m, j, j, 0))
                w3 = float(wig.wigner_6j(j, j, m, j, j, k))
                cj = Cj0[:, m] if m <= nlev else 0.0
                out[k // 2 - 1, i - 1] += (2 * j + 1) ** 2 * (-1) ** m * (2 * m + 1) * w1 * w1 * (w2 - w3) * cj
    return out


def test_depolarization_coefficients_against_sympy():
    mol = synth.linear_rotor(7)
    got = oracle.de_polarization(mol, 6)
    want = _depol_restated(mol, 6)
    assert np.abs(want).max() > 1e-12
    np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-30)
    # J = 0 has no K >= 2 component; K above 2J gives nothing
    assert not got[:, 0].any() and not got[1:, 1].any()
    # the reference's own assumption, j_lev(i) = i - 1
    import dataclasses
    shifted = dataclasses.replace(mol, j_lev=mol.j_lev + 1)
    assert oracle.de_polarization(shifted, 6) is None


def test_depolarization_enters_the_se_only_when_switched_on():
    """mode 0 is the reference's run (D0 = 0); modes 1 and 2 change the
    alignment, mode 2 (col_dep carried to the later entries, as the
    reference's code reads it) the populations as well; the temperature
    interpolation is make_depolarization_temp's last bracket."""
    cloud, mol, rc = synth.config_cloud("sphere4k", n_points=1024)
    rc.nth = rc.nph = 8
    P0 = oracle.OracleProblem(cloud, mol)
    J0, J2, _, _, _ = P0.radiation_field(rc, 1, 32)
    p0 = P0.solve_se(rc.kmax, J0, J2, 1, 32)[0][:32]
    p1 = oracle.OracleProblem(cloud, mol, depol=1).solve_se(rc.kmax, J0, J2, 1, 32)[0][:32]
    p2 = oracle.OracleProblem(cloud, mol, depol=2).solve_se(rc.kmax, J0, J2, 1, 32)[0][:32]
    d1 = np.abs(p1[:, 1::2] - p0[:, 1::2]).max() / np.abs(p0[:, 1::2]).max()
    assert d1 > 1e-3                                   # the alignment is depolarised
    assert np.all(np.abs(p1[:, 1::2]) <= np.abs(p0[:, 1::2]) * (1 + 1e-9) + 1e-300)
    assert np.abs(p2 - p1).max() > 1e-6 * np.abs(p1).max()
    # make_depolarization_temp at T: the last bracket, times n_H2 1e-6
    D = oracle.de_polarization(mol, rc.kmax)
    T, nH2 = 20.0, 3e10
    tt = mol.col_temps
    f = (T - tt[-2]) / (tt[-1] - tt[-2])
    want = (D[..., -2] + f * (D[..., -1] - D[..., -2])) * nH2 * 1e-6
    got = np.zeros(D.shape[:2])          # D0(nlev, kmax/2) column-major == (kmax/2, nlev)
    oracle.lib().orc_make_depolarization_temp(oracle._p(np.ascontiguousarray(D)), mol.nlev, mol.c_temp, rc.kmax,
                                              oracle._p(np.ascontiguousarray(tt)), C.c_double(T), C.c_double(nH2),
                                              oracle._p(got))
    np.testing.assert_allclose(got, want, rtol=1e-14)
