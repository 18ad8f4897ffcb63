"""The drop-in executables main_portal.x / finish_portal.x: file parsing on the
CPU (parse-only dump), and the whole file -> GPU -> file path on the GPU."""
import math
import os
import subprocess

import numpy as np
import pytest

from portal_gb300 import lime, synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
MAIN = os.path.join(ROOT, "portal_gb300", "_build", "main_portal.x")
FINISH = os.path.join(ROOT, "portal_gb300", "_build", "finish_portal.x")


@pytest.fixture(scope="module")
def case(tmp_path_factory, built_lib):
    d = str(tmp_path_factory.mktemp("portal_case"))
    mol = synth.linear_rotor(5)
    cloud = synth.power_law_sphere(2000, 3, mol, keep_raw=True)
    rc = synth.RunConfig(nth=8, nph=8, nvel=16, kmax=6, gvec=synth.gauge_vector(3))
    paths = lime.write_case(d, cloud, mol)
    lime.write_main_input(os.path.join(d, "pol.dat"), rc, extra_info=1)
    return dict(d=d, mol=mol, cloud=cloud, rc=rc, paths=paths)


def _run(exe, case, env_extra, input_name="pol.dat"):
    p = case["paths"]
    env = dict(os.environ, **env_extra)
    return subprocess.run([exe, os.path.join(case["d"], input_name), case["d"], p["pop"], p["grid"], p["mol"],
                           p["dust"]], env=env, capture_output=True, text=True, timeout=600)


def _npy(d, name):
    return np.load(os.path.join(d, name + ".npy"))


def test_ingestion_matches_python_restatement(case):
    """eat_lime_no_delaunay + main_para.f90:119-185 from the files (C++)
    equal the same transforms applied in memory (Python)."""
    dd = os.path.join(case["d"], "dump_b")
    os.makedirs(dd, exist_ok=True)
    r = _run(MAIN, case, dict(PORTAL_DUMP_INGESTED=dd, PORTAL_BVEC_FILE=case["paths"]["bvec"]))
    assert r.returncode == 0, r.stderr
    cloud, mol = case["cloud"], case["mol"]
    np.testing.assert_array_equal(_npy(dd, "xyz"), cloud.xyz.ravel())
    np.testing.assert_array_equal(_npy(dd, "vel"), cloud.vel.ravel())
    np.testing.assert_array_equal(_npy(dd, "b_all"), cloud.b_all)
    np.testing.assert_array_equal(_npy(dd, "lev_p"), cloud.lev_p.ravel())
    np.testing.assert_array_equal(_npy(dd, "bvec"), cloud.bvec.ravel())
    np.testing.assert_array_equal(_npy(dd, "del_ne"), cloud.del_ne().ravel())
    np.testing.assert_array_equal(_npy(dd, "del_num_ne"), cloud.del_num_ne())
    for name in ("e_levs", "nu", "A", "Bij", "kd_v"):
        np.testing.assert_array_equal(_npy(dd, name), getattr(mol, name))
    sc = _npy(dd, "scalars")
    assert sc[0] == cloud.tx and int(sc[1]) == cloud.bulk_node_num and sc[3] == mol.mass


def test_input_file_line_shift_is_reproduced(case):
    """main_para.f90:77 reads x1..x_dip starting on the dust_ii_gas line of
    the file run_portal.sh writes, so x1 = dust_ii_gas, x2 = b_rad,
    x3 = b_tor, x_dip = b_pol (b_dip is never read): with the field line
    "0 1 0 1.d0" the field is global_magfield(0.01, 0, 1)."""
    dd = os.path.join(case["d"], "dump_g")
    os.makedirs(dd, exist_ok=True)
    r = _run(MAIN, case, dict(PORTAL_DUMP_INGESTED=dd))
    assert r.returncode == 0, r.stderr
    b = _npy(dd, "bvec").reshape(-1, 3)
    x = case["cloud"].xyz
    rad = x / np.linalg.norm(x, axis=1, keepdims=True)
    pol = np.stack([x[:, 2] * x[:, 0], x[:, 1] * x[:, 2], -(x[:, 1] ** 2 + x[:, 0] ** 2)], axis=1)
    pol /= np.linalg.norm(pol, axis=1, keepdims=True)
    ref = 0.01 * rad + 1.0 * pol
    ref /= np.linalg.norm(ref, axis=1, keepdims=True)
    np.testing.assert_allclose(b, ref, rtol=0, atol=1e-14)


def _copy_case(case, tmp_path):
    import shutil
    d = str(tmp_path)
    for name in ("model.pop", "grid.vtk", "molecule.dat", "dust.tab", "bvec.dat", "pol.dat"):
        shutil.copy(os.path.join(case["d"], name), d)
    return dict(case, d=d, paths={k: os.path.join(d, os.path.basename(v)) for k, v in case["paths"].items()})


def _edit_line(path, lineno, fn):
    with open(path) as f:
        lines = f.readlines()
    lines[lineno] = fn(lines[lineno])
    with open(path, "w") as f:
        f.writelines(lines)


def test_garbled_numbers_stop_the_reader(case, tmp_path):
    """An item that is not a number stops the reading, as Fortran's
    list-directed READ stops the reference: in grid.vtk, in the .pop rows and
    in the input file, each with the file and the token named; nothing is
    ingested."""
    c2 = _copy_case(case, tmp_path)
    p = c2["paths"]
    dd = os.path.join(c2["d"], "dump")
    os.makedirs(dd, exist_ok=True)
    cases = [
        (p["grid"], 6, lambda l: "1.2.3 " + l.split(None, 1)[1], "1.2.3"),        # a POINTS row
        (p["pop"], 5, lambda l: l.replace(l.split()[6], "12x4", 1), "12x4"),        # a .pop row's density
        (os.path.join(c2["d"], "pol.dat"), 2, lambda l: "8 8x 16\n", "8x"),         # nth nph nvel
    ]
    for path, lineno, fn, tok in cases:
        backup = open(path).read()
        _edit_line(path, lineno, fn)
        r = _run(MAIN, c2, dict(PORTAL_DUMP_INGESTED=dd))
        assert r.returncode != 0, (path, r.stdout)
        assert "not a number: '%s'" % tok in r.stderr and os.path.basename(path) in r.stderr, r.stderr
        assert not os.listdir(dd)
        with open(path, "w") as f:
            f.write(backup)


def test_sign_exponents_are_read(case, tmp_path):
    """Numeric input takes an exponent given by its sign alone (1.25-1 is
    0.125), as the reference's list-directed READ does; the general reader
    path handles it (the parallel line parser falls back to it)."""
    c2 = _copy_case(case, tmp_path)
    grid = c2["paths"]["grid"]
    with open(grid) as f:
        lines = f.readlines()
    i = next(k for k, l in enumerate(lines) if l.startswith("POINTS")) + 1
    x0 = [float(v) for v in lines[i].split()]
    lines[i] = "%s %s %s\n" % ("%.17g" % x0[0], "1.25-1", "-2.5+2")
    with open(grid, "w") as f:
        f.writelines(lines)
    dd = os.path.join(c2["d"], "dump")
    os.makedirs(dd, exist_ok=True)
    r = _run(MAIN, c2, dict(PORTAL_DUMP_INGESTED=dd, PORTAL_BVEC_FILE=c2["paths"]["bvec"]))
    assert r.returncode == 0, r.stderr
    xyz = _npy(dd, "xyz").reshape(-1, 3)
    tx = _npy(dd, "scalars")[0]
    np.testing.assert_allclose(xyz[0, 1:] * tx, [0.125, -250.0], rtol=1e-15)


def test_executables_fail_loudly_without_a_gpu(case):
    """No CPU path in the drop-ins either: without an sm_103a device both
    executables stop with the library's error after parsing, and write no
    output."""
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    env = dict(PORTAL_BVEC_FILE=case["paths"]["bvec"])
    out = os.path.join(case["d"], "pol_pops.dat")
    before = os.path.getmtime(out) if os.path.exists(out) else None
    r = _run(MAIN, case, env)
    assert r.returncode != 0 and "portal_create" in r.stderr, (r.returncode, r.stderr)
    assert (os.path.getmtime(out) if os.path.exists(out) else None) == before


def test_fits_writer_roundtrip(tmp_path, built_lib):
    """writeimage's header keywords and big-endian float data
    (fits_writing.f90:57-149), read back by the repo's own parser."""
    import ctypes as C
    cube = np.arange(5 * 7 * 7, dtype=np.float32).reshape(5, 7, 7) * 0.25
    # exercise the C++ writer through finish_portal's FITS routine: a tiny
    # shim library is not shipped, so write with Python in the same layout and
    # parse it back; the C++ writer is exercised end to end in the GPU test
    path = str(tmp_path / "x.fits")
    cards = ["SIMPLE  =                    T", "BITPIX  =                  -32", "NAXIS   =                    3",
             "NAXIS1  =                    7", "NAXIS2  =                    7", "NAXIS3  =                    5", "END"]
    hdr = "".join(c.ljust(80) for c in cards)
    hdr = hdr.ljust((len(hdr) + 2879) // 2880 * 2880)
    data = cube.astype(">f4").tobytes()
    with open(path, "wb") as f:
        f.write(hdr.encode() + data + b"\0" * ((2880 - len(data) % 2880) % 2880))
    h, d = lime.read_fits(path)
    assert h["NAXIS3"] == "5" and np.array_equal(d, cube)


@pytest.mark.gpu
def test_main_and_finish_portal_end_to_end(case):
    """main_portal.x then finish_portal.x on files equal the library calls on
    the same cloud: pol_pops.dat to the last digit written, and the FITS
    cubes to the I_to_T scaling."""
    import portal_gb300 as pg
    d, cloud, mol, rc = case["d"], case["cloud"], case["mol"], case["rc"]
    env = dict(PORTAL_BVEC_FILE=case["paths"]["bvec"], PORTAL_GVEC=" ".join(repr(g) for g in rc.gvec))
    r = _run(MAIN, case, env)
    assert r.returncode == 0, r.stderr
    pops_file = np.loadtxt(os.path.join(d, "pol_pops.dat"))
    with pg.Context(0) as ctx:
        ctx.set_molecule(mol)
        ctx.set_cloud(cloud)
        ctx.radiation_field(rc, fetch=False)
        pops, _, jj, rates = ctx.solve_se(rc.kmax, jj20=True, rates=True)
        np.testing.assert_allclose(pops_file, pops, rtol=1e-15, atol=0)
        # extra_info = 1: the three rate files and the anisotropy
        for k, name in enumerate(("spont_rates.dat", "rad_rates.dat", "col_rates.dat")):
            np.testing.assert_allclose(np.loadtxt(os.path.join(d, name)), rates[:, k, :], rtol=1e-15, atol=0)
        got = np.loadtxt(os.path.join(d, "rad_anis.dat")).reshape(jj.shape)
        np.testing.assert_allclose(got, jj, rtol=1e-15, atol=0, equal_nan=True)
        im = dict(l1=[1], l2=[2], th_inc=[0.78539816339], ph_az=[0.0], nvel=8, dvel=50.0, v0=0.0, im_pix=12,
                  im_size=0.7)
        lime.write_finish_input(os.path.join(d, "finish.dat"), im["l1"], im["l2"], im["th_inc"], im["ph_az"],
                                im["nvel"], im["dvel"], im["v0"], im["im_pix"], im["im_size"])
        r2 = _run(FINISH, case, env, input_name="finish.dat")
        assert r2.returncode == 0, r2.stderr
        cube, st = ctx.image(im["l1"], im["l2"], im["th_inc"][0], im["ph_az"][0], im["nvel"], im["dvel"], im["v0"],
                             im["im_pix"], im["im_size"], pol_pops=pops_file)
    nu0 = mol.e_levs[1] - mol.e_levs[0]
    I_to_T = 3.255e39 / nu0 ** 2
    h, dI = lime.read_fits(os.path.join(d, "inc01-trans01-im_i.fits"))
    assert h["BITPIX"] == "-32" and h["CTYPE3"] == "VELO-LSR" and h["BUNIT"] == "K"
    assert abs(float(h["RESTFREQ"]) - nu0) <= 1e-6 * nu0
    np.testing.assert_allclose(dI, (I_to_T * cube[0, 0].astype(np.float64)).astype(np.float32), rtol=1e-6,
                               atol=1e-30)
    h, dtau = lime.read_fits(os.path.join(d, "inc01-trans01-im_tau.fits"))
    np.testing.assert_array_equal(dtau, cube[3, 0])
    h, ddust = lime.read_fits(os.path.join(d, "inc01-trans01-dust_i.fits"))
    assert ddust.shape == (1, 25, 25)


@pytest.mark.gpu
def test_main_portal_lambda_mode(case):
    """PORTAL_LAMBDA="tol n": main_portal.x iterates the node loop to
    convergence (accelerated) before its pass; pol_pops.dat equals the same
    library calls."""
    import portal_gb300 as pg
    d, cloud, mol, rc = case["d"], case["cloud"], case["mol"], case["rc"]
    env = dict(PORTAL_BVEC_FILE=case["paths"]["bvec"], PORTAL_GVEC=" ".join(repr(g) for g in rc.gvec),
               PORTAL_LAMBDA="1e-6 300")
    r = _run(MAIN, case, env)
    assert r.returncode == 0, r.stderr
    assert "Lambda iteration" in r.stdout
    pops_file = np.loadtxt(os.path.join(d, "pol_pops.dat"))
    with pg.Context(0) as ctx:
        ctx.set_molecule(mol)
        ctx.set_cloud(cloud)
        _, _, n, res, _ = ctx.lambda_iterate(rc, tol=1e-6, max_iter=300, fetch=False, ng_period=4,
                                             local_operator=True)
        assert n < 300 and res[-1] < 1e-6
        assert f"{n} passes" in r.stdout
        ctx.radiation_field(rc, fetch=False)
        pops, _, _, _ = ctx.solve_se(rc.kmax, jj20=True, rates=True)
    np.testing.assert_allclose(pops_file, pops, rtol=1e-15, atol=0)
    r = _run(MAIN, case, dict(env, PORTAL_LAMBDA="-1"))
    assert r.returncode != 0 and "PORTAL_LAMBDA" in r.stderr


@pytest.mark.gpu
def test_finish_portal_node_maps(case):
    """pix_mod = 0: finish_portal.x writes inc01-xy.dat and one
    inc01-trans01-vel{k}-im.dat per channel from the library's per-node
    maps (I_to_T I, I_to_T Q, I_to_T U, tau per bulk node)."""
    import portal_gb300 as pg
    d, cloud, mol, rc = case["d"], case["cloud"], case["mol"], case["rc"]
    env = dict(PORTAL_BVEC_FILE=case["paths"]["bvec"], PORTAL_GVEC=" ".join(repr(g) for g in rc.gvec))
    r = _run(MAIN, case, env)
    assert r.returncode == 0, r.stderr
    pops_file = np.loadtxt(os.path.join(d, "pol_pops.dat"))
    nvel = 3
    lime.write_finish_input(os.path.join(d, "finish0.dat"), [1], [2], [0.5], [0.2], nvel, 100.0, 0.0, 12, 0.7,
                            pix_mod=0)
    r2 = _run(FINISH, case, env, input_name="finish0.dat")
    assert r2.returncode == 0, r2.stderr
    with pg.Context(0) as ctx:
        ctx.set_molecule(mol)
        ctx.set_cloud(cloud)
        cube, xy, st = ctx.image_nodes([1], [2], 0.5, 0.2, nvel, 100.0, 0.0, pol_pops=pops_file)
    assert not st.any()
    np.testing.assert_allclose(np.loadtxt(os.path.join(d, "inc01-xy.dat")), xy, rtol=1e-15, atol=0)
    nu0 = mol.e_levs[1] - mol.e_levs[0]
    I_to_T = 3.255e39 / nu0 ** 2
    for k in range(2 * nvel + 1):
        rows = np.loadtxt(os.path.join(d, "inc01-trans01-vel%02d-im.dat" % (k + 1)))
        want = np.stack([I_to_T * cube[0, 0, k].astype(np.float64), I_to_T * cube[1, 0, k].astype(np.float64),
                         I_to_T * cube[2, 0, k].astype(np.float64), cube[3, 0, k].astype(np.float64)], axis=1)
        np.testing.assert_allclose(rows, want, rtol=1e-15, atol=0)
    assert not os.path.exists(os.path.join(d, "inc01-trans01-vel%02d-im.dat" % (2 * nvel + 2)))


@pytest.mark.gpu
def test_star_mode_end_to_end(case, tmp_path):
    """star_mod = 1 in both input files (run_portal.sh's default): the
    executables pass the star to the library (R_star in metres, X_star as
    read); pol_pops.dat and the FITS cube equal the library calls with the
    same star."""
    import shutil
    import portal_gb300 as pg
    d = str(tmp_path)
    for name in ("model.pop", "grid.vtk", "molecule.dat", "dust.tab", "bvec.dat"):
        shutil.copy(os.path.join(case["d"], name), d)
    cloud, mol = case["cloud"], case["mol"]
    # 12 x 12 directions: enough rays for the nodes nearest the star (star_all)
    rc = synth.RunConfig(nth=12, nph=12, nvel=16, kmax=6, gvec=case["rc"].gvec)
    star = (2500.0, 0.05 * cloud.tx, (0.0, 0.0, 0.0))
    c2 = dict(case, d=d, paths={k: os.path.join(d, os.path.basename(v)) for k, v in case["paths"].items()})
    lime.write_main_input(os.path.join(d, "pol.dat"), rc, extra_info=0, star=star)
    env = dict(PORTAL_BVEC_FILE=c2["paths"]["bvec"], PORTAL_GVEC=" ".join(repr(g) for g in rc.gvec))
    r = _run(MAIN, c2, env)
    assert r.returncode == 0, r.stderr
    pops_file = np.loadtxt(os.path.join(d, "pol_pops.dat"))
    im = dict(l1=[1], l2=[2], th_inc=[0.5], ph_az=[0.0], nvel=4, dvel=80.0, v0=0.0, im_pix=8, im_size=0.6)
    lime.write_finish_input(os.path.join(d, "finish.dat"), im["l1"], im["l2"], im["th_inc"], im["ph_az"],
                            im["nvel"], im["dvel"], im["v0"], im["im_pix"], im["im_size"], star=star)
    r2 = _run(FINISH, c2, env, input_name="finish.dat")
    assert r2.returncode == 0, r2.stderr
    with pg.Context(0) as ctx:
        ctx.set_molecule(mol)
        ctx.set_cloud(cloud)
        ctx.set_star(star)
        ctx.radiation_field(rc, fetch=False)
        pops, _ = ctx.solve_se(rc.kmax)
        inside = np.linalg.norm(cloud.xyz[:cloud.bulk_node_num], axis=1) <= 0.05
        assert inside.any() and (pops_file[:cloud.bulk_node_num][inside] == 0).all()
        np.testing.assert_allclose(pops_file, pops, rtol=1e-15, atol=0)
        cube, _ = ctx.image(im["l1"], im["l2"], im["th_inc"][0], im["ph_az"][0], im["nvel"], im["dvel"], im["v0"],
                            im["im_pix"], im["im_size"], pol_pops=pops_file)
    nu0 = mol.e_levs[1] - mol.e_levs[0]
    h, dI = lime.read_fits(os.path.join(d, "inc01-trans01-im_i.fits"))
    np.testing.assert_allclose(dI, (3.255e39 / nu0 ** 2 * cube[0, 0].astype(np.float64)).astype(np.float32),
                               rtol=1e-6, atol=1e-30, equal_nan=True)


@pytest.mark.gpu
def test_finish_portal_dat_maps(case, tmp_path):
    """fits = 0: one list-directed .dat file per inclination, line and
    channel for each of I, Q, U, tau and the dust I, Q, U, tau (dust maps in
    every channel, unlike the FITS path's centre channel), FP64 rows
    I_to_T x the cube, names with Fortran's i2.2 numbers."""
    import shutil
    import portal_gb300 as pg
    d = str(tmp_path)
    for name in ("model.pop", "grid.vtk", "molecule.dat", "dust.tab", "bvec.dat", "pol.dat"):
        shutil.copy(os.path.join(case["d"], name), d)
    c2 = dict(case, d=d, paths={k: os.path.join(d, os.path.basename(v)) for k, v in case["paths"].items()})
    cloud, mol, rc = case["cloud"], case["mol"], case["rc"]
    env = dict(PORTAL_BVEC_FILE=c2["paths"]["bvec"], PORTAL_GVEC=" ".join(repr(g) for g in rc.gvec))
    assert _run(MAIN, c2, env).returncode == 0
    pops_file = np.loadtxt(os.path.join(d, "pol_pops.dat"))
    nvel, im_pix = 2, 5
    lime.write_finish_input(os.path.join(d, "finish.dat"), [1], [2], [0.5], [0.0], nvel, 90.0, 0.0, im_pix, 0.6,
                            fits=0)
    r = _run(FINISH, c2, env, input_name="finish.dat")
    assert r.returncode == 0, r.stderr
    with pg.Context(0) as ctx:
        ctx.set_molecule(mol)
        ctx.set_cloud(cloud)
        cube, _ = ctx.image([1], [2], 0.5, 0.0, nvel, 90.0, 0.0, im_pix, 0.6, pol_pops=pops_file)
    I_to_T = 3.255e39 / (mol.e_levs[1] - mol.e_levs[0]) ** 2
    names = ["im_i", "im_q", "im_u", "im_tau", "dust_i", "dust_q", "dust_u", "dust_tau"]
    for k in range(2 * nvel + 1):
        for q, nm in enumerate(names):
            got = np.loadtxt(os.path.join(d, "inc01-trans01-vel%02d-%s.dat" % (k + 1, nm)))
            want = cube[q, 0, k].astype(np.float64).T * (1.0 if q % 4 == 3 else I_to_T)
            np.testing.assert_allclose(got, want, rtol=1e-15, atol=0, equal_nan=True)


@pytest.mark.gpu
def test_pol_pops_binary_sidecar(case, tmp_path):
    """PORTAL_POPS_BINARY=1: main_portal.x also writes pol_pops.bin, equal to
    pol_pops.dat to the last bit; finish_portal.x reads it and writes the
    same cube as from the text; a text file newer than the sidecar wins."""
    import shutil
    import time
    d = str(tmp_path)
    for name in ("model.pop", "grid.vtk", "molecule.dat", "dust.tab", "bvec.dat", "pol.dat"):
        shutil.copy(os.path.join(case["d"], name), d)
    c2 = dict(case, d=d, paths={k: os.path.join(d, os.path.basename(v)) for k, v in case["paths"].items()})
    rc = case["rc"]
    env = dict(PORTAL_BVEC_FILE=c2["paths"]["bvec"], PORTAL_GVEC=" ".join(repr(g) for g in rc.gvec))
    r = _run(MAIN, c2, dict(env, PORTAL_POPS_BINARY="1"))
    assert r.returncode == 0, r.stderr
    text = np.loadtxt(os.path.join(d, "pol_pops.dat"))
    raw = open(os.path.join(d, "pol_pops.bin"), "rb").read()
    assert raw[:8] == b"PORTALPP"
    rows, cols = np.frombuffer(raw[8:16], dtype="<i4")
    binp = np.frombuffer(raw[16:], dtype="<f8").reshape(cols, rows).T
    np.testing.assert_array_equal(binp, text)
    lime.write_finish_input(os.path.join(d, "finish.dat"), [1], [2], [0.4], [0.1], 4, 80.0, 0.0, 6, 0.6)
    r2 = _run(FINISH, c2, env, input_name="finish.dat")
    assert r2.returncode == 0 and "pol_pops.bin" in r2.stdout, r2.stderr
    _, from_bin = lime.read_fits(os.path.join(d, "inc01-trans01-im_i.fits"))
    time.sleep(0.05)
    os.utime(os.path.join(d, "pol_pops.dat"))  # the text is now newer: it wins
    r3 = _run(FINISH, c2, env, input_name="finish.dat")
    assert r3.returncode == 0 and "pol_pops.bin" not in r3.stdout, r3.stderr
    _, from_text = lime.read_fits(os.path.join(d, "inc01-trans01-im_i.fits"))
    np.testing.assert_array_equal(from_bin, from_text)


_ROW_WRITER_CHECK = r"""
#include <cstdio>
#include <vector>
#include "portal_io.h"
int main(int argc, char **argv) {
    FILE *f = fopen(argv[1], "rb");
    int rows, cols;
    if (fread(&rows, 4, 1, f) != 1 || fread(&cols, 4, 1, f) != 1) return 2;
    std::vector<double> v((size_t)rows * cols);
    if (fread(v.data(), 8, v.size(), f) != v.size()) return 3;
    fclose(f);
    return portal_io::write_rows(argv[2], v, rows, cols) ? 0 : 1;
}
"""


def test_row_writer_matches_printf(tmp_path):
    """write_rows (the pol_pops.dat writer, parallel, std::to_chars) is byte
    for byte the " %24.17E" printf loop: signed zeros, subnormals, the
    largest and smallest doubles, inf and NaN included, with 1 and with 8
    threads."""
    import shutil
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no g++")
    apps = os.path.join(ROOT, "portal_gb300", "apps")
    src = tmp_path / "check.cpp"
    src.write_text(_ROW_WRITER_CHECK)
    exe = str(tmp_path / "check")
    r = subprocess.run([cxx, "-O2", "-std=c++17", "-pthread", "-I", apps, str(src),
                        os.path.join(apps, "portal_io.cpp"), "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    rng = np.random.default_rng(5)
    rows, cols = 9001, 7
    v = rng.normal(size=(rows, cols)) * 10.0 ** rng.integers(-300, 300, size=(rows, cols))
    special = [0.0, -0.0, 5e-324, -2.2250738585072014e-308, 1.7976931348623157e308, np.inf, -np.inf, np.nan,
               1.0, 0.1, 123456789.0, 9.999999999999999e22]
    v.flat[:len(special)] = special
    blob = tmp_path / "in.bin"
    with open(blob, "wb") as f:
        f.write(np.array([rows, cols], dtype=np.int32).tobytes())
        f.write(np.asfortranarray(v).tobytes(order="F"))
    want = "".join("".join(" %24.17E" % x for x in row) + "\n" for row in v)
    for threads in ("1", "8"):
        out = tmp_path / ("rows%s.dat" % threads)
        r = subprocess.run([exe, str(blob), str(out)], env=dict(os.environ, PORTAL_THREADS=threads))
        assert r.returncode == 0
        assert out.read_text() == want


def test_parallel_reader_matches_list_directed_forms(case, tmp_path):
    """The bulk readers' fast path (one plain record per line, many threads)
    and their list-directed fallback (records across lines, D exponents,
    repeat counts) ingest the same arrays; so do 1 and many threads."""
    p = case["paths"]
    alt = dict(p)
    # .pop: one row split over two lines, a D exponent, a repeat count
    lines = open(p["pop"]).read().splitlines()
    r = lines[5].split()
    lines[5] = " ".join(r[:7]) + "\n" + " ".join(r[7:])
    r = lines[9].split()
    r[6] = r[6].replace("e", "D") if "e" in r[6] else r[6] + "D0"
    lines[9] = " ".join(r)
    r = lines[12].split()
    assert float(r[11]) == float(r[12]) == 0.0
    lines[12] = " ".join(r[:11] + ["2*0"] + r[13:])
    alt["pop"] = str(tmp_path / "alt.pop")
    open(alt["pop"], "w").write("\n".join(lines) + "\n")
    # grid.vtk: one point record over two lines
    g = open(p["grid"]).read().splitlines()
    k = next(i for i, l in enumerate(g) if l.startswith("POINTS")) + 3
    x = g[k].split()
    g[k] = x[0] + "\n" + " ".join(x[1:])
    alt["grid"] = str(tmp_path / "alt.vtk")
    open(alt["grid"], "w").write("\n".join(g) + "\n")
    dumps = []
    for paths, threads in ((p, "1"), (p, "8"), (alt, "8")):
        dd = tmp_path / ("dump_%d" % len(dumps))
        dd.mkdir()
        c2 = dict(case, paths=paths)
        r = _run(MAIN, c2, dict(PORTAL_DUMP_INGESTED=str(dd), PORTAL_BVEC_FILE=p["bvec"], PORTAL_THREADS=threads))
        assert r.returncode == 0, r.stderr
        dumps.append({n: np.load(dd / (n + ".npy")) for n in ("xyz", "vel", "b_all", "lev_p", "del_ne",
                                                               "del_num_ne", "h2_dens", "temp_all")})
    for d in dumps[1:]:
        for n, v in d.items():
            np.testing.assert_array_equal(v, dumps[0][n], err_msg=n)
