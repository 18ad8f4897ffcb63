"""Writers of the input files PORTAL's executables read.

A synthetic cloud (synth.power_law_sphere with keep_raw) is written as the
LIME grid.vtk / .pop pair, the molecule as a LAMDA file, plus a 67-row dust
table and the two whitespace input files in the layout run_portal.sh writes
(run_portal.sh:118-152).  Numbers are written with 17 significant digits so
that reading them back gives the same doubles.
"""
from __future__ import annotations

import os

import numpy as np


def _g(x) -> str:
    return repr(float(x))


def write_grid_vtk(path, pos_m, tets):
    """LIME's grid.vtk: points in metres, then the Delaunay tetrahedra
    (0-based), the records eat_lime.f90:21-34 and miscellaneous.f90:937-972
    read."""
    with open(path, "w") as f:
        f.write("# vtk DataFile Version 3.0\nLime grid\nASCII\nDATASET UNSTRUCTURED_GRID\n")
        f.write("POINTS %d float\n" % len(pos_m))
        np.savetxt(f, pos_m, fmt="%.17g")
        f.write("\nCELLS %d %d\n" % (len(tets), 5 * len(tets)))
        np.savetxt(f, np.column_stack([np.full(len(tets), 4), tets]), fmt="%d")
        f.write("CELL_TYPES %d\n" % len(tets))
        np.savetxt(f, np.full(len(tets), 10), fmt="%d")


def write_pop(path, raw, nbulk):
    """LIME's .pop rows: x y z vx vy vz n_H2 T_kin T_dust b abundance
    gas-to-dust (unused column) populations (eat_lime.f90:213-214)."""
    cols = [raw["pos_m"][:nbulk], raw["vel"][:nbulk], raw["n_h2"][:nbulk, None], raw["t_kin"][:nbulk, None],
            raw["t_dust"][:nbulk, None], raw["b"][:nbulk, None], raw["ab"][:nbulk, None],
            raw["gas_ii_dust"][:nbulk, None], np.zeros((nbulk, 1)), raw["frac"][:nbulk]]
    with open(path, "w") as f:
        f.write("# x y z vx vy vz density temperature tdust doppler abundance gas_to_dust - populations\n")
        np.savetxt(f, np.hstack(cols), fmt="%.17g")


def write_lamda(path, mol, name="SYNROT"):
    """LAMDA layout with the records eat_lime.f90:38-62 and :151-196 read."""
    from .synth import C_LIGHT_CGS, H_CGS, KB_CGS
    with open(path, "w") as f:
        f.write("!MOLECULE\n%s\n!MOLECULAR WEIGHT\n%s\n" % (name, _g(mol.mass)))
        f.write("!NUMBER OF ENERGY LEVELS\n%d\n!LEVEL + ENERGIES(cm^-1) + WEIGHT + J\n" % mol.nlev)
        for i in range(mol.nlev):
            f.write("%d %s %s %d\n" % (i + 1, _g(mol.e_cm[i]), _g(2 * mol.j_lev[i] + 1), mol.j_lev[i]))
        f.write("!NUMBER OF RADIATIVE TRANSITIONS\n%d\n!TRANS + UP + LOW + EINSTEINA(s^-1) + FREQ(GHz) + E_u(K)\n"
                % mol.r_num)
        for i in range(mol.r_num):
            lo, up = int(mol.r_trans[i, 0]), int(mol.r_trans[i, 1])
            eu = H_CGS * C_LIGHT_CGS * mol.e_cm[up - 1] / KB_CGS
            f.write("%d %d %d %s %s %s\n" % (i + 1, up, lo, _g(mol.A[i]), _g(mol.freq_ghz[i]), _g(eu)))
        f.write("!NUMBER OF COLL PARTNERS\n%d\n" % mol.c_par)
        for p in range(mol.c_par):
            f.write("!COLLISIONS BETWEEN\n%d SYNROT-H2\n!NUMBER OF COLL TRANS\n%d\n" % (p + 1, mol.c_num))
            f.write("!NUMBER OF COLL TEMPS\n%d\n!COLL TEMPS\n%s\n" % (mol.c_temp, " ".join(_g(t) for t in mol.col_temps)))
            f.write("!TRANS + UP + LOW + COLLRATES(cm^3 s^-1)\n")
            for i in range(mol.c_num):
                lo, up = int(mol.c_trans[i, 0]), int(mol.c_trans[i, 1])
                f.write("%d %d %d %s\n" % (i + 1, up, lo, " ".join(_g(v) for v in mol.C[p, i])))


def write_dust(path, table):
    np.savetxt(path, table, fmt="%.17g")


def _star_line(star):
    """The star record (star_mod T_star R_star X Y Z, run_portal.sh:120):
    star = None (star_mod 0 with run_portal.sh's values) or (T_star [K],
    R_star [m], (x, y, z))."""
    if star is None:
        return "0 2.5E3 2.99196E11 0.d0 0.d0 0.d0"
    T_s, R_s, X_s = star
    return "1 %s %s %s" % (_g(T_s), _g(R_s), " ".join(_g(v) for v in X_s))


def write_main_input(path, rc, kmax=None, extra_info=0, max_ne_temp=10000, dust_ii_gas=0.01,
                     field=(0, 1, 0, "1.d0"), star=None):
    """The input file of main_portal.x as run_portal.sh:118-128 writes it."""
    with open(path, "w") as f:
        f.write("\n%s\n" % _star_line(star))
        f.write("%d %d %d\n" % (rc.nth, rc.nph, rc.nvel))
        f.write("%s\n" % dust_ii_gas)
        f.write("%s %s %s %s\n" % field)
        f.write("%d %d\n" % (rc.kmax if kmax is None else kmax, extra_info))
        f.write("%d %d\n\n" % (max_ne_temp, rc.n_depth))


def write_finish_input(path, l1, l2, th_inc, ph_az, nvel, dvel, v0, im_pix, im_size, kmax=6, fits=1,
                       distance=3.086e16, max_ne_temp=10000, n_depth_rt=10000, dust_ii_gas=0.01,
                       field=(0, 1, 0, "1.d0"), pix_mod=1, star=None):
    """The input file of finish_portal.x as run_portal.sh:133-152 writes it."""
    with open(path, "w") as f:
        f.write("\n%d\n%s\n%s\n\n" % (len(l1), " ".join(map(str, l1)), " ".join(map(str, l2))))
        f.write("%d\n%s\n%s\n\n" % (len(th_inc), " ".join(_g(t) for t in th_inc), " ".join(_g(p) for p in ph_az)))
        f.write("%d %s %s\n\n" % (nvel, _g(dvel), _g(v0)))
        f.write("%s\n%s\n" % (_star_line(star), dust_ii_gas))
        f.write("%s %s %s %s\n" % field)
        f.write("%d 0\n%d %d %s\n%d %s\n%d %d\n\n" % (kmax, pix_mod, im_pix, _g(im_size), fits, _g(distance),
                                                   max_ne_temp, n_depth_rt))


def write_case(directory, cloud, mol, dust_table=None):
    """All model files of one cloud; returns their paths (pop, grid, mol,
    dust, bvec)."""
    from .synth import default_dust_table
    if cloud.raw is None or cloud.tets is None:
        raise ValueError("the cloud must be generated with keep_raw=True")
    os.makedirs(directory, exist_ok=True)
    p = {k: os.path.join(directory, v) for k, v in
         dict(pop="model.pop", grid="grid.vtk", mol="molecule.dat", dust="dust.tab", bvec="bvec.dat").items()}
    write_grid_vtk(p["grid"], cloud.raw["pos_m"], cloud.tets)
    write_pop(p["pop"], cloud.raw, cloud.bulk_node_num)
    write_lamda(p["mol"], mol)
    write_dust(p["dust"], default_dust_table() if dust_table is None else dust_table)
    np.savetxt(p["bvec"], cloud.bvec, fmt="%.17g")
    return p


def read_fits(path):
    """Minimal reader of the cubes finish_portal writes: (header dict, data
    as a (naxis3, naxis2, naxis1) float32 array)."""
    with open(path, "rb") as f:
        raw = f.read()
    hdr, pos = {}, 0
    while True:
        card = raw[pos:pos + 80].decode("ascii")
        pos += 80
        key = card[:8].strip()
        if key == "END":
            break
        if card[8:10] == "= ":
            v = card[10:].split("/")[0].strip()
            hdr[key] = v.strip("'").strip() if v.startswith("'") else v
    pos = (pos + 2879) // 2880 * 2880
    n1, n2, n3 = int(hdr["NAXIS1"]), int(hdr["NAXIS2"]), int(hdr["NAXIS3"])
    data = np.frombuffer(raw[pos:pos + 4 * n1 * n2 * n3], dtype=">f4").reshape(n3, n2, n1)
    return hdr, data.astype(np.float32)
