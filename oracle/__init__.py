"""ctypes front end of the FP64 oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this package; it is the checker, never the thing measured or shipped.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

P_D = C.POINTER(C.c_double)
P_I = C.POINTER(C.c_int)
P_L = C.POINTER(C.c_int64)


class OrcCloud(C.Structure):
    _fields_ = [("node_num", C.c_int), ("bulk_node_num", C.c_int), ("nlev", C.c_int),
                ("maxne", C.c_int), ("xyz", P_D), ("vel", P_D), ("b_all", P_D), ("t_kin", P_D),
                ("t_dust", P_D), ("dust_p", P_D), ("h2_dens", P_D), ("ab_all", P_D),
                ("lev_p", P_D), ("bvec", P_D), ("del_ne", P_I), ("del_num_ne", P_I),
                ("tx", C.c_double), ("star_mod", C.c_int), ("T_star", C.c_double), ("R_star", C.c_double),
                ("X_star", C.c_double * 3)]


class OrcMolecule(C.Structure):
    _fields_ = [("nlev", C.c_int), ("r_num", C.c_int), ("c_num", C.c_int), ("c_temp", C.c_int),
                ("c_par", C.c_int), ("j_lev", P_I), ("e_levs", P_D), ("r_trans", P_I),
                ("A", P_D), ("nu", P_D), ("Bij", P_D), ("kd_v", P_D), ("c_trans", P_I),
                ("col_temps", P_D), ("C", P_D), ("depol", C.c_int)]


def build() -> str:
    """Compile the oracle with its Makefile (gcc, OpenMP)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH) or (
                os.path.getmtime(_LIB_PATH) < os.path.getmtime(os.path.join(_HERE, "portal_oracle.c"))):
            build()
        L = C.CDLL(_LIB_PATH)
        L.orc_black_body.restype = C.c_double
        L.orc_black_body.argtypes = [C.c_double, C.c_double]
        L.orc_wigner3j.restype = C.c_double
        L.orc_wigner3j.argtypes = [C.c_int] * 6
        L.orc_wigner6j.restype = C.c_double
        L.orc_wigner6j.argtypes = [C.c_int] * 6
        L.orc_legendre_all.restype = C.c_int
        L.orc_gauss_legendre.restype = None
        L.orc_radiation_field.restype = C.c_int
        L.orc_solve_se.restype = C.c_int
        L.orc_image.restype = C.c_int
        L.orc_coupling_constants.restype = None
        _lib = L
    return _lib


def _p(a, t=P_D):
    return a.ctypes.data_as(t)


class OracleProblem:
    """Holds the reference-layout arrays of one cloud + molecule so that the
    C structs' pointers stay valid."""

    def __init__(self, cloud, mol, star=None, depol=0):
        """star: None, or (T_star [K], R_star [m], (x, y, z) as the input file
        gives them) for star_mod = 1.  depol: the depolarising collisions of
        the SE (0 off as main_sub.f90:96, 1 at the K = K' >= 2 diagonal
        entries, 2 as setup_stateq's code reads col_dep)."""
        self.cloud, self.mol = cloud, mol
        N = cloud.node_num
        self.xyz = np.ascontiguousarray(cloud.xyz, dtype=np.float64)          # (N,3) == X(3,N)
        self.vel = np.ascontiguousarray(cloud.vel, dtype=np.float64)
        self.b_all = np.ascontiguousarray(cloud.b_all, dtype=np.float64)
        self.t_kin = np.ascontiguousarray(cloud.t_kin, dtype=np.float64)
        self.t_dust = np.ascontiguousarray(cloud.t_dust, dtype=np.float64)
        self.dust_p = np.ascontiguousarray(cloud.dust_p, dtype=np.float64)
        self.h2 = np.ascontiguousarray(cloud.h2_dens, dtype=np.float64)
        self.ab = np.ascontiguousarray(cloud.ab_all, dtype=np.float64)
        # own copy: callers iterate the oracle by updating this array in place
        self.lev_p = np.array(cloud.lev_p, dtype=np.float64, order="C", copy=True)  # == lev_p(nlev,N)
        self.bvec = np.ascontiguousarray(cloud.bvec, dtype=np.float64)
        self.del_ne = np.ascontiguousarray(cloud.del_ne(), dtype=np.int32)    # (maxne,N) == del_ne(N,maxne)
        self.del_num_ne = np.ascontiguousarray(cloud.del_num_ne(), dtype=np.int32)
        self.c = OrcCloud(N, cloud.bulk_node_num, cloud.nlev, self.del_ne.shape[0], _p(self.xyz),
                          _p(self.vel), _p(self.b_all), _p(self.t_kin), _p(self.t_dust),
                          _p(self.dust_p), _p(self.h2), _p(self.ab), _p(self.lev_p), _p(self.bvec),
                          _p(self.del_ne, P_I), _p(self.del_num_ne, P_I), float(cloud.tx))
        if star is not None:
            T_s, R_s, X_s = star
            self.c.star_mod = 1
            self.c.T_star = float(T_s)
            self.c.R_star = float(R_s) / float(cloud.tx)   # main_para.f90:122
            for k in range(3):
                self.c.X_star[k] = float(X_s[k])
        self.j_lev = np.ascontiguousarray(mol.j_lev, dtype=np.int32)
        self.e_levs = np.ascontiguousarray(mol.e_levs, dtype=np.float64)
        self.r_trans = np.ascontiguousarray(mol.r_trans, dtype=np.int32)      # (r,2) == r_trans(2,r)
        self.A = np.ascontiguousarray(mol.A, dtype=np.float64)
        self.nu = np.ascontiguousarray(mol.nu, dtype=np.float64)
        self.Bij = np.ascontiguousarray(mol.Bij, dtype=np.float64)
        self.kd_v = np.ascontiguousarray(mol.kd_v, dtype=np.float64)
        self.c_trans = np.ascontiguousarray(mol.c_trans, dtype=np.int32)
        self.col_temps = np.ascontiguousarray(mol.col_temps, dtype=np.float64)
        self.Cr = np.ascontiguousarray(mol.C, dtype=np.float64)               # (P,C,T) == C(T,C,P)
        self.m = OrcMolecule(mol.nlev, mol.r_num, mol.c_num, mol.c_temp, mol.c_par, _p(self.j_lev, P_I),
                             _p(self.e_levs), _p(self.r_trans, P_I), _p(self.A), _p(self.nu),
                             _p(self.Bij), _p(self.kd_v), _p(self.c_trans, P_I),
                             _p(self.col_temps), _p(self.Cr), int(depol))

    def radiation_field(self, rc, node_lo=1, node_hi=None, nthreads=0):
        """J0, J2 of shape (N, r_num), per-node status, total segments."""
        N, R = self.cloud.node_num, self.mol.r_num
        node_hi = self.cloud.bulk_node_num if node_hi is None else node_hi
        J0 = np.zeros((N, R)); J2 = np.zeros((N, R))
        st = np.zeros(N, dtype=np.int32)
        nseg = C.c_int64(0)
        g = np.ascontiguousarray(rc.gvec, dtype=np.float64)
        nfail = lib().orc_radiation_field(C.byref(self.c), C.byref(self.m), rc.nth, rc.nph, rc.nvel,
                                          _p(g), C.c_double(rc.dx), rc.n_depth, node_lo, node_hi,
                                          nthreads, _p(J0), _p(J2), _p(st, P_I), C.byref(nseg))
        return J0, J2, st, int(nseg.value), nfail

    def radiation_field_split(self, rc, node_lo=1, node_hi=None, nthreads=0):
        """J0, J2, J_eff, L* of shape (N, r_num) and the per-node status."""
        N, R = self.cloud.node_num, self.mol.r_num
        node_hi = self.cloud.bulk_node_num if node_hi is None else node_hi
        J0, J2, JE, LS = (np.zeros((N, R)) for _ in range(4))
        st = np.zeros(N, dtype=np.int32)
        nseg = C.c_int64(0)
        g = np.ascontiguousarray(rc.gvec, dtype=np.float64)
        lib().orc_radiation_field_split(C.byref(self.c), C.byref(self.m), rc.nth, rc.nph, rc.nvel, _p(g),
                                        C.c_double(rc.dx), rc.n_depth, node_lo, node_hi, nthreads, _p(J0),
                                        _p(J2), _p(JE), _p(LS), _p(st, P_I), C.byref(nseg))
        return J0, J2, JE, LS, st

    def radiation_field_nodes(self, rc, nodes, nthreads=0, split=False):
        """The node loop over a list of 0-based bulk node ids: J0, J2 (and
        J_eff, L* with split) of shape (N, r_num) filled at the listed rows,
        the status and the segment count of each listed node."""
        N, R = self.cloud.node_num, self.mol.r_num
        ids = np.ascontiguousarray(np.asarray(nodes, dtype=np.int64) + 1, dtype=np.int32)
        J0 = np.zeros((N, R)); J2 = np.zeros((N, R))
        JE = np.zeros((N, R)) if split else None
        LS = np.zeros((N, R)) if split else None
        st = np.zeros(len(ids), dtype=np.int32)
        seg = np.zeros(len(ids), dtype=np.int64)
        g = np.ascontiguousarray(rc.gvec, dtype=np.float64)
        lib().orc_radiation_field_nodes(C.byref(self.c), C.byref(self.m), rc.nth, rc.nph, rc.nvel, _p(g),
                                        C.c_double(rc.dx), rc.n_depth, _p(ids, P_I), len(ids), nthreads,
                                        _p(J0), _p(J2), _p(JE) if split else None, _p(LS) if split else None,
                                        _p(st, P_I), _p(seg, P_L))
        if split:
            return J0, J2, JE, LS, st, seg
        return J0, J2, st, seg

    def solve_se_nodes(self, kmax, J0, J2, nodes, nthreads=0):
        """pol_pops (N, 2*nlev) at the listed 0-based bulk nodes' rows (0
        elsewhere) and the status per listed node."""
        N, nlev = self.cloud.node_num, self.mol.nlev
        ids = np.ascontiguousarray(np.asarray(nodes, dtype=np.int64) + 1, dtype=np.int32)
        pp = np.zeros((2 * nlev, N))
        st = np.zeros(len(ids), dtype=np.int32)
        J0c = np.ascontiguousarray(J0, dtype=np.float64)
        J2c = np.ascontiguousarray(J2, dtype=np.float64)
        lib().orc_solve_se_nodes(C.byref(self.c), C.byref(self.m), kmax, _p(J0c), _p(J2c), _p(ids, P_I),
                                 len(ids), nthreads, _p(pp), None, _p(st, P_I))
        return pp.T.copy(), st

    def solve_se(self, kmax, J0, J2, node_lo=1, node_hi=None, nthreads=0, rates=False):
        """pol_pops as an (N, 2*nlev) array (reference pol_pops(node,:))."""
        N, nlev = self.cloud.node_num, self.mol.nlev
        node_hi = self.cloud.bulk_node_num if node_hi is None else node_hi
        pp = np.zeros((2 * nlev, N))              # == Fortran pol_pops(N, 2 nlev)
        rt = np.zeros((2 * nlev, 3, N)) if rates else None
        st = np.zeros(N, dtype=np.int32)
        J0c = np.ascontiguousarray(J0, dtype=np.float64)
        J2c = np.ascontiguousarray(J2, dtype=np.float64)
        nfail = lib().orc_solve_se(C.byref(self.c), C.byref(self.m), kmax, _p(J0c), _p(J2c), node_lo,
                                   node_hi, nthreads, _p(pp), _p(rt) if rates else None, _p(st, P_I))
        out = (pp.T.copy(), st, nfail)
        if rates:
            out = out + (np.transpose(rt, (2, 1, 0)).copy(),)
        return out

    def node_matrix(self, kmax, node, J0, J2):
        cdim = C.c_int(0)
        A = np.zeros(80 * 80)
        J0c = np.ascontiguousarray(J0, dtype=np.float64)
        J2c = np.ascontiguousarray(J2, dtype=np.float64)
        lib().orc_node_matrix(C.byref(self.c), C.byref(self.m), kmax, node, _p(J0c), _p(J2c), _p(A),
                              C.byref(cdim))
        n = cdim.value
        return A[: n * n].reshape(n, n).T.copy()   # row-major view of the column-major matrix

    def image(self, lines_l1, lines_l2, pol_pops, th_inc, ph_az, nvel, dvel, v0, im_pix, im_size,
              alpha=0.15, n_depth_rt=10000, pix_lo=0, pix_hi=None, nthreads=0):
        """Raw (unscaled) cube (8, n_rt, nlines, nchan): I,Q,U,tau,dust I,Q,U,tau."""
        N, nlev = self.cloud.node_num, self.mol.nlev
        nl = len(lines_l1)
        l1 = np.ascontiguousarray(lines_l1, dtype=np.int32)
        l2 = np.ascontiguousarray(lines_l2, dtype=np.int32)
        ppF = np.ascontiguousarray(np.asarray(pol_pops, dtype=np.float64).T)   # (2nlev, N)
        n_rt = (2 * im_pix + 1) ** 2
        nch = 2 * nvel + 1
        out = np.zeros((8, n_rt, nl, nch))
        st = np.zeros(n_rt, dtype=np.int32)
        pix_hi = n_rt - 1 if pix_hi is None else pix_hi
        nfail = lib().orc_image(C.byref(self.c), C.byref(self.m), nl, _p(l1, P_I), _p(l2, P_I), _p(ppF),
                                C.c_double(th_inc), C.c_double(ph_az), nvel, C.c_double(dvel),
                                C.c_double(v0), im_pix, C.c_double(im_size), C.c_double(alpha),
                                n_depth_rt, pix_lo, pix_hi, nthreads, _p(out), _p(st, P_I))
        return out, st, nfail

    def image_nodes(self, lines_l1, lines_l2, pol_pops, th_inc, ph_az, nvel, dvel, v0, alpha=0.15,
                    n_depth_rt=10000, node_lo=0, node_hi=None, nthreads=0):
        """Per-node mode (pix_mod = 0): raw cube (8, n_bulk, nlines, nchan) for
        the bulk nodes node_lo..node_hi (the others stay 0), the xy rows
        (n_bulk, 2) and the status per node."""
        nb = self.cloud.bulk_node_num
        nl = len(lines_l1)
        l1 = np.ascontiguousarray(lines_l1, dtype=np.int32)
        l2 = np.ascontiguousarray(lines_l2, dtype=np.int32)
        ppF = np.ascontiguousarray(np.asarray(pol_pops, dtype=np.float64).T)
        nch = 2 * nvel + 1
        out = np.zeros((8, nb, nl, nch))
        xy = np.zeros((nb, 2))
        st = np.zeros(nb, dtype=np.int32)
        node_hi = nb - 1 if node_hi is None else node_hi
        nfail = lib().orc_image_nodes(C.byref(self.c), C.byref(self.m), nl, _p(l1, P_I), _p(l2, P_I), _p(ppF),
                                      C.c_double(th_inc), C.c_double(ph_az), nvel, C.c_double(dvel),
                                      C.c_double(v0), C.c_double(alpha), n_depth_rt, node_lo, node_hi, nthreads,
                                      _p(xy), _p(out), _p(st, P_I))
        return out, xy, st, nfail


def star_all(nth, nph, kvec, gvec, bvec, dOm):
    """The star-mode ray set of one node: (xth (n, 3) = cos th, ph, weight
    relative to bvec; n_star), or None where the reference stops."""
    xth = np.zeros((nth * nph, 3))
    ns = C.c_int(0)
    k, g, b = (np.ascontiguousarray(v, dtype=np.float64) for v in (kvec, gvec, bvec))
    n = lib().orc_star_all(nth, nph, _p(k), _p(g), _p(b), C.c_double(dOm), C.byref(ns), _p(xth))
    return None if n < 0 else (xth[:n].copy(), ns.value)


def de_polarization(mol, kmax):
    """D0_all of de_polarization (depol.f90:242-317) as an array (kmax/2,
    nlev, c_temp): [K/2 - 1, level, temperature] in cm^3/s; None where the
    reference's assumption j_lev(i) = i - 1 fails."""
    P = OracleProblem.__new__(OracleProblem)
    j = np.ascontiguousarray(mol.j_lev, dtype=np.int32)
    ct = np.ascontiguousarray(mol.c_trans, dtype=np.int32)
    cr = np.ascontiguousarray(mol.C, dtype=np.float64)
    tt = np.ascontiguousarray(mol.col_temps, dtype=np.float64)
    m = OrcMolecule(mol.nlev, mol.r_num, mol.c_num, mol.c_temp, mol.c_par, _p(j, P_I), None, None, None, None,
                    None, None, _p(ct, P_I), _p(tt), _p(cr), 1)
    out = np.zeros((kmax // 2, mol.nlev, mol.c_temp))
    rc = lib().orc_de_polarization(C.byref(m), kmax, _p(out))
    del P
    return None if rc != 0 else out


def legendre_all(nth, nph):
    xth = np.zeros((nth * nph, 3))
    n = lib().orc_legendre_all(nth, nph, _p(xth))
    return xth[:n].copy()


def gauss_legendre(n):
    x = np.zeros(n); w = np.zeros(n)
    lib().orc_gauss_legendre(n, _p(x), _p(w))
    return x, w


def wigner3j(tj1, tj2, tj3, tm1, tm2, tm3):
    return lib().orc_wigner3j(tj1, tj2, tj3, tm1, tm2, tm3)


def wigner6j(tj1, tj2, tj3, tj4, tj5, tj6):
    return lib().orc_wigner6j(tj1, tj2, tj3, tj4, tj5, tj6)


def coupling_constant(which, j, k, j2, k2):
    c0 = C.c_double(0); c2 = C.c_double(0)
    lib().orc_coupling_constants(which, j, k, j2, k2, C.byref(c0), C.byref(c2))
    return c0.value, c2.value


def black_body(T, nu):
    return lib().orc_black_body(T, nu)
