"""PORTAL's polarized line-transfer hot path on GB300 (sm_103a).

The product is the C-ABI shared library ``_build/libportal_gb300.so`` built
from ``csrc/`` (declared in ``include/portal_gb300.h``).  This module is the
host-side mirror of the reference's node loop for Python callers: it loads the
library with ctypes and exposes one method per entry point, taking the
reference's arrays (``synth.Cloud`` / ``synth.Molecule`` or plain numpy arrays
in the reference layouts).

There is no CPU fallback: if the library is missing or no sm_103a device is
present, every call raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libportal_gb300.so")

P_D = C.POINTER(C.c_double)
P_I = C.POINTER(C.c_int)

PORTAL_OK = 0
NODE_DEPTH, NODE_SINGULAR, NODE_REFINE, NODE_STAR = 1, 2, 4, 8
KERNEL_SLOTS = ("line_table", "radiation_field", "solve_se", "emcoefs", "image_walk", "image_rt")

EXPORTS = (
    "portal_strerror", "portal_last_error", "portal_create", "portal_destroy",
    "portal_set_molecule", "portal_set_cloud", "portal_set_populations",
    "portal_radiation_field", "portal_radiation_field_split", "portal_solve_se", "portal_image", "portal_image_nodes", "portal_set_star", "portal_last_kernel_times",
    "portal_set_stream",
    "portal_wigner3j", "portal_wigner6j", "portal_coupling_constant",
    "portal_radiation_field_static", "portal_radiation_field_static_limits",
    "portal_lambda_iterate",
    "portal_mlp_create", "portal_mlp_destroy", "portal_mlp_last_error", "portal_mlp_num_params",
    "portal_mlp_get_params", "portal_mlp_set_params", "portal_mlp_gradients", "portal_mlp_train",
    "portal_mlp_predict", "portal_warmstart_features", "portal_get_results",
    "portal_batch_create", "portal_batch_destroy", "portal_batch_last_error", "portal_batch_add",
    "portal_batch_prepare", "portal_batch_run", "portal_batch_config", "portal_node_segments",
    "portal_set_depolarization", "portal_adj_list", "portal_field_moments",
)

_lib = None


class PortalError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"PORTAL error {code}: {msg}")
        self.code = code


def lib() -> C.CDLL:
    """Load the library (it must have been built; see build.py)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: run portal_gb300.build.build() first")
    L = C.CDLL(LIB_PATH)
    L.portal_strerror.restype = C.c_char_p
    L.portal_strerror.argtypes = [C.c_int]
    L.portal_last_error.restype = C.c_char_p
    L.portal_last_error.argtypes = [C.c_void_p]
    L.portal_create.argtypes = [C.POINTER(C.c_void_p), C.c_int]
    L.portal_destroy.argtypes = [C.c_void_p]
    L.portal_set_molecule.argtypes = [C.c_void_p, C.c_int, P_I, P_D, C.c_int, P_I, P_D, P_D, P_D, P_D,
                                      C.c_int, P_I, C.c_int, C.c_int, P_D, P_D]
    L.portal_set_cloud.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, P_D, P_D, P_D, P_D, P_D, P_D,
                                   P_D, P_D, P_D, C.c_int, P_I, P_I, C.c_double]
    L.portal_set_populations.argtypes = [C.c_void_p, P_D]
    L.portal_radiation_field.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, P_D, C.c_double, C.c_int,
                                         P_D, P_D, P_I, C.POINTER(C.c_longlong)]
    L.portal_radiation_field_split.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, P_D, C.c_double, C.c_int,
                                               P_D, P_D, P_D, P_D, P_I, C.POINTER(C.c_longlong)]
    L.portal_solve_se.argtypes = [C.c_void_p, C.c_int, P_D, P_D, P_D, P_D, P_D, P_I]
    L.portal_last_kernel_times.argtypes = [C.c_void_p, P_D, P_I, C.c_int]
    L.portal_set_stream.argtypes = [C.c_void_p, C.c_void_p]
    P_F = C.POINTER(C.c_float)
    L.portal_image.argtypes = [C.c_void_p, P_D, C.c_int, P_I, P_I, C.c_double, C.c_double, C.c_int, C.c_double,
                               C.c_double, C.c_int, C.c_double, C.c_double, C.c_double, C.c_int] + [P_F] * 8 + [P_I]
    L.portal_set_star.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_double, P_D]
    L.portal_image_nodes.argtypes = [C.c_void_p, P_D, C.c_int, P_I, P_I, C.c_double, C.c_double, C.c_int,
                                     C.c_double, C.c_double, C.c_double, C.c_double, C.c_int, P_D] + \
        [C.POINTER(C.c_float)] * 8 + [P_I]
    L.portal_wigner3j.restype = C.c_double
    L.portal_wigner3j.argtypes = [C.c_int] * 6
    L.portal_wigner6j.restype = C.c_double
    L.portal_wigner6j.argtypes = [C.c_int] * 6
    L.portal_coupling_constant.restype = None
    L.portal_coupling_constant.argtypes = [C.c_int] * 5 + [P_D, P_D]
    # the allocation-free entry point takes raw device addresses
    V = C.c_void_p
    L.portal_radiation_field_static.argtypes = (
        [V, C.c_int, C.c_int, C.c_int] + [V] * 8 + [C.c_int, V, V, C.c_double] +
        [P_I, C.c_int, P_I, P_D, P_D, P_D, P_D, C.c_int, C.c_int, C.c_int, P_D, C.c_double, C.c_int] + [V] * 3)
    L.portal_lambda_iterate.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, P_D, C.c_double, C.c_int, C.c_int,
                                        C.c_double, C.c_int, C.c_int, C.c_int, P_D, P_D, P_D, P_I, P_D, C.POINTER(C.c_longlong)]
    L.portal_radiation_field_static_limits.restype = None
    L.portal_radiation_field_static_limits.argtypes = [P_I, P_I, P_I, P_I, C.POINTER(C.c_longlong)]
    P_F = C.POINTER(C.c_float)
    L.portal_mlp_create.argtypes = [C.POINTER(C.c_void_p), C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                    C.c_ulonglong]
    L.portal_mlp_destroy.argtypes = [C.c_void_p]
    L.portal_mlp_last_error.restype = C.c_char_p
    L.portal_mlp_last_error.argtypes = [C.c_void_p]
    L.portal_mlp_num_params.restype = C.c_longlong
    L.portal_mlp_num_params.argtypes = [C.c_void_p]
    L.portal_mlp_get_params.argtypes = [C.c_void_p, P_F, P_F]
    L.portal_mlp_set_params.argtypes = [C.c_void_p, P_F, P_F]
    L.portal_mlp_gradients.argtypes = [C.c_void_p, P_F, P_F, C.c_int, P_F, P_F]
    L.portal_mlp_train.argtypes = [C.c_void_p, P_F, P_F, C.c_int, C.c_int, C.c_int, C.c_float, C.c_ulonglong, P_F]
    L.portal_mlp_predict.argtypes = [C.c_void_p, P_F, C.c_int, P_F]
    L.portal_warmstart_features.argtypes = [C.c_void_p, P_F]
    L.portal_get_results.argtypes = [C.c_void_p, P_D, P_D, P_D, P_I]
    L.portal_node_segments.argtypes = [C.c_void_p, P_I]
    L.portal_set_depolarization.argtypes = [C.c_void_p, C.c_int]
    L.portal_field_moments.argtypes = [C.c_void_p, P_D]
    L.portal_adj_list.argtypes = [C.c_void_p, C.c_int, C.c_longlong, P_I, C.c_int, P_I, P_I, P_I, P_D]
    L.portal_batch_create.argtypes = [C.POINTER(C.c_void_p), C.c_int]
    L.portal_batch_destroy.argtypes = [C.c_void_p]
    L.portal_batch_last_error.restype = C.c_char_p
    L.portal_batch_last_error.argtypes = [C.c_void_p]
    L.portal_batch_add.argtypes = [C.c_void_p, C.c_void_p]
    L.portal_batch_prepare.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, P_D, C.c_double, C.c_int, C.c_int,
                                       C.c_int]
    L.portal_batch_run.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_longlong), C.POINTER(C.c_double)]
    L.portal_batch_config.argtypes = [C.c_void_p, P_I, P_D, C.c_int]
    _lib = L
    return L


def _p(a, t=P_D):
    return None if a is None else a.ctypes.data_as(t)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


class Context:
    """One device context (portal_create / portal_destroy)."""

    def __init__(self, device: int = 0):
        self._h = C.c_void_p()
        rc = lib().portal_create(C.byref(self._h), device)
        if rc != PORTAL_OK:
            raise PortalError(rc, lib().portal_last_error(None).decode())
        self.nlev = self.r_num = self.N = self.bulk = 0

    def close(self):
        if self._h:
            lib().portal_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc: int):
        if rc != PORTAL_OK:
            msg = lib().portal_last_error(self._h).decode() or lib().portal_strerror(rc).decode()
            raise PortalError(rc, msg)

    # ---- set-up -----------------------------------------------------------
    def set_molecule(self, mol):
        self._mol = dict(j=_i32(mol.j_lev), e=_f64(mol.e_levs), rt=_i32(mol.r_trans), A=_f64(mol.A),
                         nu=_f64(mol.nu), B=_f64(mol.Bij), kd=_f64(mol.kd_v), ct=_i32(mol.c_trans),
                         tc=_f64(mol.col_temps), C=_f64(mol.C))
        m = self._mol
        self._check(lib().portal_set_molecule(
            self._h, mol.nlev, _p(m["j"], P_I), _p(m["e"]), mol.r_num, _p(m["rt"], P_I), _p(m["A"]),
            _p(m["nu"]), _p(m["B"]), _p(m["kd"]), mol.c_num, _p(m["ct"], P_I), mol.c_temp, mol.c_par,
            _p(m["tc"]), _p(m["C"])))
        self.nlev, self.r_num = mol.nlev, mol.r_num

    def set_cloud(self, cloud, del_ne=None, del_num_ne=None):
        """cloud: synth.Cloud.  del_ne / del_num_ne default to the cloud's
        reference-layout neighbour arrays."""
        N = cloud.node_num
        temp = np.empty((N, 2))
        temp[:, 0] = cloud.t_kin
        temp[:, 1] = cloud.t_dust
        dn = _i32(cloud.del_ne() if del_ne is None else del_ne)
        dnn = _i32(cloud.del_num_ne() if del_num_ne is None else del_num_ne)
        arrs = [_f64(cloud.xyz), _f64(cloud.vel), _f64(cloud.b_all), _f64(temp), _f64(cloud.dust_p),
                _f64(cloud.h2_dens), _f64(cloud.ab_all), _f64(cloud.lev_p), _f64(cloud.bvec)]
        self._check(lib().portal_set_cloud(self._h, N, cloud.bulk_node_num, cloud.nlev,
                                           *[_p(a) for a in arrs], dn.shape[0], _p(dn, P_I), _p(dnn, P_I),
                                           float(cloud.tx)))
        self.N, self.bulk = N, cloud.bulk_node_num

    def set_cloud_arrays(self, N, bulk, nlev, xyz, vel, b_all, temp_all, dust_p, h2_dens, ab_all, lev_p,
                         bvec, del_ne, del_num_ne, tx):
        """portal_set_cloud with the reference-layout arrays as given (no
        copies: float64 / int32 C-contiguous arrays, e.g. in pinned memory)."""
        self._check(lib().portal_set_cloud(self._h, N, bulk, nlev, _p(xyz), _p(vel), _p(b_all), _p(temp_all),
                                           _p(dust_p), _p(h2_dens), _p(ab_all), _p(lev_p), _p(bvec),
                                           del_ne.shape[0], _p(del_ne, P_I), _p(del_num_ne, P_I), float(tx)))
        self.N, self.bulk = N, bulk

    def set_star(self, star=None):
        """Star mode: star = (T_star [K], R_star [m], (x, y, z) as the input
        file gives them), or None for star_mod = 0."""
        if star is None:
            self._check(lib().portal_set_star(self._h, 0, 0.0, 0.0, None))
            return
        T_s, R_s, X_s = star
        x = _f64(np.asarray(X_s, dtype=np.float64))
        self._check(lib().portal_set_star(self._h, 1, float(T_s), float(R_s), _p(x)))

    def set_depolarization(self, mode: int):
        """Depolarising collisions in the SE: 0 off (default), 1 on the
        K = K' >= 2 diagonal entries, 2 as setup_stateq's code reads its
        col_dep variable (see portal_set_depolarization)."""
        self._check(lib().portal_set_depolarization(self._h, int(mode)))

    def set_populations(self, lev_p):
        self._check(lib().portal_set_populations(self._h, _p(_f64(lev_p))))

    # ---- the node loop ------------------------------------------------------
    def radiation_field(self, rc, fetch: bool = True):
        """J0, J2 as (N, r_num) arrays (the reference's (r_num, N) memory),
        status (N,), number of ray segments."""
        g = _f64(rc.gvec)
        nseg = C.c_longlong(0)
        J0 = np.zeros((self.N, self.r_num)) if fetch else None
        J2 = np.zeros((self.N, self.r_num)) if fetch else None
        st = np.zeros(self.N, dtype=np.int32) if fetch else None
        self._check(lib().portal_radiation_field(self._h, rc.nth, rc.nph, rc.nvel, _p(g), float(rc.dx),
                                                 rc.n_depth, _p(J0), _p(J2), _p(st, P_I), C.byref(nseg)))
        return J0, J2, st, int(nseg.value)

    def radiation_field_split(self, rc):
        """J0, J2, J_eff, L* as (N, r_num) arrays and the status; the split
        stays on the device for a following solve_se (preconditioned SE)."""
        g = _f64(rc.gvec)
        nseg = C.c_longlong(0)
        J0, J2, JE, LS = (np.zeros((self.N, self.r_num)) for _ in range(4))
        st = np.zeros(self.N, dtype=np.int32)
        self._check(lib().portal_radiation_field_split(self._h, rc.nth, rc.nph, rc.nvel, _p(g), float(rc.dx),
                                                       rc.n_depth, _p(J0), _p(J2), _p(JE), _p(LS), _p(st, P_I),
                                                       C.byref(nseg)))
        return J0, J2, JE, LS, st

    def solve_se(self, kmax, J0=None, J2=None, fetch: bool = True, jj20: bool = False, out=None,
                 rates: bool = False):
        """pol_pops as (N, 2*nlev) (reference pol_pops(node,:)), status.
        out: a float64 (2*nlev, N) C-contiguous buffer (the reference's
        pol_pops(N, 2*nlev) memory) to receive the result without a copy.
        jj20 / rates append J2/J0 (N, r_num) and the extra_info rates
        (N, 3, 2*nlev: spontaneous, radiative, collisional)."""
        if out is not None:
            self._check(lib().portal_solve_se(self._h, kmax, None, None, _p(out), None, None, None))
            return out, None
        pp = np.zeros((2 * self.nlev, self.N)) if fetch else None      # Fortran (N, 2 nlev)
        jj = np.zeros((self.r_num, self.N)) if jj20 else None
        st = np.zeros(self.N, dtype=np.int32) if fetch else None
        j0 = None if J0 is None else _f64(J0)
        j2 = None if J2 is None else _f64(J2)
        rt = np.zeros((2 * self.nlev, 3, self.N)) if rates else None  # Fortran (N, 3, 2 nlev)
        self._check(lib().portal_solve_se(self._h, kmax, _p(j0), _p(j2), _p(pp), _p(rt), _p(jj), _p(st, P_I)))
        out = (None if pp is None else pp.T.copy(), st)
        if jj20:
            out = out + (jj.T.copy(),)
        if rates:
            out = out + (np.transpose(rt, (2, 1, 0)).copy(),)
        return out

    def image(self, l1, l2, th_inc, ph_az, nvel, dvel, v0, im_pix, im_size, alpha=0.15,
              dx=float(np.float32(1e-4)), n_depth_rt=10000, pol_pops=None, quantities=8):
        """Stokes cubes of one inclination.  Returns an (8, nlines, nchan,
        npx(y), npx(x)) float32 array (I, Q, U, tau, dust I, Q, U, tau; the
        memory of eight Fortran (npx, npx, nchan, nlines) arrays) and the
        per-pixel status.  pol_pops: (N, 2*nlev) or None for the result of the
        last solve_se."""
        l1 = _i32(l1); l2 = _i32(l2)
        nl, npx, nch = len(l1), 2 * im_pix + 1, 2 * nvel + 1
        out = np.zeros((8, nl, nch, npx, npx), dtype=np.float32)
        st = np.zeros(npx * npx, dtype=np.int32)
        pp = None if pol_pops is None else np.ascontiguousarray(np.asarray(pol_pops, dtype=np.float64).T)
        P_F = C.POINTER(C.c_float)
        ptrs = [out[q].ctypes.data_as(P_F) if q < quantities else None for q in range(8)]
        self._check(lib().portal_image(self._h, _p(pp), nl, _p(l1, P_I), _p(l2, P_I), float(th_inc), float(ph_az),
                                       nvel, float(dvel), float(v0), im_pix, float(im_size), float(alpha), float(dx),
                                       n_depth_rt, *ptrs, _p(st, P_I)))
        return out, st

    def image_nodes(self, l1, l2, th_inc, ph_az, nvel, dvel, v0, alpha=0.15, dx=float(np.float32(1e-4)),
                    n_depth_rt=10000, pol_pops=None, quantities=4):
        """Per-node maps of one inclination (pix_mod = 0).  Returns an (8,
        nlines, nchan, n_bulk) float32 array (I, Q, U, tau, dust I, Q, U, tau;
        the first `quantities` filled), the xy rows (n_bulk, 2) and the
        per-node status."""
        l1 = _i32(l1); l2 = _i32(l2)
        nl, nch, nb = len(l1), 2 * nvel + 1, self.bulk
        out = np.zeros((8, nl, nch, nb), dtype=np.float32)
        xy = np.zeros((nb, 2))
        st = np.zeros(nb, dtype=np.int32)
        pp = None if pol_pops is None else np.ascontiguousarray(np.asarray(pol_pops, dtype=np.float64).T)
        P_F = C.POINTER(C.c_float)
        ptrs = [out[q].ctypes.data_as(P_F) if q < quantities else None for q in range(8)]
        self._check(lib().portal_image_nodes(self._h, _p(pp), nl, _p(l1, P_I), _p(l2, P_I), float(th_inc),
                                             float(ph_az), nvel, float(dvel), float(v0), float(alpha), float(dx),
                                             n_depth_rt, _p(xy), *ptrs, _p(st, P_I)))
        return out, xy, st

    def lambda_iterate(self, rc, tol=1e-6, max_iter=100, start_pops=None, fetch=True, ng_period=0,
                       local_operator=False):
        """Lambda iteration: plain, with Ng extrapolation every ng_period
        passes, and/or with the local (diagonal) Lambda operator.  Returns
        (pol_pops (N, 2 nlev), lev_p (N, nlev), passes, residual per pass,
        segments)."""
        pp = np.zeros((2 * self.nlev, self.N)) if fetch else None
        lp = np.zeros((self.N, self.nlev)) if fetch else None
        res = np.zeros(max_iter)
        it = C.c_int(0)
        nseg = C.c_longlong(0)
        sp = None if start_pops is None else np.ascontiguousarray(np.asarray(start_pops, dtype=np.float64).T)
        g = _f64(rc.gvec)
        self._check(lib().portal_lambda_iterate(self._h, rc.nth, rc.nph, rc.nvel, _p(g), float(rc.dx), rc.n_depth,
                                                rc.kmax, float(tol), int(max_iter), int(ng_period),
                                                int(bool(local_operator)), _p(sp),
                                                _p(pp), _p(lp),
                                                C.byref(it), _p(res), C.byref(nseg)))
        n = it.value
        return (None if pp is None else pp.T.copy()), lp, n, res[:n].copy(), int(nseg.value)

    def set_stream(self, stream_ptr: int | None):
        """Run on a caller-owned cudaStream_t (e.g. torch.cuda.current_stream().cuda_stream)."""
        self._check(lib().portal_set_stream(self._h, C.c_void_p(stream_ptr or 0)))

    def kernel_times(self):
        t = np.zeros(len(KERNEL_SLOTS))
        n = np.zeros(len(KERNEL_SLOTS), dtype=np.int32)
        self._check(lib().portal_last_kernel_times(self._h, _p(t), _p(n, P_I), len(KERNEL_SLOTS)))
        return {k: (float(t[i]), int(n[i])) for i, k in enumerate(KERNEL_SLOTS)}


    def results(self, field=True, pops=True):
        """Device-resident results of the last pass: (J0, J2) as (N, r_num)
        and pol_pops (N, 2 nlev), each None when not asked for."""
        J0 = np.zeros((self.N, self.r_num)) if field else None
        J2 = np.zeros((self.N, self.r_num)) if field else None
        pp = np.zeros((2 * self.nlev, self.N)) if pops else None
        self._check(lib().portal_get_results(self._h, _p(J0), _p(J2), _p(pp), None))
        return J0, J2, (None if pp is None else pp.T.copy())

    def adj_list(self, node_num, tets, max_ne_temp=None):
        """Delaunay neighbour lists built on the device from the tetrahedra
        (ntet, 4) 0-based: (del_ne as a (max_ne, node_num) C array == the
        reference's del_ne(node_num, max_ne), del_num_ne, device ms).  The
        CSR of synth.neighbours_from_tets follows from these two arrays."""
        t = _i32(tets)
        cap = int(max_ne_temp or 12 * 64)
        dne = np.zeros((cap, node_num), dtype=np.int32)
        num = np.zeros(node_num, dtype=np.int32)
        mx = C.c_int(0)
        ms = C.c_double(0.0)
        self._check(lib().portal_adj_list(self._h, int(node_num), int(t.shape[0]), _p(t, P_I), cap, _p(dne, P_I),
                                          _p(num, P_I), C.byref(mx), C.byref(ms)))
        return dne[:mx.value].copy(), num, float(ms.value)

    def field_moments(self) -> np.ndarray:
        """Second moment of line 1's field per node (N, 6): xx yy zz xy xz yz
        of sum w Ibar n n from the last radiation_field call."""
        m = np.zeros((self.N, 6))
        self._check(lib().portal_field_moments(self._h, _p(m)))
        return m

    def node_segments(self) -> np.ndarray:
        """Ray segments of every node in the last radiation-field pass (N,)."""
        seg = np.zeros(self.N, dtype=np.int32)
        self._check(lib().portal_node_segments(self._h, _p(seg, P_I)))
        return seg

    def warmstart_features(self) -> np.ndarray:
        """Features (N, 8) of the warm start from the device-resident
        radiation field of the last radiation_field call."""
        f = np.zeros((self.N, 8), dtype=np.float32)
        self._check(lib().portal_warmstart_features(self._h, _p(f, P_F)))
        return f


P_F = C.POINTER(C.c_float)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


class MLP:
    """The warm start's network (portal_mlp_*): n_in -> width (SiLU) x depth
    -> n_out, trained and evaluated by the library's own BF16 kernels."""

    def __init__(self, n_in: int, width: int, depth: int, n_out: int, seed: int = 0, device: int = 0):
        self._h = C.c_void_p()
        rc = lib().portal_mlp_create(C.byref(self._h), device, n_in, width, depth, n_out, seed)
        if rc != PORTAL_OK:
            raise PortalError(rc, "portal_mlp_create")
        self.n_in, self.width, self.depth, self.n_out = n_in, width, depth, n_out

    def close(self):
        if self._h:
            lib().portal_mlp_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc):
        if rc != PORTAL_OK:
            raise PortalError(rc, lib().portal_mlp_last_error(self._h).decode())

    @property
    def num_params(self) -> int:
        return int(lib().portal_mlp_num_params(self._h))

    def layer_shapes(self):
        """[(fan_out, fan_in)] per layer, the order of the flat parameters."""
        dims = [self.n_in] + [self.width] * self.depth + [self.n_out]
        return [(dims[i + 1], dims[i]) for i in range(len(dims) - 1)]

    def get_params(self):
        p = np.zeros(self.num_params, dtype=np.float32)
        st = np.zeros(2 * (self.n_in + self.n_out), dtype=np.float32)
        self._check(lib().portal_mlp_get_params(self._h, _p(p, P_F), _p(st, P_F)))
        return p, st

    def set_params(self, params=None, stats=None):
        p = None if params is None else _f32(params)
        st = None if stats is None else _f32(stats)
        self._check(lib().portal_mlp_set_params(self._h, _p(p, P_F), _p(st, P_F)))

    def gradients(self, X, T):
        """(loss, flat gradient) of the MSE on standardised X (B, n_in), T (B, n_out)."""
        X, T = _f32(X), _f32(T)
        g = np.zeros(self.num_params, dtype=np.float32)
        loss = C.c_float(0.0)
        self._check(lib().portal_mlp_gradients(self._h, _p(X, P_F), _p(T, P_F), X.shape[0], _p(g, P_F),
                                               C.byref(loss)))
        return float(loss.value), g

    def train(self, X, Y, epochs: int, batch: int, lr: float, seed: int = 0):
        X, Y = _f32(X), _f32(Y)
        losses = np.zeros(epochs, dtype=np.float32)
        self._check(lib().portal_mlp_train(self._h, _p(X, P_F), _p(Y, P_F), X.shape[0], epochs, batch, float(lr),
                                           seed, _p(losses, P_F)))
        return losses

    def predict(self, X):
        X = _f32(X)
        Y = np.zeros((X.shape[0], self.n_out), dtype=np.float32)
        self._check(lib().portal_mlp_predict(self._h, _p(X, P_F), X.shape[0], _p(Y, P_F)))
        return Y


class Batch:
    """Many models in one launch (portal_batch_*): add contexts, prepare
    (tunes the launch shapes, captures the CUDA graph), run passes."""

    def __init__(self, device: int = 0):
        self._h = C.c_void_p()
        rc = lib().portal_batch_create(C.byref(self._h), device)
        if rc != PORTAL_OK:
            raise PortalError(rc, "portal_batch_create")
        self.models = []

    def close(self):
        if self._h:
            lib().portal_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc):
        if rc < 0:
            raise PortalError(rc, lib().portal_batch_last_error(self._h).decode())
        return rc

    def add(self, ctx: "Context") -> int:
        i = self._check(lib().portal_batch_add(self._h, ctx._h))
        self.models.append(ctx)
        return i

    def prepare(self, rc, autotune: bool = True):
        g = _f64(rc.gvec)
        self._check(lib().portal_batch_prepare(self._h, rc.nth, rc.nph, rc.nvel, _p(g), float(rc.dx), rc.n_depth,
                                               rc.kmax, int(bool(autotune))))

    def run(self, use_graph: bool = True):
        """One pass over every model: (segments, device ms)."""
        nseg, ms = C.c_longlong(0), C.c_double(0.0)
        self._check(lib().portal_batch_run(self._h, int(bool(use_graph)), C.byref(nseg), C.byref(ms)))
        return int(nseg.value), float(ms.value)

    def config(self):
        """(line group, RF blocks/SM, SE warps/block, SE blocks/SM) and the
        tuner's (shape, shape, ms) rows."""
        cfg = np.zeros(4, dtype=np.int32)
        tune = np.zeros(64)
        n = self._check(lib().portal_batch_config(self._h, _p(cfg, P_I), _p(tune), 64))
        return tuple(int(v) for v in cfg), tune[:n].reshape(-1, 3)


def wigner3j(tj1, tj2, tj3, tm1, tm2, tm3) -> float:
    return lib().portal_wigner3j(tj1, tj2, tj3, tm1, tm2, tm3)


def wigner6j(tj1, tj2, tj3, tj4, tj5, tj6) -> float:
    return lib().portal_wigner6j(tj1, tj2, tj3, tj4, tj5, tj6)


def coupling_constant(which, j, k, j2, k2):
    c0, c2 = C.c_double(), C.c_double()
    lib().portal_coupling_constant(which, j, k, j2, k2, C.byref(c0), C.byref(c2))
    return c0.value, c2.value
