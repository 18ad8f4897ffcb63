"""Seeded synthetic clouds and molecules in PORTAL's input conventions.

PORTAL post-processes LIME grids: a point set with a Delaunay tetrahedral
mesh (``grid.vtk``), per-point physical columns (``.pop``) and a LAMDA
molecule file.  No such inputs ship with the reference, so this module
builds them from the recipes of the benchmark configurations:

* power-law sphere: radius 1e4 AU, point density ~ r^-1.5 outside a 200 AU
  core (constant inside), n_H2 = 1e5 (r/1000 AU)^-1.5 cm^-3, infall
  v_r = -0.5 (r/1000 AU)^-0.5 km/s, 0.2 km/s microturbulence, LTE
  populations, dust off (gas-to-dust column 0);
* linear rotor: B_rot = 57.6 GHz, dipole 0.11 D, collision rates
  1e-11 |dJ|^-1 cm^3/s downward for every level pair (upward rates come from
  detailed balance inside the SE assembly, pop_eqs.f90:535).

Radii below the core radius are clamped to it in the n_H2, v_r and T laws.

The returned arrays are already in the state that the reference's ingestion
leaves them in (eat_lime.f90:207-311, main_para.f90:119-185): coordinates
divided by r_max, b with thermal broadening added, level number densities,
frequencies in Hz computed with the reference's REAL*4 literals.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

AU = 1.495978707e11          # m
C_LIGHT_CGS = 2.99792458e10   # cm/s
H_CGS = 6.62607015e-27        # erg s
KB_CGS = 1.380649e-16         # erg/K
DEBYE = 1e-18                 # esu cm

F4 = lambda x: float(np.float32(x))  # REAL*4 literal promoted to FP64


@dataclasses.dataclass
class Molecule:
    """A LAMDA molecule after main_para.f90:119-120 and :180-185."""

    nlev: int
    mass: float                 # Daltons
    j_lev: np.ndarray           # (nlev,) int32
    e_cm: np.ndarray            # (nlev,) cm^-1, as in the LAMDA file
    e_levs: np.ndarray          # (nlev,) Hz  (29.9792458E9 REAL*4 * e_cm)
    r_trans: np.ndarray         # (r_num, 2) int32 (lower, upper), 1-based
    A: np.ndarray               # (r_num,)
    freq_ghz: np.ndarray        # (r_num,) as in the LAMDA file
    nu: np.ndarray              # (r_num,) Hz (1E9 REAL*4 * GHz)
    Bij: np.ndarray             # (r_num,)
    kd_v: np.ndarray            # (r_num,) dust opacity m^2/kg
    c_trans: np.ndarray         # (c_num, 2) int32 (lower, upper), 1-based
    col_temps: np.ndarray       # (c_temp,)
    C: np.ndarray               # (c_par, c_num, c_temp) cm^3/s

    @property
    def r_num(self) -> int:
        return int(self.r_trans.shape[0])

    @property
    def c_num(self) -> int:
        return int(self.c_trans.shape[0])

    @property
    def c_temp(self) -> int:
        return int(self.col_temps.shape[0])

    @property
    def c_par(self) -> int:
        return int(self.C.shape[0])


@dataclasses.dataclass
class Cloud:
    """A LIME grid after eat_lime.f90's transforms, plus neighbour CSR."""

    xyz: np.ndarray        # (N,3) normalised by r_max
    vel: np.ndarray        # (N,3) m/s
    b_all: np.ndarray      # (N,) m/s incl. thermal broadening
    t_kin: np.ndarray      # (N,)
    t_dust: np.ndarray     # (N,)
    dust_p: np.ndarray     # (N,) kg/m^3
    h2_dens: np.ndarray    # (N,) m^-3
    ab_all: np.ndarray     # (N,)
    lev_p: np.ndarray      # (N,nlev) m^-3
    bvec: np.ndarray       # (N,3) unit
    nb_off: np.ndarray     # (N+1,) int64 CSR offsets
    nb_idx: np.ndarray     # (nnz,) int32, 0-based, ascending within a node
    tx: float              # r_max in metres
    bulk_node_num: int
    tets: np.ndarray | None = None   # (ntet,4) 0-based, for the grid.vtk writer
    raw: dict | None = None          # LIME columns before ingestion (file writers)

    @property
    def node_num(self) -> int:
        return int(self.xyz.shape[0])

    @property
    def nlev(self) -> int:
        return int(self.lev_p.shape[1])

    @property
    def maxne(self) -> int:
        return int(np.diff(self.nb_off).max())

    def del_ne(self) -> np.ndarray:
        """Reference layout del_ne(N,maxne): returned as a C array of shape
        (maxne, N) so that its memory equals the Fortran column-major array;
        1-based ids, 0 = unused slot."""
        N, maxne = self.node_num, self.maxne
        out = np.zeros((maxne, N), dtype=np.int32)
        deg = np.diff(self.nb_off)
        rows = np.repeat(np.arange(N), deg)
        slot = np.arange(self.nb_idx.shape[0]) - np.repeat(self.nb_off[:-1], deg)
        out[slot, rows] = self.nb_idx + 1
        return out

    def del_num_ne(self) -> np.ndarray:
        return np.diff(self.nb_off).astype(np.int32)


@dataclasses.dataclass
class RunConfig:
    """The parameters that main_portal.x reads from its input file."""

    nth: int
    nph: int
    nvel: int
    kmax: int
    n_depth: int = 10000
    dx: float = F4(1e-6)          # main_para.f90:135
    gvec: tuple = (0.0, 0.0, 1.0)


# --------------------------------------------------------------------------
# molecule
# --------------------------------------------------------------------------

def linear_rotor(nlev: int, b_rot_hz: float = 57.6e9, dipole_debye: float = 0.11,
                 mass: float = 28.0, k0: float = 1e-11,
                 col_temps=(5.0, 10.0, 20.0, 30.0, 40.0, 50.0, 60.0, 80.0, 100.0),
                 dust_table: np.ndarray | None = None) -> Molecule:
    """Synthetic linear rotor in LAMDA conventions.

    E_J = B J(J+1), lines J -> J-1 at 2 B J with the standard dipole
    Einstein A, one collision partner with temperature-independent downward
    rates k0/|dJ| for every pair of levels."""
    J = np.arange(nlev, dtype=np.int32)
    e_cm = b_rot_hz * J * (J + 1) / C_LIGHT_CGS
    e_levs = F4(29.9792458e9) * e_cm                      # main_para.f90:120
    ju = np.arange(1, nlev, dtype=np.int32)
    freq_hz_true = 2.0 * b_rot_hz * ju
    mu = dipole_debye * DEBYE
    A = (64.0 * math.pi ** 4 * freq_hz_true ** 3 * mu * mu /
         (3.0 * H_CGS * C_LIGHT_CGS ** 3)) * ju / (2 * ju + 1)
    freq_ghz = freq_hz_true / 1e9
    nu = F4(1e9) * freq_ghz                               # main_para.f90:119
    r_trans = np.stack([ju, ju + 1], axis=1).astype(np.int32)   # (lower, upper) 1-based
    g = 2 * J + 1
    a_to_b = 1.6179542e57                                 # main_para.f90:178
    g1 = g[r_trans[:, 0] - 1].astype(np.float64)
    g2 = g[r_trans[:, 1] - 1].astype(np.float64)
    Bij = (g2 / g1) * A * a_to_b / nu ** 3                # main_para.f90:184
    pairs = [(lo, up) for up in range(2, nlev + 1) for lo in range(1, up)]
    c_trans = np.array(pairs, dtype=np.int32).reshape(-1, 2)
    dJ = (c_trans[:, 1] - c_trans[:, 0]).astype(np.float64)
    ct = np.asarray(col_temps, dtype=np.float64)
    C = np.repeat((k0 / dJ)[None, :, None], ct.shape[0], axis=2)
    if dust_table is None:
        dust_table = default_dust_table()
    kd_v = dust_to_opacities(nu, dust_table)
    return Molecule(nlev=nlev, mass=mass, j_lev=J, e_cm=e_cm, e_levs=e_levs, r_trans=r_trans,
                    A=A, freq_ghz=freq_ghz, nu=nu, Bij=Bij, kd_v=kd_v, c_trans=c_trans,
                    col_temps=ct, C=C)


def default_dust_table(n: int = 67) -> np.ndarray:
    """67-row (wavelength micron, kappa cm^2/g) power-law table, the row
    count eat_lime.f90:84 expects."""
    lam = np.logspace(-1, 4, n)
    kap = 1e3 * (lam / 1.0) ** -1.5
    return np.stack([lam, kap], axis=1)


def dust_to_opacities(nu_hz: np.ndarray, table: np.ndarray) -> np.ndarray:
    """dust_to_opacities miscellaneous.f90:643-700 (table log10 per
    eat_lime.f90:290-293; the reference's argument is nu*1E9 with nu in
    GHz, i.e. the nu_hz here)."""
    lt = np.log10(table[:, 0])
    lk = np.log10(table[:, 1])
    out = np.zeros(nu_hz.shape[0])
    n_dt = lt.shape[0]
    for i, nu in enumerate(nu_hz):
        mu0 = math.log10(F4(2.998e14) / nu)
        kd_m = float("nan")
        for j in range(n_dt - 1):
            if lt[j] < mu0 < lt[j + 1]:
                mu_res = (mu0 - lt[j]) / (lt[j + 1] - lt[j])
                kd_m = lk[j] + mu_res * (lk[j + 1] - lk[j])
                break
        if mu0 > lt[n_dt - 1]:
            mu_res = (mu0 - lt[n_dt - 1]) / (lt[n_dt - 1] - lt[n_dt - 2])
            kd_m = lk[n_dt - 1] + mu_res * (lk[n_dt - 1] - lk[n_dt - 2])
        out[i] = 10.0 ** kd_m * F4(1e-1)
    return out


# --------------------------------------------------------------------------
# cloud
# --------------------------------------------------------------------------

def neighbours_from_tets(tets: np.ndarray, n: int):
    """adj_list_no_delaunay miscellaneous.f90:910-1015 + SortUnique
    unique.f90:43-59: every tetrahedron gives each of its vertices the other
    three; the per-node lists are sorted ascending and de-duplicated."""
    t = tets.astype(np.int64)
    src = np.repeat(t, 3, axis=1).reshape(-1)
    others = np.stack([t[:, [1, 2, 3]], t[:, [0, 2, 3]], t[:, [0, 1, 3]], t[:, [0, 1, 2]]],
                      axis=1).reshape(-1)
    key = np.unique(src * n + others)
    s = key // n
    d = (key % n).astype(np.int32)
    off = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(np.bincount(s, minlength=n), out=off[1:])
    return off, d


def _radii_power_law(rng, n, r_out, r_core, p=1.5):
    """Radii of points with density ~ r^-p outside r_core, uniform inside."""
    q = 3.0 - p
    m_in = r_core ** q / 3.0
    m_out = (1.0 / q) * (r_out ** q - r_core ** q)
    u = rng.random(n) * (m_in + m_out)
    r = np.empty(n)
    inner = u < m_in
    r[inner] = np.cbrt(3.0 * u[inner] * r_core ** p)
    r[~inner] = (q * (u[~inner] - m_in) + r_core ** q) ** (1.0 / q)
    return r


def lte_fractions(mol: Molecule, T: np.ndarray) -> np.ndarray:
    g = (2 * mol.j_lev + 1).astype(np.float64)
    e_k = H_CGS * C_LIGHT_CGS * mol.e_cm / KB_CGS      # level energies in K
    w = g[None, :] * np.exp(-e_k[None, :] / T[:, None])
    return w / w.sum(axis=1, keepdims=True)


def power_law_sphere(n_points: int, seed: int, mol: Molecule, *, t_law: str = "uniform",
                     t_uniform: float = 20.0, b_random: float = 0.0,
                     abundance: float = 1e-4, r_out_au: float = 1e4, r_core_au: float = 200.0,
                     micro_turb: float = 200.0, keep_raw: bool = False, density_exp: float = 1.5,
                     n0_cm3: float = 1e5, b_dir=(0.0, 0.0, 1.0)) -> Cloud:
    """The power-law sphere of the benchmark configurations: points and
    n_H2 = n0_cm3 (r/1000 AU)^-density_exp outside a core of r_core_au.

    t_law "uniform" (T = t_uniform) or "loglinear" (40 K at the core radius
    falling linearly in log r to 10 K at the edge).  b_random is the rms of
    an isotropic Gaussian component added to a unit field along b_dir."""
    from scipy.spatial import Delaunay

    rng = np.random.default_rng(seed)
    r = _radii_power_law(rng, n_points, r_out_au, r_core_au, density_exp)
    u = rng.normal(size=(n_points, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    pos_au = u * r[:, None]
    pos_m = pos_au * AU
    tri = Delaunay(pos_m)
    tets = tri.simplices.astype(np.int32)
    off, idx = neighbours_from_tets(tets, n_points)

    r_eff = np.maximum(r, r_core_au)
    n_h2 = n0_cm3 * 1e6 * (r_eff / 1000.0) ** -density_exp          # m^-3
    if t_law == "uniform":
        T = np.full(n_points, float(t_uniform))
    else:
        f = np.log(r_eff / r_core_au) / math.log(r_out_au / r_core_au)
        T = 40.0 - 30.0 * f
    v_r = -0.5e3 * (r_eff / 1000.0) ** -0.5                          # m/s
    vel = u * v_r[:, None]
    b_turb = np.full(n_points, micro_turb)
    ab = np.full(n_points, abundance)
    gas_ii_dust = np.zeros(n_points)
    bvec = np.tile(np.asarray(b_dir, dtype=np.float64), (n_points, 1))
    if b_random > 0.0:
        bvec = bvec + b_random * rng.normal(size=(n_points, 3))
    bvec /= np.linalg.norm(bvec, axis=1, keepdims=True)
    frac = lte_fractions(mol, T)

    raw = dict(pos_m=pos_m, vel=vel, n_h2=n_h2, t_kin=T.copy(), t_dust=T.copy(), b=b_turb,
               ab=ab, gas_ii_dust=gas_ii_dust, frac=frac)
    return ingest(raw, mol, off, idx, bvec, bulk_node_num=n_points,
                  tets=tets if keep_raw else None, keep_raw=keep_raw)


def ingest(raw: dict, mol: Molecule, off, idx, bvec, bulk_node_num: int, tets=None,
           keep_raw=False) -> Cloud:
    """eat_lime_no_delaunay eat_lime.f90:207-311 applied to LIME columns."""
    pos = np.asarray(raw["pos_m"], dtype=np.float64)
    n = pos.shape[0]
    nb = bulk_node_num
    vel = np.zeros((n, 3)); vel[:nb] = raw["vel"][:nb]
    h2 = np.ones(n); h2[:nb] = raw["n_h2"][:nb]
    tk = np.zeros(n); tk[:nb] = raw["t_kin"][:nb]
    td = np.zeros(n); td[:nb] = raw["t_dust"][:nb]
    b = np.full(n, 200.0); b[:nb] = raw["b"][:nb]
    ab = np.full(n, 1e-3); ab[:nb] = raw["ab"][:nb]
    g2d = np.zeros(n); g2d[:nb] = raw["gas_ii_dust"][:nb]
    lev = np.zeros((n, mol.nlev)); lev[:nb] = raw["frac"][:nb]
    if nb < n:                                         # eat_lime.f90:227-245
        s = np.ones(n - nb)
        lev[nb:, 0] = 1.0
        for k in range(1, mol.nlev):
            lev[nb:, k] = np.exp(-mol.e_cm[k] * 0.527)
            s = s + lev[nb:, k]
        lev[nb:] /= s[:, None]
    b = np.sqrt(b ** 2 + 2.0 * 8314.462 * tk / mol.mass)               # :250-258
    lev = lev * (ab * h2)[:, None]                                     # :261-263
    rmax = float(np.sqrt((pos ** 2).sum(axis=1)).max())                # :269-274
    xyz = pos / rmax
    dust_p = np.where(g2d != 0.0, h2 * F4(2.32e-27) / np.where(g2d != 0.0, g2d, 1.0), 0.0)
    return Cloud(xyz=np.ascontiguousarray(xyz), vel=np.ascontiguousarray(vel), b_all=b,
                 t_kin=tk, t_dust=td, dust_p=dust_p, h2_dens=h2, ab_all=ab,
                 lev_p=np.ascontiguousarray(lev), bvec=np.ascontiguousarray(bvec),
                 nb_off=off, nb_idx=idx, tx=rmax, bulk_node_num=nb, tets=tets,
                 raw=raw if keep_raw else None)


def gaussian_field(rng, n: int, slope: float = -11.0 / 3.0, components: int = 1) -> np.ndarray:
    """Periodic Gaussian random field on an n^3 grid with power spectrum
    P(k) ~ k^slope, zero mean, unit rms per component; shape (components, n, n, n)."""
    k = np.fft.fftfreq(n) * n
    kx, ky, kz = np.meshgrid(k, k, k, indexing="ij")
    kk = np.sqrt(kx * kx + ky * ky + kz * kz)
    amp = np.zeros_like(kk)
    amp[kk > 0] = kk[kk > 0] ** (slope / 2.0)
    out = np.empty((components, n, n, n))
    for c in range(components):
        w = np.fft.fftn(rng.normal(size=(n, n, n)))
        f = np.fft.ifftn(w * amp).real
        f -= f.mean()
        out[c] = f / f.std()
    return out


def _trilinear(field: np.ndarray, u: np.ndarray) -> np.ndarray:
    """Periodic trilinear interpolation of field (C, n, n, n) at points u in
    [0, 1)^3 (shape (M, 3)); returns (M, C)."""
    n = field.shape[1]
    g = u * n
    i0 = np.floor(g).astype(np.int64)
    f = g - i0
    out = np.zeros((u.shape[0], field.shape[0]))
    for dx in (0, 1):
        wx = f[:, 0] if dx else 1 - f[:, 0]
        for dy in (0, 1):
            wy = f[:, 1] if dy else 1 - f[:, 1]
            for dz in (0, 1):
                wz = f[:, 2] if dz else 1 - f[:, 2]
                ix = (i0[:, 0] + dx) % n
                iy = (i0[:, 1] + dy) % n
                iz = (i0[:, 2] + dz) % n
                out += (wx * wy * wz)[:, None] * field[:, ix, iy, iz].T
    return out


def turbulent_cube(n_points: int, seed: int, mol: Molecule, *, grid: int = 64, sigma_ln: float = 1.5,
                   n_mean_cm3: float = 1e4, v_rms: float = 1.0e3, T: float = 20.0, abundance: float = 1e-4,
                   micro_turb: float = 200.0, size_pc: float = 1.0, keep_raw: bool = False) -> Cloud:
    """The turbulent cloud of the 1M-point configuration: points uniform in a
    cube of side size_pc; ln(density) a k^-11/3 Gaussian random field with
    sigma_ln, scaled to mean n_mean_cm3; velocity a k^-11/3 Gaussian random
    field with v_rms (3D); field = unit mean along x plus an equal-rms
    turbulent part with the same spectrum.  The periodic fields are sampled
    trilinearly; the reference's domain is the unit sphere around the
    points (eat_lime.f90:269-279), so the cube is treated as non-periodic."""
    from scipy.spatial import Delaunay

    PC = 3.0856775814913673e16
    rng = np.random.default_rng(seed)
    u = rng.random((n_points, 3))
    pos_m = (u - 0.5) * size_pc * PC
    lnrho = gaussian_field(rng, grid)
    vel_f = gaussian_field(rng, grid, components=3)
    b_f = gaussian_field(rng, grid, components=3)
    s = _trilinear(lnrho, u)[:, 0] * sigma_ln
    n_h2 = np.exp(s)
    n_h2 *= n_mean_cm3 / n_h2.mean()
    n_h2 *= 1e6                                                   # m^-3
    vel = _trilinear(vel_f, u) * (v_rms / math.sqrt(3.0))
    bt = _trilinear(b_f, u) / math.sqrt(3.0)
    bvec = bt + np.array([1.0, 0.0, 0.0])
    bvec /= np.linalg.norm(bvec, axis=1, keepdims=True)
    tri = Delaunay(pos_m)
    tets = tri.simplices.astype(np.int32)
    off, idx = neighbours_from_tets(tets, n_points)
    Tk = np.full(n_points, float(T))
    raw = dict(pos_m=pos_m, vel=vel, n_h2=n_h2, t_kin=Tk, t_dust=Tk.copy(), b=np.full(n_points, micro_turb),
               ab=np.full(n_points, abundance), gas_ii_dust=np.zeros(n_points), frac=lte_fractions(mol, Tk))
    return ingest(raw, mol, off, idx, bvec, bulk_node_num=n_points, tets=tets if keep_raw else None,
                  keep_raw=keep_raw)


def batch_cloud(i: int, points_scale: float = 1.0, n_min: int = 10000, n_max: int = 300000):
    """Cloud i of the batched uneven configuration: seed 100 + i, a point
    count log-uniform in [n_min, n_max] (times points_scale), a linear rotor
    of 5..20 levels, density exponent uniform in 1..2, n0 log-uniform in
    1e4..1e7 cm^-3 and an isotropically drawn field direction; T = 20 K.
    Returns (cloud, molecule)."""
    rng = np.random.default_rng(100 + i)
    n = int(round(math.exp(rng.uniform(math.log(n_min), math.log(n_max))) * points_scale))
    nlev = int(rng.integers(5, 21))
    p = float(rng.uniform(1.0, 2.0))
    n0 = float(10.0 ** rng.uniform(4.0, 7.0))
    b = rng.normal(size=3)
    b /= np.linalg.norm(b)
    mol = linear_rotor(nlev)
    cloud = power_law_sphere(max(n, 64), 100 + i, mol, density_exp=p, n0_cm3=n0, b_dir=tuple(b))
    return cloud, mol


BATCH_RUN_CONFIG = dict(nth=16, nph=16, nvel=32, kmax=2)


def batch_clouds(n_clouds: int = 64, points_scale: float = 1.0, n_min: int = 10000, n_max: int = 300000):
    """The batched uneven configuration: clouds batch_cloud(0..n_clouds-1).
    Returns [(cloud, molecule)] and the run configuration shared by all
    (16x16 directions, 65 channels, kmax 2)."""
    out = [batch_cloud(i, points_scale, n_min, n_max) for i in range(n_clouds)]
    rc = RunConfig(gvec=gauge_vector(3), **BATCH_RUN_CONFIG)
    return out, rc


def gauge_vector(seed: int) -> tuple:
    """main_para.f90:172-176 draws three uniform numbers and normalises
    them; here the draw is seeded so both paths share it."""
    g = np.random.default_rng(seed + 7919).random(3)
    g = g / math.sqrt(g[0] ** 2 + g[1] ** 2 + g[2] ** 2)
    return tuple(float(x) for x in g)


# --------------------------------------------------------------------------
# the benchmark configurations
# --------------------------------------------------------------------------

def config_cloud(name: str, n_points: int | None = None, keep_raw: bool = False):
    """(cloud, molecule, run config) for a named configuration.

    "sphere4k": 4,096 points, seed 0, 5-level rotor, T = 20 K, B along z,
            16x16 directions, 65 channels (nvel = 32);
    "sphere262k": 262,144 points, seed 1, 10-level rotor, T 10-40 K linear in
            log r, B along z + 30% Gaussian component, 24x24 directions,
            129 channels (nvel = 64);
    "cube1m": 1,048,576 points of the turbulent cube (seed 4), 20-level
            rotor, 32x32 directions, 129 channels, kmax 2.
    n_points overrides the point count (smaller parity cases); keep_raw
    keeps the tetrahedra and the LIME columns (file writers, neighbour-list
    checks)."""
    if name == "sphere4k":
        mol = linear_rotor(5)
        n = n_points or 4096
        cloud = power_law_sphere(n, 0, mol, t_law="uniform", t_uniform=20.0, keep_raw=keep_raw)
        rc = RunConfig(nth=16, nph=16, nvel=32, kmax=6, gvec=gauge_vector(0))
    elif name == "sphere262k":
        mol = linear_rotor(10)
        n = n_points or 262144
        cloud = power_law_sphere(n, 1, mol, t_law="loglinear", b_random=0.3, keep_raw=keep_raw)
        rc = RunConfig(nth=24, nph=24, nvel=64, kmax=6, gvec=gauge_vector(1))
    elif name == "cube1m":
        mol = linear_rotor(20)
        n = n_points or 1048576
        cloud = turbulent_cube(n, 4, mol, grid=128 if n > 200000 else 64, keep_raw=keep_raw)
        rc = RunConfig(nth=32, nph=32, nvel=64, kmax=2, gvec=gauge_vector(4))
    else:
        raise ValueError(f"unknown configuration {name!r}")
    return cloud, mol, rc
