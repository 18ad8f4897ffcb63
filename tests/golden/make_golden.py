"""Generate the golden fixtures that pin the oracle (run from the repo root:
``python tests/golden/make_golden.py``).

The reference ships no tests, fixtures or data, so the oracle is pinned at the
boundaries where PORTAL calls third-party arithmetic, against independent
exact or library values:

* wigner.json   -- Wigner 3j / 6j symbols from sympy's exact evaluation
                   (wigxjpf's fwig3jj / fwig6jj call sites: pop_eqs.f90:48-61,
                   :127-140, :194, :252-265, :331-344, em_coefs.f90:42-46);
* leggauss.json -- Gauss-Legendre knots / weights from numpy (IQPACK's cdgqf,
                   legendre_rule.f90:1-84, as called by miscellaneous.f90:1117)
                   and the direction counts of legendre_all;
* lapack.json   -- LAPACK dgetrf + dgetri (scipy) on a fixed polarized SE
                   matrix, the first column of the inverse (em_coefs.f90:169-186).
"""
import json
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def wigner():
    from sympy import N
    from sympy.physics.wigner import wigner_3j, wigner_6j

    rng = np.random.default_rng(12345)
    three, six = [], []
    # the families the coupling constants use, up to J = 20
    for j in range(0, 21):
        for k in range(0, min(2 * j, 8) + 1, 2):
            for m in range(-j, j + 1, max(1, j // 3)):
                three.append((j, j, k, m, -m, 0))
        for jp in (j - 1, j + 1):
            if jp < 0:
                continue
            for m in range(-j, j + 1, max(1, j // 2)):
                for q in (-1, 0, 1):
                    if abs(m - q) <= jp:
                        three.append((jp, j, 1, -(m - q), m, -q))
    for q in (-1, 0, 1):
        three.append((1, 1, 0, q, -q, 0))
        three.append((1, 1, 2, q, -q, 0))
    # random generic ones
    while len(three) < 600:
        j1, j2 = int(rng.integers(0, 25)), int(rng.integers(0, 25))
        j3 = int(rng.integers(abs(j1 - j2), j1 + j2 + 1))
        m1 = int(rng.integers(-j1, j1 + 1)); m2 = int(rng.integers(-j2, j2 + 1))
        if abs(m1 + m2) <= j3:
            three.append((j1, j2, j3, m1, m2, -m1 - m2))
    for j in range(0, 21):
        for k in range(0, min(2 * j, 8) + 1, 2):
            for jp in (j - 1, j, j + 1):
                if jp >= 0:
                    six.append((jp, jp, k, j, j, 1))
        for jp in (j - 1, j + 1):
            if jp >= 0:
                six.append((1, 1, 2, j, j, jp))
    while len(six) < 300:
        a = [int(x) for x in rng.integers(0, 16, size=6)]
        six.append(tuple(a))
    out3 = [list(t) + [str(N(wigner_3j(*t), 30))] for t in three]
    out6 = [list(t) + [str(N(wigner_6j(*t), 30))] for t in six]
    with open(os.path.join(HERE, "wigner.json"), "w") as f:
        json.dump({"source": "sympy.physics.wigner (exact), 30 digits", "w3j": out3, "w6j": out6}, f)


def _gl_mpmath(n, dps=40):
    """Gauss-Legendre rule to 40 digits: Newton on P_n in mpmath."""
    import mpmath as mp
    mp.mp.dps = dps
    xs, ws = [], []
    for i in range(n):
        z = mp.cos(mp.pi * (i + mp.mpf(3) / 4) / (n + mp.mpf(1) / 2))
        for _ in range(100):
            p0, p1 = mp.mpf(1), z
            for k in range(2, n + 1):
                p0, p1 = p1, ((2 * k - 1) * z * p1 - (k - 1) * p0) / k
            dp = n * (z * p1 - p0) / (z * z - 1)
            dz = p1 / dp
            z -= dz
            if abs(dz) < mp.mpf(10) ** (-dps + 5):
                break
        p0, p1 = mp.mpf(1), z
        for k in range(2, n + 1):
            p0, p1 = p1, ((2 * k - 1) * z * p1 - (k - 1) * p0) / k
        dp = n * (z * p1 - p0) / (z * z - 1)
        xs.append(z); ws.append(2 / ((1 - z * z) * dp * dp))
    order = sorted(range(n), key=lambda i: xs[i])
    return [mp.nstr(xs[i], 30) for i in order], [mp.nstr(ws[i], 30) for i in order]


def leggauss():
    out = {"source": "numpy.polynomial.legendre.leggauss and a 40-digit mpmath Newton iteration",
           "rules": {}, "exact": {}, "n_sphere": {}}
    for n in (8, 16, 24, 32, 64):
        x, w = np.polynomial.legendre.leggauss(n)
        out["rules"][str(n)] = {"x": [float(v) for v in x], "w": [float(v) for v in w]}
        xe, we = _gl_mpmath(n)
        out["exact"][str(n)] = {"x": xe, "w": we}
        cnt = sum(int(math.ceil(n * math.sin(math.acos(xi)))) for xi in x)
        out["n_sphere"][str(n)] = cnt
    with open(os.path.join(HERE, "leggauss.json"), "w") as f:
        json.dump(out, f)


def lapack():
    """dgetrf/dgetri on a polarized SE matrix built by the oracle for node 1
    of the 4,096-point configuration (J from the oracle's radiation field)."""
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    import oracle
    from portal_gb300 import synth
    from scipy.linalg import lapack as la

    cloud, mol, rc = synth.config_cloud("sphere4k")
    P = oracle.OracleProblem(cloud, mol)
    J0, J2, _, _, _ = P.radiation_field(rc, 1, 4)
    out = {"source": "scipy.linalg.lapack dgetrf + dgetri", "cases": []}
    for node in (1, 2, 3, 4):
        A = P.node_matrix(rc.kmax, node, J0, J2)
        n = A.shape[0]
        ca, c = [], 0
        for j in mol.j_lev:
            ca.append(c)
            c += len(range(0, min(2 * int(j), rc.kmax) + 1, 2))
        A[0, :] = 0.0
        for i, j in enumerate(mol.j_lev):
            A[0, ca[i]] = math.sqrt(2 * int(j) + 1)
        lu, piv, info = la.dgetrf(A)
        inv, info2 = la.dgetri(lu, piv)
        out["cases"].append({"node": node, "kmax": rc.kmax, "A": A.tolist(), "rho": inv[:, 0].tolist(),
                             "J0": J0[node - 1].tolist(), "J2": J2[node - 1].tolist()})
    with open(os.path.join(HERE, "lapack.json"), "w") as f:
        json.dump(out, f)


if __name__ == "__main__":
    wigner()
    leggauss()
    lapack()
