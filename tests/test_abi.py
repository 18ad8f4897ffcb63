"""The C-ABI library: it builds, loads, exports what include/ declares, and its
host-side numerics (Wigner tables, coupling constants) are pinned.  CPU only."""
import ctypes as C
import json
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")


def declared_symbols():
    syms = set()
    for name in os.listdir(os.path.join(ROOT, "include")):
        if name.endswith(".h"):
            text = open(os.path.join(ROOT, "include", name)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            syms |= set(re.findall(r"\b(portal_\w+)\s*\(", text))
    return sorted(syms)


def test_library_exports_every_declared_symbol(built_lib):
    L = C.CDLL(built_lib)
    syms = declared_symbols()
    assert len(syms) >= 13
    missing = [s for s in syms if not hasattr(L, s)]
    assert not missing, missing


def test_python_mirror_binds_every_declared_symbol(built_lib):
    import portal_gb300 as pg
    assert set(declared_symbols()) <= set(pg.EXPORTS)


def _c_param_counts():
    text = open(os.path.join(ROOT, "include", "portal_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    out = {}
    for m in re.finditer(r"\b(portal_\w+)\s*\(([^;{]*?)\)\s*;", text):
        params = m.group(2).strip()
        out[m.group(1)] = 0 if params in ("", "void") else len(params.split(","))
    return out


def test_fortran_interface_matches_header():
    """include/portal_gb300.f90 (the ISO_C_BINDING module a Fortran caller
    uses): every bind(C) name is a header entry point with the same number of
    arguments, and every dummy argument has a declaration."""
    f = re.sub(r"!.*", "", open(os.path.join(ROOT, "include", "portal_gb300.f90")).read())
    f = f.replace("&\n", " ").replace("&", " ")
    c = _c_param_counts()
    found = 0
    for m in re.finditer(r"function\s+(\w+)\s*\(([^)]*)\)\s*bind\(C,\s*name=\"(\w+)\"\)(.*?)end function", f,
                         flags=re.S):
        name, args, cname, body = m.group(1), m.group(2), m.group(3), m.group(4)
        assert name == cname and cname in c, cname
        dummies = [a.strip() for a in args.split(",") if a.strip()]
        assert len(dummies) == c[cname], (cname, len(dummies), c[cname])
        declared = set(re.findall(r"::\s*([^\n]+)", body))
        names = {v.strip() for d in declared for v in re.sub(r"\([^)]*\)", "", d).split(",")}
        assert set(dummies) <= names, (cname, set(dummies) - names)
        found += 1
    assert found >= 10


def test_create_without_device_fails_loudly(built_lib):
    """No silent CPU path: without an sm_103a device portal_create refuses."""
    import portal_gb300 as pg
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("a GPU is present")
    with pytest.raises(pg.PortalError) as e:
        pg.Context(0)
    assert e.value.code == -7


def test_strerror_covers_codes(built_lib):
    import portal_gb300 as pg
    for code in range(0, -8, -1):
        assert pg.lib().portal_strerror(code).decode() != "unknown error"


def test_product_wigner_against_sympy(built_lib):
    import portal_gb300 as pg
    with open(os.path.join(GOLD, "wigner.json")) as f:
        g = json.load(f)
    worst = 0.0
    for row in g["w3j"]:
        *a, v = row
        ex = float(v)
        got = pg.wigner3j(*[2 * x for x in a])
        worst = max(worst, abs(got - ex) / abs(ex) if ex != 0 else abs(got))
    for row in g["w6j"]:
        *a, v = row
        ex = float(v)
        got = pg.wigner6j(*[2 * x for x in a])
        worst = max(worst, abs(got - ex) / abs(ex) if ex != 0 else abs(got))
    assert worst < 1e-14, worst


def test_product_coupling_constants_match_oracle(built_lib):
    import oracle
    import portal_gb300 as pg
    for which in range(5):
        for j in range(0, 20):
            for j2 in (j - 1, j, j + 1):
                if j2 < 0:
                    continue
                for k in range(0, min(2 * j, 6) + 1, 2):
                    for k2 in range(0, min(2 * j2, 6) + 1, 2):
                        a = pg.coupling_constant(which, j, k, j2, k2)
                        b = oracle.coupling_constant(which, j, k, j2, k2)
                        for x, y in zip(a, b):
                            assert abs(x - y) <= 1e-13 * max(1.0, abs(y)), (which, j, k, j2, k2, x, y)
