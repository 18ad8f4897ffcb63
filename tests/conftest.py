import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs an sm_103a GPU (GB300)")


@pytest.fixture(scope="session")
def built_lib():
    from portal_gb300 import build
    return build.build()


@pytest.fixture(scope="session")
def sphere4k():
    from portal_gb300 import synth
    return synth.config_cloud("sphere4k")


@pytest.fixture(scope="session")
def sphere4k_oracle(sphere4k):
    """Oracle radiation field + SE of all sphere4k nodes (FP64, OpenMP)."""
    import oracle
    cloud, mol, rc = sphere4k
    P = oracle.OracleProblem(cloud, mol)
    J0, J2, st, nseg, nfail = P.radiation_field(rc)
    pp, st2, nf2 = P.solve_se(rc.kmax, J0, J2)
    return dict(P=P, J0=J0, J2=J2, nseg=nseg, pops=pp)
