"""The named workloads and the bench's bookkeeping (CPU only): the seeded
stand-ins have the shapes the measurements quote, and the per-segment ncu
figures the bench reads from profiles/ are present."""
import os
import sys

import numpy as np
import pytest

from portal_gb300 import synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("name,nlev,nth,nvel,kmax", [("sphere4k", 5, 16, 32, 6), ("sphere262k", 10, 24, 64, 6),
                                                     ("cube1m", 20, 32, 64, 2)])
def test_named_workloads_have_the_quoted_shapes(name, nlev, nth, nvel, kmax):
    """sphere4k / sphere262k / cube1m at a reduced point count: levels,
    directions (nth = nph), channels (2 nvel + 1) and kmax as quoted; lines =
    levels - 1 for the linear rotor; seeded (two builds are identical)."""
    cloud, mol, rc = synth.config_cloud(name, n_points=2048)
    assert mol.nlev == nlev and mol.r_num == nlev - 1
    assert rc.nth == rc.nph == nth and 2 * rc.nvel + 1 == 2 * nvel + 1 and rc.kmax == kmax
    assert cloud.node_num >= 2048 and cloud.bulk_node_num <= cloud.node_num
    assert np.all(np.linalg.norm(cloud.xyz, axis=1) <= 1.0 + 1e-12)
    cloud2, _, _ = synth.config_cloud(name, n_points=2048)
    np.testing.assert_array_equal(cloud.xyz, cloud2.xyz)
    np.testing.assert_array_equal(cloud.lev_p, cloud2.lev_p)


def test_direction_counts_match_legendre_all():
    """388 rays per node at 24 x 24 and 678 at 32 x 32 (ceil(nph sin th) per
    Gauss-Legendre ring, miscellaneous.f90:1100-1137), the counts the
    throughput figures use."""
    import oracle
    assert len(oracle.legendre_all(24, 24)) == 388
    assert len(oracle.legendre_all(32, 32)) == 678
    assert len(oracle.legendre_all(16, 16)) == 178


def test_bench_reads_the_profile_figures():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.profile_constant("dram_bytes_per_segment") == pytest.approx(0.40)
    assert bench.profile_constant("warp_instructions_per_segment") == pytest.approx(373.0)
    assert bench.profile_constant("no_such_figure") is None


def test_se_lu_rates():
    """The SE stages' FP32 factorisation rate: 2/3 n^3 flop per node, against
    SMs x 128 lanes x 2 flop x clock."""
    import bench
    r = bench.lu_rates(262144, 34, 15.0, 152, 2070.0)
    assert r["fp32_lu_flop_per_s"] == pytest.approx(262144 * (2.0 / 3.0) * 34 ** 3 / 0.015)
    assert r["fp32_peak_flop_per_s"] == pytest.approx(152 * 128 * 2 * 2070e6)
    assert r["fp32_lu_frac"] == pytest.approx(r["fp32_lu_flop_per_s"] / r["fp32_peak_flop_per_s"])
    assert set(bench.lu_rates(10, 34, 1.0)) == {"fp32_lu_flop_per_s"}
