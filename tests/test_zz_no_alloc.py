"""The allocation-free radiation-field entry point.

portal_radiation_field_static exists for callers that cannot call cudaMalloc
(their device memory belongs to a pool they do not control, or they may not
allocate between simulation steps).  They keep the reference-layout cloud
arrays on the device themselves and hand the library only device pointers;
the library's scratch is a fixed array in its own image.

These tests play such a caller: torch allocates the device arrays (the
caller may allocate; the entry point may not), the entry point is called
through the C ABI -- twice in a row on the same arrays -- and its results are
checked against the context-based portal_radiation_field and against the
FP64 oracle within the tolerances of the parity tests, over every channel
layout of its kernel, with surface nodes (bulk < N) whose rows the caller
left as garbage, and with walks that overflow n_depth.  The file is
collected last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _limits():
    import portal_gb300 as pg
    L = pg.lib()
    max_depth = C.c_int()
    scratch = C.c_longlong()
    L.portal_radiation_field_static_limits(C.byref(max_depth), None, None, None, C.byref(scratch))
    return max_depth.value, scratch.value


def _call_static(cloud, mol, rc, calls=1):
    """portal_radiation_field_static on device copies of the cloud; J0/J2
    prefilled with NaN and status with -1 before each call.  Returns the
    host copies of (J0, J2, status) of every call."""
    import torch

    import portal_gb300 as pg
    L = pg.lib()
    dev = torch.device("cuda:0")
    N, R = cloud.node_num, mol.r_num
    temp = np.stack([cloud.t_kin, cloud.t_dust], axis=1)
    host = [cloud.xyz, cloud.vel, cloud.b_all, temp, cloud.dust_p, cloud.ab_all, cloud.lev_p, cloud.bvec]
    d = [torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).to(dev) for a in host]
    del_ne = torch.from_numpy(np.ascontiguousarray(cloud.del_ne(), dtype=np.int32)).to(dev)
    del_num = torch.from_numpy(np.ascontiguousarray(cloud.del_num_ne(), dtype=np.int32)).to(dev)
    mol_h = [np.ascontiguousarray(mol.j_lev, dtype=np.int32), np.ascontiguousarray(mol.r_trans, dtype=np.int32),
             np.ascontiguousarray(mol.A), np.ascontiguousarray(mol.nu), np.ascontiguousarray(mol.Bij),
             np.ascontiguousarray(mol.kd_v)]
    g = np.ascontiguousarray(rc.gvec, dtype=np.float64)
    stream = torch.cuda.current_stream().cuda_stream
    out = []
    for call in range(calls):
        J0 = torch.full((N, R), float("nan"), dtype=torch.float64, device=dev)
        J2 = torch.full((N, R), float("nan"), dtype=torch.float64, device=dev)
        st = torch.full((N,), -1, dtype=torch.int32, device=dev)
        code = L.portal_radiation_field_static(
            stream, N, cloud.bulk_node_num, cloud.nlev, *[t.data_ptr() for t in d], del_ne.shape[0],
            del_ne.data_ptr(), del_num.data_ptr(), float(cloud.tx),
            mol_h[0].ctypes.data_as(pg.P_I), R, mol_h[1].ctypes.data_as(pg.P_I),
            *[a.ctypes.data_as(pg.P_D) for a in mol_h[2:]], rc.nth, rc.nph, rc.nvel,
            g.ctypes.data_as(pg.P_D), float(rc.dx), rc.n_depth, J0.data_ptr(), J2.data_ptr(), st.data_ptr())
        assert code == 0, (call, code)
        torch.cuda.synchronize()
        out.append((J0.cpu().numpy(), J2.cpu().numpy(), st.cpu().numpy()))
    return out


def test_static_scratch_entry_point_matches_context_path_and_oracle(built_lib, sphere4k, sphere4k_oracle):
    import portal_gb300 as pg
    from test_gpu_parity import _check_J

    max_depth, scratch = _limits()
    assert scratch == 64 << 20 and max_depth >= 512
    cloud, mol, rc = sphere4k
    rc = type(rc)(**{**rc.__dict__, "n_depth": max_depth})
    with pg.Context(0) as ctx:
        ctx.set_molecule(mol)
        ctx.set_cloud(cloud)
        J0_ref, J2_ref, st_ref, _ = ctx.radiation_field(rc)
    assert not st_ref.any()
    for J0, J2, st in _call_static(cloud, mol, rc, calls=2):
        assert (st == 0).all()
        _check_J(J0, J2, J0_ref, J2_ref)
        _check_J(J0, J2, sphere4k_oracle["J0"], sphere4k_oracle["J2"])


@pytest.mark.parametrize("nvel", [8, 64, 100])
def test_static_entry_point_channel_layouts_and_surface_nodes(built_lib, nvel):
    """nvel 8, 64 and 100 run the kernel's 1-, 5- and 9-slot variants (17,
    129 and 201 channels); the last 64 nodes are surface nodes (bulk < N),
    whose rows must come back zero although the caller's buffers held NaN
    and -1 before the call."""
    import oracle
    from portal_gb300 import synth
    from test_gpu_parity import _check_J
    mol = synth.linear_rotor(5)
    cloud = synth.power_law_sphere(1024, 7, mol, t_uniform=20.0)
    cloud.bulk_node_num = cloud.node_num - 64
    cloud.ab_all[[5, 17]] = 0.0
    rc = synth.RunConfig(nth=8, nph=8, nvel=nvel, kmax=2, gvec=synth.gauge_vector(7))
    rc.n_depth = _limits()[0]
    P = oracle.OracleProblem(cloud, mol)
    oJ0, oJ2, ost, _, nf = P.radiation_field(rc, 1, 96)
    assert nf == 0
    live = np.ones(96, dtype=bool)
    live[[5, 17]] = False
    bulk = cloud.bulk_node_num
    for J0, J2, st in _call_static(cloud, mol, rc, calls=2):
        assert (st == 0).all()
        assert (J0[bulk:] == 0).all() and (J2[bulk:] == 0).all()
        assert (J0[[5, 17]] == 0).all() and (J2[[5, 17]] == 0).all()
        assert np.isfinite(J0).all() and np.isfinite(J2).all()
        _check_J(J0[:96], J2[:96], oJ0[:96], oJ2[:96], mask=live)


def test_static_entry_point_reports_walk_overflow(built_lib):
    """n_depth 24: the nodes whose walks need more cells (about one in
    twenty here) get status PORTAL_NODE_DEPTH and J = 0 (inverse_rt.f90:
    206-210 stops the reference there), the same nodes as the oracle's (one
    node may differ: a walk of exactly n_depth cells flips on a single
    near-degenerate crossing); the other nodes' J match the oracle's."""
    import oracle
    import portal_gb300 as pg
    from portal_gb300 import synth
    from test_gpu_parity import _check_J
    mol = synth.linear_rotor(5)
    cloud = synth.power_law_sphere(1024, 8, mol, t_uniform=20.0)
    rc = synth.RunConfig(nth=8, nph=8, nvel=16, kmax=2, gvec=synth.gauge_vector(8), n_depth=24)
    P = oracle.OracleProblem(cloud, mol)
    oJ0, oJ2, ost, _, nf = P.radiation_field(rc)
    over = ost == 1
    assert 0 < over.sum() < cloud.bulk_node_num
    for J0, J2, st in _call_static(cloud, mol, rc, calls=2):
        gover = st == pg.NODE_DEPTH
        assert (gover != over).sum() <= 1 and gover.sum() > 0
        assert ((st == 0) | gover).all()
        assert (J0[gover] == 0).all() and (J2[gover] == 0).all()
        _check_J(J0, J2, oJ0, oJ2, mask=~(over | gover))


def test_static_entry_point_rejects_oversized_walks(built_lib):
    import portal_gb300 as pg
    L = pg.lib()
    max_depth = _limits()[0]
    one = np.ones(8)
    ione = np.ones(8, dtype=np.int32)
    p = one.ctypes.data
    code = L.portal_radiation_field_static(
        None, 4, 4, 2, p, p, p, p, p, p, p, p, 1, ione.ctypes.data, ione.ctypes.data, 1.0,
        ione.ctypes.data_as(pg.P_I), 1, ione.ctypes.data_as(pg.P_I), one.ctypes.data_as(pg.P_D),
        one.ctypes.data_as(pg.P_D), one.ctypes.data_as(pg.P_D), one.ctypes.data_as(pg.P_D), 4, 4, 4,
        one.ctypes.data_as(pg.P_D), 1e-6, max_depth + 1, p, p, None)
    assert code == -2
