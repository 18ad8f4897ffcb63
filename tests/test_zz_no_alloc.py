"""The allocation-free radiation-field entry point.

portal_radiation_field_static exists for callers that cannot call cudaMalloc
(their device memory belongs to a pool they do not control, or they may not
allocate between simulation steps).  They keep the reference-layout cloud
arrays on the device themselves and hand the library only device pointers;
the library's scratch is a fixed array in its own image.

This test plays such a caller: torch allocates the device arrays (the caller
may allocate; the entry point may not), the new entry point is called twice
in a row through the C ABI, and both results are checked against the
context-based portal_radiation_field within the tolerance of the parity
tests.  It lives in its own file, collected last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_static_scratch_entry_point_matches_context_path(built_lib):
    import torch

    import portal_gb300 as pg
    from portal_gb300 import synth
    from test_gpu_parity import _check_J

    L = pg.lib()
    max_depth = C.c_int()
    scratch = C.c_longlong()
    L.portal_radiation_field_static_limits(C.byref(max_depth), None, None, None, C.byref(scratch))
    assert scratch.value == 64 << 20 and max_depth.value >= 512

    cloud, mol, rc = synth.config_cloud("sphere4k")
    rc.n_depth = max_depth.value
    with pg.Context(0) as ctx:
        ctx.set_molecule(mol)
        ctx.set_cloud(cloud)
        J0_ref, J2_ref, st_ref, _ = ctx.radiation_field(rc)
    assert not st_ref.any()

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
    for call in range(2):
        J0 = torch.full((N, R), float("nan"), dtype=torch.float64, device=dev)
        J2 = torch.full((N, R), float("nan"), dtype=torch.float64, device=dev)
        st = torch.full((N,), -1, dtype=torch.int32, device=dev)
        rc_code = L.portal_radiation_field_static(
            stream, N, cloud.bulk_node_num, cloud.nlev, *[t.data_ptr() for t in d], del_ne.shape[0],
            del_ne.data_ptr(), del_num.data_ptr(), float(cloud.tx),
            mol_h[0].ctypes.data_as(pg.P_I), R, mol_h[1].ctypes.data_as(pg.P_I),
            *[a.ctypes.data_as(pg.P_D) for a in mol_h[2:]], rc.nth, rc.nph, rc.nvel,
            g.ctypes.data_as(pg.P_D), float(rc.dx), rc.n_depth, J0.data_ptr(), J2.data_ptr(), st.data_ptr())
        assert rc_code == 0, (call, rc_code)
        torch.cuda.synchronize()
        assert (st.cpu().numpy() == 0).all(), call
        _check_J(J0.cpu().numpy(), J2.cpu().numpy(), J0_ref, J2_ref)


def test_static_entry_point_rejects_oversized_walks(built_lib):
    import portal_gb300 as pg
    L = pg.lib()
    max_depth = C.c_int()
    L.portal_radiation_field_static_limits(C.byref(max_depth), None, None, None, None)
    one = np.ones(8)
    ione = np.ones(8, dtype=np.int32)
    p = one.ctypes.data
    code = L.portal_radiation_field_static(
        None, 4, 4, 2, p, p, p, p, p, p, p, p, 1, ione.ctypes.data, ione.ctypes.data, 1.0,
        ione.ctypes.data_as(pg.P_I), 1, ione.ctypes.data_as(pg.P_I), one.ctypes.data_as(pg.P_D),
        one.ctypes.data_as(pg.P_D), one.ctypes.data_as(pg.P_D), one.ctypes.data_as(pg.P_D), 4, 4, 4,
        one.ctypes.data_as(pg.P_D), 1e-6, max_depth.value + 1, p, p, None)
    assert code == -2
