"""The allocation-free Apply (ouranos_rt_apply_noalloc) against the regular Apply.

For callers that cannot allocate device memory while applying the operator
(a framework that owns the device memory pool, a driver that allows
allocations only at set-up): the entry point keeps all of its scratch in one
fixed-size device array inside the library.  Collected last (file name) so a
run that stops at the first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# the FP64 parity tolerance used by the other GPU tests
TOL64 = 1e-12


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("which", ["2d-p3-expanded", "3d-p0-fused", "2d-cell-order"])
def test_apply_noalloc_matches_apply_twice(which):
    torch = pytest.importorskip("torch")
    import ouranos_gb300 as og
    from ouranos_gb300 import _capi
    if which == "2d-p3-expanded":
        prob = og.heterogeneous_2d(seed=51, n=24, fe_order=2, sn=8, l_max=3, blocks=3)
    elif which == "3d-p0-fused":
        prob = og.thick_3d(seed=2051, n=10, sn=4, block=2, width=2.0)
    else:
        prob = og.heterogeneous_2d(seed=52, n=8, fe_order=1, sn=4, l_max=1, blocks=2)
        prob.cell_order = np.random.default_rng(3).permutation(64).astype(np.int64)
    lib = _capi.lib()
    with og.RadiativeTransfer(prob) as rt:
        x = torch.randn(prob.vector_length, dtype=torch.float64, device="cuda",
                        generator=torch.Generator(device="cuda").manual_seed(7))
        y_ref = torch.empty_like(x)
        rt.Apply(x, y_ref)
        torch.cuda.synchronize()
        ref = y_ref.cpu().numpy()
        for call in range(2):
            y = torch.full_like(x, float("nan"))
            torch.cuda.synchronize()
            free_before = torch.cuda.mem_get_info()[0]
            rc = lib.ouranos_rt_apply_noalloc(rt._h, C.c_void_p(x.data_ptr()),
                                              C.c_void_p(y.data_ptr()))
            torch.cuda.synchronize()
            free_after = torch.cuda.mem_get_info()[0]
            assert rc == _capi.OK, _capi.last_error(rt._h)
            assert _rel(y.cpu().numpy(), ref) < TOL64, (which, call)
            if call == 1:
                assert free_after == free_before  # nothing allocated by the call


def test_apply_noalloc_rejects_oversized_and_host_pointers():
    torch = pytest.importorskip("torch")
    import ouranos_gb300 as og
    from ouranos_gb300 import _capi
    lib = _capi.lib()
    big = og.heterogeneous_2d(seed=53, n=128, fe_order=2, sn=16, l_max=3, blocks=4)
    with og.RadiativeTransfer(big) as rt:
        x = torch.zeros(big.vector_length, dtype=torch.float64, device="cuda")
        y = torch.empty_like(x)
        rc = lib.ouranos_rt_apply_noalloc(rt._h, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()))
        assert rc == _capi.ERR_BAD_INPUT
        assert "scratch" in _capi.last_error(rt._h)
    small = og.config_small(n=8, sn=4)
    with og.RadiativeTransfer(small) as rt:
        xh = np.zeros(small.vector_length)
        yh = np.zeros(small.vector_length)
        rc = lib.ouranos_rt_apply_noalloc(rt._h, C.c_void_p(xh.ctypes.data), C.c_void_p(yh.ctypes.data))
        assert rc == _capi.ERR_BAD_INPUT
