"""The allocation-free Apply (ouranos_rt_apply_noalloc) against the regular Apply.

For callers that cannot allocate device memory while applying the operator
(a framework that owns the device memory pool, a driver that allows
allocations only at set-up): the entry point keeps all of its scratch in one
fixed-size device array inside the library, placed on the device when the
handle is created.  Collected last (file name) so a run that stops at the
first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# the tolerances the other GPU tests use: FP64 parity, FP32 sweep
TOL = {"fp64": 1e-12, "fp32": 2e-6}


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _problem(og, which):
    if which == "2d-p3-expanded":
        return og.heterogeneous_2d(seed=51, n=24, fe_order=2, sn=8, l_max=3, blocks=3)
    if which == "3d-p0-fused":
        return og.thick_3d(seed=2051, n=10, sn=4, block=2, width=2.0)
    prob = og.heterogeneous_2d(seed=52, n=8, fe_order=1, sn=4, l_max=1, blocks=2)
    prob.cell_order = np.random.default_rng(3).permutation(64).astype(np.int64)
    return prob


def _noalloc(lib, rt, x, y):
    return lib.ouranos_rt_apply_noalloc(rt._h, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()))


@pytest.mark.parametrize("arith", ["fp64", "fp64-native", "fp64-df64", "fp64-tc", "fp32"])
@pytest.mark.parametrize("which", ["2d-p3-expanded", "3d-p0-fused", "2d-cell-order"])
def test_apply_noalloc_matches_apply_twice(which, arith):
    """Two calls in a row give the regular Apply's result for the handle's
    arithmetic (the same kernels: bit for bit), and neither changes the free
    device memory."""
    torch = pytest.importorskip("torch")
    import ouranos_gb300 as og
    from ouranos_gb300 import _capi
    prob = _problem(og, which)
    lib = _capi.lib()
    prec = "fp32" if arith == "fp32" else "fp64"
    with og.RadiativeTransfer(prob, precision=prec) as rt:
        if arith == "fp64-native":
            rt.set_fp64_contractions("native")
        elif arith == "fp64-df64":
            rt.set_fp64_contractions("df64")
        elif arith == "fp64-tc":
            rt.set_fp64_contractions("df64_sweep_tc")
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
            rc = _noalloc(lib, rt, x, y)
            torch.cuda.synchronize()
            free_after = torch.cuda.mem_get_info()[0]
            assert rc == _capi.OK, _capi.last_error(rt._h)
            got = y.cpu().numpy()
            assert _rel(got, ref) < TOL[prec], (which, arith, call)
            assert np.array_equal(got, ref), (which, arith, call)
            assert free_after == free_before, (which, arith, call)  # nothing allocated by the call


def test_apply_noalloc_first_call_on_a_fresh_handle():
    """The scratch array is placed on the device when the handle is created:
    the first call of a handle that has made no other call leaves the free
    device memory unchanged and matches the regular Apply.  (A regular Apply
    on another handle runs first, so that CUDA's lazy loading has already
    loaded the kernels both entry points launch.)"""
    torch = pytest.importorskip("torch")
    import ouranos_gb300 as og
    from ouranos_gb300 import _capi
    lib = _capi.lib()
    prob = _problem(og, "2d-p3-expanded")
    x = torch.randn(prob.vector_length, dtype=torch.float64, device="cuda",
                    generator=torch.Generator(device="cuda").manual_seed(9))
    with og.RadiativeTransfer(prob) as warm:
        y_ref = torch.empty_like(x)
        warm.Apply(x, y_ref)
        torch.cuda.synchronize()
    with og.RadiativeTransfer(prob) as rt:
        y = torch.full_like(x, float("nan"))
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        rc = _noalloc(lib, rt, x, y)
        torch.cuda.synchronize()
        free_after = torch.cuda.mem_get_info()[0]
        assert rc == _capi.OK, _capi.last_error(rt._h)
        assert free_after == free_before
        assert _rel(y.cpu().numpy(), y_ref.cpu().numpy()) < TOL["fp64"]


def test_apply_noalloc_wait_timeout_and_recovery():
    """A dependency wait that cannot be satisfied (target biased past the
    end) runs out after the wait limit: the call returns OURANOS_ERR_TIMEOUT
    with the context usable, and the next call is correct."""
    torch = pytest.importorskip("torch")
    import ouranos_gb300 as og
    from ouranos_gb300 import _capi
    lib = _capi.lib()
    prob = og.config_small(n=40, sn=4)  # several tiles -> inter-tile waits
    with og.RadiativeTransfer(prob) as rt:
        rt.set_tiling(8, 1, 4)
        x = torch.randn(prob.vector_length, dtype=torch.float64, device="cuda",
                        generator=torch.Generator(device="cuda").manual_seed(11))
        y_ref = torch.empty_like(x)
        rt.Apply(x, y_ref)
        y = torch.empty_like(x)
        rt.set_wait_limit(2e7)  # 20 ms
        rt.debug_wait_bias(1 << 20)
        assert _noalloc(lib, rt, x, y) == _capi.ERR_TIMEOUT
        assert "timed out" in _capi.last_error(rt._h)
        rt.debug_wait_bias(0)
        rt.set_wait_limit(2e9)
        assert _noalloc(lib, rt, x, y) == _capi.OK
        torch.cuda.synchronize()
        assert _rel(y.cpu().numpy(), y_ref.cpu().numpy()) < TOL["fp64"]


def test_apply_noalloc_rejects_oversized_and_host_pointers():
    torch = pytest.importorskip("torch")
    import ouranos_gb300 as og
    from ouranos_gb300 import _capi
    lib = _capi.lib()
    big = og.heterogeneous_2d(seed=53, n=128, fe_order=2, sn=16, l_max=3, blocks=4)
    with og.RadiativeTransfer(big) as rt:
        x = torch.zeros(big.vector_length, dtype=torch.float64, device="cuda")
        y = torch.empty_like(x)
        assert _noalloc(lib, rt, x, y) == _capi.ERR_BAD_INPUT
        assert "scratch" in _capi.last_error(rt._h)
    small = og.config_small(n=8, sn=4)
    with og.RadiativeTransfer(small) as rt:
        xh = np.zeros(small.vector_length)
        yh = np.zeros(small.vector_length)
        rc = lib.ouranos_rt_apply_noalloc(rt._h, C.c_void_p(xh.ctypes.data), C.c_void_p(yh.ctypes.data))
        assert rc == _capi.ERR_BAD_INPUT
