"""afx_residual_noalloc: the residual for callers that cannot let the
library allocate device memory (a coupling code that owns all device memory
through its own pool).  It must give the same residual as afx_residual — bit
for bit in FP64, the tolerance of the other FP64 parity tests — on two calls
in a row through the C ABI, with the state and the result in the caller's
own device arrays, and without taking any device memory.

Kept in its own file, collected last, so a stop-at-first-failure run has
already run every other test."""
import ctypes

import numpy as np
import pytest

from tests.cases import channel_case, gpu_solver, omesh_case

pytestmark = pytest.mark.gpu


def _noalloc(afx, g, q_host, check_memory=False):
    import torch

    qd = torch.from_numpy(np.ascontiguousarray(q_host)).to("cuda")
    Rd = torch.full_like(qd, float("nan"))
    torch.cuda.synchronize()  # q_dev must be complete before the call
    free0 = torch.cuda.mem_get_info()[0]
    rc = afx.lib().afx_residual_noalloc(g.h, ctypes.c_void_p(qd.data_ptr()), ctypes.c_void_p(Rd.data_ptr()),
                                        qd.numel())
    free1 = torch.cuda.mem_get_info()[0]
    if rc != 0:
        raise afx.AfxError(rc, afx.lib().afx_last_error().decode())
    if check_memory:
        assert free1 == free0, "the call took %d bytes of device memory" % (free0 - free1)
    return Rd.cpu().numpy()


@pytest.mark.parametrize("case", ["omesh", "channel"])
def test_residual_noalloc_matches_afx_residual(afx, case):
    if case == "omesh":
        m, bcs = omesh_case(48, 24)
        g = gpu_solver(afx, m, bcs, kernel_variant="tile")
        g.init()
        g.iterate(12)
    else:
        m, bcs, q = channel_case(128, 64)
        g = gpu_solver(afx, m, bcs, kernel_variant="gather")
        g.init()
        g.set_q(q)
    q1 = g.get_q()
    r1 = _noalloc(afx, g, q1)
    np.testing.assert_array_equal(g.get_q(), q1)  # the solver's own state is untouched
    np.testing.assert_array_equal(r1, g.residual())
    # second call, another state: the fixed scratch keeps the first call's contents
    g.iterate(3)
    q2 = g.get_q()
    r2 = _noalloc(afx, g, q2, check_memory=True)
    np.testing.assert_array_equal(r2, g.residual())
    assert not np.array_equal(r1, r2)


def test_residual_noalloc_keeps_the_pending_stage_residual(afx):
    """iterate -> noalloc -> run_solver gives the same run as iterate ->
    run_solver: the last iteration's stage residual (which run_solver's
    normaliser reads) is formed before the call overwrites the gradients."""
    m, bcs = omesh_case(48, 24)
    runs = []
    for with_call in (False, True):
        g = gpu_solver(afx, m, bcs, kernel_variant="tile")
        g.init()
        g.iterate(7)
        if with_call:
            _noalloc(afx, g, g.get_q() * 1.01)
        g.run_solver(1e-30, 40)
        runs.append((g.get_q(), np.asarray(g.history())))
    np.testing.assert_array_equal(runs[1][0], runs[0][0])
    np.testing.assert_array_equal(runs[1][1], runs[0][1])


def test_residual_noalloc_rejects_bad_calls(afx):
    m, bcs = omesh_case(16, 8)
    g = gpu_solver(afx, m, bcs)
    g.init()
    q = g.get_q()
    with pytest.raises(afx.AfxError) as e:  # host pointers are refused
        qh = np.ascontiguousarray(q)
        R = np.empty_like(qh)
        rc = afx.lib().afx_residual_noalloc(g.h, qh.ctypes.data_as(ctypes.c_void_p),
                                            R.ctypes.data_as(ctypes.c_void_p), qh.size)
        if rc != 0:
            raise afx.AfxError(rc, afx.lib().afx_last_error().decode())
    assert e.value.code == 8
    g32 = gpu_solver(afx, m, bcs, precision="fp32-mixed")
    with pytest.raises(afx.AfxError) as e:
        _noalloc(afx, g32, q)
    assert e.value.code == 2
