"""Behaviour of the C-ABI around the compute: which device an entry point
runs on, and recovery after a failed allocation (GPU)."""
import numpy as np
import pytest

import nsmp_gb300 as ng
from helpers import small_case

pytestmark = pytest.mark.gpu


def _run(prm, mesh):
    s = ng.Solver(prm, mesh)
    s.user_initial(*ng.initial_channel(prm, s.ncell, seed=1))
    rc, _ = s.step(3, 1)
    assert rc >= 0
    u = s.download(ng.F_U)
    s.close()
    return u


def test_entry_points_keep_the_callers_current_device():
    """Every entry point runs on the context's device and gives the caller's
    current device back; with a second GPU the caller's device is another
    ordinal while a context on device 0 steps."""
    import torch
    prm, mesh = small_case(8, 6, layers=6)
    before = torch.cuda.current_device()
    ref = _run(dict(prm, device=0), mesh)
    assert torch.cuda.current_device() == before
    if torch.cuda.device_count() > 1:
        torch.cuda.set_device(1)
        try:
            u = _run(dict(prm, device=0), mesh)
            assert torch.cuda.current_device() == 1
            assert np.array_equal(u, ref)
        finally:
            torch.cuda.set_device(before)


def test_failed_allocation_does_not_poison_the_next_call():
    """An adjoint whose pressure tape cannot be allocated fails with
    NSMP_ERR_CUDA; the error is not reported again by the next call, which
    steps normally."""
    prm, mesh = small_case(8, 6, layers=6)
    s = ng.Solver(prm, mesh)
    s.user_initial(*ng.initial_channel(prm, s.ncell, seed=1))
    fx = np.zeros((s.n0, s.nz), order="F")
    with pytest.raises(ng.NsmpError) as ei:
        s.adjoint(10**8, 10**8, fx)  # ~0.7 TB of tape
    assert ei.value.code == ng.ERR_CUDA
    assert "tape" in str(ei.value)
    rc, info = s.step(3, 1)
    assert rc >= 0 and info["converged"] == 1
    s.close()
