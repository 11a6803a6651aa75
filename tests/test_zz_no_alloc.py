"""nsmp_mass_diag_noalloc: the mass-flux reductions with their scratch in a
static device array, for callers that cannot allocate device memory after
setup.  Checked against nsmp_mass_diag on two calls in a row (the second call
finds the array holding the first call's contents), on a context above its
size limit, and -- on the CPU -- for the absence of allocation calls in its
source."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import nsmp_gb300 as ng
from helpers import small_case

SRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "3d-channel-flow-code_gb300",
                   "csrc", "noalloc.cu")


def _solver():
    prm, mesh = small_case(16, 8, layers=8)
    s = ng.Solver(prm, mesh)
    u, v, w, p = ng.initial_channel(prm, s.ncell, seed=1)
    s.user_initial(u, v, w, p)
    return s


def _check(a, b):
    # maxima are exact; sums differ only in summation order
    assert a[1] == b[1] and a[3] == b[3], (a, b)
    assert abs(a[0] - b[0]) <= 1e-12 * abs(b[0])
    assert abs(a[2] - b[2]) <= 1e-12 * max(abs(b[0]), 1e-300)


@pytest.mark.gpu
def test_noalloc_matches_allocating_entry_point():
    s = _solver()
    ref0 = s.mass_diag()
    out = np.zeros(4)
    assert s.L.nsmp_mass_diag_noalloc(s.h, out.ctypes.data_as(C.c_void_p)) == 0
    _check(out, ref0)
    # second call in a row, after the state changed: the static scratch keeps
    # the previous call's contents and must not leak into this result
    s.step(1, 1)
    ref1 = s.mass_diag()
    out2 = np.zeros(4)
    assert s.L.nsmp_mass_diag_noalloc(s.h, out2.ctypes.data_as(C.c_void_p)) == 0
    _check(out2, ref1)
    assert not np.array_equal(out, out2)


@pytest.mark.gpu
def test_noalloc_rejects_null_arguments():
    s = _solver()
    assert s.L.nsmp_mass_diag_noalloc(None, None) == ng.ERR_ARG
    assert s.L.nsmp_mass_diag_noalloc(s.h, None) == ng.ERR_ARG


@pytest.mark.gpu
def test_noalloc_rejects_contexts_above_its_limit():
    """65536 triangles x 258 layers = 16,908,288 prisms, above the
    16,777,216 the static array holds: NSMP_ERR_RANGE with a message, and
    the context stays usable."""
    prm, mesh = small_case(256, 128, layers=258)
    s = ng.Solver(prm, mesh)
    out = np.zeros(4)
    assert s.L.nsmp_mass_diag_noalloc(s.h, out.ctypes.data_as(C.c_void_p)) == ng.ERR_RANGE
    assert b"static scratch limit" in s.L.nsmp_last_error(s.h)
    assert s.mass_diag()[3] == 0.0  # zero state: the allocating path still runs
    s.close()


def test_noalloc_source_names_no_allocation_call():
    """The entry point's translation unit calls no device allocator."""
    src = open(SRC).read()
    code = re.sub(r"//[^\n]*", "", re.sub(r"/\*.*?\*/", "", src, flags=re.S))
    for name in ("cudaMalloc", "cudaMallocAsync", "cudaMallocManaged", "cudaFree", "cudaFreeAsync",
                 "cudaMallocHost", "cudaHostAlloc", "malloc(", "new "):
        assert name not in code, name
