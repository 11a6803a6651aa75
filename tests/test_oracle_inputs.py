"""The oracle's own copy of the synthetic inputs equals the library's, bit
for bit (CPU only).  The CPU baseline builds its workload from the oracle's
copy so that it never loads the product library."""
import numpy as np
import pytest

import nsmp_gb300 as ng
from oracle import oracle_ctypes as oc


@pytest.mark.parametrize("nx,ny,seed,jitter", [(8, 6, 0, 0.2), (32, 16, 0, 0.2), (17, 9, 5, 0.1), (4, 3, 0, 0.0)])
def test_mesh_generators_agree(nx, ny, seed, jitter):
    a = ng.make_mesh(nx, ny, seed=seed, jitter=jitter)
    b = oc.make_mesh(nx, ny, seed=seed, jitter=jitter)
    for k in ("No_vp", "No_cp", "nbe", "nbev", "xv", "yv"):
        assert a[k].dtype == b[k].dtype, k
        assert np.array_equal(np.ascontiguousarray(a[k]).view(np.uint8), np.ascontiguousarray(b[k]).view(np.uint8)), k


@pytest.mark.parametrize("grid_kind", [0, 1])
def test_initial_states_agree(grid_kind):
    nx, ny, layers = 16, 8, 12
    prm = ng.channel_params(nx, ny, layers, 1e-3, grid_kind=grid_kind)
    oprm = oc.channel_params(nx, ny, layers, 1e-3, grid_kind=grid_kind)
    o = oc.Oracle(oprm, oc.make_mesh(nx, ny))
    mine = ng.initial_channel(prm, o.ncell, seed=1)
    theirs = o.initial_channel(seed=1)
    for a, b in zip(mine, theirs):
        assert np.array_equal(np.ascontiguousarray(a).view(np.uint64), np.ascontiguousarray(b).view(np.uint64))


def test_channel_parameters_agree():
    prm = ng.channel_params(256, 128, 96, 2.5e-4)
    oprm = oc.channel_params(256, 128, 96, 2.5e-4)
    for k, v in oprm.items():
        assert prm[k] == v, k
