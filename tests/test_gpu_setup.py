"""Setup on the GPU: nsmp_create computes the floating-point geometry of
calcul_geometry (cell centres, areas, edges and normals; doe; the LSQ sums
and Kim-Choi factors; the inverse-distance vertex weights) on the device and
keeps the integer topology on the host.  Every array equals the host setup's
bit for bit (which tests/test_setup_geometry.py pins against the oracle)."""
import numpy as np
import pytest

import nsmp_gb300 as ng
from helpers import small_case

pytestmark = pytest.mark.gpu

ALL = [ng.G_XC, ng.G_YC, ng.G_AREA, ng.G_DLVV, ng.G_DLCC, ng.G_DLE1, ng.G_DLE2, ng.G_DOE, ng.G_XNN, ng.G_YNN,
       ng.G_DXCC, ng.G_DYCC, ng.G_SUMXC2, ng.G_SUMYC2, ng.G_SUMXCYC, ng.G_SIG, ng.G_DSIG, ng.G_SIGV, ng.G_DSIGV,
       ng.G_DLVSUM, ng.G_NOCP, ng.G_PERM]


@pytest.mark.parametrize("nx,ny,layers,grid_kind", [(8, 6, 6, 0), (32, 16, 32, 1), (128, 64, 8, 1)])
def test_device_setup_equals_host_setup(nx, ny, layers, grid_kind):
    prm, mesh = small_case(nx, ny, layers=layers, grid_kind=grid_kind)
    for which in ALL:
        h = ng.geometry(prm, mesh, which)
        d = ng.geometry(prm, mesh, which, device=True)
        assert h.shape == d.shape, which
        assert np.array_equal(h.view(np.uint64), d.view(np.uint64)), which


def test_device_setup_on_the_uniform_mesh():
    """A mesh with every quad split the same way and no jitter (many exactly
    symmetric stencils and axis-parallel edges)."""
    from helpers import uniform_mesh
    prm = ng.channel_params(12, 10, 6, 1e-3, lx=2.0, ly=2.0)
    mesh = uniform_mesh(12, 10, 2.0, 2.0)
    for which in ALL:
        assert np.array_equal(ng.geometry(prm, mesh, which).view(np.uint64),
                              ng.geometry(prm, mesh, which, device=True).view(np.uint64)), which
