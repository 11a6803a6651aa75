"""Vertex fields of the output path against the oracle's interpolation3D +
BCvelvertex3D/BCpvertex + bc_periodic (tagdir 2 and 3)."""
import numpy as np
import pytest

import nsmp_gb300 as ng
from oracle import oracle_ctypes as oc
from helpers import oracle_params, rel_l2, small_case

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("top_bc", [0, 1])
def test_vertex_output_against_oracle(top_bc):
    prm, mesh = small_case(8, 6, layers=6, eps=1e-14, max_iters=2000, top_bc=top_bc)
    o = oc.Oracle(oracle_params(prm), mesh)
    s = ng.Solver(prm, mesh)
    u, v, w, p = ng.initial_channel(prm, o.ncell, seed=1)
    o.user_initial(u, v, w, p)
    s.user_initial(u, v, w, p)
    for _ in range(2):
        o.step(3)
        s.step(3, 1)
    cases = [(ng.F_U, oc.F_U, False, 1), (ng.F_V, oc.F_V, False, 2), (ng.F_W, oc.F_W, False, 3),
             (ng.F_P, oc.F_P, True, 0)]
    for fg, fo, is_p, tag in cases:
        for tagdir in (2, 3):
            ref = o.vertex_interp(o.get(fo), is_pressure=is_p, tag_bc=tag, tagdir=tagdir)
            got = s.download_vertex(fg, tagdir)
            assert got.shape == ref.shape
            assert rel_l2(got, ref) <= 1e-11, (fg, tagdir, rel_l2(got, ref))
    s.close()
