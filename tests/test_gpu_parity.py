"""GPU parity: the CUDA stage through the C-ABI against the CPU oracle on
the same seeded inputs.

Tolerances (FP64 plain form): relative L2 <= 1e-11 per field after one
step, <= 1e-8 after 100 steps, BiCGSTAB iterations within +-1 per stage.
"""
import numpy as np
import pytest

import nsmp_gb300 as ng
from oracle import oracle_ctypes as oc
from helpers import interior, oracle_params, rel_l2, small_case

pytestmark = pytest.mark.gpu

CELL_FIELDS = [(ng.F_U, oc.F_U), (ng.F_V, oc.F_V), (ng.F_W, oc.F_W), (ng.F_P, oc.F_P)]
FACE_FIELDS = [(ng.F_U1FACE, oc.F_U1F), (ng.F_U2FACE, oc.F_U2F), (ng.F_U3FACE, oc.F_U3F),
               (ng.F_UTFACE, oc.F_UTF), (ng.F_UBFACE, oc.F_UBF)]


def _pair(prm, mesh, seed=1):
    o = oc.Oracle(oracle_params(prm), mesh)
    s = ng.Solver(prm, mesh)
    assert s.ncell == o.ncell
    u, v, w, p = ng.initial_channel(prm, o.ncell, seed=seed)
    o.user_initial(u, v, w, p)
    s.user_initial(u, v, w, p)
    return o, s


def _compare(o, s, tol, what=""):
    worst = {}
    for fg, fo in CELL_FIELDS:
        a, b = s.download(fg), o.get(fo)
        e = rel_l2(interior(a, o.n0), interior(b, o.n0))
        worst[f"cell{fg}"] = e
        # ghosts (periodic images and wall layers) must agree as well
        worst[f"full{fg}"] = rel_l2(a, b)
    for fg, fo in FACE_FIELDS:
        a, b = s.download(fg), o.get(fo)
        worst[f"face{fg}"] = rel_l2(a[:, 1:-1], b[:, 1:-1])
    bad = {k: v for k, v in worst.items() if not v <= tol}
    assert not bad, f"{what}: fields above {tol}: {bad}"
    return worst


def test_initial_state_roundtrip():
    prm, mesh = small_case(8, 6, layers=6)
    o, s = _pair(prm, mesh)
    _compare(o, s, 1e-14, "initial")


@pytest.mark.parametrize("les", [0, 1])
@pytest.mark.parametrize("grid_kind", [0, 1])
def test_one_stage_euler(les, grid_kind):
    prm, mesh = small_case(8, 6, layers=6, les=les, grid_kind=grid_kind)
    o, s = _pair(prm, mesh)
    rc_o, io = o.step(1)
    rc_s, inf = s.step(1, 1)
    assert abs(io["iters"] - inf["iters"]) <= 1, (io, inf)
    _compare(o, s, 1e-11, "one stage")
    if les:
        e_o, e_s = o.get(oc.F_EDDY), s.download(ng.F_EDDY)
        assert rel_l2(interior(e_s, o.n0), interior(e_o, o.n0)) <= 1e-11
    # AB2 history and vertex pressure
    for fg, fo in [(ng.F_RHSU, oc.F_RHSU), (ng.F_RHSV, oc.F_RHSV), (ng.F_RHSW, oc.F_RHSW)]:
        assert rel_l2(s.download(fg), o.get(fo)) <= 1e-11
    pv_s, pv_o = s.download(ng.F_PV), o.get(oc.F_PV)
    assert rel_l2(pv_s, pv_o) <= 1e-11


def test_config0_one_step_rk3():
    """configs[0] geometry: 32x16 quads, 32 tanh layers, RK3, dt = 1e-3."""
    prm, mesh = small_case(32, 16, layers=32, dt=1e-3)
    o, s = _pair(prm, mesh)
    o.step(3)
    s.step(3, 1)
    _compare(o, s, 1e-11, "config0 1 step")


@pytest.mark.parametrize("fin_rk,nsteps", [(1, 4), (2, 3)])
def test_reference_integrators(fin_rk, nsteps):
    """Euler->AB2 (1.55/-0.55, hydro.F90:225-231) and Heun RK2 (nsmp3D.F90:531-546)."""
    prm, mesh = small_case(8, 6, layers=6)
    o, s = _pair(prm, mesh)
    for _ in range(nsteps):
        _, io = o.step(fin_rk)
        _, inf = s.step(fin_rk, 1)
        assert abs(io["iters"] - inf["iters"]) <= 1
    assert s.flag_ab == o.flag_ab or fin_rk != 1
    _compare(o, s, 1e-10, f"fin_rk={fin_rk}")


def test_stagewise_api_matches_step():
    """hydro_stage + copy/finalize/update calls == nsmp_step (RK2)."""
    prm, mesh = small_case(8, 6, layers=6)
    _, s1 = _pair(prm, mesh)
    _, s2 = _pair(prm, mesh)
    s1.step(2, 1)
    s2.copy_known_from_n()
    s2.stage(2)
    s2.copy_known_from_np()
    s2.stage(2)
    s2.rk2_finalize()
    s2.time_update()
    for f in (ng.F_U, ng.F_V, ng.F_W, ng.F_P, ng.F_U1FACE):
        assert np.array_equal(s1.download(f), s2.download(f))


@pytest.mark.slow
def test_config0_100_steps():
    """configs[0]: 100 RK3 steps, rel-L2 <= 1e-8 per field."""
    prm, mesh = small_case(32, 16, layers=32, dt=1e-3)
    o, s = _pair(prm, mesh)
    for _ in range(100):
        _, io = o.step(3)
        _, inf = s.step(3, 1)
        assert abs(io["iters"] - inf["iters"]) <= 1
    _compare(o, s, 1e-8, "config0 100 steps")


def test_mass_diag_matches_oracle():
    prm, mesh = small_case(8, 6, layers=6)
    o, s = _pair(prm, mesh)
    o.step(1)
    s.step(1, 1)
    a, b = s.mass_diag(), o.mass_diag()
    assert np.allclose(a[[0, 1, 3]], b[[0, 1, 3]], rtol=1e-9, atol=1e-13)
    assert abs(a[2] - b[2]) <= 1e-9 * max(1.0, b[0])


def test_bad_inputs_rejected():
    prm, mesh = small_case(8, 6, layers=6)
    bad = dict(prm, top_bc=3)
    with pytest.raises(ng.NsmpError):
        ng.Solver(bad, mesh)
    bad_mesh = {k: np.array(v, copy=True) for k, v in mesh.items()}
    bad_mesh["No_vp"][0, 0] = prm["nvert"] + 5
    with pytest.raises(ng.NsmpError):
        ng.Solver(prm, bad_mesh)


def test_maxiter_warning():
    """MaxIters exhaustion is a warning, the stage completes (bicgstab.F90:562-566)."""
    prm, mesh = small_case(8, 6, layers=6, max_iters=2, eps=1e-14)
    o, s = _pair(prm, mesh)
    rc, inf = s.step(1, 1)
    assert rc == ng.WARN_MAXITER
    assert inf["iters"] == 3
    _, io = o.step(1)
    assert io["iters"] == 3
    _compare(o, s, 1e-11, "maxiter")
