"""Discrete adjoint of the SSP-RK3 step: the dot-product test of the PPE
operator and its transpose, the body-force hook of the forward stage, and
the gradient of the time-averaged wall shear stress against central finite
differences of the forward run."""
import numpy as np
import pytest

import nsmp_gb300 as ng
from helpers import oracle_params, small_case

pytestmark = pytest.mark.gpu


def _solver(nx=8, ny=6, layers=8, dt=1e-3, eps=1e-13, **kw):
    prm, mesh = small_case(nx, ny, layers, dt, eps=eps, **kw)
    s = ng.Solver(prm, mesh)
    u0, v0, w0, p0 = ng.initial_channel(prm, s.ncell, seed=1)
    s.user_initial(u0, v0, w0, p0)
    return prm, mesh, s


def _state(s):
    cells = [s.download(f) for f in (ng.F_U, ng.F_V, ng.F_W, ng.F_P)]
    faces = [s.download(f) for f in (ng.F_U1FACE, ng.F_U2FACE, ng.F_U3FACE, ng.F_UTFACE, ng.F_UBFACE)]
    hist = [s.download(f) for f in (ng.F_RHSU, ng.F_RHSV, ng.F_RHSW)]
    return cells, faces, hist


def _objective(s, state, fx, nsteps):
    """J = mean over steps 1..nsteps of the wall shear, from `state`."""
    cells, faces, hist = state
    s.upload_state(*cells, faces, hist, 0)
    s.set_body_force(fx)
    J = 0.0
    for _ in range(nsteps):
        rc, _ = s.step(3, 1)
        assert rc == 0
        J += s.wall_shear()
    return J / nsteps


def _interior_random(rng, n0, nz, scale=1.0):
    a = np.zeros((n0, nz), order="F")
    a[:, 1:-1] = scale * rng.standard_normal((n0, nz - 2))
    return a


def test_apply_A_dot_product_and_oracle():
    prm, mesh, s = _solver()
    n0, nz = prm["n0"], prm["nz"]
    rng = np.random.default_rng(5)
    v = _interior_random(rng, n0, nz)
    w = _interior_random(rng, n0, nz)
    Av = s.apply_A(v)
    ATw = s.apply_A(w, transpose=True)
    lhs, rhs = float(np.sum(Av * w)), float(np.sum(v * ATw))
    assert abs(lhs - rhs) <= 1e-13 * (np.abs(Av * w).sum())
    # A is symmetric: the transposed gather equals the row form
    Aw = s.apply_A(w)
    assert np.linalg.norm(ATw - Aw) <= 1e-13 * np.linalg.norm(Aw)
    # the row form against the oracle's operator
    from oracle import oracle_ctypes as oc
    o = oc.Oracle(oracle_params(prm), mesh, nthreads=2)
    ncell = s.ncell
    vw = np.zeros((ncell, nz), order="F")
    vw[:n0] = v
    Ao = o.apply_A(vw)[:n0]
    assert np.linalg.norm(Ao[:, 1:-1] - Av[:, 1:-1]) <= 1e-13 * np.linalg.norm(Ao[:, 1:-1])
    s.close()


def test_zero_body_force_changes_nothing():
    prm, mesh, a = _solver(eps=1e-10)
    _, _, b = _solver(eps=1e-10)
    b.set_body_force(np.zeros((prm["n0"], prm["nz"]), order="F"))
    a.step(3, 2)
    b.step(3, 2)
    for f in (ng.F_U, ng.F_V, ng.F_W, ng.F_P):
        assert np.array_equal(a.download(f), b.download(f))
    a.close()
    b.close()


def test_body_force_drives_u():
    prm, mesh, s = _solver(eps=1e-12)
    n0, nz = prm["n0"], prm["nz"]
    st = _state(s)
    J0 = _objective(s, st, np.zeros((n0, nz), order="F"), 2)
    J1 = _objective(s, st, np.full((n0, nz), 5.0, order="F"), 2)
    assert J1 > J0   # a uniform push along x raises the wall shear
    s.close()


@pytest.mark.parametrize("les", [1, 0])
def test_adjoint_gradient_against_finite_differences(les):
    prm, mesh, s = _solver(les=les)
    n0, nz = prm["n0"], prm["nz"]
    nsteps = 3
    rng = np.random.default_rng(2)
    fx = _interior_random(rng, n0, nz, 0.01)
    st = _state(s)
    s.upload_state(*st[0], st[1], st[2], 0)
    J, grad, rc = s.adjoint(nsteps, 2, fx)
    assert rc == 0
    assert np.all(grad[:, 0] == 0) and np.all(grad[:, -1] == 0)
    # the J of the adjoint run is the forward objective
    J_fwd = _objective(s, st, fx, nsteps)
    assert abs(J - J_fwd) <= 1e-14 * abs(J_fwd)
    rel = []
    for k in range(4):
        d = _interior_random(np.random.default_rng(100 + k), n0, nz)
        h = 1e-4
        Jp = _objective(s, st, fx + h * d, nsteps)
        Jm = _objective(s, st, fx - h * d, nsteps)
        fd = (Jp - Jm) / (2 * h)
        ad = float(np.sum(grad * d))
        rel.append(abs(fd - ad) / max(abs(fd), 1e-300))
    assert max(rel) <= 1e-5, rel
    s.close()


def test_adjoint_checkpoint_spacing_does_not_change_the_gradient():
    prm, mesh, s = _solver()
    n0, nz = prm["n0"], prm["nz"]
    fx = _interior_random(np.random.default_rng(2), n0, nz, 0.01)
    st = _state(s)
    out = []
    for k in (1, 2, 4):
        s.upload_state(*st[0], st[1], st[2], 0)
        J, g, rc = s.adjoint(4, k, fx)
        assert rc == 0
        out.append((J, g))
    # the recomputed segments replay the taped pressures (bitwise the forward
    # run) and every adjoint sum is taken in a fixed order: equal bits
    for J, g in out[1:]:
        assert J == out[0][0]
        assert np.array_equal(g, out[0][1])
    s.close()


def test_adjoint_is_bitwise_deterministic():
    """Two adjoint runs from the same state give the same gradient bits (no
    atomics: contributions are gathered in a fixed order)."""
    prm, mesh, s = _solver()
    n0, nz = prm["n0"], prm["nz"]
    fx = _interior_random(np.random.default_rng(2), n0, nz, 0.01)
    st = _state(s)
    out = []
    for _ in range(2):
        s.upload_state(*st[0], st[1], st[2], 0)
        J, g, rc = s.adjoint(3, 2, fx)
        assert rc == 0
        out.append((J, g))
    assert out[0][0] == out[1][0]
    assert np.array_equal(out[0][1], out[1][1])
    s.close()


def test_adjoint_inner_checkpoints_match_the_segment_store():
    """A budget too small for the stage inputs of a whole segment switches
    nsmp_adjoint to inner checkpoints; J and the gradient are bitwise the
    same."""
    prm, mesh, s = _solver()
    n0, nz = prm["n0"], prm["nz"]
    fx = _interior_random(np.random.default_rng(2), n0, nz, 0.01)
    st = _state(s)
    out = []
    for budget in (0, 1):
        s.set_adjoint_budget(budget)
        s.upload_state(*st[0], st[1], st[2], 0)
        J, g, rc = s.adjoint(5, 5, fx)
        assert rc == 0
        out.append((J, g))
    assert out[1][0] == out[0][0]
    assert np.array_equal(out[1][1], out[0][1])
    s.close()


def test_adjoint_in_mixed_precision_agrees_with_fp64():
    prm, mesh, s = _solver()
    n0, nz = prm["n0"], prm["nz"]
    fx = _interior_random(np.random.default_rng(2), n0, nz, 0.01)
    st = _state(s)
    J64, g64, rc = s.adjoint(3, 2, fx)
    assert rc == 0
    s.set_precision(ng.MIXED)
    s.upload_state(*st[0], st[1], st[2], 0)
    J32, g32, rc = s.adjoint(3, 2, fx)
    assert rc == 0
    assert abs(J32 - J64) <= 1e-9 * abs(J64)
    assert np.linalg.norm(g32 - g64) <= 1e-6 * np.linalg.norm(g64)
    s.close()


def test_autograd_function_matches_the_adjoint():
    """J.backward() through the torch.autograd.Function fills fx.grad with
    the adjoint gradient, and the Function's J matches a finite difference."""
    import torch
    from nsmp_gb300.autograd import capture_state, wall_shear_objective
    prm, mesh, s = _solver()
    n0, nz = prm["n0"], prm["nz"]
    st = capture_state(s)
    f0 = _interior_random(np.random.default_rng(2), n0, nz, 0.01)
    fx = torch.tensor(f0, dtype=torch.float64, requires_grad=True)
    J = wall_shear_objective(s, fx, st, 3, 2)
    J.backward()
    s.upload_state(*st[0], st[1], st[2], 0)
    _, g_ref, rc = s.adjoint(3, 2, f0)
    assert rc == 0
    assert np.linalg.norm(fx.grad.numpy() - g_ref) <= 1e-6 * np.linalg.norm(g_ref)
    d = _interior_random(np.random.default_rng(7), n0, nz)
    h = 1e-4
    with torch.no_grad():
        Jp = wall_shear_objective(s, torch.tensor(f0 + h * d), st, 3, 2).item()
        Jm = wall_shear_objective(s, torch.tensor(f0 - h * d), st, 3, 2).item()
    fd = (Jp - Jm) / (2 * h)
    assert abs(fd - float(np.sum(fx.grad.numpy() * d))) <= 1e-5 * abs(fd)
    s.close()


@pytest.mark.slow
def test_adjoint_config3_against_finite_differences():
    """The 1,048,576-prism mesh (128x64 quads, 64 tanh layers, dt 5e-4,
    force 0.01 N(0,1), seed 2): the adjoint gradient over 10 RK3 steps with
    a checkpoint every 5 against central differences along 8 seeded
    directions (PPE solves to 1e-13).  The step is 1e-3: J is about 0.2 and
    its directional derivatives 1e-6 to 2e-5, so with a step of 1e-6 the
    difference J+ - J- is only ~1e5 units of J's last place, and FP64
    rounding of the forward run limits the agreement to 2e-6..1.5e-4
    (measured); steps 1e-3 and 1e-4 give 2e-8..2e-6."""
    prm, mesh, s = _solver(128, 64, 64, 5e-4, eps=1e-13, max_iters=5000)
    n0, nz = prm["n0"], prm["nz"]
    fx = _interior_random(np.random.default_rng(2), n0, nz, 0.01)
    st = _state(s)
    nsteps, h = 10, 1e-3
    s.upload_state(*st[0], st[1], st[2], 0)
    J, grad, rc = s.adjoint(nsteps, 5, fx)
    assert rc == 0
    rel = []
    for k in range(8):
        d = _interior_random(np.random.default_rng(1000 + k), n0, nz)
        Jp = _objective(s, st, fx + h * d, nsteps)
        Jm = _objective(s, st, fx - h * d, nsteps)
        fd = (Jp - Jm) / (2 * h)
        ad = float(np.sum(grad * d))
        rel.append(abs(fd - ad) / max(abs(fd), 1e-300))
    print("config3 FD relative errors", rel)
    assert max(rel) <= 1e-5, rel
    s.close()
