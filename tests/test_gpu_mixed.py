"""Mixed precision (NSMP_MIXED): FP32 inner BiCGSTAB inside FP64 iterative
refinement.  The stopping test is the reference's, on the FP64 residual, so
the mixed solution agrees with the FP64 one to the solver tolerance."""
import numpy as np
import pytest

import nsmp_gb300 as ng
from oracle import oracle_ctypes as oc
from helpers import interior, oracle_params, rel_l2, small_case

pytestmark = pytest.mark.gpu


def _start(prm, mesh, seed=1):
    s = ng.Solver(prm, mesh)
    u, v, w, p = ng.initial_channel(prm, s.ncell, seed=seed)
    s.user_initial(u, v, w, p)
    return s, (u, v, w, p)


def test_mixed_one_stage_vs_oracle():
    """Refinement to 1e-13 reproduces the oracle's FP64 stage."""
    prm, mesh = small_case(8, 6, layers=8, eps=1e-13, max_iters=5000, precision=ng.MIXED)
    s, st = _start(prm, mesh)
    o = oc.Oracle(oracle_params(prm), mesh)
    o.user_initial(*st)
    o.step(1)
    rc, inf = s.step(1, 1)
    assert rc == 0 and inf["converged"] == 1
    assert min(inf["e1norm"], inf["e2norm"]) < 1e-13
    for fg, fo in ((ng.F_U, oc.F_U), (ng.F_V, oc.F_V), (ng.F_W, oc.F_W)):
        assert rel_l2(interior(s.download(fg), o.n0), interior(o.get(fo), o.n0)) <= 1e-10
    assert rel_l2(interior(s.download(ng.F_P), o.n0), interior(o.get(oc.F_P), o.n0)) <= 1e-9


def test_incremental_residual_matches_recomputed():
    """The hand-over's incremental residual r - s A (e - mean e), with A c in
    double-float FP32, stays accurate.  A mixed solve is only declared
    converged after an update that recomputes b - A x from scratch in FP64
    for the same x, so the last two updates of a converged solve report the
    incremental and the recomputed residual of one iterate.  Their norms
    agree to 1 % at eps = 1e-10 (measured: to 5 digits; the double-float
    drift bound is of order 1e-12 |b|); A c with FP32 accuracy would be off
    by orders of magnitude."""
    prm, mesh = small_case(32, 16, layers=32, dt=1e-3, eps=1e-10, max_iters=20000, precision=ng.MIXED)
    s, _ = _start(prm, mesh)
    for _ in range(3):  # three Euler/AB2 stages, each with its own solve
        rc, inf = s.step(1, 1)
        assert rc == 0 and inf["converged"] == 1
        log = s.solver_log()
        assert len(log) >= 3, log
        inc, rec = log[-2][2], log[-1][2]
        assert rec > 0.0 and abs(inc - rec) <= 0.01 * rec, (inc, rec)
    s.close()


def test_recurrence_form_matches_direct_products():
    """The p/v pass forms A D^-1 p by the recurrence v' = w - omega M w
    (w = t + beta v) between FP64 hand-overs, and directly on the pass after
    each hand-over.  With a hand-over after every FP32 iteration
    (inner_cap = 1) every product is formed directly; both solves converge
    to eps = 1e-12 on the 32,768-prism mesh and give the same fields to the
    solver tolerance."""
    prm, mesh = small_case(32, 16, layers=32, dt=1e-3, eps=1e-12, max_iters=50000, precision=ng.MIXED)
    rec, _ = _start(prm, mesh)
    direct, _ = _start(prm, mesh)
    direct.set_inner_solver(inner_tol=0.5, inner_cap=1, restart_every=300)
    its = {}
    for name, s in (("recurrence", rec), ("direct", direct)):
        it0, up0 = s.solver_counters()
        rc, inf = s.step(3, 1)
        it1, up1 = s.solver_counters()
        assert rc == 0 and inf["converged"] == 1 and min(inf["e1norm"], inf["e2norm"]) < 1e-12
        its[name] = (it1 - it0, up1 - up0)
    # the direct run hands over after every iteration, the recurrence run rarely
    assert its["direct"][1] >= its["direct"][0] and its["recurrence"][1] < its["recurrence"][0] / 10, its
    n0 = prm["n0"]
    for f in (ng.F_U, ng.F_V, ng.F_W):
        assert rel_l2(interior(rec.download(f), n0), interior(direct.download(f), n0)) <= 1e-9
    assert rel_l2(interior(rec.download(ng.F_P), n0), interior(direct.download(ng.F_P), n0)) <= 1e-7
    rec.close()
    direct.close()


def test_mixed_matches_fp64_after_steps():
    """32,768-prism mesh, 20 RK3 steps at eps = 1e-10: mixed vs FP64 GPU."""
    prm, mesh = small_case(32, 16, layers=32, dt=1e-3)
    s64, _ = _start(prm, mesh)
    s32, _ = _start(dict(prm, precision=ng.MIXED), mesh)
    for _ in range(20):
        rc64, i64 = s64.step(3, 1)
        rc32, i32 = s32.step(3, 1)
        assert rc64 == 0 and rc32 == 0
        assert i32["converged"] == 1 and min(i32["e1norm"], i32["e2norm"]) < 1e-10
    for f in (ng.F_U, ng.F_V, ng.F_W):
        assert rel_l2(interior(s32.download(f), prm["n0"]), interior(s64.download(f), prm["n0"])) <= 1e-6
    d64, d32 = s64.mass_diag(), s32.mass_diag()
    # divergence of the projected face fluxes: same to 1e-10 (relative to the flux scale)
    assert abs(d32[1] - d64[1]) <= 1e-10 * max(1.0, d64[0])


def test_set_precision_switch():
    prm, mesh = small_case(8, 6, layers=6)
    s, _ = _start(prm, mesh)
    s.step(1, 1)
    assert s.L.nsmp_set_precision(s.h, ng.MIXED) == 0
    rc, inf = s.step(1, 1)
    assert rc == 0 and inf["converged"] == 1
    assert s.L.nsmp_set_precision(s.h, 7) == ng.ERR_ARG


def test_fp32_stage_arithmetic_after_steps():
    """NSMP_MIXED_F32: the stage right-hand side (fluxes, gradients,
    Smagorinsky, diffusion) in FP32 on top of the mixed solver.  On the
    32,768-prism mesh over 20 RK3 steps the velocities stay within 1e-6 of
    the FP64 run, the divergence agrees to 1e-10 of the flux scale, and the
    fields do differ from the FP64-stage mixed run (the FP32 kernel ran)."""
    prm, mesh = small_case(32, 16, layers=32, dt=1e-3)
    s64, _ = _start(prm, mesh)
    smx, _ = _start(dict(prm, precision=ng.MIXED), mesh)
    s32, _ = _start(dict(prm, precision=ng.MIXED_F32), mesh)
    for _ in range(20):
        for s in (s64, smx, s32):
            rc, inf = s.step(3, 1)
            assert rc == 0 and inf["converged"] == 1
    n0 = prm["n0"]
    for f in (ng.F_U, ng.F_V, ng.F_W):
        e = rel_l2(interior(s32.download(f), n0), interior(s64.download(f), n0))
        assert e <= 1e-6, (f, e)
    assert not np.array_equal(s32.download(ng.F_U), smx.download(ng.F_U))
    d64, d32 = s64.mass_diag(), s32.mass_diag()
    assert abs(d32[1] - d64[1]) <= 1e-10 * max(1.0, d64[0])
    # switching back and forth at run time
    assert s32.L.nsmp_set_precision(s32.h, ng.MIXED) == 0
    assert s32.step(3, 1)[0] == 0
    assert s32.L.nsmp_set_precision(s32.h, ng.MIXED_F32) == 0
    assert s32.step(3, 1)[0] == 0
