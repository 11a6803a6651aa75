"""Setup parity on the CPU: the library's geometry (calcul_geometry,
adjust_bc, PDE_center restated in csrc/setup.cpp) against the oracle's own
restatement, bit for bit, plus mesh invariants the reference asserts."""
import numpy as np
import pytest

import nsmp_gb300 as ng
from oracle import oracle_ctypes as oc
from helpers import oracle_params, small_case

PAIRS = [
    (ng.G_XC, oc.G_XC, "cell"), (ng.G_YC, oc.G_YC, "cell"), (ng.G_AREA, oc.G_AREA, "cell"),
    (ng.G_DLVV, oc.G_DLVV, "n03"), (ng.G_DLCC, oc.G_DLCC, "n03"), (ng.G_DLE1, oc.G_DLE1, "n03"),
    (ng.G_DLE2, oc.G_DLE2, "n03"), (ng.G_DOE, oc.G_DOE, "n03"), (ng.G_XNN, oc.G_XNN, "n03"),
    (ng.G_YNN, oc.G_YNN, "n03"), (ng.G_DXCC, oc.G_DXCC, "n03"), (ng.G_DYCC, oc.G_DYCC, "n03"),
    (ng.G_SUMXC2, oc.G_SUMXC2, "n0"), (ng.G_SUMYC2, oc.G_SUMYC2, "n0"), (ng.G_SUMXCYC, oc.G_SUMXCYC, "n0"),
    (ng.G_SIG, oc.G_SIG, "nz"), (ng.G_DSIG, oc.G_DSIG, "nz"), (ng.G_SIGV, oc.G_SIGV, "nzv"),
    (ng.G_DSIGV, oc.G_DSIGV, "nzv"), (ng.G_DLVSUM, oc.G_DLVSUM, "nv"),
]


def _shape(kind, o):
    return {"cell": (o.ncell,), "n03": (o.n0, 3), "n0": (o.n0,), "nz": (o.nz,), "nzv": (o.nz - 1,),
            "nv": (o.nvert,)}[kind]


@pytest.mark.parametrize("grid_kind", [0, 1])
@pytest.mark.parametrize("nx,ny", [(8, 6), (32, 16)])
def test_geometry_bitwise(nx, ny, grid_kind):
    prm, mesh = small_case(nx, ny, layers=8, grid_kind=grid_kind)
    o = oc.Oracle(oracle_params(prm), mesh)
    for gid, oid, kind in PAIRS:
        shape = _shape(kind, o)
        ref = o.geom(oid, shape).ravel(order="F")
        got = ng.geometry(prm, mesh, gid)
        assert got.shape == ref.shape, (gid, got.shape, ref.shape)
        assert np.array_equal(got, ref), f"geometry array {gid} differs: max {np.abs(got - ref).max()}"
    # neighbour table incl. ghost images (No_cp(ghost,3))
    ref_cp = o.no_cp()
    got_cp = ng.geometry(prm, mesh, ng.G_NOCP).reshape((o.ncell, 3), order="F").astype(np.int32)
    assert np.array_equal(got_cp[:o.n0], ref_cp[:o.n0])
    assert np.array_equal(got_cp[o.n0:, 2], ref_cp[o.n0:, 2])


def test_mesh_invariants():
    prm, mesh = small_case(16, 8, layers=4)
    area = ng.geometry(prm, mesh, ng.G_AREA)
    n0 = prm["n0"]
    assert np.all(area[:n0] > 0)
    assert abs(area[:n0].sum() - prm["xdfin"] * prm["ydfin"]) < 1e-12 * prm["xdfin"] * prm["ydfin"]
    # every boundary edge became a ghost with a periodic image (calcul_geometry.F90:495-564)
    cp = ng.geometry(prm, mesh, ng.G_NOCP).reshape((-1, 3), order="F").astype(int)
    ncell = cp.shape[0]
    assert ncell == n0 + 2 * (16 + 8)
    assert np.all(cp[n0:, 2] >= 1) and np.all(cp[n0:, 2] <= n0)
    assert np.all(cp[:n0] >= 1)
    # column permutation is a permutation
    perm = ng.geometry(prm, mesh, ng.G_PERM).astype(int)
    assert np.array_equal(np.sort(perm), np.arange(n0))


def test_renumbering_is_deterministic():
    prm, mesh = small_case(16, 8, layers=4)
    a = ng.geometry(prm, mesh, ng.G_PERM)
    b = ng.geometry(prm, mesh, ng.G_PERM)
    assert np.array_equal(a, b)


def test_sigma_grid_tanh():
    prm, mesh = small_case(8, 6, layers=16, grid_kind=1, beta=2.0)
    sigv = ng.geometry(prm, mesh, ng.G_SIGV)
    assert sigv[0] == 0.0 and sigv[-1] == 2.0
    d = np.diff(sigv)
    assert np.all(d > 0)
    # clustered toward both walls, symmetric
    assert d[0] < d[len(d) // 2] and abs(d[0] - d[-1]) < 1e-12


def test_oracle_ppe_rows_sum_to_zero():
    """A*1 = 0 and the wall/Neumann checks of get_matrix_coef (bicgstab.F90:239-288)."""
    prm, mesh = small_case(8, 6, layers=6)
    o = oc.Oracle(oracle_params(prm), mesh)
    x = np.ones((o.ncell, o.nz), order="F")
    y = o.apply_A(x)
    assert np.abs(y[:o.n0, 1:-1]).max() < 1e-12 * np.abs(o.geom(oc.G_AMC0, (o.n0, o.nz))).max()
    amct = o.geom(oc.G_AMCT, (o.n0, o.nz))
    amcb = o.geom(oc.G_AMCB, (o.n0, o.nz))
    assert np.all(amct[:, o.nz - 2] == 0.0) and np.all(amcb[:, 1] == 0.0)


def test_oracle_ppe_symmetric_pattern():
    """The 7-point operator is symmetric: <Av, w> = <v, Aw> on interior fields."""
    prm, mesh = small_case(8, 6, layers=6)
    o = oc.Oracle(oracle_params(prm), mesh)
    rng = np.random.default_rng(3)
    v = np.zeros((o.ncell, o.nz), order="F")
    w = np.zeros((o.ncell, o.nz), order="F")
    v[:o.n0, 1:-1] = rng.standard_normal((o.n0, o.nz - 2))
    w[:o.n0, 1:-1] = rng.standard_normal((o.n0, o.nz - 2))
    av = o.apply_A(v)[:o.n0, 1:-1]
    aw = o.apply_A(w)[:o.n0, 1:-1]
    lhs = float(np.sum(av * w[:o.n0, 1:-1]))
    rhs = float(np.sum(v[:o.n0, 1:-1] * aw))
    assert abs(lhs - rhs) <= 1e-10 * max(abs(lhs), 1.0)


def test_oracle_body_force_zero_and_nonzero():
    """The oracle's body-force hook: a zero force changes no bit; a uniform
    push along x raises the mean of u."""
    from oracle import oracle_ctypes as oc
    prm, mesh = small_case(6, 4, layers=4, eps=1e-12)
    runs = []
    for fx in (None, 0.0, 5.0):
        o = oc.Oracle(oracle_params(prm), mesh, nthreads=2)
        u, v, w, p = ng.initial_channel(prm, o.ncell, seed=1)
        o.user_initial(u, v, w, p)
        if fx is not None:
            o.set_body_force(np.full((prm["n0"], prm["nz"]), fx, order="F"))
        o.step(3)
        runs.append(o.get(oc.F_U))
    assert np.array_equal(runs[0], runs[1])
    n0 = prm["n0"]
    assert runs[2][:n0, 1:-1].mean() > runs[0][:n0, 1:-1].mean()
