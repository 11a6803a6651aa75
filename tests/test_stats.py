"""Turbulence statistics (Stats/stats.F90): the oracle's restatement against
numpy on its own fields (CPU), and the device sums and plane averages
against the oracle (GPU)."""
import numpy as np
import pytest

import nsmp_gb300 as ng
from oracle import oracle_ctypes as oc
from helpers import oracle_params, rel_l2, small_case

FIELDS = [(ng.S_U, 0), (ng.S_V, 1), (ng.S_W, 2), (ng.S_P, 3), (ng.S_U2, 4), (ng.S_V2, 5), (ng.S_W2, 6),
          (ng.S_UV, 7), (ng.S_VW, 8), (ng.S_WU, 9), (ng.S_P2, 10), (ng.S_EDDY, 11)]


def _plane_numpy(sm, ns, n0, nz, re):
    rows = []
    tke = 0.0
    for k in range(2, nz):
        kk = k - 1
        S = [np.sum(sm[f][:n0, kk] / ns) for f in (0, 1, 2, 4, 5, 6, 7, 8, 9)]
        u1, v1, w1, u2, v2, w2, uv, vw, wu = [x / n0 for x in S]
        xr, yr, zr = u2 - u1 * u1, v2 - v1 * v1, w2 - w1 * w1
        tke += 0.5 * (xr + yr + zr)
        rows.append([re * (2 * k - 3) / (2 * nz - 4), u1, v1, w1, np.sqrt(xr), np.sqrt(yr), np.sqrt(zr),
                     u1 * v1 - uv, v1 * w1 - vw, w1 * u1 - wu])
    return np.array(rows), tke / (nz - 2)


def test_oracle_stats_against_numpy():
    prm, mesh = small_case(6, 4, layers=4, eps=1e-12)
    o = oc.Oracle(oracle_params(prm), mesh, nthreads=2)
    u, v, w, p = ng.initial_channel(prm, o.ncell, seed=1)
    o.user_initial(u, v, w, p)
    o.stats_reset()
    acc = None
    for _ in range(3):
        o.step(3)
        o.stats_sample()
        f = [o.get(x) for x in (oc.F_U, oc.F_V, oc.F_W, oc.F_P)]
        terms = [f[0], f[1], f[2], f[3], f[0] ** 2, f[1] ** 2, f[2] ** 2, f[0] * f[1], f[1] * f[2],
                 f[2] * f[0], f[3] ** 2, o.get(oc.F_EDDY)]
        acc = terms if acc is None else [a + t for a, t in zip(acc, terms)]
    n0 = o.n0
    for _, j in FIELDS:
        got = o.stats_get(j)
        assert np.allclose(got[:n0], acc[j][:n0], rtol=1e-13, atol=1e-13)
        assert np.all(got[n0:] == 0)
    ref, tke_ref = _plane_numpy([o.stats_get(j) for j in range(12)], 3, n0, prm["nz"], prm["re"])
    got, tke = o.stats_plane()
    assert np.allclose(got, ref, rtol=1e-12, atol=1e-14)
    assert abs(tke - tke_ref) <= 1e-12 * abs(tke_ref)


@pytest.mark.gpu
def test_device_stats_against_oracle():
    prm, mesh = small_case(8, 6, layers=6, eps=1e-14, max_iters=2000)
    o = oc.Oracle(oracle_params(prm), mesh)
    s = ng.Solver(prm, mesh)
    u, v, w, p = ng.initial_channel(prm, o.ncell, seed=1)
    o.user_initial(u, v, w, p)
    s.user_initial(u, v, w, p)
    o.stats_reset()
    s.stats_reset()
    for _ in range(3):
        o.step(3)
        s.step(3, 1)
        o.stats_sample()
        s.stats_sample()
    assert s.stats_count() == 3
    for g, j in FIELDS:
        a, b = s.stats_download(g), o.stats_get(j)
        assert rel_l2(a, b) <= 1e-11, (g, rel_l2(a, b))
    pg, tg = s.stats_plane()
    po, to = o.stats_plane()
    assert np.allclose(pg, po, rtol=1e-10, atol=1e-13)
    assert abs(tg - to) <= 1e-10 * abs(to)
    s.stats_reset()
    assert s.stats_count() == 0
    s.close()
