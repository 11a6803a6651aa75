"""Shared test helpers: meshes, parameters and comparisons."""
import numpy as np

import nsmp_gb300 as ng


def small_case(nx=8, ny=6, layers=6, dt=1e-3, **kw):
    """A small periodic channel: mesh + parameters (seed 0 mesh)."""
    mesh = ng.make_mesh(nx, ny, seed=kw.pop("mesh_seed", 0))
    prm = ng.channel_params(nx, ny, layers, dt, **kw)
    return prm, mesh


def oracle_params(prm):
    keys = ["n0", "nvert", "nz", "xdini", "xdfin", "ydini", "ydfin", "sigini", "sigfin", "grid_kind",
            "grid_beta", "top_bc", "bot_bc", "dt", "re", "bdx", "bdy", "bdz", "eps", "max_iters", "les",
            "les_van", "ref_bug_compat"]
    return {k: prm[k] for k in keys}


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64).ravel()
    b = np.asarray(b, dtype=np.float64).ravel()
    den = np.linalg.norm(b)
    if den == 0.0:
        return float(np.linalg.norm(a - b))
    return float(np.linalg.norm(a - b) / den)


def interior(f, n0):
    """Interior rows and interior layers of an (N_CELL,NZ) field."""
    return np.asarray(f)[:n0, 1:-1]
