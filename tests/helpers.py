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


def uniform_mesh(nx, ny, lx, ly):
    """Unjittered periodic mesh in data.txt layout with every quad split along
    the same diagonal: the triangulation is point-symmetric about each vertex,
    so the inverse-distance vertex values (interpolation2D.F90:120-135) are
    exact for linear fields and the Kim-Choi face values are consistent."""
    nv, n0 = (nx + 1) * (ny + 1), 2 * nx * ny
    ix, iy = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1))
    ix, iy = ix.ravel(), iy.ravel()
    xv = np.where(ix == nx, lx, ix * lx / nx)
    yv = np.where(iy == ny, ly, iy * ly / ny)
    nbev = ((ix == 0) | (ix == nx) | (iy == 0) | (iy == ny)).astype(np.int32)
    vp = np.zeros((n0, 3), np.int32, order="F")
    for qy in range(ny):
        for qx in range(nx):
            q = qx + qy * nx
            a = 1 + qx + qy * (nx + 1)
            b, c, d = a + 1, a + nx + 2, a + nx + 1
            vp[2 * q] = (a, b, c)
            vp[2 * q + 1] = (a, c, d)
    owner = {(vp[t, j], vp[t, (j + 1) % 3]): t + 1 for t in range(n0) for j in range(3)}
    cp = np.zeros((n0, 3), np.int32, order="F")
    for t in range(n0):
        for j in range(3):
            cp[t, j] = owner.get((vp[t, (j + 1) % 3], vp[t, j]), 0)
    nbe = (cp == 0).any(axis=1).astype(np.int32)
    return {"No_vp": vp, "No_cp": cp, "nbe": nbe, "nbev": nbev, "xv": xv.astype(np.float64),
            "yv": yv.astype(np.float64)}
