"""ctypes binding of the CPU oracle -- test infrastructure only.

Imported by tests/, by __graft_entry__.smoke() (as the checker) and by the
CPU-baseline leg of bench.py.  Arrays are numpy arrays in the reference's
Fortran layout (column-major, 1-based index values).
"""
import ctypes as C
import os

import numpy as np

from . import build_oracle

F_U, F_V, F_W, F_P, F_U1F, F_U2F, F_U3F, F_UTF, F_UBF, F_RHSU, F_RHSV, F_RHSW, \
    F_EDDY, F_UV, F_VV, F_WV, F_PV = range(17)

(G_XC, G_YC, G_AREA, G_DLVV, G_DLCC, G_DLE1, G_DLE2, G_DOE, G_XNN, G_YNN,
 G_DXCC, G_DYCC, G_SUMXC2, G_SUMYC2, G_SUMXCYC, G_SIG, G_DSIG, G_SIGV, G_DSIGV,
 G_AMC0, G_AMC1, G_AMC2, G_AMC3, G_AMCT, G_AMCB, G_DLVSUM) = range(26)


class OrcParams(C.Structure):
    _fields_ = [
        ("n0", C.c_int), ("nvert", C.c_int), ("nz", C.c_int),
        ("xdini", C.c_double), ("xdfin", C.c_double),
        ("ydini", C.c_double), ("ydfin", C.c_double),
        ("sigini", C.c_double), ("sigfin", C.c_double),
        ("grid_kind", C.c_int), ("grid_beta", C.c_double),
        ("top_bc", C.c_int), ("bot_bc", C.c_int),
        ("dt", C.c_double), ("re", C.c_double),
        ("bdx", C.c_double), ("bdy", C.c_double), ("bdz", C.c_double),
        ("eps", C.c_double), ("max_iters", C.c_int),
        ("les", C.c_int), ("les_van", C.c_int),
        ("ref_bug_compat", C.c_int), ("nthreads", C.c_int),
    ]


class OrcInfo(C.Structure):
    _fields_ = [("iters", C.c_int), ("e1norm", C.c_double), ("e2norm", C.c_double),
                ("converged", C.c_int), ("max_eddy", C.c_double), ("iters_total", C.c_int),
                ("iters_stage", C.c_int * 3)]


# glob_cfl values (the order of nsmp_cfl_diag)
CFL_NAMES = ["umax", "vmax", "wmax", "aveu", "avev", "avew", "cfl_max", "flux_total", "flux_max", "flux_bc",
             "flux_bot", "flux_top", "flux_side", "abs_div"]

PI_REF = 3.14159265359  # common.mpf:26


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        L = C.CDLL(path)
        P = C.POINTER
        L.orc_create.restype = C.c_void_p
        L.orc_create.argtypes = [P(OrcParams), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                 C.c_void_p, C.c_void_p, P(C.c_int)]
        L.orc_destroy.argtypes = [C.c_void_p]
        for name in ("orc_ncell", "orc_get_flag_ab"):
            getattr(L, name).argtypes = [C.c_void_p]
            getattr(L, name).restype = C.c_int
        L.orc_set_flag_ab.argtypes = [C.c_void_p, C.c_int]
        L.orc_set_sum_order.argtypes = [C.c_void_p, C.c_int]
        L.orc_ghost_image.argtypes = [C.c_void_p, C.c_void_p]
        L.orc_no_cp.argtypes = [C.c_void_p, C.c_void_p]
        L.orc_geom.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        L.orc_user_initial.argtypes = [C.c_void_p] + [C.c_void_p] * 4
        L.orc_get.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        L.orc_set.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        L.orc_step.argtypes = [C.c_void_p, C.c_int, P(OrcInfo)]
        L.orc_apply_A.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_set_body_force.argtypes = [C.c_void_p, C.c_void_p]
        L.orc_stats_reset.argtypes = [C.c_void_p]
        L.orc_stats_sample.argtypes = [C.c_void_p]
        L.orc_stats_get.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        L.orc_stats_plane.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_gradient_lsm.argtypes = [C.c_void_p] + [C.c_void_p] * 4
        L.orc_predictor.argtypes = [C.c_void_p] + [C.c_void_p] * 3
        L.orc_vertex_interp.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p]
        L.orc_mass_diag.argtypes = [C.c_void_p, C.c_void_p]
        L.orc_cfl_diag.argtypes = [C.c_void_p, C.c_void_p]
        L.orc_mesh_generate.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                        C.c_double, C.c_ulonglong] + [C.c_void_p] * 6
        L.orc_initial_channel.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_ulonglong] + [C.c_void_p] * 4
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def channel_params(nx, ny, layers, dt, lx=2 * PI_REF, ly=PI_REF, height=2.0, re=180.0, les=1, les_van=1,
                   grid_kind=1, beta=2.0, eps=1e-10, max_iters=10000, top_bc=0, bot_bc=0, ref_bug_compat=1):
    """Oracle parameters of the periodic channel (2pi x pi x 2, tanh layers,
    dp/dx = -1): the same values the product's channel parameters hold."""
    return dict(n0=2 * nx * ny, nvert=(nx + 1) * (ny + 1), nz=layers + 2, xdini=0.0, xdfin=lx, ydini=0.0,
                ydfin=ly, sigini=0.0, sigfin=height, grid_kind=grid_kind, grid_beta=beta, top_bc=top_bc,
                bot_bc=bot_bc, dt=dt, re=re, bdx=1.0, bdy=0.0, bdz=0.0, eps=eps, max_iters=max_iters, les=les,
                les_van=les_van, ref_bug_compat=ref_bug_compat)


def make_mesh(nx, ny, lx=2 * PI_REF, ly=PI_REF, jitter=0.2, seed=0):
    """The oracle's own periodic jittered mesh in data.txt layout."""
    n0, nv = 2 * nx * ny, (nx + 1) * (ny + 1)
    m = {"No_vp": np.zeros((n0, 3), np.int32, order="F"), "No_cp": np.zeros((n0, 3), np.int32, order="F"),
         "nbe": np.zeros(n0, np.int32), "nbev": np.zeros(nv, np.int32),
         "xv": np.zeros(nv, np.float64), "yv": np.zeros(nv, np.float64)}
    rc = lib().orc_mesh_generate(nx, ny, 0.0, lx, 0.0, ly, jitter, seed,
                                 *[_ptr(m[k]) for k in ("No_vp", "No_cp", "nbe", "nbev", "xv", "yv")])
    if rc:
        raise ValueError(f"orc_mesh_generate failed ({rc})")
    return m


class Oracle:
    """One oracle context: geometry from a mesh, then reference time steps."""

    def __init__(self, params: dict, mesh: dict, nthreads: int = 0):
        L = lib()
        p = OrcParams()
        for name, _ in OrcParams._fields_:
            if name == "nthreads":
                continue
            setattr(p, name, params[name])
        p.nthreads = nthreads
        self.params = dict(params)
        self.mesh = {k: np.asfortranarray(v, dtype=(np.int32 if k in ("No_vp", "No_cp", "nbe", "nbev") else np.float64))
                     for k, v in mesh.items()}
        err = C.c_int(0)
        m = self.mesh
        self.h = L.orc_create(C.byref(p), _ptr(m["No_vp"]), _ptr(m["No_cp"]), _ptr(m["nbe"]),
                              _ptr(m["nbev"]), _ptr(m["xv"]), _ptr(m["yv"]), C.byref(err))
        if not self.h:
            raise RuntimeError(f"orc_create failed with {err.value}")
        self.n0, self.nvert, self.nz = params["n0"], params["nvert"], params["nz"]
        self.ncell = L.orc_ncell(self.h)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    def shape(self, field):
        if field in (F_U1F, F_U2F, F_U3F, F_UTF, F_UBF):
            return (self.n0, self.nz)
        if field in (F_UV, F_VV, F_WV, F_PV):
            return (self.nvert, self.nz - 1)
        return (self.ncell, self.nz)

    def get(self, field):
        out = np.zeros(self.shape(field), dtype=np.float64, order="F")
        lib().orc_get(self.h, field, _ptr(out))
        return out

    def set(self, field, arr):
        a = np.asfortranarray(arr, dtype=np.float64)
        assert a.shape == self.shape(field)
        lib().orc_set(self.h, field, _ptr(a))

    def geom(self, which, shape):
        out = np.zeros(shape, dtype=np.float64, order="F")
        lib().orc_geom(self.h, which, _ptr(out))
        return out

    def ghost_image(self):
        img = np.zeros(self.ncell - self.n0, dtype=np.int32)
        lib().orc_ghost_image(self.h, _ptr(img))
        return img

    def no_cp(self):
        out = np.zeros((self.ncell, 3), dtype=np.int32, order="F")
        lib().orc_no_cp(self.h, _ptr(out))
        return out

    def user_initial(self, u, v, w, p):
        arrs = [np.asfortranarray(a, dtype=np.float64) for a in (u, v, w, p)]
        for a in arrs:
            assert a.shape == (self.ncell, self.nz)
        lib().orc_user_initial(self.h, *[_ptr(a) for a in arrs])

    def step(self, fin_rk=1):
        info = OrcInfo()
        rc = lib().orc_step(self.h, fin_rk, C.byref(info))
        return rc, {"iters": info.iters, "e1norm": info.e1norm, "e2norm": info.e2norm,
                    "converged": info.converged, "max_eddy": info.max_eddy, "iters_total": info.iters_total,
                    "iters_stage": list(info.iters_stage)}

    @property
    def flag_ab(self):
        return lib().orc_get_flag_ab(self.h)

    @flag_ab.setter
    def flag_ab(self, f):
        lib().orc_set_flag_ab(self.h, int(f))

    def set_sum_order(self, reverse):
        """Reverse (True) or layer order (False) of the per-layer partial sums."""
        lib().orc_set_sum_order(self.h, 1 if reverse else 0)

    def stats_reset(self):
        lib().orc_stats_reset(self.h)

    def stats_sample(self):
        lib().orc_stats_sample(self.h)

    def stats_get(self, which):
        out = np.zeros((self.ncell, self.nz), order="F")
        assert lib().orc_stats_get(self.h, int(which), _ptr(out)) == 0
        return out

    def stats_plane(self):
        out = np.zeros((self.nz - 2, 10))
        tke = C.c_double()
        assert lib().orc_stats_plane(self.h, _ptr(out), C.byref(tke)) == 0
        return out, tke.value

    def set_body_force(self, fx):
        if fx is None:
            lib().orc_set_body_force(self.h, None)
            return
        self._fx = np.asfortranarray(fx, dtype=np.float64)
        lib().orc_set_body_force(self.h, _ptr(self._fx))

    def apply_A(self, x):
        x = np.asfortranarray(x, dtype=np.float64)
        y = np.zeros_like(x)
        lib().orc_apply_A(self.h, _ptr(x), _ptr(y))
        return y

    def gradient_lsm(self, f):
        f = np.asfortranarray(f, dtype=np.float64)
        outs = [np.zeros_like(f) for _ in range(3)]
        lib().orc_gradient_lsm(self.h, _ptr(f), *[_ptr(o) for o in outs])
        return outs

    def predictor(self):
        """u*, v*, w* of one stage from the level-n state (history untouched)."""
        outs = [np.zeros((self.ncell, self.nz), order="F") for _ in range(3)]
        lib().orc_predictor(self.h, *[_ptr(o) for o in outs])
        return outs

    def vertex_interp(self, f, is_pressure=True, tag_bc=0, tagdir=2):
        f = np.asfortranarray(f, dtype=np.float64)
        out = np.zeros((self.nvert, self.nz - 1), dtype=np.float64, order="F")
        lib().orc_vertex_interp(self.h, _ptr(f), int(is_pressure), int(tag_bc), int(tagdir), _ptr(out))
        return out

    def mass_diag(self):
        out = np.zeros(4, dtype=np.float64)
        lib().orc_mass_diag(self.h, _ptr(out))
        return out

    def cfl_diag(self):
        """glob_cfl on the level-n state: dict of the CFL_NAMES values."""
        out = np.zeros(len(CFL_NAMES), dtype=np.float64)
        lib().orc_cfl_diag(self.h, _ptr(out))
        return dict(zip(CFL_NAMES, out.tolist()))

    def initial_channel(self, umax=18.0, amp=1.8, seed=1):
        """The oracle's own seeded channel state on its (N_CELL,NZ) grid."""
        arrs = [np.zeros((self.ncell, self.nz), np.float64, order="F") for _ in range(4)]
        lib().orc_initial_channel(self.h, umax, amp, seed, *[_ptr(a) for a in arrs])
        return arrs
