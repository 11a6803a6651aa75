"""Host-side mirror of the nsmp3D hot-path interface over libnsmpgpu.so.

The Fortran driver of the reference calls `hydro` once per stage and copies
time levels around it (src/nsmp3D.F90:394-564).  `Solver` exposes the same
entry points as the C-ABI in include/nsmp.h, with numpy arrays in the
reference's Fortran layout.  Compute runs only in the CUDA library: if the
library or a GPU is missing, construction raises instead of falling back.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

PI_REF = 3.14159265359  # common.mpf:26

# status codes (include/nsmp.h)
OK, WARN_MAXITER, WARN_BREAKDOWN = 0, 1, 2
ERR_ARG, ERR_MESH, ERR_CUDA, ERR_NAN, ERR_UNSUPPORTED, ERR_NOMEM, ERR_RANGE = -1, -2, -3, -4, -5, -6, -7
FP64, MIXED, MIXED_F32 = 0, 1, 2

(F_U, F_V, F_W, F_P, F_U1FACE, F_U2FACE, F_U3FACE, F_UTFACE, F_UBFACE, F_RHSU, F_RHSV,
 F_RHSW, F_EDDY, F_UNP, F_VNP, F_WNP, F_PNP, F_PV) = range(18)

(G_XC, G_YC, G_AREA, G_DLVV, G_DLCC, G_DLE1, G_DLE2, G_DOE, G_XNN, G_YNN, G_DXCC, G_DYCC,
 G_SUMXC2, G_SUMYC2, G_SUMXCYC, G_SIG, G_DSIG, G_SIGV, G_DSIGV, G_DLVSUM, G_NOCP, G_PERM) = range(22)


class Params(C.Structure):
    _fields_ = [
        ("n0", C.c_int), ("nvert", C.c_int), ("nz", C.c_int),
        ("xdini", C.c_double), ("xdfin", C.c_double), ("ydini", C.c_double), ("ydfin", C.c_double),
        ("sigini", C.c_double), ("sigfin", C.c_double),
        ("grid_kind", C.c_int), ("grid_beta", C.c_double),
        ("top_bc", C.c_int), ("bot_bc", C.c_int),
        ("dt", C.c_double), ("re", C.c_double), ("bdx", C.c_double), ("bdy", C.c_double), ("bdz", C.c_double),
        ("eps", C.c_double), ("max_iters", C.c_int),
        ("les", C.c_int), ("les_van", C.c_int), ("ref_bug_compat", C.c_int),
        ("precision", C.c_int), ("device", C.c_int),
    ]


class Mesh(C.Structure):
    _fields_ = [("No_vp", C.c_void_p), ("No_cp", C.c_void_p), ("nbe", C.c_void_p), ("nbev", C.c_void_p),
                ("xv", C.c_void_p), ("yv", C.c_void_p)]


class StageInfo(C.Structure):
    _fields_ = [("iters", C.c_int), ("e1norm", C.c_double), ("e2norm", C.c_double),
                ("converged", C.c_int), ("max_eddy", C.c_double), ("status", C.c_int),
                ("refinements", C.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


EXPORTS = [
    "nsmp_create", "nsmp_destroy", "nsmp_last_error", "nsmp_ncell", "nsmp_user_initial", "nsmp_upload_state",
    "nsmp_download", "nsmp_copy_known_from_n", "nsmp_hydro_stage", "nsmp_copy_known_from_np",
    "nsmp_rk2_finalize", "nsmp_rk_combine", "nsmp_time_update", "nsmp_step", "nsmp_mass_diag",
    "nsmp_set_precision", "nsmp_stream", "nsmp_host_register", "nsmp_host_unregister", "nsmp_mesh_size",
    "nsmp_mesh_generate", "nsmp_initial_channel",
    "nsmp_sigma_grid", "nsmp_geometry", "nsmp_prof_enable", "nsmp_prof_read", "nsmp_counters",
    "nsmp_set_inner_solver", "nsmp_solver_log", "nsmp_mass_diag_noalloc",
    "nsmp_set_body_force", "nsmp_wall_shear", "nsmp_adjoint", "nsmp_apply_A", "nsmp_apply_AT",
    "nsmp_set_adjoint_budget", "nsmp_stats_reset", "nsmp_stats_sample", "nsmp_stats_count",
    "nsmp_stats_download", "nsmp_stats_plane", "nsmp_download_vertex", "nsmp_cfl_diag",
    "nsmp_solver_counters", "nsmp_probe_fp64_fma", "nsmp_set_fp64_spmv", "nsmp_geometry_device",
]

# glob_cfl values of nsmp_cfl_diag (NSMP_CFL_* order)
CFL_NAMES = ["umax", "vmax", "wmax", "aveu", "avev", "avew", "cfl_max", "flux_total", "flux_max", "flux_bc",
             "flux_bot", "flux_top", "flux_side", "abs_div"]

(K_VERTEX4, K_STAGE_RHS, K_FACES_DIV, K_BICG_INIT, K_BICG_P, K_BICG_SPMV_V, K_BICG_S, K_BICG_SPMV_T,
 K_BICG_X, K_PMEAN, K_VERTEX1, K_PROJECT, K_IN_PV, K_IN_ST, K_MIX_UPDATE, K_MIX_SCALE, K_OTHER,
 K_COUNT) = range(18)
(S_U, S_V, S_W, S_P, S_U2, S_V2, S_W2, S_UV, S_VW, S_WU, S_P2, S_EDDY, NSTATS) = range(13)
KERNEL_NAMES = ["k_vertex4", "k_stage_rhs", "k_faces_div", "k_bicg_init", "k_bicg_p", "k_bicg_spmv_v",
                "k_bicg_s", "k_bicg_spmv_t", "k_bicg_x", "k_pmean", "k_vertex1", "k_project", "k_in_pv",
                "k_in_st", "k_mix_update", "k_mix_scale", "other"]

_lib = None


def lib_path():
    return _build.LIB


def lib(build_if_missing=True):
    """Load libnsmpgpu.so (building it in-tree if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"{path} is missing; run build()")
        _build.build()
    L = C.CDLL(path)
    vp = C.c_void_p
    P = C.POINTER
    L.nsmp_create.argtypes = [P(Params), P(Mesh), P(vp)]
    L.nsmp_destroy.argtypes = [vp]
    L.nsmp_last_error.argtypes = [vp]
    L.nsmp_last_error.restype = C.c_char_p
    L.nsmp_ncell.argtypes = [vp, P(C.c_int)]
    L.nsmp_user_initial.argtypes = [vp] + [vp] * 4
    L.nsmp_upload_state.argtypes = [vp] + [vp] * 12 + [C.c_int]
    L.nsmp_download.argtypes = [vp, C.c_int, vp]
    for n in ("nsmp_copy_known_from_n", "nsmp_copy_known_from_np", "nsmp_rk2_finalize", "nsmp_time_update"):
        getattr(L, n).argtypes = [vp]
    L.nsmp_hydro_stage.argtypes = [vp, P(C.c_int), C.c_int, P(StageInfo)]
    L.nsmp_rk_combine.argtypes = [vp, C.c_double, C.c_double]
    L.nsmp_step.argtypes = [vp, C.c_int, C.c_int, P(C.c_int), P(StageInfo)]
    L.nsmp_mass_diag.argtypes = [vp, vp]
    L.nsmp_mass_diag_noalloc.argtypes = [vp, vp]
    L.nsmp_cfl_diag.argtypes = [vp, vp]
    L.nsmp_set_precision.argtypes = [vp, C.c_int]
    L.nsmp_set_inner_solver.argtypes = [vp, C.c_double, C.c_int, C.c_int]
    L.nsmp_set_body_force.argtypes = [vp, vp]
    L.nsmp_wall_shear.argtypes = [vp, P(C.c_double)]
    L.nsmp_adjoint.argtypes = [vp, C.c_int, C.c_int, vp, vp, P(C.c_double)]
    L.nsmp_apply_A.argtypes = [vp, vp, vp]
    L.nsmp_set_adjoint_budget.argtypes = [vp, C.c_double]
    L.nsmp_download_vertex.argtypes = [vp, C.c_int, C.c_int, vp]
    L.nsmp_stats_reset.argtypes = [vp]
    L.nsmp_stats_sample.argtypes = [vp]
    L.nsmp_stats_count.argtypes = [vp, P(C.c_int)]
    L.nsmp_stats_download.argtypes = [vp, C.c_int, vp]
    L.nsmp_stats_plane.argtypes = [vp, vp, P(C.c_double)]
    L.nsmp_apply_AT.argtypes = [vp, vp, vp]
    L.nsmp_stream.argtypes = [vp]
    L.nsmp_stream.restype = vp
    L.nsmp_host_register.argtypes = [vp, vp, C.c_size_t]
    L.nsmp_host_unregister.argtypes = [vp, vp]
    L.nsmp_mesh_size.argtypes = [C.c_int, C.c_int, P(C.c_int), P(C.c_int)]
    L.nsmp_mesh_generate.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                     C.c_double, C.c_ulonglong] + [vp] * 6
    L.nsmp_initial_channel.argtypes = [P(Params), C.c_int, C.c_double, C.c_double, C.c_ulonglong] + [vp] * 4
    L.nsmp_sigma_grid.argtypes = [P(Params)] + [vp] * 4
    L.nsmp_geometry.argtypes = [P(Params), P(Mesh), C.c_int, vp, P(C.c_int)]
    L.nsmp_geometry_device.argtypes = [P(Params), P(Mesh), C.c_int, vp, P(C.c_int)]
    L.nsmp_prof_enable.argtypes = [vp, C.c_int]
    L.nsmp_prof_read.argtypes = [vp, C.c_int, P(C.c_longlong), P(C.c_double)]
    L.nsmp_counters.argtypes = [vp, P(C.c_longlong), P(C.c_longlong)]
    L.nsmp_solver_log.argtypes = [vp, C.c_int, vp, vp, vp, vp]
    L.nsmp_solver_counters.argtypes = [vp, P(C.c_longlong), P(C.c_longlong)]
    L.nsmp_set_fp64_spmv.argtypes = [vp, C.c_int]
    L.nsmp_probe_fp64_fma.argtypes = [C.c_int, C.c_int, P(C.c_double), P(C.c_double)]
    _lib = L
    return L


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def make_mesh(nx, ny, lx=2 * PI_REF, ly=PI_REF, jitter=0.2, seed=0):
    """Periodic jittered triangle mesh in data.txt layout (host only)."""
    L = lib()
    n0, nv = C.c_int(), C.c_int()
    rc = L.nsmp_mesh_size(nx, ny, C.byref(n0), C.byref(nv))
    if rc:
        raise ValueError(f"nsmp_mesh_size failed ({rc})")
    n0, nv = n0.value, nv.value
    m = {"No_vp": np.zeros((n0, 3), np.int32, order="F"), "No_cp": np.zeros((n0, 3), np.int32, order="F"),
         "nbe": np.zeros(n0, np.int32), "nbev": np.zeros(nv, np.int32),
         "xv": np.zeros(nv, np.float64), "yv": np.zeros(nv, np.float64)}
    rc = L.nsmp_mesh_generate(nx, ny, 0.0, lx, 0.0, ly, jitter, seed,
                              *[_p(m[k]) for k in ("No_vp", "No_cp", "nbe", "nbev", "xv", "yv")])
    if rc:
        raise ValueError(f"nsmp_mesh_generate failed ({rc})")
    return m


def channel_params(nx, ny, layers, dt, lx=2 * PI_REF, ly=PI_REF, height=2.0, re=180.0, les=1, les_van=1,
                   grid_kind=1, beta=2.0, eps=1e-10, max_iters=10000, top_bc=0, bot_bc=0, ref_bug_compat=1,
                   precision=FP64, device=0):
    """Parameter dict of the periodic channel (2pi x pi x 2, tanh layers, dp/dx = -1 by default)."""
    return dict(n0=2 * nx * ny, nvert=(nx + 1) * (ny + 1), nz=layers + 2, xdini=0.0, xdfin=lx, ydini=0.0,
                ydfin=ly, sigini=0.0, sigfin=height, grid_kind=grid_kind, grid_beta=beta, top_bc=top_bc,
                bot_bc=bot_bc, dt=dt, re=re, bdx=1.0, bdy=0.0, bdz=0.0, eps=eps, max_iters=max_iters, les=les,
                les_van=les_van, ref_bug_compat=ref_bug_compat, precision=precision, device=device)


def to_struct(params):
    p = Params()
    for name, _ in Params._fields_:
        setattr(p, name, params.get(name, 0))
    return p


def mesh_struct(m):
    keep = {k: np.asfortranarray(v, dtype=(np.int32 if k in ("No_vp", "No_cp", "nbe", "nbev") else np.float64))
            for k, v in m.items()}
    ms = Mesh(*[_p(keep[k]) for k in ("No_vp", "No_cp", "nbe", "nbev", "xv", "yv")])
    return ms, keep


def n_cell_of(mesh):
    return int(mesh["No_cp"].shape[0] + np.count_nonzero(np.asarray(mesh["No_cp"]) == 0))


def geometry(params, mesh, which, device=False):
    """Geometry array as computed by the library's host setup, or (device=True)
    by the setup nsmp_create runs, with its floating-point steps on the GPU."""
    L = lib()
    ms, keep = mesh_struct(mesh)
    ncell = n_cell_of(mesh)
    out = np.zeros(max(3 * ncell, params["nvert"], params["nz"]), dtype=np.float64)
    cnt = C.c_int(0)
    fn = L.nsmp_geometry_device if device else L.nsmp_geometry
    rc = fn(C.byref(to_struct(params)), C.byref(ms), which, _p(out), C.byref(cnt))
    if rc:
        raise RuntimeError(f"nsmp_geometry failed ({rc})")
    return out[:cnt.value].copy()


def initial_channel(params, n_cell, umax=18.0, amp=1.8, seed=1):
    """Seeded Poiseuille + noise state on the (N_CELL,NZ) grid (host only)."""
    L = lib()
    shape = (n_cell, params["nz"])
    arrs = [np.zeros(shape, np.float64, order="F") for _ in range(4)]
    rc = L.nsmp_initial_channel(C.byref(to_struct(params)), n_cell, umax, amp, seed, *[_p(a) for a in arrs])
    if rc:
        raise RuntimeError(f"nsmp_initial_channel failed ({rc})")
    return arrs


def probe_fp64_fma(device=0, iters=20000):
    """Measured FP64 FMA rate of a device in TFLOP/s (nsmp_probe_fp64_fma)."""
    t, ms = C.c_double(), C.c_double()
    rc = lib().nsmp_probe_fp64_fma(device, iters, C.byref(t), C.byref(ms))
    if rc:
        raise RuntimeError(f"nsmp_probe_fp64_fma failed ({rc})")
    return t.value, ms.value


class NsmpError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"nsmp error {code}: {msg}")
        self.code = code


class Solver:
    """One device-resident solver (a nsmp_ctx)."""

    def __init__(self, params, mesh):
        self.L = lib()
        self.params = dict(params)
        self._ms, self._mesh = mesh_struct(mesh)
        h = C.c_void_p()
        rc = self.L.nsmp_create(C.byref(to_struct(params)), C.byref(self._ms), C.byref(h))
        if rc != 0 or not h.value:
            raise NsmpError(rc, "nsmp_create failed")
        self.h = h
        n = C.c_int()
        self._check(self.L.nsmp_ncell(self.h, C.byref(n)))
        self.ncell = n.value
        self.n0, self.nvert, self.nz = params["n0"], params["nvert"], params["nz"]
        self.flag_ab = 0

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.L.nsmp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc < 0:
            raise NsmpError(rc, self.L.nsmp_last_error(self.h).decode(errors="replace"))
        return rc

    def shape(self, field):
        if field in (F_U1FACE, F_U2FACE, F_U3FACE, F_UTFACE, F_UBFACE):
            return (self.n0, self.nz)
        if field == F_PV:
            return (self.nvert, self.nz - 1)
        return (self.ncell, self.nz)

    def user_initial(self, u, v, w, p):
        arrs = [np.asfortranarray(a, dtype=np.float64) for a in (u, v, w, p)]
        self._check(self.L.nsmp_user_initial(self.h, *[_p(a) for a in arrs]))
        self.flag_ab = 0

    def upload_state(self, u, v, w, p, faces, hist, flag_ab):
        arrs = [np.asfortranarray(a, dtype=np.float64) for a in [u, v, w, p] + list(faces) + list(hist)]
        self._check(self.L.nsmp_upload_state(self.h, *[_p(a) for a in arrs], int(flag_ab)))
        self.flag_ab = int(flag_ab)

    def host_register(self, arr):
        """Page-lock a host array (nsmp_host_register) so uploads and
        downloads through it are direct copies."""
        self._check(self.L.nsmp_host_register(self.h, arr.ctypes.data, arr.nbytes))

    def host_unregister(self, arr):
        self._check(self.L.nsmp_host_unregister(self.h, arr.ctypes.data))

    def download(self, field, out=None):
        """Field in the reference's Fortran layout; into `out` (float64,
        Fortran-ordered, of the field's shape, e.g. pinned memory) if given."""
        shape = tuple(self.shape(field))
        if out is None:
            out = np.zeros(shape, dtype=np.float64, order="F")
        elif out.dtype != np.float64 or out.shape != shape or not out.flags.f_contiguous:
            raise ValueError("out must be a Fortran-ordered float64 array of shape %s" % (shape,))
        self._check(self.L.nsmp_download(self.h, field, _p(out)))
        return out

    def stage(self, fin_rk=1):
        fab = C.c_int(self.flag_ab)
        info = StageInfo()
        rc = self._check(self.L.nsmp_hydro_stage(self.h, C.byref(fab), fin_rk, C.byref(info)))
        self.flag_ab = fab.value
        return rc, info.as_dict()

    def copy_known_from_n(self):
        self._check(self.L.nsmp_copy_known_from_n(self.h))

    def copy_known_from_np(self):
        self._check(self.L.nsmp_copy_known_from_np(self.h))

    def rk2_finalize(self):
        self._check(self.L.nsmp_rk2_finalize(self.h))

    def rk_combine(self, a, b):
        self._check(self.L.nsmp_rk_combine(self.h, a, b))

    def time_update(self):
        self._check(self.L.nsmp_time_update(self.h))

    def step(self, fin_rk=1, nsteps=1):
        info = StageInfo()
        fab = C.c_int(self.flag_ab)
        rc = self._check(self.L.nsmp_step(self.h, fin_rk, nsteps, C.byref(fab), C.byref(info)))
        self.flag_ab = fab.value
        return rc, info.as_dict()

    def mass_diag(self):
        """(sum |div|, max |div|, sum div, max CFL) of glob_cfl."""
        out = np.zeros(4, dtype=np.float64)
        self._check(self.L.nsmp_mass_diag(self.h, _p(out)))
        return out

    def cfl_diag(self):
        """glob_cfl (cfl.F90) on the level-n state: dict of the CFL_NAMES values."""
        out = np.zeros(len(CFL_NAMES), dtype=np.float64)
        self._check(self.L.nsmp_cfl_diag(self.h, _p(out)))
        return dict(zip(CFL_NAMES, out.tolist()))

    def download_vertex(self, field, tagdir=3, out=None):
        """Vertex values (N_VERT, NZ-1) of a level-n field (F_U .. F_P); into
        `out` (float64, Fortran-ordered, e.g. pinned memory) if given."""
        shape = (self.nvert, self.nz - 1)
        if out is None:
            out = np.zeros(shape, order="F")
        elif out.dtype != np.float64 or out.shape != shape or not out.flags.f_contiguous:
            raise ValueError("out must be a Fortran-ordered float64 array of shape %s" % (shape,))
        self._check(self.L.nsmp_download_vertex(self.h, int(field), int(tagdir), _p(out)))
        return out

    # ---- turbulence statistics -------------------------------------------
    def stats_reset(self):
        self._check(self.L.nsmp_stats_reset(self.h))

    def stats_sample(self):
        self._check(self.L.nsmp_stats_sample(self.h))

    def stats_count(self):
        n = C.c_int()
        self._check(self.L.nsmp_stats_count(self.h, C.byref(n)))
        return n.value

    def stats_download(self, which):
        out = np.zeros((self.ncell, self.nz), order="F")
        self._check(self.L.nsmp_stats_download(self.h, int(which), _p(out)))
        return out

    def stats_plane(self):
        """((NZ-2) x 10 array: yplus, mean u v w, rms u v w, shear uv vw wu), tke."""
        out = np.zeros((self.nz - 2, 10))
        tke = C.c_double()
        self._check(self.L.nsmp_stats_plane(self.h, _p(out), C.byref(tke)))
        return out, tke.value

    # ---- discrete adjoint ------------------------------------------------
    def _n0nz(self, a):
        a = np.asfortranarray(np.asarray(a, dtype=np.float64))
        if a.shape != (self.n0, self.nz):
            raise ValueError(f"expected shape {(self.n0, self.nz)}, got {a.shape}")
        return a

    def set_body_force(self, fx):
        """Body force on u per cell, (N0, NZ); None removes it."""
        if fx is None:
            self._check(self.L.nsmp_set_body_force(self.h, None))
            return
        fx = self._n0nz(fx)
        self._check(self.L.nsmp_set_body_force(self.h, _p(fx)))

    def wall_shear(self):
        t = C.c_double()
        self._check(self.L.nsmp_wall_shear(self.h, C.byref(t)))
        return t.value

    def adjoint(self, nsteps, ckpt_every, fx):
        """(J, dJ/dfx, status): nsteps RK3 steps with body force fx and the
        discrete adjoint of the time-averaged wall shear stress."""
        fx = self._n0nz(fx)
        grad = np.zeros_like(fx, order="F")
        J = C.c_double()
        rc = self._check(self.L.nsmp_adjoint(self.h, int(nsteps), int(ckpt_every), _p(fx), _p(grad), C.byref(J)))
        return J.value, grad, rc

    def set_adjoint_budget(self, nbytes):
        """Bytes for the stage inputs of an adjoint segment (0: automatic)."""
        self._check(self.L.nsmp_set_adjoint_budget(self.h, float(nbytes)))

    def apply_A(self, x, transpose=False):
        x = self._n0nz(x)
        y = np.zeros_like(x, order="F")
        fn = self.L.nsmp_apply_AT if transpose else self.L.nsmp_apply_A
        self._check(fn(self.h, _p(x), _p(y)))
        return y

    def mass_diag_noalloc(self):
        """nsmp_mass_diag_noalloc: the same reductions with no allocation."""
        out = np.zeros(4, dtype=np.float64)
        self._check(self.L.nsmp_mass_diag_noalloc(self.h, _p(out)))
        return out

    @property
    def stream(self):
        return self.L.nsmp_stream(self.h)

    def set_fp64_spmv(self, matrix_free):
        """FP64 solver couplings: stored (False) or regenerated matrix-free (True)."""
        self._check(self.L.nsmp_set_fp64_spmv(self.h, 1 if matrix_free else 0))

    def set_precision(self, mode):
        self._check(self.L.nsmp_set_precision(self.h, int(mode)))

    def set_inner_solver(self, inner_tol=3e-2, inner_cap=80, restart_every=300):
        self._check(self.L.nsmp_set_inner_solver(self.h, float(inner_tol), int(inner_cap), int(restart_every)))

    def prof_enable(self, on=True):
        self._check(self.L.nsmp_prof_enable(self.h, 1 if on else 0))

    def prof_read(self):
        """{kernel name: (launches, total ms)} accumulated since prof_enable."""
        out = {}
        for k in range(K_COUNT):
            n, ms = C.c_longlong(), C.c_double()
            self._check(self.L.nsmp_prof_read(self.h, k, C.byref(n), C.byref(ms)))
            out[KERNEL_NAMES[k]] = (n.value, ms.value)
        return out

    def solver_log(self):
        """Per refinement cycle of the last mixed solve: (inner its, inner res, outer res, accepted)."""
        n = 48
        it = np.zeros(n, np.int32)
        ri = np.zeros(n)
        ro = np.zeros(n)
        ac = np.zeros(n, np.int32)
        k = self._check(self.L.nsmp_solver_log(self.h, n, _p(it), _p(ri), _p(ro), _p(ac)))
        return list(zip(it[:k].tolist(), ri[:k].tolist(), ro[:k].tolist(), ac[:k].tolist()))

    def solver_counters(self):
        """(BiCGSTAB iterations, FP64 hand-overs of the mixed solver) since creation."""
        a, b = C.c_longlong(), C.c_longlong()
        self._check(self.L.nsmp_solver_counters(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def counters(self):
        """(kernel launches, BiCGSTAB iterations) since creation."""
        a, b = C.c_longlong(), C.c_longlong()
        self._check(self.L.nsmp_counters(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value
