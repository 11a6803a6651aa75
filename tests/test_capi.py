"""The C-ABI library loads without a GPU and exports every entry point the
public header declares; host-only entry points work on the CPU."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import nsmp_gb300 as ng

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    names = []
    for h in sorted(os.listdir(os.path.join(REPO, "include"))):
        if not h.endswith(".h"):
            continue
        src = open(os.path.join(REPO, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_\s\*]*?\b(nsmp_[A-Za-z0-9_]+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_library_exports_header():
    L = ng.lib()
    names = header_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert set(ng.EXPORTS) <= set(names)


def ctx_functions():
    """Header functions whose first parameter is the context, with the C
    types of their parameters."""
    src = open(os.path.join(REPO, "include", "nsmp.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    out = []
    for ret, name, params in re.findall(r"^\s*((?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\*?)\s*(nsmp_[A-Za-z0-9_]+)\s*\(([^)]*)\)\s*;",
                                        src, flags=re.M):
        ps = [p.strip() for p in params.replace("\n", " ").split(",")]
        if ps and ps[0].startswith("nsmp_ctx"):
            out.append((ret.strip(), name, ps))
    return out


def test_null_context_is_rejected_without_a_gpu():
    """Every entry point that takes a context returns NSMP_ERR_ARG for a null
    one (before touching CUDA, so this runs on a CPU); the pointer and string
    queries return null and a message."""
    L = ng.lib()
    fns = ctx_functions()
    assert len(fns) >= 30
    for ret, name, ps in fns:
        f = getattr(L, name)
        typed = f.argtypes is not None  # else wrap values in their ctypes types
        args = []
        for p in ps[1:]:
            if "*" in p or "[" in p:
                args.append(None)
            elif p.startswith("double"):
                args.append(0.5 if typed else C.c_double(0.5))
            elif p.startswith("size_t"):
                args.append(1 if typed else C.c_size_t(1))
            else:
                args.append(1 if typed else C.c_int(1))
        rv = f(None, *args)
        if name == "nsmp_stream":
            assert rv is None
        elif name == "nsmp_last_error":
            assert rv == b"null context"
        else:
            assert rv == -1, (name, rv)  # NSMP_ERR_ARG


def header_enum(first):
    """Names of the C enum whose first member is `first`, in order."""
    src = open(os.path.join(REPO, "include", "nsmp.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    body = re.search(r"enum\s*\{([^}]*\b" + first + r"\b[^}]*)\}", src).group(1)
    return [t.split("=")[0].strip() for t in body.split(",") if t.strip()]


def test_kernel_ids_match_header():
    names = header_enum("NSMP_K_VERTEX4")
    assert names[-1] == "NSMP_K_COUNT"
    assert ng.K_COUNT == len(names) - 1 == len(ng.KERNEL_NAMES)
    for i, n in enumerate(names[:-1]):
        assert getattr(ng, n[len("NSMP_"):]) == i
        want = n[len("NSMP_K_"):].lower()
        assert ng.KERNEL_NAMES[i].replace("k_", "", 1) == want or ng.KERNEL_NAMES[i] == want


def test_field_ids_match_header():
    names = header_enum("NSMP_F_U")
    assert names[-1] == "NSMP_NFIELDS"
    for i, n in enumerate(names[:-1]):
        assert getattr(ng, n[len("NSMP_"):]) == i


def test_mesh_generator_shapes_and_determinism():
    m1 = ng.make_mesh(8, 6, seed=0)
    m2 = ng.make_mesh(8, 6, seed=0)
    m3 = ng.make_mesh(8, 6, seed=7)
    for k in m1:
        assert np.array_equal(m1[k], m2[k])
    assert not np.array_equal(m1["xv"], m3["xv"])
    assert m1["No_vp"].shape == (96, 3) and m1["xv"].shape == (63,)
    # neighbour symmetry: j is a neighbour of i iff i is a neighbour of j
    cp = m1["No_cp"]
    for i in range(cp.shape[0]):
        for j in range(3):
            n = cp[i, j]
            if n:
                assert (i + 1) in cp[n - 1]
    assert np.count_nonzero(cp == 0) == 2 * (8 + 6)


def test_initial_channel_keyed_by_cell():
    prm = ng.channel_params(8, 6, 6, 1e-3)
    ncell = ng.n_cell_of(ng.make_mesh(8, 6))
    u, v, w, p = ng.initial_channel(prm, ncell, seed=1)
    u2, _, _, _ = ng.initial_channel(prm, ncell + 10, seed=1)
    # the value of a cell does not depend on the array it is written into
    assert np.array_equal(u[:prm["n0"]], u2[:prm["n0"]])
    assert np.all(u[prm["n0"]:] == 0) and np.all(p == 0)
    sig = ng.geometry(prm, ng.make_mesh(8, 6), ng.G_SIG)
    k = 3
    prof = 18.0 * sig[k] * (2 - sig[k])
    assert np.all(np.abs(u[:prm["n0"], k] - prof) <= 1.8)
    assert np.all(u[:prm["n0"], 0] == 0)  # ghost layer below the wall


def test_bad_mesh_arguments():
    L = ng.lib()
    n0, nv = C.c_int(), C.c_int()
    assert L.nsmp_mesh_size(1, 5, C.byref(n0), C.byref(nv)) == ng.ERR_ARG
    with pytest.raises(ValueError):
        ng.make_mesh(8, 6, jitter=0.9)
