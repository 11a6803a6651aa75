"""The committed Fortran binding (fortran/nsmp_gpu.F90, not compiled: no
Fortran compiler exists here) agrees with the C header: every bind(C) name
is a declared export, and the bind(C) derived types list the C structs'
members in the same order (CPU only, text checks)."""
import os
import re

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _header():
    src = open(os.path.join(REPO, "include", "nsmp.h")).read()
    return re.sub(r"/\*.*?\*/", "", src, flags=re.S)


def _fortran():
    return open(os.path.join(REPO, "fortran", "nsmp_gpu.F90")).read()


def test_bind_names_are_header_exports():
    declared = set(re.findall(r"\b(nsmp_[a-z0-9_]+)\s*\(", _header()))
    names = re.findall(r'bind\(C,\s*name="([a-z0-9_]+)"\)', _fortran())
    assert len(names) >= 30
    assert set(names) <= declared, set(names) - declared


def _c_members(struct):
    body = re.search(r"typedef struct %s \{(.*?)\} %s;" % (struct, struct), _header(), flags=re.S).group(1)
    out = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        out += re.findall(r"(\w+)\s*(?:,|$)", decl)
    return out


def _f_members(typ):
    body = re.search(r"type, bind\(C\) :: %s\n(.*?)end type" % typ, _fortran(), flags=re.S).group(1)
    out = []
    for ln in body.splitlines():
        if "::" in ln:
            out += [n.strip() for n in ln.split("::")[1].split("!")[0].split(",") if n.strip()]
    return out


def test_derived_types_match_structs():
    for name in ("nsmp_params", "nsmp_mesh", "nsmp_stage_info"):
        assert _f_members(name) == _c_members(name), name


def test_enum_values_match_header():
    h, f = _header(), _fortran()
    for prefix in ("NSMP_F_", "NSMP_CFL_"):
        block = re.search(r"enum \{([^}]*%s[^}]*)\}" % prefix, h, flags=re.S).group(1)
        names = [n.strip().split("=")[0].strip() for n in block.replace("\n", " ").split(",") if n.strip()]
        for i, n in enumerate(names):
            if n.endswith(("COUNT", "NFIELDS")) and n not in f:
                continue
            m = re.search(r"\b%s\s*=\s*(\d+)" % n, f)
            assert m, n
            assert int(m.group(1)) == i, (n, m.group(1), i)
