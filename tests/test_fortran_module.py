"""The Fortran binding (fortran/mge_gpu_mod.f90) against the C header, read
as text (no Fortran compiler is needed): every entry point it binds is one
the header declares, its ABI version is the header's, and each bind(C) type
lists the C struct's fields in the same order with matching kinds and
array sizes (CPU only)."""
import os
import re

from code_mge_gb300 import _abi as A

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
MOD = open(os.path.join(ROOT, "fortran", "mge_gpu_mod.f90")).read()
HDR = open(os.path.join(ROOT, "include", "mge_gpu.h")).read()

KIND = {"integer(c_int)": A.C.c_int, "real(c_double)": A.C.c_double, "type(c_ptr)": A.C.c_void_p}


def fortran_fields(type_name):
    """(name, kind, element count) of a bind(C) type, in order."""
    body = re.search(r"type, bind\(C\) :: %s\n(.*?)\n\s*end type" % type_name, MOD, re.S).group(1)
    out = []
    for line in body.split("\n"):
        line = line.split("!")[0].strip()
        if not line:
            continue
        kind, names = [x.strip() for x in line.split("::")]
        for item in re.findall(r"(\w+)(?:\(([^)]*)\))?", names):
            name, dims = item
            count = 1
            for d in (dims.split(",") if dims else []):
                d = d.strip()
                count *= int(d) if d.isdigit() else int(re.search(r"%s\s*=\s*(\d+)" % d, MOD).group(1))
            out.append((name, kind, count))
    return out


def ctypes_fields(cls):
    out = []
    for name, ty in cls._fields_:
        count = 1
        while hasattr(ty, "_length_"):
            count *= ty._length_
            ty = ty._type_
        out.append((name, ty, count))
    return out


def test_bound_names_are_declared():
    bound = set(re.findall(r'bind\(C, name="(mge_\w+)"\)', MOD))
    assert bound, "no bound entry points found"
    assert bound <= set(A.HEADER_SYMBOLS), sorted(bound - set(A.HEADER_SYMBOLS))


def test_abi_version_matches_the_header():
    f = int(re.search(r"MGE_ABI_VERSION\s*=\s*(\d+)", MOD).group(1))
    c = int(re.search(r"#define MGE_ABI_VERSION (\d+)", HDR).group(1))
    assert f == c == A.MGE_ABI_VERSION


def test_types_follow_the_c_structs():
    for fname, cls in (("mge_params", A.MgeParams), ("mge_block_desc", A.MgeBlockDesc), ("mge_forces", A.MgeForces),
                       ("mge_solve_opts", A.MgeSolveOpts)):
        f = fortran_fields(fname)
        c = ctypes_fields(cls)
        assert [x[0] for x in f] == [x[0] for x in c], fname
        for (name, kind, count), (_, ty, n) in zip(f, c):
            want = KIND[kind]
            ok = ty is want or (want is A.C.c_void_p and ty not in (A.C.c_int, A.C.c_double))
            assert ok and count == n, (fname, name, kind, count, ty, n)
