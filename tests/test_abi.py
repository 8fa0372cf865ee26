"""The C-ABI boundary: every declared entry point is exported, the ctypes
mirror matches the C struct layout, and parameter validation works without a
GPU (no compute call is made here)."""
import ctypes as C
import os
import re
import subprocess

import pytest

from code_mge_gb300 import _abi as A

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "mge_gpu.h")


def header_functions():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(mge_[a-z_0-9]+)\s*\(", txt)))


def test_header_lists_match():
    assert set(header_functions()) == set(A.HEADER_SYMBOLS)


def test_library_exports_every_declared_symbol(gpulib):
    for name in header_functions():
        assert hasattr(gpulib, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", os.path.join(ROOT, "code_mge_gb300", "_build", "libmge_gpu.so")],
                         capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (mge_\w+)", out))
    assert set(header_functions()) <= exported


def test_oracle_exports_mirror(oraclelib):
    for name, _, _ in A.SIGNATURES:
        assert hasattr(oraclelib, "mgeo_" + name)


def test_struct_layout_matches_c(tmp_path):
    src = tmp_path / "lay.c"
    src.write_text('''#include <stdio.h>
#include <stddef.h>
#include "mge_gpu.h"
int main(void){
 printf("%zu %zu %zu %zu\\n", sizeof(mge_params), sizeof(mge_block_desc), sizeof(mge_forces), sizeof(mge_solve_opts));
 printf("%zu %zu %zu %zu %zu %zu\\n", offsetof(mge_params, mcyc), offsetof(mge_params, conv_drop),
        offsetof(mge_block_desc, blank), offsetof(mge_block_desc, parent), offsetof(mge_block_desc, offset),
        offsetof(mge_block_desc, psurf));
 printf("%d\\n", MGE_ABI_VERSION);
 return 0;}''')
    exe = tmp_path / "lay"
    subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    a, b, v = subprocess.run([str(exe)], capture_output=True, text=True).stdout.split("\n")[:3]
    sizes = [int(x) for x in a.split()]
    offs = [int(x) for x in b.split()]
    assert sizes == [C.sizeof(A.MgeParams), C.sizeof(A.MgeBlockDesc), C.sizeof(A.MgeForces),
                     C.sizeof(A.MgeSolveOpts)]
    assert offs == [A.MgeParams.mcyc.offset, A.MgeParams.conv_drop.offset, A.MgeBlockDesc.blank.offset,
                    A.MgeBlockDesc.parent.offset, A.MgeBlockDesc.offset.offset, A.MgeBlockDesc.psurf.offset]
    assert int(v) == A.MGE_ABI_VERSION


def test_init_rejects_bad_config_without_gpu(gpulib):
    from code_mge_gb300 import cases as K
    p = K.params(0.5, nlevel=2)
    ctx = C.c_void_p()
    p.nlevel = 0
    assert gpulib.mge_init(C.byref(p), 0, C.byref(ctx)) == A.MGE_EBADCFG
    p.nlevel = 2
    p.mstage = 99
    assert gpulib.mge_init(C.byref(p), 0, C.byref(ctx)) == A.MGE_EBADCFG
    p.mstage = 5
    p.dissip = 7
    assert gpulib.mge_init(C.byref(p), 0, C.byref(ctx)) == A.MGE_EBADCFG


def test_params_default_matches_input_param(gpulib):
    from code_mge_gb300 import cases as K
    p = A.MgeParams()
    gpulib.mge_params_default(C.byref(p), 1.4, 0.5, 0.0, 0.0)
    q = K.params(0.5)
    for f in ("p0", "c0", "ei0", "u0", "v0", "w0", "h0", "vis4"):
        assert getattr(p, f) == pytest.approx(getattr(q, f), rel=1e-15), f
