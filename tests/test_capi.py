"""The C ABI: the library builds, loads and exports every symbol include/hssgpu.h declares
(CPU only: no compute call is made without a GPU)."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
HEADER = os.path.join(ROOT, "include", "hssgpu.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(hss\w+)\s*\(", src, flags=re.M)))


@pytest.fixture(scope="module")
def lib():
    from hssc_directsolver_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        import __graft_entry__
        __graft_entry__.build()
    return _lib.lib()


def test_header_declares_the_boundary():
    names = declared_functions()
    for need in ("hss1d_compress", "hss1d_invert", "hss1d_apply", "hss1d_applyinv", "hss2d_build_tree",
                 "hss2d_compress", "hss2d_invert", "hss2d_apply", "hss2d_applyinv", "hss2d_solve"):
        assert need in names


def test_library_exports_every_declared_symbol(lib):
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_binding_covers_header():
    from hssc_directsolver_gb300 import _lib
    assert set(declared_functions()) == set(_lib.SIGNATURES)


def test_status_paths_without_gpu(lib):
    from hssc_directsolver_gb300 import _lib
    n = C.c_int32(-1)
    assert lib.hss_device_count(C.byref(n)) == _lib.HSS_OK
    assert n.value >= 0
    assert lib.hss_version() >= 100
    # NULL arguments are rejected before any device work
    assert lib.hss2d_compress(None) == _lib.HSS_ERR_ARG
    assert lib.hss1d_invert(None) == _lib.HSS_ERR_ARG
    assert b"NULL" in lib.hss_last_error()
    assert lib.hss1d_sum(None, None, 1e-10, None) == _lib.HSS_ERR_ARG
    assert lib.hss1d_compress_rect(None, None, 0, 0, None, 0, 0, 64, 1e-10, None, 0) == _lib.HSS_ERR_ARG
    assert lib.hss1d_rect_info(None, None, None, None, None, None) == _lib.HSS_ERR_ARG
    # the least squares' precision is checked first: only FP64 and DFLOAT are accepted
    assert lib.hss_batched_lstsq_device_ex(None, 8, 4, 2, 1, _lib.HSS_PREC_MIXED, None) == _lib.HSS_ERR_ARG
    assert b"HSS_PREC_DFLOAT" in lib.hss_last_error()
    assert lib.hss_batched_lstsq_device_ex(None, 8, 4, 2, 1, _lib.HSS_PREC_DFLOAT, None) == _lib.HSS_ERR_ARG
    if n.value == 0:
        h = C.c_void_p()
        p = _lib.hss2d_params(8, 4, 2, 0, 0, 0, 0, 0, 1e-10, _lib.hss_kernel_params())
        assert lib.hss2d_build_tree(C.byref(h), C.byref(p)) == _lib.HSS_ERR_CUDA
        # the HSS1D constructors need the device before they look at their inputs' values
        U = (C.c_double * 8)()
        assert lib.hss1d_compress_lr(C.byref(h), U, U, 4, 2, 4, 4, 2, 1e-10, 0) == _lib.HSS_ERR_CUDA
        kp = _lib.hss_kernel_params()
        assert lib.hss1d_compress_rect(C.byref(h), U, 4, 4, U, 4, 4, 2, 1e-10, C.byref(kp), 0) == _lib.HSS_ERR_CUDA


def test_product_fails_loudly_without_library(monkeypatch, tmp_path):
    from hssc_directsolver_gb300 import _lib
    monkeypatch.setattr(_lib, "LIB_PATH", str(tmp_path / "missing.so"))
    monkeypatch.setattr(_lib, "_lib", None)
    with pytest.raises(ImportError):
        _lib.lib()


def test_block_submatrix_apply_composition(monkeypatch):
    """BHSS1D_apply_nsym's host composition (HSS1D/BHSS1D_apply_nsym.m:38-73): four submatrix
    applies, X split after the first block column's selected rows.  The GPU submatrix apply is
    replaced by its dense definition here; the GPU path is tested on a GB300."""
    import numpy as np
    from hssc_directsolver_gb300 import hss1d as G1

    class Dense:
        def __init__(self, A):
            self.A, self.N = A, A.shape[0]

    def sub(K, bd, bu, dn, up, q):
        dn, up = np.asarray(dn, bool), np.asarray(up, bool)
        return K.A[np.ix_(dn, up)] @ np.asarray(q)[up]

    monkeypatch.setattr(G1, "HSS1D_apply_submatrix_nsym", sub)
    rng = np.random.default_rng(0)
    K = [Dense(rng.standard_normal((n, n))) for n in (7, 6, 6, 9)]
    dn1 = np.array([1, 0, 1, 0, 1, 0, 1], bool)
    dn2 = np.array([1, 1, 0, 0, 1, 0, 0, 1, 0], bool)
    I_dn = [[dn1, np.array([1, 1, 0, 1, 0, 1], bool)], [np.array([1, 0, 1, 1, 0, 1], bool), dn2]]
    I_up = [[~dn1, np.array([1, 1, 1, 0, 1, 1], bool)], [np.array([0, 1, 1, 1, 0, 0], bool), ~dn2]]
    X = rng.standard_normal(((~dn1).sum() + (~dn2).sum(), 2))
    Y = G1.BHSS1D_apply_nsym(K[0], K[1], K[2], K[3], None, None, I_dn, I_up, X)
    A = np.block([[K[0].A[np.ix_(I_dn[0][0], I_up[0][0])], K[1].A[np.ix_(I_dn[0][1], I_up[0][1])]],
                  [K[2].A[np.ix_(I_dn[1][0], I_up[1][0])], K[3].A[np.ix_(I_dn[1][1], I_up[1][1])]]])
    assert np.abs(Y - A @ X).max() <= 1e-14


def test_binding_constants_match_header():
    """Every #define HSS_* of the header has the same value in the Python binding."""
    from hssc_directsolver_gb300 import _lib
    src = open(HEADER).read()
    consts = dict(re.findall(r"^#define\s+(HSS_\w+)\s+(-?\d+)", src, flags=re.M))
    assert len(consts) >= 15
    for name, val in consts.items():
        assert getattr(_lib, name) == int(val), name


def test_struct_layouts_match_header(tmp_path):
    """The ctypes mirrors of hss_kernel_params and hss2d_params have the C layout: sizes and
    every field offset, from a C program compiled against the header (needs a C compiler)."""
    import shutil
    import subprocess
    from hssc_directsolver_gb300 import _lib
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    structs = {"hss_kernel_params": _lib.hss_kernel_params, "hss2d_params": _lib.hss2d_params}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "hssgpu.h"', "int main(void) {"]
    for sname, cls in structs.items():
        lines.append(f'printf("{sname} size %zu\\n", sizeof({sname}));')
        for f, _ in cls._fields_:
            lines.append(f'printf("{sname} {f} %zu\\n", offsetof({sname}, {f}));')
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {tuple(l.split()[:2]): int(l.split()[2]) for l in out if l.strip()}
    for sname, cls in structs.items():
        assert got[(sname, "size")] == C.sizeof(cls), sname
        for f, _ in cls._fields_:
            assert got[(sname, f)] == getattr(cls, f).offset, (sname, f)


def test_binding_arity_matches_header():
    """Each ctypes signature takes as many arguments as the header's prototype declares."""
    from hssc_directsolver_gb300 import _lib
    src = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    protos = dict(re.findall(r"\b(hss\w+)\s*\(([^)]*)\)\s*;", src))
    assert protos
    for name, params in protos.items():
        params = params.strip()
        n = 0 if params in ("", "void") else params.count(",") + 1
        assert len(_lib.SIGNATURES[name][1]) == n, name


def test_binding_argument_kinds_match_header():
    """Position by position: pointers bind as pointers, and int32_t / int64_t / uint64_t /
    double scalars as the same ctypes scalar."""
    from hssc_directsolver_gb300 import _lib
    src = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    protos = dict(re.findall(r"\b(hss\w+)\s*\(([^)]*)\)\s*;", src))
    scalars = {"int32_t": C.c_int32, "int64_t": C.c_int64, "uint64_t": C.c_uint64, "double": C.c_double,
               "float": C.c_float, "int": C.c_int}
    ptr_types = (C.c_void_p, C.c_char_p)
    for name, params in protos.items():
        params = params.strip()
        if params in ("", "void"):
            continue
        for i, (decl, ct) in enumerate(zip(params.split(","), _lib.SIGNATURES[name][1])):
            if "*" in decl:
                assert ct in ptr_types or issubclass(ct, C._Pointer), (name, i, decl)
            else:
                base = decl.replace("const", "").split()[0]
                assert ct is scalars[base], (name, i, decl)
