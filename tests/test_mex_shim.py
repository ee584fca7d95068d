"""The MATLAB MEX binding (hssc_directsolver_gb300/mex/hss_gpu_mex.c), compiled against the
host-side stand-ins of the MATLAB C API in tests/mex_stub and linked to libhssgpu.so.

CPU: the shim compiles warning-free against include/hssgpu.h and the mex.h declarations,
links against every C-ABI symbol it calls, and turns the library's status into a MATLAB
error (no GPU here: HSS_ERR_CUDA).  GPU: the reference-style call sequence through the shim
(params struct -> INFO_TREE / A_HSS structs, K_HSS cell) gives the Python binding's results.
"""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
LIBDIR = os.path.join(ROOT, "hssc_directsolver_gb300")
SRC = [os.path.join(LIBDIR, "mex", "hss_gpu_mex.c"), os.path.join(ROOT, "tests", "mex_stub", "mex_stub.c"),
       os.path.join(ROOT, "tests", "mex_stub", "mex_driver.c")]
NPAN, M = 4, 1024


def _build(tmp):
    if not os.path.exists(os.path.join(LIBDIR, "libhssgpu.so")):
        pytest.skip("libhssgpu.so not built")
    exe = os.path.join(tmp, "mex_driver")
    cmd = ["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-O1", "-I" + os.path.join(ROOT, "tests", "mex_stub"),
           "-I" + os.path.join(ROOT, "include"), "-o", exe, *SRC, "-L" + LIBDIR, "-lhssgpu",
           "-Wl,-rpath," + LIBDIR, "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def _inputs(tmp):
    from oracle import geometry as OG
    X = OG.grid_source(8, NPAN)
    N = X.shape[0]
    F = np.random.default_rng(2).standard_normal((N, 2))
    C = OG.star_curve(M)
    with open(os.path.join(tmp, "sizes.txt"), "w") as f:
        f.write(f"{N} {NPAN} {M}\n")
    np.asfortranarray(X).T.tofile(os.path.join(tmp, "x_source.bin"))   # column-major N x 2
    np.asfortranarray(F).T.tofile(os.path.join(tmp, "rhs.bin"))
    np.asfortranarray(C).T.tofile(os.path.join(tmp, "curve.bin"))
    return X, F, C


def test_mex_shim_compiles_links_and_reports_status(tmp_path):
    exe = _build(str(tmp_path))
    _inputs(str(tmp_path))
    from hssc_directsolver_gb300 import _lib
    if _lib.device_count() > 0:
        pytest.skip("a GPU is present: the GPU test covers the run")
    r = subprocess.run([exe, str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 3, r.stdout + r.stderr
    assert "MEXERR: hss:gpu:" in r.stdout and "status 2" in r.stdout   # HSS_ERR_CUDA as a MATLAB error


@pytest.mark.gpu
def test_mex_shim_matches_python_binding(gpu, tmp_path):
    from hssc_directsolver_gb300 import hss1d as G1, hss2d as G2, kernels as GK
    exe = _build(str(tmp_path))
    X, F, C = _inputs(str(tmp_path))
    r = subprocess.run([exe, str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 0 and "MEXOK" in r.stdout, r.stdout + r.stderr
    N = X.shape[0]
    y2 = np.fromfile(os.path.join(tmp_path, "y2d.bin")).reshape(2, N).T
    y1 = np.fromfile(os.path.join(tmp_path, "y1d.bin"))
    lines = open(os.path.join(tmp_path, "info.txt")).read().split("\n")
    h = 2.0 / (8 * NPAN)
    p = G2.HSS2DParams(Ng=8, npan=NPAN, kernel=GK.Kernel("SL_L_2D", h, GK.Modulation(),
                                                           GK.Modulation(0.5, 0, 0, 20.0)))
    t = G2.HSS2D_invert_nsym(G2.HSS2D_build_tree_nsym(p))
    ref = G2.HSS2D_applyinv_nsym(t, None, F)
    assert np.linalg.norm(y2 - ref) <= 1e-13 * np.linalg.norm(ref)
    depth, nb = lines[0].split()
    assert int(float(depth)) == t.depth and int(nb) == t.nboxes
    n, k, _ = t.box_sizes()
    assert [int(float(v)) for v in lines[1].split()] == list(k)
    assert [int(float(v)) for v in lines[2].split()] == list(t.export_box(1)["J"] + 1)   # 1-based
    FI0, _ = t.export_inverse(0)
    m0, v0 = lines[3].split()
    assert int(m0) == FI0.shape[0] and float(v0) == FI0[0, 0]
    H = G1.HSS1D_compress_nsym("green", C, 64, 1e-10, GK.Kernel("DL_L_2D"))
    G1.HSS1D_invert_nsym(H)
    x1 = G1.HSS1D_applyinv_nsym(H, None, None, F[:M, 0])
    assert np.linalg.norm(y1 - x1) <= 1e-13 * np.linalg.norm(x1)
    inf = H.info()
    assert int(lines[4]) == len(inf["kskel"])
    assert [int(float(v)) for v in lines[5].split()] == list(inf["kskel"])
    assert [int(float(v)) for v in lines[6].split()] == list(H.export_box(1)["I_SKUP"] + 1)
    # the complex Helmholtz curve through the shim: complex right-hand side in, complex out
    gb, gc = GK.Modulation(0.5, 0.3, 0.0, 2.0), GK.Modulation(-0.3, 0.0, -0.2, 3.0)
    hk = GK.Kernel("SL_H_2D", 0.05, gb, gc, 20.0, 0.3 + 0.1j)
    Hc = G1.HSS1D_compress_nsym("green", C, 64, 1e-10, hk)
    G1.HSS1D_invert_nsym(Hc)
    xc = G1.HSS1D_applyinv_nsym(Hc, None, None, F[:M, 0] + 1j * F[:M, 1])
    yc = np.fromfile(os.path.join(tmp_path, "y1c.bin")).view(np.complex128)
    assert np.linalg.norm(yc - xc) <= 1e-13 * np.linalg.norm(xc)
    ke = np.fromfile(os.path.join(tmp_path, "ke.bin")).view(np.complex128).reshape(8, 8, order="F")
    P = np.asfortranarray(C[:8, :2])
    ref_ke = GK.Kernel_Eval(P, P, hk)
    assert np.abs(ke - ref_ke).max() <= 1e-15 * np.abs(ref_ke).max()
