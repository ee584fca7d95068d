"""The FP64 kernel-matrix residual ||f - K x|| / ||f|| (K generated on the fly on the GPU, never
formed) against NumPy on the oracle's dense kernel matrix, and at the full HSS2D workload
for the solutions of every solve path (GPU)."""
import numpy as np
import pytest

from oracle import geometry as OG, kernels as OK

pytestmark = pytest.mark.gpu


def _params(npan, precision="fp64", Ng=8):
    from hssc_directsolver_gb300 import hss2d as G2, kernels as GK
    h = 2.0 / (Ng * npan)
    return G2.HSS2DParams(Ng=Ng, npan=npan, kernel=GK.Kernel("SL_L_2D", h, GK.Modulation(),
                                                               GK.Modulation(0.5, 0, 0, 20.0)),
                          precision=precision)


def test_hss2d_kernel_residual_matches_dense(gpu):
    from hssc_directsolver_gb300 import hss2d as G2
    npan = 4
    t = G2.HSS2D_build_tree_nsym(_params(npan))
    kp = OK.KernelParams(flag=OK.SL_L_2D, h=2.0 / (8 * npan), c=OK.Modulation(0.5, 0, 0, 20.0))
    X = OG.grid_source(8, npan)
    A = OK.kernel_eval(X, X, kp)
    r = np.random.default_rng(3)
    x = r.standard_normal((t.N, 5))
    f = A @ x + 1e-6 * r.standard_normal((t.N, 5))
    want = max(np.linalg.norm(f[:, c] - A @ x[:, c]) / np.linalg.norm(f[:, c]) for c in range(5))
    got = G2.HSS2D_kernel_residual(t, f, x)
    assert abs(got - want) <= 1e-6 * want


def test_hss1d_kernel_residual_matches_dense(gpu):
    from hssc_directsolver_gb300 import hss1d as G1, kernels as GK
    Xs = [OG.star_curve(700), OG.star_curve(333)]
    H = G1.HSS1D_compress_batch(Xs, 64, 1e-10, GK.Kernel("DL_L_2D"))
    kp = OK.KernelParams(flag=OK.DL_L_2D)
    r = np.random.default_rng(4)
    x = r.standard_normal((H.N, 3))
    f = np.zeros_like(x)
    o = 0
    for X in Xs:
        A = OK.kernel_eval(X, X, kp)
        f[o:o + len(X)] = A @ x[o:o + len(X)]
        o += len(X)
    f += 1e-7 * r.standard_normal(f.shape)
    want = 0.0
    for c in range(3):
        o, num = 0, 0.0
        for X in Xs:
            A = OK.kernel_eval(X, X, kp)
            num += np.sum((f[o:o + len(X), c] - A @ x[o:o + len(X), c]) ** 2)
            o += len(X)
        want = max(want, np.sqrt(num) / np.linalg.norm(f[:, c]))
    got = G1.HSS1D_kernel_residual(H, f, x)
    assert abs(got - want) <= 1e-6 * want


@pytest.mark.parametrize("precision", ["fp64", "dfloat", "tc"])
def test_full_size_solution_against_the_kernel_matrix(gpu, precision):
    """N = 65536: the refined solution's residual against the kernel matrix itself stays at the
    compression tolerance's level (the compressed operator is accurate to ~1e-10)."""
    from hssc_directsolver_gb300 import hss2d as G2
    t = G2.HSS2D_invert_nsym(G2.HSS2D_build_tree_nsym(_params(32, precision)))
    F = np.random.default_rng(0).standard_normal((t.N, 4))
    F /= np.linalg.norm(F, axis=0)
    x, rr, it = G2.HSS2D_solve(t, F, 1e-10, 6)
    assert rr <= 1e-10
    true = G2.HSS2D_kernel_residual(t, F, x)
    assert true <= 1e-8, true
