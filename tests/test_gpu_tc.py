"""Tensor-core (tcgen05) skinny products over bf16 digit slices, and the HSS2D inverse apply
that runs on them (HSS_PREC_TC: every level of the apply, up and down the tree, in one
cooperative launch), against FP64 products and the oracle (GPU).

The product keeps the digit pairs of weight 256^-t, t <= 7, of a fixed-point split of
each row of A and each column of B (6 digits of 8 bits each).  Per output entry the error
is bounded by a small multiple of 2^-48 * K * max_k |A(i,k)| * max_k |B(k,j)|; the tests
hold it to 2^-44 of that scale.
"""
import numpy as np
import pytest

from oracle import hss2d as O2, kernels as OK

pytestmark = pytest.mark.gpu
TOL = 2.0 ** -44


@pytest.fixture(scope="module")
def env(gpu):
    import torch
    from hssc_directsolver_gb300 import _lib
    return torch, _lib, _lib.lib()


def _tc(env, A, B):
    torch, L, lib = env
    batch, K, M = A.shape            # A[b] is M x K column-major (stored transposed)
    N = B.shape[1]
    dA = torch.from_numpy(np.ascontiguousarray(A)).cuda()
    dB = torch.from_numpy(np.ascontiguousarray(B)).cuda()
    dC = torch.full((batch, N, M), np.nan, dtype=torch.float64, device="cuda")
    L.check(lib.hss_batched_gemv_tc_device(L.ptr(dA), L.ptr(dB), L.ptr(dC), M, N, K, batch, None))
    torch.cuda.synchronize()
    return dC.cpu().numpy()


def _check(A, B, C):
    ref = np.einsum("bkm,bnk->bnm", A, B)
    rowmax = np.abs(A).max(axis=1)                   # batch x M
    colmax = np.abs(B).max(axis=2)                   # batch x N
    K = A.shape[1]
    scale = K * rowmax[:, None, :] * colmax[:, :, None]
    err = np.abs(C - ref)
    assert np.all(np.isfinite(C))
    assert np.all(err <= TOL * scale + 1e-300), (err / np.maximum(scale, 1e-300)).max()


@pytest.mark.parametrize("M,N,K,batch", [(1, 1, 1, 1), (8, 4, 16, 2), (48, 4, 64, 5), (130, 3, 300, 3),
                                         (257, 4, 1000, 2), (640, 2, 257, 1), (1500, 4, 3040, 1)])
def test_tc_product_matches_fp64(env, M, N, K, batch):
    r = np.random.default_rng(M * 7 + K)
    A = r.standard_normal((batch, K, M))
    B = r.standard_normal((batch, N, K))
    _check(A, B, _tc(env, A, B))


def test_tc_product_wide_dynamic_range(env):
    """Rows and columns spanning 40 orders of magnitude, zero rows and zero columns, and
    entries at exact powers of two (the top digit at its limit)."""
    r = np.random.default_rng(5)
    M, N, K, batch = 200, 4, 700, 2
    A = r.standard_normal((batch, K, M)) * 10.0 ** r.uniform(-20, 20, (batch, 1, M))
    A[:, :, 7] = 0.0
    A[0, :, 9] = 2.0 ** 30
    A[1, :, 11] = -(2.0 ** -30)
    B = r.standard_normal((batch, N, K)) * 10.0 ** r.uniform(-20, 20, (batch, N, 1))
    B[1, 2, :] = 0.0
    B[0, 1, ::3] = 1.0
    _check(A, B, _tc(env, A, B))


def test_tc_product_rejects_wide_blocks(env):
    torch, L, lib = env
    d = torch.zeros(64, dtype=torch.float64, device="cuda")
    assert lib.hss_batched_gemv_tc_device(L.ptr(d), L.ptr(d), L.ptr(d), 4, 5, 4, 1, None) == L.HSS_ERR_ARG


def _params(npan, precision, Ng=8):
    from hssc_directsolver_gb300 import hss2d as G2, kernels as GK
    h = 2.0 / (Ng * npan)
    return G2.HSS2DParams(Ng=Ng, npan=npan, kernel=GK.Kernel("SL_L_2D", h, GK.Modulation(),
                                                               GK.Modulation(0.5, 0, 0, 20.0)),
                          precision=precision)


@pytest.mark.parametrize("npan", [4, 8])
def test_tc_inverse_apply_matches_oracle(gpu, npan):
    from hssc_directsolver_gb300 import hss2d as G2
    t = G2.HSS2D_invert_nsym(G2.HSS2D_build_tree_nsym(_params(npan, "tc")))
    kp = OK.KernelParams(flag=OK.SL_L_2D, h=2.0 / (8 * npan), c=OK.Modulation(0.5, 0, 0, 20.0))
    prm = O2.HSS2DParams(Ng=8, npan=npan, kp=kp)
    ot = O2.build_tree_nsym(prm)
    inv = O2.invert_nsym(ot, prm, O2.compress_nsym(ot, prm))
    q = np.random.default_rng(7).standard_normal((prm.N, 6))   # 6 columns: two column groups
    x = G2.HSS2D_applyinv_nsym(t, None, q)
    xo = O2.applyinv_nsym(ot, inv, q)
    assert np.linalg.norm(x - xo) <= 1e-11 * np.linalg.norm(xo)
    # the forward apply (the refinement residual) runs on double-float products in this mode
    u = G2.HSS2D_apply_nsym(t, None, q)
    uo = O2.apply_nsym(ot, O2.compress_nsym(ot, prm), q)
    assert np.linalg.norm(u - uo) <= 1e-12 * np.linalg.norm(uo)
    xs, rr, it = G2.HSS2D_solve(t, q[:, :4], 1e-10, 3)
    assert rr <= 1e-10 and it == 1


def test_tc_full_size_solve(gpu):
    """The 256 x 256 workload (N = 65536) solves to 1e-10 with one tensor-core inverse apply,
    and its inverse apply agrees with the double-float one to the solve tolerance (measured:
    2.7e-11; the digit products carry ~2^-47 of each row's largest factor entry)."""
    from hssc_directsolver_gb300 import hss2d as G2
    f = np.random.default_rng(0).standard_normal((65536, 4))
    t = G2.HSS2D_invert_nsym(G2.HSS2D_build_tree_nsym(_params(32, "tc")))
    x, rr, it = G2.HSS2D_solve(t, f, 1e-10, 3)
    assert rr <= 1e-10 and it == 1
    d = G2.HSS2D_invert_nsym(G2.HSS2D_build_tree_nsym(_params(32, "dfloat")))
    xd = G2.HSS2D_applyinv_nsym(d, None, f)
    xt = G2.HSS2D_applyinv_nsym(t, None, f)
    dd = np.linalg.norm(xt - xd) / np.linalg.norm(xd)
    print(f"tensor-core vs double-float inverse apply: {dd:.2e}")
    assert dd <= 1e-10
    # one launch runs every level, each waiting for the one before on every SM: the same
    # input gives the same bits after an apply of another input (no stale reads)
    G2.HSS2D_applyinv_nsym(t, None, np.random.default_rng(1).standard_normal((65536, 4)))
    assert np.array_equal(G2.HSS2D_applyinv_nsym(t, None, f), xt)
