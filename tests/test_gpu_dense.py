"""Batched dense primitives of libhssgpu.so against NumPy / the oracle (GPU)."""
import ctypes as C

import numpy as np
import pytest

from oracle import geometry, idecomp, kernels

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env(gpu):
    import torch
    from hssc_directsolver_gb300 import _lib
    return torch, _lib, _lib.lib()


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("M,N,K", [(1, 1, 1), (5, 3, 7), (70, 4, 65), (130, 90, 33), (257, 8, 300)])
def test_gemm(env, M, N, K):
    torch, L, lib = env
    r = np.random.default_rng(M + N + K)
    A = r.standard_normal((3, K, M))
    B = r.standard_normal((3, N, K))
    dA, dB = _dev(torch, A), _dev(torch, B)
    dC = torch.zeros((3, N, M), dtype=torch.float64, device="cuda")
    L.check(lib.hss_batched_gemm_device(L.ptr(dA), L.ptr(dB), L.ptr(dC), M, N, K, 3, None))
    torch.cuda.synchronize()
    ref = np.einsum("bkm,bnk->bnm", A, B)
    assert np.abs(dC.cpu().numpy() - ref).max() <= 1e-13 * max(1.0, np.abs(ref).max())


@pytest.mark.parametrize("n", [1, 5, 31, 32, 33, 64, 100, 300])
def test_inverse_fp64(env, n):
    torch, L, lib = env
    r = np.random.default_rng(n)
    A = r.standard_normal((4, n, n)) + 0.1 * n * np.eye(n)[None]
    dA = _dev(torch, A)
    info = torch.zeros(4, dtype=torch.int32, device="cuda")
    L.check(lib.hss_batched_inverse_device(L.ptr(dA), n, 4, L.ptr(info), None))
    torch.cuda.synchronize()
    assert np.all(info.cpu().numpy() == 0)
    inv = dA.cpu().numpy()
    for b in range(4):
        assert np.abs(inv[b].T @ A[b].T - np.eye(n)).max() < 1e-12


def test_inverse_fp32(env):
    torch, L, lib = env
    n = 96
    A = np.random.default_rng(3).standard_normal((2, n, n)) + 10 * np.eye(n)[None]
    dA = _dev(torch, A.astype(np.float32))
    info = torch.zeros(2, dtype=torch.int32, device="cuda")
    L.check(lib.hss_batched_inverse_device_f32(L.ptr(dA), n, 2, L.ptr(info), None))
    torch.cuda.synchronize()
    inv = dA.cpu().numpy().astype(np.float64)
    for b in range(2):
        assert np.abs(inv[b].T @ A[b].T - np.eye(n)).max() < 1e-4


def test_inverse_reports_singular_block(env):
    """Host-side fault injection: a singular block must return HSS_ERR_SINGULAR-style info, not trap."""
    torch, L, lib = env
    n = 40
    A = np.random.default_rng(4).standard_normal((2, n, n))
    A[1] = 0.0
    dA = _dev(torch, A)
    info = torch.zeros(2, dtype=torch.int32, device="cuda")
    L.check(lib.hss_batched_inverse_device(L.ptr(dA), n, 2, L.ptr(info), None))
    torch.cuda.synchronize()
    inf = info.cpu().numpy()
    assert inf[0] == 0 and inf[1] == 1
    A2 = A.copy()
    A2[0, 3, 3] = np.nan
    A2[1] = np.eye(n)
    dA = _dev(torch, A2)
    L.check(lib.hss_batched_inverse_device(L.ptr(dA), n, 2, L.ptr(info), None))
    torch.cuda.synchronize()
    inf = info.cpu().numpy()
    assert inf[1] == 0 and inf[0] != 0


@pytest.mark.parametrize("m,n,kf", [(40, 30, 20), (132, 64, 48), (300, 200, 150), (2340, 2016, 1520)])
def test_lstsq(env, m, n, kf):
    torch, L, lib = env
    A = np.random.default_rng(m).standard_normal((2, n, m))
    dA = _dev(torch, A)
    L.check(lib.hss_batched_lstsq_device(L.ptr(dA), m, n, kf, 2, None))
    torch.cuda.synchronize()
    out = dA.cpu().numpy()
    for b in range(2):
        Am = A[b].T
        X = np.linalg.lstsq(Am[:, :kf], Am[:, kf:], rcond=None)[0]
        assert np.abs(X - out[b].T[:kf, kf:]).max() <= 1e-11 * np.abs(X).max()


@pytest.mark.parametrize("m,n,kf", [(40, 30, 20), (132, 64, 48), (300, 200, 150), (700, 240, 200),
                                    (2340, 2016, 1520)])
def test_lstsq_dfloat(env, m, n, kf):
    """The double-float least squares (hss_batched_lstsq_device_ex, HSS_PREC_DFLOAT): panels,
    trailing updates and back substitution in paired FP32.  Shapes cover one CTA per
    problem, the cluster panel (m > 256 with few problems), the row-split update (tall
    problems) and a last panel narrower than 32 columns.  The solution matches NumPy's to
    the double-float precision times the system's condition and the FP64 path's closely."""
    torch, L, lib = env
    r = np.random.default_rng(m + 1)
    A = r.standard_normal((3, n, m))
    A[2, :kf] *= np.logspace(0, -6, kf)[:, None]      # a graded (cond ~1e6) system
    out = {}
    for prec in (L.HSS_PREC_FP64, L.HSS_PREC_DFLOAT):
        dA = _dev(torch, A)
        L.check(lib.hss_batched_lstsq_device_ex(L.ptr(dA), m, n, kf, 3, prec, None))
        torch.cuda.synchronize()
        out[prec] = dA.cpu().numpy()
    worst = []
    for b in range(3):
        Am = A[b].T
        X = np.linalg.lstsq(Am[:, :kf], Am[:, kf:], rcond=None)[0]
        cond = np.linalg.cond(Am[:, :kf])
        X64 = out[L.HSS_PREC_FP64][b].T[:kf, kf:]
        Xdf = out[L.HSS_PREC_DFLOAT][b].T[:kf, kf:]
        e_np = np.abs(Xdf - X).max() / np.abs(X).max()
        e_64 = np.abs(Xdf - X64).max() / np.abs(X64).max()
        worst.append((e_np, e_64, cond))
        # ~2^-48 per operation, amplified by the condition of the skeleton columns
        assert e_np <= 2e-13 * max(1.0, cond) and e_64 <= 2e-13 * max(1.0, cond), (b, e_np, e_64, cond)
        # what the solution does: the residual of the normal equations is as small as FP64's
        res_df = np.linalg.norm(Am[:, :kf].T @ (Am[:, :kf] @ Xdf - Am[:, kf:]))
        res_64 = np.linalg.norm(Am[:, :kf].T @ (Am[:, :kf] @ X64 - Am[:, kf:]))
        scale = np.linalg.norm(Am[:, :kf]) ** 2 * np.linalg.norm(X) + 1e-300
        assert res_df / scale <= 1e-12 and res_64 / scale <= 1e-13
    print(f"double-float least squares {m}x{n} (kf={kf}): vs NumPy / FP64 path " +
          ", ".join(f"{a:.1e}/{b_:.1e} (cond {c:.0e})" for a, b_, c in worst))


def _id_gpu(env, A, acc, force=-1):
    torch, L, lib = env
    m, n = A.shape
    dA = _dev(torch, np.asfortranarray(A).T)
    rank = torch.zeros(1, dtype=torch.int32, device="cuda")
    perm = torch.zeros(n, dtype=torch.int32, device="cuda")
    T = torch.zeros(n * n, dtype=torch.float64, device="cuda")
    L.check(lib.hss_batched_id_device(L.ptr(dA), m, n, 1, acc, 0, force, L.ptr(rank), L.ptr(perm), L.ptr(T), None))
    torch.cuda.synchronize()
    k = int(rank.item())
    Tg = T.cpu().numpy()[:(n - k) * n].reshape(n - k, n).T[:k, :]
    return k, perm.cpu().numpy(), Tg


@pytest.mark.parametrize("rows,cols", [((300, 450), (0, 64)), ((64, 200), (0, 64)), ((100, 130), (60, 120))])
def test_id_matches_oracle(env, rows, cols):
    X = geometry.star_curve(1024)
    A = kernels.kernel_eval(X[rows[0]:rows[1]], X[cols[0]:cols[1]], kernels.KernelParams(flag=kernels.DL_L_2D))
    k, perm, Tg = _id_gpu(env, A, 1e-10)
    To, Io, ko, Ro = idecomp.id_adaptive(A, 1e-10, 0, 0)
    assert k == ko
    assert np.array_equal(perm[:k], Io[:k])
    # columns of T follow the residual order; compare by global column index
    cols_g = {c: i for i, c in enumerate(perm[k:])}
    Tal = np.stack([Tg[:, cols_g[c]] for c in Io[k:]], axis=1) if k < A.shape[1] else Tg
    err_g = np.linalg.norm(A[:, perm[:k]] @ Tg - A[:, perm[k:]]) / np.linalg.norm(A)
    assert err_g < 1e-9
    assert np.abs(Tal - To).max() <= 1e-6 * max(1.0, np.abs(To).max())
    kf = min(k + 4, min(A.shape))
    kf_, _, Tf = _id_gpu(env, A, 1e-10, kf)
    assert kf_ == kf
    err_f = np.linalg.norm(A[:, perm[:kf]] @ Tf - A[:, perm[kf:]]) / np.linalg.norm(A)
    assert err_f < 1e-9
