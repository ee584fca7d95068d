"""Kernel_Eval on the GPU (Common/Kernel_Eval.m) against the oracle: the Laplace kernel
and the complex Helmholtz / Lippmann-Schwinger kernel with its Duan-Rokhlin diagonal."""
import math

import numpy as np
import pytest

from oracle import drweights as OD
from oracle import geometry as OG
from oracle import kernels as OK

pytestmark = pytest.mark.gpu


def _points(Ng=8, npan=4, extra=37, seed=0):
    S = OG.grid_source(Ng, npan)
    rng = np.random.default_rng(seed)
    T = np.concatenate([S[rng.choice(len(S), 300, replace=False)], rng.uniform(-1.2, 1.2, (extra, 2))])
    return T, S


def _oracle_kernel(k):
    mod = lambda m: OK.Modulation(m.alpha, m.x0, m.y0, m.isig, m.kind)  # noqa: E731
    flag = {"SL_L_2D": OK.SL_L_2D, "SL_H_2D": OK.SL_H_2D}[k.flag_pot]
    return OK.KernelParams(flag=flag, h=k.h, b=mod(k.b), c=mod(k.c), kh=k.kh, dr=k.dr_weights)


def test_laplace_kernel_matches_oracle():
    from hssc_directsolver_gb300 import kernels as GK
    T, S = _points()
    h = 2.0 / 32
    for b, c in (OK.reference_modulations(0, 0, 0), OK.reference_modulations(1, 0, 0), (OK.Modulation(),) * 2):
        k = GK.Kernel("SL_L_2D", h, GK.Modulation(b.alpha, b.x0, b.y0, b.isig), GK.Modulation(c.alpha, c.x0, c.y0, c.isig))
        A = GK.Kernel_Eval(T, S, k)
        R = OK.kernel_eval(T, S, _oracle_kernel(k))
        assert A.dtype == np.float64 and A.shape == R.shape
        assert np.abs(A - R).max() <= 1e-15 * np.abs(R).max()


@pytest.mark.parametrize("sym,TI,order", [(0, 0, 4), (1, 0, 4), (0, 1, 4), (1, 1, 0), (0, 0, 6)])
def test_helmholtz_kernel_matches_oracle(sym, TI, order):
    from hssc_directsolver_gb300 import kernels as GK
    Ng, npan, kh = 8, 4, 8 * math.pi
    T, S = _points(Ng, npan)
    k = GK.helmholtz_kernel(kh, sym, Ng, npan, TI, order=order)
    if order == 4:
        c0, _ = OD.dr_corrections(k.h, kh)
        assert abs(k.dr_weights - c0) <= 1e-13 * abs(c0)
    else:
        assert k.dr_weights == 0
    A = GK.Kernel_Eval(T, S, k)
    R = OK.kernel_eval(T, S, _oracle_kernel(k))
    assert A.dtype == np.complex128 and A.shape == R.shape
    diag = np.zeros(A.shape, bool)
    for i, t in enumerate(T):
        j = np.nonzero((S[:, 0] == t[0]) & (S[:, 1] == t[1]))[0]
        diag[i, j] = True
    assert diag.sum() == 300
    # diagonal: w = 1 + kh^2 (i/4) dr, formed identically on both sides
    assert np.array_equal(A[diag], R[diag])
    q = kh * kh / 4
    w = complex(1 - q * k.dr_weights.imag, q * k.dr_weights.real)
    assert np.all(A[diag] == w)
    # off the diagonal: the library's H0 (series / Hankel integral) against SciPy's j0, y0
    off = ~diag
    err = np.abs(A[off] - R[off])
    assert err.max() <= 1e-14 * np.abs(R[off]).max()
    assert np.median(err / np.abs(R[off])) <= 1e-15
    # the Lippmann-Schwinger bump scales the rows (b) and columns (c) of the plain kernel
    plain = GK.Kernel_Eval(T, S, GK.Kernel("SL_H_2D", k.h, kh=kh, dr_weights=k.dr_weights))
    b = OK._modulation(_oracle_kernel(k).b, T[:, 0], T[:, 1], k.h)
    c = OK._modulation(_oracle_kernel(k).c, S[:, 0], S[:, 1], k.h)
    ratio = A[off] / plain[off]
    # 0.5 tanh(z) + 0.5 cancels in the bump's tail, so two tanh implementations (the host
    # library's and NumPy's) agree there only to ~1e-12 relative
    assert np.allclose(ratio, (b[:, None] * c[None, :])[off], rtol=1e-10, atol=0)


def test_kernel_eval_argument_errors():
    from hssc_directsolver_gb300 import _lib as L, kernels as GK
    T, S = _points()
    with pytest.raises(L.HSSError):
        GK.Kernel_Eval(T, S, GK.Kernel("DL_L_2D", 0.1))
    with pytest.raises(L.HSSError):
        GK.Kernel_Eval(T, S, GK.Kernel("SL_H_2D", 0.1, kh=0.0))
    with pytest.raises(L.HSSError):
        GK.Kernel_Eval(T, S, GK.Kernel("SL_H_2D", 0.1, kh=5.0, b=GK.Modulation(kind=7)))


def test_kernel_eval_device_matches_host_entry():
    import torch
    from hssc_directsolver_gb300 import _lib as L, kernels as GK
    T, S = _points()
    for k in (GK.Kernel("SL_L_2D", 2.0 / 32, GK.Modulation(0.25, 0.3, 0.6, 1.0)),
              GK.helmholtz_kernel(8 * math.pi, 0, 8, 4, 0)):
        A = GK.Kernel_Eval(T, S, k)
        d1 = torch.tensor(np.ascontiguousarray(T.T), device="cuda")
        d2 = torch.tensor(np.ascontiguousarray(S.T), device="cuda")
        cplx = k.flag_pot == "SL_H_2D"
        dA = torch.empty((2 if cplx else 1) * len(T) * len(S), dtype=torch.float64, device="cuda")
        kp = k.to_c()
        import ctypes as C
        L.check(L.lib().hss_kernel_eval_device(C.byref(kp), L.ptr(d1), len(T), L.ptr(d2), len(S), L.ptr(dA),
                                               C.c_void_p(torch.cuda.current_stream().cuda_stream)))
        got = dA.cpu().numpy()
        got = got.view(np.complex128).reshape(A.shape, order="F") if cplx else got.reshape(A.shape, order="F")
        assert np.array_equal(got, A)
