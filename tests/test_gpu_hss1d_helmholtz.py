"""The complex Helmholtz HSS1D on the GPU against the oracle (GPU).

Star curve r = 1 + 0.3 cos 5t, N = 1024, leaf 64, acc 1e-10, the SL_H_2D kernel with kh = 20,
h = 0.05, the DR diagonal weight 0.3 + 0.1i, and two different Gaussian modulations b and c, so
the matrix is neither Hermitian nor complex symmetric.  The proxy ring holds
min(max(50, round(4 kh 1.75 R + 30)), N) points (HSS1D_compress_nsym.m:111-114) and every ID is
complex (Common/ID.m:40-65 on complex blocks), run on the GPU as the pair-pivoted QR of the
real 2 x 2 embedding.  Checked: ranks, J and skeleton sets equal the oracle's in every box, T
close, the forward and inverse applies close to the oracle's, the refined solve, and the
kernel-matrix residual against NumPy's dense product.
"""
import numpy as np
import pytest

from oracle import geometry, hss1d as O1, kernels as OK

pytestmark = pytest.mark.gpu
N, LEAF, ACC, KH, H, DR = 1024, 64, 1e-10, 20.0, 0.05, 0.3 + 0.1j


def _kernels():
    from hssc_directsolver_gb300 import kernels as GK
    gb, gc = GK.Modulation(0.5, 0.3, 0.0, 2.0), GK.Modulation(-0.3, 0.0, -0.2, 3.0)
    ob, oc = OK.Modulation(0.5, 0.3, 0.0, 2.0), OK.Modulation(-0.3, 0.0, -0.2, 3.0)
    return (GK.Kernel("SL_H_2D", H, gb, gc, KH, DR),
            OK.KernelParams(flag=OK.SL_H_2D, h=H, b=ob, c=oc, kh=KH, dr=DR))


@pytest.fixture(scope="module")
def helm(gpu):
    from hssc_directsolver_gb300 import hss1d as G1
    X = geometry.star_curve(N)
    gk, ok = _kernels()
    Hg = G1.HSS1D_compress_nsym("green", X, LEAF, ACC, gk)
    Ho = O1.compress_nsym(X, LEAF, ACC, ok)
    return G1, X, ok, Hg, Ho


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def test_complex_ranks_skeletons_and_T(helm):
    G1, X, ok, Hg, Ho = helm
    assert Hg.complex and Hg.N == N
    inf = Hg.info()
    assert np.array_equal(inf["kskel"][1:], np.array(Ho.kskel[1:]))
    assert np.array_equal(inf["nskel"][1:], np.array(Ho.nskel[1:]))
    nei = O1.neighbor_list(X, Ho.tree)
    worst, worst_act = 0.0, 0.0
    for b in range(1, inf["nboxes"]):
        e = Hg.export_box(b)
        k = Ho.kskel[b]
        assert np.array_equal(e["I_SKUP"], Ho.I_SKUP[b]) and np.array_equal(e["I_SKDN"], Ho.I_SKDN[b]), b
        _, _, A_out, A_in = O1.compress_green_blocks(Ho, X, b, nei, ok, N)
        for side, J, A in (("T_UP", "J_UP", A_out), ("T_DN", "J_DN", A_in.T)):
            Jo = getattr(Ho, J)[b]
            assert np.array_equal(e[J][:k], Jo[:k]), b
            To = getattr(Ho, side)[b]
            if To.size:
                # the pivoted QR runs on past the rank, where trailing norms tie at rounding
                # level: compare T column by residual point
                pos = {c: i for i, c in enumerate(e[J][k:])}
                Tg = np.stack([e[side][:, pos[c]] for c in Jo[k:]], axis=1)
                worst = max(worst, np.abs(Tg - To).max() / max(1.0, np.abs(To).max()))
                # what T does: the interpolation of the block's residual columns
                act = np.linalg.norm(A[:, Jo[:k]] @ (Tg - To)) / np.linalg.norm(A[:, Jo[k:]])
                worst_act = max(worst_act, act)
    print(f"complex HSS1D N={N}: ranks {list(inf['kskel'][1:7])}..., T within {worst:.2e} of the oracle's "
          f"entries (R11 of condition up to 1/acc), {worst_act:.2e} in action")
    # measured 2.1e-6 (entries), the condition of R11 (|R_kk| ~ acc |R_11|) times rounding
    assert worst <= 1e-5 and worst_act <= 1e-13
    # the Helmholtz proxy ring: 4 kh 1.75 R + 30 points exceed the Laplace 50 near the root
    assert max(c[0] for c in Ho.census[1:3]) > 200


def test_complex_applies_match_oracle(helm):
    G1, X, ok, Hg, Ho = helm
    r = np.random.default_rng(7)
    q = r.standard_normal((N, 3)) + 1j * r.standard_normal((N, 3))
    u = G1.HSS1D_apply_nsym(Hg, q)
    uo = O1.apply_nsym(Ho, q)
    K = OK.kernel_eval(X, X, ok)
    da, dk = _rel(u, uo), _rel(u, K @ q)
    G1.HSS1D_invert_nsym(Hg)
    x = G1.HSS1D_applyinv_nsym(Hg, None, None, u)
    xo = O1.applyinv_nsym(Ho, O1.invert_nsym(Ho), uo)
    di, rt = _rel(x, xo), _rel(x, q)
    print(f"complex HSS1D: apply {da:.2e} (vs K {dk:.2e}), inverse apply {di:.2e}, round trip {rt:.2e}")
    assert da <= 1e-12 and dk <= 1e-9
    assert di <= 1e-11 and rt <= 1e-11
    v = G1.HSS1D_apply_nsym(Hg, q[:, 0])                # one complex vector
    assert v.shape == (N,) and np.iscomplexobj(v) and _rel(v, uo[:, 0]) <= 1e-12


def test_complex_solve_and_kernel_residual(helm):
    G1, X, ok, Hg, Ho = helm
    G1.HSS1D_invert_nsym(Hg)
    r = np.random.default_rng(8)
    f = r.standard_normal((N, 2)) + 1j * r.standard_normal((N, 2))
    x, relres, it = G1.HSS1D_solve(Hg, f, 1e-12, 4)
    K = OK.kernel_eval(X, X, ok)
    rk = G1.HSS1D_kernel_residual(Hg, f, x)
    dense = max(np.linalg.norm(f[:, c] - K @ x[:, c]) / np.linalg.norm(f[:, c]) for c in range(2))
    print(f"complex HSS1D solve: relres {relres:.2e} in {it} inverse applies; kernel residual {rk:.3e} "
          f"(NumPy {dense:.3e})")
    assert relres <= 1e-12
    assert abs(rk - dense) <= 1e-3 * dense + 1e-15 and rk <= 1e-9
    Kinv = G1.HSS1D_transforminv_nsym(Hg)            # the inverse in compressed form, complex too
    assert Kinv.complex
    assert _rel(G1.HSS1D_apply_nsym(Kinv, f), np.linalg.solve(K, f)) <= 1e-9


def test_complex_forest_matches_single_curves(gpu):
    """Two complex curves of different size in one forest: each equals its own compress."""
    from hssc_directsolver_gb300 import hss1d as G1
    gk, ok = _kernels()
    Xs = [geometry.star_curve(512), geometry.star_curve(768, eps=0.2, m=3)]
    F = G1.HSS1D_compress_batch(Xs, LEAF, ACC, gk, seeds=[0, 0])
    assert F.complex
    roots, base = G1.forest_info(F)
    kF = F.info()["kskel"]
    r = np.random.default_rng(9)
    q = r.standard_normal(1280) + 1j * r.standard_normal(1280)
    u = G1.HSS1D_apply_nsym(F, q)
    for p, X in enumerate(Xs):
        Ho = O1.compress_nsym(X, LEAF, ACC, ok)
        nb = len(Ho.kskel)
        assert np.array_equal(kF[roots[p] + 1:roots[p] + nb], np.array(Ho.kskel[1:]))
        s = slice(int(base[p]), int(base[p]) + X.shape[0])
        assert _rel(u[s], O1.apply_nsym(Ho, q[s])) <= 1e-12


def test_complex_symmetric_fsym(gpu):
    """HSS1D_compress_fsym on a complex symmetric matrix (b = c, so K.' = K): one complex ID
    per box, T_DN = T_UP and M_SIB{c2} = M_SIB{c1}.' (plain transposes,
    HSS1D_compress_fsym.m:186-198, :245).  Ranks and skeletons equal the oracle's; the applies
    match it and the dense matrix."""
    from hssc_directsolver_gb300 import hss1d as G1, kernels as GK
    gb, ob = GK.Modulation(0.5, 0.3, 0.0, 2.0), OK.Modulation(0.5, 0.3, 0.0, 2.0)
    gk = GK.Kernel("SL_H_2D", H, gb, gb, KH, DR)
    ok = OK.KernelParams(flag=OK.SL_H_2D, h=H, b=ob, c=ob, kh=KH, dr=DR)
    X = geometry.star_curve(768)
    K = OK.kernel_eval(X, X, ok)
    assert np.abs(K - K.T).max() <= 1e-15 * np.abs(K).max()
    Hg = G1.HSS1D_compress_fsym("green", X, LEAF, ACC, gk)
    Ho = O1.compress_fsym(X, LEAF, ACC, ok)
    assert Hg.complex
    assert np.array_equal(Hg.info()["kskel"][1:], np.array(Ho.kskel[1:]))
    for b in range(1, len(Ho.kskel)):
        e = Hg.export_box(b)
        assert np.array_equal(e["I_SKUP"], Ho.I_SKUP[b]) and np.array_equal(e["I_SKDN"], Ho.I_SKUP[b]), b
        assert np.array_equal(e["T_UP"], e["T_DN"]), b
    r = np.random.default_rng(10)
    q = r.standard_normal((768, 2)) + 1j * r.standard_normal((768, 2))
    u = G1.HSS1D_apply_nsym(Hg, q)
    assert _rel(u, O1.apply_nsym(Ho, q)) <= 1e-12 and _rel(u, K @ q) <= 1e-9
    G1.HSS1D_invert_nsym(Hg)
    x = G1.HSS1D_applyinv_nsym(Hg, None, None, u)
    assert _rel(x, O1.applyinv_nsym(Ho, O1.invert_nsym(Ho), u)) <= 1e-11 and _rel(x, q) <= 1e-11
