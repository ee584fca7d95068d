"""HSS1D on the GPU against the oracle and the golden fixture (GPU)."""
import os

import numpy as np
import pytest

from oracle import geometry, hss1d as O1, hss2d as O2, idecomp, kernels as OK

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def star(gpu):
    from hssc_directsolver_gb300 import hss1d as G1, kernels as GK
    g = np.load(os.path.join(GOLD, "hss1d_star4096.npz"))
    X = geometry.star_curve(int(g["N"]))
    H = G1.HSS1D_compress_nsym("green", X, int(g["leaf"]), float(g["acc"]), GK.Kernel("DL_L_2D"))
    Ho = O1.compress_nsym(X, int(g["leaf"]), float(g["acc"]), OK.KernelParams(flag=OK.DL_L_2D))
    return G1, g, X, H, Ho


def test_ranks_and_skeletons_exact(star):
    G1, g, X, H, Ho = star
    inf = H.info()
    assert np.array_equal(inf["kskel"], g["kskel"])
    nb = inf["nboxes"]
    up = np.concatenate([H.export_box(b)["I_SKUP"] for b in range(1, nb)])
    dn = np.concatenate([H.export_box(b)["I_SKDN"] for b in range(1, nb)])
    assert np.array_equal(up, g["I_SKUP"]) and np.array_equal(dn, g["I_SKDN"])
    for b in (1, 2, nb - 1):
        e = H.export_box(b)
        k = Ho.kskel[b]
        assert np.array_equal(e["J_UP"][:k], Ho.J_UP[b][:k])
        if e["T_UP"].size:
            # residual columns past the rank may be ordered differently (their norms tie at
            # rounding level); compare the interpolation coefficients column by residual point
            pos = {c: i for i, c in enumerate(e["J_UP"][k:])}
            Tg = np.stack([e["T_UP"][:, pos[c]] for c in Ho.J_UP[b][k:]], axis=1)
            assert np.abs(Tg - Ho.T_UP[b]).max() <= 1e-6 * max(1, np.abs(Ho.T_UP[b]).max())


def test_apply_matches_oracle(star):
    G1, g, X, H, Ho = star
    q = np.random.default_rng(5).standard_normal((X.shape[0], 3))
    u = G1.HSS1D_apply_nsym(H, q)
    uo = O1.apply_nsym(Ho, q)
    assert np.linalg.norm(u - uo) <= 1e-12 * np.linalg.norm(uo)


def test_applyinv_matches_oracle_1e12(star):
    G1, g, X, H, Ho = star
    G1.HSS1D_invert_nsym(H)
    x = G1.HSS1D_applyinv_nsym(H, None, None, g["f"])
    assert np.linalg.norm(x - g["x"]) <= 1e-12 * np.linalg.norm(g["x"])
    A = OK.kernel_eval(X, X, OK.KernelParams(flag=OK.DL_L_2D))
    assert np.linalg.norm(A @ x - g["f"]) / np.linalg.norm(g["f"]) < 1e-10
    F = np.random.default_rng(6).standard_normal((X.shape[0], 11))   # more than one 8-column chunk
    Y = G1.HSS1D_applyinv_nsym(H, None, None, F)
    Yo = O1.applyinv_nsym(Ho, O1.invert_nsym(Ho), F)
    assert np.linalg.norm(Y - Yo) <= 1e-12 * np.linalg.norm(Yo)


def test_reference_test_geometry(gpu):
    """Run_HSS1D_tests.m parameters: Laplace SL on the 2-layer skeleton of box 2 (Ng=7, np=16)."""
    from hssc_directsolver_gb300 import hss1d as G1, kernels as GK
    Ng, npan = 7, 16
    h = 2.0 / (Ng * npan)
    b, c = OK.reference_modulations(sym=0, proxy=1, transinv=0)
    kp = OK.KernelParams(flag=OK.SL_L_2D, h=h, b=b, c=c)
    prm = O2.HSS2DParams(Ng=Ng, npan=npan, kp=kp)
    X = prm.X_source()[O2.build_tree_nsym(prm, with_T=False).I_sk[1]]
    gk = GK.Kernel("SL_L_2D", h, GK.Modulation(b.alpha, b.x0, b.y0, b.isig), GK.Modulation(c.alpha, c.x0, c.y0, c.isig))
    H = G1.HSS1D_compress_nsym("green", X, 56, 1e-10, gk)
    Ho = O1.compress_nsym(X, 56, 1e-10, kp)
    inf = H.info()
    assert np.array_equal(inf["kskel"][1:], np.array(Ho.kskel[1:]))
    G1.HSS1D_invert_nsym(H)
    q = np.random.default_rng(0).standard_normal((X.shape[0], 10))
    A = OK.kernel_eval(X, X, kp)
    y = G1.HSS1D_applyinv_nsym(H, None, None, q)
    yd = np.linalg.solve(A, q)
    assert np.linalg.norm(y - yd) / np.linalg.norm(yd) < 1e-8       # INSTALL.txt criterion
    yo = O1.applyinv_nsym(Ho, O1.invert_nsym(Ho), q)
    assert np.linalg.norm(y - yo) <= 1e-12 * np.linalg.norm(yo)


def test_errors_are_status_codes(gpu):
    from hssc_directsolver_gb300 import hss1d as G1, kernels as GK, _lib as L
    X = geometry.star_curve(256)
    with pytest.raises(L.HSSError) as e:
        G1.HSS1D_compress_nsym("green", X, 64, 2.0, GK.Kernel("DL_L_2D"))
    assert e.value.code == L.HSS_ERR_ARG
    H = G1.HSS1D_compress_nsym("green", X, 64, 1e-10, GK.Kernel("DL_L_2D"))
    with pytest.raises(L.HSSError) as e:
        G1.HSS1D_applyinv_nsym(H, None, None, np.ones(256))
    assert e.value.code == L.HSS_ERR_STATE


def test_batched_forest_matches_per_problem_oracle(gpu):
    """Many curves of uneven N in one forest: every tree equals the oracle run on its own
    (ranks exact, inverse apply <= 1e-12), with per-problem rank-check seeds."""
    from hssc_directsolver_gb300 import hss1d as G1, kernels as GK, geometry as GG
    Xs, sizes = GG.batched_curves(5, nmin=600, nmax=3000, seed=3)
    H = G1.HSS1D_compress_batch(Xs, 64, 1e-10, GK.Kernel("DL_L_2D"), seeds=[11 * p for p in range(5)])
    roots, base = G1.forest_info(H)
    assert list(np.diff(base)) == sizes[:-1]
    inf = H.info()
    G1.HSS1D_invert_nsym(H)
    F = np.random.default_rng(4).standard_normal((sum(sizes), 2))
    X = G1.HSS1D_applyinv_nsym(H, None, None, F)
    U = G1.HSS1D_apply_nsym(H, F)
    for p, Xp in enumerate(Xs):
        Ho = O1.compress_nsym(Xp, 64, 1e-10, OK.KernelParams(flag=OK.DL_L_2D), seed=11 * p)
        nb = Ho.tree.nboxes
        kg = inf["kskel"][roots[p] + 1:roots[p] + nb]
        assert np.array_equal(kg, np.array(Ho.kskel[1:]))
        sl = slice(base[p], base[p] + sizes[p])
        xo = O1.applyinv_nsym(Ho, O1.invert_nsym(Ho), F[sl])
        assert np.linalg.norm(X[sl] - xo) <= 1e-12 * np.linalg.norm(xo)
        uo = O1.apply_nsym(Ho, F[sl])
        assert np.linalg.norm(U[sl] - uo) <= 1e-12 * np.linalg.norm(uo)


def test_refined_solve_reaches_tolerance(gpu):
    from hssc_directsolver_gb300 import hss1d as G1, kernels as GK, geometry as GG
    Xs, sizes = GG.batched_curves(6, nmin=800, nmax=2500, seed=7)
    H = G1.HSS1D_compress_batch(Xs, 64, 1e-10, GK.Kernel("DL_L_2D"))
    G1.HSS1D_invert_nsym(H)
    F = np.random.default_rng(1).standard_normal((sum(sizes), 3))
    x, rr, it = G1.HSS1D_solve(H, F, 1e-13, 4)
    assert rr <= 1e-13 and 1 <= it <= 4
    r = F - G1.HSS1D_apply_nsym(H, x)
    assert np.linalg.norm(r, axis=0).max() / np.linalg.norm(F, axis=0).min() < 1e-12


def test_transforminv_matches_oracle(star):
    """Kinv_HSS = HSS1D_transforminv_nsym: its forward apply equals the oracle's transformed
    inverse and the inverse apply; its J/T rows match the oracle's."""
    G1, g, X, H, Ho = star
    G1.HSS1D_invert_nsym(H)
    Ki = G1.HSS1D_transforminv_nsym(H, None, None)
    inv = O1.invert_nsym(Ho)
    Ko = O1.transforminv_nsym(Ho, inv)
    F = np.random.default_rng(9).standard_normal((X.shape[0], 3))
    y = G1.HSS1D_apply_nsym(Ki, F)
    yo = O1.apply_nsym(Ko, F)
    assert np.linalg.norm(y - yo) <= 1e-10 * np.linalg.norm(yo)
    x = G1.HSS1D_applyinv_nsym(H, None, None, F)
    assert np.linalg.norm(y - x) <= 1e-10 * np.linalg.norm(x)
    for b in (1, 2, H.info()["nboxes"] - 1):
        e = Ki.export_box(b)
        k = Ho.kskel[b]
        assert np.array_equal(e["J_UP"][:k], Ho.J_DN[b][:k]) and np.array_equal(e["J_DN"][:k], Ho.J_UP[b][:k])
        if e["T_UP"].size:
            pos = {c: i for i, c in enumerate(e["J_UP"][k:])}
            Tg = np.stack([e["T_UP"][:, pos[c]] for c in Ko.J_UP[b][k:]], axis=1)
            # P and Q inverses amplify rounding (cond ~1e6 here): entries agree to ~1e-6
            assert np.abs(Tg - Ko.T_UP[b]).max() <= 1e-5 * max(1.0, np.abs(Ko.T_UP[b]).max())


def test_transforminv_forest(gpu):
    from hssc_directsolver_gb300 import hss1d as G1, kernels as GK, geometry as GG
    Xs, sizes = GG.batched_curves(4, nmin=700, nmax=2500, seed=12)
    H = G1.HSS1D_compress_batch(Xs, 64, 1e-10, GK.Kernel("DL_L_2D"))
    G1.HSS1D_invert_nsym(H)
    Ki = G1.HSS1D_transforminv_nsym(H)
    F = np.random.default_rng(2).standard_normal((sum(sizes), 2))
    x = G1.HSS1D_applyinv_nsym(H, None, None, F)
    assert np.linalg.norm(G1.HSS1D_apply_nsym(Ki, F) - x) <= 1e-10 * np.linalg.norm(x)


def test_fsym_matches_oracle(gpu):
    """HSS1D_compress_fsym on the symmetric reference geometry: ranks and skeletons equal
    the oracle's, inverse apply within 1e-12 of it and 1e-8 of the dense solve."""
    from hssc_directsolver_gb300 import hss1d as G1, kernels as GK
    Ng, npan = 7, 16
    h = 2.0 / (Ng * npan)
    b, c = OK.reference_modulations(sym=1, proxy=0, transinv=0)
    kp = OK.KernelParams(flag=OK.SL_L_2D, h=h, b=b, c=c)
    prm = O2.HSS2DParams(Ng=Ng, npan=npan, kp=kp)
    X = prm.X_source()[O2.build_tree_nsym(prm, with_T=False).I_sk[1]]
    gk = GK.Kernel("SL_L_2D", h, GK.Modulation(b.alpha, b.x0, b.y0, b.isig), GK.Modulation(c.alpha, c.x0, c.y0, c.isig))
    H = G1.HSS1D_compress_fsym("green", X, 56, 1e-10, gk)
    Ho = O1.compress_fsym(X, 56, 1e-10, kp)
    inf = H.info()
    assert np.array_equal(inf["kskel"][1:], np.array(Ho.kskel[1:]))
    for bx in range(1, inf["nboxes"]):
        e = H.export_box(bx)
        assert np.array_equal(e["I_SKUP"], Ho.I_SKUP[bx]) and np.array_equal(e["I_SKDN"], Ho.I_SKUP[bx])
    G1.HSS1D_invert_fsym(H)
    q = np.random.default_rng(0).standard_normal((X.shape[0], 5))
    y = G1.HSS1D_applyinv_fsym(H, None, None, q)
    yo = O1.applyinv_nsym(Ho, O1.invert_nsym(Ho), q)
    assert np.linalg.norm(y - yo) <= 1e-12 * np.linalg.norm(yo)
    A = OK.kernel_eval(X, X, kp)
    assert np.linalg.norm(y - np.linalg.solve(A, q)) < 1e-8 * np.linalg.norm(yo)
    u = G1.HSS1D_apply_fsym(H, q)
    assert np.linalg.norm(u - O1.apply_nsym(Ho, q)) <= 1e-12 * np.linalg.norm(u)


def test_dfloat_forest_solve(gpu):
    """Double-float solve products on a forest: inverse and forward applies agree with FP64
    to ~1e-12, and the refined solve reaches 1e-12."""
    from hssc_directsolver_gb300 import hss1d as G1, kernels as GK, geometry as GG
    Xs, sizes = GG.batched_curves(5, nmin=800, nmax=3000, seed=17)
    H = G1.HSS1D_compress_batch(Xs, 64, 1e-10, GK.Kernel("DL_L_2D"))
    G1.HSS1D_invert_nsym(H)
    F = np.random.default_rng(2).standard_normal((sum(sizes), 11))
    x64 = G1.HSS1D_applyinv_nsym(H, None, None, F)
    u64 = G1.HSS1D_apply_nsym(H, F)
    H.set_precision("dfloat")
    xdf = G1.HSS1D_applyinv_nsym(H, None, None, F)
    udf = G1.HSS1D_apply_nsym(H, F)
    assert np.linalg.norm(xdf - x64) <= 1e-12 * np.linalg.norm(x64)
    assert np.linalg.norm(udf - u64) <= 1e-13 * np.linalg.norm(u64)
    x, rr, it = G1.HSS1D_solve(H, F[:, :3], 1e-12, 4)
    assert rr <= 1e-12


def test_fsym_transforminv_and_precision_errors(gpu):
    from hssc_directsolver_gb300 import hss1d as G1, kernels as GK, _lib as L
    X = geometry.star_curve(1500)
    H = G1.HSS1D_compress_fsym("green", X, 64, 1e-10, GK.Kernel("SL_L_2D", 0.01))
    G1.HSS1D_invert_fsym(H)
    K = G1.HSS1D_transforminv_nsym(H)
    f = np.random.default_rng(1).standard_normal((1500, 2))
    x = G1.HSS1D_applyinv_fsym(H, None, None, f)
    assert np.linalg.norm(G1.HSS1D_apply_nsym(K, f) - x) <= 1e-10 * np.linalg.norm(x)
    with pytest.raises(L.HSSError) as e:
        L.check(L.lib().hss1d_set_precision(H._h, L.HSS_PREC_MIXED))
    assert e.value.code == L.HSS_ERR_ARG


def test_dfloat_inv_forest(gpu):
    """HSS_PREC_DFLOAT_INV: the inversion's updates and products in double-float; the
    refined solve reaches 1e-10 and matches the FP64 inverse apply to 1e-9."""
    from hssc_directsolver_gb300 import hss1d as G1, kernels as GK, geometry as GG
    Xs, sizes = GG.batched_curves(4, nmin=800, nmax=3000, seed=19)
    H64 = G1.HSS1D_compress_batch(Xs, 64, 1e-10, GK.Kernel("DL_L_2D"))
    G1.HSS1D_invert_nsym(H64)
    H = G1.HSS1D_compress_batch(Xs, 64, 1e-10, GK.Kernel("DL_L_2D"))
    H.set_precision("dfloat_inv")
    G1.HSS1D_invert_nsym(H)
    F = np.random.default_rng(6).standard_normal((sum(sizes), 3))
    x64 = G1.HSS1D_applyinv_nsym(H64, None, None, F)
    x, rr, it = G1.HSS1D_solve(H, F, 1e-10, 4)
    assert rr <= 1e-10
    assert np.linalg.norm(x - x64) <= 1e-9 * np.linalg.norm(x64)


def test_dense_matrix_transpose_scalarmult(star):
    """HSS1D_dense_matrix / HSS1D_transpose / HSS1D_scalarmult against the oracle's
    telescoping restatements (HSS1D/HSS1D_dense_matrix.m, HSS1D_transpose.m,
    HSS1D_scalarmult.m)."""
    G1, g, X, H, Ho = star
    N = X.shape[0]
    Kd = G1.HSS1D_dense_matrix(H)
    Kdo = O1.dense_matrix(Ho)
    scale = np.abs(Kdo).max()
    assert Kd.shape == (N, N)
    assert np.abs(Kd - Kdo).max() <= 1e-12 * scale
    # the compressed matrix is the kernel matrix to the compression tolerance
    A = OK.kernel_eval(X, X, OK.KernelParams(flag=OK.DL_L_2D))
    assert np.abs(Kd - A).max() <= 1e-9 * np.abs(A).max()
    # transpose: a new handle whose apply and dense form are A^T
    At = G1.HSS1D_transpose(H)
    q = np.random.default_rng(11).standard_normal((N, 3))
    assert np.linalg.norm(G1.HSS1D_apply_nsym(At, q) - Kd.T @ q) <= 1e-13 * np.linalg.norm(Kd.T @ q)
    assert np.linalg.norm(G1.HSS1D_apply_nsym(At, q) - O1.apply_nsym(O1.transpose(Ho), q)) <= 1e-12 * np.linalg.norm(q)
    assert np.abs(G1.HSS1D_dense_matrix(At) - Kd.T).max() <= 1e-14 * scale
    # the transpose inverts and solves like the dense transpose
    G1.HSS1D_invert_nsym(At)
    f = np.random.default_rng(12).standard_normal(N)
    x = G1.HSS1D_applyinv_nsym(At, None, None, f)
    assert np.linalg.norm(Kd.T @ x - f) <= 1e-11 * np.linalg.norm(f)
    # scalar multiple (in place; the inverse is dropped until re-inverted)
    G1.HSS1D_invert_nsym(At)
    G1.HSS1D_scalarmult(-2.5, At)
    assert np.linalg.norm(G1.HSS1D_apply_nsym(At, q) + 2.5 * (Kd.T @ q)) <= 1e-13 * np.linalg.norm(Kd.T @ q)
    from hssc_directsolver_gb300 import _lib
    with pytest.raises(_lib.HSSError):
        G1.HSS1D_applyinv_nsym(At, None, None, f)
    G1.HSS1D_invert_nsym(At)
    x2 = G1.HSS1D_applyinv_nsym(At, None, None, f)
    assert np.linalg.norm(x2 + x / 2.5) <= 1e-11 * np.linalg.norm(x)
    out = np.zeros(4)
    assert _lib.lib().hss1d_dense_matrix(H._h, 3, _lib.ptr(out)) == _lib.HSS_ERR_ARG


def test_dense_matrix_of_a_forest_problem(gpu):
    from hssc_directsolver_gb300 import hss1d as G1, kernels as GK
    rng = np.random.default_rng(3)
    curves = [geometry.fourier_curve(n, rng.uniform(0, 0.3 / np.arange(1, 5)), rng.uniform(0, 2 * np.pi, 4))
              for n in (700, 1300)]
    F = G1.HSS1D_compress_batch(curves, 64, 1e-10, GK.Kernel("DL_L_2D"))
    for p, X in enumerate(curves):
        Hs = G1.HSS1D_compress_nsym("green", X, 64, 1e-10, GK.Kernel("DL_L_2D"))
        Kf = G1.HSS1D_dense_matrix(F, prob=p)
        Ks = G1.HSS1D_dense_matrix(Hs)
        assert Kf.shape == (X.shape[0], X.shape[0])
        assert np.abs(Kf - Ks).max() <= 1e-12 * np.abs(Ks).max()


def test_apply_submatrix(star):
    """HSS1D_apply_submatrix_nsym / _boxes (HSS1D/HSS1D_apply_submatrix_*.m) against the
    oracle: K(I_dn, I_up) qq(I_up) through the dense form, and the box masks."""
    G1, g, X, H, Ho = star
    N = X.shape[0]
    rng = np.random.default_rng(21)
    I_dn = np.zeros(N, bool)
    I_dn[100:900] = True
    I_dn[rng.choice(N, 200, replace=False)] = True
    I_up = np.zeros(N, bool)
    I_up[2000:3100] = True
    q = rng.standard_normal((N, 2))
    bd, bu = G1.HSS1D_apply_submatrix_boxes(H, I_dn, I_up)
    bdo, buo = O1.apply_submatrix_boxes(Ho.tree, I_dn, I_up)
    assert np.array_equal(bd, bdo) and np.array_equal(bu, buo)
    uu = G1.HSS1D_apply_submatrix_nsym(H, bd, bu, I_dn, I_up, q)
    ref = O1.apply_submatrix(Ho, I_dn, I_up, q)
    assert uu.shape == (I_dn.sum(), 2)
    assert np.linalg.norm(uu - ref) <= 1e-12 * np.linalg.norm(ref)


@pytest.mark.parametrize("N,leaf", [(50, 64), (64, 64), (65, 64), (129, 32), (1000, 17)])
def test_small_and_ragged_trees(gpu, N, leaf):
    """N <= leaf (no split: rejected with HSS_ERR_ARG, a dense solve needs no HSS form), the
    first split (65 = 33 + 32), a split into uneven halves and an odd leaf size, FP64 and
    double-float: the solve against the dense kernel matrix and the oracle's ranks."""
    from hssc_directsolver_gb300 import hss1d as G1, kernels as GK, _lib as L
    X = geometry.star_curve(N)
    kp = OK.KernelParams(flag=OK.DL_L_2D)
    if N <= leaf:
        with pytest.raises(L.HSSError) as e:
            G1.HSS1D_compress_nsym("green", X, leaf, 1e-10, GK.Kernel("DL_L_2D"))
        assert e.value.code == L.HSS_ERR_ARG
        return
    H = G1.HSS1D_compress_nsym("green", X, leaf, 1e-10, GK.Kernel("DL_L_2D"))
    Ho = O1.compress_nsym(X, leaf, 1e-10, kp)
    assert np.array_equal(H.info()["kskel"][1:], np.array(Ho.kskel[1:], dtype=np.int32))
    G1.HSS1D_invert_nsym(H)
    A = OK.kernel_eval(X, X, kp)
    f = np.random.default_rng(N).standard_normal((N, 3))
    for prec in ("fp64", "dfloat"):
        H.set_precision(prec)
        x, rr, it = G1.HSS1D_solve(H, f, 1e-12, 4)
        assert rr <= 1e-12
        assert np.linalg.norm(A @ x - f) <= 1e-9 * np.linalg.norm(f)


def test_dfloat_id_compress(gpu):
    """The IDs' pivoted QR in double-float arithmetic: ranks as the FP64 ID (ties in the
    pivot order may move a rank by one in a few boxes), the same compression accuracy and
    a solve to 1e-12 against the FP64-compressed operator's dense form."""
    from hssc_directsolver_gb300 import hss1d as G1, kernels as GK, geometry as GG
    Xs, sizes = GG.batched_curves(16, nmin=1024, nmax=4096, seed=4)
    k = GK.Kernel("DL_L_2D")
    A = G1.HSS1D_compress_batch(Xs, 64, 1e-10, k)
    B = G1.HSS1D_compress_batch(Xs, 64, 1e-10, k, id_precision="dfloat")
    ka, kb = A.info()["kskel"], B.info()["kskel"]
    assert (ka == kb).mean() >= 0.98 and np.abs(ka - kb).max() <= 2
    for p in (0, 7):
        X = Xs[p]
        Kx = OK.kernel_eval(X, X, OK.KernelParams(flag=OK.DL_L_2D))
        Kb = G1.HSS1D_dense_matrix(B, prob=p)
        assert np.abs(Kb - Kx).max() <= 1e-9 * np.abs(Kx).max()
    G1.HSS1D_invert_nsym(B)
    f = np.random.default_rng(2).standard_normal((sum(sizes), 2))
    x, rr, it = G1.HSS1D_solve(B, f, 1e-12, 4)
    assert rr <= 1e-12
    with pytest.raises(ValueError):
        G1.HSS1D_compress_batch(Xs[:1], 64, 1e-10, k, id_precision="fp32")


def _outer_star(M, s):
    P = geometry.star_curve(M).copy()
    P[:, :2] *= s
    P[:, 4] *= s
    P[:, 5] /= s
    return P


def _rect_parity(G1, H, Ho, Xin, Xout, kpo, nrhs=11, tol=1e-9):
    """Trees, ranks and skeletons equal the oracle's; the apply equals the oracle's to 1e-12
    and the dense K(Xin, Xout) to the compression tolerance."""
    inf, ri = H.info(), H.rect_info()
    nb = inf["nboxes"]
    assert ri["M"] == Xin.shape[0]
    assert np.array_equal(ri["off_in"], Ho.off_in) and np.array_equal(ri["cnt_in"], Ho.cnt_in)
    assert np.array_equal(inf["kskel"][1:], Ho.kskel[1:])
    assert np.array_equal(ri["kskel_in"][1:], Ho.kskel_in[1:])
    for b in range(1, nb):
        e = H.export_box(b)
        assert np.array_equal(e["I_SKUP"], Ho.I_SKUP[b]) and np.array_equal(e["I_SKDN"], Ho.I_SKDN[b])
    q = np.random.default_rng(3).standard_normal((Xout.shape[0], nrhs))   # more than one 8-column chunk
    u = G1.HSS1D_apply_rect_nsym(H, q)
    uo = O1.apply_rect_nsym(Ho, q)
    assert u.shape == (Xin.shape[0], nrhs)
    assert np.linalg.norm(u - uo) <= 1e-12 * np.linalg.norm(uo)
    K = OK.kernel_eval(Xin, Xout, kpo)
    assert np.linalg.norm(u - K @ q) <= tol * np.linalg.norm(K @ q)
    return u, q


@pytest.mark.parametrize("N,M,leaf,s", [(1500, 1100, 64, 1.2), (700, 1000, 50, 0.85)])
def test_rect_compress_apply_matches_oracle(gpu, N, M, leaf, s):
    """HSS1D_compress_rectangular_nsym + HSS1D_apply_rect_nsym on two curves (M < N and
    M > N); the double-float apply agrees with the FP64 one; square-only calls refuse."""
    from hssc_directsolver_gb300 import hss1d as G1, kernels as GK
    Xout, Xin = geometry.star_curve(N), _outer_star(M, s)
    kpo = OK.KernelParams(flag=OK.DL_L_2D)
    H = G1.HSS1D_compress_rectangular_nsym("green", Xin, Xout, leaf, 1e-10, GK.Kernel("DL_L_2D"))
    Ho = O1.compress_rectangular_nsym(Xin, Xout, leaf, 1e-10, kpo)
    u, q = _rect_parity(G1, H, Ho, Xin, Xout, kpo)
    H.set_precision("dfloat")
    ud = G1.HSS1D_apply_rect_nsym(H, q)
    assert np.linalg.norm(ud - u) <= 1e-12 * np.linalg.norm(u)
    for call in (lambda: G1.HSS1D_invert_nsym(H), lambda: G1.HSS1D_transpose(H),
                 lambda: G1.HSS1D_dense_matrix(H)):
        with pytest.raises(Exception):
            call()


def test_rect_reference_call_site(gpu):
    """The reference's use (interpolation_operator_HSS.m:64): K(X_proxy, X1) between a level-1
    box's proxy layers and its skeleton (Ng=8, np=16, SL_L_2D), nbox_max 108, acc/10."""
    from hssc_directsolver_gb300 import hss1d as G1, kernels as GK
    Ng, npan = 8, 16
    h = 2.0 / (Ng * npan)
    b, c = OK.reference_modulations(sym=0, proxy=1, transinv=0)
    kp = OK.KernelParams(flag=OK.SL_L_2D, h=h, b=b, c=c)
    prm = O2.HSS2DParams(Ng=Ng, npan=npan, kp=kp)
    tree = O2.build_tree_nsym(prm, with_T=False)
    X1 = prm.X_source()[tree.I_sk[1]]
    colrad, rowrad = O2.box_radii(1)
    Xp = O2.build_box_proxy(tree.cent[1], colrad, rowrad, O2.lay_prox(prm, 1), h)
    Xp = Xp[np.argsort(np.arctan2(Xp[:, 1] - tree.cent[1][1], Xp[:, 0] - tree.cent[1][0]), kind="stable")]
    gk = GK.Kernel("SL_L_2D", h, GK.Modulation(b.alpha, b.x0, b.y0, b.isig), GK.Modulation(c.alpha, c.x0, c.y0, c.isig))
    H = G1.HSS1D_compress_rectangular_nsym("green", Xp, X1, 108, 1e-11, gk)
    Ho = O1.compress_rectangular_nsym(Xp, X1, 108, 1e-11, kp)
    _rect_parity(G1, H, Ho, Xp, X1, kp, nrhs=4, tol=1e-9)


def test_sum_matches_oracle(gpu):
    """HSS1D_sum_nsym(A, A^T): ranks and skeletons equal the oracle's, the apply equals the
    oracle's and the dense K + K^T; the sum inverts and solves like any compressed matrix;
    operands on different trees are refused."""
    from hssc_directsolver_gb300 import hss1d as G1, kernels as GK
    X = geometry.star_curve(1536)
    kpo = OK.KernelParams(flag=OK.DL_L_2D)
    A = G1.HSS1D_compress_nsym("green", X, 64, 1e-10, GK.Kernel("DL_L_2D"))
    At = G1.HSS1D_transpose(A)
    Cg = G1.HSS1D_sum_nsym(A, At, 1e-10)
    Ao = O1.compress_nsym(X, 64, 1e-10, kpo)
    Co = O1.sum_nsym(Ao, O1.transpose(Ao), 1e-10)
    inf, infA = Cg.info(), A.info()
    nb = inf["nboxes"]
    # on a leaf the IDs read exact copies of the operands' [I T] forms: with the operands
    # exported from the GPU, the oracle's IDs give the same ranks
    for b in range(1, nb):
        if inf["c1"][b] >= 0:
            continue
        ea, eb = A.export_box(b), At.export_box(b)
        n, k = int(infA["cnt"][b]), int(infA["kskel"][b])
        RC = np.vstack([O1._rform(ea["T_UP"], ea["J_UP"], k, n), O1._rform(eb["T_UP"], eb["J_UP"], k, n)])
        LCt = np.vstack([O1._rform(ea["T_DN"], ea["J_DN"], k, n), O1._rform(eb["T_DN"], eb["J_DN"], k, n)])
        ko = idecomp.id_adaptive(RC, 1e-10, 0, 2 * b)[2]
        ki = idecomp.id_adaptive(LCt, 1e-10, 0, 2 * b + 1)[2]
        assert inf["kskel"][b] == max(ko, ki), (b, inf["kskel"][b], ko, ki, Co.kskel[b])
    # against the oracle's own operands (whose T differ from the GPU's in the last bits) and
    # above the leaves (products whose rounding differs from numpy's) a rank sitting at the
    # tolerance may move by one: 7 of 62 boxes here
    kd = np.abs(inf["kskel"][1:] - np.array(Co.kskel[1:]))
    assert kd.max() <= 1 and np.mean(kd == 0) >= 0.8, (np.nonzero(kd)[0] + 1, kd[kd > 0])
    q = np.random.default_rng(8).standard_normal((X.shape[0], 3))
    u = G1.HSS1D_apply_nsym(Cg, q)
    uo = O1.apply_nsym(Co, q)
    assert np.linalg.norm(u - uo) <= 1e-9 * np.linalg.norm(uo)
    K = OK.kernel_eval(X, X, kpo)
    assert np.linalg.norm(u - (K + K.T) @ q) <= 1e-9 * np.linalg.norm((K + K.T) @ q)
    G1.HSS1D_invert_nsym(Cg)
    x, rr, _ = G1.HSS1D_solve(Cg, u, tol=1e-10)
    assert rr < 1e-10 and np.linalg.norm(x - q) <= 1e-8 * np.linalg.norm(q)
    B = G1.HSS1D_compress_nsym("green", geometry.star_curve(1024), 64, 1e-10, GK.Kernel("DL_L_2D"))
    with pytest.raises(Exception):
        G1.HSS1D_sum_nsym(A, B, 1e-10)


def test_sum_forest(gpu):
    """The sum of two forests of curves (one launch per level across problems) equals the
    oracle's per-problem sums."""
    from hssc_directsolver_gb300 import hss1d as G1, kernels as GK
    Xs = [geometry.star_curve(900), geometry.fourier_curve(1300, np.array([0.0, 0.1, 0.05]), np.array([0.0, 1.0, 2.0]))]
    kpo = OK.KernelParams(flag=OK.DL_L_2D)
    A = G1.HSS1D_compress_batch(Xs, 64, 1e-10, GK.Kernel("DL_L_2D"))
    Cg = G1.HSS1D_sum_nsym(A, G1.HSS1D_scalarmult(-0.5, G1.HSS1D_transpose(A)), 1e-10)
    q = np.random.default_rng(9).standard_normal((sum(x.shape[0] for x in Xs), 2))
    u = G1.HSS1D_apply_nsym(Cg, q)
    r0 = 0
    for p, X in enumerate(Xs):
        Ao = O1.compress_nsym(X, 64, 1e-10, kpo, seed=p)
        Co = O1.sum_nsym(Ao, O1.scalarmult(-0.5, O1.transpose(Ao)), 1e-10, seed=p)
        uo = O1.apply_nsym(Co, q[r0:r0 + X.shape[0]])
        assert np.linalg.norm(u[r0:r0 + X.shape[0]] - uo) <= 1e-9 * np.linalg.norm(uo)
        r0 += X.shape[0]


def test_compress_lr_and_low_rank_update(gpu):
    """HSS1D_compressLR_nsym: the IDs read exact copies of U and V rows, so ranks, skeletons
    and the apply equal the oracle's; K + U V^T (HSS1D_sum_nsym of a kernel compression and
    the low-rank one) inverts and solves to 1e-10 against the dense matrix."""
    from hssc_directsolver_gb300 import hss1d as G1, kernels as GK
    rng = np.random.default_rng(4)
    N, r = 2000, 11
    U, V = rng.standard_normal((N, r)), rng.standard_normal((N, r))
    H = G1.HSS1D_compressLR_nsym(U, V, 64, 1e-10)
    Ho = O1.compress_lr_nsym(U, V, 64, 1e-10)
    inf = H.info()
    assert np.array_equal(inf["kskel"][1:], Ho.kskel[1:])
    for b in range(1, inf["nboxes"]):
        e = H.export_box(b)
        assert np.array_equal(e["I_SKUP"], Ho.I_SKUP[b]) and np.array_equal(e["I_SKDN"], Ho.I_SKDN[b])
    q = rng.standard_normal((N, 3))
    u = G1.HSS1D_apply_nsym(H, q)
    assert np.linalg.norm(u - O1.apply_nsym(Ho, q)) <= 1e-12 * np.linalg.norm(u)
    assert np.linalg.norm(u - U @ (V.T @ q)) <= 1e-12 * np.linalg.norm(u)
    X = geometry.star_curve(N)
    kpo = OK.KernelParams(flag=OK.DL_L_2D)
    A = G1.HSS1D_compress_nsym("green", X, 64, 1e-10, GK.Kernel("DL_L_2D"))
    Cg = G1.HSS1D_sum_nsym(A, G1.HSS1D_scalarmult(1e-3, H), 1e-10)
    Kd = OK.kernel_eval(X, X, kpo) + 1e-3 * U @ V.T
    f = rng.standard_normal(N)
    G1.HSS1D_invert_nsym(Cg)
    x, rr, _ = G1.HSS1D_solve(Cg, f, tol=1e-10)
    assert rr < 1e-10
    xd = np.linalg.solve(Kd, f)
    assert np.linalg.norm(x - xd) <= 1e-8 * np.linalg.norm(xd)


def test_block_submatrix_apply(gpu):
    """BHSS1D_apply_nsym: the submatrix of a 2 x 2 block matrix whose blocks are four
    compressed curves, applied through four GPU submatrix applies, equals the dense product."""
    from hssc_directsolver_gb300 import hss1d as G1, kernels as GK
    rng = np.random.default_rng(12)
    kpo = OK.KernelParams(flag=OK.DL_L_2D)
    n1, n2 = 700, 900
    Xa, Xb = geometry.star_curve(n1), geometry.star_curve(n2, eps=0.2, m=3)
    Xc, Xd = geometry.star_curve(800), geometry.star_curve(800, eps=0.1, m=4)
    Ks = [G1.HSS1D_compress_nsym("green", X, 64, 1e-10, GK.Kernel("DL_L_2D")) for X in (Xa, Xc, Xd, Xb)]
    Kd = [OK.kernel_eval(X, X, kpo) for X in (Xa, Xc, Xd, Xb)]
    sizes = [n1, 800, 800, n2]
    # row masks of the block row i and column masks of the block column j: K11 rows/cols split
    # into complementary parts as in the reference's use (k1 + r1 = n1)
    dn1 = rng.random(n1) < 0.5
    up1 = ~dn1
    dn2 = rng.random(n2) < 0.4
    up2 = ~dn2
    k1, r1, k2, r2 = dn1.sum(), up1.sum(), dn2.sum(), up2.sum()
    def mask(n, cnt, seed):
        m = np.zeros(n, bool)
        m[np.random.default_rng(seed).choice(n, cnt, replace=False)] = True
        return m
    I_dn = [[dn1, mask(800, k1, 1)], [mask(800, k2, 2), dn2]]
    I_up = [[up1, mask(800, r2, 3)], [mask(800, r1, 4), up2]]
    X = rng.standard_normal((r1 + r2, 2))
    Y = G1.BHSS1D_apply_nsym(Ks[0], Ks[1], Ks[2], Ks[3], None, None, I_dn, I_up, X)
    A = np.block([[Kd[0][np.ix_(I_dn[0][0], I_up[0][0])], Kd[1][np.ix_(I_dn[0][1], I_up[0][1])]],
                  [Kd[2][np.ix_(I_dn[1][0], I_up[1][0])], Kd[3][np.ix_(I_dn[1][1], I_up[1][1])]]])
    assert Y.shape == (k1 + k2, 2)
    assert np.linalg.norm(Y - A @ X) <= 1e-9 * np.linalg.norm(A @ X)


def test_fsym_sum_and_low_rank_forms(gpu):
    """HSS1D_sum_fsym and HSS1D_compressLR_fsym (the nsym algorithms, which take fsym
    operands, T_DN = T_UP, unchanged): the sum of two fsym compressions of symmetric kernels
    and the compressed U U^T equal their dense matrices to the tolerance, and the sum inverts
    and solves against its dense matrix."""
    from hssc_directsolver_gb300 import hss1d as G1, kernels as GK
    rng = np.random.default_rng(21)
    N = 1500
    X = geometry.star_curve(N)
    h = 2 * np.pi / N
    ka = GK.Kernel("SL_L_2D", np.sqrt(h))
    A = G1.HSS1D_compress_fsym("green", X, 64, 1e-12, ka)
    B = G1.HSS1D_scalarmult(0.5, G1.HSS1D_compress_fsym("green", X, 64, 1e-12, ka))
    Ad = G1.HSS1D_dense_matrix(A)
    C = G1.HSS1D_sum_fsym(A, B, 1e-10)
    Cd = G1.HSS1D_dense_matrix(C)
    assert np.linalg.norm(Cd - 1.5 * Ad) <= 1e-9 * np.linalg.norm(Ad)
    U = rng.standard_normal((N, 7))
    H = G1.HSS1D_compressLR_fsym(U, U, 64, 1e-10)
    Hd = G1.HSS1D_dense_matrix(H)
    assert np.linalg.norm(Hd - U @ U.T) <= 1e-10 * np.linalg.norm(U @ U.T)
    S = G1.HSS1D_sum_fsym(C, G1.HSS1D_scalarmult(1e-4, H), 1e-10)
    Sd = 1.5 * Ad + 1e-4 * U @ U.T
    G1.HSS1D_invert_nsym(S)
    f = rng.standard_normal(N)
    x, rr, _ = G1.HSS1D_solve(S, f, tol=1e-10)
    assert rr < 1e-10
    xd = np.linalg.solve(Sd, f)
    assert np.linalg.norm(x - xd) <= 1e-7 * np.linalg.norm(xd)


@pytest.mark.parametrize("acc", [1e-6, 1e-9])
def test_recompress_matches_oracle(gpu, acc):
    """HSS1D_recompress_nsym (HSS1D/HSS1D_recompress_nsym.m:26-247) on the GPU: a star-curve
    compression at 1e-12 recompressed at acc.  The SVD truncation ranks, the full-rank IDs'
    skeletons and the operator equal the oracle's restatement on the same (exported-equal)
    operand; the ranks drop and the operator stays within ~acc of the original."""
    from hssc_directsolver_gb300 import hss1d as G1, kernels as GK
    X = geometry.star_curve(1024)
    kp = OK.KernelParams(flag=OK.DL_L_2D)
    A = G1.HSS1D_compress_nsym("green", X, 64, 1e-12, GK.Kernel("DL_L_2D"))
    Ao = O1.compress_nsym(X, 64, 1e-12, kp)
    inf = A.info()
    assert np.array_equal(inf["kskel"][1:], np.array(Ao.kskel[1:]))
    R = G1.HSS1D_recompress_nsym(A, acc)
    Ro = O1.recompress_nsym(Ao, acc)
    ri = R.info()
    print(f"recompress {acc:g}: ranks {list(inf['kskel'][1:5])} -> {list(ri['kskel'][1:5])} "
          f"(oracle {Ro.kskel[1:5]})")
    assert np.array_equal(ri["kskel"][1:], np.array(Ro.kskel[1:]))
    assert max(ri["kskel"][1:]) < max(inf["kskel"][1:])
    nb = ri["nboxes"]
    same = 0
    for b in range(1, nb):
        e = R.export_box(b)
        same += int(np.array_equal(e["I_SKUP"], Ro.I_SKUP[b]) and np.array_equal(e["I_SKDN"], Ro.I_SKDN[b]))
    q = np.random.default_rng(11).standard_normal((1024, 3))
    u, uo, ua = G1.HSS1D_apply_nsym(R, q), O1.apply_nsym(Ro, q), G1.HSS1D_apply_nsym(A, q)
    d_or, d_a = np.linalg.norm(u - uo) / np.linalg.norm(uo), np.linalg.norm(u - ua) / np.linalg.norm(ua)
    print(f"  skeletons equal in {same}/{nb - 1} boxes; apply vs oracle {d_or:.2e}, vs the operand {d_a:.2e}")
    assert same >= nb - 1 - 2
    assert d_or <= 1e-8 and d_a <= 50 * acc
    G1.HSS1D_invert_nsym(R)
    x = G1.HSS1D_applyinv_nsym(R, None, None, u)
    assert np.linalg.norm(x - q) <= 1e-8 * np.linalg.norm(q)
