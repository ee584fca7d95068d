"""HSS2D on the GPU against the oracle, the golden fixture and full-size properties (GPU)."""
import os

import numpy as np
import pytest

from oracle import hss2d as O2, kernels as OK

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def params(npan, precision="fp64", Ng=8):
    from hssc_directsolver_gb300 import hss2d as G2, kernels as GK
    h = 2.0 / (Ng * npan)
    return G2.HSS2DParams(Ng=Ng, npan=npan, kernel=GK.Kernel("SL_L_2D", h, GK.Modulation(),
                                                               GK.Modulation(0.5, 0, 0, 20.0)),
                          precision=precision)


def oracle(npan, Ng=8):
    kp = OK.KernelParams(flag=OK.SL_L_2D, h=2.0 / (Ng * npan), c=OK.Modulation(0.5, 0, 0, 20.0))
    prm = O2.HSS2DParams(Ng=Ng, npan=npan, kp=kp)
    tree = O2.build_tree_nsym(prm)
    blk = O2.compress_nsym(tree, prm)
    return prm, tree, blk, O2.invert_nsym(tree, prm, blk)


@pytest.fixture(scope="module", params=[4, 8])
def case(request, gpu):
    from hssc_directsolver_gb300 import hss2d as G2
    npan = request.param
    t = G2.HSS2D_build_tree_nsym(params(npan))
    G2.HSS2D_compress_nsym(t)
    G2.HSS2D_invert_nsym(t)
    return G2, t, oracle(npan)


def test_tree_exact(case):
    G2, t, (prm, ot, blk, inv) = case
    n, k, p = t.box_sizes()
    for b in range(t.nboxes):
        e = t.export_box(b)
        assert np.array_equal(e["J"], ot.J[b]) and np.array_equal(e["I_src"], ot.I_src[b])
        assert k[b] == ot.k[b] and p[b] == ot.proxy[b].shape[0]
        if b > 0 and ot.T_up[b].size:
            s = max(1.0, np.abs(ot.T_up[b]).max())
            assert np.abs(e["T_up"] - ot.T_up[b]).max() <= 1e-7 * s
            assert np.abs(e["T_dn"] - ot.T_dn[b]).max() <= 1e-7 * s


def test_inverse_factors(case):
    G2, t, (prm, ot, blk, inv) = case
    for b in (0, 1, t.nboxes - 1):
        FI, E = t.export_inverse(b)
        assert np.abs(FI - inv["FI"][b]).max() <= 1e-7 * np.abs(inv["FI"][b]).max()
        if b > 0:
            assert np.abs(E - inv["E"][b]).max() <= 1e-7 * np.abs(inv["E"][b]).max()


def test_apply_and_applyinv_match_oracle(case):
    G2, t, (prm, ot, blk, inv) = case
    q = np.random.default_rng(7).standard_normal((prm.N, 5))
    u = G2.HSS2D_apply_nsym(t, None, q)
    assert np.linalg.norm(u - O2.apply_nsym(ot, blk, q)) <= 1e-13 * np.linalg.norm(u)
    x = G2.HSS2D_applyinv_nsym(t, None, q)
    xo = O2.applyinv_nsym(ot, inv, q)
    assert np.linalg.norm(x - xo) <= 1e-12 * np.linalg.norm(xo)
    X = prm.X_source()
    A = OK.kernel_eval(X, X, prm.kp)
    assert np.linalg.norm(q - A @ x) / np.linalg.norm(q) < 1e-9


def test_golden_fixture(gpu):
    from hssc_directsolver_gb300 import hss2d as G2
    g = np.load(os.path.join(GOLD, "hss2d_npan4.npz"))
    t = G2.HSS2D_invert_nsym(G2.HSS2D_build_tree_nsym(params(4)))
    x = G2.HSS2D_applyinv_nsym(t, None, g["f"])
    assert np.linalg.norm(x - g["x"]) <= 1e-12 * np.linalg.norm(g["x"])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_solve_refinement(gpu, precision):
    from hssc_directsolver_gb300 import hss2d as G2
    t = G2.HSS2D_invert_nsym(G2.HSS2D_build_tree_nsym(params(8, precision)))
    prm, ot, blk, inv = oracle(8)
    f = np.random.default_rng(8).standard_normal((prm.N, 4))
    x, rr, it = G2.HSS2D_solve(t, f, 1e-12, 8)
    assert rr <= 1e-12
    r = f - O2.apply_nsym(ot, blk, x)
    assert np.linalg.norm(r, axis=0).max() / np.linalg.norm(f, axis=0).min() < 1e-11


def test_full_size_properties(gpu):
    """The 256x256 workload (N = 65536): forward(inverse(f)) = f to 1e-10, linearity."""
    from hssc_directsolver_gb300 import hss2d as G2
    t = G2.HSS2D_invert_nsym(G2.HSS2D_build_tree_nsym(params(32)))
    assert t.N == 65536 and t.depth == 10
    r = np.random.default_rng(0)
    f = r.standard_normal((t.N, 4))
    x = G2.HSS2D_applyinv_nsym(t, None, f)
    back = G2.HSS2D_apply_nsym(t, None, x)
    assert np.linalg.norm(back - f, axis=0).max() / np.linalg.norm(f, axis=0).min() < 1e-10
    x2 = G2.HSS2D_applyinv_nsym(t, None, 2.0 * f[:, :2] - 3.0 * f[:, 2:])
    assert np.linalg.norm(x2 - (2.0 * x[:, :2] - 3.0 * x[:, 2:])) <= 1e-11 * np.linalg.norm(x2)
    xs, rr, it = G2.HSS2D_solve(t, f, 1e-10, 3)
    assert rr <= 1e-10 and it == 1


def test_status_codes(gpu):
    from hssc_directsolver_gb300 import hss2d as G2, _lib as L
    with pytest.raises(L.HSSError) as e:
        G2.HSS2D_build_tree_nsym(params(6))       # npan must be a power of two
    assert e.value.code == L.HSS_ERR_ARG
    t = G2.HSS2D_build_tree_nsym(params(4))
    with pytest.raises(L.HSSError) as e:
        G2.HSS2D_applyinv_nsym(t, None, np.ones(t.N))
    assert e.value.code == L.HSS_ERR_STATE
    G2.HSS2D_invert_nsym(t)
    f = np.ones(t.N)
    f[3] = np.nan
    with pytest.raises(L.HSSError) as e:
        G2.HSS2D_solve(t, f, 1e-10, 2)
    assert e.value.code == L.HSS_ERR_NONFINITE


@pytest.mark.parametrize("npan", [4, 8])
def test_translation_invariant_mode(gpu, npan):
    """transinv = 1 (one factor set per level, INFO_TREE.LEV) on the unmodulated kernel agrees with
    the per-box (NTI) oracle, whose boxes of a level are all translates of each other."""
    from hssc_directsolver_gb300 import hss2d as G2, kernels as GK
    Ng = 8
    h = 2.0 / (Ng * npan)
    gp = G2.HSS2DParams(Ng=Ng, npan=npan, kernel=GK.Kernel("SL_L_2D", h), transinv=1)
    t = G2.HSS2D_invert_nsym(G2.HSS2D_build_tree_nsym(gp))
    kp = OK.KernelParams(flag=OK.SL_L_2D, h=h)
    prm = O2.HSS2DParams(Ng=Ng, npan=npan, kp=kp)
    ot = O2.build_tree_nsym(prm)
    blk = O2.compress_nsym(ot, prm)
    inv = O2.invert_nsym(ot, prm, blk)
    f = np.random.default_rng(9).standard_normal((prm.N, 3))
    x = G2.HSS2D_applyinv_nsym(t, None, f)
    xo = O2.applyinv_nsym(ot, inv, f)
    assert np.linalg.norm(x - xo) <= 1e-11 * np.linalg.norm(xo)
    u = G2.HSS2D_apply_nsym(t, None, f)
    assert np.linalg.norm(u - O2.apply_nsym(ot, blk, f)) <= 1e-12 * np.linalg.norm(u)
    with pytest.raises(Exception):
        G2.HSS2D_build_tree_nsym(G2.HSS2DParams(Ng=Ng, npan=npan, transinv=1,
                                                kernel=GK.Kernel("SL_L_2D", h, GK.Modulation(),
                                                                 GK.Modulation(0.5, 0, 0, 20.0))))


# ---- INTERform 'lowrank' (the reference default): randomized ID of K21, T = T.U T.V^T ----

@pytest.fixture(scope="module")
def lowrank8(gpu):
    from hssc_directsolver_gb300 import hss2d as G2
    prm = params(8)
    prm.INTERform = "lowrank"
    t = G2.HSS2D_build_tree_nsym(prm)
    G2.HSS2D_compress_nsym(t)
    G2.HSS2D_invert_nsym(t)
    kp = OK.KernelParams(flag=OK.SL_L_2D, h=2.0 / 64, c=OK.Modulation(0.5, 0, 0, 20.0))
    oprm = O2.HSS2DParams(Ng=8, npan=8, kp=kp, INTERform="lowrank")
    ot = O2.build_tree_nsym(oprm)
    return G2, t, oprm, ot


def test_lowrank_ranks_and_T_match_oracle(lowrank8):
    """Randomized ranks of every low-rank T equal the oracle's (same Gaussian samples from
    the counter RNG); T = T.U T.V^T agrees to the least-squares conditioning."""
    G2, t, oprm, ot = lowrank8
    qu, qd = t.interp_ranks()
    assert len(ot.lowrank) > 0
    for b in range(t.nboxes):
        if b in ot.lowrank:
            lr = ot.lowrank[b]
            assert qu[b] == lr["Uu"].shape[1] and qd[b] == lr["Ud"].shape[1]
        else:
            assert qu[b] == -1 and qd[b] == -1
    for b in ot.lowrank:
        e = t.export_box(b)
        s = max(1.0, np.abs(ot.T_up[b]).max())
        assert np.abs(e["T_up"] - ot.T_up[b]).max() <= 1e-6 * s
        assert np.abs(e["T_dn"] - ot.T_dn[b]).max() <= 1e-6 * s


def test_lowrank_solve_accuracy(lowrank8):
    """The low-rank compressed inverse solves to the dense path's accuracy: relative
    residual against the kernel matrix ~acc before refinement, <= 1e-10 after."""
    G2, t, oprm, ot = lowrank8
    f = np.random.default_rng(0).standard_normal((oprm.N, 2))
    x = G2.HSS2D_applyinv_nsym(t, t, f)
    r = O2.kernel_matvec(oprm, x) - f
    assert np.linalg.norm(r) / np.linalg.norm(f) < 1e-8
    xs, relres, its = G2.HSS2D_solve(t, f, 1e-10, 5)
    r = O2.kernel_matvec(oprm, xs) - f
    assert np.linalg.norm(r) / np.linalg.norm(f) < 5e-10


def test_levhss_matches_oracle(case):
    G2, t, (prm, ot, blk, inv) = case
    for n_cut in (10, 40, 100, 400, 10 ** 6):
        assert G2.levHSS(t, n_cut) == O2.lev_hss(ot, n_cut)


def test_dfloat_solve_matches_fp64(gpu):
    """HSS_PREC_DFLOAT: the same FP64 factors, solve products in paired-FP32 arithmetic.
    Forward and inverse applies agree with the FP64 mode to ~1e-13 and the refined solve
    reaches 1e-10."""
    from hssc_directsolver_gb300 import hss2d as G2
    ts = {}
    for prec in ("fp64", "dfloat"):
        t = G2.HSS2D_build_tree_nsym(params(8, prec))
        G2.HSS2D_compress_nsym(t)
        G2.HSS2D_invert_nsym(t)
        ts[prec] = t
    f = np.random.default_rng(3).standard_normal((ts["fp64"].N, 4))
    y64 = G2.HSS2D_apply_nsym(ts["fp64"], ts["fp64"], f)
    ydf = G2.HSS2D_apply_nsym(ts["dfloat"], ts["dfloat"], f)
    assert np.linalg.norm(ydf - y64) <= 1e-13 * np.linalg.norm(y64)
    x64 = G2.HSS2D_applyinv_nsym(ts["fp64"], ts["fp64"], f)
    xdf = G2.HSS2D_applyinv_nsym(ts["dfloat"], ts["dfloat"], f)
    assert np.linalg.norm(xdf - x64) <= 1e-11 * np.linalg.norm(x64)
    x, rr, it = G2.HSS2D_solve(ts["dfloat"], f, 1e-10, 5)
    assert rr <= 1e-10
    assert np.linalg.norm(x - x64) <= 1e-10 * np.linalg.norm(x64)
    f11 = np.random.default_rng(4).standard_normal((ts["fp64"].N, 11))   # 8 + 3 columns
    a = G2.HSS2D_applyinv_nsym(ts["fp64"], ts["fp64"], f11)
    b = G2.HSS2D_applyinv_nsym(ts["dfloat"], ts["dfloat"], f11)
    assert np.linalg.norm(b - a) <= 1e-11 * np.linalg.norm(a)


def test_dfloat_inv_solves_to_tolerance(gpu):
    """HSS_PREC_DFLOAT_INV: the inversion's updates and products in paired FP32 too. The
    factors are a few bits short of FP64, so the refined solve is the contract: relres
    <= 1e-10 and the solution within 1e-9 of the FP64 path."""
    from hssc_directsolver_gb300 import hss2d as G2
    t64 = G2.HSS2D_build_tree_nsym(params(8, "fp64"))
    G2.HSS2D_compress_nsym(t64)
    G2.HSS2D_invert_nsym(t64)
    t = G2.HSS2D_build_tree_nsym(params(8, "dfloat_inv"))
    G2.HSS2D_compress_nsym(t)
    G2.HSS2D_invert_nsym(t)
    f = np.random.default_rng(8).standard_normal((t.N, 4))
    x64 = G2.HSS2D_applyinv_nsym(t64, t64, f)
    x = G2.HSS2D_applyinv_nsym(t, t, f)
    assert np.linalg.norm(x - x64) <= 1e-9 * np.linalg.norm(x64)
    xs, rr, it = G2.HSS2D_solve(t, f, 1e-10, 5)
    assert rr <= 1e-10 and it <= 2
    assert np.linalg.norm(xs - x64) <= 1e-9 * np.linalg.norm(x64)
    # the interpolation operators come from a double-float least squares too: the
    # solution still solves the kernel system to the compression tolerance
    kp = OK.KernelParams(flag=OK.SL_L_2D, h=2.0 / 64, c=OK.Modulation(0.5, 0, 0, 20.0))
    oprm = O2.HSS2DParams(Ng=8, npan=8, kp=kp)
    r = O2.kernel_matvec(oprm, xs) - f
    assert np.linalg.norm(r) / np.linalg.norm(f) < 1e-9


def test_bicgstab_with_translation_invariant_preconditioner(gpu):
    """The reference's iterative solution: BiCGSTAB on the variable-coefficient operator,
    preconditioned by the inverse of the translation-invariant (b = c = 1) tree. Converges
    to 1e-10 and agrees with the direct solve."""
    from hssc_directsolver_gb300 import hss2d as G2, kernels as GK
    A = G2.HSS2D_build_tree_nsym(params(8))
    G2.HSS2D_compress_nsym(A)
    G2.HSS2D_invert_nsym(A)
    prm_ti = G2.HSS2DParams(Ng=8, npan=8, kernel=GK.Kernel("SL_L_2D", 2.0 / 64), transinv=1)
    M = G2.HSS2D_build_tree_nsym(prm_ti)
    G2.HSS2D_compress_nsym(M)
    G2.HSS2D_invert_nsym(M)
    f = np.random.default_rng(11).standard_normal((A.N, 3))
    x, rr, it = G2.HSS2D_bicgstab(A, f, 1e-10, 100, PRECOND=M)
    assert rr <= 1e-10 and it < 100
    xd = G2.HSS2D_applyinv_nsym(A, A, f)
    assert np.linalg.norm(x - xd) <= 1e-8 * np.linalg.norm(xd)
    # with the operator's own inverse as preconditioner it is a one-step method
    x1, rr1, it1 = G2.HSS2D_bicgstab(A, f, 1e-10, 10, PRECOND=A)
    assert rr1 <= 1e-10 and it1 <= 2


def test_translation_invariant_lowrank_dfloat(gpu):
    """Mode combinations: translation-invariant tree (one factor set per level) with the
    low-rank interpolation operators and double-float solves agrees with the same tree in
    FP64 dense form to the compression tolerance."""
    from hssc_directsolver_gb300 import hss2d as G2, kernels as GK
    out = {}
    for form, prec in (("dense", "fp64"), ("lowrank", "dfloat")):
        prm = G2.HSS2DParams(Ng=8, npan=8, kernel=GK.Kernel("SL_L_2D", 2.0 / 64), transinv=1, INTERform=form,
                             precision=prec)
        t = G2.HSS2D_build_tree_nsym(prm)
        G2.HSS2D_compress_nsym(t)
        G2.HSS2D_invert_nsym(t)
        f = np.random.default_rng(5).standard_normal((t.N, 2))
        x, rr, it = G2.HSS2D_solve(t, f, 1e-10, 4)
        assert rr <= 1e-10
        out[form] = x
        if form == "lowrank":
            qu, qd = t.interp_ranks()
            assert (qu > 0).any()
    assert np.linalg.norm(out["lowrank"] - out["dense"]) <= 1e-8 * np.linalg.norm(out["dense"])


def test_krylov_argument_errors(gpu):
    from hssc_directsolver_gb300 import hss2d as G2, _lib as L
    A = G2.HSS2D_build_tree_nsym(params(4))
    G2.HSS2D_compress_nsym(A)
    M = G2.HSS2D_build_tree_nsym(params(8))
    G2.HSS2D_compress_nsym(M)
    f = np.ones((A.N, 1))
    with pytest.raises(L.HSSError) as e:
        G2.HSS2D_bicgstab(A, f, 1e-10, 10, PRECOND=M)   # M not inverted
    assert e.value.code == L.HSS_ERR_STATE
    G2.HSS2D_invert_nsym(M)
    with pytest.raises(L.HSSError) as e:
        G2.HSS2D_bicgstab(A, f, 1e-10, 10, PRECOND=M)   # sizes differ
    assert e.value.code == L.HSS_ERR_ARG


@pytest.mark.parametrize("precision", ["fp64", "dfloat", "dfloat_inv"])
def test_smallest_grid_and_rhs_chunks(gpu, precision):
    """npan = 2 (a depth-2 tree), 1 and 17 right-hand sides (two full 8-column chunks and a
    ragged one), every precision: solves to 1e-11 against the oracle's forward operator."""
    from hssc_directsolver_gb300 import hss2d as G2
    t = G2.HSS2D_invert_nsym(G2.HSS2D_build_tree_nsym(params(2, precision)))
    prm, ot, blk, inv = oracle(2)
    for nrhs in (1, 17):
        f = np.random.default_rng(nrhs).standard_normal((prm.N, nrhs))
        x, rr, it = G2.HSS2D_solve(t, f, 1e-11, 4)
        assert rr <= 1e-11
        r = f - O2.apply_nsym(ot, blk, x)
        assert np.linalg.norm(r, axis=0).max() / np.linalg.norm(f, axis=0).min() < 1e-10


@pytest.mark.parametrize("inter", ["dense", "lowrank"])
def test_skeleton_interpolation_error(gpu, inter):
    """Test_HSS2D_skeletons.m on the GPU tree (exported J, T_up per box): the per-level
    interpolation error on a 2*layers box proxy is below 1e-8 and within 2x of the
    oracle tree's."""
    from hssc_directsolver_gb300 import hss2d as G2, kernels as GK
    from test_oracle import skeleton_errors
    npan = 8
    prm = G2.HSS2DParams(Ng=8, npan=npan, kernel=GK.Kernel("SL_L_2D", 2.0 / 64, GK.Modulation(),
                                                             GK.Modulation(0.5, 0, 0, 20.0)), INTERform=inter)
    t = G2.HSS2D_build_tree_nsym(prm)
    kp = OK.KernelParams(flag=OK.SL_L_2D, h=2.0 / 64, c=OK.Modulation(0.5, 0, 0, 20.0))
    oprm = O2.HSS2DParams(Ng=8, npan=npan, kp=kp, INTERform=inter)
    ot = O2.build_tree_nsym(oprm)
    cent = O2.box_centers(ot.depth)
    n, k, _ = t.box_sizes()

    def gbox(b):
        e = t.export_box(b)
        return e["I_src"], e["J"], int(k[b]), e["T_up"], cent[b]

    X = oprm.X_source()
    eg = skeleton_errors(X, oprm.h, oprm.layers, ot.depth, kp, gbox)
    eo = skeleton_errors(X, oprm.h, oprm.layers, ot.depth, kp,
                         lambda b: (np.asarray(ot.I_src[b]), np.asarray(ot.J[b]), ot.k[b], ot.T_up[b], ot.cent[b]))
    assert max(eg) < 1e-8, eg
    assert all(g <= 2 * o + 1e-12 for g, o in zip(eg, eo)), (eg, eo)


def test_autotuned_plans(gpu):
    """hss2d_set_autotune: tuned solve plans give the untuned solution to rounding, the same
    refinement count, and bit-identical results from one tuned solve to the next."""
    from hssc_directsolver_gb300 import hss2d as G2
    t = G2.HSS2D_invert_nsym(G2.HSS2D_build_tree_nsym(params(16, "dfloat")))
    f = np.random.default_rng(9).standard_normal((t.N, 5))
    x0, r0, i0 = G2.HSS2D_solve(t, f, 1e-10, 4)
    t.set_autotune(True)
    x1, r1, i1 = G2.HSS2D_solve(t, f, 1e-10, 4)
    x2, r2, i2 = G2.HSS2D_solve(t, f, 1e-10, 4)
    assert i1 == i0 and r1 <= 1e-10
    assert np.linalg.norm(x1 - x0) <= 1e-12 * np.linalg.norm(x0)
    assert np.array_equal(x1, x2)
    y = G2.HSS2D_apply_nsym(t, None, x1)
    assert np.linalg.norm(y - f, axis=0).max() / np.linalg.norm(f, axis=0).min() <= 1e-10


@pytest.mark.parametrize("rule,npan", [("rand", 4), ("rand", 8), ("wdec", 4), ("wdec", 8)])
def test_skeleton_rules_match_oracle(gpu, rule, npan):
    """params.skel_rule = 'rand' (LOCAL_Preset_Skeleton_Info :703-730: a random sample of each
    box's points, the Mersenne Twister reset to seed 5489 per box as the reference's
    rng('default')) and 'wdec' (:668-701: the Whitney decomposition of
    Common/Whitney_decomposition.m); every box of a level raised to the level's largest count
    by promoting the residual points nearest its boundary.  Skeletons equal the oracle's; the
    forward apply agrees to 1e-13 and the inverse apply to the FP64 parity level."""
    from hssc_directsolver_gb300 import hss2d as G2
    p = params(npan, "fp64")
    p.skel_rule = rule
    p.INTERform = "dense"
    kp = OK.KernelParams(flag=OK.SL_L_2D, h=2.0 / (8 * npan), c=OK.Modulation(0.5, 0, 0, 20.0))
    prm = O2.HSS2DParams(Ng=8, npan=npan, kp=kp, skel_rule=rule, uniform_ranks=True)
    ot = O2.build_tree_nsym(prm)
    blk = O2.compress_nsym(ot, prm)
    inv = O2.invert_nsym(ot, prm, blk)
    t = G2.HSS2D_invert_nsym(G2.HSS2D_build_tree_nsym(p))
    _, k, _ = t.box_sizes()
    for b in range(t.nboxes):
        e = t.export_box(b)
        assert k[b] == ot.k[b] and np.array_equal(e["J"], ot.J[b]) and np.array_equal(e["I_src"], ot.I_src[b]), b
    q = np.random.default_rng(5).standard_normal((prm.N, 3))
    y = G2.HSS2D_apply_nsym(t, None, q)
    yo = O2.apply_nsym(ot, blk, q)
    x = G2.HSS2D_applyinv_nsym(t, None, q)
    xo = O2.applyinv_nsym(ot, inv, q)
    df, di = np.linalg.norm(y - yo) / np.linalg.norm(yo), np.linalg.norm(x - xo) / np.linalg.norm(xo)
    print(f"{rule} npan {npan}: forward {df:.2e}, inverse {di:.2e}")
    # the proxy systems of these skeletons are numerically rank deficient (the Whitney
    # skeletons hold 60 of a leaf's 64 points): both sides solve them damped, and the inverse
    # factors agree to ~1e-11 (measured 2.4e-12 / 1.7e-11 for 'rand' at npan 4 / 8)
    assert df <= 1e-13 and di <= 1e-10
