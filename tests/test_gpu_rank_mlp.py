"""Learned ranks on the GPU: MLP kernels against the oracle, and the learned HSS1D
compress against the plain one (GPU)."""
import numpy as np
import pytest

from oracle import mlp as OM

pytestmark = pytest.mark.gpu


def _data(B, nin=8, seed=0):
    r = np.random.default_rng(seed)
    X = r.standard_normal((B, nin)).astype(np.float32)
    t = r.uniform(0.05, 0.95, B).astype(np.float32)
    return X, t


def test_init_matches_oracle(gpu):
    from hssc_directsolver_gb300.rank_mlp import RankPredictor
    P = RankPredictor(seed=9)
    assert np.array_equal(P.params(), OM.init_params(8, 32, seed=9))


@pytest.mark.parametrize("B", [1, 77, 1000])
def test_gradient_matches_oracle(gpu, B):
    from hssc_directsolver_gb300.rank_mlp import RankPredictor
    P = RankPredictor(seed=2)
    p = OM.init_params(8, 32, seed=2).copy()
    p[256:288] = 0.05
    P.set_params(p)
    X, t = _data(B, seed=B)
    loss, g = P.grad(X, t)
    lo, go = OM.loss_and_grad(p, X, t, 8, 32)
    assert abs(loss - lo) <= 1e-5 * lo + 1e-7
    assert np.linalg.norm(g - go) <= 2e-5 * np.linalg.norm(go) + 1e-7
    y = P.predict(X)
    yo, _ = OM.forward(p, X, 8, 32)
    assert np.abs(y - yo).max() <= 1e-6


def test_gradient_is_reproducible(gpu):
    from hssc_directsolver_gb300.rank_mlp import RankPredictor
    P = RankPredictor(seed=4)
    X, t = _data(5000, seed=1)
    g1 = P.grad(X, t)[1]
    g2 = P.grad(X, t)[1]
    assert np.array_equal(g1, g2)


def test_adam_steps_match_oracle(gpu):
    from hssc_directsolver_gb300.rank_mlp import RankPredictor
    P = RankPredictor(seed=5)
    X, t = _data(256, seed=3)
    P.train(X, t, epochs=5, batch=64, lr=1e-3)
    p = OM.init_params(8, 32, seed=5).astype(np.float64)
    m = np.zeros_like(p)
    v = np.zeros_like(p)
    s = 0
    for _ in range(5):
        for b0 in range(0, 256, 64):
            s += 1
            _, g = OM.loss_and_grad(p, X[b0:b0 + 64], t[b0:b0 + 64], 8, 32)
            p, m, v = OM.adam_step(p, g, m, v, s, 1e-3)
    assert np.abs(P.params() - p).max() <= 2e-4


@pytest.fixture(scope="module")
def curves(gpu):
    from hssc_directsolver_gb300 import hss1d as G1, kernels as GK, geometry as GG
    from hssc_directsolver_gb300.rank_mlp import RankPredictor, training_set
    Xs, sizes = GG.batched_curves(12, nmin=1000, nmax=6000, seed=21)
    kern = GK.Kernel("DL_L_2D")
    H = G1.HSS1D_compress_batch(Xs, 64, 1e-10, kern)
    F, y = training_set(H)
    P = RankPredictor(seed=0)
    loss = P.train(F, y, epochs=300, batch=256, lr=3e-3)
    return G1, GK, GG, Xs, sizes, kern, H, P, loss, F, y


def test_predictor_learns_ranks(curves):
    G1, GK, GG, Xs, sizes, kern, H, P, loss, F, y = curves
    l0 = 0.5 * np.mean((y - y.mean()) ** 2)
    assert loss < 0.2 * l0
    assert np.abs(P.predict(F) - y).mean() < 0.05


def _same_compress(G1, A, B):
    ia, ib = A.info(), B.info()
    assert np.array_equal(ia["kskel"], ib["kskel"]) and np.array_equal(ia["nskel"], ib["nskel"])
    for b in range(ia["nboxes"]):
        if ia["level"][b] == 0:
            continue
        ea, eb = A.export_box(b), B.export_box(b)
        assert np.array_equal(ea["I_SKUP"], eb["I_SKUP"]) and np.array_equal(ea["I_SKDN"], eb["I_SKDN"])
        k = int(ia["kskel"][b])
        for J, T in (("J_UP", "T_UP"), ("J_DN", "T_DN")):
            if ea[T].size:
                pos = {c: i for i, c in enumerate(eb[J][k:])}
                Tb = np.stack([eb[T][:, pos[c]] for c in ea[J][k:]], axis=1)
                assert np.array_equal(ea[T], Tb)


def test_learned_compress_equals_plain(curves):
    """New curves: the learned compress gives the same ranks, skeletons and T bit for bit
    with fewer QR steps.  Only the order of the residual (non-skeleton) columns past the
    truncation differs, which reorders sums in the inversion: inverse applies agree to
    rounding."""
    G1, GK, GG, Xs, sizes, kern, H, P, loss, F, y = curves
    Xn, sn = GG.batched_curves(6, nmin=1500, nmax=5000, seed=99)
    A = G1.HSS1D_compress_batch(Xn, 64, 1e-10, kern)
    B = G1.HSS1D_compress_batch(Xn, 64, 1e-10, kern, predictor=P)
    _same_compress(G1, A, B)
    done, full, reruns = B.id_stats()
    done_a, full_a, _ = A.id_stats()
    assert done_a == full_a == full and done < 0.8 * full
    G1.HSS1D_invert_nsym(A)
    G1.HSS1D_invert_nsym(B)
    f = np.random.default_rng(3).standard_normal((sum(sn), 2))
    xa = G1.HSS1D_applyinv_nsym(A, None, None, f)
    xb = G1.HSS1D_applyinv_nsym(B, None, None, f)
    assert np.linalg.norm(xa - xb) <= 1e-13 * np.linalg.norm(xa)


def test_untrained_predictor_still_exact(curves):
    """A predictor that is far off only costs QR steps: results stay identical."""
    G1, GK, GG, Xs, sizes, kern, H, P, loss, F, y = curves
    from hssc_directsolver_gb300.rank_mlp import RankPredictor
    Q = RankPredictor(seed=1)
    p = Q.params()
    p[:] = 0.0
    p[-1] = -6.0                       # predicts k/n ~ 0.0025: every QR is checked from step 5 on
    Q.set_params(p)
    Xn = Xs[:4]
    A = G1.HSS1D_compress_batch(Xn, 64, 1e-10, kern)
    B = G1.HSS1D_compress_batch(Xn, 64, 1e-10, kern, predictor=Q)
    _same_compress(G1, A, B)
    done, full, _ = B.id_stats()
    assert done <= full


def test_learned_against_the_per_step_rule(curves):
    """The model-free baseline the learned mode must be weighed against: the same stop rule
    tested at every step of every pivoted QR (HSS_ID_STEP_TEST).  Both give the plain
    compress's ranks, skeletons and T; the QR steps and reruns of each are reported (the
    per-step rule can stop no later than the hint, and pays in reruns when the randomized
    check relaxes the threshold past where it stopped)."""
    import time
    G1, GK, GG, Xs, sizes, kern, H, P, loss, F, y = curves
    Xn, sn = GG.batched_curves(6, nmin=1500, nmax=5000, seed=99)
    t = {}
    mats = {}
    for name, kw in (("plain", {}), ("learned", {"predictor": P}), ("per_step", {"step_test": True})):
        t0 = time.perf_counter()
        mats[name] = G1.HSS1D_compress_batch(Xn, 64, 1e-10, kern, **kw)
        t[name] = time.perf_counter() - t0
    _same_compress(G1, mats["plain"], mats["learned"])
    _same_compress(G1, mats["plain"], mats["per_step"])
    done_p, full, _ = mats["plain"].id_stats()
    done_l, _, re_l = mats["learned"].id_stats()
    done_s, _, re_s = mats["per_step"].id_stats()
    print(f"QR steps: full {full}, learned {done_l} ({re_l} reruns), per-step rule {done_s} ({re_s} reruns); "
          f"compress s: plain {t['plain']:.3f}, learned {t['learned']:.3f}, per-step {t['per_step']:.3f}")
    assert done_p == full and done_l < full and done_s < full
