"""LOCAL_Build_Proxy on the host (no GPU): the library's proxy points of a box equal the
oracle's, point for point, for the 'bdry' rule (build_box_proxy.m:52-88 with the layer count
of HSS2D_build_tree_nsym.m:360-368, Laplace and kh > 0), the 'rand' rule (LOCAL_Build_Proxy
:883-905 over LOCAL_random_sampler :964-1001: the Mersenne Twister reset to seed 5489 on every
call, its 53-bit uniforms) and the 'wdec' rule (:877-881 over
Common/Whitney_decomposition_1Dcurve.m)."""
import numpy as np
import pytest

from oracle import hss2d as O2, kernels as OK


def _both(npan, kh, rule, lam=2.0, layers=3):
    from hssc_directsolver_gb300 import hss2d as G2, kernels as GK
    flag = "SL_H_2D" if kh > 0 else "SL_L_2D"
    gp = G2.HSS2DParams(Ng=8, npan=npan, layers=layers, kernel=GK.Kernel(flag, 2.0 / (8 * npan), kh=kh),
                        proxy_rule=rule, lambda_=lam)
    kp = OK.KernelParams(flag=OK.SL_H_2D if kh > 0 else OK.SL_L_2D, h=gp.h, kh=kh)
    op = O2.HSS2DParams(Ng=8, npan=npan, kp=kp, layers=layers, proxy_rule=rule, lambda_=lam)
    return gp, op


def _oracle_proxy(op, box, n_src):
    lev = int(np.floor(np.log2(box + 1)))
    colrad, rowrad = O2.box_radii(lev)
    cent = O2.box_centers(op.depth)
    Xp = O2.build_box_proxy(cent[box], colrad, rowrad, O2.lay_prox(op, lev), op.h)
    if op.proxy_rule == "rand":
        Xp = O2.random_proxy(Xp, n_src, cent[box], colrad, rowrad, lev, op)
    elif op.proxy_rule == "wdec":
        Xp = Xp[O2.whitney_curve_mask(Xp, cent[box], np.array([colrad, rowrad]), 2 * op.layers, op.h)]
    return Xp


@pytest.mark.parametrize("npan,kh,rule", [(4, 0.0, "bdry"), (8, 0.0, "bdry"), (8, 20.0, "bdry"),
                                          (4, 0.0, "rand"), (8, 20.0, "rand"), (16, 20.0, "rand"),
                                          (4, 0.0, "wdec"), (8, 0.0, "wdec"), (8, 20.0, "wdec")])
def test_proxy_points_equal_oracle(npan, kh, rule):
    from hssc_directsolver_gb300 import hss2d as G2
    gp, op = _both(npan, kh, rule)
    depth = op.depth
    boxes = sorted({1, 2, 5, 2 ** (depth - 1) - 1 + 3, 2 ** depth - 1, 2 ** (depth + 1) - 2})
    for box in boxes:
        for n_src in (64, 150, 400):
            got = G2.proxy_points(gp, box, n_src)
            want = _oracle_proxy(op, box, n_src)
            assert got.shape == want.shape, (box, n_src, got.shape, want.shape)
            assert np.array_equal(got, want), (box, n_src)


def test_rand_rule_retries_with_smaller_lambda():
    """A target above what one sampling keeps makes the rule sample again with 0.9 lambda
    (and again on the previous sample); the count then reaches ceil(2/3 n) or stops after 10."""
    from hssc_directsolver_gb300 import hss2d as G2
    gp, op = _both(8, 20.0, "rand", lam=6.0)
    for box in (1, 4, 20):
        for n_src in (100, 2000):
            got = G2.proxy_points(gp, box, n_src)
            assert np.array_equal(got, _oracle_proxy(op, box, n_src))


def test_grid_points_equal_oracle_source_points():
    from oracle.geometry import grid_source
    from hssc_directsolver_gb300.geometry import grid_points
    for Ng, npan in ((8, 4), (7, 8), (8, 32)):
        assert np.array_equal(grid_points(Ng, npan), grid_source(Ng, npan))
