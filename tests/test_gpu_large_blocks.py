"""Blocks above the single-launch size limits (GPU): the two-level (Schur complement) block
inversion and the row-blocked (TSQR) least squares, reached at small sizes by lowering the
limit (HSS2D_PANEL_LIMIT), give the operator and the inverse of the single-launch kernels.
At the Lippmann-Schwinger configuration's 512 x 512 grid the root block (~17400 embedded
rows) and the top interpolation systems (~21000 rows) need them."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _laplace():
    from hssc_directsolver_gb300 import hss2d as G2, kernels as GK
    return G2.HSS2DParams(Ng=8, npan=8, kernel=GK.Kernel("SL_L_2D", 2.0 / 64, GK.Modulation(),
                                                          GK.Modulation(0.5, 0, 0, 20.0)))


def _helmholtz():
    from tests.test_gpu_hss2d_helmholtz import _params
    return _params(8, rule="rand")[0]


@pytest.mark.parametrize("case,limit", [("laplace", "400"), ("helmholtz", "1200")])
def test_large_block_paths_match_single_launch(gpu, monkeypatch, case, limit):
    from hssc_directsolver_gb300 import hss2d as G2
    prm = _laplace() if case == "laplace" else _helmholtz()
    r = np.random.default_rng(4)
    x = r.standard_normal((prm.N, 2))
    if case == "helmholtz":
        x = x + 1j * r.standard_normal((prm.N, 2))

    def run():
        t = G2.HSS2D_invert_nsym(G2.HSS2D_build_tree_nsym(prm))
        y = G2.HSS2D_apply_nsym(t, None, x)
        return y, G2.HSS2D_applyinv_nsym(t, None, y)

    y0, z0 = run()
    monkeypatch.setenv("HSS2D_PANEL_LIMIT", limit)
    y1, z1 = run()
    rel = lambda a, b: np.linalg.norm(a - b) / np.linalg.norm(b)
    print(f"{case}: apply {rel(y1, y0):.2e}, inverse {rel(z1, z0):.2e}, round trip {rel(z1, x):.2e}")
    assert rel(y1, y0) <= 1e-12
    assert rel(z1, x) <= 1e-10
    assert rel(z1, z0) <= 1e-10
