"""Entry points called from several host threads at once (GPU).

The library sets its per-device state (function attributes of the cluster panels) once
per device under a lock, and the Helmholtz kernel's quadrature weights travel in the
kernel's parameters.  Two host threads that each evaluate the Helmholtz kernel and invert
large blocks (the cluster-panel path) must get the same results as one thread does.
"""
import math
import threading

import numpy as np
import pytest

from oracle import geometry as OG

pytestmark = pytest.mark.gpu


def _work(seed):
    import torch
    from hssc_directsolver_gb300 import _lib as L, kernels as GK
    lib = L.lib()
    rng = np.random.default_rng(seed)
    S = OG.grid_source(8, 4)
    T = S[rng.choice(len(S), 200, replace=False)]
    k = GK.helmholtz_kernel(20.0, 0, 8, 4, 0, order=4)
    A = GK.Kernel_Eval(T, S, k)
    n, batch = 1100, 2                         # above 256 rows: the cluster Gauss-Jordan panel
    M = rng.standard_normal((batch, n, n)) + 0.1 * n * np.eye(n)[None]
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        dM = torch.from_numpy(np.ascontiguousarray(M)).cuda()
        info = torch.zeros(batch, dtype=torch.int32, device="cuda")
    s.synchronize()
    L.check(lib.hss_batched_inverse_device(L.ptr(dM), n, batch, L.ptr(info), s.cuda_stream))
    s.synchronize()
    return A, dM.cpu().numpy(), info.cpu().numpy()


def test_two_host_threads_match_one(gpu):
    ref = [_work(seed) for seed in (1, 2)]
    out = [None, None]
    errs = []

    def run(i, seed):
        try:
            out[i] = _work(seed)
        except Exception as e:  # pragma: no cover - reported below
            errs.append(e)

    th = [threading.Thread(target=run, args=(i, seed)) for i, seed in enumerate((1, 2))]
    for t in th:
        t.start()
    for t in th:
        t.join()
    assert not errs, errs
    for (A0, M0, i0), (A1, M1, i1) in zip(ref, out):
        assert np.all(i0 == 0) and np.all(i1 == 0)
        assert np.array_equal(A0, A1)          # same kernel, same points: bit-equal
        assert np.array_equal(M0, M1)          # deterministic inversion
        assert np.isfinite(A0).all() and np.abs(A0).max() > 0 and math.isfinite(np.abs(M0).max())
