"""The allocation-free batched inversion, checked against the allocating one (GPU).

For callers that cannot allocate device memory while they run (their device
memory belongs to their own pool allocator, or allocation would synchronise
the device in a latency-bound loop): hss_batched_inverse_noalloc_device takes
its scratch from a fixed array in device global memory.  Two calls in a row
must each match hss_batched_inverse_device, which allocates its workspace, to
the tolerance of the other inversion tests; this file is collected last.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _inv(torch, L, lib, fn, A, n, batch):
    dA = torch.from_numpy(np.ascontiguousarray(A)).cuda()
    info = torch.full((batch,), 7, dtype=torch.int32, device="cuda")
    L.check(fn(L.ptr(dA), n, batch, L.ptr(info), None))
    torch.cuda.synchronize()
    return dA.cpu().numpy(), info.cpu().numpy()


def test_noalloc_inverse_matches_allocating_inverse_twice(gpu):
    import torch
    from hssc_directsolver_gb300 import _lib as L
    lib = L.lib()
    rng = np.random.default_rng(42)
    for n, batch in ((100, 3), (257, 2)):     # second call reuses the scratch left by the first
        A = rng.standard_normal((batch, n, n)) + 0.1 * n * np.eye(n)[None]
        ref, info_ref = _inv(torch, L, lib, lib.hss_batched_inverse_device, A, n, batch)
        got, info = _inv(torch, L, lib, lib.hss_batched_inverse_noalloc_device, A, n, batch)
        assert np.all(info == 0) and np.all(info_ref == 0)
        assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()
        for b in range(batch):
            assert np.abs(got[b].T @ A[b].T - np.eye(n)).max() < 1e-12


def test_noalloc_rejects_sizes_beyond_the_scratch(gpu):
    import torch
    from hssc_directsolver_gb300 import _lib as L
    lib = L.lib()
    n = 1500                                   # 1500^2 doubles alone exceed the 16 MiB array
    dA = torch.zeros((n, n), dtype=torch.float64, device="cuda")
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    assert lib.hss_batched_inverse_noalloc_device(L.ptr(dA), n, 1, L.ptr(info), None) == L.HSS_ERR_ARG
    assert b"scratch" in lib.hss_last_error()
