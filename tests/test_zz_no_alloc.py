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


def _inv(torch, L, fn, A, n, batch):
    dA = torch.from_numpy(np.ascontiguousarray(A)).cuda()
    info = torch.full((batch,), 7, dtype=torch.int32, device="cuda")
    L.check(fn(L.ptr(dA), n, batch, L.ptr(info), None))
    torch.cuda.synchronize()
    return dA.cpu().numpy(), info.cpu().numpy()


def _free_device_bytes():
    """cudaMemGetInfo's free bytes, read through the CUDA runtime itself."""
    import torch
    free, _ = torch.cuda.mem_get_info()
    return free


def test_noalloc_inverse_matches_allocating_inverse_twice(gpu):
    import torch
    from hssc_directsolver_gb300 import _lib as L
    lib = L.lib()
    rng = np.random.default_rng(42)
    for n, batch in ((100, 3), (257, 2)):     # second call reuses the scratch left by the first
        A = rng.standard_normal((batch, n, n)) + 0.1 * n * np.eye(n)[None]
        ref, info_ref = _inv(torch, L, lib.hss_batched_inverse_device, A, n, batch)
        got, info = _inv(torch, L, lib.hss_batched_inverse_noalloc_device, A, n, batch)
        assert np.all(info == 0) and np.all(info_ref == 0)
        assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()
        for b in range(batch):
            assert np.abs(got[b].T @ A[b].T - np.eye(n)).max() < 1e-12


def test_noalloc_allocates_no_device_memory(gpu):
    """After one call on the device, further calls leave cudaMemGetInfo's free bytes unchanged."""
    import torch
    from hssc_directsolver_gb300 import _lib as L
    lib = L.lib()
    n, batch = 200, 4
    A = np.random.default_rng(3).standard_normal((batch, n, n)) + 0.1 * n * np.eye(n)[None]
    dA = torch.from_numpy(np.ascontiguousarray(A)).cuda()
    info = torch.zeros(batch, dtype=torch.int32, device="cuda")
    L.check(lib.hss_batched_inverse_noalloc_device(L.ptr(dA), n, batch, L.ptr(info), None))  # set-up call
    torch.cuda.synchronize()
    before = _free_device_bytes()
    for _ in range(3):
        dA.copy_(torch.from_numpy(np.ascontiguousarray(A)))
        L.check(lib.hss_batched_inverse_noalloc_device(L.ptr(dA), n, batch, L.ptr(info), None))
    torch.cuda.synchronize()
    assert _free_device_bytes() == before
    assert int(info.abs().sum()) == 0


def _largest_accepted_n(lib, L, dA, info):
    """Largest n for one matrix: rejected calls return HSS_ERR_ARG before any work."""
    lo, hi = 1, 1500                           # 1500^2 doubles alone exceed the 16 MiB array
    assert lib.hss_batched_inverse_noalloc_device(L.ptr(dA), hi, 1, L.ptr(info), None) == L.HSS_ERR_ARG
    import torch
    while hi - lo > 1:
        mid = (lo + hi) // 2
        # only size checks run for n >= the answer; for smaller n the call inverts the
        # identity written into the leading mid*mid entries of the buffer
        dA[: mid * mid].copy_(torch.eye(mid, dtype=torch.float64, device="cuda").reshape(-1))
        rc = lib.hss_batched_inverse_noalloc_device(L.ptr(dA), mid, 1, L.ptr(info), None)
        if rc == L.HSS_OK:
            lo = mid
        else:
            assert rc == L.HSS_ERR_ARG
            hi = mid
    return lo


def test_noalloc_size_limit_edges(gpu):
    """The largest accepted size matches the allocating inversion; the next size up is
    rejected with a message naming the scratch, and its matrix is left untouched."""
    import torch
    from hssc_directsolver_gb300 import _lib as L
    lib = L.lib()
    cap = 1500
    buf = torch.zeros(cap * cap, dtype=torch.float64, device="cuda")
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    n = _largest_accepted_n(lib, L, buf, info)
    assert 1300 < n < 1500
    A = np.random.default_rng(11).standard_normal((1, n, n)) + 0.1 * n * np.eye(n)[None]
    ref, info_ref = _inv(torch, L, lib.hss_batched_inverse_device, A, n, 1)
    got, info_got = _inv(torch, L, lib.hss_batched_inverse_noalloc_device, A, n, 1)
    assert info_ref[0] == 0 and info_got[0] == 0
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()
    m = n + 1
    B = np.random.default_rng(12).standard_normal((m, m))
    dB = torch.from_numpy(np.ascontiguousarray(B)).cuda()
    info.fill_(5)
    assert lib.hss_batched_inverse_noalloc_device(L.ptr(dB), m, 1, L.ptr(info), None) == L.HSS_ERR_ARG
    assert b"scratch" in lib.hss_last_error()
    torch.cuda.synchronize()
    assert np.array_equal(dB.cpu().numpy(), B)
    assert int(info[0]) == 5


def test_noalloc_rejects_sizes_beyond_the_scratch(gpu):
    import torch
    from hssc_directsolver_gb300 import _lib as L
    lib = L.lib()
    n = 1500                                   # 1500^2 doubles alone exceed the 16 MiB array
    dA = torch.zeros((n, n), dtype=torch.float64, device="cuda")
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    assert lib.hss_batched_inverse_noalloc_device(L.ptr(dA), n, 1, L.ptr(info), None) == L.HSS_ERR_ARG
    assert b"scratch" in lib.hss_last_error()
