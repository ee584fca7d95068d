#!/usr/bin/env python3
"""Benchmark of the HSS2D direct-solver hot path on GB300.

Workload (the HSS2D plain-FP64 configuration): volume integral equation
u + int log|x-y| b(y) u(y) dy = f on [-1,1]^2, 256 x 256 midpoint grid (Ng = 8
points per panel side, 32 x 32 panels, N = 65536, leaf 8 x 8), Laplace kernel
(den==0) + h^2/2 log(den) c(y) with c(y) = 1 + 0.5 exp(-|y|^2/0.05) (NTI,
nsym), two boundary layers, ID tolerance 1e-10, 4 right-hand sides N(0,1)
(seed 0, unit columns as the reference test normalises them).

One step = one direct solve of the 4 right-hand sides to a max-column relative
residual <= 1e-10 against the FP64 forward HSS operator (inverse apply +
residual + refinement rounds when needed), with the inverse factors resident in
HBM.  value = solves/s.  compress+invert seconds (tree with interpolation
operators, kernel blocks, inverse factors) are measured beside it for the plain
FP64 and the mixed (FP32 factors + FP64 refinement) paths.

Inputs are larger than L2: the factors read by every solve are ~1.9 GB (FP64)
or ~0.94 GB (FP32) against a 129 MB L2, so no flush is needed between steps.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "compress+invert s and solves/s at 1e-10 residual: mixed/batched vs plain FP64"

# DRAM bytes (read + write) of the skinny-product kernels of one inverse apply at this
# workload, summed over the kernels of one ncu capture (dram__bytes_read.sum +
# dram__bytes_write.sum per launch)
TRAFFIC_PER_APPLYINV = {"dfloat": 2.0057e9, "dfloat_inv": 2.0057e9, "fp64": 1.9471e9}
WORKLOAD = "HSS2D 256x256 grid (Ng=8, 32x32 panels, N=65536), leaf 8x8, tol 1e-10, 4 RHS"


def workload_params(precision: str, npan: int = 32):
    from hssc_directsolver_gb300 import hss2d as G2, kernels as GK
    Ng = 8
    h = 2.0 / (Ng * npan)
    return G2.HSS2DParams(Ng=Ng, npan=npan, acc=1e-10, layers=2,
                          kernel=GK.Kernel("SL_L_2D", h, GK.Modulation(), GK.Modulation(0.5, 0.0, 0.0, 20.0)),
                          precision=precision)


def rhs(N: int, nrhs: int = 4, seed: int = 0) -> np.ndarray:
    F = np.random.default_rng(seed).standard_normal((N, nrhs))
    F /= np.linalg.norm(F, axis=0, keepdims=True)
    return np.asfortranarray(F)


# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int = 0):
        self.gpu = gpu_index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                if out.returncode == 0 and out.stdout.strip():
                    self.samples.append([x.strip() for x in out.stdout.strip().split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4)
                          if len(s) > 3 + i and s[3 + i].lower().startswith("active")})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


# ---------------------------------------------------------------------------
def cpu_model() -> str:
    """The host CPU's model name (the CPU baseline's hardware)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=5).stdout
        for line in out.splitlines():
            k, _, v = line.partition(":")
            if k.strip() == "Model name" and v.strip():
                return v.strip()
    except Exception:
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                k, _, v = line.partition(":")
                if k.strip() in ("model name", "Model", "CPU part") and v.strip():
                    return v.strip()
    except OSError:
        pass
    import platform
    return platform.processor() or platform.machine()


def cpu_sample(npan: int = 32, nrhs: int = 4, budget_s: float = 20.0):
    """One step of the GPU arm on the host cores: the oracle's inverse apply
    (HSS2D_applyinv_nsym restated in NumPy), its forward apply (HSS2D_apply_nsym, the
    refinement's residual operator) and the residual norms, over factors and blocks of the
    workload's exact shapes.  Factors and blocks are random (the applies' cost does not
    depend on their values), so the sample is bounded by the solve itself rather than the
    oracle's ~60 s factorization."""
    from oracle import hss2d as O2, kernels as OK
    prm = O2.HSS2DParams(Ng=8, npan=npan, acc=1e-10, layers=2,
                         kp=OK.KernelParams(flag=OK.SL_L_2D, h=2.0 / (8 * npan)))
    tree = O2.build_tree_nsym(prm, with_T=False)
    rng = np.random.default_rng(1)
    nb = tree.nboxes
    for b in range(nb):
        if b > 0:
            k, n = tree.k[b], len(tree.J[b])
            tree.T_up[b] = rng.standard_normal((k, n - k)) * 1e-2
            tree.T_dn[b] = rng.standard_normal((k, n - k)) * 1e-2
    inv = {"FI": [None] * nb, "E": [None] * nb}
    for b in range(nb):
        n, k = len(tree.J[b]), tree.k[b]
        inv["FI"][b] = rng.standard_normal((n, n)) * (1.0 / n)
        if b > 0:
            inv["E"][b] = rng.standard_normal((k, k)) * (1.0 / k)
    Bs, B12, B21 = {}, {}, {}
    for b in range(nb):
        if tree.is_leaf(b):
            n = len(tree.I_src[b])
            Bs[b] = rng.standard_normal((n, n)) * (1.0 / n)
        else:
            c1, c2 = tree.children(b)
            B12[b] = rng.standard_normal((tree.k[c1], tree.k[c2])) * 1e-3
            B21[b] = rng.standard_normal((tree.k[c2], tree.k[c1])) * 1e-3
    blk = O2.HSS2DBlocks(Bs, B12, B21)
    F = rhs(prm.N, nrhs)

    def step():
        x = O2.applyinv_nsym(tree, inv, F)
        r = F - O2.apply_nsym(tree, blk, x)
        return np.linalg.norm(r, axis=0).max() / np.linalg.norm(F, axis=0).min()

    step()  # warm
    times = []
    t_end = time.perf_counter() + budget_s
    while time.perf_counter() < t_end or len(times) < 2:
        t0 = time.perf_counter()
        step()
        times.append(time.perf_counter() - t0)
        if len(times) >= 50:
            break
    return float(np.median(times)), len(times)


def cpu_compress_invert(npan: int = 32):
    """Seconds of the oracle's tree build (interpolation operators), compress and invert
    (HSS2D_build_tree_nsym / HSS2D_compress_nsym / HSS2D_invert_nsym restated in NumPy,
    dense T) on the workload's grid and kernel, on the host cores: the CPU side of the
    metric's compress+invert comparison."""
    from oracle import hss2d as O2, kernels as OK
    h = 2.0 / (8 * npan)
    kp = OK.KernelParams(flag=OK.SL_L_2D, h=h, c=OK.Modulation(0.5, 0.0, 0.0, 20.0))
    prm = O2.HSS2DParams(Ng=8, npan=npan, kp=kp, layers=2, acc=1e-10, INTERform="dense")
    t0 = time.perf_counter()
    tree = O2.build_tree_nsym(prm)
    blk = O2.compress_nsym(tree, prm)
    O2.invert_nsym(tree, prm, blk)
    return time.perf_counter() - t0


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    cores = os.cpu_count() or 1
    os.environ.setdefault("OPENBLAS_NUM_THREADS", str(cores))
    steps = []
    t_solve, n = cpu_sample(budget_s=max(5.0, 2.0 * (args.steps + args.warmup)))
    value = 1.0 / t_solve
    t_ci = cpu_compress_invert(args.npan) if not args.no_cpu_ci else None
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_solve * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "nrhs": 4, "l2": "inputs larger than L2"},
        "cpu_baseline": {"value": value, "unit": "solves/s", "cores": cores, "kind": "port", "cpu": cpu_model(),
                         "sample": f"oracle HSS2D_applyinv_nsym + HSS2D_apply_nsym residual (NumPy/OpenBLAS) over "
                                   f"factors and blocks of the workload's shapes, {n} timed steps of 4 RHS, median"},
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    if t_ci is not None:
        line["compress_invert_s"] = {"fp64": t_ci}
        line["cpu_baseline"]["compress_invert_s"] = t_ci
        line["cpu_baseline"]["compress_invert_sample"] = ("oracle build_tree (dense T) + compress + invert at the "
                                                          "full workload, once")
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
def bench_batched(args, L, dev):
    """The batched-curves workload: 512 double-layer curves r = 1 + sum_k a_k cos(k t + phi_k)
    (a_k ~ U(0, 0.3/k), k <= 8), N log-uniform in [1024, 16384], leaf 64, tol 1e-10, 8 RHS per
    curve, all curves compressed / inverted / solved as one forest: the IDs' QR in FP64 and in
    double-float (timed; the second forest is kept), the inversion in FP64 and in double-float,
    every solve refined to 1e-10 against the FP64 forward operator."""
    import torch
    from hssc_directsolver_gb300 import hss1d as G1, kernels as GK, geometry as GG
    Xs, sizes = GG.batched_curves(args.curves, seed=0)
    torch.cuda.synchronize()
    # the IDs' pivoted QR in FP64 (the reference's arithmetic), then in double-float; the
    # second forest is the one inverted and solved
    tf0 = time.perf_counter()
    H64 = G1.HSS1D_compress_batch(Xs, 64, 1e-10, GK.Kernel("DL_L_2D"))
    compress_fp64_id = time.perf_counter() - tf0
    k64 = H64.info()["kskel"]
    del H64
    t0 = time.perf_counter()
    H = G1.HSS1D_compress_batch(Xs, 64, 1e-10, GK.Kernel("DL_L_2D"), id_precision="dfloat")
    t1 = time.perf_counter()
    rank_agree = float((H.info()["kskel"] == k64).mean())
    # FP64 inversion (timed solves in the fp64 and dfloat paths), then the double-float
    # inversion the dfloat_inv path solves with (both refine to 1e-10 in two solves)
    H.set_precision("fp64")
    ti0 = time.perf_counter()
    G1.HSS1D_invert_nsym(H)
    torch.cuda.synchronize()
    invert_fp64 = time.perf_counter() - ti0
    Nt = sum(sizes)
    F = np.random.default_rng(0).standard_normal((8, Nt))
    dF = torch.from_numpy(F).to(dev)
    dX = torch.zeros_like(dF)
    stream = torch.cuda.current_stream(dev)
    sp = C.c_void_p(stream.cuda_stream)
    rr = C.c_double()
    it = C.c_int32()

    def solve():
        L.check(L.lib().hss1d_solve_device(H._h, L.ptr(dF), L.ptr(dX), 8, 1e-10, 4, C.byref(rr), C.byref(it), sp))

    out = {}
    inv_s = {"fp64": invert_fp64, "dfloat": invert_fp64}
    for prec in ("fp64", "dfloat", "dfloat_inv"):
        H.set_precision(prec)
        if prec == "dfloat_inv":
            torch.cuda.synchronize()
            ti0 = time.perf_counter()
            G1.HSS1D_invert_nsym(H)
            torch.cuda.synchronize()
            inv_s[prec] = time.perf_counter() - ti0
        for _ in range(2):
            solve()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        steps = max(3, args.steps // 4)
        e0.record(stream)
        for _ in range(steps):
            solve()
        e1.record(stream)
        torch.cuda.synchronize()
        out[prec] = (e0.elapsed_time(e1) / steps, rr.value, it.value)
    ok = [p for p in out if out[p][1] <= 1e-10]
    # fastest solve, then the cheaper inversion among equally fast solves
    best = min(ok, key=lambda p: (round(out[p][0], 1), inv_s[p])) if ok else "fp64"
    ms, rel, used = out[best]
    return {"workload": f"{args.curves} Laplace double-layer curves, N log-uniform [1024,16384] "
                        f"(total {Nt}), leaf 64, tol 1e-10, 8 RHS each, one forest",
            "compress_s": t1 - t0, "invert_s": inv_s[best], "compress_invert_s": t1 - t0 + inv_s[best],
            "invert_s_by_path": inv_s,
            "id_precision": "dfloat", "compress_s_fp64_id": compress_fp64_id,
            "ranks_equal_to_fp64_id": rank_agree,
            "solve_ms": ms, "solves_per_s": 1e3 / ms, "relres": rel, "solves_used": used, "path": best,
            "solve_ms_by_path": {p: out[p][0] for p in out}, "dtype": "f64"}


def bench_kernel_gen(L, dev, m=8192, n=8192, reps=3):
    """Kernel_Eval throughput (entries/s) on device buffers: the Laplace log kernel and the
    complex Lippmann-Schwinger kernel (H0 with the order-4 Duan-Rokhlin diagonal)."""
    import torch
    from hssc_directsolver_gb300 import kernels as GK
    rng = np.random.default_rng(0)
    X1 = torch.tensor(rng.uniform(-1, 1, (2, m)), dtype=torch.float64, device=dev)  # x row, y row
    X2 = torch.tensor(rng.uniform(-1, 1, (2, n)), dtype=torch.float64, device=dev)
    out = {}
    for name, k in (("SL_L_2D", GK.Kernel("SL_L_2D", 2.0 / 256, GK.Modulation(0.25, 0.3, 0.6, 1.0))),
                    ("SL_H_2D", GK.helmholtz_kernel(20.0, 0, 8, 32, 0))):
        A = torch.empty((2 if name == "SL_H_2D" else 1) * m * n, dtype=torch.float64, device=dev)
        kp = k.to_c()
        sp = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        call = lambda: L.check(L.lib().hss_kernel_eval_device(C.byref(kp), L.ptr(X1), m, L.ptr(X2), n,  # noqa: E731
                                                             L.ptr(A), sp))
        call()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            call()
        torch.cuda.synchronize()
        dt = (time.perf_counter() - t0) / reps
        out[name] = {"entries_per_s": m * n / dt, "ms": dt * 1e3,
                     "bytes_written_gbs": A.numel() * 8 / dt / 1e9}
        del A
    out["block"] = f"{m} x {n} random points in [-1,1]^2, kh = 20 for SL_H_2D, FP64 entries"
    out["bound"] = "fp64 pipe (log / series and Hankel-integral H0 in FP64); call includes the point upload"
    return out


def bench_hss1d_algebra(N=32768, M=24576, r=16, leaf=64, acc=1e-10):
    """Seconds of the HSS1D algebra entry points on one star curve (Laplace double layer):
    compress, transpose, A + A^T (HSS1D_sum_nsym), U V^T (HSS1D_compressLR_nsym), the
    low-rank update A + U V^T, and the rectangular K(Xin, Xout) between the curve and the
    curve scaled by 1.2 (HSS1D_compress_rectangular_nsym) with its 8-column apply."""
    from hssc_directsolver_gb300 import hss1d as G1, kernels as GK, geometry as GG
    rng = np.random.default_rng(0)
    X = GG.star_curve(N)
    Xin = GG.star_curve(M).copy()
    Xin[:, :2] *= 1.2
    Xin[:, 4] *= 1.2
    Xin[:, 5] /= 1.2
    U, V = rng.standard_normal((N, r)), rng.standard_normal((N, r))
    k = GK.Kernel("DL_L_2D")
    out = {"workload": f"star curve N={N} (rows of the rectangular case: M={M}, the curve scaled by 1.2), "
                       f"leaf {leaf}, tol {acc:g}, U V^T of rank {r}; host wall seconds per call"}
    t = time.perf_counter
    t0 = t()
    A = G1.HSS1D_compress_nsym("green", X, leaf, acc, k)
    t1 = t()
    At = G1.HSS1D_transpose(A)
    t2 = t()
    S = G1.HSS1D_sum_nsym(A, At, acc)
    t3 = t()
    H = G1.HSS1D_compressLR_nsym(U, V, leaf, acc)
    t4 = t()
    C2 = G1.HSS1D_sum_nsym(A, H, acc)
    t5 = t()
    R = G1.HSS1D_compress_rectangular_nsym("green", Xin, X, leaf, acc, k)
    t6 = t()
    q = rng.standard_normal((N, 8))
    G1.HSS1D_apply_rect_nsym(R, q)
    t7 = t()
    G1.HSS1D_apply_rect_nsym(R, q)
    t8 = t()
    out.update(compress_s=t1 - t0, transpose_s=t2 - t1, sum_AAt_s=t3 - t2, compress_lr_s=t4 - t3,
               sum_lowrank_update_s=t5 - t4, compress_rect_s=t6 - t5, apply_rect_8rhs_ms=(t8 - t7) * 1e3,
               max_rank={"A": int(A.info()["kskel"][1:].max()), "A+A^T": int(S.info()["kskel"][1:].max()),
                         "A+UV^T": int(C2.info()["kskel"][1:].max()),
                         "rect_in": int(R.rect_info()["kskel_in"][1:].max())})
    del A, At, S, H, C2, R
    return out


def bench_config5(args, L, dev):
    """The learned-rank configuration at scale: 2048 double-layer curves (N log-uniform in
    [2048, 32768], ~23 M points) compressed plainly and with the rank MLP trained on the
    ranks of a 256-curve batched compress, plus the 1024 x 1024 HSS2D grid
    (N = 1,048,576) in the double-float inversion mode.  Reports seconds and the QR steps
    the network saved; the adaptive ID still decides every rank."""
    import torch
    from hssc_directsolver_gb300 import hss1d as G1, hss2d as G2, kernels as GK, geometry as GG
    from hssc_directsolver_gb300.rank_mlp import RankPredictor, training_set
    kern = GK.Kernel("DL_L_2D")
    Xt, _ = GG.batched_curves(256, nmin=1024, nmax=16384, seed=1)
    Ht = G1.HSS1D_compress_batch(Xt, 64, 1e-10, kern)
    Ft, yt = training_set(Ht)
    del Ht
    P = RankPredictor(seed=0)
    t0 = time.perf_counter()
    loss = P.train(Ft, yt, epochs=100, batch=512, lr=3e-3)
    t_train = time.perf_counter() - t0
    Xs, ss = GG.batched_curves(2048, nmin=2048, nmax=32768, seed=5)
    out = {"curves": {"workload": f"2048 Laplace double-layer curves, N log-uniform [2048,32768] (total "
                                  f"{sum(ss)}), leaf 64, tol 1e-10",
                      "mlp": {"train_boxes": int(len(yt)), "train_s": t_train, "loss": loss}}}
    for mode in ("plain", "learned"):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        H = G1.HSS1D_compress_batch(Xs, 64, 1e-10, kern, predictor=(P if mode == "learned" else None))
        t1 = time.perf_counter()
        H.set_precision("dfloat_inv")
        G1.HSS1D_invert_nsym(H)
        t2 = time.perf_counter()
        f = np.random.default_rng(0).standard_normal((sum(ss), 1))
        _, rr, it = G1.HSS1D_solve(H, f, 1e-10, 4)
        done, full, reruns = H.id_stats()
        out["curves"][mode] = {"compress_s": t1 - t0, "invert_s": t2 - t1, "relres": rr, "solves_used": it,
                               "qr_steps": done, "qr_steps_full": full, "reruns": reruns}
        del H
    prm = workload_params("dfloat_inv", 128)
    t0 = time.perf_counter()
    tree = G2.HSS2D_build_tree_nsym(prm)
    G2.HSS2D_compress_nsym(tree)
    G2.HSS2D_invert_nsym(tree)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    F = rhs(prm.N)
    _, rr, it = G2.HSS2D_solve(tree, F, 1e-10, 6)
    t2 = time.perf_counter()
    _, rr, it = G2.HSS2D_solve(tree, F, 1e-10, 6)
    t3 = time.perf_counter()
    out["hss2d_1024"] = {"workload": "HSS2D 1024x1024 grid (N=1048576), dfloat_inv", "compress_invert_s": t1 - t0,
                         "solve_s_host_buffers": t3 - t2, "relres": rr, "solves_used": it,
                         "factor_bytes_per_solve": tree.solve_bytes()}
    return out


def bench_lippmann_schwinger(npan: int = 64, kh: float = 20.0):
    """The Lippmann-Schwinger configuration: kh = 20, the Gaussian contrast exp(-|x|^2/0.1)
    taken symmetrically, the order-4 Duan-Rokhlin diagonal, (8 npan)^2 grid with leaf 8 x 8,
    tol 1e-10, 'rand' proxies, dense T; compress and invert in HSS_PREC_MIXED (FP32 inverse
    factors: the complex64 inverse), complex128 GMRES on the compressed operator to 1e-8
    preconditioned by that inverse.  Reports the stage seconds, GMRES steps and time, the
    relative residual against the compressed operator and against the kernel matrix itself
    on three samples of 4096 rows (the full O(N^2) product is not formed)."""
    import torch
    from hssc_directsolver_gb300 import hss2d as G2, kernels as GK
    h = 2.0 / (8 * npan)
    _, w, _ = GK.DR_stencil(h, kh, 8 * npan, 4)
    sq = GK.Modulation(alpha=1.0, isig=5.0, kind=GK.MOD_GAUSS0)
    prm = G2.HSS2DParams(Ng=8, npan=npan, layers=3, acc=1e-10, INTERform="dense", precision="mixed",
                         kernel=GK.Kernel("SL_H_2D", h, sq, sq, kh, complex(w[0])), proxy_rule="rand")
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    tree = G2.HSS2D_build_tree_nsym(prm)
    G2.HSS2D_compress_nsym(tree)
    G2.HSS2D_invert_nsym(tree)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    ph = tree.phase_times()
    from hssc_directsolver_gb300.geometry import grid_points
    X = grid_points(8, npan)
    f = np.exp(-(X[:, 0] ** 2 + X[:, 1] ** 2) / 0.2) * np.exp(1j * kh * X[:, 0])
    F = np.stack([f, np.random.default_rng(0).standard_normal(prm.N) + 0j], axis=1)
    G2.HSS2D_gmres(tree, F[:, :1], tol=1e-8, restart=30, maxit=60, PRECOND=tree)  # warm the plans
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    x, rr, its = G2.HSS2D_gmres(tree, F, tol=1e-8, restart=30, maxit=60, PRECOND=tree)
    t3 = time.perf_counter()
    kr = []
    for row0 in (0, prm.N // 2 - 2048, prm.N - 4096):
        kr.append(G2.HSS2D_kernel_residual_rows(tree, row0, F[row0:row0 + 4096], x))
    n, k, _ = tree.box_sizes()
    return {"workload": f"HSS2D Lippmann-Schwinger kappa={kh:g}, contrast exp(-|x|^2/0.1) (symmetric), "
                        f"{8 * npan}x{8 * npan} grid (N={prm.N}), leaf 8x8, tol 1e-10, 'rand' proxies, dense T",
            "precision": "compress/invert HSS_PREC_MIXED (FP32 inverse factors), complex128 GMRES",
            "compress_invert_s": t1 - t0,
            "stages_s": {"tree_geometry_and_ID": float(ph[0]), "uploads": float(ph[1]),
                         "interpolation_lstsq": float(ph[2]), "compress": float(ph[3]), "invert": float(ph[4])},
            "gmres": {"nrhs": 2, "steps": its, "s_host_buffers": t3 - t2, "relres_compressed_operator": rr,
                      "restart": 30, "tol": 1e-8},
            "kernel_relres_rows": {"rows": "3 samples of 4096 rows (start, middle, end)", "values": kr},
            "root_n": int(n[0]), "root_k_children": int(k[1])}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--npan", type=int, default=32)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true", help="skip the 512-curve batched HSS1D section")
    ap.add_argument("--curves", type=int, default=512)
    ap.add_argument("--no-algebra", action="store_true", help="skip the HSS1D algebra section")
    ap.add_argument("--no-cpu-ci", action="store_true",
                    help="skip the CPU oracle's compress+invert (about a minute at the full workload)")
    ap.add_argument("--no-ls", action="store_true",
                    help="skip the Lippmann-Schwinger (complex HSS2D, 512 x 512) section")
    ap.add_argument("--ls-npan", type=int, default=64)
    ap.add_argument("--only-ls", action="store_true",
                    help="run only the Lippmann-Schwinger section and print its JSON (profiling)")
    ap.add_argument("--config5", action="store_true",
                    help="also run the learned-rank configuration at scale (2048 curves, 1024^2 grid; ~1 min)")
    ap.add_argument("--paths", default="fp64,mixed,dfloat,dfloat_inv,tc",
                    help="solve paths to measure (comma list of fp64, mixed, dfloat, dfloat_inv, tc)")
    ap.add_argument("--no-kernel-residual", action="store_true",
                    help="skip the FP64 residual against the kernel matrix itself (~0.5 s per path)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.only_ls:
        print(json.dumps({"lippmann_schwinger": bench_lippmann_schwinger(args.ls_npan)}), flush=True)
        return

    import torch
    import torch.distributed as dist
    from hssc_directsolver_gb300 import _lib as L, hss2d as G2

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()

    def max_over_ranks(x: float) -> float:
        if world == 1:
            return x
        t = torch.tensor([x], dtype=torch.float64, device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    F = rhs(workload_params("fp64", args.npan).N)
    results = {}
    paths = [p for p in args.paths.split(",") if p]
    for prec in paths:
        prm = workload_params(prec, args.npan)
        # built twice: the first build of a process also pays the first use of each kernel
        # (module loading, one-time attributes); the second, warm build is the one reported
        first_ci = None
        for rep in range(2):
            tree = None
            barrier()
            t0 = time.perf_counter()
            tree = G2.HSS2D_build_tree_nsym(prm)
            t1 = time.perf_counter()
            G2.HSS2D_compress_nsym(tree)
            t2 = time.perf_counter()
            G2.HSS2D_invert_nsym(tree)
            torch.cuda.synchronize()
            t3 = time.perf_counter()
            if rep == 0:
                first_ci = max_over_ranks(t3 - t0)
        ci = max_over_ranks(t3 - t0)
        # the solve plans tune their K splits when first built (in the warm-up solves)
        tree.set_autotune(True)
        dF = torch.from_numpy(F.T.copy()).to(dev)  # (nrhs, N) row-major == N x nrhs column-major
        dX = torch.zeros_like(dF)
        rr = C.c_double()
        it = C.c_int32()
        stream = torch.cuda.current_stream(dev)
        sp = C.c_void_p(stream.cuda_stream)

        def solve():
            L.check(L.lib().hss2d_solve_device(tree._h, L.ptr(dF), L.ptr(dX), dF.shape[0], 1e-10, 10,
                                               C.byref(rr), C.byref(it), sp))

        for _ in range(args.warmup):
            solve()
        barrier()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        with ClockSampler(local) as clk:
            ev0.record(stream)
            for _ in range(args.steps):
                solve()
            ev1.record(stream)
            torch.cuda.synchronize()
        ms = ev0.elapsed_time(ev1) / args.steps
        ms = max_over_ranks(ms)
        # inverse apply alone (the chain of skinny factor products) for the roofline
        dY = torch.zeros_like(dF)
        for _ in range(3):
            L.check(L.lib().hss2d_applyinv_device(tree._h, L.ptr(dF), L.ptr(dY), dF.shape[0], sp))
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            L.check(L.lib().hss2d_applyinv_device(tree._h, L.ptr(dF), L.ptr(dY), dF.shape[0], sp))
        e1.record(stream)
        torch.cuda.synchronize()
        inv_ms = e0.elapsed_time(e1) / args.steps
        # forward FP64 apply (the refinement residual operator)
        e0.record(stream)
        for _ in range(args.steps):
            L.check(L.lib().hss2d_apply_device(tree._h, L.ptr(dY), L.ptr(dX), dF.shape[0], sp))
        e1.record(stream)
        torch.cuda.synchronize()
        fwd_ms = e0.elapsed_time(e1) / args.steps
        # end to end through the C ABI with host buffers (H2D of f, D2H of x each step)
        # pinned host buffers: (nrhs, N) row-major storage viewed as the N x nrhs
        # column-major arrays the C ABI takes
        Fp = torch.empty((F.shape[1], F.shape[0]), dtype=torch.float64, pin_memory=True)
        Xp = torch.empty((F.shape[1], F.shape[0]), dtype=torch.float64, pin_memory=True)
        Fp.numpy()[:] = np.asarray(F).T
        Xp.zero_()
        Fh = Fp.numpy().T
        Xh = Xp.numpy().T
        assert Fh.flags.f_contiguous and Xh.flags.f_contiguous
        rr2 = C.c_double()
        it2 = C.c_int32()
        for _ in range(2):
            L.check(L.lib().hss2d_solve(tree._h, L.ptr(Fh), L.ptr(Xh), Fh.shape[1], 1e-10, 10, C.byref(rr2),
                                        C.byref(it2)))
        barrier()
        te0 = time.perf_counter()
        for _ in range(args.steps):
            L.check(L.lib().hss2d_solve(tree._h, L.ptr(Fh), L.ptr(Xh), Fh.shape[1], 1e-10, 10, C.byref(rr2),
                                        C.byref(it2)))
        barrier()
        e2e_s = max_over_ranks((time.perf_counter() - te0) / args.steps)
        # the solution's residual against the kernel matrix itself (generated on the fly in
        # FP64, never formed), outside the timed region
        kres = None
        if not args.no_kernel_residual:
            kres = G2.HSS2D_kernel_residual(tree, F, np.asfortranarray(Xh))
        gm = None
        if prec == "mixed":
            # the FP32 inverse as a GMRES preconditioner instead of the refinement's
            # preconditioner-only iteration (host buffers, like e2e)
            Fg = np.asfortranarray(F)
            G2.HSS2D_gmres(tree, Fg, tol=1e-10, restart=20, maxit=40, PRECOND=tree)
            tg0 = time.perf_counter()
            for _ in range(max(1, args.steps // 4)):
                _, grr, gits = G2.HSS2D_gmres(tree, Fg, tol=1e-10, restart=20, maxit=40, PRECOND=tree)
            gm = {"ms_host_buffers": (time.perf_counter() - tg0) / max(1, args.steps // 4) * 1e3, "steps": gits,
                  "relres": grr}
        results[prec] = dict(kernel_relres=kres, compress_invert_s=ci, first_compress_invert_s=first_ci, tree_s=t1 - t0, compress_s=t2 - t1, invert_s=t3 - t2, gmres=gm,
                             solve_ms=ms, relres=rr.value, solves_used=it.value, applyinv_ms=inv_ms,
                             apply_ms=fwd_ms,
                             solve_bytes=tree.solve_bytes(), launches=tree.solve_launches(dF.shape[0]),
                             e2e_s=e2e_s, e2e_relres=rr2.value, clocks=clk.summary())
        del tree
        torch.cuda.empty_cache()

    batched = None
    if not args.no_batched:
        batched = bench_batched(args, L, dev)
    kgen = bench_kernel_gen(L, dev) if rank == 0 else None
    algebra = None
    if rank == 0 and not args.no_algebra:
        try:
            algebra = bench_hss1d_algebra()
        except Exception as e:  # the section is reported, never allowed to drop the bench line
            algebra = {"error": str(e)}

    ok = [p for p in results if results[p]["relres"] <= 1e-10]
    best = min(ok, key=lambda p: results[p]["solve_ms"]) if ok else next(iter(results))
    r = results[best]
    peaks = {}
    try:
        with open(os.path.join(HERE, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except Exception:
        pass
    hbm = peaks.get("hbm_gbs")
    peak_src = "measured" if hbm else "fallback"
    hbm = hbm or 6800.0
    achieved = r["solve_bytes"] / (r["applyinv_ms"] * 1e-3) / 1e9
    N = workload_params("fp64", args.npan).N
    nrhs = F.shape[1]
    launches_per_solve = r["launches"] * r["solves_used"]
    line = {
        "metric": METRIC, "value": 1e3 / r["solve_ms"] * world, "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["solve_ms"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": {"mixed": "f32+f64", "dfloat": "f64 (products as f32 pairs)",
                  "dfloat_inv": "f64 (products and inversion as f32 pairs)",
                  "tc": "f64 (inverse-apply products as bf16 digit slices on tensor cores, exact fp32 "
                        "accumulation)"}.get(best, "f64"),
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "nrhs": nrhs, "path": best, "parallelism": f"replicas{world}",
                   "l2": "inputs larger than L2 (factors %.2f GB per solve)" % (r["solve_bytes"] / 1e9)},
        "compress_invert_s": {p: results[p]["compress_invert_s"] for p in results},
        "compress_invert_first_build_s": {p: results[p]["first_compress_invert_s"] for p in results},
        "stages_s": {p: {k: results[p][k] for k in ("tree_s", "compress_s", "invert_s")} for p in results},
        "solves_per_s": {p: 1e3 / results[p]["solve_ms"] for p in results},
        "mixed_gmres": results.get("mixed", {}).get("gmres"),
        "relres": {p: results[p]["relres"] for p in results},
        "kernel_relres": {p: results[p]["kernel_relres"] for p in results},
        "solves_used": {p: results[p]["solves_used"] for p in results},
        "applyinv_ms": {p: results[p]["applyinv_ms"] for p in results},
        "apply_fp64_ms": {p: results[p]["apply_ms"] for p in results},
        "e2e": {"value": 1.0 / r["e2e_s"] * world, "unit": "solves/s",
                "h2d_bytes_per_step": int(N * nrhs * 8), "d2h_bytes_per_step": int(N * nrhs * 8),
                "host_buffers": "pinned", "call": "hss2d_solve"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": TRAFFIC_PER_APPLYINV.get(best),
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of the inverse apply's "
                                       "kernels, summed over one capture of this workload's solve; not measured "
                                       "in this run",
                     "kernel": {"dfloat": "k_skinny_df", "dfloat_inv": "k_skinny_df", "tc": "k_skinny_tc",
                                "mixed": "k_skinny<float>"}.get(best, "k_skinny<double>")
                               + " chain of one inverse apply",
                     "peak_source": peak_src,
                     "algorithmic_bytes": r["solve_bytes"]},
        "gpu_launches": int(args.steps * launches_per_solve),
        "clocks": r["clocks"],
    }
    if batched is not None:
        line["batched_hss1d"] = batched
    if kgen is not None:
        line["kernel_gen"] = kgen
    if algebra is not None:
        line["hss1d_algebra"] = algebra
    if not args.no_ls:
        try:
            line["lippmann_schwinger"] = bench_lippmann_schwinger(args.ls_npan)
        except Exception as e:  # reported, not fatal: the headline line still prints
            line["lippmann_schwinger"] = {"error": str(e)}
    if args.config5:
        line["config5"] = bench_config5(args, L, dev)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:  # the CPU baseline is an N=1 figure
        try:
            cores = os.cpu_count() or 1
            t_cpu, n_cpu = cpu_sample(args.npan, nrhs, budget_s=15.0)
            line["cpu_baseline"] = {"value": 1.0 / t_cpu, "unit": "solves/s", "cores": cores, "kind": "port",
                                    "cpu": cpu_model(),
                                    "sample": f"oracle HSS2D_applyinv_nsym + HSS2D_apply_nsym residual over factors "
                                              f"and blocks of the workload's shapes, {n_cpu} steps of 4 RHS, median"}
            if not args.no_cpu_ci:
                try:
                    t_ci = cpu_compress_invert(args.npan)
                    line["cpu_baseline"]["compress_invert_s"] = t_ci
                    line["cpu_baseline"]["compress_invert_sample"] = ("oracle build_tree (dense T) + compress + "
                                                                      "invert at the full workload, once")
                except Exception as e:  # reported, never required
                    line["cpu_baseline"]["compress_invert_sample"] = f"failed: {e}"
        except Exception as e:  # the CPU baseline is reported, never required
            line["cpu_baseline"] = {"value": None, "unit": "solves/s", "cores": os.cpu_count(), "kind": "port",
                                    "sample": f"failed: {e}"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
