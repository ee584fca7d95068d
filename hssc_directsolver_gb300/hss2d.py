"""HSS2D host interface mirroring the reference's MATLAB entry points.

    params    = HSS_tree_parameters(pot, kh, sym, Ng, np, acc, lay, n_cut, TI)
    INFO_TREE = HSS2D_build_tree_nsym(params)
    A_HSS     = HSS2D_compress_nsym(INFO_TREE, params)
    A_HSS     = HSS2D_invert_nsym(INFO_TREE, params)          (params.Fopts = 'dense')
    Y         = HSS2D_apply_nsym(INFO_TREE, A_HSS, X, params)
    Y         = HSS2D_applyinv_nsym(INFO_TREE, A_HSS, X, params)
    X, hist   = Iterative_Refinement(...)                      (hss2d_solve)

(Common/HSS_tree_parameters.m:1, HSS2D/HSS2D_build_tree_nsym.m:1,
HSS2D_compress_nsym.m:1, HSS2D_invert_nsym.m:1, HSS2D_apply_nsym.m:1,
HSS2D_applyinv_nsym.m:1, Common/Iterative_Refinement.m:1).  Every stage runs
in libhssgpu.so on the GPU; INFO_TREE owns the device state.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
import math

import numpy as np

from . import _lib as L
from .kernels import Kernel, Modulation, reference_modulations


@dataclass
class HSS2DParams:
    """The params struct of Common/HSS_tree_parameters.m:115-139 (dense path fields)."""

    Ng: int
    npan: int
    acc: float = 1e-10
    layers: int = 2
    kernel: Kernel = field(default_factory=Kernel)
    INTERform: str = "dense"
    transinv: int = 0
    sym: int = 0
    precision: str = "fp64"   # "fp64", "mixed", "dfloat" (FP64 factors, paired-FP32 solve products)
                              # or "dfloat_inv" (also the inversion in paired FP32) or "tc"
                              # (FP64 factors, inverse-apply products on the tensor cores)
    n_cut: int = 400
    Fopts: str = "dense"
    k_cut: int = 2500         # low-rank T only where k < k_cut
    seed: int = 0             # key of the randomized ID's Gaussian samples
    proxy_rule: str = "bdry"  # params.proxy_rule: "bdry", "rand" (sampled layers) or "wdec" (Whitney-thinned)
    skel_rule: str = "bdry"   # params.skel_rule: "bdry", "rand" (sampled box points), "wdec" (Whitney) or "ID" (kh > 0)
    lambda_: float = 2.0      # params.lambda of the "rand" rule

    @property
    def h(self) -> float:
        return 2.0 / (self.Ng * self.npan)

    @property
    def depth(self) -> int:
        return int(round(2 * (math.log(self.npan) / math.log(2) - 1) + 3)) - 1

    @property
    def N(self) -> int:
        return self.npan * self.npan * self.Ng * self.Ng

    def to_c(self) -> L.hss2d_params:
        forms = {"dense": L.HSS_INTER_DENSE, "lowrank": L.HSS_INTER_LOWRANK}
        if self.INTERform not in forms:
            raise ValueError("INTERform must be 'dense' or 'lowrank'")
        if self.Fopts != "dense":
            raise ValueError("Fopts 'dense' (HSS-D) is the implemented inverse storage")
        prec = {"fp64": L.HSS_PREC_FP64, "mixed": L.HSS_PREC_MIXED, "dfloat": L.HSS_PREC_DFLOAT,
                "dfloat_inv": L.HSS_PREC_DFLOAT_INV, "tc": L.HSS_PREC_TC}[self.precision]
        k = self.kernel
        k.h = self.h
        rules = {"bdry": L.HSS_PROXY_BDRY, "rand": L.HSS_PROXY_RAND, "wdec": L.HSS_PROXY_WDEC}
        if self.proxy_rule not in rules:
            raise ValueError("proxy_rule must be 'bdry', 'rand' or 'wdec'")
        skels = {"bdry": L.HSS_SKEL_BDRY, "rand": L.HSS_SKEL_RAND, "ID": L.HSS_SKEL_ID, "wdec": L.HSS_SKEL_WDEC}
        if self.skel_rule not in skels:
            raise ValueError("skel_rule must be 'bdry', 'rand', 'wdec' or 'ID'")
        return L.hss2d_params(self.Ng, self.npan, self.layers, forms[self.INTERform], self.transinv, self.sym, prec,
                              0, float(self.acc), k.to_c(), int(self.k_cut), 0, int(self.seed),
                              rules[self.proxy_rule], 0, float(self.lambda_), skels[self.skel_rule], 0)

    @property
    def complex(self) -> bool:
        """The Helmholtz / Lippmann-Schwinger operator (SL_H_2D) is complex."""
        return self.kernel.flag_pot == "SL_H_2D"


def HSS_tree_parameters(pot: str, kh: float, sym: int, Ng: int, npan: int, acc: float, lay: int, n_cut: int,
                        TI: int, proxy: int = 0) -> HSS2DParams:
    """Common/HSS_tree_parameters.m:108-139.  kh > 0: the Lippmann-Schwinger kernel SL_H_2D
    with the order-4 Duan-Rokhlin diagonal and the bump contrast of LOCAL_get_bc, dense T
    (the complex GPU tree's interpolation form)."""
    if kh != 0:
        from .kernels import helmholtz_kernel
        return HSS2DParams(Ng=Ng, npan=npan, acc=acc, layers=lay, kernel=helmholtz_kernel(kh, sym, Ng, npan, TI, proxy),
                           transinv=TI, sym=sym, n_cut=n_cut, INTERform="dense")
    # transinv = 1 keeps one factor set per tree level (INFO_TREE.LEV); the kernel has b = c = 1
    b, c = reference_modulations(sym, proxy, TI)
    # INTERform 'lowrank' and k_cut 2500 are the reference's defaults (HSS_tree_parameters.m:131-134)
    return HSS2DParams(Ng=Ng, npan=npan, acc=acc, layers=lay, kernel=Kernel(pot, 2.0 / (Ng * npan), b, c),
                       transinv=TI, sym=sym, n_cut=n_cut, INTERform="lowrank", k_cut=2500)


class InfoTree:
    """INFO_TREE (and the A_HSS factors once compressed / inverted) on the GPU."""

    def __init__(self, params: HSS2DParams):
        self.params = params
        self._h = C.c_void_p()
        self._cp = params.to_c()
        L.check(L.lib().hss2d_build_tree(C.byref(self._h), C.byref(self._cp)))
        d, nb, n = C.c_int32(), C.c_int32(), C.c_int64()
        L.check(L.lib().hss2d_info(self._h, C.byref(d), C.byref(nb), C.byref(n)))
        self.depth, self.nboxes, self.N = d.value, nb.value, n.value
        self.complex = params.complex
        self.compressed = False
        self.inverted = False

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                L.lib().hss2d_destroy(h)
            except Exception:
                pass
            self._h = None

    def box_sizes(self):
        n = np.zeros(self.nboxes, np.int32)
        k = np.zeros(self.nboxes, np.int32)
        p = np.zeros(self.nboxes, np.int32)
        ip = lambda a: a.ctypes.data_as(L._I32P)
        L.check(L.lib().hss2d_box_sizes(self._h, ip(n), ip(k), ip(p)))
        return n, k, p

    def phase_times(self):
        """Host wall seconds: tree geometry, uploads, interpolation operators, compress, invert."""
        t = np.zeros(5)
        L.check(L.lib().hss2d_phase_times(self._h, t.ctypes.data_as(L._DP)))
        return t

    def set_autotune(self, on: bool = True):
        """Tune the K split of every batched solve product when a solve plan is built
        (``hss2d_set_autotune``)."""
        L.check(L.lib().hss2d_set_autotune(self._h, 1 if on else 0))

    def interp_ranks(self):
        """(q_up, q_dn): rank of each box's low-rank T_up / T_dn, -1 where T is dense."""
        qu = np.zeros(self.nboxes, np.int32)
        qd = np.zeros(self.nboxes, np.int32)
        L.check(L.lib().hss2d_interp_ranks(self._h, qu.ctypes.data_as(L._I32P), qd.ctypes.data_as(L._I32P)))
        return qu, qd

    def export_box(self, box: int):
        n, k, _ = self.box_sizes()
        nb, kb = int(n[box]), int(k[box])
        dt = np.complex128 if self.complex else np.float64
        out = dict(I_src=np.zeros(nb, np.int32), J=np.zeros(nb, np.int32),
                   T_up=np.zeros((kb, nb - kb), dtype=dt, order="F"), T_dn=np.zeros((kb, nb - kb), dtype=dt, order="F"))
        ip = lambda a: a.ctypes.data_as(L._I32P)
        dp = lambda a: a.ctypes.data_as(L._DP)
        L.check(L.lib().hss2d_export_box(self._h, box, ip(out["I_src"]), ip(out["J"]), dp(out["T_up"]),
                                         dp(out["T_dn"])))
        return out

    def export_inverse(self, box: int):
        n, k, _ = self.box_sizes()
        nb, kb = int(n[box]), int(k[box])
        dt = np.complex128 if self.complex else np.float64
        FI = np.zeros((nb, nb), dtype=dt, order="F")
        E = np.zeros((kb, kb), dtype=dt, order="F")
        L.check(L.lib().hss2d_export_inverse(self._h, box, FI.ctypes.data_as(L._DP), E.ctypes.data_as(L._DP)))
        return FI, E

    def solve_bytes(self) -> int:
        b = C.c_int64()
        L.check(L.lib().hss2d_solve_bytes(self._h, C.byref(b)))
        return b.value

    def solve_launches(self, nrhs: int) -> int:
        n = C.c_int32()
        L.check(L.lib().hss2d_solve_launches(self._h, nrhs, C.byref(n)))
        return n.value


def levHSS(INFO_TREE: InfoTree, n_cut: int, trinv: int = 0) -> int:
    """lev_HSS = levHSS(INFO_TREE, n_cut, trinv), HSS2D/levHSS.m:33-65: the first tree
    level whose smallest skeleton is <= n_cut (forced even), -1 when the top boxes are
    already below it.  It selects where the compressed-block (HSS-C) inverse would start."""
    _, k, _ = INFO_TREE.box_sizes()
    n_min = max(int(k[0]), int(k[1]), int(k[2]))
    lev = 0
    while n_min > n_cut and lev < INFO_TREE.depth - 1:
        lev += 1
        n_min = int(k[2 ** lev - 1:2 ** (lev + 1) - 1].min())
    if lev > 0:
        return lev - 1 if lev % 2 == 1 else lev
    return -1


def HSS2D_build_tree_nsym(params: HSS2DParams) -> InfoTree:
    return InfoTree(params)


def HSS2D_compress_nsym(INFO_TREE: InfoTree, params: HSS2DParams | None = None) -> InfoTree:
    L.check(L.lib().hss2d_compress(INFO_TREE._h))
    INFO_TREE.compressed = True
    return INFO_TREE


def HSS2D_invert_nsym(INFO_TREE: InfoTree, params: HSS2DParams | None = None) -> InfoTree:
    if not INFO_TREE.compressed:
        HSS2D_compress_nsym(INFO_TREE, params)
    L.check(L.lib().hss2d_invert(INFO_TREE._h))
    INFO_TREE.inverted = True
    return INFO_TREE


def _vec(INFO_TREE, X):
    """Column-major N x r vectors in the tree's arithmetic: complex128 for a complex tree
    (passed to the library as interleaved (re, im) doubles), float64 otherwise."""
    dt = np.complex128 if INFO_TREE.complex else np.float64
    X = np.asfortranarray(np.asarray(X, dtype=dt))
    vec = X.ndim == 1
    X2 = X.reshape(INFO_TREE.N, -1, order="F")
    return X2, vec


def _out(X2, vec):
    return X2[:, 0] if vec else X2


def HSS2D_apply_nsym(INFO_TREE: InfoTree, A_HSS, X, params=None) -> np.ndarray:
    X2, vec = _vec(INFO_TREE, X)
    Y = np.zeros_like(X2, order="F")
    L.check(L.lib().hss2d_apply(INFO_TREE._h, L.ptr(X2), L.ptr(Y), X2.shape[1]))
    return _out(Y, vec)


def HSS2D_applyinv_nsym(INFO_TREE: InfoTree, A_HSS, X, params=None) -> np.ndarray:
    X2, vec = _vec(INFO_TREE, X)
    Y = np.zeros_like(X2, order="F")
    L.check(L.lib().hss2d_applyinv(INFO_TREE._h, L.ptr(X2), L.ptr(Y), X2.shape[1]))
    return _out(Y, vec)


def HSS2D_gmres(INFO_TREE: InfoTree, F, tol: float = 1e-8, restart: int = 30, maxit: int = 200,
                PRECOND: InfoTree | None = None):
    """x = A^-1 f by restarted GMRES on INFO_TREE's forward operator, right-preconditioned by
    the inverse apply of PRECOND (an inverted tree; INFO_TREE itself in "mixed" precision is
    the Lippmann-Schwinger configuration's complex64 inverse), complex128 on a complex tree
    (the reference's Krylov solves: HSS2D/Test/Test_HSS2D_InverseCompression.m:201-228).
    Returns (x, relres, iterations)."""
    F2, vec = _vec(INFO_TREE, F)
    Xs = np.zeros_like(F2, order="F")
    rr = C.c_double()
    it = C.c_int32()
    L.check(L.lib().hss2d_gmres(INFO_TREE._h, PRECOND._h if PRECOND is not None else None, L.ptr(F2), L.ptr(Xs),
                                F2.shape[1], float(tol), int(restart), int(maxit), C.byref(rr), C.byref(it)))
    return _out(Xs, vec), rr.value, it.value


def HSS2D_kernel_residual_rows(INFO_TREE: InfoTree, row0: int, F_rows, X) -> float:
    """max over columns of ||f - K x|| / ||f|| over the rows row0 .. row0 + len(F_rows) only:
    the kernel-matrix residual on a sample of rows (O(rows N) work)."""
    dt = np.complex128 if INFO_TREE.complex else np.float64
    Fr = np.asfortranarray(np.asarray(F_rows, dtype=dt))
    Fr = Fr.reshape(Fr.shape[0], -1, order="F")
    X2, _ = _vec(INFO_TREE, X)
    assert Fr.shape[1] == X2.shape[1]
    rr = C.c_double()
    L.check(L.lib().hss2d_kernel_residual_rows(INFO_TREE._h, int(row0), Fr.shape[0], L.ptr(Fr), L.ptr(X2),
                                               X2.shape[1], C.byref(rr)))
    return rr.value


def proxy_points(params: HSS2DParams, box: int, n_src: int) -> np.ndarray:
    """LOCAL_Build_Proxy of one box (host computation): the proxy points (p x 2) of heap box
    ``box`` with ``n_src`` sources under params' proxy rule."""
    cp = params.to_c()
    cap = 1 << 22
    xy = np.zeros(2 * cap)
    cnt = C.c_int32()
    L.check(L.lib().hss2d_proxy_points(C.byref(cp), int(box), int(n_src), xy.ctypes.data_as(L._DP), cap,
                                       C.byref(cnt)))
    n = cnt.value
    return np.stack([xy[:n], xy[cap:cap + n]], axis=1)


def HSS2D_solve(INFO_TREE: InfoTree, F, tol: float = 1e-10, maxit: int = 5):
    """x = A^-1 f with iterative refinement (Common/Iterative_Refinement.m:20-35).

    Returns (x, relres, solves used)."""
    F2, vec = _vec(INFO_TREE, F)
    Xs = np.zeros_like(F2, order="F")
    rr = C.c_double()
    it = C.c_int32()
    L.check(L.lib().hss2d_solve(INFO_TREE._h, L.ptr(F2), L.ptr(Xs), F2.shape[1], tol, maxit, C.byref(rr),
                                C.byref(it)))
    return _out(Xs, vec), rr.value, it.value


def HSS2D_kernel_residual(INFO_TREE: InfoTree, F, X) -> float:
    """max over columns of ||f - K x|| / ||f|| with K the kernel matrix of the grid itself
    (Kernel_Eval entries generated in FP64 on the GPU and applied on the fly, never formed):
    the residual of HSS2D/Test/Test_HSS2D_InverseCompression.m:300-324 against the dense
    operator rather than the compressed one."""
    F2, _ = _vec(INFO_TREE, F)
    X2, _ = _vec(INFO_TREE, X)
    assert F2.shape == X2.shape
    rr = C.c_double()
    L.check(L.lib().hss2d_kernel_residual(INFO_TREE._h, L.ptr(F2), L.ptr(X2), F2.shape[1], C.byref(rr)))
    return rr.value


def HSS2D_bicgstab(INFO_TREE: InfoTree, F, tol: float = 1e-10, maxit: int = 200, PRECOND: InfoTree | None = None):
    """[x, flag, relres, iter] = bicgstab(Mapp, F, tol, maxit, Iapp) of the reference's
    iterative solution (HSS2D/Test/Test_HSS2D_InverseCompression.m:201-228): Mapp is the
    forward apply of INFO_TREE's compressed operator, Iapp the inverse apply of PRECOND
    (an inverted tree, e.g. the translation-invariant one).  Returns (x, relres, iters)."""
    F2, vec = _vec(INFO_TREE, F)
    Xs = np.zeros_like(F2, order="F")
    rr = C.c_double()
    it = C.c_int32()
    L.check(L.lib().hss2d_bicgstab(INFO_TREE._h, PRECOND._h if PRECOND is not None else None, L.ptr(F2), L.ptr(Xs),
                                   F2.shape[1], float(tol), int(maxit), C.byref(rr), C.byref(it)))
    return (Xs[:, 0] if vec else Xs), rr.value, it.value
