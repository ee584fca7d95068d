"""HSS1D host interface mirroring the reference's MATLAB entry points.

    K_HSS          = HSS1D_compress_nsym('green', X, TREE, acc, knl_params)
    [HSSinv,FTinv] = HSS1D_invert_nsym(K_HSS, acc)
    uu             = HSS1D_apply_nsym(K_HSS, qq)
    xx             = HSS1D_applyinv_nsym(K_HSS, HSSinv, FTinv, ff)
    K_HSS          = HSS1D_compress_rectangular_nsym('green', Xin, Xout, TREE, acc, params)
    uu             = HSS1D_apply_rect_nsym(K_HSS, qq)

(HSS1D/HSS1D_compress_nsym.m:1, HSS1D_invert_nsym.m:1, HSS1D_apply_nsym.m:1,
HSS1D_applyinv_nsym.m:1, HSS1D_compress_rectangular_nsym.m:1, HSS1D_apply_rect_nsym.m:1).  All work runs in libhssgpu.so on the GPU; the
returned K_HSS object owns the device factors.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from .kernels import Kernel


class HSS1DMatrix:
    """K_HSS: tree, skeletons, interpolation matrices and self/sibling blocks on the GPU."""

    def __init__(self, handle: C.c_void_p, N: int):
        self._h = handle
        self.N = N
        self.inverted = False
        flag = C.c_int32(0)
        L.check(L.lib().hss1d_is_complex(handle, C.byref(flag)))
        # a complex (SL_H_2D) matrix takes and returns complex128 vectors
        self.complex = bool(flag.value)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                L.lib().hss1d_destroy(h)
            except Exception:
                pass
            self._h = None

    # --- box_constants.m rows -------------------------------------------------
    def info(self):
        lib = L.lib()
        nb = C.c_int32(0)
        L.check(lib.hss1d_info(self._h, C.byref(nb), *([None] * 8)))
        n = nb.value
        arrs = {k: np.zeros(n, dtype=np.int32) for k in
                ("level", "parent", "c1", "c2", "off", "cnt", "nskel", "kskel")}
        p = lambda a: a.ctypes.data_as(L._I32P)
        L.check(lib.hss1d_info(self._h, C.byref(nb), p(arrs["level"]), p(arrs["parent"]), p(arrs["c1"]),
                               p(arrs["c2"]), p(arrs["off"]), p(arrs["cnt"]), p(arrs["nskel"]),
                               p(arrs["kskel"])))
        arrs["nboxes"] = n
        return arrs

    def rect_info(self):
        """Row side (K_HSS rows 16:19): M and per box off_in, cnt_in, nskel_in, kskel_in
        (the column side again on a square matrix)."""
        n = self.info()["nboxes"]
        M = C.c_int64()
        arrs = {k: np.zeros(n, dtype=np.int32) for k in ("off_in", "cnt_in", "nskel_in", "kskel_in")}
        p = lambda a: a.ctypes.data_as(L._I32P)
        L.check(L.lib().hss1d_rect_info(self._h, C.byref(M), p(arrs["off_in"]), p(arrs["cnt_in"]),
                                        p(arrs["nskel_in"]), p(arrs["kskel_in"])))
        arrs["M"] = M.value
        return arrs

    def export_box(self, box: int):
        inf = self.info()
        rinf = self.rect_info()
        n, k = int(inf["nskel"][box]), int(inf["kskel"][box])
        nd, kd = int(rinf["nskel_in"][box]), int(rinf["kskel_in"][box])
        dt = np.complex128 if self.complex else np.float64
        out = dict(I_SKUP=np.zeros(k, np.int32), I_SKDN=np.zeros(kd, np.int32),
                   J_UP=np.zeros(n, np.int32), J_DN=np.zeros(nd, np.int32),
                   T_UP=np.zeros((k, n - k), dt, order="F"), T_DN=np.zeros((kd, nd - kd), dt, order="F"))
        ip = lambda a: a.ctypes.data_as(L._I32P)
        dp = lambda a: a.ctypes.data_as(L._DP)
        L.check(L.lib().hss1d_export_box(self._h, box, ip(out["I_SKUP"]), ip(out["I_SKDN"]), ip(out["J_UP"]),
                                         ip(out["J_DN"]), dp(out["T_UP"]), dp(out["T_DN"])))
        return out

    def set_precision(self, precision: str):
        """'fp64', 'dfloat' (double-float apply / inverse-apply products) or 'dfloat_inv'
        (also the next hss1d_invert's updates and products in double-float)."""
        code = {"fp64": L.HSS_PREC_FP64, "dfloat": L.HSS_PREC_DFLOAT, "dfloat_inv": L.HSS_PREC_DFLOAT_INV}[precision]
        L.check(L.lib().hss1d_set_precision(self._h, code))

    # --- learned ranks ----------------------------------------------------------
    def features(self):
        """(nboxes x 8 rank features, k/n of each box's plain ID) of the last compress."""
        n = self.info()["nboxes"]
        F = np.zeros((n, 8), np.float32)
        y = np.zeros(n, np.float32)
        L.check(L.lib().hss1d_features(self._h, L.ptr(F), L.ptr(y)))
        return F, y

    def phase_times(self):
        """Host wall seconds of the last compress: setup, level geometry, level uploads,
        level GPU work, level bookkeeping, final blocks."""
        t = np.zeros(6)
        L.check(L.lib().hss1d_phase_times(self._h, t.ctypes.data_as(L._DP)))
        return t

    def id_stats(self):
        """(QR steps done, QR steps of full factorizations, boxes redone in full)."""
        a, b, c = C.c_int64(), C.c_int64(), C.c_int32()
        L.check(L.lib().hss1d_id_stats(self._h, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value


def _as_f64(a):
    a = np.asarray(a, dtype=np.float64)
    return np.asfortranarray(a)


def _vec(K_HSS: HSS1DMatrix, a, rows=None):
    """Column-major rows x r vectors in the matrix's arithmetic (complex128 for a complex
    matrix, passed to the library as interleaved (re, im) doubles) and whether a was 1-D."""
    dt = np.complex128 if K_HSS.complex else np.float64
    a = np.asfortranarray(np.asarray(a, dtype=dt))
    return a.reshape(K_HSS.N if rows is None else rows, -1, order="F"), a.ndim == 1


def HSS1D_compress_nsym(type_: str, X, TREE: int, acc: float, knl_params: Kernel, seed: int = 0) -> HSS1DMatrix:
    if type_ != "green":
        raise ValueError("only the 'green' construction is implemented on the GPU")
    X = np.asarray(X, dtype=np.float64)
    if X.ndim != 2 or X.shape[1] not in (2, 6):
        raise ValueError("X must be N x 2 or N x 6 ([x y nx ny w kappa])")
    if X.shape[1] == 2:
        X6 = np.zeros((X.shape[0], 6))
        X6[:, :2] = X
        X = X6
    Xf = np.asfortranarray(X)
    h = C.c_void_p()
    kp = knl_params.to_c()
    L.check(L.lib().hss1d_compress(C.byref(h), L.ptr(Xf), Xf.shape[0], Xf.shape[0], int(TREE), float(acc),
                                   C.byref(kp), int(seed)))
    return HSS1DMatrix(h, Xf.shape[0])


def HSS1D_compress_fsym(type_: str, X, TREE: int, acc: float, knl_params: Kernel, seed: int = 0) -> HSS1DMatrix:
    """K_HSS = HSS1D_compress_fsym('green', X, TREE, acc, knl_params): one ID per box, for
    kernels the caller treats as symmetric (HSS1D/HSS1D_compress_fsym.m:98-248)."""
    if type_ != "green":
        raise ValueError("only the 'green' construction is implemented on the GPU")
    X = np.asarray(X, dtype=np.float64)
    if X.ndim != 2 or X.shape[1] not in (2, 6):
        raise ValueError("X must be N x 2 or N x 6 ([x y nx ny w kappa])")
    if X.shape[1] == 2:
        X6 = np.zeros((X.shape[0], 6))
        X6[:, :2] = X
        X = X6
    Xf = np.asfortranarray(X)
    h = C.c_void_p()
    kp = knl_params.to_c()
    L.check(L.lib().hss1d_compress_fsym(C.byref(h), L.ptr(Xf), Xf.shape[0], Xf.shape[0], int(TREE), float(acc),
                                        C.byref(kp), int(seed)))
    return HSS1DMatrix(h, Xf.shape[0])


def _points6(X):
    X = np.asarray(X, dtype=np.float64)
    if X.ndim != 2 or X.shape[1] not in (2, 6):
        raise ValueError("points must be n x 2 or n x 6 ([x y nx ny w kappa])")
    if X.shape[1] == 2:
        X6 = np.zeros((X.shape[0], 6))
        X6[:, :2] = X
        X = X6
    return np.asfortranarray(X)


def HSS1D_compress_rectangular_nsym(type_: str, Xin, Xout, TREE: int, acc: float, params: Kernel,
                                    seed: int = 0) -> HSS1DMatrix:
    """K_HSS = HSS1D_compress_rectangular_nsym('green', Xin, Xout, TREE, acc, params)
    (HSS1D/HSS1D_compress_rectangular_nsym.m:1): the M x N matrix K(Xin, Xout) with a
    column tree over Xout and a row tree of the same shape over Xin.  Apply it with
    ``HSS1D_apply_rect_nsym``."""
    if type_ != "green":
        raise ValueError("only the 'green' construction is implemented on the GPU")
    Xi, Xo = _points6(Xin), _points6(Xout)
    h = C.c_void_p()
    kp = params.to_c()
    L.check(L.lib().hss1d_compress_rect(C.byref(h), L.ptr(Xi), Xi.shape[0], Xi.shape[0], L.ptr(Xo), Xo.shape[0],
                                        Xo.shape[0], int(TREE), float(acc), C.byref(kp), int(seed)))
    K = HSS1DMatrix(h, Xo.shape[0])
    K.M = Xi.shape[0]
    return K


def HSS1D_apply_rect_nsym(K_HSS: HSS1DMatrix, qq) -> np.ndarray:
    """uu = HSS1D_apply_rect_nsym(K_HSS, qq) (HSS1D/HSS1D_apply_rect_nsym.m:1): qq has N rows
    (Xout), uu has M rows (Xin)."""
    q = _as_f64(qq)
    vec = q.ndim == 1
    q2 = q.reshape(K_HSS.N, -1, order="F")
    out = np.zeros((getattr(K_HSS, "M", K_HSS.N), q2.shape[1]), order="F")
    L.check(L.lib().hss1d_apply(K_HSS._h, L.ptr(q2), L.ptr(out), q2.shape[1]))
    return out[:, 0] if vec else out


def HSS1D_compress_batch(Xs, TREE: int, acc: float, knl_params: Kernel, seeds=None,
                         predictor=None, id_precision: str = "fp64", step_test: bool = False) -> HSS1DMatrix:
    """Many independent curves compressed together (every level of every tree in the
    same launches).  Vectors of the returned matrix are the problems' vectors stacked.
    With a ``RankPredictor`` the IDs stop their pivoted QR early at the predicted rank;
    the result equals the plain compress.  ``step_test=True`` (no predictor) is the
    model-free baseline: every pivoted QR tests the same stop rule at every step.
    ``id_precision="dfloat"`` runs the IDs' pivoted QR in double-float arithmetic (rank, T
    and the randomized check in FP64)."""
    mats = []
    for X in Xs:
        X = np.asarray(X, dtype=np.float64)
        if X.shape[1] == 2:
            X6 = np.zeros((X.shape[0], 6))
            X6[:, :2] = X
            X = X6
        mats.append(np.asfortranarray(X))
    P = len(mats)
    N = (C.c_int64 * P)(*[m.shape[0] for m in mats])
    ptrs = (C.c_void_p * P)(*[m.ctypes.data for m in mats])
    seeds = list(range(P)) if seeds is None else list(seeds)
    sd = (C.c_uint64 * P)(*seeds)
    h = C.c_void_p()
    kp = knl_params.to_c()
    if id_precision != "fp64" or step_test:
        prec = {"fp64": L.HSS_PREC_FP64, "dfloat": L.HSS_PREC_DFLOAT}.get(id_precision)
        if prec is None:
            raise ValueError("id_precision must be 'fp64' or 'dfloat'")
        if step_test:
            prec |= L.HSS_ID_STEP_TEST
        L.check(L.lib().hss1d_compress_batch_ex(C.byref(h), P, N, ptrs, N, int(TREE), float(acc), C.byref(kp), sd,
                                                predictor._h if predictor is not None else None, prec))
    elif predictor is None:
        L.check(L.lib().hss1d_compress_batch(C.byref(h), P, N, ptrs, N, int(TREE), float(acc), C.byref(kp), sd))
    else:
        L.check(L.lib().hss1d_compress_batch_learned(C.byref(h), P, N, ptrs, N, int(TREE), float(acc),
                                                     C.byref(kp), sd, predictor._h))
    M = HSS1DMatrix(h, int(sum(m.shape[0] for m in mats)))
    M.sizes = [m.shape[0] for m in mats]
    return M


def forest_info(K_HSS: HSS1DMatrix):
    P = C.c_int32()
    Nt = C.c_int64()
    L.check(L.lib().hss1d_forest_info(K_HSS._h, C.byref(P), C.byref(Nt), None, None))
    roots = np.zeros(P.value, np.int32)
    base = np.zeros(P.value, np.int64)
    L.check(L.lib().hss1d_forest_info(K_HSS._h, None, None, roots.ctypes.data_as(L._I32P),
                                      base.ctypes.data_as(L._I64P)))
    return roots, base


def HSS1D_invert_nsym(K_HSS: HSS1DMatrix, acc: float = 0.0):
    """Returns (HSSinv, FTinv); both are views of the factors kept inside K_HSS."""
    L.check(L.lib().hss1d_invert(K_HSS._h))
    K_HSS.inverted = True
    return K_HSS, K_HSS


def HSS1D_transforminv_nsym(K_HSS: HSS1DMatrix, HSSinv=None, FTinv=None) -> HSS1DMatrix:
    """Kinv_HSS: the inverse rewritten in K_HSS's compressed format
    (HSS1D/HSS1D_transforminv_nsym.m:38-161); ``HSS1D_apply_nsym(Kinv_HSS, f)`` applies
    the inverse.  HSSinv/FTinv are the factors inside K_HSS (from HSS1D_invert_nsym)."""
    h = C.c_void_p()
    L.check(L.lib().hss1d_transforminv(K_HSS._h, C.byref(h)))
    K = HSS1DMatrix(h, K_HSS.N)
    if hasattr(K_HSS, "sizes"):
        K.sizes = K_HSS.sizes
    return K


def HSS1D_transpose(A_HSS: HSS1DMatrix) -> HSS1DMatrix:
    """At_HSS = HSS1D_transpose(A_HSS) (HSS1D/HSS1D_transpose.m:1): the transpose in compressed
    form, as a new (not inverted) matrix."""
    h = C.c_void_p()
    L.check(L.lib().hss1d_transpose(A_HSS._h, C.byref(h)))
    K = HSS1DMatrix(h, A_HSS.N)
    if hasattr(A_HSS, "sizes"):
        K.sizes = A_HSS.sizes
    return K


def HSS1D_sum_nsym(A_HSS: HSS1DMatrix, B_HSS: HSS1DMatrix, acc: float) -> HSS1DMatrix:
    """C_HSS = HSS1D_sum_nsym(A_HSS, B_HSS, acc) (HSS1D/HSS1D_sum_nsym.m:1): A + B as a new
    compressed matrix on the operands' common tree, re-skeletonized at tolerance acc."""
    h = C.c_void_p()
    L.check(L.lib().hss1d_sum(A_HSS._h, B_HSS._h, float(acc), C.byref(h)))
    K = HSS1DMatrix(h, A_HSS.N)
    if hasattr(A_HSS, "sizes"):
        K.sizes = A_HSS.sizes
    return K


def HSS1D_recompress_nsym(A_HSS: HSS1DMatrix, acc: float) -> HSS1DMatrix:
    """A_NEW = HSS1D_recompress_nsym(A, acc) (HSS1D/HSS1D_recompress_nsym.m:1): A with its
    ranks reduced to what acc needs, as a new (not inverted) compressed matrix."""
    h = C.c_void_p()
    L.check(L.lib().hss1d_recompress(A_HSS._h, float(acc), C.byref(h)))
    K = HSS1DMatrix(h, A_HSS.N)
    if hasattr(A_HSS, "sizes"):
        K.sizes = A_HSS.sizes
    return K


def HSS1D_compressLR_nsym(U, V, TREE: int, acc: float, seed: int = 0) -> HSS1DMatrix:
    """K_HSS = HSS1D_compressLR_nsym(U, V, TREE, acc) (HSS1D/HSS1D_compressLR_nsym.m:1): the
    N x N matrix U V^T in compressed form on the halving tree of leaf size TREE."""
    Uf = np.asfortranarray(np.asarray(U, dtype=np.float64))
    Vf = np.asfortranarray(np.asarray(V, dtype=np.float64))
    if Uf.ndim != 2 or Uf.shape != Vf.shape:
        raise ValueError("U and V must both be N x r")
    h = C.c_void_p()
    L.check(L.lib().hss1d_compress_lr(C.byref(h), L.ptr(Uf), L.ptr(Vf), Uf.shape[0], Uf.shape[1], Uf.shape[0],
                                      Vf.shape[0], int(TREE), float(acc), int(seed)))
    return HSS1DMatrix(h, Uf.shape[0])


def HSS1D_scalarmult(c: float, A_HSS: HSS1DMatrix) -> HSS1DMatrix:
    """A = HSS1D_scalarmult(c, A) (HSS1D/HSS1D_scalarmult.m:1).  The matrix is scaled in place
    (and returned); its inverse factors are dropped, so invert again before applyinv."""
    L.check(L.lib().hss1d_scalarmult(A_HSS._h, float(c)))
    A_HSS.inverted = False
    return A_HSS


def HSS1D_dense_matrix(K_HSS: HSS1DMatrix, sym: int = 0, prob: int = 0) -> np.ndarray:
    """Kd = HSS1D_dense_matrix(K_HSS, sym) (HSS1D/HSS1D_dense_matrix.m:1): the dense matrix of
    problem ``prob`` (0 for a single curve).  ``sym`` is implied by the handle."""
    sizes = getattr(K_HSS, "sizes", [K_HSS.N])
    n = sizes[prob]
    Kd = np.zeros((n, n), order="F")
    L.check(L.lib().hss1d_dense_matrix(K_HSS._h, int(prob), L.ptr(Kd)))
    return Kd


def HSS1D_apply_submatrix_boxes(TREE: HSS1DMatrix, I_dn, I_up):
    """[Box_dn, Box_up] = HSS1D_apply_submatrix_boxes(TREE, I_dn, I_up)
    (HSS1D/HSS1D_apply_submatrix_boxes.m:1): boolean masks over the boxes."""
    dn = np.ascontiguousarray(np.asarray(I_dn, dtype=bool).astype(np.uint8))
    up = np.ascontiguousarray(np.asarray(I_up, dtype=bool).astype(np.uint8))
    nb = TREE.info()["nboxes"]
    bd = np.zeros(nb, np.uint8)
    bu = np.zeros(nb, np.uint8)
    L.check(L.lib().hss1d_apply_submatrix_boxes(TREE._h, L.ptr(dn), L.ptr(up), L.ptr(bd), L.ptr(bu)))
    return bd.astype(bool), bu.astype(bool)


def HSS1D_apply_submatrix_nsym(K_HSS: HSS1DMatrix, Box_dn, Box_up, I_dn, I_up, qq) -> np.ndarray:
    """uu = HSS1D_apply_submatrix_nsym(K_HSS, Box_dn, Box_up, I_dn, I_up, qq)
    (HSS1D/HSS1D_apply_submatrix_nsym.m:1): uu = K(I_dn, I_up) qq(I_up), qq of full length N.
    Box_dn / Box_up are accepted for the reference's signature and not needed."""
    dn = np.ascontiguousarray(np.asarray(I_dn, dtype=bool).astype(np.uint8))
    up = np.ascontiguousarray(np.asarray(I_up, dtype=bool).astype(np.uint8))
    q = _as_f64(qq)
    vec = q.ndim == 1
    q2 = q.reshape(K_HSS.N, -1, order="F")
    out = np.zeros((int(dn.sum()), q2.shape[1]), order="F")
    L.check(L.lib().hss1d_apply_submatrix(K_HSS._h, L.ptr(dn), L.ptr(up), L.ptr(q2), q2.shape[1], L.ptr(out)))
    return out[:, 0] if vec else out


HSS1D_apply_submatrix_fsym = HSS1D_apply_submatrix_nsym


def BHSS1D_apply_nsym(K11, K12, K21, K22, B_dn, B_up, I_dn, I_up, X) -> np.ndarray:
    """Y = BHSS1D_apply_nsym(K11,K12,K21,K22,B_dn,B_up,I_dn,I_up,X) (HSS1D/BHSS1D_apply_nsym.m:1):
    Y = A X for the submatrix A = [K11(I_dn{1,1},I_up{1,1}) K12(I_dn{1,2},I_up{1,2});
    K21(I_dn{2,1},I_up{2,1}) K22(I_dn{2,2},I_up{2,2})] of a 2 x 2 block matrix of compressed
    matrices, through four submatrix applies on the GPU.  I_dn / I_up are 2 x 2 nested lists
    of boolean masks over each block's points; B_dn / B_up (box masks) are accepted for the
    reference's signature and not needed.  X stacks X1 (sum of I_up{1,1} rows) over X2."""
    X = np.asarray(X, dtype=np.float64)
    vec = X.ndim == 1
    X2d = X.reshape(X.shape[0], -1)
    r1 = int(np.count_nonzero(I_up[0][0]))
    parts = (X2d[:r1], X2d[r1:])
    rows = []
    for i, (Ka, Kb) in enumerate(((K11, K12), (K21, K22))):
        y = 0.0
        for j, K in enumerate((Ka, Kb)):
            up = np.asarray(I_up[i][j], dtype=bool)
            v = np.zeros((up.size, X2d.shape[1]), order="F")
            v[up] = parts[j]
            y = y + HSS1D_apply_submatrix_nsym(K, None, None, I_dn[i][j], up, v)
        rows.append(y)
    Y = np.vstack(rows)
    return Y[:, 0] if vec else Y


BHSS1D_apply_fsym = BHSS1D_apply_nsym


def HSS1D_apply_nsym(K_HSS: HSS1DMatrix, qq) -> np.ndarray:
    q2, vec = _vec(K_HSS, qq)
    out = np.zeros((getattr(K_HSS, "M", K_HSS.N), q2.shape[1]), q2.dtype, order="F")
    L.check(L.lib().hss1d_apply(K_HSS._h, L.ptr(q2), L.ptr(out), q2.shape[1]))
    return out[:, 0] if vec else out


def HSS1D_applyinv_nsym(K_HSS: HSS1DMatrix, HSSinv, FTinv, ff) -> np.ndarray:
    f2, vec = _vec(K_HSS, ff)
    out = np.zeros_like(f2, order="F")
    L.check(L.lib().hss1d_applyinv(K_HSS._h, L.ptr(f2), L.ptr(out), f2.shape[1]))
    return out[:, 0] if vec else out


def HSS1D_solve(K_HSS: HSS1DMatrix, ff, tol: float = 1e-10, maxit: int = 5):
    """x = A^-1 f refined against the FP64 HSS1D forward operator
    (Common/Iterative_Refinement.m:20-35).  Returns (x, relres, inverse applies used)."""
    f2, vec = _vec(K_HSS, ff)
    out = np.zeros_like(f2, order="F")
    rr = C.c_double()
    it = C.c_int32()
    L.check(L.lib().hss1d_solve(K_HSS._h, L.ptr(f2), L.ptr(out), f2.shape[1], tol, maxit, C.byref(rr),
                                C.byref(it)))
    return (out[:, 0] if vec else out), rr.value, it.value


def HSS1D_kernel_residual(K_HSS: HSS1DMatrix, ff, xx) -> float:
    """max over columns of ||f - K x|| / ||f|| with K the kernel matrix of each curve itself
    (generated in FP64 on the GPU and applied on the fly, never formed): the dense-matrix
    residual the reference's tests print (Common/Iterative_Refinement.m:20-35)."""
    f2, _ = _vec(K_HSS, ff)
    x2, _ = _vec(K_HSS, xx)
    assert f2.shape == x2.shape
    rr = C.c_double()
    L.check(L.lib().hss1d_kernel_residual(K_HSS._h, L.ptr(f2), L.ptr(x2), f2.shape[1], C.byref(rr)))
    return rr.value


# HSS1D_sum_fsym / HSS1D_compressLR_fsym (one ID per box for symmetric operands,
# HSS1D/HSS1D_sum_fsym.m, HSS1D_compressLR_fsym.m): the nsym forms accept the same
# operands and return matrices every call here takes (incoming and outgoing skeletons
# kept separately).
HSS1D_sum_fsym = HSS1D_sum_nsym
HSS1D_compressLR_fsym = HSS1D_compressLR_nsym

# fsym handles carry T_DN = T_UP; the nsym algorithms are the fsym ones on them
# (HSS1D_invert_fsym.m:47-90 with E at :79, HSS1D_apply_fsym.m:1-118, HSS1D_applyinv_fsym.m:38-86)
HSS1D_invert_fsym = HSS1D_invert_nsym
HSS1D_apply_fsym = HSS1D_apply_nsym
HSS1D_applyinv_fsym = HSS1D_applyinv_nsym
