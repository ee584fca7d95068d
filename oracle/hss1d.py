"""HSS1D compress / invert / apply / applyinv / transforminv (oracle restatement).

Follows, function by function:
  HSS1D/HSS1D_compress_nsym.m   (compress, 'green' and 'brute'; tree :277-334,
                                  circle :339-371, neighbour list :376-412)
  HSS1D/HSS1D_invert_nsym.m     (:44-91)
  HSS1D/HSS1D_apply_nsym.m      (:38-130)
  HSS1D/HSS1D_applyinv_nsym.m   (:43-86)
  HSS1D/HSS1D_transforminv_nsym.m (:38-161)
  HSS1D/HSS1D_compress_rectangular_nsym.m, HSS1D/HSS1D_apply_rect_nsym.m (rectangular K(Xin, Xout))
  HSS1D/HSS1D_sum_nsym.m        (C = A + B on one tree)
  HSS1D/HSS1D_compressLR_nsym.m (U V^T in compressed form)
  HSS1D/HSS1D_recompress_nsym.m (rank reduction by SVDs of the far-field blocks)

The cell array ``K_HSS{row, ibox}`` of Common/box_constants.m:33-52 becomes an
``HSS1DMatrix`` whose per-box lists are indexed by the 0-based box id (box 0 is
the reference's box 1, the root).  Index arrays are 0-based here.
"""
from __future__ import annotations

from dataclasses import dataclass, field
import math

import numpy as np

from .kernels import KernelParams, kernel_eval, DL_L_2D, SL_L_2D, SL_H_2D
from . import cid, idecomp

RADIUS_REL = 1.75   # HSS1D_compress_nsym.m:51
NPROXY = 50         # HSS1D_compress_nsym.m:52


def _mround(x: float) -> int:
    """MATLAB's round (half away from zero), exact for x >= 0."""
    t = math.floor(x)
    return int(t) + (1 if x - t >= 0.5 else 0)


def proxy_count(kp: KernelParams, R: float, ntot: int) -> int:
    """Proxy points of a box, HSS1D_compress_nsym.m:111-114: 50, or for the Helmholtz
    kernel min(max(50, round(4 kh 1.75 R + 30)), ntot) (four points per wavelength)."""
    if kp.flag == SL_H_2D:
        return min(max(NPROXY, _mround(4.0 * kp.kh * RADIUS_REL * R + 30.0)), ntot)
    return NPROXY


def _id_out(A, acc, seed, problem):
    """ID(A, acc) of Common/ID.m:40-65, complex through oracle.cid for complex blocks."""
    if np.iscomplexobj(A):
        return cid.id_adaptive_complex(A, acc, seed, problem)
    return idecomp.id_adaptive(A, acc, seed, problem)


def _id_fixed(R, J, k):
    if np.iscomplexobj(R):
        return cid.id_fixed_complex(R, J, k)
    return idecomp.id_fixed_from_qr(R, J, k)


@dataclass
class HSS1DTree:
    level: np.ndarray
    parent: np.ndarray
    c1: np.ndarray
    c2: np.ndarray
    off: np.ndarray   # 0-based first point (END1 - 1)
    cnt: np.ndarray   # number of points (END2)

    @property
    def nboxes(self):
        return len(self.level)

    def is_leaf(self, b):
        return self.c1[b] < 0 and self.c2[b] < 0


def get_tree(ntot: int, nbox_max: int) -> HSS1DTree:
    """LOCAL_get_tree, HSS1D_compress_nsym.m:277-334 (BFS halving, son1 = ceil(n/2))."""
    level = [0]
    parent = [-1]
    c1 = [-1]
    c2 = [-1]
    off = [0]
    cnt = [ntot]
    ibox_last = -1
    ncreated = 1
    ilevel = 0
    while ncreated > 0:
        ibox_first = ibox_last + 1
        ibox_last = ibox_last + ncreated
        ncreated = 0
        for ibox in range(ibox_first, ibox_last + 1):
            nbox = cnt[ibox]
            if nbox > nbox_max:
                nhalf = (nbox + 1) // 2
                s1 = ibox_last + ncreated + 1
                s2 = s1 + 1
                c1[ibox] = s1
                c2[ibox] = s2
                for s, o, c in ((s1, off[ibox], nhalf), (s2, off[ibox] + nhalf, nbox - nhalf)):
                    assert len(level) == s
                    level.append(ilevel + 1)
                    parent.append(ibox)
                    c1.append(-1)
                    c2.append(-1)
                    off.append(o)
                    cnt.append(c)
                ncreated += 2
        ilevel += 1
    a = lambda v: np.asarray(v, dtype=np.int64)
    return HSS1DTree(a(level), a(parent), a(c1), a(c2), a(off), a(cnt))


def circum_circle(X: np.ndarray):
    """LOCAL_get_circum_circle, HSS1D_compress_nsym.m:339-356."""
    nloc = X.shape[0]
    xxc = 0.5 * (X[0, :2] + X[-1, :2])
    d = (X[:, 0] - xxc[0]) ** 2 + (X[:, 1] - xxc[1]) ** 2
    R = math.sqrt(np.max(d))
    e = (X[0, 0] - X[-1, 0]) ** 2 + (X[0, 1] - X[-1, 1]) ** 2
    if (1.2 * R * R) > e:
        sx = sy = 0.0
        for a, b in zip(X[:, 0].tolist(), X[:, 1].tolist()):   # sequential sums
            sx += a
            sy += b
        xxc = np.array([sx, sy]) * (1.0 / nloc)
        d = (X[:, 0] - xxc[0]) ** 2 + (X[:, 1] - xxc[1]) ** 2
        R = math.sqrt(np.max(d))
    return xxc, R


def proxy_circle(xxc, R, n):
    """LOCAL_construct_circle (HSS1D_compress_nsym.m:361-371) as (n,6) points.

    The normal (cos t, sin t) and weight 2 pi R / n are what the double-layer
    kernel uses for proxy sources; curvature 1/R.
    """
    tt = np.linspace(0.0, 2.0 * math.pi * (1.0 - 1.0 / n), n)
    P = np.zeros((n, 6))
    c = np.array([math.cos(t) for t in tt.tolist()])   # libm, as the host C++ does
    s = np.array([math.sin(t) for t in tt.tolist()])
    P[:, 0] = xxc[0] + R * c
    P[:, 1] = xxc[1] + R * s
    P[:, 2] = c
    P[:, 3] = s
    P[:, 4] = 2.0 * math.pi * R / n
    P[:, 5] = 1.0 / R
    return P


def neighbor_list(X: np.ndarray, tree: HSS1DTree, radius_rel=RADIUS_REL):
    """LOCAL_construct_potential_neighborlist, HSS1D_compress_nsym.m:376-412."""
    nb = tree.nboxes
    nei = [[] for _ in range(nb)]
    nei[0] = [0]
    for ibox in range(1, nb):
        o, c = tree.off[ibox], tree.cnt[ibox]
        xxc, R = circum_circle(X[o:o + c])
        pot = []
        for jbox in nei[tree.parent[ibox]]:
            if tree.c1[jbox] >= 0:
                pot.append(int(tree.c1[jbox]))
            if tree.c2[jbox] >= 0:
                pot.append(int(tree.c2[jbox]))
        rr = radius_rel * radius_rel * R * R
        for jbox in pot:
            oj, cj = tree.off[jbox], tree.cnt[jbox]
            d = (X[oj:oj + cj, 0] - xxc[0]) ** 2 + (X[oj:oj + cj, 1] - xxc[1]) ** 2
            if np.min(d) < rr:
                nei[ibox].append(jbox)
    for ibox in range(1, nb):
        lst = list(nei[ibox])
        if ibox in lst:
            lst.remove(ibox)
        nei[ibox] = sorted(lst)
    return nei


@dataclass
class HSS1DMatrix:
    tree: HSS1DTree
    nskel: list = field(default_factory=list)
    kskel: list = field(default_factory=list)
    I_SKUP: list = field(default_factory=list)
    I_SKDN: list = field(default_factory=list)
    T_UP: list = field(default_factory=list)
    J_UP: list = field(default_factory=list)
    T_DN: list = field(default_factory=list)
    J_DN: list = field(default_factory=list)
    M_SELF: list = field(default_factory=list)
    M_SIB: list = field(default_factory=list)
    # diagnostics: per-box ID problem shapes (m_out, m_in, n, k)
    census: list = field(default_factory=list)


def _leaf_range(tree, b):
    return np.arange(tree.off[b], tree.off[b] + tree.cnt[b])


def _box_skel_sets(H, b):
    """indskel_out / indskel_in of HSS1D_compress_nsym.m:87-100."""
    t = H.tree
    if t.is_leaf(b):
        ind = _leaf_range(t, b)
        return ind, ind
    if t.c1[b] >= 0 and t.c2[b] >= 0:
        s1, s2 = t.c1[b], t.c2[b]
        return (np.concatenate([H.I_SKUP[s1], H.I_SKUP[s2]]),
                np.concatenate([H.I_SKDN[s1], H.I_SKDN[s2]]))
    s = max(t.c1[b], t.c2[b])
    return H.I_SKUP[s], H.I_SKDN[s]


def compress_green_blocks(H, X, ibox, nei, kp: KernelParams, ntot):
    """A_out and A_in of HSS1D_compress_nsym.m:106-156 (the 'green' trick)."""
    t = H.tree
    out, inn = _box_skel_sets(H, ibox)
    both = np.sort(np.concatenate([out, inn]), kind="stable")
    xxc, R = circum_circle(X[both])
    nproxy = proxy_count(kp, R, ntot)
    Cp = proxy_circle(xxc, RADIUS_REL * R, nproxy)
    out_maybe, in_maybe = [], []
    for j in nei[ibox]:
        if t.is_leaf(j):
            r = _leaf_range(t, j)
            out_maybe.append(r)
            in_maybe.append(r)
        elif t.c1[j] >= 0 and t.c2[j] >= 0:
            out_maybe += [H.I_SKUP[t.c1[j]], H.I_SKUP[t.c2[j]]]
            in_maybe += [H.I_SKDN[t.c1[j]], H.I_SKDN[t.c2[j]]]
        else:
            s = max(t.c1[j], t.c2[j])
            out_maybe.append(H.I_SKUP[s])
            in_maybe.append(H.I_SKDN[s])
    cat = lambda L: np.concatenate(L) if L else np.zeros(0, dtype=np.int64)
    out_maybe = cat(out_maybe)
    in_maybe = cat(in_maybe)
    rr = (RADIUS_REL * R) ** 2
    d = (X[out_maybe, 0] - xxc[0]) ** 2 + (X[out_maybe, 1] - xxc[1]) ** 2
    out_inside = out_maybe[d < rr]
    d = (X[in_maybe, 0] - xxc[0]) ** 2 + (X[in_maybe, 1] - xxc[1]) ** 2
    in_inside = in_maybe[d < rr]
    A_out = np.vstack([kernel_eval(X[in_inside], X[out], kp), kernel_eval(Cp, X[out], kp)])
    A_in = np.hstack([kernel_eval(X[inn], X[out_inside], kp), kernel_eval(X[inn], Cp, kp)])
    return out, inn, A_out, A_in


def compress_nsym(X: np.ndarray, leaf: int, acc: float, kp: KernelParams, seed: int = 0,
                  tree: HSS1DTree | None = None) -> HSS1DMatrix:
    """K_HSS = HSS1D_compress_nsym('green', X, TREE, acc, knl_params).

    ID problem numbering for the shared RNG: box b's outgoing ID is problem
    2*b, its incoming ID 2*b+1.  With the Helmholtz kernel (SL_H_2D) every block is
    complex: the proxy ring holds proxy_count points and the IDs are complex
    (oracle.cid); T_DN is the ID's T of A_in.' (plain transpose), as in the reference.
    """
    X = np.asarray(X, dtype=np.float64)
    ntot = X.shape[0]
    t = tree if tree is not None else get_tree(ntot, leaf)
    nb = t.nboxes
    H = HSS1DMatrix(t)
    for name in ("nskel", "kskel", "I_SKUP", "I_SKDN", "T_UP", "J_UP", "T_DN", "J_DN",
                 "M_SELF", "M_SIB", "census"):
        setattr(H, name, [None] * nb)
    nei = neighbor_list(X, t)
    for ibox in range(nb - 1, 0, -1):
        out, inn, A_out, A_in = compress_green_blocks(H, X, ibox, nei, kp, ntot)
        Tout, Jout, kout, Rout = _id_out(A_out, acc, seed, 2 * ibox)
        Tin, Jin, kin, Rin = _id_out(A_in.T, acc, seed, 2 * ibox + 1)
        k = max(kout, kin)
        if k != kout:
            Tout = _id_fixed(Rout, Jout, k)
        elif k != kin:
            Tin = _id_fixed(Rin, Jin, k)
        H.I_SKUP[ibox] = out[Jout[:k]]
        H.T_UP[ibox] = Tout
        H.J_UP[ibox] = Jout
        H.I_SKDN[ibox] = inn[Jin[:k]]
        H.T_DN[ibox] = Tin
        H.J_DN[ibox] = Jin
        H.nskel[ibox] = len(out)
        H.kskel[ibox] = k
        H.census[ibox] = (A_out.shape[0], A_in.shape[1], len(out), k, kout, kin)
    for ibox in range(nb - 1, -1, -1):
        if t.is_leaf(ibox):
            ind = _leaf_range(t, ibox)
            H.M_SELF[ibox] = kernel_eval(X[ind], X[ind], kp)
        elif t.c1[ibox] >= 0 and t.c2[ibox] >= 0:
            s1, s2 = t.c1[ibox], t.c2[ibox]
            H.M_SIB[s1] = kernel_eval(X[H.I_SKDN[s1]], X[H.I_SKUP[s2]], kp)
            H.M_SIB[s2] = kernel_eval(X[H.I_SKDN[s2]], X[H.I_SKUP[s1]], kp)
    return H


def compress_fsym(X: np.ndarray, leaf: int, acc: float, kp: KernelParams, seed: int = 0,
                  tree: HSS1DTree | None = None) -> HSS1DMatrix:
    """K_HSS = HSS1D_compress_fsym('green', X, TREE, acc, knl_params),
    HSS1D/HSS1D_compress_fsym.m:98-248: one ID per box on A_out = K([X_inside; X_proxy],
    X_skel) (:114-164, :186-198; problem 2*b of the shared RNG), incoming skeletons equal
    to the outgoing ones, and M_SIB{c2} = M_SIB{c1}.' (:245).  The nsym invert and apply
    functions run on the result unchanged (their L is the transpose of R here)."""
    X = np.asarray(X, dtype=np.float64)
    ntot = X.shape[0]
    t = tree if tree is not None else get_tree(ntot, leaf)
    nb = t.nboxes
    H = HSS1DMatrix(t)
    for name in ("nskel", "kskel", "I_SKUP", "I_SKDN", "T_UP", "J_UP", "T_DN", "J_DN",
                 "M_SELF", "M_SIB", "census"):
        setattr(H, name, [None] * nb)
    nei = neighbor_list(X, t)
    for ibox in range(nb - 1, 0, -1):
        out, _, A_out, _ = compress_green_blocks(H, X, ibox, nei, kp, ntot)
        T, J, k, _ = _id_out(A_out, acc, seed, 2 * ibox)
        H.I_SKUP[ibox] = H.I_SKDN[ibox] = out[J[:k]]
        H.T_UP[ibox] = H.T_DN[ibox] = T
        H.J_UP[ibox] = H.J_DN[ibox] = J
        H.nskel[ibox] = len(out)
        H.kskel[ibox] = k
        H.census[ibox] = (A_out.shape[0], A_out.shape[0], len(out), k, k, k)
    for ibox in range(nb - 1, -1, -1):
        if t.is_leaf(ibox):
            ind = _leaf_range(t, ibox)
            H.M_SELF[ibox] = kernel_eval(X[ind], X[ind], kp)
        elif t.c1[ibox] >= 0 and t.c2[ibox] >= 0:
            s1, s2 = t.c1[ibox], t.c2[ibox]
            H.M_SIB[s1] = kernel_eval(X[H.I_SKUP[s1]], X[H.I_SKUP[s2]], kp)
            H.M_SIB[s2] = H.M_SIB[s1].T.copy()
    return H


def _RL(H, b):
    """R (k x n) and L (n x k) of HSS1D_invert_nsym.m:63-72."""
    n, k = H.nskel[b], H.kskel[b]
    dt = np.result_type(H.T_UP[b], H.T_DN[b], np.float64)
    R = np.zeros((k, n), dtype=dt)
    R[:, H.J_UP[b][:k]] = np.eye(k)
    R[:, H.J_UP[b][k:]] = H.T_UP[b]
    L = np.zeros((n, k), dtype=dt)
    L[H.J_DN[b][:k], :] = np.eye(k)
    L[H.J_DN[b][k:], :] = H.T_DN[b].T
    return R, L


def invert_nsym(H: HSS1DMatrix):
    """[HSSinv, FTinv] = HSS1D_invert_nsym(K_HSS, acc), HSS1D_invert_nsym.m:44-91.

    Returns dict with lists Linv, Rinv, Dinv (index = box) and FTinv.
    """
    t = H.tree
    nb = t.nboxes
    E = [None] * nb
    Linv = [None] * nb
    Rinv = [None] * nb
    Dinv = [None] * nb
    for b in range(nb - 1, 0, -1):
        F = _diag_block(H, E, b)
        R, L = _RL(H, b)
        Finv = np.linalg.inv(F)
        Eb = np.linalg.inv(R @ Finv @ L)
        E[b] = Eb
        Linv[b] = Finv @ L @ Eb
        Rinv[b] = Eb @ R @ Finv
        Dinv[b] = Finv - Linv[b] @ (R @ Finv)
    FT = np.block([[E[1], H.M_SIB[1]], [H.M_SIB[2], E[2]]])
    return {"Linv": Linv, "Rinv": Rinv, "Dinv": Dinv, "FTinv": np.linalg.inv(FT), "E": E}


def _diag_block(H, E, b):
    t = H.tree
    if t.is_leaf(b):
        return H.M_SELF[b]
    if t.c1[b] >= 0 and t.c2[b] >= 0:
        s1, s2 = t.c1[b], t.c2[b]
        return np.block([[E[s1], H.M_SIB[s1]], [H.M_SIB[s2], E[s2]]])
    return E[max(t.c1[b], t.c2[b])]


def _skel_proj(T, J, q):
    """LOCAL_skel_proj, HSS1D_apply_nsym.m:108-115."""
    if T.shape[1] == 0:
        return q[J]
    k = T.shape[0]
    return q[J[:k]] + T @ q[J[k:]]


def _skel_eval(T, J, u):
    """LOCAL_skel_eval, HSS1D_apply_nsym.m:121-130."""
    out = np.zeros((len(J), u.shape[1]), dtype=np.result_type(T, u))
    if T.shape[1] == 0:
        out[J] = u
    else:
        k = T.shape[0]
        out[J[:k]] = u
        out[J[k:]] = T.T @ u
    return out


def _dtype(H: HSS1DMatrix, v):
    """complex128 when the compressed matrix or the vector is complex, else float64."""
    cplx = np.iscomplexobj(v) or any(m is not None and np.iscomplexobj(m) for m in H.M_SELF)
    return np.complex128 if cplx else np.float64


def apply_nsym(H: HSS1DMatrix, qq: np.ndarray) -> np.ndarray:
    """uu = HSS1D_apply_nsym(K_HSS, qq), HSS1D_apply_nsym.m:38-100."""
    t = H.tree
    nb = t.nboxes
    qq = np.asarray(qq, dtype=_dtype(H, qq))
    vec = qq.ndim == 1
    if vec:
        qq = qq[:, None]
    up = [None] * nb
    dn = [None] * nb
    for b in range(nb - 1, 0, -1):
        if t.is_leaf(b):
            up[b] = _skel_proj(H.T_UP[b], H.J_UP[b], qq[_leaf_range(t, b)])
    for b in range(nb - 1, 0, -1):
        if not t.is_leaf(b):
            parts = [up[s] for s in (t.c1[b], t.c2[b]) if s >= 0]
            up[b] = _skel_proj(H.T_UP[b], H.J_UP[b], np.vstack(parts))
    dn[1] = H.M_SIB[1] @ up[2]
    dn[2] = H.M_SIB[2] @ up[1]
    for b in range(1, nb):
        if not t.is_leaf(b):
            s1, s2 = t.c1[b], t.c2[b]
            if s1 >= 0 and s2 >= 0:
                n1 = len(H.I_SKDN[s1])
                u = _skel_eval(H.T_DN[b], H.J_DN[b], dn[b])
                dn[s1] = u[:n1] + H.M_SIB[s1] @ up[s2]
                dn[s2] = u[n1:] + H.M_SIB[s2] @ up[s1]
            else:
                dn[max(s1, s2)] = _skel_eval(H.T_DN[b], H.J_DN[b], dn[b])
    uu = np.zeros_like(qq)
    for b in range(nb - 1, 0, -1):
        if t.is_leaf(b):
            ind = _leaf_range(t, b)
            uu[ind] = _skel_eval(H.T_DN[b], H.J_DN[b], dn[b]) + H.M_SELF[b] @ qq[ind]
    return uu[:, 0] if vec else uu


def applyinv_nsym(H: HSS1DMatrix, inv: dict, ff: np.ndarray) -> np.ndarray:
    """xx = HSS1D_applyinv_nsym(K_HSS, HSSinv, FTinv, ff), HSS1D_applyinv_nsym.m:43-86."""
    t = H.tree
    nb = t.nboxes
    ff = np.asarray(ff, dtype=_dtype(H, ff))
    vec = ff.ndim == 1
    if vec:
        ff = ff[:, None]
    f1 = [None] * nb
    f2 = [None] * nb
    for b in range(nb - 1, 0, -1):
        if t.is_leaf(b):
            f1[b] = inv["Rinv"][b] @ ff[_leaf_range(t, b)]
        else:
            parts = [f1[s] for s in (t.c1[b], t.c2[b]) if s >= 0]
            f1[b] = inv["Rinv"][b] @ np.vstack(parts)
    x_top = inv["FTinv"] @ np.vstack([f1[1], f1[2]])
    k2 = inv["Linv"][1].shape[1]
    f2[1] = x_top[:k2]
    f2[2] = x_top[k2:]
    xx = np.zeros_like(ff)
    for b in range(1, nb):
        if t.is_leaf(b):
            ind = _leaf_range(t, b)
            xx[ind] = inv["Linv"][b] @ f2[b] + inv["Dinv"][b] @ ff[ind]
        else:
            s1, s2 = t.c1[b], t.c2[b]
            if s1 >= 0 and s2 >= 0:
                k1 = H.kskel[s1]
                xl = inv["Linv"][b] @ f2[b] + inv["Dinv"][b] @ np.vstack([f1[s1], f1[s2]])
                f2[s1] = xl[:k1]
                f2[s2] = xl[k1:]
            else:
                s = max(s1, s2)
                f2[s] = inv["Linv"][b] @ f2[b] + inv["Dinv"][b] @ f1[s]
    return xx[:, 0] if vec else xx


def transforminv_nsym(H: HSS1DMatrix, inv: dict) -> HSS1DMatrix:
    """Kinv_HSS = HSS1D_transforminv_nsym(K_HSS, HSSinv, FTinv), :38-161."""
    t = H.tree
    nb = t.nboxes
    Lv = [None if x is None else x.copy() for x in inv["Linv"]]
    Rv = [None if x is None else x.copy() for x in inv["Rinv"]]
    Dv = [None if x is None else x.copy() for x in inv["Dinv"]]
    FT = inv["FTinv"].copy()
    k1, k2 = H.kskel[1], H.kskel[2]
    i1 = slice(0, k1)
    i2 = slice(k1, k1 + k2)
    Dv[1] = Dv[1] + Lv[1] @ FT[i1, i1] @ Rv[1]
    Dv[2] = Dv[2] + Lv[2] @ FT[i2, i2] @ Rv[2]
    FT[i1, i1] = 0.0
    FT[i2, i2] = 0.0
    for b in range(1, nb):
        s1, s2 = t.c1[b], t.c2[b]
        if s1 >= 0 and s2 >= 0:
            ka, kb = H.kskel[s1], H.kskel[s2]
            ia = slice(0, ka)
            ib = slice(ka, ka + kb)
            Dv[s1] = Dv[s1] + Lv[s1] @ Dv[b][ia, ia] @ Rv[s1]
            Dv[s2] = Dv[s2] + Lv[s2] @ Dv[b][ib, ib] @ Rv[s2]
            Dv[b][ia, ia] = 0.0
            Dv[b][ib, ib] = 0.0
        elif s1 >= 0 or s2 >= 0:
            s = max(s1, s2)
            Dv[s] = Dv[s] + Lv[s] @ Dv[b] @ Rv[s]
            Dv[b] = np.zeros((H.kskel[s], H.kskel[s]))
    for b in range(nb - 1, 0, -1):
        n, k = H.nskel[b], H.kskel[b]
        JC, JR = H.J_UP[b], H.J_DN[b]
        L, R = Lv[b], Rv[b]
        P = L[JC[:k], :]
        Q = R[:, JR[:k]]
        Lnew = np.zeros((n, k))
        Lnew[JC[:k]] = np.eye(k)
        Lnew[JC[k:]] = np.linalg.solve(P.T, L[JC[k:], :].T).T
        Rnew = np.zeros((k, n))
        Rnew[:, JR[:k]] = np.eye(k)
        Rnew[:, JR[k:]] = np.linalg.solve(Q, R[:, JR[k:]])
        Lv[b] = Lnew
        Rv[b] = Rnew
        f = t.parent[b]
        if b == t.c2[f] and t.c1[f] >= 0:
            ind = slice(H.kskel[t.c1[f]], H.kskel[t.c1[f]] + k)
        else:
            ind = slice(0, k)
        if t.level[b] > 1:
            Lv[f][ind, :] = P @ Lv[f][ind, :]
            Rv[f][:, ind] = Rv[f][:, ind] @ Q
            Dv[f][ind, :] = P @ Dv[f][ind, :]
            Dv[f][:, ind] = Dv[f][:, ind] @ Q
        else:
            FT[ind, :] = P @ FT[ind, :]
            FT[:, ind] = FT[:, ind] @ Q
    K = HSS1DMatrix(t)
    K.nskel = list(H.nskel)
    K.kskel = list(H.kskel)
    K.I_SKUP = list(H.I_SKUP)
    K.I_SKDN = list(H.I_SKDN)
    K.T_UP = [None] * nb
    K.J_UP = [None] * nb
    K.T_DN = [None] * nb
    K.J_DN = [None] * nb
    K.M_SELF = [None] * nb
    K.M_SIB = [None] * nb
    for b in range(1, nb):
        n, k = H.nskel[b], H.kskel[b]
        JC, JR = H.J_UP[b], H.J_DN[b]
        K.T_UP[b] = Rv[b][:, JR[k:]]
        K.J_UP[b] = JR
        K.T_DN[b] = Lv[b][JC[k:], :].T
        K.J_DN[b] = JC
    ka = H.kskel[1]
    kb = H.kskel[2]
    K.M_SIB[1] = FT[0:ka, ka:ka + kb]
    K.M_SIB[2] = FT[ka:ka + kb, 0:ka]
    for b in range(1, nb):
        s1, s2 = t.c1[b], t.c2[b]
        if s1 >= 0 and s2 >= 0:
            ka, kb = H.kskel[s1], H.kskel[s2]
            K.M_SIB[s1] = Dv[b][0:ka, ka:ka + kb]
            K.M_SIB[s2] = Dv[b][ka:ka + kb, 0:ka]
        elif t.is_leaf(b):
            K.M_SELF[b] = Dv[b]
    return K


def dense_from_points(X, kp):
    return kernel_eval(X, X, kp)


def transpose(H: HSS1DMatrix) -> HSS1DMatrix:
    """At_HSS = HSS1D_transpose(A_HSS), HSS1D/HSS1D_transpose.m:24-50: up/down skeletons and
    interpolation matrices swap, M_SELF is transposed, sibling blocks swap and transpose."""
    t = H.tree
    nb = t.nboxes
    At = HSS1DMatrix(tree=t, nskel=list(H.nskel), kskel=list(H.kskel),
                     I_SKUP=list(H.I_SKDN), I_SKDN=list(H.I_SKUP),
                     T_UP=list(H.T_DN), J_UP=list(H.J_DN), T_DN=list(H.T_UP), J_DN=list(H.J_UP),
                     M_SELF=[None if m is None else np.array(m).T.copy() for m in H.M_SELF],
                     M_SIB=list(H.M_SIB), census=list(H.census))
    for b in range(nb):
        s1, s2 = t.c1[b], t.c2[b]
        if s1 >= 0 and s2 >= 0:
            At.M_SIB[s1] = np.array(H.M_SIB[s2]).T.copy()
            At.M_SIB[s2] = np.array(H.M_SIB[s1]).T.copy()
    return At


def scalarmult(c: float, H: HSS1DMatrix) -> HSS1DMatrix:
    """A = HSS1D_scalarmult(c, A), HSS1D/HSS1D_scalarmult.m:19-33 (a scaled copy)."""
    t = H.tree
    A = HSS1DMatrix(tree=t, nskel=list(H.nskel), kskel=list(H.kskel), I_SKUP=list(H.I_SKUP),
                    I_SKDN=list(H.I_SKDN), T_UP=list(H.T_UP), J_UP=list(H.J_UP), T_DN=list(H.T_DN),
                    J_DN=list(H.J_DN), M_SELF=list(H.M_SELF), M_SIB=list(H.M_SIB), census=list(H.census))
    for b in range(t.nboxes):
        s1, s2 = t.c1[b], t.c2[b]
        if s1 >= 0 and s2 >= 0:
            A.M_SIB[s1] = c * np.asarray(H.M_SIB[s1])
            A.M_SIB[s2] = c * np.asarray(H.M_SIB[s2])
        if t.is_leaf(b) and H.M_SELF[b] is not None:
            A.M_SELF[b] = c * np.asarray(H.M_SELF[b])
    return A


def dense_matrix(H: HSS1DMatrix) -> np.ndarray:
    """Kd = HSS1D_dense_matrix(K_HSS, sym), HSS1D/HSS1D_dense_matrix.m:17-92: leaves to root,
    Rho_b (k x points) maps a box's points to its up skeleton and Lambda_b (points x k) its
    down skeleton to its points; each sibling pair fills Kd(ind1, ind2) =
    Lambda_1 M_SIB_1 Rho_2 and Kd(ind2, ind1) = Lambda_2 M_SIB_2 Rho_1.

    A parent's Lambda uses the down interpolation (T_DN, J_DN); the reference's nsym branch
    (:58-61) passes T_UP / J_UP there, which only agrees when T_DN = T_UP (fsym)."""
    t = H.tree
    nb = t.nboxes
    Rho = [None] * nb
    Lam = [None] * nb
    sl = lambda b: slice(int(t.off[b]), int(t.off[b] + t.cnt[b]))  # noqa: E731
    Kd = np.zeros((int(t.cnt[0]), int(t.cnt[0])))
    for b in range(nb - 1, -1, -1):
        if t.is_leaf(b):
            Kd[sl(b), sl(b)] = H.M_SELF[b]
            if b == 0:
                continue
            I = np.eye(int(t.cnt[b]))
            Rho[b] = _skel_proj(H.T_UP[b], H.J_UP[b], I)
            Lam[b] = _skel_proj(H.T_DN[b], H.J_DN[b], I).T
            continue
        s1, s2 = t.c1[b], t.c2[b]
        Kd[sl(s1), sl(s2)] = Lam[s1] @ H.M_SIB[s1] @ Rho[s2]
        Kd[sl(s2), sl(s1)] = Lam[s2] @ H.M_SIB[s2] @ Rho[s1]
        if b == 0:
            continue
        n1, n2 = Rho[s1].shape[1], Rho[s2].shape[1]
        k1, k2 = Rho[s1].shape[0], Rho[s2].shape[0]
        Rc = np.zeros((k1 + k2, n1 + n2))
        Rc[:k1, :n1] = Rho[s1]
        Rc[k1:, n1:] = Rho[s2]
        Lc = np.zeros((n1 + n2, k1 + k2))
        Lc[:n1, :k1] = Lam[s1]
        Lc[n1:, k1:] = Lam[s2]
        Rho[b] = _skel_proj(H.T_UP[b], H.J_UP[b], Rc)
        Lam[b] = _skel_proj(H.T_DN[b], H.J_DN[b], Lc.T).T
    return Kd


def apply_submatrix_boxes(tree: HSS1DTree, I_dn, I_up):
    """[Box_dn, Box_up] = HSS1D_apply_submatrix_boxes(TREE, I_dn, I_up),
    HSS1D/HSS1D_apply_submatrix_boxes.m:19-62: a leaf is marked when it holds any selected
    row / column, a parent when a child is marked."""
    I_dn = np.asarray(I_dn, dtype=bool)
    I_up = np.asarray(I_up, dtype=bool)
    nb = tree.nboxes
    bd = np.zeros(nb, bool)
    bu = np.zeros(nb, bool)
    for b in range(nb - 1, -1, -1):
        if tree.is_leaf(b):
            ind = _leaf_range(tree, b)
            bd[b] = I_dn[ind].any()
            bu[b] = I_up[ind].any()
        else:
            kids = [s for s in (tree.c1[b], tree.c2[b]) if s >= 0]
            bd[b] = any(bd[s] for s in kids)
            bu[b] = any(bu[s] for s in kids)
    return bd, bu


def apply_submatrix(H: HSS1DMatrix, I_dn, I_up, qq):
    """uu = K(I_dn, I_up) qq(I_up) (HSS1D_apply_submatrix_nsym.m output), through the dense
    form of the compressed matrix."""
    I_dn = np.asarray(I_dn, dtype=bool)
    I_up = np.asarray(I_up, dtype=bool)
    Kd = dense_matrix(H)
    return Kd[np.ix_(I_dn, I_up)] @ np.asarray(qq)[I_up]


# ---------------------------------------------------------------------------
# Rectangular HSS1D: K(Xin, Xout), HSS1D/HSS1D_compress_rectangular_nsym.m and
# HSS1D/HSS1D_apply_rect_nsym.m
# ---------------------------------------------------------------------------
@dataclass
class HSS1DRectMatrix(HSS1DMatrix):
    """K_HSS of HSS1D_compress_rectangular_nsym: ``tree`` is the column (out) tree over
    Xout; the row (in) tree has the same shape with offsets/counts ``off_in``/``cnt_in``
    over Xin (K_HSS rows 16:17) and skeleton sizes ``nskel_in``/``kskel_in`` (rows 18:19).
    I_SKUP indexes Xout, I_SKDN indexes Xin."""
    off_in: np.ndarray = None
    cnt_in: np.ndarray = None
    nskel_in: list = field(default_factory=list)
    kskel_in: list = field(default_factory=list)
    mtot: int = 0


def get_tree_in(mtot: int, tree: HSS1DTree):
    """LOCAL_get_tree_in, HSS1D_compress_rectangular_nsym.m:325-356: the row tree takes the
    column tree's shape; a parent's rows split as ceil(m/2) | rest (parents come first)."""
    nb = tree.nboxes
    off = np.zeros(nb, dtype=np.int64)
    cnt = np.zeros(nb, dtype=np.int64)
    cnt[0] = mtot
    for b in range(nb):
        s1, s2 = tree.c1[b], tree.c2[b]
        if s1 >= 0 and s2 >= 0:
            half = (cnt[b] + 1) // 2
            off[s1], cnt[s1] = off[b], half
            off[s2], cnt[s2] = off[b] + half, cnt[b] - half
    return off, cnt


def neighbor_list_rect(Xin, Xout, tree: HSS1DTree, off_in, cnt_in, radius_rel=RADIUS_REL):
    """LOCAL_construct_potential_neighborlist, HSS1D_compress_rectangular_nsym.m:397-462.
    One circle per box around its rows and columns; nei_in keeps the boxes whose COLUMN
    points come inside it, nei_out those whose ROW points do."""
    nb = tree.nboxes
    nei_in = [[] for _ in range(nb)]
    nei_out = [[] for _ in range(nb)]
    nei_in[0] = [0]
    nei_out[0] = [0]
    for ibox in range(1, nb):
        P = np.vstack([Xin[off_in[ibox]:off_in[ibox] + cnt_in[ibox]],
                       Xout[tree.off[ibox]:tree.off[ibox] + tree.cnt[ibox]]])
        xxc, R = circum_circle(P)
        rr = radius_rel * radius_rel * R * R
        for lst, pts, offs, cnts in ((nei_in, Xout, tree.off, tree.cnt), (nei_out, Xin, off_in, cnt_in)):
            pot = []
            for jbox in lst[tree.parent[ibox]]:
                if tree.c1[jbox] >= 0:
                    pot.append(int(tree.c1[jbox]))
                if tree.c2[jbox] >= 0:
                    pot.append(int(tree.c2[jbox]))
            for jbox in pot:
                o, c = offs[jbox], cnts[jbox]
                d = (pts[o:o + c, 0] - xxc[0]) ** 2 + (pts[o:o + c, 1] - xxc[1]) ** 2
                if c > 0 and np.min(d) < rr:
                    lst[ibox].append(jbox)
    for lst in (nei_in, nei_out):
        for ibox in range(1, nb):
            l = list(lst[ibox])
            if ibox in l:
                l.remove(ibox)
            lst[ibox] = sorted(l)
    return nei_in, nei_out


def compress_rectangular_nsym(Xin: np.ndarray, Xout: np.ndarray, leaf: int, acc: float, kp: KernelParams,
                              seed: int = 0) -> HSS1DRectMatrix:
    """K_HSS = HSS1D_compress_rectangular_nsym('green', Xin, Xout, TREE, acc, params) for the
    M x N matrix K(Xin, Xout), HSS1D_compress_rectangular_nsym.m:70-266.

    Per box (fine to coarse, :112-236): one circle around the box's row and column
    skeleton candidates, one proxy ring on it (50 points for Laplace kernels),
    A_out = [K(rows inside, cols); K(ring, cols)] and A_in = [K(rows, cols inside),
    K(rows, ring)], then ID(A_out) and ID(A_in.') with independent ranks (no rank
    equalisation, unlike the square compress).  Problem numbers of the shared RNG:
    2*b (outgoing) and 2*b+1 (incoming), as in compress_nsym.  Leaves keep
    M_SELF = K(Xin(rows), Xout(cols)); siblings M_SIB{s1} = K(Xin(I_SKDN{s1}),
    Xout(I_SKUP{s2})) (:240-266)."""
    Xin = np.asarray(Xin, dtype=np.float64)
    Xout = np.asarray(Xout, dtype=np.float64)
    mtot, ntot = Xin.shape[0], Xout.shape[0]
    t = get_tree(ntot, leaf)
    off_in, cnt_in = get_tree_in(mtot, t)
    nb = t.nboxes
    H = HSS1DRectMatrix(t, off_in=off_in, cnt_in=cnt_in, mtot=mtot)
    for name in ("nskel", "kskel", "I_SKUP", "I_SKDN", "T_UP", "J_UP", "T_DN", "J_DN",
                 "M_SELF", "M_SIB", "census", "nskel_in", "kskel_in"):
        setattr(H, name, [None] * nb)
    nei_in, nei_out = neighbor_list_rect(Xin, Xout, t, off_in, cnt_in)
    cat = lambda L: np.concatenate(L) if L else np.zeros(0, dtype=np.int64)
    in_range = lambda b: np.arange(off_in[b], off_in[b] + cnt_in[b])
    for ibox in range(nb - 1, 0, -1):
        if t.is_leaf(ibox):
            out, inn = _leaf_range(t, ibox), in_range(ibox)
        else:
            s1, s2 = t.c1[ibox], t.c2[ibox]
            out = np.concatenate([H.I_SKUP[s1], H.I_SKUP[s2]])
            inn = np.concatenate([H.I_SKDN[s1], H.I_SKDN[s2]])
        xxc, R = circum_circle(np.vstack([Xin[np.sort(inn, kind="stable")], Xout[np.sort(out, kind="stable")]]))
        Cp = proxy_circle(xxc, RADIUS_REL * R, NPROXY)
        out_maybe, in_maybe = [], []
        for j in nei_in[ibox]:
            out_maybe += [_leaf_range(t, j)] if t.is_leaf(j) else [H.I_SKUP[t.c1[j]], H.I_SKUP[t.c2[j]]]
        for j in nei_out[ibox]:
            in_maybe += [in_range(j)] if t.is_leaf(j) else [H.I_SKDN[t.c1[j]], H.I_SKDN[t.c2[j]]]
        out_maybe, in_maybe = cat(out_maybe), cat(in_maybe)
        rr = (RADIUS_REL * R) ** 2
        out_inside = out_maybe[(Xout[out_maybe, 0] - xxc[0]) ** 2 + (Xout[out_maybe, 1] - xxc[1]) ** 2 < rr]
        in_inside = in_maybe[(Xin[in_maybe, 0] - xxc[0]) ** 2 + (Xin[in_maybe, 1] - xxc[1]) ** 2 < rr]
        A_out = np.vstack([kernel_eval(Xin[in_inside], Xout[out], kp), kernel_eval(Cp, Xout[out], kp)])
        A_in = np.hstack([kernel_eval(Xin[inn], Xout[out_inside], kp), kernel_eval(Xin[inn], Cp, kp)])
        Tout, Jout, kout, _ = idecomp.id_adaptive(A_out, acc, seed, 2 * ibox)
        Tin, Jin, kin, _ = idecomp.id_adaptive(A_in.T, acc, seed, 2 * ibox + 1)
        H.I_SKUP[ibox] = out[Jout[:kout]]
        H.T_UP[ibox] = Tout
        H.J_UP[ibox] = Jout
        H.I_SKDN[ibox] = inn[Jin[:kin]]
        H.T_DN[ibox] = Tin
        H.J_DN[ibox] = Jin
        H.nskel[ibox], H.kskel[ibox] = len(out), kout
        H.nskel_in[ibox], H.kskel_in[ibox] = len(inn), kin
        H.census[ibox] = (A_out.shape[0], A_in.shape[1], len(out), len(inn), kout, kin)
    for ibox in range(nb - 1, -1, -1):
        if t.is_leaf(ibox):
            H.M_SELF[ibox] = kernel_eval(Xin[in_range(ibox)], Xout[_leaf_range(t, ibox)], kp)
        elif t.c1[ibox] >= 0 and t.c2[ibox] >= 0:
            s1, s2 = t.c1[ibox], t.c2[ibox]
            H.M_SIB[s1] = kernel_eval(Xin[H.I_SKDN[s1]], Xout[H.I_SKUP[s2]], kp)
            H.M_SIB[s2] = kernel_eval(Xin[H.I_SKDN[s2]], Xout[H.I_SKUP[s1]], kp)
    return H


def apply_rect_nsym(H: HSS1DRectMatrix, qq: np.ndarray) -> np.ndarray:
    """uu = HSS1D_apply_rect_nsym(K_HSS, qq), HSS1D_apply_rect_nsym.m:30-106: the upward
    projections run on the column tree, the downward evaluations on the row tree, and
    the leaves add M_SELF qq(cols) into uu(rows) (uu has mtot rows)."""
    t = H.tree
    nb = t.nboxes
    qq = np.asarray(qq, dtype=np.float64)
    vec = qq.ndim == 1
    if vec:
        qq = qq[:, None]
    up = [None] * nb
    dn = [None] * nb
    for b in range(nb - 1, 0, -1):
        if t.is_leaf(b):
            up[b] = _skel_proj(H.T_UP[b], H.J_UP[b], qq[_leaf_range(t, b)])
    for b in range(nb - 1, 0, -1):
        if not t.is_leaf(b):
            up[b] = _skel_proj(H.T_UP[b], H.J_UP[b], np.vstack([up[t.c1[b]], up[t.c2[b]]]))
    dn[1] = H.M_SIB[1] @ up[2]
    dn[2] = H.M_SIB[2] @ up[1]
    for b in range(1, nb):
        if not t.is_leaf(b):
            s1, s2 = t.c1[b], t.c2[b]
            n1 = len(H.I_SKDN[s1])
            u = _skel_eval(H.T_DN[b], H.J_DN[b], dn[b])
            dn[s1] = u[:n1] + H.M_SIB[s1] @ up[s2]
            dn[s2] = u[n1:] + H.M_SIB[s2] @ up[s1]
    uu = np.zeros((H.mtot, qq.shape[1]))
    for b in range(nb - 1, 0, -1):
        if t.is_leaf(b):
            rows = np.arange(H.off_in[b], H.off_in[b] + H.cnt_in[b])
            uu[rows] = _skel_eval(H.T_DN[b], H.J_DN[b], dn[b]) + H.M_SELF[b] @ qq[_leaf_range(t, b)]
    return uu[:, 0] if vec else uu


# ---------------------------------------------------------------------------
# C = A + B on one tree, HSS1D/HSS1D_sum_nsym.m
# ---------------------------------------------------------------------------
def _rform(T, J, k, n):
    """R with R(:, J) = [I T] (k x n), HSS1D_sum_nsym.m:40-43; for the incoming side the
    same form of (T_DN, J_DN) is L^T."""
    R = np.zeros((k, n))
    R[:, np.asarray(J)] = np.hstack([np.eye(k), np.asarray(T).reshape(k, n - k)])
    return R


def sum_nsym(A: HSS1DMatrix, B: HSS1DMatrix, acc: float, seed: int = 0) -> HSS1DMatrix:
    """C_HSS = HSS1D_sum_nsym(A_HSS, B_HSS, acc), HSS1D_sum_nsym.m:30-160, for A and B on
    one tree.  Bottom-up, each box stacks the two operands' outgoing bases
    RC = [R_A P_A; R_B P_B] and incoming bases LC^T (P: the sons' RHO, the identity on a
    leaf), IDs both (problems 2*b and 2*b+1 of the shared RNG) with the rank equalised to
    k = max(k_out, k_in) by the fixed-rank ID (:57-66), and keeps RHO = RC(:, J_out(1:k)),
    LAMBDA = LC(J_in(1:k), :).  Sibling blocks become
    LAMBDA_s1 [M_SIB_A 0; 0 M_SIB_B] RHO_s2 (:79-86) and self blocks add."""
    t = A.tree
    for f in ("level", "parent", "c1", "c2", "off", "cnt"):
        if not np.array_equal(getattr(t, f), getattr(B.tree, f)):
            raise ValueError("HSS1D_sum_nsym needs both operands on one tree")
    nb = t.nboxes
    C = HSS1DMatrix(t)
    for name in ("nskel", "kskel", "I_SKUP", "I_SKDN", "T_UP", "J_UP", "T_DN", "J_DN",
                 "M_SELF", "M_SIB", "census"):
        setattr(C, name, [None] * nb)
    rho = [None] * nb
    sig = [None] * nb   # LAMBDA^T
    for ibox in range(nb - 1, -1, -1):
        if t.is_leaf(ibox):
            ind = _leaf_range(t, ibox)
            n = len(ind)
            C.M_SELF[ibox] = A.M_SELF[ibox] + B.M_SELF[ibox]
            if ibox == 0:
                continue
            kA, kB = A.kskel[ibox], B.kskel[ibox]
            RC = np.vstack([_rform(A.T_UP[ibox], A.J_UP[ibox], kA, n), _rform(B.T_UP[ibox], B.J_UP[ibox], kB, n)])
            LCt = np.vstack([_rform(A.T_DN[ibox], A.J_DN[ibox], kA, n), _rform(B.T_DN[ibox], B.J_DN[ibox], kB, n)])
            out_set = in_set = ind
        else:
            s1, s2 = t.c1[ibox], t.c2[ibox]
            kA1, kA2 = A.kskel[s1], A.kskel[s2]
            C.M_SIB[s1] = sig[s1][:kA1].T @ A.M_SIB[s1] @ rho[s2][:kA2] + sig[s1][kA1:].T @ B.M_SIB[s1] @ rho[s2][kA2:]
            C.M_SIB[s2] = sig[s2][:kA2].T @ A.M_SIB[s2] @ rho[s1][:kA1] + sig[s2][kA2:].T @ B.M_SIB[s2] @ rho[s1][kA1:]
            if ibox == 0:
                continue
            kB1, kB2 = B.kskel[s1], B.kskel[s2]
            kA, kB = A.kskel[ibox], B.kskel[ibox]
            out_set = np.concatenate([C.I_SKUP[s1], C.I_SKUP[s2]])
            in_set = np.concatenate([C.I_SKDN[s1], C.I_SKDN[s2]])

            def stack(TA, JA, TB, JB, P):
                RA = _rform(TA, JA, kA, kA1 + kA2)
                RB = _rform(TB, JB, kB, kB1 + kB2)
                return np.vstack([np.hstack([RA[:, :kA1] @ P[s1][:kA1], RA[:, kA1:] @ P[s2][:kA2]]),
                                  np.hstack([RB[:, :kB1] @ P[s1][kA1:], RB[:, kB1:] @ P[s2][kA2:]])])
            RC = stack(A.T_UP[ibox], A.J_UP[ibox], B.T_UP[ibox], B.J_UP[ibox], rho)
            LCt = stack(A.T_DN[ibox], A.J_DN[ibox], B.T_DN[ibox], B.J_DN[ibox], sig)
        Tout, Jout, kout, Rout = idecomp.id_adaptive(RC, acc, seed, 2 * ibox)
        Tin, Jin, kin, Rin = idecomp.id_adaptive(LCt, acc, seed, 2 * ibox + 1)
        k = max(kout, kin)
        if k != kout:
            Tout = idecomp.id_fixed_from_qr(Rout, Jout, k)
        elif k != kin:
            Tin = idecomp.id_fixed_from_qr(Rin, Jin, k)
        C.I_SKUP[ibox] = out_set[Jout[:k]]
        C.T_UP[ibox] = Tout
        C.J_UP[ibox] = Jout
        C.I_SKDN[ibox] = in_set[Jin[:k]]
        C.T_DN[ibox] = Tin
        C.J_DN[ibox] = Jin
        C.nskel[ibox] = len(out_set)
        C.kskel[ibox] = k
        C.census[ibox] = (RC.shape[0], LCt.shape[0], len(out_set), k, kout, kin)
        rho[ibox] = RC[:, Jout[:k]]
        sig[ibox] = LCt[:, Jin[:k]]
    return C


# ---------------------------------------------------------------------------
# K = U V^T in compressed form, HSS1D/HSS1D_compressLR_nsym.m
# ---------------------------------------------------------------------------
def compress_lr_nsym(U: np.ndarray, V: np.ndarray, leaf: int, acc: float, seed: int = 0) -> HSS1DMatrix:
    """K_HSS = HSS1D_compressLR_nsym(U, V, TREE, acc), HSS1D_compressLR_nsym.m:25-88: the
    N x N matrix U V^T on the halving tree.  Per box (fine to coarse) ID(V(out,:).') and
    ID(U(in,:).') (problems 2*b and 2*b+1 of the shared RNG), rank equalised by the
    fixed-rank ID; M_SELF = U(ind,:) V(ind,:).' and M_SIB{s1} = U(I_SKDN{s1},:)
    V(I_SKUP{s2},:).'."""
    U = np.asarray(U, dtype=np.float64)
    V = np.asarray(V, dtype=np.float64)
    t = get_tree(U.shape[0], leaf)
    nb = t.nboxes
    H = HSS1DMatrix(t)
    for name in ("nskel", "kskel", "I_SKUP", "I_SKDN", "T_UP", "J_UP", "T_DN", "J_DN",
                 "M_SELF", "M_SIB", "census"):
        setattr(H, name, [None] * nb)
    for ibox in range(nb - 1, 0, -1):
        out, inn = _box_skel_sets(H, ibox)
        A21 = V[out].T
        A12t = U[inn].T
        Tout, Jout, kout, Rout = idecomp.id_adaptive(A21, acc, seed, 2 * ibox)
        Tin, Jin, kin, Rin = idecomp.id_adaptive(A12t, acc, seed, 2 * ibox + 1)
        k = max(kout, kin)
        if k != kout:
            Tout = idecomp.id_fixed_from_qr(Rout, Jout, k)
        elif k != kin:
            Tin = idecomp.id_fixed_from_qr(Rin, Jin, k)
        H.I_SKUP[ibox] = out[Jout[:k]]
        H.T_UP[ibox] = Tout
        H.J_UP[ibox] = Jout
        H.I_SKDN[ibox] = inn[Jin[:k]]
        H.T_DN[ibox] = Tin
        H.J_DN[ibox] = Jin
        H.nskel[ibox] = len(out)
        H.kskel[ibox] = k
        H.census[ibox] = (A21.shape[0], A12t.shape[0], len(out), k, kout, kin)
    for ibox in range(nb - 1, -1, -1):
        if t.is_leaf(ibox):
            ind = _leaf_range(t, ibox)
            H.M_SELF[ibox] = U[ind] @ V[ind].T
        elif t.c1[ibox] >= 0 and t.c2[ibox] >= 0:
            s1, s2 = t.c1[ibox], t.c2[ibox]
            H.M_SIB[s1] = U[H.I_SKDN[s1]] @ V[H.I_SKUP[s2]].T
            H.M_SIB[s2] = U[H.I_SKDN[s2]] @ V[H.I_SKUP[s1]].T
    return H


# ---------------------------------------------------------------------------
# Rank reduction of a compressed matrix, HSS1D/HSS1D_recompress_nsym.m
# ---------------------------------------------------------------------------
def recompress_nsym(A: HSS1DMatrix, acc: float) -> HSS1DMatrix:
    """A_NEW = HSS1D_recompress_nsym(A, acc), HSS1D_recompress_nsym.m:26-247.

    Top-down (:30-146): the root's sibling blocks are truncated by their SVDs (singular
    values above the absolute acc); every other parent stacks its sons' sibling blocks with
    the parent's far-field factors (Sson = [B, Lp S], Tson = [B; T Rp]) and truncates them
    by SVD, giving each son a reduced row basis Q' R and column basis L P.  Bottom-up
    (:148-246): each box IDs its reduced bases at full rank (ID(RNEW, k), k = min(size)),
    keeps RHO / LAMBDA, and the sibling blocks become LAMBDA_s1 M_SIB RHO_s2."""
    t = A.tree
    nb = t.nboxes
    sv = lambda M: np.linalg.svd(M, full_matrices=False)
    Rf = lambda b: _rform(A.T_UP[b], A.J_UP[b], A.kskel[b], A.nskel[b])
    Lf = lambda b: _rform(A.T_DN[b], A.J_DN[b], A.kskel[b], A.nskel[b]).T
    Tp, Sp, Rp, Lp = {}, {}, {}, {}
    sib = {}
    for ib in range(nb):
        s1, s2 = t.c1[ib], t.c2[ib]
        if s1 < 0 or s2 < 0:
            continue
        k1, k2 = A.kskel[s1], A.kskel[s2]
        R1, R2, L1, L2 = Rf(s1), Rf(s2), Lf(s1), Lf(s2)
        B1, B2 = A.M_SIB[s1], A.M_SIB[s2]
        if ib == 0:
            P1, D1, Q2h = sv(B1)
            P2, D2, Q1h = sv(B2)
            k1n, k2n = int(np.sum(D1 > acc)), int(np.sum(D2 > acc))
            Q1, Q2 = Q1h.conj().T[:, :k1n], Q2h.conj().T[:, :k2n]
            P1, P2 = P1[:, :k1n], P2[:, :k2n]
            D1m = np.diag(D1)[:k1n, :k2n]
            D2m = np.diag(D2)[:k2n, :k1n]
            sib[s1], sib[s2] = D1m, D2m
            Tp[s1], Tp[s2] = D2m, D1m
            Sp[s1], Sp[s2] = D1m, D2m
        else:
            T0, S0, R0, L0 = Tp.pop(ib), Sp.pop(ib), Rp[ib], Lp[ib]
            Sson1 = np.hstack([B1, L0[:k1] @ S0])
            Sson2 = np.hstack([B2, L0[k1:] @ S0])
            Tson2 = np.vstack([B1, T0 @ R0[:, k1:]])
            Tson1 = np.vstack([B2, T0 @ R0[:, :k1]])
            Y2, DT2, Q2h = sv(Tson2)
            Y1, DT1, Q1h = sv(Tson1)
            P1, DS1, _ = sv(Sson1)
            P2, DS2, _ = sv(Sson2)
            k2n = max(int(np.sum(DT2 > acc)), int(np.sum(DS2 > acc)))
            k1n = max(int(np.sum(DT1 > acc)), int(np.sum(DS1 > acc)))
            Y1, Y2 = Y1[:, :k1n], Y2[:, :k2n]
            Q1, Q2 = Q1h.conj().T[:, :k1n], Q2h.conj().T[:, :k2n]
            P1, P2 = P1[:, :k1n], P2[:, :k2n]
            DT1m, DT2m = np.diag(DT1[:k1n]), np.diag(DT2[:k2n])
            sib[s1] = P1.conj().T @ Y2[:k1] @ DT2m
            sib[s2] = P2.conj().T @ Y1[:k2] @ DT1m
            Tp[s1], Tp[s2] = DT1m, DT2m
            Sp[s1], Sp[s2] = np.diag(DS1[:k1n]), np.diag(DS2[:k2n])
            Rp[ib] = np.hstack([R0[:, :k1] @ Q1, R0[:, k1:] @ Q2])
            Lp[ib] = np.vstack([P1.conj().T @ L0[:k1], P2.conj().T @ L0[k1:]])
        Rp[s1], Rp[s2] = Q1.conj().T @ R1, Q2.conj().T @ R2
        Lp[s1], Lp[s2] = L1 @ P1, L2 @ P2
    N = HSS1DMatrix(t)
    for name in ("nskel", "kskel", "I_SKUP", "I_SKDN", "T_UP", "J_UP", "T_DN", "J_DN",
                 "M_SELF", "M_SIB", "census"):
        setattr(N, name, [None] * nb)
    rho, lam = [None] * nb, [None] * nb
    for ib in range(nb - 1, -1, -1):
        if t.is_leaf(ib):
            out = inn = _leaf_range(t, ib)
            N.M_SELF[ib] = A.M_SELF[ib]
            RNEW, LNEW = Rp.get(ib), Lp.get(ib)
        else:
            s1, s2 = t.c1[ib], t.c2[ib]
            out = np.concatenate([N.I_SKUP[s1], N.I_SKUP[s2]])
            inn = np.concatenate([N.I_SKDN[s1], N.I_SKDN[s2]])
            N.M_SIB[s1] = lam[s1] @ sib[s1] @ rho[s2]
            N.M_SIB[s2] = lam[s2] @ sib[s2] @ rho[s1]
            if ib > 0:
                RA, LA = Rp[ib], Lp[ib]
                ka1 = rho[s1].shape[0]
                RNEW = np.hstack([RA[:, :ka1] @ rho[s1], RA[:, ka1:] @ rho[s2]])
                LNEW = np.vstack([lam[s1] @ LA[:ka1], lam[s2] @ LA[ka1:]])
        if ib == 0:
            continue
        k = min(RNEW.shape)
        Rq, Jout = idecomp.pivoted_qr(RNEW)
        Tout = idecomp.id_fixed_from_qr(Rq, Jout, k)
        Rq2, Jin = idecomp.pivoted_qr(LNEW.T)
        Tin = idecomp.id_fixed_from_qr(Rq2, Jin, k)
        N.I_SKUP[ib], N.T_UP[ib], N.J_UP[ib] = out[Jout[:k]], Tout, Jout
        N.I_SKDN[ib], N.T_DN[ib], N.J_DN[ib] = inn[Jin[:k]], Tin, Jin
        N.nskel[ib], N.kskel[ib] = len(out), k
        N.census[ib] = (RNEW.shape[0], LNEW.shape[1], len(out), k, k, k)
        rho[ib] = RNEW[:, Jout[:k]]
        lam[ib] = LNEW[Jin[:k], :]
    return N
