"""HSS2D (compressed-block HSS, dense-block "HSS-D" path) oracle restatement.

Follows:
  Common/HSS_tree_parameters.m:108-162     (params, X_source)
  HSS2D/HSS2D_build_tree_nsym.m            (uniform tree :145-277 with bisect_level
                                            :1183-1240; Build_I_source_unif :1097-1124;
                                            upward skeleton pass :342-559; 'bdry' preset
                                            skeletons :732-792; orient :794-811; dense
                                            interpolation operators :814-868; proxy
                                            :870-961)
  HSS2D/build_box_proxy.m:52-88
  HSS2D/interpolation_operator.m:57-77     (dense T = K11 \\ K21)
  HSS2D/HSS2D_compress_nsym.m:67-125       (dense Bself, B12, B21)
  HSS2D/HSS2D_invert_nsym.m:70-155         (Fopts='dense')
  HSS2D/HSS2D_build_Finv_nsym.m:92-100     (dense FI = inv([E1 K12; K21 E2]))
  HSS2D/HSS2D_build_E_nsym.m:43-51         (dense, LR = 0: E = inv(R FI L))
  HSS2D/HSS2D_apply_nsym.m:74-218
  HSS2D/HSS2D_applyinv_nsym.m:74-243 with HSS2D_applyFinv_nsym.m:30-31

Boxes are 0-based heap-numbered (box b has children 2b+1, 2b+2), which is the
reference's 1-based numbering (children 2B, 2B+1) shifted by one.  Index arrays
are 0-based.
"""
from __future__ import annotations

from dataclasses import dataclass, field
import math

import numpy as np

from .kernels import KernelParams, kernel_eval, SL_L_2D, SL_H_2D
from . import geometry
from . import idecomp


@dataclass
class HSS2DParams:
    """The fields of params (HSS_tree_parameters.m:115-139) the dense path reads."""

    Ng: int
    npan: int
    acc: float = 1e-10
    layers: int = 2
    kp: KernelParams = field(default_factory=KernelParams)
    INTERform: str = "dense"
    transinv: int = 0
    sym: int = 0
    k_cut: int = 2500
    seed: int = 0
    # uniform level layout of the GPU build (the reference keeps per-box ranks): on the ID
    # levels of the Helmholtz tree every box takes the level's largest rank (promote_id), on
    # the preset levels above them the level's largest boundary count (promote_skeleton)
    uniform_ranks: bool = False
    # params.proxy_rule / lambda / skel_extra_pts (HSS_tree_parameters.m:121-124)
    proxy_rule: str = "bdry"
    # params.skel_rule (HSS2D_build_tree_nsym.m:399-412, :668-730): 'bdry' boundary layers,
    # 'rand' a random sample of the box's points, 'wdec' a Whitney decomposition of the box,
    # 'ID' the ID of K(proxies, box) on every level
    skel_rule: str = "bdry"
    lambda_: float = 2.0
    skel_extra_pts: int = 0

    @property
    def h(self):
        return 2.0 / (self.Ng * self.npan)

    @property
    def depth(self):
        nlevels = int(round(2 * (math.log(self.npan) / math.log(2) - 1) + 3))
        return nlevels - 1

    @property
    def N(self):
        return self.npan * self.npan * self.Ng * self.Ng

    def X_source(self):
        return geometry.grid_source(self.Ng, self.npan)


def box_radii(lev):
    """(colrad, rowrad) of a level (HSS2D_build_tree_nsym.m:343-347)."""
    scl = lev // 2
    rowrad = 2.0 ** (-scl)
    colrad = rowrad / (2 ** (lev % 2))
    return colrad, rowrad


def box_centers(depth):
    """cent of bisect_level (:1183-1240): level-even boxes split in x, odd in y."""
    nb = 2 ** (depth + 1) - 1
    cent = np.zeros((nb, 2))
    for lev in range(depth):
        scl = lev // 2
        d = 0.5 * (0.5 ** scl)
        for b in range(2 ** lev - 1, 2 ** (lev + 1) - 1):
            c = cent[b]
            if lev % 2 == 0:
                cent[2 * b + 1] = (c[0] - d, c[1])
                cent[2 * b + 2] = (c[0] + d, c[1])
            else:
                cent[2 * b + 1] = (c[0], c[1] + d)
                cent[2 * b + 2] = (c[0], c[1] - d)
    return cent


def _colon(a, step, b):
    """MATLAB a:step:b for values on an h-grid."""
    n = int(math.floor((b - a) / step + 1e-9)) + 1
    if n <= 0:
        return np.zeros(0)
    return a + step * np.arange(n)


def build_box_proxy(cB, colrad, rowrad, layers, h):
    """build_box_proxy.m:52-88; returns [X_proxy; X_extra] as the 'bdry' rule uses it."""
    cx, cy = cB
    width = (layers - 0.5) * h
    xs1 = _colon(cx - colrad - width, h, cx - colrad - h / 2)
    ys1 = _colon(cy - rowrad - width, h, cy + rowrad + width)
    X1 = np.stack([np.tile(xs1, len(ys1)), np.repeat(ys1, len(xs1))], axis=1)
    xs2 = _colon(cx - colrad + h / 2, h, cx + colrad - h / 2)
    ys2 = _colon(cy + rowrad + width, -h, cy + rowrad + h / 2)
    X2 = np.stack([np.repeat(xs2, len(ys2)), np.tile(ys2, len(xs2))], axis=1)
    xs3 = _colon(cx + colrad + h / 2, h, cx + colrad + width)
    ys3 = _colon(cy + rowrad + width, -h, cy - rowrad - width)
    X3 = np.stack([np.tile(xs3, len(ys3)), np.repeat(ys3, len(xs3))], axis=1)
    xs4 = _colon(cx + colrad - h / 2, -h, cx - colrad + h / 2)
    ys4 = _colon(cy - rowrad - h / 2, -h, cy - rowrad - width)
    X4 = np.stack([np.repeat(xs4, len(ys4)), np.tile(ys4, len(xs4))], axis=1)
    r1 = layers * layers - 0.5
    r2 = layers * layers + 0.5
    W = rowrad + width
    V = colrad + width
    I1 = ((np.abs(X1[:, 0] - cx) > (V - h / 2)) & ((X1[:, 1] - cy > (W - r1 * h)) | (X1[:, 1] - cy < -(W - r2 * h)))) \
        | (np.abs(X1[:, 1] - cy) > (W - h / 2))
    I2 = (np.abs(X2[:, 1] - cy) > (W - h / 2)) & ((X2[:, 0] - cx > (V - r1 * h)) | (X2[:, 0] - cx < -(V - r2 * h)))
    I3 = ((np.abs(X3[:, 0] - cx) > (V - h / 2)) & ((X3[:, 1] - cy > (W - r2 * h)) | (X3[:, 1] - cy < -(W - r1 * h)))) \
        | (np.abs(X3[:, 1] - cy) > (W - h / 2))
    I4 = (np.abs(X4[:, 1] - cy) > (W - h / 2)) & ((X4[:, 0] - cx > (V - r2 * h)) | (X4[:, 0] - cx < -(V - r1 * h)))
    return np.vstack([X1[~I1], X2[~I2], X3[~I3], X4[~I4], X1[I1], X2[I2], X3[I3], X4[I4]])


def orient_residual(X_rs, nrm, tan):
    """LOCAL_orient_residual, HSS2D_build_tree_nsym.m:805-811 (stable sorts)."""
    J1 = np.argsort(X_rs[:, nrm], kind="stable")
    J2 = np.argsort(-X_rs[J1, tan], kind="stable")
    return J1[J2]


def orient_skeleton(X_sk, cB, th0):
    """LOCAL_orient_skeleton, HSS2D_build_tree_nsym.m:794-802."""
    dx = X_sk[:, 0] - cB[0]
    dy = X_sk[:, 1] - cB[1]
    # libm atan2/hypot (cart2pol), the same calls the host C++ tree builder makes
    th = np.array([math.atan2(a, b) for a, b in zip(dy.tolist(), dx.tolist())])
    rho = np.array([math.hypot(a, b) for a, b in zip(dx.tolist(), dy.tolist())])
    th = np.where(th < th0, th + 2.0 * math.pi, th)
    J1 = np.argsort(rho, kind="stable")
    J2 = np.argsort(th[J1], kind="stable")
    return J1[J2]


def preset_skeleton(X_src, cB, lev, colrad, rowrad, layers, h):
    """LOCAL_Preset_Skeleton_Info 'bdry' branch, :732-792. Returns (J, k)."""
    width = layers * h
    bdry = (np.abs(X_src[:, 0] - cB[0]) > (colrad - width)) | (np.abs(X_src[:, 1] - cB[1]) > (rowrad - width))
    if lev % 2 == 0:
        nrm, tan, th0 = 0, 1, math.pi / 2
    else:
        nrm, tan, th0 = 1, 0, 0.0
    idx = np.arange(X_src.shape[0])
    I_rs = idx[~bdry]
    I_rs = I_rs[orient_residual(X_src[~bdry], nrm, tan)]
    I_sk = idx[bdry]
    I_sk = I_sk[orient_skeleton(X_src[bdry], cB, th0)]
    return np.concatenate([I_sk, I_rs]), len(I_sk)


@dataclass
class HSS2DTree:
    depth: int
    cent: np.ndarray
    I_src: list
    I_sk: list
    J: list
    k: list
    T_up: list
    T_dn: list
    proxy: list
    leaf_of_panel: np.ndarray

    @property
    def nboxes(self):
        return len(self.I_src)

    def children(self, b):
        return 2 * b + 1, 2 * b + 2

    def is_leaf(self, b):
        return 2 * b + 1 >= self.nboxes


def lay_prox(prm: HSS2DParams, lev):
    """HSS2D_build_tree_nsym.m:360-368."""
    if lev > 0:
        if prm.kp.flag == SL_L_2D:
            return prm.layers + 1
        colrad, rowrad = box_radii(lev)
        return 2 * int(round(min(colrad, rowrad) / prm.h))
    return prm.layers


def leaf_sources(prm: HSS2DParams, cent):
    """Build_I_source_unif (:1097-1124): the panel whose first point a leaf holds."""
    depth = prm.depth
    J = prm.Ng * prm.Ng
    X = prm.X_source()
    first = X[0::J]
    colrad, rowrad = box_radii(depth)
    l0 = 2 ** depth - 1
    leaf_of_panel = np.empty(first.shape[0], dtype=np.int64)
    lc = cent[l0:]
    for i, p in enumerate(first):
        hit = np.nonzero((np.abs(p[0] - lc[:, 0]) < colrad) & (np.abs(p[1] - lc[:, 1]) < rowrad))[0]
        assert hit.size == 1
        leaf_of_panel[i] = l0 + hit[0]
    return leaf_of_panel


def build_tree_nsym(prm: HSS2DParams, with_T: bool = True) -> HSS2DTree:
    """INFO_TREE = HSS2D_build_tree_nsym(params), 'uniform'/'bdry'/'bdry'.  With transinv
    (:421-438, :507-548) the first box of each level computes (J, k, T) and every other
    box of the level takes them over on its own source set."""
    depth = prm.depth
    h = prm.h
    X = prm.X_source()
    cent = box_centers(depth)
    nb = 2 ** (depth + 1) - 1
    lop = leaf_sources(prm, cent)
    J = prm.Ng * prm.Ng
    I_src = [None] * nb
    for i, b in enumerate(lop):
        I_src[b] = np.arange(J * i, J * (i + 1))
    I_sk = [None] * nb
    Js = [None] * nb
    ks = [0] * nb
    T_up = [None] * nb
    T_dn = [None] * nb
    proxy = [None] * nb
    lowrank = {}
    q = [0] * (depth + 1)          # q(lev+1) of the reference: widest T.U of each level
    for lev in range(depth, -1, -1):
        colrad, rowrad = box_radii(lev)
        lp = lay_prox(prm, lev)
        qlev = 0
        ids = {}
        presets = {}
        first = 2 ** lev - 1
        followers = []
        for b in range(2 ** lev - 1, 2 ** (lev + 1) - 1):
            if 2 * b + 1 < nb:
                I_src[b] = np.concatenate([I_sk[2 * b + 1], I_sk[2 * b + 2]])
            X_src = X[I_src[b]]
            Xp = build_box_proxy(cent[b], colrad, rowrad, lp, h)
            if prm.proxy_rule == "rand":
                Xp = random_proxy(Xp, len(I_src[b]), cent[b], colrad, rowrad, lev, prm)
            elif prm.proxy_rule == "wdec":
                Xp = Xp[whitney_curve_mask(Xp, cent[b], np.array([colrad, rowrad]), 2 * prm.layers, h)]
            proxy[b] = Xp
            if prm.transinv and b != first:
                followers.append(b)
                continue
            if prm.skel_rule == "ID" or (prm.kp.flag == SL_H_2D and lev >= depth - 1):
                # :399-412 -- kh > 0: skeletons by the ID on the two finest levels (on
                # every level with skel_rule 'ID')
                ids[b] = (X_src, id_box(prm, Xp, X_src, b))
                continue
            if prm.skel_rule == "rand":
                presets[b] = random_skeleton(X_src, cent[b], lev, colrad, rowrad, prm)
            elif prm.skel_rule == "wdec":
                presets[b] = whitney_skeleton(X_src, cent[b], lev, colrad, rowrad, prm)
            else:
                presets[b] = preset_skeleton(X_src, cent[b], lev, colrad, rowrad, prm.layers, h)
        if prm.uniform_ranks and presets:
            # the boundary-layer counts of boxes above ID levels differ; every box takes the
            # level's largest count, promoting the residual points nearest its boundary
            kl = max(kb for _, kb in presets.values())
            for b, (Jb, kb) in presets.items():
                if kb < kl:
                    presets[b] = promote_skeleton(X[I_src[b]], Jb, kb, kl, cent[b], colrad, rowrad, lev)
        for b, (Jb, kb) in presets.items():
            X_src = X[I_src[b]]
            Xp = proxy[b]
            Js[b] = Jb
            ks[b] = kb
            I_sk[b] = I_src[b][Jb[:kb]]
            if with_T and lev > 0:
                X_sk, X_rs = X_src[Jb[:kb]], X_src[Jb[kb:]]
                if uses_lowrank(prm, lev, depth, kb, X_rs.shape[0]):
                    lr = interpolation_lowrank(prm, Xp, X_sk, X_rs, q, lev, b)
                    lowrank[b] = lr
                    T_up[b] = lr["Uu"] @ lr["Vu"].T
                    T_dn[b] = lr["Ud"] @ lr["Vd"].T
                    qlev = max(qlev, lr["Uu"].shape[1], lr["Ud"].shape[1])
                else:
                    T_up[b], T_dn[b] = interpolation_dense(prm, Xp, X_sk, X_rs)
                    qlev = max(qlev, T_up[b].shape[1])
                if prm.skel_extra_pts and len(Jb) - kb > 0:
                    # T = T.U T.V' is kept dense after the update (the reference keeps the
                    # factors, :1111-1121; their product is this T)
                    lowrank.pop(b, None)
                    T_up[b], T_dn[b], Jb, kb = extra_points(prm, T_up[b], T_dn[b], Jb, kb, Xp, X_src, cent[b],
                                                            lev, b)
                    Js[b], ks[b] = Jb, kb
                    I_sk[b] = I_src[b][Jb[:kb]]
        if ids:
            # the ID level's skeletons; with uniform_ranks every box holds the level's
            # largest rank: residual points join the skeleton with zero rows of T
            kl = max(r[2] for _, r in ids.values())
            for b, (X_src, (Tt, Jp, k, R)) in ids.items():
                if prm.uniform_ranks and k < kl:
                    Tt, Jp, k = promote_id(Tt, Jp, k, kl, X_src, cent[b], colrad, rowrad)
                Tb, Jb, kb = orient_id(Tt, Jp, k, X_src, cent[b], lev)
                Js[b] = Jb
                ks[b] = kb
                I_sk[b] = I_src[b][Jb[:kb]]
                T_up[b] = T_dn[b] = Tb
                qlev = max(qlev, Tb.shape[1])
        for b in followers:   # transinv: the level's first box's skeleton data
            Js[b], ks[b], T_up[b], T_dn[b] = Js[first], ks[first], T_up[first], T_dn[first]
            I_sk[b] = I_src[b][Js[first][:ks[first]]]
        if lev > 0:
            q[lev] = qlev
    tree = HSS2DTree(depth, cent, I_src, I_sk, Js, ks, T_up, T_dn, proxy, lop)
    tree.lowrank = lowrank
    tree.q = q
    return tree


def promote_skeleton(X_src, J, k, kl, cB, colrad, rowrad, lev):
    """The uniform level layout above the ID levels of a kh > 0 tree (the GPU build's; the
    reference keeps per-box counts): a box with k < kl boundary points promotes the kl - k
    residual points nearest its boundary (distance min(colrad - |x - cx|, rowrad - |y - cy|),
    ties in the residual order), then orders both sets as LOCAL_Preset_Skeleton_Info does.
    Returns (J, kl)."""
    rs = J[k:]
    d = np.minimum(colrad - np.abs(X_src[rs, 0] - cB[0]), rowrad - np.abs(X_src[rs, 1] - cB[1]))
    o = np.argsort(d, kind="stable")[:kl - k]
    take = np.zeros(len(rs), dtype=bool)
    take[o] = True
    sk = np.concatenate([J[:k], rs[o]])
    rest = rs[~take]
    if lev % 2 == 0:
        nrm, tan, th0 = 0, 1, math.pi / 2
    else:
        nrm, tan, th0 = 1, 0, 0.0
    sk = sk[orient_skeleton(X_src[sk], cB, th0)]
    rest = rest[orient_residual(X_src[rest], nrm, tan)]
    return np.concatenate([sk, rest]), kl


def promote_id(T, J, k, kl, X_src, cB, colrad, rowrad):
    """The uniform level layout of the ID levels (the GPU build's; the reference keeps
    per-box ranks): a box of rank k < kl moves the kl - k residual points nearest its boundary
    (distance min(colrad - |x - cx|, rowrad - |y - cy|), ties in the ID's residual order) into
    its skeleton.  Their rows of T are zero: A(:, sk) T = A(:, rs) holds unchanged for the
    remaining residual points, so the interpolation error is the ID's own.
    Returns (T, J, kl) with the promoted points after the ID's skeleton."""
    rs = J[k:]
    d = np.minimum(colrad - np.abs(X_src[rs, 0] - cB[0]), rowrad - np.abs(X_src[rs, 1] - cB[1]))
    o = np.argsort(d, kind="stable")[:kl - k]
    take = np.zeros(len(rs), dtype=bool)
    take[o] = True
    keep = np.flatnonzero(~take)
    Tn = np.vstack([T[:, keep], np.zeros((kl - k, len(keep)), dtype=T.dtype)])
    return Tn, np.concatenate([J[:k], rs[o], rs[keep]]), kl


def random_sampler(X, cB, colrad, rowrad, lam, lay, h):
    """LOCAL_random_sampler, HSS2D_build_tree_nsym.m:964-1001: points within lay*h of the
    box are kept, farther ones with probability 2^(-lam * l) by dyadic distance band l.
    The reference resets MATLAB's generator (rng('default'): the Mersenne Twister with its
    default seed, 5489) on every call; numpy's RandomState(5489) is that generator, so the
    same uniforms are drawn (not verified against MATLAB here)."""
    return X[sampler_mask(X, cB, colrad, rowrad, lam, lay, h)]


def mround(x):
    """MATLAB's round: half away from zero, exact (x - trunc(x) has no rounding error).
    Returns int64."""
    x = np.asarray(x, dtype=np.float64)
    t = np.trunc(x)
    return (t + np.sign(x) * (np.abs(x - t) >= 0.5)).astype(np.int64)


def whitney_curve_mask(G, cB, rB, layers, h):
    """Common/Whitney_decomposition_1Dcurve.m with C = (0, 0), R = (1, 1) (its only call,
    LOCAL_Build_Proxy 'wdec', HSS2D_build_tree_nsym.m:877-881): a quadtree over [-1, 1]^2
    refines every box that holds more than one point and lies within freq 1.5 rad of the
    box boundary (freq = min(ceil(layers / 2), 2)), marking the points of least and largest
    integer coordinate in each direction (first on ties) of every box it splits; the points
    within layers h of the box boundary are added.  Returns the mask."""
    N = G.shape[0]
    coord = mround((0.0 + (1.0 - h / 2) + G) / h)
    dmax = max(int(coord[:, 0].max() - coord[:, 0].min()), int(coord[:, 1].max() - coord[:, 1].min()))
    depth = math.ceil(math.log2(dmax))
    freq = min(math.ceil(layers / 2), 2)
    B = np.zeros(N, dtype=bool)
    level = [(np.zeros(2), np.arange(N))]   # (centre, point indices) of the level's boxes
    cta = np.array([[-0.5, -0.5], [-0.5, 0.5], [0.5, -0.5], [0.5, 0.5]])
    for lev in range(depth):
        nxt = []
        for cent, J in level:
            if len(J) == 0:
                continue
            bc = coord[J]
            id_mn = np.argmin(bc, axis=0)
            id_mx = np.argmax(bc, axis=0)
            d = np.abs(cent - cB)
            i = int(np.argmax(d))
            dist = abs(rB[i] - d[i])
            rad = 2.0 ** (-lev)
            if len(J) > 1 and dist < freq * 1.5 * rad:
                cbc = mround((0.0 + (1.0 - h / 2) + cent) / h)
                rowmid, colmid = int(cbc[0]), int(cbc[1])
                masks = [(bc[:, 0] < rowmid) & (bc[:, 1] < colmid), (bc[:, 0] < rowmid) & (bc[:, 1] >= colmid),
                         (bc[:, 0] >= rowmid) & (bc[:, 1] < colmid), (bc[:, 0] >= rowmid) & (bc[:, 1] >= colmid)]
                for j in range(4):
                    nxt.append((cent + 2.0 ** (-lev) * cta[j], J[masks[j]]))
                B[J[[id_mn[0], id_mn[1], id_mx[0], id_mx[1]]]] = True
        level = nxt
    inf_nrm = np.abs(G - cB[None, :])
    dist = np.min(np.abs(rB[None, :] - inf_nrm), axis=1)
    bdry = (dist < layers * h) & (inf_nrm[:, 0] < rB[0] + layers * h) & (inf_nrm[:, 1] < rB[1] + layers * h)
    return B | bdry


def random_skeleton(X_src, cB, lev, colrad, rowrad, prm: HSS2DParams):
    """LOCAL_Preset_Skeleton_Info 'rand' (:703-730): the box's own points sampled by
    LOCAL_random_sampler (each retry on the full set with 0.9 lambda) until the sample
    reaches k0 / 1.1, k0 = ceil(2/3 n) (even levels) or ceil(3/4 n); skeleton and residual
    ordered as the 'bdry' rule orders them.  Returns (J, k)."""
    n = X_src.shape[0]
    k0 = math.ceil((2 / 3) * n) if lev % 2 == 0 else math.ceil((3 / 4) * n)
    lam, k = prm.lambda_, 0
    keep = np.zeros(n, dtype=bool)
    while k0 > 1.1 * k:
        keep = sampler_mask(X_src, cB, colrad, rowrad, lam, prm.layers, prm.h)
        k = int(keep.sum())
        if k0 > 1.1 * k:
            lam = 0.9 * lam
    if lev % 2 == 0:
        nrm, tan, th0 = 0, 1, math.pi / 2
    else:
        nrm, tan, th0 = 1, 0, 0.0
    idx = np.arange(n)
    I_rs = idx[~keep]
    I_rs = I_rs[orient_residual(X_src[~keep], nrm, tan)]
    I_sk = idx[keep]
    I_sk = I_sk[orient_skeleton(X_src[keep], cB, th0)]
    return np.concatenate([I_sk, I_rs]), len(I_sk)


def whitney_mask(X, cB, colrad, rowrad, layers, h, Ng):
    """Common/Whitney_decomposition.m: on the box's integer grid coordinates, the full
    boundary layers, then for each finer dyadic scale i the lines at distance c_i from the
    box edges sampled every 2^max(i - ceil(layers/2), 0) points (c_i a power of two below
    Ng, or Ng times one: the Ng x Ng panel grid).  Returns the skeleton mask."""
    c1 = mround((-cB[0] + (colrad - h / 2) + X[:, 0]) / h)
    c2 = mround((-cB[1] + (rowrad - h / 2) + X[:, 1]) / h)
    max1, max2 = int(c1.max()), int(c2.max())
    dmax = max(max1, max2)
    depth = math.ceil(math.log2(dmax)) + 1
    B = (c1 < layers) | (max1 - c1 < layers) | (c2 < layers) | (max2 - c2 < layers)
    freq = math.ceil(layers / 2)
    lNg = math.ceil(math.log2(Ng))
    for i in range(2, depth + 1):
        if 2 ** (i - 1) < Ng:
            ci, mi = 2 ** (i - 1), Ng
        else:
            ci = Ng * 2 ** (i - 1 - lNg)
            mi = 2 * ci
        e = 2 ** max(i - freq, 0)
        w = ((c1 == ci) | (c1 == max1 - ci)) & (((c2 % mi) % e == 0) | (c2 == max2 - ci))
        w |= ((c2 == ci) | (c2 == max2 - ci)) & (((c1 % mi) % e == 0) | (c1 == max1 - ci))
        B |= w
    return B


def whitney_skeleton(X_src, cB, lev, colrad, rowrad, prm: HSS2DParams):
    """LOCAL_Preset_Skeleton_Info 'wdec' (:668-701): the Whitney decomposition's points,
    ordered as the 'bdry' rule orders its sets.  Returns (J, k)."""
    keep = whitney_mask(X_src, cB, colrad, rowrad, prm.layers, prm.h, prm.Ng)
    if lev % 2 == 0:
        nrm, tan, th0 = 0, 1, math.pi / 2
    else:
        nrm, tan, th0 = 1, 0, 0.0
    idx = np.arange(X_src.shape[0])
    I_rs = idx[~keep]
    I_rs = I_rs[orient_residual(X_src[~keep], nrm, tan)]
    I_sk = idx[keep]
    I_sk = I_sk[orient_skeleton(X_src[keep], cB, th0)]
    return np.concatenate([I_sk, I_rs]), len(I_sk)


def sampler_mask(X, cB, colrad, rowrad, lam, lay, h):
    """The kept-point mask of LOCAL_random_sampler (random_sampler returns X[mask])."""
    D = np.abs(np.minimum(colrad - np.abs(X[:, 0] - cB[0]), rowrad - np.abs(X[:, 1] - cB[1])))
    width = lay * h
    rad = D.max()
    sz = -math.floor(math.log2(width / rad)) + 1
    prob = 2.0 ** (-lam * np.arange(sz - 1, -1, -1, dtype=np.float64))
    B = D < width
    with np.errstate(divide="ignore"):
        Ld = np.minimum(-np.ceil(np.log2(D / rad)), sz - 2) + 1
    Ld[B] = sz
    if sz > 0:
        P = prob[Ld.astype(np.int64) - 1]
        B = np.random.RandomState(5489).random_sample(P.shape[0]) < P
    return B


def random_proxy(X_ext, n_skel, cB, colrad, rowrad, lev, prm: HSS2DParams):
    """LOCAL_Build_Proxy, 'rand' rule (:883-905): the 'bdry' layers sampled until at least
    k0 = ceil(2/3 n) (even levels) or ceil(3/4 n) (odd) points remain; each retry samples
    the previous sample again with a wider target and 0.9 lambda, as the reference does."""
    k0 = math.ceil((2 / 3) * n_skel) if lev % 2 == 0 else math.ceil((3 / 4) * n_skel)
    k0 = min(k0, X_ext.shape[0])
    lam, k, c = prm.lambda_, 0, 0
    while k0 > k and c < 10:
        X_ext = random_sampler(X_ext, cB, colrad, rowrad, lam, prm.layers, prm.h)
        k = X_ext.shape[0]
        if k0 > k:
            lam = 0.9 * lam
        c += 1
    return X_ext


def extra_points(prm: HSS2DParams, Tu0, Td0, J0, k0, X_ext, X_src, cB, lev, box):
    """LOCAL_ID_rand_update (:1069-1124) with dense T, and the re-orientation of the NTI
    (:468-487) or TI (:516-528) branch: a randomized ID of the interpolation residual
    [K(X_ext, X_rs) - K(X_ext, X_sk) T_up; K(X_rs, X_ext).' - K(X_sk, X_ext).' T_dn]
    (2p x n_rs, q0 = 8 layers ceil(log2 k0), C = q0/2, problem 2*box of the shared RNG)
    promotes k1 residual points to skeletons; T = [T(:, J1_rs) - T(:, J1_sk) T1; T1].
    (The reference's Res_apply stacks the full A_sk twice; only its transpose, which
    splits A_sk correctly, enters the randomized ID.)  Returns (T_up, T_dn, J, k)."""
    from . import cid, randid
    kp = prm.kp
    J0_sk, J0_rs = J0[:k0], J0[k0:]
    Xrs, Xsk = X_src[J0_rs], X_src[J0_sk]
    p = X_ext.shape[0]
    A_rs = np.vstack([kernel_eval(X_ext, Xrs, kp), kernel_eval(Xrs, X_ext, kp).T])
    A_sk = np.vstack([kernel_eval(X_ext, Xsk, kp), kernel_eval(Xsk, X_ext, kp).T])
    Res = A_rs - np.vstack([A_sk[:p] @ Tu0, A_sk[p:] @ Td0])
    q0 = 8 * prm.layers * math.ceil(math.log2(k0))
    if np.iscomplexobj(Res):
        T1, J1, k1 = cid.id_rand_complex(Res, q0, q0 // 2, prm.acc, prm.seed, 2 * box)
    else:
        T1, J1, k1 = randid.id_rand(Res, q0, q0 // 2, prm.acc, prm.seed, 2 * box)
    J1_sk, J1_rs = J1[:k1], J1[k1:]
    kf = k0 + k1
    Jf = np.concatenate([J0_sk, J0_rs[J1]])
    Tfu = np.vstack([Tu0[:, J1_rs] - Tu0[:, J1_sk] @ T1, T1])
    Tfd = np.vstack([Td0[:, J1_rs] - Td0[:, J1_sk] @ T1, T1])
    if lev % 2 == 0:
        th = math.pi / 2 if (box + 1) % 2 == 0 else -math.pi / 2
        nrm, tan = 0, 1
    else:
        th = 0.0 if (box + 1) % 2 == 0 else -math.pi
        nrm, tan = 1, 0
    Js = orient_skeleton(X_src[Jf[:kf]], cB, th)
    # the translation-invariant branch (:520-528) also orders the residual points
    Jr = orient_residual(X_src[Jf[kf:]], nrm, tan) if prm.transinv else np.arange(len(Jf) - kf)
    return Tfu[np.ix_(Js, Jr)], Tfd[np.ix_(Js, Jr)], np.concatenate([Jf[:kf][Js], Jf[kf:][Jr]]), kf


def id_box(prm: HSS2DParams, X_ext, X_src, box):
    """The ID of LOCAL_Non_Preset_Skeleton_Info (HSS2D_build_tree_nsym.m:614-627): [T, J] =
    ID(K(X_ext, X_src), acc), the complex ID with problem 2*box of the shared RNG.
    Returns (T, J, k, R)."""
    from . import cid
    return cid.id_adaptive_complex(kernel_eval(X_ext, X_src, prm.kp), prm.acc, prm.seed, 2 * box)


def orient_id(Ttmp, J, k, X_src, cB, lev):
    """The rest of LOCAL_Non_Preset_Skeleton_Info (:629-656): skeleton points sorted around
    the box centre, residual points along the interface, T = T(Js, Jr), which serves both
    directions (T_dn = T_up).  Returns (T, J, k)."""
    if lev % 2 == 0:
        nrm, tan, th0 = 0, 1, math.pi / 2
    else:
        nrm, tan, th0 = 1, 0, 0.0
    I_sk, I_rs = J[:k], J[k:]
    Jr = orient_residual(X_src[I_rs], nrm, tan)
    Js = orient_skeleton(X_src[I_sk], cB, th0)
    return Ttmp[np.ix_(Js, Jr)], np.concatenate([I_sk[Js], I_rs[Jr]]), k


def uses_lowrank(prm: HSS2DParams, lev: int, depth: int, k: int, nr: int) -> bool:
    """LOCAL_Interpolation_Operators (HSS2D_build_tree_nsym.m:842-846): the low-rank T of
    INTERform 'lowrank' on levels above the leaves' parents with k < k_cut (the k >= k_cut
    branch, interpolation_operator_HSS, is the compressed-block path and is not built)."""
    return prm.INTERform == "lowrank" and lev < depth - 1 and k < prm.k_cut and k > 0 and nr > 0


def sample_guess(q, lev, m, n, up: bool):
    """First sample count k0 and block size C of the randomized ID
    (interpolation_operator.m:98-116 for box_2_proxy, :143-152 for proxy_2_box).

    The boxes of a level are processed together, so the same-level guess
    ``q(lev+1) + 1`` of the reference's box-by-box loop (:99-101) is never available:
    every box takes the finer-level guess.  ``q[l]`` = widest T.U on level l (0 if none).
    """
    mn = min(m, n)
    if sum(1 for v in q if v > 0) < 5:
        return min(math.ceil(9 * math.log2(mn) - 20), mn), 5
    a, b = q[lev + 2], q[lev + 4]
    if up:
        return min(max(math.ceil(2 * a - b + 2), a), mn), math.ceil(abs(a - b) / 2) + 1
    return min(math.ceil(2 * a - b + 2), mn), math.ceil(a - b / 2) + 1


def interpolation_lowrank(prm: HSS2DParams, Xp, X_sk, X_rs, q, lev, box):
    """interpolation_operator.m:79-131 (lr = 1): K21 ~ U V^T by LRID_rand, T.U = K11 \\ U,
    T.V = V, for box_2_proxy (randomized problem 2*box) and proxy_2_box (2*box+1)."""
    from . import randid
    kp = prm.kp
    out = {}
    for up, tag in ((True, "u"), (False, "d")):
        if up:
            K11 = kernel_eval(Xp, X_sk, kp)
            A = kernel_eval(Xp, X_rs, kp)          # p x nr; matvec K21*x
        else:
            K11 = kernel_eval(X_sk, Xp, kp).T
            A = kernel_eval(X_rs, Xp, kp).T        # p x nr; matvec K21.'*x
        m, n = A.shape
        k0, C = sample_guess(q, lev, m, n, up)
        if np.iscomplexobj(A):
            from . import cid
            U, V = cid.lrid_rand_complex(A, k0, C, prm.acc, prm.seed, 2 * box + (0 if up else 1))
            out["U" + tag] = np.linalg.lstsq(K11, U, rcond=None)[0]
        else:
            U, V = randid.lrid_rand(A, k0, C, prm.acc, prm.seed, 2 * box + (0 if up else 1))
            out["U" + tag] = idecomp.lstsq_qr(K11, U)
        out["V" + tag] = V
        out["k0" + tag] = k0
        out["C" + tag] = C
    return out


TIKHONOV_REL = 2.0 ** -40


def lstsq_tikhonov(A, B):
    """T = argmin ||A T - B||^2 + lam^2 ||T||^2, lam = 2^-40 ||A||_F, by the Householder QR of
    [A; lam I] (the complex interpolation systems' rule, GPU and oracle alike).  The
    Helmholtz proxy systems K11 of the preset levels are numerically rank deficient (cond
    ~1e14): the reference's K11 \\ K21 takes MATLAB's basic solution from a column-pivoted
    QR; an unpivoted QR's solution has 10-100x that norm and costs the inverse five digits.
    The damping keeps ||T|| near the minimum-norm solution's at an interpolation error of
    ~acc."""
    k = A.shape[1]
    lam = TIKHONOV_REL * np.linalg.norm(A)
    Aa = np.vstack([A, lam * np.eye(k)])
    Ba = np.vstack([B, np.zeros((k, B.shape[1]), dtype=np.result_type(A, B))])
    Q, R = np.linalg.qr(Aa)
    return np.linalg.solve(R, Q.conj().T @ Ba)


def interpolation_dense(prm: HSS2DParams, Xp, X_sk, X_rs):
    """interpolation_operator.m:57-77 with lr = 0: T_up (box_2_proxy), T_dn (proxy_2_box)."""
    k = X_sk.shape[0]
    if k == 0 or X_rs.shape[0] == 0:
        z = np.zeros((k, X_rs.shape[0]))
        return z, z
    kp = prm.kp
    # the damped least squares for the complex kernel and for the sampled / Whitney skeletons,
    # whose proxy systems are numerically rank deficient; the boundary-layer rule keeps the
    # plain Householder solve
    ls = lstsq_tikhonov if (kp.flag == SL_H_2D or prm.skel_rule != "bdry") else idecomp.lstsq_qr
    K11 = kernel_eval(Xp, X_sk, kp)
    K21 = kernel_eval(Xp, X_rs, kp)
    Tu = ls(K11, K21)
    K11d = kernel_eval(X_sk, Xp, kp).T
    K21d = kernel_eval(X_rs, Xp, kp).T
    Td = ls(K11d, K21d)
    return Tu, Td


@dataclass
class HSS2DBlocks:
    Bself: dict
    B12: dict
    B21: dict


def _as_vectors(Xv, tree):
    """Right-hand sides in the tree's arithmetic: complex when its T are (Helmholtz)."""
    Xv = np.asarray(Xv)
    cplx = any(t is not None and np.iscomplexobj(t) for t in tree.T_up)
    return Xv.astype(np.complex128 if cplx or np.iscomplexobj(Xv) else np.float64, copy=False)


def compress_nsym(tree: HSS2DTree, prm: HSS2DParams) -> HSS2DBlocks:
    """A_HSS = HSS2D_compress_nsym(INFO_TREE, params), dense branch (:81-107)."""
    X = prm.X_source()
    kp = prm.kp
    Bs, B12, B21 = {}, {}, {}
    for b in range(tree.nboxes):
        if tree.is_leaf(b):
            Xi = X[tree.I_src[b]]
            Bs[b] = kernel_eval(Xi, Xi, kp)
        else:
            c1, c2 = tree.children(b)
            X1 = X[tree.I_sk[c1]]
            X2 = X[tree.I_sk[c2]]
            B12[b] = kernel_eval(X1, X2, kp)
            B21[b] = kernel_eval(X2, X1, kp)
    return HSS2DBlocks(Bs, B12, B21)


def _R_L(tree, b):
    k = tree.k[b]
    Jb = tree.J[b]
    n = len(Jb)
    dt = np.result_type(tree.T_up[b], tree.T_dn[b])
    R = np.zeros((k, n), dtype=dt)
    R[:, Jb] = np.hstack([np.eye(k), tree.T_up[b]])
    L = np.zeros((n, k), dtype=dt)
    L[Jb, :] = np.hstack([np.eye(k), tree.T_dn[b]]).T
    return R, L


def invert_nsym(tree: HSS2DTree, prm: HSS2DParams, blocks: HSS2DBlocks | None = None):
    """A_HSS = HSS2D_invert_nsym(INFO_TREE, params) with Fopts = 'dense'.

    Returns dict with FI (per box) and E (per non-root box).
    """
    X = prm.X_source()
    kp = prm.kp
    nb = tree.nboxes
    FI = [None] * nb
    E = [None] * nb
    for lev in range(tree.depth, -1, -1):
        for b in range(2 ** lev - 1, 2 ** (lev + 1) - 1):
            if tree.is_leaf(b):
                Xi = X[tree.I_src[b]]
                A = blocks.Bself[b] if blocks is not None else kernel_eval(Xi, Xi, kp)
                FI[b] = np.linalg.inv(A)
            else:
                c1, c2 = tree.children(b)
                if blocks is not None:
                    K12, K21 = blocks.B12[b], blocks.B21[b]
                else:
                    X1, X2 = X[tree.I_sk[c1]], X[tree.I_sk[c2]]
                    K12, K21 = kernel_eval(X1, X2, kp), kernel_eval(X2, X1, kp)
                F = np.block([[E[c1], K12], [K21, E[c2]]])
                FI[b] = np.linalg.inv(F)
            if lev > 0:
                R, L = _R_L(tree, b)
                E[b] = np.linalg.inv(R @ (FI[b] @ L))
    return {"FI": FI, "E": E}


def apply_nsym(tree: HSS2DTree, blocks: HSS2DBlocks, Xv: np.ndarray) -> np.ndarray:
    """Y = HSS2D_apply_nsym(INFO_TREE, A_HSS, X, params), :74-218 (LR = 0)."""
    Xv = _as_vectors(Xv, tree)
    vec = Xv.ndim == 1
    if vec:
        Xv = Xv[:, None]
    nb = tree.nboxes
    up = [None] * nb
    dn = [None] * nb
    for lev in range(tree.depth, 0, -1):
        for b in range(2 ** lev - 1, 2 ** (lev + 1) - 1):
            if tree.is_leaf(b):
                q = Xv[tree.I_src[b]]
            else:
                c1, c2 = tree.children(b)
                q = np.vstack([up[c1], up[c2]])
            k = tree.k[b]
            Jb = tree.J[b]
            if k < len(Jb):
                up[b] = q[Jb[:k]] + tree.T_up[b] @ q[Jb[k:]]
            else:
                up[b] = q[Jb]
    Y = np.zeros_like(Xv)
    for lev in range(0, tree.depth + 1):
        for b in range(2 ** lev - 1, 2 ** (lev + 1) - 1):
            if tree.is_leaf(b):
                lam = blocks.Bself[b] @ Xv[tree.I_src[b]]
            else:
                c1, c2 = tree.children(b)
                lam = np.vstack([blocks.B12[b] @ up[c2], blocks.B21[b] @ up[c1]])
            eta = np.zeros_like(lam)
            if lev > 0:
                k = tree.k[b]
                Jb = tree.J[b]
                tmp = dn[b]
                if k < len(Jb):
                    eta[Jb] = np.vstack([tmp, tree.T_dn[b].T @ tmp])
                else:
                    eta[Jb] = tmp
            phi = eta + lam
            if tree.is_leaf(b):
                Y[tree.I_src[b]] = phi
            else:
                c1, c2 = tree.children(b)
                k1 = tree.k[c1]
                dn[c1] = phi[:k1]
                dn[c2] = phi[k1:]
    return Y[:, 0] if vec else Y


def applyinv_nsym(tree: HSS2DTree, inv: dict, Xv: np.ndarray) -> np.ndarray:
    """Y = HSS2D_applyinv_nsym(INFO_TREE, A_HSS, X, params), :74-243 (dense, LR = 0)."""
    Xv = _as_vectors(Xv, tree)
    vec = Xv.ndim == 1
    if vec:
        Xv = Xv[:, None]
    nb = tree.nboxes
    FI, E = inv["FI"], inv["E"]
    up = [None] * nb
    dn = [None] * nb
    for lev in range(tree.depth, 0, -1):
        for b in range(2 ** lev - 1, 2 ** (lev + 1) - 1):
            if tree.is_leaf(b):
                q = Xv[tree.I_src[b]]
            else:
                c1, c2 = tree.children(b)
                q = np.vstack([up[c1], up[c2]])
            psi = FI[b] @ q
            k = tree.k[b]
            Jb = tree.J[b]
            if k < len(Jb):
                tmp = psi[Jb[:k]] + tree.T_up[b] @ psi[Jb[k:]]
            else:
                tmp = psi[Jb]
            up[b] = E[b] @ tmp
    Y = np.zeros_like(Xv)
    for lev in range(0, tree.depth + 1):
        for b in range(2 ** lev - 1, 2 ** (lev + 1) - 1):
            k = tree.k[b]
            Jb = tree.J[b]
            n = len(Jb)
            if lev == 0:
                lam = np.vstack([up[1], up[2]])
                eta = np.zeros_like(lam)
            else:
                tmp = np.zeros((n, Xv.shape[1]), dtype=Xv.dtype)
                if k < n:
                    tmp[Jb] = np.vstack([up[b], tree.T_dn[b].T @ up[b]])
                else:
                    tmp[Jb] = up[b]
                if tree.is_leaf(b):
                    q = Xv[tree.I_src[b]]
                else:
                    c1, c2 = tree.children(b)
                    q = np.vstack([up[c1], up[c2]])
                lam = q - tmp
                t2 = E[b] @ dn[b]
                eta = np.zeros_like(lam)
                if k < n:
                    eta[Jb] = np.vstack([t2, tree.T_dn[b].T @ t2])
                else:
                    eta[Jb] = t2
            phi = FI[b] @ (eta + lam)
            if tree.is_leaf(b):
                Y[tree.I_src[b]] = phi
            else:
                c1, c2 = tree.children(b)
                k1 = tree.k[c1]
                dn[c1] = phi[:k1]
                dn[c2] = phi[k1:]
    return Y[:, 0] if vec else Y


def kernel_matvec(prm: HSS2DParams, Xv: np.ndarray, block: int = 4096) -> np.ndarray:
    """A @ Xv for the dense kernel matrix A = K[X_source, X_source], blockwise."""
    X = prm.X_source()
    Xv = np.asarray(Xv)
    cplx = np.iscomplexobj(Xv) or prm.kp.flag == SL_H_2D
    Xv = Xv.astype(np.complex128 if cplx else np.float64, copy=False)
    out = np.zeros_like(Xv)
    for i in range(0, X.shape[0], block):
        out[i:i + block] = kernel_eval(X[i:i + block], X, prm.kp) @ Xv
    return out


def iterative_refinement(apply_A, apply_inv, B, acc, maxit=10):
    """Common/Iterative_Refinement.m:20-35 (absolute-norm stop, as the reference)."""
    Xs = apply_inv(B)
    res = B - apply_A(Xs)
    err = np.linalg.norm(res)
    it = 1
    hist = [err]
    while err > acc and it < maxit:
        Xs = Xs + apply_inv(res)
        res = B - apply_A(Xs)
        err = np.linalg.norm(res)
        it += 1
        hist.append(err)
    return Xs, hist


def lev_hss(tree: HSS2DTree, n_cut: int, trinv: int = 0) -> int:
    """lHSS = levHSS(TREE, n_cut, trinv), HSS2D/levHSS.m:33-65: the first level whose
    smallest skeleton is <= n_cut (searched from the top; forced even), -1 if the top
    boxes are already small enough.  With the uniform tree every box of a level has the
    same k, which is also the translation-invariant LEV(l).k."""
    k = tree.k
    n_min = max(k[0], k[1], k[2])
    lev = 0
    while n_min > n_cut and lev < tree.depth - 1:
        lev += 1
        n_min = min(k[b] for b in range(2 ** lev - 1, 2 ** (lev + 1) - 1))
    if lev > 0:
        return lev - 1 if lev % 2 == 1 else lev
    return -1
