"""Generate the golden fixtures under tests/golden/ from the oracle.

    python tests/golden/make_golden.py

The reference is MATLAB and cannot run here, and its own tests hold no
golden vectors (they print errors against dense solves), so the fixtures are
oracle outputs for the small cases the parity tests use; the oracle itself is
pinned by tests/test_oracle_*.py to the reference tests' error criteria.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.abspath(os.path.join(HERE, "..", "..")))

from oracle import geometry, hss1d, hss2d, kernels, rng  # noqa: E402


def hss1d_star(N=4096, leaf=64, acc=1e-10):
    X = geometry.star_curve(N)
    kp = kernels.KernelParams(flag=kernels.DL_L_2D)
    H = hss1d.compress_nsym(X, leaf, acc, kp)
    inv = hss1d.invert_nsym(H)
    f = np.random.default_rng(0).standard_normal(N)
    x = hss1d.applyinv_nsym(H, inv, f)
    nb = H.tree.nboxes
    k = np.array([H.kskel[b] if b else 0 for b in range(nb)], np.int32)
    up = np.concatenate([H.I_SKUP[b] for b in range(1, nb)]).astype(np.int32)
    dn = np.concatenate([H.I_SKDN[b] for b in range(1, nb)]).astype(np.int32)
    return dict(N=N, leaf=leaf, acc=acc, kskel=k, I_SKUP=up, I_SKDN=dn, f=f, x=x)


def hss2d_small(npan=4, Ng=8):
    kp = kernels.KernelParams(flag=kernels.SL_L_2D, h=2.0 / (Ng * npan), c=kernels.Modulation(0.5, 0.0, 0.0, 20.0))
    prm = hss2d.HSS2DParams(Ng=Ng, npan=npan, acc=1e-10, layers=2, kp=kp)
    tree = hss2d.build_tree_nsym(prm)
    blk = hss2d.compress_nsym(tree, prm)
    inv = hss2d.invert_nsym(tree, prm, blk)
    f = np.random.default_rng(0).standard_normal(prm.N)
    x = hss2d.applyinv_nsym(tree, inv, f)
    J = np.concatenate([tree.J[b] for b in range(tree.nboxes)]).astype(np.int32)
    k = np.array(tree.k, np.int32)
    return dict(npan=npan, Ng=Ng, J=J, k=k, f=f, x=x)


def rng_kat():
    return dict(u=rng.uniform(0, rng.id_stream(5, 1), 8), u2=rng.uniform(12345, 7, 4))


if __name__ == "__main__":
    np.savez_compressed(os.path.join(HERE, "hss1d_star4096.npz"), **hss1d_star())
    np.savez_compressed(os.path.join(HERE, "hss2d_npan4.npz"), **hss2d_small())
    np.savez_compressed(os.path.join(HERE, "rng_kat.npz"), **rng_kat())
    print("wrote fixtures to", HERE)
