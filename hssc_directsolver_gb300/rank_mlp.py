"""Learned ID ranks: a small MLP trained on the ranks the plain ID produces.

The reference predicts skeleton sizes with a hand-fitted table
``rank ~ m*log10(n) - b`` per kernel and precision (HSS2D/predict_rank.m:5-23).
Here the network (8 -> 32 -> 32 -> 1, ReLU, sigmoid) maps per-box features
(``HSS1DMatrix.features``) to the rank fraction k/n, and
``HSS1D_compress_batch(..., predictor=P)`` uses the prediction to stop each
pivoted QR early.  Forward, backward and Adam are CUDA kernels in libhssgpu.so.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L

NFEAT = 8
HIDDEN = 32


class RankPredictor:
    def __init__(self, nin: int = NFEAT, hidden: int = HIDDEN, seed: int = 0):
        self._h = C.c_void_p()
        L.check(L.lib().hss_mlp_create(C.byref(self._h), int(nin), int(hidden), int(seed)))
        self.nin, self.hidden = nin, hidden

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                L.lib().hss_mlp_destroy(h)
            except Exception:
                pass
            self._h = None

    @property
    def nparams(self) -> int:
        n = C.c_int32()
        L.check(L.lib().hss_mlp_nparams(self._h, C.byref(n)))
        return n.value

    def params(self) -> np.ndarray:
        p = np.zeros(self.nparams, np.float32)
        L.check(L.lib().hss_mlp_get_params(self._h, L.ptr(p)))
        return p

    def set_params(self, p) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        if p.size != self.nparams:
            raise ValueError("parameter vector has the wrong length")
        L.check(L.lib().hss_mlp_set_params(self._h, L.ptr(p)))

    def _xt(self, X, t=None):
        X = np.ascontiguousarray(X, dtype=np.float32)
        if X.ndim != 2 or X.shape[1] != self.nin:
            raise ValueError(f"X must be B x {self.nin}")
        if t is None:
            return X, None
        t = np.ascontiguousarray(t, dtype=np.float32)
        if t.shape != (X.shape[0],):
            raise ValueError("t must have one target per row of X")
        return X, t

    def grad(self, X, t):
        """(loss, gradient) of 0.5*mean((y - t)^2)."""
        X, t = self._xt(X, t)
        g = np.zeros(self.nparams, np.float32)
        loss = C.c_float()
        L.check(L.lib().hss_mlp_grad(self._h, L.ptr(X), L.ptr(t), X.shape[0], L.ptr(g), C.byref(loss)))
        return loss.value, g

    def train(self, X, t, epochs: int = 200, batch: int = 256, lr: float = 3e-3) -> float:
        X, t = self._xt(X, t)
        loss = C.c_float()
        L.check(L.lib().hss_mlp_train(self._h, L.ptr(X), L.ptr(t), X.shape[0], int(epochs), int(batch),
                                      float(lr), C.byref(loss)))
        return loss.value

    def predict(self, X) -> np.ndarray:
        X, _ = self._xt(X)
        y = np.zeros(X.shape[0], np.float32)
        L.check(L.lib().hss_mlp_predict(self._h, L.ptr(X), X.shape[0], L.ptr(y)))
        return y


def training_set(K_HSS):
    """(features, rank fractions) of every non-root box of a plain compress."""
    F, y = K_HSS.features()
    inf = K_HSS.info()
    keep = inf["level"] > 0
    return F[keep], y[keep]
