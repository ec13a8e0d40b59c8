"""Learned-proposal form of SGMA from Python: recording traces of the exact
SGMA scores, training the proposal network on the GPU and installing it (C
API: irwls_mlp_*, irwls_sgma_traces, irwls_set_sgma_proposer in
include/irwls_gpu.h). The proposer acts on the precision form of SGMA
(irwls_set_precision(1)) with RBF kernels."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import load

PF = C.POINTER(C.c_float)


def _f32(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float32))


class Proposer:
    """The proposal network (8 features -> 128 -> 128 -> 1, ReLU)."""

    def __init__(self, seed: int = 0):
        self.lib = load()
        self.h = self.lib.irwls_mlp_create(seed)
        if not self.h:
            raise RuntimeError("cannot create the proposal network: " + self.lib.irwls_last_error_message().decode())
        self.n_params = self.lib.irwls_mlp_param_count()
        self.n_features = self.lib.irwls_mlp_feature_count()

    def close(self):
        if self.h:
            self.lib.irwls_set_sgma_proposer(None, 0)
            self.lib.irwls_mlp_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self) -> np.ndarray:
        out = np.zeros(self.n_params, np.float32)
        if self.lib.irwls_mlp_get_params(self.h, out.ctypes.data_as(PF)) != 0:
            raise RuntimeError(self.lib.irwls_last_error_message().decode())
        return out

    def set_params(self, theta) -> None:
        t = _f32(theta)
        assert t.size == self.n_params
        if self.lib.irwls_mlp_set_params(self.h, t.ctypes.data_as(PF)) != 0:
            raise RuntimeError(self.lib.irwls_last_error_message().decode())

    def loss_grad(self, X, T):
        X, T = _f32(X), _f32(T)
        g = np.zeros(self.n_params, np.float32)
        loss = self.lib.irwls_mlp_loss_grad(self.h, X.ctypes.data_as(PF), T.ctypes.data_as(PF), len(T),
                                            g.ctypes.data_as(PF))
        if loss < 0:
            raise RuntimeError(self.lib.irwls_last_error_message().decode())
        return loss, g

    def predict(self, X) -> np.ndarray:
        X = _f32(X)
        out = np.zeros(X.shape[0], np.float32)
        if self.lib.irwls_mlp_predict_host(self.h, X.ctypes.data_as(PF), X.shape[0], out.ctypes.data_as(PF)) != 0:
            raise RuntimeError(self.lib.irwls_last_error_message().decode())
        return out

    def train(self, X, T, epochs=30, batch=1024, lr=1e-3, seed=0) -> float:
        X, T = _f32(X), _f32(T)
        loss = self.lib.irwls_mlp_train(self.h, X.ctypes.data_as(PF), T.ctypes.data_as(PF), len(T), epochs, batch,
                                        lr, seed)
        if loss < 0:
            raise RuntimeError("training failed: " + self.lib.irwls_last_error_message().decode())
        return loss

    def install(self, pool: int = 4096) -> None:
        self.lib.irwls_set_sgma_proposer(self.h, pool)

    def uninstall(self) -> None:
        self.lib.irwls_set_sgma_proposer(None, 0)


def traces(hd, props):
    """Features ((m - 2) x 64 x 8) and exact scores ((m - 2) x 64) of the random
    candidates of one precision-form SGMA run on a host dataset."""
    lib = load()
    m, nf = props.size, lib.irwls_mlp_feature_count()
    feat = np.zeros((m - 2, 64, nf), np.float32)
    score = np.zeros((m - 2, 64), np.float32)
    if lib.irwls_sgma_traces(hd.struct, props, feat.ctypes.data_as(PF), score.ctypes.data_as(PF)) != 0:
        raise RuntimeError(lib.irwls_last_error_message().decode())
    return feat, score


def targets(score) -> np.ndarray:
    """Per step: log score minus the step's mean log score."""
    ls = np.log(np.maximum(np.asarray(score, dtype=np.float64), 1e-30))
    return (ls - ls.mean(axis=1, keepdims=True)).astype(np.float32)


def training_set(runs):
    """Stacked features and targets of the traces of (dataset, props) runs."""
    Xs, Ts = [], []
    for hd, props in runs:
        f, s = traces(hd, props)
        Xs.append(f.reshape(-1, f.shape[-1]))
        Ts.append(targets(s).reshape(-1))
    return np.concatenate(Xs), np.concatenate(Ts)


def fit(runs, seed=0, rounds=2, epochs=10, batch=1024, lr=1e-3, pool=4096):
    """Trains a proposer on traces of the (dataset, props) runs: the first
    round on random candidates, each later round adds the exact scores of the
    candidates the current network proposes (on-policy traces, which teach
    it where it over-ranks) and continues training on all of them."""
    net = Proposer(seed)
    X, T = training_set(runs)
    net.train(X, T, epochs=epochs, batch=batch, lr=lr, seed=seed)
    for r in range(1, rounds):
        net.install(pool)
        try:
            X2, T2 = training_set(runs)
        finally:
            net.uninstall()
        X, T = np.concatenate([X, X2]), np.concatenate([T, T2])
        net.train(X, T, epochs=epochs, batch=batch, lr=lr, seed=seed + r)
    return net, len(T)
