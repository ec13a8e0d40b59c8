"""Learned-proposal form of SGMA: the GPU network's loss and gradients
against the CPU oracle, its training, and what its proposals gain over the
reference's random candidates (the Nystrom residual at equal budget) on a
held-out set of the data family it was trained on."""
import os
import sys

import numpy as np
import pytest

import harness as H
from libirwls_gb300 import _abi, learned, load, synth

sys.path.insert(0, os.path.join(H.ROOT, "oracle"))
import mlp  # noqa: E402

pytestmark = pytest.mark.gpu


def _theta(seed):
    rng = np.random.default_rng(seed)
    parts = {}
    for name, shape in mlp.SIZES:
        fan = shape[-1] if len(shape) == 2 else 128
        parts[name] = rng.normal(0.0, np.sqrt(2.0 / fan), shape) if len(shape) == 2 else rng.normal(0.0, 0.1, shape)
    return mlp.pack(parts).astype(np.float32)


def test_gradients_match_oracle():
    net = learned.Proposer(seed=1)
    theta = _theta(3)
    net.set_params(theta)
    rng = np.random.default_rng(4)
    X = rng.normal(0.0, 1.0, (300, mlp.LF)).astype(np.float32)
    T = rng.normal(0.0, 1.0, 300).astype(np.float32)
    loss, g = net.loss_grad(X, T)
    ref_loss, ref_g = mlp.loss_grad(theta.astype(np.float64), X.astype(np.float64), T.astype(np.float64))
    assert abs(loss - ref_loss) <= 1e-5 * ref_loss
    k = 0
    for name, shape in mlp.SIZES:
        n = int(np.prod(shape))
        a, b = g[k:k + n], ref_g[k:k + n]
        assert np.abs(a - b).max() <= 1e-4 * max(np.abs(b).max(), 1e-6), name
        k += n
    net.close()


def test_training_fits_and_matches_oracle_forward():
    net = learned.Proposer(seed=2)
    rng = np.random.default_rng(5)
    X = rng.normal(0.0, 1.0, (8192, mlp.LF)).astype(np.float32)
    T = (np.sin(X[:, 0]) + 0.5 * X[:, 1] * X[:, 2] - 0.3 * np.abs(X[:, 3])).astype(np.float32)
    final = net.train(X, T, epochs=40, batch=512, lr=3e-3, seed=1)
    assert final < 0.1 * float(T.var())
    theta = net.params().astype(np.float64)
    P_ref, _ = mlp.forward(theta, X[:500].astype(np.float64))
    P = net.predict(X[:500])
    assert np.abs(P - P_ref).max() <= 1e-4 * max(np.abs(P_ref).max(), 1.0)
    net.close()


def _family_set(n, seed, family):
    X, y = synth.gauss_mixture(n, seed, family_seed=family)
    d = synth.from_dense(X, y, keep_zeros=True)
    return _abi.build_dataset(d.indptr, d.indices, d.values, d.y)


def test_learned_proposals_lower_the_nystrom_residual():
    lib = load()
    m = 60
    props = _abi.make_properties(gamma=0.5, C_=10.0, size=m, algorithm=1)
    runs = [(_family_set(4000, 10 + k, 300 + k), props) for k in range(4)]
    lib.initMemory(1, m)
    H.LIBC.srand(1)
    net, _ = learned.fit(runs, seed=7, rounds=2, epochs=20, batch=512, pool=1024)
    test_set = _family_set(8000, 99, 399)
    lib.irwls_set_precision(1)
    try:
        res = {}
        for name in ("random", "learned"):
            if name == "learned":
                net.install(pool=1024)
            H.LIBC.srand(1)
            c = lib.SGMA(test_set.struct, props)
            assert c, lib.irwls_last_error_message()
            res[name] = lib.irwls_last_nystrom_residual()
            w = lib.IRWLSpar(test_set.struct, c, props)
            assert w
            net.uninstall()
    finally:
        lib.irwls_set_precision(0)
        net.close()
    print("Nystrom residual: random %.2f, learned %.2f (%.1f%%)" % (res["random"], res["learned"],
                                                                     100 * (1 - res["learned"] / res["random"])))
    assert 0 < res["learned"] < res["random"]
