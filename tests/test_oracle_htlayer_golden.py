"""Pin the HT-layer part of the oracle to the reference's own code.

tests/golden/ref_htlayer_s7.npz holds what HT_tensor_layer/FC_MNIST/mnist_ht.py
computes, run as written by tests/golden/make_golden.py: its ``ht()``
initialisation of a seeded 80 x 96 weight (N = 4, 4, 6; M = 4, 5, 4; rank 4),
the einsum chain of ``tNet.forward`` on a seeded batch, and the gradients torch
autograd gives that chain for a seeded output cotangent (float32)."""
import os

import numpy as np
import pytest

import ht_oracle as O

FIX = os.path.join(os.path.dirname(__file__), "golden", "ref_htlayer_s7.npz")
NAMES = ("u1", "u2", "u3", "b2", "b1")


@pytest.fixture(scope="module")
def z():
    return np.load(FIX)


def _f64(z, names):
    return [z[k].astype(np.float64) for k in names]


def test_chain_matches_reference_forward(z):
    y = O.ht_layer_chain(z["x"], *_f64(z, NAMES), bias=z["bias"])
    ref = z["y"].astype(np.float64)
    assert y.shape == ref.shape
    assert np.abs(y - ref).max() <= 2e-6 * np.abs(ref).max()


def test_dense_weight_matches_reference_forward(z):
    W = O.ht_layer_weight(*_f64(z, NAMES))
    y = z["x"].astype(np.float64) @ W.T + z["bias"].astype(np.float64).reshape(1, -1)
    ref = z["y"].astype(np.float64)
    assert np.abs(y - ref).max() <= 2e-6 * np.abs(ref).max()


@pytest.mark.parametrize("name", NAMES + ("bias", "x"))
def test_chain_gradients_match_reference_autograd(z, name):
    """The chain is linear in each of its arguments, so a central difference of
    <chain, dy> along a random direction is its exact directional derivative;
    it equals <reference gradient, direction>."""
    p = {k: z[k].astype(np.float64) for k in NAMES + ("bias", "x")}
    dy = z["dy"].astype(np.float64)

    def f(q):
        return float((O.ht_layer_chain(q["x"], *[q[k] for k in NAMES], bias=q["bias"]) * dy).sum())

    d = np.random.default_rng(len(name)).standard_normal(p[name].shape)
    h = 1e-2
    hi, lo = dict(p), dict(p)
    hi[name] = p[name] + h * d
    lo[name] = p[name] - h * d
    fd = (f(hi) - f(lo)) / (2 * h)
    g = float((z["g_" + name].astype(np.float64) * d).sum())
    scale = np.abs(z["g_" + name]).sum() * np.abs(d).max()
    assert abs(fd - g) <= 1e-5 * scale + 1e-6, (fd, g)


def test_init_unfoldings_and_transfers_match_reference(z):
    """ht(): the reference's leaves are eigenvectors of the oracle's unfolding
    Grams, and the oracle's transfer contractions (node 1's basis from the
    oracle's SVD, the reference's leaves) rebuild the reference's layer weight."""
    N, M, r = [int(v) for v in z["N"]], [int(v) for v in z["M"]], int(z["rank"])
    a, b, c = N[0] * M[0], N[1] * M[1], N[2] * M[2]
    X, U3m, U4m, U2m, U1m = O.ht_layer_unfoldings(z["W"], N, M)
    U3 = z["u1"].astype(np.float64).reshape(a, r)
    U4 = z["u2"].astype(np.float64).reshape(b, r)
    U2 = z["u3"].astype(np.float64).reshape(c, r)
    for A, U in ((U3m, U3), (U4m, U4), (U2m, U2)):
        G = A @ A.T
        lam = np.einsum("ij,ij->j", U, G @ U)
        # float32 ?geev vectors (not orthogonalised by the routine): 1e-4
        assert np.abs(U.T @ U - np.eye(r)).max() < 1e-4
        assert np.linalg.norm(G @ U - U * lam, axis=0).max() <= 1e-4 * np.linalg.norm(G, 2)
    U1 = np.linalg.svd(U1m, full_matrices=False)[0][:, :r].reshape(a, b, r)
    B1, B0 = O.ht_layer_transfers(X, U1, U2, U3, U4)
    assert B1.shape == z["b2"].shape and B0.shape == z["b1"].shape
    W_ref = O.ht_layer_weight(*_f64(z, NAMES))
    W_or = O.ht_layer_weight(z["u1"], z["u2"], z["u3"], B1, B0)
    assert np.abs(W_or - W_ref).max() <= 1e-5 * np.abs(W_ref).max()
