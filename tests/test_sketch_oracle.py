"""CPU checks of the learned-sketch objective: the oracle's closed-form
adjoint equals central finite differences of the oracle loss (float64)."""
import numpy as np

import ht_oracle as O


def test_sketch_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    n, s = 20, 5
    A = rng.standard_normal((n, 40)) * (0.7 ** np.arange(40))
    G = A @ A.T
    S = rng.standard_normal((n, s))
    g = O.sketch_grad(G, S)
    fd = np.zeros_like(S)
    h = 1e-6
    for i in range(n):
        for j in range(s):
            Sp, Sm = S.copy(), S.copy()
            Sp[i, j] += h
            Sm[i, j] -= h
            fd[i, j] = (O.sketch_loss(G, Sp) - O.sketch_loss(G, Sm)) / (2 * h)
    assert np.linalg.norm(g - fd) / np.linalg.norm(fd) < 1e-6


def test_sketch_loss_invariances():
    rng = np.random.default_rng(1)
    n, s = 16, 4
    A = rng.standard_normal((n, n))
    G = A @ A.T
    S = rng.standard_normal((n, s))
    M = rng.standard_normal((s, s)) + 3 * np.eye(s)
    # the loss depends on span(G S) only
    assert abs(O.sketch_loss(G, S) - O.sketch_loss(G, S @ M)) < 1e-12
    assert 0.0 <= O.sketch_loss(G, S) <= 1.0
    # a sketch spanning the top-s eigenvectors attains the optimum
    w, V = np.linalg.eigh(G)
    best = 1 - w[::-1][:s].sum() / w.sum()
    assert abs(O.sketch_loss(G, V[:, ::-1][:, :s]) - best) < 1e-12


def test_sketch_loss_rank_deficient_gram_stays_in_range():
    """A Gram of rank below the sketch width (the separable-bumps family: rank
    <= 32 < 34) makes Y = G S rank deficient.  The dependent columns are left
    out of Q, so the loss stays in [0, 1] and equals the exact value 0 (the
    kept columns span the whole range)."""
    rng = np.random.default_rng(2)
    n, r, s = 40, 6, 9
    A = rng.standard_normal((n, r)) * (0.5 ** np.arange(r))
    G = A @ A.T
    S = rng.standard_normal((n, s))
    loss = O.sketch_loss(G, S)
    assert 0.0 <= loss < 1e-9, loss
    _, _, _, keep = O._sketch_parts(G, S)
    assert keep.sum() == r
    g = O.sketch_grad(G, S)
    assert np.isfinite(g).all()
    assert np.abs(g[:, ~keep]).max() == 0.0
