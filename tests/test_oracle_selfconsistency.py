"""Self-consistency pins of the oracle that need no reference data: exact HT
tensors decomposed at their true ranks are reproduced to machine precision
(every 3rd-order tree and the 4th-order balanced tree), and an orthogonally
decomposable tensor's HT error equals the closed-form truncation error."""
import numpy as np
import pytest

import ht_oracle as O
import ht_tensor_learning_using_gpu_tensor_cores_gb300 as ht
from ht_tensor_learning_using_gpu_tensor_cores_gb300 import synth

TREES3 = [ht.reference_tree_3d, ht.left_first_tree_3d, ht.middle_tree_3d]


@pytest.mark.parametrize("mk", TREES3)
def test_exact_ht_3d_reproduced_at_true_ranks(mk):
    tree = mk([1, 7, 5, 4, 6])
    dims = (20, 18, 22)
    tree.check_ranks(dims)
    X = synth.exact_ht(dims, tree, noise_rel=0.0, seed=4, dtype=np.float64)
    U, B, _ = O.ht_decompose(X, tree, dtype=np.float64)
    assert O.ht_error(X, tree, U, B) < 1e-12
    for t in tree.leaves():
        assert O.orthogonality_defect(U[t]) < 1e-12


def test_exact_ht_4d_reproduced_at_true_ranks():
    tree = ht.balanced_tree_4d([1, 6, 5, 3, 2, 3, 4])
    dims = (8, 9, 7, 10)
    tree.check_ranks(dims)
    X = synth.exact_ht(dims, tree, noise_rel=0.0, seed=5, dtype=np.float64)
    U, B, _ = O.ht_decompose(X, tree, dtype=np.float64)
    assert O.ht_error(X, tree, U, B) < 1e-12


@pytest.mark.parametrize("k", [4, 8, 12])
def test_odeco_error_is_the_closed_form_optimum(k):
    n = 24
    X = synth.odeco(n, decay=1.5, seed=2).astype(np.float64)
    tree = ht.reference_tree_3d([1, k, k, k, k])
    U, B, _ = O.ht_decompose(X, tree, dtype=np.float64)
    e = O.ht_error(X, tree, U, B)
    opt = synth.odeco_optimal_error(n, k, 1.5)
    assert abs(e - opt) <= 1e-6 * opt + 1e-7, (e, opt)


def test_error_grows_when_ranks_are_cut():
    tree_full = ht.reference_tree_3d([1, 6, 6, 6, 6])
    X = synth.exact_ht((16, 16, 16), tree_full, noise_rel=0.0, seed=8, dtype=np.float64)
    errs = []
    for k in (6, 4, 2):
        tree = ht.reference_tree_3d([1, k, k, k, k])
        U, B, _ = O.ht_decompose(X, tree, dtype=np.float64)
        errs.append(O.ht_error(X, tree, U, B))
    assert errs[0] < 1e-12 < errs[1] < errs[2]
