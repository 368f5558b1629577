"""HT-format file round trips and validation on the host (no GPU), and the
oracle's leaf-to-root entry contraction against its full reconstruction."""
import numpy as np
import pytest

import ht_tensor_learning_using_gpu_tensor_cores_gb300 as ht
from ht_tensor_learning_using_gpu_tensor_cores_gb300 import htformat
import ht_oracle as O


def factors(tree, dims, seed):
    rng = np.random.default_rng(seed)
    U = {t: rng.standard_normal((dims[tree.modes[t][0]], tree.ranks[t])).astype(np.float32) for t in tree.leaves()}
    B = {t: rng.standard_normal((tree.ranks[tree.left[t]], tree.ranks[tree.right[t]], tree.ranks[t]))
         .astype(np.float32) for t in [0] + tree.interior()}
    return U, B


TREES = [(ht.reference_tree_3d([1, 4, 3, 2, 3]), (6, 5, 7)),
         (ht.left_first_tree_3d([1, 3, 4, 3, 2]), (4, 6, 5)),
         (ht.middle_tree_3d([1, 3, 4, 2, 3]), (5, 4, 6)),
         (ht.balanced_tree_4d([1, 3, 2, 2, 3, 2, 2]), (3, 4, 5, 2))]


@pytest.mark.parametrize("tree,dims", TREES)
def test_save_load_roundtrip(tmp_path, tree, dims):
    U, B = factors(tree, dims, 1)
    p = str(tmp_path / "h.npz")
    htformat.save(p, tree, dims, U, B)
    h = htformat.load(p)
    assert h.dims == dims
    assert h.tree.modes == tree.modes and h.tree.left == tree.left and h.tree.right == tree.right
    assert h.tree.ranks == tree.ranks
    for t in U:
        assert np.array_equal(h.U[t], U[t])
    for t in B:
        assert np.array_equal(h.B[t], B[t])
    assert h.n_parameters() == sum(a.size for a in U.values()) + sum(a.size for a in B.values())
    full0 = O.ht_reconstruct(tree, dims, U, B)
    full1 = O.ht_reconstruct(h.tree, h.dims, h.U, h.B)
    assert np.array_equal(full0, full1)


def test_save_rejects_wrong_shapes(tmp_path):
    tree, dims = TREES[0]
    U, B = factors(tree, dims, 2)
    U[3] = U[3][:, :1]
    with pytest.raises(ValueError, match="shape"):
        htformat.save(str(tmp_path / "bad.npz"), tree, dims, U, B)
    U, B = factors(tree, dims, 2)
    del B[1]
    with pytest.raises(ValueError, match="missing"):
        htformat.save(str(tmp_path / "bad.npz"), tree, dims, U, B)


def test_load_rejects_foreign_or_damaged_files(tmp_path):
    p = str(tmp_path / "other.npz")
    np.savez(p, a=np.zeros(3))
    with pytest.raises(ValueError, match="not an"):
        htformat.load(p)
    tree, dims = TREES[1]
    U, B = factors(tree, dims, 3)
    good = str(tmp_path / "good.npz")
    htformat.save(good, tree, dims, U, B)
    with np.load(good) as z:
        arrays = {k: z[k] for k in z.files}
    arrays["B2"] = arrays["B2"][:, :, :1]
    damaged = str(tmp_path / "damaged.npz")
    np.savez(damaged, **arrays)
    with pytest.raises(ValueError, match="B2"):
        htformat.load(damaged)


@pytest.mark.parametrize("tree,dims", TREES)
def test_oracle_entries_match_reconstruction(tree, dims):
    U, B = factors(tree, dims, 4)
    U = {t: a.astype(np.float64) for t, a in U.items()}
    B = {t: a.astype(np.float64) for t, a in B.items()}
    full = O.ht_reconstruct(tree, dims, U, B)
    idx = np.array(list(np.ndindex(*dims)), dtype=np.int64)
    got = O.ht_entries(tree, U, B, idx)
    assert np.allclose(got, full[tuple(idx.T)], rtol=1e-12, atol=1e-12 * np.abs(full).max())
