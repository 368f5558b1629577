"""The batched path (ht_decompose_batched, c4-style many small tensors) against
single-tensor calls and the FP64 oracle, and the CUDA-graph replay: a second
call with the same buffers replays the recorded graph and gives the same
factors; new contents in the same buffers give the new tensors' factors.

Tolerances as in the single-tensor parity tests: |err - err_fp64| <= 1e-5
(FP32 path), <= 1e-3 (mixed BF16 path).
"""
import numpy as np
import pytest
import torch

import ht_tensor_learning_using_gpu_tensor_cores_gb300 as ht
from ht_tensor_learning_using_gpu_tensor_cores_gb300 import synth
import ht_oracle as O

pytestmark = pytest.mark.gpu

TOL = {"fp32": 1e-5, "bf16": 1e-3}


def to_dev(X):
    return torch.from_numpy(np.ascontiguousarray(X.transpose(tuple(range(X.ndim))[::-1]))).cuda()


@pytest.fixture(scope="module")
def family():
    return synth.batch_family(12, seed=5, dim_range=(24, 72), rank_range=(4, 10))


@pytest.mark.parametrize("prec", ["fp32", "bf16"])
def test_batched_matches_oracle_and_single_calls(family, prec):
    trees = [t for _, t in family]
    dims = [X.shape for X, _ in family]
    xs = [to_dev(X) for X, _ in family]
    bd = ht.BatchDecomposer(trees, dims, precision=prec, compute_error=True)
    res, rep = bd(xs)
    torch.cuda.synchronize()
    errs = []
    for (X, tree), r in zip(family, res):
        U = {t: r.U[t].cpu().numpy().astype(np.float64) for t in r.U}
        B = {t: r.B[t].cpu().numpy().astype(np.float64) for t in r.B}
        e = O.ht_error(X, tree, U, B)
        Uo, Bo, _ = O.ht_decompose(X, tree)
        e64 = O.ht_error(X, tree, Uo, Bo)
        assert abs(e - e64) <= TOL[prec], (prec, e, e64)
        assert abs(r.report["rel_err"] - e) <= 1e-5 + 1e-4 * e
        single = ht.decompose(to_dev(X), tree, precision=prec, compute_error=True)
        assert abs(single.report["rel_err"] - r.report["rel_err"]) <= (1e-6 if prec == "fp32" else 2e-4)
        errs.append(r.report["rel_err"])
    s = np.sort(errs)
    assert rep["rel_err_p50"] == pytest.approx(s[int(np.ceil(0.5 * len(s))) - 1])
    assert rep["rel_err_p99"] == pytest.approx(s[int(np.ceil(0.99 * len(s))) - 1])
    assert rep["rel_err_max"] == pytest.approx(s[-1])
    assert rep["gpu_launches"] > 0 and rep["lanes"] >= 1


def test_graph_replay_same_and_new_contents(family):
    trees = [t for _, t in family]
    dims = [X.shape for X, _ in family]
    xs = [to_dev(X) for X, _ in family]
    bd = ht.BatchDecomposer(trees, dims, precision="bf16", compute_error=True)
    r1, rep1 = bd(xs)
    assert rep1["note"] == "", rep1["note"]   # the batch was recorded into a graph
    U1 = [{t: r.U[t].cpu().numpy().copy() for t in r.U} for r in r1]
    e1 = [r.report["rel_err"] for r in r1]
    r2, rep2 = bd(xs)
    assert rep2["graph_replayed"], "identical second call must replay the recorded graph"
    # small modes: every leaf in one grouped solver launch, timed inside the graph
    assert rep2["grouped"] and min(rep2["ms_phase"].values()) >= 0 and rep2["ms_phase"]["leaf_solver"] > 0, rep2
    assert sum(rep2["ms_phase"].values()) <= rep2["ms_total"] * 1.01 + 0.05
    for a, r in zip(U1, r2):
        for t in a:
            np.testing.assert_array_equal(a[t], r.U[t].cpu().numpy())
    # new contents, same buffers: the replay must decompose the new tensors

    for i, (x, (X, tree)) in enumerate(zip(xs, family)):
        Y = synth.exact_ht(X.shape, tree, noise_rel=1e-2, seed=1000 + i)
        x.copy_(to_dev(Y))
    r3, rep3 = bd(xs)
    assert rep3["graph_replayed"]
    for i, (x, (X, tree)) in enumerate(zip(xs, family)):
        single = ht.decompose(x, tree, precision="bf16", compute_error=True)
        assert abs(single.report["rel_err"] - r3[i].report["rel_err"]) <= 2e-4
        assert r3[i].report["rel_err"] > 5e-3 > e1[i]   # the 1e-2 noise now dominates



def test_batched_rejects_host_inputs(family):
    X, tree = family[0]
    bd = ht.BatchDecomposer([tree], [X.shape], precision="bf16")
    with pytest.raises(TypeError):
        bd([X])


def _check_batch(pairs, prec):
    trees = [t for _, t in pairs]
    dims = [X.shape for X, _ in pairs]
    bd = ht.BatchDecomposer(trees, dims, precision=prec, compute_error=True)
    res, rep = bd([to_dev(X) for X, _ in pairs])
    for (X, tree), r in zip(pairs, res):
        U = {t: r.U[t].cpu().numpy().astype(np.float64) for t in r.U}
        B = {t: r.B[t].cpu().numpy().astype(np.float64) for t in r.B}
        e = O.ht_error(X, tree, U, B)
        Uo, Bo, _ = O.ht_decompose(X, tree)
        assert abs(e - O.ht_error(X, tree, Uo, Bo)) <= TOL[prec], (prec, X.shape, e)
        assert abs(r.report["rel_err"] - e) <= 1e-5 + 1e-4 * e
        for t in tree.leaves():
            assert O.orthogonality_defect(U[t]) < 1e-4
    return rep


@pytest.mark.parametrize("prec", ["fp32", "bf16"])
def test_batched_large_mode_uses_per_lane_solver(prec):
    """A batch with a mode above the grouped solver's 512 runs every tensor's
    leaf solver as a cooperative launch of its own; results as before."""
    pairs = []
    for i, d in enumerate([(520, 24, 20), (40, 36, 32), (33, 47, 61)]):
        tree = ht.reference_tree_3d([1, 8, 6, 5, 7])
        pairs.append((synth.exact_ht(d, tree, noise_rel=1e-3, seed=300 + i), tree))
    rep = _check_batch(pairs, prec)
    assert not rep["grouped"]


@pytest.mark.parametrize("prec", ["fp32", "bf16"])
def test_batched_4d_and_direct_leaves(prec):
    """4th-order tensors (four leaves each, the root's range finder after the
    grouped leaf solver); leaves no larger than k + oversampling are solved
    directly, the others iterated, in one batch."""
    pairs = []
    for i, d in enumerate([(20, 24, 18, 22), (30, 16, 26, 20), (12, 28, 20, 24)]):
        tree = ht.balanced_tree_4d([1, 12, 12, 6, 6, 6, 6])
        pairs.append((synth.exact_ht(d, tree, noise_rel=1e-3, seed=400 + i), tree))
    _check_batch(pairs, prec)


@pytest.mark.parametrize("prec", ["fp32", "bf16"])
def test_batched_grouped_gram_classes(prec):
    """Modes of at most 128 and 129..256 (the two grouped Gram tile classes),
    a mode of 260 (its Gram launched on its own inside a grouped batch), first
    modes that are not multiples of 8 (padded BF16 copies) and one that is."""
    pairs = []
    for i, d in enumerate([(150, 40, 200), (260, 30, 24), (64, 129, 33), (37, 256, 45)]):
        tree = ht.reference_tree_3d([1, 10, 8, 9, 7])
        pairs.append((synth.exact_ht(d, tree, noise_rel=1e-3, seed=500 + i), tree))
    rep = _check_batch(pairs, prec)
    assert rep["grouped"]


@pytest.mark.parametrize("prec", ["fp32", "bf16"])
def test_batched_other_trees_take_the_general_grouped_paths(prec):
    """Trees {1},{2,3} and {2},{1,3}: the complementary leaf is not the last
    mode, so the grouped core pass runs FP32 tiles and the error pass the
    expansion + fused tiles; mixed with reference-tree tensors in one batch."""
    pairs = []
    trees = [ht.left_first_tree_3d, ht.middle_tree_3d, ht.reference_tree_3d, ht.left_first_tree_3d]
    for i, (tf, d) in enumerate(zip(trees, [(40, 52, 36), (61, 33, 47), (48, 40, 56), (130, 24, 40)])):
        tree = tf([1, 9, 8, 7, 6])
        pairs.append((synth.exact_ht(d, tree, noise_rel=1e-3, seed=600 + i), tree))
    rep = _check_batch(pairs, prec)
    assert rep["grouped"]


@pytest.mark.parametrize("prec", ["fp32", "bf16"])
def test_batched_tiny_tensors_and_single_tensor_batch(prec):
    """Modes of 3..12 (first modes padded for TMA, fewer than 32 rows in the
    mode product, leaf problems solved directly) in one grouped batch; then a
    batch of one tensor."""
    pairs = []
    for i, d in enumerate([(5, 6, 7), (3, 12, 4), (9, 4, 11), (12, 12, 12), (7, 3, 5)]):
        r = [1, min(3, d[2]), min(3, d[2]), min(2, d[0]), min(3, d[1])]
        tree = ht.reference_tree_3d(r)
        pairs.append((synth.exact_ht(d, tree, noise_rel=1e-3, seed=700 + i), tree))
    rep = _check_batch(pairs, prec)
    assert rep["grouped"]
    rep1 = _check_batch(pairs[3:4], prec)
    assert rep1["grouped"] and rep1["gpu_launches"] > 0
