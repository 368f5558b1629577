"""Parity of the GPU HT decomposition with the CPU oracle (the reference's
algorithm restated in numpy, pinned to the reference's own outputs by
tests/test_oracle_golden.py).

Tolerances (relative reconstruction error ||X - Xhat|| / ||X||, compared with
the FP64 oracle's error on the same input):
  plain FP32 path  |err_gpu - err_fp64| <= 1e-5
  mixed BF16 path  |err_gpu - err_fp64| <= 1e-3
The factors themselves are unique only up to an orthogonal change of basis
per node (and arbitrary inside exactly degenerate or null eigenspaces), so
factor parity is checked through principal angles of the leaf subspaces when
the spectrum has a gap, and through the full reconstruction otherwise.
"""
import glob
import os

import numpy as np
import pytest
import torch

import ht_tensor_learning_using_gpu_tensor_cores_gb300 as ht
from ht_tensor_learning_using_gpu_tensor_cores_gb300 import synth
from ht_tensor_learning_using_gpu_tensor_cores_gb300.tree import DimTree
import ht_oracle as O

pytestmark = pytest.mark.gpu

TOL = {"fp32": 1e-5, "bf16": 1e-3}


def to_dev(X):
    return torch.from_numpy(np.ascontiguousarray(X.transpose(tuple(range(X.ndim))[::-1]))).cuda()


def run(X, tree, prec, **kw):
    res = ht.decompose(to_dev(X), tree, precision=prec, compute_error=True, **kw)
    torch.cuda.synchronize()
    U = {t: res.U[t].cpu().numpy().astype(np.float64) for t in res.U}
    B = {t: res.B[t].cpu().numpy().astype(np.float64) for t in res.B}
    return res, U, B


def check_against_oracle(X, tree, prec, angle_tol=None, **kw):
    res, U, B = run(X, tree, prec, **kw)
    Uo, Bo, _ = O.ht_decompose(X, tree, dtype=np.float64)
    e64 = O.ht_error(X, tree, Uo, Bo)
    e = O.ht_error(X, tree, U, B)
    assert abs(e - e64) <= TOL[prec], (prec, e, e64)
    # the device-side error pass agrees with the oracle's reconstruction of the same factors
    assert abs(res.report["rel_err"] - e) <= 1e-5 + 1e-4 * e, (res.report["rel_err"], e)
    for t in tree.leaves():
        assert O.orthogonality_defect(U[t]) < (2e-5 if prec == "fp32" else 2e-4)
        if angle_tol is not None:
            assert O.principal_angles(U[t], Uo[t]).max() < angle_tol, t
    return res, e, e64


@pytest.mark.parametrize("prec", ["fp32", "bf16"])
def test_c1_shape_left_first_tree(prec):
    """256^3, tree {1,2,3}->{1},{2,3}->{2},{3}, ranks 16, exact HT + 1e-3 noise."""
    tree = ht.left_first_tree_3d([1, 16, 16, 16, 16])
    X = synth.exact_ht((256, 256, 256), tree, noise_rel=1e-3, seed=1)
    res, e, e64 = check_against_oracle(X, tree, prec, angle_tol=1e-2 if prec == "fp32" else 5e-2)
    assert res.report["path"]["tcgen05"] == (prec == "bf16")


@pytest.mark.parametrize("tree_fn", [ht.reference_tree_3d, ht.left_first_tree_3d, ht.middle_tree_3d])
@pytest.mark.parametrize("prec", ["fp32", "bf16"])
def test_all_3d_trees(tree_fn, prec):
    tree = tree_fn([1, 8, 8, 8, 8])
    X = synth.exact_ht((64, 56, 48), tree, noise_rel=1e-3, seed=2)
    check_against_oracle(X, tree, prec)


@pytest.mark.parametrize("prec", ["fp32", "bf16"])
def test_uneven_ranks_interior_differs_from_complement(prec):
    # k_t > k_c and k_t < k_c, uneven dims
    for k in ([1, 12, 6, 5, 4], [1, 5, 9, 4, 3]):
        tree = ht.reference_tree_3d(k)
        X = synth.exact_ht((72, 64, 80), ht.reference_tree_3d([1, 10, 10, 6, 5]), noise_rel=1e-3, seed=3)
        check_against_oracle(X, tree, prec)


@pytest.mark.parametrize("prec", ["fp32", "bf16"])
def test_rank_deficient_reference_style(prec):
    """The reference's own test data (genHtensor recipe): true ranks 3..7,
    decomposition ranks above them, so some directions are null."""
    X, k = synth.reference_style(64, seed=4)
    tree = ht.reference_tree_3d([1, 10, 10, 10, 10])
    res, e, e64 = check_against_oracle(X, tree, prec)
    assert e < (1e-5 if prec == "fp32" else 1e-3)
    assert all(np.isfinite(res.B[t].cpu().numpy()).all() for t in res.B)


@pytest.mark.parametrize("prec", ["fp32", "bf16"])
def test_odeco_decaying_spectrum(prec):
    """c2-style data at reduced size: spectrum r^-1.5 on every unfolding."""
    n, k = 128, 32
    X = synth.odeco(n, seed=5)
    tree = ht.reference_tree_3d([1, k, k, k, k])
    res, e, e64 = check_against_oracle(X, tree, prec)
    assert abs(e64 - synth.odeco_optimal_error(n, k)) < 1e-6


@pytest.mark.parametrize("prec", ["fp32", "bf16"])
def test_4d_balanced(prec):
    tree = ht.balanced_tree_4d([1, 12, 12, 6, 6, 6, 6])
    X = synth.exact_ht((32, 24, 32, 16), tree, noise_rel=1e-4, seed=6)
    check_against_oracle(X, tree, prec)


def test_4d_c3_shape_properties():
    """128^4 (1 GiB), leaf ranks 24, interior 48, exact HT + 1e-4 noise: the
    error sits at the noise level and the bases are orthonormal."""
    tree = ht.balanced_tree_4d([1, 48, 48, 24, 24, 24, 24])
    X = synth.exact_ht((128, 128, 128, 128), tree, noise_rel=1e-4, seed=7)
    for prec in ("fp32", "bf16"):
        res, U, B = run(X, tree, prec)
        e = res.report["rel_err"]
        assert e < 2e-4, (prec, e)
        for t in tree.leaves():
            assert O.orthogonality_defect(U[t]) < 2e-4


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "ref_*_3d_*.npz"))),
                         ids=os.path.basename)
def test_golden_inputs_through_gpu(path):
    """The reference's own test tensors through the GPU path: FP32 error at or
    below the error the reference printed (FP32 rounding level)."""
    from test_oracle_golden import _load3
    z, X, tree, Uref, Bref = _load3(path)
    res, U, B = run(X, tree, "fp32")
    e = O.ht_error(X, tree, U, B)
    assert e <= max(float(z["err"]), 1e-6) * 1.5 + 1e-6


def test_reconstruct_error_matches_oracle():
    tree = ht.middle_tree_3d([1, 6, 6, 6, 6])
    X = synth.exact_ht((40, 48, 56), tree, noise_rel=1e-2, seed=8)
    U, B, _ = O.ht_decompose(X, tree)
    e = O.ht_error(X, tree, U, B)
    U32 = {t: U[t].astype(np.float32) for t in U if tree.is_leaf(t)}
    B32 = {t: B[t].astype(np.float32) for t in B}
    assert abs(ht.reconstruct_error(X, tree, U32, B32) - e) < 1e-6
    tree4 = ht.balanced_tree_4d([1, 8, 8, 4, 4, 4, 4])
    X4 = synth.exact_ht((16, 24, 16, 8), tree4, noise_rel=1e-2, seed=9)
    U, B, _ = O.ht_decompose(X4, tree4)
    U32 = {t: U[t].astype(np.float32) for t in U if tree4.is_leaf(t)}
    B32 = {t: B[t].astype(np.float32) for t in B}
    assert abs(ht.reconstruct_error(X4, tree4, U32, B32) - O.ht_error(X4, tree4, U, B)) < 1e-6


def test_reference_shims():
    X, k = synth.reference_style(48, seed=10)
    e = ht.htd(X, [1, 8, 8, 8, 8])
    assert 0 <= e < 1e-3
    tree4 = ht.balanced_tree_4d([1, 6, 6, 3, 3, 3, 3])
    X4 = synth.exact_ht((16, 16, 16, 16), tree4, noise_rel=0.0, seed=11)
    ht.htd4(X4, [1, 6, 6, 3, 3, 3, 3])


def test_host_and_device_inputs_agree():
    tree = ht.reference_tree_3d([1, 8, 8, 8, 8])
    X = synth.exact_ht((48, 40, 32), tree, noise_rel=1e-3, seed=12)
    rh = ht.decompose(X, tree, precision="bf16", compute_error=True)
    rd = ht.decompose(to_dev(X), tree, precision="bf16", compute_error=True)
    for t in rh.U:
        np.testing.assert_array_equal(rh.U[t], rd.U[t].cpu().numpy())
    for t in rh.B:
        np.testing.assert_array_equal(rh.B[t], rd.B[t].cpu().numpy())
    assert rh.report["rel_err"] == rd.report["rel_err"]


def test_deterministic_repeat():
    tree = ht.reference_tree_3d([1, 16, 16, 16, 16])
    X = synth.odeco(96, seed=13)
    a = ht.decompose(X, tree, precision="bf16")
    b = ht.decompose(X, tree, precision="bf16")
    for t in a.U:
        np.testing.assert_array_equal(a.U[t], b.U[t])


def test_user_start_block():
    tree = ht.reference_tree_3d([1, 8, 8, 8, 8])
    X = synth.exact_ht((48, 48, 48), tree, noise_rel=1e-3, seed=14)
    rng = np.random.default_rng(0)
    sk = [rng.standard_normal((48, 24)).astype(np.float32) for _ in range(3)]
    res = ht.decompose(X, tree, precision="fp32", compute_error=True, sketch=sk, oversample=16)
    Uo, Bo, _ = O.ht_decompose(X, tree)
    assert abs(res.report["rel_err"] - O.ht_error(X, tree, Uo, Bo)) < 1e-5


@pytest.mark.parametrize("prec", ["fp32", "bf16"])
def test_numerically_rank_deficient_large_modes(prec):
    """Separable-bumps tensor at 128^3, rank 24: the mode Grams have ~20 eigenvalues
    above 1e-12 of the largest and the rest at rounding level, so the leaf
    solver runs its subspace iteration (n > 64) on numerically rank-deficient
    blocks.  FP32 arithmetic cannot resolve directions below ~1e-7 of the
    largest eigenvalue: the float32 restatement of the reference algorithm
    (LAPACK ssyevd/sgesvd in the oracle) itself lands near 1.5e-4 here, not at
    the FP64 error (3e-8).  Bar: within 2x of that float32 error (plain path),
    and the mixed path within the mixed tolerance of it."""
    X = synth.bumps(128, seed=20000)
    tree = ht.reference_tree_3d([1, 24, 24, 24, 24])
    U32, B32, _ = O.ht_decompose(X.astype(np.float32), tree, dtype=np.float32)
    e32 = O.ht_error(X, tree, {t: U32[t].astype(np.float64) for t in U32}, {t: B32[t].astype(np.float64) for t in B32})
    res, U, B = run(X, tree, prec)
    e = O.ht_error(X, tree, U, B)
    if prec == "fp32":
        assert e <= 2.0 * e32 + 1e-6, (e, e32)
    else:
        assert e <= e32 + TOL["bf16"], (e, e32)
    for t in tree.leaves():
        assert O.orthogonality_defect(U[t]) < 2e-5


@pytest.mark.parametrize("where", ["device", "host"])
def test_slab_pipelined_input_512cubed(where):
    """3rd-order BF16 Gram-path host inputs of 256 MiB and more run slab by slab:
    the mode-1/2 Grams accumulate over 8 slabs along mode 3 while the next slab
    is copied (device inputs take the plain path).  At 512^3 on the r^-1.5
    family the error matches the closed-form FP64 optimum within 1e-3 and the
    plain path's (not pipelined) within 1e-3, the leaf bases are orthonormal, and
    the leading leaf subspaces agree with the plain path's."""
    n, k = 512, 32
    tree = ht.reference_tree_3d([1, k, k, k, k])
    X = synth.odeco(n, decay=1.5, seed=2, assemble_on=torch.device("cuda"))
    e_opt = synth.odeco_optimal_error(n, k)
    plain = ht.decompose(X, tree, precision="fp32", compute_error=True)
    x = X if where == "device" else X.cpu().numpy().reshape(-1)
    kw = {} if where == "device" else {"dims": (n, n, n)}
    mixed = ht.decompose(x, tree, precision="bf16", compute_error=True, **kw)
    assert abs(mixed.report["rel_err"] - e_opt) <= 1e-3
    assert abs(mixed.report["rel_err"] - plain.report["rel_err"]) <= 1e-3
    for t in tree.leaves():
        Um = np.asarray(mixed.U[t].cpu() if hasattr(mixed.U[t], "cpu") else mixed.U[t], np.float64)
        Up = plain.U[t].cpu().numpy().astype(np.float64)
        assert O.orthogonality_defect(Um) < 2e-4
        # the leading 8 directions are well separated on this spectrum
        assert O.principal_angles(Um[:, :8], Up[:, :8]).max() < 3e-2


@pytest.mark.parametrize("dims", [(37, 45, 51), (61, 64, 40), (45, 32, 24, 17)])
def test_unaligned_first_mode_uses_padded_bf16_grams(dims):
    """A first mode that is not a multiple of 8 cannot be addressed by TMA in
    place; the mixed path then reads its leaf Grams from a zero-padded BF16
    copy and still runs them on tcgen05, within the BF16 bar of the oracle."""
    if len(dims) == 3:
        tree = ht.reference_tree_3d([1, 8, 6, 7, 6])
    else:
        tree = ht.balanced_tree_4d([1, 10, 10, 5, 5, 5, 5])
    X = synth.exact_ht(dims, tree, noise_rel=1e-3, seed=17)
    res, e, e64 = check_against_oracle(X, tree, "bf16")
    assert res.report["path"]["tcgen05"]
