"""The Gram-free leaf range finder (leaf_method="sketch", HT_LEAF_SKETCH) and
the Householder TSQR (ht_tsqr) on the GPU.

TSQR against numpy's float64 QR: R with a non-negative diagonal is unique for
a full-rank A, so it is compared directly on well-conditioned inputs
(1e-5 relative, Frobenius); R^T R = A^T A (1e-5 relative) holds for any A,
rank-deficient or ill-conditioned.

The sketch path against the FP64 oracle (the reference's algorithm restated):
its subspaces come from a randomized range finder, so it is held to the
mixed-precision bar |err - err_fp64| <= 1e-3 on both precisions, with
orthonormal leaf bases, the device-reported error equal to the oracle's
reconstruction of the returned factors, and leaf principal angles to the
oracle's subspaces below 1e-2 rad wherever the spectrum has a gap.
"""
import numpy as np
import pytest
import torch

import ht_tensor_learning_using_gpu_tensor_cores_gb300 as ht
from ht_tensor_learning_using_gpu_tensor_cores_gb300 import learn, synth
import ht_oracle as O

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


def r_fp64(A):
    R = np.linalg.qr(np.asarray(A, np.float64), mode="r")
    return R * np.where(np.diag(R) < 0, -1.0, 1.0)[:, None]


@pytest.mark.parametrize("m,k", [(1000, 7), (65536, 32), (100003, 33), (262144, 48), (1 << 20, 64), (64, 64),
                                 (129, 1)])
def test_tsqr_matches_fp64_qr(m, k):
    A = np.random.default_rng(m + k).standard_normal((m, k)).astype(np.float32)
    Ad = torch.from_numpy(np.ascontiguousarray(A.T)).cuda().t()   # (m, k), contiguous columns
    R = ht.tsqr(Ad).cpu().numpy()
    assert np.allclose(np.tril(R, -1), 0.0)
    assert (np.diag(R) >= 0).all()
    if m >= 4 * k:   # well conditioned: R itself is determined to FP32 rounding
        assert rel(R, r_fp64(A)) < 1e-5, rel(R, r_fp64(A))
    G = A.astype(np.float64).T @ A.astype(np.float64)
    assert rel(R.astype(np.float64).T @ R, G) < 1e-5


def test_tsqr_host_input_leading_dimension_and_rank_deficiency():
    """Host A with lda > m, and A of rank 5 < k (R^T R = A^T A still holds);
    an ill-conditioned A (column scales 1 .. 1e-4) likewise."""
    rng = np.random.default_rng(5)
    m, k, lda = 5000, 12, 5003
    buf = np.zeros((lda, k), dtype=np.float32, order="F")
    buf[:m] = rng.standard_normal((m, 5)) @ rng.standard_normal((5, k))
    R = np.zeros((k, k), dtype=np.float32, order="F")
    from ht_tensor_learning_using_gpu_tensor_cores_gb300._lib import lib, check
    import ctypes
    check(lib().ht_tsqr(ctypes.c_void_p(buf.ctypes.data), m, k, lda, ctypes.c_void_p(R.ctypes.data), None))
    A = buf[:m].astype(np.float64)
    assert rel(R.astype(np.float64).T @ R, A.T @ A) < 1e-5
    B = (rng.standard_normal((40000, 20)) * np.logspace(0, -4, 20)).astype(np.float32)
    Rb = ht.tsqr(B)
    assert rel(Rb.astype(np.float64).T @ Rb, B.astype(np.float64).T @ B) < 1e-5


def sketch_vs_oracle(X, tree, prec, angle_tol=None, tol=1e-3, **kw):
    xd = torch.from_numpy(np.ascontiguousarray(X.transpose(tuple(range(X.ndim))[::-1]))).cuda()
    res = ht.decompose(xd, tree, precision=prec, compute_error=True, leaf_method="sketch", **kw)
    U = {t: res.U[t].cpu().numpy().astype(np.float64) for t in res.U}
    B = {t: res.B[t].cpu().numpy().astype(np.float64) for t in res.B}
    Uo, Bo, _ = O.ht_decompose(X, tree, dtype=np.float64)
    e64 = O.ht_error(X, tree, Uo, Bo)
    e = O.ht_error(X, tree, U, B)
    assert e - e64 <= tol, (prec, e, e64)
    assert abs(res.report["rel_err"] - e) <= 1e-5 + 1e-3 * e, (res.report["rel_err"], e)
    angles = {}
    for t in tree.leaves():
        assert O.orthogonality_defect(U[t]) < 1e-4, t
        angles[t] = float(O.principal_angles(U[t], Uo[t]).max())
        if angle_tol is not None:
            assert angles[t] < angle_tol, (t, angles)
    return e, e64, angles


@pytest.mark.parametrize("tree_fn", [ht.reference_tree_3d, ht.left_first_tree_3d, ht.middle_tree_3d])
@pytest.mark.parametrize("prec", ["fp32", "bf16"])
def test_sketch_exact_ht_all_trees(tree_fn, prec):
    """Exact HT rank 12 + 1e-3 noise (a clear spectral gap): the range finder
    recovers the oracle's subspaces."""
    tree = tree_fn([1, 12, 12, 12, 12])
    X = synth.exact_ht((160, 144, 128), tree, noise_rel=1e-3, seed=21)
    sketch_vs_oracle(X, tree, prec, angle_tol=1e-2)


@pytest.mark.parametrize("prec", ["fp32", "bf16"])
def test_sketch_decaying_spectrum_c2_style(prec):
    """The headline family at 256^3 (every matricisation with singular values
    r^-1.5, rank 32), oversampling 10 and one power step as the configuration
    names; no gap, so the bar is the error alone."""
    tree = ht.reference_tree_3d([1, 32, 32, 32, 32])
    X = synth.odeco(256, 3, 1.5, seed=3)
    e, e64, _ = sketch_vs_oracle(X, tree, prec, oversample=10, power_steps=1)
    assert e >= e64 - 1e-6


def test_sketch_uneven_ranks():
    """k_{12} > k_3: the complementary leaf's basis has kw = k_{12} columns and
    the TSQR of X_(12) V is kw wide."""
    tree = ht.reference_tree_3d([1, 20, 9, 8, 7])
    X = synth.exact_ht((96, 80, 112), tree, noise_rel=1e-3, seed=8)
    sketch_vs_oracle(X, tree, "bf16", angle_tol=2e-2)


@pytest.mark.parametrize("prec", ["fp32", "bf16"])
def test_sketch_4d_balanced(prec):
    tree = ht.balanced_tree_4d([1, 20, 20, 10, 10, 10, 10])
    X = synth.exact_ht((40, 36, 32, 44), tree, noise_rel=1e-3, seed=9)
    sketch_vs_oracle(X, tree, prec, angle_tol=1e-2)


def test_sketch_small_modes_and_power_steps():
    """Modes below the sketch width (s = n: the block spans the whole mode),
    and zero or two power steps."""
    tree = ht.reference_tree_3d([1, 8, 6, 8, 8])
    X = synth.exact_ht((24, 40, 30), tree, noise_rel=1e-3, seed=10)
    for q in (0, 2):
        sketch_vs_oracle(X, tree, "bf16", power_steps=q)


def test_sketch_bumps_gaussian_and_learned_blocks():
    """The separable-bumps family (rank <= 32, target 24, block width 34): the
    Gaussian block and a block trained on the family's Grams both stay within
    1e-3 of the exact-Gram path's error, which is itself within 1e-3 of FP64."""
    n, k, p = 256, 24, 10
    tree = ht.reference_tree_3d([1, k, k, k, k])
    X = synth.bumps(n, seed=931, assemble_on=torch.device("cuda"))
    Xnp = np.asfortranarray(X.cpu().numpy().transpose(2, 1, 0))
    exact = ht.decompose(X, tree, precision="bf16", compute_error=True).report["rel_err"]
    G, trg = learn.family_grams(range(940, 946), n, precision="bf16")
    sketches, _ = learn.train_mode_sketches(G, trg, s=k + p, steps=40, batch=6, lr=2e-3, seed=4)
    for sk in (None, [learn.to_bf16(S) for S in sketches]):
        res = ht.decompose(X, tree, precision="bf16", compute_error=True, leaf_method="sketch", oversample=p,
                           sketch=sk)
        U = {t: res.U[t].cpu().numpy() for t in res.U}
        B = {t: res.B[t].cpu().numpy() for t in res.B}
        e = O.ht_error(Xnp, tree, U, B)
        assert e <= exact + 1e-3, (e, exact)


def test_sketch_rejected_where_grams_are_needed():
    tree = ht.reference_tree_3d([1, 4, 4, 4, 4])
    X = np.asfortranarray(np.random.default_rng(0).standard_normal((16, 16, 16)).astype(np.float32))
    with pytest.raises(ht.HTError, match="UNSUPPORTED"):
        _streaming_sketch(X, tree)


def _streaming_sketch(X, tree):
    import ctypes
    from ht_tensor_learning_using_gpu_tensor_cores_gb300 import _config, _tree_struct, _out_buffers
    from ht_tensor_learning_using_gpu_tensor_cores_gb300._lib import HtReport, check, lib
    cfg, _ = _config("bf16", 16, 10, 1, 1234, 0, None, 0.0, "sketch")
    ts = _tree_struct(tree)
    U, B, up, bp = _out_buffers(tree, X.shape, None)
    rep = HtReport()
    check(lib().ht_decompose_streaming(ctypes.c_void_p(X.ctypes.data), (ctypes.c_long * 4)(*X.shape), 3,
                                       ctypes.byref(ts), ctypes.byref(cfg), up, bp, ctypes.c_ulonglong(1 << 20),
                                       ctypes.byref(rep), None))
