"""Out-of-core decomposition (ht_decompose_streaming): the tensor stays in host
memory and is streamed through two device slab buffers.  Checked against the
FP64 oracle's error on the same input (tolerances as the in-core parity tests:
FP32 1e-5, BF16 1e-3), against the in-core decomposition of the same tensor,
and its own error pass against the oracle's reconstruction of its factors.
"""
import numpy as np
import pytest
import torch

import ht_tensor_learning_using_gpu_tensor_cores_gb300 as ht
from ht_tensor_learning_using_gpu_tensor_cores_gb300 import synth
from ht_tensor_learning_using_gpu_tensor_cores_gb300._lib import HTError
import ht_oracle as O

pytestmark = pytest.mark.gpu

TOL = {"fp32": 1e-5, "bf16": 1e-3}

TREES = [ht.reference_tree_3d, ht.left_first_tree_3d, ht.middle_tree_3d]


def slab_budget(dims, slices):
    """Bytes for two FP32 slabs of `slices` frontal slices."""
    return 2 * 4 * dims[0] * dims[1] * slices


@pytest.mark.parametrize("mk", TREES)
@pytest.mark.parametrize("prec", ["fp32", "bf16"])
def test_streaming_matches_oracle_and_in_core(mk, prec):
    dims = (96, 80, 112)
    tree = mk([1, 10, 8, 6, 7])
    tree.check_ranks(dims)
    X = synth.exact_ht(dims, tree, noise_rel=1e-3, seed=7)
    # 13 slices per slab along mode 3 (the last slab ragged), and the matching
    # mode-2 slabs: 9 passes' worth of copies per pass
    res = ht.decompose_streaming(X, tree, slab_bytes=slab_budget(dims, 13), precision=prec, compute_error=True)
    U = {t: np.asarray(a, np.float64) for t, a in res.U.items()}
    B = {t: np.asarray(a, np.float64) for t, a in res.B.items()}
    Uo, Bo, _ = O.ht_decompose(X, tree, dtype=np.float64)
    e64 = O.ht_error(X, tree, Uo, Bo)
    e = O.ht_error(X, tree, U, B)
    assert abs(e - e64) <= TOL[prec], (e, e64)
    assert abs(res.report["rel_err"] - e) <= 1e-5 + 1e-4 * e
    assert abs(res.report["norm_x"] - np.linalg.norm(X.astype(np.float64).ravel())) <= 1e-6 * res.report["norm_x"]
    ref = ht.decompose(X, tree, precision=prec, compute_error=True)
    assert abs(res.report["rel_err"] - ref.report["rel_err"]) <= (1e-6 if prec == "fp32" else 5e-5)
    for t in tree.leaves():
        assert O.orthogonality_defect(U[t]) < (2e-5 if prec == "fp32" else 2e-4)


def test_streaming_one_slice_slabs_and_pinned_input():
    """The smallest budget (one slice per slab) and a page-locked torch input."""
    dims = (40, 24, 56)
    tree = ht.reference_tree_3d([1, 12, 6, 5, 7])
    X = synth.exact_ht(dims, tree, noise_rel=1e-2, seed=3)
    Xt = torch.from_numpy(np.ascontiguousarray(X.transpose(2, 1, 0))).pin_memory()
    res = ht.decompose_streaming(Xt, tree, slab_bytes=1, precision="bf16", compute_error=True)
    ref = ht.decompose(X, tree, precision="bf16", compute_error=True)
    assert abs(res.report["rel_err"] - ref.report["rel_err"]) <= 5e-5
    e = O.ht_error(X, tree, {t: np.asarray(a, np.float64) for t, a in res.U.items()},
                   {t: np.asarray(a, np.float64) for t, a in res.B.items()})
    assert abs(res.report["rel_err"] - e) <= 1e-5 + 1e-4 * e


def test_streaming_large_matches_in_core():
    """512^3 (512 MiB) through 64 MiB of slab buffers, BF16: the error equals the
    in-core path's on the same tensor."""
    n, k = 512, 24
    tree = ht.reference_tree_3d([1, k, k, k, k])
    Xd = synth.exact_ht_device((n, n, n), tree, noise_rel=1e-3, seed=11)
    Xh = Xd.cpu().pin_memory()
    ref = ht.decompose(Xd, tree, precision="bf16", compute_error=True)
    del Xd
    torch.cuda.empty_cache()
    res = ht.decompose_streaming(Xh, tree, slab_bytes=64 << 20, precision="bf16", compute_error=True)
    assert abs(res.report["rel_err"] - ref.report["rel_err"]) <= 2e-5, (res.report["rel_err"], ref.report["rel_err"])
    assert abs(res.report["rel_err"] - 1e-3) < 1e-4


def test_streaming_rejects_device_input_and_4th_order():
    tree = ht.reference_tree_3d([1, 2, 2, 2, 2])
    with pytest.raises(TypeError):
        ht.decompose_streaming(torch.zeros(8, 8, 8, device="cuda"), tree, slab_bytes=1 << 20)
    t4 = ht.balanced_tree_4d([1, 2, 2, 2, 2, 2, 2])
    with pytest.raises((ValueError, HTError)):
        ht.decompose_streaming(np.zeros((4, 4, 4, 4), np.float32, order="F"), t4, slab_bytes=1 << 20)


def test_pipelined_host_input_matches_device_input():
    """Host input of a large 3rd-order tensor goes through the pipelined copy
    (slabs along mode 3, conversion and mode-1/2 Gram shares as each lands): the
    result equals the device-input path's."""
    n, k = 512, 24
    tree = ht.reference_tree_3d([1, k, k, k, k])
    Xd = synth.exact_ht_device((n, n, n), tree, noise_rel=1e-3, seed=13)
    ref = ht.decompose(Xd, tree, precision="bf16", compute_error=True)
    Xh = Xd.cpu().pin_memory().numpy().reshape(-1)
    res = ht.decompose(Xh, tree, dims=(n, n, n), precision="bf16", compute_error=True)
    assert abs(res.report["rel_err"] - ref.report["rel_err"]) <= 2e-6, (res.report["rel_err"], ref.report["rel_err"])
    assert abs(res.report["norm_x"] - ref.report["norm_x"]) <= 1e-6 * ref.report["norm_x"]
    for t in tree.leaves():
        assert O.principal_angles(np.asarray(res.U[t], np.float64), ref.U[t].cpu().numpy().astype(np.float64)).max() < 1e-3
