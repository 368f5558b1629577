"""Argument checks of the Python API that run on the host before any device
call (no GPU): each bad call raises ValueError / TypeError, and a good call
reaches the library (which, without a device, reports HT_ERR_NO_DEVICE)."""
import numpy as np
import pytest

import ht_tensor_learning_using_gpu_tensor_cores_gb300 as ht


def _no_gpu():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")


def _x(shape=(8, 8, 8), dtype=np.float32):
    return np.zeros(shape, dtype=dtype, order="F")


def test_decompose_rejects_bad_arguments_before_the_device():
    tree = ht.reference_tree_3d([1, 2, 2, 2, 2])
    with pytest.raises(ValueError, match="precision"):
        ht.decompose(_x(), tree, precision="fp16")
    with pytest.raises(ValueError, match="leaf_method"):
        ht.decompose(_x(), tree, leaf_method="qr")
    with pytest.raises(TypeError, match="float32"):
        ht.decompose(_x(dtype=np.float64), tree)
    with pytest.raises(ValueError, match="buffer size"):
        ht.decompose(np.zeros(100, dtype=np.float32), tree, dims=(8, 8, 8))
    with pytest.raises(ValueError, match="dims"):
        ht.decompose(np.zeros(512, dtype=np.float32), tree)          # flat buffer without dims
    with pytest.raises(ValueError, match="order"):
        ht.decompose(_x(), tree, dims=(8, 8, 8, 8))
    with pytest.raises(ValueError, match="rank"):
        ht.decompose(_x((8, 8, 2)), ht.reference_tree_3d([1, 2, 3, 2, 2]))   # leaf {3}: k = 3 > n = 2


def test_rank_rules_of_interior_nodes():
    # the interior node {1,2} carries at most k_1 k_2 columns
    with pytest.raises(ValueError):
        ht.reference_tree_3d([1, 5, 5, 2, 2]).check_ranks((8, 8, 8))
    ht.reference_tree_3d([1, 4, 4, 2, 2]).check_ranks((8, 8, 8))


def test_good_call_reaches_the_library():
    _no_gpu()
    tree = ht.reference_tree_3d([1, 2, 2, 2, 2])
    for kw in ({}, {"precision": "fp32"}, {"leaf_method": "sketch"}):
        with pytest.raises(ht.HTError) as ei:
            ht.decompose(_x(), tree, **kw)
        assert ei.value.status == 7          # HT_ERR_NO_DEVICE: no CPU fallback
    # a flat buffer with dims, in the reference's column-major order
    with pytest.raises(ht.HTError):
        ht.decompose(np.zeros(512, dtype=np.float32), tree, dims=(8, 8, 8))


def test_reference_shims_check_the_order():
    with pytest.raises(ValueError, match="3rd-order"):
        ht.htd(_x((4, 4, 4, 4)), [1, 2, 2, 2, 2])
    with pytest.raises(ValueError, match="4th-order"):
        ht.htd4(_x(), [1, 2, 2, 2, 2, 2, 2])


def test_streaming_takes_third_order_host_tensors():
    t4 = ht.balanced_tree_4d([1, 4, 4, 2, 2, 2, 2])
    with pytest.raises(ValueError, match="3rd-order"):
        ht.decompose_streaming(_x((4, 4, 4, 4)), t4, slab_bytes=1 << 20)


def test_batch_decomposer_checks_its_tensors():
    t3 = ht.reference_tree_3d([1, 2, 2, 2, 2])
    t4 = ht.balanced_tree_4d([1, 4, 4, 2, 2, 2, 2])
    with pytest.raises(ValueError, match="one tree per tensor"):
        ht.BatchDecomposer([t3, t3], [(8, 8, 8)])
    with pytest.raises(ValueError, match="one tree per tensor"):
        ht.BatchDecomposer([], [])
    with pytest.raises(ValueError, match="same order"):
        ht.BatchDecomposer([t3, t4], [(8, 8, 8), (4, 4, 4, 4)])
    with pytest.raises(ValueError, match="rank"):
        ht.BatchDecomposer([ht.reference_tree_3d([1, 2, 2, 9, 2])], [(8, 8, 8)])
