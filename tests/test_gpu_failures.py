"""Failure detection on the device path: a non-finite input is reported as
HT_ERR_NUMERICAL (status code, no fault, no hang), for device- and host-resident
inputs and for one tensor of a batch, and the context stays usable: the next
decomposition on the same device succeeds with the usual error."""
import numpy as np
import pytest
import torch

import ht_tensor_learning_using_gpu_tensor_cores_gb300 as ht
from ht_tensor_learning_using_gpu_tensor_cores_gb300 import synth
from ht_tensor_learning_using_gpu_tensor_cores_gb300._lib import HTError

pytestmark = pytest.mark.gpu
HT_ERR_NUMERICAL = 8


def _tensor(seed=3):
    tree = ht.reference_tree_3d([1, 6, 5, 4, 6])
    X = synth.exact_ht((48, 40, 56), tree, noise_rel=1e-3, seed=seed)
    return tree, X


@pytest.mark.parametrize("bad", [np.nan, np.inf, -np.inf])
@pytest.mark.parametrize("where", ["device", "host"])
@pytest.mark.parametrize("prec", ["fp32", "bf16"])
def test_non_finite_input_is_reported(bad, where, prec):
    tree, X = _tensor()   # a fresh column-major array
    X[5, 7, 11] = bad
    x = torch.from_numpy(np.ascontiguousarray(X.transpose(2, 1, 0))).cuda() if where == "device" else X
    with pytest.raises(HTError) as e:
        ht.decompose(x, tree, precision=prec)
    assert e.value.status == HT_ERR_NUMERICAL
    # the device and the library are still usable
    ref = ht.decompose(_tensor()[1], tree, precision=prec, compute_error=True)
    assert abs(ref.report["rel_err"] - 1e-3) < 1e-4


def test_non_finite_tensor_in_a_batch_is_reported():
    fam = synth.batch_family(6, seed=5, device="cuda")
    xs = [x.clone() for x, _ in fam]
    trees = [t for _, t in fam]
    dims = [tuple(reversed(x.shape)) for x in xs]
    xs[3].view(-1)[17] = float("nan")
    bd = ht.BatchDecomposer(trees, dims, precision="bf16", compute_error=True)
    with pytest.raises(HTError) as e:
        bd(xs)
    assert e.value.status == HT_ERR_NUMERICAL
    assert "tensor 3" in str(e.value)
    del bd
    ht.release_batch()


@pytest.mark.parametrize("ctas", [1, 8])
def test_bounded_wait_runs_out_and_the_device_stays_usable(ctas):
    """A grid barrier that waits for one CTA more than its grid holds can only
    run out (ht_selftest_wait_timeout, a 20 ms limit instead of the library's
    2 s): every CTA gives up, the call returns HT_ERR_TIMEOUT, and the next
    decomposition on the same context succeeds with the usual error."""
    import time
    from ht_tensor_learning_using_gpu_tensor_cores_gb300._lib import lib
    HT_ERR_TIMEOUT = 5
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    rc = lib().ht_selftest_wait_timeout(ctas, 20.0, None)
    dt = time.perf_counter() - t0
    assert rc == HT_ERR_TIMEOUT, lib().ht_last_error()
    assert b"ran out" in lib().ht_last_error()
    assert 0.02 <= dt < 5.0, dt
    tree, X = _tensor()
    ref = ht.decompose(X, tree, precision="bf16", compute_error=True)
    assert abs(ref.report["rel_err"] - 1e-3) < 1e-4
