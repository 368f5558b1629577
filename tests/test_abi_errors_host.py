"""Error behaviour of the C ABI that needs no device (no GPU): every entry point
checks its arguments before it looks for a device, returns a status code (never
aborts) and leaves the reason in ht_last_error()."""
import ctypes
from ctypes import POINTER, c_double, c_long, c_void_p

import numpy as np
import pytest

import ht_tensor_learning_using_gpu_tensor_cores_gb300 as ht
from ht_tensor_learning_using_gpu_tensor_cores_gb300._lib import (HtBatchReport, HtConfig, HtReport, HtTree, MAX_NODES,
                                                                   lib)

OK, INVALID_ARG, UNSUPPORTED, NO_DEVICE = 0, 1, 6, 7


def _tree3(k):
    t = HtTree()
    ks = (ctypes.c_int * 5)(*k)
    assert lib().ht_tree_reference_3d(ctypes.byref(t), ks) == OK
    return t


def _cfg(**kw):
    c = HtConfig()
    assert lib().ht_config_default(ctypes.byref(c)) == OK
    for k, v in kw.items():
        setattr(c, k, v)
    return c


def _last():
    return lib().ht_last_error().decode()


def _decompose(x, dims, tree, cfg):
    U = (c_void_p * MAX_NODES)()
    B = (c_void_p * MAX_NODES)()
    bufs = [np.zeros(64 * 64, dtype=np.float32) for _ in range(MAX_NODES)]
    for i in range(MAX_NODES):
        U[i] = bufs[i].ctypes.data
        B[i] = bufs[i].ctypes.data
    rep = HtReport()
    cd = (c_long * 4)(*dims)
    return lib().ht_decompose(x, cd, len(dims), ctypes.byref(tree), ctypes.byref(cfg), U, B, ctypes.byref(rep),
                              None)


def test_decompose_checks_arguments_first():
    x = np.zeros(8 * 8 * 8, dtype=np.float32)
    xp = c_void_p(x.ctypes.data)
    t = _tree3([1, 2, 2, 2, 2])
    assert _decompose(None, (8, 8, 8), t, _cfg()) == INVALID_ARG
    assert "NULL" in _last()
    assert _decompose(xp, (8, 8, 8), t, _cfg(precision=9)) == INVALID_ARG
    assert "precision" in _last()
    assert _decompose(xp, (8, 8, 8), t, _cfg(leaf_method=9)) == INVALID_ARG
    assert _decompose(xp, (8, 8, 8), t, _cfg(oversample=-1)) == INVALID_ARG
    assert _decompose(xp, (8, 8, 2), _tree3([1, 2, 3, 2, 2]), _cfg()) == INVALID_ARG   # k_{3} = 3 > n_3 = 2
    assert _decompose(xp, (8, 8, 0), t, _cfg()) == INVALID_ARG


def test_valid_call_without_device_reports_no_device():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    x = np.zeros(8 * 8 * 8, dtype=np.float32)
    assert _decompose(c_void_p(x.ctypes.data), (8, 8, 8), _tree3([1, 2, 2, 2, 2]), _cfg()) == NO_DEVICE
    assert _last()


def test_batched_entry_checks_arguments_first():
    L = lib()
    rep = HtBatchReport()
    errs = (c_double * 1)()
    xs = (c_void_p * 1)()
    U = (c_void_p * MAX_NODES)()
    B = (c_void_p * MAX_NODES)()
    dims = (c_long * 3)(8, 8, 8)
    t = _tree3([1, 2, 2, 2, 2])
    cfg = _cfg()
    assert L.ht_decompose_batched(0, xs, dims, 3, ctypes.byref(t), ctypes.byref(cfg), U, B, errs,
                                  ctypes.byref(rep), None) == INVALID_ARG
    sk = _cfg(leaf_method=1)   # HT_LEAF_SKETCH: the batched path computes Grams
    x = np.zeros(512, dtype=np.float32)
    xs[0] = x.ctypes.data
    assert L.ht_decompose_batched(1, xs, dims, 3, ctypes.byref(t), ctypes.byref(sk), U, B, errs,
                                  ctypes.byref(rep), None) == UNSUPPORTED
    assert "ht_decompose" in _last()
    assert L.ht_batch_set_tuning(-1, 0) == INVALID_ARG
    assert L.ht_batch_set_tuning(1 << 20, 0) == INVALID_ARG
    assert L.ht_batch_set_tuning(0, -1) == INVALID_ARG


def test_primitives_check_arguments_first():
    L = lib()
    a = np.zeros(64, dtype=np.float32)
    p = c_void_p(a.ctypes.data)
    dims = (c_long * 3)(4, 4, 4)
    assert L.ht_tsqr(None, 16, 4, 16, p, None) == INVALID_ARG
    assert L.ht_tsqr(p, 16, 4, 8, p, None) == INVALID_ARG          # lda < m
    assert L.ht_tsqr(p, 16, 65, 16, p, None) == UNSUPPORTED        # k above 64
    assert L.ht_mode_gram_noalloc(None, dims, 3, 0, 0, p, None) == INVALID_ARG
    assert L.ht_mode_gram_noalloc(p, dims, 3, 2, 1, p, None) == INVALID_ARG   # hi < lo
    assert L.ht_mode_gram_noalloc(p, dims, 5, 0, 0, p, None) == INVALID_ARG   # order above 4
    loss = c_double()
    assert L.ht_sketch_loss_grad(None, p, 1, 4, 2, p, p, ctypes.byref(loss), None) == INVALID_ARG
    assert L.ht_sketch_loss_grad(p, p, 1, 4, 5, p, p, ctypes.byref(loss), None) == INVALID_ARG   # s > n
    assert L.ht_selftest_wait_timeout(0, 10.0, None) == INVALID_ARG
    assert L.ht_selftest_wait_timeout(1, 5000.0, None) == INVALID_ARG


def test_status_strings_name_every_code():
    L = lib()
    names = [L.ht_status_string(s).decode() for s in range(9)]
    assert names[0] == "ok"
    assert all(names) and len(set(names)) == 9
    assert L.ht_status_string(99)   # an unknown code still maps to a string


def test_python_errors_carry_the_status_and_reason():
    err = ht.HTError(INVALID_ARG, "dims must be positive")
    assert err.status == INVALID_ARG
    assert "dims must be positive" in str(err)
