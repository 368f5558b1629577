"""The allocation-free Gram entry point (ht_mode_gram_noalloc), called through
the C ABI on device buffers, against numpy's float64 X_(g) X_(g)^T and against
the allocating entry point (ht_mode_gram, FP32).  FP32 tolerance as elsewhere:
1e-5 relative (Frobenius).

Two calls in a row on different shapes share the one static scratch array;
the second must not see the first's leftovers.  The file is named so that
pytest collects it last; it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest
import torch

from ht_tensor_learning_using_gpu_tensor_cores_gb300 import _lib

pytestmark = pytest.mark.gpu

TOL = 1e-5
HT_ERR_UNSUPPORTED = 6


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


def device_tensor(dims, seed):
    x = np.random.default_rng(seed).standard_normal(int(np.prod(dims))).astype(np.float32)
    return torch.from_numpy(x).cuda()   # flat column-major storage of a tensor with these dims


def n_of(dims, lo, hi):
    return int(np.prod(dims[lo:hi + 1]))


def gram_fp64(x, dims, lo, hi):
    """X_(g) X_(g)^T in float64: rows over modes lo..hi, columns over the rest."""
    L = int(np.prod(dims[:lo]))
    N = n_of(dims, lo, hi)
    R = int(np.prod(dims[hi + 1:]))
    X3 = x.cpu().numpy().astype(np.float64).reshape((L, N, R), order="F")
    Xg = X3.transpose(1, 0, 2).reshape(N, L * R)
    return Xg @ Xg.T


def call_noalloc(L, x, dims, lo, hi, G, stream):
    return L.ht_mode_gram_noalloc(ctypes.c_void_p(x.data_ptr()), (ctypes.c_long * 4)(*dims), len(dims), lo, hi,
                                  ctypes.c_void_p(G.data_ptr()), ctypes.c_void_p(stream))


def call_alloc(L, x, dims, lo, hi, G, stream):
    return L.ht_mode_gram(ctypes.c_void_p(x.data_ptr()), (ctypes.c_long * 4)(*dims), len(dims), lo, hi,
                          _lib.PREC_FP32, ctypes.c_void_p(G.data_ptr()), ctypes.c_void_p(stream))


def test_noalloc_gram_matches_allocating_gram_twice():
    L = _lib.lib()
    stream = torch.cuda.current_stream().cuda_stream
    cases = [((96, 256, 80), 1, 1),          # split-K Gram, n = 256
             ((24, 16, 20, 32), 0, 1)]       # a different shape and split count, n = 384
    inputs = [device_tensor(d, 100 + i) for i, (d, _, _) in enumerate(cases)]
    outs = [torch.full((n_of(d, lo, hi),) * 2, float("nan"), device="cuda") for d, lo, hi in cases]
    refs = [torch.empty((n_of(d, lo, hi),) * 2, device="cuda") for d, lo, hi in cases]
    for (d, lo, hi), x, G, R in zip(cases, inputs, outs, refs):
        assert call_alloc(L, x, d, lo, hi, R, stream) == 0, _lib.lib().ht_last_error()
    torch.cuda.synchronize()
    free_before = None
    for i, ((d, lo, hi), x, G) in enumerate(zip(cases, inputs, outs)):
        if i == 1:
            free_before = torch.cuda.mem_get_info()[0]
        rc = call_noalloc(L, x, d, lo, hi, G, stream)
        assert rc == 0, L.ht_last_error()
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free_before, "the no-alloc call changed free device memory"
    for (d, lo, hi), x, G, R in zip(cases, inputs, outs, refs):
        g, r = G.cpu().numpy(), R.cpu().numpy()
        assert np.isfinite(g).all()
        assert np.array_equal(g, g.T)
        assert rel(g, gram_fp64(x, d, lo, hi)) < TOL, (d, lo, hi, rel(g, gram_fp64(x, d, lo, hi)))
        assert rel(g, r) < TOL, (d, lo, hi, rel(g, r))
    # the first shape again, after the second call left its partials in the scratch
    d, lo, hi = cases[0]
    G = torch.full_like(outs[0], float("nan"))
    assert call_noalloc(L, inputs[0], d, lo, hi, G, stream) == 0
    torch.cuda.synchronize()
    assert rel(G.cpu().numpy(), gram_fp64(inputs[0], d, lo, hi)) < TOL
    assert rel(G.cpu().numpy(), refs[0].cpu().numpy()) < TOL


def test_noalloc_gram_rejects_sizes_above_its_maximum():
    L = _lib.lib()
    x = torch.zeros(4, device="cuda")
    G = torch.zeros(4, device="cuda")
    dims = (2049, 1, 1)
    rc = call_noalloc(L, x, dims, 0, 0, G, torch.cuda.current_stream().cuda_stream)
    assert rc == HT_ERR_UNSUPPORTED
    assert b"maximum" in L.ht_last_error()
