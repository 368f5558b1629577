"""Kernel-level GPU tests: the three unfolding products on both paths against
numpy in FP64, over every operand layout the engine uses (K-major, MN-major,
co-range with the (l, r) K order), aligned and unaligned shapes, and shapes
large enough to need many tiles and split-K.

FP32 path tolerance: 1e-5 relative (Frobenius) to FP64.  BF16 path: against
FP64 products of the BF16-rounded operands, 1e-5 relative (FP32 accumulation
is the only remaining error), and against the exact product, 1e-2.
"""
import numpy as np
import pytest
import torch

import ht_tensor_learning_using_gpu_tensor_cores_gb300 as ht
import ht_oracle as O

pytestmark = pytest.mark.gpu


def bf16(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).to(torch.bfloat16).float().numpy()


def rel(a, b):
    return float(np.linalg.norm((np.asarray(a, np.float64) - np.asarray(b, np.float64)).ravel()) /
                 max(np.linalg.norm(np.asarray(b, np.float64).ravel()), 1e-300))


def rnd(shape, seed):
    return np.asfortranarray(np.random.default_rng(seed).standard_normal(shape).astype(np.float32))


def group(dims, lo, hi):
    return tuple(range(lo, hi + 1))


def view(dims, lo, hi):
    L = int(np.prod(dims[:lo])) if lo else 1
    N = int(np.prod(dims[lo:hi + 1]))
    R = int(np.prod(dims[hi + 1:])) if hi + 1 < len(dims) else 1
    return L, N, R


def tc_expressible(op, dims, lo, hi):
    """The BF16 request runs on tcgen05 only when every TMA operand's innermost
    extent is a multiple of 8 elements; otherwise the FP32 kernel runs."""
    L, N, R = view(dims, lo, hi)
    a0 = L if L > 1 else N
    if op == "gram":
        return a0 % 8 == 0
    if op == "product":
        return a0 % 8 == 0 and N % 8 == 0
    return a0 % 8 == 0 and (L if L > 1 else R) % 8 == 0


def check_bf16(op, dims, lo, hi, got, exact, exact_bf16):
    if tc_expressible(op, dims, lo, hi):
        assert rel(got, exact_bf16) < 1e-5
        assert rel(got, exact) < 1e-2
    else:
        assert rel(got, exact) < 1e-5


CASES_GRAM = [((64, 48, 40), 0, 0), ((64, 48, 40), 1, 1), ((64, 48, 40), 2, 2), ((30, 20, 18), 0, 0),
              ((30, 20, 18), 1, 1), ((256, 256, 256), 0, 0), ((256, 256, 256), 2, 2), ((24, 16, 16, 32), 0, 1),
              ((24, 16, 16, 32), 2, 3), ((24, 16, 16, 32), 1, 1), ((16, 24, 24, 24), 3, 3), ((8, 600, 40), 1, 1)]


@pytest.mark.parametrize("dims,lo,hi", CASES_GRAM)
@pytest.mark.parametrize("prec", ["fp32", "bf16"])
def test_mode_gram(dims, lo, hi, prec):
    X = rnd(dims, hash((dims, lo)) % 1000)
    G = ht.mode_gram(X, dims, lo, hi, precision=prec)
    A = O.unfold(X.astype(np.float64), group(dims, lo, hi))
    Gx = A @ A.T
    assert np.array_equal(G, G.T), "Gram must be exactly symmetric"
    if prec == "fp32":
        assert rel(G, Gx) < 1e-5
    else:
        Ab = O.unfold(bf16(X).astype(np.float64), group(dims, lo, hi))
        check_bf16("gram", dims, lo, hi, G, Gx, Ab @ Ab.T)


CASES_PROD = [((64, 48, 40), 0, 0, 16), ((64, 48, 40), 1, 1, 24), ((64, 48, 40), 2, 2, 32), ((30, 20, 18), 2, 2, 5),
              ((16, 16, 16, 16), 2, 3, 48), ((16, 16, 16, 16), 0, 1, 12), ((128, 96, 64), 2, 2, 64),
              ((40, 8, 200), 1, 1, 8)]


@pytest.mark.parametrize("dims,lo,hi,k", CASES_PROD)
@pytest.mark.parametrize("prec", ["fp32", "bf16"])
def test_mode_product(dims, lo, hi, k, prec):
    X = rnd(dims, 11)
    A = O.unfold(X.astype(np.float64), group(dims, lo, hi))   # N x (L*R), columns (l, r) l fastest
    W = rnd((A.shape[0], k), 12)
    Z = ht.mode_product(X, dims, lo, W, hi, precision=prec)
    Zx = A.T @ W.astype(np.float64)
    if prec == "fp32":
        assert rel(Z, Zx) < 1e-5
    else:
        Ab = O.unfold(bf16(X).astype(np.float64), group(dims, lo, hi))
        check_bf16("product", dims, lo, hi, Z, Zx, Ab.T @ bf16(W).astype(np.float64))


@pytest.mark.parametrize("dims,lo,hi,k", CASES_PROD)
@pytest.mark.parametrize("prec", ["fp32", "bf16"])
def test_corange_product(dims, lo, hi, k, prec):
    X = rnd(dims, 21)
    A = O.unfold(X.astype(np.float64), group(dims, lo, hi))
    Q = rnd((A.shape[1], k), 22)
    Z = ht.corange_product(X, dims, lo, Q, hi, precision=prec)
    Zx = A @ Q.astype(np.float64)
    if prec == "fp32":
        assert rel(Z, Zx) < 1e-5
    else:
        Ab = O.unfold(bf16(X).astype(np.float64), group(dims, lo, hi))
        check_bf16("corange", dims, lo, hi, Z, Zx, Ab @ bf16(Q).astype(np.float64))


def test_primitives_accept_device_tensors():
    dims = (64, 32, 48)
    X = rnd(dims, 5)
    xd = torch.from_numpy(np.ascontiguousarray(X.transpose(2, 1, 0))).cuda()
    G = ht.mode_gram(xd, dims, 1, precision="bf16")
    assert G.is_cuda and G.shape == (32, 32)
    Gh = ht.mode_gram(X, dims, 1, precision="bf16")
    np.testing.assert_array_equal(G.cpu().numpy(), Gh)
