"""HT tensor layer on the GPU against the reference's einsum chain
(HT_tensor_layer/FC_MNIST/mnist_ht.py:233-241, restated in the oracle in
float64) and, for gradients, against float64 autograd of that chain.

Tolerances (relative Frobenius error against float64):
  FP32 products   forward 1e-5, weight 1e-5, gradients 1e-4
  BF16 products   forward 1e-2 against the float64 chain on the FP32 operands;
                  gradients 1e-4 (dx 2e-4) against float64 on the BF16-rounded
                  operands the products consume (BF16 operands, FP32 sums)
  ht_init         weight from our factors vs the oracle's ht(): 1e-4 on an
                  input with a clear spectral gap
"""
import numpy as np
import pytest
import torch

from ht_tensor_learning_using_gpu_tensor_cores_gb300 import htlayer, synth
from ht_tensor_learning_using_gpu_tensor_cores_gb300._lib import HTError
import ht_oracle as O

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


def factors(N, M, r, seed):
    """r = (r_u1, r_u2, r_u3, r_b2); scaled so that y has entries of order one."""
    g = torch.Generator().manual_seed(seed)
    mk = lambda *s: torch.randn(*s, generator=g, dtype=torch.float64) / np.sqrt(s[0] * s[-1])
    return [mk(N[0], M[0], r[0]), mk(N[1], M[1], r[1]), mk(N[2], M[2], r[2]), mk(r[0], r[1], r[3]),
            mk(r[3], r[2])]


def cuda32(ts):
    return [t.to(device="cuda", dtype=torch.float32).contiguous() for t in ts]


SHAPES = [
    ((8, 8, 16), (8, 8, 16), (16, 16, 16, 16), 128),      # the MNIST layer, tNet fc1 (mnist_ht.py:202)
    ((16, 16, 25), (16, 16, 16), (8, 8, 8, 8), 64),      # the AlexNet layer 1 modes (alexnet.py:141-146)
    ((3, 5, 7), (2, 3, 4), (2, 3, 4, 5), 33),             # ragged modes and ranks
    ((4, 2, 8), (8, 4, 2), (1, 2, 3, 1), 1),              # rank one, batch one
]


@pytest.mark.parametrize("N,M,r,batch", SHAPES)
def test_forward_fp32_matches_chain(N, M, r, batch):
    f64 = factors(N, M, r, seed=batch)
    g = torch.Generator().manual_seed(500 + batch)
    bias = torch.randn(M[0], M[1], M[2], dtype=torch.float64, generator=g)
    x = torch.randn(batch, int(np.prod(N)), dtype=torch.float64, generator=g)
    want = O.ht_layer_chain(x.numpy(), *[t.numpy() for t in f64], bias=bias.numpy())
    f = cuda32(f64)
    y = htlayer.layer_forward(x.float().cuda(), *f, bias=bias.float().cuda())
    assert y.shape == (batch, int(np.prod(M)))
    assert rel(y.cpu().numpy(), want) <= 1e-5
    yr = htlayer.layer_forward(x.float().cuda(), *f, bias=bias.float().cuda(), relu=True)
    assert rel(yr.cpu().numpy(), np.maximum(want, 0.0)) <= 1e-5
    W = htlayer.layer_weight(*f)
    assert rel(W.cpu().numpy(), O.ht_layer_weight(*[t.numpy() for t in f64])) <= 1e-5


@pytest.mark.parametrize("N,M,r,batch", [s for s in SHAPES if np.prod(s[0]) % 8 == 0 and np.prod(s[1]) % 8 == 0])
def test_forward_bf16(N, M, r, batch):
    f64 = factors(N, M, r, seed=batch + 1)
    x = torch.randn(batch, int(np.prod(N)), dtype=torch.float64, generator=torch.Generator().manual_seed(600 + batch))
    want = O.ht_layer_chain(x.numpy(), *[t.numpy() for t in f64])
    y = htlayer.layer_forward(x.float().cuda(), *cuda32(f64), precision="bf16")
    assert rel(y.cpu().numpy(), want) <= 1e-2


def test_bf16_rejects_unaligned_modes():
    f = cuda32(factors((3, 5, 7), (2, 3, 4), (2, 3, 4, 5), 0))
    with pytest.raises(HTError, match="divisible by 8"):
        htlayer.layer_forward(torch.zeros(2, 105, device="cuda"), *f, precision="bf16")


def test_rejects_host_tensors_and_bad_ranks():
    f = cuda32(factors((4, 4, 4), (4, 4, 4), (2, 2, 2, 2), 0))
    with pytest.raises(TypeError):
        htlayer.layer_forward(torch.zeros(2, 64), *f)
    big = cuda32(factors((4, 4, 4), (4, 4, 4), (65, 2, 2, 2), 0))
    with pytest.raises(HTError, match="ranks"):
        htlayer.layer_forward(torch.zeros(2, 64, device="cuda"), *big)


def chain_grads(x, f64, bias, dy):
    """float64 autograd of the reference chain (torch on the CPU)."""
    xs = x.clone().requires_grad_(True)
    ps = [t.clone().requires_grad_(True) for t in f64]
    bs = bias.clone().requires_grad_(True)
    t = xs.reshape(x.shape[0], ps[0].shape[0], ps[1].shape[0], ps[2].shape[0])
    t = torch.einsum("zabc,ade->zbcde", t, ps[0])
    t = torch.einsum("zabcd,def->zabcef", t, ps[3])
    t = torch.einsum("zabcde,afd->zbcef", t, ps[1])
    t = torch.einsum("zabcd,ce->zabde", t, ps[4])
    t = torch.einsum("zabcd,aed->zbce", t, ps[2])
    y = (t + bs).reshape(x.shape[0], -1)
    (y * dy).sum().backward()
    return xs.grad, [p.grad for p in ps], bs.grad


def bf16_round(t):
    """float64 copy of t rounded to BF16 (what the tcgen05 products consume)."""
    return t.to(torch.float32).to(torch.bfloat16).to(torch.float64)


@pytest.mark.parametrize("N,M,r,batch", SHAPES)
@pytest.mark.parametrize("prec", ["fp32", "bf16"])
def test_backward_matches_autograd(N, M, r, batch, prec):
    """FP32 path against float64 autograd of the chain.  BF16 path: its products
    consume bf16(x), bf16(dy) and bf16(W) and sum in FP32, so it is compared
    with float64 on exactly those operands: dx = bf16(dy) bf16(W), the factor
    gradients from the chain at bf16(x), bf16(dy).  What remains is FP32
    rounding, hence the same bars as the FP32 path (a flat BF16 tolerance
    cannot hold where a gradient is a short sum with cancellation)."""
    if prec == "bf16" and (np.prod(N) % 8 or np.prod(M) % 8):
        pytest.skip("BF16 products need mode products divisible by 8")
    g = torch.Generator().manual_seed(1000 + 7 * batch + (1 if prec == "bf16" else 0))
    f64 = [t.float().double() for t in factors(N, M, r, seed=3 * batch)]   # the FP32 factors the GPU gets
    bias = torch.randn(M[0], M[1], M[2], dtype=torch.float64, generator=g)
    x = torch.randn(batch, int(np.prod(N)), dtype=torch.float64, generator=g).float().double()
    dy = torch.randn(batch, int(np.prod(M)), dtype=torch.float64, generator=g).float().double()
    if prec == "fp32":
        gx, gf, gb = chain_grads(x, f64, bias, dy)
    else:
        _, gf, gb = chain_grads(bf16_round(x), f64, bias, bf16_round(dy))
        W = torch.from_numpy(O.ht_layer_weight(*[t.numpy() for t in f64]))
        gx = bf16_round(dy) @ bf16_round(W)
    dx, *gr, dbias = htlayer.layer_backward(x.float().cuda(), dy.float().cuda(), *cuda32(f64), precision=prec)
    assert rel(dx.cpu().numpy(), gx.numpy()) <= (1e-4 if prec == "fp32" else 2e-4)
    for name, got, want in zip(("u1", "u2", "u3", "b2", "b1"), gr, gf):
        assert got.shape == want.shape
        assert rel(got.cpu().numpy(), want.numpy()) <= 1e-4, name
    # dbias = column sums of the FP32 dy on both paths
    assert rel(dbias.cpu().numpy(), dy.sum(0).numpy()) <= 1e-5
    if prec == "fp32":
        assert rel(dbias.cpu().numpy(), gb.reshape(-1).numpy()) <= 1e-5


def test_autograd_module_trains():
    """HTLinear through torch autograd: the gradients of a loss reach every
    factor and an Adam loop fits a target HT layer."""
    torch.manual_seed(0)
    N, M, r = (4, 4, 8), (4, 4, 8), 4
    target = htlayer.HTLinear(N, M, r)
    layer = htlayer.HTLinear(N, M, r)
    opt = torch.optim.Adam(layer.parameters(), lr=1e-2)
    x = torch.randn(256, 128, device="cuda")
    with torch.no_grad():
        yt = target(x)
    first = None
    for _ in range(300):
        opt.zero_grad()
        loss = ((layer(x) - yt) ** 2).mean()
        loss.backward()
        if first is None:
            first = float(loss.detach())
            assert all(p.grad is not None and torch.isfinite(p.grad).all() for p in layer.parameters())
        opt.step()
    assert loss.item() < 0.05 * first


def test_ht_init_matches_reference_init():
    """ht_init (the GPU decomposition) and the oracle's ht() give the same layer
    weight on a weight whose reshaped tensor has HT rank 16 plus noise."""
    N, M, rank = (8, 8, 16), (8, 8, 16), 16
    a, b, c = N[0] * M[0], N[1] * M[1], N[2] * M[2]
    from ht_tensor_learning_using_gpu_tensor_cores_gb300 import left_first_tree_3d
    # column-major (c, b, a) = C-order (a, b, c); the tree {c}, {b, a} is ht()'s tree
    tree = left_first_tree_3d([1, rank, rank, rank, rank])
    T = synth.exact_ht((c, b, a), tree, noise_rel=1e-3, seed=4)
    w = np.ascontiguousarray(T.transpose(2, 1, 0)).reshape(a * b * c // 1024, 1024)
    ours = htlayer.ht_init(torch.from_numpy(w).cuda(), rank, N, M)
    ref = O.ht_layer_init(w, rank, N, M)
    for got, want in zip(ours, ref):
        assert tuple(got.shape) == want.shape
    Wo = htlayer.layer_weight(*ours).cpu().numpy()
    Wr = O.ht_layer_weight(*ref)
    assert rel(Wo, Wr) <= 1e-4
    # the factors have orthonormal columns, as the reference's do
    for u in ours[:3]:
        m = u.reshape(-1, rank).double()
        assert torch.allclose(m.T @ m, torch.eye(rank, dtype=torch.float64, device="cuda"), atol=1e-5)
