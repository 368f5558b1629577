// HT tensor layer: a fully connected layer whose weight is held in HT format.
//
// The reference's layer (HT_tensor_layer/FC_MNIST/mnist_ht.py:232-245 and
// Alex_ImageNet/model/alexnet.py:157-170) maps x[z, n0, n1, n2] to
// y[z, m0, m1, m2] through the einsum chain
//   x u1[n0,m0,r3] -> b2[r3,r4,r1] -> u2[n1,m1,r4] -> b1[r1,r2] -> u3[n2,m2,r2],
// i.e. y = x W^T with
//   W[(m0,m1,m2), (n0,n1,n2)] = sum_{r1} P[a, b, r1] Q[c, r1],
//   P[a, b, r1] = sum_{r3,r4} u1[a, r3] u2[b, r4] b2[r3, r4, r1],   a = n0 M0 + m0, b = n1 M1 + m1
//   Q[c, r1]    = sum_{r2} b1[r1, r2] u3[c, r2],                     c = n2 M2 + m2.
// The chain costs more multiply-adds per sample than the dense product at the
// reference's shapes (rank 16 on 8 x 8 x 16 modes), so here the weight is formed
// once per call from the factors (batch-independent, L2-resident) and the batch
// goes through one GEMM; the kernels in this file form P, Q and W, add the
// bias, and carry the gradients back from dW to the factors.
//
// All parameter tensors use the reference's C-order layouts:
// u_j (N_j, M_j, r_j), b2 (r3, r4, r1), b1 (r1, r2), bias (M0, M1, M2).
#include <cuda_bf16.h>

#include "common.cuh"
#include "engine.h"

namespace htgb {
namespace {

constexpr int kLayerThreads = 256;

int grid_for_layer(long long n) {
  long long g = (n + kLayerThreads - 1) / kLayerThreads;
  if (g > 32ll * device_sm_count()) g = 32ll * device_sm_count();
  return static_cast<int>(g < 1 ? 1 : g);
}

// Blocks [0, A): T1[a] = u1[a, :] b2 (r4 x r1, in shared memory, also written to
// T1g when non-null), then P[a, b, r1] for every b.  Blocks [A, A + qb): Q.
__global__ void __launch_bounds__(kLayerThreads) layer_pq_kernel(const LayerShape sh, const float *__restrict__ u1,
                                                                 const float *__restrict__ u2,
                                                                 const float *__restrict__ u3,
                                                                 const float *__restrict__ b2,
                                                                 const float *__restrict__ b1, float *__restrict__ P,
                                                                 float *__restrict__ Q, float *__restrict__ T1g) {
  __shared__ float T1[kLayerMaxRank * kLayerMaxRank];
  const int A = sh.n[0] * sh.m[0], B = sh.n[1] * sh.m[1], C = sh.n[2] * sh.m[2];
  const int R1 = sh.r1, R2 = sh.r2, R3 = sh.r3, R4 = sh.r4;
  if (static_cast<int>(blockIdx.x) < A) {
    const int a = blockIdx.x;
    for (int e = threadIdx.x; e < R4 * R1; e += kLayerThreads) {
      const int r4 = e / R1, r1 = e - r4 * R1;
      float s = 0.f;
      for (int r3 = 0; r3 < R3; ++r3) s = fmaf(u1[a * R3 + r3], b2[(r3 * R4 + r4) * R1 + r1], s);
      T1[e] = s;
      if (T1g) T1g[static_cast<long long>(a) * R4 * R1 + e] = s;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < B * R1; e += kLayerThreads) {
      const int b = e / R1, r1 = e - b * R1;
      float s = 0.f;
      for (int r4 = 0; r4 < R4; ++r4) s = fmaf(T1[r4 * R1 + r1], u2[b * R4 + r4], s);
      P[(static_cast<long long>(a) * B + b) * R1 + r1] = s;
    }
  } else {
    const long long e = static_cast<long long>(blockIdx.x - A) * kLayerThreads + threadIdx.x;
    if (e >= static_cast<long long>(C) * R1) return;
    const int c = static_cast<int>(e / R1), r1 = static_cast<int>(e - static_cast<long long>(c) * R1);
    float s = 0.f;
    for (int r2 = 0; r2 < R2; ++r2) s = fmaf(b1[r1 * R2 + r2], u3[c * R2 + r2], s);
    Q[e] = s;
  }
}

template <class T>
HT_DEV T from_f32(float v);
template <>
HT_DEV float from_f32<float>(float v) { return v; }
template <>
HT_DEV __nv_bfloat16 from_f32<__nv_bfloat16>(float v) { return __float2bfloat16_rn(v); }

// W[o * Nin + i] = sum_r1 P[a, b, r1] Q[c, r1]; i = (n0 N1 + n1) N2 + n2 runs
// fastest, so consecutive threads share (a, b) and read P's row once.
template <class T>
__global__ void __launch_bounds__(kLayerThreads) layer_weight_kernel(const LayerShape sh, const float *__restrict__ P,
                                                                     const float *__restrict__ Q, T *__restrict__ W) {
  const int N1 = sh.n[1], N2 = sh.n[2], M0 = sh.m[0], M1 = sh.m[1], M2 = sh.m[2];
  const long long Nin = static_cast<long long>(sh.n[0]) * N1 * N2, Nout = static_cast<long long>(M0) * M1 * M2;
  const int B = N1 * M1, R1 = sh.r1;
  for (long long e = blockIdx.x * static_cast<long long>(kLayerThreads) + threadIdx.x; e < Nin * Nout;
       e += static_cast<long long>(gridDim.x) * kLayerThreads) {
    const long long o = e / Nin, i = e - o * Nin;
    const int n2 = static_cast<int>(i % N2), n1 = static_cast<int>((i / N2) % N1), n0 = static_cast<int>(i / N2 / N1);
    const int m2 = static_cast<int>(o % M2), m1 = static_cast<int>((o / M2) % M1), m0 = static_cast<int>(o / M2 / M1);
    const int a = n0 * M0 + m0, b = n1 * M1 + m1, c = n2 * M2 + m2;
    const float *p = P + (static_cast<long long>(a) * B + b) * R1;
    const float *q = Q + static_cast<long long>(c) * R1;
    float s = 0.f;
    for (int r = 0; r < R1; ++r) s = fmaf(p[r], q[r], s);
    W[e] = from_f32<T>(s);
  }
}

// The same W, a block per (m0, m1, group of kWeightG m2 rows): the P slice
// Ps[(n0, n1)][r] = P[n0 M0 + m0, n1 M1 + m1, r] and Qt[r][g][n2] =
// Q[n2 M2 + m2_0 + g, r] sit in shared memory, each thread keeps kWeightG
// accumulators for one input index i and writes kWeightG rows of W, consecutive
// threads on consecutive i (coalesced rows).
constexpr int kWeightG = 8;
template <class T>
__global__ void __launch_bounds__(kLayerThreads) layer_weight_tiled_kernel(const LayerShape sh,
                                                                           const float *__restrict__ P,
                                                                           const float *__restrict__ Q,
                                                                           T *__restrict__ W) {
  extern __shared__ float sm[];
  const int N0 = sh.n[0], N1 = sh.n[1], N2 = sh.n[2], M0 = sh.m[0], M1 = sh.m[1], M2 = sh.m[2];
  const int R1 = sh.r1, B = N1 * M1, NP = N0 * N1;
  const long long Nin = static_cast<long long>(NP) * N2;
  const int groups = (M2 + kWeightG - 1) / kWeightG;
  const int gi = blockIdx.x % groups, mm = blockIdx.x / groups, m1 = mm % M1, m0 = mm / M1;
  const int m2_0 = gi * kWeightG, G = min(kWeightG, M2 - m2_0);
  float *Ps = sm;                                    // NP x R1
  float *Qt = sm + static_cast<size_t>(NP) * R1;     // R1 x kWeightG x N2
  for (int e = threadIdx.x; e < NP * R1; e += kLayerThreads) {
    const int pr = e / R1, r = e - pr * R1, n0 = pr / N1, n1 = pr - n0 * N1;
    Ps[e] = P[(static_cast<long long>(n0 * M0 + m0) * B + (n1 * M1 + m1)) * R1 + r];
  }
  for (int e = threadIdx.x; e < R1 * kWeightG * N2; e += kLayerThreads) {
    const int n2 = e % N2, g = (e / N2) % kWeightG, r = e / (N2 * kWeightG);
    Qt[e] = g < G ? Q[static_cast<long long>(n2 * M2 + m2_0 + g) * R1 + r] : 0.f;
  }
  __syncthreads();
  const long long o0 = (static_cast<long long>(m0) * M1 + m1) * M2 + m2_0;
  for (long long i = threadIdx.x; i < Nin; i += kLayerThreads) {
    const int pr = static_cast<int>(i / N2), n2 = static_cast<int>(i - static_cast<long long>(pr) * N2);
    float acc[kWeightG];
#pragma unroll
    for (int g = 0; g < kWeightG; ++g) acc[g] = 0.f;
    const float *ps = Ps + static_cast<size_t>(pr) * R1;
    for (int r = 0; r < R1; ++r) {
      const float pv = ps[r];
      const float *q = Qt + static_cast<size_t>(r) * kWeightG * N2 + n2;
#pragma unroll
      for (int g = 0; g < kWeightG; ++g) acc[g] = fmaf(pv, q[g * N2], acc[g]);
    }
#pragma unroll
    for (int g = 0; g < kWeightG; ++g)
      if (g < G) W[(o0 + g) * Nin + i] = from_f32<T>(acc[g]);
  }
}

// y[z, o] = act(y[z, o] + bias[o]), act 0 = identity, 1 = ReLU
__global__ void bias_act_kernel(float *__restrict__ y, const float *__restrict__ bias, long long batch, long long nout,
                                int act) {
  for (long long e = blockIdx.x * static_cast<long long>(kLayerThreads) + threadIdx.x; e < batch * nout;
       e += static_cast<long long>(gridDim.x) * kLayerThreads) {
    float v = y[e];
    if (bias) v += bias[e % nout];
    if (act == 1) v = fmaxf(v, 0.f);
    y[e] = v;
  }
}

// dbias[o] = sum_z dy[z, o]: one thread per o, the batch split over blockIdx.y
// partials summed in a fixed order by layer_colsum_finish_kernel.
__global__ void layer_colsum_kernel(const float *__restrict__ dy, long long batch, long long nout, int chunks,
                                    float *__restrict__ part) {
  const long long o = blockIdx.x * static_cast<long long>(kLayerThreads) + threadIdx.x;
  if (o >= nout) return;
  const long long per = (batch + chunks - 1) / chunks;
  const long long z0 = per * blockIdx.y, z1 = min(batch, z0 + per);
  float s = 0.f;
  for (long long z = z0; z < z1; ++z) s += dy[z * nout + o];
  part[static_cast<long long>(blockIdx.y) * nout + o] = s;
}

__global__ void layer_colsum_finish_kernel(const float *__restrict__ part, long long nout, int chunks,
                                           float *__restrict__ out) {
  const long long o = blockIdx.x * static_cast<long long>(kLayerThreads) + threadIdx.x;
  if (o >= nout) return;
  float s = 0.f;
  for (int c = 0; c < chunks; ++c) s += part[static_cast<long long>(c) * nout + o];
  out[o] = s;
}

// dP[a, b, r1] = sum_{n2, m2} dW[o, i] Q[c, r1] and, in the same pass over dW,
// per-(a, b) block contributions to dQ.  One block per (a, b): the M2 x N2
// sub-block of dW it owns is staged in shared memory.
//   dQpart[(a, b), c, r1] is not formed: dQ is summed by layer_dq_kernel.
__global__ void __launch_bounds__(kLayerThreads) layer_dp_kernel(const LayerShape sh, const float *__restrict__ dW,
                                                                 const float *__restrict__ Q, float *__restrict__ dP) {
  extern __shared__ float sm[];
  const int N1 = sh.n[1], N2 = sh.n[2], M0 = sh.m[0], M1 = sh.m[1], M2 = sh.m[2];
  const long long Nin = static_cast<long long>(sh.n[0]) * N1 * N2;
  const int B = N1 * M1, C = N2 * M2, R1 = sh.r1;
  const int ab = blockIdx.x, a = ab / B, b = ab - a * B;
  const int n0 = a / M0, m0 = a - n0 * M0, n1 = b / M1, m1 = b - n1 * M1;
  float *blk = sm;   // [c = n2 M2 + m2]
  for (int e = threadIdx.x; e < C; e += kLayerThreads) {
    const int n2 = e / M2, m2 = e - n2 * M2;
    const long long o = (static_cast<long long>(m0) * M1 + m1) * M2 + m2;
    const long long i = (static_cast<long long>(n0) * N1 + n1) * N2 + n2;
    blk[e] = dW[o * Nin + i];
  }
  __syncthreads();
  for (int r1 = threadIdx.x; r1 < R1; r1 += kLayerThreads) {
    float s = 0.f;
    for (int c = 0; c < C; ++c) s = fmaf(blk[c], Q[static_cast<long long>(c) * R1 + r1], s);
    dP[static_cast<long long>(ab) * R1 + r1] = s;
  }
}

// dQ[c, r1] = sum_{a, b} dW[o, i] P[a, b, r1]: one block per c, the (a, b)
// range split over the threads, a fixed-order tree reduction at the end.
__global__ void __launch_bounds__(kLayerThreads) layer_dq_kernel(const LayerShape sh, const float *__restrict__ dW,
                                                                 const float *__restrict__ P, float *__restrict__ dQ) {
  __shared__ float red[kLayerThreads / 32][kLayerMaxRank];
  const int N1 = sh.n[1], N2 = sh.n[2], M0 = sh.m[0], M1 = sh.m[1], M2 = sh.m[2];
  const long long Nin = static_cast<long long>(sh.n[0]) * N1 * N2;
  const int A = sh.n[0] * M0, B = N1 * M1, R1 = sh.r1;
  const int c = blockIdx.x, n2 = c / M2, m2 = c - n2 * M2;
  float acc[kLayerMaxRank];
#pragma unroll
  for (int r = 0; r < kLayerMaxRank; ++r) acc[r] = 0.f;
  for (int ab = threadIdx.x; ab < A * B; ab += kLayerThreads) {
    const int a = ab / B, b = ab - a * B;
    const int n0 = a / M0, m0 = a - n0 * M0, n1 = b / M1, m1 = b - n1 * M1;
    const long long o = (static_cast<long long>(m0) * M1 + m1) * M2 + m2;
    const long long i = (static_cast<long long>(n0) * N1 + n1) * N2 + n2;
    const float g = dW[o * Nin + i];
    const float *p = P + static_cast<long long>(ab) * R1;
#pragma unroll
    for (int r = 0; r < kLayerMaxRank; ++r)
      if (r < R1) acc[r] = fmaf(g, p[r], acc[r]);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int r = 0; r < kLayerMaxRank; ++r) {
    float v = acc[r];
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    if (lane == 0) red[warp][r] = v;
  }
  __syncthreads();
  for (int r = threadIdx.x; r < R1; r += kLayerThreads) {
    float s = 0.f;
    for (int w = 0; w < kLayerThreads / 32; ++w) s += red[w][r];
    dQ[static_cast<long long>(c) * R1 + r] = s;
  }
}

// dP and per-block dQ partials in one pass over dW, a block per (m0, m1) and
// range of m2 (several ranges give dP partials, summed afterwards): the block
// reads its rows o = (m0 M1 + m1) M2 + m2 of dW (coalesced, staged in
// shared memory with an odd pair stride), and with Q (C x R1) and the P slice
// Ps[(n0, n1)][r] resident accumulates
//   dPs[(n0, n1)][r] += sum_n2 dW[o, (n0, n1, n2)] Q[n2 M2 + m2, r]
//   dQpart[blk][n2 M2 + m2][r] = sum_(n0, n1) dW[o, (n0, n1, n2)] Ps[(n0, n1)][r].
// Every accumulator has one owning thread, so the sums are deterministic.
__global__ void __launch_bounds__(kLayerThreads) layer_dpq_kernel(const LayerShape sh, const float *__restrict__ dW,
                                                                  const float *__restrict__ P,
                                                                  const float *__restrict__ Q,
                                                                  float *__restrict__ dP,
                                                                  float *__restrict__ dQpart) {
  extern __shared__ float sm[];
  const int N0 = sh.n[0], N1 = sh.n[1], N2 = sh.n[2], M0 = sh.m[0], M1 = sh.m[1], M2 = sh.m[2];
  const int R1 = sh.r1, B = N1 * M1, NP = N0 * N1, C = N2 * M2;
  const int rs = N2 | 1;                             // odd stride between pairs: conflict-free column reads
  const long long Nin = static_cast<long long>(NP) * N2;
  const int chunks = gridDim.x / (M0 * M1);          // m2 ranges per (m0, m1): dP partials per range
  const int blk = blockIdx.x / chunks, ch = blockIdx.x - blk * chunks, m1 = blk % M1, m0 = blk / M1;
  const int mg = (M2 + chunks - 1) / chunks, m2_lo = ch * mg, m2_hi = min(M2, m2_lo + mg);
  float *row = sm;                                   // NP x rs
  float *Qs = row + static_cast<size_t>(NP) * rs;    // C x R1
  float *Ps = Qs + static_cast<size_t>(C) * R1;      // NP x R1
  float *dPs = Ps + static_cast<size_t>(NP) * R1;    // NP x R1
  for (int e = threadIdx.x; e < C * R1; e += kLayerThreads) Qs[e] = Q[e];
  for (int e = threadIdx.x; e < NP * R1; e += kLayerThreads) {
    const int pr = e / R1, r = e - pr * R1, n0 = pr / N1, n1 = pr - n0 * N1;
    Ps[e] = P[(static_cast<long long>(n0 * M0 + m0) * B + (n1 * M1 + m1)) * R1 + r];
    dPs[e] = 0.f;
  }
  for (int m2 = m2_lo; m2 < m2_hi; ++m2) {
    __syncthreads();   // previous row fully consumed (and Qs / Ps written on the first pass)
    const float *src = dW + ((static_cast<long long>(m0) * M1 + m1) * M2 + m2) * Nin;
    for (long long i = threadIdx.x; i < Nin; i += kLayerThreads) {
      const int pr = static_cast<int>(i / N2), n2 = static_cast<int>(i - static_cast<long long>(pr) * N2);
      row[pr * rs + n2] = src[i];
    }
    __syncthreads();
    for (int e = threadIdx.x; e < NP * R1; e += kLayerThreads) {
      const int pr = e / R1, r = e - pr * R1;
      const float *rw = row + pr * rs;
      float s = dPs[e];
      for (int n2 = 0; n2 < N2; ++n2) s = fmaf(rw[n2], Qs[(n2 * M2 + m2) * R1 + r], s);
      dPs[e] = s;
    }
    for (int e = threadIdx.x; e < N2 * R1; e += kLayerThreads) {
      const int r = e / N2, n2 = e - r * N2;
      float s[4] = {0.f, 0.f, 0.f, 0.f};   // four independent chains, combined in a fixed order
      int pr = 0;
      for (; pr + 4 <= NP; pr += 4)
#pragma unroll
        for (int j = 0; j < 4; ++j) s[j] = fmaf(row[(pr + j) * rs + n2], Ps[(pr + j) * R1 + r], s[j]);
      for (; pr < NP; ++pr) s[0] = fmaf(row[pr * rs + n2], Ps[pr * R1 + r], s[0]);
      dQpart[(static_cast<long long>(blk) * C + (n2 * M2 + m2)) * R1 + r] = (s[0] + s[1]) + (s[2] + s[3]);
    }
  }
  __syncthreads();
  // chunks > 1: dP points at the partial buffer [chunks][A B R1]
  float *dPo = dP + static_cast<long long>(ch) * (static_cast<long long>(sh.n[0]) * M0 * B * R1);
  for (int e = threadIdx.x; e < NP * R1; e += kLayerThreads) {
    const int pr = e / R1, r = e - pr * R1, n0 = pr / N1, n1 = pr - n0 * N1;
    dPo[(static_cast<long long>(n0 * M0 + m0) * B + (n1 * M1 + m1)) * R1 + r] = dPs[e];
  }
}

// dQ[c, r] = sum over the (m0, m1) blocks of dQpart, in block order.
__global__ void layer_dq_reduce_kernel(const float *__restrict__ dQpart, int blocks, long long count,
                                       float *__restrict__ dQ) {
  const long long e = blockIdx.x * static_cast<long long>(kLayerThreads) + threadIdx.x;
  if (e >= count) return;
  float s[4] = {0.f, 0.f, 0.f, 0.f};   // four independent chains, combined in a fixed order
  int b = 0;
  for (; b + 4 <= blocks; b += 4)
#pragma unroll
    for (int q = 0; q < 4; ++q) s[q] += dQpart[static_cast<long long>(b + q) * count + e];
  for (; b < blocks; ++b) s[0] += dQpart[static_cast<long long>(b) * count + e];
  dQ[e] = (s[0] + s[1]) + (s[2] + s[3]);
}

// dT1[a, r4, r1] = sum_b u2[b, r4] dP[a, b, r1]: a block per a, the b range
// staged through shared memory in chunks of kDtChunk rows of dP[a] and u2,
// each thread owning fixed (r4, r1) outputs.  Blocks [A, A + du3 blocks):
// du3[c, r2] = sum_r1 dQ[c, r1] b1[r1, r2], a thread per entry.
constexpr int kDtChunk = 64;
__global__ void __launch_bounds__(kLayerThreads) layer_dt1_kernel(const LayerShape sh, const float *__restrict__ u2,
                                                                  const float *__restrict__ b1,
                                                                  const float *__restrict__ dP,
                                                                  const float *__restrict__ dQ,
                                                                  float *__restrict__ dT1, float *__restrict__ du3) {
  const int A = sh.n[0] * sh.m[0], B = sh.n[1] * sh.m[1], C = sh.n[2] * sh.m[2];
  const int R1 = sh.r1, R2 = sh.r2, R4 = sh.r4, t = threadIdx.x;
  if (static_cast<int>(blockIdx.x) >= A) {
    const long long f = (blockIdx.x - A) * static_cast<long long>(kLayerThreads) + t;
    if (f >= static_cast<long long>(C) * R2) return;
    const int c = static_cast<int>(f / R2), r2 = static_cast<int>(f - static_cast<long long>(c) * R2);
    float v = 0.f;
    for (int r1 = 0; r1 < R1; ++r1) v = fmaf(dQ[static_cast<long long>(c) * R1 + r1], b1[r1 * R2 + r2], v);
    du3[f] = v;
    return;
  }
  __shared__ float sP[kDtChunk * kLayerMaxRank];   // [b][r1]
  __shared__ float sU[kDtChunk * kLayerMaxRank];   // [b][r4]
  constexpr int kOut = kLayerMaxRank * kLayerMaxRank / kLayerThreads;
  const int a = blockIdx.x, nout = R4 * R1;
  float acc[kOut];
#pragma unroll
  for (int q = 0; q < kOut; ++q) acc[q] = 0.f;
  for (int b0 = 0; b0 < B; b0 += kDtChunk) {
    const int nb = min(kDtChunk, B - b0);
    __syncthreads();
    for (int e = t; e < nb * R1; e += kLayerThreads) sP[e] = dP[(static_cast<long long>(a) * B + b0) * R1 + e];
    for (int e = t; e < nb * R4; e += kLayerThreads) sU[e] = u2[static_cast<long long>(b0) * R4 + e];
    __syncthreads();
#pragma unroll
    for (int q = 0; q < kOut; ++q) {
      const int o = t + q * kLayerThreads;
      if (o < nout) {
        const int r4 = o / R1, r1 = o - r4 * R1;
        float v = acc[q];
        for (int b = 0; b < nb; ++b) v = fmaf(sU[b * R4 + r4], sP[b * R1 + r1], v);
        acc[q] = v;
      }
    }
  }
#pragma unroll
  for (int q = 0; q < kOut; ++q) {
    const int o = t + q * kLayerThreads;
    if (o < nout) dT1[static_cast<long long>(a) * nout + o] = acc[q];
  }
}

// du1[a, r3] = sum_q dT1[a, q] b2[r3, q] (q = (r4, r1)): a warp per entry,
// lanes striding q, a fixed shuffle tree.  Blocks past the du1 ones:
// db2[r3, q] = sum_a u1[a, r3] dT1[a, q], a thread per entry with four
// independent chains over a combined in a fixed order.
__global__ void __launch_bounds__(kLayerThreads) layer_dt1_back_kernel(const LayerShape sh, const float *__restrict__ u1,
                                                                       const float *__restrict__ b2,
                                                                       const float *__restrict__ dT1,
                                                                       float *__restrict__ du1,
                                                                       float *__restrict__ db2, int du1_blocks) {
  const int A = sh.n[0] * sh.m[0];
  const int R1 = sh.r1, R3 = sh.r3, R4 = sh.r4, Qn = R4 * R1;
  if (static_cast<int>(blockIdx.x) < du1_blocks) {
    const long long w = blockIdx.x * static_cast<long long>(kLayerThreads / 32) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (w >= static_cast<long long>(A) * R3) return;
    const int a = static_cast<int>(w / R3), r3 = static_cast<int>(w - static_cast<long long>(a) * R3);
    const float *d = dT1 + static_cast<long long>(a) * Qn;
    const float *g = b2 + static_cast<long long>(r3) * Qn;
    float v = 0.f;
    for (int q = lane; q < Qn; q += 32) v = fmaf(d[q], g[q], v);
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    if (lane == 0) du1[w] = v;
    return;
  }
  const long long f = (blockIdx.x - du1_blocks) * static_cast<long long>(kLayerThreads) + threadIdx.x;
  if (f >= static_cast<long long>(R3) * Qn) return;
  const int r3 = static_cast<int>(f / Qn), q = static_cast<int>(f - static_cast<long long>(r3) * Qn);
  float s[4] = {0.f, 0.f, 0.f, 0.f};
  int a = 0;
  for (; a + 4 <= A; a += 4)
#pragma unroll
    for (int j = 0; j < 4; ++j) s[j] = fmaf(u1[(a + j) * R3 + r3], dT1[static_cast<long long>(a + j) * Qn + q], s[j]);
  for (; a < A; ++a) s[0] = fmaf(u1[a * R3 + r3], dT1[static_cast<long long>(a) * Qn + q], s[0]);
  db2[f] = (s[0] + s[1]) + (s[2] + s[3]);
}

// The factor gradients from dP, dQ (all small):
//   du3[c, r2] = sum_r1 dQ[c, r1] b1[r1, r2]        db1[r1, r2] = sum_c dQ[c, r1] u3[c, r2]
//   dT1[a, r4, r1] = sum_b dP[a, b, r1] u2[b, r4]   du2[b, r4] = sum_{a, r1} dP[a, b, r1] T1[a, r4, r1]
//   du1[a, r3] = sum_{r4, r1} dT1[a, r4, r1] b2[r3, r4, r1]
//   db2[r3, r4, r1] = sum_a u1[a, r3] dT1[a, r4, r1]
// dT1 and du3 come from layer_dt1_kernel, du1 and db2 from
// layer_dt1_back_kernel, du2 and db1 from the two kernels below.
// du2[b, r4] = sum_{a, r1} dP[a, b, r1] T1[a, r4, r1]: a block per b, the
// (a, r1) pairs split over the threads with R4 accumulators each, then a
// fixed-order reduction (deterministic).
template <int RB>   // rank bound: R4 <= RB
__global__ void __launch_bounds__(kLayerThreads) layer_du2_kernel(const LayerShape sh, const float *__restrict__ dP,
                                                                  const float *__restrict__ T1, float *__restrict__ du2) {
  __shared__ float red[kLayerThreads / 32][RB];
  const int A = sh.n[0] * sh.m[0], B = sh.n[1] * sh.m[1];
  const int R1 = sh.r1, R4 = sh.r4, b = blockIdx.x;
  float acc[RB];
#pragma unroll
  for (int r = 0; r < RB; ++r) acc[r] = 0.f;
  for (int e = threadIdx.x; e < A * R1; e += kLayerThreads) {
    const int a = e / R1, r1 = e - a * R1;
    const float g = dP[(static_cast<long long>(a) * B + b) * R1 + r1];
    const float *t = T1 + static_cast<long long>(a) * R4 * R1 + r1;
#pragma unroll
    for (int r = 0; r < RB; ++r)
      if (r < R4) acc[r] = fmaf(g, t[r * R1], acc[r]);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int r = 0; r < RB; ++r) {
    float v = acc[r];
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    if (lane == 0) red[warp][r] = v;
  }
  __syncthreads();
  for (int r = threadIdx.x; r < R4; r += kLayerThreads) {
    float v = 0.f;
    for (int w = 0; w < kLayerThreads / 32; ++w) v += red[w][r];
    du2[static_cast<long long>(b) * R4 + r] = v;
  }
}

// db1[r1, r2] = sum_c dQ[c, r1] u3[c, r2]: a block per r1, c split over the
// threads with R2 accumulators each, fixed-order reduction.
template <int RB>   // rank bound: R2 <= RB
__global__ void __launch_bounds__(kLayerThreads) layer_db1_kernel(const LayerShape sh, const float *__restrict__ dQ,
                                                                  const float *__restrict__ u3, float *__restrict__ db1) {
  __shared__ float red[kLayerThreads / 32][RB];
  const int C = sh.n[2] * sh.m[2], R1 = sh.r1, R2 = sh.r2, r1 = blockIdx.x;
  float acc[RB];
#pragma unroll
  for (int r = 0; r < RB; ++r) acc[r] = 0.f;
  for (int c = threadIdx.x; c < C; c += kLayerThreads) {
    const float g = dQ[static_cast<long long>(c) * R1 + r1];
    const float *u = u3 + static_cast<long long>(c) * R2;
#pragma unroll
    for (int r = 0; r < RB; ++r)
      if (r < R2) acc[r] = fmaf(g, u[r], acc[r]);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int r = 0; r < RB; ++r) {
    float v = acc[r];
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    if (lane == 0) red[warp][r] = v;
  }
  __syncthreads();
  for (int r = threadIdx.x; r < R2; r += kLayerThreads) {
    float v = 0.f;
    for (int w = 0; w < kLayerThreads / 32; ++w) v += red[w][r];
    db1[static_cast<long long>(r1) * R2 + r] = v;
  }
}

}  // namespace

cudaError_t layer_pq_launch(const LayerShape &sh, const float *u1, const float *u2, const float *u3, const float *b2,
                            const float *b1, float *P, float *Q, float *T1, cudaStream_t s) {
  const int A = sh.n[0] * sh.m[0], C = sh.n[2] * sh.m[2];
  const long long qb = (static_cast<long long>(C) * sh.r1 + kLayerThreads - 1) / kLayerThreads;
  layer_pq_kernel<<<static_cast<unsigned>(A + qb), kLayerThreads, 0, s>>>(sh, u1, u2, u3, b2, b1, P, Q, T1);
  return cudaGetLastError();
}

size_t layer_weight_smem(const LayerShape &sh) {
  return sizeof(float) * (static_cast<size_t>(sh.n[0]) * sh.n[1] * sh.r1 +
                          static_cast<size_t>(sh.r1) * kWeightG * sh.n[2]);
}

size_t layer_dpq_smem(const LayerShape &sh) {
  const size_t NP = static_cast<size_t>(sh.n[0]) * sh.n[1], C = static_cast<size_t>(sh.n[2]) * sh.m[2];
  return sizeof(float) * (NP * (sh.n[2] | 1) + C * sh.r1 + 2 * NP * sh.r1);
}

constexpr size_t kLayerSmemMax = 200 * 1024;

template <class K>
cudaError_t allow_smem(K kernel, size_t bytes) {
  if (bytes <= 48 * 1024) return cudaSuccess;
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(bytes));
}

cudaError_t layer_weight_launch(const LayerShape &sh, const float *P, const float *Q, float *W32, __nv_bfloat16 *W16,
                                cudaStream_t s) {
  const long long total = static_cast<long long>(sh.n[0]) * sh.n[1] * sh.n[2] * sh.m[0] * sh.m[1] * sh.m[2];
  const size_t smem = layer_weight_smem(sh);
  if (smem <= kLayerSmemMax) {
    const unsigned grid =
        static_cast<unsigned>(sh.m[0]) * sh.m[1] * ((sh.m[2] + kWeightG - 1) / kWeightG);
    cudaError_t e;
    if (W32) {
      if ((e = allow_smem(layer_weight_tiled_kernel<float>, smem)) != cudaSuccess) return e;
      layer_weight_tiled_kernel<float><<<grid, kLayerThreads, smem, s>>>(sh, P, Q, W32);
    } else {
      if ((e = allow_smem(layer_weight_tiled_kernel<__nv_bfloat16>, smem)) != cudaSuccess) return e;
      layer_weight_tiled_kernel<__nv_bfloat16><<<grid, kLayerThreads, smem, s>>>(sh, P, Q, W16);
    }
    return cudaGetLastError();
  }
  if (W32) layer_weight_kernel<float><<<grid_for_layer(total), kLayerThreads, 0, s>>>(sh, P, Q, W32);
  else layer_weight_kernel<__nv_bfloat16><<<grid_for_layer(total), kLayerThreads, 0, s>>>(sh, P, Q, W16);
  return cudaGetLastError();
}

cudaError_t bias_act_launch(float *y, const float *bias, long long batch, long long nout, int act, cudaStream_t s) {
  bias_act_kernel<<<grid_for_layer(batch * nout), kLayerThreads, 0, s>>>(y, bias, batch, nout, act);
  return cudaGetLastError();
}

int layer_colsum_chunks(long long batch) {
  long long c = (batch + 15) / 16;   // at most 16 rows of dy per thread at small batch
  if (c < 1) c = 1;
  if (c > 64) c = 64;
  return static_cast<int>(c);
}

cudaError_t layer_colsum_launch(const float *dy, long long batch, long long nout, float *part, float *out,
                                cudaStream_t s) {
  const int chunks = layer_colsum_chunks(batch);
  const unsigned gx = static_cast<unsigned>((nout + kLayerThreads - 1) / kLayerThreads);
  layer_colsum_kernel<<<dim3(gx, chunks), kLayerThreads, 0, s>>>(dy, batch, nout, chunks, part);
  layer_colsum_finish_kernel<<<gx, kLayerThreads, 0, s>>>(part, nout, chunks, out);
  return cudaGetLastError();
}

int layer_dpq_chunks(const LayerShape &sh) {
  const int blocks = sh.m[0] * sh.m[1];
  int ch = (2 * device_sm_count() + blocks - 1) / blocks;
  return ch < 1 ? 1 : (ch > sh.m[2] ? sh.m[2] : ch);
}

size_t layer_dq_part_count(const LayerShape &sh) {
  if (layer_dpq_smem(sh) > kLayerSmemMax) return 0;
  const size_t dq = static_cast<size_t>(sh.m[0]) * sh.m[1] * sh.n[2] * sh.m[2] * sh.r1;
  const int ch = layer_dpq_chunks(sh);
  const size_t dp = ch > 1 ? static_cast<size_t>(ch) * sh.n[0] * sh.m[0] * sh.n[1] * sh.m[1] * sh.r1 : 0;
  return dq + dp;   // dQ partials, then dP partials
}

cudaError_t layer_factor_grads_launch(const LayerShape &sh, const float *dW, const float *u1, const float *u2,
                                      const float *u3, const float *b2, const float *b1, const float *P,
                                      const float *Q, const float *T1, float *dP, float *dQ, float *dT1, float *dQpart,
                                      float *du1, float *du2, float *du3, float *db2, float *db1, cudaStream_t s) {
  const int A = sh.n[0] * sh.m[0], B = sh.n[1] * sh.m[1], C = sh.n[2] * sh.m[2];
  const size_t smem_dpq = layer_dpq_smem(sh);
  if (smem_dpq <= kLayerSmemMax && dQpart) {
    cudaError_t e = allow_smem(layer_dpq_kernel, smem_dpq);
    if (e != cudaSuccess) return e;
    const int blocks = sh.m[0] * sh.m[1], ch = layer_dpq_chunks(sh);
    float *dPpart = dQpart + static_cast<size_t>(blocks) * C * sh.r1;
    layer_dpq_kernel<<<static_cast<unsigned>(blocks * ch), kLayerThreads, smem_dpq, s>>>(sh, dW, P, Q,
                                                                                         ch > 1 ? dPpart : dP, dQpart);
    const long long cnt = static_cast<long long>(C) * sh.r1;
    layer_dq_reduce_kernel<<<static_cast<unsigned>((cnt + kLayerThreads - 1) / kLayerThreads), kLayerThreads, 0, s>>>(
        dQpart, blocks, cnt, dQ);
    if (ch > 1) {
      const long long pc = static_cast<long long>(A) * B * sh.r1;
      layer_dq_reduce_kernel<<<static_cast<unsigned>((pc + kLayerThreads - 1) / kLayerThreads), kLayerThreads, 0,
                               s>>>(dPpart, ch, pc, dP);
    }
  } else {
    const size_t smem = sizeof(float) * static_cast<size_t>(C);
    if (smem > 48 * 1024) return cudaErrorInvalidValue;
    layer_dp_kernel<<<static_cast<unsigned>(A * B), kLayerThreads, smem, s>>>(sh, dW, Q, dP);
    layer_dq_kernel<<<static_cast<unsigned>(C), kLayerThreads, 0, s>>>(sh, dW, P, dQ);
  }
  const long long du3_blocks = (static_cast<long long>(C) * sh.r2 + kLayerThreads - 1) / kLayerThreads;
  layer_dt1_kernel<<<static_cast<unsigned>(A + du3_blocks), kLayerThreads, 0, s>>>(sh, u2, b1, dP, dQ, dT1, du3);
  if (sh.r4 <= 16) layer_du2_kernel<16><<<static_cast<unsigned>(B), kLayerThreads, 0, s>>>(sh, dP, T1, du2);
  else if (sh.r4 <= 32) layer_du2_kernel<32><<<static_cast<unsigned>(B), kLayerThreads, 0, s>>>(sh, dP, T1, du2);
  else layer_du2_kernel<kLayerMaxRank><<<static_cast<unsigned>(B), kLayerThreads, 0, s>>>(sh, dP, T1, du2);
  if (sh.r2 <= 16) layer_db1_kernel<16><<<static_cast<unsigned>(sh.r1), kLayerThreads, 0, s>>>(sh, dQ, u3, db1);
  else if (sh.r2 <= 32) layer_db1_kernel<32><<<static_cast<unsigned>(sh.r1), kLayerThreads, 0, s>>>(sh, dQ, u3, db1);
  else layer_db1_kernel<kLayerMaxRank><<<static_cast<unsigned>(sh.r1), kLayerThreads, 0, s>>>(sh, dQ, u3, db1);
  const long long du1_blocks = (static_cast<long long>(A) * sh.r3 + kLayerThreads / 32 - 1) / (kLayerThreads / 32);
  const long long db2_blocks =
      (static_cast<long long>(sh.r3) * sh.r4 * sh.r1 + kLayerThreads - 1) / kLayerThreads;
  layer_dt1_back_kernel<<<static_cast<unsigned>(du1_blocks + db2_blocks), kLayerThreads, 0, s>>>(
      sh, u1, b2, dT1, du1, db2, static_cast<int>(du1_blocks));
  return cudaGetLastError();
}

}  // namespace htgb
