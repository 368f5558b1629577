// Householder TSQR: the R factor of a tall-skinny FP32 matrix A (m x k,
// k <= 64, column-major), all row blocks in one launch.
//
// Replaces the reference's tsqr_svd / tsqr_svd_half
// (third_order_tensor_decompsition/CUDA/TSQR/kernel.cu:500-949), which splits
// the n^2 x n unfolding into four row blocks on the host, QR-factors each with
// cuSOLVER (geqrf, kernel.cu:326-350), stacks the four R factors and factors
// them again.  Here:
//   * every warp owns a k x k R in shared memory and folds 64-row panels of A
//     into it with Householder reflections on [R; panel] (rows held two per
//     lane, column norms and the reflector-column dot products as warp-shuffle
//     reductions); the reflector of column j touches only row j of R and the
//     panel, because R is upper triangular;
//   * the warps' R factors are combined in a shared-memory binary tree (each
//     partner's R is the next panel);
//   * the CTAs' R factors are combined in a tree of fan-in 8 across the grid:
//     the last CTA of a group to finish (an atomic counter, no waiting) loads
//     the group's R factors and combines them, until one remains.  No CTA ever
//     waits for another, so the launch needs no co-residency.
// The result has a non-negative diagonal (R's rows take the sign of their
// pivot); optionally R^T R is formed in compensated FP32.
#include "common.cuh"
#include "engine.h"

namespace htgb {
namespace {

constexpr int TQ_PROWS = 64;   // rows of a panel (two per lane)
constexpr int TQ_FAN = 8;      // fan-in of the cross-CTA tree

template <int KM>
struct TqCfg {
  static constexpr int WARPS = KM == 32 ? 8 : 4;
  static constexpr int THREADS = WARPS * 32;
  static constexpr int LD = KM + 1;                                  // row stride (floats): conflict-free rows
  static constexpr int WARP_FLOATS = (KM + TQ_PROWS) * LD;           // R (KM rows) + panel (64 rows)
  static constexpr size_t SMEM = size_t(WARPS) * WARP_FLOATS * sizeof(float);
  static constexpr int RPL = KM == 32 ? 4 : 2;                       // panel rows per lane in the main loop
  static constexpr int PANEL = 32 * RPL;                             // main-loop panel height
};

// Sum over the warp, the same value in every lane (lane 0's reduction order).
HT_DEV float warp_sum_bcast(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return __shfl_sync(0xffffffffu, v, 0);
}

// Sum of v[i] over the warp for 32 columns i at once (reduce-scatter): lane l
// returns the total of column l.  31 shuffles, all independent per level.
HT_DEV float warp_reduce_scatter32(float (&v)[32]) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) {
    const bool up = (lane & o) != 0;
#pragma unroll
    for (int i = 0; i < o; ++i) {
      const float send = up ? v[i] : v[i + o];
      const float keep = up ? v[i + o] : v[i];
      v[i] = keep + __shfl_xor_sync(0xffffffffu, send, o);
    }
  }
  return v[0];
}

// [R; P] -> R' with R' upper triangular and R'^T R' = R^T R + P^T P: k
// Householder reflections.  R: k x k row-major (stride LD), P: prow x k
// row-major (stride LD, prow <= 64, destroyed).  One warp; lane l holds panel
// rows l and l + 32 and, while column j is reduced, entries l + 32 b of R's row
// j (the only row of R the reflector changes, R being upper triangular).  For
// each column j the dot products of the reflector with all later columns are
// formed together, 32 columns per reduce-scatter, so the shuffles of different
// columns overlap instead of forming one long dependent chain per column.
template <int KM, int LD>
HT_DEV void warp_qr_fold(float *R, float *P, int prow, int k) {
  constexpr int NB = KM / 32;
  const int lane = threadIdx.x & 31;
  const bool h0 = lane < prow, h1 = lane + 32 < prow;
  float *p0 = P + lane * LD, *p1 = P + (lane + 32) * LD;
  for (int j = 0; j < k; ++j) {
    float r[NB];
#pragma unroll
    for (int b = 0; b < NB; ++b) r[b] = lane + 32 * b < k ? R[j * LD + lane + 32 * b] : 0.f;
    const float x0 = h0 ? p0[j] : 0.f, x1 = h1 ? p1[j] : 0.f;
    const float sig = warp_sum_bcast(fmaf(x0, x0, x1 * x1));
    const float rjj = __shfl_sync(0xffffffffu, NB == 1 || j < 32 ? r[0] : r[NB - 1], j & 31);
    if (sig != 0.f) {   // else the column below the pivot is already zero
      const float nrm = sqrtf(fmaf(rjj, rjj, sig));
      const float alpha = rjj > 0.f ? -nrm : nrm;
      const float v0 = rjj - alpha;            // reflector v = [v0; x], tau = 2 / v^T v
      const float tau = -1.f / (alpha * v0);
#pragma unroll
      for (int b = 0; b < NB; ++b) {
        if (32 * b + 31 <= j) continue;        // every column of this block is done
        float a0[32], a1[32], v[32];
#pragma unroll
        for (int i = 0; i < 32; ++i) {
          const int c = 32 * b + i;
          const bool live = c > j && c < k;
          a0[i] = (live && h0) ? p0[c] : 0.f;
          a1[i] = (live && h1) ? p1[c] : 0.f;
          v[i] = fmaf(x0, a0[i], x1 * a1[i]);
        }
        const int cl = 32 * b + lane;        // this lane's column
        const float w = fmaf(v0, r[b], warp_reduce_scatter32(v));
        const float tw = (cl > j && cl < k) ? tau * w : 0.f;
        r[b] = fmaf(-tw, v0, r[b]);
#pragma unroll
        for (int i = 0; i < 32; ++i) {
          const int c = 32 * b + i;
          const float twi = __shfl_sync(0xffffffffu, tw, i);
          if (c > j && c < k) {
            if (h0) p0[c] = fmaf(-twi, x0, a0[i]);
            if (h1) p1[c] = fmaf(-twi, x1, a1[i]);
          }
        }
      }
      if (lane == (j & 31)) r[NB == 1 ? 0 : j / 32] = alpha;
    }
#pragma unroll
    for (int b = 0; b < NB; ++b)
      if (lane + 32 * b < k) R[j * LD + lane + 32 * b] = r[b];
    __syncwarp();
  }
}

// The same fold for k <= 32 with the panel in registers: lane l holds rows
// l + 32 q (q < RPL) of all 32 columns.  The column extraction is a select over
// the unrolled register array; the shuffles of one column step (the column
// norm, the 32-column reduce-scatter and the broadcast of the 32 updates) are
// shared by all 32 RPL rows of the panel, so taller panels amortise them.
template <int LD, int RPL>
HT_DEV void warp_qr_fold32(float *R, float (&p)[RPL][32], int k) {
  const int lane = threadIdx.x & 31;
  for (int j = 0; j < k; ++j) {
    float r = lane < k ? R[j * LD + lane] : 0.f;
    float x[RPL];
#pragma unroll
    for (int q = 0; q < RPL; ++q) {
      x[q] = 0.f;
#pragma unroll
      for (int c = 0; c < 32; ++c)
        if (c == j) x[q] = p[q][c];
    }
    float ss = 0.f;
#pragma unroll
    for (int q = 0; q < RPL; ++q) ss = fmaf(x[q], x[q], ss);
    const float sig = warp_sum_bcast(ss);
    const float rjj = __shfl_sync(0xffffffffu, r, j);
    if (sig != 0.f) {   // else the column below the pivot is already zero
      const float nrm = sqrtf(fmaf(rjj, rjj, sig));
      const float alpha = rjj > 0.f ? -nrm : nrm;
      const float v0 = rjj - alpha;
      const float tau = -1.f / (alpha * v0);
      float v[32];
#pragma unroll
      for (int c = 0; c < 32; ++c) {
        float a = 0.f;
#pragma unroll
        for (int q = 0; q < RPL; ++q) a = fmaf(x[q], p[q][c], a);
        v[c] = c > j ? a : 0.f;
      }
      const float w = fmaf(v0, r, warp_reduce_scatter32(v));
      const float tw = (lane > j && lane < k) ? tau * w : 0.f;
      r = fmaf(-tw, v0, r);
#pragma unroll
      for (int c = 0; c < 32; ++c) {
        const float twc = __shfl_sync(0xffffffffu, tw, c);
        if (c > j) {
#pragma unroll
          for (int q = 0; q < RPL; ++q) p[q][c] = fmaf(-twc, x[q], p[q][c]);
        }
      }
      if (lane == j) r = alpha;
    }
    if (lane < k) R[j * LD + lane] = r;
    __syncwarp();
  }
}

// Fold a row-major panel in shared memory (prow <= 64 rows, stride LD) into R.
template <int KM, int LD>
HT_DEV void warp_fold_smem(float *R, float *P, int prow, int k) {
  if constexpr (KM == 32) {
    const int lane = threadIdx.x & 31;
    float p[2][32];
#pragma unroll
    for (int c = 0; c < 32; ++c) {
      p[0][c] = (lane < prow && c < k) ? P[lane * LD + c] : 0.f;
      p[1][c] = (lane + 32 < prow && c < k) ? P[(lane + 32) * LD + c] : 0.f;
    }
    warp_qr_fold32<LD, 2>(R, p, k);
  } else {
    warp_qr_fold<KM, LD>(R, P, prow, k);
  }
}

struct TqParams {
  const float *A;
  long long m, lda;
  int k;
  long long rows_per_cta;   // a multiple of warps x panel rows
  float *slots;             // per level: count_l x k x k floats (row-major R)
  long long slot_off[8];    // float offset of level l's slots
  int cnt_off[8];           // offset of level l's group counters
  int *counters;            // zeroed before the launch
  float *R_out;             // k x k column-major (lower triangle zero), diagonal >= 0
  float *RtR_out;           // optional k x k R^T R (compensated FP32)
};

template <int KM>
__global__ void __launch_bounds__(TqCfg<KM>::THREADS, 1) tsqr_kernel(const TqParams p) {
  using C = TqCfg<KM>;
  constexpr int LD = C::LD;
  extern __shared__ float tq_sm[];
  __shared__ int s_last;
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const int k = p.k;
  float *R = tq_sm + warp * C::WARP_FLOATS;
  float *P = R + KM * LD;
  for (int e = lane; e < KM * LD; e += 32) R[e] = 0.f;
  __syncwarp();

  // 1. this CTA's rows, in 64-row panels dealt round-robin to the warps
  const long long r_begin = static_cast<long long>(blockIdx.x) * p.rows_per_cta;
  const long long r_end = min(p.m, r_begin + p.rows_per_cta);
  for (long long r0 = r_begin + static_cast<long long>(warp) * C::PANEL; r0 < r_end;
       r0 += static_cast<long long>(C::WARPS) * C::PANEL) {
    const int prow = static_cast<int>(min(static_cast<long long>(C::PANEL), r_end - r0));
    if constexpr (KM == 32) {   // the panel straight into registers
      float pr[TqCfg<KM>::RPL][32];
#pragma unroll
      for (int c = 0; c < 32; ++c) {
        const float *col = p.A + r0 + p.lda * c;
#pragma unroll
        for (int q = 0; q < TqCfg<KM>::RPL; ++q)
          pr[q][c] = (c < k && lane + 32 * q < prow) ? __ldg(col + lane + 32 * q) : 0.f;
      }
      warp_qr_fold32<LD, TqCfg<KM>::RPL>(R, pr, k);
    } else {
#pragma unroll 4
      for (int c = 0; c < k; ++c) {
        const float *col = p.A + r0 + p.lda * c;
        P[lane * LD + c] = lane < prow ? __ldg(col + lane) : 0.f;
        P[(lane + 32) * LD + c] = lane + 32 < prow ? __ldg(col + lane + 32) : 0.f;
      }
      __syncwarp();
      warp_qr_fold<KM, LD>(R, P, prow, k);
    }
  }
  __syncthreads();

  // 2. the warps' R factors, combined pairwise in shared memory
  auto tree = [&]() {
    for (int half = C::WARPS / 2; half >= 1; half >>= 1) {
      if (warp < half) warp_fold_smem<KM, LD>(R, tq_sm + (warp + half) * C::WARP_FLOATS, k, k);
      __syncthreads();
    }
  };
  tree();

  // 3. across CTAs: the last CTA of each group of TQ_FAN combines the group
  float *R0 = tq_sm;   // warp 0's R: the CTA's result
  long long node = blockIdx.x, count = gridDim.x;
  int level = 0;
  while (count > 1) {
    float *slot = p.slots + p.slot_off[level] + node * k * k;
    for (int e = t; e < k * k; e += C::THREADS) slot[e] = R0[(e / k) * LD + e % k];
    __threadfence();
    __syncthreads();
    const long long group = node / TQ_FAN;
    const int gsize = static_cast<int>(min(static_cast<long long>(TQ_FAN), count - group * TQ_FAN));
    if (t == 0) s_last = atomicAdd(p.counters + p.cnt_off[level] + group, 1) == gsize - 1;
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    // warp w takes member w into its R (zero when the group is smaller) and
    // folds in members w + WARPS, w + 2 WARPS, ... as panels
    auto load_member = [&](float *dst, long long member) {
      const float *src = p.slots + p.slot_off[level] + member * k * k;
      for (int e = lane; e < KM * LD; e += 32) {
        const int i = e / LD, c = e % LD;
        dst[e] = (i < k && c < k) ? __ldcg(src + i * k + c) : 0.f;
      }
      __syncwarp();
    };
    if (warp < gsize) {
      load_member(R, group * TQ_FAN + warp);
    } else {
      for (int e = lane; e < KM * LD; e += 32) R[e] = 0.f;
      __syncwarp();
    }
    for (int w = warp + C::WARPS; w < gsize; w += C::WARPS) {
      load_member(P, group * TQ_FAN + w);
      warp_fold_smem<KM, LD>(R, P, k, k);
    }
    __syncthreads();
    tree();
    node = group;
    count = (count + TQ_FAN - 1) / TQ_FAN;
    ++level;
  }

  // 4. one R left: non-negative diagonal, column-major out, R^T R if asked
  __shared__ float sgn[64];
  for (int i = t; i < k; i += C::THREADS) sgn[i] = R0[i * LD + i] < 0.f ? -1.f : 1.f;
  __syncthreads();
  for (int e = t; e < k * k; e += C::THREADS) {
    const int i = e % k, j = e / k;
    p.R_out[e] = i <= j ? sgn[i] * R0[i * LD + j] : 0.f;
  }
  if (p.RtR_out) {
    for (int e = t; e < k * k; e += C::THREADS) {
      const int a = e % k, b = e / k;
      Acc2 acc{0.f, 0.f};
      for (int i = 0; i <= min(a, b); ++i) acc2_add_prod(acc, R0[i * LD + a], R0[i * LD + b]);
      p.RtR_out[e] = acc.s + acc.c;
    }
  }
}

int tq_levels(long long count, long long *counts) {
  int L = 0;
  while (count > 1 && L < 8) {
    counts[L++] = count;
    count = (count + TQ_FAN - 1) / TQ_FAN;
  }
  return L;
}

long long tq_grid(long long m) {
  const long long want = (m + 4 * TQ_PROWS - 1) / (4 * TQ_PROWS);   // at least ~4 panels per CTA
  const long long cap = device_sm_count();
  return want < 1 ? 1 : (want < cap ? want : cap);
}

}  // namespace

size_t tsqr_workspace_bytes(long long m, int k) {
  long long counts[8];
  const int L = tq_levels(tq_grid(m), counts);
  size_t floats = 0, ints = 0;
  for (int l = 0; l < L; ++l) {
    floats += static_cast<size_t>(counts[l]) * k * k;
    ints += static_cast<size_t>((counts[l] + TQ_FAN - 1) / TQ_FAN);
  }
  return ((floats * sizeof(float) + 255) & ~size_t(255)) + ((ints * sizeof(int) + 255) & ~size_t(255)) + 256;
}

cudaError_t tsqr_launch(const float *A, long long m, int k, long long lda, float *R, float *RtR, void *ws,
                        size_t ws_bytes, cudaStream_t st, int *launches) {
  if (k < 1 || k > 64 || m < 1 || lda < m) return cudaErrorInvalidValue;
  if (tsqr_workspace_bytes(m, k) > ws_bytes) return cudaErrorInvalidValue;
  TqParams p{};
  p.A = A;
  p.m = m;
  p.lda = lda;
  p.k = k;
  const long long grid = tq_grid(m);
  // a CTA's rows are a whole number of rounds of panels over its warps, so the
  // warps finish together (the tree that follows waits for the slowest)
  const long long round = k <= 32 ? TqCfg<32>::WARPS * TqCfg<32>::PANEL : TqCfg<64>::WARPS * TqCfg<64>::PANEL;
  p.rows_per_cta = ((m + grid - 1) / grid + round - 1) / round * round;
  const long long g = (m + p.rows_per_cta - 1) / p.rows_per_cta;   // CTAs that own rows
  long long counts[8];
  const int L = tq_levels(g, counts);
  if (g > 1 && L >= 8) return cudaErrorInvalidValue;
  size_t floats = 0;
  int ints = 0;
  for (int l = 0; l < L; ++l) {
    p.slot_off[l] = static_cast<long long>(floats);
    p.cnt_off[l] = ints;
    floats += static_cast<size_t>(counts[l]) * k * k;
    ints += static_cast<int>((counts[l] + TQ_FAN - 1) / TQ_FAN);
  }
  char *w = static_cast<char *>(ws);
  p.slots = reinterpret_cast<float *>(w);
  p.counters = reinterpret_cast<int *>(w + ((floats * sizeof(float) + 255) & ~size_t(255)));
  p.R_out = R;
  p.RtR_out = RtR;
  if (ints > 0) {
    const cudaError_t e = cudaMemsetAsync(p.counters, 0, sizeof(int) * ints, st);
    if (e != cudaSuccess) return e;
  }
  static bool attr32[64] = {}, attr64[64] = {};
  if (k <= 32) {
    const cudaError_t e = opt_in_smem(tsqr_kernel<32>, static_cast<int>(TqCfg<32>::SMEM), attr32);
    if (e != cudaSuccess) return e;
    tsqr_kernel<32><<<static_cast<unsigned>(g), TqCfg<32>::THREADS, TqCfg<32>::SMEM, st>>>(p);
  } else {
    const cudaError_t e = opt_in_smem(tsqr_kernel<64>, static_cast<int>(TqCfg<64>::SMEM), attr64);
    if (e != cudaSuccess) return e;
    tsqr_kernel<64><<<static_cast<unsigned>(g), TqCfg<64>::THREADS, TqCfg<64>::SMEM, st>>>(p);
  }
  if (launches) *launches += 1;
  return cudaGetLastError();
}

}  // namespace htgb
