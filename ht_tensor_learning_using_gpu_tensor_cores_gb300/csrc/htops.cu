// Operations on a tensor held in HT format (tree, ranks, leaf bases U_t,
// transfer tensors B_t): full reconstruction and evaluation of single entries.
//
// The reference reconstructs only the whole tensor, with cuBLAS calls on the
// node bases (third_order_tensor_decompsition/CUDA/Optimized/htd_tensorcore.cu:
// 295-331); it has no entry-wise evaluation.  Here the reconstruction is one
// expansion of the interior node basis (small.cu expand2) and one NT product
// written straight into the column-major tensor.  Single entries are read from
// precontracted matrices: every transfer tensor is folded with its parent's
// and one child's factors into a matrix with one row per index of that child's
// mode, so an entry costs one or two k x k row-vector products.
#include "common.cuh"
#include "engine.h"

namespace htgb {
namespace {

constexpr int RT_M = 128, RT_N = 64, RT_K = 64;

// Slab z of a batch: C_z (m x n, ldc) = A_z (m x k, lda) B^T (B: n x k, ldb),
// k <= 64, column-major, A_z = A + z sA, C_z = C + z sC.  256 threads: thread
// (tx = t % 32, ty = t / 32) owns rows 4 tx .. 4 tx + 3 and columns
// 8 ty .. 8 ty + 7 of the 128 x 64 tile, read from shared memory as one and two
// 16-byte vectors per k step (the column vectors are warp-uniform broadcasts),
// so the loop is bound by the FMA pipe; rows go out as 16-byte stores when the
// output is 16-byte aligned.
__global__ void __launch_bounds__(256) gemm_nt_kernel(const float *__restrict__ A0, long long lda, long long sA,
                                                      const float *__restrict__ B, long long ldb, float *__restrict__ C0,
                                                      long long ldc, long long sC, long long m, long long n, int k,
                                                      long long batch) {
  __shared__ __align__(16) float As[RT_K][RT_M];
  __shared__ __align__(16) float Bs[RT_K][RT_N];
  const long long r0 = static_cast<long long>(blockIdx.x) * RT_M, c0 = static_cast<long long>(blockIdx.y) * RT_N;
  const int t = threadIdx.x, tx = t & 31, ty = t >> 5;
  for (int e = t; e < RT_N * k; e += 256) {
    const int c = e % RT_N, kk = e / RT_N;
    Bs[kk][c] = (c0 + c < n) ? B[(c0 + c) + ldb * kk] : 0.f;
  }
  for (long long z = blockIdx.z; z < batch; z += gridDim.z) {
    const float *A = A0 + z * sA;
    float *C = C0 + z * sC;
    __syncthreads();
    for (int e = t; e < RT_M * k; e += 256) {
      const int r = e % RT_M, kk = e / RT_M;
      As[kk][r] = (r0 + r < m) ? A[(r0 + r) + lda * kk] : 0.f;
    }
    __syncthreads();
    float acc[4][8];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 8; ++j) acc[i][j] = 0.f;
    for (int kk = 0; kk < k; ++kk) {
      const float4 a = *reinterpret_cast<const float4 *>(&As[kk][4 * tx]);
      const float4 b0 = *reinterpret_cast<const float4 *>(&Bs[kk][8 * ty]);
      const float4 b1 = *reinterpret_cast<const float4 *>(&Bs[kk][8 * ty + 4]);
      const float av[4] = {a.x, a.y, a.z, a.w};
      const float bv[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
    }
    const long long r = r0 + 4 * tx;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const long long c = c0 + 8 * ty + j;
      if (c >= n || r >= m) continue;
      float *dst = C + r + ldc * c;
      if (r + 3 < m && (reinterpret_cast<uintptr_t>(dst) & 15u) == 0) {
        *reinterpret_cast<float4 *>(dst) = make_float4(acc[0][j], acc[1][j], acc[2][j], acc[3][j]);
      } else {
#pragma unroll
        for (int i = 0; i < 4; ++i)
          if (r + i < m) dst[i] = acc[i][j];
      }
    }
  }
}

// out[(c + kc b) + kc kq a] = sum_rt Bt[a + kp b + kp kq rt] M[rt + kt c]
// (M: kt x kc; M null = the identity, kc = kt): a transfer tensor with its
// parent's factor folded in, reordered so that a row of out's product with a
// leaf basis is contiguous in (c, b).
__global__ void eval_core_kernel(const float *__restrict__ Bt, int kp, int kq, int kt, const float *__restrict__ M,
                                 int kc, float *__restrict__ out) {
  const int total = kc * kq * kp;
  for (int e = blockIdx.x * 256 + threadIdx.x; e < total; e += gridDim.x * 256) {
    const int c = e % kc, b = (e / kc) % kq, a = e / (kc * kq);
    float s;
    if (!M) {
      s = Bt[a + kp * b + kp * kq * c];
    } else {
      s = 0.f;
      for (int rt = 0; rt < kt; ++rt) s = fmaf(Bt[a + kp * b + kp * kq * rt], M[rt + kt * c], s);
    }
    out[e] = s;
  }
}

HT_DEV long long eval_index(const long long *idx, long long e, int order, int m, long long dim, int *err, int lane) {
  long long i = idx[e * order + m];
  if (i < 0 || i >= dim) {
    if (lane == 0) atomicOr(err, 1);
    i = i < 0 ? 0 : dim - 1;
  }
  return i;
}

// One warp per entry, lanes over y < ky (two per lane):
//   a[y] = sum_x W0[i_row0][y + ky x] U0v[i_vec0 + n_vec0 x]
//   c[y] = side 1 the same, or U1v[i_vec1 + n_vec1 y] when W1 is null
//   entry = sum_y a[y] c[y].
__global__ void __launch_bounds__(256) evaluate_kernel(const EvalPlan ep, const long long *__restrict__ idx,
                                                       long long count, float *__restrict__ out, int *err) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ky = ep.ky;
  for (long long e = static_cast<long long>(blockIdx.x) * 8 + warp; e < count;
       e += static_cast<long long>(gridDim.x) * 8) {
    float v[2][2];
#pragma unroll
    for (int sd = 0; sd < 2; ++sd) {
      const EvalSide &S = ep.side[sd];
      const long long iv = eval_index(idx, e, ep.order, S.mode_vec, S.n_vec, err, lane);
      if (S.W) {
        const long long ir = eval_index(idx, e, ep.order, S.mode_row, S.n_row, err, lane);
        const float *row = S.W + ir * static_cast<long long>(ky) * S.kx;
        float s0 = 0.f, s1 = 0.f;
        for (int x = 0; x < S.kx; ++x) {
          const float u = __ldg(S.Uv + iv + S.n_vec * x);
          if (lane < ky) s0 = fmaf(row[lane + ky * x], u, s0);
          if (lane + 32 < ky) s1 = fmaf(row[lane + 32 + ky * x], u, s1);
        }
        v[sd][0] = s0;
        v[sd][1] = s1;
      } else {
        v[sd][0] = lane < ky ? S.Uv[iv + S.n_vec * lane] : 0.f;
        v[sd][1] = lane + 32 < ky ? S.Uv[iv + S.n_vec * (lane + 32)] : 0.f;
      }
    }
    float s = v[0][0] * v[1][0] + v[0][1] * v[1][1];
    for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    if (lane == 0) out[e] = s;
  }
}

}  // namespace

cudaError_t gemm_nt_launch(const float *A, long long lda, long long sA, const float *B, long long ldb, float *C,
                           long long ldc, long long sC, long long m, long long n, int k, long long batch,
                           cudaStream_t s) {
  if (k < 1 || k > RT_K || batch < 1) return cudaErrorInvalidValue;
  const long long gx = (m + RT_M - 1) / RT_M;
  if (gx > 0x7fffffffll) return cudaErrorInvalidValue;
  const long long gz = batch < 65535 ? batch : 65535;
  const long long chunk = 65535ll * RT_N;   // columns per launch (grid y limit)
  for (long long c0 = 0; c0 < n; c0 += chunk) {
    const long long nc = n - c0 < chunk ? n - c0 : chunk;
    const unsigned gy = static_cast<unsigned>((nc + RT_N - 1) / RT_N);
    gemm_nt_kernel<<<dim3(static_cast<unsigned>(gx), gy, static_cast<unsigned>(gz)), 256, 0, s>>>(
        A, lda, sA, B + c0, ldb, C + c0 * ldc, ldc, sC, m, nc, k, batch);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t eval_core_launch(const float *Bt, int kp, int kq, int kt, const float *M, int kc, float *out,
                             cudaStream_t s) {
  const int total = kc * kq * kp;
  int grid = (total + 255) / 256;
  if (grid > 8 * device_sm_count()) grid = 8 * device_sm_count();
  eval_core_kernel<<<grid < 1 ? 1 : grid, 256, 0, s>>>(Bt, kp, kq, kt, M, kc, out);
  return cudaGetLastError();
}

cudaError_t evaluate_launch(const EvalPlan &ep, const long long *idx, long long count, float *out, int *err,
                            cudaStream_t s) {
  if (ep.ky < 1 || ep.ky > 64) return cudaErrorInvalidValue;
  long long grid = (count + 7) / 8;
  if (grid > 16ll * device_sm_count()) grid = 16ll * device_sm_count();
  if (grid < 1) grid = 1;
  evaluate_kernel<<<static_cast<unsigned>(grid), 256, 0, s>>>(ep, idx, count, out, err);
  return cudaGetLastError();
}

}  // namespace htgb
