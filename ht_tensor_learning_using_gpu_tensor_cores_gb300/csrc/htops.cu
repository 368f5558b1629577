// Operations on a tensor held in HT format (tree, ranks, leaf bases U_t,
// transfer tensors B_t): full reconstruction and evaluation of single entries.
//
// The reference reconstructs only the whole tensor, with cuBLAS calls on the
// node bases (third_order_tensor_decompsition/CUDA/Optimized/htd_tensorcore.cu:
// 295-331); it has no entry-wise evaluation.  Here the reconstruction is one
// expansion of the interior node basis (small.cu expand2) and one NT product
// written straight into the column-major tensor, and single entries are
// contracted leaf-to-root without touching the rest of the tensor.
#include "common.cuh"
#include "engine.h"

namespace htgb {
namespace {

constexpr int RT_M = 128, RT_N = 64, RT_K = 64;

// Slab z of a batch: C_z (m x n, ldc) = A_z (m x k, lda) B^T (B: n x k, ldb),
// k <= 64, column-major, A_z = A + z sA, C_z = C + z sC.  256 threads: thread
// (tx = t % 32, ty = t / 32) owns rows tx + 32 i (i < 4) and columns ty + 8 j
// (j < 8) of the 128 x 64 tile.
__global__ void __launch_bounds__(256) gemm_nt_kernel(const float *__restrict__ A0, long long lda, long long sA,
                                                      const float *__restrict__ B, long long ldb, float *__restrict__ C0,
                                                      long long ldc, long long sC, long long m, long long n, int k,
                                                      long long batch) {
  __shared__ float As[RT_K][RT_M];   // rows are read and written by consecutive lanes: no padding
  __shared__ float Bs[RT_K][RT_N];
  const long long r0 = static_cast<long long>(blockIdx.x) * RT_M, c0 = static_cast<long long>(blockIdx.y) * RT_N;
  const int t = threadIdx.x, tx = t & 31, ty = t >> 5;
  for (long long z = blockIdx.z; z < batch; z += gridDim.z) {
  const float *A = A0 + z * sA;
  float *C = C0 + z * sC;
  __syncthreads();
  for (int e = t; e < RT_M * k; e += 256) {
    const int r = e % RT_M, kk = e / RT_M;
    As[kk][r] = (r0 + r < m) ? A[(r0 + r) + lda * kk] : 0.f;
  }
  for (int e = t; e < RT_N * k; e += 256) {
    const int c = e % RT_N, kk = e / RT_N;
    Bs[kk][c] = (c0 + c < n) ? B[(c0 + c) + ldb * kk] : 0.f;
  }
  __syncthreads();
  float acc[4][8];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[i][j] = 0.f;
  for (int kk = 0; kk < k; ++kk) {
    float a[4], b[8];
#pragma unroll
    for (int i = 0; i < 4; ++i) a[i] = As[kk][tx + 32 * i];
#pragma unroll
    for (int j = 0; j < 8; ++j) b[j] = Bs[kk][ty + 8 * j];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 8; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
  }
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const long long c = c0 + ty + 8 * j;
    if (c >= n) continue;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const long long r = r0 + tx + 32 * i;
      if (r < m) C[r + ldc * c] = acc[i][j];
    }
  }
  }
}

// One warp per entry: leaf rows, then every interior node bottom-up
// (v_t[c] = sum_{a,b} B_t[a + kl b + kl kr c] v_l[a] v_r[b]), then the root.
// An index outside its mode sets *err = 1 and is read as the nearest valid one.
__global__ void __launch_bounds__(256) evaluate_kernel(const EvalTree et, const long long *__restrict__ idx,
                                                       long long count, float *__restrict__ out, int *err) {
  __shared__ float vs[8][kEvalNodes][64];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float (*v)[64] = vs[warp];
  for (long long e = static_cast<long long>(blockIdx.x) * 8 + warp; e < count; e += static_cast<long long>(gridDim.x) * 8) {
    for (int q = 0; q < et.n_nodes; ++q) {
      const int t = et.post[q];
      if (et.left[t] < 0) {
        const int m = et.mode[t];
        long long i = idx[e * et.order + m];
        if (i < 0 || i >= et.dim[m]) {
          if (lane == 0) atomicOr(err, 1);
          i = i < 0 ? 0 : et.dim[m] - 1;
        }
        for (int c = lane; c < et.rank[t]; c += 32) v[t][c] = et.U[t][i + et.dim[m] * static_cast<long long>(c)];
      } else {
        const int l = et.left[t], r = et.right[t], kl = et.rank[l], kr = et.rank[r], kt = et.rank[t];
        const float *Bt = et.B[t];
        for (int c = lane; c < kt; c += 32) {
          float s = 0.f;
          for (int b = 0; b < kr; ++b) {
            float inner = 0.f;
            const float *col = Bt + static_cast<long long>(kl) * (b + static_cast<long long>(kr) * c);
            for (int a = 0; a < kl; ++a) inner = fmaf(col[a], v[l][a], inner);
            s = fmaf(inner, v[r][b], s);
          }
          v[t][c] = s;
        }
      }
      __syncwarp();
    }
    if (lane == 0) out[e] = v[0][0];
    __syncwarp();
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

cudaError_t evaluate_launch(const EvalTree &et, const long long *idx, long long count, float *out, int *err,
                            cudaStream_t s) {
  long long grid = (count + 7) / 8;
  if (grid > 152 * 16) grid = 152 * 16;
  if (grid < 1) grid = 1;
  evaluate_kernel<<<static_cast<unsigned>(grid), 256, 0, s>>>(et, idx, count, out, err);
  return cudaGetLastError();
}

}  // namespace htgb
