// Streaming and small dense kernels of the HT path:
//   * FP32 -> BF16 conversion of the tensor with a compensated ||X||^2 (the
//     reference's f2h, third_order_tensor_decompsition/CUDA/Optimized/kernel.cu:31-45);
//   * the small contractions that turn the core pass into transfer tensors
//     (the reference's ttm chain, ttm.cu:2-36);
//   * expansion of HT factors and a fused reconstruct-and-reduce error pass
//     that never materialises Xhat (the reference writes Xhat and runs
//     Saxpy + 2 x Snrm2, htd_batch.cu:196-244).
#include "common.cuh"
#include "engine.h"

namespace htgb {
namespace {

__global__ void __launch_bounds__(256, 8) convert_bf16_kernel(const float *__restrict__ x, __nv_bfloat16 *__restrict__ xb,
                                                           long long n, double *partials) {
  Acc2 a = {0.f, 0.f};
  const long long n4 = n / 4;
  const float4 *x4 = reinterpret_cast<const float4 *>(x);
  for (long long i = blockIdx.x * 256ll + threadIdx.x; i < n4; i += gridDim.x * 256ll) {
    const float4 v = __ldcs(x4 + i);   // streamed once: do not keep in L2
    acc2_add_prod(a, v.x, v.x);
    acc2_add_prod(a, v.y, v.y);
    acc2_add_prod(a, v.z, v.z);
    acc2_add_prod(a, v.w, v.w);
    __nv_bfloat162 lo = __floats2bfloat162_rn(v.x, v.y);
    __nv_bfloat162 hi = __floats2bfloat162_rn(v.z, v.w);
    uint2 pk;
    pk.x = *reinterpret_cast<uint32_t *>(&lo);
    pk.y = *reinterpret_cast<uint32_t *>(&hi);
    reinterpret_cast<uint2 *>(xb)[i] = pk;
  }
  for (long long i = n4 * 4 + blockIdx.x * 256ll + threadIdx.x; i < n; i += gridDim.x * 256ll) {
    const float v = x[i];
    acc2_add_prod(a, v, v);
    xb[i] = __float2bfloat16_rn(v);
  }
  __shared__ double red[256];
  red[threadIdx.x] = static_cast<double>(a.s) + static_cast<double>(a.c);
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partials[blockIdx.x] = red[0];
}

// X (n1 x rest, FP32, first index fastest) -> xp (n1p x rest, BF16, zero rows
// n1 <= i < n1p) and the compensated sum of squares per block.  The padded copy
// gives every matricisation a leading dimension that TMA can address (a
// multiple of 8 BF16 elements) when n1 itself is not one.
__global__ void __launch_bounds__(256) convert_bf16_pad_kernel(const float *__restrict__ x, __nv_bfloat16 *__restrict__ xp,
                                                             long long n1, long long n1p, long long rest,
                                                             double *partials) {
  Acc2 a = {0.f, 0.f};
  const long long total = n1p * rest;
  for (long long e = blockIdx.x * 256ll + threadIdx.x; e < total; e += gridDim.x * 256ll) {
    const long long r = e / n1p, i = e - r * n1p;
    const float v = i < n1 ? __ldcs(x + i + n1 * r) : 0.f;
    acc2_add_prod(a, v, v);
    xp[e] = __float2bfloat16_rn(v);
  }
  __shared__ double red[256];
  red[threadIdx.x] = static_cast<double>(a.s) + static_cast<double>(a.c);
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partials[blockIdx.x] = red[0];
}

// X (L x N, l fastest, FP32) -> xb (the same layout, BF16) and xbt, a second
// BF16 copy in l-blocks of B = 2^lb elements: xbt[((l / B) N + n) B + l % B],
// plus the compensated sum of squares per block, over the columns n in
// [n_begin, n_begin + n_count).  Work goes in tiles of B l by
// TN n (TN = 2^(12 - lb), 4096 elements a tile), l-blocks fastest: the grid's blocks
// then read and write xb inside TN columns at a time, and each tile's xbt part
// is one contiguous run of 2 B TN bytes (8 KiB), so all three streams stay
// within a few hundred 2 MiB pages.  In xbt the rows of the last mode's Gram
// (rows n, K = l) are 2B bytes apart inside each l-block, where in xb they lie
// 2L bytes apart (one 2 MiB page per row at 1024^3).  Needs L % B == 0 and
// N % TN == 0.
__global__ void __launch_bounds__(256, 8) convert_bf16_dual_kernel(const float *__restrict__ x,
                                                                __nv_bfloat16 *__restrict__ xb,
                                                                __nv_bfloat16 *__restrict__ xbt, long long L,
                                                                long long N, long long n_begin, long long n_count,
                                                                int lb, double *partials) {
  Acc2 a = {0.f, 0.f};
  const int TN = 1 << (12 - lb);
  const long long B = 1ll << lb, nlb = L >> lb, tiles = nlb * (n_count / TN);
  const int row4 = static_cast<int>(B / 4);          // float4 per tile column
  // every tile holds B * TN = 4096 elements: 4 float4 per thread, loaded together
  for (long long ti = blockIdx.x; ti < tiles; ti += gridDim.x) {
    const long long lblk = ti % nlb, n0 = n_begin + (ti / nlb) * TN;
    float4 v[4];
    long long off[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int q = threadIdx.x + 256 * j, nn = q / row4, l4 = q - nn * row4;
      off[j] = (lblk << lb) + 4 * l4 + L * (n0 + nn);
      v[j] = __ldcs(reinterpret_cast<const float4 *>(x + off[j]));
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      acc2_add_prod(a, v[j].x, v[j].x);
      acc2_add_prod(a, v[j].y, v[j].y);
      acc2_add_prod(a, v[j].z, v[j].z);
      acc2_add_prod(a, v[j].w, v[j].w);
      __nv_bfloat162 lo = __floats2bfloat162_rn(v[j].x, v[j].y);
      __nv_bfloat162 hi = __floats2bfloat162_rn(v[j].z, v[j].w);
      uint2 pk;
      pk.x = *reinterpret_cast<uint32_t *>(&lo);
      pk.y = *reinterpret_cast<uint32_t *>(&hi);
      *reinterpret_cast<uint2 *>(xb + off[j]) = pk;
      // the tile's xbt part is contiguous and in the same element order as q
      *reinterpret_cast<uint2 *>(xbt + ((lblk * N + n0) << lb) + 4 * (threadIdx.x + 256 * j)) = pk;
    }
  }
  __shared__ double red[256];
  red[threadIdx.x] = static_cast<double>(a.s) + static_cast<double>(a.c);
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partials[blockIdx.x] = red[0];
}

// dst = src (first) or dst + src, n floats
__global__ void accumulate_kernel(float *__restrict__ dst, const float *__restrict__ src, long long n, int first) {
  for (long long i = blockIdx.x * 256ll + threadIdx.x; i < n; i += gridDim.x * 256ll)
    dst[i] = first ? src[i] : dst[i] + src[i];
}

__global__ void sumsq_kernel(const float *__restrict__ x, long long n, double *partials) {
  Acc2 a = {0.f, 0.f};
  for (long long i = blockIdx.x * 256ll + threadIdx.x; i < n; i += gridDim.x * 256ll) {
    const float v = x[i];
    acc2_add_prod(a, v, v);
  }
  __shared__ double red[256];
  red[threadIdx.x] = static_cast<double>(a.s) + static_cast<double>(a.c);
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partials[blockIdx.x] = red[0];
}

// Grouped conversion of a batch: job j owns blocks [blk0, blk0 + nblk) of the
// launch and converts its tensor x (n1 x rest, FP32) to xb (n1p x rest, BF16,
// rows padded with zeros; xb null: sums only), writing one compensated
// partial sum of squares per block; the finish kernel (a block per job) sums
// a job's partials in block order into its dsum[0].
// Job j of a grouped launch into shared memory, one 4-byte word per thread.
template <class Job>
HT_DEV void load_job(const Job *__restrict__ jobs, int j, Job &J) {
  static_assert(sizeof(Job) % 4 == 0 && sizeof(Job) <= 4 * 256, "job table entries are copied word by word");
  if (threadIdx.x < sizeof(Job) / 4)
    reinterpret_cast<uint32_t *>(&J)[threadIdx.x] = reinterpret_cast<const uint32_t *>(jobs + j)[threadIdx.x];
  __syncthreads();
}

__global__ void __launch_bounds__(256) convert_grouped_kernel(const ConvJob *__restrict__ jobs,
                                                              const int *__restrict__ job_of_block) {
  __shared__ ConvJob J;
  load_job(jobs, job_of_block[blockIdx.x], J);
  const int b = blockIdx.x - J.blk0;
  Acc2 a = {0.f, 0.f};
  // a warp per row of n1 inputs (n1p outputs), four loads in flight per lane
  const int lane = threadIdx.x & 31, n1 = static_cast<int>(J.n1), n1p = static_cast<int>(J.n1p);
  for (long long r = static_cast<long long>(b) * 8 + (threadIdx.x >> 5); r < J.rest; r += J.nblk * 8ll) {
    const float *src = J.x + J.n1 * r;
    __nv_bfloat16 *dst = J.xb ? J.xb + J.n1p * r : nullptr;
    for (int i0 = lane; i0 < n1p; i0 += 128) {
      float v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int i = i0 + 32 * u;
        v[u] = i < n1 ? __ldcs(src + i) : 0.f;
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int i = i0 + 32 * u;
        if (i < n1p) {
          acc2_add_prod(a, v[u], v[u]);
          if (dst) dst[i] = __float2bfloat16_rn(v[u]);
        }
      }
    }
  }
  __shared__ double red[256];
  red[threadIdx.x] = static_cast<double>(a.s) + static_cast<double>(a.c);
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) J.partials[b] = red[0];
}

__global__ void convert_grouped_finish_kernel(const ConvJob *__restrict__ jobs) {
  const ConvJob &J = jobs[blockIdx.x];
  __shared__ double red[256];
  double s = 0.0;
  for (int i = threadIdx.x; i < J.nblk; i += 256) s += J.partials[i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) J.dsum[0] = red[0];
}

// Grouped copy: block i copies segment segs[i] (count floats).
__global__ void copy_segments_kernel(const CopySeg *__restrict__ segs) {
  const CopySeg g = segs[blockIdx.x];
  for (long long e = threadIdx.x; e < g.count; e += 256) g.dst[e] = g.src[e];
}

// x[i] = the BF16 rounding of x[i] (kept in FP32), and the BF16 copy in y.
__global__ void round_bf16_kernel(float *__restrict__ x, __nv_bfloat16 *__restrict__ y, long long n) {
  for (long long i = blockIdx.x * 256ll + threadIdx.x; i < n; i += gridDim.x * 256ll) {
    const __nv_bfloat16 b = __float2bfloat16_rn(x[i]);
    y[i] = b;
    x[i] = __bfloat162float(b);
  }
}

__global__ void f32_to_bf16_kernel(const float *__restrict__ x, __nv_bfloat16 *__restrict__ y, long long n) {
  for (long long i = blockIdx.x * 256ll + threadIdx.x; i < n; i += gridDim.x * 256ll) y[i] = __float2bfloat16_rn(x[i]);
}

__global__ void split_bf16_kernel(const float *__restrict__ W, long long rows, int k, int h,
                                  __nv_bfloat16 *__restrict__ Y) {
  const long long total = rows * 2 * h;
  for (long long i = blockIdx.x * 256ll + threadIdx.x; i < total; i += gridDim.x * 256ll) {
    const long long r = i % rows;
    const int col = static_cast<int>(i / rows);
    const int j = col < h ? col : col - h;
    float v = 0.f;
    if (j < k) {
      const float w = W[r + rows * j];
      const float hi = __bfloat162float(__float2bfloat16_rn(w));
      v = col < h ? hi : w - hi;   // w - hi is exact in FP32
    }
    Y[i] = __float2bfloat16_rn(v);
  }
}

__global__ void sumsq_finish_kernel(const double *partials, int n, double *out) {
  __shared__ double red[256];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += 256) s += partials[i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = red[0];
}

// C (m x n) = A^T B, A (K x m), B (K x n), column-major.  One warp per output
// element, compensated accumulation.
__global__ void gemm_tn_small_kernel(const float *__restrict__ A, int lda, const float *__restrict__ B, int ldb,
                                     float *__restrict__ C, int ldc, int m, int n, int K) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= m * n) return;
  const int i = warp % m, j = warp / m;
  Acc2 a = {0.f, 0.f};
  for (int k = lane; k < K; k += 32) acc2_add_prod(a, A[k + static_cast<long long>(lda) * i], B[k + static_cast<long long>(ldb) * j]);
  double v = static_cast<double>(a.s) + static_cast<double>(a.c);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if (lane == 0) C[i + static_cast<long long>(ldc) * j] = static_cast<float>(v);
}

// C[a, b, c] = sum_j T1[(j + nq*c) + ldt*a] * Uq[j + nq*b]: a CTA per (c, range
// of jc values of j); with several ranges C points at partials [range][kp kq kc].
// Entries (:, :, c) of C from the j range [j_lo, j_hi); writes Co[pr + kp kq c].
HT_DEV void core_step2_body(const float *__restrict__ T1, long long ldt, int nq, int kp, const float *__restrict__ Uq,
                            int kq, int c, int j_lo, int j_hi, float *__restrict__ Co) {
  __shared__ float Ts[64][65];
  __shared__ float Us[64][65];
  const int t = threadIdx.x;
  const int npair = kp * kq;
  float acc[16];
#pragma unroll
  for (int q = 0; q < 16; ++q) acc[q] = 0.f;
  for (int j0 = j_lo; j0 < j_hi; j0 += 64) {
    __syncthreads();
    for (int e = t; e < 64 * 64; e += 256) {
      const int jj = e % 64, a = e / 64;
      Ts[jj][a] = (j0 + jj < j_hi && a < kp) ? T1[(j0 + jj + static_cast<long long>(nq) * c) + ldt * a] : 0.f;
      Us[jj][a] = (j0 + jj < j_hi && a < kq) ? Uq[(j0 + jj) + static_cast<long long>(nq) * a] : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      const int pr = t + 256 * q;
      if (pr < npair) {
        const int a = pr % kp, b = pr / kp;
        float s = acc[q];
        for (int jj = 0; jj < 64; ++jj) s = fmaf(Ts[jj][a], Us[jj][b], s);
        acc[q] = s;
      }
    }
  }
#pragma unroll
  for (int q = 0; q < 16; ++q) {
    const int pr = t + 256 * q;
    if (pr < npair) Co[pr + static_cast<long long>(npair) * c] = acc[q];
  }
}

__global__ void __launch_bounds__(256) core_step2_kernel(const float *__restrict__ T1, long long ldt, int nq, int kp,
                                                         const float *__restrict__ Uq, int kq, int jc,
                                                         float *__restrict__ C) {
  const int c = blockIdx.x, j_lo = blockIdx.y * jc, j_hi = min(nq, j_lo + jc);
  core_step2_body(T1, ldt, nq, kp, Uq, kq, c, j_lo, j_hi,
                  C + static_cast<long long>(blockIdx.y) * kp * kq * gridDim.x);
}

// Grouped narrow mode product of the batched path (the 3rd-order core pass,
// rows of X contiguous): Z[row + L R j] = sum_i X[l + L (i + N r)] V[i + N j]
// for row = l + L r, j < kz <= KB.  A thread per row, V staged in 64-row chunks
// of shared memory; the job's blocks stride over its rows.
template <int KB>
__global__ void __launch_bounds__(256) modeprod_narrow_grouped_kernel(const NarrowJob *__restrict__ jobs,
                                                                      const int *__restrict__ job_of_block) {
  __shared__ NarrowJob J;
  __shared__ __align__(16) float Vs[64][KB];
  load_job(jobs, job_of_block[blockIdx.x], J);
  const int t = threadIdx.x, kz = J.kz, N = J.N;
  const long long L = J.L, total = J.L * J.R;
  for (long long base = static_cast<long long>(blockIdx.x - J.blk0) * 256; base < total; base += J.nblk * 256ll) {
    const long long row = base + t;
    const bool valid = row < total;
    const long long r = valid ? row / L : 0, l = valid ? row - r * L : 0;
    const float *x = J.X + l + L * N * r;
    float acc[KB];
#pragma unroll
    for (int j = 0; j < KB; ++j) acc[j] = 0.f;
    for (int i0 = 0; i0 < N; i0 += 64) {
      const int ni = min(64, N - i0);
      __syncthreads();
      for (int e = t; e < 64 * KB; e += 256) {
        const int ii = e / KB, j = e - ii * KB;
        Vs[ii][j] = (ii < ni && j < kz) ? J.V[(i0 + ii) + static_cast<long long>(N) * j] : 0.f;
      }
      __syncthreads();
      if (valid) {
        for (int ii = 0; ii < ni; ii += 8) {
          float xv[8];   // eight independent loads in flight before the products
#pragma unroll
          for (int u = 0; u < 8; ++u) xv[u] = ii + u < ni ? __ldg(x + L * (i0 + ii + u)) : 0.f;
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            const float4 *v4 = reinterpret_cast<const float4 *>(&Vs[(ii + u) & 63][0]);
#pragma unroll
            for (int j4 = 0; j4 < KB / 4; ++j4) {
              const float4 v = v4[j4];
              acc[4 * j4] = fmaf(xv[u], v.x, acc[4 * j4]);
              acc[4 * j4 + 1] = fmaf(xv[u], v.y, acc[4 * j4 + 1]);
              acc[4 * j4 + 2] = fmaf(xv[u], v.z, acc[4 * j4 + 2]);
              acc[4 * j4 + 3] = fmaf(xv[u], v.w, acc[4 * j4 + 3]);
            }
          }
        }
      }
    }
    if (valid)
#pragma unroll
      for (int j = 0; j < KB; ++j)
        if (j < kz) J.Z[row + total * j] = acc[j];
  }
}

// First core contraction: T1[row + rows a] = sum_i Z[i + np row] Up[i + np a],
// a < kp <= 4 M.  Block `blk` of `nblk` strides over tiles of 64 rows
// (consecutive rows of Z are contiguous); Z and Up staged in 64-wide chunks of
// i; thread (row t % 64, a = t / 64 + 4 m).
template <int M>
HT_DEV void core_t1_body(const T1Job &J, long long blk, long long nblk) {
  __shared__ float Zs[64][65];   // [i][row]
  __shared__ float Us[64][65];   // [i][a]
  const int t = threadIdx.x, np = J.np, kp = J.kp, rr = t & 63, ag = t >> 6;
  for (long long r0 = blk * 64; r0 < J.rows; r0 += nblk * 64) {
    const int nr = static_cast<int>(min(64ll, J.rows - r0));
    float acc[M];
#pragma unroll
    for (int m = 0; m < M; ++m) acc[m] = 0.f;
    for (int i0 = 0; i0 < np; i0 += 64) {
      const int ni = min(64, np - i0);
      __syncthreads();
      for (int e = t; e < 64 * 64; e += 256) {
        const int a = e >> 6, ii = e & 63;   // i fastest: contiguous reads of a Z row and of an Up column
        Zs[ii][a] = (ii < ni && a < nr) ? J.Z[(i0 + ii) + static_cast<long long>(np) * (r0 + a)] : 0.f;
        if (a < 4 * M) Us[ii][a] = (ii < ni && a < kp) ? J.Up[(i0 + ii) + static_cast<long long>(np) * a] : 0.f;
      }
      __syncthreads();
      for (int ii = 0; ii < ni; ++ii) {
        const float z = Zs[ii][rr];
#pragma unroll
        for (int m = 0; m < M; ++m) acc[m] = fmaf(z, Us[ii][ag + 4 * m], acc[m]);
      }
    }
    if (rr < nr)
#pragma unroll
      for (int m = 0; m < M; ++m) {
        const int a = ag + 4 * m;
        if (a < kp) J.T1[r0 + rr + J.rows * a] = acc[m];
      }
  }
}

// Grouped (batched path): the job of block b is job_of_block[b].
template <int M>
__global__ void __launch_bounds__(256) core_t1_grouped_kernel(const T1Job *__restrict__ jobs,
                                                              const int *__restrict__ job_of_block) {
  __shared__ T1Job J;
  load_job(jobs, job_of_block[blockIdx.x], J);
  core_t1_body<M>(J, blockIdx.x - J.blk0, J.nblk);
}

// Grouped second core-contraction step of the batched path: block b is
// entry c = b - blk0 of job job_of_block[b] (the whole j range).
__global__ void __launch_bounds__(256) core_step2_grouped_kernel(const Step2Job *__restrict__ jobs,
                                                                 const int *__restrict__ job_of_block) {
  __shared__ Step2Job J;
  if (threadIdx.x == 0) J = jobs[job_of_block[blockIdx.x]];
  __syncthreads();
  core_step2_body(J.T1, J.ldt, J.nq, J.kp, J.Uq, J.kq, static_cast<int>(blockIdx.x) - J.blk0, 0, J.nq, J.C);
}

// out[e] = sum_r part[r * count + e], r in order
__global__ void sum_parts_kernel(const float *__restrict__ part, int nparts, long long count, float *__restrict__ out) {
  for (long long e = blockIdx.x * 256ll + threadIdx.x; e < count; e += gridDim.x * 256ll) {
    float v = 0.f;
    for (int r = 0; r < nparts; ++r) v += part[static_cast<long long>(r) * count + e];
    out[e] = v;
  }
}

// W[i0 + n0*i1, c] = sum_{a,b} U0[i0,a] U1[i1,b] core[a + k0*b + k0*k1*c]
// step 1: T[i0, b, c] = sum_a U0[i0,a] core[a,b,c]
HT_DEV void expand_step1_body(const float *__restrict__ U0, int n0, int k0, const float *__restrict__ core, int k1,
                              int k2, float *__restrict__ T, long long blk, long long nblk) {
  const long long total = static_cast<long long>(n0) * k1 * k2;
  for (long long idx = blk * 256ll + threadIdx.x; idx < total; idx += nblk * 256ll) {
    const int i0 = static_cast<int>(idx % n0);
    const long long bc = idx / n0;   // b + k1*c
    float s = 0.f;
    for (int a = 0; a < k0; ++a) s = fmaf(U0[i0 + static_cast<long long>(n0) * a], core[a + k0 * bc], s);
    T[idx] = s;
  }
}
__global__ void expand_step1_kernel(const float *__restrict__ U0, int n0, int k0, const float *__restrict__ core,
                                    int k1, int k2, float *__restrict__ T) {
  expand_step1_body(U0, n0, k0, core, k1, k2, T, blockIdx.x, gridDim.x);
}
// step 2: W[i0 + n0*i1 + n0*n1*c] = sum_b T[i0 + n0*(b + k1*c)] U1[i1 + n1*b]
HT_DEV void expand_step2_body(const float *__restrict__ T, int n0, int k1, const float *__restrict__ U1, int n1, int k2,
                              float *__restrict__ W, long long blk, long long nblk) {
  const long long total = static_cast<long long>(n0) * n1 * k2;
  for (long long idx = blk * 256ll + threadIdx.x; idx < total; idx += nblk * 256ll) {
    const int i0 = static_cast<int>(idx % n0);
    const long long r = idx / n0;
    const int i1 = static_cast<int>(r % n1);
    const int c = static_cast<int>(r / n1);
    float s = 0.f;
    for (int b = 0; b < k1; ++b)
      s = fmaf(T[i0 + static_cast<long long>(n0) * (b + static_cast<long long>(k1) * c)], U1[i1 + static_cast<long long>(n1) * b], s);
    W[idx] = s;
  }
}
__global__ void expand_step2_kernel(const float *__restrict__ T, int n0, int k1, const float *__restrict__ U1, int n1,
                                    int k2, float *__restrict__ W) {
  expand_step2_body(T, n0, k1, U1, n1, k2, W, blockIdx.x, gridDim.x);
}

// C (m x n) = A (m x K) * B (K x n), column-major, small K and n
__global__ void matmul_nn_kernel(const float *__restrict__ A, long long lda, const float *__restrict__ B, int ldb,
                                 float *__restrict__ C, long long ldc, long long m, int n, int K) {
  const long long total = m * n;
  for (long long idx = blockIdx.x * 256ll + threadIdx.x; idx < total; idx += gridDim.x * 256ll) {
    const long long i = idx % m;
    const int j = static_cast<int>(idx / m);
    float s = 0.f;
    for (int k = 0; k < K; ++k) s = fmaf(A[i + lda * k], B[k + static_cast<long long>(ldb) * j], s);
    C[i + ldc * j] = s;
  }
}

// err partial over a 128 x 64 tile: sum (X[r + R*c] - sum_k A[r + R*k] B[c + Cn*k])^2.
// Thread layout: 32 row groups of 4 rows x 8 column groups of 8 columns, so a
// warp reads 128 consecutive rows of one column of X.
// Tile `tile` of slab `y` (X and A advanced by sx, sa per slab); the tile's
// partial goes to partials[tile + ntiles * y].
HT_DEV void error_fused_body(const float *__restrict__ X, long long ldx, long long sx, const float *__restrict__ A,
                             long long lda, long long sa, const float *__restrict__ B, long long ldb, long long R,
                             long long Cn, int kk, double *partials, long long tile, long long ntiles, long long y) {
  X += sx * y;
  A += sa * y;
  __shared__ __align__(16) float As[32][128];
  __shared__ float Bs[32][64];
  __shared__ double red[256];
  const long long tiles_r = (R + 127) / 128;
  const long long tr = tile % tiles_r, tc = tile / tiles_r;
  const long long r0 = tr * 128, c0 = tc * 64;
  const int t = threadIdx.x;
  const int rg = t % 32, cg = t / 32;
  float acc[4][8];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[i][j] = 0.f;
  for (int k0 = 0; k0 < kk; k0 += 32) {
    __syncthreads();
    for (int e = t; e < 32 * 128; e += 256) {
      const int rr = e % 128, k = e / 128;
      As[k][rr] = (k0 + k < kk && r0 + rr < R) ? A[r0 + rr + lda * (k0 + k)] : 0.f;
    }
    for (int e = t; e < 32 * 64; e += 256) {
      const int cc = e % 64, k = e / 64;
      Bs[k][cc] = (k0 + k < kk && c0 + cc < Cn) ? B[c0 + cc + ldb * (k0 + k)] : 0.f;
    }
    __syncthreads();
    const int kn = kk - k0 < 32 ? kk - k0 : 32;   // no products with the zero-padded k slices
#pragma unroll 4
    for (int k = 0; k < kn; ++k) {
      const float4 a4 = *reinterpret_cast<const float4 *>(&As[k][rg * 4]);
      const float a[4] = {a4.x, a4.y, a4.z, a4.w};
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const float b = Bs[k][cg * 8 + j];
#pragma unroll
        for (int i = 0; i < 4; ++i) acc[i][j] = fmaf(a[i], b, acc[i][j]);
      }
    }
  }
  Acc2 s = {0.f, 0.f};
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const long long c = c0 + cg * 8 + j;
    if (c >= Cn) continue;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const long long r = r0 + rg * 4 + i;
      if (r >= R) continue;
      const float d = __ldcs(X + r + ldx * c) - acc[i][j];
      acc2_add_prod(s, d, d);
    }
  }
  red[t] = static_cast<double>(s.s) + static_cast<double>(s.c);
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (t < w) red[t] += red[t + w];
    __syncthreads();
  }
  if (t == 0) partials[tile + ntiles * y] = red[0];
}

__global__ void __launch_bounds__(256) error_fused_kernel(const float *__restrict__ X, long long ldx, long long sx,
                                                          const float *__restrict__ A, long long lda, long long sa,
                                                          const float *__restrict__ B, long long ldb, long long R,
                                                          long long Cn, int kk, double *partials) {
  error_fused_body(X, ldx, sx, A, lda, sa, B, ldb, R, Cn, kk, partials, blockIdx.x, gridDim.x, blockIdx.y);
}

// Grouped error pass of the batched path (3rd order), one launch per step
// for every job; job_of_block[step] maps a block of launch `step` to its job.

// step 0: core (kpq x kc) = Bt (kpq x kt) Bkt (kt x kc); Bkt is B0 itself when
// t is the root's left child, else B0 is its transpose (kc x kt)
__global__ void __launch_bounds__(256) err_core_grouped_kernel(const ErrJob *__restrict__ jobs, const int *__restrict__ job_of_block) {
  __shared__ ErrJob J;
  load_job(jobs, job_of_block[blockIdx.x], J);
  const long long b = blockIdx.x - J.blk0[0], total = J.kpq * J.kc;
  for (long long idx = b * 256 + threadIdx.x; idx < total; idx += J.nblk[0] * 256ll) {
    const long long i = idx % J.kpq;
    const int u = static_cast<int>(idx / J.kpq);
    float s = 0.f;
    for (int r = 0; r < J.kt; ++r)
      s = fmaf(J.Bt[i + J.kpq * r], J.t_is_left ? J.B0[r + J.kt * u] : J.B0[u + J.kc * r], s);
    J.core[idx] = s;
  }
}

__global__ void __launch_bounds__(256) err_expand1_grouped_kernel(const ErrJob *__restrict__ jobs, const int *__restrict__ job_of_block) {
  __shared__ ErrJob J;
  load_job(jobs, job_of_block[blockIdx.x], J);
  expand_step1_body(J.Up, J.np, J.kp, J.core, J.kq, J.kc, J.Tm, blockIdx.x - J.blk0[1], J.nblk[1]);
}

__global__ void __launch_bounds__(256) err_expand2_grouped_kernel(const ErrJob *__restrict__ jobs, const int *__restrict__ job_of_block) {
  __shared__ ErrJob J;
  load_job(jobs, job_of_block[blockIdx.x], J);
  expand_step2_body(J.Tm, J.np, J.kq, J.Uq, J.nq, J.kc, J.Wm, blockIdx.x - J.blk0[2], J.nblk[2]);
}

__global__ void __launch_bounds__(256) err_fused_grouped_kernel(const ErrJob *__restrict__ jobs, const int *__restrict__ job_of_block) {
  __shared__ ErrJob J;
  load_job(jobs, job_of_block[blockIdx.x], J);
  const long long ntiles = J.ntile / J.slabs;
  for (long long tb = blockIdx.x - J.blk0[3]; tb < J.ntile; tb += J.nblk[3])
    error_fused_body(J.X, J.ldx, J.sx, J.A, J.lda, J.sa, J.B, J.ldb, J.R, J.Cn, J.kk, J.parts, tb % ntiles, ntiles,
                     tb / ntiles);
}

// Expansion of a narrow error job: W[i1 + np i2 + L c] = sum_b T[i1 + np (b + kq c)]
// Uq[i2 + nq b] (L = np nq), kq <= KQ.  Block (c, i1 range of 256): a thread
// per i1 keeps its row of T_c in registers, Uq is staged in 64-row chunks of
// shared memory, and the thread loops over every i2.
template <int KQ>
__global__ void __launch_bounds__(256) err_expand2w_grouped_kernel(const ErrJob *__restrict__ jobs,
                                                                   const int *__restrict__ job_of_block) {
  __shared__ ErrJob J;
  __shared__ float Us[64][KQ + 1];
  load_job(jobs, job_of_block[blockIdx.x], J);
  const int np = J.np, nq = J.nq, kq = J.kq, t = threadIdx.x;
  const int chunks = (np + 255) / 256;
  const int b = blockIdx.x - J.blk0[5], c = b / chunks, i1 = (b - c * chunks) * 256 + t;
  const bool valid = i1 < np;
  const long long L = static_cast<long long>(np) * nq;
  float tr[KQ];
#pragma unroll
  for (int q = 0; q < KQ; ++q)
    tr[q] = (valid && q < kq) ? J.Tm[i1 + static_cast<long long>(np) * (q + static_cast<long long>(kq) * c)] : 0.f;
  for (int j0 = 0; j0 < nq; j0 += 64) {
    const int nj = min(64, nq - j0);
    __syncthreads();
    for (int e = t; e < 64 * KQ; e += 256) {
      const int jj = e / KQ, q = e - jj * KQ;
      Us[jj][q] = (jj < nj && q < kq) ? J.Uq[(j0 + jj) + static_cast<long long>(nq) * q] : 0.f;
    }
    __syncthreads();
    if (valid)
      for (int jj = 0; jj < nj; ++jj) {
        float v = 0.f;
#pragma unroll
        for (int q = 0; q < KQ; ++q) v = fmaf(tr[q], Us[jj][q], v);
        J.Wm[i1 + static_cast<long long>(np) * (j0 + jj) + L * c] = v;
      }
  }
}

// Narrow error pass (complementary leaf = the last mode, rows l = i1 + np i2
// of X contiguous): a thread per row takes its row W[l, :] of the expansion,
// then for every i3 the difference
// X[l + L i3] - sum_c W[l, c] U3[i3 + nc c] (U3 staged in 64-row chunks of
// shared memory); the compensated sum of squares of a block's rows is its
// partial (ntile = nblk[4] partials).
template <int KB>
__global__ void __launch_bounds__(256) err_narrow_grouped_kernel(const ErrJob *__restrict__ jobs,
                                                                 const int *__restrict__ job_of_block) {
  __shared__ ErrJob J;
  __shared__ __align__(16) float Us[64][KB];
  __shared__ double red[256];
  load_job(jobs, job_of_block[blockIdx.x], J);
  const int t = threadIdx.x, kc = J.kc, np = J.np, kq = J.kq;
  const long long L = J.R, nc = J.Cn;
  const long long b = blockIdx.x - J.blk0[4];
  Acc2 acc = {0.f, 0.f};
  for (long long base = b * 256; base < L; base += J.nblk[4] * 256ll) {
    const long long l = base + t;
    const bool valid = l < L;
    const int i1 = valid ? static_cast<int>(l % np) : 0, i2 = valid ? static_cast<int>(l / np) : 0;
    float w[KB];   // this row of the expansion (err_expand2w_grouped_kernel)
#pragma unroll
    for (int c = 0; c < KB; ++c) w[c] = (valid && c < kc) ? J.Wm[l + L * c] : 0.f;
    for (long long i0 = 0; i0 < nc; i0 += 64) {
      const int ni = static_cast<int>(min(64ll, nc - i0));
      __syncthreads();
      for (int e = t; e < 64 * KB; e += 256) {
        const int ii = e / KB, c = e - ii * KB;
        Us[ii][c] = (ii < ni && c < kc) ? J.B[(i0 + ii) + J.ldb * c] : 0.f;
      }
      __syncthreads();
      if (valid)
        for (int ii = 0; ii < ni; ii += 8) {
          float xv[8];   // eight independent loads in flight before the products
#pragma unroll
          for (int u = 0; u < 8; ++u) xv[u] = ii + u < ni ? __ldcs(J.X + l + L * (i0 + ii + u)) : 0.f;
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            if (ii + u < ni) {
              const float4 *u4 = reinterpret_cast<const float4 *>(&Us[ii + u][0]);
              float xh = 0.f;
#pragma unroll
              for (int c4 = 0; c4 < KB / 4; ++c4) {
                const float4 v = u4[c4];
                xh = fmaf(w[4 * c4], v.x, xh);
                xh = fmaf(w[4 * c4 + 1], v.y, xh);
                xh = fmaf(w[4 * c4 + 2], v.z, xh);
                xh = fmaf(w[4 * c4 + 3], v.w, xh);
              }
              const float d = xv[u] - xh;
              acc2_add_prod(acc, d, d);
            }
          }
        }
    }
  }
  red[t] = static_cast<double>(acc.s) + static_cast<double>(acc.c);
  __syncthreads();
  for (int w2 = 128; w2 > 0; w2 >>= 1) {
    if (t < w2) red[t] += red[t + w2];
    __syncthreads();
  }
  if (t == 0) J.parts[b] = red[0];
}

// the sum of a job's tile partials, as sumsq_finish_kernel sums them
__global__ void err_finish_grouped_kernel(const ErrJob *__restrict__ jobs) {
  const ErrJob &J = jobs[blockIdx.x];
  __shared__ double red[256];
  double s = 0.0;
  for (int i = threadIdx.x; i < J.ntile; i += 256) s += J.parts[i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) J.out[0] = red[0];
}

__global__ void gaussian_fill_kernel(float *dst, long long n, unsigned long long seed, unsigned long long stream) {
  for (long long i = blockIdx.x * 256ll + threadIdx.x; i < n; i += gridDim.x * 256ll) dst[i] = gaussian(seed, stream, i);
}

__global__ void transpose_small_kernel(const float *A, int m, int n, float *AT) {
  for (int idx = blockIdx.x * 256 + threadIdx.x; idx < m * n; idx += gridDim.x * 256) {
    const int i = idx % m, j = idx / m;
    AT[j + n * i] = A[i + m * j];
  }
}

}  // namespace

// Multiprocessor count of the current device (cached per device).
int device_sm_count() {
  static int cached[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
    cudaGetLastError();
    return 1;
  }
  if (cached[dev] <= 0) {
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) {
      cudaGetLastError();
      v = 1;
    }
    cached[dev] = v;
  }
  return cached[dev];
}

namespace {

int grid_for(long long n, int cap = 0) {
  if (cap <= 0) cap = 8 * device_sm_count();
  long long g = (n + 255) / 256;
  if (g < 1) g = 1;
  if (g > cap) g = cap;
  return static_cast<int>(g);
}

}  // namespace

cudaError_t convert_bf16_pad_launch(const float *x, __nv_bfloat16 *xp, long long n1, long long n1p, long long rest,
                                    double *partials, int num_partials, cudaStream_t s) {
  if (n1 < 1 || n1p < n1 || rest < 1 || num_partials < 1) return cudaErrorInvalidValue;
  convert_bf16_pad_kernel<<<num_partials, 256, 0, s>>>(x, xp, n1, n1p, rest, partials);
  return cudaGetLastError();
}

cudaError_t convert_bf16_launch(const float *x, __nv_bfloat16 *xb, long long n, double *partials, int num_partials,
                                cudaStream_t s) {
  if (reinterpret_cast<uintptr_t>(x) % 16 == 0 && reinterpret_cast<uintptr_t>(xb) % 8 == 0)
    convert_bf16_kernel<<<num_partials, 256, 0, s>>>(x, xb, n, partials);
  else
    return cudaErrorInvalidValue;
  return cudaGetLastError();
}

cudaError_t convert_bf16_dual_launch(const float *x, __nv_bfloat16 *xb, __nv_bfloat16 *xbt, long long L, long long N,
                                     int lb, double *partials, int num_partials, cudaStream_t s, long long n_begin,
                                     long long n_count) {
  const int TN = 1 << (12 - lb);
  if (n_count < 0) n_count = N - n_begin;
  if (lb < 6 || lb > 12 || L % (1ll << lb) || N < TN || N % TN || n_begin < 0 || n_begin % TN || n_count % TN ||
      n_begin + n_count > N || num_partials < 1 || num_partials > 4096 ||
      (reinterpret_cast<uintptr_t>(x) & 15u) || (reinterpret_cast<uintptr_t>(xb) & 7u) ||
      (reinterpret_cast<uintptr_t>(xbt) & 7u))
    return cudaErrorInvalidValue;
  convert_bf16_dual_kernel<<<num_partials, 256, 0, s>>>(x, xb, xbt, L, N, n_begin, n_count, lb, partials);
  return cudaGetLastError();
}

cudaError_t accumulate_launch(float *dst, const float *src, long long n, int first, cudaStream_t s) {
  accumulate_kernel<<<grid_for(n), 256, 0, s>>>(dst, src, n, first);
  return cudaGetLastError();
}

cudaError_t sumsq_launch(const float *x, long long n, double *partials, int num_partials, cudaStream_t s) {
  sumsq_kernel<<<num_partials, 256, 0, s>>>(x, n, partials);
  return cudaGetLastError();
}

cudaError_t f32_to_bf16_launch(const float *x, __nv_bfloat16 *y, long long n, cudaStream_t s) {
  f32_to_bf16_kernel<<<grid_for(n), 256, 0, s>>>(x, y, n);
  return cudaGetLastError();
}

cudaError_t round_bf16_launch(float *x, __nv_bfloat16 *y, long long n, cudaStream_t s) {
  round_bf16_kernel<<<grid_for(n), 256, 0, s>>>(x, y, n);
  return cudaGetLastError();
}

cudaError_t split_bf16_launch(const float *W, long long rows, int k, int h, __nv_bfloat16 *Y, cudaStream_t s) {
  split_bf16_kernel<<<grid_for(rows * 2 * h), 256, 0, s>>>(W, rows, k, h, Y);
  return cudaGetLastError();
}

cudaError_t convert_grouped_launch(const ConvJob *jobs_dev, int njobs, int total_blocks, const int *job_of_block,
                                   cudaStream_t s) {
  if (njobs < 1) return cudaSuccess;
  if (!jobs_dev || !job_of_block || total_blocks < njobs) return cudaErrorInvalidValue;
  convert_grouped_kernel<<<total_blocks, 256, 0, s>>>(jobs_dev, job_of_block);
  convert_grouped_finish_kernel<<<njobs, 256, 0, s>>>(jobs_dev);
  return cudaGetLastError();
}

cudaError_t copy_segments_launch(const CopySeg *segs_dev, int nseg, cudaStream_t s) {
  if (nseg < 1) return cudaSuccess;
  if (!segs_dev) return cudaErrorInvalidValue;
  copy_segments_kernel<<<nseg, 256, 0, s>>>(segs_dev);
  return cudaGetLastError();
}

cudaError_t sumsq_finish_launch(const double *partials, int n, double *out, cudaStream_t s) {
  sumsq_finish_kernel<<<1, 256, 0, s>>>(partials, n, out);
  return cudaGetLastError();
}

cudaError_t gemm_tn_small_launch(const float *A, int lda, const float *B, int ldb, float *C, int ldc, int m, int n,
                                 int K, cudaStream_t s) {
  const long long warps = static_cast<long long>(m) * n;
  const int blocks = static_cast<int>((warps * 32 + 255) / 256);
  gemm_tn_small_kernel<<<blocks, 256, 0, s>>>(A, lda, B, ldb, C, ldc, m, n, K);
  return cudaGetLastError();
}

int core_step2_ranges(int nq, int kc) {
  const int chunks64 = (nq + 63) / 64;
  int want = (2 * device_sm_count() + kc - 1) / kc;
  if (want > chunks64) want = chunks64;
  if (want < 1) want = 1;
  const int per = (chunks64 + want - 1) / want;   // 64-blocks of j per range
  return (chunks64 + per - 1) / per;
}

cudaError_t core_step2_launch(const float *T1, long long ldt, int nq, int kp, const float *Uq, int kq, int kc, float *C,
                              float *scratch, cudaStream_t s) {
  if (kp > 64 || kq > 64 || kp * kq > 16 * 256) return cudaErrorInvalidValue;
  const int ranges = scratch ? core_step2_ranges(nq, kc) : 1;
  const int chunks64 = (nq + 63) / 64;
  const int jc = 64 * ((chunks64 + ranges - 1) / ranges);
  core_step2_kernel<<<dim3(kc, ranges), 256, 0, s>>>(T1, ldt, nq, kp, Uq, kq, jc, ranges > 1 ? scratch : C);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || ranges == 1) return e;
  const long long count = static_cast<long long>(kp) * kq * kc;
  sum_parts_kernel<<<grid_for(count), 256, 0, s>>>(scratch, ranges, count, C);
  return cudaGetLastError();
}

cudaError_t modeprod_narrow_grouped_launch(const NarrowJob *jobs_dev, const int *job_of_block, int nblocks, int kb,
                                          cudaStream_t s) {
  if (nblocks < 1) return cudaSuccess;
  if (!jobs_dev || !job_of_block) return cudaErrorInvalidValue;
  if (kb <= 16) modeprod_narrow_grouped_kernel<16><<<nblocks, 256, 0, s>>>(jobs_dev, job_of_block);
  else if (kb <= 32) modeprod_narrow_grouped_kernel<32><<<nblocks, 256, 0, s>>>(jobs_dev, job_of_block);
  else if (kb <= 64) modeprod_narrow_grouped_kernel<64><<<nblocks, 256, 0, s>>>(jobs_dev, job_of_block);
  else return cudaErrorInvalidValue;
  return cudaGetLastError();
}

cudaError_t core_t1_grouped_launch(const T1Job *jobs_dev, const int *job_of_block, int nblocks, int kp_max,
                                   cudaStream_t s) {
  if (nblocks < 1) return cudaSuccess;
  if (!jobs_dev || !job_of_block) return cudaErrorInvalidValue;
  if (kp_max <= 16) core_t1_grouped_kernel<4><<<nblocks, 256, 0, s>>>(jobs_dev, job_of_block);
  else if (kp_max <= 32) core_t1_grouped_kernel<8><<<nblocks, 256, 0, s>>>(jobs_dev, job_of_block);
  else if (kp_max <= 64) core_t1_grouped_kernel<16><<<nblocks, 256, 0, s>>>(jobs_dev, job_of_block);
  else return cudaErrorInvalidValue;
  return cudaGetLastError();
}

cudaError_t core_step2_grouped_launch(const Step2Job *jobs_dev, const int *job_of_block, int nblocks, cudaStream_t s) {
  if (nblocks < 1) return cudaSuccess;
  if (!jobs_dev || !job_of_block) return cudaErrorInvalidValue;
  core_step2_grouped_kernel<<<nblocks, 256, 0, s>>>(jobs_dev, job_of_block);
  return cudaGetLastError();
}

cudaError_t expand2_launch(const float *U0, int n0, int k0, const float *core, const float *U1, int n1, int k1, int k2,
                           float *T, float *W, cudaStream_t s) {
  expand_step1_kernel<<<grid_for(static_cast<long long>(n0) * k1 * k2), 256, 0, s>>>(U0, n0, k0, core, k1, k2, T);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  expand_step2_kernel<<<grid_for(static_cast<long long>(n0) * n1 * k2), 256, 0, s>>>(T, n0, k1, U1, n1, k2, W);
  return cudaGetLastError();
}

cudaError_t matmul_nn_launch(const float *A, long long lda, const float *B, int ldb, float *C, long long ldc,
                             long long m, int n, int K, cudaStream_t s) {
  matmul_nn_kernel<<<grid_for(m * n), 256, 0, s>>>(A, lda, B, ldb, C, ldc, m, n, K);
  return cudaGetLastError();
}

int error_fused_blocks(long long R, long long Cn) { return static_cast<int>(((R + 127) / 128) * ((Cn + 63) / 64)); }

cudaError_t error_fused_launch(const float *X, long long ldx, long long sx, const float *A, long long lda, long long sa,
                               const float *B, long long ldb, long long R, long long Cn, int kk, int batch,
                               double *partials, cudaStream_t s) {
  if (kk > 64 || batch < 1 || batch > 65535) return cudaErrorInvalidValue;
  error_fused_kernel<<<dim3(error_fused_blocks(R, Cn), batch), 256, 0, s>>>(X, ldx, sx, A, lda, sa, B, ldb, R, Cn, kk,
                                                                           partials);
  return cudaGetLastError();
}

cudaError_t error_grouped_launch(const ErrJob *jobs_dev, int njobs, const int *blocks, const int *const *job_of_block,
                                 int narrow_kb, int narrow_kq, cudaStream_t s) {
  if (njobs < 1) return cudaSuccess;
  if (!jobs_dev) return cudaErrorInvalidValue;
  for (int k = 0; k < 6; ++k)
    if (blocks[k] > 0 && !job_of_block[k]) return cudaErrorInvalidValue;
  if (blocks[0] < njobs || blocks[1] < njobs) return cudaErrorInvalidValue;
  err_core_grouped_kernel<<<blocks[0], 256, 0, s>>>(jobs_dev, job_of_block[0]);
  err_expand1_grouped_kernel<<<blocks[1], 256, 0, s>>>(jobs_dev, job_of_block[1]);
  if (blocks[5] > 0) {
    if (narrow_kq <= 16) err_expand2w_grouped_kernel<16><<<blocks[5], 256, 0, s>>>(jobs_dev, job_of_block[5]);
    else if (narrow_kq <= 32) err_expand2w_grouped_kernel<32><<<blocks[5], 256, 0, s>>>(jobs_dev, job_of_block[5]);
    else if (narrow_kq <= 64) err_expand2w_grouped_kernel<64><<<blocks[5], 256, 0, s>>>(jobs_dev, job_of_block[5]);
    else return cudaErrorInvalidValue;
  }
  if (blocks[2] > 0) err_expand2_grouped_kernel<<<blocks[2], 256, 0, s>>>(jobs_dev, job_of_block[2]);
  if (blocks[3] > 0) err_fused_grouped_kernel<<<blocks[3], 256, 0, s>>>(jobs_dev, job_of_block[3]);
  if (blocks[4] > 0) {
    if (narrow_kb <= 16) err_narrow_grouped_kernel<16><<<blocks[4], 256, 0, s>>>(jobs_dev, job_of_block[4]);
    else if (narrow_kb <= 32) err_narrow_grouped_kernel<32><<<blocks[4], 256, 0, s>>>(jobs_dev, job_of_block[4]);
    else if (narrow_kb <= 64) err_narrow_grouped_kernel<64><<<blocks[4], 256, 0, s>>>(jobs_dev, job_of_block[4]);
    else return cudaErrorInvalidValue;
  }
  err_finish_grouped_kernel<<<njobs, 256, 0, s>>>(jobs_dev);
  return cudaGetLastError();
}

cudaError_t gaussian_fill_launch(float *dst, long long n, uint64_t seed, uint64_t stream, cudaStream_t s) {
  gaussian_fill_kernel<<<grid_for(n), 256, 0, s>>>(dst, n, seed, stream);
  return cudaGetLastError();
}

cudaError_t transpose_small_launch(const float *A, int m, int n, float *AT, cudaStream_t s) {
  transpose_small_kernel<<<grid_for(static_cast<long long>(m) * n), 256, 0, s>>>(A, m, n, AT);
  return cudaGetLastError();
}

}  // namespace htgb
