// Learned per-mode sketch: forward and adjoint kernels.
//
// A sketch S (n x s) is the test matrix of the leaf range finder on a mode
// Gram G = X_(t) X_(t)^T: Y = G S, Q = orth(Y) (CholeskyQR, Y = Q R), and the
// leaf basis is the top-k Rayleigh-Ritz vectors of span(Q) (the eigen-solver
// with start block S and one iteration).  Training minimises, over a family of
// Grams, the energy the subspace misses:
//
//   L(S) = mean_b [ 1 - tr(Q_b^T G_b Q_b) / tr(G_b) ]
//        = mean_b [ 1 - tr(C_b^-1 H_b) / tr(G_b) ],   C = Y^T Y = R^T R,  H = Y^T G Y,
//
// with C and H restricted to the columns of Y that the CholeskyQR keeps (a
// column in the span of the earlier ones to rounding is left out, see kDrop).
//
// Its adjoint through CholeskyQR (dC, dH back to dY, then dS = G dY):
//
//   dL/dS = -(2 / B) sum_b G_b E_b C_b^-1 / tr(G_b),   E = G Y - Y C^-1 H = (I - Q Q^T) G Q R.
//
// Kernels: a batched n x n by n x s product (FP32, the three large products),
// a per-Gram kernel for the s x s algebra (C and H accumulated in FP64, FP64
// Cholesky and solves, E formed in FP64), and a deterministic batch reduction
// of the gradient, plus an Adam step.  The reference has no learned component;
// the Gaussian start block it would use (the rsvd test matrix,
// 3D/Opt/kernel.cu:595-680) is what the learned sketch replaces.
#include "common.cuh"
#include "engine.h"

namespace htgb {
namespace {

constexpr int LS_MAX = 64;    // sketch width limit
constexpr int LT_ROWS = 64;   // rows per CTA of the batched product
constexpr int LT_K = 32;      // k chunk

// out[b] (n x s) = G[b] (n x n) * M[b] (n x s), column-major; M is shared by
// the batch when m_stride == 0.
__global__ void __launch_bounds__(256) ls_bgemm_kernel(const float *__restrict__ G, const float *__restrict__ M,
                                                       long long m_stride, float *__restrict__ out, int n, int s) {
  __shared__ float Gs[LT_K][LT_ROWS + 1];
  __shared__ float Ms[LT_K][LS_MAX + 1];
  const int b = blockIdx.y, r0 = blockIdx.x * LT_ROWS, t = threadIdx.x;
  const float *Gb = G + static_cast<long long>(b) * n * n;
  const float *Mb = M + static_cast<long long>(b) * m_stride;
  float *Ob = out + static_cast<long long>(b) * n * s;
  const int r = t & 63, cg = t >> 6;   // row, column group (columns cg + 4 j)
  float acc[16];
#pragma unroll
  for (int j = 0; j < 16; ++j) acc[j] = 0.f;
  for (int k0 = 0; k0 < n; k0 += LT_K) {
    for (int e = t; e < LT_K * LT_ROWS; e += 256) {
      const int rr = e % LT_ROWS, kk = e / LT_ROWS;
      Gs[kk][rr] = (r0 + rr < n && k0 + kk < n) ? Gb[(r0 + rr) + static_cast<long long>(n) * (k0 + kk)] : 0.f;
    }
    for (int e = t; e < LT_K * LS_MAX; e += 256) {
      const int kk = e % LT_K, c = e / LT_K;
      Ms[kk][c] = (c < s && k0 + kk < n) ? Mb[(k0 + kk) + static_cast<long long>(n) * c] : 0.f;
    }
    __syncthreads();
#pragma unroll 8
    for (int kk = 0; kk < LT_K; ++kk) {
      const float g = Gs[kk][r];
#pragma unroll
      for (int j = 0; j < 16; ++j) acc[j] = fmaf(g, Ms[kk][cg + 4 * j], acc[j]);
    }
    __syncthreads();
  }
  if (r0 + r < n) {
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      const int c = cg + 4 * j;
      if (c < s) Ob[(r0 + r) + static_cast<long long>(n) * c] = acc[j];
    }
  }
}

// A column of Y whose pivot (Schur complement) is below kDrop times its
// squared norm lies in the span of the earlier columns to rounding and is left
// out of Q: Y = G S is rank deficient whenever the Gram's rank is below the
// sketch width (the separable-bumps family: rank <= 32 < 34), and keeping such
// a column would turn rounding noise into a basis vector (and the loss
// negative).  The oracle (sketch_loss) applies the same rule.
constexpr double kDrop = 1e-8;

// In-place Cholesky C = R^T R of an s x s FP64 matrix (upper triangle of A,
// row-major stride LS_MAX) by one CTA, dropping dependent columns: a dropped
// column j gets R[j, j] = 1 and a zero row, and keep[j] = 0.  *s_bad is set
// on a non-finite pivot.
__device__ void ls_cholesky(double *A, int s, int *keep, double *d0, int *s_bad) {
  const int t = threadIdx.x;
  if (t == 0) *s_bad = 0;
  for (int j = t; j < s; j += 256) d0[j] = A[j * LS_MAX + j];
  __syncthreads();
  for (int j = 0; j < s; ++j) {
    if (t == 0) {
      const double d = A[j * LS_MAX + j];
      if (!isfinite(d)) *s_bad = 1;
      keep[j] = d > kDrop * d0[j] ? 1 : 0;
      A[j * LS_MAX + j] = keep[j] ? sqrt(d) : 1.0;
    }
    __syncthreads();
    const double inv = keep[j] ? 1.0 / A[j * LS_MAX + j] : 0.0;
    for (int k = j + 1 + t; k < s; k += 256) A[j * LS_MAX + k] *= inv;
    __syncthreads();
    if (keep[j])
      for (int e = t; e < (s - j - 1) * (s - j - 1); e += 256) {
        const int i = j + 1 + e / (s - j - 1), k = j + 1 + e % (s - j - 1);
        if (k >= i) A[i * LS_MAX + k] -= A[j * LS_MAX + i] * A[j * LS_MAX + k];
      }
    __syncthreads();
  }
}

// Per Gram b: C = Y^T Y, H = Y^T P (FP64 accumulation), X = C_KK^-1 H_KK on the
// kept columns K (zero rows and columns elsewhere), loss_b = 1 - tr(X) / trG_b,
// E = P - Y X, and Ci = C_KK^-1 (FP64, zero outside K) for the gradient.  One
// CTA per Gram.
__global__ void __launch_bounds__(256) ls_small_kernel(const float *__restrict__ Y, const float *__restrict__ P,
                                                       const float *__restrict__ trG, int n, int s,
                                                       float *__restrict__ E, double *__restrict__ Ci,
                                                       double *__restrict__ loss, int *__restrict__ bad) {
  extern __shared__ double ls_sm[];
  double *C = ls_sm;                        // LS_MAX x LS_MAX
  double *W = ls_sm + LS_MAX * LS_MAX;      // H, then X = C^-1 H
  __shared__ int s_bad;
  __shared__ int keep[LS_MAX];
  __shared__ double d0[LS_MAX];
  const int b = blockIdx.x, t = threadIdx.x;
  const float *Yb = Y + static_cast<long long>(b) * n * s;
  const float *Pb = P + static_cast<long long>(b) * n * s;
  for (int e = t; e < s * s; e += 256) {
    const int i = e / s, j = e % s;
    double c = 0.0, h = 0.0;
    for (int r = 0; r < n; ++r) {
      const double yi = Yb[r + static_cast<long long>(n) * i];
      c = fma(yi, static_cast<double>(Yb[r + static_cast<long long>(n) * j]), c);
      h = fma(yi, static_cast<double>(Pb[r + static_cast<long long>(n) * j]), h);
    }
    C[i * LS_MAX + j] = c;
    W[i * LS_MAX + j] = h;
  }
  __syncthreads();
  ls_cholesky(C, s, keep, d0, &s_bad);
  if (s_bad && t == 0) atomicOr(bad, 1);
  // X = R^-1 R^-T H on K: forward substitution with R^T, then back substitution
  // with R (column per thread); dropped rows and columns are zero
  for (int j = t; j < s; j += 256) {
    for (int i = 0; i < s; ++i) {   // R^T z = h
      double v = (keep[i] && keep[j]) ? W[i * LS_MAX + j] : 0.0;
      if (keep[i])
        for (int k = 0; k < i; ++k) v -= C[k * LS_MAX + i] * W[k * LS_MAX + j];
      W[i * LS_MAX + j] = keep[i] ? v / C[i * LS_MAX + i] : 0.0;
    }
    for (int i = s - 1; i >= 0; --i) {   // R x = z
      double v = W[i * LS_MAX + j];
      if (keep[i])
        for (int k = i + 1; k < s; ++k) v -= C[i * LS_MAX + k] * W[k * LS_MAX + j];
      W[i * LS_MAX + j] = keep[i] ? v / C[i * LS_MAX + i] : 0.0;
    }
  }
  __syncthreads();
  // C_KK^-1 = R^-1 R^-T on K, column j by thread j
  double *Cib = Ci + static_cast<long long>(b) * LS_MAX * LS_MAX;
  for (int j = t; j < s; j += 256) {
    double z[LS_MAX];
    for (int i = 0; i < s; ++i) {   // R^T z = e_j
      double v = (i == j && keep[j]) ? 1.0 : 0.0;
      if (keep[i])
        for (int k = 0; k < i; ++k) v -= C[k * LS_MAX + i] * z[k];
      z[i] = keep[i] ? v / C[i * LS_MAX + i] : 0.0;
    }
    for (int i = s - 1; i >= 0; --i) {   // R x = z
      double v = z[i];
      if (keep[i])
        for (int k = i + 1; k < s; ++k) v -= C[i * LS_MAX + k] * Cib[k * LS_MAX + j];
      Cib[i * LS_MAX + j] = keep[i] ? v / C[i * LS_MAX + i] : 0.0;
    }
  }
  if (t == 0) {
    double tr = 0.0;
    for (int i = 0; i < s; ++i) tr += W[i * LS_MAX + i];
    loss[b] = 1.0 - tr / static_cast<double>(trG[b]);
  }
  // E = P - Y X (columns outside K are multiplied by zero rows of Ci later)
  float *Eb = E + static_cast<long long>(b) * n * s;
  for (int e = t; e < n * s; e += 256) {
    const int r = e % n, j = e / n;
    double v = Pb[r + static_cast<long long>(n) * j];
    for (int k = 0; k < s; ++k) v -= static_cast<double>(Yb[r + static_cast<long long>(n) * k]) * W[k * LS_MAX + j];
    Eb[e] = static_cast<float>(v);
  }
}

// grad[r, j] = -(2 / B) sum_b (1 / trG_b) sum_k GE_b[r, k] Ci_b[k, j], batch summed in order.
__global__ void __launch_bounds__(256) ls_grad_kernel(const float *__restrict__ GE, const double *__restrict__ Ci,
                                                      const float *__restrict__ trG, int batch, int n, int s,
                                                      float *__restrict__ grad) {
  const long long e = blockIdx.x * 256ll + threadIdx.x;
  if (e >= static_cast<long long>(n) * s) return;
  const int r = static_cast<int>(e % n), j = static_cast<int>(e / n);
  double acc = 0.0;
  for (int b = 0; b < batch; ++b) {
    const float *GEb = GE + static_cast<long long>(b) * n * s;
    const double *Cib = Ci + static_cast<long long>(b) * LS_MAX * LS_MAX;
    double v = 0.0;
    for (int k = 0; k < s; ++k) v = fma(static_cast<double>(GEb[r + static_cast<long long>(n) * k]), Cib[k * LS_MAX + j], v);
    acc += v / static_cast<double>(trG[b]);
  }
  grad[e] = static_cast<float>(-2.0 * acc / batch);
}

__global__ void ls_adam_kernel(float *__restrict__ S, const float *__restrict__ g, float *__restrict__ m,
                               float *__restrict__ v, long long count, float lr, float b1, float b2, float eps,
                               float c1, float c2) {
  const long long i = blockIdx.x * 256ll + threadIdx.x;
  if (i >= count) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  S[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

}  // namespace

size_t sketch_workspace_bytes(int batch, int n, int s) {
  const size_t ns = static_cast<size_t>(n) * s * batch;
  return 4 * ns * sizeof(float) + static_cast<size_t>(batch) * LS_MAX * LS_MAX * sizeof(double) +
         static_cast<size_t>(batch) * sizeof(double) + 256;
}

cudaError_t sketch_loss_grad(const float *G, const float *trG, int batch, int n, int s, const float *S, float *grad,
                             double *loss, int *bad, void *ws, cudaStream_t st, int *launches) {
  if (s < 1 || s > LS_MAX || n < s || batch < 1) return cudaErrorInvalidValue;
  const size_t ns = static_cast<size_t>(n) * s * batch;
  float *Y = static_cast<float *>(ws), *P = Y + ns, *E = P + ns, *GE = E + ns;
  double *Ci = reinterpret_cast<double *>(GE + ns);
  const dim3 grid((n + LT_ROWS - 1) / LT_ROWS, batch);
  ls_bgemm_kernel<<<grid, 256, 0, st>>>(G, S, 0, Y, n, s);                                   // Y = G S
  ls_bgemm_kernel<<<grid, 256, 0, st>>>(G, Y, static_cast<long long>(n) * s, P, n, s);       // P = G Y
  static bool attr_set[64] = {};
  constexpr int kSmallSmem = 2 * LS_MAX * LS_MAX * sizeof(double);
  {
    const cudaError_t e = opt_in_smem(ls_small_kernel, kSmallSmem, attr_set);
    if (e != cudaSuccess) return e;
  }
  ls_small_kernel<<<batch, 256, kSmallSmem, st>>>(Y, P, trG, n, s, E, Ci, loss, bad);     // E, C^-1, loss
  ls_bgemm_kernel<<<grid, 256, 0, st>>>(G, E, static_cast<long long>(n) * s, GE, n, s);      // G E
  const long long cnt = static_cast<long long>(n) * s;
  ls_grad_kernel<<<static_cast<int>((cnt + 255) / 256), 256, 0, st>>>(GE, Ci, trG, batch, n, s, grad);
  if (launches) *launches += 5;
  return cudaGetLastError();
}

cudaError_t sketch_adam(float *S, const float *g, float *m, float *v, long long count, float lr, float b1, float b2,
                        float eps, int step, cudaStream_t st) {
  const float c1 = 1.f - powf(b1, static_cast<float>(step)), c2 = 1.f - powf(b2, static_cast<float>(step));
  ls_adam_kernel<<<static_cast<int>((count + 255) / 256), 256, 0, st>>>(S, g, m, v, count, lr, b1, b2, eps, c1, c2);
  return cudaGetLastError();
}

}  // namespace htgb
