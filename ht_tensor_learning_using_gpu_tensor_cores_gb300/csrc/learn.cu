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
//   dL/dS = -(2 / B) sum_b G_b E_b C_b^-1 / tr(G_b),   E = G Y - Y C^-1 H = (I - Q Q^T) G Q R,
//         = -(2 / B) sum_b G_b (I - Q_b Q_b^T) G_b Q_b R_b^-T / tr(G_b).
//
// Kernels: a batched n x n by n x s product (FP32, the three large products
// Y = G S, P = G Q, G E), a per-Gram factor kernel (C in FP64, the
// column-dropping Cholesky, R^-1 and Q = Y R^-1 in FP64), a per-Gram loss
// kernel (H = Q^T P, E = P - Q H in FP64), a deterministic batch reduction of
// the gradient, plus an Adam step.  The reference has no learned component;
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

// Per Gram b: C = Y^T Y (FP64 accumulation), the column-dropping Cholesky
// C_KK = R^T R, Rinv = R^-1 (FP64, zero outside K) and the orthonormal basis
// Q = Y Rinv (FP64 sums, stored FP32; dropped columns zero).  Forming Q keeps
// the loss well conditioned: tr(Q^T G Q) from a fresh product G Q cannot
// exceed tr(G), whereas tr(C^-1 Y^T G Y) carries the rounding of G Y through
// C^-1.  One CTA per Gram.
__global__ void __launch_bounds__(256) ls_factor_kernel(const float *__restrict__ Y, int n, int s,
                                                        float *__restrict__ Q, double *__restrict__ Rinv,
                                                        int *__restrict__ bad) {
  extern __shared__ double ls_sm[];
  double *C = ls_sm;                        // LS_MAX x LS_MAX: C, then R (upper triangle)
  double *Ri = ls_sm + LS_MAX * LS_MAX;     // LS_MAX x LS_MAX: R^-1
  __shared__ int s_bad;
  __shared__ int keep[LS_MAX];
  __shared__ double d0[LS_MAX];
  const int b = blockIdx.x, t = threadIdx.x;
  const float *Yb = Y + static_cast<long long>(b) * n * s;
  for (int e = t; e < s * s; e += 256) {
    const int i = e / s, j = e % s;
    double c = 0.0;
    for (int r = 0; r < n; ++r)
      c = fma(static_cast<double>(Yb[r + static_cast<long long>(n) * i]),
              static_cast<double>(Yb[r + static_cast<long long>(n) * j]), c);
    C[i * LS_MAX + j] = c;
  }
  __syncthreads();
  ls_cholesky(C, s, keep, d0, &s_bad);
  if (s_bad && t == 0) atomicOr(bad, 1);
  // R^-1, column j by thread j (back substitution; zero rows/columns off K)
  for (int j = t; j < s; j += 256) {
    for (int i = s - 1; i >= 0; --i) {
      double v = (i == j) ? 1.0 : 0.0;
      if (keep[i] && keep[j]) {
        for (int k = i + 1; k <= j; ++k) v -= C[i * LS_MAX + k] * Ri[k * LS_MAX + j];
        v /= C[i * LS_MAX + i];
      } else {
        v = 0.0;
      }
      Ri[i * LS_MAX + j] = v;
    }
  }
  __syncthreads();
  double *Rb = Rinv + static_cast<long long>(b) * LS_MAX * LS_MAX;
  for (int e = t; e < LS_MAX * LS_MAX; e += 256) Rb[e] = Ri[e];
  float *Qb = Q + static_cast<long long>(b) * n * s;
  for (int e = t; e < n * s; e += 256) {
    const int r = e % n, j = e / n;
    double v = 0.0;
    for (int k = 0; k <= j; ++k) v = fma(static_cast<double>(Yb[r + static_cast<long long>(n) * k]), Ri[k * LS_MAX + j], v);
    Qb[e] = static_cast<float>(v);
  }
}

// Per Gram b, with P = G Q: H = Q^T P (FP64), loss_b = 1 - tr(H) / trG_b and
// E = P - Q H (the part of G Q outside span(Q)).  One CTA per Gram.
__global__ void __launch_bounds__(256) ls_loss_kernel(const float *__restrict__ Q, const float *__restrict__ P,
                                                      const float *__restrict__ trG, int n, int s,
                                                      float *__restrict__ E, double *__restrict__ loss) {
  __shared__ double H[LS_MAX * LS_MAX];
  const int b = blockIdx.x, t = threadIdx.x;
  const float *Qb = Q + static_cast<long long>(b) * n * s;
  const float *Pb = P + static_cast<long long>(b) * n * s;
  for (int e = t; e < s * s; e += 256) {
    const int i = e / s, j = e % s;
    double h = 0.0;
    for (int r = 0; r < n; ++r)
      h = fma(static_cast<double>(Qb[r + static_cast<long long>(n) * i]),
              static_cast<double>(Pb[r + static_cast<long long>(n) * j]), h);
    H[i * LS_MAX + j] = h;
  }
  __syncthreads();
  if (t == 0) {
    double tr = 0.0;
    for (int i = 0; i < s; ++i) tr += H[i * LS_MAX + i];
    loss[b] = 1.0 - tr / static_cast<double>(trG[b]);
  }
  float *Eb = E + static_cast<long long>(b) * n * s;
  for (int e = t; e < n * s; e += 256) {
    const int r = e % n, j = e / n;
    double v = Pb[r + static_cast<long long>(n) * j];
    for (int k = 0; k < s; ++k) v -= static_cast<double>(Qb[r + static_cast<long long>(n) * k]) * H[k * LS_MAX + j];
    Eb[e] = static_cast<float>(v);
  }
}

// grad[r, j] = -(2 / B) sum_b (1 / trG_b) sum_k GE_b[r, k] Rinv_b[j, k], batch
// summed in order (dL/dS = -(2 / tr G) G (I - Q Q^T) G Q R^-T).
__global__ void __launch_bounds__(256) ls_grad_kernel(const float *__restrict__ GE, const double *__restrict__ Rinv,
                                                      const float *__restrict__ trG, int batch, int n, int s,
                                                      float *__restrict__ grad) {
  const long long e = blockIdx.x * 256ll + threadIdx.x;
  if (e >= static_cast<long long>(n) * s) return;
  const int r = static_cast<int>(e % n), j = static_cast<int>(e / n);
  double acc = 0.0;
  for (int b = 0; b < batch; ++b) {
    const float *GEb = GE + static_cast<long long>(b) * n * s;
    const double *Rb = Rinv + static_cast<long long>(b) * LS_MAX * LS_MAX;
    double v = 0.0;
    for (int k = j; k < s; ++k) v = fma(static_cast<double>(GEb[r + static_cast<long long>(n) * k]), Rb[j * LS_MAX + k], v);
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
  return 5 * ns * sizeof(float) + static_cast<size_t>(batch) * LS_MAX * LS_MAX * sizeof(double) +
         static_cast<size_t>(batch) * sizeof(double) + 256;
}

cudaError_t sketch_loss_grad(const float *G, const float *trG, int batch, int n, int s, const float *S, float *grad,
                             double *loss, int *bad, void *ws, cudaStream_t st, int *launches) {
  if (s < 1 || s > LS_MAX || n < s || batch < 1) return cudaErrorInvalidValue;
  const size_t ns = static_cast<size_t>(n) * s * batch;
  float *Y = static_cast<float *>(ws), *Q = Y + ns, *P = Q + ns, *E = P + ns, *GE = E + ns;
  double *Rinv = reinterpret_cast<double *>(GE + ns);
  const dim3 grid((n + LT_ROWS - 1) / LT_ROWS, batch);
  static bool attr_set[64] = {};
  constexpr int kFactorSmem = 2 * LS_MAX * LS_MAX * sizeof(double);
  {
    const cudaError_t e = opt_in_smem(ls_factor_kernel, kFactorSmem, attr_set);
    if (e != cudaSuccess) return e;
  }
  ls_bgemm_kernel<<<grid, 256, 0, st>>>(G, S, 0, Y, n, s);                                   // Y = G S
  ls_factor_kernel<<<batch, 256, kFactorSmem, st>>>(Y, n, s, Q, Rinv, bad);                 // Q = Y R^-1
  ls_bgemm_kernel<<<grid, 256, 0, st>>>(G, Q, static_cast<long long>(n) * s, P, n, s);       // P = G Q
  ls_loss_kernel<<<batch, 256, 0, st>>>(Q, P, trG, n, s, E, loss);                          // loss, E
  ls_bgemm_kernel<<<grid, 256, 0, st>>>(G, E, static_cast<long long>(n) * s, GE, n, s);      // G E
  const long long cnt = static_cast<long long>(n) * s;
  ls_grad_kernel<<<static_cast<int>((cnt + 255) / 256), 256, 0, st>>>(GE, Rinv, trG, batch, n, s, grad);
  if (launches) *launches += 6;
  return cudaGetLastError();
}

cudaError_t sketch_adam(float *S, const float *g, float *m, float *v, long long count, float lr, float b1, float b2,
                        float eps, int step, cudaStream_t st) {
  const float c1 = 1.f - powf(b1, static_cast<float>(step)), c2 = 1.f - powf(b2, static_cast<float>(step));
  ls_adam_kernel<<<static_cast<int>((count + 255) / 256), 256, 0, st>>>(S, g, m, v, count, lr, b1, b2, eps, c1, c2);
  return cudaGetLastError();
}

}  // namespace htgb
