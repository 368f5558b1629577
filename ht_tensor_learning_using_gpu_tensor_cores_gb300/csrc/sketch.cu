// Small kernels of the Gram-free leaf range finder (api.cu, HT_LEAF_SKETCH).
//
// A leaf's range finder never forms the mode Gram G = X_(m) X_(m)^T: each
// application Y = G Q runs as two streaming products over the tensor
// (Z = X_(m)^T Q, Y = X_(m) Z).  After the last application the leaf basis
// comes from the Nystrom approximation of G in the test block Q,
//   G ~ Y (Q^T Y)^-1 Y^T,
// taken with a small shift nu for stability (Tropp, Yurtsever, Udell and
// Cevher, "Fixed-rank approximation of a positive-semidefinite matrix from
// streaming data", NeurIPS 2017, Alg. 3): with Y_nu = Y + nu Q = Q1 R1 and
// W = Q^T Y,
//   G + nu I ~ Q1 R1 (W + nu I)^-1 R1^T Q1^T,
// so the leaf basis is Q1 times the top eigenvectors of the s x s matrix
// H = R1 (W + nu I)^-1 R1^T.  The reference's range finder (rsvd,
// third_order_tensor_decompsition/CUDA/Optimized/kernel.cu:595-680) instead
// forms B = C^T A from its sketch C = A Omega and takes the SVD of B.
#include "common.cuh"
#include "engine.h"

namespace htgb {
namespace {

constexpr int NY_MAX = 64;

// nu = nu_rel * tr(W), summed in FP64 in index order (the two kernels below
// must agree on it bit for bit).
HT_DEV double nystrom_nu(const float *W, int s, float nu_rel) {
  double tr = 0.0;
  for (int i = 0; i < s; ++i) tr += static_cast<double>(W[i + s * i]);
  return static_cast<double>(nu_rel) * (tr > 0.0 ? tr : 0.0);
}

__global__ void nystrom_shift_kernel(const float *__restrict__ Y, const float *__restrict__ Q, long long n, int s,
                                     const float *__restrict__ W, float nu_rel, float *__restrict__ Yn) {
  __shared__ float s_nu;
  if (threadIdx.x == 0) s_nu = static_cast<float>(nystrom_nu(W, s, nu_rel));
  __syncthreads();
  const float nu = s_nu;
  const long long total = n * s;
  for (long long i = blockIdx.x * 256ll + threadIdx.x; i < total; i += gridDim.x * 256ll) Yn[i] = fmaf(nu, Q[i], Y[i]);
}

// H = R1 (sym(W) + nu I)^-1 R1^T in FP64 (Cholesky of the shifted W; a pivot
// that rounding drove to or below zero is floored at nu).  One CTA.
struct NystromBatch {
  NystromProb p[4];
};

__global__ void __launch_bounds__(256) nystrom_core_kernel(const NystromBatch batch, float nu_rel,
                                                           int *__restrict__ err) {
  const float *__restrict__ W = batch.p[blockIdx.x].W;
  const float *__restrict__ R1 = batch.p[blockIdx.x].R1;
  const int s = batch.p[blockIdx.x].s;
  float *__restrict__ H = batch.p[blockIdx.x].H;
  extern __shared__ double ny_sm[];
  double *L = ny_sm;                       // upper Cholesky factor, row-major: (W + nu I) = L^T L
  double *F = ny_sm + NY_MAX * NY_MAX;     // F = R1 L^-1, row-major
  __shared__ double s_nu;
  const int t = threadIdx.x;
  if (t == 0) s_nu = nystrom_nu(W, s, nu_rel);
  __syncthreads();
  const double nu = s_nu;
  for (int e = t; e < s * s; e += 256) {
    const int i = e / s, j = e % s;
    L[i * NY_MAX + j] = 0.5 * (static_cast<double>(W[i + s * j]) + static_cast<double>(W[j + s * i])) +
                        (i == j ? nu : 0.0);
  }
  __syncthreads();
  for (int j = 0; j < s; ++j) {
    if (t == 0) {
      double d = L[j * NY_MAX + j];
      if (!isfinite(d)) report_error(err, kErrNonFinite);
      if (!(d > nu)) d = nu > 0.0 ? nu : 1.0;
      L[j * NY_MAX + j] = sqrt(d);
    }
    __syncthreads();
    const double inv = 1.0 / L[j * NY_MAX + j];
    for (int c = j + 1 + t; c < s; c += 256) L[j * NY_MAX + c] *= inv;
    __syncthreads();
    for (int e = t; e < (s - j - 1) * (s - j - 1); e += 256) {
      const int i = j + 1 + e / (s - j - 1), c = j + 1 + e % (s - j - 1);
      if (c >= i) L[i * NY_MAX + c] -= L[j * NY_MAX + i] * L[j * NY_MAX + c];
    }
    __syncthreads();
  }
  // F[i, :] L = R1[i, :]: forward substitution along the columns, row i by thread i
  for (int i = t; i < s; i += 256) {
    for (int c = 0; c < s; ++c) {
      double v = static_cast<double>(R1[i + s * c]);
      for (int d = 0; d < c; ++d) v -= F[i * NY_MAX + d] * L[d * NY_MAX + c];
      F[i * NY_MAX + c] = v / L[c * NY_MAX + c];
    }
  }
  __syncthreads();
  for (int e = t; e < s * s; e += 256) {
    const int i = e % s, j = e / s;
    double v = 0.0;
    for (int c = 0; c < s; ++c) v = fma(F[i * NY_MAX + c], F[j * NY_MAX + c], v);
    H[i + s * j] = static_cast<float>(v);
  }
}

}  // namespace

cudaError_t nystrom_shift_launch(const float *Y, const float *Q, long long n, int s, const float *W, float nu_rel,
                                 float *Yn, cudaStream_t st) {
  if (s < 1 || s > NY_MAX) return cudaErrorInvalidValue;
  long long blocks = (n * s + 255) / 256;
  const long long cap = 4ll * device_sm_count();
  if (blocks > cap) blocks = cap;
  nystrom_shift_kernel<<<static_cast<unsigned>(blocks < 1 ? 1 : blocks), 256, 0, st>>>(Y, Q, n, s, W, nu_rel, Yn);
  return cudaGetLastError();
}

cudaError_t nystrom_core_launch(const NystromProb *probs, int nprob, float nu_rel, int *err, cudaStream_t st) {
  if (nprob < 1 || nprob > 4) return cudaErrorInvalidValue;
  NystromBatch b;
  for (int i = 0; i < 4; ++i) b.p[i] = NystromProb{nullptr, nullptr, 0, nullptr};
  for (int i = 0; i < nprob; ++i) {
    if (probs[i].s < 1 || probs[i].s > NY_MAX) return cudaErrorInvalidValue;
    b.p[i] = probs[i];
  }
  constexpr int kSmem = 2 * NY_MAX * NY_MAX * sizeof(double);
  static bool attr_set[64] = {};
  const cudaError_t e = opt_in_smem(nystrom_core_kernel, kSmem, attr_set);
  if (e != cudaSuccess) return e;
  nystrom_core_kernel<<<nprob, 256, kSmem, st>>>(b, nu_rel, err);
  return cudaGetLastError();
}

}  // namespace htgb
