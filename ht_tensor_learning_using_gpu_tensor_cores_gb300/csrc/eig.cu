// Top-K eigenpairs of the leaf Grams on the GPU.
//
// Replaces the reference's full cuSOLVER syevd of every n x n Gram followed by
// a copy of the last k columns (third_order_tensor_decompsition/CUDA/Optimized/
// kernel.cu:682-718, htd_tensorcore.cu:133-140).  Only the top K eigenvectors
// are needed, so this is block subspace iteration on G with an oversampled
// block of s <= 64 columns:
//
//   Q <- Gaussian (or a supplied start block)
//   repeat iters:  Y = (G + mu I) Q ;  Q = Y R^-1   (CholeskyQR, shifted)
//   two more CholeskyQR passes on Q (orthonormal to FP32 rounding)
//   Rayleigh-Ritz: H = Q^T G Q, Jacobi eigen-decomposition of H (s x s),
//   U = Q V[:, top K], GU = G U, residual max_j ||G u_j - theta_j u_j|| / theta_1.
//
// Precision: G and Q are FP32; the s x s Gram matrices Y^T Y and Q^T G Q are
// accumulated with compensated FP32 (TwoProduct/TwoSum), which is as accurate
// as FP64 accumulation while running at FP32 rate -- GB300's FP64 throughput
// is 1/64 of FP32.  The Cholesky runs on the unit-diagonal scaled matrix with
// a small shift, so it cannot break down on rank-deficient blocks.
// mu = 1e-9 * trace(G) keeps Y nonzero on exactly null directions without
// moving any eigenvector or slowing convergence.  When the block covers the
// whole space (s == n, small modes) the iteration is skipped: Q = I and the
// Rayleigh-Ritz step is a Jacobi eigen-decomposition of G itself.
#include <vector>

#include "common.cuh"
#include "engine.h"

namespace htgb {
namespace {

constexpr int SMAX = 64;
constexpr int ESMAX = SMAX * (SMAX + 1) / 2;
constexpr int RB = 16;   // rows per CTA

constexpr int kMaxProb = 8;

struct EigDev {
  const float *G;
  int n, s, K, nrb;
  float *Q, *Y, *U, *GU, *theta, *resid;
  const float *start;
  unsigned long long seed, stream_id;
  float *partS;    // [nrb][ESMAX][2]
  float *partH;    // [nrb][SMAX*SMAX][2]
  double *S;       // [ESMAX]
  double *H;       // [SMAX*SMAX]
  float *V;        // [SMAX*SMAX] sorted eigenvectors of H
  float *mu;       // [1]
  float *colss;    // [nrb][SMAX]
};

struct EigBatch {
  EigDev p[kMaxProb];
};

HT_DEV void tri_index(int e, int &i, int &j) {
  // packed upper triangle, column-major: e = j(j+1)/2 + i, i <= j
  int jj = static_cast<int>((sqrtf(8.f * e + 1.f) - 1.f) * 0.5f);
  while (jj * (jj + 1) / 2 > e) --jj;
  while ((jj + 1) * (jj + 2) / 2 <= e) ++jj;
  j = jj;
  i = e - jj * (jj + 1) / 2;
}

__global__ void eig_init_kernel(const EigBatch probs) {
  const EigDev &P = probs.p[blockIdx.y];
  const long long total = static_cast<long long>(P.n) * P.s;
  for (long long idx = blockIdx.x * 256ll + threadIdx.x; idx < total; idx += gridDim.x * 256ll) {
    float v;
    if (P.s == P.n) v = (idx % P.n == idx / P.n) ? 1.f : 0.f;   // direct: Q = I
    else if (P.start) v = P.start[idx];
    else v = gaussian(P.seed, P.stream_id, static_cast<unsigned long long>(idx));
    P.Q[idx] = v;
  }
  if (blockIdx.x == 0) {
    __shared__ float red[256];
    float t = 0.f;
    for (int i = threadIdx.x; i < P.n; i += 256) t += P.G[i + static_cast<long long>(P.n) * i];
    red[threadIdx.x] = t;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
      if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
      __syncthreads();
    }
    // far below the FP32 noise floor of G (~1e-7 ||G||): it only keeps Y
    // nonzero on exactly null directions, and never slows convergence
    if (threadIdx.x == 0) P.mu[0] = 1e-9f * fmaxf(red[0], 0.f);
  }
}

// mode 0: Y = (G + mu I) Q, partial Y^T Y
// mode 1: partial Q^T Q (Y untouched)
// mode 2: Y = G Q, partial Q^T Y (Rayleigh quotient)
__global__ void __launch_bounds__(256) eig_gq_kernel(const EigBatch probs, int mode) {
  const EigDev &P = probs.p[blockIdx.y];
  const int rb = blockIdx.x;
  if (rb >= P.nrb) return;
  if (mode != 2 && P.s == P.n && P.G) return;   // direct problems skip the iteration
  const int n = P.n, s = P.s;
  const int r0 = rb * RB;
  const int t = threadIdx.x;
  __shared__ float Gs[64][RB + 1];
  __shared__ float Qs[64][SMAX + 1];
  __shared__ float Ys[RB][SMAX + 1];
  __shared__ float Qr[RB][SMAX + 1];

  // rows of Q owned by this CTA
  for (int e = t; e < RB * SMAX; e += 256) {
    const int i = e % RB, j = e / RB;
    float v = 0.f;
    if (r0 + i < n && j < s) v = P.Q[(r0 + i) + static_cast<long long>(n) * j];
    Qr[i][j] = v;
  }
  if (mode != 1) {
    const int i = t / 16;            // row within the block
    const int jb = t % 16;           // columns jb, jb+16, jb+32, jb+48
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
    for (int kc = 0; kc < n; kc += 64) {
      __syncthreads();
      for (int e = t; e < 64 * RB; e += 256) {
        const int kk = e % 64, ii = e / 64;
        float v = 0.f;
        if (kc + kk < n && r0 + ii < n) v = P.G[(kc + kk) + static_cast<long long>(n) * (r0 + ii)];   // G symmetric
        Gs[kk][ii] = v;
      }
      for (int e = t; e < 64 * SMAX; e += 256) {
        const int kk = e % 64, j = e / 64;
        float v = 0.f;
        if (kc + kk < n && j < s) v = P.Q[(kc + kk) + static_cast<long long>(n) * j];
        Qs[kk][j] = v;
      }
      __syncthreads();
#pragma unroll 8
      for (int kk = 0; kk < 64; ++kk) {
        const float g = Gs[kk][i];
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[c] = fmaf(g, Qs[kk][jb + 16 * c], acc[c]);
      }
    }
    const float mu = (mode == 0) ? P.mu[0] : 0.f;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const int j = jb + 16 * c;
      float y = acc[c] + mu * Qr[i][j];
      if (r0 + i >= n || j >= s) y = 0.f;
      Ys[i][j] = y;
      if (r0 + i < n && j < s) P.Y[(r0 + i) + static_cast<long long>(n) * j] = y;
    }
  } else {
    for (int e = t; e < RB * SMAX; e += 256) Ys[e % RB][e / RB] = Qr[e % RB][e / RB];
  }
  __syncthreads();
  const int rows = min(RB, n - r0);
  if (mode != 2) {
    const int E = s * (s + 1) / 2;
    for (int e = t; e < E; e += 256) {
      int i, j;
      tri_index(e, i, j);
      Acc2 a = {0.f, 0.f};
      for (int r = 0; r < rows; ++r) acc2_add_prod(a, Ys[r][i], Ys[r][j]);
      float *dst = P.partS + (static_cast<long long>(rb) * ESMAX + e) * 2;
      dst[0] = a.s;
      dst[1] = a.c;
    }
  } else {
    for (int e = t; e < s * s; e += 256) {
      const int i = e % s, j = e / s;
      Acc2 a = {0.f, 0.f};
      for (int r = 0; r < rows; ++r) acc2_add_prod(a, Qr[r][i], Ys[r][j]);
      float *dst = P.partH + (static_cast<long long>(rb) * SMAX * SMAX + e) * 2;
      dst[0] = a.s;
      dst[1] = a.c;
    }
  }
}

// which 0: S (packed triangle), which 1: H (s x s)
__global__ void eig_reduce_kernel(const EigBatch probs, int which) {
  const EigDev &P = probs.p[blockIdx.y];
  const int E = which == 0 ? P.s * (P.s + 1) / 2 : P.s * P.s;
  const int stride = which == 0 ? ESMAX : SMAX * SMAX;
  const float *part = which == 0 ? P.partS : P.partH;
  if (which == 0 && P.s == P.n && P.G) return;
  for (int e = blockIdx.x * 256 + threadIdx.x; e < E; e += gridDim.x * 256) {
    Acc2 a = {0.f, 0.f};
    for (int r = 0; r < P.nrb; ++r) {
      const float *src = part + (static_cast<long long>(r) * stride + e) * 2;
      acc2_add(a, src[0], src[1]);
    }
    const double v = static_cast<double>(a.s) + static_cast<double>(a.c);
    if (which == 0) P.S[e] = v;
    else P.H[e] = v;
  }
}

// Q[rows] = X[rows] D^-1/2 R^-1 where R^T R = D^-1/2 S D^-1/2 + shift I and X
// is Y (src 0) or Q itself (src 1).
__global__ void __launch_bounds__(256) eig_orth_kernel(const EigBatch probs, int src, float shift) {
  const EigDev &P = probs.p[blockIdx.y];
  const int rb = blockIdx.x;
  if (rb >= P.nrb) return;
  if (P.s == P.n && P.G) return;   // direct problems skip the iteration
  const int n = P.n, s = P.s;
  __shared__ float A[SMAX][SMAX + 1];   // scaled S, overwritten by R (upper)
  __shared__ float dsc[SMAX];
  const int t = threadIdx.x;
  // scaling
  for (int j = t; j < s; j += 256) {
    const double d = P.S[j * (j + 1) / 2 + j];
    dsc[j] = d > 1e-300 ? static_cast<float>(1.0 / sqrt(d)) : 0.f;
  }
  __syncthreads();
  const int E = s * (s + 1) / 2;
  for (int e = t; e < E; e += 256) {
    int i, j;
    tri_index(e, i, j);
    const double sc = static_cast<double>(dsc[i]) * static_cast<double>(dsc[j]);
    float v = static_cast<float>(P.S[e] * sc);
    if (i == j) v = (dsc[j] > 0.f ? 1.f : 0.f) + shift;
    A[i][j] = v;
  }
  __syncthreads();
  // Right-looking Cholesky A = R^T R on the upper triangle with all threads.
  // Step j updates rows > j from the still-unscaled row j, then scales row j;
  // the next step never touches row j again, so one barrier per step suffices.
  for (int j = 0; j < s; ++j) {
    const float d = sqrtf(fmaxf(A[j][j], 1e-30f));
    const float inv = 1.f / d;
    const int m = s - j - 1;
    for (int e = t; e < m * m; e += 256) {
      const int ii = e % m, kk = e / m;
      if (ii <= kk) {
        const int i = j + 1 + ii, k = j + 1 + kk;
        A[i][k] = fmaf(-(A[j][i] * inv), A[j][k] * inv, A[i][k]);
      }
    }
    __syncthreads();
    for (int k = j + t; k < s; k += 256) A[j][k] = (k == j) ? d : A[j][k] * inv;
  }
  __syncthreads();
  // forward substitution q R = x D^-1/2, one half-warp per row
  const int half = t / 16, l = t % 16;
  const int row = rb * RB + half;
  const bool valid = row < n;
  const float *X = src == 0 ? P.Y : P.Q;
  float tv[4];
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const int j = l + 16 * c;
    tv[c] = (valid && j < s) ? X[row + static_cast<long long>(n) * j] * dsc[j] : 0.f;
  }
  float q[4] = {0.f, 0.f, 0.f, 0.f};
  const unsigned mask = 0xFFFFu << (16 * ((t / 16) & 1));
  for (int j = 0; j < s; ++j) {
    const int owner = j % 16, c = j / 16;
    float qj = 0.f;
    if (l == owner) {
      qj = tv[c] / A[j][j];
      q[c] = qj;
    }
    qj = __shfl_sync(mask, qj, owner, 16);
#pragma unroll
    for (int cc = 0; cc < 4; ++cc) {
      const int k = l + 16 * cc;
      if (k > j && k < s) tv[cc] = fmaf(-qj, A[j][k], tv[cc]);
    }
  }
  if (valid) {
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const int j = l + 16 * c;
      if (j < s) P.Q[row + static_cast<long long>(n) * j] = q[c];
    }
  }
}

// Cyclic Jacobi on a symmetric s x s matrix held in shared memory (s <= SMAX),
// 256 threads, round-robin ("circle method") ordering so every round rotates
// s/2 disjoint pairs in parallel.  On return A is diagonal to FP32 rounding,
// V holds the eigenvectors and order[] the indices by descending eigenvalue.
HT_DEV void jacobi_smem(float (*A)[SMAX + 1], float (*V)[SMAX + 1], int s, int *order) {
  __shared__ float cs[SMAX / 2], sn[SMAX / 2];
  __shared__ int pp[SMAX / 2], qq[SMAX / 2];
  __shared__ float red[256];
  const int t = threadIdx.x;
  const int m = (s + 1) & ~1;   // even number of players (a dummy index when s is odd)
  for (int e = t; e < SMAX * SMAX; e += 256) {
    const int i = e % SMAX, j = e / SMAX;
    V[i][j] = (i == j) ? 1.f : 0.f;
  }
  __syncthreads();
  for (int sweep = 0; sweep < 16 && m > 1; ++sweep) {
    float off = 0.f, dia = 0.f;
    for (int e = t; e < s * s; e += 256) {
      const int i = e % s, j = e / s;
      const float v = A[i][j];
      if (i == j) dia += v * v; else off += v * v;
    }
    red[t] = off;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
      if (t < w) red[t] += red[t + w];
      __syncthreads();
    }
    const float offs = red[0];
    __syncthreads();
    red[t] = dia;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
      if (t < w) red[t] += red[t + w];
      __syncthreads();
    }
    const float dias = red[0];
    __syncthreads();
    // FP32 rounding leaves off-diagonal mass near s * eps^2 * diag mass
    if (offs <= 1e-11f * dias || offs == 0.f) break;
    for (int round = 0; round < m - 1; ++round) {
      if (t < m / 2) {
        // position 0 is fixed, positions 1..m-1 rotate by one each round
        const int pa = t, pb = m - 1 - t;
        int p = pa == 0 ? 0 : 1 + ((pa - 1 + round) % (m - 1));
        int q = pb == 0 ? 0 : 1 + ((pb - 1 + round) % (m - 1));
        if (p > q) { const int tmp = p; p = q; q = tmp; }
        float c = 1.f, sv = 0.f;
        if (q < s) {
          const float apq = A[p][q];
          if (fabsf(apq) > 1e-30f && fabsf(apq) > 1e-9f * sqrtf(fabsf(A[p][p] * A[q][q]))) {
            const float tau = (A[q][q] - A[p][p]) / (2.f * apq);
            const float tt = (tau >= 0.f ? 1.f : -1.f) / (fabsf(tau) + sqrtf(1.f + tau * tau));
            c = rsqrtf(1.f + tt * tt);
            sv = tt * c;
          }
        }
        pp[t] = p; qq[t] = q; cs[t] = c; sn[t] = sv;
      }
      __syncthreads();
      for (int e = t; e < (m / 2) * s; e += 256) {   // rows: A <- J^T A
        const int pr = e / s, j = e % s;
        const int p = pp[pr], q = qq[pr];
        if (q >= s) continue;
        const float c = cs[pr], sv = sn[pr];
        const float ap = A[p][j], aq = A[q][j];
        A[p][j] = c * ap - sv * aq;
        A[q][j] = sv * ap + c * aq;
      }
      __syncthreads();
      for (int e = t; e < (m / 2) * s; e += 256) {   // columns: A <- A J, V <- V J
        const int pr = e / s, i = e % s;
        const int p = pp[pr], q = qq[pr];
        if (q >= s) continue;
        const float c = cs[pr], sv = sn[pr];
        const float ap = A[i][p], aq = A[i][q];
        A[i][p] = c * ap - sv * aq;
        A[i][q] = sv * ap + c * aq;
        const float vp = V[i][p], vq = V[i][q];
        V[i][p] = c * vp - sv * vq;
        V[i][q] = sv * vp + c * vq;
      }
      __syncthreads();
    }
  }
  for (int j = t; j < s; j += 256) {   // rank by counting: descending eigenvalues
    const float dj = A[j][j];
    int rank = 0;
    for (int i = 0; i < s; ++i) {
      const float di = A[i][i];
      if (di > dj || (di == dj && i < j)) ++rank;
    }
    order[rank] = j;
  }
  __syncthreads();
}

// Rayleigh-Ritz: eigen-decomposition of H = Q^T G Q, one CTA per problem.
__global__ void __launch_bounds__(256) eig_jacobi_kernel(const EigBatch probs) {
  const EigDev &P = probs.p[blockIdx.x];
  const int s = P.s;
  __shared__ float A[SMAX][SMAX + 1];
  __shared__ float V[SMAX][SMAX + 1];
  __shared__ int order[SMAX];
  const int t = threadIdx.x;
  for (int e = t; e < SMAX * SMAX; e += 256) {
    const int i = e % SMAX, j = e / SMAX;
    A[i][j] = (i < s && j < s) ? static_cast<float>(0.5 * (P.H[i + s * j] + P.H[j + s * i])) : 0.f;
  }
  __syncthreads();
  jacobi_smem(A, V, s, order);
  for (int e = t; e < s * s; e += 256) {
    const int i = e % s, r = e / s;
    P.V[i + s * r] = V[i][order[r]];
  }
  for (int r = t; r < P.K; r += 256) P.theta[r] = A[order[r]][order[r]];
}

// Transfer-tensor step of the complementary-leaf construction.  WG = W^T G_c W
// (kw x kw, leading dimension kw) for the complementary leaf's Ritz block W;
// V = W[:, :kt].  With GV = V^T G_c V = P diag(lam) P^T:
//   M     = P diag(lam^-1/2)   (columns with lam <= 1e-12 lam_max are zero)
//   Broot = M^T V^T G_c U_c    (kt x kc; stored transposed when the interior
//                               node is the root's right child)
// and the caller forms B_t = C_V M.
__global__ void __launch_bounds__(256) transfer_eig_kernel(const float *WG, int kw, int kt, int kc, int t_is_left,
                                                           float *M, float *Broot) {
  __shared__ float A[SMAX][SMAX + 1];
  __shared__ float V[SMAX][SMAX + 1];
  __shared__ int order[SMAX];
  __shared__ float inv[SMAX];
  const int t = threadIdx.x;
  for (int e = t; e < SMAX * SMAX; e += 256) {
    const int i = e % SMAX, j = e / SMAX;
    A[i][j] = (i < kt && j < kt) ? 0.5f * (WG[i + kw * j] + WG[j + kw * i]) : 0.f;
  }
  __syncthreads();
  jacobi_smem(A, V, kt, order);
  if (t == 0) {
    const float lmax = A[order[0]][order[0]];
    for (int r = 0; r < kt; ++r) {
      const float l = A[order[r]][order[r]];
      inv[r] = (lmax > 0.f && l > 1e-12f * lmax) ? rsqrtf(l) : 0.f;
    }
  }
  __syncthreads();
  for (int e = t; e < kt * kt; e += 256) {
    const int i = e % kt, r = e / kt;
    M[i + kt * r] = V[i][order[r]] * inv[r];
  }
  __syncthreads();
  for (int e = t; e < kt * kc; e += 256) {
    const int r = e % kt, u = e / kt;
    float acc = 0.f;
    const int oc = order[r];
    for (int c = 0; c < kt; ++c) acc = fmaf(V[c][oc] * inv[r], 0.5f * (WG[c + kw * u] + WG[u + kw * c]), acc);
    if (t_is_left) Broot[r + kt * u] = acc;
    else Broot[u + kc * r] = acc;
  }
}

// U = Q V[:, :K], GU = Y V[:, :K], residual partials.
__global__ void __launch_bounds__(256) eig_finalize_kernel(const EigBatch probs) {
  const EigDev &P = probs.p[blockIdx.y];
  const int rb = blockIdx.x;
  if (rb >= P.nrb) return;
  const int n = P.n, s = P.s, K = P.K;
  __shared__ float Vs[SMAX][SMAX + 1];
  __shared__ float Qr[RB][SMAX + 1];
  __shared__ float Yr[RB][SMAX + 1];
  __shared__ float res[RB][SMAX + 1];
  const int t = threadIdx.x;
  const int r0 = rb * RB;
  for (int e = t; e < SMAX * SMAX; e += 256) {
    const int i = e % SMAX, j = e / SMAX;
    Vs[i][j] = (i < s && j < s) ? P.V[i + s * j] : 0.f;
  }
  for (int e = t; e < RB * SMAX; e += 256) {
    const int i = e % RB, j = e / RB;
    const bool ok = r0 + i < n && j < s;
    Qr[i][j] = ok ? P.Q[(r0 + i) + static_cast<long long>(n) * j] : 0.f;
    Yr[i][j] = ok ? P.Y[(r0 + i) + static_cast<long long>(n) * j] : 0.f;
  }
  __syncthreads();
  const int i = t / 16, jb = t % 16;
  for (int c = 0; c < 4; ++c) {
    const int j = jb + 16 * c;
    float u = 0.f, gu = 0.f;
    if (j < K) {
      for (int k = 0; k < s; ++k) {
        u = fmaf(Qr[i][k], Vs[k][j], u);
        gu = fmaf(Yr[i][k], Vs[k][j], gu);
      }
    }
    const bool ok = (r0 + i < n) && j < K;
    if (ok) {
      P.U[(r0 + i) + static_cast<long long>(n) * j] = u;
      P.GU[(r0 + i) + static_cast<long long>(n) * j] = gu;
    }
    const float d = ok ? gu - P.theta[j] * u : 0.f;
    res[i][j] = d * d;
  }
  __syncthreads();
  for (int j = t; j < K; j += 256) {
    float a = 0.f;
    for (int r = 0; r < RB; ++r) a += res[r][j];
    P.colss[static_cast<long long>(rb) * SMAX + j] = a;
  }
}

__global__ void eig_resid_kernel(const EigBatch probs) {
  const EigDev &P = probs.p[blockIdx.x];
  __shared__ float red[64];
  const int j = threadIdx.x;
  float a = 0.f;
  if (j < P.K)
    for (int r = 0; r < P.nrb; ++r) a += P.colss[static_cast<long long>(r) * SMAX + j];
  red[j] = sqrtf(a);
  __syncthreads();
  if (j == 0) {
    float m = 0.f;
    for (int i = 0; i < P.K; ++i) m = fmaxf(m, red[i]);
    const float th = P.theta[0];
    P.resid[0] = th > 0.f ? m / th : m;
  }
}

// SVD of a tall W from its Gram GW = W^T W (s x s): GW = U diag(sigma^2) U^T.
// M1 = U[:, :k1], M2 = U[:, :k2] diag(1/sigma) (zero where sigma <= 1e-6 sigma_1),
// Broot = M1^T GW M2 (k1 x k2).
__global__ void __launch_bounds__(256) svd_from_gram_kernel(const float *GW, int s, int k1, int k2, float *M1,
                                                            float *M2, float *Broot) {
  __shared__ float A[SMAX][SMAX + 1];
  __shared__ float V[SMAX][SMAX + 1];
  __shared__ int order[SMAX];
  __shared__ float inv[SMAX];
  const int t = threadIdx.x;
  for (int e = t; e < SMAX * SMAX; e += 256) {
    const int i = e % SMAX, j = e / SMAX;
    A[i][j] = (i < s && j < s) ? 0.5f * (GW[i + s * j] + GW[j + s * i]) : 0.f;
  }
  __syncthreads();
  jacobi_smem(A, V, s, order);
  if (t == 0) {
    const float s1 = sqrtf(fmaxf(A[order[0]][order[0]], 0.f));
    for (int r = 0; r < s; ++r) {
      const float sg = sqrtf(fmaxf(A[order[r]][order[r]], 0.f));
      inv[r] = (s1 > 0.f && sg > 1e-6f * s1) ? 1.f / sg : 0.f;
    }
  }
  __syncthreads();
  for (int e = t; e < s * k1; e += 256) {
    const int i = e % s, r = e / s;
    M1[i + s * r] = V[i][order[r]];
  }
  for (int e = t; e < s * k2; e += 256) {
    const int i = e % s, r = e / s;
    M2[i + s * r] = V[i][order[r]] * inv[r];
  }
  for (int e = t; e < k1 * k2; e += 256) {
    const int i = e % k1, j = e / k1;
    const int oi = order[i], oj = order[j];
    float acc = 0.f;
    for (int a = 0; a < s; ++a) {
      float g = 0.f;
      for (int c = 0; c < s; ++c) g = fmaf(0.5f * (GW[a + s * c] + GW[c + s * a]), V[c][oj], g);
      acc = fmaf(V[a][oi], g, acc);
    }
    Broot[i + k1 * j] = acc * inv[j];
  }
}

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

}  // namespace

size_t eig_workspace_bytes(const EigProblem *probs, int nprob) {
  size_t b = align256(sizeof(EigDev) * nprob);
  for (int i = 0; i < nprob; ++i) {
    const int nrb = (probs[i].n + RB - 1) / RB;
    b += align256(sizeof(float) * nrb * ESMAX * 2);
    b += align256(sizeof(float) * nrb * SMAX * SMAX * 2);
    b += align256(sizeof(double) * ESMAX);
    b += align256(sizeof(double) * SMAX * SMAX);
    b += align256(sizeof(float) * SMAX * SMAX);
    b += align256(sizeof(float) * 4);
    b += align256(sizeof(float) * nrb * SMAX);
  }
  return b;
}

static cudaError_t build_batch(const EigProblem *probs, int nprob, void *ws, size_t ws_bytes, EigBatch &b,
                               int &max_nrb) {
  if (nprob > kMaxProb) return cudaErrorInvalidValue;
  if (eig_workspace_bytes(probs, nprob) > ws_bytes) return cudaErrorInvalidValue;
  char *p = static_cast<char *>(ws);
  p += align256(sizeof(EigDev) * nprob);
  max_nrb = 0;
  for (int i = 0; i < nprob; ++i) {
    const EigProblem &q = probs[i];
    if (q.s > SMAX || q.s < 1 || q.K > q.s || q.s > q.n) return cudaErrorInvalidValue;
    EigDev &d = b.p[i];
    d.G = q.G; d.n = q.n; d.s = q.s; d.K = q.K;
    d.nrb = (q.n + RB - 1) / RB;
    max_nrb = d.nrb > max_nrb ? d.nrb : max_nrb;
    d.Q = q.Q; d.Y = q.Y; d.U = q.U; d.GU = q.GU; d.theta = q.theta; d.resid = q.resid;
    d.start = q.start; d.seed = q.seed; d.stream_id = q.stream_id;
    d.partS = reinterpret_cast<float *>(p); p += align256(sizeof(float) * d.nrb * ESMAX * 2);
    d.partH = reinterpret_cast<float *>(p); p += align256(sizeof(float) * d.nrb * SMAX * SMAX * 2);
    d.S = reinterpret_cast<double *>(p); p += align256(sizeof(double) * ESMAX);
    d.H = reinterpret_cast<double *>(p); p += align256(sizeof(double) * SMAX * SMAX);
    d.V = reinterpret_cast<float *>(p); p += align256(sizeof(float) * SMAX * SMAX);
    d.mu = reinterpret_cast<float *>(p); p += align256(sizeof(float) * 4);
    d.colss = reinterpret_cast<float *>(p); p += align256(sizeof(float) * d.nrb * SMAX);
  }
  return cudaSuccess;
}

cudaError_t eig_batched(EigProblem *probs, int nprob, int iters, void *ws, size_t ws_bytes, int *err, cudaStream_t st,
                        int *launches) {
  if (nprob <= 0) return cudaSuccess;
  (void)err;
  EigBatch b;
  int max_nrb = 0;
  cudaError_t e = build_batch(probs, nprob, ws, ws_bytes, b, max_nrb);
  if (e != cudaSuccess) return e;
  int nl = 0;
  const dim3 rows(max_nrb, nprob);
  eig_init_kernel<<<dim3(64, nprob), 256, 0, st>>>(b); ++nl;
  for (int it = 0; it < iters; ++it) {
    eig_gq_kernel<<<rows, 256, 0, st>>>(b, 0); ++nl;
    eig_reduce_kernel<<<dim3((ESMAX + 255) / 256, nprob), 256, 0, st>>>(b, 0); ++nl;
    eig_orth_kernel<<<rows, 256, 0, st>>>(b, 0, 1e-5f); ++nl;
  }
  for (int pass = 0; pass < 2; ++pass) {
    eig_gq_kernel<<<rows, 256, 0, st>>>(b, 1); ++nl;
    eig_reduce_kernel<<<dim3((ESMAX + 255) / 256, nprob), 256, 0, st>>>(b, 0); ++nl;
    eig_orth_kernel<<<rows, 256, 0, st>>>(b, 1, pass == 0 ? 1e-6f : 0.f); ++nl;
  }
  eig_gq_kernel<<<rows, 256, 0, st>>>(b, 2); ++nl;
  eig_reduce_kernel<<<dim3((SMAX * SMAX + 255) / 256, nprob), 256, 0, st>>>(b, 1); ++nl;
  eig_jacobi_kernel<<<nprob, 256, 0, st>>>(b); ++nl;
  eig_finalize_kernel<<<rows, 256, 0, st>>>(b); ++nl;
  eig_resid_kernel<<<nprob, 64, 0, st>>>(b); ++nl;
  if (launches) *launches += nl;
  return cudaGetLastError();
}

cudaError_t cholqr_batched(EigProblem *probs, int nprob, int passes, void *ws, size_t ws_bytes, cudaStream_t st,
                           int *launches) {
  if (nprob <= 0) return cudaSuccess;
  EigBatch b;
  int max_nrb = 0;
  cudaError_t e = build_batch(probs, nprob, ws, ws_bytes, b, max_nrb);
  if (e != cudaSuccess) return e;
  int nl = 0;
  const dim3 rows(max_nrb, nprob);
  for (int pass = 0; pass < passes; ++pass) {
    eig_gq_kernel<<<rows, 256, 0, st>>>(b, 1); ++nl;
    eig_reduce_kernel<<<dim3((ESMAX + 255) / 256, nprob), 256, 0, st>>>(b, 0); ++nl;
    eig_orth_kernel<<<rows, 256, 0, st>>>(b, 1, pass == 0 ? 1e-6f : 0.f); ++nl;
  }
  if (launches) *launches += nl;
  return cudaGetLastError();
}

cudaError_t svd_from_gram_launch(const float *GW, int s, int k1, int k2, float *M1, float *M2, float *Broot,
                                 cudaStream_t st) {
  if (s > SMAX || k1 > s || k2 > s) return cudaErrorInvalidValue;
  svd_from_gram_kernel<<<1, 256, 0, st>>>(GW, s, k1, k2, M1, M2, Broot);
  return cudaGetLastError();
}

cudaError_t transfer_eig_launch(const float *WG, int kw, int kt, int kc, int t_is_left, float *M, float *Broot,
                                cudaStream_t st) {
  if (kt > SMAX || kc > kw || kt > kw) return cudaErrorInvalidValue;
  transfer_eig_kernel<<<1, 256, 0, st>>>(WG, kw, kt, kc, t_is_left, M, Broot);
  return cudaGetLastError();
}

}  // namespace htgb
