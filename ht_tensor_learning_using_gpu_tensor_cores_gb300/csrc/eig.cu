// Top-K eigenpairs of the leaf Grams on the GPU.
//
// Replaces the reference's full cuSOLVER syevd of every n x n Gram followed by
// a copy of the last k columns (third_order_tensor_decompsition/CUDA/Optimized/
// kernel.cu:682-718, htd_tensorcore.cu:133-140).  Only the top K eigenvectors
// are needed, so this is block subspace iteration on G with an oversampled
// block of s <= 64 columns:
//
//   Q_0 = Gaussian (or a supplied start block)
//   Y_i = (G + mu I) Q_i,  Q_{i+1} = Y_i T_i   (T_i: shifted CholeskyQR factor of Y_i)
//   three more CholeskyQR transforms (orthonormal to FP32 rounding)
//   Rayleigh-Ritz: H = Q^T G Q, Jacobi eigen-decomposition of H (s x s),
//   U = Q V[:, top K], GU = G U, residual max_j ||G u_j - theta_j u_j|| / theta_1.
//
// One launch per iteration: since Q_{i+1} = Y_i T_i, a CTA computes its rows
// of Y_{i+1} = (G Y_i + mu Y_i) T_i from the complete Y_i of the previous
// launch, applies T_i by forward substitution, and writes its partial of the
// s x s Gram Y_{i+1}^T Y_{i+1}.  The last CTA to finish (a two-level
// "last block" reduction: atomic tickets, no waiting) sums the partials in a
// fixed order and factors T_{i+1} for the next launch.
//
// Precision: G and the n x s blocks are FP32; the s x s Gram matrices are
// accumulated with compensated FP32 (TwoProduct/TwoSum), as accurate as FP64
// accumulation at FP32 rate -- GB300's FP64 throughput is 1/64 of FP32.  The
// Cholesky runs on the unit-diagonal scaled matrix with a small shift, so it
// cannot break down on rank-deficient blocks.  mu = 1e-9 trace(G) keeps Y
// nonzero on exactly null directions without moving any eigenvector or
// slowing convergence.  Modes with n <= 64 (s == n) skip the iteration: Q = I
// and the Rayleigh-Ritz step is a Jacobi eigen-decomposition of G itself.
#include <vector>

#include "common.cuh"
#include "engine.h"

namespace htgb {
namespace {

constexpr int SMAX = 64;
constexpr int ESMAX = SMAX * (SMAX + 1) / 2;   // packed upper triangle
constexpr int RB = 16;                          // rows per CTA
constexpr int GROUP = 8;                        // CTAs per first-level reduction group
constexpr int kMaxProb = 8;
constexpr int kThreads = 256;

enum StepMode : int { STEP_ITER = 0, STEP_APPLY = 1, STEP_RR = 2 };

struct EigDev {
  const float *G;
  int n, s, K, nrb, ngroups, direct;
  float *buf[4];            // n x s work blocks
  float *U, *GU, *theta, *resid;
  const float *start;
  unsigned long long seed, stream_id;
  float *part;              // [nrb][ESMAX][2]
  float *gpart;             // [ngroups][ESMAX][2]
  int *cnt;                 // [ngroups + 1] tickets, zero between launches
  float *R[2];              // [SMAX*SMAX] upper factors, row-major, ping-pong slots
  float *dsc[2];            // [SMAX] column scaling
  float *V;                 // [SMAX*SMAX] Ritz vectors of H, descending
  float *mu;                // [1]
  float *colss;             // [nrb][SMAX]
};

struct EigBatch {
  EigDev p[kMaxProb];
};

struct StepArgs {
  int mode, src, dst, dst2, tslot, t_identity, want_s;
  float shift, mu_scale;
};

// packed upper triangle, column-major: e = j(j+1)/2 + i, i <= j
HT_DEV void tri_index(int e, int &i, int &j) {
  int jj = static_cast<int>((sqrtf(8.f * e + 1.f) - 1.f) * 0.5f);
  while (jj * (jj + 1) / 2 > e) --jj;
  while ((jj + 1) * (jj + 2) / 2 <= e) ++jj;
  j = jj;
  i = e - jj * (jj + 1) / 2;
}

// fill = 0: only reset the bookkeeping (tickets), for in-place CholeskyQR.
__global__ void eig_init_kernel(const EigBatch probs, int fill) {
  const EigDev &P = probs.p[blockIdx.y];
  const long long total = fill ? static_cast<long long>(P.n) * P.s : 0;
  // direct problems start the Rayleigh-Ritz step from Q = I in buffer 2
  float *dst = P.direct ? P.buf[2] : P.buf[0];
  for (long long idx = blockIdx.x * 256ll + threadIdx.x; idx < total; idx += gridDim.x * 256ll) {
    float v;
    if (P.direct) v = (idx % P.n == idx / P.n) ? 1.f : 0.f;
    else if (P.start) v = P.start[idx];
    else v = gaussian(P.seed, P.stream_id, static_cast<unsigned long long>(idx));
    dst[idx] = v;
  }
  if (blockIdx.x == 0) {
    __shared__ float red[256];
    float t = 0.f;
    for (int i = threadIdx.x; i < P.n; i += 256) t += P.G ? P.G[i + static_cast<long long>(P.n) * i] : 0.f;
    red[threadIdx.x] = t;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
      if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
      __syncthreads();
    }
    if (threadIdx.x == 0) P.mu[0] = 1e-9f * fmaxf(red[0], 0.f);
    for (int i = threadIdx.x; i <= P.ngroups; i += 256) P.cnt[i] = 0;
  }
}

// Forward substitution of one row (one half-warp): x <- (x .* dsc) R^-1 with R
// upper triangular (row-major, stride SMAX) in shared memory.  Lane l owns
// columns l, l+16, l+32, l+48.
HT_DEV void apply_factor_row(float *row, const float *Rs, const float *ds, int s, int l, unsigned mask) {
  float tv[4], q[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const int j = l + 16 * c;
    tv[c] = j < s ? row[j] * ds[j] : 0.f;
  }
  for (int j = 0; j < s; ++j) {
    const int owner = j & 15, cj = j >> 4;
    float qj = 0.f;
#pragma unroll
    for (int c = 0; c < 4; ++c)
      if (l == owner && c == cj) {
        qj = tv[c] / Rs[j * SMAX + j];
        q[c] = qj;
      }
    qj = __shfl_sync(mask, qj, owner, 16);
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const int k = l + 16 * c;
      if (k > j && k < s) tv[c] = fmaf(-qj, Rs[j * SMAX + k], tv[c]);
    }
  }
  __syncwarp(mask);
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const int j = l + 16 * c;
    if (j < s) row[j] = q[c];
  }
}

// 16-byte asynchronous global->shared copy; src_bytes < 16 zero-fills the rest.
HT_DEV void cp_async16(void *smem_dst, const void *gsrc, int src_bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_u32(smem_dst)), "l"(gsrc), "r"(src_bytes)
               : "memory");
}
HT_DEV void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
HT_DEV void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

constexpr int KC = 64;       // k chunk of the G * src product
constexpr int NSTAGE = 3;    // cp.async pipeline depth
constexpr int LDK = KC + 4;  // padded row length (keeps float4 alignment)

// Z[i][j] (16 x s, in Zs) = sum_k G[r0+i, k] src[k, j], G symmetric so row
// r0+i of G is read as column r0+i (contiguous).  Thread t owns rows
// 4*(t>>6)..+3 of column t&63.  Chunks of KC rows of src stream through a
// NSTAGE-deep cp.async ring.  Requires n % 4 == 0 and 16-byte aligned bases.
HT_DEV void gsrc_product_async(const float *G, const float *src, int n, int s, int r0, int rows, float *ring,
                               float (&acc)[4]) {
  const int t = threadIdx.x;
  const int nchunks = (n + KC - 1) / KC;
  auto issue = [&](int c) {
    const int kc = c * KC;
    float *Gd = ring + (c % NSTAGE) * (RB + SMAX) * LDK, *Sd_ = Gd + RB * LDK;
    // G: RB rows x KC/4 float4 = 256 copies
    {
      const int i = t >> 4, k4 = (t & 15) * 4;
      const int kk = kc + k4;
      const int bytes = (i < rows && kk < n) ? 4 * min(4, n - kk) : 0;
      const float *g = G + (bytes ? (static_cast<long long>(kk) + static_cast<long long>(n) * (r0 + i)) : 0);
      cp_async16(Gd + i * LDK + k4, g, bytes);
    }
    // src: SMAX columns x KC/4 float4 = 1024 copies, 4 per thread
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int idx = t + 256 * q;
      const int j = idx >> 4, k4 = (idx & 15) * 4;
      const int kk = kc + k4;
      const int bytes = (j < s && kk < n) ? 4 * min(4, n - kk) : 0;
      const float *g = src + (bytes ? (static_cast<long long>(kk) + static_cast<long long>(n) * j) : 0);
      cp_async16(Sd_ + j * LDK + k4, g, bytes);
    }
  };
  for (int c = 0; c < NSTAGE - 1; ++c) {
    if (c < nchunks) issue(c);
    cp_async_commit();
  }
  const int ig = t >> 6, j = t & 63;
#pragma unroll
  for (int c4 = 0; c4 < 4; ++c4) acc[c4] = 0.f;
  for (int c = 0; c < nchunks; ++c) {
    if (c + NSTAGE - 1 < nchunks) issue(c + NSTAGE - 1);
    cp_async_commit();
    cp_async_wait<NSTAGE - 1>();   // chunk c has landed
    __syncthreads();
    const float *Gd = ring + (c % NSTAGE) * (RB + SMAX) * LDK, *Sd_ = Gd + RB * LDK;
#pragma unroll 4
    for (int kk = 0; kk < KC; kk += 4) {
      const float4 q = *reinterpret_cast<const float4 *>(Sd_ + j * LDK + kk);
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const float4 g = *reinterpret_cast<const float4 *>(Gd + (4 * ig + r) * LDK + kk);
        acc[r] = fmaf(g.x, q.x, fmaf(g.y, q.y, fmaf(g.z, q.z, fmaf(g.w, q.w, acc[r]))));
      }
    }
    __syncthreads();   // the stage is refilled NSTAGE-1 chunks later
  }
  cp_async_wait<0>();
}

// Last-block bookkeeping: returns true in exactly one CTA of the group /
// of the whole problem once every member has published its partial.
HT_DEV bool arrive(int *counter, int members, int *s_flag) {
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    const int tk = atomicAdd(counter, 1);
    const int last = (tk == members - 1) ? 1 : 0;
    if (last) *counter = 0;   // every member has arrived: reset for the next launch
    *s_flag = last;
  }
  __syncthreads();
  const bool last = *s_flag != 0;
  if (last) __threadfence();
  return last;
}

// acc += sum of the (hi, lo) pairs of entry e in partials [first, first+count),
// in order; loads are issued GROUP at a time so their latencies overlap.
HT_DEV void sum_pairs(Acc2 &acc, const float *base, int first, int count, int e) {
  for (int r0 = 0; r0 < count; r0 += GROUP) {
    float hi[GROUP], lo[GROUP];
#pragma unroll
    for (int q = 0; q < GROUP; ++q) {
      if (r0 + q < count) {
        const float *p = base + (static_cast<long long>(first + r0 + q) * ESMAX + e) * 2;
        hi[q] = __ldcg(p);
        lo[q] = __ldcg(p + 1);
      } else {
        hi[q] = 0.f;
        lo[q] = 0.f;
      }
    }
#pragma unroll
    for (int q = 0; q < GROUP; ++q) acc2_add(acc, hi[q], lo[q]);
  }
}

// Scaled, shifted Cholesky of the packed s x s matrix Sd (double): writes the
// upper factor R (row-major, stride SMAX) and the scaling dsc to global memory.
HT_DEV void factor_and_store(const double *Sd, int s, float shift, float *A, float *dsc_sm, float *Rout, float *dout) {
  const int t = threadIdx.x;
  for (int j = t; j < s; j += kThreads) {
    const double d = Sd[j * (j + 1) / 2 + j];
    dsc_sm[j] = d > 1e-300 ? static_cast<float>(1.0 / sqrt(d)) : 0.f;
  }
  __syncthreads();
  const int E = s * (s + 1) / 2;
  for (int e = t; e < E; e += kThreads) {
    int i, j;
    tri_index(e, i, j);
    float v = static_cast<float>(Sd[e] * static_cast<double>(dsc_sm[i]) * static_cast<double>(dsc_sm[j]));
    if (i == j) v = (dsc_sm[j] > 0.f ? 1.f : 0.f) + shift;
    A[i * SMAX + j] = v;
  }
  __syncthreads();
  // right-looking Cholesky A = R^T R on the upper triangle; step j updates rows
  // > j from the unscaled row j, then scales row j (never touched again)
  const int warp = t >> 5, lane = t & 31;
  for (int j = 0; j < s; ++j) {
    const float d = sqrtf(fmaxf(A[j * SMAX + j], 1e-30f));
    const float inv = 1.f / d;
    for (int i = j + 1 + warp; i < s; i += kThreads / 32) {
      const float rji = A[j * SMAX + i] * inv;
      for (int k = i + lane; k < s; k += 32) A[i * SMAX + k] = fmaf(-rji, A[j * SMAX + k] * inv, A[i * SMAX + k]);
    }
    __syncthreads();
    for (int k = j + t; k < s; k += kThreads) A[j * SMAX + k] = (k == j) ? d : A[j * SMAX + k] * inv;
  }
  __syncthreads();
  for (int e = t; e < s * SMAX; e += kThreads) {
    const int i = e / SMAX, k = e % SMAX;
    Rout[e] = (k >= i && k < s) ? A[e] : 0.f;
  }
  for (int j = t; j < s; j += kThreads) dout[j] = dsc_sm[j];
}

// Cyclic Jacobi on a symmetric s x s matrix held in shared memory (s <= SMAX),
// 256 threads, round-robin ("circle method") ordering so every round rotates
// s/2 disjoint pairs in parallel.  On return A is diagonal to FP32 rounding,
// V holds the eigenvectors and order[] the indices by descending eigenvalue.
HT_DEV void jacobi_smem(float (*A)[SMAX + 1], float (*V)[SMAX + 1], int s, int *order) {
  __shared__ float rh[SMAX / 2], sn[SMAX / 2];
  __shared__ int pp[SMAX / 2], qq[SMAX / 2];
  const int t = threadIdx.x;
  const int m = (s + 1) & ~1;   // even number of players (a dummy index when s is odd)
  for (int e = t; e < SMAX * SMAX; e += 256) {
    const int i = e % SMAX, j = e / SMAX;
    V[i][j] = (i == j) ? 1.f : 0.f;
  }
  __syncthreads();
  // A pair rotates while its coupling is above 2.4e-7 (two FP32 units of
  // rounding) relative to sqrt(a_pp a_qq), the test that keeps small
  // eigenvalues' vectors accurate (Demmel and Veselic, "Jacobi's method is
  // more accurate than QR", 1992).  The rotated pair's new diagonal is
  // formed as a_pp - t a_pq, a_qq + t a_pq and its coupling set to exactly
  // zero (Rutishauser's update), so rounding does not regenerate it and the
  // test terminates even between null directions.  Sweeps stop after one
  // that rotated nothing.  Rotations are applied as x - s (y + rho x),
  // y + s (x - rho y) with rho = s / (1 + c): for the many tiny late
  // rotations c rounds to 1, and the plain c x - s y form would then grow every
  // column of V by s^2/2 per rotation (a 1e-5 loss of orthogonality after ten
  // sweeps); this form carries that second-order term explicitly.
  for (int sweep = 0; sweep < 20 && m > 1; ++sweep) {
    int rotated = 0;
    for (int round = 0; round < m - 1; ++round) {
      int did = 0, pme = 0, qme = 0;
      float tt = 0.f, app = 0.f, aqq = 0.f;
      if (t < m / 2) {
        // position 0 is fixed, positions 1..m-1 rotate by one each round
        const int pa = t, pb = m - 1 - t;
        int p = pa == 0 ? 0 : 1 + ((pa - 1 + round) % (m - 1));
        int q = pb == 0 ? 0 : 1 + ((pb - 1 + round) % (m - 1));
        if (p > q) { const int tmp = p; p = q; q = tmp; }
        float rho = 0.f, sv = 0.f;
        if (q < s) {
          const float apq = A[p][q];
          if (fabsf(apq) > 1e-30f && fabsf(apq) > 2.4e-7f * sqrtf(fabsf(A[p][p] * A[q][q]))) {
            const float tau = (A[q][q] - A[p][p]) / (2.f * apq);
            tt = (tau >= 0.f ? 1.f : -1.f) / (fabsf(tau) + sqrtf(1.f + tau * tau));
            const float c = 1.f / sqrtf(1.f + tt * tt);
            sv = tt * c;
            rho = sv / (1.f + c);
            app = A[p][p] - tt * apq;
            aqq = A[q][q] + tt * apq;
            did = 1;
          }
        }
        pp[t] = p; qq[t] = q; rh[t] = rho; sn[t] = sv;
        pme = p; qme = q;
      }
      rotated |= __syncthreads_or(did);
      for (int e = t; e < (m / 2) * s; e += 256) {   // rows: A <- J^T A
        const int pr = e / s, j = e % s;
        const int p = pp[pr], q = qq[pr];
        if (q >= s) continue;
        const float sv = sn[pr], rho = rh[pr];
        const float ap = A[p][j], aq = A[q][j];
        A[p][j] = ap - sv * (aq + rho * ap);
        A[q][j] = aq + sv * (ap - rho * aq);
      }
      __syncthreads();
      for (int e = t; e < (m / 2) * s; e += 256) {   // columns: A <- A J, V <- V J
        const int pr = e / s, i = e % s;
        const int p = pp[pr], q = qq[pr];
        if (q >= s) continue;
        const float sv = sn[pr], rho = rh[pr];
        const float ap = A[i][p], aq = A[i][q];
        A[i][p] = ap - sv * (aq + rho * ap);
        A[i][q] = aq + sv * (ap - rho * aq);
        const float vp = V[i][p], vq = V[i][q];
        V[i][p] = vp - sv * (vq + rho * vp);
        V[i][q] = vq + sv * (vp - rho * vq);
      }
      __syncthreads();
      if (did) {
        A[pme][pme] = app;
        A[qme][qme] = aqq;
        A[pme][qme] = 0.f;
        A[qme][pme] = 0.f;
      }
      __syncthreads();
    }
    if (!rotated) break;
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

// One step of the eigen-solver for every problem of the batch (see the file
// comment).  ITER: dst = (G src + mu src) T; APPLY: dst = src T (in place
// allowed); RR: dst = src T, dst2 = (G src) T and the Rayleigh quotient.
__global__ void __launch_bounds__(kThreads) eig_step_kernel(const EigBatch probs, const StepArgs a) {
  const EigDev &P = probs.p[blockIdx.y];
  const int rb = blockIdx.x;
  if (rb >= P.nrb) return;
  if (P.direct && a.mode != STEP_RR) return;
  extern __shared__ __align__(16) float sm[];
  float *Rs = sm;                                   // SMAX*SMAX
  float *ds = Rs + SMAX * SMAX;                     // SMAX
  float *Zs = ds + SMAX;                            // RB*SMAX  (rows of the result)
  float *Qr = Zs + RB * SMAX;                       // RB*SMAX  (RR: rows of Q)
  float *Gs = Qr + RB * SMAX;                       // 64*(RB+1)   (scalar path)
  float *Ss = Gs + 64 * (RB + 1);                   // ring of NSTAGE*(RB+SMAX)*LDK floats (async path),
                                                    // or 64*68 (scalar path); 16-byte aligned
  // the final reducer's scratch aliases the ring (dead once the product is done)
  double *Sd = reinterpret_cast<double *>(Ss);              // ESMAX
  float *Vs = reinterpret_cast<float *>(Sd + ESMAX);        // SMAX*(SMAX+1) (RR Jacobi)
  __shared__ int s_flag;
  __shared__ int order[SMAX];
  const int n = P.n, s = P.s, t = threadIdx.x;
  const int r0 = rb * RB;
  const int rows = min(RB, n - r0);
  const float *src = P.buf[a.src];
  const bool ident = a.t_identity || P.direct;

  if (!ident) {
    for (int e = t; e < SMAX * SMAX; e += kThreads) Rs[e] = P.R[a.tslot][e];
    for (int j = t; j < SMAX; j += kThreads) ds[j] = P.dsc[a.tslot][j];
  }
  // rows of src owned by this CTA
  for (int e = t; e < RB * SMAX; e += kThreads) {
    const int i = e % RB, j = e / RB;
    const float v = (i < rows && j < s) ? src[(r0 + i) + static_cast<long long>(n) * j] : 0.f;
    if (a.mode == STEP_APPLY) Zs[i * SMAX + j] = v;
    else Qr[i * SMAX + j] = v;
  }
  if (a.mode != STEP_APPLY) {
    const float mu = (a.mode == STEP_ITER) ? P.mu[0] * a.mu_scale : 0.f;
    const bool vec = (n % 4 == 0) && ((reinterpret_cast<uintptr_t>(P.G) | reinterpret_cast<uintptr_t>(src)) & 15u) == 0;
    if (vec) {
      float acc[4];
      gsrc_product_async(P.G, src, n, s, r0, rows, Ss, acc);
      const int ig = t >> 6, j = t & 63;
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const int i = 4 * ig + r;
        Zs[i * SMAX + j] = (i < rows && j < s) ? acc[r] + mu * Qr[i * SMAX + j] : 0.f;
      }
    } else {
      // Z = G[rows, :] src, scalar loads (unaligned shapes)
      const int i = t >> 4, cg = t & 15;
      float acc[4] = {0.f, 0.f, 0.f, 0.f};
      for (int kc = 0; kc < n; kc += 64) {
        __syncthreads();
        for (int e = t; e < 64 * RB; e += kThreads) {
          const int kk = e % 64, ii = e / 64;
          Gs[kk * (RB + 1) + ii] =
              (kc + kk < n && ii < rows) ? P.G[(kc + kk) + static_cast<long long>(n) * (r0 + ii)] : 0.f;
        }
        for (int e = t; e < 64 * SMAX; e += kThreads) {
          const int kk = e % 64, jj = e / 64;
          Ss[kk * 68 + jj] = (kc + kk < n && jj < s) ? src[(kc + kk) + static_cast<long long>(n) * jj] : 0.f;
        }
        __syncthreads();
#pragma unroll 8
        for (int kk = 0; kk < 64; ++kk) {
          const float g = Gs[kk * (RB + 1) + i];
          const float4 q4 = *reinterpret_cast<const float4 *>(&Ss[kk * 68 + 4 * cg]);
          acc[0] = fmaf(g, q4.x, acc[0]);
          acc[1] = fmaf(g, q4.y, acc[1]);
          acc[2] = fmaf(g, q4.z, acc[2]);
          acc[3] = fmaf(g, q4.w, acc[3]);
        }
      }
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const int j = 4 * cg + c;
        Zs[i * SMAX + j] = (i < rows && j < s) ? acc[c] + mu * Qr[i * SMAX + j] : 0.f;
      }
    }
  }
  __syncthreads();
  // apply the previous factor: one half-warp per row
  if (!ident) {
    const int half = t >> 4, l = t & 15;
    const unsigned mask = 0xFFFFu << (16 * (half & 1));
    apply_factor_row(Zs + half * SMAX, Rs, ds, s, l, mask);
    if (a.mode == STEP_RR) apply_factor_row(Qr + half * SMAX, Rs, ds, s, l, mask);
  }
  __syncthreads();
  float *dst = P.buf[a.dst];
  if (a.mode == STEP_RR) {
    float *dst2 = P.buf[a.dst2];
    for (int e = t; e < RB * SMAX; e += kThreads) {
      const int i = e % RB, j = e / RB;
      if (i < rows && j < s) {
        dst[(r0 + i) + static_cast<long long>(n) * j] = Qr[i * SMAX + j];
        dst2[(r0 + i) + static_cast<long long>(n) * j] = Zs[i * SMAX + j];
      }
    }
  } else {
    for (int e = t; e < RB * SMAX; e += kThreads) {
      const int i = e % RB, j = e / RB;
      if (i < rows && j < s) dst[(r0 + i) + static_cast<long long>(n) * j] = Zs[i * SMAX + j];
    }
  }
  if (!a.want_s) return;
  // partial of the s x s Gram (ITER/APPLY: Y^T Y, RR: Q^T Y), packed upper triangle
  const int E = s * (s + 1) / 2;
  const float *L = (a.mode == STEP_RR) ? Qr : Zs;
  {
    const int j = t & 63, ib = t >> 6;   // column j, rows ib, ib+4, ... <= j
    if (j < s) {
      float zc[RB];
#pragma unroll
      for (int r = 0; r < RB; ++r) zc[r] = Zs[r * SMAX + j];
      for (int i = ib; i <= j; i += 4) {
        Acc2 acc = {0.f, 0.f};
#pragma unroll
        for (int r = 0; r < RB; ++r) acc2_add_prod(acc, L[r * SMAX + i], zc[r]);   // rows >= `rows` are zero
        float *d = P.part + (static_cast<long long>(rb) * ESMAX + j * (j + 1) / 2 + i) * 2;
        d[0] = acc.s;
        d[1] = acc.c;
      }
    }
  }
  // two-level deterministic reduction by the last CTAs to arrive
  const int g = rb / GROUP;
  const int gsize = min(GROUP, P.nrb - g * GROUP);
  if (!arrive(&P.cnt[g], gsize, &s_flag)) return;
  for (int e = t; e < E; e += kThreads) {
    Acc2 acc = {0.f, 0.f};
    sum_pairs(acc, P.part, g * GROUP, gsize, e);
    float *d = P.gpart + (static_cast<long long>(g) * ESMAX + e) * 2;
    d[0] = acc.s;
    d[1] = acc.c;
  }
  if (!arrive(&P.cnt[P.ngroups], P.ngroups, &s_flag)) return;
  for (int e = t; e < E; e += kThreads) {
    Acc2 acc = {0.f, 0.f};
    sum_pairs(acc, P.gpart, 0, P.ngroups, e);
    Sd[e] = static_cast<double>(acc.s) + static_cast<double>(acc.c);
  }
  __syncthreads();
  if (a.mode != STEP_RR) {
    factor_and_store(Sd, s, a.shift, Rs, ds, P.R[a.tslot ^ 1], P.dsc[a.tslot ^ 1]);
    return;
  }
  // Rayleigh-Ritz: Jacobi on H (symmetrised from the upper triangle)
  float (*A)[SMAX + 1] = reinterpret_cast<float (*)[SMAX + 1]>(Rs);
  float (*VV)[SMAX + 1] = reinterpret_cast<float (*)[SMAX + 1]>(Vs);
  for (int e = t; e < SMAX * SMAX; e += kThreads) {
    const int i = e % SMAX, j = e / SMAX;
    float v = 0.f;
    if (i < s && j < s) v = static_cast<float>(i <= j ? Sd[j * (j + 1) / 2 + i] : Sd[i * (i + 1) / 2 + j]);
    A[i][j] = v;
  }
  __syncthreads();
  jacobi_smem(A, VV, s, order);
  for (int e = t; e < s * s; e += kThreads) {
    const int i = e % s, r = e / s;
    P.V[i + s * r] = VV[i][order[r]];
  }
  for (int r = t; r < P.K; r += kThreads) P.theta[r] = A[order[r]][order[r]];
}

// U = Q V[:, :K], GU = Y V[:, :K], residual max_j ||GU_j - theta_j U_j|| / theta_1.
__global__ void __launch_bounds__(kThreads) eig_final_kernel(const EigBatch probs, int qbuf, int ybuf) {
  const EigDev &P = probs.p[blockIdx.y];
  const int rb = blockIdx.x;
  if (rb >= P.nrb) return;
  const int n = P.n, s = P.s, K = P.K;
  __shared__ float Vsm[SMAX][SMAX + 1];
  __shared__ float Qr[RB][SMAX + 1];
  __shared__ float Yr[RB][SMAX + 1];
  __shared__ float res[RB][SMAX + 1];
  __shared__ int s_flag;
  const int t = threadIdx.x;
  const int r0 = rb * RB;
  const float *Q = P.buf[qbuf], *Y = P.buf[ybuf];
  for (int e = t; e < SMAX * SMAX; e += kThreads) {
    const int i = e % SMAX, j = e / SMAX;
    Vsm[i][j] = (i < s && j < s) ? P.V[i + s * j] : 0.f;
  }
  for (int e = t; e < RB * SMAX; e += kThreads) {
    const int i = e % RB, j = e / RB;
    const bool ok = r0 + i < n && j < s;
    Qr[i][j] = ok ? Q[(r0 + i) + static_cast<long long>(n) * j] : 0.f;
    Yr[i][j] = ok ? Y[(r0 + i) + static_cast<long long>(n) * j] : 0.f;
  }
  __syncthreads();
  const int i = t / 16, jb = t % 16;
  for (int c = 0; c < 4; ++c) {
    const int j = jb + 16 * c;
    float u = 0.f, gu = 0.f;
    if (j < K) {
      for (int k = 0; k < s; ++k) {
        u = fmaf(Qr[i][k], Vsm[k][j], u);
        gu = fmaf(Yr[i][k], Vsm[k][j], gu);
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
  for (int j = t; j < K; j += kThreads) {
    float acc = 0.f;
    for (int r = 0; r < RB; ++r) acc += res[r][j];
    P.colss[static_cast<long long>(rb) * SMAX + j] = acc;
  }
  if (!arrive(&P.cnt[P.ngroups], P.nrb, &s_flag)) return;
  __shared__ float colmax[SMAX];
  if (t < SMAX) {
    float acc = 0.f;
    if (t < K) {
      for (int r0 = 0; r0 < P.nrb; r0 += 8) {
        float v[8];
#pragma unroll
        for (int q = 0; q < 8; ++q)
          v[q] = (r0 + q < P.nrb) ? __ldcg(P.colss + static_cast<long long>(r0 + q) * SMAX + t) : 0.f;
#pragma unroll
        for (int q = 0; q < 8; ++q) acc += v[q];
      }
    }
    colmax[t] = sqrtf(acc);
  }
  __syncthreads();
  if (t == 0) {
    float m = 0.f;
    for (int j = 0; j < K; ++j) m = fmaxf(m, colmax[j]);
    const float th = P.theta[0];
    P.resid[0] = th > 0.f ? m / th : m;
  }
}

// Transfer-tensor step of the complementary-leaf construction.  WG = W^T G_c W
// (kw x kw, leading dimension kw) for the complementary leaf's Ritz block W;
// V = W[:, :kt].  With GV = V^T G_c V = P diag(lam) P^T:
//   M     = P diag(lam^-1/2)   (columns with lam <= 1e-12 lam_max are zero)
//   Broot = M^T V^T G_c U_c    (kt x kc)
// and the caller forms B_t = C_V M.  On the columns U_c shares with V
// (u < min(kt, kc)) V^T G_c U_c = GV[:, u], so Broot = diag(lam^1/2) P^T there:
// writing it that way makes B_t Broot = C_V P P^T exactly, instead of relying on
// lam^-1 * lam cancelling in FP32, which fails for ill-conditioned Grams.
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
    const int oc = order[r];
    float acc;
    if (u < kt) {
      acc = inv[r] > 0.f ? sqrtf(A[oc][oc]) * V[u][oc] : 0.f;
    } else {
      acc = 0.f;
      for (int c = 0; c < kt; ++c) acc = fmaf(V[c][oc] * inv[r], 0.5f * (WG[c + kw * u] + WG[u + kw * c]), acc);
    }
    if (t_is_left) Broot[r + kt * u] = acc;
    else Broot[u + kc * r] = acc;
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

constexpr size_t kRingFloats = NSTAGE * (RB + SMAX) * LDK;
constexpr size_t kReducerFloats = 2 * ESMAX + SMAX * (SMAX + 1);
constexpr size_t kStepSmem = sizeof(float) * (SMAX * SMAX + SMAX + 2 * RB * SMAX + 64 * (RB + 1) +
                                              (kRingFloats > kReducerFloats ? kRingFloats : kReducerFloats)) +
                             64;

}  // namespace

size_t eig_workspace_bytes(const EigProblem *probs, int nprob) {
  size_t b = 0;
  for (int i = 0; i < nprob; ++i) {
    const int nrb = (probs[i].n + RB - 1) / RB;
    const int ng = (nrb + GROUP - 1) / GROUP;
    b += 4 * align256(sizeof(float) * static_cast<size_t>(probs[i].n) * SMAX);
    b += align256(sizeof(float) * nrb * ESMAX * 2);
    b += align256(sizeof(float) * ng * ESMAX * 2);
    b += align256(sizeof(int) * (ng + 1));
    b += 2 * align256(sizeof(float) * SMAX * SMAX) + 2 * align256(sizeof(float) * SMAX);
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
  max_nrb = 0;
  for (int i = 0; i < nprob; ++i) {
    const EigProblem &q = probs[i];
    if (q.s > SMAX || q.s < 1 || q.K > q.s || q.s > q.n) return cudaErrorInvalidValue;
    EigDev &d = b.p[i];
    d.G = q.G; d.n = q.n; d.s = q.s; d.K = q.K;
    d.nrb = (q.n + RB - 1) / RB;
    d.ngroups = (d.nrb + GROUP - 1) / GROUP;
    d.direct = (q.G != nullptr && q.s == q.n) ? 1 : 0;
    max_nrb = d.nrb > max_nrb ? d.nrb : max_nrb;
    d.U = q.U; d.GU = q.GU; d.theta = q.theta; d.resid = q.resid;
    d.start = q.start; d.seed = q.seed; d.stream_id = q.stream_id;
    for (int k = 0; k < 4; ++k) {
      d.buf[k] = reinterpret_cast<float *>(p);
      p += align256(sizeof(float) * static_cast<size_t>(q.n) * SMAX);
    }
    d.part = reinterpret_cast<float *>(p); p += align256(sizeof(float) * d.nrb * ESMAX * 2);
    d.gpart = reinterpret_cast<float *>(p); p += align256(sizeof(float) * d.ngroups * ESMAX * 2);
    d.cnt = reinterpret_cast<int *>(p); p += align256(sizeof(int) * (d.ngroups + 1));
    for (int k = 0; k < 2; ++k) {
      d.R[k] = reinterpret_cast<float *>(p); p += align256(sizeof(float) * SMAX * SMAX);
      d.dsc[k] = reinterpret_cast<float *>(p); p += align256(sizeof(float) * SMAX);
    }
    d.V = reinterpret_cast<float *>(p); p += align256(sizeof(float) * SMAX * SMAX);
    d.mu = reinterpret_cast<float *>(p); p += align256(sizeof(float) * 4);
    d.colss = reinterpret_cast<float *>(p); p += align256(sizeof(float) * d.nrb * SMAX);
  }
  return cudaSuccess;
}

static cudaError_t launch_step(const EigBatch &b, int nprob, int max_nrb, StepArgs a, cudaStream_t st) {
  eig_step_kernel<<<dim3(max_nrb, nprob), kThreads, kStepSmem, st>>>(b, a);
  return cudaGetLastError();
}

cudaError_t eig_batched(EigProblem *probs, int nprob, int iters, void *ws, size_t ws_bytes, int *err, cudaStream_t st,
                        int *launches) {
  if (nprob <= 0) return cudaSuccess;
  (void)err;
  EigBatch b;
  int max_nrb = 0;
  cudaError_t e = build_batch(probs, nprob, ws, ws_bytes, b, max_nrb);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(eig_step_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(kStepSmem));
  if (e != cudaSuccess) return e;
  int nl = 0;
  eig_init_kernel<<<dim3(64, nprob), 256, 0, st>>>(b, 1); ++nl;
  int cur = 0, tslot = 0, ident = 1;
  for (int it = 0; it < iters; ++it) {
    StepArgs a{STEP_ITER, cur, cur ^ 1, 0, tslot, ident, 1, 1e-5f, 1.f};
    if ((e = launch_step(b, nprob, max_nrb, a, st)) != cudaSuccess) return e;
    ++nl;
    ident = 0; tslot ^= 1; cur ^= 1;
  }
  // three CholeskyQR transforms: Y_L T_L -> buffer 2, then twice in place
  StepArgs f1{STEP_APPLY, cur, 2, 0, tslot, ident, 1, 1e-6f, 0.f};
  if ((e = launch_step(b, nprob, max_nrb, f1, st)) != cudaSuccess) return e;
  tslot ^= 1;
  StepArgs f2{STEP_APPLY, 2, 2, 0, tslot, 0, 1, 0.f, 0.f};
  if ((e = launch_step(b, nprob, max_nrb, f2, st)) != cudaSuccess) return e;
  tslot ^= 1;
  StepArgs rr{STEP_RR, 2, 3, 0, tslot, 0, 1, 0.f, 0.f};
  if ((e = launch_step(b, nprob, max_nrb, rr, st)) != cudaSuccess) return e;
  eig_final_kernel<<<dim3(max_nrb, nprob), kThreads, 0, st>>>(b, 3, 0);
  nl += 4;
  if (launches) *launches += nl;
  return cudaGetLastError();
}

// In-place CholeskyQR3 of tall blocks (G == nullptr problems, buffer 0 = the matrix).
cudaError_t cholqr_batched(EigProblem *probs, int nprob, int passes, void *ws, size_t ws_bytes, cudaStream_t st,
                           int *launches) {
  if (nprob <= 0) return cudaSuccess;
  EigBatch b;
  int max_nrb = 0;
  cudaError_t e = build_batch(probs, nprob, ws, ws_bytes, b, max_nrb);
  if (e != cudaSuccess) return e;
  for (int i = 0; i < nprob; ++i) b.p[i].buf[0] = probs[i].Q;   // operate on the caller's matrix in place
  e = cudaFuncSetAttribute(eig_step_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(kStepSmem));
  if (e != cudaSuccess) return e;
  int nl = 0;
  eig_init_kernel<<<dim3(1, nprob), 256, 0, st>>>(b, 0);   // zeroes the tickets only
  ++nl;
  int tslot = 0;
  for (int pass = 0; pass <= passes; ++pass) {
    StepArgs a{STEP_APPLY, 0, 0, 0, tslot, pass == 0 ? 1 : 0, pass < passes ? 1 : 0, pass == 0 ? 1e-6f : 0.f, 0.f};
    if ((e = launch_step(b, nprob, max_nrb, a, st)) != cudaSuccess) return e;
    ++nl;
    if (pass < passes) tslot ^= 1;
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
