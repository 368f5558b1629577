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
//   (the float-pair factor leaves Q_L = Y_L T_L orthonormal to ~1e-7)
//   Rayleigh-Ritz: H = Q^T G Q, Jacobi eigen-decomposition of H (s x s),
//   U = Q V[:, top K], GU = G U, residual max_j ||G u_j - theta_j u_j|| / theta_1.
//
// All iterations of every problem run in ONE cooperative launch
// (eig_coop_kernel): since Q_{i+1} = Y_i T_i, a CTA computes its rows of
// Y_{i+1} = (G Y_i + mu Y_i) T_i from the complete Y_i and writes its partial
// of the s x s Gram Y_{i+1}^T Y_{i+1}; after a grid barrier all CTAs reduce
// the partials in a fixed order, and after a second one every CTA of the
// problem factors T_{i+1} itself.  The same kernel, in its CholeskyQR mode,
// orthonormalises tall blocks without a Gram (the 4th-order range finder).
//
// Precision: G and the n x s blocks are FP32; the s x s Gram matrices are
// accumulated with compensated FP32 (TwoProduct/TwoSum), as accurate as FP64
// accumulation at FP32 rate -- GB300's FP64 throughput is 1/64 of FP32.  The
// Cholesky runs on the unit-diagonal scaled matrix with a small shift, so it
// cannot break down on rank-deficient blocks.  mu = 1e-9 trace(G) keeps Y
// nonzero on exactly null directions without moving any eigenvector or
// slowing convergence.  Modes no larger than the block (s == n) skip the iteration: Q = I
// and the Rayleigh-Ritz step is a Jacobi eigen-decomposition of G itself.
#include <algorithm>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "engine.h"

namespace htgb {
namespace {

constexpr int SMAX = 64;
constexpr int ESMAX = SMAX * (SMAX + 1) / 2;   // packed upper triangle
constexpr int GROUP = 8;                        // partials loaded at once by the reduction
constexpr int kMaxProb = 8;

// packed upper triangle, column-major: e = j(j+1)/2 + i, i <= j
HT_DEV void tri_index(int e, int &i, int &j) {
  int jj = static_cast<int>((sqrtf(8.f * e + 1.f) - 1.f) * 0.5f);
  while (jj * (jj + 1) / 2 > e) --jj;
  while ((jj + 1) * (jj + 2) / 2 <= e) ++jj;
  j = jj;
  i = e - jj * (jj + 1) / 2;
}

// 16-byte asynchronous global->shared copy; src_bytes < 16 zero-fills the rest.
HT_DEV void cp_async16(void *smem_dst, const void *gsrc, int src_bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_u32(smem_dst)), "l"(gsrc), "r"(src_bytes)
               : "memory");
}
HT_DEV void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
HT_DEV void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// Cyclic Jacobi on a symmetric s x s matrix held in shared memory (s <= SMAX),
// 256 threads, round-robin ("circle method") ordering: every round rotates up
// to s/2 disjoint pairs.  On return A is diagonal to FP32 rounding, V holds the
// eigenvectors and order[] the indices by descending eigenvalue.  A2 is
// scratch of the same shape.
//
// Rotation rule.  A pair rotates while its coupling is above 2.4e-7 (two FP32
// units of rounding) relative to sqrt(a_pp a_qq), the test that keeps small
// eigenvalues' vectors accurate (Demmel and Veselic, "Jacobi's method is more
// accurate than QR", 1992).  The rotated pair's new diagonal is formed as
// a_pp - t a_pq, a_qq + t a_pq and its coupling set to exactly zero
// (Rutishauser's update), so rounding does not regenerate it and the test
// terminates even between null directions.  Rotations are applied as
// x - s (y + rho x), y + s (x - rho y) with rho = s / (1 + c): for the many
// tiny late rotations c rounds to 1, and the plain c x - s y form would then
// grow every column of V by s^2/2 per rotation (a 1e-5 loss of orthogonality
// after ten sweeps); this form carries that second-order term explicitly.
// The cosine uses a correctly rounded square root (an approximate one makes
// every rotation slightly non-orthogonal, which the exact diagonal update then
// turns into absolute errors on small eigenvalues).
//
// Schedule.  One round is one phase between two barriers: A2 = J^T A J is
// formed block by block (the 2x2 block of pairs (P, P') only depends on A's
// old block and the two pairs' rotations), V's columns are rotated, and the
// threads owning the NEXT round's pairs recompute the three entries they need
// from the old A with the same arithmetic and choose their rotations.  The
// iteration stops once m - 1 consecutive rounds (every pair once) chose no
// rotation, i.e. a full sweep left the matrix unchanged.
struct JacRot {
  int p, q, rot;
  float rho, sn, tt;
};

HT_DEV JacRot jac_choose(int p, int q, int s, float app, float aqq, float apq) {
  JacRot r{p, q, 0, 0.f, 0.f, 0.f};
  if (q < s && fabsf(apq) > 1e-30f && fabsf(apq) > 2.4e-7f * sqrtf(fabsf(app * aqq))) {
    const float tau = (aqq - app) / (2.f * apq);
    r.tt = (tau >= 0.f ? 1.f : -1.f) / (fabsf(tau) + sqrtf(1.f + tau * tau));
    const float c = 1.f / sqrtf(1.f + r.tt * r.tt);
    r.sn = r.tt * c;
    r.rho = r.sn / (1.f + c);
    r.rot = 1;
  }
  return r;
}

HT_DEV void jac_pair(int round, int m, int idx, int &p, int &q) {
  const int pa = idx, pb = m - 1 - idx;
  p = pa == 0 ? 0 : 1 + ((pa - 1 + round) % (m - 1));
  q = pb == 0 ? 0 : 1 + ((pb - 1 + round) % (m - 1));
  if (p > q) {
    const int tmp = p;
    p = q;
    q = tmp;
  }
}

// New 2x2 block (rows of pair a, columns of pair b) of J^T A J.
HT_DEV void jac_block(const float (*A)[SMAX + 1], const JacRot &ja, const JacRot &jb, bool diag, float &a2, float &b2,
                      float &c2, float &d2) {
  const float a = A[ja.p][jb.p], b = A[ja.p][jb.q], c = A[ja.q][jb.p], d = A[ja.q][jb.q];
  if (diag) {
    if (ja.rot) {
      a2 = __fmaf_rn(-ja.tt, b, a);
      d2 = __fmaf_rn(ja.tt, b, d);
      b2 = 0.f;
      c2 = 0.f;
    } else {
      a2 = a; b2 = b; c2 = c; d2 = d;
    }
    return;
  }
  // x - s (y + rho x) and y + s (x - rho y), as explicit fused operations so
  // that every thread that evaluates an entry gets the same bits
  const float a1 = __fmaf_rn(-ja.sn, __fmaf_rn(ja.rho, a, c), a), c1 = __fmaf_rn(ja.sn, __fmaf_rn(-ja.rho, c, a), c);
  const float b1 = __fmaf_rn(-ja.sn, __fmaf_rn(ja.rho, b, d), b), d1 = __fmaf_rn(ja.sn, __fmaf_rn(-ja.rho, d, b), d);
  a2 = __fmaf_rn(-jb.sn, __fmaf_rn(jb.rho, a1, b1), a1);
  b2 = __fmaf_rn(jb.sn, __fmaf_rn(-jb.rho, b1, a1), b1);
  c2 = __fmaf_rn(-jb.sn, __fmaf_rn(jb.rho, c1, d1), c1);
  d2 = __fmaf_rn(jb.sn, __fmaf_rn(-jb.rho, d1, c1), d1);
}

// Entry (i, j) of J^T A J, computed exactly as the block owner computes it.
HT_DEV float jac_entry(const float (*A)[SMAX + 1], const JacRot *J, const int *owner, int i, int j) {
  const int oi = owner[i], oj = owner[j];
  const int a = oi >> 1, b = oj >> 1;
  float v0, v1, v2, v3;
  int r, c;   // row / column position inside the computed block
  if (a <= b) {
    jac_block(A, J[a], J[b], a == b, v0, v1, v2, v3);
    r = oi & 1;
    c = oj & 1;
  } else {
    jac_block(A, J[b], J[a], false, v0, v1, v2, v3);
    r = oj & 1;
    c = oi & 1;
  }
  return r ? (c ? v3 : v2) : (c ? v1 : v0);
}

HT_DEV void jacobi_smem(float (*A)[SMAX + 1], float (*A2)[SMAX + 1], float (*V)[SMAX + 1], int s, int *order) {
  __shared__ JacRot Jbuf[2][SMAX / 2];
  __shared__ int own[2][SMAX];
  __shared__ unsigned short blk_ab[(SMAX / 2) * (SMAX / 2 + 1) / 2];   // upper block (a, b): a | b << 8
  __shared__ unsigned char pair_tab[SMAX - 1][SMAX / 2][2];            // round-robin pairs of every round
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const int m = (s + 1) & ~1;   // even number of players (a dummy index when s is odd)
  const int np = m / 2;
  const int nb = np * (np + 1) / 2;
  for (int e = t; e < SMAX * SMAX; e += 256) {
    const int i = e % SMAX, j = e / SMAX;
    V[i][j] = (i == j) ? 1.f : 0.f;
  }
  for (int e = t; e < nb; e += 256) {
    int a, b;
    tri_index(e, a, b);
    blk_ab[e] = static_cast<unsigned short>(a | (b << 8));
  }
  for (int e = t; e < (m - 1) * np; e += 256) {
    const int r = e / np, idx = e % np;
    int p, q;
    jac_pair(r, m, idx, p, q);
    pair_tab[r][idx][0] = static_cast<unsigned char>(p);
    pair_tab[r][idx][1] = static_cast<unsigned char>(q);
  }
  __syncthreads();
  int cur = 0;
  float (*Ac)[SMAX + 1] = A;
  float (*An)[SMAX + 1] = A2;
  int any = 0;
  if (t < np && m > 1) {
    const int p = pair_tab[0][t][0], q = pair_tab[0][t][1];
    Jbuf[0][t] = jac_choose(p, q, s, A[p][p], A[q][q], A[p][q]);
    own[0][p] = 2 * t;
    own[0][q] = 2 * t + 1;
    any = Jbuf[0][t].rot;
  }
  int quiet = __syncthreads_or(any) ? 0 : 1;
  const int max_rounds = m > 1 ? 20 * (m - 1) : 0;
  int rr = 0;   // round index within the sweep
  for (int round = 0; round < max_rounds && quiet < m - 1; ++round) {
    const JacRot *J = Jbuf[cur];
    const int *ow = own[cur];
    const int rn = rr + 1 == m - 1 ? 0 : rr + 1;
    any = 0;
    if (warp < 7) {
      // A2 = J^T A J: upper blocks (a <= b) and their mirror
      for (int e = t; e < nb; e += 224) {
        const int ab = blk_ab[e], a = ab & 255, b = ab >> 8;
        const JacRot &ja = J[a], &jb = J[b];
        float a2, b2, c2, d2;
        jac_block(Ac, ja, jb, a == b, a2, b2, c2, d2);
        An[ja.p][jb.p] = a2; An[ja.p][jb.q] = b2; An[ja.q][jb.p] = c2; An[ja.q][jb.q] = d2;
        An[jb.p][ja.p] = a2; An[jb.q][ja.p] = b2; An[jb.p][ja.q] = c2; An[jb.q][ja.q] = d2;
      }
      // V <- V J: warp w rotates pairs w, w + 7, ...; lanes own rows lane, lane + 32
      for (int a = warp; a < np; a += 7) {
        const JacRot ja = J[a];
        if (!ja.rot) continue;
        for (int i = lane; i < s; i += 32) {
          const float vp = V[i][ja.p], vq = V[i][ja.q];
          V[i][ja.p] = __fmaf_rn(-ja.sn, __fmaf_rn(ja.rho, vp, vq), vp);
          V[i][ja.q] = __fmaf_rn(ja.sn, __fmaf_rn(-ja.rho, vq, vp), vq);
        }
      }
    } else if (lane < np) {
      // the next round's rotations, from the entries this round produces
      const int p = pair_tab[rn][lane][0], q = pair_tab[rn][lane][1];
      const float app = jac_entry(Ac, J, ow, p, p), aqq = jac_entry(Ac, J, ow, q, q), apq = jac_entry(Ac, J, ow, p, q);
      const JacRot jn = jac_choose(p, q, s, app, aqq, apq);
      Jbuf[cur ^ 1][lane] = jn;
      own[cur ^ 1][p] = 2 * lane;
      own[cur ^ 1][q] = 2 * lane + 1;
      any = jn.rot;
    }
    quiet = __syncthreads_or(any) ? 0 : quiet + 1;
    cur ^= 1;
    rr = rn;
    float (*tmp)[SMAX + 1] = Ac;
    Ac = An;
    An = tmp;
    // first quiet round: if no pair of the whole matrix would rotate (the
    // criterion of jac_choose), the remaining quiet rounds of the sweep would
    // change nothing
    if (quiet == 1) {
      int bad = 0;
      for (int e = t; e < s * (s + 1) / 2; e += 256) {
        int i, j;
        tri_index(e, i, j);
        const float apq = Ac[i][j];
        if (i != j && fabsf(apq) > 1e-30f && fabsf(apq) > 2.4e-7f * sqrtf(fabsf(Ac[i][i] * Ac[j][j]))) bad = 1;
      }
      if (!__syncthreads_or(bad)) break;
    }
  }
  if (Ac != A) {
    for (int e = t; e < s * s; e += 256) A[e % s][e / s] = Ac[e % s][e / s];
    __syncthreads();
  }
  // rank by counting: descending eigenvalues.  NaN counts as -inf and ties go
  // by index, so the ranks always form a permutation (order[] is used as an
  // index: a hole would be an out-of-range shared-memory access)
  for (int j = t; j < s; j += 256) {
    const float dj = isnan(A[j][j]) ? -INFINITY : A[j][j];
    int rank = 0;
    for (int i = 0; i < s; ++i) {
      const float di = isnan(A[i][i]) ? -INFINITY : A[i][i];
      if (di > dj || (di == dj && i < j)) ++rank;
    }
    order[rank] = j;
  }
  __syncthreads();
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
// Transfer-tensor eigen step on WG (kw x kw, leading dimension kw, global or
// shared memory): the top-kt eigenpairs of sym(WG[:kt, :kt]) by Jacobi give
// M (kt x kt) = V diag(lambda^-1/2) and the root transfer tensor
// Broot (kt x kc, or kc x kt when !t_is_left).
HT_DEV void transfer_eig_body(const float *WG, int kw, int kt, int kc, int t_is_left, float *M, float *Broot,
                              float (*A)[SMAX + 1], float (*V)[SMAX + 1], float (*A2)[SMAX + 1], int *order,
                              float *inv) {
  const int t = threadIdx.x;
  for (int e = t; e < SMAX * SMAX; e += 256) {
    const int i = e % SMAX, j = e / SMAX;
    A[i][j] = (i < kt && j < kt) ? 0.5f * (WG[i + kw * j] + WG[j + kw * i]) : 0.f;
  }
  __syncthreads();
  jacobi_smem(A, A2, V, kt, order);
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

__global__ void __launch_bounds__(256) transfer_eig_kernel(const float *WG, int kw, int kt, int kc, int t_is_left,
                                                           float *M, float *Broot) {
  __shared__ float A[SMAX][SMAX + 1];
  __shared__ float V[SMAX][SMAX + 1];
  extern __shared__ float jac_scratch[];   // SMAX * (SMAX + 1) floats
  float (*A2)[SMAX + 1] = reinterpret_cast<float (*)[SMAX + 1]>(jac_scratch);
  __shared__ int order[SMAX];
  __shared__ float inv[SMAX];
  transfer_eig_body(WG, kw, kt, kc, t_is_left, M, Broot, A, V, A2, order, inv);
}

// Grouped transfer tail of the batched path, a CTA per tensor:
//   WG = U^T GU (kw x kw, compensated dot products as gemm_tn_small),
//   the transfer eigen step (M, Bkt; Broot = Bkt^T when t is the right child),
//   Bt = C M (kpq x kt, as matmul_nn).
__global__ void __launch_bounds__(256) transfer_tail_grouped_kernel(const TailJob *__restrict__ jobs) {
  __shared__ float A[SMAX][SMAX + 1];
  __shared__ float V[SMAX][SMAX + 1];
  extern __shared__ float tail_sm[];   // A2 (SMAX * (SMAX + 1)), WG (SMAX * SMAX), M (SMAX * SMAX)
  float (*A2)[SMAX + 1] = reinterpret_cast<float (*)[SMAX + 1]>(tail_sm);
  float *WG = tail_sm + SMAX * (SMAX + 1);
  float *Ms = WG + SMAX * SMAX;
  __shared__ int order[SMAX];
  __shared__ float inv[SMAX];
  __shared__ TailJob J;
  if (threadIdx.x == 0) J = jobs[blockIdx.x];
  __syncthreads();
  const int kw = J.kw, kt = J.kt, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int e = warp; e < kw * kw; e += 8) {
    const int i = e % kw, j = e / kw;
    Acc2 acc = {0.f, 0.f};
    for (int k = lane; k < J.nc; k += 32)
      acc2_add_prod(acc, J.U[k + static_cast<long long>(J.nc) * i], J.GU[k + static_cast<long long>(J.nc) * j]);
    double v = static_cast<double>(acc.s) + static_cast<double>(acc.c);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) WG[i + kw * j] = static_cast<float>(v);
  }
  __syncthreads();
  transfer_eig_body(WG, kw, kt, J.kc, 1, Ms, J.Bkt, A, V, A2, order, inv);
  __syncthreads();
  for (int e = threadIdx.x; e < kt * J.kc && !J.t_is_left; e += 256) {
    const int i = e % kt, j = e / kt;
    J.Broot[j + J.kc * i] = J.Bkt[i + kt * j];
  }
  for (long long idx = threadIdx.x; idx < J.kpq * kt; idx += 256) {
    const long long i = idx % J.kpq;
    const int j = static_cast<int>(idx / J.kpq);
    float sacc = 0.f;
    for (int k = 0; k < kt; ++k) sacc = fmaf(J.C[i + J.kpq * k], Ms[k + kt * j], sacc);
    J.Bt[i + J.kpq * j] = sacc;
  }
}

// SVD of a tall W from its Gram GW = W^T W (s x s): GW = U diag(sigma^2) U^T.
// M1 = U[:, :k1], M2 = U[:, :k2] diag(1/sigma) (zero where sigma <= 1e-6 sigma_1),
// Broot = M1^T GW M2 (k1 x k2).
// Up to four independent problems, one CTA each (blockIdx.x).
struct SvdGramBatch {
  SvdGramProb p[4];
};

__global__ void __launch_bounds__(256) svd_from_gram_kernel(const SvdGramBatch batch) {
  const SvdGramProb &pb = batch.p[blockIdx.x];
  const float *GW = pb.GW;
  const int s = pb.s, k1 = pb.k1, k2 = pb.k2;
  float *M1 = pb.M1, *M2 = pb.M2, *Broot = pb.Broot;
  __shared__ float A[SMAX][SMAX + 1];
  __shared__ float V[SMAX][SMAX + 1];
  extern __shared__ float jac_scratch[];   // SMAX * (SMAX + 1) floats
  float (*A2)[SMAX + 1] = reinterpret_cast<float (*)[SMAX + 1]>(jac_scratch);
  __shared__ int order[SMAX];
  __shared__ float inv[SMAX];
  const int t = threadIdx.x;
  for (int e = t; e < SMAX * SMAX; e += 256) {
    const int i = e % SMAX, j = e / SMAX;
    A[i][j] = (i < s && j < s) ? 0.5f * (GW[i + s * j] + GW[j + s * i]) : 0.f;
  }
  __syncthreads();
  jacobi_smem(A, A2, V, s, order);
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
  // Broot = M1^T (GW_sym V[:, order[:k2]]) diag(inv): the symmetrised Gram in
  // the Jacobi scratch, the product P = GW_sym V_k2 in A (its diagonal is read
  // above), both in shared memory
  for (int e = t; e < s * s; e += 256) {
    const int a = e % s, c = e / s;
    A2[a][c] = 0.5f * (GW[a + s * c] + GW[c + s * a]);
  }
  __syncthreads();
  for (int e = t; e < s * k2; e += 256) {
    const int a = e % s, j = e / s;
    const int oj = order[j];
    float g = 0.f;
    for (int c = 0; c < s; ++c) g = fmaf(A2[a][c], V[c][oj], g);
    A[a][j] = g;
  }
  __syncthreads();
  for (int e = t; e < k1 * k2; e += 256) {
    const int i = e % k1, j = e / k1;
    const int oi = order[i];
    float acc = 0.f;
    for (int a = 0; a < s; ++a) acc = fmaf(V[a][oi], A[a][j], acc);
    Broot[i + k1 * j] = acc * inv[j];
  }
}

// ------------------------------------------------------------------------
// Cooperative eigen-solver: the whole subspace iteration of every problem of
// the batch in ONE launch.  CTAs of one problem own consecutive row ranges;
// grid-wide barriers (bounded spins on a counter / generation pair) separate
// the phases, so there is no single-CTA tail per iteration: the s x s Gram
// partials are reduced by all CTAs (each sums a slice of the entries over the
// problem's CTAs, in CTA order) and every CTA of the problem factors the
// reduced Gram itself.  Direct problems (s == n) run in CTAs of their own that
// take no part in the barriers.
constexpr int RBMAX = 32;                 // rows per sub-block
constexpr int CNS = 4;                    // cp.async stages of the G * Y product
constexpr int CLD = 68;                   // padded k length of a staged row
constexpr int kCoopMaxCta = 160;          // cap on the cooperative grid (sizes the per-CTA partials)
constexpr int kMaxEntPerThread = (ESMAX + 255) / 256;

struct CoopProb {
  const float *G;
  int n, s, K;
  int cta0, ncta, rows;                   // CTAs [cta0, cta0 + ncta), `rows` rows each (last fewer)
  float *buf[4];                          // n x s blocks (column stride n)
  float *U, *GU, *theta, *resid;
  const float *start;
  unsigned long long seed, stream_id;
  float *part;                            // [ncta][ESMAX][2]
  double *S;                              // [ESMAX] reduced Gram / Rayleigh quotient
  float *V;                               // [SMAX * SMAX] Ritz vectors of H (column j = vector j)
  float *colss;                           // [ncta][SMAX] residual partials
};

struct CoopBatch {
  CoopProb p[kMaxProb];
  int nprob, iters, refine, orth_passes, nsync, ent_total;
  int ent_off[kMaxProb + 1];
  int direct_idx[kMaxProb];               // problem index of direct CTA d (blockIdx.x - nsync)
  unsigned *bar;                          // [2]: arrivals, generation (zero at launch)
  int *err;
};

constexpr size_t kCoopAlias = 2 * ESMAX + 3 * SMAX * (SMAX + 1);                // Sd (doubles) + A + V + A2
// dynamic shared memory of a solver whose G * Y product runs a `stages`-deep ring
constexpr size_t coop_smem(int stages) {
  return sizeof(float) * (SMAX * SMAX + SMAX + 2 * RBMAX * SMAX +
                          (size_t(stages) * (RBMAX + SMAX) * CLD > kCoopAlias ? size_t(stages) * (RBMAX + SMAX) * CLD
                                                                                : kCoopAlias)) +
         64;
}
constexpr size_t kCoopSmem = coop_smem(CNS);
// the grouped solver (a CTA per problem): a 2-stage ring, so that two CTAs share an SM
constexpr int kGroupedStages = 2;
constexpr size_t kGroupedSmem = coop_smem(kGroupedStages);

// Bounded grid barrier over the first `members` CTAs.  False (and the error
// word set) when the wait ran past limit_ns; the caller then returns.
HT_DEV bool grid_barrier(unsigned *bar, unsigned members, int *err, int *s_ok, uint64_t limit_ns = kWaitLimitNs) {
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned *gen = bar + 1;
    const unsigned g = *gen;
    __threadfence();
    int ok = 1;
    if (atomicAdd(bar, 1u) == members - 1) {
      atomicExch(bar, 0u);
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      const uint64_t t0 = global_timer_ns();
      while (*gen == g) {
        __nanosleep(64);
        if (global_timer_ns() - t0 > limit_ns) {
          ok = 0;
          break;
        }
      }
    }
    __threadfence();
    if (!ok) report_error(err, kErrTimeout);
    *s_ok = ok;
  }
  __syncthreads();
  return *s_ok != 0;
}

// G * Y product for the CTA's rows, K split across the 8 warps: warp w takes
// k = 8w .. 8w+7 of every 64-wide chunk, lane l columns l and l + 32, and
// every row (RT >= rows, padded); the G operand is a broadcast shared-memory
// load.  The eight partial blocks are summed in a fixed order at the end.
template <int RT, int NC, int NS>
HT_DEV void coop_product_t(const float *G, const float *Y, int n, int s, int r0, int rows, float *ring, float *Zs) {
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const bool vec = (n % 4 == 0) && ((reinterpret_cast<uintptr_t>(G) | reinterpret_cast<uintptr_t>(Y)) & 15u) == 0;
  const int nchunks = (n + 63) / 64;
  constexpr int STAGE = (RBMAX + SMAX) * CLD;
  auto issue = [&](int c) {
    const int kc = c * 64;
    float *Gd = ring + (c % NS) * STAGE, *Yd = Gd + RBMAX * CLD;
    if (vec) {
      for (int idx = t; idx < RT * 16; idx += 256) {
        const int i = idx >> 4, k4 = (idx & 15) * 4, kk = kc + k4;
        const int bytes = (i < rows && kk < n) ? 4 * min(4, n - kk) : 0;
        const float *g = bytes ? G + static_cast<long long>(r0 + i) * n + kk : G;
        cp_async16(Gd + i * CLD + k4, g, bytes);
      }
      for (int idx = t; idx < 32 * NC * 16; idx += 256) {
        const int j = idx >> 4, k4 = (idx & 15) * 4, kk = kc + k4;
        const int bytes = (j < s && kk < n) ? 4 * min(4, n - kk) : 0;
        const float *y = bytes ? Y + static_cast<long long>(j) * n + kk : Y;
        cp_async16(Yd + j * CLD + k4, y, bytes);
      }
    } else {
      for (int idx = t; idx < RT * 64; idx += 256) {
        const int i = idx >> 6, k = idx & 63, kk = kc + k;
        Gd[i * CLD + k] = (i < rows && kk < n) ? __ldcg(G + static_cast<long long>(r0 + i) * n + kk) : 0.f;
      }
      for (int idx = t; idx < 32 * NC * 64; idx += 256) {
        const int j = idx >> 6, k = idx & 63, kk = kc + k;
        Yd[j * CLD + k] = (j < s && kk < n) ? __ldcg(Y + static_cast<long long>(j) * n + kk) : 0.f;
      }
    }
  };
  float acc[RT][NC];
#pragma unroll
  for (int r = 0; r < RT; ++r)
#pragma unroll
    for (int c = 0; c < NC; ++c) acc[r][c] = 0.f;
  for (int c = 0; c < NS - 1; ++c) {
    if (c < nchunks) issue(c);
    cp_async_commit();
  }
  for (int c = 0; c < nchunks; ++c) {
    if (c + NS - 1 < nchunks) issue(c + NS - 1);
    cp_async_commit();
    cp_async_wait<NS - 1>();
    __syncthreads();
    const float *Gd = ring + (c % NS) * STAGE, *Yd = Gd + RBMAX * CLD;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int kk = 8 * warp + 4 * h;
      float4 y[NC];
#pragma unroll
      for (int q = 0; q < NC; ++q) y[q] = *reinterpret_cast<const float4 *>(Yd + (lane + 32 * q) * CLD + kk);
#pragma unroll
      for (int r = 0; r < RT; ++r) {
        const float4 g = *reinterpret_cast<const float4 *>(Gd + r * CLD + kk);
#pragma unroll
        for (int q = 0; q < NC; ++q)
          acc[r][q] = fmaf(g.x, y[q].x, fmaf(g.y, y[q].y, fmaf(g.z, y[q].z, fmaf(g.w, y[q].w, acc[r][q]))));
      }
    }
    __syncthreads();   // this stage is refilled NS-1 chunks later
  }
  cp_async_wait<0>();
  __syncthreads();
  // partials [warp][row][col] in the (now idle) ring, then a fixed-order sum
  float *red = ring;
#pragma unroll
  for (int r = 0; r < RT; ++r)
#pragma unroll
    for (int q = 0; q < NC; ++q) red[(warp * RT + r) * SMAX + lane + 32 * q] = acc[r][q];
  __syncthreads();
  for (int e = t; e < RBMAX * SMAX; e += 256) {
    const int i = e / SMAX, j = e % SMAX;
    float v = 0.f;
    if (i < rows && j < s) {
#pragma unroll
      for (int w = 0; w < 8; ++w) v += red[(w * RT + i) * SMAX + j];
    }
    Zs[e] = v;
  }
  __syncthreads();
}

template <int NS>
HT_DEV void coop_product(const float *G, const float *Y, int n, int s, int r0, int rows, float *ring, float *Zs) {
  if (s <= 32) {
    if (rows <= 8) coop_product_t<8, 1, NS>(G, Y, n, s, r0, rows, ring, Zs);
    else if (rows <= 16) coop_product_t<16, 1, NS>(G, Y, n, s, r0, rows, ring, Zs);
    else if (rows <= 24) coop_product_t<24, 1, NS>(G, Y, n, s, r0, rows, ring, Zs);
    else coop_product_t<32, 1, NS>(G, Y, n, s, r0, rows, ring, Zs);
  } else {
    if (rows <= 8) coop_product_t<8, 2, NS>(G, Y, n, s, r0, rows, ring, Zs);
    else if (rows <= 16) coop_product_t<16, 2, NS>(G, Y, n, s, r0, rows, ring, Zs);
    else if (rows <= 24) coop_product_t<24, 2, NS>(G, Y, n, s, r0, rows, ring, Zs);
    else coop_product_t<32, 2, NS>(G, Y, n, s, r0, rows, ring, Zs);
  }
}

// 1 / sqrt(max(x, 1e-24)) in FP64 from an FP32 seed and two Newton steps
// y <- y (3 - x y^2) / 2 (each squares the relative error): a few FP64
// multiplies instead of the FP64 square-root and division sequences, which
// are long on GB300's narrow FP64 pipe.
HT_DEV double frsqrt_fp64(double x) {
  x = fmax(x, 1e-24);
  double y = static_cast<double>(rsqrtf(static_cast<float>(x)));
  y = y * fma(-0.5 * x, y * y, 1.5);
  y = y * fma(-0.5 * x, y * y, 1.5);
  return y;
}

// Pairs of floats (hi + lo, |lo| <= ulp(hi)/2) as a ~48-bit format: sums by
// Knuth's two-sum, products by the FMA two-product (Dekker's double-float
// arithmetic).  The rounded intrinsics keep the compiler from contracting or
// reordering the error terms.
struct DF {
  float h, l;
};
HT_DEV DF df_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b), bb = __fsub_rn(s, a);
  return DF{s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
HT_DEV DF df_quick(float a, float b) {
  const float s = __fadd_rn(a, b);
  return DF{s, __fsub_rn(b, __fsub_rn(s, a))};
}
HT_DEV DF df_add(DF x, DF y) {
  DF s = df_two_sum(x.h, y.h);
  const DF t = df_two_sum(x.l, y.l);
  s = df_quick(s.h, __fadd_rn(s.l, t.h));
  return df_quick(s.h, __fadd_rn(s.l, t.l));
}
HT_DEV DF df_mul(DF x, DF y) {
  const float p = __fmul_rn(x.h, y.h);
  float e = __fmaf_rn(x.h, y.h, -p);
  e = __fmaf_rn(x.h, y.l, __fmaf_rn(x.l, y.h, e));
  return df_quick(p, e);
}
HT_DEV DF df_of(double v) {
  const float h = static_cast<float>(v);
  return DF{h, static_cast<float>(v - static_cast<double>(h))};
}
// 1 / sqrt(x) from the FP32 estimate and one Newton step y + y (1 - x y^2) / 2
// in pair arithmetic (the step squares the estimate's ~2^-23 relative error).
HT_DEV DF df_rsqrt(DF x) {
  const float y0 = rsqrtf(x.h);
  const DF y = DF{y0, 0.f};
  const DF r = df_mul(x, df_mul(y, y));
  const DF e = df_add(DF{1.f, 0.f}, DF{-r.h, -r.l});
  return df_add(y, df_mul(y, DF{__fmul_rn(0.5f, e.h), __fmul_rn(0.5f, e.l)}));
}

// Scaled, shifted Cholesky of the packed s x s matrix Sd followed by the
// explicit transform T = diag(dsc) R^-1 (row-major, stride SMAX, upper
// triangular, FP32) in Ts, so that applying it is a small matrix product.
//
// On numerically rank-deficient blocks the scaled Gram has pivots far below
// FP32 resolution, and an FP32 factor (or a large shift) would discard the weak
// directions every iteration.  The elimination therefore runs in float-pair
// arithmetic (~48 bits) on the unit-diagonal scaled matrix: A's storage (SMAX x
// SMAX doubles) holds the high and the low floats.  GB300 issues FP64 at a
// small fraction of the FP32 rate and with long latency (measured with clock64
// on the FP64 version of this loop: ~1000 cycles a step for the pivot alone,
// ~1900 a step in all); pair arithmetic runs on the FP32 pipe.  Shifts are
// tiny (1e-12; 1e-14 in a second refinement pass) and pivots are floored at
// 1e-24, so T stays finite.  Every trailing update is spread over all 256
// threads (packed triangle, consecutive threads on consecutive words of a
// row), and the triangular inverse runs in FP32 from the factor: T only has to
// keep the block well conditioned; the span is that of Y for any invertible T.
HT_DEV void factor_transform(const double *Sd, int s, double shift, double *A, double *d, float *R32, float *Ts) {
  const int t = threadIdx.x;
  float *Ah = reinterpret_cast<float *>(A), *Al = Ah + SMAX * SMAX;   // the pair's high and low floats
  for (int j = t; j < s; j += 256) {
    const double v = Sd[j * (j + 1) / 2 + j];
    d[j] = v > 1e-300 ? (v >= 1e-24 ? frsqrt_fp64(v) : 1.0 / sqrt(v)) : 0.0;
  }
  __syncthreads();
  const int E = s * (s + 1) / 2;
  for (int e = t; e < E; e += 256) {
    int i, j;
    tri_index(e, i, j);
    double v = Sd[e] * d[i] * d[j];
    if (i == j) v = (d[j] > 0.0 ? 1.0 : 0.0) + shift;
    const DF p = df_of(v);
    Ah[i * SMAX + j] = p.h;
    Al[i * SMAX + j] = p.l;
  }
  __syncthreads();
  // Row 0 of R: warp 0 forms the pivot (every lane) and scales the row.
  if (t < 32) {
    DF piv = DF{Ah[0], Al[0]};
    if (!(piv.h >= 1e-24f)) piv = DF{1e-24f, 0.f};
    const DF ri = df_rsqrt(piv);
    for (int k = 1 + t; k < s; k += 32) {
      const DF r = df_mul(DF{Ah[k], Al[k]}, ri);
      Ah[k] = r.h;
      Al[k] = r.l;
    }
    if (t == 0) {
      const DF r = df_mul(piv, ri);
      Ah[0] = r.h;
      Al[0] = r.l;
    }
  }
  __syncthreads();
  // Step j (row j of R final): warp 0 applies row j to row j + 1, forms its
  // pivot from registers and scales it -- the next step's row -- while warps
  // 1-7 apply row j to rows j + 2 .. s - 1.  One barrier a step, and the
  // pivot's dependent chain overlaps the bulk of the update.  Every entry sees
  // the same operations in the same order as a plain right-looking sweep.
  for (int j = 0; j + 1 < s; ++j) {
    const int j1 = j + 1;
    if (t < 32) {
      const DF rj = DF{Ah[j * SMAX + j1], Al[j * SMAX + j1]};
      DF v[2] = {DF{0.f, 0.f}, DF{0.f, 0.f}};
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        const int k = j1 + t + 32 * q;
        if (k < s) {
          const DF p = df_mul(rj, DF{Ah[j * SMAX + k], Al[j * SMAX + k]});
          v[q] = df_add(DF{Ah[j1 * SMAX + k], Al[j1 * SMAX + k]}, DF{-p.h, -p.l});
        }
      }
      DF piv = DF{__shfl_sync(0xffffffffu, v[0].h, 0), __shfl_sync(0xffffffffu, v[0].l, 0)};
      if (!(piv.h >= 1e-24f)) piv = DF{1e-24f, 0.f};
      const DF ri = df_rsqrt(piv);
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        const int k = j1 + t + 32 * q;
        if (k < s) {
          const DF r = df_mul(k == j1 ? piv : v[q], ri);
          Ah[j1 * SMAX + k] = r.h;
          Al[j1 * SMAX + k] = r.l;
        }
      }
    } else {
      const int L = s - 2 - j;   // A[i][k] -= R[j][i] R[j][k], j + 1 < i <= k
      for (int e = t - 32; e < L * (L + 1) / 2; e += 224) {
        // tri_index varies its first index fastest; mapping it to the column
        // k (reversed) makes consecutive threads touch consecutive words of a row
        int a, b;
        tri_index(e, a, b);
        const int i = s - 1 - b, k = s - 1 - a;
        const DF p = df_mul(DF{Ah[j * SMAX + i], Al[j * SMAX + i]}, DF{Ah[j * SMAX + k], Al[j * SMAX + k]});
        const DF r = df_add(DF{Ah[i * SMAX + k], Al[i * SMAX + k]}, DF{-p.h, -p.l});
        Ah[i * SMAX + k] = r.h;
        Al[i * SMAX + k] = r.l;
      }
    }
    __syncthreads();
  }
  for (int e = t; e < E; e += 256) {
    int i, k;
    tri_index(e, i, k);
    R32[i * SMAX + k] = __fadd_rn(Ah[i * SMAX + k], Al[i * SMAX + k]);
  }
  __syncthreads();
  // W = R^-1 in 32 x 32 blocks, R = [R11 R12; 0 R22]:
  //   W11 = R11^-1, W22 = R22^-1  (warp 0 / warp 1: lane = column, back substitution
  //                                 with the column in registers, R rows broadcast)
  //   W12 = -W11 (R12 W22)        (two 32 x 32 products over all threads)
  // then T = diag(dsc) W.  W lives in A's storage (free once R is formed).
  {
    __shared__ float rinv[SMAX];
    constexpr int WS = SMAX + 1;
    float *W = Ah;
    const int n1 = s < 32 ? s : 32, n2 = s - n1;
    for (int i = t; i < s; i += 256) rinv[i] = 1.f / R32[i * SMAX + i];
    for (int e = t; e < SMAX * WS; e += 256) W[e] = 0.f;
    __syncthreads();
    if (t < 64) {
      const int w = t >> 5, lane = t & 31, base = 32 * w, nb = w == 0 ? n1 : n2;
      if (lane < nb) {
        float wv[32];
#pragma unroll
        for (int ii = 31; ii >= 0; --ii) {
          float acc = ii == lane ? 1.f : 0.f;
#pragma unroll
          for (int jj = ii + 1; jj < 32; ++jj)
            if (jj <= lane) acc = fmaf(-R32[(base + ii) * SMAX + base + jj], wv[jj], acc);
          wv[ii] = (ii <= lane) ? acc * rinv[base + (ii < nb ? ii : 0)] : 0.f;
        }
#pragma unroll
        for (int ii = 0; ii < 32; ++ii)
          if (ii <= lane) W[(base + ii) * WS + base + lane] = wv[ii];
      }
    }
    __syncthreads();
    if (n2 > 0) {
      // P = R12 W22 (n1 x n2) into the strictly lower part's rows (W[32 + i][*] is free below the diagonal)
      float *Pm = Ts;   // Ts is written last: use it as scratch (n1 rows, stride SMAX)
      for (int e = t; e < n1 * n2; e += 256) {
        const int i = e / n2, k = e % n2;
        float acc = 0.f;
        for (int j = 0; j <= k; ++j) acc = fmaf(R32[i * SMAX + 32 + j], W[(32 + j) * WS + 32 + k], acc);
        Pm[i * SMAX + k] = acc;
      }
      __syncthreads();
      for (int e = t; e < n1 * n2; e += 256) {
        const int i = e / n2, k = e % n2;
        float acc = 0.f;
        for (int j = i; j < n1; ++j) acc = fmaf(W[i * WS + j], Pm[j * SMAX + k], acc);
        W[i * WS + 32 + k] = -acc;
      }
      __syncthreads();
    }
    for (int e = t; e < SMAX * SMAX; e += 256) {
      const int i = e / SMAX, k = e % SMAX;
      Ts[e] = (i < s && k < s && k >= i) ? W[i * WS + k] * static_cast<float>(d[i]) : 0.f;
    }
    __syncthreads();
  }
}

// X (RBMAX x SMAX rows) <- X T for the upper-triangular T (s x s): thread
// (row t / 8, columns t % 8 + 8 b) forms its eight outputs, then writes back.
HT_DEV void coop_apply(float *X, const float *Ts, int s) {
  const int t = threadIdx.x, r = t >> 3, cb = t & 7;
  float o[8];
#pragma unroll
  for (int b = 0; b < 8; ++b) o[b] = 0.f;
  for (int j = 0; j < s; ++j) {
    const float x = X[r * SMAX + j];
#pragma unroll
    for (int b = 0; b < 8; ++b) o[b] = fmaf(x, Ts[j * SMAX + cb + 8 * b], o[b]);
  }
  __syncthreads();
#pragma unroll
  for (int b = 0; b < 8; ++b) X[r * SMAX + cb + 8 * b] = (cb + 8 * b < s) ? o[b] : 0.f;
  __syncthreads();
}

// Rows [r0, r0 + rows) of an n x s block into X[i * SMAX + j] (zero padded).
HT_DEV void coop_load_rows(const float *src, int n, int s, int r0, int rows, float *X) {
  for (int e = threadIdx.x; e < RBMAX * SMAX; e += 256) {
    const int i = e % RBMAX, j = e / RBMAX;
    X[i * SMAX + j] = (i < rows && j < s) ? __ldcg(src + (r0 + i) + static_cast<long long>(n) * j) : 0.f;
  }
}

HT_DEV void coop_store_rows(const float *X, int n, int s, int r0, int rows, float *dst) {
  for (int e = threadIdx.x; e < RBMAX * SMAX; e += 256) {
    const int i = e % RBMAX, j = e / RBMAX;
    if (i < rows && j < s) dst[(r0 + i) + static_cast<long long>(n) * j] = X[i * SMAX + j];
  }
}

// acc[q] += partial of entry e = t + 256 q (packed upper triangle, i <= j) of L^T R.
HT_DEV void coop_gram_partial(const float *L, const float *R, int s, Acc2 (&acc)[kMaxEntPerThread]) {
  const int E = s * (s + 1) / 2;
#pragma unroll
  for (int q = 0; q < kMaxEntPerThread; ++q) {
    const int e = threadIdx.x + 256 * q;
    if (e < E) {
      int i, j;
      tri_index(e, i, j);
#pragma unroll 8
      for (int r = 0; r < RBMAX; ++r) acc2_add_prod(acc[q], L[r * SMAX + i], R[r * SMAX + j]);
    }
  }
}

HT_DEV void coop_gram_store(const Acc2 (&acc)[kMaxEntPerThread], int s, float *part) {
  const int E = s * (s + 1) / 2;
#pragma unroll
  for (int q = 0; q < kMaxEntPerThread; ++q) {
    const int e = threadIdx.x + 256 * q;
    if (e < E) {
      part[2 * e] = acc[q].s;
      part[2 * e + 1] = acc[q].c;
    }
  }
}

// Every synchronising CTA sums a slice of all problems' entries over the
// problem's CTA partials, in CTA order.
HT_DEV void coop_reduce(const CoopBatch &B) {
  for (int g = blockIdx.x * 256 + threadIdx.x; g < B.ent_total; g += B.nsync * 256) {
    int p = 0;
    while (g >= B.ent_off[p + 1]) ++p;
    const CoopProb &P = B.p[p];
    const int e = g - B.ent_off[p];
    Acc2 acc = {0.f, 0.f};
    for (int c0 = 0; c0 < P.ncta; c0 += GROUP) {
      float hi[GROUP], lo[GROUP];
#pragma unroll
      for (int q = 0; q < GROUP; ++q) {
        const bool ok = c0 + q < P.ncta;
        const float *src = P.part + (static_cast<long long>(c0 + q) * ESMAX + e) * 2;
        hi[q] = ok ? __ldcg(src) : 0.f;
        lo[q] = ok ? __ldcg(src + 1) : 0.f;
      }
#pragma unroll
      for (int q = 0; q < GROUP; ++q) acc2_add(acc, hi[q], lo[q]);
    }
    P.S[e] = static_cast<double>(acc.s) + static_cast<double>(acc.c);
  }
}

HT_DEV void coop_load_S(const CoopProb &P, double *Sd) {
  const int E = P.s * (P.s + 1) / 2;
  for (int e = threadIdx.x; e < E; e += 256) Sd[e] = __ldcg(P.S + e);
  __syncthreads();
}

// One CholeskyQR-type step over the CTA's rows: X = src rows (optionally
// G * src + mu src), apply the current transform Rs (unless identity), store to dst,
// accumulate the Gram partial.  mode 0: ITER, 1: APPLY, 2: RR (also Q rows).
template <int NS>
HT_DEV void coop_step(const CoopProb &P, int cl, int mode, const float *src, float *dst, float *dst2, bool ident,
                      float mu, const float *Rs, float *Zs, float *Qr, float *ring, bool want_s = true) {
  Acc2 acc[kMaxEntPerThread];
#pragma unroll
  for (int q = 0; q < kMaxEntPerThread; ++q) acc[q] = Acc2{0.f, 0.f};
  const int rb = cl * P.rows, re = min(P.n, rb + P.rows);
  for (int r0 = rb; r0 < re; r0 += RBMAX) {
    const int rows = min(RBMAX, re - r0);
    coop_load_rows(src, P.n, P.s, r0, rows, Qr);
    if (mode != 1) {
      coop_product<NS>(P.G, src, P.n, P.s, r0, rows, ring, Zs);
      if (mode == 0)
        for (int e = threadIdx.x; e < RBMAX * SMAX; e += 256) Zs[e] = fmaf(mu, Qr[e], Zs[e]);
    } else {
      __syncthreads();
      for (int e = threadIdx.x; e < RBMAX * SMAX; e += 256) Zs[e] = Qr[e];
    }
    __syncthreads();
    if (!ident) {
      coop_apply(Zs, Rs, P.s);
      if (mode == 2) coop_apply(Qr, Rs, P.s);
    }
    if (mode == 2) {
      coop_store_rows(Qr, P.n, P.s, r0, rows, dst);
      coop_store_rows(Zs, P.n, P.s, r0, rows, dst2);
      coop_gram_partial(Qr, Zs, P.s, acc);
    } else {
      coop_store_rows(Zs, P.n, P.s, r0, rows, dst);
      if (want_s) coop_gram_partial(Zs, Zs, P.s, acc);
    }
    __syncthreads();
  }
  if (want_s) coop_gram_store(acc, P.s, P.part + static_cast<long long>(cl) * ESMAX * 2);
}

// U = Q V[:, :K], GU = Y V[:, :K] on the CTA's rows, column sums of squares of
// GU - theta U into colss[cl].
HT_DEV void coop_final_rows(const CoopProb &P, int cl, const float *Q, const float *Y, float (*Vsm)[SMAX + 1],
                            const float *th, float *Qr, float *Zs) {
  const int t = threadIdx.x, n = P.n, s = P.s, K = P.K;
  __shared__ float colsum[SMAX];
  if (t < SMAX) colsum[t] = 0.f;
  const int rb = cl * P.rows, re = min(n, rb + P.rows);
  for (int r0 = rb; r0 < re; r0 += RBMAX) {
    const int rows = min(RBMAX, re - r0);
    coop_load_rows(Q, n, s, r0, rows, Qr);
    coop_load_rows(Y, n, s, r0, rows, Zs);
    __syncthreads();
    // thread: row i = t / 8 (32 rows), columns j = t % 8 + 8 c
    const int i = t >> 3, jb = t & 7;
    float dsq[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      const int j = jb + 8 * c;
      float u = 0.f, gu = 0.f;
      if (j < K && i < rows) {
        for (int k = 0; k < s; ++k) {
          u = fmaf(Qr[i * SMAX + k], Vsm[k][j], u);
          gu = fmaf(Zs[i * SMAX + k], Vsm[k][j], gu);
        }
        P.U[(r0 + i) + static_cast<long long>(n) * j] = u;
        P.GU[(r0 + i) + static_cast<long long>(n) * j] = gu;
      }
      const float d = (j < K && i < rows) ? gu - th[j] * u : 0.f;
      dsq[c] = d * d;
    }
    __syncthreads();
    // column sums over the 32 rows: reuse Qr as scratch [row][col]
#pragma unroll
    for (int c = 0; c < 8; ++c) Qr[i * SMAX + jb + 8 * c] = dsq[c];
    __syncthreads();
    if (t < SMAX) {
      float a = 0.f;
      for (int r = 0; r < RBMAX; ++r) a += Qr[r * SMAX + t];
      colsum[t] += a;
    }
    __syncthreads();
  }
  if (t < SMAX) P.colss[static_cast<long long>(cl) * SMAX + t] = colsum[t];
}

// Shared memory of the eigen-solver kernels: the dynamic block (kCoopSmem)
// carved as the cooperative kernel always has, plus small static arrays.
struct EigSmem {
  float *Rs;                    // SMAX*SMAX (upper factor, row-major)
  float *Zs, *Qr;               // RBMAX*SMAX each
  float *ring;                  // product ring, or (aliased) the reducer / Jacobi scratch
  double *Sd;
  float (*A)[SMAX + 1], (*VV)[SMAX + 1], (*A2)[SMAX + 1];
  int *s_ok, *order;
  float *red, *th_sm;
  double *piv64;
};

HT_DEV EigSmem eig_smem(float *sm) {
  __shared__ int s_ok;
  __shared__ int order[SMAX];
  __shared__ float red[256];
  __shared__ float th_sm[SMAX];
  __shared__ double piv64[SMAX];
  EigSmem m;
  m.Rs = sm;
  m.Zs = m.Rs + SMAX * SMAX + SMAX;   // SMAX floats after the factor are reserved
  m.Qr = m.Zs + RBMAX * SMAX;
  m.ring = m.Qr + RBMAX * SMAX;
  m.Sd = reinterpret_cast<double *>(m.ring);
  m.A = reinterpret_cast<float (*)[SMAX + 1]>(m.ring + 2 * ESMAX);
  m.VV = reinterpret_cast<float (*)[SMAX + 1]>(m.ring + 2 * ESMAX + SMAX * (SMAX + 1));
  m.A2 = reinterpret_cast<float (*)[SMAX + 1]>(m.ring + 2 * ESMAX + 2 * SMAX * (SMAX + 1));
  m.s_ok = &s_ok;
  m.order = order;
  m.red = red;
  m.th_sm = th_sm;
  m.piv64 = piv64;
  return m;
}

// Direct problem (s == n): Jacobi eigen-decomposition of G itself.
HT_DEV void eig_direct(const CoopProb &P, const EigSmem &m) {
  const int t = threadIdx.x, n = P.n, K = P.K;
  float (*A)[SMAX + 1] = m.A;
  float (*VV)[SMAX + 1] = m.VV;
  const int *order = m.order;
  for (int e = t; e < SMAX * SMAX; e += 256) {
    const int i = e % SMAX, j = e / SMAX;
    A[i][j] = (i < n && j < n) ? P.G[i + static_cast<long long>(n) * j] : 0.f;
  }
  __syncthreads();
  jacobi_smem(A, m.A2, VV, n, m.order);
  for (int r = t; r < K; r += 256) P.theta[r] = A[order[r]][order[r]];
  // U = V[:, order[:K]], GU = G U, residual
  for (int e = t; e < n * K; e += 256) {
    const int i = e % n, j = e / n;
    float gu = 0.f;
    for (int k = 0; k < n; ++k) gu = fmaf(P.G[i + static_cast<long long>(n) * k], VV[k][order[j]], gu);
    const float u = VV[i][order[j]];
    P.U[i + static_cast<long long>(n) * j] = u;
    P.GU[i + static_cast<long long>(n) * j] = gu;
    const float d = gu - A[order[j]][order[j]] * u;
    m.Zs[e] = d * d;   // n * K <= 64 * 64 fits Zs + Qr (contiguous)
  }
  __syncthreads();
  if (t == 0) {
    float mx = 0.f;
    for (int j = 0; j < K; ++j) {
      float a = 0.f;
      for (int i = 0; i < n; ++i) a += m.Zs[i + n * j];
      mx = fmaxf(mx, sqrtf(a));
    }
    const float th = A[order[0]][order[0]];
    P.resid[0] = th > 0.f ? mx / th : mx;
  }
}

// Synchronisation of the phases of one problem.  Cooperative: the problem's
// rows are spread over several CTAs of a cooperative grid -- bounded grid
// barriers, and the Gram partials reduced by all CTAs of the grid.  Local:
// the problem is one CTA's (the grouped solver) -- block barriers, and the
// CTA reduces its own partials.
struct CoopSync {
  const CoopBatch *B;
  unsigned members;
  int *s_ok;
  HT_DEV bool bar() const { return grid_barrier(B->bar, members, B->err, s_ok); }
  HT_DEV void reduce() const { coop_reduce(*B); }
};

HT_DEV void coop_reduce_one(const CoopProb &P) {
  const int E = P.s * (P.s + 1) / 2;
  for (int e = threadIdx.x; e < E; e += 256) {
    Acc2 acc = {0.f, 0.f};
    for (int c = 0; c < P.ncta; ++c) {
      const float *src = P.part + (static_cast<long long>(c) * ESMAX + e) * 2;
      acc2_add(acc, __ldcg(src), __ldcg(src + 1));
    }
    P.S[e] = static_cast<double>(acc.s) + static_cast<double>(acc.c);
  }
}

struct LocalSync {
  const CoopProb *P;
  HT_DEV bool bar() const {
    __syncthreads();
    return true;
  }
  HT_DEV void reduce() const { coop_reduce_one(*P); }
};

// Subspace iteration, Rayleigh-Ritz and the final U / GU / residual of one
// problem; CTA `cl` of the problem's P.ncta owns rows [cl * P.rows, ...).
template <class Sync, int NS>
HT_DEV void eig_iterate(const CoopProb &P, int cl, const Sync &sy, int iters, int refine, const EigSmem &m) {
  const int t = threadIdx.x;
  float *Rs = m.Rs, *Zs = m.Zs, *Qr = m.Qr, *ring = m.ring, *red = m.red;
  double *Sd = m.Sd;
  // mu = 1e-9 trace(G), computed identically by every CTA of the problem
  {
    float tr = 0.f;
    for (int i = t; i < P.n; i += 256) tr += __ldg(P.G + i + static_cast<long long>(P.n) * i);
    red[t] = tr;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
      if (t < w) red[t] += red[t + w];
      __syncthreads();
    }
  }
  const float mu = 1e-9f * fmaxf(red[0], 0.f);
  // start block rows
  {
    const int rb = cl * P.rows, re = min(P.n, rb + P.rows);
    for (int e = t; e < (re - rb) * P.s; e += 256) {
      const int i = rb + e % (re - rb), j = e / (re - rb);
      const long long idx = i + static_cast<long long>(P.n) * j;
      P.buf[0][idx] = P.start ? P.start[idx] : gaussian(P.seed, P.stream_id, static_cast<unsigned long long>(idx));
    }
  }
  if (!sy.bar()) return;

  auto reduce_and_factor = [&](double shift) -> bool {
    if (!sy.bar()) return false;
    sy.reduce();
    if (!sy.bar()) return false;
    coop_load_S(P, Sd);
    double *A64 = Sd + ESMAX;                  // SMAX*SMAX doubles after the reduced Gram
    factor_transform(Sd, P.s, shift, A64, m.piv64, reinterpret_cast<float *>(A64 + SMAX * SMAX), Rs);
    return true;
  };

  int cur = 0;
  bool ident = true;
  for (int it = 0; it < iters; ++it) {
    coop_step<NS>(P, cl, 0, P.buf[cur], P.buf[cur ^ 1], nullptr, ident, mu, Rs, Zs, Qr, ring);
    if (!reduce_and_factor(1e-12)) return;
    ident = false;
    cur ^= 1;
  }
  // Q_L = Y_L T_L -> buffer 2.  The float-pair factor leaves Q_L orthonormal
  // to ~1e-7 (scaled off-diagonal of Q_L^T Q_L, 1e-6 on clustered spectra), so
  // Rayleigh-Ritz takes it as it is: no further CholeskyQR pass.  G Q is formed
  // from Q_L itself, not as (G Y_L) T_L, whose sum over the ill-scaled columns of
  // Y_L loses digits to cancellation.
  // The FP32 path asks for `refine` CholeskyQR passes on Q_L all the same
  // (orthonormal to FP32 rounding, the last digit of its error).
  coop_step<NS>(P, cl, 1, P.buf[cur], P.buf[2], nullptr, ident, 0.f, Rs, Zs, Qr, ring, ident || refine > 0);
  bool rr_ident = true;
  if (ident || refine > 0) {   // ident: no iteration ran, orthonormalise the start block
    if (!reduce_and_factor(1e-12)) return;
    rr_ident = false;
    for (int r = 1; r < refine; ++r) {   // row-local, so in place
      coop_step<NS>(P, cl, 1, P.buf[2], P.buf[2], nullptr, false, 0.f, Rs, Zs, Qr, ring);
      if (!reduce_and_factor(1e-14)) return;
    }
  } else if (!sy.bar()) {
    return;
  }
  // Rayleigh-Ritz: Q -> buf3, G Q -> buf0, H = Q^T G Q
  coop_step<NS>(P, cl, 2, P.buf[2], P.buf[3], P.buf[0], rr_ident, 0.f, Rs, Zs, Qr, ring);
  if (!sy.bar()) return;
  sy.reduce();
  if (!sy.bar()) return;
  if (cl == 0) {
    coop_load_S(P, Sd);
    const int s = P.s;
    for (int e = t; e < SMAX * SMAX; e += 256) {
      const int i = e % SMAX, j = e / SMAX;
      float v = 0.f;
      if (i < s && j < s) v = static_cast<float>(i <= j ? Sd[j * (j + 1) / 2 + i] : Sd[i * (i + 1) / 2 + j]);
      m.A[i][j] = v;
    }
    __syncthreads();
    jacobi_smem(m.A, m.A2, m.VV, s, m.order);
    for (int e = t; e < s * s; e += 256) {
      const int i = e % s, r = e / s;
      P.V[i + s * r] = m.VV[i][m.order[r]];
    }
    for (int r = t; r < P.K; r += 256) P.theta[r] = m.A[m.order[r]][m.order[r]];
  }
  if (!sy.bar()) return;
  // final: U, GU and the residual partials
  {
    float (*Vsm)[SMAX + 1] = m.VV;
    const int s = P.s;
    for (int e = t; e < SMAX * SMAX; e += 256) {
      const int i = e % SMAX, j = e / SMAX;
      Vsm[i][j] = (i < s && j < s) ? __ldcg(P.V + i + s * j) : 0.f;
    }
    for (int j = t; j < SMAX; j += 256) m.th_sm[j] = j < P.K ? __ldcg(P.theta + j) : 0.f;
    __syncthreads();
    coop_final_rows(P, cl, P.buf[3], P.buf[0], Vsm, m.th_sm, Qr, Zs);
  }
  if (!sy.bar()) return;
  if (cl == 0 && t < SMAX) {
    float a = 0.f;
    if (t < P.K)
      for (int c = 0; c < P.ncta; ++c) a += __ldcg(P.colss + static_cast<long long>(c) * SMAX + t);
    red[t] = sqrtf(a);
  }
  __syncthreads();
  if (cl == 0 && t == 0) {
    float mx = 0.f;
    for (int j = 0; j < P.K; ++j) mx = fmaxf(mx, red[j]);
    const float th = __ldcg(P.theta);
    P.resid[0] = th > 0.f ? mx / th : mx;
  }
}

__global__ void __launch_bounds__(256, 1) eig_coop_kernel(const __grid_constant__ CoopBatch B) {
  extern __shared__ __align__(16) float sm[];
  const EigSmem m = eig_smem(sm);

  if (static_cast<int>(blockIdx.x) >= B.nsync) {
    // ---- direct problem (s == n): Jacobi on G itself, no barriers
    eig_direct(B.p[B.direct_idx[blockIdx.x - B.nsync]], m);
    return;
  }

  int pi = 0;
  while (!(static_cast<int>(blockIdx.x) >= B.p[pi].cta0 && static_cast<int>(blockIdx.x) < B.p[pi].cta0 + B.p[pi].ncta)) ++pi;
  const CoopProb &P = B.p[pi];
  const int cl = blockIdx.x - P.cta0;
  const unsigned members = static_cast<unsigned>(B.nsync);

  if (B.orth_passes > 0) {
    // In-place CholeskyQR of buffer 0 (problems without a Gram): each pass
    // applies the previous transform to the CTA's rows and accumulates their
    // Gram partial, all CTAs reduce, every CTA factors (float pairs, pivots
    // floored, so it cannot break down; the first pass shifted by 1e-12 of the
    // unit diagonal, as the eigen-solver's iterations).  The Gram and the
    // factor carry ~48 bits, so after one pass only the FP32 rounding of the
    // applied transform remains (~u * cond(Y)); a second pass removes it.
    float *Q = P.buf[0];
    double *A64 = m.Sd + ESMAX;
    for (int pass = 0; pass <= B.orth_passes; ++pass) {
      // row-local: in place; the last pass only applies the transform
      coop_step<CNS>(P, cl, 1, Q, Q, nullptr, pass == 0, 0.f, m.Rs, m.Zs, m.Qr, m.ring, pass < B.orth_passes);
      if (pass == B.orth_passes) break;
      if (!grid_barrier(B.bar, members, B.err, m.s_ok)) return;
      coop_reduce(B);
      if (!grid_barrier(B.bar, members, B.err, m.s_ok)) return;
      coop_load_S(P, m.Sd);
      factor_transform(m.Sd, P.s, pass == 0 ? 1e-12 : 0.0, A64, m.piv64, reinterpret_cast<float *>(A64 + SMAX * SMAX),
                       m.Rs);
    }
    return;
  }
  const CoopSync sy{&B, members, m.s_ok};
  eig_iterate<CoopSync, CNS>(P, cl, sy, B.iters, B.refine, m);
}

// Grouped solver of the batched path: CTA b solves problem tab[b] alone (all
// of its rows, block barriers only), so one ordinary launch covers every leaf
// of every tensor of a batch and no CTA waits on another.
__global__ void __launch_bounds__(256, 2) eig_grouped_kernel(const CoopProb *__restrict__ tab, int iters, int refine) {
  extern __shared__ __align__(16) float sm[];
  const EigSmem m = eig_smem(sm);
  __shared__ CoopProb sP;
  if (threadIdx.x == 0) sP = tab[blockIdx.x];
  __syncthreads();
  const CoopProb &P = sP;
  if (P.s == P.n) {
    eig_direct(P, m);
    return;
  }
  const LocalSync sy{&P};
  eig_iterate<LocalSync, kGroupedStages>(P, 0, sy, iters, refine, m);
}

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

constexpr size_t kJacScratch = sizeof(float) * SMAX * (SMAX + 1);   // dynamic smem of the one-CTA Jacobi kernels

}  // namespace

namespace {
size_t coop_workspace_bytes(const EigProblem *probs, int nprob) {
  size_t b = align256(4 * sizeof(unsigned));
  for (int i = 0; i < nprob; ++i) {
    b += 4 * align256(sizeof(float) * static_cast<size_t>(probs[i].n) * SMAX);
    b += align256(sizeof(float) * kCoopMaxCta * ESMAX * 2);
    b += align256(sizeof(double) * ESMAX);
    b += align256(sizeof(float) * SMAX * SMAX);
    b += align256(sizeof(float) * kCoopMaxCta * SMAX);
  }
  return b;
}
}  // namespace

size_t eig_workspace_bytes(const EigProblem *probs, int nprob) { return coop_workspace_bytes(probs, nprob); }

// Resources of the cooperative solver on the current device (cached).
static int coop_max_ctas() {
  static int cached[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 0;
  if (cached[dev]) return cached[dev];
  int sms = 0, occ = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
  if (cudaFuncSetAttribute(eig_coop_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           static_cast<int>(kCoopSmem)) != cudaSuccess)
    return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, eig_coop_kernel, 256, kCoopSmem) != cudaSuccess) return 0;
  const int m = sms * occ;
  cached[dev] = m < kCoopMaxCta ? m : kCoopMaxCta;
  return cached[dev];
}

cudaError_t eig_prepare() {
  if (coop_max_ctas() <= 0) return cudaErrorInvalidConfiguration;
  cudaError_t e = cudaFuncSetAttribute(transfer_eig_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           static_cast<int>(kJacScratch));
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(eig_grouped_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           static_cast<int>(kGroupedSmem));
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(svd_from_gram_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              static_cast<int>(kJacScratch));
}

cudaError_t eig_batched(EigProblem *probs, int nprob, int iters, void *ws, size_t ws_bytes, int *err, cudaStream_t st,
                        int *launches, int max_ctas, int refine) {
  if (nprob <= 0) return cudaSuccess;
  if (nprob > kMaxProb) return cudaErrorInvalidValue;
  if (coop_workspace_bytes(probs, nprob) > ws_bytes) return cudaErrorInvalidValue;
  int budget = coop_max_ctas();
  if (max_ctas > 0 && max_ctas < budget) budget = max_ctas;
  if (budget <= 0) return cudaErrorInvalidConfiguration;
  CoopBatch B;
  std::memset(&B, 0, sizeof(B));
  char *p = static_cast<char *>(ws);
  B.bar = reinterpret_cast<unsigned *>(p);
  p += align256(4 * sizeof(unsigned));
  B.err = err;
  B.nprob = nprob;
  B.iters = iters;
  B.refine = refine < 0 ? 0 : (refine > 2 ? 2 : refine);
  long long n_iter = 0;
  int n_direct = 0, n_iterating = 0;
  for (int i = 0; i < nprob; ++i) {
    const EigProblem &q = probs[i];
    if (!q.G || q.s > SMAX || q.s < 1 || q.K > q.s || q.s > q.n) return cudaErrorInvalidValue;
    if (q.s == q.n) {
      ++n_direct;
    } else {
      n_iter += q.n;
      ++n_iterating;
    }
  }
  const int budget_it = budget - n_direct;
  if (n_iterating > 0 && budget_it < n_iterating) return cudaErrorInvalidConfiguration;
  int cta = 0, d = 0, ent = 0;
  for (int i = 0; i < nprob; ++i) {
    const EigProblem &q = probs[i];
    CoopProb &c = B.p[i];
    c.G = q.G; c.n = q.n; c.s = q.s; c.K = q.K;
    c.U = q.U; c.GU = q.GU; c.theta = q.theta; c.resid = q.resid;
    c.start = q.start; c.seed = q.seed; c.stream_id = q.stream_id;
    for (int k = 0; k < 4; ++k) {
      c.buf[k] = reinterpret_cast<float *>(p);
      p += align256(sizeof(float) * static_cast<size_t>(q.n) * SMAX);
    }
    c.part = reinterpret_cast<float *>(p); p += align256(sizeof(float) * kCoopMaxCta * ESMAX * 2);
    c.S = reinterpret_cast<double *>(p); p += align256(sizeof(double) * ESMAX);
    c.V = reinterpret_cast<float *>(p); p += align256(sizeof(float) * SMAX * SMAX);
    c.colss = reinterpret_cast<float *>(p); p += align256(sizeof(float) * kCoopMaxCta * SMAX);
    B.ent_off[i] = ent;
    if (q.s == q.n) {
      c.cta0 = -1; c.ncta = 0; c.rows = 0;
      B.direct_idx[d++] = i;
    } else {
      int nc = static_cast<int>(static_cast<long long>(budget_it) * q.n / n_iter);
      nc = nc < 1 ? 1 : nc;
      const int rows = (q.n + nc - 1) / nc;
      c.rows = rows;
      c.ncta = (q.n + rows - 1) / rows;
      c.cta0 = cta;
      cta += c.ncta;
      ent += q.s * (q.s + 1) / 2;
    }
  }
  B.ent_off[nprob] = ent;
  B.ent_total = ent;
  B.nsync = cta;
  const int grid = cta + n_direct;
  if (grid > budget) return cudaErrorInvalidConfiguration;
  cudaError_t e = cudaMemsetAsync(B.bar, 0, 4 * sizeof(unsigned), st);
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg;
  std::memset(&cfg, 0, sizeof(cfg));
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(256);
  cfg.dynamicSmemBytes = kCoopSmem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  e = cudaLaunchKernelEx(&cfg, eig_coop_kernel, B);
  if (e != cudaSuccess) return e;
  if (launches) *launches += 1;
  return cudaSuccess;
}

// ---- grouped solver (batched path): one CTA per problem, so a problem's
// workspace holds one CTA's Gram and residual partials
namespace {
size_t grouped_prob_bytes(const EigProblem &q) {
  return 4 * align256(sizeof(float) * static_cast<size_t>(q.n) * SMAX) + align256(sizeof(float) * ESMAX * 2) +
         align256(sizeof(double) * ESMAX) + align256(sizeof(float) * SMAX * SMAX) + align256(sizeof(float) * SMAX);
}
}  // namespace

size_t eig_grouped_workspace_bytes(const EigProblem *probs, int nprob) {
  size_t b = 0;
  for (int i = 0; i < nprob; ++i) b += grouped_prob_bytes(probs[i]);
  return b;
}

size_t eig_grouped_entry_bytes() { return sizeof(CoopProb); }

cudaError_t eig_grouped_fill(const EigProblem *probs, int nprob, void *ws, size_t ws_bytes,
                             std::vector<unsigned char> &table) {
  if (eig_grouped_workspace_bytes(probs, nprob) > ws_bytes) return cudaErrorInvalidValue;
  char *p = static_cast<char *>(ws);
  for (int i = 0; i < nprob; ++i) {
    const EigProblem &q = probs[i];
    if (!q.G || q.s > SMAX || q.s < 1 || q.K > q.s || q.s > q.n) return cudaErrorInvalidValue;
    CoopProb c;
    std::memset(&c, 0, sizeof(c));
    c.G = q.G; c.n = q.n; c.s = q.s; c.K = q.K;
    c.cta0 = 0; c.ncta = 1; c.rows = q.n;
    c.U = q.U; c.GU = q.GU; c.theta = q.theta; c.resid = q.resid;
    c.start = q.start; c.seed = q.seed; c.stream_id = q.stream_id;
    for (int k = 0; k < 4; ++k) {
      c.buf[k] = reinterpret_cast<float *>(p);
      p += align256(sizeof(float) * static_cast<size_t>(q.n) * SMAX);
    }
    c.part = reinterpret_cast<float *>(p); p += align256(sizeof(float) * ESMAX * 2);
    c.S = reinterpret_cast<double *>(p); p += align256(sizeof(double) * ESMAX);
    c.V = reinterpret_cast<float *>(p); p += align256(sizeof(float) * SMAX * SMAX);
    c.colss = reinterpret_cast<float *>(p); p += align256(sizeof(float) * SMAX);
    const unsigned char *raw = reinterpret_cast<const unsigned char *>(&c);
    table.insert(table.end(), raw, raw + sizeof(c));
  }
  return cudaSuccess;
}

void eig_grouped_order(std::vector<unsigned char> &table) {
  // CTAs start in index order, so the longest problems go first and the short
  // ones fill the last wave: Jacobi sweeps on the whole Gram (s == n, cost
  // ~n^3 per sweep) before iterating problems (~n^2 s per iteration)
  const size_t nb = sizeof(CoopProb), np = table.size() / nb;
  std::vector<CoopProb> v(np);
  std::memcpy(v.data(), table.data(), np * nb);
  auto cost = [](const CoopProb &q) {
    return q.s == q.n ? 4.0 * q.n * q.n * q.n : static_cast<double>(q.n) * q.n * q.s + 64.0 * q.s * q.s * q.s;
  };
  std::stable_sort(v.begin(), v.end(), [&](const CoopProb &a, const CoopProb &b) { return cost(a) > cost(b); });
  std::memcpy(table.data(), v.data(), np * nb);
}

cudaError_t eig_grouped_launch(const void *table_dev, int nprob, int iters, int refine, cudaStream_t st) {
  if (nprob <= 0) return cudaSuccess;
  if (!table_dev || (reinterpret_cast<uintptr_t>(table_dev) % alignof(CoopProb)) != 0) return cudaErrorInvalidValue;
  eig_grouped_kernel<<<nprob, 256, kGroupedSmem, st>>>(static_cast<const CoopProb *>(table_dev), iters,
                                                    refine < 0 ? 0 : (refine > 2 ? 2 : refine));
  return cudaGetLastError();
}

// In-place CholeskyQR (`passes` factorisations, the first shifted) of tall
// blocks: G == nullptr problems, Q = the matrix.  One cooperative launch of the
// eigen-solver's kernel in its CholeskyQR mode.
cudaError_t cholqr_batched(EigProblem *probs, int nprob, int passes, void *ws, size_t ws_bytes, int *err, cudaStream_t st,
                           int *launches) {
  if (nprob <= 0) return cudaSuccess;
  if (nprob > kMaxProb || passes < 1) return cudaErrorInvalidValue;
  if (coop_workspace_bytes(probs, nprob) > ws_bytes) return cudaErrorInvalidValue;
  const int budget = coop_max_ctas();
  if (budget < nprob) return cudaErrorInvalidConfiguration;
  CoopBatch B;
  std::memset(&B, 0, sizeof(B));
  char *p = static_cast<char *>(ws);
  B.bar = reinterpret_cast<unsigned *>(p);
  p += align256(4 * sizeof(unsigned));
  B.err = err;
  B.nprob = nprob;
  B.orth_passes = passes;
  long long n_all = 0;
  for (int i = 0; i < nprob; ++i) {
    const EigProblem &q = probs[i];
    if (q.G || !q.Q || q.s > SMAX || q.s < 1 || q.s > q.n) return cudaErrorInvalidValue;
    n_all += q.n;
  }
  int cta = 0, ent = 0;
  for (int i = 0; i < nprob; ++i) {
    const EigProblem &q = probs[i];
    CoopProb &c = B.p[i];
    c.G = nullptr; c.n = q.n; c.s = q.s; c.K = q.s;
    for (int k = 0; k < 4; ++k) {
      c.buf[k] = reinterpret_cast<float *>(p);
      p += align256(sizeof(float) * static_cast<size_t>(q.n) * SMAX);
    }
    c.buf[0] = q.Q;   // operate on the caller's matrix in place
    c.part = reinterpret_cast<float *>(p); p += align256(sizeof(float) * kCoopMaxCta * ESMAX * 2);
    c.S = reinterpret_cast<double *>(p); p += align256(sizeof(double) * ESMAX);
    c.V = reinterpret_cast<float *>(p); p += align256(sizeof(float) * SMAX * SMAX);
    c.colss = reinterpret_cast<float *>(p); p += align256(sizeof(float) * kCoopMaxCta * SMAX);
    B.ent_off[i] = ent;
    int nc = static_cast<int>(static_cast<long long>(budget) * q.n / n_all);
    nc = nc < 1 ? 1 : nc;
    const int rows = (q.n + nc - 1) / nc;
    c.rows = rows;
    c.ncta = (q.n + rows - 1) / rows;
    c.cta0 = cta;
    cta += c.ncta;
    ent += q.s * (q.s + 1) / 2;
  }
  B.ent_off[nprob] = ent;
  B.ent_total = ent;
  B.nsync = cta;
  if (cta > budget) return cudaErrorInvalidConfiguration;
  cudaError_t e = cudaMemsetAsync(B.bar, 0, 4 * sizeof(unsigned), st);
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg;
  std::memset(&cfg, 0, sizeof(cfg));
  cfg.gridDim = dim3(cta);
  cfg.blockDim = dim3(256);
  cfg.dynamicSmemBytes = kCoopSmem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  e = cudaLaunchKernelEx(&cfg, eig_coop_kernel, B);
  if (e != cudaSuccess) return e;
  if (launches) *launches += 1;
  return cudaSuccess;
}

cudaError_t svd_from_gram_batched_launch(const SvdGramProb *probs, int nprob, cudaStream_t st) {
  if (nprob < 1 || nprob > 4) return cudaErrorInvalidValue;
  SvdGramBatch b;
  std::memset(&b, 0, sizeof(b));
  for (int i = 0; i < nprob; ++i) {
    const SvdGramProb &q = probs[i];
    if (q.s > SMAX || q.s < 1 || q.k1 > q.s || q.k2 > q.s) return cudaErrorInvalidValue;
    b.p[i] = q;
  }
  static bool attr_set[64] = {};
  const cudaError_t e = opt_in_smem(svd_from_gram_kernel, static_cast<int>(kJacScratch), attr_set);
  if (e != cudaSuccess) return e;
  svd_from_gram_kernel<<<nprob, 256, kJacScratch, st>>>(b);
  return cudaGetLastError();
}

cudaError_t svd_from_gram_launch(const float *GW, int s, int k1, int k2, float *M1, float *M2, float *Broot,
                                 cudaStream_t st) {
  SvdGramProb q{GW, s, k1, k2, M1, M2, Broot};
  return svd_from_gram_batched_launch(&q, 1, st);
}

cudaError_t transfer_tail_grouped_launch(const TailJob *jobs_dev, int njobs, cudaStream_t st) {
  if (njobs < 1) return cudaSuccess;
  if (!jobs_dev) return cudaErrorInvalidValue;
  constexpr size_t kSmem = sizeof(float) * (SMAX * (SMAX + 1) + 2 * SMAX * SMAX);
  static bool attr_set[64] = {};
  const cudaError_t e = opt_in_smem(transfer_tail_grouped_kernel, static_cast<int>(kSmem), attr_set);
  if (e != cudaSuccess) return e;
  transfer_tail_grouped_kernel<<<njobs, 256, kSmem, st>>>(jobs_dev);
  return cudaGetLastError();
}

cudaError_t transfer_eig_launch(const float *WG, int kw, int kt, int kc, int t_is_left, float *M, float *Broot,
                                cudaStream_t st) {
  if (kt > SMAX || kc > kw || kt > kw) return cudaErrorInvalidValue;
  static bool attr_set[64] = {};
  const cudaError_t e = opt_in_smem(transfer_eig_kernel, static_cast<int>(kJacScratch), attr_set);
  if (e != cudaSuccess) return e;
  transfer_eig_kernel<<<1, 256, kJacScratch, st>>>(WG, kw, kt, kc, t_is_left, M, Broot);
  return cudaGetLastError();
}

// Self-test of the bounded waits: a cooperative grid whose barrier expects one
// more member than the grid holds, so it can never complete.  Every CTA gives
// up after limit_ns, sets kErrTimeout in *err and returns; nothing hangs and
// the context stays usable.  Used by the failure-detection tests.
namespace {
__global__ void wait_probe_kernel(unsigned *bar, unsigned members, uint64_t limit_ns, int *err) {
  __shared__ int s_ok;
  grid_barrier(bar, members, err, &s_ok, limit_ns);
}
}  // namespace

cudaError_t wait_probe_launch(int ctas, uint64_t limit_ns, void *ws, int *err, cudaStream_t st) {
  if (ctas < 1 || ctas > device_sm_count() || limit_ns > kWaitLimitNs) return cudaErrorInvalidValue;
  unsigned *bar = static_cast<unsigned *>(ws);
  cudaError_t e = cudaMemsetAsync(bar, 0, 4 * sizeof(unsigned), st);
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg;
  std::memset(&cfg, 0, sizeof(cfg));
  cfg.gridDim = dim3(ctas);
  cfg.blockDim = dim3(32);
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, wait_probe_kernel, bar, static_cast<unsigned>(ctas) + 1u, limit_ns, err);
}

}  // namespace htgb
