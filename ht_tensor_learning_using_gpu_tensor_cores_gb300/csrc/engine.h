// Internal interfaces between the host orchestration (api.cu) and the kernel
// translation units.  Not part of the public C ABI.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

namespace htgb {

// ----------------------------------------------------------------- views
// A column-major tensor seen as (L, N, R): element (l, n, r) at l + L*n + L*N*r.
// The matricisation over a contiguous group of modes has N = product of the
// group's dims, L = product of the dims before it, R = product after it.
struct View {
  long L, N, R;
};

// ------------------------------------------------------ GEMM over unfoldings
// D[m, j] = sum_k A(m, k) * B(j, k).  Each operand is a 3-D strided tensor
// (d0 innermost) read in one of three patterns:
enum OpKind : int {
  OP_KM3 = 0,   // K-major: row index on d1, k = (l on d0, r on d2), element l + d0*row + d0*d1*r
  OP_KM3Q = 1,  // K-major: row index on d2, k = (l on d0, r on d1), element l + d0*r + d0*d1*row
  OP_MN3 = 2    // MN-major: row index on d0, k on d1, fixed z on d2, element row + d0*k + d0*d1*z
};

struct Operand {
  int kind;
  const void *ptr;      // __nv_bfloat16* for the tcgen05 path, float* for the SIMT path
  long d0, d1, d2;
};

// One output tile.  a_row / b_row: first row of the A / B operand;
// a_z: d2 coordinate of an OP_MN3 A operand.  out_row/out_col: where the tile
// lands in a column-major output (OUT_COLMAJOR); valid_rows/cols clip it.
struct Tile {
  int a_row, a_z, b_row, valid_rows;
  long long out_row;
  int out_col, valid_cols;
};

enum OutMode : int { OUT_PARTIAL = 0, OUT_COLMAJOR = 1 };

// Output tiles are generated from a small descriptor passed by value in the
// kernel parameters (no host->device copy on the launch path).
enum TileKind : int {
  TILES_ROWS = 0,   // rows [0, rows) in blocks of 128, one column block
  TILES_SLABS = 1,  // (l-block, r) blocks of a (L, *, R) view, out_row = l + L*r
  TILES_GRAM = 2,   // blocks of an n x n symmetric matrix on or above the diagonal
  TILES_GRID = 3    // bm x bn blocks of a rows x n output, row block fastest
};
constexpr int kMaxGramRows = 256;   // n <= 32768
struct TileGen {
  int kind, count, bn, cols;
  int bm;                            // rows per tile: 128, or 256 for the paired-accumulator Gram tiles
  long long rows, L, R, n;
  int ni;                            // gram: number of 128-row blocks
  int prefix[kMaxGramRows + 1];      // gram: tiles before row block i
  int jmin[kMaxGramRows];            // gram: first column block of row block i
};

struct GemmArgs {
  Operand a, b;
  TileGen gen;
  int num_tiles;
  int splits;            // split-K factor (work items = num_tiles * splits)
  int out_mode;
  float *out;            // partial buffer [splits][num_tiles][BM][BN] or column-major output
  long long ld_out;
  int *err;              // device error word
  // tcgen05 path, column-major output only: the B operand holds two halves of
  // BN/2 rows each (a BF16 matrix split into high and low parts) and the
  // epilogue writes column j as acc[j] + acc[j + BN/2].
  int fold = 0;
  // tcgen05 path: 2 = each CTA computes a 256-row tile as two 128-row
  // accumulators that share every B stage (TileGen::bm must be 256)
  int mt = 1;
  // tcgen05 path, column-major output only: non-null = write the output in
  // BF16 here instead of FP32 to `out`
  __nv_bfloat16 *out16 = nullptr;
};

// tcgen05 path (BF16 operands), BM = 128, BN in {64, 128, 256}.
// Returns false (and fills *why) when the operand shapes cannot be expressed as
// TMA tensor maps (strides not multiples of 16 bytes, dims too large).
bool tc_gemm_supported(const GemmArgs &g, int bn, std::string *why);
// Grouped Grams of the batched path: one CTA per n x n Gram (n <= 256), the
// whole K range as one tile written column-major to G (ld = n).  Class 0:
// n <= 128 (128 x 128 tiles), class 1: n <= 256 (256 x 256); -1: not grouped.
// tc_gram_item appends an item (tensor maps included) to `out` (false: the
// operand cannot be read by TMA; why says so); the items of one class are
// copied to device memory (64-byte aligned) for tc_gram_grouped_launch.
int tc_gram_class(long n);
size_t tc_gram_item_bytes();
bool tc_gram_item(const Operand &a, long n, float *G, int *err, std::vector<unsigned char> &out, std::string *why);
cudaError_t tc_gram_grouped_launch(int cls, const void *items_dev, int count, cudaStream_t s);
cudaError_t tc_gemm_launch(const GemmArgs &g, int bn, cudaStream_t s);
// One-time set-up (kernel attributes, the tensor-map encoder) so that later
// launches can be recorded into a CUDA graph.
cudaError_t tc_prepare();
// number of 64-wide K blocks of an operand pair (tcgen05 path)
long tc_num_kblocks(const Operand &a);

// SIMT FP32 path (float operands), BM = 128, BN in {64, 128}.
// Grouped FP32 GEMMs of the batched path (the 3rd-order core pass): every
// tile of every GEMM of a group in one launch, each block a whole tile over
// the full K range (128 x 64 tiles, column-major output, row or slab tile
// generators).  simt_grouped_add appends the GEMM's parameters and its tiles
// (false: not a groupable GEMM); both tables are copied to device memory
// (8-byte aligned) for simt_grouped_launch.  The blobs are opaque storage.
struct SParamsBlob {
  unsigned long long w[24];
};
struct SimtBlockBlob {
  unsigned long long w[6];
};
bool simt_grouped_add(const GemmArgs &g, std::vector<SParamsBlob> &gemms, std::vector<SimtBlockBlob> &blocks);
cudaError_t simt_grouped_launch(const SParamsBlob *gemms_dev, const SimtBlockBlob *blocks_dev, int nblocks,
                                cudaStream_t s);
cudaError_t simt_gemm_launch(const GemmArgs &g, int bn, cudaStream_t s);
long simt_k_total(const Operand &a);

// Sum split-K partial tiles ([splits][tiles][gen.bm][bn]) into out.  symmetric
// bit 0 clear: plain column-major tiles; set: a symmetric Gram (tiles on/above
// the diagonal, mirrored into the lower triangle).  Bit 1: add the sums to what
// out holds instead of overwriting it (a Gram accumulated over slabs).
cudaError_t reduce_partials_launch(const float *partial, const TileGen &gen, int splits, int bn, float *out,
                                   long long ld_out, int symmetric, cudaStream_t s);
TileGen make_rows_gen(long long rows, int cols, int bn);
TileGen make_slabs_gen(long long L, long long R, int cols, int bn);
// rows x cols output in 128 x bn tiles (TILES_GRID); false when the tile count overflows
bool make_grid_gen(long long rows, long long cols, int bn, TileGen *g);
bool make_gram_gen(long long n, int bn, TileGen *g, int bm = 128);

// Multiprocessor count of the current device (cached per device).
int device_sm_count();

// --------------------------------------------------------------- small ops
cudaError_t convert_bf16_launch(const float *x, __nv_bfloat16 *xb, long long n, double *sumsq_partials,
                                int num_partials, cudaStream_t s);
cudaError_t sumsq_launch(const float *x, long long n, double *partials, int num_partials, cudaStream_t s);
// X (n1 x rest, FP32) -> xp (n1p x rest, BF16, rows n1..n1p-1 zero) + sum-of-squares partials
cudaError_t convert_bf16_pad_launch(const float *x, __nv_bfloat16 *xp, long long n1, long long n1p, long long rest,
                                    double *partials, int num_partials, cudaStream_t s);
// dst = src (first != 0) or dst += src, n floats
cudaError_t accumulate_launch(float *dst, const float *src, long long n, int first, cudaStream_t s);
// X (L x N) -> xb (same layout) and xbt (l-blocks of B = 2^lb: xbt[((l/B) N + n) B + l%B])
// in BF16 + sum-of-squares partials; 6 <= lb <= 12, L % B == 0, x 16-byte aligned
// Only the columns n in [n_begin, n_begin + n_count) (n_count < 0: to the end; both
// multiples of 2^(12 - lb)).
cudaError_t convert_bf16_dual_launch(const float *x, __nv_bfloat16 *xb, __nv_bfloat16 *xbt, long long L, long long N,
                                     int lb, double *partials, int num_partials, cudaStream_t s,
                                     long long n_begin = 0, long long n_count = -1);
cudaError_t f32_to_bf16_launch(const float *x, __nv_bfloat16 *y, long long n, cudaStream_t s);
// x <- bf16(x) in place (values kept in FP32) and y = the BF16 copy.
cudaError_t round_bf16_launch(float *x, __nv_bfloat16 *y, long long n, cudaStream_t s);
// W (rows x k, column-major FP32) -> Y (rows x 2h BF16): columns [0, k) the
// BF16 rounding hi(W), columns [h, h + k) the rounding of W - hi(W), the rest 0.
cudaError_t split_bf16_launch(const float *W, long long rows, int k, int h, __nv_bfloat16 *Y, cudaStream_t s);
cudaError_t sumsq_finish_launch(const double *partials, int n, double *out, cudaStream_t s);
// Grouped conversion of a batch (one launch for every tensor, then one finish
// launch): job j converts x (n1 x rest, FP32) to xb (n1p x rest BF16, rows
// zero-padded; null: sums only) in blocks [blk0, blk0 + nblk) of the launch
// (nblk <= the capacity of partials; job_of_block, in device memory, maps each
// block of the launch to its job) and leaves ||x||^2 in dsum[0].  The job
// table lives in device memory.
struct ConvJob {
  const float *x;
  __nv_bfloat16 *xb;
  double *partials, *dsum;
  long long n1, n1p, rest;
  int blk0, nblk;
};
// Grouped error pass of the batched path (3rd order): core = Bt Bkt (launch
// 0) and the first expansion step into Tm (1) for every job; then either the
// second expansion step into Wm (2) and the fused error tiles (3, as
// error_fused_launch, ntile = tiles x slabs of X) or, for a narrow job (the
// complementary leaf is the last mode, kc <= narrow_kb <= 64, kq <= narrow_kq
// <= 64), the second expansion step as small products (5, a block per (c, 256
// values of i1)) and the narrow error kernel (4, ntile = nblk[4] partials);
// then the sum of the partials into out[0].  blk0[k] / nblk[k]: the job's blocks in launch
// k (grid-stride within the job, 0 when it takes no part); blocks[k] = the
// launch sizes and job_of_block[k] (device) the job of each block of launch
// k.  Job table in device memory.
struct ErrJob {
  const float *Bt, *B0;        // B_t (kpq x kt); B0 = Bkt (kt x kc) or its transpose
  float *core, *Tm, *Wm;
  const float *Up, *Uq;        // leaves p (np x kp) and q (nq x kq)
  const float *X, *A, *B;      // error tiles: X (R x Cn per slab) against A B^T
  double *parts, *out;
  long long kpq, ldx, sx, lda, sa, ldb, R, Cn;
  int kt, kc, t_is_left, np, nq, kp, kq, kk, slabs, ntile, narrow;
  int blk0[6], nblk[6];
};
cudaError_t error_grouped_launch(const ErrJob *jobs_dev, int njobs, const int *blocks, const int *const *job_of_block,
                                 int narrow_kb, int narrow_kq, cudaStream_t s);
// Grouped narrow mode product (3rd-order core pass, rows of X contiguous,
// L >= 32): Z[row + L R j] = sum_i X[l + L (i + N r)] V[i + N j], row = l + L r,
// j < kz <= kb (kb <= 64, the largest kz of the launch).  Blocks
// [blk0, blk0 + nblk) of the launch stride over the job's rows.
struct NarrowJob {
  const float *X, *V;
  float *Z;
  long long L, R;
  int N, kz, blk0, nblk;
};
cudaError_t modeprod_narrow_grouped_launch(const NarrowJob *jobs_dev, const int *job_of_block, int nblocks, int kb,
                                          cudaStream_t s);
// Grouped first core contraction: T1[row + rows a] = sum_i Z[i + np row] Up[i + np a],
// a < kp <= 64; blocks [blk0, blk0 + nblk) stride over tiles of 64 rows.
struct T1Job {
  const float *Z, *Up;
  float *T1;
  long long rows;
  int np, kp, blk0, nblk;
};
// kp_max: the largest kp of the launch's jobs
cudaError_t core_t1_grouped_launch(const T1Job *jobs_dev, const int *job_of_block, int nblocks, int kp_max,
                                   cudaStream_t s);
// Grouped second core-contraction step (C[a, b, c] = sum_j T1[(j + nq c) +
// ldt a] Uq[j + nq b], as core_step2_launch without j ranges): job j owns the
// blocks [blk0, blk0 + kc) of the launch, one per c; job_of_block (device)
// maps the launch's blocks to jobs.  kp, kq <= 64, kp kq <= 4096.
struct Step2Job {
  const float *T1, *Uq;
  float *C;
  long long ldt;
  int nq, kp, kq, kc, blk0, pad;
};
cudaError_t core_step2_grouped_launch(const Step2Job *jobs_dev, const int *job_of_block, int nblocks, cudaStream_t s);
cudaError_t convert_grouped_launch(const ConvJob *jobs_dev, int njobs, int total_blocks, const int *job_of_block,
                                   cudaStream_t s);
// dst[0, count) = src[0, count) for every segment, one launch (table in device memory).
struct CopySeg {
  const float *src;
  float *dst;
  long long count;
};
cudaError_t copy_segments_launch(const CopySeg *segs_dev, int nseg, cudaStream_t s);

// C (m x n) = A^T B with A (K x m), B (K x n), column-major, compensated FP32.
cudaError_t gemm_tn_small_launch(const float *A, int lda, const float *B, int ldb, float *C, int ldc, int m, int n,
                                 int K, cudaStream_t s);
// C[a + kp*b + kp*kq*c] = sum_j T1[(j + nq*c) + ldt*a] * Uq[j + nq*b].  scratch (or
// null: one CTA per c) holds core_step2_ranges(nq, kc) * kp*kq*kc floats of partial
// sums over ranges of j, summed in order afterwards.
int core_step2_ranges(int nq, int kc);
cudaError_t core_step2_launch(const float *T1, long long ldt, int nq, int kp, const float *Uq, int kq, int kc, float *C,
                              float *scratch, cudaStream_t s);
// W[i0 + n0*i1 + n0*n1*c] = sum_{a,b} U0[i0,a] U1[i1,b] core[a + k0*b + k0*k1*c]  (T: n0*k1*k2 scratch)
cudaError_t expand2_launch(const float *U0, int n0, int k0, const float *core, const float *U1, int n1, int k1, int k2,
                           float *T, float *W, cudaStream_t s);
// C (m x n) = A (m x K) B (K x n), column-major
cudaError_t matmul_nn_launch(const float *A, long long lda, const float *B, int ldb, float *C, long long ldc,
                             long long m, int n, int K, cudaStream_t s);
// per-block partial sums of (X[r + ldx*c] - sum_k A[r + lda*k] B[c + ldb*k])^2 over an R x Cn
// matrix, repeated for `batch` slices offset by the given strides
int error_fused_blocks(long long R, long long Cn);
cudaError_t error_fused_launch(const float *X, long long ldx, long long sx, const float *A, long long lda, long long sa,
                               const float *B, long long ldb, long long R, long long Cn, int kk, int batch,
                               double *partials, cudaStream_t s);
cudaError_t transpose_small_launch(const float *A, int m, int n, float *AT, cudaStream_t s);
cudaError_t gaussian_fill_launch(float *dst, long long n, uint64_t seed, uint64_t stream, cudaStream_t s);

// ------------------------------------------------------- eigen-solver (batched)
// Top-K eigenpairs of symmetric PSD FP32 matrices by subspace iteration with
// CholeskyQR and a final Rayleigh-Ritz step.  All arrays column-major.
struct EigProblem {
  const float *G;    // n x n
  int n, s, K;       // subspace size s (<= 64, <= n), wanted K <= s
  float *Q, *Y;      // n x s work
  float *U;          // n x K out: Ritz vectors, descending Ritz values
  float *GU;         // n x K out: G * U
  float *theta;      // K out: Ritz values
  float *resid;      // 1 out: max_j ||G u_j - theta_j u_j|| / theta_1
  const float *start; // optional n x s start block (NULL = Gaussian)
  uint64_t seed, stream_id;
};
size_t eig_workspace_bytes(const EigProblem *probs, int nprob);
// One-time set-up of the eigen-solver kernels (attributes, occupancy).
cudaError_t eig_prepare();
// max_ctas > 0 caps the cooperative grid (several batches running at once).
// refine (0-2): CholeskyQR passes on the last block before Rayleigh-Ritz.
cudaError_t eig_batched(EigProblem *probs, int nprob, int iters, void *ws, size_t ws_bytes, int *err,
                        cudaStream_t s, int *launches, int max_ctas = 0, int refine = 0);
// Grouped solver of the batched path: every problem of a batch in one launch,
// one CTA per problem (no cooperative launch, no CTA waits on another).
// eig_grouped_fill appends one table entry per problem (entry_bytes each) to
// `table`, carving the problems' buffers from ws; the table is copied to
// device memory (16-byte aligned) before eig_grouped_launch reads it.
size_t eig_grouped_workspace_bytes(const EigProblem *probs, int nprob);
size_t eig_grouped_entry_bytes();
cudaError_t eig_grouped_fill(const EigProblem *probs, int nprob, void *ws, size_t ws_bytes,
                             std::vector<unsigned char> &table);
// Longest problems first (CTAs start in index order).
void eig_grouped_order(std::vector<unsigned char> &table);
cudaError_t eig_grouped_launch(const void *table_dev, int nprob, int iters, int refine, cudaStream_t st);
// Orthonormalise the columns of tall matrices in place (CholeskyQR, `passes`
// times; the first pass shifted).  Uses the eigen-solver's workspace layout;
// a wait that runs out sets bits in *err.
cudaError_t cholqr_batched(EigProblem *probs, int nprob, int passes, void *ws, size_t ws_bytes, int *err, cudaStream_t s,
                           int *launches);
// Self-test of the bounded waits: a cooperative grid of `ctas` CTAs (<= SMs)
// whose barrier expects ctas + 1 members; every CTA gives up after limit_ns
// (<= the library's 2 s wait limit) and sets kErrTimeout in *err.  ws: 16 bytes.
cudaError_t wait_probe_launch(int ctas, uint64_t limit_ns, void *ws, int *err, cudaStream_t st);
// Grouped transfer tail of the batched path (3rd order), a CTA per tensor:
// WG = U^T GU, the transfer eigen step into M and Bkt (Broot = Bkt^T when
// !t_is_left), Bt = C M.  kw, kt <= 64.  Job table in device memory.
struct TailJob {
  const float *U, *GU;   // complementary leaf: basis and G U, nc x kw
  const float *C;        // kpq x kt core product
  float *M, *Bkt, *Broot, *Bt;
  long long kpq;
  int nc, kw, kt, kc, t_is_left;
};
cudaError_t transfer_tail_grouped_launch(const TailJob *jobs_dev, int njobs, cudaStream_t st);
// Transfer-tensor eigen step (see eig.cu).  WG: kw x kw.  M: kt x kt, Bkt: kt x kc.
cudaError_t transfer_eig_launch(const float *WG, int kw, int kt, int kc, int t_is_left, float *M, float *Broot,
                                cudaStream_t st);
// Small SVD from a Gram: GW (s x s) = W^T W.  M1 (s x k1) = top-k1 eigenvectors,
// M2 (s x k2) = top-k2 eigenvectors scaled by sigma^-1, Broot (k1 x k2) = M1^T GW M2.
cudaError_t svd_from_gram_launch(const float *GW, int s, int k1, int k2, float *M1, float *M2, float *Broot,
                                 cudaStream_t st);
// The same for up to four independent problems in one launch (a CTA each).
struct SvdGramProb {
  const float *GW;
  int s, k1, k2;
  float *M1, *M2, *Broot;
};
cudaError_t svd_from_gram_batched_launch(const SvdGramProb *probs, int nprob, cudaStream_t st);

// ------------------------------------------------------- Householder TSQR (tsqr.cu)
size_t tsqr_workspace_bytes(long long m, int k);
// R (k x k, column-major, upper triangular, diagonal >= 0) of A = Q R for A
// (m x k, column-major, leading dimension lda), k <= 64; RtR (optional, may be
// null) = R^T R in compensated FP32.  ws holds tsqr_workspace_bytes(m, k).
cudaError_t tsqr_launch(const float *A, long long m, int k, long long lda, float *R, float *RtR, void *ws,
                        size_t ws_bytes, cudaStream_t st, int *launches);

// ------------------------------------------- Gram-free leaf range finder (sketch.cu)
// Yn = Y + nu Q (n x s), nu = nu_rel * tr(W) for the s x s matrix W.
cudaError_t nystrom_shift_launch(const float *Y, const float *Q, long long n, int s, const float *W, float nu_rel,
                                 float *Yn, cudaStream_t st);
// H (s x s) = R1 (sym(W) + nu I)^-1 R1^T, nu as above (FP64, one CTA per
// problem; up to four problems in one launch).
struct NystromProb {
  const float *W, *R1;
  int s;
  float *H;
};
cudaError_t nystrom_core_launch(const NystromProb *probs, int nprob, float nu_rel, int *err, cudaStream_t st);

// ------------------------------------------------------- learned sketch (learn.cu)
size_t sketch_workspace_bytes(int batch, int n, int s);
// loss[b] and the batch-mean gradient of L(S) = mean_b [1 - tr(Q_b^T G_b Q_b) / tr(G_b)],
// Q_b = orth(G_b S); G: batch x n x n, S and grad: n x s, all column-major device memory.
cudaError_t sketch_loss_grad(const float *G, const float *trG, int batch, int n, int s, const float *S, float *grad,
                             double *loss, int *bad, void *ws, cudaStream_t st, int *launches);
cudaError_t sketch_adam(float *S, const float *g, float *m, float *v, long long count, float lr, float b1, float b2,
                        float eps, int step, cudaStream_t st);

// ------------------------------------------------ HT-format operations (htops.cu)
// Slab z < batch: C + z sC (m x n, ldc) = (A + z sA) (m x k, lda) B^T (n x k, ldb),
// column-major, k <= 64.
cudaError_t gemm_nt_launch(const float *A, long long lda, long long sA, const float *B, long long ldb, float *C,
                           long long ldc, long long sC, long long m, long long n, int k, long long batch,
                           cudaStream_t s);
// out[(c + kc b) + kc kq a] = sum_rt Bt[a + kp b + kp kq rt] M[rt + kt c]; M null: identity (kc = kt)
cudaError_t eval_core_launch(const float *Bt, int kp, int kq, int kt, const float *M, int kc, float *out,
                             cudaStream_t s);
// One side of an entry: with W, a[y] = sum_x W[i_row (ky kx) + y + ky x] Uv[i_vec + n_vec x];
// without W, a[y] = Uv[i_vec + n_vec y].
struct EvalSide {
  const float *W;
  const float *Uv;
  long long n_row, n_vec;
  int mode_row, mode_vec, kx;
};
struct EvalPlan {
  int order, ky;
  EvalSide side[2];
};
// out[e] = sum_y a0[y] a1[y] at the index tuple idx[e*order .. e*order + order);
// an index out of range sets *err to 1.
cudaError_t evaluate_launch(const EvalPlan &ep, const long long *idx, long long count, float *out, int *err,
                            cudaStream_t s);

// ------------------------------------------------------ HT tensor layer (layer.cu)
constexpr int kLayerMaxRank = 64;
// u1 (n0, m0, r3), u2 (n1, m1, r4), u3 (n2, m2, r2), b2 (r3, r4, r1), b1 (r1, r2), C-order
struct LayerShape {
  int n[3], m[3];
  int r1, r2, r3, r4;
};
// P[a, b, r1] (A x B x r1), Q[c, r1] (C x r1) and, when T1 is non-null,
// T1[a, r4, r1] = sum_r3 u1[a, r3] b2[r3, r4, r1]
cudaError_t layer_pq_launch(const LayerShape &sh, const float *u1, const float *u2, const float *u3, const float *b2,
                            const float *b1, float *P, float *Q, float *T1, cudaStream_t s);
// W (Nout x Nin, row-major) from P and Q, into W32 (FP32) or, when W32 is null, W16 (BF16)
cudaError_t layer_weight_launch(const LayerShape &sh, const float *P, const float *Q, float *W32, __nv_bfloat16 *W16,
                                cudaStream_t s);
// y[z, o] = act(y[z, o] + bias[o]) (bias may be null; act 0 identity, 1 ReLU)
cudaError_t bias_act_launch(float *y, const float *bias, long long batch, long long nout, int act, cudaStream_t s);
// out[o] = sum_z dy[z, o]; part holds layer_colsum_chunks(batch) * nout floats
int layer_colsum_chunks(long long batch);
cudaError_t layer_colsum_launch(const float *dy, long long batch, long long nout, float *part, float *out,
                                cudaStream_t s);
// Floats of the dQ partial buffer layer_factor_grads_launch wants (0: the shape
// takes the unfused path, which needs none).
size_t layer_dq_part_count(const LayerShape &sh);
// du1, du2, du3, db2, db1 from dW (Nout x Nin, row-major), via dP, dQ, dT1 (scratch of P, Q, T1's sizes)
cudaError_t layer_factor_grads_launch(const LayerShape &sh, const float *dW, const float *u1, const float *u2,
                                      const float *u3, const float *b2, const float *b1, const float *P,
                                      const float *Q, const float *T1, float *dP, float *dQ, float *dT1, float *dQpart,
                                      float *du1, float *du2, float *du3, float *db2, float *db1, cudaStream_t s);

}  // namespace htgb
