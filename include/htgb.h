/*
 * htgb -- hierarchical Tucker (HT) decomposition on one GB300 (sm_103a).
 *
 * C ABI.  Plain pointers and sizes only; no exceptions cross this boundary and
 * every entry point except the two reference-compatible shims returns an
 * ht_status_t.  The last error message of the calling thread is available from
 * ht_last_error().
 *
 * Tensors are column-major (first index fastest), as in the reference's CUDA
 * code (third_order_tensor_decompsition/CUDA/Optimized/htd_tensorcore.cu:12):
 * element (i1, i2, i3) of an n1 x n2 x n3 tensor is x[i1 + n1*i2 + n1*n2*i3].
 *
 * Dimension tree and ranks: node 0 is the root.  Leaves hold one mode.  The
 * reference's node numbering and rank vector k[] (k[0] = 1) are kept:
 *   3rd order (ht_init.cu:16-20, HT_TensorLy.py:23-24): 0 root, 1 = {1,2},
 *             2 = {3}, 3 = {1}, 4 = {2};
 *   4th order (4D/.../Optimized/ht_init.cu:19-23): 0 root, 1 = {1,2},
 *             2 = {3,4}, 3..6 = {1}..{4}.
 *
 * Outputs follow the reference's transfer-tensor layout (CUDA/Optimized/ttm.cu:2-36):
 *   U[t] for every leaf t: n_t x k_t, column-major, orthonormal columns in
 *        descending order of the mode Gram's eigenvalues;
 *   B[t] for every interior node t (root included): k_left x k_right x k_t,
 *        column-major, so that U_t = (U_right kron U_left) B_t and the tensor
 *        is X ~= reshape(U_left_root B_0 U_right_root^T).
 */
#ifndef HTGB_H
#define HTGB_H

#ifdef __cplusplus
extern "C" {
#endif

#define HT_MAX_ORDER 4
#define HT_MAX_NODES 7

typedef enum {
    HT_OK = 0,
    HT_ERR_INVALID_ARG = 1,    /* bad dims, tree, ranks or pointers            */
    HT_ERR_CUDA = 2,           /* a CUDA runtime call failed                   */
    HT_ERR_OUT_OF_MEMORY = 3,  /* device workspace could not be allocated      */
    HT_ERR_NOT_CONVERGED = 4,  /* eigen-solver residual above tolerance        */
    HT_ERR_TIMEOUT = 5,        /* a kernel's bounded wait expired (no hang)    */
    HT_ERR_UNSUPPORTED = 6,    /* shape/tree combination not implemented       */
    HT_ERR_NO_DEVICE = 7,      /* no CUDA device / not an sm_103 device        */
    HT_ERR_NUMERICAL = 8       /* NaN/Inf in the input or a breakdown          */
} ht_status_t;

typedef enum {
    HT_PREC_FP32 = 0,  /* plain path: every product in FP32 on CUDA cores          */
    HT_PREC_BF16 = 1   /* mixed path: BF16 tcgen05 GEMMs, FP32 accumulation in TMEM */
} ht_precision_t;

typedef enum {
    HT_LEAF_GRAM = 0,   /* leaf bases from the mode Gram X_(t) X_(t)^T               */
    HT_LEAF_SKETCH = 1  /* leaf bases from a randomized range finder on X_(t) that
                           never forms the Gram: test matrix X_(t)^T S for a per-mode
                           block S (n_t x (k_t + oversample): sketch[t] or Gaussian),
                           power_steps applications of X_(t) X_(t)^T as two streaming
                           products each, CholeskyQR2 between them, a Nystrom core
                           for the leaf basis; 3rd order: the interior node from the
                           Householder TSQR of X_(t) V (ht_decompose only)          */
} ht_leaf_method_t;

/* Flags */
#define HT_FLAG_COMPUTE_ERROR  1   /* fill ht_report_t.rel_err (one extra pass)   */
#define HT_FLAG_SYNC_TIMING    2   /* per-stage times in ht_report_t.ms_stage    */

typedef struct {
    int order;                   /* 3 or 4                                        */
    int n_nodes;                 /* 2*order-1                                     */
    int parent[HT_MAX_NODES];    /* -1 for the root                               */
    int left[HT_MAX_NODES];      /* -1 for leaves                                 */
    int right[HT_MAX_NODES];
    int mode_mask[HT_MAX_NODES]; /* bit m set when mode m (0-based) is in node t  */
    int rank[HT_MAX_NODES];      /* k_t; rank[0] = 1                              */
} ht_tree_t;

typedef struct {
    int precision;        /* ht_precision_t                                      */
    int leaf_method;      /* ht_leaf_method_t                                    */
    int oversample;       /* subspace size = k + oversample (default 16)         */
    int eig_iters;        /* subspace iterations per leaf Gram (default 0 =
                             10 on the FP32 path, 6 on the mixed path)           */
    int power_steps;      /* power steps of the range finder (default 1)         */
    unsigned long long seed;  /* Gaussian start / test matrices (default 1234)   */
    const float *sketch[HT_MAX_ORDER]; /* optional start matrices per mode, n_m x (k+p),
                                          column-major, host or device; NULL = Gaussian.
                                          HT_LEAF_GRAM: the eigen-solver's start block;
                                          HT_LEAF_SKETCH: the range finder's block S   */
    int flags;            /* HT_FLAG_*                                           */
    double eig_tol;       /* residual tolerance reported as HT_ERR_NOT_CONVERGED
                             when exceeded (0 = do not check)                    */
} ht_config_t;

typedef struct {
    double rel_err;          /* ||X - Xhat||_F / ||X||_F (HT_FLAG_COMPUTE_ERROR)  */
    double norm_x;           /* ||X||_F                                           */
    float ms_total;          /* device time of the decomposition (CUDA events)    */
    float ms_stage[8];       /* 0 input/convert, 1 grams, 2 eig, 3 core pass,
                                4 transfer tensors, 5 error, 6 h2d, 7 d2h.  When a
                                3rd-order BF16 Gram-path call with host input
                                takes X in slabs (tensors of 256 MiB and more),
                                stage 0 also holds the mode-1/2 Grams, which
                                overlap the copy, and stage 1 the last mode's
                                Gram alone.  With
                                HT_LEAF_SKETCH stage 1 is the whole range finder
                                and stage 2 is empty.                             */
    double eig_residual[HT_MAX_NODES]; /* max_j ||G u_j - theta_j u_j|| / theta_1   */
    int gpu_launches;        /* kernels launched by this call                     */
    int path_flags;          /* bit 0: tcgen05 path used, bit 1: SIMT path used   */
} ht_report_t;

/* ------------------------------------------------------------------ setup */
ht_status_t ht_config_default(ht_config_t *cfg);
/* Trees of the reference: htd (3rd order) and htd4 (4th order).  k has
 * 5 / 7 entries indexed by node id; k[0] is ignored (set to 1). */
ht_status_t ht_tree_reference_3d(ht_tree_t *tree, const int *k);
ht_status_t ht_tree_balanced_4d(ht_tree_t *tree, const int *k);
ht_status_t ht_tree_validate(const ht_tree_t *tree, const long *dims, int order);

/* -------------------------------------------------------------- decompose */
/*
 * HT decomposition of x (host or device pointer, column-major, dims[0..order)).
 * Replaces htd() (3D/Opt/htd_tensorcore.cu:2, 3D/Opt/htd_batch.cu:2,
 * 3D/Base/htd_unopt.cu:2) and htd4() (4D/Opt/htd4_tensorcore.cu:2) with the
 * factors returned instead of freed.
 * U[t] (leaves) and B[t] (interior nodes, root) are caller-allocated, host or
 * device; other entries of U/B are ignored and may be NULL.  stream may be
 * NULL (legacy default stream).  The call is synchronous with respect to the
 * host: it returns after the outputs are written.
 */
ht_status_t ht_decompose(const float *x, const long *dims, int order,
                         const ht_tree_t *tree, const ht_config_t *cfg,
                         float *const *U, float *const *B,
                         ht_report_t *report, void *stream);

/* Out-of-core variant for 3rd-order tensors that stay in host memory (pinned
 * memory gives the full copy bandwidth; pageable memory works through the
 * driver's staging).  The reference's 3D/TSQR variant streams the tensor in
 * four slabs of frontal slices (third_order_tensor_decompsition/CUDA/TSQR/
 * htd_tensorcore.cu:58-111).  Here X goes through two device slab buffers of at
 * most slab_bytes together, three times (four with HT_FLAG_COMPUTE_ERROR):
 * slabs along mode 3 for the mode-1 and mode-2 Grams, slabs along mode 2 for
 * the mode-3 Gram, slabs along mode 3 for the core pass (and the error); each
 * copy overlaps the work on the previous slab.  Same outputs and
 * configuration as ht_decompose.  report->ms_stage: 0 first pass (Grams 1, 2),
 * 1 second pass (Gram 3), 2 eigen-solver, 3 core pass, 4 transfer tensors,
 * 5 error pass. */
ht_status_t ht_decompose_streaming(const float *x, const long *dims, int order,
                                   const ht_tree_t *tree, const ht_config_t *cfg,
                                   float *const *U, float *const *B,
                                   unsigned long long slab_bytes,
                                   ht_report_t *report, void *stream);

/* Relative reconstruction error ||X - Xhat||_F / ||X||_F of an HT
 * representation (one fused pass over x on the GPU; htd_batch.cu:196-244). */
ht_status_t ht_reconstruct_error(const float *x, const long *dims, int order,
                                 const ht_tree_t *tree,
                                 const float *const *U, const float *const *B,
                                 double *rel_err, void *stream);

/* ------------------------------------------------------ HT-format operations */
/* Full tensor Xhat (column-major, dims[0..order)) of an HT representation.
 * Replaces the reference's reconstruction by node bases
 * (third_order_tensor_decompsition/CUDA/Optimized/htd_tensorcore.cu:295-331,
 * htd_batch.cu:196-244), which it only uses to measure the error.  Factors and
 * x_out may be host or device memory; returns after the result is complete. */
ht_status_t ht_reconstruct(const long *dims, int order, const ht_tree_t *tree,
                           const float *const *U, const float *const *B,
                           float *x_out, void *stream);

/* Entries of an HT representation at count index tuples, without forming the
 * tensor: out[e] = Xhat(idx[e*order], ..., idx[e*order + order - 1]), 0-based.
 * Each entry is contracted from the leaf rows to the root (cost
 * sum_t k_l k_r k_t per entry).  An index outside its mode returns
 * HT_ERR_INVALID_ARG.  idx and out may be host or device memory. */
ht_status_t ht_evaluate(const long *dims, int order, const ht_tree_t *tree,
                        const float *const *U, const float *const *B,
                        const long long *idx, long long count, float *out, void *stream);

/* ---------------------------------------------------- unfolding primitives */
/* The three matricisation products the decomposition is built from, exposed
 * for direct use.  Modes lo..hi (0-based, contiguous) form the group g; with
 * L = prod(dims[<lo]), N = prod(dims[lo..hi]), R = prod(dims[>hi]) the tensor
 * is seen as (L, N, R) and X_(g) is N x (L*R).  precision: ht_precision_t.
 * All pointers may be host or device; outputs are column-major.
 *
 * ht_mode_gram:     G (N x N) = X_(g) X_(g)^T
 *   (the leaf Gram GEMMs, 3D/Opt/htd_tensorcore.cu:83-121, htd_batch.cu:83-106)
 * ht_mode_product:  Z ((L*R) x k) = X_(g)^T W, W: N x k
 *   (the mode-n TTM, 3D/Opt/ttm.cu:2-36 and the root transfer htd_batch.cu:165)
 * ht_corange_product: Z (N x k) = X_(g) Q, Q: (L*R) x k
 *   (the rsvd products B = C^T A, 3D/Opt/kernel.cu:618) */
ht_status_t ht_mode_gram(const float *x, const long *dims, int order, int lo, int hi, int precision,
                         float *G, void *stream);
ht_status_t ht_mode_product(const float *x, const long *dims, int order, int lo, int hi, const float *W, int k,
                            int precision, float *Z, void *stream);
ht_status_t ht_corange_product(const float *x, const long *dims, int order, int lo, int hi, const float *Q, int k,
                               int precision, float *Z, void *stream);

/* R factor of A = Q R for a tall-skinny A (m x k, column-major, leading
 * dimension lda >= m, 1 <= k <= 64) by Householder TSQR on the GPU: every
 * row block folded into per-warp R factors with Householder reflections
 * (warp-shuffle reductions), the warps' factors combined in a shared-memory
 * tree and the CTAs' in a fan-in-8 tree across the grid, in one launch.
 * Replaces the reference's tsqr_svd / tsqr_svd_half row-block QR
 * (third_order_tensor_decompsition/CUDA/TSQR/kernel.cu:500-949, geqrf at
 * :326-350), which factors four host-split blocks with cuSOLVER.
 * R (k x k, column-major) is upper triangular with a non-negative diagonal.
 * A and R may be host or device memory; returns after R is written. */
ht_status_t ht_tsqr(const float *A, long long m, int k, long long lda, float *R, void *stream);

/* ht_mode_gram_noalloc: the FP32 mode Gram G (N x N) = X_(g) X_(g)^T with no
 * memory allocation at all.  It has no counterpart in the reference.
 *
 * It is for callers that must not allocate device memory while they run:
 * code inside a host-side memory pool or allocator callback, a caller whose
 * memory budget is fixed when it starts, or one whose device memory belongs to
 * another framework's caching allocator.  ht_mode_gram may grow the library's
 * cached workspace with cudaMalloc and stage host data; this entry point never
 * calls cudaMalloc, cudaFree or any allocating library routine.
 *
 * x (the column-major tensor) and G must both be device memory.  The split-K
 * partial sums live in one fixed scratch array of HT_NOALLOC_SCRATCH_BYTES,
 * compiled into the library as a static device array: every GPU that loads
 * the library holds it until the process exits.  N = prod(dims[lo..hi]) may
 * be at most HT_NOALLOC_MAX_GRAM; larger N returns HT_ERR_UNSUPPORTED.
 * The first call on each device looks the array's device address up once
 * (cudaGetSymbolAddress); make that first call before any stream capture.
 * All calls on a device share the one array and it keeps the last call's
 * contents (every partial tile is rewritten before it is read, so nothing
 * needs clearing): calls whose work overlaps on the GPU, on different streams
 * or from different threads, race and give wrong results; order them on one
 * stream.  Work is queued on `stream`; the call returns without waiting. */
#define HT_NOALLOC_SCRATCH_BYTES (16u << 20)
#define HT_NOALLOC_MAX_GRAM 2048
ht_status_t ht_mode_gram_noalloc(const float *x, const long *dims, int order, int lo, int hi, float *G,
                                 void *stream);

/* Self-test of failure detection (no counterpart in the reference): launches a
 * cooperative grid of `ctas` CTAs (at most the device's multiprocessor count)
 * whose grid barrier waits for ctas + 1 members, so the wait can only run
 * out.  Every CTA gives up after limit_ms (0 < limit_ms <= 2000; the library's
 * own waits give up after 2000 ms) and the call returns HT_ERR_TIMEOUT, as a
 * decomposition does when one of its waits runs out; nothing hangs and the
 * device stays usable for the next call. */
ht_status_t ht_selftest_wait_timeout(int ctas, double limit_ms, void *stream);

/* ------------------------------------------------------------ batched path */
typedef struct {
    double rel_err_p50;      /* median relative error over the batch (HT_FLAG_COMPUTE_ERROR) */
    double rel_err_p99;      /* 99th percentile (nearest rank)                               */
    double rel_err_max;
    float ms_total;          /* device time of the batch (CUDA events around the launch)     */
    int gpu_launches;        /* kernels launched per batch                                   */
    int graph_replayed;      /* 1 when the cached CUDA graph of an identical batch ran       */
    int lanes;               /* concurrent streams the batch was spread over                 */
    int grouped;             /* 1: the batch ran as grouped stages (every mode <= 512)       */
    float ms_phase[6];       /* grouped: device ms of (0) conversion and leaf Grams, (1) the
                                leaf solver, (2) the core pass, (3) the transfer tails,
                                (4) the error pass, (5) the copies to the caller's buffers
                                (else 0)                                                      */
} ht_batch_report_t;

/* Decompose `count` tensors of the same order in one call.  Replaces the
 * reference's driver loop that calls htd() once per tensor size
 * (3D/Opt/ht_init.cu:9-47) for the many-small-tensors case.
 *   x[i]   DEVICE pointer to tensor i (column-major, dims[i*order .. +order));
 *   trees  count trees (trees[i] for tensor i);
 *   U, B   count x HT_MAX_NODES tables of DEVICE output pointers: U[i*HT_MAX_NODES + t]
 *          and B[i*HT_MAX_NODES + t] as in ht_decompose for tensor i;
 *   rel_err host array of count (HT_FLAG_COMPUTE_ERROR) or NULL.
 * When every mode of the batch is at most 512 it runs stage by stage, one launch
 * per stage for all tensors (conversion, leaf Grams, leaf solver, core pass,
 * transfer tensors, error, copies), each tensor in a workspace region of its
 * own; otherwise the tensors are spread over concurrent streams.
 * The first call records the whole batch into a CUDA graph; a later call with
 * the same count, dims, trees, config and pointers replays it (fixed buffers,
 * new contents).  Synchronous with respect to the host. */
ht_status_t ht_decompose_batched(int count, const float *const *x, const long *dims, int order,
                                 const ht_tree_t *trees, const ht_config_t *cfg,
                                 float *const *U, float *const *B, double *rel_err,
                                 ht_batch_report_t *report, void *stream);
/* Free the batched path's cached graph and workspace on the current device. */
ht_status_t ht_release_batch(void);
/* Launch shape of later ht_decompose_batched calls on the current device:
 * lanes = concurrent streams (1..32, 0 = the default 16) and eig_ctas = cap on
 * each lane's cooperative eigen-solver grid (0 = SMs / lanes, at least 8).  The
 * library's autotuner (autotune.tune_batched) picks them per size bucket; no
 * counterpart in the reference, which has no batched path. */
ht_status_t ht_batch_set_tuning(int lanes, int eig_ctas);

/* ---------------------------------------------------------- learned sketch */
/* Training of a per-mode sketch S (n x s): the start block of the leaf range
 * finder, used as ht_config_t.sketch[m] with eig_iters = 1 (Y = G S, Rayleigh-
 * Ritz on span(Y)).  No counterpart in the reference, whose range finder draws a
 * Gaussian test matrix (3D/Opt/kernel.cu:595-680); the Gaussian start block
 * stays the default and the yardstick of the learned one.
 *
 * ht_sketch_loss_grad: for `batch` mode Grams G (batch x n x n, column-major,
 * device) with traces trG (device), the forward value
 *   loss[b] = 1 - tr(Q_b^T G_b Q_b) / tr(G_b),   Q_b = orth(G_b S)  (CholeskyQR)
 * (host array of batch) and the adjoint grad = d mean_b loss[b] / dS (n x s,
 * device).  A column of G_b S in the span of the earlier columns to rounding
 * (a Gram of rank below s) is left out of Q_b, so loss[b] stays in [0, 1].
 * Synchronous; HT_ERR_NUMERICAL when a Gram, S or a factor holds NaN/Inf.
 * ht_sketch_adam: one Adam step on S with moments m, v (count = n*s, device),
 * step >= 1, beta1 0.9, beta2 0.999, eps 1e-8.  Asynchronous on `stream`. */
ht_status_t ht_sketch_loss_grad(const float *G, const float *trG, int batch, int n, int s, const float *S,
                                float *grad, double *loss, void *stream);
ht_status_t ht_sketch_adam(float *S, const float *grad, float *m, float *v, long long count, float lr, int step,
                           void *stream);

/* -------------------------------------------------------- HT tensor layer */
/* A fully connected layer whose weight is an HT tensor, as the reference's
 * tNet / AlexNet_ht layers (HT_tensor_layer/FC_MNIST/mnist_ht.py:199-245,
 * Alex_ImageNet/model/alexnet.py:157-170).  x is (batch, n[0], n[1], n[2]) and
 * y is (batch, m[0], m[1], m[2]), both C-order; the parameters keep the
 * reference's C-order layouts:
 *   u1 (n[0], m[0], r[0])   u2 (n[1], m[1], r[1])   u3 (n[2], m[2], r[2])
 *   b2 (r[0], r[1], r[3])   b1 (r[3], r[2])         bias (m[0], m[1], m[2])
 * and y[z, m0, m1, m2] = sum x[z, n0, n1, n2] u1[n0, m0, e] b2[e, f, g]
 *   u2[n1, m1, f] b1[g, h] u3[n2, m2, h]  (+ bias), the reference's einsum chain.
 * Ranks <= 64.  All pointers are device memory.  The calls are asynchronous on
 * `stream` and use a per-device workspace of their own: calls that may overlap
 * on the GPU (different streams) must be ordered by the caller.
 * precision: HT_PREC_FP32 (FP32 SIMT products) or HT_PREC_BF16 (tcgen05
 * products on BF16 operands, FP32 accumulation; needs n and m products that are
 * multiples of 8). */
typedef struct {
    int n[3];   /* input modes  */
    int m[3];   /* output modes */
    int r[4];   /* ranks of u1, u2, u3 and the third dimension of b2 */
} ht_layer_shape_t;

/* W (m0*m1*m2 x n0*n1*n2, row-major: an nn.Linear weight) from the factors. */
ht_status_t ht_layer_weight(const ht_layer_shape_t *shape, const float *u1, const float *u2, const float *u3,
                            const float *b2, const float *b1, float *W, void *stream);
/* y = act(x W^T + bias); bias may be NULL; activation 0 = none, 1 = ReLU. */
ht_status_t ht_layer_forward(const ht_layer_shape_t *shape, const float *u1, const float *u2, const float *u3,
                             const float *b2, const float *b1, const float *bias, int activation, int precision,
                             const float *x, long long batch, float *y, void *stream);
/* Gradients of sum(dy * y) for y = x W^T + bias: dx (may be NULL), the five
 * factor gradients (same layouts as the factors) and dbias (may be NULL). */
ht_status_t ht_layer_backward(const ht_layer_shape_t *shape, const float *u1, const float *u2, const float *u3,
                              const float *b2, const float *b1, int precision, const float *x, const float *dy,
                              long long batch, float *dx, float *du1, float *du2, float *du3, float *db2,
                              float *db1, float *dbias, void *stream);
/* Synchronise the device and report (then clear) a wait that timed out inside
 * an earlier layer call on this device: HT_ERR_TIMEOUT, else HT_OK. */
ht_status_t ht_layer_check(void);
/* Free the layer workspace of the current device. */
ht_status_t ht_layer_release(void);

/* Bytes of device workspace ht_decompose needs for this problem. */
ht_status_t ht_workspace_size(const long *dims, int order, const ht_tree_t *tree,
                              const ht_config_t *cfg, unsigned long long *bytes);
/* Free the cached device workspace of the current device. */
ht_status_t ht_release_workspace(void);

const char *ht_status_string(ht_status_t s);
const char *ht_last_error(void);
/* Number of kernels this library launched since load (all threads). */
unsigned long long ht_kernel_launch_count(void);

/* ----------------------------------------------- reference-compatible shims */
/* float htd(dt *x, long a, long b, long c, int *k)
 *   third_order_tensor_decompsition/CUDA/Optimized/function.h:6 (htd_tensorcore.cu:2).
 * x: host tensor a x b x c (column-major), k[5] ranks by node id.  Runs the
 * mixed-precision path and returns the relative reconstruction error, as the
 * reference does; returns a negative value on failure (see ht_last_error). */
float htd(float *x, long a, long b, long c, int *k);

/* void htd4(dt *X, long a, long b, long c, long d, int *k, cublasHandle_t, cusolverDnHandle_t)
 *   fourth_order_tensor_decomposition/single_GPU/CUDA/Optimized/function.h:6
 *   (htd4_tensorcore.cu:2).  The two handle arguments are accepted and ignored.
 * The error is printed to stdout as the reference does. */
void htd4(float *x, long a, long b, long c, long d, int *k, void *cublas_handle, void *cusolver_handle);

#ifdef __cplusplus
}
#endif
#endif /* HTGB_H */
