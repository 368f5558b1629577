// C ABI and host orchestration of the HT decomposition (see include/htgb.h).
//
// Algorithm (root-to-leaf hierarchical SVD, the reference's algorithm:
// third_order_tensor_decompsition/CUDA/Optimized/htd_batch.cu:78-165,
// Python/HT_TensorLy.py:52-72, 4D/.../htd4_tensorcore.cu:2-228):
//   leaves      U_t = top-k_t eigenvectors of G_t = X_(t) X_(t)^T
//   interior    U_t = top-k_t left singular vectors of X_(t)
//   transfer    B_t = (U_r kron U_l)^T U_t,   B_root = U_l^T X_(l) U_r
//
// 3rd order.  The root's children are an interior node t = {p,q} and a leaf c
// (the complementary mode).  X_(t)^T X_(t) = G_c, so with V = the top-k_t
// eigenvectors of G_c the top-k_t left singular vectors of X_(t) are
// U_t = X_(t) V P Lambda^-1/2, where V^T G_c V = P Lambda P^T.  Therefore
//   B_t    = (U_q kron U_p)^T X_(t) V P Lambda^-1/2 = C_V P Lambda^-1/2
//   B_root = U_t^T X_(t) U_c = Lambda^-1/2 P^T V^T G_c U_c
// where C_V = X x_p U_p^T x_q U_q^T x_c V^T is the projected core.  The
// interior node costs one streaming pass over X (the mode-c product) instead
// of the reference's QR + SVD of the n^2 x n matricisation (kernel.cu:719-830).
//
// 4th order (balanced tree {1,2},{3,4}).  Both root children are interior:
// a randomized range finder on A = X_(12) (Gaussian test matrix, oversampling
// p, q power steps, CholeskyQR) gives Q with A ~ Q Q^T A; W = A^T Q and the
// SVD of W from its Gram give U_12 = Q U_s, U_34 = W U_s Sigma^-1 and
// B_root = Sigma (the reference uses the same range-finder idea,
// 4D/.../Optimized/kernel.cu:419-500).
//
// Workspace: one cached device buffer per device, carved by a bump arena.
// The whole pipeline first runs as a dry run (no launches) to size it.
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/htgb.h"
#include "common.cuh"
#include "engine.h"

using namespace htgb;

namespace {

thread_local std::string g_last_error;
std::atomic<unsigned long long> g_launches{0};

ht_status_t fail(ht_status_t s, const std::string &msg) {
  g_last_error = msg;
  return s;
}

#define HT_CUDA(expr)                                                                                   \
  do {                                                                                                  \
    cudaError_t _e = (expr);                                                                            \
    if (_e != cudaSuccess)                                                                              \
      return fail(_e == cudaErrorMemoryAllocation ? HT_ERR_OUT_OF_MEMORY : HT_ERR_CUDA,                 \
                  std::string(#expr) + ": " + cudaGetErrorString(_e));                                  \
  } while (0)

#define HT_TRY(expr)            \
  do {                          \
    ht_status_t _s = (expr);    \
    if (_s != HT_OK) return _s; \
  } while (0)

// ------------------------------------------------------------ workspace cache
struct DeviceWorkspace {
  void *ptr = nullptr;
  size_t bytes = 0;
};
std::mutex g_ws_mutex;
DeviceWorkspace g_ws[64];

// Per-device host state of the single-tensor call, guarded by g_ws_mutex:
// a page-locked block that receives the call's status words in one copy (a
// pageable copy costs a full host round trip each), the timing events (made
// once, not per call), and the workspace sizes of recent call signatures (the
// dry run that sizes a call plans every launch on the host).
struct CallHostState {
  char *status = nullptr;      // cudaHostAlloc'd, kStatusBytes
  cudaEvent_t ev[10] = {};
  bool ev_made = false;
  std::vector<std::pair<std::string, size_t>> sizes;
};
CallHostState g_call[64];
constexpr size_t kStatusBytes = 352;

// Bump allocator over one device buffer.  In dry-run mode it only counts.
struct Arena {
  char *base = nullptr;
  size_t cap = 0, off = 0, peak = 0;
  bool dry = false;
  template <class T>
  T *take(size_t count) {
    const size_t bytes = (count * sizeof(T) + 255) & ~size_t(255);
    T *p = reinterpret_cast<T *>(base + off);
    off += bytes;
    peak = std::max(peak, off);
    if (dry) return reinterpret_cast<T *>(static_cast<uintptr_t>(256));   // non-null, aligned placeholder
    if (off > cap) return nullptr;
    return p;
  }
};

struct Tree {
  int order = 0, n_nodes = 0;
  int parent[HT_MAX_NODES], left[HT_MAX_NODES], right[HT_MAX_NODES], mask[HT_MAX_NODES], rank[HT_MAX_NODES];
  bool leaf(int t) const { return left[t] < 0; }
  int mode_of_leaf(int t) const {
    for (int m = 0; m < order; ++m)
      if (mask[t] == (1 << m)) return m;
    return -1;
  }
  int leaf_of_mode(int m) const {
    for (int t = 0; t < n_nodes; ++t)
      if (leaf(t) && mask[t] == (1 << m)) return t;
    return -1;
  }
};

ht_status_t parse_tree(const ht_tree_t *in, const long *dims, int order, Tree &t) {
  if (!in) return fail(HT_ERR_INVALID_ARG, "tree is NULL");
  if (order != 3 && order != 4) return fail(HT_ERR_UNSUPPORTED, "only 3rd and 4th order tensors are supported");
  if (in->order != order) return fail(HT_ERR_INVALID_ARG, "tree order does not match the tensor order");
  if (in->n_nodes != 2 * order - 1) return fail(HT_ERR_INVALID_ARG, "a binary dimension tree has 2*order-1 nodes");
  t.order = order;
  t.n_nodes = in->n_nodes;
  for (int i = 0; i < t.n_nodes; ++i) {
    t.parent[i] = in->parent[i];
    t.left[i] = in->left[i];
    t.right[i] = in->right[i];
    t.mask[i] = in->mode_mask[i];
    t.rank[i] = in->rank[i];
  }
  if (t.mask[0] != (1 << order) - 1) return fail(HT_ERR_INVALID_ARG, "node 0 must be the root holding every mode");
  if (t.parent[0] != -1) return fail(HT_ERR_INVALID_ARG, "the root has no parent");
  int leaves = 0;
  for (int i = 0; i < t.n_nodes; ++i) {
    const int l = t.left[i], r = t.right[i];
    if ((l < 0) != (r < 0)) return fail(HT_ERR_INVALID_ARG, "node " + std::to_string(i) + " needs zero or two children");
    if (l >= t.n_nodes || r >= t.n_nodes || l == 0 || r == 0 || (l >= 0 && l == r))
      return fail(HT_ERR_INVALID_ARG, "bad child index at node " + std::to_string(i));
    if (l >= 0) {
      if ((t.mask[l] | t.mask[r]) != t.mask[i] || (t.mask[l] & t.mask[r]) || !t.mask[l] || !t.mask[r])
        return fail(HT_ERR_INVALID_ARG, "children of node " + std::to_string(i) + " must partition its modes");
      if (t.parent[l] != i || t.parent[r] != i)
        return fail(HT_ERR_INVALID_ARG, "parent[] inconsistent with left[]/right[] at node " + std::to_string(i));
      if (i != 0) {
        int hi_l = -1, lo_r = 64;
        for (int m = 0; m < order; ++m) {
          if (t.mask[l] & (1 << m)) hi_l = m;
          if ((t.mask[r] & (1 << m)) && m < lo_r) lo_r = m;
        }
        if (hi_l > lo_r)
          return fail(HT_ERR_INVALID_ARG, "node " + std::to_string(i) + ": left child's modes must precede the right child's");
      }
    } else {
      if (__builtin_popcount(static_cast<unsigned>(t.mask[i])) != 1)
        return fail(HT_ERR_INVALID_ARG, "leaf " + std::to_string(i) + " must hold one mode");
      ++leaves;
    }
  }
  if (leaves != order) return fail(HT_ERR_INVALID_ARG, "tree must have one leaf per mode");
  for (int i = 0; i < order; ++i)
    if (dims[i] < 1 || dims[i] > (1l << 30)) return fail(HT_ERR_INVALID_ARG, "dims must be positive");
  long long total = 1;
  for (int i = 0; i < order; ++i) total *= dims[i];
  if (total > (1ll << 36)) return fail(HT_ERR_UNSUPPORTED, "tensor larger than 2^36 elements");
  for (int i = 1; i < t.n_nodes; ++i) {
    long long rows = 1, cols = 1;
    for (int m = 0; m < order; ++m) (t.mask[i] & (1 << m) ? rows : cols) *= dims[m];
    const int k = t.rank[i];
    if (k < 1 || k > rows || k > cols)
      return fail(HT_ERR_INVALID_ARG, "rank of node " + std::to_string(i) + " must lie in [1, min(rows, cols)]");
    if (k > 64) return fail(HT_ERR_UNSUPPORTED, "ranks above 64 are not supported");
    if (!t.leaf(i) && k > t.rank[t.left[i]] * t.rank[t.right[i]])
      return fail(HT_ERR_INVALID_ARG, "rank of node " + std::to_string(i) + " exceeds k_left * k_right");
  }
  if (order == 4) {
    const int l = t.left[0], r = t.right[0];
    if (t.leaf(l) || t.leaf(r) || t.mask[l] != 0x3 || t.mask[r] != 0xC)
      return fail(HT_ERR_UNSUPPORTED, "4th order: the root's children must be {1,2} (left) and {3,4} (right)");
  } else {
    if (t.leaf(t.left[0]) == t.leaf(t.right[0]))
      return fail(HT_ERR_INVALID_ARG, "3rd order: the root needs one leaf and one interior child");
  }
  return HT_OK;
}

struct Ctx {
  cudaStream_t st = nullptr;
  int *err = nullptr;   // device error word
  float *resid_slots = nullptr;   // per-leaf eigen residuals inside the call's status block (or null)
  Arena ar;
  int launches = 0;
  int path = 0;         // bit 0 tcgen05, bit 1 SIMT
  bool tc = false;
  int eig_ctas = 0;     // cap on the cooperative eigen-solver's grid (0 = every SM)
  // Staged enqueue of the batched path.  eig_mode 0: leaf_eigs launches the
  // cooperative solver; 1: it appends its problems to eig_table (the grouped
  // solver's entries) and launches nothing; 2: it launches nothing (the batch
  // launches the grouped solver).  Every launch belongs to a stage -- 0 before
  // the leaf solver, 1 after it, 2 the 3rd-order transfer tail, 3 the error
  // pass (4 for 3rd order) -- and only the stages in `live` launch; the arena still hands out
  // the same real pointers, so a tensor's passes agree on every buffer.
  int eig_mode = 0;
  std::vector<unsigned char> *eig_table = nullptr;
  int eig_iters_used = 0, eig_refine_used = 0;
  int stage = 0;
  unsigned live = ~0u;
  std::vector<TailJob> *tail_out = nullptr;   // grouped transfer tails (3rd order)
  std::vector<ErrJob> *err_out = nullptr;     // grouped error passes (3rd order, stage 4)
  // grouped 3rd-order core pass: the mode product (group 0) and the first
  // core contraction (group 1) as grouped FP32 GEMM tiles, the second
  // contraction as a grouped step; set by enqueue_body for a grouped batch
  bool core_grouped = false;
  int core_seq = 0;
  std::vector<SParamsBlob> *core_gemms = nullptr;
  std::vector<SimtBlockBlob> *core_blocks[2] = {nullptr, nullptr};
  std::vector<Step2Job> *step2_out = nullptr;
  std::vector<NarrowJob> *narrow_out = nullptr;   // mode products with contiguous rows of X
  std::vector<T1Job> *t1_out = nullptr;           // first core contractions
  // Batched path: the tensor's conversion (with its ||X||^2) and the copies of
  // its factors to the caller's buffers are left to one grouped launch each
  // (defer_io), described into conv_out / copy_out when those are set.
  bool defer_io = false;
  std::vector<ConvJob> *conv_out = nullptr;
  std::vector<CopySeg> *copy_out = nullptr;
  std::vector<unsigned char> *gram_out[2] = {nullptr, nullptr};   // grouped Gram items by class
  bool dry() const { return ar.dry || !((live >> stage) & 1u); }
};

View view_of_group(const long *dims, int order, int lo, int hi) {   // modes [lo, hi]
  View v{1, 1, 1};
  for (int m = 0; m < order; ++m) {
    if (m < lo) v.L *= dims[m];
    else if (m <= hi) v.N *= dims[m];
    else v.R *= dims[m];
  }
  return v;
}

// Operand whose rows are the middle index of v and whose K runs over (l, r).
Operand gram_operand(const View &v, const void *x) {
  Operand o;
  o.ptr = x;
  if (v.L == 1) {
    o.kind = OP_MN3; o.d0 = v.N; o.d1 = v.R; o.d2 = 1;
  } else {
    o.kind = OP_KM3; o.d0 = v.L; o.d1 = v.N; o.d2 = v.R;
  }
  return o;
}

int sm_count() { return device_sm_count(); }

struct GemmReq {
  Operand a32, b32;                 // FP32 operands (SIMT path)
  Operand a16, b16;                 // BF16 operands (tcgen05 path); ptr null = unavailable
  int bn_tc = 128, bn_simt = 128;
  // tile generator for a given BN (the SIMT and tcgen05 paths may use different BN)
  int tiles_kind = TILES_ROWS;
  long long t_rows = 0, t_L = 0, t_R = 0, t_n = 0;
  int t_cols = 0;
  int out_mode = OUT_COLMAJOR;
  float *out = nullptr;
  long long ld_out = 0;
  bool symmetric = false;
  bool accumulate = false;          // OUT_PARTIAL reductions add to q.out
  bool allow_split = true;
  bool fold = false;                // tcgen05 only: b16 is a high/low split (GemmArgs::fold)
  int mt_tc = 1;                    // tcgen05 only: 2 = 256-row tiles (GemmArgs::mt)
  __nv_bfloat16 *out16 = nullptr;   // column-major output wanted in BF16 here (q.out may then be scratch)
  // split-K partials into the caller's buffer with exactly force_splits
  // splits, no reduction (the caller reduces several launches' partials at once)
  float *part_ext = nullptr;
  int force_splits = 0;
};

// D = A B^T over the tiles: tcgen05 on the BF16 operands when the context
// allows it and the shapes map to TMA, else SIMT on the FP32 operands.
ht_status_t run_gemm(Ctx &c, const GemmReq &q) {
  bool use_tc = c.tc && q.a16.ptr && q.b16.ptr;
  if (use_tc) {
    GemmArgs probe;
    probe.a = q.a16; probe.b = q.b16; probe.splits = 1;
    std::string why;
    if (!tc_gemm_supported(probe, q.bn_tc, &why)) use_tc = false;
  }
  // grouped 3rd-order batch: the core pass's products are grouped FP32 GEMMs
  if (c.core_grouped && c.stage == 1) {
    if (c.core_seq > 1 || q.out_mode != OUT_COLMAJOR ||
        (q.tiles_kind != TILES_ROWS && q.tiles_kind != TILES_SLABS))
      return fail(HT_ERR_UNSUPPORTED, "grouped core pass: unexpected product");
    const int seq = c.core_seq++;
    if (!c.core_gemms || c.ar.dry) return HT_OK;
    if (seq == 0 && q.a32.kind == OP_MN3 && q.a32.d0 >= 32 && q.b32.kind == OP_KM3 && q.t_cols <= 64 &&
        q.ld_out == q.a32.d0 * q.a32.d2) {   // Z = X_(t) V, a thread per row of X
      NarrowJob j;
      j.X = static_cast<const float *>(q.a32.ptr); j.V = static_cast<const float *>(q.b32.ptr); j.Z = q.out;
      j.L = q.a32.d0; j.R = q.a32.d2; j.N = static_cast<int>(q.a32.d1); j.kz = q.t_cols;
      j.blk0 = 0;
      j.nblk = static_cast<int>(std::min<long long>(32, (j.L * j.R + 255) / 256));
      c.narrow_out->push_back(j);
      return HT_OK;
    }
    if (seq == 1 && q.a32.kind == OP_KM3 && q.b32.kind == OP_KM3 && q.a32.d2 == 1 && q.t_cols <= 64 &&
        q.ld_out == q.a32.d1 && q.tiles_kind == TILES_ROWS) {   // T1 = Z-rows x Up
      T1Job j;
      j.Z = static_cast<const float *>(q.a32.ptr); j.Up = static_cast<const float *>(q.b32.ptr); j.T1 = q.out;
      j.rows = q.a32.d1; j.np = static_cast<int>(q.a32.d0); j.kp = q.t_cols;
      j.blk0 = 0;
      j.nblk = static_cast<int>(std::min<long long>(16, (j.rows + 63) / 64));
      c.t1_out->push_back(j);
      return HT_OK;
    }
    {
      GemmArgs g;
      g.a = q.a32;
      g.b = q.b32;
      g.gen = q.tiles_kind == TILES_ROWS ? make_rows_gen(q.t_rows, q.t_cols, 64) : make_slabs_gen(q.t_L, q.t_R, q.t_cols, 64);
      g.num_tiles = g.gen.count;
      g.splits = 1;
      g.out_mode = OUT_COLMAJOR;
      g.out = q.out;
      g.ld_out = q.ld_out;
      g.err = c.err;
      g.fold = 0;
      g.out16 = nullptr;
      g.mt = 1;
      if (!simt_grouped_add(g, *c.core_gemms, *c.core_blocks[seq]))
        return fail(HT_ERR_UNSUPPORTED, "grouped core pass: product not groupable");
    }
    return HT_OK;
  }
  // grouped batch (eig_mode != 0): a leaf Gram of a mode of at most 256 is one
  // item of the batch's grouped Gram launch -- described by the plan pass,
  // launched by the batch, never launched here
  const int gcls = tc_gram_class(q.t_n);
  if (c.eig_mode != 0 && use_tc && q.tiles_kind == TILES_GRAM && q.a16.ptr == q.b16.ptr && !q.accumulate &&
      !q.part_ext && gcls >= 0) {
    if (c.gram_out[gcls] && !c.ar.dry) {
      std::string why;
      if (!tc_gram_item(q.a16, q.t_n, q.out, c.err, *c.gram_out[gcls], &why))
        return fail(HT_ERR_CUDA, "grouped Gram item: " + why);
    }
    return HT_OK;
  }
  const int bn = use_tc ? q.bn_tc : q.bn_simt;
  const int mt = use_tc ? q.mt_tc : 1;
  TileGen gen;
  if (q.tiles_kind == TILES_ROWS) gen = make_rows_gen(q.t_rows, q.t_cols, bn);
  else if (q.tiles_kind == TILES_SLABS) gen = make_slabs_gen(q.t_L, q.t_R, q.t_cols, bn);
  else if (q.tiles_kind == TILES_GRID) {
    if (!make_grid_gen(q.t_rows, q.t_n, bn, &gen)) return fail(HT_ERR_UNSUPPORTED, "product too large for one grid");
  } else if (!make_gram_gen(q.t_n, bn, &gen, 128 * mt)) return fail(HT_ERR_UNSUPPORTED, "Gram larger than 32768");
  const int nt = gen.count;
  int splits = 1;
  if (q.allow_split && nt < sm_count()) splits = std::max(1, sm_count() / nt);
  if (q.force_splits > 0) {
    splits = q.force_splits;
  } else if (use_tc) {
    const long nkb = tc_num_kblocks(q.a16);
    long per = (nkb + splits - 1) / splits;
    per = std::max<long>(per, std::min<long>(nkb, 16));   // keep the smem pipeline busy
    splits = static_cast<int>((nkb + per - 1) / per);
  } else {
    const long kt = simt_k_total(q.a32);
    long per = (kt + splits - 1) / splits;
    per = std::max<long>((per + 15) / 16 * 16, 256);
    splits = static_cast<int>(std::max<long>(1, (kt + per - 1) / per));
  }
  const bool partial = splits > 1 || q.out_mode == OUT_PARTIAL;
  const size_t mark = c.ar.off;
  float *part = q.part_ext ? q.part_ext
                           : (partial ? c.ar.take<float>(static_cast<size_t>(splits) * nt * gen.bm * bn) : nullptr);
  if (c.dry()) {
    c.ar.off = mark;
    return HT_OK;
  }
  if (partial && !part) return fail(HT_ERR_OUT_OF_MEMORY, "workspace too small (gemm scratch)");
  GemmArgs g;
  g.a = use_tc ? q.a16 : q.a32;
  g.b = use_tc ? q.b16 : q.b32;
  g.gen = gen;
  g.num_tiles = nt;
  g.splits = splits;
  g.out_mode = partial ? OUT_PARTIAL : OUT_COLMAJOR;
  g.out = partial ? part : q.out;
  g.ld_out = q.ld_out;
  g.err = c.err;
  g.fold = (use_tc && q.fold) ? 1 : 0;
  g.mt = mt;
  // a BF16 column-major output comes straight from the tcgen05 epilogue, else
  // from the FP32 result converted afterwards
  const bool direct16 = q.out16 && use_tc && !partial;
  g.out16 = direct16 ? q.out16 : nullptr;
  if (use_tc) {
    HT_CUDA(tc_gemm_launch(g, bn, c.st));
    c.path |= 1;
  } else {
    HT_CUDA(simt_gemm_launch(g, bn, c.st));
    c.path |= 2;
  }
  ++c.launches;
  if (partial && !q.part_ext) {
    HT_CUDA(reduce_partials_launch(part, gen, splits, bn, q.out, q.ld_out,
                                   (q.symmetric ? 1 : 0) | (q.accumulate ? 2 : 0), c.st));
    ++c.launches;
  }
  if (q.out16 && !direct16) {   // rows x cols column-major, ld = rows
    HT_CUDA(f32_to_bf16_launch(q.out, q.out16, q.ld_out * q.t_cols, c.st));
    ++c.launches;
  }
  c.ar.off = mark;   // scratch is stream-ordered: later work may reuse it
  return HT_OK;
}

// tcgen05 tile of an n x n Gram: 256 x 256 (two M = 128 accumulators) from n = 256 up
int gram_bn_tc(long n) { return n >= 256 ? 256 : (n > 64 ? 128 : 64); }
int gram_mt_tc(long n) { return n >= 256 ? 2 : 1; }

// G (n x n, column-major, symmetric) = X_(group) X_(group)^T, n = v.N
// (accumulate: G += X_(group) X_(group)^T).  part_ext: leave the split-K
// partials (force_splits of them) in that buffer unreduced.
ht_status_t gram(Ctx &c, const View &v, const float *x32, const __nv_bfloat16 *x16, float *G,
                 bool accumulate = false, float *part_ext = nullptr, int force_splits = 0) {
  GemmReq q;
  q.a32 = q.b32 = gram_operand(v, x32);
  if (x16) q.a16 = q.b16 = gram_operand(v, x16);
  else q.a16.ptr = q.b16.ptr = nullptr;
  q.part_ext = part_ext;
  q.force_splits = force_splits;
  q.bn_tc = gram_bn_tc(v.N);
  q.mt_tc = gram_mt_tc(v.N);   // 256 x 256 tiles, diagonal ones loading a single panel
  q.bn_simt = v.N > 64 ? 128 : 64;
  q.tiles_kind = TILES_GRAM;
  q.t_n = v.N;
  q.out_mode = OUT_PARTIAL;
  q.out = G;
  q.ld_out = v.N;
  q.symmetric = true;
  q.accumulate = accumulate;
  return run_gemm(c, q);
}

// The Gram of view v (FP32 operands from x32) with its BF16 operands read from
// the first-mode-padded copy x16p, whose view of the same mode group is vp
// (vp.N = n1p for the first mode; rows beyond v.N are zero and clipped).
ht_status_t gram_padded(Ctx &c, const View &v, const View &vp, const float *x32, const __nv_bfloat16 *x16p,
                        float *G) {
  GemmReq q;
  q.a32 = q.b32 = gram_operand(v, x32);
  q.a16 = q.b16 = gram_operand(vp, x16p);
  q.bn_tc = gram_bn_tc(v.N);
  q.mt_tc = gram_mt_tc(v.N);
  q.bn_simt = v.N > 64 ? 128 : 64;
  q.tiles_kind = TILES_GRAM;
  q.t_n = v.N;
  q.out_mode = OUT_PARTIAL;
  q.out = G;
  q.ld_out = v.N;
  q.symmetric = true;
  return run_gemm(c, q);
}

// l-block exponent of the last mode's second BF16 copy (0: no copy).
int last_mode_block(const long *dims, int order) {
  if (order != 3) return 0;
  const long long N = dims[2], L = static_cast<long long>(dims[0]) * dims[1];
  if (N < 256 || L < 65536) return 0;
  if (N % 16 == 0 && L % 256 == 0) return 8;   // 256-element l-blocks: 512-byte rows, 16-column tiles
  if (N % 64 == 0 && L % 64 == 0) return 6;    // 64-element l-blocks: 128-byte rows, 64-column tiles
  return 0;
}

// Gram of the last mode (v.R == 1) from the l-blocked BF16 copy x16t
// (x16t[((l/B) N + n) B + l%B], B = 2^lb): a K-major operand whose rows are 2B
// bytes apart.  Read in place, the last mode's K-major rows are 2L bytes apart,
// so every 256-row TMA box touches 256 different 2 MiB pages; at 1024^3 that
// Gram read X three times from DRAM and ran at half the speed of the other two.
ht_status_t gram_transposed(Ctx &c, const View &v, const float *x32, const __nv_bfloat16 *x16t, int lb, float *G) {
  GemmReq q;
  q.a32 = q.b32 = gram_operand(v, x32);
  Operand o;
  o.kind = OP_KM3; o.ptr = x16t; o.d0 = 1l << lb; o.d1 = v.N; o.d2 = v.L >> lb;
  q.a16 = q.b16 = o;
  q.bn_tc = v.N >= 256 ? 256 : (v.N > 64 ? 128 : 64);
  q.mt_tc = v.N >= 256 ? 2 : 1;
  q.bn_simt = v.N > 64 ? 128 : 64;
  q.tiles_kind = TILES_GRAM;
  q.t_n = v.N;
  q.out_mode = OUT_PARTIAL;
  q.out = G;
  q.ld_out = v.N;
  q.symmetric = true;
  return run_gemm(c, q);
}

// Z ((L*R) x k, column-major) = contraction of the middle index of view v with W (v.N x k)
// fold_h > 0: W16 is the split_bf16 form of W32 (v.N x 2*fold_h, high part in
// columns [0, k), low part in [fold_h, fold_h + k)), so the tcgen05 product
// carries W to about 16 significant bits instead of BF16's 8.
// Z16 non-null: the product is wanted in BF16 there (Z is then FP32 scratch).
ht_status_t mode_product(Ctx &c, const View &v, const float *x32, const __nv_bfloat16 *x16, const float *W32,
                         const __nv_bfloat16 *W16, int k, float *Z, int fold_h = 0, __nv_bfloat16 *Z16 = nullptr) {
  GemmReq q;
  auto opA = [&](const void *x) {
    Operand o;
    o.ptr = x;
    if (v.L == 1) {
      o.kind = OP_KM3; o.d0 = v.N; o.d1 = v.R; o.d2 = 1;
    } else {
      o.kind = OP_MN3; o.d0 = v.L; o.d1 = v.N; o.d2 = v.R;
    }
    return o;
  };
  auto opB = [&](const void *w, int cols) {
    Operand o;
    o.ptr = w; o.kind = OP_KM3; o.d0 = v.N; o.d1 = cols; o.d2 = 1;
    return o;
  };
  q.a32 = opA(x32); q.b32 = opB(W32, k);
  if (x16 && W16) { q.a16 = opA(x16); q.b16 = opB(W16, fold_h > 0 ? 2 * fold_h : k); }
  else q.a16.ptr = q.b16.ptr = nullptr;
  q.bn_tc = fold_h > 0 ? 2 * fold_h : 64; q.bn_simt = k <= 32 ? 32 : 64;
  q.fold = fold_h > 0;
  if (v.L == 1) {
    q.tiles_kind = TILES_ROWS; q.t_rows = v.R; q.t_cols = k;
  } else {
    q.tiles_kind = TILES_SLABS; q.t_L = v.L; q.t_R = v.R; q.t_cols = k;
  }
  q.out_mode = OUT_COLMAJOR;
  q.out = Z;
  q.out16 = Z16;
  q.ld_out = v.L * v.R;
  return run_gemm(c, q);
}

// Z (v.N x k, column-major) = X_(group) Q with Q ((L*R) x k): contract every index but the middle one
// a16: optional BF16 A operand in place of X_(group) read from x16 (the
// l-blocked copy of the last mode, see gram_transposed)
ht_status_t corange_product(Ctx &c, const View &v, const float *x32, const __nv_bfloat16 *x16, const float *Q32,
                            const __nv_bfloat16 *Q16, int k, float *Z, const Operand *a16 = nullptr) {
  GemmReq q;
  auto opB = [&](const void *p) {
    Operand o;
    o.ptr = p;
    if (v.L == 1) {
      o.kind = OP_KM3; o.d0 = v.R; o.d1 = k; o.d2 = 1;
    } else {
      o.kind = OP_KM3Q; o.d0 = v.L; o.d1 = v.R; o.d2 = k;
    }
    return o;
  };
  q.a32 = gram_operand(v, x32); q.b32 = opB(Q32);
  if ((x16 || a16) && Q16) { q.a16 = a16 ? *a16 : gram_operand(v, x16); q.b16 = opB(Q16); }
  else q.a16.ptr = q.b16.ptr = nullptr;
  q.bn_tc = 64; q.bn_simt = k <= 32 ? 32 : 64;
  q.tiles_kind = TILES_ROWS; q.t_rows = v.N; q.t_cols = k;
  q.out_mode = OUT_COLMAJOR;
  q.out = Z;
  q.ld_out = v.N;
  return run_gemm(c, q);
}

// C[a + kp*b + kp*kq*u] = sum_{i,j} Up[i,a] Uq[j,b] Z[i + np*j, u]   (FP32)
ht_status_t core_contract(Ctx &c, const float *Z, int np, int nq, int ku, const float *Up, int kp, const float *Uq,
                          int kq, float *C) {
  const size_t mark = c.ar.off;
  const long long rows = static_cast<long long>(nq) * ku;
  float *T1 = c.ar.take<float>(static_cast<size_t>(rows) * kp);
  const int ranges = c.core_grouped ? 1 : core_step2_ranges(nq, ku);
  float *parts = ranges > 1 ? c.ar.take<float>(static_cast<size_t>(ranges) * kp * kq * ku) : nullptr;
  if (!T1 || (ranges > 1 && !parts)) return fail(HT_ERR_OUT_OF_MEMORY, "workspace too small (core)");
  // T1[(j + nq*u) + rows*a] = sum_i Z[i + np*(j + nq*u)] Up[i + np*a]
  GemmReq q;
  q.a32.kind = OP_KM3; q.a32.ptr = Z; q.a32.d0 = np; q.a32.d1 = rows; q.a32.d2 = 1;
  q.b32.kind = OP_KM3; q.b32.ptr = Up; q.b32.d0 = np; q.b32.d1 = kp; q.b32.d2 = 1;
  q.a16.ptr = q.b16.ptr = nullptr;
  q.bn_simt = kp <= 32 ? 32 : 64;
  q.tiles_kind = TILES_ROWS; q.t_rows = rows; q.t_cols = kp;
  q.out_mode = OUT_COLMAJOR;
  q.out = T1;
  q.ld_out = rows;
  HT_TRY(run_gemm(c, q));
  // grouped: the batch's step reads T1 later; its memory, released below, is
  // only written again by this tensor's error pass, which runs after the step
  if (c.core_grouped) {
    if (c.step2_out && !c.ar.dry) c.step2_out->push_back(Step2Job{T1, Uq, C, rows, nq, kp, kq, ku, 0, 0});
  } else if (!c.dry()) {
    HT_CUDA(core_step2_launch(T1, rows, nq, kp, Uq, kq, ku, C, parts, c.st));
    c.launches += ranges > 1 ? 2 : 1;
  }
  c.ar.off = mark;
  return HT_OK;
}

bool is_device_ptr(const void *p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

int g_dev_ok[64];   // 0 unknown, 1 sm_103, -1 other
ht_status_t check_device() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return fail(HT_ERR_NO_DEVICE, "no CUDA device");
  }
  if (dev >= 0 && dev < 64 && g_dev_ok[dev] == 1) return HT_OK;
  int major = 0, minor = 0;
  if (cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev) != cudaSuccess) {
    cudaGetLastError();
    return fail(HT_ERR_NO_DEVICE, "cannot query the CUDA device");
  }
  if (!(major == 10 && minor == 3))
    return fail(HT_ERR_NO_DEVICE, "the library is compiled for sm_103a (GB300); device is sm_" + std::to_string(major) +
                                      std::to_string(minor));
  if (dev >= 0 && dev < 64) g_dev_ok[dev] = 1;
  return HT_OK;
}

ht_status_t acquire_workspace(size_t bytes, void **ptr, cudaStream_t st) {
  int dev = 0;
  HT_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(HT_ERR_INVALID_ARG, "device index out of range");
  DeviceWorkspace &w = g_ws[dev];
  if (w.bytes < bytes) {
    if (w.ptr) {
      HT_CUDA(cudaStreamSynchronize(st));
      HT_CUDA(cudaDeviceSynchronize());
      HT_CUDA(cudaFree(w.ptr));
      w.ptr = nullptr;
      w.bytes = 0;
    }
    HT_CUDA(cudaMalloc(&w.ptr, bytes));
    w.bytes = bytes;
  }
  *ptr = w.ptr;
  return HT_OK;
}

// ----------------------------------------------------------------- pipeline
struct Plan3 {
  int t, c, p, q;           // interior root child, complementary leaf, t's children
  int mc, mp, mq;           // modes of c, p, q
  int kt, kc, kp, kq, kw;   // kw = max(kc, kt)
  bool t_is_left;
};

Plan3 plan3(const Tree &T) {
  Plan3 P;
  const int l = T.left[0], r = T.right[0];
  P.t_is_left = !T.leaf(l);
  P.t = P.t_is_left ? l : r;
  P.c = P.t_is_left ? r : l;
  P.p = T.left[P.t];
  P.q = T.right[P.t];
  P.mc = T.mode_of_leaf(P.c);
  P.mp = T.mode_of_leaf(P.p);
  P.mq = T.mode_of_leaf(P.q);
  P.kt = T.rank[P.t]; P.kc = T.rank[P.c]; P.kp = T.rank[P.p]; P.kq = T.rank[P.q];
  P.kw = std::max(P.kc, P.kt);
  return P;
}

// Device-resident results of one decomposition (workspace pointers).
struct Result {
  const float *U[HT_MAX_NODES] = {};   // leaves: n_t x k_t (leading columns of the Ritz block)
  const float *B[HT_MAX_NODES] = {};   // interior nodes and root
  const float *resid[HT_MAX_NODES] = {};
};

struct Timeline {
  cudaEvent_t ev[8];
  int n = 0;
  bool on = false;
  void mark(cudaStream_t s) {
    if (on && n < 8) cudaEventRecord(ev[n++], s);
  }
};

// 2. top-K eigenvectors of every leaf Gram G[m], one batched launch; the leaf
// bases land in res.U (arena memory taken here).
ht_status_t leaf_eigs(Ctx &c, const Tree &T, const ht_config_t &cfg, const long *dims, int order, float *const *G,
                      EigProblem *ep, Result &res) {
  const int p_over = cfg.oversample > 0 ? cfg.oversample : 16;
  // eig_iters 0: ten iterations on the FP32 path, six on the mixed path, whose
  // BF16 Gram error is well above what the last four iterations change (at
  // 1024^3 on the r^-1.5 family: 3e-7 of relative error against 7e-6 from BF16)
  const int iters = cfg.eig_iters > 0 ? cfg.eig_iters : (cfg.precision == HT_PREC_BF16 ? 6 : 10);
  const bool d3 = order == 3;
  Plan3 P3{};
  if (d3) P3 = plan3(T);
  for (int m = 0; m < order; ++m) {
    const int leaf = T.leaf_of_mode(m);
    const int K = (d3 && leaf == P3.c) ? P3.kw : T.rank[leaf];
    const int n = static_cast<int>(dims[m]);
    // s = k + oversampling (at most 64); a mode no larger than that is the
    // whole block, and the eigen-solver reduces to a Jacobi eigen-decomposition
    // of the Gram itself.  A mode of at most 64 above s takes whichever of the
    // two is cheaper by a cost model (µs, one CTA) from measured costs: a Jacobi
    // round on an m x m matrix ~0.85 (m / 64)^2 and ~10 sweeps of m - 1 rounds
    // (~2e-3 m^3; 535 µs at m = 64, 172 at 48), against per iteration a fixed
    // ~10 µs of barriers and pivots, the float-pair factor (~2.5e-4 s^3) and the
    // product (~2e-5 n^2 s), plus the Rayleigh-Ritz Jacobi on s x s.
    int s = std::max(K, std::min<int>({static_cast<int>(n), K + p_over, 64}));
    if (s < n && n <= 64) {
      const double direct = 2e-3 * n * n * n;
      const double iterate = iters * (10.0 + 2.5e-4 * s * s * s + 2e-5 * n * n * s) + 2e-3 * s * s * s;
      if (direct <= iterate) s = static_cast<int>(n);
    }
    if (s > 64) return fail(HT_ERR_UNSUPPORTED, "subspace size above 64");
    EigProblem &e = ep[m];
    e.G = G[m]; e.n = n; e.s = s; e.K = K;
    e.Q = c.ar.take<float>(static_cast<size_t>(n) * s);
    e.Y = c.ar.take<float>(static_cast<size_t>(n) * s);
    e.U = c.ar.take<float>(static_cast<size_t>(n) * K);
    e.GU = c.ar.take<float>(static_cast<size_t>(n) * K);
    e.theta = c.ar.take<float>(64);
    e.resid = c.resid_slots ? c.resid_slots + leaf : c.ar.take<float>(4);
    e.seed = cfg.seed;
    e.stream_id = static_cast<uint64_t>(m);
    e.start = nullptr;
    if (cfg.sketch[m]) {
      if (is_device_ptr(cfg.sketch[m])) {
        e.start = cfg.sketch[m];
      } else {
        float *d = c.ar.take<float>(static_cast<size_t>(n) * s);
        if (!d) return fail(HT_ERR_OUT_OF_MEMORY, "workspace too small (start block)");
        if (!c.dry()) HT_CUDA(cudaMemcpyAsync(d, cfg.sketch[m], sizeof(float) * n * s, cudaMemcpyHostToDevice, c.st));
        e.start = d;
      }
    }
    if (!e.Q || !e.Y || !e.U || !e.GU) return fail(HT_ERR_OUT_OF_MEMORY, "workspace too small (eig)");
    res.U[leaf] = e.U;
    res.resid[leaf] = e.resid;
  }
  {
    const size_t mark = c.ar.off;
    const size_t eb = c.eig_mode ? eig_grouped_workspace_bytes(ep, order) : eig_workspace_bytes(ep, order);
    void *ews = c.ar.take<char>(eb);
    if (!ews) return fail(HT_ERR_OUT_OF_MEMORY, "workspace too small (eig)");
    // the FP32 path keeps two CholeskyQR refinement passes (its error sits at
    // FP32 rounding, where the last pass still moves it); the mixed path's
    // BF16 Gram error is four orders above what they change once the block has
    // converged.  With few iterations, or a caller's start block, the last
    // block need not be: Y = G S is rank deficient whenever the Gram's rank is
    // below s (the separable-bumps family: rank <= 32 < 34), and one shifted
    // CholeskyQR of it leaves noise columns that are not orthogonal to the
    // rest.  Those paths refine on both precisions.
    bool sketched = false;
    for (int m = 0; m < order; ++m) sketched = sketched || cfg.sketch[m] != nullptr;
    const int refine = (cfg.precision == HT_PREC_FP32 || iters < 4 || sketched) ? 2 : 0;
    c.stage = 1;
    c.eig_iters_used = iters;
    c.eig_refine_used = refine;
    if (c.eig_mode == 1 && !c.ar.dry) HT_CUDA(eig_grouped_fill(ep, order, ews, eb, *c.eig_table));
    if (c.eig_mode == 0 && !c.dry()) HT_CUDA(eig_batched(ep, order, iters, ews, eb, c.err, c.st, &c.launches, c.eig_ctas, refine));
    c.ar.off = mark;
  }
  return HT_OK;
}

// 2'. Leaf bases without the mode Grams (HT_LEAF_SKETCH): a randomized range
// finder on X_(m) whose test matrix is Omega = X_(m)^T Q for a per-mode block
// Q (n_m x s, s = k + oversample): the caller's sketch[m] or a Gaussian one.
// Each application Y = G Q = X_(m) (X_(m)^T Q) is two streaming products
// over the tensor (mode product, then co-range product); G is never formed.
//   Q = orth(S);  power_steps times: Q = orth(G Q);  Y = G Q
// and the leaf basis is Q1 times the top-k eigenvectors of the Nystrom core
// H = R1 (Q^T Y + nu I)^-1 R1^T, Y + nu Q = Q1 R1 (sketch.cu).  Orthonormal
// blocks come from the eigen-solver's cooperative CholeskyQR2 (float-pair
// factor).  The reference's range finder (rsvd, 3D/Opt/kernel.cu:595-680)
// draws a Gaussian Omega for X_(12) and SVDs the projected B = Q^T A; no
// residual is reported on this path (there is no Gram to measure it on).
constexpr float kNystromShift = 1e-7f;   // nu / tr(Q^T G Q)

ht_status_t leaf_sketch(Ctx &c, const Tree &T, const ht_config_t &cfg, const long *dims, int order,
                        const float *x32, const __nv_bfloat16 *x16, const __nv_bfloat16 *x16t, int lb,
                        EigProblem *ep, Result &res) {
  const int p_over = cfg.oversample > 0 ? cfg.oversample : 16;
  const int qsteps = cfg.power_steps >= 0 ? cfg.power_steps : 1;
  const bool d3 = order == 3;
  Plan3 P3{};
  if (d3) P3 = plan3(T);
  int K[4], S[4];
  long long LRmax = 0, nmax = 0;
  int smax = 1;
  for (int m = 0; m < order; ++m) {
    const int leaf = T.leaf_of_mode(m);
    K[m] = (d3 && leaf == P3.c) ? P3.kw : T.rank[leaf];
    const int n = static_cast<int>(dims[m]);
    S[m] = std::max(K[m], std::min({n, K[m] + p_over, 64}));
    if (S[m] > 64) return fail(HT_ERR_UNSUPPORTED, "sketch width above 64");
    const View v = view_of_group(dims, order, m, m);
    LRmax = std::max(LRmax, static_cast<long long>(v.L * v.R));
    nmax = std::max(nmax, static_cast<long long>(n));
    smax = std::max(smax, S[m]);
  }
  // results (kept): U per leaf; work (released at the end)
  for (int m = 0; m < order; ++m) {
    const int leaf = T.leaf_of_mode(m);
    EigProblem &e = ep[m];
    e = EigProblem{};
    e.n = static_cast<int>(dims[m]); e.s = S[m]; e.K = K[m];
    e.U = c.ar.take<float>(static_cast<size_t>(e.n) * K[m]);
    if (!e.U) return fail(HT_ERR_OUT_OF_MEMORY, "workspace too small (sketch bases)");
    res.U[leaf] = e.U;
    res.resid[leaf] = nullptr;
  }
  const size_t mark = c.ar.off;
  float *Z32 = c.ar.take<float>(static_cast<size_t>(LRmax) * smax);
  __nv_bfloat16 *Z16 = c.tc ? c.ar.take<__nv_bfloat16>(static_cast<size_t>(LRmax) * smax + 64) : nullptr;
  __nv_bfloat16 *Q16 = c.tc ? c.ar.take<__nv_bfloat16>(static_cast<size_t>(nmax) * smax + 64) : nullptr;
  if (!Z32 || (c.tc && (!Z16 || !Q16))) return fail(HT_ERR_OUT_OF_MEMORY, "workspace too small (sketch products)");
  float *Qm[4], *Ym[4], *Q1[4], *Wm[4], *R1[4], *Hm[4], *Tm[4], *M2[4], *Br[4];
  for (int m = 0; m < order; ++m) {
    const size_t ns = static_cast<size_t>(dims[m]) * S[m], ss = static_cast<size_t>(S[m]) * S[m];
    Qm[m] = c.ar.take<float>(ns);
    Ym[m] = c.ar.take<float>(ns);
    Q1[m] = c.ar.take<float>(ns);
    Wm[m] = c.ar.take<float>(ss);
    R1[m] = c.ar.take<float>(ss);
    Hm[m] = c.ar.take<float>(ss);
    Tm[m] = c.ar.take<float>(static_cast<size_t>(S[m]) * K[m]);
    M2[m] = c.ar.take<float>(static_cast<size_t>(S[m]) * K[m]);
    Br[m] = c.ar.take<float>(static_cast<size_t>(K[m]) * K[m]);
    if (!Qm[m] || !Ym[m] || !Q1[m] || !Wm[m] || !R1[m] || !Hm[m] || !Tm[m] || !M2[m] || !Br[m])
      return fail(HT_ERR_OUT_OF_MEMORY, "workspace too small (sketch)");
  }
  EigProblem cq[4];
  for (int m = 0; m < order; ++m) {
    cq[m] = EigProblem{};
    cq[m].n = static_cast<int>(dims[m]); cq[m].s = S[m]; cq[m].K = S[m];
  }
  const size_t cbytes = eig_workspace_bytes(cq, order);
  void *cws = c.ar.take<char>(cbytes);
  if (!cws) return fail(HT_ERR_OUT_OF_MEMORY, "workspace too small (sketch CholeskyQR)");
  auto orth_all = [&](float *const *M) -> ht_status_t {   // CholeskyQR2 of every mode's block, one launch
    for (int m = 0; m < order; ++m) {
      cq[m].Q = M[m];
      cq[m].G = nullptr; cq[m].Y = cq[m].U = cq[m].GU = cq[m].theta = cq[m].resid = nullptr;
      cq[m].start = nullptr;
    }
    HT_CUDA(cholqr_batched(cq, order, 2, cws, cbytes, c.err, c.st, &c.launches));
    return HT_OK;
  };
  // Y = G Q for mode m, as X_(m) (X_(m)^T Q).  On the mixed path Q is first
  // rounded to BF16 in place, so the products see exactly the block that the
  // Nystrom core later pairs with Y (any block serves as a test matrix).
  auto apply_gram = [&](int m, float *Qsrc, float *Ydst) -> ht_status_t {
    const View v = view_of_group(dims, order, m, m);
    const int s = S[m];
    if (c.tc && !c.dry()) {
      HT_CUDA(round_bf16_launch(Qsrc, Q16, dims[m] * s, c.st));
      ++c.launches;
    }
    HT_TRY(mode_product(c, v, x32, x16, Qsrc, Q16, s, Z32, 0, c.tc ? Z16 : nullptr));
    if (c.tc && m == order - 1 && x16t) {
      Operand o;
      o.kind = OP_KM3; o.ptr = x16t; o.d0 = 1l << lb; o.d1 = v.N; o.d2 = v.L >> lb;
      return corange_product(c, v, x32, x16, Z32, Z16, s, Ydst, &o);
    }
    return corange_product(c, v, x32, x16, Z32, Z16, s, Ydst);
  };
  if (c.dry()) {   // size the products' split-K scratch
    for (int m = 0; m < order; ++m) HT_TRY(apply_gram(m, Qm[m], Ym[m]));
    c.ar.off = mark;
    return HT_OK;
  }
  // start blocks
  for (int m = 0; m < order; ++m) {
    const size_t ns = static_cast<size_t>(dims[m]) * S[m];
    if (cfg.sketch[m]) {
      HT_CUDA(cudaMemcpyAsync(Qm[m], cfg.sketch[m], sizeof(float) * ns, cudaMemcpyDefault, c.st));
    } else {
      HT_CUDA(gaussian_fill_launch(Qm[m], static_cast<long long>(ns), cfg.seed, 200 + m, c.st));
      ++c.launches;
    }
  }
  HT_TRY(orth_all(Qm));
  for (int it = 0; it < qsteps; ++it) {
    for (int m = 0; m < order; ++m) HT_TRY(apply_gram(m, Qm[m], Ym[m]));
    for (int m = 0; m < order; ++m) std::swap(Qm[m], Ym[m]);
    HT_TRY(orth_all(Qm));
  }
  for (int m = 0; m < order; ++m) HT_TRY(apply_gram(m, Qm[m], Ym[m]));
  // Nystrom: W = Q^T Y, Y_nu = Y + nu Q -> Q1 R1, H = R1 (W + nu I)^-1 R1^T, U = Q1 * top-K(H)
  for (int m = 0; m < order; ++m) {
    const int n = static_cast<int>(dims[m]), s = S[m];
    HT_CUDA(gemm_tn_small_launch(Qm[m], n, Ym[m], n, Wm[m], s, s, s, n, c.st));
    HT_CUDA(nystrom_shift_launch(Ym[m], Qm[m], n, s, Wm[m], kNystromShift, Q1[m], c.st));
    HT_CUDA(cudaMemcpyAsync(Ym[m], Q1[m], sizeof(float) * n * s, cudaMemcpyDeviceToDevice, c.st));   // Y_nu
    c.launches += 2;
  }
  HT_TRY(orth_all(Q1));
  NystromProb np_[4];
  SvdGramProb sp[4];
  for (int m = 0; m < order; ++m) {
    const int n = static_cast<int>(dims[m]), s = S[m];
    HT_CUDA(gemm_tn_small_launch(Q1[m], n, Ym[m], n, R1[m], s, s, s, n, c.st));
    ++c.launches;
    np_[m] = NystromProb{Wm[m], R1[m], s, Hm[m]};
    sp[m] = SvdGramProb{Hm[m], s, K[m], K[m], Tm[m], M2[m], Br[m]};
  }
  HT_CUDA(nystrom_core_launch(np_, order, kNystromShift, c.err, c.st));       // all modes, a CTA each
  HT_CUDA(svd_from_gram_batched_launch(sp, order, c.st));                     // top-K eigenvectors of each H
  c.launches += 2;
  for (int m = 0; m < order; ++m) {
    const int n = static_cast<int>(dims[m]), s = S[m];
    HT_CUDA(matmul_nn_launch(Q1[m], n, Tm[m], s, ep[m].U, n, n, K[m], s, c.st));
    ++c.launches;
  }
  c.ar.off = mark;
  return HT_OK;
}

// Buffers of the 3rd-order transfer step (taken before the core pass's scratch).
struct Transfer3 {
  float *C, *WG, *M, *Bkt, *Broot, *Bt;
};

ht_status_t take_transfer3(Ctx &c, const Plan3 &P, Transfer3 &tr) {
  tr.C = c.ar.take<float>(static_cast<size_t>(P.kp) * P.kq * P.kt);
  tr.WG = c.ar.take<float>(static_cast<size_t>(P.kw) * P.kw);
  tr.M = c.ar.take<float>(static_cast<size_t>(P.kt) * P.kt);
  tr.Bkt = c.ar.take<float>(static_cast<size_t>(P.kt) * P.kc);
  tr.Broot = c.ar.take<float>(static_cast<size_t>(P.kt) * P.kc);
  tr.Bt = c.ar.take<float>(static_cast<size_t>(P.kp) * P.kq * P.kt);
  if (!tr.C || !tr.WG || !tr.M || !tr.Bkt || !tr.Broot || !tr.Bt)
    return fail(HT_ERR_OUT_OF_MEMORY, "workspace too small (transfer)");
  return HT_OK;
}

// 4. transfer tensors from the core-pass product Z = X_(t) V (3rd order).
// WG_ready: W^T G_c W is already in tr.WG (the sketch path's TSQR of Z).
ht_status_t transfer3_from_z(Ctx &c, const Plan3 &P, const long *dims, const EigProblem *ep, const float *Z,
                             const Transfer3 &tr, Result &res, bool WG_ready = false) {
  const EigProblem &ec = ep[P.mc];
  HT_TRY(core_contract(c, Z, static_cast<int>(dims[P.mp]), static_cast<int>(dims[P.mq]), P.kt, ep[P.mp].U, P.kp,
                       ep[P.mq].U, P.kq, tr.C));
  const int stage_before = c.stage;
  c.stage = 2;
  if (c.tail_out && !c.ar.dry && !WG_ready) {
    TailJob j;
    j.U = ec.U; j.GU = ec.GU; j.C = tr.C;
    j.M = tr.M; j.Bkt = tr.Bkt; j.Broot = tr.Broot; j.Bt = tr.Bt;
    j.kpq = static_cast<long long>(P.kp) * P.kq;
    j.nc = static_cast<int>(dims[P.mc]); j.kw = P.kw; j.kt = P.kt; j.kc = P.kc; j.t_is_left = P.t_is_left ? 1 : 0;
    c.tail_out->push_back(j);
  }
  if (!c.dry()) {
    const int nc = static_cast<int>(dims[P.mc]);
    if (!WG_ready) {
      HT_CUDA(gemm_tn_small_launch(ec.U, nc, ec.GU, nc, tr.WG, P.kw, P.kw, P.kw, nc, c.st));
      ++c.launches;
    }
    HT_CUDA(transfer_eig_launch(tr.WG, P.kw, P.kt, P.kc, 1, tr.M, tr.Bkt, c.st));
    const long long kpq = static_cast<long long>(P.kp) * P.kq;
    HT_CUDA(matmul_nn_launch(tr.C, kpq, tr.M, P.kt, tr.Bt, kpq, kpq, P.kt, P.kt, c.st));
    c.launches += 2;
    if (!P.t_is_left) {
      HT_CUDA(transpose_small_launch(tr.Bkt, P.kt, P.kc, tr.Broot, c.st));
      ++c.launches;
    }
  }
  c.stage = stage_before;
  res.B[P.t] = tr.Bt;
  res.B[0] = P.t_is_left ? tr.Bkt : tr.Broot;
  return HT_OK;
}

// G_pre[m] non-null: the mode-m Gram is already there (the pipelined input path).
// x16p: a BF16 copy with the first mode padded to n1p rows (zeros), used by the
// leaf Grams when n1 is not a multiple of 8 (TMA needs 16-byte rows).
ht_status_t decompose_core(Ctx &c, const Tree &T, const ht_config_t &cfg, const float *x32,
                           const __nv_bfloat16 *x16, const __nv_bfloat16 *x16t, int lb, const long *dims,
                           int order, Result &res, Timeline &tl, float *const *G_pre = nullptr,
                           const __nv_bfloat16 *x16p = nullptr, long n1p = 0) {
  const int p_over = cfg.oversample > 0 ? cfg.oversample : 16;
  const bool d3 = order == 3;
  Plan3 P3{};
  if (d3) P3 = plan3(T);

  const bool sketch = cfg.leaf_method == HT_LEAF_SKETCH;
  EigProblem ep[4];
  if (sketch) {
    // 1'-2'. leaf bases from the Gram-free range finder (stage "grams" holds
    // all of it, stage "eig" is empty)
    HT_TRY(leaf_sketch(c, T, cfg, dims, order, x32, x16, x16t, lb, ep, res));
    tl.mark(c.st);
    tl.mark(c.st);
  } else {
    // 1. leaf Grams
    float *G[4] = {};
    for (int m = 0; m < order; ++m) {
      G[m] = (G_pre && G_pre[m]) ? G_pre[m] : c.ar.take<float>(static_cast<size_t>(dims[m]) * dims[m]);
      if (!G[m]) return fail(HT_ERR_OUT_OF_MEMORY, "workspace too small (Gram)");
    }
    long pdims[HT_MAX_ORDER];
    for (int m = 0; m < order; ++m) pdims[m] = (m == 0 && x16p) ? n1p : dims[m];
    for (int m = 0; m < order; ++m) {
      if (G_pre && G_pre[m]) continue;
      const View v = view_of_group(dims, order, m, m);
      if (x16p) HT_TRY(gram_padded(c, v, view_of_group(pdims, order, m, m), x32, x16p, G[m]));
      else if (m == order - 1 && x16t) HT_TRY(gram_transposed(c, v, x32, x16t, lb, G[m]));
      else HT_TRY(gram(c, v, x32, x16, G[m]));
    }
    tl.mark(c.st);
    HT_TRY(leaf_eigs(c, T, cfg, dims, order, G, ep, res));
    tl.mark(c.st);
  }

  if (d3) {
    const Plan3 &P = P3;
    const View vc = view_of_group(dims, 3, P.mc, P.mc);
    const long long zrows = vc.L * vc.R;
    const EigProblem &ec = ep[P.mc];
    Transfer3 tr;
    HT_TRY(take_transfer3(c, P, tr));
    const size_t mark = c.ar.off;
    // the sketch path has no Gram of the complementary mode: Z gets all kw
    // columns of its basis W and W^T G_c W = Z^T Z comes from the Householder
    // TSQR of Z (R^T R)
    const int kz = sketch ? P.kw : P.kt;
    float *Z = c.ar.take<float>(static_cast<size_t>(zrows) * kz);
    // V enters the BF16 product as high + low BF16 parts (one MMA tile of
    // 2*fold_h columns): rounding V itself to BF16 would tilt every column of
    // Z = X_(t) V by ~2^-9 of X's energy, which dominates the error of nearly
    // exact low-rank inputs.
    const int fold_h = kz <= 32 ? 32 : 64;
    // (no BF16 copy of X in its plain layout -- a first mode padded for the
    // Grams -- means an FP32 product: no split V either)
    __nv_bfloat16 *V16 =
        (c.tc && x16 && !c.core_grouped) ? c.ar.take<__nv_bfloat16>(static_cast<size_t>(dims[P.mc]) * 2 * fold_h + 64)
                                         : nullptr;
    float *Rz = sketch ? c.ar.take<float>(static_cast<size_t>(kz) * kz) : nullptr;
    const size_t qbytes = sketch ? tsqr_workspace_bytes(zrows, kz) : 0;
    void *qws = sketch ? c.ar.take<char>(qbytes) : nullptr;
    if (!Z || (c.tc && x16 && !c.core_grouped && !V16) || (sketch && (!Rz || !qws)))
      return fail(HT_ERR_OUT_OF_MEMORY, "workspace too small (core pass)");
    // 3. core pass: Z = X_(t) V, V = leading kz columns of the complementary leaf's basis
    if (V16 && !c.dry()) {
      HT_CUDA(split_bf16_launch(ec.U, dims[P.mc], kz, fold_h, V16, c.st));
      ++c.launches;
    }
    HT_TRY(mode_product(c, vc, x32, x16, ec.U, V16, kz, Z, fold_h));
    if (sketch && !c.dry()) HT_CUDA(tsqr_launch(Z, zrows, kz, zrows, Rz, tr.WG, qws, qbytes, c.st, &c.launches));
    tl.mark(c.st);
    HT_TRY(transfer3_from_z(c, P, dims, ep, Z, tr, res, sketch));
    c.ar.off = mark;
    tl.mark(c.st);
    return HT_OK;
  }

  // 4th order: range finder on A = X_(12) (nA x mA, column-major)
  const int t1 = T.left[0], t2 = T.right[0];
  const int k1 = T.rank[t1], k2 = T.rank[t2];
  const long long nA = static_cast<long long>(dims[0]) * dims[1], mA = static_cast<long long>(dims[2]) * dims[3];
  const int s = static_cast<int>(std::min<long long>({static_cast<long long>(std::max(k1, k2) + p_over), 64ll, nA, mA}));
  const int qsteps = cfg.power_steps >= 0 ? cfg.power_steps : 1;
  const int a1 = T.left[t1], b1 = T.right[t1], a2 = T.left[t2], b2 = T.right[t2];
  float *Broot = c.ar.take<float>(static_cast<size_t>(k1) * k2);
  float *B12 = c.ar.take<float>(static_cast<size_t>(T.rank[a1]) * T.rank[b1] * k1);
  float *B34 = c.ar.take<float>(static_cast<size_t>(T.rank[a2]) * T.rank[b2] * k2);
  if (!Broot || !B12 || !B34) return fail(HT_ERR_OUT_OF_MEMORY, "workspace too small (transfer)");
  const size_t mark = c.ar.off;
  float *Om = c.ar.take<float>(static_cast<size_t>(mA) * s);
  float *Yq = c.ar.take<float>(static_cast<size_t>(nA) * s);
  float *Wz = c.ar.take<float>(static_cast<size_t>(mA) * s);
  __nv_bfloat16 *B16 = c.tc ? c.ar.take<__nv_bfloat16>(static_cast<size_t>(std::max(nA, mA)) * s + 64) : nullptr;
  float *GW = c.ar.take<float>(static_cast<size_t>(s) * s);
  float *M1 = c.ar.take<float>(static_cast<size_t>(s) * s);
  float *M2 = c.ar.take<float>(static_cast<size_t>(s) * s);
  float *U12 = c.ar.take<float>(static_cast<size_t>(nA) * k1);
  float *U34 = c.ar.take<float>(static_cast<size_t>(mA) * k2);
  EigProblem cq;
  cq.G = nullptr; cq.n = static_cast<int>(std::max(nA, mA)); cq.s = s; cq.K = s;
  const size_t cbytes = eig_workspace_bytes(&cq, 1);
  void *cws = c.ar.take<char>(cbytes);
  if (!Om || !Yq || !Wz || !GW || !M1 || !M2 || !U12 || !U34 || !cws || (c.tc && !B16))
    return fail(HT_ERR_OUT_OF_MEMORY, "workspace too small (range finder)");
  const View vy{static_cast<long>(nA), static_cast<long>(mA), 1};
  auto orth = [&](float *Qm, long long rows) -> ht_status_t {
    if (c.dry()) return HT_OK;
    EigProblem e;
    e.G = nullptr; e.n = static_cast<int>(rows); e.s = s; e.K = s; e.Q = Qm; e.Y = nullptr;
    e.U = e.GU = e.theta = e.resid = nullptr; e.start = nullptr; e.seed = 0; e.stream_id = 0;
    HT_CUDA(cholqr_batched(&e, 1, 2, cws, cbytes, c.err, c.st, &c.launches));
    return HT_OK;
  };
  auto to16 = [&](const float *src, long long count) -> const __nv_bfloat16 * {
    if (!B16) return nullptr;
    if (!c.dry()) {
      if (f32_to_bf16_launch(src, B16, count, c.st) != cudaSuccess) return nullptr;
      ++c.launches;
    }
    return B16;
  };
  if (!c.dry()) {
    HT_CUDA(gaussian_fill_launch(Om, mA * s, cfg.seed, 100, c.st));
    ++c.launches;
  }
  HT_TRY(mode_product(c, vy, x32, x16, Om, to16(Om, mA * s), s, Yq));        // Y = A Omega
  HT_TRY(orth(Yq, nA));
  for (int it = 0; it < qsteps; ++it) {
    HT_TRY(corange_product(c, vy, x32, x16, Yq, to16(Yq, nA * s), s, Wz));   // Z = A^T Q
    HT_TRY(orth(Wz, mA));
    HT_TRY(mode_product(c, vy, x32, x16, Wz, to16(Wz, mA * s), s, Yq));      // Y = A Z
    HT_TRY(orth(Yq, nA));
  }
  HT_TRY(corange_product(c, vy, x32, x16, Yq, to16(Yq, nA * s), s, Wz));     // W = A^T Q
  tl.mark(c.st);
  if (!c.dry()) {
    HT_CUDA(gemm_tn_small_launch(Wz, static_cast<int>(mA), Wz, static_cast<int>(mA), GW, s, s, s, static_cast<int>(mA), c.st));
    HT_CUDA(svd_from_gram_launch(GW, s, k1, k2, M1, M2, Broot, c.st));
    HT_CUDA(matmul_nn_launch(Yq, nA, M1, s, U12, nA, nA, k1, s, c.st));
    HT_CUDA(matmul_nn_launch(Wz, mA, M2, s, U34, mA, mA, k2, s, c.st));
    c.launches += 4;
  }
  HT_TRY(core_contract(c, U12, static_cast<int>(dims[0]), static_cast<int>(dims[1]), k1, ep[0].U, T.rank[a1], ep[1].U,
                       T.rank[b1], B12));
  HT_TRY(core_contract(c, U34, static_cast<int>(dims[2]), static_cast<int>(dims[3]), k2, ep[2].U, T.rank[a2], ep[3].U,
                       T.rank[b2], B34));
  c.ar.off = mark;
  res.B[t1] = B12;
  res.B[t2] = B34;
  res.B[0] = Broot;
  tl.mark(c.st);
  return HT_OK;
}

// ||X - Xhat||_F^2 of an HT representation, into *dev_out (device double).
ht_status_t error_core(Ctx &c, const Tree &T, const float *x32, const long *dims, int order, const float *const *U,
                       const float *const *B, double *dev_out) {
  const size_t mark = c.ar.off;
  int nb = 0;
  double *parts = nullptr;
  if (order == 3) {
    const Plan3 P = plan3(T);
    const long np_ = dims[P.mp], nq_ = dims[P.mq], nc_ = dims[P.mc];
    float *Bkt = c.ar.take<float>(static_cast<size_t>(P.kt) * P.kc);
    float *core = c.ar.take<float>(static_cast<size_t>(P.kp) * P.kq * P.kc);
    float *Tm = c.ar.take<float>(static_cast<size_t>(np_) * P.kq * P.kc);
    float *Wm = c.ar.take<float>(static_cast<size_t>(np_) * nq_ * P.kc);
    long long Rr, Cc;
    int batch = 1;
    if (P.mc == 2) { Rr = np_ * nq_; Cc = nc_; }
    else if (P.mc == 0) { Rr = nc_; Cc = np_ * nq_; }
    else { Rr = np_; Cc = nc_; batch = static_cast<int>(nq_); }
    nb = error_fused_blocks(Rr, Cc) * batch;
    parts = c.ar.take<double>(static_cast<size_t>(nb) + 8);
    if (!Bkt || !core || !Tm || !Wm || !parts) return fail(HT_ERR_OUT_OF_MEMORY, "workspace too small (error)");
    c.stage = 4;
    if (c.err_out && !c.ar.dry) {   // the batch's grouped error pass
      ErrJob j;
      j.Bt = B[P.t]; j.B0 = B[0]; j.t_is_left = P.t_is_left ? 1 : 0;
      j.kpq = static_cast<long long>(P.kp) * P.kq; j.kt = P.kt; j.kc = P.kc;
      j.core = core; j.Tm = Tm; j.Wm = Wm;
      j.Up = U[P.p]; j.Uq = U[P.q];
      j.np = static_cast<int>(np_); j.nq = static_cast<int>(nq_); j.kp = P.kp; j.kq = P.kq;
      j.X = x32; j.R = Rr; j.Cn = Cc; j.kk = P.kc; j.slabs = batch;
      if (P.mc == 2) {
        j.ldx = Rr; j.sx = 0; j.A = Wm; j.lda = Rr; j.sa = 0; j.B = U[P.c]; j.ldb = nc_;
      } else if (P.mc == 0) {
        j.ldx = Rr; j.sx = 0; j.A = U[P.c]; j.lda = nc_; j.sa = 0; j.B = Wm; j.ldb = np_ * nq_;
      } else {
        j.ldx = np_; j.sx = np_ * nc_; j.A = Wm; j.lda = np_ * nq_; j.sa = np_; j.B = U[P.c]; j.ldb = nc_;
      }
      j.parts = parts; j.out = dev_out;
      auto blocks = [](long long n, long long cap) {
        return static_cast<int>(std::min<long long>(cap, std::max<long long>(1, (n + 255) / 256)));
      };
      j.nblk[0] = blocks(j.kpq * P.kc, 8);
      j.nblk[1] = blocks(np_ * P.kq * P.kc, 16);
      // narrow: the last mode is the complementary leaf (rows of X contiguous)
      j.narrow = (P.mc == 2 && P.kc <= 64 && Rr >= 32) ? 1 : 0;
      if (j.narrow) {
        j.nblk[2] = j.nblk[3] = 0;
        j.nblk[4] = static_cast<int>(std::min<long long>(32, (Rr + 255) / 256));
        j.nblk[5] = P.kc * static_cast<int>((np_ + 255) / 256);
        j.ntile = j.nblk[4];
      } else {
        j.nblk[2] = blocks(np_ * nq_ * P.kc, 32);
        j.nblk[3] = std::min(nb, 32);
        j.nblk[4] = j.nblk[5] = 0;
        j.ntile = nb;
      }
      for (int k = 0; k < 6; ++k) j.blk0[k] = 0;
      c.err_out->push_back(j);
    }
    if (!c.dry()) {
      if (P.t_is_left) HT_CUDA(cudaMemcpyAsync(Bkt, B[0], sizeof(float) * P.kt * P.kc, cudaMemcpyDeviceToDevice, c.st));
      else HT_CUDA(transpose_small_launch(B[0], P.kc, P.kt, Bkt, c.st));
      const long long kpq = static_cast<long long>(P.kp) * P.kq;
      HT_CUDA(matmul_nn_launch(B[P.t], kpq, Bkt, P.kt, core, kpq, kpq, P.kc, P.kt, c.st));
      HT_CUDA(expand2_launch(U[P.p], static_cast<int>(np_), P.kp, core, U[P.q], static_cast<int>(nq_), P.kq, P.kc, Tm,
                             Wm, c.st));
      if (P.mc == 2)         // X_(01) = W U_c^T
        HT_CUDA(error_fused_launch(x32, Rr, 0, Wm, Rr, 0, U[P.c], nc_, Rr, Cc, P.kc, 1, parts, c.st));
      else if (P.mc == 0)    // X_(0) = U_c W^T
        HT_CUDA(error_fused_launch(x32, Rr, 0, U[P.c], nc_, 0, Wm, np_ * nq_, Rr, Cc, P.kc, 1, parts, c.st));
      else                   // slab i2 of X (n0 x n1) = W[(i0, i2), :] U_1^T
        HT_CUDA(error_fused_launch(x32, np_, np_ * nc_, Wm, np_ * nq_, np_, U[P.c], nc_, Rr, Cc, P.kc, batch, parts,
                                   c.st));
      c.launches += 5;
    }
  } else {
    const int t1 = T.left[0], t2 = T.right[0];
    const int k1 = T.rank[t1], k2 = T.rank[t2];
    const int a1 = T.left[t1], b1 = T.right[t1], a2 = T.left[t2], b2 = T.right[t2];
    const long long R = static_cast<long long>(dims[0]) * dims[1], Cn = static_cast<long long>(dims[2]) * dims[3];
    float *T1 = c.ar.take<float>(static_cast<size_t>(dims[0]) * T.rank[b1] * k1);
    float *W12 = c.ar.take<float>(static_cast<size_t>(R) * k1);
    float *A12 = c.ar.take<float>(static_cast<size_t>(R) * k2);
    float *T2 = c.ar.take<float>(static_cast<size_t>(dims[2]) * T.rank[b2] * k2);
    float *W34 = c.ar.take<float>(static_cast<size_t>(Cn) * k2);
    nb = error_fused_blocks(R, Cn);
    parts = c.ar.take<double>(static_cast<size_t>(nb) + 8);
    if (!T1 || !W12 || !A12 || !T2 || !W34 || !parts) return fail(HT_ERR_OUT_OF_MEMORY, "workspace too small (error)");
    if (!c.dry()) {
      HT_CUDA(expand2_launch(U[a1], static_cast<int>(dims[0]), T.rank[a1], B[t1], U[b1], static_cast<int>(dims[1]),
                             T.rank[b1], k1, T1, W12, c.st));
      HT_CUDA(expand2_launch(U[a2], static_cast<int>(dims[2]), T.rank[a2], B[t2], U[b2], static_cast<int>(dims[3]),
                             T.rank[b2], k2, T2, W34, c.st));
      HT_CUDA(matmul_nn_launch(W12, R, B[0], k1, A12, R, R, k2, k1, c.st));
      HT_CUDA(error_fused_launch(x32, R, 0, A12, R, 0, W34, Cn, R, Cn, k2, 1, parts, c.st));
      c.launches += 6;
    }
  }
  if (!c.dry()) {   // (stage 4 for 3rd order: part of the grouped error pass)
    HT_CUDA(sumsq_finish_launch(parts, nb, dev_out, c.st));
    ++c.launches;
  }
  c.ar.off = mark;
  return HT_OK;
}

size_t factor_count(const Tree &T, const long *dims, int t) {
  if (T.leaf(t)) return static_cast<size_t>(dims[T.mode_of_leaf(t)]) * T.rank[t];
  return static_cast<size_t>(T.rank[T.left[t]]) * T.rank[T.right[t]] * T.rank[t];
}

// ------------------------------------------------------------ out-of-core path
// A 3rd-order tensor that stays in host memory (the reference's 3D/TSQR variant
// streams four slabs of frontal slices: htd_tensorcore.cu:58-111).  Passes over
// host X, each through two device slab buffers (the copy of slab s+1 on its own
// stream overlaps the work on slab s):
//   A  slabs along mode 2 (contiguous):    ||X||^2, G_0 += X_s(0) X_s(0)^T, G_1 likewise
//   B  slabs along mode 1 (2-D copies):    G_2 += X_s(2) X_s(2)^T
//      (a Gram accumulates over slabs along any mode but its own)
//   -  leaf eigen-solver on the three Grams, in core
//   C  slabs along mode 2:                 Z = X_(t) V, accumulated (c = mode 2) or
//                                          written by row blocks (c = mode 0 or 1)
//   -  transfer tensors from Z, in core
//   D  (error) slabs along mode 2:         ||X_s - Xhat_s||^2 from the fused error kernel
struct StreamArgs {
  const float *xh;
  const long *dims;
  float *const *U;
  float *const *B;
  bool want_err;
  long long slab2, slab1;   // slab lengths along modes 2 and 1
};

struct SlabIo {
  cudaStream_t cs = nullptr;
  cudaEvent_t copied[2] = {}, freed[2] = {};
  float *buf[2] = {};
};

// Streams `count` slabs through io.buf: copy(s, dst, cs) issues slab s's copy
// on the copy stream, compute(s, src) enqueues its work on c.st.  In a dry run
// only slab 0's work is sized.
template <class Copy, class Compute>
ht_status_t stream_slabs(Ctx &c, SlabIo &io, long long count, Copy copy, Compute compute) {
  if (c.dry()) return count > 0 ? compute(0, io.buf[0]) : HT_OK;
  // the buffers may still be read by an earlier pass's work on c.st
  HT_CUDA(cudaEventRecord(io.freed[0], c.st));
  HT_CUDA(cudaStreamWaitEvent(io.cs, io.freed[0], 0));
  auto issue = [&](long long s) -> ht_status_t {
    const int b = static_cast<int>(s & 1);
    if (s >= 2) HT_CUDA(cudaStreamWaitEvent(io.cs, io.freed[b], 0));
    HT_TRY(copy(s, io.buf[b], io.cs));
    HT_CUDA(cudaEventRecord(io.copied[b], io.cs));
    return HT_OK;
  };
  HT_TRY(issue(0));
  for (long long s = 0; s < count; ++s) {
    if (s + 1 < count) HT_TRY(issue(s + 1));
    const int b = static_cast<int>(s & 1);
    HT_CUDA(cudaStreamWaitEvent(c.st, io.copied[b], 0));
    HT_TRY(compute(s, io.buf[b]));
    HT_CUDA(cudaEventRecord(io.freed[b], c.st));
  }
  return HT_OK;
}

ht_status_t stream_call(Ctx &c, const Tree &T, const ht_config_t &cfg, const StreamArgs &a, SlabIo &io,
                        Timeline &tl, double *dsum) {
  const long n0 = a.dims[0], n1 = a.dims[1], n2 = a.dims[2];
  const long long s2 = a.slab2, s1 = a.slab1;
  const long long cnt2 = (n2 + s2 - 1) / s2, cnt1 = (n1 + s1 - 1) / s1;
  const long long slab_floats = std::max(s2 * n0 * n1, s1 * n0 * n2);
  const Plan3 P = plan3(T);
  const long nmax = std::max({n0, n1, n2});
  io.buf[0] = c.ar.take<float>(static_cast<size_t>(slab_floats));
  io.buf[1] = c.ar.take<float>(static_cast<size_t>(slab_floats));
  __nv_bfloat16 *b16 = c.tc ? c.ar.take<__nv_bfloat16>(static_cast<size_t>(slab_floats) + 64) : nullptr;
  __nv_bfloat16 *b16t = c.tc ? c.ar.take<__nv_bfloat16>(static_cast<size_t>(slab_floats) + 64) : nullptr;
  double *nparts = c.ar.take<double>(static_cast<size_t>(cnt2) * 1024);
  double *scratch_parts = c.ar.take<double>(1024);
  float *G[3];
  for (int m = 0; m < 3; ++m) G[m] = c.ar.take<float>(static_cast<size_t>(a.dims[m]) * a.dims[m]);
  float *Gt = c.ar.take<float>(static_cast<size_t>(nmax) * nmax);
  if (!io.buf[0] || !io.buf[1] || (c.tc && (!b16 || !b16t)) || !nparts || !scratch_parts || !G[0] || !G[1] ||
      !G[2] || !Gt)
    return fail(HT_ERR_OUT_OF_MEMORY, "workspace too small (streaming buffers)");
  const size_t slab_row_bytes2 = sizeof(float) * static_cast<size_t>(n0) * n1;
  auto copy2 = [&](long long s, float *dst, cudaStream_t cs) -> ht_status_t {   // X[:, :, c0:c0+len]
    const long long c0 = s * s2, len = std::min(s2, n2 - c0);
    HT_CUDA(cudaMemcpyAsync(dst, a.xh + static_cast<size_t>(n0) * n1 * c0, slab_row_bytes2 * len,
                            cudaMemcpyHostToDevice, cs));
    return HT_OK;
  };
  auto copy1 = [&](long long s, float *dst, cudaStream_t cs) -> ht_status_t {   // X[:, j0:j0+len, :]
    const long long j0 = s * s1, len = std::min(s1, n1 - j0);
    const size_t w = sizeof(float) * static_cast<size_t>(n0) * len;
    HT_CUDA(cudaMemcpy2DAsync(dst, w, a.xh + static_cast<size_t>(n0) * j0, sizeof(float) * n0 * n1, w, n2,
                              cudaMemcpyHostToDevice, cs));
    return HT_OK;
  };
  auto bf16_of = [&](const float *x, long long count, double *parts) -> ht_status_t {
    if (c.dry()) return HT_OK;
    if (c.tc) HT_CUDA(convert_bf16_launch(x, b16, count, parts, 1024, c.st));
    else HT_CUDA(sumsq_launch(x, count, parts, 1024, c.st));
    ++c.launches;
    return HT_OK;
  };
  auto accumulate = [&](float *dst, const float *src, long long count, bool first) -> ht_status_t {
    if (!c.dry()) {
      HT_CUDA(accumulate_launch(dst, src, count, first ? 1 : 0, c.st));
      ++c.launches;
    }
    return HT_OK;
  };

  // pass A: ||X||^2, G_0, G_1
  HT_TRY(stream_slabs(c, io, cnt2, copy2, [&](long long s, const float *x) -> ht_status_t {
    const long long len = std::min(s2, n2 - s * s2);
    const long dd[3] = {n0, n1, static_cast<long>(len)};
    HT_TRY(bf16_of(x, n0 * n1 * len, nparts + s * 1024));
    for (int m = 0; m < 2; ++m) {
      HT_TRY(gram(c, view_of_group(dd, 3, m, m), x, b16, Gt));
      HT_TRY(accumulate(G[m], Gt, static_cast<long long>(a.dims[m]) * a.dims[m], s == 0));
    }
    return HT_OK;
  }));
  if (!c.dry()) {
    HT_CUDA(sumsq_finish_launch(nparts, static_cast<int>(cnt2 * 1024), dsum, c.st));
    ++c.launches;
  }
  tl.mark(c.st);
  // pass B: G_2
  HT_TRY(stream_slabs(c, io, cnt1, copy1, [&](long long s, const float *x) -> ht_status_t {
    const long long len = std::min(s1, n1 - s * s1);
    const long dd[3] = {n0, static_cast<long>(len), n2};
    const View v = view_of_group(dd, 3, 2, 2);
    const int lb = c.tc ? last_mode_block(dd, 3) : 0;
    if (lb && !c.dry()) {
      HT_CUDA(convert_bf16_dual_launch(x, b16, b16t, v.L, v.N, lb, scratch_parts, 1024, c.st));
      ++c.launches;
    } else {
      HT_TRY(bf16_of(x, n0 * len * n2, scratch_parts));
    }
    if (lb) HT_TRY(gram_transposed(c, v, x, b16t, lb, Gt));
    else HT_TRY(gram(c, v, x, b16, Gt));
    return accumulate(G[2], Gt, static_cast<long long>(n2) * n2, s == 0);
  }));
  tl.mark(c.st);

  // leaf eigen-solver
  Result res;
  EigProblem ep[4];
  HT_TRY(leaf_eigs(c, T, cfg, a.dims, 3, G, ep, res));
  tl.mark(c.st);

  // pass C: Z = X_(t) V
  const EigProblem &ec = ep[P.mc];
  const View vc = view_of_group(a.dims, 3, P.mc, P.mc);
  const long long zrows = vc.L * vc.R;
  Transfer3 tr;
  HT_TRY(take_transfer3(c, P, tr));
  const size_t mark = c.ar.off;
  const int fold_h = P.kt <= 32 ? 32 : 64;
  float *Z = c.ar.take<float>(static_cast<size_t>(zrows) * P.kt);
  const long long zs_rows = P.mc == 2 ? zrows : (P.mc == 0 ? static_cast<long long>(n1) * s2 : static_cast<long long>(n0) * s2);
  float *Zs = c.ar.take<float>(static_cast<size_t>(zs_rows) * P.kt);
  const long vrows = P.mc == 2 ? static_cast<long>(s2) : static_cast<long>(a.dims[P.mc]);
  float *Vs = c.ar.take<float>(static_cast<size_t>(vrows) * P.kt);
  __nv_bfloat16 *V16 = c.tc ? c.ar.take<__nv_bfloat16>(static_cast<size_t>(vrows) * 2 * fold_h + 64) : nullptr;
  if (!Z || !Zs || !Vs || (c.tc && !V16)) return fail(HT_ERR_OUT_OF_MEMORY, "workspace too small (core pass)");
  if (P.mc != 2 && !c.dry()) {   // V is used whole by every slab
    HT_CUDA(cudaMemcpyAsync(Vs, ec.U, sizeof(float) * a.dims[P.mc] * P.kt, cudaMemcpyDeviceToDevice, c.st));
    if (V16) {
      HT_CUDA(split_bf16_launch(Vs, a.dims[P.mc], P.kt, fold_h, V16, c.st));
      ++c.launches;
    }
  }
  HT_TRY(stream_slabs(c, io, cnt2, copy2, [&](long long s, const float *x) -> ht_status_t {
    const long long c0 = s * s2, len = std::min(s2, n2 - c0);
    const long dd[3] = {n0, n1, static_cast<long>(len)};
    if (c.tc) HT_TRY(bf16_of(x, n0 * n1 * len, scratch_parts));
    const View v = view_of_group(dd, 3, P.mc, P.mc);
    if (P.mc == 2) {   // V rows of this slab
      if (!c.dry()) {
        HT_CUDA(cudaMemcpy2DAsync(Vs, sizeof(float) * len, ec.U + c0, sizeof(float) * n2, sizeof(float) * len, P.kt,
                                  cudaMemcpyDeviceToDevice, c.st));
        if (V16) {
          HT_CUDA(split_bf16_launch(Vs, len, P.kt, fold_h, V16, c.st));
          ++c.launches;
        }
      }
      HT_TRY(mode_product(c, v, x, c.tc ? b16 : nullptr, Vs, V16, P.kt, Zs, fold_h));
      return accumulate(Z, Zs, zrows * P.kt, s == 0);
    }
    HT_TRY(mode_product(c, v, x, c.tc ? b16 : nullptr, Vs, V16, P.kt, Zs, fold_h));
    if (!c.dry()) {   // rows (i1 or i0, i2 in the slab) of Z
      const long long per = P.mc == 0 ? n1 : n0;
      HT_CUDA(cudaMemcpy2DAsync(Z + per * c0, sizeof(float) * zrows, Zs, sizeof(float) * per * len,
                                sizeof(float) * per * len, P.kt, cudaMemcpyDeviceToDevice, c.st));
    }
    return HT_OK;
  }));
  tl.mark(c.st);
  HT_TRY(transfer3_from_z(c, P, a.dims, ep, Z, tr, res));
  c.ar.off = mark;
  tl.mark(c.st);

  // outputs
  for (int t = 0; t < T.n_nodes; ++t) {
    float *dst = T.leaf(t) ? a.U[t] : a.B[t];
    const float *src = T.leaf(t) ? res.U[t] : res.B[t];
    if (dst && !c.dry())
      HT_CUDA(cudaMemcpyAsync(dst, src, factor_count(T, a.dims, t) * sizeof(float), cudaMemcpyDefault, c.st));
  }

  // pass D: ||X - Xhat||^2
  if (a.want_err) {
    const long np_ = a.dims[P.mp], nq_ = a.dims[P.mq], nc_ = a.dims[P.mc];
    float *Bkt = c.ar.take<float>(static_cast<size_t>(P.kt) * P.kc);
    float *core = c.ar.take<float>(static_cast<size_t>(P.kp) * P.kq * P.kc);
    float *Tm = c.ar.take<float>(static_cast<size_t>(np_) * P.kq * P.kc);
    float *Wm = c.ar.take<float>(static_cast<size_t>(np_) * nq_ * P.kc);
    long long nb = 0;
    if (P.mc == 2) nb = error_fused_blocks(static_cast<long long>(n0) * n1, s2);
    else if (P.mc == 0) nb = error_fused_blocks(n0, static_cast<long long>(n1) * s2);
    else nb = static_cast<long long>(error_fused_blocks(n0, n1)) * s2;
    double *eparts = c.ar.take<double>(static_cast<size_t>(nb * cnt2) + 8);
    if (!Bkt || !core || !Tm || !Wm || !eparts) return fail(HT_ERR_OUT_OF_MEMORY, "workspace too small (error)");
    if (!c.dry()) {
      HT_CUDA(cudaMemsetAsync(eparts, 0, sizeof(double) * nb * cnt2, c.st));
      if (P.t_is_left)
        HT_CUDA(cudaMemcpyAsync(Bkt, res.B[0], sizeof(float) * P.kt * P.kc, cudaMemcpyDeviceToDevice, c.st));
      else HT_CUDA(transpose_small_launch(res.B[0], P.kc, P.kt, Bkt, c.st));
      const long long kpq = static_cast<long long>(P.kp) * P.kq;
      HT_CUDA(matmul_nn_launch(res.B[P.t], kpq, Bkt, P.kt, core, kpq, kpq, P.kc, P.kt, c.st));
      HT_CUDA(expand2_launch(res.U[P.p], static_cast<int>(np_), P.kp, core, res.U[P.q], static_cast<int>(nq_), P.kq,
                             P.kc, Tm, Wm, c.st));
      c.launches += 4;
    }
    HT_TRY(stream_slabs(c, io, cnt2, copy2, [&](long long s, const float *x) -> ht_status_t {
      if (c.dry()) return HT_OK;
      const long long c0 = s * s2, len = std::min(s2, n2 - c0);
      double *pp = eparts + s * nb;
      if (P.mc == 2) {   // X_s (n0 n1 x len) = W U_2[c0:c0+len]^T
        const long long R = static_cast<long long>(n0) * n1;
        HT_CUDA(error_fused_launch(x, R, 0, Wm, R, 0, res.U[P.c] + c0, nc_, R, len, P.kc, 1, pp, c.st));
      } else if (P.mc == 0) {   // X_s (n0 x n1 len) = U_0 W[rows (i1, i2 in slab)]^T
        HT_CUDA(error_fused_launch(x, n0, 0, res.U[P.c], n0, 0, Wm + static_cast<long long>(n1) * c0,
                                   static_cast<long long>(np_) * nq_, n0, static_cast<long long>(n1) * len, P.kc, 1,
                                   pp, c.st));
      } else {   // slice i2 of X_s (n0 x n1) = W[rows (i0, i2)] U_1^T
        HT_CUDA(error_fused_launch(x, n0, static_cast<long long>(n0) * n1, Wm + static_cast<long long>(n0) * c0,
                                   static_cast<long long>(np_) * nq_, n0, res.U[P.c], nc_, n0, n1, P.kc,
                                   static_cast<int>(len), pp, c.st));
      }
      ++c.launches;
      return HT_OK;
    }));
    if (!c.dry()) {
      HT_CUDA(sumsq_finish_launch(eparts, static_cast<int>(nb * cnt2), dsum + 1, c.st));
      ++c.launches;
    }
    tl.mark(c.st);
  }
  return HT_OK;
}

// One full call (decomposition, outputs, optional error), used both as the
// dry run that sizes the workspace and for the real run.
struct CallArgs {
  const float *x;
  bool x_dev;
  const long *dims;
  int order;
  float *const *U;
  float *const *B;
  bool want_err;
};

// The asynchronous part of a call, X already on the device: BF16 copy and
// ||X||^2 (dsum[0]), the decomposition, the factors copied to the caller's
// buffers, and the error pass (dsum[1]) when asked.  No host synchronisation,
// so it can be captured into a CUDA graph.
ht_status_t enqueue_body(Ctx &c, const Tree &T, const ht_config_t &cfg, const float *xd, const CallArgs &a,
                         double *nparts, double *dsum, Timeline &tl, Result &res) {
  c.core_grouped = c.eig_mode != 0 && a.order == 3 && cfg.leaf_method == HT_LEAF_GRAM;
  long long total = 1;
  for (int m = 0; m < a.order; ++m) total *= a.dims[m];
  __nv_bfloat16 *xb = nullptr, *xbt = nullptr, *xp = nullptr;
  int lb = c.tc ? last_mode_block(a.dims, a.order) : 0;
  // first mode not a multiple of 8: the Grams read a copy padded to n1p rows
  // (the tcgen05 path's TMA rows must be 16-byte multiples); the other products
  // of such a tensor run on the FP32 operands
  const long n1 = a.dims[0], n1p = (n1 + 7) / 8 * 8;
  // grouped conversion job of the batched path (plain or padded copy, or sums only)
  auto defer = [&](__nv_bfloat16 *dst, long pad) {
    if (c.conv_out) {
      ConvJob j;
      j.x = xd; j.xb = dst; j.partials = nparts; j.dsum = dsum;
      j.n1 = n1; j.n1p = pad; j.rest = total / n1;
      j.blk0 = 0;
      j.nblk = static_cast<int>(std::min<long long>(32, std::max<long long>(1, (pad * (total / n1)) / 16384)));
      c.conv_out->push_back(j);
    }
  };
  if (c.tc && n1 % 8 != 0 && cfg.leaf_method == HT_LEAF_GRAM) {
    xp = c.ar.take<__nv_bfloat16>(static_cast<size_t>(total / n1 * n1p) + 64);
    if (!xp) return fail(HT_ERR_OUT_OF_MEMORY, "workspace too small (padded bf16 tensor)");
    if (c.defer_io) defer(xp, n1p);
    else if (!c.dry()) HT_CUDA(convert_bf16_pad_launch(xd, xp, n1, n1p, total / n1, nparts, 1024, c.st));
    lb = 0;
  } else if (c.tc && c.defer_io && !(lb && (reinterpret_cast<uintptr_t>(xd) & 15u) == 0)) {
    xb = c.ar.take<__nv_bfloat16>(static_cast<size_t>(total) + 64);
    if (!xb) return fail(HT_ERR_OUT_OF_MEMORY, "workspace too small (bf16 tensor)");
    defer(xb, n1);
  } else if (!c.tc && c.defer_io) {
    defer(nullptr, n1);
  } else if (c.tc) {
    xb = c.ar.take<__nv_bfloat16>(static_cast<size_t>(total) + 64);
    if (!xb) return fail(HT_ERR_OUT_OF_MEMORY, "workspace too small (bf16 tensor)");
    if (lb && (reinterpret_cast<uintptr_t>(xd) & 15u) == 0) {
      const long long N = a.dims[a.order - 1], L = total / N;
      xbt = c.ar.take<__nv_bfloat16>(static_cast<size_t>(total) + 64);
      if (!xbt) return fail(HT_ERR_OUT_OF_MEMORY, "workspace too small (bf16 tensor)");
      if (!c.dry()) HT_CUDA(convert_bf16_dual_launch(xd, xb, xbt, L, N, lb, nparts, 1024, c.st));
    } else if (!c.dry()) {
      HT_CUDA(convert_bf16_launch(xd, xb, total, nparts, 1024, c.st));
    }
  } else if (!c.dry()) {
    HT_CUDA(sumsq_launch(xd, total, nparts, 1024, c.st));
  }
  const bool deferred = c.defer_io && !xbt;
  if (!c.dry() && !deferred) {
    HT_CUDA(sumsq_finish_launch(nparts, 1024, dsum, c.st));
    c.launches += 2;
  }
  tl.mark(c.st);
  if (!xbt) lb = 0;
  HT_TRY(decompose_core(c, T, cfg, xd, xb, xbt, lb, a.dims, a.order, res, tl, nullptr, xp, n1p));
  // outputs to the caller's buffers (host or device)
  for (int t = 0; t < T.n_nodes; ++t) {
    float *dst = T.leaf(t) ? a.U[t] : a.B[t];
    const float *src = T.leaf(t) ? res.U[t] : res.B[t];
    if (!dst) continue;
    if (c.defer_io) {
      if (c.copy_out) c.copy_out->push_back(CopySeg{src, dst, static_cast<long long>(factor_count(T, a.dims, t))});
    } else if (!c.dry()) {
      HT_CUDA(cudaMemcpyAsync(dst, src, factor_count(T, a.dims, t) * sizeof(float), cudaMemcpyDefault, c.st));
    }
  }
  c.stage = 3;
  if (a.want_err) HT_TRY(error_core(c, T, xd, a.dims, a.order, res.U, res.B, dsum + 1));
  return HT_OK;
}

// Mixed path, 3rd order with the l-blocked copy, Gram leaves: X is taken in
// slabs along mode 3 and the mode-1 and mode-2 Grams accumulate slab by slab
// (split-K reductions that add into G), so that they overlap the work that
// produces the slabs:
//   host input    the host->device copy of slab s+1 (its own stream) overlaps
//                 the conversion and the Gram shares of slab s;
//   device input  the BF16 conversion of slab s+1 (its own stream, HBM-bound)
//                 overlaps the Gram shares of slab s (tensor-bound).
// Only the last slab's work, the mode-3 Gram and the rest of the
// decomposition follow.  The whole tensor ends up resident as in the plain path.
constexpr int kPipeSlabs = 8;

bool pipelined_input(const Ctx &c, const CallArgs &a, const ht_config_t &cfg) {
  // device input stays on the plain path: measured at 1024^3, the conversion on
  // a side stream did not overlap the slab Grams (5.63 ms against 5.38 ms)
  if (a.x_dev || !c.tc || a.order != 3 || cfg.leaf_method != HT_LEAF_GRAM) return false;
  const int lb = last_mode_block(a.dims, a.order);
  if (lb != 8) return false;   // 16-column conversion tiles: slabs of multiples of 16 columns
  if (a.x_dev && (reinterpret_cast<uintptr_t>(a.x) & 15u) != 0) return false;
  const long long total = static_cast<long long>(a.dims[0]) * a.dims[1] * a.dims[2];
  return total * 4 >= (256ll << 20) && a.dims[2] >= 16 * kPipeSlabs;
}

// Side stream and slab events of the pipelined path, created once per device.
struct PipeRes {
  cudaStream_t cs = nullptr;
  cudaEvent_t ev[kPipeSlabs + 1] = {};
};
PipeRes g_pipe[64];

ht_status_t pipe_resources(PipeRes **out) {
  int dev = 0;
  HT_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(HT_ERR_INVALID_ARG, "device index out of range");
  PipeRes &r = g_pipe[dev];
  if (!r.cs) {
    HT_CUDA(cudaStreamCreateWithFlags(&r.cs, cudaStreamNonBlocking));
    for (int i = 0; i <= kPipeSlabs; ++i) HT_CUDA(cudaEventCreateWithFlags(&r.ev[i], cudaEventDisableTiming));
  }
  *out = &r;
  return HT_OK;
}

ht_status_t enqueue_pipelined(Ctx &c, const Tree &T, const ht_config_t &cfg, const CallArgs &a, double *dsum,
                              Timeline &tl, Result &res, cudaEvent_t h2d_done) {
  const long n0 = a.dims[0], n1 = a.dims[1], n2 = a.dims[2];
  const long long L = static_cast<long long>(n0) * n1, total = L * n2;
  const int lb = last_mode_block(a.dims, a.order);
  long long len = (n2 + kPipeSlabs - 1) / kPipeSlabs;
  len = (len + 15) / 16 * 16;
  const long long S = (n2 + len - 1) / len;
  float *xd = a.x_dev ? const_cast<float *>(a.x) : c.ar.take<float>(static_cast<size_t>(total));
  __nv_bfloat16 *xb = c.ar.take<__nv_bfloat16>(static_cast<size_t>(total) + 64);
  __nv_bfloat16 *xbt = c.ar.take<__nv_bfloat16>(static_cast<size_t>(total) + 64);
  // device input: the conversion runs beside the Grams, so it takes 5 CTAs per
  // SM (32 registers x 256 threads each), which leaves an SM's registers and
  // threads for one Gram CTA (192 threads x 80 registers)
  const int np_conv = a.x_dev ? std::min(1024, 5 * sm_count()) : 1024;
  double *parts = c.ar.take<double>(static_cast<size_t>(S) * np_conv);
  float *G[4] = {};
  G[0] = c.ar.take<float>(static_cast<size_t>(n0) * n0);
  G[1] = c.ar.take<float>(static_cast<size_t>(n1) * n1);
  // the slab Grams of modes 1 and 2 leave their split-K partials side by side
  // (slab-major) and each mode is reduced once after the last slab
  TileGen ggen[2];
  int gsplits[2];
  float *gpart[2];
  for (int m = 0; m < 2; ++m) {
    const long nm = a.dims[m];
    const int bn = gram_bn_tc(nm), mt = gram_mt_tc(nm);
    if (!make_gram_gen(nm, bn, &ggen[m], 128 * mt)) return fail(HT_ERR_UNSUPPORTED, "Gram larger than 32768");
    const int nt = ggen[m].count;
    int sp = nt < sm_count() ? std::max(1, sm_count() / nt) : 1;
    const long long kb = (static_cast<long long>(a.dims[1 - m]) * len + 63) / 64;   // K blocks of a full slab
    long long per = (kb + sp - 1) / sp;
    per = std::max<long long>(per, std::min<long long>(kb, 16));
    gsplits[m] = static_cast<int>((kb + per - 1) / per);
    gpart[m] = c.ar.take<float>(static_cast<size_t>(S) * gsplits[m] * nt * ggen[m].bm * bn);
    if (!gpart[m]) return fail(HT_ERR_OUT_OF_MEMORY, "workspace too small (pipelined Gram partials)");
  }
  if (!xd || !xb || !xbt || !parts || !G[0] || !G[1])
    return fail(HT_ERR_OUT_OF_MEMORY, "workspace too small (pipelined input)");
  PipeRes *pr = nullptr;
  if (!c.dry()) {
    HT_TRY(pipe_resources(&pr));
    // the side stream may start only after earlier work on c.st (the workspace is shared)
    HT_CUDA(cudaEventRecord(pr->ev[S], c.st));
    HT_CUDA(cudaStreamWaitEvent(pr->cs, pr->ev[S], 0));
    for (long long s = 0; s < S; ++s) {
      const long long c0 = s * len, w = std::min(len, n2 - c0);
      if (a.x_dev) {
        HT_CUDA(convert_bf16_dual_launch(xd, xb, xbt, L, n2, lb, parts + s * np_conv, np_conv, pr->cs, c0, w));
        ++c.launches;
      } else {
        HT_CUDA(cudaMemcpyAsync(xd + L * c0, a.x + L * c0, sizeof(float) * L * w, cudaMemcpyHostToDevice, pr->cs));
      }
      HT_CUDA(cudaEventRecord(pr->ev[s], pr->cs));
    }
    if (h2d_done && !a.x_dev) HT_CUDA(cudaEventRecord(h2d_done, pr->cs));
  }
  for (long long s = 0; s < S; ++s) {
    const long long c0 = s * len, w = std::min(len, n2 - c0);
    if (!c.dry()) {
      HT_CUDA(cudaStreamWaitEvent(c.st, pr->ev[s], 0));
      if (!a.x_dev) {
        HT_CUDA(convert_bf16_dual_launch(xd, xb, xbt, L, n2, lb, parts + s * np_conv, np_conv, c.st, c0, w));
        ++c.launches;
      }
    }
    const long dd[3] = {n0, n1, static_cast<long>(w)};
    for (int m = 0; m < 2; ++m) {
      const size_t slab_part = static_cast<size_t>(gsplits[m]) * ggen[m].count * ggen[m].bm * ggen[m].bn;
      HT_TRY(gram(c, view_of_group(dd, 3, m, m), xd + L * c0, xb + L * c0, G[m], false, gpart[m] + s * slab_part,
                  gsplits[m]));
    }
  }
  if (!c.dry()) {
    for (int m = 0; m < 2; ++m) {
      HT_CUDA(reduce_partials_launch(gpart[m], ggen[m], static_cast<int>(S) * gsplits[m], ggen[m].bn, G[m], a.dims[m],
                                     1, c.st));
      ++c.launches;
    }
    HT_CUDA(sumsq_finish_launch(parts, static_cast<int>(S * np_conv), dsum, c.st));
    ++c.launches;
  }
  tl.mark(c.st);
  HT_TRY(decompose_core(c, T, cfg, xd, xb, xbt, lb, a.dims, a.order, res, tl, G));
  for (int t = 0; t < T.n_nodes; ++t) {
    float *dst = T.leaf(t) ? a.U[t] : a.B[t];
    const float *src = T.leaf(t) ? res.U[t] : res.B[t];
    if (!dst) continue;
    if (c.defer_io) {
      if (c.copy_out) c.copy_out->push_back(CopySeg{src, dst, static_cast<long long>(factor_count(T, a.dims, t))});
    } else if (!c.dry()) {
      HT_CUDA(cudaMemcpyAsync(dst, src, factor_count(T, a.dims, t) * sizeof(float), cudaMemcpyDefault, c.st));
    }
  }
  c.stage = 3;
  if (a.want_err) HT_TRY(error_core(c, T, xd, a.dims, a.order, res.U, res.B, dsum + 1));
  return HT_OK;
}

ht_status_t run_call(Ctx &c, const Tree &T, const ht_config_t &cfg, const CallArgs &a, ht_report_t *rep) {
  long long total = 1;
  for (int m = 0; m < a.order; ++m) total *= a.dims[m];
  // the call's status block, read back in one copy: ||X||^2 and the error
  // pass's sum (8 doubles, bytes 0-63), the error word (64 ints, 64-319) and
  // the leaf eigen residuals (8 floats, 320-351)
  char *status = reinterpret_cast<char *>(c.ar.take<double>(kStatusBytes / sizeof(double)));
  double *nparts = c.ar.take<double>(1024);
  if (!status || !nparts) return fail(HT_ERR_OUT_OF_MEMORY, "workspace too small");
  double *dsum = reinterpret_cast<double *>(status);
  c.err = reinterpret_cast<int *>(status + 64);
  c.resid_slots = reinterpret_cast<float *>(status + 320);
  Timeline tl;
  tl.on = rep != nullptr && !c.dry();
  cudaEvent_t h0 = nullptr, h1 = nullptr;
  CallHostState *hs = nullptr;
  if (!c.dry()) {
    int dev = 0;
    HT_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return fail(HT_ERR_INVALID_ARG, "device index out of range");
    hs = &g_call[dev];
    if (!hs->status) HT_CUDA(cudaHostAlloc(reinterpret_cast<void **>(&hs->status), kStatusBytes, cudaHostAllocDefault));
    if (tl.on && !hs->ev_made) {
      for (int i = 0; i < 10; ++i) HT_CUDA(cudaEventCreate(&hs->ev[i]));
      hs->ev_made = true;
    }
    if (tl.on) {
      for (int i = 0; i < 8; ++i) tl.ev[i] = hs->ev[i];
      h0 = hs->ev[8];
      h1 = hs->ev[9];
    }
  }
  if (!c.dry()) HT_CUDA(cudaMemsetAsync(c.err, 0, sizeof(int), c.st));
  if (tl.on) HT_CUDA(cudaEventRecord(h0, c.st));
  Result res;
  if (pipelined_input(c, a, cfg)) {
    if (a.x_dev && tl.on) HT_CUDA(cudaEventRecord(h1, c.st));
    tl.mark(c.st);
    HT_TRY(enqueue_pipelined(c, T, cfg, a, dsum, tl, res, tl.on ? h1 : nullptr));
  } else {
    const float *xd = a.x;
    if (!a.x_dev) {
      float *t = c.ar.take<float>(static_cast<size_t>(total));
      if (!t) return fail(HT_ERR_OUT_OF_MEMORY, "workspace too small (tensor)");
      if (!c.dry()) HT_CUDA(cudaMemcpyAsync(t, a.x, sizeof(float) * total, cudaMemcpyHostToDevice, c.st));
      xd = t;
    }
    if (tl.on) HT_CUDA(cudaEventRecord(h1, c.st));
    tl.mark(c.st);
    HT_TRY(enqueue_body(c, T, cfg, xd, a, nparts, dsum, tl, res));
  }
  if (c.dry()) return HT_OK;
  HT_CUDA(cudaMemcpyAsync(hs->status, status, kStatusBytes, cudaMemcpyDeviceToHost, c.st));
  HT_CUDA(cudaStreamSynchronize(c.st));
  HT_CUDA(cudaGetLastError());
  double host_sums[2] = {0.0, 0.0};
  std::memcpy(host_sums, hs->status, sizeof(double) * (a.want_err ? 2 : 1));
  int errword = 0;
  std::memcpy(&errword, hs->status + 64, sizeof(int));
  float resid[HT_MAX_NODES] = {};
  for (int t = 0; t < T.n_nodes; ++t)
    if (T.leaf(t) && res.resid[t]) std::memcpy(&resid[t], hs->status + 320 + sizeof(float) * t, sizeof(float));
  if (errword & kErrTimeout) return fail(HT_ERR_TIMEOUT, "a kernel's bounded wait expired; results are invalid");
  if (!std::isfinite(host_sums[0])) return fail(HT_ERR_NUMERICAL, "input tensor contains NaN or Inf");
  if (errword & kErrBreakdown) return fail(HT_ERR_NUMERICAL, "a factorisation broke down (non-orthonormal basis)");
  // X^ is X projected onto the tensor product of orthonormal node bases, so
  // ||X - X^|| <= ||X||: a larger error means a basis is not orthonormal
  if (a.want_err && host_sums[0] > 0 && !(host_sums[1] <= host_sums[0] * (1.0 + 1e-3)))
    return fail(HT_ERR_NUMERICAL, "relative error above 1: a node basis is not orthonormal");
  if (rep) {
    std::memset(rep, 0, sizeof(*rep));
    rep->norm_x = std::sqrt(host_sums[0]);
    rep->rel_err = a.want_err ? (host_sums[0] > 0 ? std::sqrt(std::max(host_sums[1], 0.0) / host_sums[0]) : 0.0) : -1.0;
    float ms = 0.f;
    if (tl.on) {
      cudaEventElapsedTime(&ms, h0, h1);
      rep->ms_stage[6] = ms;
      // marks: 0 start, 1 input ready, 2 grams, 3 eig, 4 core pass, 5 transfer
      for (int i = 1; i < tl.n && i <= 5; ++i) {
        cudaEventElapsedTime(&ms, tl.ev[i - 1], tl.ev[i]);
        rep->ms_stage[i - 1] = ms;
      }
      if (tl.n >= 2) {
        cudaEventElapsedTime(&ms, tl.ev[0], tl.ev[std::min(tl.n, 6) - 1]);
        rep->ms_total = ms;
      }
    }
    for (int t = 0; t < T.n_nodes; ++t) rep->eig_residual[t] = resid[t];
    rep->gpu_launches = c.launches;
    rep->path_flags = c.path;
  }
  g_launches += static_cast<unsigned long long>(c.launches);
  if (rep && cfg.eig_tol > 0.0)
    for (int t = 0; t < T.n_nodes; ++t)
      if (T.leaf(t) && rep->eig_residual[t] > cfg.eig_tol)
        return fail(HT_ERR_NOT_CONVERGED, "eigen-solver residual above eig_tol at leaf " + std::to_string(t));
  return HT_OK;
}

size_t dry_run_bytes(const Tree &T, const ht_config_t &cfg, const CallArgs &a, int eig_mode = 0) {
  Ctx d;
  d.ar.dry = true;
  d.eig_mode = eig_mode;
  d.tc = cfg.precision == HT_PREC_BF16;
  run_call(d, T, cfg, a, nullptr);
  return d.ar.peak + (1 << 20);
}

// ------------------------------------------------------------ batched path
constexpr int kLanes = 32;          // streams a batch may be spread over (at most)
constexpr int kDefaultLanes = 16;

// Launch shape of the batched path, per device: lanes (concurrent streams) and
// the cap on each lane's cooperative eigen-solver grid (0: SMs / lanes, at
// least 8).  Set by ht_batch_set_tuning (an autotuner's table), read per call.
struct BatchTuning {
  int lanes = kDefaultLanes;
  int eig_ctas = 0;
};
BatchTuning g_batch_tuning[64];

struct BatchState {
  std::vector<unsigned long long> key;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  void *ws = nullptr;
  size_t ws_bytes = 0;
  cudaStream_t lane[kLanes] = {};
  cudaStream_t cap = nullptr;   // capture origin (the caller's stream may be the legacy stream)
  cudaEvent_t fork = nullptr, join[kLanes] = {}, t0 = nullptr, t1 = nullptr;
  cudaEvent_t tp[5] = {};   // grouped mode: ends of the first five phases (ms_phase)

  bool grouped = false;
  double *sums = nullptr;   // device: [count][2] (||X||^2, ||X - Xhat||^2)
  int *errw = nullptr;      // device: one error word per lane
  int launches = 0, lanes = 0;
  void *table = nullptr;    // device: the grouped leaf solver's problem table
  size_t table_bytes = 0;
  void *conv = nullptr;     // device: grouped conversion jobs
  size_t conv_bytes = 0;
  void *copies = nullptr;   // device: grouped output copies
  size_t copies_bytes = 0;
  void *grams = nullptr;    // device: grouped Gram items, class 0 then class 1
  size_t grams_bytes = 0;
  void *tails = nullptr;    // device: grouped transfer tails
  size_t tails_bytes = 0;
  void *errs = nullptr;     // device: grouped error passes
  size_t errs_bytes = 0;
  void *maps = nullptr;     // device: block -> job maps of the grouped conversion, step-2 and error launches
  size_t maps_bytes = 0;
  void *core = nullptr;     // device: grouped core-pass GEMM parameters, then their tiles (group 0, group 1)
  size_t core_bytes = 0;
  void *step2 = nullptr;    // device: grouped step-2 jobs
  size_t step2_bytes = 0;
  void *narrow = nullptr;   // device: grouped narrow mode products
  size_t narrow_bytes = 0;
  void *t1jobs = nullptr;   // device: grouped first core contractions
  size_t t1jobs_bytes = 0;
};

// Workspace layout of one batch.  Per-lane mode: tensor i runs in lane
// i % lanes's region (lane_bytes each), after the previous tensor of that
// lane.  Grouped mode: tensor i has the region [off[i], off[i + 1]) of its
// own, so that its state survives between the two phases around the grouped
// leaf solver (nprob problems, iters / refine as every tensor's leaf_eigs).
struct BatchLayout {
  bool grouped = false;
  size_t lane_bytes = 0;
  std::vector<size_t> off;
  int nprob = 0, iters = 0, refine = 0;
  int nconv = 0, conv_blocks = 0, ncopy = 0;   // grouped conversion jobs (their blocks), output copies
  int ngram[2] = {0, 0};                       // grouped Grams per class
  int ntail = 0, nerr = 0;                     // grouped transfer tails and error passes
  int err_blocks[6] = {};                      // launch sizes of the error steps
  int err_narrow_kb = 0, err_narrow_kq = 0;    // widest kc and kq of the narrow error jobs
  size_t map_off[8] = {};                      // ints into BatchState::maps: conversion, step 2, error steps 0-5
  int ncore_blocks[2] = {0, 0}, nstep2_blocks = 0;   // grouped core pass: GEMM tiles per group, step-2 blocks
  size_t core_params = 0;                      // bytes of GEMM parameters before the tiles in BatchState::core
  int nnarrow_blocks = 0, narrow_kb = 0, nt1_blocks = 0, t1_kp = 0;   // narrow mode products (widest kz), T1 (widest kp)
  size_t map_narrow = 0, map_t1 = 0;           // their block -> job maps in BatchState::maps
};
// Leaves of at most this size go through the grouped solver (one CTA each);
// batches with larger modes keep the per-lane cooperative solver.
constexpr long kGroupedMaxN = 512;
BatchState g_batch[64];
std::mutex g_batch_mutex;

void batch_drop_graph(BatchState &b) {
  if (b.exec) cudaGraphExecDestroy(b.exec);
  if (b.graph) cudaGraphDestroy(b.graph);
  b.exec = nullptr;
  b.graph = nullptr;
  b.key.clear();
}

ht_status_t batch_streams(BatchState &b) {
  if (b.fork) return HT_OK;
  for (int l = 0; l < kLanes; ++l) {
    HT_CUDA(cudaStreamCreateWithFlags(&b.lane[l], cudaStreamNonBlocking));
    HT_CUDA(cudaEventCreateWithFlags(&b.join[l], cudaEventDisableTiming));
  }
  HT_CUDA(cudaStreamCreateWithFlags(&b.cap, cudaStreamNonBlocking));
  HT_CUDA(cudaEventCreateWithFlags(&b.fork, cudaEventDisableTiming));
  HT_CUDA(cudaEventCreate(&b.t0));
  HT_CUDA(cudaEventCreate(&b.t1));
  for (int i = 0; i < 5; ++i) HT_CUDA(cudaEventCreate(&b.tp[i]));

  return HT_OK;
}

// Host-side tables of a grouped batch, filled by its plan pass.
struct BatchPlanOut {
  std::vector<unsigned char> table;          // grouped leaf solver problems
  std::vector<ConvJob> conv;
  std::vector<CopySeg> copies;
  std::vector<unsigned char> grams[2];       // grouped Gram items by class
  std::vector<TailJob> tails;
  std::vector<ErrJob> errs;
  std::vector<SParamsBlob> core_gemms;
  std::vector<SimtBlockBlob> core_blocks[2];
  std::vector<Step2Job> step2;
  std::vector<NarrowJob> narrow;
  std::vector<T1Job> t1;
  int iters = 0, refine = 0;
};

// One pass over every tensor of the batch.  phase 0: the whole chain of each
// tensor (per-lane mode); 1, 2, 3: the tensor's launches of stage 0 (up to the
// leaf Grams), stage 1 (after the leaf solver) or stage 3 (the error pass);
// 4: no launches, the grouped stages' tables are filled into *plan_out (host
// only).  Phases 0-3 run on the lanes, forked from and joined back into `st`.
ht_status_t batch_pass(BatchState &b, const BatchLayout &L, int phase, cudaStream_t st, int count,
                       const float *const *x, const long *dims, int order, const std::vector<Tree> &trees,
                       const ht_config_t &cfg, float *const *U, float *const *B, bool want_err, int eig_ctas,
                       BatchPlanOut *plan_out = nullptr) {
  const bool plan = phase == 4;
  if (!plan) {
    HT_CUDA(cudaEventRecord(b.fork, st));
    for (int l = 0; l < b.lanes; ++l) HT_CUDA(cudaStreamWaitEvent(b.lane[l], b.fork, 0));
  }
  for (int i = 0; i < count; ++i) {
    const int l = i % b.lanes;
    Ctx c;
    c.st = b.lane[l];
    c.tc = cfg.precision == HT_PREC_BF16;
    c.eig_ctas = eig_ctas;
    c.err = b.errw + l;
    if (L.grouped) {
      c.ar.base = static_cast<char *>(b.ws) + L.off[i];
      c.ar.cap = L.off[i + 1] - L.off[i];
      c.eig_mode = plan ? 1 : 2;
      c.live = plan ? 0u : (phase == 1 ? 1u : (phase == 2 ? 2u : 8u));
      c.defer_io = true;
      if (plan) {
        c.eig_table = &plan_out->table;
        c.tail_out = &plan_out->tails;
        c.err_out = &plan_out->errs;
        c.conv_out = &plan_out->conv;
        c.copy_out = &plan_out->copies;
        c.gram_out[0] = &plan_out->grams[0];
        c.gram_out[1] = &plan_out->grams[1];
        c.core_gemms = &plan_out->core_gemms;
        c.core_blocks[0] = &plan_out->core_blocks[0];
        c.core_blocks[1] = &plan_out->core_blocks[1];
        c.step2_out = &plan_out->step2;
        c.narrow_out = &plan_out->narrow;
        c.t1_out = &plan_out->t1;
      }
    } else {
      c.ar.base = static_cast<char *>(b.ws) + static_cast<size_t>(l) * L.lane_bytes;
      c.ar.cap = L.lane_bytes;
    }
    double *nparts = c.ar.take<double>(1024);
    if (!nparts) return fail(HT_ERR_OUT_OF_MEMORY, "batch workspace too small");
    CallArgs a{x[i], true, dims + static_cast<size_t>(i) * order, order, U + static_cast<size_t>(i) * HT_MAX_NODES,
               B + static_cast<size_t>(i) * HT_MAX_NODES, want_err};
    Timeline tl;
    Result res;
    HT_TRY(enqueue_body(c, trees[i], cfg, x[i], a, nparts, b.sums + 2 * static_cast<size_t>(i), tl, res));
    b.launches += c.launches;
    if (plan) {
      plan_out->iters = c.eig_iters_used;
      plan_out->refine = c.eig_refine_used;
    }
  }
  if (!plan) {
    for (int l = 0; l < b.lanes; ++l) {
      HT_CUDA(cudaEventRecord(b.join[l], b.lane[l]));
      HT_CUDA(cudaStreamWaitEvent(st, b.join[l], 0));
    }
  }
  return HT_OK;
}

// Enqueue the whole batch on `st`.  Grouped mode: one conversion launch, the
// grouped Grams, one launch of the grouped leaf solver for every leaf of every
// tensor (tables uploaded beforehand by batch_plan_grouped), the core pass
// (grouped for 3rd order, on the lanes for 4th), the grouped transfer tails
// and error passes, and one copy of every factor to the caller's buffers.
ht_status_t batch_enqueue(BatchState &b, const BatchLayout &L, cudaStream_t st, int count, const float *const *x,
                          const long *dims, int order, const std::vector<Tree> &trees, const ht_config_t &cfg,
                          float *const *U, float *const *B, bool want_err, int eig_ctas) {
  HT_CUDA(cudaMemsetAsync(b.errw, 0, sizeof(int) * kLanes, st));
  b.launches = 0;
  if (!L.grouped) return batch_pass(b, L, 0, st, count, x, dims, order, trees, cfg, U, B, want_err, eig_ctas);
  const int *maps = static_cast<const int *>(b.maps);
  HT_CUDA(convert_grouped_launch(static_cast<const ConvJob *>(b.conv), L.nconv, L.conv_blocks, maps + L.map_off[0], st));
  b.launches += L.nconv > 0 ? 2 : 0;
  HT_CUDA(tc_gram_grouped_launch(0, b.grams, L.ngram[0], st));
  HT_CUDA(tc_gram_grouped_launch(1, static_cast<char *>(b.grams) + tc_gram_item_bytes() * L.ngram[0], L.ngram[1], st));
  b.launches += (L.ngram[0] > 0) + (L.ngram[1] > 0);
  HT_TRY(batch_pass(b, L, 1, st, count, x, dims, order, trees, cfg, U, B, want_err, eig_ctas));
  // external records: inside a capture they become event-record nodes of the graph
  HT_CUDA(cudaEventRecordWithFlags(b.tp[0], st, cudaEventRecordExternal));
  HT_CUDA(eig_grouped_launch(b.table, L.nprob, L.iters, L.refine, st));
  HT_CUDA(cudaEventRecordWithFlags(b.tp[1], st, cudaEventRecordExternal));
  b.launches += 1;
  if (L.nstep2_blocks > 0) {   // 3rd order: the grouped core pass
    const SParamsBlob *params = static_cast<const SParamsBlob *>(b.core);
    const SimtBlockBlob *tiles =
        reinterpret_cast<const SimtBlockBlob *>(static_cast<const char *>(b.core) + L.core_params);
    HT_CUDA(modeprod_narrow_grouped_launch(static_cast<const NarrowJob *>(b.narrow), maps + L.map_narrow,
                                           L.nnarrow_blocks, L.narrow_kb, st));
    HT_CUDA(simt_grouped_launch(params, tiles, L.ncore_blocks[0], st));
    HT_CUDA(core_t1_grouped_launch(static_cast<const T1Job *>(b.t1jobs), maps + L.map_t1, L.nt1_blocks, L.t1_kp, st));
    HT_CUDA(simt_grouped_launch(params, tiles + L.ncore_blocks[0], L.ncore_blocks[1], st));
    HT_CUDA(core_step2_grouped_launch(static_cast<const Step2Job *>(b.step2), maps + L.map_off[1], L.nstep2_blocks,
                                      st));
    b.launches += (L.nnarrow_blocks > 0) + (L.ncore_blocks[0] > 0) + (L.nt1_blocks > 0) + (L.ncore_blocks[1] > 0) + 1;
  }
  HT_TRY(batch_pass(b, L, 2, st, count, x, dims, order, trees, cfg, U, B, want_err, eig_ctas));
  HT_CUDA(cudaEventRecordWithFlags(b.tp[2], st, cudaEventRecordExternal));
  HT_CUDA(transfer_tail_grouped_launch(static_cast<const TailJob *>(b.tails), L.ntail, st));
  b.launches += L.ntail > 0 ? 1 : 0;
  HT_CUDA(cudaEventRecordWithFlags(b.tp[3], st, cudaEventRecordExternal));
  if (L.nerr > 0) {
    const int *emaps[6];
    for (int k = 0; k < 6; ++k) emaps[k] = maps + L.map_off[2 + k];
    HT_CUDA(error_grouped_launch(static_cast<const ErrJob *>(b.errs), L.nerr, L.err_blocks, emaps, L.err_narrow_kb,
                                 L.err_narrow_kq, st));
    for (int k = 0; k < 6; ++k) b.launches += L.err_blocks[k] > 0 ? 1 : 0;
    b.launches += 1;
  }
  HT_TRY(batch_pass(b, L, 3, st, count, x, dims, order, trees, cfg, U, B, want_err, eig_ctas));
  HT_CUDA(cudaEventRecordWithFlags(b.tp[4], st, cudaEventRecordExternal));
  HT_CUDA(copy_segments_launch(static_cast<const CopySeg *>(b.copies), L.ncopy, st));
  b.launches += L.ncopy > 0 ? 1 : 0;
  return HT_OK;
}

// Copy a host table into a device buffer that grows as needed.
ht_status_t upload_table(void *&buf, size_t &cap, const void *data, size_t bytes) {
  if (bytes > cap) {
    if (buf) HT_CUDA(cudaFree(buf));
    buf = nullptr;
    cap = 0;
    HT_CUDA(cudaMalloc(&buf, bytes));
    cap = bytes;
  }
  if (bytes) HT_CUDA(cudaMemcpy(buf, data, bytes, cudaMemcpyHostToDevice));
  return HT_OK;
}

// Host-only pass that lays out every leaf problem of the batch for the
// grouped solver and copies the table to the device (outside any capture).
ht_status_t batch_plan_grouped(BatchState &b, BatchLayout &L, int count, const float *const *x, const long *dims,
                               int order, const std::vector<Tree> &trees, const ht_config_t &cfg, float *const *U,
                               float *const *B, bool want_err) {
  BatchPlanOut P;
  const int launches = b.launches;
  HT_TRY(batch_pass(b, L, 4, nullptr, count, x, dims, order, trees, cfg, U, B, want_err, 0, &P));
  b.launches = launches;
  // block -> job maps: the conversion, the core pass's step 2, the four error steps
  std::vector<int> maps;
  int blk = 0;
  for (size_t j = 0; j < P.conv.size(); ++j) {
    P.conv[j].blk0 = blk;
    blk += P.conv[j].nblk;
    maps.insert(maps.end(), P.conv[j].nblk, static_cast<int>(j));
  }
  L.map_off[0] = 0;
  L.nconv = static_cast<int>(P.conv.size());
  L.conv_blocks = blk;
  L.map_off[1] = maps.size();
  blk = 0;
  for (size_t j = 0; j < P.step2.size(); ++j) {
    P.step2[j].blk0 = blk;
    blk += P.step2[j].kc;
    maps.insert(maps.end(), P.step2[j].kc, static_cast<int>(j));
  }
  L.nstep2_blocks = blk;
  L.map_narrow = maps.size();
  blk = 0;
  L.narrow_kb = 0;
  for (size_t j = 0; j < P.narrow.size(); ++j) {
    P.narrow[j].blk0 = blk;
    blk += P.narrow[j].nblk;
    maps.insert(maps.end(), P.narrow[j].nblk, static_cast<int>(j));
    L.narrow_kb = std::max(L.narrow_kb, P.narrow[j].kz);
  }
  L.nnarrow_blocks = blk;
  L.map_t1 = maps.size();
  blk = 0;
  for (size_t j = 0; j < P.t1.size(); ++j) {
    P.t1[j].blk0 = blk;
    blk += P.t1[j].nblk;
    L.t1_kp = std::max(L.t1_kp, P.t1[j].kp);
    maps.insert(maps.end(), P.t1[j].nblk, static_cast<int>(j));
  }
  L.nt1_blocks = blk;
  HT_TRY(upload_table(b.narrow, b.narrow_bytes, P.narrow.data(), sizeof(NarrowJob) * P.narrow.size()));
  HT_TRY(upload_table(b.t1jobs, b.t1jobs_bytes, P.t1.data(), sizeof(T1Job) * P.t1.size()));
  for (int k = 0; k < 6; ++k) {
    L.map_off[2 + k] = maps.size();
    int eb = 0;
    for (size_t i = 0; i < P.errs.size(); ++i) {
      P.errs[i].blk0[k] = eb;
      eb += P.errs[i].nblk[k];
      maps.insert(maps.end(), P.errs[i].nblk[k], static_cast<int>(i));
    }
    L.err_blocks[k] = eb;
  }
  L.err_narrow_kb = L.err_narrow_kq = 0;
  for (const ErrJob &j : P.errs)
    if (j.narrow) {
      L.err_narrow_kb = std::max(L.err_narrow_kb, j.kc);
      L.err_narrow_kq = std::max(L.err_narrow_kq, j.kq);
    }
  L.nerr = static_cast<int>(P.errs.size());
  L.ntail = static_cast<int>(P.tails.size());
  // core pass: the GEMM parameters, then group 0's tiles, then group 1's
  L.ncore_blocks[0] = static_cast<int>(P.core_blocks[0].size());
  L.ncore_blocks[1] = static_cast<int>(P.core_blocks[1].size());
  L.core_params = sizeof(SParamsBlob) * P.core_gemms.size();
  std::vector<unsigned char> core(L.core_params + sizeof(SimtBlockBlob) * (L.ncore_blocks[0] + L.ncore_blocks[1]));
  if (!core.empty()) {
    std::memcpy(core.data(), P.core_gemms.data(), L.core_params);
    std::memcpy(core.data() + L.core_params, P.core_blocks[0].data(), sizeof(SimtBlockBlob) * L.ncore_blocks[0]);
    std::memcpy(core.data() + L.core_params + sizeof(SimtBlockBlob) * L.ncore_blocks[0], P.core_blocks[1].data(),
                sizeof(SimtBlockBlob) * L.ncore_blocks[1]);
  }
  HT_TRY(upload_table(b.core, b.core_bytes, core.data(), core.size()));
  HT_TRY(upload_table(b.step2, b.step2_bytes, P.step2.data(), sizeof(Step2Job) * P.step2.size()));
  L.ngram[0] = static_cast<int>(P.grams[0].size() / tc_gram_item_bytes());
  L.ngram[1] = static_cast<int>(P.grams[1].size() / tc_gram_item_bytes());
  P.grams[0].insert(P.grams[0].end(), P.grams[1].begin(), P.grams[1].end());
  eig_grouped_order(P.table);
  L.nprob = static_cast<int>(P.table.size() / eig_grouped_entry_bytes());
  L.iters = P.iters;
  L.refine = P.refine;
  L.ncopy = static_cast<int>(P.copies.size());
  HT_TRY(upload_table(b.maps, b.maps_bytes, maps.data(), sizeof(int) * maps.size()));
  HT_TRY(upload_table(b.errs, b.errs_bytes, P.errs.data(), sizeof(ErrJob) * P.errs.size()));
  HT_TRY(upload_table(b.tails, b.tails_bytes, P.tails.data(), sizeof(TailJob) * P.tails.size()));
  HT_TRY(upload_table(b.grams, b.grams_bytes, P.grams[0].data(), P.grams[0].size()));
  HT_TRY(upload_table(b.table, b.table_bytes, P.table.data(), P.table.size()));
  HT_TRY(upload_table(b.conv, b.conv_bytes, P.conv.data(), sizeof(ConvJob) * P.conv.size()));
  HT_TRY(upload_table(b.copies, b.copies_bytes, P.copies.data(), sizeof(CopySeg) * P.copies.size()));
  return HT_OK;
}

}  // namespace

// ====================================================================== C ABI
extern "C" {

ht_status_t ht_config_default(ht_config_t *cfg) {
  if (!cfg) return fail(HT_ERR_INVALID_ARG, "cfg is NULL");
  std::memset(cfg, 0, sizeof(*cfg));
  cfg->precision = HT_PREC_BF16;
  cfg->leaf_method = HT_LEAF_GRAM;
  cfg->oversample = 16;
  cfg->eig_iters = 0;
  cfg->power_steps = 1;
  cfg->seed = 1234ull;
  return HT_OK;
}

static void fill_tree(ht_tree_t *t, int order, const int *mask, const int *left, const int *right, const int *k) {
  std::memset(t, 0, sizeof(*t));
  t->order = order;
  t->n_nodes = 2 * order - 1;
  for (int i = 0; i < HT_MAX_NODES; ++i) t->parent[i] = t->left[i] = t->right[i] = -1;
  for (int i = 0; i < t->n_nodes; ++i) {
    t->mode_mask[i] = mask[i];
    t->left[i] = left[i];
    t->right[i] = right[i];
    t->rank[i] = (i == 0) ? 1 : (k ? k[i] : 1);
  }
  for (int i = 0; i < t->n_nodes; ++i)
    if (left[i] >= 0) {
      t->parent[left[i]] = i;
      t->parent[right[i]] = i;
    }
}

ht_status_t ht_tree_reference_3d(ht_tree_t *tree, const int *k) {
  if (!tree) return fail(HT_ERR_INVALID_ARG, "tree is NULL");
  const int mask[5] = {7, 3, 4, 1, 2};
  const int left[5] = {1, 3, -1, -1, -1};
  const int right[5] = {2, 4, -1, -1, -1};
  fill_tree(tree, 3, mask, left, right, k);
  return HT_OK;
}

ht_status_t ht_tree_balanced_4d(ht_tree_t *tree, const int *k) {
  if (!tree) return fail(HT_ERR_INVALID_ARG, "tree is NULL");
  const int mask[7] = {15, 3, 12, 1, 2, 4, 8};
  const int left[7] = {1, 3, 5, -1, -1, -1, -1};
  const int right[7] = {2, 4, 6, -1, -1, -1, -1};
  fill_tree(tree, 4, mask, left, right, k);
  return HT_OK;
}

ht_status_t ht_tree_validate(const ht_tree_t *tree, const long *dims, int order) {
  if (!dims) return fail(HT_ERR_INVALID_ARG, "dims is NULL");
  Tree T;
  return parse_tree(tree, dims, order, T);
}

ht_status_t ht_workspace_size(const long *dims, int order, const ht_tree_t *tree, const ht_config_t *cfg,
                              unsigned long long *bytes) {
  if (!dims || !bytes) return fail(HT_ERR_INVALID_ARG, "NULL argument");
  Tree T;
  HT_TRY(parse_tree(tree, dims, order, T));
  ht_config_t def;
  ht_config_default(&def);
  float *none[HT_MAX_NODES] = {};
  CallArgs a{nullptr, true, dims, order, none, none, cfg ? (cfg->flags & HT_FLAG_COMPUTE_ERROR) != 0 : false};
  *bytes = dry_run_bytes(T, cfg ? *cfg : def, a);
  return HT_OK;
}

ht_status_t ht_release_workspace(void) {
  std::lock_guard<std::mutex> lk(g_ws_mutex);
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return HT_OK;
  }
  if (dev >= 0 && dev < 64 && g_ws[dev].ptr) {
    HT_CUDA(cudaDeviceSynchronize());
    HT_CUDA(cudaFree(g_ws[dev].ptr));
    g_ws[dev].ptr = nullptr;
    g_ws[dev].bytes = 0;
  }
  return HT_OK;
}

// Workspace bytes of a single-tensor call, from the cache of recent call
// signatures on this device or a dry run.  The signature holds everything the
// dry run's plan depends on: the device, the dims, the tree, the configuration
// (its sketch blocks as absent / host / device), where X lives and its 16-byte
// alignment, and whether the error pass runs.  Call with g_ws_mutex held.
ht_status_t sized_call_bytes(const Tree &T, const ht_config_t &cfg, const CallArgs &a, size_t *bytes) {
  int dev = 0;
  HT_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(HT_ERR_INVALID_ARG, "device index out of range");
  long long key[64];
  int n = 0;
  key[n++] = dev;
  key[n++] = a.order;
  for (int m = 0; m < a.order; ++m) key[n++] = a.dims[m];
  key[n++] = T.n_nodes;
  for (int t = 0; t < T.n_nodes; ++t)
    key[n++] = (static_cast<long long>(T.left[t] + 1) << 48) | (static_cast<long long>(T.right[t] + 1) << 40) |
               (static_cast<long long>(T.mask[t]) << 32) | static_cast<unsigned>(T.rank[t]);
  key[n++] = cfg.precision;
  key[n++] = cfg.leaf_method;
  key[n++] = cfg.oversample;
  key[n++] = cfg.eig_iters;
  key[n++] = cfg.power_steps;
  key[n++] = cfg.flags;
  for (int m = 0; m < a.order; ++m) key[n++] = cfg.sketch[m] ? (is_device_ptr(cfg.sketch[m]) ? 2 : 1) : 0;
  key[n++] = a.x_dev;
  key[n++] = static_cast<long long>(reinterpret_cast<uintptr_t>(a.x) & 15u);
  key[n++] = a.want_err;
  const std::string k(reinterpret_cast<const char *>(key), sizeof(long long) * n);
  auto &cache = g_call[dev].sizes;
  for (const auto &e : cache)
    if (e.first == k) {
      *bytes = e.second;
      return HT_OK;
    }
  *bytes = dry_run_bytes(T, cfg, a);
  if (cache.size() >= 64) cache.erase(cache.begin());
  cache.emplace_back(k, *bytes);
  return HT_OK;
}

ht_status_t ht_decompose(const float *x, const long *dims, int order, const ht_tree_t *tree, const ht_config_t *cfg_in,
                         float *const *U, float *const *B, ht_report_t *report, void *stream) {
  if (!x || !dims || !U || !B) return fail(HT_ERR_INVALID_ARG, "NULL argument");
  Tree T;
  HT_TRY(parse_tree(tree, dims, order, T));
  ht_config_t cfg;
  if (cfg_in) cfg = *cfg_in;
  else ht_config_default(&cfg);
  if (cfg.precision != HT_PREC_FP32 && cfg.precision != HT_PREC_BF16) return fail(HT_ERR_INVALID_ARG, "unknown precision");
  if (cfg.leaf_method != HT_LEAF_GRAM && cfg.leaf_method != HT_LEAF_SKETCH)
    return fail(HT_ERR_INVALID_ARG, "unknown leaf method");
  if (cfg.oversample < 0 || cfg.eig_iters < 0) return fail(HT_ERR_INVALID_ARG, "negative oversample / eig_iters");
  for (int t = 0; t < T.n_nodes; ++t) {
    if (T.leaf(t) && !U[t]) return fail(HT_ERR_INVALID_ARG, "U[t] is NULL for leaf " + std::to_string(t));
    if (!T.leaf(t) && !B[t]) return fail(HT_ERR_INVALID_ARG, "B[t] is NULL for interior node " + std::to_string(t));
  }
  HT_TRY(check_device());
  std::lock_guard<std::mutex> lk(g_ws_mutex);
  CallArgs a{x, is_device_ptr(x), dims, order, U, B, (cfg.flags & HT_FLAG_COMPUTE_ERROR) != 0};
  size_t bytes = 0;
  HT_TRY(sized_call_bytes(T, cfg, a, &bytes));
  void *ws = nullptr;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  HT_TRY(acquire_workspace(bytes, &ws, st));
  Ctx c;
  c.st = st;
  c.tc = cfg.precision == HT_PREC_BF16;
  c.ar.base = static_cast<char *>(ws);
  c.ar.cap = bytes;
  return run_call(c, T, cfg, a, report);
}

ht_status_t ht_decompose_streaming(const float *x, const long *dims, int order, const ht_tree_t *tree,
                                   const ht_config_t *cfg_in, float *const *U, float *const *B,
                                   unsigned long long slab_bytes, ht_report_t *report, void *stream) {
  if (!x || !dims || !U || !B) return fail(HT_ERR_INVALID_ARG, "NULL argument");
  if (order != 3) return fail(HT_ERR_UNSUPPORTED, "the streaming path handles 3rd-order tensors");
  Tree T;
  HT_TRY(parse_tree(tree, dims, order, T));
  ht_config_t cfg;
  if (cfg_in) cfg = *cfg_in;
  else ht_config_default(&cfg);
  if (cfg.precision != HT_PREC_FP32 && cfg.precision != HT_PREC_BF16) return fail(HT_ERR_INVALID_ARG, "unknown precision");
  if (cfg.leaf_method == HT_LEAF_SKETCH)
    return fail(HT_ERR_UNSUPPORTED, "the streaming path computes leaf Grams; HT_LEAF_SKETCH runs in ht_decompose");
  if (cfg.leaf_method != HT_LEAF_GRAM) return fail(HT_ERR_INVALID_ARG, "unknown leaf method");
  if (cfg.oversample < 0 || cfg.eig_iters < 0) return fail(HT_ERR_INVALID_ARG, "negative oversample / eig_iters");
  for (int t = 0; t < T.n_nodes; ++t) {
    if (T.leaf(t) && !U[t]) return fail(HT_ERR_INVALID_ARG, "U[t] is NULL for leaf " + std::to_string(t));
    if (!T.leaf(t) && !B[t]) return fail(HT_ERR_INVALID_ARG, "B[t] is NULL for interior node " + std::to_string(t));
  }
  HT_TRY(check_device());
  if (is_device_ptr(x)) return fail(HT_ERR_INVALID_ARG, "the streaming path reads x from host memory; use ht_decompose");
  // slab lengths: two FP32 slab buffers within slab_bytes, multiples of 8 where possible
  auto slab_len = [&](long long per_index, long long extent) {
    long long len = static_cast<long long>(slab_bytes / (2ull * sizeof(float) * static_cast<unsigned long long>(per_index)));
    if (len >= 8) len -= len % 8;
    return std::max(1ll, std::min(len, extent));
  };
  StreamArgs a;
  a.xh = x;
  a.dims = dims;
  a.U = U;
  a.B = B;
  a.want_err = (cfg.flags & HT_FLAG_COMPUTE_ERROR) != 0;
  a.slab2 = slab_len(static_cast<long long>(dims[0]) * dims[1], dims[2]);
  a.slab1 = slab_len(static_cast<long long>(dims[0]) * dims[2], dims[1]);
  std::lock_guard<std::mutex> lk(g_ws_mutex);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  auto plan = [&](Ctx &c, SlabIo &io, Timeline &tl, double **dsum) -> ht_status_t {
    c.err = c.ar.take<int>(64);
    *dsum = c.ar.take<double>(8);
    if (!c.err || !*dsum) return fail(HT_ERR_OUT_OF_MEMORY, "workspace too small");
    if (!c.dry()) HT_CUDA(cudaMemsetAsync(c.err, 0, sizeof(int), c.st));
    tl.mark(c.st);
    return stream_call(c, T, cfg, a, io, tl, *dsum);
  };
  size_t bytes = 0;
  {
    Ctx d;
    d.ar.dry = true;
    d.tc = cfg.precision == HT_PREC_BF16;
    SlabIo io;
    Timeline tl;
    double *ds = nullptr;
    HT_TRY(plan(d, io, tl, &ds));
    bytes = d.ar.peak + (1 << 20);
  }
  void *ws = nullptr;
  HT_TRY(acquire_workspace(bytes, &ws, st));
  Ctx c;
  c.st = st;
  c.tc = cfg.precision == HT_PREC_BF16;
  c.ar.base = static_cast<char *>(ws);
  c.ar.cap = bytes;
  SlabIo io;
  Timeline tl;
  tl.on = report != nullptr;
  struct Cleanup {
    SlabIo &io;
    Timeline &tl;
    ~Cleanup() {
      if (io.cs) {
        cudaStreamSynchronize(io.cs);
        cudaStreamDestroy(io.cs);
      }
      for (int b = 0; b < 2; ++b) {
        if (io.copied[b]) cudaEventDestroy(io.copied[b]);
        if (io.freed[b]) cudaEventDestroy(io.freed[b]);
      }
      if (tl.on)
        for (int i = 0; i < 8; ++i)
          if (tl.ev[i]) cudaEventDestroy(tl.ev[i]);
    }
  } cleanup{io, tl};
  HT_CUDA(cudaStreamCreateWithFlags(&io.cs, cudaStreamNonBlocking));
  for (int b = 0; b < 2; ++b) {
    HT_CUDA(cudaEventCreateWithFlags(&io.copied[b], cudaEventDisableTiming));
    HT_CUDA(cudaEventCreateWithFlags(&io.freed[b], cudaEventDisableTiming));
  }
  if (tl.on)
    for (int i = 0; i < 8; ++i) HT_CUDA(cudaEventCreate(&tl.ev[i]));
  double *dsum = nullptr;
  HT_TRY(plan(c, io, tl, &dsum));
  double host_sums[2] = {0.0, 0.0};
  HT_CUDA(cudaMemcpyAsync(host_sums, dsum, sizeof(double) * (a.want_err ? 2 : 1), cudaMemcpyDeviceToHost, c.st));
  int errword = 0;
  HT_CUDA(cudaMemcpyAsync(&errword, c.err, sizeof(int), cudaMemcpyDeviceToHost, c.st));
  HT_CUDA(cudaStreamSynchronize(c.st));
  HT_CUDA(cudaGetLastError());
  g_launches += static_cast<unsigned long long>(c.launches);
  if (errword & kErrTimeout) return fail(HT_ERR_TIMEOUT, "a kernel's bounded wait expired; results are invalid");
  if (!std::isfinite(host_sums[0])) return fail(HT_ERR_NUMERICAL, "input tensor contains NaN or Inf");
  if (errword & kErrBreakdown) return fail(HT_ERR_NUMERICAL, "a factorisation broke down (non-orthonormal basis)");
  // X^ is X projected onto the tensor product of orthonormal node bases, so
  // ||X - X^|| <= ||X||: a larger error means a basis is not orthonormal
  if (a.want_err && host_sums[0] > 0 && !(host_sums[1] <= host_sums[0] * (1.0 + 1e-3)))
    return fail(HT_ERR_NUMERICAL, "relative error above 1: a node basis is not orthonormal");
  if (report) {
    std::memset(report, 0, sizeof(*report));
    report->norm_x = std::sqrt(host_sums[0]);
    report->rel_err =
        a.want_err ? (host_sums[0] > 0 ? std::sqrt(std::max(host_sums[1], 0.0) / host_sums[0]) : 0.0) : -1.0;
    // marks: 0 start, 1 pass A, 2 pass B, 3 eig, 4 pass C, 5 transfer, 6 error pass
    float ms = 0.f;
    for (int i = 1; i < tl.n && i <= 6; ++i) {
      cudaEventElapsedTime(&ms, tl.ev[i - 1], tl.ev[i]);
      report->ms_stage[i - 1] = ms;
    }
    if (tl.n >= 2) {
      cudaEventElapsedTime(&ms, tl.ev[0], tl.ev[tl.n - 1]);
      report->ms_total = ms;
    }
    report->gpu_launches = c.launches;
    report->path_flags = c.path;
  }
  return HT_OK;
}

ht_status_t ht_decompose_batched(int count, const float *const *x, const long *dims, int order,
                                 const ht_tree_t *trees, const ht_config_t *cfg_in, float *const *U, float *const *B,
                                 double *rel_err, ht_batch_report_t *report, void *stream) {
  if (count < 1 || !x || !dims || !trees || !U || !B) return fail(HT_ERR_INVALID_ARG, "NULL argument or count < 1");
  g_last_error.clear();   // after a successful call: empty, or why no graph was recorded
  ht_config_t cfg;
  if (cfg_in) cfg = *cfg_in;
  else ht_config_default(&cfg);
  if (cfg.precision != HT_PREC_FP32 && cfg.precision != HT_PREC_BF16) return fail(HT_ERR_INVALID_ARG, "unknown precision");
  if (cfg.leaf_method == HT_LEAF_SKETCH)
    return fail(HT_ERR_UNSUPPORTED, "the batched path computes leaf Grams; HT_LEAF_SKETCH runs in ht_decompose");
  if (cfg.leaf_method != HT_LEAF_GRAM) return fail(HT_ERR_INVALID_ARG, "unknown leaf method");
  if (cfg.oversample < 0 || cfg.eig_iters < 0) return fail(HT_ERR_INVALID_ARG, "negative oversample / eig_iters");
  const bool want_err = (cfg.flags & HT_FLAG_COMPUTE_ERROR) != 0;
  HT_TRY(check_device());
  int dev = 0;
  HT_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(HT_ERR_INVALID_ARG, "device index out of range");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  std::lock_guard<std::mutex> lk(g_batch_mutex);
  BatchState &b = g_batch[dev];
  const BatchTuning tune = g_batch_tuning[dev];
  // identity of the batch: shapes, trees, config, launch shape and every pointer
  std::vector<unsigned long long> key;
  key.reserve(static_cast<size_t>(count) * (order + 2 * HT_MAX_NODES + 2 + sizeof(ht_tree_t) / 4) + 16);
  key.push_back(static_cast<unsigned long long>(count));
  key.push_back(static_cast<unsigned long long>(order));
  key.push_back(static_cast<unsigned long long>(tune.lanes));
  key.push_back(static_cast<unsigned long long>(tune.eig_ctas));
  {
    const unsigned char *cb = reinterpret_cast<const unsigned char *>(&cfg);
    for (size_t q = 0; q < sizeof(cfg); ++q) key.push_back(cb[q]);
  }
  for (int i = 0; i < count; ++i) {
    key.push_back(reinterpret_cast<uintptr_t>(x[i]));
    for (int m = 0; m < order; ++m) key.push_back(static_cast<unsigned long long>(dims[static_cast<size_t>(i) * order + m]));
    const int *tw = reinterpret_cast<const int *>(&trees[i]);
    for (size_t q = 0; q < sizeof(ht_tree_t) / sizeof(int); ++q) key.push_back(static_cast<unsigned long long>(tw[q]));
    for (int t = 0; t < HT_MAX_NODES; ++t) {
      key.push_back(reinterpret_cast<uintptr_t>(U[static_cast<size_t>(i) * HT_MAX_NODES + t]));
      key.push_back(reinterpret_cast<uintptr_t>(B[static_cast<size_t>(i) * HT_MAX_NODES + t]));
    }
  }
  const bool replay = b.exec && key == b.key;
  if (!replay) {
    std::vector<Tree> T(count);
    BatchLayout L;
    L.grouped = true;
    for (int i = 0; i < count; ++i)
      for (int m = 0; m < order; ++m) L.grouped = L.grouped && dims[static_cast<size_t>(i) * order + m] <= kGroupedMaxN;
    L.off.assign(static_cast<size_t>(count) + 1, 0);
    for (int i = 0; i < count; ++i) {
      const long *di = dims + static_cast<size_t>(i) * order;
      HT_TRY(parse_tree(&trees[i], di, order, T[i]));
      if (!is_device_ptr(x[i])) return fail(HT_ERR_INVALID_ARG, "x[" + std::to_string(i) + "] must be device memory");
      for (int t = 0; t < T[i].n_nodes; ++t) {
        float *o = T[i].leaf(t) ? U[static_cast<size_t>(i) * HT_MAX_NODES + t] : B[static_cast<size_t>(i) * HT_MAX_NODES + t];
        if (!o || !is_device_ptr(o))
          return fail(HT_ERR_INVALID_ARG, "output of node " + std::to_string(t) + " of tensor " + std::to_string(i) +
                                              " must be device memory");
      }
      CallArgs a{x[i], true, di, order, U + static_cast<size_t>(i) * HT_MAX_NODES, B + static_cast<size_t>(i) * HT_MAX_NODES,
                 want_err};
      const size_t bi = (dry_run_bytes(T[i], cfg, a, L.grouped ? 1 : 0) + 1024 * sizeof(double) + 4095) & ~size_t(4095);
      L.lane_bytes = std::max(L.lane_bytes, bi);
      L.off[i + 1] = L.off[i] + bi;
    }
    batch_drop_graph(b);
    HT_TRY(batch_streams(b));
    b.lanes = std::min(tune.lanes, count);
    b.grouped = L.grouped;
    const size_t regions = L.grouped ? L.off[count] : static_cast<size_t>(b.lanes) * L.lane_bytes;
    const size_t need = regions + sizeof(double) * 2 * count + 4096;
    if (b.ws_bytes < need) {
      if (b.ws) {
        HT_CUDA(cudaDeviceSynchronize());
        HT_CUDA(cudaFree(b.ws));
        b.ws = nullptr;
        b.ws_bytes = 0;
      }
      HT_CUDA(cudaMalloc(&b.ws, need));
      b.ws_bytes = need;
    }
    char *tail = static_cast<char *>(b.ws) + regions;
    b.errw = reinterpret_cast<int *>(tail);
    b.sums = reinterpret_cast<double *>(tail + 256);
    const int eig_ctas = tune.eig_ctas > 0 ? tune.eig_ctas : std::max(8, sm_count() / b.lanes);
    HT_CUDA(tc_prepare());   // one-time kernel attributes outside the capture
    HT_CUDA(eig_prepare());
    if (L.grouped) HT_TRY(batch_plan_grouped(b, L, count, x, dims, order, T, cfg, U, B, want_err));
    // record the batch into a graph (captured from a private stream: the
    // caller's may be the legacy stream); if capture is refused, run it directly
    bool captured = false;
    std::string why;
    cudaError_t ce = cudaStreamBeginCapture(b.cap, cudaStreamCaptureModeThreadLocal);
    if (ce == cudaSuccess) {
      const ht_status_t s = batch_enqueue(b, L, b.cap, count, x, dims, order, T, cfg, U, B, want_err, eig_ctas);
      if (s != HT_OK) why = ht_last_error();
      cudaGraph_t g = nullptr;
      ce = cudaStreamEndCapture(b.cap, &g);
      cudaError_t ie = cudaErrorUnknown;
      if (s == HT_OK && ce == cudaSuccess && g) ie = cudaGraphInstantiate(&b.exec, g, 0);
      if (s == HT_OK && ce == cudaSuccess && g && ie == cudaSuccess) {
        b.graph = g;
        b.key = key;
        captured = true;
      } else {   // not capturable here (or a launch failed): run the batch directly below
        if (why.empty()) why = std::string("capture: ") + cudaGetErrorString(ce != cudaSuccess ? ce : ie);
        if (g) cudaGraphDestroy(g);
        b.exec = nullptr;
        cudaGetLastError();
      }
    } else {
      why = std::string("begin capture: ") + cudaGetErrorString(ce);
      cudaGetLastError();
    }
    if (!captured) g_last_error = "batch ran without a CUDA graph (" + why + ")";
    if (!captured) {
      HT_CUDA(cudaEventRecord(b.t0, st));
      HT_TRY(batch_enqueue(b, L, st, count, x, dims, order, T, cfg, U, B, want_err, eig_ctas));
      HT_CUDA(cudaEventRecord(b.t1, st));
    }
    if (captured) {
      HT_CUDA(cudaEventRecord(b.t0, st));
      HT_CUDA(cudaGraphLaunch(b.exec, st));
      HT_CUDA(cudaEventRecord(b.t1, st));
    }
  } else {
    HT_CUDA(cudaEventRecord(b.t0, st));
    HT_CUDA(cudaGraphLaunch(b.exec, st));
    HT_CUDA(cudaEventRecord(b.t1, st));
  }
  std::vector<double> sums(2 * static_cast<size_t>(count));
  int errw[kLanes] = {};
  HT_CUDA(cudaMemcpyAsync(sums.data(), b.sums, sizeof(double) * sums.size(), cudaMemcpyDeviceToHost, st));
  HT_CUDA(cudaMemcpyAsync(errw, b.errw, sizeof(errw), cudaMemcpyDeviceToHost, st));
  HT_CUDA(cudaStreamSynchronize(st));
  HT_CUDA(cudaGetLastError());
  for (int l = 0; l < kLanes; ++l)
    if (errw[l] & kErrTimeout) return fail(HT_ERR_TIMEOUT, "a kernel's bounded wait expired; results are invalid");
  std::vector<double> errs;
  for (int i = 0; i < count; ++i) {
    const double nx = sums[2 * static_cast<size_t>(i)], ne = sums[2 * static_cast<size_t>(i) + 1];
    if (!std::isfinite(nx)) return fail(HT_ERR_NUMERICAL, "tensor " + std::to_string(i) + " contains NaN or Inf");
    const double e = want_err ? (nx > 0 ? std::sqrt(std::max(ne, 0.0) / nx) : 0.0) : -1.0;
    if (rel_err) rel_err[i] = e;
    errs.push_back(e);
  }
  g_launches += static_cast<unsigned long long>(b.launches);
  if (report) {
    std::memset(report, 0, sizeof(*report));
    std::vector<double> sorted = errs;
    std::sort(sorted.begin(), sorted.end());
    auto rank_pct = [&](double q) {
      const size_t idx = static_cast<size_t>(std::ceil(q * sorted.size())) - 1;
      return sorted[std::min(idx, sorted.size() - 1)];
    };
    report->rel_err_p50 = want_err ? rank_pct(0.50) : -1.0;
    report->rel_err_p99 = want_err ? rank_pct(0.99) : -1.0;
    report->rel_err_max = want_err ? sorted.back() : -1.0;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, b.t0, b.t1);
    report->ms_total = ms;
    report->gpu_launches = b.launches;
    report->graph_replayed = replay ? 1 : 0;
    report->lanes = b.lanes;
    report->grouped = b.grouped ? 1 : 0;
    if (b.grouped) {
      const cudaEvent_t ev[7] = {b.t0, b.tp[0], b.tp[1], b.tp[2], b.tp[3], b.tp[4], b.t1};
      for (int i = 0; i < 6; ++i)
        if (cudaEventElapsedTime(&report->ms_phase[i], ev[i], ev[i + 1]) != cudaSuccess) {
          cudaGetLastError();   // timing unavailable: report zeros, leave no error behind
          for (int j = 0; j < 6; ++j) report->ms_phase[j] = 0.f;
          break;
        }
    }
  }
  return HT_OK;
}

ht_status_t ht_batch_set_tuning(int lanes, int eig_ctas) {
  if (lanes < 0 || lanes > kLanes || eig_ctas < 0)
    return fail(HT_ERR_INVALID_ARG, "lanes must lie in [0, " + std::to_string(kLanes) + "], eig_ctas >= 0");
  int dev = 0;
  HT_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(HT_ERR_INVALID_ARG, "device index out of range");
  std::lock_guard<std::mutex> lk(g_batch_mutex);
  g_batch_tuning[dev].lanes = lanes > 0 ? lanes : kDefaultLanes;
  g_batch_tuning[dev].eig_ctas = eig_ctas;
  return HT_OK;
}

ht_status_t ht_release_batch(void) {
  std::lock_guard<std::mutex> lk(g_batch_mutex);
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
    cudaGetLastError();
    return HT_OK;
  }
  BatchState &b = g_batch[dev];
  HT_CUDA(cudaDeviceSynchronize());
  batch_drop_graph(b);
  if (b.ws) HT_CUDA(cudaFree(b.ws));
  b.ws = nullptr;
  b.ws_bytes = 0;
  if (b.table) HT_CUDA(cudaFree(b.table));
  b.table = nullptr;
  b.table_bytes = 0;
  if (b.conv) HT_CUDA(cudaFree(b.conv));
  b.conv = nullptr;
  b.conv_bytes = 0;
  if (b.copies) HT_CUDA(cudaFree(b.copies));
  b.copies = nullptr;
  b.copies_bytes = 0;
  if (b.grams) HT_CUDA(cudaFree(b.grams));
  b.grams = nullptr;
  b.grams_bytes = 0;
  if (b.tails) HT_CUDA(cudaFree(b.tails));
  b.tails = nullptr;
  b.tails_bytes = 0;
  if (b.errs) HT_CUDA(cudaFree(b.errs));
  b.errs = nullptr;
  b.errs_bytes = 0;
  if (b.maps) HT_CUDA(cudaFree(b.maps));
  b.maps = nullptr;
  b.maps_bytes = 0;
  if (b.core) HT_CUDA(cudaFree(b.core));
  b.core = nullptr;
  b.core_bytes = 0;
  if (b.step2) HT_CUDA(cudaFree(b.step2));
  b.step2 = nullptr;
  b.step2_bytes = 0;
  if (b.narrow) HT_CUDA(cudaFree(b.narrow));
  b.narrow = nullptr;
  b.narrow_bytes = 0;
  if (b.t1jobs) HT_CUDA(cudaFree(b.t1jobs));
  b.t1jobs = nullptr;
  b.t1jobs_bytes = 0;
  return HT_OK;
}

ht_status_t ht_sketch_loss_grad(const float *G, const float *trG, int batch, int n, int s, const float *S,
                                float *grad, double *loss, void *stream) {
  if (!G || !trG || !S || !grad || !loss) return fail(HT_ERR_INVALID_ARG, "NULL argument");
  if (batch < 1 || n < 1 || s < 1 || s > 64 || s > n) return fail(HT_ERR_INVALID_ARG, "need batch >= 1, 1 <= s <= min(n, 64)");
  HT_TRY(check_device());
  if (!is_device_ptr(G) || !is_device_ptr(trG) || !is_device_ptr(S) || !is_device_ptr(grad))
    return fail(HT_ERR_INVALID_ARG, "G, trG, S and grad must be device memory");
  std::lock_guard<std::mutex> lk(g_ws_mutex);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const size_t bytes = sketch_workspace_bytes(batch, n, s) + sizeof(double) * batch + 512;
  void *ws = nullptr;
  HT_TRY(acquire_workspace(bytes, &ws, st));
  char *p = static_cast<char *>(ws);
  double *dloss = reinterpret_cast<double *>(p);
  int *bad = reinterpret_cast<int *>(p + ((sizeof(double) * batch + 255) & ~size_t(255)));
  void *scratch = p + ((sizeof(double) * batch + 255) & ~size_t(255)) + 256;
  int launches = 0;
  HT_CUDA(cudaMemsetAsync(bad, 0, sizeof(int), st));
  HT_CUDA(sketch_loss_grad(G, trG, batch, n, s, S, grad, dloss, bad, scratch, st, &launches));
  int hbad = 0;
  HT_CUDA(cudaMemcpyAsync(loss, dloss, sizeof(double) * batch, cudaMemcpyDeviceToHost, st));
  HT_CUDA(cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, st));
  HT_CUDA(cudaStreamSynchronize(st));
  g_launches += static_cast<unsigned long long>(launches);
  if (hbad) return fail(HT_ERR_NUMERICAL, "non-finite value in a Gram, the sketch or its CholeskyQR factor");
  for (int b = 0; b < batch; ++b)
    if (!(loss[b] >= -1e-4 && loss[b] <= 1.0 + 1e-4))
      return fail(HT_ERR_NUMERICAL, "sketch loss of Gram " + std::to_string(b) + " outside [0, 1]");
  return HT_OK;
}

ht_status_t ht_sketch_adam(float *S, const float *grad, float *m, float *v, long long count, float lr, int step,
                           void *stream) {
  if (!S || !grad || !m || !v || count < 1 || step < 1) return fail(HT_ERR_INVALID_ARG, "bad argument");
  HT_CUDA(sketch_adam(S, grad, m, v, count, lr, 0.9f, 0.999f, 1e-8f, step, static_cast<cudaStream_t>(stream)));
  g_launches += 1;
  return HT_OK;
}

ht_status_t ht_reconstruct_error(const float *x, const long *dims, int order, const ht_tree_t *tree,
                                 const float *const *U, const float *const *B, double *rel_err, void *stream) {
  if (!x || !dims || !U || !B || !rel_err) return fail(HT_ERR_INVALID_ARG, "NULL argument");
  Tree T;
  HT_TRY(parse_tree(tree, dims, order, T));
  for (int t = 0; t < T.n_nodes; ++t)
    if (!(T.leaf(t) ? U[t] : B[t])) return fail(HT_ERR_INVALID_ARG, "missing factor for node " + std::to_string(t));
  HT_TRY(check_device());
  std::lock_guard<std::mutex> lk(g_ws_mutex);
  long long total = 1;
  for (int m = 0; m < order; ++m) total *= dims[m];
  const bool x_dev = is_device_ptr(x);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // size: staged tensor + staged factors + error scratch (dry run of error_core)
  auto plan = [&](Ctx &c, const float **xd, const float **Ud, const float **Bd, double **sums) -> ht_status_t {
    c.err = c.ar.take<int>(64);
    double *np_ = c.ar.take<double>(1024);
    *sums = c.ar.take<double>(8);
    *xd = x;
    if (!x_dev) {
      float *t = c.ar.take<float>(static_cast<size_t>(total));
      if (!t) return fail(HT_ERR_OUT_OF_MEMORY, "workspace too small");
      if (!c.dry()) HT_CUDA(cudaMemcpyAsync(t, x, sizeof(float) * total, cudaMemcpyHostToDevice, c.st));
      *xd = t;
    }
    for (int t = 0; t < T.n_nodes; ++t) {
      const float *src = T.leaf(t) ? U[t] : B[t];
      const size_t count = factor_count(T, dims, t);
      const float *d = src;
      if (!is_device_ptr(src)) {
        float *tmp = c.ar.take<float>(count);
        if (!tmp) return fail(HT_ERR_OUT_OF_MEMORY, "workspace too small");
        if (!c.dry()) HT_CUDA(cudaMemcpyAsync(tmp, src, count * sizeof(float), cudaMemcpyHostToDevice, c.st));
        d = tmp;
      }
      (T.leaf(t) ? Ud : Bd)[t] = d;
    }
    if (!c.dry()) {
      HT_CUDA(sumsq_launch(*xd, total, np_, 1024, c.st));
      HT_CUDA(sumsq_finish_launch(np_, 1024, *sums, c.st));
      c.launches += 2;
    }
    return error_core(c, T, *xd, dims, order, Ud, Bd, *sums + 1);
  };
  const float *xd = nullptr, *Ud[HT_MAX_NODES] = {}, *Bd[HT_MAX_NODES] = {};
  double *sums = nullptr;
  Ctx d;
  d.ar.dry = true;
  plan(d, &xd, Ud, Bd, &sums);
  const size_t bytes = d.ar.peak + (1 << 20);
  void *ws = nullptr;
  HT_TRY(acquire_workspace(bytes, &ws, st));
  Ctx c;
  c.st = st;
  c.ar.base = static_cast<char *>(ws);
  c.ar.cap = bytes;
  HT_TRY(plan(c, &xd, Ud, Bd, &sums));
  double h[2] = {0.0, 0.0};
  HT_CUDA(cudaMemcpyAsync(h, sums, sizeof(h), cudaMemcpyDeviceToHost, c.st));
  HT_CUDA(cudaStreamSynchronize(c.st));
  *rel_err = h[0] > 0 ? std::sqrt(std::max(h[1], 0.0) / h[0]) : 0.0;
  g_launches += static_cast<unsigned long long>(c.launches);
  return HT_OK;
}

// Factors on the device: host factors are staged into the arena.
static ht_status_t stage_factors(Ctx &c, const Tree &T, const long *dims, const float *const *U, const float *const *B,
                                 const float **Ud, const float **Bd) {
  for (int t = 0; t < T.n_nodes; ++t) {
    const float *src = T.leaf(t) ? U[t] : B[t];
    const size_t count = factor_count(T, dims, t);
    const float *d = src;
    if (!is_device_ptr(src)) {
      float *tmp = c.ar.take<float>(count);
      if (!tmp) return fail(HT_ERR_OUT_OF_MEMORY, "workspace too small");
      if (!c.dry()) HT_CUDA(cudaMemcpyAsync(tmp, src, count * sizeof(float), cudaMemcpyHostToDevice, c.st));
      d = tmp;
    }
    (T.leaf(t) ? Ud : Bd)[t] = d;
  }
  return HT_OK;
}

// Xhat into out (device, column-major).  3rd order: X_(t) = W U_c^T with
// W = (U_p x U_q) (B_t B_root'), the unfolding chosen by which mode c holds;
// 4th order: X_(12) = (W12 B_root) W34^T.  Interior children list their modes
// in increasing order, so W's rows are the column-major (i_p, i_q) pairs.
static ht_status_t reconstruct_core(Ctx &c, const Tree &T, const long *dims, int order, const float *const *U,
                                    const float *const *B, float *out) {
  const size_t mark = c.ar.off;
  if (order == 3) {
    const Plan3 P = plan3(T);
    const long long np_ = dims[P.mp], nq_ = dims[P.mq], nc_ = dims[P.mc];
    float *Bkt = c.ar.take<float>(static_cast<size_t>(P.kt) * P.kc);
    float *core = c.ar.take<float>(static_cast<size_t>(P.kp) * P.kq * P.kc);
    float *Tm = c.ar.take<float>(static_cast<size_t>(np_) * P.kq * P.kc);
    float *Wm = c.ar.take<float>(static_cast<size_t>(np_) * nq_ * P.kc);
    if (!Bkt || !core || !Tm || !Wm) return fail(HT_ERR_OUT_OF_MEMORY, "workspace too small (reconstruct)");
    if (!c.dry()) {
      if (P.t_is_left) HT_CUDA(cudaMemcpyAsync(Bkt, B[0], sizeof(float) * P.kt * P.kc, cudaMemcpyDeviceToDevice, c.st));
      else HT_CUDA(transpose_small_launch(B[0], P.kc, P.kt, Bkt, c.st));
      const long long kpq = static_cast<long long>(P.kp) * P.kq;
      HT_CUDA(matmul_nn_launch(B[P.t], kpq, Bkt, P.kt, core, kpq, kpq, P.kc, P.kt, c.st));
      HT_CUDA(expand2_launch(U[P.p], static_cast<int>(np_), P.kp, core, U[P.q], static_cast<int>(nq_), P.kq, P.kc, Tm,
                             Wm, c.st));
      if (P.mc == 2)        // X_(01) = W U_2^T
        HT_CUDA(gemm_nt_launch(Wm, np_ * nq_, 0, U[P.c], nc_, out, np_ * nq_, 0, np_ * nq_, nc_, P.kc, 1, c.st));
      else if (P.mc == 0)   // X_(0) = U_0 W^T
        HT_CUDA(gemm_nt_launch(U[P.c], nc_, 0, Wm, np_ * nq_, out, nc_, 0, nc_, np_ * nq_, P.kc, 1, c.st));
      else                  // slab i2: X(:, :, i2) = W[(:, i2), :] U_1^T
        HT_CUDA(gemm_nt_launch(Wm, np_ * nq_, np_, U[P.c], nc_, out, np_, np_ * nc_, np_, nc_, P.kc, nq_, c.st));
      c.launches += 4;
    }
  } else {
    const int t1 = T.left[0], t2 = T.right[0];
    const int k1 = T.rank[t1], k2 = T.rank[t2];
    const int a1 = T.left[t1], b1 = T.right[t1], a2 = T.left[t2], b2 = T.right[t2];
    const long long R = static_cast<long long>(dims[0]) * dims[1], Cn = static_cast<long long>(dims[2]) * dims[3];
    float *T1 = c.ar.take<float>(static_cast<size_t>(dims[0]) * T.rank[b1] * k1);
    float *W12 = c.ar.take<float>(static_cast<size_t>(R) * k1);
    float *A12 = c.ar.take<float>(static_cast<size_t>(R) * k2);
    float *T2 = c.ar.take<float>(static_cast<size_t>(dims[2]) * T.rank[b2] * k2);
    float *W34 = c.ar.take<float>(static_cast<size_t>(Cn) * k2);
    if (!T1 || !W12 || !A12 || !T2 || !W34) return fail(HT_ERR_OUT_OF_MEMORY, "workspace too small (reconstruct)");
    if (!c.dry()) {
      HT_CUDA(expand2_launch(U[a1], static_cast<int>(dims[0]), T.rank[a1], B[t1], U[b1], static_cast<int>(dims[1]),
                             T.rank[b1], k1, T1, W12, c.st));
      HT_CUDA(expand2_launch(U[a2], static_cast<int>(dims[2]), T.rank[a2], B[t2], U[b2], static_cast<int>(dims[3]),
                             T.rank[b2], k2, T2, W34, c.st));
      HT_CUDA(matmul_nn_launch(W12, R, B[0], k1, A12, R, R, k2, k1, c.st));
      HT_CUDA(gemm_nt_launch(A12, R, 0, W34, Cn, out, R, 0, R, Cn, k2, 1, c.st));
      c.launches += 6;
    }
  }
  c.ar.off = mark;
  return HT_OK;
}

ht_status_t ht_reconstruct(const long *dims, int order, const ht_tree_t *tree, const float *const *U,
                           const float *const *B, float *x_out, void *stream) {
  if (!dims || !U || !B || !x_out) return fail(HT_ERR_INVALID_ARG, "NULL argument");
  Tree T;
  HT_TRY(parse_tree(tree, dims, order, T));
  for (int t = 0; t < T.n_nodes; ++t)
    if (!(T.leaf(t) ? U[t] : B[t])) return fail(HT_ERR_INVALID_ARG, "missing factor for node " + std::to_string(t));
  HT_TRY(check_device());
  std::lock_guard<std::mutex> lk(g_ws_mutex);
  long long total = 1;
  for (int m = 0; m < order; ++m) total *= dims[m];
  const bool out_dev = is_device_ptr(x_out);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  auto plan = [&](Ctx &c) -> ht_status_t {
    const float *Ud[HT_MAX_NODES] = {}, *Bd[HT_MAX_NODES] = {};
    HT_TRY(stage_factors(c, T, dims, U, B, Ud, Bd));
    float *o = out_dev ? x_out : c.ar.take<float>(static_cast<size_t>(total));
    if (!o) return fail(HT_ERR_OUT_OF_MEMORY, "workspace too small");
    HT_TRY(reconstruct_core(c, T, dims, order, Ud, Bd, o));
    if (!out_dev && !c.dry())
      HT_CUDA(cudaMemcpyAsync(x_out, o, sizeof(float) * total, cudaMemcpyDeviceToHost, c.st));
    return HT_OK;
  };
  Ctx d;
  d.ar.dry = true;
  HT_TRY(plan(d));
  const size_t bytes = d.ar.peak + (1 << 20);
  void *ws = nullptr;
  HT_TRY(acquire_workspace(bytes, &ws, st));
  Ctx c;
  c.st = st;
  c.ar.base = static_cast<char *>(ws);
  c.ar.cap = bytes;
  HT_TRY(plan(c));
  HT_CUDA(cudaStreamSynchronize(c.st));
  g_launches += static_cast<unsigned long long>(c.launches);
  return HT_OK;
}

ht_status_t ht_evaluate(const long *dims, int order, const ht_tree_t *tree, const float *const *U,
                        const float *const *B, const long long *idx, long long count, float *out, void *stream) {
  if (!dims || !U || !B || count < 0) return fail(HT_ERR_INVALID_ARG, "NULL argument or negative count");
  if (count == 0) return HT_OK;
  if (!idx || !out) return fail(HT_ERR_INVALID_ARG, "NULL argument");
  Tree T;
  HT_TRY(parse_tree(tree, dims, order, T));
  for (int t = 0; t < T.n_nodes; ++t)
    if (!(T.leaf(t) ? U[t] : B[t])) return fail(HT_ERR_INVALID_ARG, "missing factor for node " + std::to_string(t));
  HT_TRY(check_device());
  std::lock_guard<std::mutex> lk(g_ws_mutex);
  const bool idx_dev = is_device_ptr(idx), out_dev = is_device_ptr(out);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // Precontracted rows (3rd order, root -> t = {p, q}, c):
  //   Wp[i_p][(y = r_c) + k_c b] = sum_{a, r_t} U_p[i_p, a] B_t[a, b, r_t] B_root'[r_t, r_c],
  //   entry = sum_y (sum_b Wp[i_p][y, b] U_q[i_q, b]) U_c[i_c, y];
  // 4th order (root -> t1 = {0, 1}, t2 = {2, 3}):
  //   W12[i0][r1 + k1 b] = sum_a U_a1[i0, a] B_t1[a, b, r1]
  //   W34[i2][r1 + k1 d] = sum_{c, r2} U_a2[i2, c] B_t2[c, d, r2] B_root[r1, r2]
  //   entry = sum_r1 (sum_b W12[i0][r1, b] U_b1[i1, b]) (sum_d W34[i2][r1, d] U_b2[i3, d]).
  auto plan = [&](Ctx &c) -> ht_status_t {
    const float *Ud[HT_MAX_NODES] = {}, *Bd[HT_MAX_NODES] = {};
    c.err = c.ar.take<int>(64);
    if (!c.err) return fail(HT_ERR_OUT_OF_MEMORY, "workspace too small");
    HT_TRY(stage_factors(c, T, dims, U, B, Ud, Bd));
    const long long *ix = idx;
    if (!idx_dev) {
      long long *tmp = c.ar.take<long long>(static_cast<size_t>(count) * order);
      if (!tmp) return fail(HT_ERR_OUT_OF_MEMORY, "workspace too small");
      if (!c.dry())
        HT_CUDA(cudaMemcpyAsync(tmp, idx, sizeof(long long) * count * order, cudaMemcpyHostToDevice, c.st));
      ix = tmp;
    }
    float *o = out_dev ? out : c.ar.take<float>(static_cast<size_t>(count));
    if (!o) return fail(HT_ERR_OUT_OF_MEMORY, "workspace too small");
    EvalPlan ep{};
    ep.order = order;
    if (order == 3) {
      const Plan3 P = plan3(T);
      float *Bkt = c.ar.take<float>(static_cast<size_t>(P.kt) * P.kc);
      float *core = c.ar.take<float>(static_cast<size_t>(P.kc) * P.kq * P.kp);
      float *Wp = c.ar.take<float>(static_cast<size_t>(dims[P.mp]) * P.kq * P.kc);
      if (!Bkt || !core || !Wp) return fail(HT_ERR_OUT_OF_MEMORY, "workspace too small");
      if (!c.dry()) {
        if (P.t_is_left)
          HT_CUDA(cudaMemcpyAsync(Bkt, Bd[0], sizeof(float) * P.kt * P.kc, cudaMemcpyDeviceToDevice, c.st));
        else HT_CUDA(transpose_small_launch(Bd[0], P.kc, P.kt, Bkt, c.st));
        HT_CUDA(eval_core_launch(Bd[P.t], P.kp, P.kq, P.kt, Bkt, P.kc, core, c.st));
        const long long rw = static_cast<long long>(P.kc) * P.kq;
        HT_CUDA(gemm_nt_launch(core, rw, 0, Ud[P.p], dims[P.mp], Wp, rw, 0, rw, dims[P.mp], P.kp, 1, c.st));
        c.launches += 3;
      }
      ep.ky = P.kc;
      ep.side[0] = EvalSide{Wp, Ud[P.q], dims[P.mp], dims[P.mq], P.mp, P.mq, P.kq};
      ep.side[1] = EvalSide{nullptr, Ud[P.c], 0, dims[P.mc], 0, P.mc, 0};
    } else {
      const int t1 = T.left[0], t2 = T.right[0];
      const int k1 = T.rank[t1], k2 = T.rank[t2];
      const int a1 = T.left[t1], b1 = T.right[t1], a2 = T.left[t2], b2 = T.right[t2];
      const int ka1 = T.rank[a1], kb1 = T.rank[b1], ka2 = T.rank[a2], kb2 = T.rank[b2];
      float *c12 = c.ar.take<float>(static_cast<size_t>(k1) * kb1 * ka1);
      float *B0T = c.ar.take<float>(static_cast<size_t>(k2) * k1);
      float *c34 = c.ar.take<float>(static_cast<size_t>(k1) * kb2 * ka2);
      float *W12 = c.ar.take<float>(static_cast<size_t>(dims[0]) * k1 * kb1);
      float *W34 = c.ar.take<float>(static_cast<size_t>(dims[2]) * k1 * kb2);
      if (!c12 || !B0T || !c34 || !W12 || !W34) return fail(HT_ERR_OUT_OF_MEMORY, "workspace too small");
      if (!c.dry()) {
        HT_CUDA(eval_core_launch(Bd[t1], ka1, kb1, k1, nullptr, k1, c12, c.st));
        HT_CUDA(transpose_small_launch(Bd[0], k1, k2, B0T, c.st));
        HT_CUDA(eval_core_launch(Bd[t2], ka2, kb2, k2, B0T, k1, c34, c.st));
        const long long r12 = static_cast<long long>(k1) * kb1, r34 = static_cast<long long>(k1) * kb2;
        HT_CUDA(gemm_nt_launch(c12, r12, 0, Ud[a1], dims[0], W12, r12, 0, r12, dims[0], ka1, 1, c.st));
        HT_CUDA(gemm_nt_launch(c34, r34, 0, Ud[a2], dims[2], W34, r34, 0, r34, dims[2], ka2, 1, c.st));
        c.launches += 5;
      }
      ep.ky = k1;
      ep.side[0] = EvalSide{W12, Ud[b1], dims[0], dims[1], 0, 1, kb1};
      ep.side[1] = EvalSide{W34, Ud[b2], dims[2], dims[3], 2, 3, kb2};
    }
    if (!c.dry()) {
      HT_CUDA(cudaMemsetAsync(c.err, 0, sizeof(int), c.st));
      HT_CUDA(evaluate_launch(ep, ix, count, o, c.err, c.st));
      ++c.launches;
      if (!out_dev) HT_CUDA(cudaMemcpyAsync(out, o, sizeof(float) * count, cudaMemcpyDeviceToHost, c.st));
    }
    return HT_OK;
  };
  Ctx d;
  d.ar.dry = true;
  HT_TRY(plan(d));
  const size_t bytes = d.ar.peak + (1 << 20);
  void *ws = nullptr;
  HT_TRY(acquire_workspace(bytes, &ws, st));
  Ctx c;
  c.st = st;
  c.ar.base = static_cast<char *>(ws);
  c.ar.cap = bytes;
  HT_TRY(plan(c));
  int errword = 0;
  HT_CUDA(cudaMemcpyAsync(&errword, c.err, sizeof(int), cudaMemcpyDeviceToHost, c.st));
  HT_CUDA(cudaStreamSynchronize(c.st));
  g_launches += static_cast<unsigned long long>(c.launches);
  if (errword) return fail(HT_ERR_INVALID_ARG, "an index lies outside its mode");
  return HT_OK;
}

// Shared driver of the three unfolding primitives.  op 0: Gram, 1: mode product, 2: co-range product.
static ht_status_t unfolding_op(int op, const float *x, const long *dims, int order, int lo, int hi, const float *Mat,
                                int k, int precision, float *out, void *stream) {
  if (!x || !dims || !out || (op != 0 && !Mat)) return fail(HT_ERR_INVALID_ARG, "NULL argument");
  if (order < 1 || order > HT_MAX_ORDER) return fail(HT_ERR_INVALID_ARG, "order must be 1..4");
  if (lo < 0 || hi < lo || hi >= order) return fail(HT_ERR_INVALID_ARG, "bad mode group");
  if (precision != HT_PREC_FP32 && precision != HT_PREC_BF16) return fail(HT_ERR_INVALID_ARG, "unknown precision");
  for (int m = 0; m < order; ++m)
    if (dims[m] < 1) return fail(HT_ERR_INVALID_ARG, "dims must be positive");
  const View v = view_of_group(dims, order, lo, hi);
  if (op != 0 && (k < 1 || k > 64)) return fail(HT_ERR_UNSUPPORTED, "k must lie in [1, 64]");
  if (op == 0 && v.N > 32768) return fail(HT_ERR_UNSUPPORTED, "Gram size above 32768");
  HT_TRY(check_device());
  std::lock_guard<std::mutex> lk(g_ws_mutex);
  const long long total = v.L * v.N * v.R;
  const long long mat_rows = op == 1 ? v.N : v.L * v.R;
  const long long out_count = op == 0 ? v.N * v.N : (op == 1 ? v.L * v.R * k : v.N * k);
  const bool x_dev = is_device_ptr(x), m_dev = Mat && is_device_ptr(Mat), o_dev = is_device_ptr(out);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  auto body = [&](Ctx &c) -> ht_status_t {
    c.err = c.ar.take<int>(64);
    const float *xd = x, *md = Mat;
    if (!x_dev) {
      float *t = c.ar.take<float>(static_cast<size_t>(total));
      if (!t) return fail(HT_ERR_OUT_OF_MEMORY, "workspace");
      if (!c.dry()) HT_CUDA(cudaMemcpyAsync(t, x, sizeof(float) * total, cudaMemcpyHostToDevice, c.st));
      xd = t;
    }
    if (Mat && !m_dev) {
      float *t = c.ar.take<float>(static_cast<size_t>(mat_rows) * k);
      if (!t) return fail(HT_ERR_OUT_OF_MEMORY, "workspace");
      if (!c.dry()) HT_CUDA(cudaMemcpyAsync(t, Mat, sizeof(float) * mat_rows * k, cudaMemcpyHostToDevice, c.st));
      md = t;
    }
    float *od = out;
    if (!o_dev) {
      od = c.ar.take<float>(static_cast<size_t>(out_count));
      if (!od) return fail(HT_ERR_OUT_OF_MEMORY, "workspace");
    }
    __nv_bfloat16 *x16 = nullptr, *m16 = nullptr;
    if (c.tc) {
      x16 = c.ar.take<__nv_bfloat16>(static_cast<size_t>(total) + 64);
      double *parts = c.ar.take<double>(1024);
      if (!x16 || !parts) return fail(HT_ERR_OUT_OF_MEMORY, "workspace");
      if (!c.dry()) HT_CUDA(convert_bf16_launch(xd, x16, total, parts, 1024, c.st));
      if (Mat) {
        m16 = c.ar.take<__nv_bfloat16>(static_cast<size_t>(mat_rows) * k + 64);
        if (!m16) return fail(HT_ERR_OUT_OF_MEMORY, "workspace");
        if (!c.dry()) HT_CUDA(f32_to_bf16_launch(md, m16, mat_rows * k, c.st));
      }
    }
    if (!c.dry()) HT_CUDA(cudaMemsetAsync(c.err, 0, sizeof(int), c.st));
    if (op == 0) HT_TRY(gram(c, v, xd, x16, od));
    else if (op == 1) HT_TRY(mode_product(c, v, xd, x16, md, m16, k, od));
    else HT_TRY(corange_product(c, v, xd, x16, md, m16, k, od));
    if (c.dry()) return HT_OK;
    if (!o_dev) HT_CUDA(cudaMemcpyAsync(out, od, sizeof(float) * out_count, cudaMemcpyDeviceToHost, c.st));
    int errword = 0;
    HT_CUDA(cudaMemcpyAsync(&errword, c.err, sizeof(int), cudaMemcpyDeviceToHost, c.st));
    HT_CUDA(cudaStreamSynchronize(c.st));
    HT_CUDA(cudaGetLastError());
    if (errword & kErrTimeout) return fail(HT_ERR_TIMEOUT, "a kernel's bounded wait expired; results are invalid");
    g_launches += static_cast<unsigned long long>(c.launches);
    return HT_OK;
  };
  Ctx d;
  d.ar.dry = true;
  d.tc = precision == HT_PREC_BF16;
  body(d);
  const size_t bytes = d.ar.peak + (1 << 20);
  void *ws = nullptr;
  HT_TRY(acquire_workspace(bytes, &ws, st));
  Ctx c;
  c.st = st;
  c.tc = precision == HT_PREC_BF16;
  c.ar.base = static_cast<char *>(ws);
  c.ar.cap = bytes;
  return body(c);
}

ht_status_t ht_mode_gram(const float *x, const long *dims, int order, int lo, int hi, int precision, float *G,
                         void *stream) {
  return unfolding_op(0, x, dims, order, lo, hi, nullptr, 0, precision, G, stream);
}

ht_status_t ht_mode_product(const float *x, const long *dims, int order, int lo, int hi, const float *W, int k,
                            int precision, float *Z, void *stream) {
  return unfolding_op(1, x, dims, order, lo, hi, W, k, precision, Z, stream);
}

ht_status_t ht_corange_product(const float *x, const long *dims, int order, int lo, int hi, const float *Q, int k,
                               int precision, float *Z, void *stream) {
  return unfolding_op(2, x, dims, order, lo, hi, Q, k, precision, Z, stream);
}

ht_status_t ht_selftest_wait_timeout(int ctas, double limit_ms, void *stream) {
  if (ctas < 1 || !(limit_ms > 0.0) || limit_ms > 2000.0)
    return fail(HT_ERR_INVALID_ARG, "need ctas >= 1 and 0 < limit_ms <= 2000");
  HT_TRY(check_device());
  if (ctas > sm_count()) return fail(HT_ERR_INVALID_ARG, "ctas above the device's multiprocessor count");
  std::lock_guard<std::mutex> lk(g_ws_mutex);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  void *ws = nullptr;
  HT_TRY(acquire_workspace(1 << 20, &ws, st));
  int *err = reinterpret_cast<int *>(static_cast<char *>(ws) + 256);
  HT_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));
  HT_CUDA(wait_probe_launch(ctas, static_cast<uint64_t>(limit_ms * 1e6), ws, err, st));
  int h = 0;
  HT_CUDA(cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, st));
  HT_CUDA(cudaStreamSynchronize(st));
  HT_CUDA(cudaGetLastError());
  ++g_launches;
  if (h & kErrTimeout) return fail(HT_ERR_TIMEOUT, "the probe's grid barrier wait ran out, as intended");
  return fail(HT_ERR_CUDA, "the probe's wait did not report a timeout");
}

ht_status_t ht_tsqr(const float *A, long long m, int k, long long lda, float *R, void *stream) {
  if (!A || !R) return fail(HT_ERR_INVALID_ARG, "NULL argument");
  if (m < 1 || k < 1 || lda < m) return fail(HT_ERR_INVALID_ARG, "need m >= 1, k >= 1 and lda >= m");
  if (k > 64) return fail(HT_ERR_UNSUPPORTED, "k above 64");
  HT_TRY(check_device());
  std::lock_guard<std::mutex> lk(g_ws_mutex);
  const bool a_dev = is_device_ptr(A), r_dev = is_device_ptr(R);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  auto body = [&](Ctx &c) -> ht_status_t {
    const float *Ad = A;
    long long ld = lda;
    if (!a_dev) {
      float *t = c.ar.take<float>(static_cast<size_t>(m) * k);
      if (!t) return fail(HT_ERR_OUT_OF_MEMORY, "workspace");
      if (!c.dry())
        HT_CUDA(cudaMemcpy2DAsync(t, sizeof(float) * m, A, sizeof(float) * lda, sizeof(float) * m, k,
                                  cudaMemcpyHostToDevice, c.st));
      Ad = t;
      ld = m;
    }
    float *Rd = R;
    if (!r_dev) {
      Rd = c.ar.take<float>(static_cast<size_t>(k) * k);
      if (!Rd) return fail(HT_ERR_OUT_OF_MEMORY, "workspace");
    }
    const size_t qb = tsqr_workspace_bytes(m, k);
    void *qws = c.ar.take<char>(qb);
    if (!qws) return fail(HT_ERR_OUT_OF_MEMORY, "workspace");
    if (c.dry()) return HT_OK;
    HT_CUDA(tsqr_launch(Ad, m, k, ld, Rd, nullptr, qws, qb, c.st, &c.launches));
    if (!r_dev) HT_CUDA(cudaMemcpyAsync(R, Rd, sizeof(float) * k * k, cudaMemcpyDeviceToHost, c.st));
    HT_CUDA(cudaStreamSynchronize(c.st));
    HT_CUDA(cudaGetLastError());
    g_launches += static_cast<unsigned long long>(c.launches);
    return HT_OK;
  };
  Ctx d;
  d.ar.dry = true;
  body(d);
  const size_t bytes = d.ar.peak + (1 << 20);
  void *ws = nullptr;
  HT_TRY(acquire_workspace(bytes, &ws, st));
  Ctx c;
  c.st = st;
  c.ar.base = static_cast<char *>(ws);
  c.ar.cap = bytes;
  return body(c);
}

}  // extern "C"

// ------------------------------------------------ allocation-free Gram entry
// Scratch of ht_mode_gram_noalloc: the split-K partial tiles of the FP32 Gram.
// A static device array, so it exists on every device that loads this module
// and is never allocated or freed by the library.
__device__ __align__(256) float g_noalloc_scratch[HT_NOALLOC_SCRATCH_BYTES / sizeof(float)];

namespace {

std::mutex g_noalloc_mutex;
struct NoallocSlot {
  float *ptr = nullptr;            // device address of g_noalloc_scratch
  unsigned long long ctx = 0;      // id of the context it was looked up in
};
NoallocSlot g_noalloc_slot[64];

// Id of the current context (0 when the driver cannot say).  A device's
// primary context is destroyed by cudaDeviceReset and a new one gets a new id,
// so an address looked up in the old one is not reused.
unsigned long long current_context_id() {
  using GetCurrent = CUresult (*)(CUcontext *);
  using GetId = CUresult (*)(CUcontext, unsigned long long *);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<GetCurrent>(f);
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<GetId>(f);
    cudaGetLastError();
  });
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS)
    return 0;
  return id;
}

// The host-side symbol g_noalloc_scratch is not a device address; look the
// real address up once per device (and again in a new context), with that
// device current.
ht_status_t noalloc_scratch(float **out) {
  int dev = 0;
  HT_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(HT_ERR_INVALID_ARG, "device index out of range");
  std::lock_guard<std::mutex> lk(g_noalloc_mutex);
  NoallocSlot &slot = g_noalloc_slot[dev];
  const unsigned long long ctx = current_context_id();
  if (!slot.ptr || ctx == 0 || slot.ctx != ctx) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      slot.ptr = nullptr;
      return fail(HT_ERR_CUDA, std::string("ht_mode_gram_noalloc: cudaGetSymbolAddress failed: ") +
                                   cudaGetErrorString(e));
    }
    slot.ptr = static_cast<float *>(p);
    slot.ctx = ctx;
  }
  *out = slot.ptr;
  return HT_OK;
}

}  // namespace

extern "C" {

ht_status_t ht_mode_gram_noalloc(const float *x, const long *dims, int order, int lo, int hi, float *G,
                                 void *stream) {
  if (!x || !dims || !G) return fail(HT_ERR_INVALID_ARG, "NULL argument");
  if (order < 1 || order > HT_MAX_ORDER) return fail(HT_ERR_INVALID_ARG, "order must be 1..4");
  if (lo < 0 || hi < lo || hi >= order) return fail(HT_ERR_INVALID_ARG, "bad mode group");
  for (int m = 0; m < order; ++m)
    if (dims[m] < 1) return fail(HT_ERR_INVALID_ARG, "dims must be positive");
  const View v = view_of_group(dims, order, lo, hi);
  if (v.N > HT_NOALLOC_MAX_GRAM)
    return fail(HT_ERR_UNSUPPORTED, "ht_mode_gram_noalloc: Gram size " + std::to_string(v.N) +
                                        " is above the maximum " + std::to_string(HT_NOALLOC_MAX_GRAM) +
                                        " that its fixed scratch holds; use ht_mode_gram");
  HT_TRY(check_device());
  if (!is_device_ptr(x) || !is_device_ptr(G))
    return fail(HT_ERR_INVALID_ARG, "ht_mode_gram_noalloc: x and G must be device memory");
  float *scratch = nullptr;
  HT_TRY(noalloc_scratch(&scratch));
  const int bn = v.N > 64 ? 128 : 64;
  TileGen gen;
  if (!make_gram_gen(v.N, bn, &gen)) return fail(HT_ERR_UNSUPPORTED, "Gram too large");
  const int nt = gen.count;
  const long long tile_floats = 128ll * bn;
  const long long cap_splits = static_cast<long long>(HT_NOALLOC_SCRATCH_BYTES / sizeof(float)) / (tile_floats * nt);
  if (cap_splits < 1) return fail(HT_ERR_UNSUPPORTED, "ht_mode_gram_noalloc: scratch too small");
  // split K as the allocating path does, then clip to what the scratch holds
  int splits = nt < sm_count() ? std::max(1, sm_count() / nt) : 1;
  GemmArgs g;
  g.a = g.b = gram_operand(v, x);
  const long kt = simt_k_total(g.a);
  long per = (kt + splits - 1) / splits;
  per = std::max<long>((per + 15) / 16 * 16, 256);
  splits = static_cast<int>(std::max<long>(1, (kt + per - 1) / per));
  if (splits > cap_splits) {
    splits = static_cast<int>(cap_splits);
    per = (kt + splits - 1) / splits;
    per = (per + 15) / 16 * 16;
    splits = static_cast<int>(std::max<long>(1, (kt + per - 1) / per));
  }
  g.gen = gen;
  g.num_tiles = nt;
  g.splits = splits;
  g.out_mode = OUT_PARTIAL;
  g.out = scratch;
  g.ld_out = v.N;
  g.err = nullptr;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  HT_CUDA(simt_gemm_launch(g, bn, st));
  HT_CUDA(reduce_partials_launch(scratch, gen, splits, bn, G, v.N, 1, st));
  g_launches += 2;
  return HT_OK;
}

const char *ht_status_string(ht_status_t s) {
  switch (s) {
    case HT_OK: return "ok";
    case HT_ERR_INVALID_ARG: return "invalid argument";
    case HT_ERR_CUDA: return "CUDA error";
    case HT_ERR_OUT_OF_MEMORY: return "out of device memory";
    case HT_ERR_NOT_CONVERGED: return "eigen-solver did not converge";
    case HT_ERR_TIMEOUT: return "kernel wait timed out";
    case HT_ERR_UNSUPPORTED: return "unsupported";
    case HT_ERR_NO_DEVICE: return "no suitable device";
    case HT_ERR_NUMERICAL: return "numerical failure";
  }
  return "unknown status";
}

const char *ht_last_error(void) { return g_last_error.c_str(); }

unsigned long long ht_kernel_launch_count(void) { return g_launches.load(); }

float htd(float *x, long a, long b, long c, int *k) {
  ht_tree_t tree;
  if (!x || !k || ht_tree_reference_3d(&tree, k) != HT_OK) return -1.f;
  const long dims[3] = {a, b, c};
  ht_config_t cfg;
  ht_config_default(&cfg);
  cfg.flags |= HT_FLAG_COMPUTE_ERROR;
  std::vector<float> u1(static_cast<size_t>(a) * std::max(k[3], 1)), u2(static_cast<size_t>(b) * std::max(k[4], 1)),
      u3(static_cast<size_t>(c) * std::max(k[2], 1));
  std::vector<float> b1(static_cast<size_t>(std::max(k[3] * k[4] * k[1], 1))), b0(static_cast<size_t>(std::max(k[1] * k[2], 1)));
  float *U[5] = {nullptr, nullptr, u3.data(), u1.data(), u2.data()};
  float *B[5] = {b0.data(), b1.data(), nullptr, nullptr, nullptr};
  ht_report_t rep;
  std::memset(&rep, 0, sizeof(rep));
  if (ht_decompose(x, dims, 3, &tree, &cfg, U, B, &rep, nullptr) != HT_OK) return -1.f;
  return static_cast<float>(rep.rel_err);
}

void htd4(float *x, long a, long b, long c, long d, int *k, void *cublas_handle, void *cusolver_handle) {
  (void)cublas_handle;
  (void)cusolver_handle;
  ht_tree_t tree;
  if (!x || !k || ht_tree_balanced_4d(&tree, k) != HT_OK) {
    std::printf("htd4: invalid arguments\n");
    return;
  }
  const long dims[4] = {a, b, c, d};
  ht_config_t cfg;
  ht_config_default(&cfg);
  cfg.flags |= HT_FLAG_COMPUTE_ERROR;
  std::vector<float> u[4] = {std::vector<float>(static_cast<size_t>(a) * std::max(k[3], 1)),
                             std::vector<float>(static_cast<size_t>(b) * std::max(k[4], 1)),
                             std::vector<float>(static_cast<size_t>(c) * std::max(k[5], 1)),
                             std::vector<float>(static_cast<size_t>(d) * std::max(k[6], 1))};
  std::vector<float> b1(static_cast<size_t>(std::max(k[3] * k[4] * k[1], 1))),
      b2(static_cast<size_t>(std::max(k[5] * k[6] * k[2], 1))), b0(static_cast<size_t>(std::max(k[1] * k[2], 1)));
  float *U[7] = {nullptr, nullptr, nullptr, u[0].data(), u[1].data(), u[2].data(), u[3].data()};
  float *B[7] = {b0.data(), b1.data(), b2.data(), nullptr, nullptr, nullptr, nullptr};
  ht_report_t rep;
  std::memset(&rep, 0, sizeof(rep));
  const ht_status_t s = ht_decompose(x, dims, 4, &tree, &cfg, U, B, &rep, nullptr);
  if (s != HT_OK) {
    std::printf("htd4: %s (%s)\n", ht_status_string(s), ht_last_error());
    return;
  }
  std::printf("error rate %g\n", rep.rel_err);
}

}  // extern "C"

// ------------------------------------------------------------ HT tensor layer
// Forward:  P, Q from the factors; W (Nout x Nin) from P, Q; one GEMM
//           y^T = W x^T (rows o, columns z, i.e. y row-major); bias + activation.
// Backward: P, Q, T1 and W again; dx = dy W and dW = dy^T x as GEMMs; dbias as
//           column sums of dy; dP, dQ from dW; the factor gradients from dP, dQ.
namespace {

std::mutex g_layer_mutex;
DeviceWorkspace g_layer_ws[64];
int *g_layer_err[64];   // first 256 bytes of each device's layer workspace

ht_status_t layer_shape(const ht_layer_shape_t *in, LayerShape *sh) {
  if (!in) return fail(HT_ERR_INVALID_ARG, "shape is NULL");
  long long nin = 1, nout = 1;
  for (int j = 0; j < 3; ++j) {
    if (in->n[j] < 1 || in->m[j] < 1) return fail(HT_ERR_INVALID_ARG, "mode sizes must be positive");
    sh->n[j] = in->n[j];
    sh->m[j] = in->m[j];
    nin *= in->n[j];
    nout *= in->m[j];
  }
  for (int j = 0; j < 4; ++j)
    if (in->r[j] < 1 || in->r[j] > kLayerMaxRank) return fail(HT_ERR_UNSUPPORTED, "layer ranks must lie in [1, 64]");
  if (nin > (1ll << 28) || nout > (1ll << 28) || nin * nout > (1ll << 34))
    return fail(HT_ERR_UNSUPPORTED, "layer too large");
  const long long A = static_cast<long long>(in->n[0]) * in->m[0], B = static_cast<long long>(in->n[1]) * in->m[1],
                  C = static_cast<long long>(in->n[2]) * in->m[2];
  if (A * B > (1ll << 31) - 1 || C * 4 > 48 * 1024)
    return fail(HT_ERR_UNSUPPORTED, "layer mode products too large (n[2]*m[2] <= 12288)");
  sh->r3 = in->r[0];
  sh->r4 = in->r[1];
  sh->r2 = in->r[2];
  sh->r1 = in->r[3];
  return HT_OK;
}

long long layer_nin(const LayerShape &s) { return static_cast<long long>(s.n[0]) * s.n[1] * s.n[2]; }
long long layer_nout(const LayerShape &s) { return static_cast<long long>(s.m[0]) * s.m[1] * s.m[2]; }
size_t layer_p_count(const LayerShape &s) {
  return static_cast<size_t>(s.n[0]) * s.m[0] * s.n[1] * s.m[1] * s.r1;
}
size_t layer_q_count(const LayerShape &s) { return static_cast<size_t>(s.n[2]) * s.m[2] * s.r1; }
size_t layer_t1_count(const LayerShape &s) { return static_cast<size_t>(s.n[0]) * s.m[0] * s.r4 * s.r1; }

ht_status_t layer_check_ptrs(std::initializer_list<const void *> ptrs) {
  for (const void *p : ptrs)
    if (p && !is_device_ptr(p)) return fail(HT_ERR_INVALID_ARG, "HT layer arguments must be device memory");
  return HT_OK;
}

// Run plan() as a dry run to size the workspace, grow the device's layer
// workspace if needed (synchronising only then) and run it for real.
template <class F>
ht_status_t layer_run(cudaStream_t st, bool tc, F &&plan) {
  int dev = 0;
  HT_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(HT_ERR_INVALID_ARG, "device index out of range");
  Ctx d;
  d.ar.dry = true;
  d.tc = tc;
  HT_TRY(plan(d));
  const size_t bytes = d.ar.peak + 256 + (1 << 16);
  std::lock_guard<std::mutex> lk(g_layer_mutex);
  DeviceWorkspace &w = g_layer_ws[dev];
  if (w.bytes < bytes) {
    if (w.ptr) {
      HT_CUDA(cudaDeviceSynchronize());
      HT_CUDA(cudaFree(w.ptr));
      w.ptr = nullptr;
      w.bytes = 0;
    }
    HT_CUDA(cudaMalloc(&w.ptr, bytes));
    HT_CUDA(cudaMemset(w.ptr, 0, 256));
    HT_CUDA(cudaDeviceSynchronize());
    w.bytes = bytes;
    g_layer_err[dev] = static_cast<int *>(w.ptr);
  }
  Ctx c;
  c.st = st;
  c.tc = tc;
  c.err = g_layer_err[dev];
  c.ar.base = static_cast<char *>(w.ptr) + 256;
  c.ar.cap = w.bytes - 256;
  HT_TRY(plan(c));
  g_launches += static_cast<unsigned long long>(c.launches);
  return HT_OK;
}

// D (rows x cols, column-major, ld = rows) = A B^T over the two operand pairs.
ht_status_t layer_gemm(Ctx &c, const Operand &a32, const Operand &b32, const Operand &a16, const Operand &b16,
                       long long rows, long long cols, float *D) {
  GemmReq q;
  q.a32 = a32;
  q.b32 = b32;
  q.a16 = a16;
  q.b16 = b16;
  q.bn_tc = cols >= 256 ? 256 : (cols > 64 ? 128 : 64);
  q.bn_simt = cols > 64 ? 128 : 64;
  q.tiles_kind = TILES_GRID;
  q.t_rows = rows;
  q.t_n = cols;
  q.out_mode = OUT_COLMAJOR;
  q.out = D;
  q.ld_out = rows;
  if (c.tc) {   // the FP32 operands may be absent here: no SIMT fallback
    GemmArgs probe;
    probe.a = a16;
    probe.b = b16;
    probe.splits = 1;
    std::string why;
    if (!a16.ptr || !b16.ptr || !tc_gemm_supported(probe, q.bn_tc, &why))
      return fail(HT_ERR_UNSUPPORTED, "BF16 layer product not expressible as TMA tiles: " + why);
  }
  return run_gemm(c, q);
}

Operand op_of(int kind, const void *p, long d0, long d1) {
  Operand o;
  o.kind = kind;
  o.ptr = p;
  o.d0 = d0;
  o.d1 = d1;
  o.d2 = 1;
  return o;
}

}  // namespace

extern "C" {

ht_status_t ht_layer_weight(const ht_layer_shape_t *shape, const float *u1, const float *u2, const float *u3,
                            const float *b2, const float *b1, float *W, void *stream) {
  LayerShape sh;
  HT_TRY(layer_shape(shape, &sh));
  if (!u1 || !u2 || !u3 || !b2 || !b1 || !W) return fail(HT_ERR_INVALID_ARG, "NULL argument");
  HT_TRY(check_device());
  HT_TRY(layer_check_ptrs({u1, u2, u3, b2, b1, W}));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  return layer_run(st, false, [&](Ctx &c) -> ht_status_t {
    float *P = c.ar.take<float>(layer_p_count(sh));
    float *Q = c.ar.take<float>(layer_q_count(sh));
    if (!P || !Q) return fail(HT_ERR_OUT_OF_MEMORY, "layer workspace too small");
    if (c.dry()) return HT_OK;
    HT_CUDA(layer_pq_launch(sh, u1, u2, u3, b2, b1, P, Q, nullptr, c.st));
    HT_CUDA(layer_weight_launch(sh, P, Q, W, nullptr, c.st));
    c.launches += 2;
    return HT_OK;
  });
}

ht_status_t ht_layer_forward(const ht_layer_shape_t *shape, const float *u1, const float *u2, const float *u3,
                             const float *b2, const float *b1, const float *bias, int activation, int precision,
                             const float *x, long long batch, float *y, void *stream) {
  LayerShape sh;
  HT_TRY(layer_shape(shape, &sh));
  if (!u1 || !u2 || !u3 || !b2 || !b1 || !x || !y) return fail(HT_ERR_INVALID_ARG, "NULL argument");
  if (batch < 1 || batch > (1ll << 31) - 256) return fail(HT_ERR_INVALID_ARG, "batch must lie in [1, 2^31)");
  if (activation != 0 && activation != 1) return fail(HT_ERR_INVALID_ARG, "activation must be 0 or 1");
  if (precision != HT_PREC_FP32 && precision != HT_PREC_BF16) return fail(HT_ERR_INVALID_ARG, "bad precision");
  const long long nin = layer_nin(sh), nout = layer_nout(sh);
  const bool tc = precision == HT_PREC_BF16;
  if (tc && (nin % 8 || nout % 8))
    return fail(HT_ERR_UNSUPPORTED, "the BF16 layer needs n0*n1*n2 and m0*m1*m2 divisible by 8");
  HT_TRY(check_device());
  HT_TRY(layer_check_ptrs({u1, u2, u3, b2, b1, bias, x, y}));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  return layer_run(st, tc, [&](Ctx &c) -> ht_status_t {
    float *P = c.ar.take<float>(layer_p_count(sh));
    float *Q = c.ar.take<float>(layer_q_count(sh));
    float *W32 = tc ? nullptr : c.ar.take<float>(static_cast<size_t>(nin * nout));
    __nv_bfloat16 *W16 = tc ? c.ar.take<__nv_bfloat16>(static_cast<size_t>(nin * nout)) : nullptr;
    __nv_bfloat16 *x16 = tc ? c.ar.take<__nv_bfloat16>(static_cast<size_t>(batch * nin)) : nullptr;
    if (!P || !Q || !(W32 || W16) || (tc && !x16)) return fail(HT_ERR_OUT_OF_MEMORY, "layer workspace too small");
    if (!c.dry()) {
      HT_CUDA(layer_pq_launch(sh, u1, u2, u3, b2, b1, P, Q, nullptr, c.st));
      HT_CUDA(layer_weight_launch(sh, P, Q, W32, W16, c.st));
      if (tc) HT_CUDA(f32_to_bf16_launch(x, x16, batch * nin, c.st));
      c.launches += tc ? 3 : 2;
    }
    // y^T (nout x batch, column-major) = W x^T: A = W (rows o, K-major), B = x (rows z, K-major)
    HT_TRY(layer_gemm(c, op_of(OP_KM3, W32, nin, nout), op_of(OP_KM3, x, nin, batch),
                      op_of(OP_KM3, W16, nin, nout), op_of(OP_KM3, x16, nin, batch), nout, batch, y));
    if (!c.dry() && (bias || activation)) {
      HT_CUDA(bias_act_launch(y, bias, batch, nout, activation, c.st));
      ++c.launches;
    }
    return HT_OK;
  });
}

ht_status_t ht_layer_backward(const ht_layer_shape_t *shape, const float *u1, const float *u2, const float *u3,
                              const float *b2, const float *b1, int precision, const float *x, const float *dy,
                              long long batch, float *dx, float *du1, float *du2, float *du3, float *db2,
                              float *db1, float *dbias, void *stream) {
  LayerShape sh;
  HT_TRY(layer_shape(shape, &sh));
  if (!u1 || !u2 || !u3 || !b2 || !b1 || !x || !dy || !du1 || !du2 || !du3 || !db2 || !db1)
    return fail(HT_ERR_INVALID_ARG, "NULL argument");
  if (batch < 1 || batch > (1ll << 31) - 256) return fail(HT_ERR_INVALID_ARG, "batch must lie in [1, 2^31)");
  if (precision != HT_PREC_FP32 && precision != HT_PREC_BF16) return fail(HT_ERR_INVALID_ARG, "bad precision");
  const long long nin = layer_nin(sh), nout = layer_nout(sh);
  const bool tc = precision == HT_PREC_BF16;
  if (tc && (nin % 8 || nout % 8))
    return fail(HT_ERR_UNSUPPORTED, "the BF16 layer needs n0*n1*n2 and m0*m1*m2 divisible by 8");
  HT_TRY(check_device());
  HT_TRY(layer_check_ptrs({u1, u2, u3, b2, b1, x, dy, dx, du1, du2, du3, db2, db1, dbias}));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  return layer_run(st, tc, [&](Ctx &c) -> ht_status_t {
    float *P = c.ar.take<float>(layer_p_count(sh));
    float *Q = c.ar.take<float>(layer_q_count(sh));
    float *T1 = c.ar.take<float>(layer_t1_count(sh));
    float *dP = c.ar.take<float>(layer_p_count(sh));
    float *dQ = c.ar.take<float>(layer_q_count(sh));
    float *dT1 = c.ar.take<float>(layer_t1_count(sh));
    float *dW = c.ar.take<float>(static_cast<size_t>(nin * nout));
    float *W32 = (!tc && dx) ? c.ar.take<float>(static_cast<size_t>(nin * nout)) : nullptr;
    __nv_bfloat16 *W16 = (tc && dx) ? c.ar.take<__nv_bfloat16>(static_cast<size_t>(nin * nout)) : nullptr;
    __nv_bfloat16 *x16 = tc ? c.ar.take<__nv_bfloat16>(static_cast<size_t>(batch * nin)) : nullptr;
    __nv_bfloat16 *dy16 = tc ? c.ar.take<__nv_bfloat16>(static_cast<size_t>(batch * nout)) : nullptr;
    float *part = dbias ? c.ar.take<float>(static_cast<size_t>(layer_colsum_chunks(batch)) * nout) : nullptr;
    const size_t nqp = layer_dq_part_count(sh);
    float *dQpart = nqp ? c.ar.take<float>(nqp) : nullptr;
    if (!P || !Q || !T1 || !dP || !dQ || !dT1 || !dW || (dx && !(W32 || W16)) || (tc && (!x16 || !dy16)) ||
        (dbias && !part) || (nqp && !dQpart))
      return fail(HT_ERR_OUT_OF_MEMORY, "layer workspace too small");
    if (!c.dry()) {
      HT_CUDA(layer_pq_launch(sh, u1, u2, u3, b2, b1, P, Q, T1, c.st));
      ++c.launches;
      if (dx) {
        HT_CUDA(layer_weight_launch(sh, P, Q, W32, W16, c.st));
        ++c.launches;
      }
      if (tc) {
        HT_CUDA(f32_to_bf16_launch(x, x16, batch * nin, c.st));
        HT_CUDA(f32_to_bf16_launch(dy, dy16, batch * nout, c.st));
        c.launches += 2;
      }
    }
    if (dx)   // dx^T (nin x batch) = W^T dy^T: A = W^T (rows i, MN-major), B = dy (rows z, K-major)
      HT_TRY(layer_gemm(c, op_of(OP_MN3, W32, nin, nout), op_of(OP_KM3, dy, nout, batch),
                        op_of(OP_MN3, W16, nin, nout), op_of(OP_KM3, dy16, nout, batch), nin, batch, dx));
    // dW^T (nin x nout, column-major = dW row-major) = x^T dy: A = x^T (rows i), B = dy^T (rows o), K = z
    HT_TRY(layer_gemm(c, op_of(OP_MN3, x, nin, batch), op_of(OP_MN3, dy, nout, batch),
                      op_of(OP_MN3, x16, nin, batch), op_of(OP_MN3, dy16, nout, batch), nin, nout, dW));
    if (!c.dry()) {
      if (dbias) {
        HT_CUDA(layer_colsum_launch(dy, batch, nout, part, dbias, c.st));
        c.launches += 2;
      }
      HT_CUDA(layer_factor_grads_launch(sh, dW, u1, u2, u3, b2, b1, P, Q, T1, dP, dQ, dT1, dQpart, du1, du2, du3,
                                        db2, db1, c.st));
      c.launches += 4;
    }
    return HT_OK;
  });
}

ht_status_t ht_layer_check(void) {
  int dev = 0;
  HT_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(HT_ERR_INVALID_ARG, "device index out of range");
  HT_CUDA(cudaDeviceSynchronize());
  std::lock_guard<std::mutex> lk(g_layer_mutex);
  if (!g_layer_err[dev]) return HT_OK;
  int w = 0;
  HT_CUDA(cudaMemcpy(&w, g_layer_err[dev], sizeof(int), cudaMemcpyDeviceToHost));
  HT_CUDA(cudaMemset(g_layer_err[dev], 0, sizeof(int)));
  if (w & kErrTimeout) return fail(HT_ERR_TIMEOUT, "a wait inside an HT layer kernel timed out");
  return HT_OK;
}

ht_status_t ht_layer_release(void) {
  int dev = 0;
  HT_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(HT_ERR_INVALID_ARG, "device index out of range");
  std::lock_guard<std::mutex> lk(g_layer_mutex);
  DeviceWorkspace &w = g_layer_ws[dev];
  if (w.ptr) {
    HT_CUDA(cudaDeviceSynchronize());
    HT_CUDA(cudaFree(w.ptr));
  }
  w.ptr = nullptr;
  w.bytes = 0;
  g_layer_err[dev] = nullptr;
  return HT_OK;
}

}  // extern "C"
