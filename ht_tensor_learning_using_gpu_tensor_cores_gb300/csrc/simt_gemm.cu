// FP32 GEMM over tensor matricisations on CUDA cores (the plain FP32 path),
// plus the deterministic split-K reduction shared with the tcgen05 path.
//
// This is the GB300 restatement of the reference's FP32 cuBLAS calls
// (third_order_tensor_decompsition/CUDA/Optimized/htd_batch.cu:83-106 leaf
// Grams with cublasSgemm, ttm.cu:2-36 TTM chains).  Same operand/tile model as
// tc_gemm.cu: operands are read in place from the column-major tensor.
//
// Tile 128 x BN (BN = 128, 64 or 32), K step 16, 256 threads, 8 x (BN/16)
// register tile per thread, double-buffered shared memory.  BN = 32 serves
// products with at most 32 columns (rank-32 core contractions), which a 64-wide
// tile would compute half in padding.
#include <algorithm>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "engine.h"
#include "tiles.cuh"

namespace htgb {
namespace {

constexpr int BM = 128;
constexpr int BKS = 16;

struct SParams {
  int a_kind, b_kind;
  const float *a, *b;
  long long a0, a1, a2, b0, b1, b2;
  long long k_total;
  long long k_per_split;
  int num_tiles, out_mode;
  float *out;
  long long ld_out;
  int a_rows, b_rows;   // operand row extents (for bounds)
  int a_vec, b_vec;     // 0 scalar, 1 float4 along k, 2 float4 along rows
};

// Vector load geometry of an operand tile of ROWS x BKS: returns per-thread
// float4 loads; K-contiguous tiles (vec 1) or row-contiguous tiles (vec 2).
template <int ROWS>
HT_DEV void load_vec(int vec, int kind, const float *base, long long d0, long long d1, long long k0, int row0, int z,
                     int rows_total, float *out) {
  constexpr int NV = ROWS * BKS / 4 / 256;   // float4 per thread
#pragma unroll
  for (int i = 0; i < NV; ++i) {
    const int idx = threadIdx.x + 256 * i;
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    if (vec == 1) {
      const int row = row0 + (idx >> 2), kq = (idx & 3) * 4;
      if (row < rows_total) {
        const float *ptr;
        if (kind == OP_KM3) {
          const long long r0 = k0 / d0, l0 = k0 - r0 * d0;
          ptr = base + l0 + d0 * (static_cast<long long>(row) + d1 * r0) + kq;
        } else {
          ptr = base + k0 + d0 * d1 * static_cast<long long>(row) + kq;
        }
        v = __ldg(reinterpret_cast<const float4 *>(ptr));
      }
    } else {
      const int kk = idx / (ROWS / 4), rq = (idx % (ROWS / 4)) * 4;
      const int row = row0 + rq;
      if (row < rows_total)
        v = __ldg(reinterpret_cast<const float4 *>(base + row + d0 * (k0 + kk + d1 * static_cast<long long>(z))));
    }
    out[4 * i] = v.x; out[4 * i + 1] = v.y; out[4 * i + 2] = v.z; out[4 * i + 3] = v.w;
  }
}

template <int ROWS>
HT_DEV void store_vec(int vec, const float *in, float (*S)[ROWS + 4]) {
  constexpr int NV = ROWS * BKS / 4 / 256;
#pragma unroll
  for (int i = 0; i < NV; ++i) {
    const int idx = threadIdx.x + 256 * i;
    if (vec == 1) {
      const int row = idx >> 2, kq = (idx & 3) * 4;
#pragma unroll
      for (int c = 0; c < 4; ++c) S[kq + c][row] = in[4 * i + c];
    } else {
      const int kk = idx / (ROWS / 4), rq = (idx % (ROWS / 4)) * 4;
      *reinterpret_cast<float4 *>(&S[kk][rq]) = make_float4(in[4 * i], in[4 * i + 1], in[4 * i + 2], in[4 * i + 3]);
    }
  }
}

HT_DEV const float *op_ptr(int kind, const float *p, long long d0, long long d1, long long row, long long k,
                           int z) {
  if (kind == OP_KM3) {
    const long long r = k / d0, l = k - r * d0;
    return p + l + d0 * (row + d1 * r);
  }
  if (kind == OP_KM3Q) return p + k + d0 * d1 * row;
  return p + row + d0 * (k + d1 * static_cast<long long>(z));
}

// One output tile (split `split` of its K range) of a CTA.
template <int BN>
HT_DEV void simt_gemm_tile(const SParams &p, const Tile &tile, int tile_idx, int split) {
  constexpr int TN = BN / 16;   // columns per thread (8, 4 or 2)
  constexpr int A_PER = BM * BKS / 256;   // 8
  constexpr int B_PER = BN * BKS / 256;   // 8, 4 or 2
  // a 32-row B tile is 128 float4: fewer than one per thread, so it loads scalar
  constexpr bool kBVec = BN >= 64;
  __shared__ __align__(16) float As[2][BKS][BM + 4];
  __shared__ __align__(16) float Bs[2][BKS][BN + 4];

  const int tid = threadIdx.x;
  const long long kbeg = static_cast<long long>(split) * p.k_per_split;
  const long long kend = min(p.k_total, kbeg + p.k_per_split);

  // load-slot geometry: K-contiguous operands load k-fast, MN3 loads row-fast
  const bool a_kfast = p.a_kind != OP_MN3;
  const bool b_kfast = p.b_kind != OP_MN3;

  float ra[A_PER], rb[B_PER];
  // KM3 operands whose contiguous extent d0 is a multiple of BKS never split a
  // 16-wide K step across two outer indices: decompose k once per step.
  const bool a_fast = p.a_kind == OP_KM3 && (p.a0 % BKS) == 0;
  const bool b_fast = p.b_kind == OP_KM3 && (p.b0 % BKS) == 0;
  // per k-tile: vector loads when the operand allows them and the tile is full
  bool a_v = false, b_v = false;
  auto load_tiles = [&](long long k0) {
    a_v = p.a_vec != 0 && k0 + BKS <= kend;
    b_v = kBVec && p.b_vec != 0 && k0 + BKS <= kend;
    if (a_v) load_vec<BM>(p.a_vec, p.a_kind, p.a, p.a0, p.a1, k0, tile.a_row, tile.a_z, p.a_rows, ra);
    if (b_v) load_vec<BN>(p.b_vec, p.b_kind, p.b, p.b0, p.b1, k0, tile.b_row, 0, p.b_rows, rb);
    if (a_v && b_v) return;
    const float *abase = nullptr, *bbase = nullptr;
    if (a_fast) {
      const long long r0 = k0 / p.a0, l0 = k0 - r0 * p.a0;
      abase = p.a + l0 + p.a0 * p.a1 * r0;
    }
    if (b_fast) {
      const long long r0 = k0 / p.b0, l0 = k0 - r0 * p.b0;
      bbase = p.b + l0 + p.b0 * p.b1 * r0;
    }
#pragma unroll
    for (int i = 0; i < A_PER; ++i) {
      if (a_v) break;
      const int e = tid + 256 * i;
      const int kk = a_kfast ? (e % BKS) : (e / BM);
      const int rr = a_kfast ? (e / BKS) : (e % BM);
      const long long k = k0 + kk;
      const long long row = tile.a_row + rr;
      float v = 0.f;
      if (k < kend && row < p.a_rows)
        v = __ldg(a_fast ? abase + kk + p.a0 * row : op_ptr(p.a_kind, p.a, p.a0, p.a1, row, k, tile.a_z));
      ra[i] = v;
    }
#pragma unroll
    for (int i = 0; i < B_PER; ++i) {
      if (b_v) break;
      const int e = tid + 256 * i;
      const int kk = b_kfast ? (e % BKS) : (e / BN);
      const int rr = b_kfast ? (e / BKS) : (e % BN);
      const long long k = k0 + kk;
      const long long row = tile.b_row + rr;
      float v = 0.f;
      if (k < kend && row < p.b_rows)
        v = __ldg(b_fast ? bbase + kk + p.b0 * row : op_ptr(p.b_kind, p.b, p.b0, p.b1, row, k, 0));
      rb[i] = v;
    }
  };
  auto store_tiles = [&](int buf) {
    if (a_v) store_vec<BM>(p.a_vec, ra, As[buf]);
    if (b_v) store_vec<BN>(p.b_vec, rb, Bs[buf]);
    if (a_v && b_v) return;
#pragma unroll
    for (int i = 0; i < A_PER; ++i) {
      if (a_v) break;
      const int e = tid + 256 * i;
      const int kk = a_kfast ? (e % BKS) : (e / BM);
      const int rr = a_kfast ? (e / BKS) : (e % BM);
      As[buf][kk][rr] = ra[i];
    }
#pragma unroll
    for (int i = 0; i < B_PER; ++i) {
      if (b_v) break;
      const int e = tid + 256 * i;
      const int kk = b_kfast ? (e % BKS) : (e / BN);
      const int rr = b_kfast ? (e / BKS) : (e % BN);
      Bs[buf][kk][rr] = rb[i];
    }
  };

  const int tx = tid % 16, ty = tid / 16;
  float acc[8][TN];
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) acc[i][j] = 0.f;

  int buf = 0;
  if (kbeg < kend) {
    load_tiles(kbeg);
    store_tiles(0);
  }
  __syncthreads();
  for (long long k0 = kbeg; k0 < kend; k0 += BKS) {
    const bool more = k0 + BKS < kend;
    if (more) load_tiles(k0 + BKS);
#pragma unroll
    for (int kk = 0; kk < BKS; ++kk) {
      float a[8], b[TN];
      const float4 a0 = *reinterpret_cast<const float4 *>(&As[buf][kk][ty * 4]);
      const float4 a1 = *reinterpret_cast<const float4 *>(&As[buf][kk][64 + ty * 4]);
      a[0] = a0.x; a[1] = a0.y; a[2] = a0.z; a[3] = a0.w;
      a[4] = a1.x; a[5] = a1.y; a[6] = a1.z; a[7] = a1.w;
      if constexpr (TN == 2) {
        const float2 b0 = *reinterpret_cast<const float2 *>(&Bs[buf][kk][tx * 2]);
        b[0] = b0.x; b[1] = b0.y;
      } else {
        const float4 b0 = *reinterpret_cast<const float4 *>(&Bs[buf][kk][tx * 4]);
        b[0] = b0.x; b[1] = b0.y; b[2] = b0.z; b[3] = b0.w;
      }
      if constexpr (TN == 8) {
        const float4 b1 = *reinterpret_cast<const float4 *>(&Bs[buf][kk][64 + tx * 4]);
        b[4] = b1.x; b[5] = b1.y; b[6] = b1.z; b[7] = b1.w;
      }
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    if (more) store_tiles(buf ^ 1);
    __syncthreads();
    buf ^= 1;
  }

  // write out
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int row = (i < 4) ? (ty * 4 + i) : (64 + ty * 4 + i - 4);
#pragma unroll
    for (int j = 0; j < TN; ++j) {
      const int col = TN == 2 ? tx * 2 + j : ((j < 4) ? (tx * 4 + j) : (64 + tx * 4 + j - 4));
      if (p.out_mode == OUT_PARTIAL) {
        p.out[((static_cast<size_t>(split) * p.num_tiles + tile_idx) * BM + row) * BN + col] = acc[i][j];
      } else if (row < tile.valid_rows && col < tile.valid_cols) {
        p.out[tile.out_row + row + p.ld_out * static_cast<long long>(tile.out_col + col)] = acc[i][j];
      }
    }
  }
}

template <int BN>
__global__ void __launch_bounds__(256) simt_gemm_kernel(const SParams p, const TileGen gen) {
  const int tile_idx = blockIdx.x % p.num_tiles;
  simt_gemm_tile<BN>(p, gen_tile(gen, tile_idx), tile_idx, blockIdx.x / p.num_tiles);
}

// 32-column tiles at three blocks per SM (80 registers, no spills)
__global__ void __launch_bounds__(256, 3) simt_gemm_narrow_kernel(const SParams p, const TileGen gen) {
  const int tile_idx = blockIdx.x % p.num_tiles;
  simt_gemm_tile<32>(p, gen_tile(gen, tile_idx), tile_idx, blockIdx.x / p.num_tiles);
}

// Grouped GEMMs of the batched path: block i computes the tile blocks[i].tile
// of GEMM gemms[blocks[i].gemm] over its whole K range (column-major output).
struct SimtBlock {
  int gemm, pad;
  Tile tile;
};

// The tables hold one SParams / SimtBlock per blob-sized slot.
__global__ void __launch_bounds__(256, 2) simt_gemm_grouped_kernel(const SParamsBlob *__restrict__ gemms,
                                                                const SimtBlockBlob *__restrict__ blocks) {
  __shared__ SParams P;
  __shared__ Tile T;
  if (threadIdx.x == 0) {
    const SimtBlock b = *reinterpret_cast<const SimtBlock *>(blocks + blockIdx.x);
    P = *reinterpret_cast<const SParams *>(gemms + b.gemm);
    T = b.tile;
  }
  __syncthreads();
  simt_gemm_tile<64>(P, T, 0, 0);
}

// Sum partial tiles [splits][num_tiles][128][bn] in a fixed order.  A block
// is (256 / G) consecutive outputs x G split groups: thread (o, g) sums the
// partials of group g in order (8 loads in flight), then the G group sums are
// added in group order.  Splitting the split range keeps enough loads in
// flight when there are few outputs and many splits (small Grams).
__global__ void __launch_bounds__(256) reduce_partials_kernel(const float *__restrict__ part, const TileGen gen,
                                                              int num_tiles, int splits, int bn, int groups,
                                                              float *__restrict__ out, long long ld, int symmetric) {
  __shared__ float red[256];
  const int nout = 256 / groups;
  const int o = threadIdx.x % nout, g = threadIdx.x / nout;
  const int per = (splits + groups - 1) / groups;
  const int k_begin = g * per, k_end = min(splits, k_begin + per);
  const long long per_tile = static_cast<long long>(gen.bm) * bn;
  const long long total = per_tile * num_tiles;
  for (long long base = static_cast<long long>(blockIdx.x) * nout; base < total;
       base += static_cast<long long>(gridDim.x) * nout) {
    const long long idx = base + o;
    const bool live = idx < total;
    const int t = live ? static_cast<int>(idx / per_tile) : 0;
    const int within = live ? static_cast<int>(idx - t * per_tile) : 0;
    float s = 0.f;
    if (live) {
      for (int k0 = k_begin; k0 < k_end; k0 += 8) {   // 8 loads in flight, summed in order
        float v[8];
#pragma unroll
        for (int q = 0; q < 8; ++q)
          v[q] = (k0 + q < k_end) ? part[(static_cast<long long>(k0 + q) * num_tiles + t) * per_tile + within] : 0.f;
#pragma unroll
        for (int q = 0; q < 8; ++q) s += v[q];
      }
    }
    red[threadIdx.x] = s;
    __syncthreads();
    if (g == 0 && live) {
      for (int q = 1; q < groups; ++q) s += red[q * nout + o];
      const int row = within / bn, col = within % bn;
      const Tile tl = gen_tile(gen, t);
      if (row < tl.valid_rows && col < tl.valid_cols) {
        const long long gr = tl.out_row + row, gc = tl.out_col + col;
        const bool acc = (symmetric & 2) != 0;   // add to what out holds
        if (!(symmetric & 1)) {
          out[gr + ld * gc] = acc ? out[gr + ld * gc] + s : s;
        } else if (gc >= gr) {   // the mirror element is produced by the tile holding (gc, gr)
          const long long a = gr + ld * gc, b = gc + ld * gr;
          const float v = acc ? out[a] + s : s;
          out[a] = v;
          if (b != a) out[b] = v;
        }
      }
    }
    __syncthreads();
  }
}

int rows_of(int kind, long long d0, long long d1, long long d2) {
  return static_cast<int>(kind == OP_KM3 ? d1 : (kind == OP_KM3Q ? d2 : d0));
}

}  // namespace

long simt_k_total(const Operand &a) {
  if (a.kind == OP_KM3) return a.d0 * a.d2;
  if (a.kind == OP_KM3Q) return a.d0 * a.d1;
  return a.d1;
}

namespace {
bool make_sparams(const GemmArgs &g, SParams &p) {
  p.a_kind = g.a.kind;
  p.b_kind = g.b.kind;
  p.a = static_cast<const float *>(g.a.ptr);
  p.b = static_cast<const float *>(g.b.ptr);
  p.a0 = g.a.d0; p.a1 = g.a.d1; p.a2 = g.a.d2;
  p.b0 = g.b.d0; p.b1 = g.b.d1; p.b2 = g.b.d2;
  p.k_total = simt_k_total(g.a);
  if (simt_k_total(g.b) != p.k_total) return false;
  const int splits = g.splits < 1 ? 1 : g.splits;
  long long kps = (p.k_total + splits - 1) / splits;
  kps = (kps + BKS - 1) / BKS * BKS;
  p.k_per_split = kps;
  p.num_tiles = g.num_tiles;
  p.out_mode = g.out_mode;
  p.out = g.out;
  p.ld_out = g.ld_out;
  p.a_rows = rows_of(g.a.kind, g.a.d0, g.a.d1, g.a.d2);
  p.b_rows = rows_of(g.b.kind, g.b.d0, g.b.d1, g.b.d2);
  auto vec_of = [](const Operand &o) {
    if ((reinterpret_cast<uintptr_t>(o.ptr) & 15u) != 0) return 0;
    if (o.kind == OP_KM3 && o.d0 % BKS == 0) return 1;
    if (o.kind == OP_KM3Q && (o.d0 * o.d1) % 4 == 0) return 1;
    if (o.kind == OP_MN3 && o.d0 % 4 == 0) return 2;
    return 0;
  };
  p.a_vec = vec_of(g.a);
  p.b_vec = vec_of(g.b);
  return true;
}

// The host's copy of gen_tile for the row and slab generators.
bool host_tile(const TileGen &g, int idx, Tile &t) {
  t.a_z = 0;
  t.b_row = 0;
  t.out_col = 0;
  if (g.kind == TILES_ROWS) {
    t.a_row = 128 * idx;
    t.out_row = 128ll * idx;
    t.valid_rows = static_cast<int>(std::min(128ll, g.rows - 128ll * idx));
    t.valid_cols = std::min(g.cols, g.bn);
    return true;
  }
  if (g.kind == TILES_SLABS) {
    const long long nlb = (g.L + 127) / 128;
    const long long r = idx / nlb, lb = idx - r * nlb;
    t.a_row = static_cast<int>(128 * lb);
    t.a_z = static_cast<int>(r);
    t.out_row = 128 * lb + g.L * r;
    t.valid_rows = static_cast<int>(std::min(128ll, g.L - 128 * lb));
    t.valid_cols = std::min(g.cols, g.bn);
    return true;
  }
  return false;
}
}  // namespace

bool simt_grouped_add(const GemmArgs &g, std::vector<SParamsBlob> &gemms, std::vector<SimtBlockBlob> &blocks) {
  static_assert(sizeof(SParams) <= sizeof(SParamsBlob) && sizeof(SimtBlock) <= sizeof(SimtBlockBlob) &&
                    alignof(SParams) <= alignof(SParamsBlob) && alignof(SimtBlock) <= alignof(SimtBlockBlob),
                "blob sizes");
  if (g.gen.bn != 64 || g.out_mode != OUT_COLMAJOR || (g.gen.kind != TILES_ROWS && g.gen.kind != TILES_SLABS))
    return false;
  GemmArgs g1 = g;
  g1.splits = 1;
  SParams p;
  std::memset(&p, 0, sizeof(p));
  if (!make_sparams(g1, p)) return false;
  SParamsBlob pb;
  std::memset(&pb, 0, sizeof(pb));
  std::memcpy(&pb, &p, sizeof(p));
  const int gi = static_cast<int>(gemms.size());
  gemms.push_back(pb);
  for (int t = 0; t < g.num_tiles; ++t) {
    SimtBlock b;
    std::memset(&b, 0, sizeof(b));
    b.gemm = gi;
    if (!host_tile(g.gen, t, b.tile)) return false;
    SimtBlockBlob bb;
    std::memset(&bb, 0, sizeof(bb));
    std::memcpy(&bb, &b, sizeof(b));
    blocks.push_back(bb);
  }
  return true;
}

cudaError_t simt_grouped_launch(const SParamsBlob *gemms_dev, const SimtBlockBlob *blocks_dev, int nblocks,
                                cudaStream_t s) {
  if (nblocks < 1) return cudaSuccess;
  if (!gemms_dev || !blocks_dev) return cudaErrorInvalidValue;
  simt_gemm_grouped_kernel<<<nblocks, 256, 0, s>>>(gemms_dev, blocks_dev);
  return cudaGetLastError();
}

cudaError_t simt_gemm_launch(const GemmArgs &g, int bn, cudaStream_t s) {
  SParams p;
  if (!make_sparams(g, p)) return cudaErrorInvalidValue;
  const int splits = g.splits < 1 ? 1 : g.splits;
  const int grid = g.num_tiles * splits;
  if (bn == 128)
    simt_gemm_kernel<128><<<grid, 256, 0, s>>>(p, g.gen);
  else if (bn == 64)
    simt_gemm_kernel<64><<<grid, 256, 0, s>>>(p, g.gen);
  else if (bn == 32)
    simt_gemm_narrow_kernel<<<grid, 256, 0, s>>>(p, g.gen);
  else
    return cudaErrorInvalidValue;
  return cudaGetLastError();
}

cudaError_t reduce_partials_launch(const float *partial, const TileGen &gen, int splits, int bn, float *out,
                                   long long ld_out, int symmetric, cudaStream_t s) {
  const long long total = static_cast<long long>(gen.bm) * bn * gen.count;
  // split groups: about 8 partials per thread, at most 8 groups
  int groups = 1;
  while (groups < 8 && splits > 8 * groups) groups *= 2;
  const int nout = 256 / groups;
  long long blocks = (total + nout - 1) / nout;
  const long long cap = 16ll * device_sm_count();
  const int grid = static_cast<int>(blocks < cap ? blocks : cap);
  reduce_partials_kernel<<<grid, 256, 0, s>>>(partial, gen, gen.count, splits, bn, groups, out, ld_out, symmetric);
  return cudaGetLastError();
}

TileGen make_rows_gen(long long rows, int cols, int bn) {
  TileGen g{};
  g.kind = TILES_ROWS;
  g.bm = 128;
  g.rows = rows;
  g.cols = cols;
  g.bn = bn;
  g.count = static_cast<int>((rows + 127) / 128);
  return g;
}

TileGen make_slabs_gen(long long L, long long R, int cols, int bn) {
  TileGen g{};
  g.bm = 128;
  g.kind = TILES_SLABS;
  g.L = L;
  g.R = R;
  g.cols = cols;
  g.bn = bn;
  g.count = static_cast<int>(((L + 127) / 128) * R);
  return g;
}

bool make_grid_gen(long long rows, long long cols, int bn, TileGen *g) {
  *g = TileGen{};
  g->kind = TILES_GRID;
  g->bm = 128;
  g->bn = bn;
  g->rows = rows;
  g->n = cols;
  g->cols = bn;
  const long long count = ((rows + 127) / 128) * ((cols + bn - 1) / bn);
  if (rows < 1 || cols < 1 || count > (1ll << 30) || rows > (1ll << 31) - 256 || cols > (1ll << 31) - 256) return false;
  g->count = static_cast<int>(count);
  return true;
}

bool make_gram_gen(long long n, int bn, TileGen *g, int bm) {
  *g = TileGen{};
  g->kind = TILES_GRAM;
  g->n = n;
  g->bn = bn;
  g->bm = bm;
  const long long ni = (n + bm - 1) / bm, nj = (n + bn - 1) / bn;
  if (ni > kMaxGramRows) return false;
  g->ni = static_cast<int>(ni);
  int c = 0;
  for (long long i = 0; i < ni; ++i) {
    // first column block that reaches the diagonal: bn*(j+1) - 1 >= bm*i
    long long j0 = (static_cast<long long>(bm) * i + 1 + bn - 1) / bn - 1;
    if (j0 < 0) j0 = 0;
    g->prefix[i] = c;
    g->jmin[i] = static_cast<int>(j0);
    c += static_cast<int>(nj - j0);
  }
  g->prefix[ni] = c;
  g->count = c;
  return true;
}

}  // namespace htgb
