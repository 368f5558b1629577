// tcgen05 + TMA GEMM over tensor matricisations (BF16 in, FP32 accumulation in TMEM).
//
// One kernel serves the three unfolding products of the HT path, replacing the
// reference's cuBLAS calls (third_order_tensor_decompsition/CUDA/Optimized/
// htd_tensorcore.cu:83-121 leaf Grams, ttm.cu:38-87 TTMs, kernel.cu:610/618
// rsvd products):
//   Gram        G = X_(t) X_(t)^T           (A = B = the matricisation)
//   mode product Z = X_(t)^T-side * W       (contract one mode with a small matrix)
//   co-range    Z = X_(t) * Q               (contract all other modes)
// Operands are read straight from the column-major tensor through 3-D TMA
// tensor maps -- no permutation pass (the reference's mode2/mode2h kernels,
// kernel.cu:46-72) -- either K-major or MN-major, both with 128-byte swizzle.
//
// CTA layout (192 threads, one CTA per SM):
//   warp 0      TMA producer (one elected thread), STAGES-deep smem ring
//   warp 1      TMEM allocator + MMA issuer (one thread issues tcgen05.mma)
//   warps 2..5  epilogue: tcgen05.ld TMEM -> registers -> global
// Tile: M = 128 (TMEM lanes), N = BN (TMEM columns), K block = 64 (one 128 B row).
// Split-K across CTAs writes deterministic partial tiles that a separate
// kernel sums in a fixed order.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstring>
#include <mutex>

#include "common.cuh"
#include "engine.h"
#include "tiles.cuh"

namespace htgb {
namespace {

constexpr int BM = 128;
constexpr int BK = 64;
constexpr int kThreads = 192;

// MT = 2: a 256-row tile as two 128-row accumulators (TMEM columns [0, BN)
// and [BN, 2 BN)) that share every B stage: a third less shared-memory
// traffic per MMA than 128-row tiles, and a deeper ring in time.
template <int BN, int MT>
struct TcCfg {
  static constexpr int STAGES = MT == 2 ? (BN == 256 ? 3 : 4) : (BN == 256 ? 4 : (BN == 128 ? 6 : 3));
  static constexpr uint32_t A_BYTES = MT * BM * BK * 2;
  static constexpr uint32_t B_BYTES = BN * BK * 2;
  static constexpr uint32_t STAGE_BYTES = A_BYTES + B_BYTES;
  static constexpr size_t SMEM = 1024 + size_t(STAGES) * STAGE_BYTES + 256;
  static constexpr uint32_t TMEM_COLS = BN * MT;
};

struct KParams {
  int a_kind, b_kind;
  int a_lblocks, b_lblocks;
  int num_kb, kb_per_split;
  int num_tiles, out_mode;
  float *out;
  long long ld_out;
  int *err;
  int fold;
  int same;    // A and B are the same operand: a tile with a_row == b_row loads one panel
  __nv_bfloat16 *out16;   // OUT_COLMAJOR only: write the tile in BF16 here instead of FP32 to out
};

// Issue the TMA loads of one operand tile (ROWS x 64 K) for k-block kb.
template <int ROWS>
HT_DEV void load_operand(const CUtensorMap *map, int kind, int lblocks, int kb, int row, int z, uint8_t *dst,
                         uint64_t *bar) {
  if (kind == OP_MN3) {
    // ROWS/64 chunks of 64 MN-contiguous elements x 64 K rows (8 KiB each)
#pragma unroll
    for (int c = 0; c < ROWS / 64; ++c) tma_load_3d(dst + c * 8192, map, bar, row + 64 * c, kb * BK, z);
  } else {
    const int lb = kb % lblocks, r = kb / lblocks;
    if (kind == OP_KM3)
      tma_load_3d(dst, map, bar, lb * BK, row, r);
    else
      tma_load_3d(dst, map, bar, lb * BK, r, row);
  }
}

// Descriptor of the kk-th 16-wide K slice of an operand tile at smem address base.
HT_DEV uint64_t op_desc(int kind, uint32_t base, int kk) {
  if (kind == OP_MN3) return make_sdesc_sw128(base + kk * 2048, 8192, 1024);
  return make_sdesc_sw128(base + kk * 32, 16, 1024);
}

// One output tile (split `split` of its K range) of a CTA; the tensor maps
// may live in the kernel parameters or in global memory.
template <int BN, int MT>
HT_DEV void tc_gemm_tile(const CUtensorMap *tmA, const CUtensorMap *tmB, const KParams &p, const Tile &tile,
                         int tile_idx, int split) {
  using C = TcCfg<BN, MT>;
  constexpr int BMT = BM * MT;
  extern __shared__ uint8_t smem_raw[];
  uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t *full = reinterpret_cast<uint64_t *>(smem + C::STAGES * C::STAGE_BYTES);
  uint64_t *empty = full + C::STAGES;
  uint64_t *done = empty + C::STAGES;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(done + 1);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int kb0 = split * p.kb_per_split;
  const int nk = max(0, min(p.num_kb, kb0 + p.kb_per_split) - kb0);
  // a diagonal tile of a Gram with BN == BMT: A's rows are B's rows, so A is
  // read from B's stage instead of being loaded
  const bool a_in_b = (BN == BMT) && p.same && tile.a_row == tile.b_row;

  if (threadIdx.x == 0) {
    for (int s = 0; s < C::STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(done, 1);
    *abort_flag = 0;
    mbar_fence_init();
    tma_prefetch_desc(tmA);
    tma_prefetch_desc(tmB);
  }
  if (warp == 1) {
    tmem_alloc(tmem_slot, C::TMEM_COLS);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      int issued = 0;
      for (int i = 0; i < nk; ++i) {
        const int s = i % C::STAGES;
        const uint32_t ph = (i / C::STAGES) & 1;
        if (!mbar_wait_bounded(&empty[s], ph ^ 1, abort_flag)) {
          *abort_flag = 1;
          report_error(p.err, kErrTimeout);
          break;
        }
        uint8_t *sa = smem + s * C::STAGE_BYTES;
        uint8_t *sb = sa + C::A_BYTES;
        mbar_arrive_expect_tx(&full[s], a_in_b ? C::B_BYTES : C::STAGE_BYTES);
        if (!a_in_b) load_operand<BMT>(tmA, p.a_kind, p.a_lblocks, kb0 + i, tile.a_row, tile.a_z, sa, &full[s]);
        load_operand<BN>(tmB, p.b_kind, p.b_lblocks, kb0 + i, tile.b_row, 0, sb, &full[s]);
        issued = i + 1;
      }
      if (*abort_flag) {
        // let copies still in flight land before the CTA's smem is released
        for (int i = max(0, issued - C::STAGES); i < issued; ++i) {
          int dummy = 0;
          mbar_wait_bounded(&full[i % C::STAGES], (i / C::STAGES) & 1, &dummy);
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      const uint32_t idesc = make_idesc_bf16(BN, p.a_kind == OP_MN3, p.b_kind == OP_MN3);
      for (int i = 0; i < nk; ++i) {
        const int s = i % C::STAGES;
        const uint32_t ph = (i / C::STAGES) & 1;
        if (!mbar_wait_bounded(&full[s], ph, abort_flag)) {
          *abort_flag = 1;
          report_error(p.err, kErrTimeout);
          break;
        }
        tc_fence_after();
        const uint32_t sb = smem_u32(smem + s * C::STAGE_BYTES) + C::A_BYTES;
        const uint32_t sa = a_in_b ? sb : sb - C::A_BYTES;
#pragma unroll
        for (int kk = 0; kk < BK / 16; ++kk)
#pragma unroll
          for (int mt = 0; mt < MT; ++mt)   // rows mt*128.. of A start 16 KiB apart in both layouts
            umma_f16(tmem + static_cast<uint32_t>(mt * BN), op_desc(p.a_kind, sa + mt * (BM * BK * 2), kk),
                     op_desc(p.b_kind, sb, kk), idesc, (i | kk) != 0 ? 1u : 0u);
        umma_commit(&empty[s]);   // frees the stage once these MMAs have read it
      }
      umma_commit(done);           // accumulator complete (or abandoned)
    }
    __syncwarp();
  } else {
    const int q = warp & 3;        // TMEM lane quarter this warp may access
    bool ok = true;
    if (nk > 0) ok = mbar_wait_bounded(done, 0, abort_flag);
    ok = __all_sync(0xffffffffu, ok);
    if (!ok) report_error(p.err, kErrTimeout);
    tc_fence_after();
    const bool have = (nk > 0) && ok;
    const int cols = p.fold ? BN / 2 : BN;
#pragma unroll 1
    for (int it = 0; it < MT * (cols / 32); ++it) {
      const int mt = it / (cols / 32), c0 = (it % (cols / 32)) * 32;
      const int row = mt * BM + q * 32 + lane;
      float v[32];
      if (have) {
        const uint32_t lane_base = tmem + (static_cast<uint32_t>(q * 32) << 16) + static_cast<uint32_t>(mt * BN);
        tmem_ld_32x32b_x32(lane_base + static_cast<uint32_t>(c0), v);
        tmem_ld_wait();
        if (p.fold) {   // low half of the split B operand: add its product
          float w[32];
          tmem_ld_32x32b_x32(lane_base + static_cast<uint32_t>(c0 + BN / 2), w);
          tmem_ld_wait();
#pragma unroll
          for (int j = 0; j < 32; ++j) v[j] += w[j];
        }
      } else {
#pragma unroll
        for (int j = 0; j < 32; ++j) v[j] = 0.f;
      }
      if (p.out_mode == OUT_PARTIAL) {
        float *dst = p.out + ((static_cast<size_t>(split) * p.num_tiles + tile_idx) * BMT + row) * BN + c0;
#pragma unroll
        for (int j = 0; j < 32; j += 4) *reinterpret_cast<float4 *>(dst + j) = make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]);
      } else if (row < tile.valid_rows) {
        const long long off = tile.out_row + row + p.ld_out * static_cast<long long>(tile.out_col + c0);
        if (p.out16) {
          __nv_bfloat16 *dst = p.out16 + off;
#pragma unroll
          for (int j = 0; j < 32; ++j)
            if (c0 + j < tile.valid_cols) dst[p.ld_out * j] = __float2bfloat16_rn(v[j]);
        } else {
          float *dst = p.out + off;
#pragma unroll
          for (int j = 0; j < 32; ++j)
            if (c0 + j < tile.valid_cols) dst[p.ld_out * j] = v[j];
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem, C::TMEM_COLS);
  }
}

template <int BN, int MT>
__global__ void __launch_bounds__(kThreads, 1)
    tc_gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                   const KParams p, const TileGen gen) {
  const int tile_idx = blockIdx.x % p.num_tiles;
  tc_gemm_tile<BN, MT>(&tmA, &tmB, p, gen_tile(gen, tile_idx), tile_idx, blockIdx.x / p.num_tiles);
}

// Grouped Grams of a batch: CTA i computes items[i]'s whole n x n Gram
// (n <= BM * MT) as one tile over its full K range, written column-major.
struct GramItem {
  CUtensorMap map_a, map_b;   // 64-byte aligned (CUtensorMap's own alignment)
  KParams p;
  Tile tile;
};

template <int BN, int MT>
__global__ void __launch_bounds__(kThreads, 1) tc_gram_grouped_kernel(const GramItem *__restrict__ items) {
  const GramItem &it = items[blockIdx.x];
  const KParams p = it.p;
  const Tile tile = it.tile;
  tc_gemm_tile<BN, MT>(&it.map_a, &it.map_b, p, tile, 0, 0);
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
  });
  return fn;
}

bool check_operand(const Operand &o, std::string *why) {
  const long long d[3] = {o.d0, o.d1, o.d2};
  for (int i = 0; i < 3; ++i)
    if (d[i] < 1 || d[i] > (1ll << 31) - 1) {
      if (why) *why = "tensor-map dimension out of range";
      return false;
    }
  if ((o.d0 * 2) % 16 != 0) {
    if (why) *why = "innermost extent must be a multiple of 8 bf16 elements for TMA";
    return false;
  }
  if ((reinterpret_cast<uintptr_t>(o.ptr) & 15u) != 0) {
    if (why) *why = "operand base not 16-byte aligned";
    return false;
  }
  return true;
}

bool make_map(const Operand &o, int rows_box, CUtensorMap *map, std::string *why) {
  auto enc = encode_fn();
  if (!enc) {
    if (why) *why = "cuTensorMapEncodeTiled unavailable";
    return false;
  }
  cuuint64_t dims[3] = {cuuint64_t(o.d0), cuuint64_t(o.d1), cuuint64_t(o.d2)};
  cuuint64_t strides[2] = {cuuint64_t(o.d0) * 2, cuuint64_t(o.d0) * cuuint64_t(o.d1) * 2};
  cuuint32_t box[3];
  if (o.kind == OP_KM3) {
    box[0] = BK; box[1] = rows_box; box[2] = 1;
  } else if (o.kind == OP_KM3Q) {
    box[0] = BK; box[1] = 1; box[2] = rows_box;
  } else {
    box[0] = 64; box[1] = BK; box[2] = 1;
  }
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void *>(o.ptr), dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    if (why) *why = "cuTensorMapEncodeTiled failed (" + std::to_string(int(r)) + ")";
    return false;
  }
  return true;
}

long kblocks_of(const Operand &o) {
  if (o.kind == OP_MN3) return (o.d1 + BK - 1) / BK;
  const long lb = (o.d0 + BK - 1) / BK;
  return lb * (o.kind == OP_KM3 ? o.d2 : o.d1);
}

// Opt-in shared memory size, set once per instantiation and device.
template <int BN, int MT>
cudaError_t set_smem() {
  static bool done[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  if (done[dev]) return cudaSuccess;
  const cudaError_t e = cudaFuncSetAttribute(tc_gemm_kernel<BN, MT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             int(TcCfg<BN, MT>::SMEM));
  if (e == cudaSuccess) done[dev] = true;
  return e;
}

template <int BN, int MT>
cudaError_t launch_bn(const GemmArgs &g, cudaStream_t s) {
  using C = TcCfg<BN, MT>;
  if (g.gen.bm != BM * MT) return cudaErrorInvalidValue;
  CUtensorMap ma, mb;
  std::string why;
  if (!make_map(g.a, BM * MT, &ma, &why) || !make_map(g.b, BN, &mb, &why)) return cudaErrorInvalidValue;
  KParams p;
  p.a_kind = g.a.kind;
  p.b_kind = g.b.kind;
  p.a_lblocks = int((g.a.d0 + BK - 1) / BK);
  p.b_lblocks = int((g.b.d0 + BK - 1) / BK);
  p.num_kb = int(kblocks_of(g.a));
  const int splits = g.splits < 1 ? 1 : g.splits;
  p.kb_per_split = (p.num_kb + splits - 1) / splits;
  p.num_tiles = g.num_tiles;
  p.out_mode = g.out_mode;
  p.out = g.out;
  p.ld_out = g.ld_out;
  p.err = g.err;
  p.fold = (g.fold && g.out_mode == OUT_COLMAJOR) ? 1 : 0;
  p.out16 = g.out_mode == OUT_COLMAJOR ? g.out16 : nullptr;
  p.same = (g.a.ptr == g.b.ptr && g.a.kind == g.b.kind && g.a.d0 == g.b.d0 && g.a.d1 == g.b.d1 && g.a.d2 == g.b.d2) ? 1 : 0;
  cudaError_t e = set_smem<BN, MT>();
  if (e != cudaSuccess) return e;
  tc_gemm_kernel<BN, MT><<<g.num_tiles * splits, kThreads, C::SMEM, s>>>(ma, mb, p, g.gen);
  return cudaGetLastError();
}

}  // namespace

long tc_num_kblocks(const Operand &a) { return kblocks_of(a); }

// ---- grouped Grams of the batched path
int tc_gram_class(long n) { return n <= BM ? 0 : (n <= 2 * BM ? 1 : -1); }

size_t tc_gram_item_bytes() { return sizeof(GramItem); }

bool tc_gram_item(const Operand &a, long n, float *G, int *err, std::vector<unsigned char> &out, std::string *why) {
  const int cls = tc_gram_class(n);
  if (cls < 0 || !check_operand(a, why)) return false;
  GramItem it;
  std::memset(&it, 0, sizeof(it));
  const int bmt = cls == 0 ? BM : 2 * BM, bn = cls == 0 ? BM : 2 * BM;
  if (!make_map(a, bmt, &it.map_a, why) || !make_map(a, bn, &it.map_b, why)) return false;
  KParams &p = it.p;
  p.a_kind = p.b_kind = a.kind;
  p.a_lblocks = p.b_lblocks = int((a.d0 + BK - 1) / BK);
  p.num_kb = int(kblocks_of(a));
  p.kb_per_split = p.num_kb;
  p.num_tiles = 1;
  p.out_mode = OUT_COLMAJOR;
  p.out = G;
  p.ld_out = n;
  p.err = err;
  p.fold = 0;
  p.same = 1;
  p.out16 = nullptr;
  it.tile.a_row = it.tile.b_row = it.tile.a_z = 0;
  it.tile.valid_rows = int(n);
  it.tile.out_row = 0;
  it.tile.out_col = 0;
  it.tile.valid_cols = int(n);
  const unsigned char *raw = reinterpret_cast<const unsigned char *>(&it);
  out.insert(out.end(), raw, raw + sizeof(it));
  return true;
}

template <int BN, int MT>
cudaError_t set_grouped_smem() {
  static bool done[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  if (done[dev]) return cudaSuccess;
  const cudaError_t e = cudaFuncSetAttribute(tc_gram_grouped_kernel<BN, MT>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, int(TcCfg<BN, MT>::SMEM));
  if (e == cudaSuccess) done[dev] = true;
  return e;
}

cudaError_t tc_gram_grouped_launch(int cls, const void *items_dev, int count, cudaStream_t s) {
  if (count < 1) return cudaSuccess;
  if (!items_dev || (reinterpret_cast<uintptr_t>(items_dev) % alignof(GramItem)) != 0) return cudaErrorInvalidValue;
  const GramItem *it = static_cast<const GramItem *>(items_dev);
  if (cls == 0) {
    tc_gram_grouped_kernel<128, 1><<<count, kThreads, TcCfg<128, 1>::SMEM, s>>>(it);
  } else if (cls == 1) {
    tc_gram_grouped_kernel<256, 2><<<count, kThreads, TcCfg<256, 2>::SMEM, s>>>(it);
  } else {
    return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t tc_prepare() {
  if (!encode_fn()) return cudaErrorNotSupported;
  cudaError_t e;
  if ((e = set_grouped_smem<128, 1>()) != cudaSuccess) return e;
  if ((e = set_grouped_smem<256, 2>()) != cudaSuccess) return e;
  if ((e = set_smem<64, 1>()) != cudaSuccess) return e;
  if ((e = set_smem<128, 1>()) != cudaSuccess) return e;
  if ((e = set_smem<256, 1>()) != cudaSuccess) return e;
  return set_smem<256, 2>();
}

bool tc_gemm_supported(const GemmArgs &g, int bn, std::string *why) {
  if (bn != 64 && bn != 128 && bn != 256) {
    if (why) *why = "BN must be 64, 128 or 256";
    return false;
  }
  if (!check_operand(g.a, why) || !check_operand(g.b, why)) return false;
  if (g.b.kind == OP_MN3 && bn % 64 != 0) return false;
  if (kblocks_of(g.a) != kblocks_of(g.b)) {
    if (why) *why = "operand K extents differ";
    return false;
  }
  if (kblocks_of(g.a) > (1l << 30)) {
    if (why) *why = "K too large";
    return false;
  }
  if (!encode_fn()) {
    if (why) *why = "cuTensorMapEncodeTiled unavailable";
    return false;
  }
  return true;
}

cudaError_t tc_gemm_launch(const GemmArgs &g, int bn, cudaStream_t s) {
  if (g.mt == 2) {
    if (bn == 256) return launch_bn<256, 2>(g, s);
    return cudaErrorInvalidValue;
  }
  switch (bn) {
    case 64: return launch_bn<64, 1>(g, s);
    case 128: return launch_bn<128, 1>(g, s);
    case 256: return launch_bn<256, 1>(g, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace htgb
