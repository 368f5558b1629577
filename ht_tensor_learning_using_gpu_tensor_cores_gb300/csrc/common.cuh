// Shared device helpers: PTX wrappers for mbarrier / TMA / tcgen05, bounded
// waits, compensated (two-float) accumulation, a counter-based Gaussian RNG.
#pragma once
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <stdint.h>

#define HT_DEV __device__ __forceinline__

namespace htgb {

// Every spin-wait in this library gives up after this many nanoseconds of
// wall time, records an error and lets the kernel exit.
constexpr uint64_t kWaitLimitNs = 2000000000ull;   // 2 s

// Error bits written to the per-call device error word.
enum : int { kErrTimeout = 1, kErrNonFinite = 2, kErrBreakdown = 4 };

// Opt-in dynamic shared memory above 48 KB for `func`, once per device
// (`done` holds 64 per-device flags owned by the caller).
template <typename F>
inline cudaError_t opt_in_smem(F *func, int bytes, bool *done) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  if (done[dev]) return cudaSuccess;
  const cudaError_t e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess) done[dev] = true;
  return e;
}

HT_DEV uint32_t smem_u32(const void *p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

HT_DEV uint64_t global_timer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// ------------------------------------------------------------------ mbarrier
HT_DEV void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
HT_DEV void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
HT_DEV void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
HT_DEV bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Wait until the phase with the given parity has completed.  Returns false if
// the wait limit expired or another role of the CTA raised *abort.
HT_DEV bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, volatile int *abort) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_timer_ns();
  for (;;) {
#pragma unroll 1
    for (int i = 0; i < 32; ++i)
      if (mbar_try_wait(bar, parity)) return true;
    if (*abort) return false;
    if (global_timer_ns() - t0 > kWaitLimitNs) return false;
  }
}

// ----------------------------------------------------------------------- TMA
HT_DEV void tma_load_3d(void *smem_dst, const void *tmap, uint64_t *bar, int c0, int c1, int c2) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%3, %4, %5}], [%2];" ::"r"(smem_u32(smem_dst)),
      "l"(tmap), "r"(smem_u32(bar)), "r"(c0), "r"(c1), "r"(c2)
      : "memory");
}
HT_DEV void tma_prefetch_desc(const void *tmap) {
  asm volatile("prefetch.tensormap [%0];" ::"l"(tmap) : "memory");
}

// ------------------------------------------------------------------- tcgen05
HT_DEV void tmem_alloc(uint32_t *dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst_smem)),
               "r"(ncols)
               : "memory");
}
HT_DEV void tmem_relinquish() { asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory"); }
HT_DEV void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
HT_DEV void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
HT_DEV void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// D(tmem) (+)= A(smem) * B(smem)^T, BF16 inputs, FP32 accumulation.
HT_DEV void umma_f16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
// Arrive on an mbarrier once all previously issued tcgen05.mma of this thread complete.
HT_DEV void umma_commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}
HT_DEV void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// 32 lanes x 32 consecutive 32-bit columns: thread i of the warp receives lane
// (warp_quarter*32 + i), columns [col, col+32).
HT_DEV void tmem_ld_32x32b_x32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// Shared-memory matrix descriptor for tcgen05.mma, 128-byte swizzle.
//   K-major tiles : rows of 128 B (64 bf16 along K), 8-row atoms of 1 KiB: SBO = 1024.
//   MN-major tiles: 64-element MN chunks of (K rows x 128 B): LBO = chunk stride, SBO = 1024.
HT_DEV uint64_t make_sdesc_sw128(uint32_t saddr, uint32_t lbo_bytes, uint32_t sbo_bytes) {
  uint64_t d = 0;
  d |= static_cast<uint64_t>((saddr & 0x3FFFFu) >> 4);
  d |= static_cast<uint64_t>((lbo_bytes >> 4) & 0x3FFFu) << 16;
  d |= static_cast<uint64_t>((sbo_bytes >> 4) & 0x3FFFu) << 32;
  d |= 1ull << 46;   // descriptor version for tcgen05
  d |= 2ull << 61;   // SWIZZLE_128B
  return d;
}

// Instruction descriptor, kind::f16 with BF16 A/B and FP32 D, M = 128.
HT_DEV constexpr uint32_t make_idesc_bf16(int n, int a_mn_major, int b_mn_major) {
  return (1u << 4)                                  // D format: F32
         | (1u << 7)                                // A format: BF16
         | (1u << 10)                               // B format: BF16
         | (static_cast<uint32_t>(a_mn_major) << 15) // A major-ness
         | (static_cast<uint32_t>(b_mn_major) << 16) // B major-ness
         | (static_cast<uint32_t>(n >> 3) << 17)     // N / 8
         | (static_cast<uint32_t>(128 >> 4) << 24);  // M / 16
}

// ------------------------------------------------- compensated accumulation
// (s, c) holds an unevaluated sum s + c; add_prod adds a*b exactly up to the
// final rounding (TwoProduct via FMA + TwoSum; Ogita-Rump-Oishi "Dot2").
struct Acc2 {
  float s, c;
};
HT_DEV void acc2_add_prod(Acc2 &a, float x, float y) {
  const float p = x * y;
  const float e = fmaf(x, y, -p);
  const float t = a.s + p;
  const float z = t - a.s;
  a.c += (a.s - (t - z)) + (p - z) + e;
  a.s = t;
}
HT_DEV void acc2_add(Acc2 &a, float hi, float lo) {
  const float t = a.s + hi;
  const float z = t - a.s;
  a.c += (a.s - (t - z)) + (hi - z) + lo;
  a.s = t;
}

// ------------------------------------------------------------------- random
// Counter-based generator: splitmix64 of (seed, stream, index) -> standard
// normal by Box-Muller.  Deterministic for a given (seed, stream, index).
HT_DEV uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}
HT_DEV float gaussian(uint64_t seed, uint64_t stream, uint64_t idx) {
  const uint64_t h = splitmix64(seed ^ splitmix64(stream * 0xD1B54A32D192ED03ull + idx));
  const float u1 = (static_cast<float>(h >> 40) + 0.5f) * (1.0f / 16777216.0f);   // (0,1)
  const float u2 = static_cast<float>((h >> 16) & 0xFFFFFFu) * (1.0f / 16777216.0f);
  return sqrtf(-2.0f * logf(u1)) * cospif(2.0f * u2);
}

HT_DEV void report_error(int *err, int bits) {
  if (err) atomicOr(err, bits);
}

}  // namespace htgb
