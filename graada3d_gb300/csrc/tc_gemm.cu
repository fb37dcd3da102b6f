// Block products on the 5th-generation tensor cores: Y = G X and X = G^T Y
// for 16 right-hand sides with G stored in FP32 or as 16-bit entries with a
// per-row scale.
//
// Reference: sixteen of the reference's dense G_vec_mul / GT_vec_mul
// (src/Forward_modelling/Fwd.cpp:145, :111) at once.  With 16 right-hand
// sides the product reads G once for all of them, so it stays bound by HBM
// (8 FLOP/B for FP32 G, 16 for 16-bit G) while doing 16x the work of one
// product -- more multiply-adds than the FP32 CUDA cores retire at HBM speed,
// hence the tensor cores.
//
// Precision.  The MMA multiplies 32-bit-container TF32 (FP32 G) or 16-bit
// operands and accumulates in FP32 in tensor memory:
//  * FP32 G: split precision.  Each staged tile of G is split in shared
//    memory into big + small TF32 parts, each right-hand side likewise into
//    two TF32 parts; one MMA with N = 32 multiplies a G part by both
//    right-hand-side parts, so big*x_big + big*x_small + small*x_big
//    (+ small*x_small) recovers an FP32-accurate product.  The tensor core
//    reads an FP32 bit pattern as TF32 by truncation (checked on GB300), so
//    where the staged tile is already K-major (G^T Y) it is the big part
//    itself, big = trunc(g), and only small = rna(g - big) is written; for
//    G X the tile must be transposed to K-major (TF32 operands cannot be
//    MN-major) and big = rna(g), small = rna(g - big) are both written.
//  * 16-bit G: the stored entries are exact MMA operands; each right-hand
//    side is split into hi + lo 16-bit parts (N = 32 again).  Each column
//    is first scaled by a power of two so that its largest entry is in
//    [0.5, 1), which keeps FP16 parts in range; the scale is undone in FP64.
// Partial sums over K ranges are added in FP64 in a fixed order.
//
// Kernel structure (one persistent CTA per SM, warp-specialised):
//  warp 0     TMA producer: G tile and right-hand-side tile per stage into
//             a ring of shared-memory stages (128-byte swizzle), completion
//             on the stage's "full" mbarrier;
//  warp 1     MMA issuer (one thread): tcgen05.mma into one of two TMEM
//             accumulators, tcgen05.commit frees the stage;
//  warps 2-5  (FP32 G only) split each G tile into its two TF32 parts;
//  4 warps    epilogue: tcgen05.ld of the 128 x 32 accumulator, hi + lo
//             columns added, FP32 partial rows to global memory.
// Shapes: Y = G X takes M = rows of G (G is column-major, so the A tile is
// MN-major), N = 32, K = cells; X = G^T Y takes M = cells (A = G^T tile,
// K-major), K = rows.  The right-hand sides are prepared as a K-major
// [32][K] array (hi rows 0-15, lo rows 16-31).
//
// Every mbarrier wait is bounded (globaltimer): on expiry the CTA raises a
// flag in `err`, stops issuing, waits (bounded) for its own TMA loads and
// MMAs, frees its tensor memory and exits; the host turns the flag into an
// error status.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <mutex>

#include "../../include/grada_gpu.h"
#include "cg_kernels.h"
#include "common.cuh"
#include "kernels.h"

namespace grada {

namespace {

enum : int { ELT_TF32 = 0, ELT_BF16 = 1, ELT_F16 = 2 };
enum : int { MODE_GX = 0, MODE_GTY = 1 };

constexpr int TC_M = 128;                 // MMA M = TMEM lanes
constexpr int TC_N = 32;                  // MMA N = 16 columns x (hi, lo)
constexpr int SWB = 128;                  // swizzle span (bytes)
constexpr int A_BYTES = TC_M * SWB;       // 16 KB per stage, both modes
constexpr int B_BYTES = TC_N * SWB;       // 4 KB per stage
constexpr int TMEM_COLS = 2 * TC_N;       // two accumulators
constexpr uint64_t kWaitLimitNs = 1000000000ull;  // 1 s per wait
// try_wait suspends the thread until the phase completes or this many ns
// pass, so waiting warps do not spin on the issue slots
constexpr uint32_t kSuspendHintNs = 200000u;

// err bits
enum : int {
  TCERR_PRODUCER = 1,
  TCERR_CONVERT = 2,
  TCERR_MMA_FULL = 4,
  TCERR_MMA_ACC = 8,
  TCERR_EPILOGUE = 16,
  TCERR_DRAIN = 32
};

template <int ELT>
struct EltCfg {
  static constexpr int bytes = (ELT == ELT_TF32) ? 4 : 2;
  static constexpr int KS = SWB / bytes;         // K elements per stage (one 128 B row)
  static constexpr int KMMA = (ELT == ELT_TF32) ? 8 : 16;
  static constexpr int STEPS = KS / KMMA;        // MMAs per stage per G part
  static constexpr bool split_a = ELT == ELT_TF32;
  // TMA ring: A tile + right-hand-side tile per stage
  static constexpr int STAGE_BYTES = A_BYTES + B_BYTES;
  static constexpr int STAGES = split_a ? 6 : 10;
  // TF32 only: ring of converted slots (K-major big and small parts of A),
  // read by the MMAs together with the right-hand-side tile of the TMA stage
  static constexpr int CSLOT_BYTES = 2 * A_BYTES;
  static constexpr int CSLOTS = split_a ? 3 : 0;
#ifndef GRADA_TC_CONV_WARPS
#define GRADA_TC_CONV_WARPS 8
#endif
  static constexpr int NCONV_WARPS = split_a ? GRADA_TC_CONV_WARPS : 0;
  static constexpr int THREADS = 64 + 32 * NCONV_WARPS + 128;
  static constexpr int W_EPI0 = 2 + NCONV_WARPS;  // first epilogue warp
  static constexpr int SMEM = STAGES * STAGE_BYTES + CSLOTS * CSLOT_BYTES + 1024;
  static constexpr int ATOM_M = SWB / bytes;     // MN-major atom: rows of G per 128 B
};

// Ring sizes per product.  TF32 G^T Y keeps only the small part in a
// converted slot (the staged tile is the big part), so its slots are half the
// size and the TMA ring gets the room; TF32 G X keeps both parts.
#ifndef GRADA_TC_GX_STAGES
#define GRADA_TC_GX_STAGES 6
#endif
#ifndef GRADA_TC_GX_SLOTS
#define GRADA_TC_GX_SLOTS 3
#endif
#ifndef GRADA_TC_GTY_STAGES
#define GRADA_TC_GTY_STAGES 8
#endif
template <int MODE, int ELT>
struct Cfg : EltCfg<ELT> {
  using E = EltCfg<ELT>;
  static constexpr int STAGES =
      !E::split_a ? E::STAGES : (MODE == 0 ? GRADA_TC_GX_STAGES : GRADA_TC_GTY_STAGES);
  static constexpr int CSLOT_BYTES = (MODE == 0 ? 2 : 1) * A_BYTES;
  static constexpr int CSLOTS = !E::split_a ? 0 : (MODE == 0 ? GRADA_TC_GX_SLOTS : 3);
  static constexpr int SMEM = STAGES * E::STAGE_BYTES + CSLOTS * CSLOT_BYTES + 1024;
  static_assert(SMEM <= 227 * 1024, "shared memory budget");
};

struct TcParams {
  int64_t m_rows;      // rows of the output (GX: ld, GTY: cells)
  int n_mtiles;
  int n_splits;
  int kst_total;       // K stages in all
  int kst_per_split;
  int64_t m_pad;       // n_mtiles * TC_M
  float *partial;      // [n_splits][m_pad][16]
  int *err;
  const int *skip;
};

// ---- PTX helpers ------------------------------------------------------------

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ uint64_t gtimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void mbar_arrive_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity), "r"(kSuspendHintNs)
      : "memory");
  return ok != 0;
}

// Non-blocking test of the phase of parity `parity` of `bar`.
__device__ __forceinline__ bool mbar_test(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait for the phase of parity `parity` of `bar`.  Returns false when
// the CTA is aborting (watch_abort) or the time limit ran out; the latter
// raises the abort flag and `code` in err.  limit_ns = 0 (the expiry test of
// grada_inject_fault) does not wait at all: a phase not complete at the first
// test expires.
__device__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int *abort_flag, int *err,
                          int code, uint64_t limit_ns, bool watch_abort = true) {
  if (limit_ns == 0) {
    if (mbar_test(bar, parity)) return true;
    if (watch_abort && *abort_flag) return false;
    *abort_flag = 1;
    atomicOr(err, code);
    return false;
  }
  if (mbar_try(bar, parity)) return true;
  const uint64_t t0 = gtimer();
  for (uint32_t n = 1;; n++) {
    if (mbar_try(bar, parity)) return true;
    if ((n & 15) == 0) {
      if (watch_abort && *abort_flag) return false;
      if (gtimer() - t0 > limit_ns) {
        *abort_flag = 1;
        atomicOr(err, code);
        return false;
      }
    }
  }
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int x, int y,
                                            uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
      : "memory");
}

// Shared-memory matrix descriptor: 128-byte swizzle, sm_100-family version 1.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}

// Instruction descriptor: FP32 accumulator, A/B format, A major-ness,
// N = TC_N, M = TC_M.
__host__ __device__ constexpr uint32_t idesc(int elt, bool a_mn_major) {
  const uint32_t f = elt == ELT_TF32 ? 2u : (elt == ELT_BF16 ? 1u : 0u);
  return (1u << 4) | (f << 7) | (f << 10) | ((a_mn_major ? 1u : 0u) << 15) |
         ((uint32_t)(TC_N >> 3) << 17) | ((uint32_t)(TC_M >> 4) << 24);
}

template <int ELT>
__device__ __forceinline__ void mma(uint32_t dt, uint64_t a, uint64_t b, uint32_t id,
                                    uint32_t accum) {
  if constexpr (ELT == ELT_TF32) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(dt),
        "l"(a), "l"(b), "r"(id), "r"(accum)
        : "memory");
  } else {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(dt),
        "l"(a), "l"(b), "r"(id), "r"(accum)
        : "memory");
  }
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
      : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// FP32 -> TF32, round to nearest with ties away from zero (the rounding of
// cvt.rna.tf32.f32) on the integer pipe: adding half a TF32 ulp (bit 12) to
// the sign-magnitude bit pattern carries into the kept bits exactly when the
// dropped 13 bits are >= half an ulp.  Conversions run on a narrow pipe on
// this GPU; two integer operations do not.
__device__ __forceinline__ uint32_t f32_to_tf32(float x) {
  return (__float_as_uint(x) + 0x1000u) & 0xFFFFE000u;
}

// 32 lanes x 32 columns of FP32 from TMEM (this warp's lane quarter).
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
        "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
        "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int k = 0; k < 32; k++) v[k] = __uint_as_float(r[k]);
}

// ---- the kernel -------------------------------------------------------------

template <int MODE, int ELT>
__global__ void __launch_bounds__(EltCfg<ELT>::THREADS, 1)
    tc_gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                   const TcParams p) {
  using C = Cfg<MODE, ELT>;
  if (p.skip && *p.skip) return;
  extern __shared__ uint8_t smem_raw[];
  constexpr int NCS = C::CSLOTS > 0 ? C::CSLOTS : 1;
  __shared__ __align__(8) uint64_t bar_full[C::STAGES], bar_empty[C::STAGES];
  __shared__ __align__(8) uint64_t bar_cfull[NCS], bar_cempty[NCS];
  __shared__ __align__(8) uint64_t bar_acc_full[2], bar_acc_empty[2], bar_drain;
  __shared__ uint32_t tmem_base_s;
  __shared__ volatile int abort_flag;

  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const uint32_t base = (smem_u32(smem_raw) + 1023u) & ~1023u;
  auto stage_a = [&](int s) { return base + (uint32_t)s * C::STAGE_BYTES; };
  auto stage_b = [&](int s) { return stage_a(s) + A_BYTES; };
  const uint32_t cbase = base + (uint32_t)C::STAGES * C::STAGE_BYTES;
  auto cslot_big = [&](int c) { return cbase + (uint32_t)c * C::CSLOT_BYTES; };
  // G X slots: [big][small]; G^T Y slots: [small]
  auto cslot_small = [&](int c) { return cslot_big(c) + (MODE == MODE_GX ? A_BYTES : 0); };
  uint8_t *base_ptr = smem_raw + (base - smem_u32(smem_raw));

  if (threadIdx.x == 0) {
    abort_flag = 0;
    for (int s = 0; s < C::STAGES; s++) {
      mbar_init(smem_u32(&bar_full[s]), 1);
      mbar_init(smem_u32(&bar_empty[s]), 1);  // freed by the MMA commit
    }
    for (int c = 0; c < NCS; c++) {
      mbar_init(smem_u32(&bar_cfull[c]), C::NCONV_WARPS > 0 ? C::NCONV_WARPS : 1);
      mbar_init(smem_u32(&bar_cempty[c]), 1);
    }
    for (int a = 0; a < 2; a++) {
      mbar_init(smem_u32(&bar_acc_full[a]), 1);
      mbar_init(smem_u32(&bar_acc_empty[a]), 4);
    }
    mbar_init(smem_u32(&bar_drain), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_base_s)),
                 "r"((uint32_t)TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base_s;

  // main-loop waits: the usual limit, or none at all while the expiry test of
  // grada_inject_fault (err[1]) is armed; drains always keep the usual limit
  const uint64_t wait_ns = (p.err && p.err[1]) ? 0ull : kWaitLimitNs;
  const int n_units = p.n_mtiles * p.n_splits;
  auto unit_mtile = [&](int u) { return u % p.n_mtiles; };
  auto unit_split = [&](int u) { return u / p.n_mtiles; };
  auto unit_kst = [&](int u, int &k0, int &k1) {
    k0 = unit_split(u) * p.kst_per_split;
    k1 = min(p.kst_total, k0 + p.kst_per_split);
  };

  if (warp == 0) {
    // ---------------- TMA producer ----------------
    if (lane == 0) {
      uint32_t it = 0;
      bool ok = true;
      for (int u = blockIdx.x; u < n_units && ok; u += gridDim.x) {
        const int mt = unit_mtile(u);
        int k0, k1;
        unit_kst(u, k0, k1);
        for (int ks = k0; ks < k1; ks++, it++) {
          const int s = (int)(it % C::STAGES);
          const uint32_t ph = (it / C::STAGES) & 1u;
          if (!mbar_wait(smem_u32(&bar_empty[s]), ph ^ 1u, &abort_flag, p.err, TCERR_PRODUCER, wait_ns)) {
            ok = false;
            break;
          }
          const uint32_t fb = smem_u32(&bar_full[s]);
          mbar_arrive_tx(fb, A_BYTES + B_BYTES);
          const int kx = ks * C::KS;
          if constexpr (MODE == MODE_GX) {
            // A = G rows [mt*128, +128) x cells [kx, +KS): TC_M / ATOM_M boxes of
            // ATOM_M rows x KS cells, each KS x 128 B
#pragma unroll
            for (int a = 0; a < TC_M / C::ATOM_M; a++)
              tma_load_2d(stage_a(s) + (uint32_t)a * (C::KS * SWB), &tmA,
                          mt * TC_M + a * C::ATOM_M, kx, fb);
          } else {
            // A = G^T tile: rows [kx, +KS) x cells [mt*128, +128): 128 x 128 B
            tma_load_2d(stage_a(s), &tmA, kx, mt * TC_M, fb);
          }
          tma_load_2d(stage_b(s), &tmB, kx, 0, fb);
        }
      }
      // wait for the loads still in flight (their stages may be unconsumed
      // when the CTA aborts)
      const uint32_t n_out = it < (uint32_t)C::STAGES ? it : (uint32_t)C::STAGES;
      for (uint32_t q = 0; q < n_out; q++) {
        const uint32_t j = it - 1 - q;
        mbar_wait(smem_u32(&bar_full[j % C::STAGES]), (j / C::STAGES) & 1u, &abort_flag, p.err,
                  TCERR_DRAIN, kWaitLimitNs, false);
      }
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      uint32_t it = 0, uc = 0;
      bool ok = true;
      constexpr uint32_t id = idesc(ELT, (MODE == MODE_GX) && !C::split_a);
      // A descriptor geometry: MN-major only for 16-bit G in G X (TF32 operands
      // must be K-major; the split warps transpose those tiles)
      constexpr bool a_mn = (MODE == MODE_GX) && !C::split_a;
      constexpr uint32_t a_lbo = a_mn ? (uint32_t)(C::KS * SWB) : 16u;
      constexpr uint32_t a_sbo = 1024u;
      constexpr uint32_t a_step = a_mn ? (uint32_t)(C::KMMA / 8 * 1024)
                                       : (uint32_t)(C::KMMA * C::bytes);
      constexpr uint32_t b_step = (uint32_t)(C::KMMA * C::bytes);
      for (int u = blockIdx.x; u < n_units && ok; u += gridDim.x, uc++) {
        const int acc = (int)(uc & 1u);
        const uint32_t aph = (uc >> 1) & 1u;
        if (!mbar_wait(smem_u32(&bar_acc_empty[acc]), aph ^ 1u, &abort_flag, p.err,
                       TCERR_MMA_ACC, wait_ns)) {
          ok = false;
          break;
        }
        tc_fence_after();
        const uint32_t dt = tmem + (uint32_t)(acc * TC_N);
        int k0, k1;
        unit_kst(u, k0, k1);
        uint32_t accum = 0;
        for (int ks = k0; ks < k1; ks++, it++) {
          const int s = (int)(it % C::STAGES);
          uint32_t ph, wb, a_s;
          const uint32_t b_s = stage_b(s);
          int c = 0;
          if constexpr (C::split_a) {
            c = (int)(it % NCS);
            ph = (it / NCS) & 1u;
            wb = smem_u32(&bar_cfull[c]);  // implies the stage's TMA completed
            a_s = cslot_big(c);
          } else {
            ph = (it / C::STAGES) & 1u;
            wb = smem_u32(&bar_full[s]);
            a_s = stage_a(s);
          }
          if (!mbar_wait(wb, ph, &abort_flag, p.err, TCERR_MMA_FULL, wait_ns)) {
            ok = false;
            break;
          }
          if constexpr (C::split_a) {
            // the right-hand-side tile comes straight from the TMA stage
            if (!mbar_wait(smem_u32(&bar_full[s]), (it / C::STAGES) & 1u, &abort_flag, p.err,
                           TCERR_MMA_FULL, wait_ns)) {
              ok = false;
              break;
            }
          }
          tc_fence_after();
          // TF32: the big part is the converted slot's (G X) or, for G^T Y, the
          // staged FP32 tile itself, which the tensor core reads truncated to
          // TF32; the small part is always the slot's
          uint32_t a_big = a_s;
          if constexpr (C::split_a && MODE == MODE_GTY) a_big = stage_a(s);
#pragma unroll
          for (int st = 0; st < C::STEPS; st++) {
            const uint64_t bd = sdesc(b_s + st * b_step, 16u, 1024u);
            mma<ELT>(dt, sdesc(a_big + st * a_step, a_lbo, a_sbo), bd, id, accum);
            accum = 1;
            if constexpr (C::split_a)
              mma<ELT>(dt, sdesc(cslot_small(c) + st * a_step, a_lbo, a_sbo), bd, id, 1);
          }
          mma_commit(smem_u32(&bar_empty[s]));  // stage free once these MMAs are done
          if constexpr (C::split_a) mma_commit(smem_u32(&bar_cempty[c]));
        }
        if (!ok) break;
        mma_commit(smem_u32(&bar_acc_full[acc]));
      }
      // all MMAs of this thread complete before the CTA releases TMEM
      mma_commit(smem_u32(&bar_drain));
      mbar_wait(smem_u32(&bar_drain), 0, &abort_flag, p.err, TCERR_DRAIN, kWaitLimitNs, false);
    }
  } else if (C::split_a && warp < C::W_EPI0) {
    // ---------------- TF32 split (and K-major transpose) of the G tile ----------
    // The big and small TF32 parts of a TMA stage's A tile go to a converted
    // slot in the K-major 128B-swizzled layout (row m of 128 B holds k =
    // 0..31; 16-byte chunk j of row m at chunk j ^ (m & 7)); the MMAs read the
    // right-hand-side tile from the TMA stage, which their commit frees.
    // (16-bit instantiations have no split warps and never get here; the
    // floor of TC_M keeps their compile-time arithmetic defined)
    constexpr int NCT = C::NCONV_WARPS > 0 ? 32 * C::NCONV_WARPS : TC_M;
    const int ct = threadIdx.x - 64;  // 0..NCT-1
    uint32_t it = 0;
    bool ok = true;
    for (int u = blockIdx.x; u < n_units && ok; u += gridDim.x) {
      int k0, k1;
      unit_kst(u, k0, k1);
      for (int ks = k0; ks < k1; ks++, it++) {
        const int s = (int)(it % C::STAGES);
        const uint32_t ph = (it / C::STAGES) & 1u;
        const int c = (int)(it % NCS);
        const uint32_t cph = (it / NCS) & 1u;
        if (!mbar_wait(smem_u32(&bar_full[s]), ph, &abort_flag, p.err, TCERR_CONVERT, wait_ns) ||
            !mbar_wait(smem_u32(&bar_cempty[c]), cph ^ 1u, &abort_flag, p.err, TCERR_CONVERT, wait_ns)) {
          ok = false;
          break;
        }
        const float *raw = reinterpret_cast<const float *>(base_ptr + (stage_a(s) - base));
        float4 *big = reinterpret_cast<float4 *>(base_ptr + (cslot_big(c) - base));
        float4 *small = reinterpret_cast<float4 *>(base_ptr + (cslot_small(c) - base));
        auto split4 = [&](const float (&v)[4], int idx4) {
          float b[4], sm[4];
#pragma unroll
          for (int q = 0; q < 4; q++) {
            b[q] = __uint_as_float(f32_to_tf32(v[q]));
            sm[q] = __uint_as_float(f32_to_tf32(v[q] - b[q]));
          }
          big[idx4] = make_float4(b[0], b[1], b[2], b[3]);
          small[idx4] = make_float4(sm[0], sm[1], sm[2], sm[3]);
        };
        if constexpr (MODE == MODE_GX) {
          // raw: 4 MN-major atoms (32 rows x 32 k, row k of 128 B holds 32 m);
          // thread = row m of the K-major result, NCT / 128 threads per row
          // sharing its eight 16-byte chunks
          constexpr int TPR = NCT / TC_M;
          const int m = ct % TC_M, atom = m >> 5, mm = m & 31;
#pragma unroll
          for (int jj = 0; jj < 8 / TPR; jj++) {
            const int j = jj * TPR + ct / TC_M;
            float v[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
              const int k = 4 * j + q;
              const int off = atom * (C::KS * SWB) + k * SWB + ((((mm >> 2) ^ (k & 7))) << 4) +
                              (mm & 3) * 4;
              v[q] = raw[off >> 2];
            }
            split4(v, (m * SWB + ((j ^ (m & 7)) << 4)) >> 4);
          }
        } else {
          // raw is already K-major and serves as the big part (read truncated
          // to TF32 by the tensor core): only small = rna(g - trunc(g)) is
          // written, element-wise
          const float4 *r4 = reinterpret_cast<const float4 *>(raw);
#pragma unroll
          for (int j = 0; j < A_BYTES / 16 / NCT; j++) {
            const int idx = ct + NCT * j;
            const float4 v4 = r4[idx];
            const float v[4] = {v4.x, v4.y, v4.z, v4.w};
            float sm[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
              const float t = __uint_as_float(__float_as_uint(v[q]) & 0xFFFFE000u);
              sm[q] = __uint_as_float(f32_to_tf32(v[q] - t));
            }
            small[idx] = make_float4(sm[0], sm[1], sm[2], sm[3]);
          }
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncwarp();
        if (lane == 0) mbar_arrive(smem_u32(&bar_cfull[c]));
      }
    }
  } else if (warp >= C::W_EPI0) {
    // ---------------- epilogue ----------------
    const int quarter = warp % 4;  // TMEM lanes 32*quarter .. +31
    uint32_t uc = 0;
    for (int u = blockIdx.x; u < n_units; u += gridDim.x, uc++) {
      const int acc = (int)(uc & 1u);
      const uint32_t aph = (uc >> 1) & 1u;
      if (!mbar_wait(smem_u32(&bar_acc_full[acc]), aph, &abort_flag, p.err, TCERR_EPILOGUE, wait_ns))
        break;
      tc_fence_after();
      __syncwarp();
      float v[32];
      tmem_ld32(tmem + ((uint32_t)(32 * quarter) << 16) + (uint32_t)(acc * TC_N), v);
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(smem_u32(&bar_acc_empty[acc]));
      const int64_t row = (int64_t)unit_mtile(u) * TC_M + 32 * quarter + lane;
      if (row < p.m_rows) {
        float4 *out = reinterpret_cast<float4 *>(
            p.partial + ((int64_t)unit_split(u) * p.m_pad + row) * kBW);
#pragma unroll
        for (int q = 0; q < 4; q++)
          out[q] = make_float4(v[4 * q] + v[16 + 4 * q], v[4 * q + 1] + v[17 + 4 * q],
                               v[4 * q + 2] + v[18 + 4 * q], v[4 * q + 3] + v[19 + 4 * q]);
      }
    }
  }

  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    __syncwarp();
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"((uint32_t)TMEM_COLS)
                 : "memory");
  }
}

// ---- right-hand-side preparation and the final sums ---------------------

constexpr int PT = 256;

// Per-column max |x * pre * rs| over rows [0, n): partial[b][c].
__global__ void colmax_kernel(const double *__restrict__ x, int64_t n,
                              const double *__restrict__ pre, const float *__restrict__ rs,
                              double *__restrict__ partial, const int *__restrict__ skip) {
  if (skip && *skip) return;
  __shared__ double red[PT / kBW][kBW];
  const int rl = threadIdx.x / kBW, c = threadIdx.x % kBW;
  double m = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * (PT / kBW) + rl; i < n;
       i += (int64_t)gridDim.x * (PT / kBW)) {
    double v = x[i * kBW + c];
    if (pre) v *= pre[i];
    if (rs) v *= (double)rs[i];
    m = fmax(m, fabs(v));
  }
  red[rl][c] = m;
  __syncthreads();
  if (threadIdx.x < kBW) {
    double s = 0.0;
    for (int k = 0; k < PT / kBW; k++) s = fmax(s, red[k][threadIdx.x]);
    partial[(int64_t)blockIdx.x * kBW + threadIdx.x] = s;
  }
}

// scale[c] = 2^-e with max_c = f 2^e, f in [0.5, 1) (1 for an all-zero column).
__global__ void colscale_kernel(const double *__restrict__ partial, int nb,
                                double *__restrict__ scale, const int *__restrict__ skip) {
  if (skip && *skip) return;
  const int c = threadIdx.x;
  if (c >= kBW) return;
  double m = 0.0;
  for (int b = 0; b < nb; b++) m = fmax(m, partial[(int64_t)b * kBW + c]);
  double sc = 1.0;
  if (m > 0.0 && isfinite(m)) {
    int e;
    frexp(m, &e);
    sc = ldexp(1.0, -e);
  }
  scale[c] = sc;
}

template <int ELT>
__device__ __forceinline__ void split_value(double v, uint32_t &hi, uint32_t &lo) {
  if constexpr (ELT == ELT_TF32) {
    const float f = (float)v;
    hi = f32_to_tf32(f);
    lo = f32_to_tf32((float)(v - (double)__uint_as_float(hi)));
  } else if constexpr (ELT == ELT_BF16) {
    const __nv_bfloat16 h = __double2bfloat16(v);
    hi = __bfloat16_as_ushort(h);
    lo = __bfloat16_as_ushort(__double2bfloat16(v - (double)__bfloat162float(h)));
  } else {
    const __half h = __double2half(v);
    hi = __half_as_ushort(h);
    lo = __half_as_ushort(__double2half(v - (double)__half2float(h)));
  }
}

// bt[c][k] = hi(x(k, c) s_c), bt[16 + c][k] = lo(...) for k < kpad (0 for k >= n).
// A block transposes 64 rows x 16 columns through shared memory.
template <int ELT>
__global__ void split_kernel(const double *__restrict__ x, int64_t n, int64_t kpad,
                             const double *__restrict__ pre, const float *__restrict__ rs,
                             const double *__restrict__ scale, void *__restrict__ bt,
                             const int *__restrict__ skip) {
  if (skip && *skip) return;
  constexpr int TK = 64;
  __shared__ uint32_t th[2 * kBW][TK + 1];
  const int64_t k0 = (int64_t)blockIdx.x * TK;
  for (int e = threadIdx.x; e < TK * kBW; e += PT) {
    const int kk = e / kBW, c = e % kBW;
    const int64_t k = k0 + kk;
    uint32_t hi = 0, lo = 0;
    if (k < n) {
      double v = x[k * kBW + c];
      if (pre) v *= pre[k];
      if (rs) v *= (double)rs[k];
      split_value<ELT>(v * scale[c], hi, lo);
    }
    th[c][kk] = hi;
    th[kBW + c][kk] = lo;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < 2 * kBW * TK; e += PT) {
    const int r = e / TK, kk = e % TK;
    const int64_t k = k0 + kk;
    if (k >= kpad) continue;
    if constexpr (ELT == ELT_TF32)
      static_cast<uint32_t *>(bt)[r * kpad + k] = th[r][kk];
    else
      static_cast<uint16_t *>(bt)[r * kpad + k] = (uint16_t)th[r][kk];
  }
}

// out(r, c) = post(r) * rs(r) * (sum over splits of partial) / scale_c, r < n.
__global__ void tc_finish_kernel(const float *__restrict__ partial, int n_split, int64_t m_pad,
                                 int64_t n, const double *__restrict__ scale,
                                 const float *__restrict__ rs, const double *__restrict__ post,
                                 double *__restrict__ out, const int *__restrict__ skip) {
  if (skip && *skip) return;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n * kBW) return;
  const int64_t r = e / kBW;
  double s = 0.0;
  for (int k = 0; k < n_split; k++) s += (double)partial[(int64_t)k * m_pad * kBW + e];
  s /= scale[e % kBW];
  if (rs) s *= (double)rs[r];
  if (post) s *= post[r];
  out[e] = s;
}

// ---- host side --------------------------------------------------------------

int elt_of(const DevG &G) {
  switch (G.kind) {
    case GKind::FP32: return ELT_TF32;
    case GKind::BF16: return ELT_BF16;
    case GKind::FP16: return ELT_F16;
    default: throw Error(GRADA_ERR_INVALID_ARGUMENT, "tensor-core products need FP32 or 16-bit G");
  }
}

int elt_bytes(int elt) { return elt == ELT_TF32 ? 4 : 2; }
int elt_ks(int elt) { return SWB / elt_bytes(elt); }

struct TcLayout {
  int n_mtiles, n_splits, kst_total, kst_per_split;
  int64_t m_rows, m_pad, k_len, kpad;
  int colmax_blocks;
  // byte offsets in the scratch
  int64_t off_bt, off_partial, off_colmax, off_scale, total;
};

int pick_splits(int n_mtiles, int kst_total, int sm_count) {
  const int max_s = std::max(1, std::min(64, kst_total / 8));
  int best = 1;
  double best_eff = -1.0;
  for (int s = 1; s <= max_s; s++) {
    const int64_t units = (int64_t)n_mtiles * s;
    const int64_t waves = ceil_div(units, sm_count);
    const double eff = (double)units / (double)(waves * sm_count);
    if (eff > best_eff + 1e-9) {
      best_eff = eff;
      best = s;
    }
    if (eff > 0.97 && units >= sm_count) break;
  }
  return best;
}

TcLayout tc_layout(const DevG &G, int mode, int sm_count) {
  const int elt = elt_of(G);
  TcLayout L;
  L.m_rows = (mode == MODE_GX) ? G.ld : G.nm;
  L.k_len = (mode == MODE_GX) ? G.nm : G.ld;
  L.n_mtiles = (int)ceil_div(L.m_rows, TC_M);
  L.m_pad = (int64_t)L.n_mtiles * TC_M;
  L.kst_total = (int)ceil_div(L.k_len, elt_ks(elt));
  L.n_splits = pick_splits(L.n_mtiles, L.kst_total, sm_count);
  L.kst_per_split = (int)ceil_div(L.kst_total, L.n_splits);
  L.n_splits = (int)ceil_div(L.kst_total, L.kst_per_split);  // no empty split
  L.kpad = round_up(L.k_len, 64);
  const int64_t kin = (mode == MODE_GX) ? G.nm : G.nd;  // rows of the input block
  L.colmax_blocks = (int)std::max<int64_t>(1, std::min<int64_t>(sm_count * 2, ceil_div(kin, PT / kBW)));
  L.off_bt = 0;
  L.off_partial = round_up(2 * kBW * L.kpad * elt_bytes(elt), 256);
  L.off_colmax =
      L.off_partial + round_up((int64_t)L.n_splits * L.m_pad * kBW * (int64_t)sizeof(float), 256);
  L.off_scale = L.off_colmax + round_up((int64_t)L.colmax_blocks * kBW * 8, 256);
  L.total = L.off_scale + 256;
  return L;
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static std::mutex mu;
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  std::lock_guard<std::mutex> lock(mu);
  if (!fn) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    GRADA_CUDA_CHECK(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                                      cudaEnableDefault, &q));
    if (q != cudaDriverEntryPointSuccess || !p)
      throw Error(GRADA_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
    fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

CUtensorMap make_map(const void *ptr, int elt, uint64_t dim0, uint64_t dim1, uint64_t stride1_bytes,
                     uint32_t box0, uint32_t box1) {
  CUtensorMap m;
  const CUtensorMapDataType dt = elt == ELT_TF32   ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32
                                 : elt == ELT_BF16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16
                                                   : CU_TENSOR_MAP_DATA_TYPE_FLOAT16;
  const cuuint64_t dims[2] = {dim0, dim1};
  const cuuint64_t strides[1] = {stride1_bytes};
  const cuuint32_t box[2] = {box0, box1};
  const cuuint32_t es[2] = {1, 1};
  const CUresult r = encode_fn()(&m, dt, 2, const_cast<void *>(ptr), dims, strides, box, es,
                                 CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                 CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                 CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS)
    throw Error(GRADA_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
  return m;
}

template <int MODE, int ELT>
void launch_kernel(const CUtensorMap &a, const CUtensorMap &b, const TcParams &p, int grid,
                   cudaStream_t s) {
  using C = Cfg<MODE, ELT>;
  static std::mutex mu;
  static bool attr_set[64] = {};
  int dev = 0;
  GRADA_CUDA_CHECK(cudaGetDevice(&dev));
  {
    std::lock_guard<std::mutex> lock(mu);
    if (dev < 0 || dev >= 64 || !attr_set[dev]) {
      GRADA_CUDA_CHECK(cudaFuncSetAttribute(tc_gemm_kernel<MODE, ELT>,
                                            cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM));
      if (dev >= 0 && dev < 64) attr_set[dev] = true;
    }
  }
  tc_gemm_kernel<MODE, ELT><<<grid, C::THREADS, C::SMEM, s>>>(a, b, p);
  GRADA_LAUNCH_CHECK();
}

template <int MODE>
void dispatch(int elt, const CUtensorMap &a, const CUtensorMap &b, const TcParams &p, int grid,
              cudaStream_t s) {
  if (elt == ELT_TF32) launch_kernel<MODE, ELT_TF32>(a, b, p, grid, s);
  else if (elt == ELT_BF16) launch_kernel<MODE, ELT_BF16>(a, b, p, grid, s);
  else launch_kernel<MODE, ELT_F16>(a, b, p, grid, s);
}

void launch_split(int elt, const double *x, int64_t n, int64_t kpad, const double *pre,
                  const float *rs, const double *scale, void *bt, const int *skip,
                  cudaStream_t s) {
  const unsigned grid = (unsigned)ceil_div(kpad, 64);
  if (elt == ELT_TF32) split_kernel<ELT_TF32><<<grid, PT, 0, s>>>(x, n, kpad, pre, rs, scale, bt, skip);
  else if (elt == ELT_BF16) split_kernel<ELT_BF16><<<grid, PT, 0, s>>>(x, n, kpad, pre, rs, scale, bt, skip);
  else split_kernel<ELT_F16><<<grid, PT, 0, s>>>(x, n, kpad, pre, rs, scale, bt, skip);
  GRADA_LAUNCH_CHECK();
}

void launch_tc(const DevG &G, int mode, const double *in, double *out, void *scratch,
               int sm_count, cudaStream_t s, const GemvOpts &o, int *err) {
  const int elt = elt_of(G);
  const TcLayout L = tc_layout(G, mode, sm_count);
  uint8_t *sc = static_cast<uint8_t *>(scratch);
  void *bt = sc + L.off_bt;
  float *partial = reinterpret_cast<float *>(sc + L.off_partial);
  double *cm = reinterpret_cast<double *>(sc + L.off_colmax);
  double *scale = reinterpret_cast<double *>(sc + L.off_scale);
  // G^T Y: rows of Y carry the optional data weight and the 16-bit row scale
  const int64_t kin = (mode == MODE_GX) ? G.nm : G.nd;
  const double *pre = (mode == MODE_GTY) ? o.scale : nullptr;
  const float *rs_in = (mode == MODE_GTY) ? G.row_scale : nullptr;
  colmax_kernel<<<L.colmax_blocks, PT, 0, s>>>(in, kin, pre, rs_in, cm, o.skip);
  GRADA_LAUNCH_CHECK();
  colscale_kernel<<<1, 32, 0, s>>>(cm, L.colmax_blocks, scale, o.skip);
  GRADA_LAUNCH_CHECK();
  launch_split(elt, in, kin, L.kpad, pre, rs_in, scale, bt, o.skip, s);

  const int eb = elt_bytes(elt), ks = elt_ks(elt);
  CUtensorMap ma;
  if (mode == MODE_GX)
    ma = make_map(G.data, elt, (uint64_t)G.ld, (uint64_t)G.nm, (uint64_t)G.ld * eb,
                  (uint32_t)(SWB / eb), (uint32_t)ks);
  else
    ma = make_map(G.data, elt, (uint64_t)G.ld, (uint64_t)G.nm, (uint64_t)G.ld * eb, (uint32_t)ks,
                  (uint32_t)TC_M);
  const CUtensorMap mb = make_map(bt, elt, (uint64_t)L.k_len, (uint64_t)(2 * kBW),
                                  (uint64_t)L.kpad * eb, (uint32_t)ks, (uint32_t)(2 * kBW));
  TcParams p;
  p.m_rows = L.m_rows;
  p.n_mtiles = L.n_mtiles;
  p.n_splits = L.n_splits;
  p.kst_total = L.kst_total;
  p.kst_per_split = L.kst_per_split;
  p.m_pad = L.m_pad;
  p.partial = partial;
  p.err = err;
  p.skip = o.skip;
  const int units = L.n_mtiles * L.n_splits;
  const int grid = std::min(units, sm_count);
  if (mode == MODE_GX) dispatch<MODE_GX>(elt, ma, mb, p, grid, s);
  else dispatch<MODE_GTY>(elt, ma, mb, p, grid, s);

  const int64_t n_out = (mode == MODE_GX) ? G.nd : G.nm;
  const float *rs_out = (mode == MODE_GX) ? G.row_scale : nullptr;
  const double *post = (mode == MODE_GX) ? o.scale : nullptr;
  tc_finish_kernel<<<(unsigned)ceil_div(n_out * kBW, 256), 256, 0, s>>>(
      partial, L.n_splits, L.m_pad, n_out, scale, rs_out, post, out, o.skip);
  GRADA_LAUNCH_CHECK();
}

}  // namespace

bool tc_supported(const DevG &G) {
  return G.kind == GKind::FP32 || G.kind == GKind::BF16 || G.kind == GKind::FP16;
}

int64_t tc_scratch_bytes(const DevG &G, int sm_count) {
  const TcLayout a = tc_layout(G, MODE_GX, sm_count);
  const TcLayout b = tc_layout(G, MODE_GTY, sm_count);
  return std::max(a.total, b.total);
}

void launch_tc_G_mat_mul(const DevG &G, const double *X, double *Y, void *scratch, int sm_count,
                         cudaStream_t s, const GemvOpts &o, int *err) {
  launch_tc(G, MODE_GX, X, Y, scratch, sm_count, s, o, err);
}

void launch_tc_GT_mat_mul(const DevG &G, const double *Y, double *X, void *scratch, int sm_count,
                          cudaStream_t s, const GemvOpts &o, int *err) {
  launch_tc(G, MODE_GTY, Y, X, scratch, sm_count, s, o, err);
}

}  // namespace grada
