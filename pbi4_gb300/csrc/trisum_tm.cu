// trisum_tm.cu -- triangle sums on tcgen05 with the pair products in tensor memory.
//
// The "Last sum" loops of measure_bk / measure_bk_multipoles
// (bispectrumI4.f90:160-195, 476-513), S(l,j,i) = sum_x M_i M_j M_l (and the
// B2/B4 sums with the delta_2 / delta_4 maps of shell l), recast as a
// contraction over the grid points x:
//     C[p, q] = sum_x A[p, x] B[q, x],  A[p, x] = M_i(x) M_j(x) for the pair p = (i, j),
//                                       B[q, x] = map q (maps in set-major, shell-minor order).
// Only the (p, q) entries that are triangles are kept.
//
// Operand forms (FP32 accumulation in every form):
//   TF32 split: hi = v with the 13 low mantissa bits cleared (exact in TF32),
//     lo = v - hi; A_hi.B_hi + A_hi.B_lo + A_lo.B_hi with kind::tf32 (K = 8).
//     The FP32 exponent range needs no scaling; every product carries a
//     relative error below 2^-20.
//   FP16 split: every operand scaled by a power of two so |v| <= 2^14 (a
//     per-map bound from Parseval: |M| <= sqrt(nmodes * sum |H|^2)), hi =
//     fp16(v), lo = fp16(v - hi); the same three products with kind::f16 (K = 16).
//   BF16: one bf16 product, kind::f16 with bf16 operands (K = 16).
//
// Data path per chunk of 64 grid points (one CTA per (M tile of 128 pairs,
// N tile of 64 maps, K range)):
//   * the x pass of the map transform writes the maps as operand planes
//     [map][point] (FP16 hi / lo, BF16, or TF32 hi / lo) plus the set-0 maps in
//     FP32 (the pair factors), so the B tiles need no conversion here;
//   * a TMA warp loads each chunk's B tile(s) (64 maps x 64 points, 128-byte
//     swizzled: the K-major operand layout itself) and the FP32 set-0 maps of
//     the chunk into a ring of shared-memory stages;
//   * three producer warpgroups take the chunks in turn (thread = TMEM lane =
//     pair row): they form the 64 products of their pair, split them and store
//     them straight into a tensor-memory A stage with tcgen05.st (the A operand
//     never touches shared memory);
//   * an MMA warp issues the MMAs (A in TMEM, B from the stage) into one of
//     two TMEM accumulators, a fresh one per chunk, and commits them to a
//     per-chunk completion barrier that frees the A stage, the accumulator and
//     (with the producers' release) the shared-memory stage.  The tensor core
//     adds the products of one instruction to the accumulator with truncation,
//     so keeping each accumulation to one chunk keeps that error near 1e-6;
//   * two drain warpgroups (32 accumulator columns each) add each chunk's
//     accumulator into FP32 registers (round to nearest) and fold those into a
//     Kahan-compensated sum every 16 chunks (kept in the TMEM columns the
//     accumulators and A stages leave free), then write the final sums (FP64,
//     scaled back by the FP16 exponents) of the triangle slots.
// Every wait is bounded: a wait that runs out sets an abort flag that ends all
// roles, records the error for the host, and the CTA waits (bounded) for its
// own MMAs and copies in flight before it frees its tensor memory.
#include <cuda.h>  // CUtensorMap and its enums (the encoder is fetched through the runtime)
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <vector>

#include "bispec.cuh"
#include "tc_ptx.cuh"
#include "trisum_tm.cuh"

namespace pbi4g {

namespace {

using namespace tcx;

constexpr int kM = 128;          // pairs per unit (MMA M = TMEM lanes)
constexpr int kN = 64;           // maps per unit (MMA N)
constexpr int kKB = 32;          // FP32 values per 128-byte swizzle row (one K block)
constexpr int kBlocks = 2;       // K blocks per chunk
constexpr int kKC = kKB * kBlocks;  // grid points per chunk
constexpr int kMaxStages = 10;   // TMA staging slots (released by the producers and the MMAs)
constexpr int kGroups = 3;       // producer warpgroups, chunks assigned round robin (2: 8% slower at 256^3)
constexpr int kProdWarps = 4 * kGroups;
constexpr int kDrainWarps = 8;   // two warpgroups, 32 accumulator columns each
constexpr int kMmaWarp = kProdWarps + kDrainWarps;
constexpr int kMmaWarps = 2;     // MMA issuers, chunks alternating (a thread's MMAs of a chunk stay in order)
constexpr int kTmaWarp = kMmaWarp + kMmaWarps;
constexpr int kThreads = (kTmaWarp + 1) * 32;  // 736
#ifndef PBI4G_TM_FOLD
#define PBI4G_TM_FOLD 16
#endif
constexpr int kFold = PBI4G_TM_FOLD;  // chunks summed in registers before a Kahan fold
constexpr int kFoldGroup = 8;    // running sums a drain thread folds per batch of loads (one TMEM x8 load)
// TMEM accumulators (one chunk each) and the FP16 form's A stages (build-time tuning)
#ifndef PBI4G_TM_ACC
#define PBI4G_TM_ACC 2
#endif
#ifndef PBI4G_TM_F16_ASTAGES
#define PBI4G_TM_F16_ASTAGES 4
#endif
constexpr int kAcc = PBI4G_TM_ACC;
constexpr int kDone = 16;        // per-chunk MMA completion barriers (ring)
constexpr int kMaxAStages = 6;   // producer -> MMA barriers (one per A stage)
constexpr uint32_t kColAcc = 0;  // kAcc accumulators of kN columns, then the A stages
constexpr uint32_t kColA = kAcc * kN;
constexpr uint32_t kTmemCols = 512;
constexpr uint32_t kBTile = kN * 128;    // one B tile: 64 maps x 128 bytes
static_assert(kMaxStages <= kDone, "a stage's MMA barrier must not have cycled when the stage is reused");
constexpr uint32_t kTfMask = 0xFFFFE000u;

enum : int { kFormTF32 = 0, kFormF16 = 1, kFormBF16 = 2 };

template <int F> struct Form;
// TF32 split: A stage = 64 hi + 64 lo columns, 8 K-steps of 8, 3 products
template <> struct Form<kFormTF32> {
    static constexpr uint32_t kACols = 2 * kKC;
    static constexpr int kAStages = 2;
    static constexpr int kBTiles = 4;  // hi, hi, lo, lo: 32 FP32 points per 128-byte row
    static constexpr int kKStep = 8;
    static constexpr bool kSplit = true;
    static constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(kN >> 3) << 17) |
                                       ((uint32_t)(kM >> 4) << 24);
};
// FP16 split: A stage = 32 hi + 32 lo packed columns, 4 K-steps of 16, 3 products
template <> struct Form<kFormF16> {
    static constexpr uint32_t kACols = kKC;
    static constexpr int kAStages = PBI4G_TM_F16_ASTAGES;
    static constexpr int kBTiles = 2;  // hi, lo: 64 FP16 points per 128-byte row
    static constexpr int kKStep = 16;
    static constexpr bool kSplit = true;
    static constexpr uint32_t kIdesc = (1u << 4) | (0u << 7) | (0u << 10) | ((uint32_t)(kN >> 3) << 17) |
                                       ((uint32_t)(kM >> 4) << 24);
};
// BF16: A stage = 32 packed columns, 4 K-steps of 16, 1 product
template <> struct Form<kFormBF16> {
    static constexpr uint32_t kACols = kKC / 2;
    static constexpr int kAStages = 4;
    static constexpr int kBTiles = 1;
    static constexpr int kKStep = 16;
    static constexpr bool kSplit = false;
    static constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kN >> 3) << 17) |
                                       ((uint32_t)(kM >> 4) << 24);
};
// A waiter on an mbarrier names the phase by its parity, so each A stage and each
// accumulator must be consumed by one issuing thread, chunk after chunk: issuer w
// takes chunks w + k kMmaWarps, which use stage (and accumulator) i % count only if
// count is a multiple of kMmaWarps.  Otherwise an issuer two phases ahead of a stage
// would read a stale parity as complete.
static_assert(kAcc % kMmaWarps == 0, "accumulators per issuer");
// the producer -> MMA barriers (one per A stage) are an array of kMaxAStages
static_assert(Form<kFormTF32>::kAStages <= kMaxAStages && Form<kFormF16>::kAStages <= kMaxAStages &&
                  Form<kFormBF16>::kAStages <= kMaxAStages,
              "A stages beyond the barrier array");
static_assert(Form<kFormTF32>::kAStages % kMmaWarps == 0 && Form<kFormF16>::kAStages % kMmaWarps == 0 &&
                  Form<kFormBF16>::kAStages % kMmaWarps == 0,
              "A stages per issuer");
static_assert(kColA + Form<kFormTF32>::kAStages * Form<kFormTF32>::kACols <= kTmemCols, "TMEM budget");
static_assert(kColA + Form<kFormF16>::kAStages * Form<kFormF16>::kACols <= kTmemCols, "TMEM budget");

// D[tmem] (+)= A[tmem] . B[smem]^T
template <int F>
__device__ __forceinline__ void umma_ta(uint32_t d_tmem, uint32_t a_tmem, uint64_t b, uint32_t accum) {
    if constexpr (F == kFormTF32)
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "setp.ne.b32 p, %3, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %4, p;\n\t}" ::"r"(d_tmem),
            "r"(a_tmem), "l"(b), "r"(accum), "r"(Form<F>::kIdesc)
            : "memory");
    else
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "setp.ne.b32 p, %3, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %4, p;\n\t}" ::"r"(d_tmem),
            "r"(a_tmem), "l"(b), "r"(accum), "r"(Form<F>::kIdesc)
            : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *tm, int x, int y, int z, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(tm)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}

// Suspend-time hint of the main-loop waits (ns; 0: plain polling).
#ifndef PBI4G_TM_WAIT_HINT_NS
#define PBI4G_TM_WAIT_HINT_NS 0
#endif

// Bounded wait of the main loop that also gives up once another role has
// aborted: kWaitNs of device time (the abort flag and the timer read every 256
// polls).  The diagnostic instantiation (D) polls `limit` times without
// blocking instead, so that such waits run out on healthy work
// (pbi4g_plan_debug_wait_limit); everything else in the kernel is the same.
template <bool D>
__device__ __forceinline__ bool wait_or_abort(uint64_t *bar, uint32_t parity, volatile int *abort_flag,
                                              uint32_t limit) {
    if constexpr (D) {
        for (uint32_t i = 0; i < limit; i++)
            if (mbar_test_wait(bar, parity)) return true;
        return false;
    } else {
        if (mbar_try_wait(bar, parity)) return true;
        const uint32_t t0 = global_ns();
        for (uint32_t i = 1;; i++) {
            if (PBI4G_TM_WAIT_HINT_NS > 0 ? mbar_try_wait_sleep(bar, parity, PBI4G_TM_WAIT_HINT_NS)
                                          : mbar_try_wait(bar, parity))
                return true;
            if ((i & 255) == 0 && (*abort_flag || global_ns() - t0 > kWaitNs)) return false;
        }
    }
}

// The same, with one answer for the whole warp (the tcgen05 loads and stores
// that follow are warp-collective: every lane takes the same branch).
template <bool D>
__device__ __forceinline__ bool warp_wait(uint64_t *bar, uint32_t parity, volatile int *abort_flag, uint32_t limit) {
    return __all_sync(0xffffffffu, wait_or_abort<D>(bar, parity, abort_flag, limit));
}

// Barrier parity of the completion, for chunk i, of a barrier used every `every` chunks.
__device__ __forceinline__ uint32_t ph(int i, int every) { return (uint32_t)((i / every) & 1); }

// Slot and phase of a ring of `size` barriers, advanced by additions: the roles'
// loops run on a single thread or warp per chunk, where a division by the
// runtime stage count is a long dependent chain.
struct Ring {
    int idx, phase;
    __device__ __forceinline__ Ring(int start, int size) : idx(start % size), phase((start / size) & 1) {}
    __device__ __forceinline__ void step(int k, int size) {  // k <= size
        idx += k;
        if (idx >= size) {
            idx -= size;
            phase ^= 1;
        }
    }
};

// two products u0 v0, u1 v1 -> packed 16-bit hi, and for the FP16 split lo =
// u v - hi (the FMA keeps the product's own rounding error out of lo).  The
// packed FP32 pair instructions round each element as the scalar ones do; they
// made the triangle sums 5% faster at 256^3.
template <int F>
__device__ __forceinline__ void pack_prod2(float u0, float v0, float u1, float v1, uint32_t &hi, uint32_t &lo) {
    if constexpr (F == kFormF16) {
        // packed FP32 pairs: the same roundings as two scalar products and FMAs
        const float2 u = make_float2(u0, u1), v = make_float2(v0, v1);
        const __half2 h = __float22half2_rn(__fmul2_rn(u, v));
        const float2 back = __half22float2(h);
        const __half2 l = __float22half2_rn(__ffma2_rn(u, v, make_float2(-back.x, -back.y)));
        hi = *reinterpret_cast<const uint32_t *>(&h);
        lo = *reinterpret_cast<const uint32_t *>(&l);
    } else {
        const __nv_bfloat162 h = __float22bfloat162_rn(__fmul2_rn(make_float2(u0, u1), make_float2(v0, v1)));
        hi = *reinterpret_cast<const uint32_t *>(&h);
        lo = 0u;
    }
}

// The drain's Kahan sums live in the TMEM columns the accumulators and A stages
// leave free when there are 2 kN of them (every form with two accumulators),
// else in an L2-resident global scratch per CTA.  In TMEM the folds cost no L2
// round trips: with two accumulators the triangle sums at 256^3 took 1.00 ms
// against 1.08 ms for four accumulators and the sums in L2 (two A stages instead
// of four: 1.33 ms).
template <int F>
constexpr bool kahan_in_tmem() {
    return kColA + (uint32_t)Form<F>::kAStages * Form<F>::kACols + 2 * kN <= kTmemCols;
}

struct TmArgs {
    long long nchunks;     // points / kKC, rounded up
    int nunits, ksplit, nslots, nA, nstages, nmaps;
    uint32_t stage_bytes, ablock;
    float *kahan;          // [grid][2][kN][kM] running sums of each CTA (forms whose sums do not fit in TMEM)
    const int2 *units;     // (M tile, N tile) per unit
    const int2 *prow;      // [nunits][kM] staged rows (i, j) of each pair's factors, (-1, -1) for none
    const int *slots;      // [nunits][kM][kN] output slot or -1
    const int *mexp;       // FP16 form: per-map exponent e, map stored times 2^e (|M| 2^e <= 2^14)
    double *partial;       // [ksplit][nslots]
    int *err;              // set to 1 when a bounded wait gives up
    uint32_t wait_limit;   // polls of a main-loop wait (kWaitLimit unless a diagnostic limit is set)
};

template <int F, bool D>
__global__ void __launch_bounds__(kThreads, 1)
    trisum_tm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmBh,
                     const __grid_constant__ CUtensorMap tmBl, const TmArgs a) {
    using FM = Form<F>;
    constexpr int AST = FM::kAStages;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char *base =
        reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    const int nst = a.nstages;
    // barriers: full per stage (TMA -> producers, MMA), sfree per stage (producers -> TMA),
    // prod per A stage (producers -> MMA), done per chunk ring (MMA completion -> TMA,
    // producers, drain), accfree per accumulator (drain -> MMA)
    // smem: nst stages | barriers and tables
    uint64_t *bars = reinterpret_cast<uint64_t *>(base + (size_t)nst * a.stage_bytes);
    uint64_t *full = bars, *sfree = full + kMaxStages, *prod = sfree + kMaxStages, *done = prod + kMaxAStages;
    uint64_t *accfree = done + kDone;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(accfree + kAcc);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);
    int2 *prow_s = reinterpret_cast<int2 *>(tmem_slot + 4);
    int *qexp_s = reinterpret_cast<int *>(prow_s + kM);  // [kN] FP16 exponent of each B row
    // running sums of the drain, then the compensation: TMEM columns kColK .. kColK + 2 kN
    // of the thread's lane, or [kN][kM] floats each in a global scratch per CTA (each
    // thread reads back only what it wrote)
    constexpr bool KT = kahan_in_tmem<F>();
    constexpr uint32_t kColK = kColA + (uint32_t)AST * FM::kACols;
    float *run_g = KT ? nullptr : a.kahan + (size_t)blockIdx.x * 2 * kN * kM;
    float *comp_g = KT ? nullptr : run_g + kN * kM;

    const int unit = blockIdx.x % a.nunits, split = blockIdx.x / a.nunits;
    const int2 U = a.units[unit];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const long long cb = a.nchunks * split / a.ksplit, ce = a.nchunks * (split + 1) / a.ksplit;
    const int n = (int)(ce - cb);

    for (int r = tid; r < kM; r += kThreads) prow_s[r] = a.prow[(size_t)unit * kM + r];
    for (int r = tid; r < kN; r += kThreads) {
        const int q = U.y * kN + r;
        qexp_s[r] = (F == kFormF16 && q < a.nmaps) ? a.mexp[q] : 0;
    }
    if (tid == 0) {
        for (int s = 0; s < kMaxStages; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&sfree[s], 128);  // the warpgroup that consumed the stage's pair factors
        }
        for (int s = 0; s < kMaxAStages; s++) mbar_init(&prod[s], 128);  // one warpgroup per chunk
        for (int s = 0; s < kDone; s++) mbar_init(&done[s], 1);
        for (int s = 0; s < kAcc; s++) mbar_init(&accfree[s], kDrainWarps * 32);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        tmem_alloc(tmem_slot, kTmemCols);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    // stage: pair-factor blocks [kBlocks][ablock] (FP32, 32 points a row) | B tiles [kBTiles][kBTile]
    auto stage_ptr = [&](int s) { return base + (size_t)s * a.stage_bytes; };
    auto fail = [&]() {
        *abort_flag = 1;
        atomicExch(a.err, 1);
    };

    if (warp < kProdWarps) {
        // ------------------------------------------------------------ producers
        const int quad = warp & 3, grp = warp >> 2;
        const int row = quad * 32 + lane;
        const int2 pr = prow_s[row];
        const uint32_t lane_addr = tmem + ((uint32_t)(quad * 32) << 16);
        Ring rs(grp, nst);  // stage and full-barrier phase of chunk i
        for (int i = grp; i < n; i += kGroups, rs.step(kGroups, nst)) {
            const int s = rs.idx, as = i % AST;
            if (!warp_wait<D>(&full[s], (uint32_t)rs.phase, abort_flag, a.wait_limit)) { fail(); break; }
            // the A stage is free once the MMAs of chunk i - AST completed (MMAs complete in order)
            if (i >= AST && !warp_wait<D>(&done[(i - AST) % kDone], ph(i - AST, kDone), abort_flag, a.wait_limit)) {
                fail();
                break;
            }
            const unsigned char *stg = stage_ptr(s);
            const uint32_t acol = kColA + (uint32_t)as * FM::kACols;
#pragma unroll
            for (int kb = 0; kb < kBlocks; kb++) {
                const unsigned char *blk = stg + kb * a.ablock;
                if constexpr (F == kFormTF32) {
#pragma unroll
                    for (int q16 = 0; q16 < 2; q16++) {
                        uint32_t hi[16], lo[16];
                        if (pr.x >= 0) {
#pragma unroll
                            for (int c4 = 0; c4 < 4; c4++) {
                                const int c = 4 * q16 + c4;
                                const float4 u =
                                    *reinterpret_cast<const float4 *>(blk + pr.x * 128 + ((c ^ (pr.x & 7)) << 4));
                                const float4 v =
                                    *reinterpret_cast<const float4 *>(blk + pr.y * 128 + ((c ^ (pr.y & 7)) << 4));
                                const float2 p01 = __fmul2_rn(make_float2(u.x, u.y), make_float2(v.x, v.y));
                                const float2 p23 = __fmul2_rn(make_float2(u.z, u.w), make_float2(v.z, v.w));
                                const float2 h01 = make_float2(__uint_as_float(__float_as_uint(p01.x) & kTfMask),
                                                               __uint_as_float(__float_as_uint(p01.y) & kTfMask));
                                const float2 h23 = make_float2(__uint_as_float(__float_as_uint(p23.x) & kTfMask),
                                                               __uint_as_float(__float_as_uint(p23.y) & kTfMask));
                                const float2 l01 = __fadd2_rn(p01, make_float2(-h01.x, -h01.y));
                                const float2 l23 = __fadd2_rn(p23, make_float2(-h23.x, -h23.y));
                                hi[4 * c4 + 0] = __float_as_uint(h01.x);
                                hi[4 * c4 + 1] = __float_as_uint(h01.y);
                                hi[4 * c4 + 2] = __float_as_uint(h23.x);
                                hi[4 * c4 + 3] = __float_as_uint(h23.y);
                                lo[4 * c4 + 0] = __float_as_uint(l01.x);
                                lo[4 * c4 + 1] = __float_as_uint(l01.y);
                                lo[4 * c4 + 2] = __float_as_uint(l23.x);
                                lo[4 * c4 + 3] = __float_as_uint(l23.y);
                            }
                        } else {
#pragma unroll
                            for (int e = 0; e < 16; e++) hi[e] = lo[e] = 0u;
                        }
                        const uint32_t col = acol + (uint32_t)(kb * kKB + 16 * q16);
                        tmem_st16(lane_addr + col, hi);
                        tmem_st16(lane_addr + col + kKC, lo);
                    }
                } else {
                    // 32 points -> 16 packed columns (point 2c in the low half of column c), in
                    // two halves of 16 points (fewer live registers: 23 warps fit in 80 each)
#pragma unroll
                    for (int q8 = 0; q8 < 2; q8++) {
                        uint32_t hi[8], lo[8];
                        if (pr.x >= 0) {
#pragma unroll
                            for (int c4 = 0; c4 < 4; c4++) {
                                const int c = 4 * q8 + c4;
                                const float4 u =
                                    *reinterpret_cast<const float4 *>(blk + pr.x * 128 + ((c ^ (pr.x & 7)) << 4));
                                const float4 v =
                                    *reinterpret_cast<const float4 *>(blk + pr.y * 128 + ((c ^ (pr.y & 7)) << 4));
                                pack_prod2<F>(u.x, v.x, u.y, v.y, hi[2 * c4], lo[2 * c4]);
                                pack_prod2<F>(u.z, v.z, u.w, v.w, hi[2 * c4 + 1], lo[2 * c4 + 1]);
                            }
                        } else {
#pragma unroll
                            for (int e = 0; e < 8; e++) hi[e] = lo[e] = 0u;
                        }
                        const uint32_t col = acol + (uint32_t)(kb * (kKB / 2) + 8 * q8);
                        tmem_st8(lane_addr + col, hi);
                        if (FM::kSplit) tmem_st8(lane_addr + col + kKC / 2, lo);
                    }
                }
            }
            mbar_arrive(&sfree[s]);  // the stage's pair factors are consumed
            tmem_wait_st();
            tc_fence_before();
            mbar_arrive(&prod[as]);
        }
    } else if (warp < kMmaWarp) {
        // ---------------------------------------------------------------- drain
        // each chunk's accumulator is added into FP32 registers (round to nearest);
        // every kFold chunks those are folded into a Kahan-compensated sum (in TMEM, or
        // an L2-resident scratch), written out at the end
        const int quad = warp & 3, cgrp = (warp - kProdWarps) >> 2;
        const int row = quad * 32 + lane, c0 = 32 * cgrp;
        const uint32_t lane_addr = tmem + ((uint32_t)(quad * 32) << 16);
        const uint32_t krun = lane_addr + kColK + (uint32_t)c0, kcomp = krun + kN;
        float mid[32];
#pragma unroll
        for (int e = 0; e < 32; e++) mid[e] = 0.f;
        if constexpr (KT) {
            const uint32_t z[8] = {0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u};
#pragma unroll
            for (int h = 0; h < 32; h += 8) {
                tmem_st8(krun + h, z);
                tmem_st8(kcomp + h, z);
            }
            tmem_wait_st();
        } else {
#pragma unroll
            for (int e = 0; e < 32; e++) {
                run_g[(c0 + e) * kM + row] = 0.f;
                comp_g[(c0 + e) * kM + row] = 0.f;
            }
        }
        bool ok = true;
#pragma unroll 1
        for (int i = 0; i < n; i++) {
            const int b = i % kAcc;
            if (!warp_wait<D>(&done[i % kDone], ph(i, kDone), abort_flag, a.wait_limit)) { fail(); ok = false; break; }
            tc_fence_after();
#pragma unroll
            for (int h = 0; h < 2; h++) {
                uint32_t ac[16];
                tmem_ld16(lane_addr + kColAcc + (uint32_t)b * kN + c0 + 16 * h, ac);
                tmem_wait_ld();
#pragma unroll
                for (int e = 0; e < 16; e++) mid[16 * h + e] += __uint_as_float(ac[e]);
            }
            tc_fence_before();
            mbar_arrive(&accfree[b]);
            if ((i + 1) % kFold == 0 || i == n - 1) {
                // each group's loads are issued before its first store, so the fold
                // costs a few TMEM (or L2) round trips
#pragma unroll
                for (int h = 0; h < 32; h += kFoldGroup) {
                    if constexpr (KT) {
                        uint32_t rr[kFoldGroup], cc[kFoldGroup];
                        tmem_ld8(krun + h, rr);
                        tmem_ld8(kcomp + h, cc);
                        tmem_wait_ld();
#pragma unroll
                        for (int e = 0; e < kFoldGroup; e++) {
                            const float rv = __uint_as_float(rr[e]), y = mid[h + e] - __uint_as_float(cc[e]);
                            const float t2 = rv + y;
                            cc[e] = __float_as_uint((t2 - rv) - y);
                            rr[e] = __float_as_uint(t2);
                            mid[h + e] = 0.f;
                        }
                        tmem_st8(krun + h, rr);
                        tmem_st8(kcomp + h, cc);
                    } else {
                        float rv[kFoldGroup], cv[kFoldGroup];
#pragma unroll
                        for (int e = 0; e < kFoldGroup; e++) {
                            rv[e] = __ldcg(run_g + (c0 + h + e) * kM + row);
                            cv[e] = __ldcg(comp_g + (c0 + h + e) * kM + row);
                        }
#pragma unroll
                        for (int e = 0; e < kFoldGroup; e++) {
                            const float y = mid[h + e] - cv[e];
                            const float t2 = rv[e] + y;
                            cv[e] = (t2 - rv[e]) - y;
                            rv[e] = t2;
                            mid[h + e] = 0.f;
                        }
#pragma unroll
                        for (int e = 0; e < kFoldGroup; e++) {
                            __stcg(run_g + (c0 + h + e) * kM + row, rv[e]);
                            __stcg(comp_g + (c0 + h + e) * kM + row, cv[e]);
                        }
                    }
                }
                if constexpr (KT) tmem_wait_st();  // the next fold reads these columns back
            }
        }
        if (__all_sync(0xffffffffu, ok && !*abort_flag)) {
            const int *sl = a.slots + ((size_t)unit * kM + row) * kN;
            const int2 pr = prow_s[row];
            const int pe = (F == kFormF16 && pr.x >= 0) ? a.mexp[pr.x] + a.mexp[pr.y] - 14 : 0;
            if constexpr (KT) {
#pragma unroll 1
                for (int h = 0; h < 32; h += 8) {
                    uint32_t rr[8], cc[8];
                    tmem_ld8(krun + h, rr);
                    tmem_ld8(kcomp + h, cc);
                    tmem_wait_ld();
#pragma unroll
                    for (int e = 0; e < 8; e++) {
                        const int slot = sl[c0 + h + e];
                        if (slot < 0) continue;
                        const double v = (double)__uint_as_float(rr[e]) - (double)__uint_as_float(cc[e]);
                        a.partial[(size_t)split * a.nslots + slot] =
                            F == kFormF16 ? ldexp(v, -(pe + qexp_s[c0 + h + e])) : v;
                    }
                }
            } else {
#pragma unroll 4
                for (int e = 0; e < 32; e++) {
                    const int slot = sl[c0 + e];
                    if (slot < 0) continue;
                    const double v = (double)run_g[(c0 + e) * kM + row] - (double)comp_g[(c0 + e) * kM + row];
                    a.partial[(size_t)split * a.nslots + slot] = F == kFormF16 ? ldexp(v, -(pe + qexp_s[c0 + e])) : v;
                }
            }
        }
    } else if (warp < kTmaWarp) {
        // ------------------------------------------ MMA issue (one thread per MMA warp)
        // issuer w takes chunks w, w + kMmaWarps, ...: each chunk has its own
        // accumulator, A stage and completion barrier, and tcgen05.commit tracks the
        // issuing thread's own MMAs, so the two streams need no ordering between them
        if (lane == 0) {
            const int mw = warp - kMmaWarp;
            int last_commit = -1;
            bool ok = true;
            Ring rs(mw, nst);
            for (int i = mw; i < n; i += kMmaWarps, rs.step(kMmaWarps, nst)) {
                const int b = i % kAcc, as = i % AST, s = rs.idx;
                if (i >= kAcc && !wait_or_abort<D>(&accfree[b], ph(i - kAcc, kAcc), abort_flag, a.wait_limit)) { ok = false; break; }
                if (!wait_or_abort<D>(&full[s], (uint32_t)rs.phase, abort_flag, a.wait_limit)) { ok = false; break; }  // B tiles
                if (!wait_or_abort<D>(&prod[as], ph(i, AST), abort_flag, a.wait_limit)) { ok = false; break; }  // A stage
                tc_fence_after();
                // descriptors advance by 16-byte units within the stage (no carry out of the address field)
                const uint64_t db = sw128_desc(smem_u32(stage_ptr(s)) + kBlocks * a.ablock);
                const uint32_t ahi = tmem + kColA + (uint32_t)as * FM::kACols;
                const uint32_t d = tmem + kColAcc + (uint32_t)b * kN;
#pragma unroll
                for (int kk = 0; kk < kKC / FM::kKStep; kk++) {
                    uint64_t dh, dl;
                    uint32_t a_hi, a_lo;
                    if constexpr (F == kFormTF32) {
                        // FP32 rows: K-step of 8 = 32 bytes; tiles hi0, hi1, lo0, lo1
                        dh = db + (((uint32_t)(kk / 4) * kBTile + (uint32_t)(kk % 4) * 32) >> 4);
                        dl = dh + ((2 * kBTile) >> 4);
                        a_hi = ahi + 8 * kk;
                        a_lo = a_hi + kKC;
                    } else {
                        // 16-bit rows: K-step of 16 = 32 bytes; tiles hi, lo
                        dh = db + (uint32_t)kk * 2;
                        dl = dh + (kBTile >> 4);
                        a_hi = ahi + 8 * kk;
                        a_lo = a_hi + kKC / 2;
                    }
                    umma_ta<F>(d, a_hi, dh, kk == 0 ? 0u : 1u);
                    if (FM::kSplit) {
                        umma_ta<F>(d, a_hi, dl, 1u);
                        umma_ta<F>(d, a_lo, dh, 1u);
                    }
                }
                umma_commit(&done[i % kDone]);
                last_commit = i;
            }
            if (!ok) fail();
            // this thread's MMAs still in flight (and their barrier arrival) land before TMEM goes away
            if (last_commit >= 0) mbar_wait(&done[last_commit % kDone], ph(last_commit, kDone));
        }
    } else if (lane == 0) {
        // --------------------------------------------------------- TMA issue (one thread)
        const uint32_t tx = kBlocks * (uint32_t)a.nA * 128 + FM::kBTiles * kBTile;
        const int q0 = U.y * kN;
        int issued = 0;
        bool ok = true;
        Ring rs(0, nst);
        for (int j = 0; j < n; j++, rs.step(1, nst)) {
            const int s = rs.idx;
            // stage s is free once the producers took the pair factors of chunk j - nst
            // (the ring's previous phase) and the MMAs of that chunk (which read its B
            // tiles) completed
            if (j >= nst && (!wait_or_abort<D>(&sfree[s], (uint32_t)(rs.phase ^ 1), abort_flag, a.wait_limit) ||
                             !wait_or_abort<D>(&done[(j - nst) % kDone], ph(j - nst, kDone), abort_flag, a.wait_limit))) {
                ok = false;
                break;
            }
            unsigned char *stg = stage_ptr(s);
            unsigned char *bt = stg + kBlocks * a.ablock;
            mbar_expect_tx(&full[s], tx);
            const int c = (int)(cb + j);  // chunk: 64 consecutive points, one block of every plane
#pragma unroll
            for (int kb = 0; kb < kBlocks; kb++) tma_load_3d(stg + kb * a.ablock, &tmA, kb * kKB, 0, c, &full[s]);
            if constexpr (F == kFormTF32) {
#pragma unroll
                for (int kb = 0; kb < kBlocks; kb++) {
                    tma_load_3d(bt + kb * kBTile, &tmBh, kb * kKB, q0, c, &full[s]);
                    tma_load_3d(bt + (2 + kb) * kBTile, &tmBl, kb * kKB, q0, c, &full[s]);
                }
            } else {
                tma_load_3d(bt, &tmBh, 0, q0, c, &full[s]);
                if (FM::kSplit) tma_load_3d(bt + kBTile, &tmBl, 0, q0, c, &full[s]);
            }
            issued = j + 1;
        }
        if (!ok) fail();
        // copies in flight land (bounded) before the shared memory goes away: after an
        // abort of any role, and (already complete, so at once) at a normal end
        for (int j = std::max(0, issued - nst); j < issued; j++) mbar_wait(&full[j % nst], ph(j, nst));
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, kTmemCols);
    }
}

// Per-map power-of-two scale of the FP16 form: |M(x)| <= sum_k |H(k)| <=
// sqrt(nmodes * sum_k |H(k)|^2) (triangle and Cauchy-Schwarz inequalities over
// the shell's modes).  Sets without their own power use the delta set's times
// max |L_l(mu)| (lfac).
__global__ void map_exponents_kernel(int nmaps, int nb, const double *__restrict__ powsum, int pow_mask,
                                     double lf1, double lf2, const double *__restrict__ nmodes, int *__restrict__ e) {
    for (int m = threadIdx.x; m < nmaps; m += blockDim.x) {
        const int s = m / nb, b = m % nb;
        const double p = (pow_mask >> s & 1) ? powsum[s * nb + b] : powsum[b];
        const double lf = s == 0 ? 1.0 : (s == 1 ? lf1 : lf2);
        const double v = sqrt(nmodes[b] * p) * ((pow_mask >> s & 1) ? 1.0 : lf);
        // scale so that |M| 2^e <= 2^14, clamped to the float exponent range
        int x = v > 0 ? 14 - (int)ceil(log2(v)) : 0;
        e[m] = x < -60 ? -60 : (x > 60 ? 60 : x);
    }
}

// ------------------------------------------------------------- tensor maps ---
using EncodeTiledFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                   const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
    static std::once_flag once;
    static EncodeTiledFn fn = nullptr;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    });
    return fn;
}

// 3D view of a chunk-major operand array [nchunks][rows][64 points] (element
// size esize): box box_pts x box_rows x 1 at (point within the chunk, first
// row, chunk), 128-byte swizzle (box_pts esize = 128 bytes: the K-major operand
// layout), zero fill past the last row.
int make_chunk_view(CUtensorMap *tm, const void *base, CUtensorMapDataType dt, int esize, long long nchunks,
                    int rows, int box_pts, int box_rows) {
    EncodeTiledFn enc = encode_fn();
    if (!enc) return set_error(PBI4G_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
    if (box_pts * esize != 128 || reinterpret_cast<uintptr_t>(base) % 16)
        return set_error(PBI4G_ERR_INVALID, "operand chunk view: alignment");
    const cuuint64_t gdim[3] = {(cuuint64_t)MapPlanes::kChunk, (cuuint64_t)rows, (cuuint64_t)nchunks};
    const cuuint64_t gstride[2] = {(cuuint64_t)MapPlanes::kChunk * esize, (cuuint64_t)rows * MapPlanes::kChunk * esize};
    const cuuint32_t box[3] = {(cuuint32_t)box_pts, (cuuint32_t)box_rows, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    const CUresult r = enc(tm, dt, 3, const_cast<void *>(base), gdim, gstride, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(PBI4G_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return PBI4G_OK;
}

}  // namespace

// ------------------------------------------------------------- host plan ---
int TmPlan::build(const Shells &sh, int nsets_) {
    nsets = nsets_;
    const int nb = sh.nb;
    nA = nb;
    // pairs (i, j) of set-0 shells, sorted by (j, i): consecutive TMEM lanes share j
    std::map<std::pair<int, int>, int> pidx;
    for (int64_t m = 0; m < sh.itot; m++) {
        const int j = sh.tri[3 * m + 1], i = sh.tri[3 * m + 2];
        pidx.emplace(std::make_pair(j - 1, i - 1), 0);
    }
    std::vector<int2> plist;
    for (auto &kv : pidx) {
        kv.second = (int)plist.size();
        plist.push_back(make_int2(kv.first.second, kv.first.first));  // (i, j)
    }
    npairs = (int)plist.size();
    nslots = (int)(sh.itot * nsets);
    const int nq = nsets * nb;  // q = map index s * nb + l - 1
    const int nmt = (npairs + kM - 1) / kM, nnt = (nq + kN - 1) / kN;
    struct E { int p, q, slot; };
    std::vector<E> ents;
    ents.reserve((size_t)sh.itot * nsets);
    std::vector<char> need((size_t)nmt * nnt, 0);
    for (int64_t m = 0; m < sh.itot; m++) {
        const int l = sh.tri[3 * m], j = sh.tri[3 * m + 1], i = sh.tri[3 * m + 2];
        const int p = pidx.at(std::make_pair(j - 1, i - 1));
        for (int s = 0; s < nsets; s++) {
            const int q = s * nb + l - 1;
            ents.push_back({p, q, (int)(m * nsets + s)});
            need[(size_t)(p / kM) * nnt + q / kN] = 1;
        }
    }
    std::vector<int2> h_units;
    std::map<std::pair<int, int>, int> uidx;
    // units ordered N tile outer, M tile inner: CTAs of one K range are adjacent in the grid
    for (int nt = 0; nt < nnt; nt++)
        for (int mt = 0; mt < nmt; mt++)
            if (need[(size_t)mt * nnt + nt]) {
                uidx[std::make_pair(mt, nt)] = (int)h_units.size();
                h_units.push_back(make_int2(mt, nt));
            }
    nunits = (int)h_units.size();
    std::vector<int2> h_prow((size_t)nunits * kM, make_int2(-1, -1));
    std::vector<int> h_slots((size_t)nunits * kM * kN, -1);
    for (int u = 0; u < nunits; u++)
        for (int r = 0; r < kM; r++) {
            const int p = h_units[u].x * kM + r;
            if (p < npairs) h_prow[(size_t)u * kM + r] = plist[p];
        }
    for (auto &e : ents) {
        const int u = uidx.at(std::make_pair(e.p / kM, e.q / kN));
        h_slots[((size_t)u * kM + e.p % kM) * kN + e.q % kN] = e.slot;
    }
    PBI4G_CHECK(units.ensure(sizeof(int2) * std::max(1, nunits)));
    PBI4G_CHECK(prow.ensure(sizeof(int2) * std::max<size_t>(1, h_prow.size())));
    PBI4G_CHECK(slots.ensure(sizeof(int) * std::max<size_t>(1, h_slots.size())));
    PBI4G_CHECK(err.ensure(sizeof(int)));
    if (nunits) {
        PBI4G_CUDA(cudaMemcpy(units.p, h_units.data(), sizeof(int2) * h_units.size(), cudaMemcpyHostToDevice));
        PBI4G_CUDA(cudaMemcpy(prow.p, h_prow.data(), sizeof(int2) * h_prow.size(), cudaMemcpyHostToDevice));
        PBI4G_CUDA(cudaMemcpy(slots.p, h_slots.data(), sizeof(int) * h_slots.size(), cudaMemcpyHostToDevice));
    }
    return PBI4G_OK;
}

bool tm_supported(const Shells &sh) {
    const long long npts = (long long)sh.Nm * sh.Nm * sh.Nm;
    return sh.nb <= 256 && sh.Nm % 4 == 0 && npts + kKC < (1LL << 31);
}

template <int F>
static int launch_tm(const CUtensorMap &tmA, const CUtensorMap &tmBh, const CUtensorMap &tmBl, const TmArgs &a,
                     size_t smem, int grid, cudaStream_t st) {
    auto kern = a.wait_limit < kWaitLimit ? trisum_tm_kernel<F, true> : trisum_tm_kernel<F, false>;
    PBI4G_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kern<<<grid, kThreads, smem, st>>>(tmA, tmBh, tmBl, a);
    PBI4G_LAUNCH_CHECK();
    return PBI4G_OK;
}

int tm_map_exponents(const Shells &sh, TmPlan &tp, int nmaps, const double *powsum, int pow_mask,
                     const double lfac[3], cudaStream_t st, int64_t *launches) {
    PBI4G_CHECK(tp.mexp.ensure(sizeof(int) * std::max(1, nmaps)));
    map_exponents_kernel<<<1, 256, 0, st>>>(nmaps, sh.nb, powsum, pow_mask, lfac[1], lfac[2],
                                            sh.nmodes_d.as<double>(), tp.mexp.as<int>());
    PBI4G_LAUNCH_CHECK();
    *launches += 1;
    return PBI4G_OK;
}

int triangle_sums_tm(const Shells &sh, TmPlan &tp, const MapPlanes &pl, DevBuf &partial, double *S,
                     bool accumulate, cudaStream_t st, int64_t *launches) {
    const int form = pl.form;
    if (!tm_supported(sh))
        return set_error(PBI4G_ERR_UNSUPPORTED, "tensor-core triangle sums: map grid %d, %d shells", sh.Nm, sh.nb);
    if (form < 0 || form > 2) return set_error(PBI4G_ERR_INVALID, "tensor-core form %d", form);
    if (tp.nunits == 0) return PBI4G_OK;
    if (form == 1 && (!pl.mexp || pl.mexp != tp.mexp.as<int>()))
        return set_error(PBI4G_ERR_INVALID, "tensor-core triangle sums: FP16 planes without the plan's exponents");
    if (pl.nb != sh.nb || pl.npts < kKC || pl.npts > (long long)sh.Nm * sh.Nm * sh.Nm || pl.nchunks * kKC != pl.npts)
        return set_error(PBI4G_ERR_INVALID, "tensor-core triangle sums: operand planes do not match the shells");
    static_assert(MapPlanes::kChunk == kKC, "a planes chunk is a contraction chunk");
    CUtensorMap tmA, tmBh, tmBl;
    const long long nc = pl.nchunks;
    PBI4G_CHECK(make_chunk_view(&tmA, pl.a32, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, nc, sh.nb, kKB, tp.nA));
    if (form == 0) {
        PBI4G_CHECK(make_chunk_view(&tmBh, pl.bhi, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, nc, pl.nmaps, kKB, kN));
        PBI4G_CHECK(make_chunk_view(&tmBl, pl.blo, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, nc, pl.nmaps, kKB, kN));
    } else if (form == 1) {
        PBI4G_CHECK(make_chunk_view(&tmBh, pl.bhi, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, nc, pl.nmaps, kKC, kN));
        PBI4G_CHECK(make_chunk_view(&tmBl, pl.blo, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, nc, pl.nmaps, kKC, kN));
    } else {
        PBI4G_CHECK(make_chunk_view(&tmBh, pl.bhi, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, nc, pl.nmaps, kKC, kN));
        tmBl = tmBh;  // unused: one product
    }
    TmArgs a;
    a.nchunks = nc;
    a.nunits = tp.nunits;
    // K split: one CTA per SM (152 SMs) in waves; the split minimising waves x
    // (chunks a CTA + a CTA's fixed cost of about 64 chunks), at least 128 chunks a CTA
    {
        long long best_cost = -1;
        a.ksplit = 1;
        for (int k = 1; k <= 152; k++) {
            if (k > 1 && a.nchunks / k < 128) break;
            const long long waves = ((long long)tp.nunits * k + 151) / 152;
            const long long cost = waves * ((a.nchunks + k - 1) / k + 64);
            if (best_cost < 0 || cost < best_cost) {
                best_cost = cost;
                a.ksplit = k;
            }
        }
    }
    a.nslots = tp.nslots;
    a.nA = tp.nA;
    a.nmaps = pl.nmaps;
    a.ablock = (uint32_t)(((tp.nA + 7) / 8) * 8 * 128);
    const int btiles = form == 0 ? Form<kFormTF32>::kBTiles : (form == 1 ? Form<kFormF16>::kBTiles : 1);
    a.stage_bytes = kBlocks * a.ablock + (uint32_t)btiles * kBTile;
    // barriers, TMEM address, abort flag, pair table, B-row exponents
    const size_t fixed =
        1024 + 8 * (2 * kMaxStages + kMaxAStages + kDone + kAcc) + 16 + sizeof(int2) * kM + sizeof(int) * kN;
    a.nstages = kMaxStages;
    while (a.nstages > 3 && fixed + (size_t)a.nstages * a.stage_bytes > 227 * 1024) a.nstages--;
    const size_t smem = fixed + (size_t)a.nstages * a.stage_bytes;
    if (smem > 227 * 1024) return set_error(PBI4G_ERR_UNSUPPORTED, "tensor-core triangle sums: %zu B smem", smem);
    a.units = tp.units.as<int2>();
    a.prow = tp.prow.as<int2>();
    a.slots = tp.slots.as<int>();
    PBI4G_CHECK(tp.mexp.ensure(sizeof(int) * std::max(1, pl.nmaps)));
    a.mexp = tp.mexp.as<int>();
    PBI4G_CHECK(partial.ensure(sizeof(double) * (size_t)a.ksplit * tp.nslots));
    a.partial = partial.as<double>();
    a.err = tp.err.as<int>();
    a.wait_limit = tp.wait_limit > 0 && tp.wait_limit < kWaitLimit ? tp.wait_limit : kWaitLimit;
    PBI4G_CUDA(cudaMemsetAsync(tp.err.p, 0, sizeof(int), st));
    const int grid = tp.nunits * a.ksplit;
    a.kahan = nullptr;
    const bool kt = form == 0 ? kahan_in_tmem<kFormTF32>()
                              : (form == 1 ? kahan_in_tmem<kFormF16>() : kahan_in_tmem<kFormBF16>());
    if (!kt) {  // the running sums do not fit beside the accumulators and A stages in TMEM
        PBI4G_CHECK(tp.kahan.ensure(sizeof(float) * 2 * kN * kM * (size_t)grid));
        a.kahan = tp.kahan.as<float>();
    }
    if (form == 0) PBI4G_CHECK(launch_tm<kFormTF32>(tmA, tmBh, tmBl, a, smem, grid, st));
    else if (form == 1) PBI4G_CHECK(launch_tm<kFormF16>(tmA, tmBh, tmBl, a, smem, grid, st));
    else PBI4G_CHECK(launch_tm<kFormBF16>(tmA, tmBh, tmBl, a, smem, grid, st));
    PBI4G_CHECK(reduce_partials(tp.nslots, a.ksplit, partial.as<double>(), S, accumulate, st));
    *launches += 2;
    return PBI4G_OK;
}

int tm_check_error(TmPlan &tp, cudaStream_t st) {
    int h = 0;
    PBI4G_CUDA(cudaMemcpyAsync(&h, tp.err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    PBI4G_CUDA(cudaStreamSynchronize(st));
    if (h) return set_error(PBI4G_ERR_TIMEOUT, "tensor-core triangle sums: a bounded wait gave up");
    return PBI4G_OK;
}

}  // namespace pbi4g
