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
//   * the C2R writes the maps row-interleaved (the x rows of all maps for one
//     (y, z) side by side), so one chunk of all maps is one contiguous read;
//     chunks are pairs of (row, 32-point x block), the last block of a row
//     zero-filled past x = Nm by the TMA bounds;
//   * a TMA warp loads the chunk's set-0 maps (the pair factors) and the 64
//     maps of the N tile, FP32, 128-byte swizzled, into a ring of shared-memory
//     stages;
//   * three producer warpgroups take the chunks in turn (thread = TMEM lane =
//     pair row): they form the 64 products of their pair, split them and store
//     them straight into a tensor-memory A stage with tcgen05.st (the A operand
//     never touches shared memory), and turn the FP32 B tile into the MMA
//     operand(s): in place for TF32 (hi) plus a lo copy; 16-bit hi / lo tiles
//     in the 128-byte swizzled K-major layout for FP16 / BF16;
//   * an MMA warp issues the MMAs (A in TMEM, B in shared memory) into one of
//     four TMEM accumulators, a fresh one per chunk, and commits them to a
//     per-chunk completion barrier that frees the shared-memory stage, the A
//     stage and the accumulator.  The tensor core adds the products of one
//     instruction to the accumulator with truncation, so keeping each
//     accumulation to one chunk keeps that error near 1e-6;
//   * two drain warpgroups (32 accumulator columns each) add each chunk's
//     accumulator into FP32 registers (round to nearest) and fold those into a
//     Kahan-compensated sum in shared memory every 16 chunks, then write the
//     final sums (FP64, scaled back by the FP16 exponents) of the triangle slots.
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
constexpr int kMaxStages = 8;    // TMA staging slots (released by the producers)
constexpr int kGroups = 3;       // producer warpgroups, chunks assigned round robin
constexpr int kProdWarps = 4 * kGroups;
constexpr int kDrainWarps = 8;   // two warpgroups, 32 accumulator columns each
constexpr int kMmaWarp = kProdWarps + kDrainWarps;
constexpr int kTmaWarp = kMmaWarp + 1;
constexpr int kThreads = (kTmaWarp + 1) * 32;  // 704
constexpr int kFold = 16;        // chunks summed in registers before a Kahan fold
constexpr int kAcc = 4;          // TMEM accumulators (one chunk each)
constexpr int kDone = 16;        // per-chunk MMA completion barriers (ring)
constexpr uint32_t kColAcc = 0;  // kAcc accumulators of kN columns, then the A stages
constexpr uint32_t kColA = kAcc * kN;
constexpr uint32_t kTmemCols = 512;
constexpr uint32_t kBBlock = kN * 128;   // bytes of one 128-byte-row tile of the N tile
constexpr uint32_t kTfMask = 0xFFFFE000u;

enum : int { kFormTF32 = 0, kFormF16 = 1, kFormBF16 = 2 };

template <int F> struct Form;
// TF32 split: A stage = 64 hi + 64 lo columns, 8 K-steps of 8, 3 products
template <> struct Form<kFormTF32> {
    static constexpr uint32_t kACols = 2 * kKC;
    static constexpr int kAStages = 2;
    static constexpr int kOpSlots = 2;
    static constexpr int kKStep = 8;
    static constexpr bool kSplit = true;
    static constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(kN >> 3) << 17) |
                                       ((uint32_t)(kM >> 4) << 24);
};
// FP16 split: A stage = 32 hi + 32 lo packed columns, 4 K-steps of 16, 3 products
template <> struct Form<kFormF16> {
    static constexpr uint32_t kACols = kKC;
    static constexpr int kAStages = 4;
    static constexpr int kOpSlots = 4;
    static constexpr int kKStep = 16;
    static constexpr bool kSplit = true;
    static constexpr uint32_t kIdesc = (1u << 4) | (0u << 7) | (0u << 10) | ((uint32_t)(kN >> 3) << 17) |
                                       ((uint32_t)(kM >> 4) << 24);
};
// BF16: A stage = 32 packed columns, 4 K-steps of 16, 1 product
template <> struct Form<kFormBF16> {
    static constexpr uint32_t kACols = kKC / 2;
    static constexpr int kAStages = 4;
    static constexpr int kOpSlots = 4;
    static constexpr int kKStep = 16;
    static constexpr bool kSplit = false;
    static constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kN >> 3) << 17) |
                                       ((uint32_t)(kM >> 4) << 24);
};
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

// Bounded wait that also gives up once another role has aborted.
__device__ __forceinline__ bool wait_or_abort(uint64_t *bar, uint32_t parity, volatile int *abort_flag) {
    for (uint32_t i = 0; i < kWaitLimit; i++) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((i & 255) == 255 && *abort_flag) return false;
    }
    return false;
}

// The same, with one answer for the whole warp (the tcgen05 loads and stores
// that follow are warp-collective: every lane takes the same branch).
__device__ __forceinline__ bool warp_wait(uint64_t *bar, uint32_t parity, volatile int *abort_flag) {
    return __all_sync(0xffffffffu, wait_or_abort(bar, parity, abort_flag));
}

// Barrier parity of the completion, for chunk i, of a barrier used every `every` chunks.
__device__ __forceinline__ uint32_t ph(long long i, int every) { return (uint32_t)((i / every) & 1); }

// two FP32 values -> packed 16-bit hi (and lo = v - hi for the split forms)
template <int F>
__device__ __forceinline__ void pack2(float x, float y, uint32_t &hi, uint32_t &lo) {
    if constexpr (F == kFormF16) {
        const __half2 h = __floats2half2_rn(x, y);
        const float2 back = __half22float2(h);
        const __half2 l = __floats2half2_rn(x - back.x, y - back.y);
        hi = *reinterpret_cast<const uint32_t *>(&h);
        lo = *reinterpret_cast<const uint32_t *>(&l);
    } else {
        const __nv_bfloat162 h = __floats2bfloat162_rn(x, y);
        hi = *reinterpret_cast<const uint32_t *>(&h);
        lo = 0u;
    }
}

struct TmArgs {
    long long nchunks;     // K / kKC
    int nunits, ksplit, nslots, nA, nstages, nmaps, nxb;
    uint32_t stage_bytes, op_bytes, ablock;
    float *kahan;          // [grid][2][kN][kM] running sum and compensation of each CTA (L2-resident)
    const int2 *units;     // (M tile, N tile) per unit
    const int2 *prow;      // [nunits][kM] staged rows (i, j) of each pair's factors, (-1, -1) for none
    const int *slots;      // [nunits][kM][kN] output slot or -1
    const int *mexp;       // FP16 form: per-map exponent e with |M| 2^e <= 2^14
    double *partial;       // [ksplit][nslots]
    int *err;              // set to 1 when a bounded wait gives up
};

template <int F>
__global__ void __launch_bounds__(kThreads, 1)
    trisum_tm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                     const TmArgs a) {
    using FM = Form<F>;
    constexpr int AST = FM::kAStages, kOpSlots = FM::kOpSlots;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char *base =
        reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    const int nst = a.nstages;
    // barriers: full per smem stage (TMA -> producers), prod per A stage (producers -> MMA),
    // done per chunk ring (MMA completion -> TMA, producers, drain), accfree per accumulator (drain -> MMA)
    // smem: nst staging slots | kOpSlots operand slots | barriers and tables
    unsigned char *opbase = base + (size_t)nst * a.stage_bytes;
    uint64_t *bars = reinterpret_cast<uint64_t *>(opbase + (size_t)kOpSlots * a.op_bytes);
    uint64_t *full = bars, *sfree = full + kMaxStages, *prod = sfree + kMaxStages, *done = prod + 4;
    uint64_t *accfree = done + kDone;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(accfree + kAcc);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);
    int2 *prow_s = reinterpret_cast<int2 *>(tmem_slot + 4);
    int *qexp_s = reinterpret_cast<int *>(prow_s + kM);  // [kN] FP16 exponent of each B row
    float *run_g = a.kahan + (size_t)blockIdx.x * 2 * kN * kM;  // [kN][kM], then the compensation
    float *comp_g = run_g + kN * kM;

    const int unit = blockIdx.x % a.nunits, split = blockIdx.x / a.nunits;
    const int2 U = a.units[unit];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const long long cb = a.nchunks * split / a.ksplit, ce = a.nchunks * (split + 1) / a.ksplit;
    const long long n = ce - cb;

    for (int r = tid; r < kM; r += kThreads) prow_s[r] = a.prow[(size_t)unit * kM + r];
    for (int r = tid; r < kN; r += kThreads) {
        const int q = U.y * kN + r;
        qexp_s[r] = (F == kFormF16 && q < a.nmaps) ? a.mexp[q] : 0;
    }
    if (tid == 0) {
        for (int s = 0; s < kMaxStages; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&sfree[s], 128);  // the warpgroup that consumed the slot
        }
        for (int s = 0; s < 4; s++) mbar_init(&prod[s], 128);  // one warpgroup per chunk
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

    // staging slot: A-source blocks [kBlocks][ablock] | B FP32 blocks [kBlocks][kBBlock]
    // operand slot: TF32 hi, lo blocks [2][kBlocks][kBBlock]; FP16/BF16 hi, lo tiles [2][kBBlock]
    auto stage_ptr = [&](int s) { return base + (size_t)s * a.stage_bytes; };
    auto op_ptr = [&](int o) { return opbase + (size_t)o * a.op_bytes; };
    auto fail = [&]() {
        *abort_flag = 1;
        atomicExch(a.err, 1);
    };

    if (warp < kProdWarps) {
        // ------------------------------------------------------------ producers
        const int quad = warp & 3, grp = warp >> 2;
        const int row = quad * 32 + lane;
        const int2 pr = prow_s[row];
        const float pscale =
            (F == kFormF16 && pr.x >= 0) ? exp2f((float)(a.mexp[pr.x] + a.mexp[pr.y] - 14)) : 1.0f;
        const uint32_t lane_addr = tmem + ((uint32_t)(quad * 32) << 16);
        const int gtid = tid & 127;
        for (long long i = grp; i < n; i += kGroups) {
            const int s = (int)(i % nst), as = (int)(i % AST), o = (int)(i % kOpSlots);
            if (!warp_wait(&full[s], ph(i, nst), abort_flag)) { fail(); break; }
            // the A stage and the operand slot are free once the MMAs of chunk
            // i - min(AST, kOpSlots) completed (MMAs complete in order)
            constexpr int kBack = AST < kOpSlots ? AST : kOpSlots;
            if (i >= kBack && !warp_wait(&done[(i - kBack) % kDone], ph(i - kBack, kDone), abort_flag)) {
                fail();
                break;
            }
            unsigned char *stg = stage_ptr(s);
            const unsigned char *bf = stg + kBlocks * a.ablock;  // FP32 B tile (kBlocks blocks)
            unsigned char *bx = op_ptr(o);
            if constexpr (F == kFormTF32) {
                // hi and lo blocks, elementwise on the swizzled bytes
                const float4 *bv = reinterpret_cast<const float4 *>(bf);
                float4 *hv = reinterpret_cast<float4 *>(bx);
                float4 *lv = reinterpret_cast<float4 *>(bx + kBlocks * kBBlock);
#pragma unroll
                for (int e = 0; e < (int)(kBlocks * kBBlock / 16) / 128; e++) {
                    const int idx = gtid + e * 128;
                    const float4 v = bv[idx];
                    float4 h, l;
                    h.x = __uint_as_float(__float_as_uint(v.x) & kTfMask); l.x = v.x - h.x;
                    h.y = __uint_as_float(__float_as_uint(v.y) & kTfMask); l.y = v.y - h.y;
                    h.z = __uint_as_float(__float_as_uint(v.z) & kTfMask); l.z = v.z - h.z;
                    h.w = __uint_as_float(__float_as_uint(v.w) & kTfMask); l.w = v.w - h.w;
                    hv[idx] = h;
                    lv[idx] = l;
                }
            } else {
                // 16-bit tiles: row r, 16-byte group g (points 8g..8g+7) at r*128 + ((g ^ (r&7)) << 4);
                // in the FP32 blocks those points are groups c, c+1 (c = 2 (g % 4)) of block g / 4
#pragma unroll
                for (int e = 0; e < 4; e++) {
                    const int t = gtid + e * 128, r = t >> 3, g = t & 7;
                    const unsigned char *blk = bf + (g >> 2) * kBBlock + r * 128;
                    const int c = 2 * (g & 3);
                    const float4 x0 = *reinterpret_cast<const float4 *>(blk + ((c ^ (r & 7)) << 4));
                    const float4 x1 = *reinterpret_cast<const float4 *>(blk + (((c + 1) ^ (r & 7)) << 4));
                    const float sc = F == kFormF16 ? exp2f((float)qexp_s[r]) : 1.0f;
                    uint32_t h[4], l[4];
                    pack2<F>(x0.x * sc, x0.y * sc, h[0], l[0]);
                    pack2<F>(x0.z * sc, x0.w * sc, h[1], l[1]);
                    pack2<F>(x1.x * sc, x1.y * sc, h[2], l[2]);
                    pack2<F>(x1.z * sc, x1.w * sc, h[3], l[3]);
                    const uint32_t off = (uint32_t)(r * 128 + ((g ^ (r & 7)) << 4));
                    *reinterpret_cast<uint4 *>(bx + off) = make_uint4(h[0], h[1], h[2], h[3]);
                    if (FM::kSplit) *reinterpret_cast<uint4 *>(bx + kBBlock + off) = make_uint4(l[0], l[1], l[2], l[3]);
                }
            }
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
                                const float p[4] = {u.x * v.x, u.y * v.y, u.z * v.z, u.w * v.w};
#pragma unroll
                                for (int e = 0; e < 4; e++) {
                                    const uint32_t h = __float_as_uint(p[e]) & kTfMask;
                                    hi[4 * c4 + e] = h;
                                    lo[4 * c4 + e] = __float_as_uint(p[e] - __uint_as_float(h));
                                }
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
                    // 32 points -> 16 packed columns (point 2c in the low half of column c)
                    uint32_t hi[16], lo[16];
                    if (pr.x >= 0) {
#pragma unroll
                        for (int c = 0; c < 8; c++) {
                            const float4 u =
                                *reinterpret_cast<const float4 *>(blk + pr.x * 128 + ((c ^ (pr.x & 7)) << 4));
                            const float4 v =
                                *reinterpret_cast<const float4 *>(blk + pr.y * 128 + ((c ^ (pr.y & 7)) << 4));
                            pack2<F>(u.x * v.x * pscale, u.y * v.y * pscale, hi[2 * c], lo[2 * c]);
                            pack2<F>(u.z * v.z * pscale, u.w * v.w * pscale, hi[2 * c + 1], lo[2 * c + 1]);
                        }
                    } else {
#pragma unroll
                        for (int e = 0; e < 16; e++) hi[e] = lo[e] = 0u;
                    }
                    const uint32_t col = acol + (uint32_t)(kb * (kKB / 2));
                    tmem_st16(lane_addr + col, hi);
                    if (FM::kSplit) tmem_st16(lane_addr + col + kKC / 2, lo);
                }
            }
            mbar_arrive(&sfree[s]);  // staging slot consumed (its values are in registers / TMEM / the operand slot)
            tmem_wait_st();
            fence_proxy_async();  // the B operand written by these threads is read by the tensor core
            tc_fence_before();
            mbar_arrive(&prod[as]);
        }
    } else if (warp < kMmaWarp) {
        // ---------------------------------------------------------------- drain
        // each chunk's accumulator is added into FP32 registers (round to nearest);
        // every kFold chunks those are folded into a Kahan-compensated sum kept in
        // shared memory ([column][row], conflict-free), written out at the end
        const int quad = warp & 3, cgrp = (warp - kProdWarps) >> 2;
        const int row = quad * 32 + lane, c0 = 32 * cgrp;
        const uint32_t lane_addr = tmem + ((uint32_t)(quad * 32) << 16);
        float mid[32];
#pragma unroll
        for (int e = 0; e < 32; e++) {
            mid[e] = 0.f;
            run_g[(c0 + e) * kM + row] = 0.f;
            comp_g[(c0 + e) * kM + row] = 0.f;
        }
        bool ok = true;
        for (long long i = 0; i < n; i++) {
            const int b = (int)(i % kAcc);
            if (!warp_wait(&done[i % kDone], ph(i, kDone), abort_flag)) { fail(); ok = false; break; }
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
#pragma unroll
                for (int e = 0; e < 32; e++) {
                    float *pr_ = run_g + (c0 + e) * kM + row, *pc = comp_g + (c0 + e) * kM + row;
                    const float y = mid[e] - *pc;
                    const float sm = *pr_;
                    const float t2 = sm + y;
                    *pc = (t2 - sm) - y;
                    *pr_ = t2;
                    mid[e] = 0.f;
                }
            }
        }
        if (__all_sync(0xffffffffu, ok && !*abort_flag)) {
            const int *sl = a.slots + ((size_t)unit * kM + row) * kN;
            const int2 pr = prow_s[row];
            const int pe = (F == kFormF16 && pr.x >= 0) ? a.mexp[pr.x] + a.mexp[pr.y] - 14 : 0;
#pragma unroll 4
            for (int e = 0; e < 32; e++) {
                const int slot = sl[c0 + e];
                if (slot < 0) continue;
                const double v = (double)run_g[(c0 + e) * kM + row] - (double)comp_g[(c0 + e) * kM + row];
                a.partial[(size_t)split * a.nslots + slot] = F == kFormF16 ? ldexp(v, -(pe + qexp_s[c0 + e])) : v;
            }
        }
    } else if (warp == kMmaWarp) {
        // --------------------------------------------------------- MMA issue (one thread)
        if (lane == 0) {
            long long last_commit = -1;
            bool ok = true;
            for (long long i = 0; i < n; i++) {
                const int b = (int)(i % kAcc), as = (int)(i % AST);
                if (i >= kAcc && !wait_or_abort(&accfree[b], ph(i - kAcc, kAcc), abort_flag)) { ok = false; break; }
                if (!wait_or_abort(&prod[as], ph(i, AST), abort_flag)) { ok = false; break; }
                tc_fence_after();
                const uint32_t b0 = smem_u32(op_ptr((int)(i % kOpSlots)));
                const uint32_t ahi = tmem + kColA + (uint32_t)as * FM::kACols;
                const uint32_t d = tmem + kColAcc + (uint32_t)b * kN;
#pragma unroll
                for (int kk = 0; kk < kKC / FM::kKStep; kk++) {
                    uint32_t bh, bl, a_hi, a_lo;
                    if constexpr (F == kFormTF32) {
                        // FP32 rows: K-step of 8 = 32 bytes; block kk / 4
                        bh = b0 + (uint32_t)(kk / 4) * kBBlock + (uint32_t)(kk % 4) * 32;
                        bl = bh + kBlocks * kBBlock;
                        a_hi = ahi + 8 * kk;
                        a_lo = a_hi + kKC;
                    } else {
                        // 16-bit rows: K-step of 16 = 32 bytes of the hi / lo tiles
                        bh = b0 + (uint32_t)kk * 32;
                        bl = bh + kBBlock;
                        a_hi = ahi + 8 * kk;
                        a_lo = a_hi + kKC / 2;
                    }
                    const uint64_t dh = sw128_desc(bh);
                    umma_ta<F>(d, a_hi, dh, kk == 0 ? 0u : 1u);
                    if (FM::kSplit) {
                        umma_ta<F>(d, a_hi, sw128_desc(bl), 1u);
                        umma_ta<F>(d, a_lo, dh, 1u);
                    }
                }
                umma_commit(&done[i % kDone]);
                last_commit = i;
            }
            if (!ok) fail();
            // the MMAs still in flight (and their barrier arrival) land before TMEM goes away
            if (last_commit >= 0) mbar_wait(&done[last_commit % kDone], ph(last_commit, kDone));
        }
    } else if (lane == 0) {
        // --------------------------------------------------------- TMA issue (one thread)
        const uint32_t tx = kBlocks * ((uint32_t)a.nA * 128 + kBBlock);
        long long issued = 0;
        bool ok = true;
        for (long long j = 0; j < n; j++) {
            const int s = (int)(j % nst);
            // staging slot s is free once the producers consumed chunk j - nst
            if (j >= nst && !wait_or_abort(&sfree[s], ph(j - nst, nst), abort_flag)) {
                ok = false;
                break;
            }
            unsigned char *stg = stage_ptr(s);
            mbar_expect_tx(&full[s], tx);
#pragma unroll
            for (int kb = 0; kb < kBlocks; kb++) {
                // K block -> (32-point x block, map row); blocks past the last row read zeros
                const long long blk = (cb + j) * kBlocks + kb;
                const int row = (int)(blk / a.nxb), x0 = (int)(blk - (long long)row * a.nxb) * kKB;
                tma_load_3d(stg + kb * a.ablock, &tmA, x0, 0, row, &full[s]);
                tma_load_3d(stg + kBlocks * a.ablock + kb * kBBlock, &tmB, x0, U.y * kN, row, &full[s]);
            }
            issued = j + 1;
        }
        if (!ok) {
            fail();
            // copies in flight land (bounded) before the shared memory goes away
            for (long long j = std::max(0LL, issued - nst); j < issued; j++)
                mbar_wait(&full[j % nst], ph(j, nst));
        }
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

// 3D FP32 view of the row-interleaved maps [Nm^2 rows][nmaps][Nm]: box 32 x
// box_rows x 1 at (x0, first map, row), 128-byte swizzle, zero fill past the
// row end (x >= Nm), past `rows` maps and past the last row.
int make_row_view(CUtensorMap *tm, const float *maps, int Nm, int nmaps, int rows, int box_rows) {
    EncodeTiledFn enc = encode_fn();
    if (!enc) return set_error(PBI4G_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
    const cuuint64_t gdim[3] = {(cuuint64_t)Nm, (cuuint64_t)rows, (cuuint64_t)Nm * Nm};
    const cuuint64_t gstride[2] = {(cuuint64_t)Nm * sizeof(float), (cuuint64_t)nmaps * Nm * sizeof(float)};
    const cuuint32_t box[3] = {(cuuint32_t)kKB, (cuuint32_t)box_rows, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    const CUresult r = enc(tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float *>(maps), gdim, gstride, box,
                           estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
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
    const long long rows = (long long)sh.Nm * sh.Nm;
    return sh.nb <= 256 && sh.Nm % 4 == 0 && rows * ((sh.Nm + kKB - 1) / kKB) < (1LL << 31);
}

template <int F>
static int launch_tm(const CUtensorMap &tmA, const CUtensorMap &tmB, const TmArgs &a, size_t smem, int grid,
                     cudaStream_t st) {
    PBI4G_CUDA(cudaFuncSetAttribute(trisum_tm_kernel<F>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    trisum_tm_kernel<F><<<grid, kThreads, smem, st>>>(tmA, tmB, a);
    PBI4G_LAUNCH_CHECK();
    return PBI4G_OK;
}

int triangle_sums_tm(const Shells &sh, TmPlan &tp, int form, const float *maps, int nmaps, const double *powsum,
                     int pow_mask, const double lfac[3], DevBuf &partial, double *S, cudaStream_t st,
                     int64_t *launches) {
    const int N = sh.Nm;
    if (!tm_supported(sh))
        return set_error(PBI4G_ERR_UNSUPPORTED, "tensor-core triangle sums: map grid %d, %d shells", N, sh.nb);
    if (form < 0 || form > 2) return set_error(PBI4G_ERR_INVALID, "tensor-core form %d", form);
    if (tp.nunits == 0) return PBI4G_OK;
    if (reinterpret_cast<uintptr_t>(maps) % 16)
        return set_error(PBI4G_ERR_INVALID, "tensor-core triangle sums: maps must be 16-byte aligned");
    PBI4G_CHECK(tp.mexp.ensure(sizeof(int) * std::max(1, nmaps)));
    if (form == 1) {
        map_exponents_kernel<<<1, 256, 0, st>>>(nmaps, sh.nb, powsum, pow_mask, lfac[1], lfac[2],
                                                sh.nmodes_d.as<double>(), tp.mexp.as<int>());
        PBI4G_LAUNCH_CHECK();
        *launches += 1;
    }
    CUtensorMap tmA, tmB;
    PBI4G_CHECK(make_row_view(&tmA, maps, N, nmaps, sh.nb, tp.nA));
    PBI4G_CHECK(make_row_view(&tmB, maps, N, nmaps, nmaps, kN));
    TmArgs a;
    // K blocks: (map row, 32-point x block), the last x block of a row zero-padded
    a.nxb = (N + kKB - 1) / kKB;
    a.nchunks = ((long long)N * N * a.nxb + kBlocks - 1) / kBlocks;
    a.nunits = tp.nunits;
    a.ksplit = std::max(1, 152 / tp.nunits);
    a.ksplit = (int)std::min<long long>(a.ksplit, std::max<long long>(1, a.nchunks / 128));
    a.nslots = tp.nslots;
    a.nA = tp.nA;
    a.nmaps = nmaps;
    a.ablock = (uint32_t)(((tp.nA + 7) / 8) * 8 * 128);
    a.stage_bytes = kBlocks * (a.ablock + kBBlock);
    a.op_bytes = form == 0 ? 2 * kBlocks * kBBlock : 2 * kBBlock;
    // barriers, TMEM address, abort flag, pair table, B-row exponents
    const size_t tail = 8 * (2 * kMaxStages + 4 + kDone + kAcc) + 16 + sizeof(int2) * kM + sizeof(int) * kN;
    const int op_slots = form == 0 ? Form<kFormTF32>::kOpSlots : Form<kFormF16>::kOpSlots;
    const size_t fixed = 1024 + (size_t)op_slots * a.op_bytes + tail;
    a.nstages = kMaxStages;
    while (a.nstages > 3 && fixed + (size_t)a.nstages * a.stage_bytes > 227 * 1024) a.nstages--;
    const size_t smem = fixed + (size_t)a.nstages * a.stage_bytes;
    if (smem > 227 * 1024) return set_error(PBI4G_ERR_UNSUPPORTED, "tensor-core triangle sums: %zu B smem", smem);
    a.units = tp.units.as<int2>();
    a.prow = tp.prow.as<int2>();
    a.slots = tp.slots.as<int>();
    a.mexp = tp.mexp.as<int>();
    PBI4G_CHECK(partial.ensure(sizeof(double) * (size_t)a.ksplit * tp.nslots));
    a.partial = partial.as<double>();
    a.err = tp.err.as<int>();
    PBI4G_CUDA(cudaMemsetAsync(tp.err.p, 0, sizeof(int), st));
    const int grid = tp.nunits * a.ksplit;
    PBI4G_CHECK(tp.kahan.ensure(sizeof(float) * 2 * kN * kM * (size_t)grid));
    a.kahan = tp.kahan.as<float>();
    if (form == 0) PBI4G_CHECK(launch_tm<kFormTF32>(tmA, tmB, a, smem, grid, st));
    else if (form == 1) PBI4G_CHECK(launch_tm<kFormF16>(tmA, tmB, a, smem, grid, st));
    else PBI4G_CHECK(launch_tm<kFormBF16>(tmA, tmB, a, smem, grid, st));
    PBI4G_CHECK(reduce_partials(tp.nslots, a.ksplit, partial.as<double>(), S, st));
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
