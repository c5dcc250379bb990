// trisum_tc.cu -- triangle sums on the 5th-generation tensor cores (tcgen05).
//
// The "Last sum" loops of measure_bk / measure_bk_multipoles
// (bispectrumI4.f90:160-195, 476-513), S(l,j,i) = sum_x M_i M_j M_l (and the
// B2/B4 sums with the delta_2 / delta_4 maps of shell l), recast as a
// contraction over the grid points x:
//     C[p, q] = sum_x A[p, x] Bq[q, x],   A[p, x] = M_i(x) M_j(x) for the pair p = (i, j),
//                                          Bq[q, x] = map q (shell l of multipole set s).
// Only the (p, q) entries that are triangles are kept.
//
// Per CTA: up to two M tiles of 128 pairs sharing one N tile of 64 q maps, a
// contiguous range of the contraction.  For every chunk of 64 grid points the
// 256 threads stage the FP32 maps the unit needs, form the operands in shared
// memory in the canonical K-major 128-byte-swizzled layout, and one thread
// issues tcgen05.mma (M=128, N=64, K=16) into TMEM accumulators.  Two operand
// stages let the tensor core run chunk c while the threads build chunk c+1.
//
// Precision forms:
//   FP16 split: every operand value v (scaled by a power of two so |v| <= 2^14)
//     is stored as hi = fp16(v), lo = fp16(v - hi); each K step issues
//     A_hi.B_hi + A_hi.B_lo + A_lo.B_hi (22-bit products, FP32 accumulate).
//   BF16: one bf16 product.
// Accumulation: FP32 in TMEM for 32 chunks (2048 points), then folded into a
// Kahan-compensated FP32 running sum that also lives in TMEM; the final sums
// leave in FP64 scaled back by the power-of-two exponents.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <map>
#include <set>

#include "bispec.cuh"
#include "trisum_tc.cuh"

namespace pbi4g {

namespace {

constexpr int kMT = 2;           // M tiles per unit
constexpr int kBM = 128;         // pairs per M tile (MMA M)
constexpr int kBN = 64;          // q maps per unit (MMA N)
constexpr int kKC = 64;          // grid points per chunk (one 128-byte swizzle row of fp16)
constexpr int kThreads = 256;
constexpr int kDrain = 32;       // chunks per TMEM accumulation period
constexpr int kStageRow = kKC + 4;
constexpr uint32_t kTmemCols = 512;
constexpr uint32_t kWaitLimit = 1u << 22;  // try_wait polls before a wait gives up

constexpr int kATile = kBM * kKC * 2;   // 16 KB
constexpr int kBTile = kBN * kKC * 2;   // 8 KB
constexpr int kStageBytes = 2 * kMT * kATile + 2 * kBTile;  // hi+lo of A (MT tiles) and B = 80 KB

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.b32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait on an mbarrier phase; false if the limit ran out.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
    for (uint32_t i = 0; i < kWaitLimit; i++)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// 8-byte asynchronous global -> shared copies (the padded C2R rows are 8-byte aligned)
__device__ __forceinline__ void cp_async8(void *smem, const void *gmem) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_u32(smem)), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait0() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_alloc(uint32_t *dst, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)), "r"(ncols)
                 : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// K-major operand, 128-byte swizzle: rows of 128 B, 8-row atoms of 1024 B.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);  // start address
    d |= (uint64_t)1 << 16;                    // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)(1024 >> 4) << 32;          // stride byte offset: 8 rows x 128 B
    d |= (uint64_t)1 << 46;                    // descriptor version (sm_100 family)
    d |= (uint64_t)2 << 61;                    // SWIZZLE_128B
    return d;
}

// kind::f16 instruction descriptor: FP32 accumulate, K-major A and B, M = 128, N = kBN.
__host__ __device__ constexpr uint32_t idesc_f16(bool bf16) {
    return (1u << 4)                            // D format F32
           | ((bf16 ? 1u : 0u) << 7)            // A format
           | ((bf16 ? 1u : 0u) << 10)           // B format
           | ((uint32_t)(kBN >> 3) << 17)       // N
           | ((uint32_t)(kBM >> 4) << 24);      // M
}

__device__ __forceinline__ void umma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accum) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accum)
        : "memory");
}

__device__ __forceinline__ void umma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

#define TC_R32(x) "=r"(x[0]), "=r"(x[1]), "=r"(x[2]), "=r"(x[3]), "=r"(x[4]), "=r"(x[5]), "=r"(x[6]), "=r"(x[7]), \
    "=r"(x[8]), "=r"(x[9]), "=r"(x[10]), "=r"(x[11]), "=r"(x[12]), "=r"(x[13]), "=r"(x[14]), "=r"(x[15]),       \
    "=r"(x[16]), "=r"(x[17]), "=r"(x[18]), "=r"(x[19]), "=r"(x[20]), "=r"(x[21]), "=r"(x[22]), "=r"(x[23]),     \
    "=r"(x[24]), "=r"(x[25]), "=r"(x[26]), "=r"(x[27]), "=r"(x[28]), "=r"(x[29]), "=r"(x[30]), "=r"(x[31])
#define TC_W32(x) "r"(x[0]), "r"(x[1]), "r"(x[2]), "r"(x[3]), "r"(x[4]), "r"(x[5]), "r"(x[6]), "r"(x[7]), \
    "r"(x[8]), "r"(x[9]), "r"(x[10]), "r"(x[11]), "r"(x[12]), "r"(x[13]), "r"(x[14]), "r"(x[15]),         \
    "r"(x[16]), "r"(x[17]), "r"(x[18]), "r"(x[19]), "r"(x[20]), "r"(x[21]), "r"(x[22]), "r"(x[23]),       \
    "r"(x[24]), "r"(x[25]), "r"(x[26]), "r"(x[27]), "r"(x[28]), "r"(x[29]), "r"(x[30]), "r"(x[31])

// 32 consecutive 32-bit TMEM columns of this thread's lane (warp quadrant lanes)
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : TC_R32(r)
        : "r"(taddr)
        : "memory");
}
__device__ __forceinline__ void tmem_st32(uint32_t taddr, const uint32_t (&r)[32]) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31, %32};" ::"r"(taddr),
        TC_W32(r)
        : "memory");
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// byte offset of the 16-byte group g (8 halves) of row r in a 128B-swizzled K-major tile
__device__ __forceinline__ uint32_t sw128_off(int r, int g) { return (uint32_t)(r * 128 + ((g ^ (r & 7)) << 4)); }

template <bool SPLIT>
__device__ __forceinline__ void split8(const float v[8], uint4 &hi, uint4 &lo) {
    uint32_t h[4], l[4];
#pragma unroll
    for (int e = 0; e < 4; e++) {
        if (SPLIT) {
            // paired conversions: hi = fp16(v), lo = fp16(v - hi)
            const __half2 hh = __floats2half2_rn(v[2 * e], v[2 * e + 1]);
            const float2 back = __half22float2(hh);
            const __half2 ll = __floats2half2_rn(v[2 * e] - back.x, v[2 * e + 1] - back.y);
            h[e] = *reinterpret_cast<const uint32_t *>(&hh);
            l[e] = *reinterpret_cast<const uint32_t *>(&ll);
        } else {
            const __nv_bfloat162 bb = __floats2bfloat162_rn(v[2 * e], v[2 * e + 1]);
            h[e] = *reinterpret_cast<const uint32_t *>(&bb);
            l[e] = 0;
        }
    }
    hi = make_uint4(h[0], h[1], h[2], h[3]);
    lo = make_uint4(l[0], l[1], l[2], l[3]);
}

struct TcArgs {
    const float *maps;     // FP32 maps, map m at maps + m * mstride, row stride rs
    size_t mstride;
    int rs, N, umax;
    long long K;           // contraction length (N^3)
    int nunits, ksplit, nslots;
    const int4 *units;     // (mt0 present, mt1 present, nU, 0)
    const int *umaps;      // [nunits][umax] staged map indices
    const int2 *psrc;      // [nunits][kMT*kBM] staging indices of the pair factors (-1: zero row)
    const int *qsrc;       // [nunits][kBN] staging index of the q map (-1: zero row)
    const int *pexp;       // [nunits][kMT*kBM] power-of-two exponent of the A row (e_i + e_j - 14)
    const int *qexp;       // [nunits][kBN] exponent of the B row (e_q)
    const int *mexp;       // [nmaps] exponent e_m with |M_m| 2^e_m <= 2^14
    const int *slots;      // [nunits][kMT*kBM][kBN] output slot or -1
    double *partial;       // [ksplit][nslots]
    int *err;              // set to 1 when a bounded wait gives up
};

template <bool SPLIT>
__global__ void __launch_bounds__(kThreads, 1) trisum_tc_kernel(const TcArgs a) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    // 1024-byte alignment of the operand stages (swizzle atoms)
    unsigned char *base = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    unsigned char *stage0 = base;
    float *stg = reinterpret_cast<float *>(base + 2 * kStageBytes);  // [2][umax][kStageRow] raw FP32 maps
    int *pexp_s = reinterpret_cast<int *>(stg + 2 * (size_t)a.umax * kStageRow);  // [kMT*kBM]
    int *qexp_s = pexp_s + kMT * kBM;                                 // [kBN]
    int2 *sps = reinterpret_cast<int2 *>(qexp_s + kBN);                // [kMT*kBM]
    int *sqs = reinterpret_cast<int *>(sps + kMT * kBM);               // [kBN]
    int *umap_s = sqs + kBN;                                           // [umax]
    float *uscale = reinterpret_cast<float *>(umap_s + a.umax);       // [umax]
    uint64_t *bars = reinterpret_cast<uint64_t *>(((reinterpret_cast<uintptr_t>(uscale + a.umax)) + 7) & ~(uintptr_t)7);
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 2);
    int *sflag = reinterpret_cast<int *>(tmem_slot + 1);

    const int unit = blockIdx.x % a.nunits, split = blockIdx.x / a.nunits;
    const int4 U = a.units[unit];
    const int nU = U.z;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const bool has_mt[2] = {U.x != 0, U.y != 0};

    for (int i = tid; i < kMT * kBM; i += kThreads) {
        sps[i] = a.psrc[(size_t)unit * kMT * kBM + i];
        pexp_s[i] = a.pexp[(size_t)unit * kMT * kBM + i];
    }
    for (int i = tid; i < kBN; i += kThreads) {
        sqs[i] = a.qsrc[(size_t)unit * kBN + i];
        qexp_s[i] = a.qexp[(size_t)unit * kBN + i];
    }
    for (int i = tid; i < nU; i += kThreads) {
        umap_s[i] = a.umaps[(size_t)unit * a.umax + i];
        uscale[i] = exp2f((float)a.mexp[umap_s[i]]);
    }
    if (tid == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        *sflag = 0;
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
    // TMEM columns: acc [0, kMT*kBN), run [kMT*kBN, 2 kMT*kBN), comp [2 kMT*kBN, 3 kMT*kBN)
    const uint32_t c_acc = 0, c_run = kMT * kBN, c_comp = 2 * kMT * kBN;
    if (warp < 4) {  // zero the running sums
        uint32_t z[32];
#pragma unroll
        for (int e = 0; e < 32; e++) z[e] = 0;
        const uint32_t lrow = tmem + ((uint32_t)(warp * 32) << 16);
        for (int c = 0; c < 2 * kMT * kBN; c += 32) tmem_st32(lrow + c_run + c, z);
        tmem_wait_st();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();

    const long long nchunks = a.K / kKC;
    const long long cb = nchunks * split / a.ksplit, ce = nchunks * (split + 1) / a.ksplit;
    const uint32_t idesc = idesc_f16(!SPLIT);
    bool failed = false;
    int in_period = 0;
    long long last_commit = -1;  // local index of the last chunk whose MMAs were committed
    // asynchronous staging of the maps of chunk ch into buffer b (one commit group per chunk)
    auto stage = [&](long long ch, int b) {
        const long long k0 = ch * kKC;
        float *dst0 = stg + (size_t)b * a.umax * kStageRow;
        for (int idx = tid; idx < nU * (kKC / 2); idx += kThreads) {
            const int u = idx / (kKC / 2), c = idx - u * (kKC / 2);
            const long long p = k0 + 2 * c;
            cp_async8(dst0 + (size_t)u * kStageRow + 2 * c,
                      a.maps + (size_t)umap_s[u] * a.mstride + (size_t)(p / a.N) * a.rs + (size_t)(p % a.N));
        }
        cp_async_commit();
    };
    if (cb < ce) stage(cb, 0);
    for (long long ch = cb; ch < ce && !failed; ch++) {
        const long long i = ch - cb;
        const int s = (int)(i & 1);
        unsigned char *st = stage0 + s * kStageBytes;
        // prefetch the next chunk into the other staging buffer, then wait for this one
        if (ch + 1 < ce) stage(ch + 1, s ^ 1);
        else cp_async_commit();
        cp_async_wait1();
        if (i >= 2) {
            if (!mbar_wait(&bars[s], (uint32_t)(((i - 2) >> 1) & 1))) *sflag = 1;
            tc_fence_after();
        }
        __syncthreads();
        const float *sg = stg + (size_t)s * a.umax * kStageRow;
        // operands: B rows (q maps) then A rows (pair products), 8 points per item
        unsigned char *Ahi = st, *Alo = st + kMT * kATile, *Bhi = st + 2 * kMT * kATile, *Blo = Bhi + kBTile;
        for (int it = tid; it < (kBN + kMT * kBM) * (kKC / 8); it += kThreads) {
            const int row = it >> 3, g = it & 7;
            float v[8];
            if (row < kBN) {
                const int src = sqs[row];
                if (src >= 0) {
                    const float4 x0 = *reinterpret_cast<const float4 *>(sg + (size_t)src * kStageRow + 8 * g);
                    const float4 x1 = *reinterpret_cast<const float4 *>(sg + (size_t)src * kStageRow + 8 * g + 4);
                    const float sc = uscale[src];
                    v[0] = x0.x * sc; v[1] = x0.y * sc; v[2] = x0.z * sc; v[3] = x0.w * sc;
                    v[4] = x1.x * sc; v[5] = x1.y * sc; v[6] = x1.z * sc; v[7] = x1.w * sc;
                } else {
#pragma unroll
                    for (int e = 0; e < 8; e++) v[e] = 0.f;
                }
                uint4 hi, lo;
                split8<SPLIT>(v, hi, lo);
                *reinterpret_cast<uint4 *>(Bhi + sw128_off(row, g)) = hi;
                if (SPLIT) *reinterpret_cast<uint4 *>(Blo + sw128_off(row, g)) = lo;
            } else {
                const int pr = row - kBN, t = pr / kBM, r = pr % kBM;
                if (!has_mt[t]) continue;
                const int2 src = sps[pr];
                if (src.x >= 0) {
                    const float *px = sg + (size_t)src.x * kStageRow + 8 * g, *py = sg + (size_t)src.y * kStageRow + 8 * g;
                    const float4 x0 = *reinterpret_cast<const float4 *>(px), x1 = *reinterpret_cast<const float4 *>(px + 4);
                    const float4 y0 = *reinterpret_cast<const float4 *>(py), y1 = *reinterpret_cast<const float4 *>(py + 4);
                    const float sc = uscale[src.x] * uscale[src.y] * 0x1p-14f;
                    v[0] = x0.x * y0.x * sc; v[1] = x0.y * y0.y * sc; v[2] = x0.z * y0.z * sc; v[3] = x0.w * y0.w * sc;
                    v[4] = x1.x * y1.x * sc; v[5] = x1.y * y1.y * sc; v[6] = x1.z * y1.z * sc; v[7] = x1.w * y1.w * sc;
                } else {
#pragma unroll
                    for (int e = 0; e < 8; e++) v[e] = 0.f;
                }
                uint4 hi, lo;
                split8<SPLIT>(v, hi, lo);
                *reinterpret_cast<uint4 *>(Ahi + t * kATile + sw128_off(r, g)) = hi;
                if (SPLIT) *reinterpret_cast<uint4 *>(Alo + t * kATile + sw128_off(r, g)) = lo;
            }
        }
        fence_proxy_async();
        __syncthreads();
        if (*sflag) failed = true;
        if (tid == 0 && !failed) {
            tc_fence_after();
            const uint32_t bh = smem_u32(Bhi), bl = smem_u32(Blo);
#pragma unroll
            for (int t = 0; t < kMT; t++) {
                if (!has_mt[t]) continue;
                const uint32_t ah = smem_u32(Ahi + t * kATile), al = smem_u32(Alo + t * kATile);
                const uint32_t d = tmem + c_acc + t * kBN;
#pragma unroll
                for (int kk = 0; kk < kKC / 16; kk++) {
                    const uint32_t first = (in_period == 0 && kk == 0) ? 0u : 1u;
                    umma(d, sw128_desc(ah + kk * 32), sw128_desc(bh + kk * 32), idesc, first);
                    if (SPLIT) {
                        umma(d, sw128_desc(ah + kk * 32), sw128_desc(bl + kk * 32), idesc, 1u);
                        umma(d, sw128_desc(al + kk * 32), sw128_desc(bh + kk * 32), idesc, 1u);
                    }
                }
            }
            umma_commit(&bars[s]);
        }
        if (!failed) last_commit = i;
        in_period++;
        const bool last = ch + 1 == ce;
        if (in_period == kDrain || last) {
            // fold the period's accumulators into the Kahan running sums
            if (!mbar_wait(&bars[s], (uint32_t)((i >> 1) & 1))) *sflag = 1;
            tc_fence_after();
            __syncthreads();
            if (warp < 4 && !*sflag) {
                const uint32_t lrow = tmem + ((uint32_t)(warp * 32) << 16);
                for (int c = 0; c < kMT * kBN; c += 32) {
                    if (!has_mt[c / kBN]) continue;
                    uint32_t ac[32], ru[32], co[32];
                    tmem_ld32(lrow + c_acc + c, ac);
                    tmem_ld32(lrow + c_run + c, ru);
                    tmem_ld32(lrow + c_comp + c, co);
                    tmem_wait_ld();
#pragma unroll
                    for (int e = 0; e < 32; e++) {
                        const float y = __uint_as_float(ac[e]) - __uint_as_float(co[e]);
                        const float sm = __uint_as_float(ru[e]);
                        const float t2 = sm + y;
                        co[e] = __float_as_uint((t2 - sm) - y);
                        ru[e] = __float_as_uint(t2);
                    }
                    tmem_st32(lrow + c_run + c, ru);
                    tmem_st32(lrow + c_comp + c, co);
                }
                tmem_wait_st();
            }
            tc_fence_before();
            __syncthreads();
            tc_fence_after();
            in_period = 0;
            if (*sflag) failed = true;
        }
    }
    cp_async_wait0();
    if (failed) {
        if (tid == 0) {
            atomicExch(a.err, 1);
            // let the MMAs still in flight finish (bounded) before TMEM is released
            if (last_commit >= 0) mbar_wait(&bars[last_commit & 1], (uint32_t)((last_commit >> 1) & 1));
        }
    } else if (warp < 4) {
        // results: (run - comp) * 2^-(pair exponent + q exponent) -> partial[split][slot]
        const uint32_t lrow = tmem + ((uint32_t)(warp * 32) << 16);
        const int r = warp * 32 + lane;
        for (int c = 0; c < kMT * kBN; c += 32) {
            const int t = c / kBN;
            if (!has_mt[t]) continue;
            uint32_t ru[32], co[32];
            tmem_ld32(lrow + c_run + c, ru);
            tmem_ld32(lrow + c_comp + c, co);
            tmem_wait_ld();
            const int prow = t * kBM + r;
            const int *sl = a.slots + ((size_t)unit * kMT * kBM + prow) * kBN;
            const int pe = pexp_s[prow];
#pragma unroll
            for (int e = 0; e < 32; e++) {
                const int qc = (c % kBN) + e;
                const int slot = sl[qc];
                if (slot < 0) continue;
                const double v = (double)__uint_as_float(ru[e]) - (double)__uint_as_float(co[e]);
                a.partial[(size_t)split * a.nslots + slot] = ldexp(v, -(pe + qexp_s[qc]));
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, kTmemCols);
    }
}

// Per-map power-of-two scale: |M(x)| <= sum_k |H(k)| <= sqrt(nmodes * sum_k |H(k)|^2)
// (triangle and Cauchy-Schwarz inequalities over the shell's modes).  Sets
// without their own power use the delta set's times max |L_l(mu)| (lfac).
__global__ void map_exponents_kernel(int nmaps, int nb, const double *__restrict__ powsum, int pow_mask,
                                     double lf1, double lf2, const double *__restrict__ nmodes, int *__restrict__ e) {
    for (int m = threadIdx.x; m < nmaps; m += blockDim.x) {
        const int s = m / nb, b = m % nb;
        const double p = (pow_mask >> s & 1) ? powsum[s * nb + b] : powsum[b];
        const double lf = s == 0 ? 1.0 : (s == 1 ? lf1 : lf2);
        const double v = sqrt(nmodes[b] * p) * ((pow_mask >> s & 1) ? 1.0 : lf);
        // scale so that |M| 2^e <= 2^14, clamped to the float exponent range of the staged values
        int x = v > 0 ? 14 - (int)ceil(log2(v)) : 0;
        e[m] = x < -100 ? -100 : (x > 100 ? 100 : x);
    }
}

__global__ void unit_exponents_kernel(int nunits, const int *__restrict__ mexp, const int2 *__restrict__ pmap,
                                      const int *__restrict__ qmapi, int *__restrict__ pexp, int *__restrict__ qexp) {
    const int n = nunits * kMT * kBM;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int2 pm = pmap[i];
        pexp[i] = pm.x >= 0 ? mexp[pm.x] + mexp[pm.y] - 14 : 0;
    }
    const int nq = nunits * kBN;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nq; i += gridDim.x * blockDim.x)
        qexp[i] = qmapi[i] >= 0 ? mexp[qmapi[i]] : 0;
}

}  // namespace

// ------------------------------------------------------------- host plan ---
int TcPlan::build(const Shells &sh, int nsets_) {
    nsets = nsets_;
    const int nb = sh.nb;
    // pairs (i, j), i <= j, in first-appearance order; q = (l-1)*nsets + s
    std::map<std::pair<int, int>, int> pidx;
    std::vector<int2> plist;
    struct E { int p, q, slot; };
    std::vector<E> ents;
    for (int64_t m = 0; m < sh.itot; m++) {
        const int l = sh.tri[3 * m], j = sh.tri[3 * m + 1], i = sh.tri[3 * m + 2];
        auto key = std::make_pair(j - 1, i - 1);
        int p;
        auto it = pidx.find(key);
        if (it == pidx.end()) { p = (int)plist.size(); pidx[key] = p; plist.push_back(make_int2(i - 1, j - 1)); }
        else p = it->second;
        for (int s = 0; s < nsets; s++) ents.push_back({p, (l - 1) * nsets + s, (int)(m * nsets + s)});
    }
    npairs = (int)plist.size();
    nslots = (int)(sh.itot * nsets);
    const int nmt = (npairs + kBM - 1) / kBM, nq = nsets * nb, nnt = (nq + kBN - 1) / kBN;
    std::vector<char> need((size_t)nmt * nnt, 0);
    for (auto &e : ents) need[(size_t)(e.p / kBM) * nnt + e.q / kBN] = 1;
    struct Unit { int mt[2]; int nt; };
    std::vector<Unit> ul;
    for (int nt = 0; nt < nnt; nt++) {
        std::vector<int> mts;
        for (int mt = 0; mt < nmt; mt++)
            if (need[(size_t)mt * nnt + nt]) mts.push_back(mt);
        for (size_t k = 0; k < mts.size(); k += kMT)
            ul.push_back({{mts[k], k + 1 < mts.size() ? mts[k + 1] : -1}, nt});
    }
    nunits = (int)ul.size();
    // staging lists
    umax = 0;
    std::vector<std::vector<int>> um(nunits);
    for (int u = 0; u < nunits; u++) {
        std::set<int> maps;
        for (int t = 0; t < kMT; t++) {
            if (ul[u].mt[t] < 0) continue;
            for (int r = 0; r < kBM; r++) {
                const int p = ul[u].mt[t] * kBM + r;
                if (p >= npairs) break;
                maps.insert(plist[p].x);  // set-0 map of shell i
                maps.insert(plist[p].y);
            }
        }
        for (int c = 0; c < kBN; c++) {
            const int q = ul[u].nt * kBN + c;
            if (q >= nq) break;
            const int l = q / nsets + 1, s = q % nsets;
            maps.insert(s * nb + l - 1);
        }
        um[u].assign(maps.begin(), maps.end());
        umax = std::max(umax, (int)um[u].size());
    }
    std::vector<int> h_umaps((size_t)nunits * umax, 0), h_qsrc((size_t)nunits * kBN, -1), h_qmap((size_t)nunits * kBN, -1);
    std::vector<int2> h_psrc((size_t)nunits * kMT * kBM, make_int2(-1, -1)), h_pmap(h_psrc);
    std::vector<int> h_slots((size_t)nunits * kMT * kBM * kBN, -1);
    std::vector<int4> h_units(nunits);
    for (int u = 0; u < nunits; u++) {
        std::map<int, int> pos;
        for (size_t k = 0; k < um[u].size(); k++) {
            pos[um[u][k]] = (int)k;
            h_umaps[(size_t)u * umax + k] = um[u][k];
        }
        h_units[u] = make_int4(ul[u].mt[0] >= 0, ul[u].mt[1] >= 0, (int)um[u].size(), 0);
        for (int t = 0; t < kMT; t++) {
            if (ul[u].mt[t] < 0) continue;
            for (int r = 0; r < kBM; r++) {
                const int p = ul[u].mt[t] * kBM + r;
                if (p >= npairs) break;
                const size_t o = (size_t)u * kMT * kBM + t * kBM + r;
                h_psrc[o] = make_int2(pos[plist[p].x], pos[plist[p].y]);
                h_pmap[o] = plist[p];
            }
        }
        for (int c = 0; c < kBN; c++) {
            const int q = ul[u].nt * kBN + c;
            if (q >= nq) break;
            const int l = q / nsets + 1, s = q % nsets, m = s * nb + l - 1;
            h_qsrc[(size_t)u * kBN + c] = pos[m];
            h_qmap[(size_t)u * kBN + c] = m;
        }
    }
    // slots: entry (p, q) lives in the unit holding (p / kBM, q / kBN)
    std::map<std::pair<int, int>, std::pair<int, int>> where;  // (mt, nt) -> (unit, t)
    for (int u = 0; u < nunits; u++)
        for (int t = 0; t < kMT; t++)
            if (ul[u].mt[t] >= 0) where[std::make_pair(ul[u].mt[t], ul[u].nt)] = std::make_pair(u, t);
    for (auto &e : ents) {
        auto w = where.at(std::make_pair(e.p / kBM, e.q / kBN));
        const size_t o = (((size_t)w.first * kMT + w.second) * kBM + e.p % kBM) * kBN + e.q % kBN;
        h_slots[o] = e.slot;
    }
    useful = (double)ents.size() / ((double)nunits * kMT * kBM * kBN);
    PBI4G_CHECK(units.ensure(sizeof(int4) * std::max(1, nunits)));
    PBI4G_CHECK(umaps.ensure(sizeof(int) * std::max<size_t>(1, h_umaps.size())));
    PBI4G_CHECK(psrc.ensure(sizeof(int2) * h_psrc.size()));
    PBI4G_CHECK(pmap.ensure(sizeof(int2) * h_pmap.size()));
    PBI4G_CHECK(qsrc.ensure(sizeof(int) * h_qsrc.size()));
    PBI4G_CHECK(qmap.ensure(sizeof(int) * h_qmap.size()));
    PBI4G_CHECK(slots.ensure(sizeof(int) * h_slots.size()));
    PBI4G_CHECK(pexp.ensure(sizeof(int) * h_psrc.size()));
    PBI4G_CHECK(qexp.ensure(sizeof(int) * h_qsrc.size()));
    PBI4G_CHECK(err.ensure(sizeof(int)));
    PBI4G_CUDA(cudaMemcpy(units.p, h_units.data(), sizeof(int4) * nunits, cudaMemcpyHostToDevice));
    PBI4G_CUDA(cudaMemcpy(umaps.p, h_umaps.data(), sizeof(int) * h_umaps.size(), cudaMemcpyHostToDevice));
    PBI4G_CUDA(cudaMemcpy(psrc.p, h_psrc.data(), sizeof(int2) * h_psrc.size(), cudaMemcpyHostToDevice));
    PBI4G_CUDA(cudaMemcpy(pmap.p, h_pmap.data(), sizeof(int2) * h_pmap.size(), cudaMemcpyHostToDevice));
    PBI4G_CUDA(cudaMemcpy(qsrc.p, h_qsrc.data(), sizeof(int) * h_qsrc.size(), cudaMemcpyHostToDevice));
    PBI4G_CUDA(cudaMemcpy(qmap.p, h_qmap.data(), sizeof(int) * h_qmap.size(), cudaMemcpyHostToDevice));
    PBI4G_CUDA(cudaMemcpy(slots.p, h_slots.data(), sizeof(int) * h_slots.size(), cudaMemcpyHostToDevice));
    return PBI4G_OK;
}

size_t tc_smem_bytes(int umax) {
    return 1024 + 2 * (size_t)kStageBytes + sizeof(float) * (2 * (size_t)umax * kStageRow + kMT * kBM + kBN) +
           sizeof(int2) * kMT * kBM + sizeof(int) * (kBN + umax) + sizeof(float) * umax + 64;
}

int triangle_sums_tc(const Shells &sh, TcPlan &tp, bool split, const float *maps, size_t mstride, int rs,
                     const double *powsum, int pow_mask, const double lfac[3], DevBuf &mexp, DevBuf &partial, double *S,
                     cudaStream_t st, int64_t *launches) {
    const int N = sh.Nm;  // maps live on the map grid
    const long long K = (long long)N * N * N;
    if (K % kKC || (rs & 1) || (mstride & 1))
        return set_error(PBI4G_ERR_UNSUPPORTED, "tensor-core triangle sums need grid^3 %% 64 == 0 (grid %d)", N);
    const int nmaps = tp.nsets * sh.nb;
    PBI4G_CHECK(mexp.ensure(sizeof(int) * nmaps));
    map_exponents_kernel<<<1, 256, 0, st>>>(nmaps, sh.nb, powsum, pow_mask, lfac[1], lfac[2],
                                            sh.nmodes_d.as<double>(), mexp.as<int>());
    PBI4G_LAUNCH_CHECK();
    unit_exponents_kernel<<<grid_blocks((size_t)tp.nunits * kMT * kBM, 256), 256, 0, st>>>(
        tp.nunits, mexp.as<int>(), tp.pmap.as<int2>(), tp.qmap.as<int>(), tp.pexp.as<int>(), tp.qexp.as<int>());
    PBI4G_LAUNCH_CHECK();
    const long long nchunks = K / kKC;
    int ksplit = std::max(1, (152 + tp.nunits - 1) / tp.nunits);
    ksplit = (int)std::min<long long>(ksplit, std::max<long long>(1, nchunks / 8));
    PBI4G_CHECK(partial.ensure(sizeof(double) * (size_t)ksplit * tp.nslots));
    PBI4G_CUDA(cudaMemsetAsync(tp.err.p, 0, sizeof(int), st));
    TcArgs a;
    a.maps = maps; a.mstride = mstride; a.rs = rs; a.N = N; a.umax = tp.umax; a.K = K;
    a.nunits = tp.nunits; a.ksplit = ksplit; a.nslots = tp.nslots;
    a.units = tp.units.as<int4>(); a.umaps = tp.umaps.as<int>(); a.psrc = tp.psrc.as<int2>();
    a.qsrc = tp.qsrc.as<int>(); a.pexp = tp.pexp.as<int>(); a.qexp = tp.qexp.as<int>();
    a.slots = tp.slots.as<int>(); a.partial = partial.as<double>(); a.err = tp.err.as<int>();
    a.mexp = mexp.as<int>();
    const size_t smem = tc_smem_bytes(tp.umax);
    if (smem > 227 * 1024) return set_error(PBI4G_ERR_UNSUPPORTED, "tensor-core triangle sums: %zu B smem", smem);
    if (split) {
        PBI4G_CUDA(cudaFuncSetAttribute(trisum_tc_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        trisum_tc_kernel<true><<<tp.nunits * ksplit, kThreads, smem, st>>>(a);
    } else {
        PBI4G_CUDA(cudaFuncSetAttribute(trisum_tc_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        trisum_tc_kernel<false><<<tp.nunits * ksplit, kThreads, smem, st>>>(a);
    }
    PBI4G_LAUNCH_CHECK();
    PBI4G_CHECK(reduce_partials(tp.nslots, ksplit, partial.as<double>(), S, st));
    *launches += 4;
    return PBI4G_OK;
}

int tc_check_error(TcPlan &tp, cudaStream_t st) {
    int h = 0;
    PBI4G_CUDA(cudaMemcpyAsync(&h, tp.err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    PBI4G_CUDA(cudaStreamSynchronize(st));
    if (h) return set_error(PBI4G_ERR_TIMEOUT, "tensor-core triangle sums: a bounded wait gave up");
    return PBI4G_OK;
}

}  // namespace pbi4g
