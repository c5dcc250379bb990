// assign_owner.cu -- mass assignment for the FP32 / mixed estimator plan:
// owner-computes 16^3 tiles, 64-bit fixed-point accumulation in shared memory,
// FP32 grids written with plain stores.
//
// Same indices and weights as powerI4.f90:68-249 (see assign.cu); the weights
// are evaluated in FP32 from the FP64 cell offset.  Every contribution
// (w_x w_y) w_z weight is rounded once to an integer at scale 2^S (|q| < 2^30,
// 2^-28 resolution for unit weights: far below the FP32 grid's rounding) and
// summed into 64-bit integers with shared-memory atomics, so the grid is
// bit-identical for any particle order and schedule.
//
// 1. prep: per particle, the first stencil cell of each grid (FP64 index math,
//    once) and the FP32 offsets; the tiles its stencils touch (1 to 8) are
//    counted.
// 2. counting sort: one 32-byte record per (particle, touched tile).
// 3. one CTA per tile, one warp per record: the lanes take distinct stencil
//    cells of the record's particle (no two lanes of a warp add to the same
//    cell), keep those inside the tile and add them into the tile's shared
//    accumulator; the tile is then converted to FP32 and stored.  No global
//    atomics, no int64 grid, no memset of the grids.
#include "assign_owner.cuh"

#include <math.h>
#include <string.h>

#include <algorithm>

namespace pbi4g {

namespace {

constexpr int kT = 16;                  // tile edge
constexpr int kTC = kT * kT * kT;       // 4096 cells
// padded shared layout of a tile's 64-bit sums: cell (x, y, z) at z * kPz + y * kPy + x.
// A stencil step's lanes are (i, j, l) in [0,4) x [0,4) x [0,2), l = lane / 16; a 64-bit
// access takes the bank pair 2 (i + 20 j + 16 l) = 2 i + 8 j (mod 32), so each half-warp
// (one wavefront of 8-byte accesses) touches 16 distinct pairs.
constexpr int kPy = 20, kPz = 336;
constexpr int kTCP = kT * kPz;          // 5376 cells per tile array
constexpr int kThreads = 512;

struct alignas(16) PRec {               // one particle, both grids (32 bytes)
    unsigned int f[2];                  // first cell x | y << 11 | z << 22 per grid
    float h[2][3];                      // cell offset per grid and axis
};

// One particle's stencil on one grid, relative to one tile (16 bytes): pack =
// base + kBias | x mask << 13 | y mask << 17 | z mask << 21, with base the
// padded offset (z kPz + y kPy + x) of the stencil's first cell from the tile
// origin and bit i of an axis mask set when the stencil's cell i on that axis
// lies inside the tile (pack 0: no cell inside).  The scatter writes them, so
// the tile kernel's lanes test one bit pattern and add one offset per cell.
struct alignas(16) PCell {
    int pack;
    float h[3];
};
struct alignas(16) PTile {              // a sorted record (particle, tile), both grids (32 bytes)
    PCell g[2];
};
// The buffers of an OwnerWork as the kernels see them.  Direct launches take
// them by value; the captured form (IND) reads them from the plan's device block
// (owner_ptrs_host), so its graphs follow the plan to another OwnerWork.  Read
// through the block the tile kernel measured 3% slower at 256^3, which is why
// the direct launches keep the kernel parameters.
struct OwnerPtrs {
    unsigned int *count, *start, *cursor;  // count: [ntiles + 2], the last two the tile counter
    PRec *rec;
    PTile *sorted;
    float *wsorted;
};
static_assert(sizeof(OwnerPtrs) <= kOwnerPtrBytes, "owner pointer block");
constexpr int kBias = 2048;             // a stencil with a cell inside starts at [-3, 15] per axis: base + kBias in [977, 7403]
constexpr int kMX = 13, kMY = 17, kMZ = 21;

__device__ __forceinline__ unsigned int pack3(int x, int y, int z) {
    return (unsigned)x | ((unsigned)y << 11) | ((unsigned)z << 22);
}

// first cell (0-based, in [0,N)) and the offset h that sets the weights
// t mod N for the cell indices: t is in [-2, 2N) for positions in [0, 1]
// (two compares), any other t takes the division
__device__ __forceinline__ int wrap_cell(long long t, int N) {
    if (t >= 0 && t < 2LL * N) return (int)(t >= N ? t - N : t);
    return (int)(t % N);
}

__device__ __forceinline__ void first_and_h(double p, int N, int nintp, bool shifted, bool cic_nint, int &f, float &h) {
    double v = __dadd_rn(__dmul_rn((double)N, p), 1.0);  // two roundings, as in assign.cu
    if (shifted) v = v - 0.5;
    long long iv;
    double hh;
    if (nintp == 4) { iv = (long long)v; f = wrap_cell(iv - 2, N); hh = v - (double)iv; }
    else if (nintp == 3) { iv = llround(v); f = wrap_cell(iv - 2, N); hh = v - (double)iv; }
    else if (nintp == 2) { iv = (long long)v; f = wrap_cell(iv, N); hh = cic_nint ? v - (double)llround(v) : v - (double)iv; }
    else { iv = llround(v); f = wrap_cell(iv - 1, N); hh = 0.0; }
    if (f < 0) f += N;
    if (f < 0 || f >= N) f = 0;
    h = (float)hh;
}

// Weight i of the per-axis stencil at offset h as a cubic in h,
// w_i(h) = c0 + h (c1 + h (c2 + h c3)): the reference's polynomials
// (powerI4.f90) expanded, e.g. PCS w0 = (1-h)^3/6, w1 = 4/6 + (h/2 - 1) h^2,
// w3 = h^3/6 and w2 = 1 - w0 - w1 - w3; TSC w0 = (1/2 - h)^2 / 2, w1 = 3/4 - h^2,
// w2 = 1 - w0 - w1; CIC 1 - h, h.  Each lane's stencil indices are fixed, so it
// picks its coefficients once and evaluates three FMAs per weight.
template <int NI>
__device__ __forceinline__ float4 axis_poly(int i) {
    if constexpr (NI == 4) {
        return i == 0 ? make_float4(1.f / 6.f, -0.5f, 0.5f, -1.f / 6.f)
             : i == 1 ? make_float4(2.f / 3.f, 0.f, -1.f, 0.5f)
             : i == 2 ? make_float4(1.f / 6.f, 0.5f, 0.5f, -0.5f)
                      : make_float4(0.f, 0.f, 0.f, 1.f / 6.f);
    } else if constexpr (NI == 3) {
        return i == 0 ? make_float4(0.125f, -0.5f, 0.5f, 0.f)
             : i == 1 ? make_float4(0.75f, 0.f, -1.f, 0.f)
                      : make_float4(0.125f, 0.5f, 0.5f, 0.f);
    } else if constexpr (NI == 2) {
        return i == 0 ? make_float4(1.f, -1.f, 0.f, 0.f) : make_float4(0.f, 1.f, 0.f, 0.f);
    } else {
        return make_float4(1.f, 0.f, 0.f, 0.f);
    }
}

__device__ __forceinline__ float horner(float4 c, float h) { return fmaf(h, fmaf(h, fmaf(h, c.w, c.z), c.y), c.x); }

// offset of a stencil's first cell from the tile origin, with the stencils that
// wrap past the upper grid edge into tile 0 shifted down by N: the lanes'
// cells are then d + c, inside the tile iff 0 <= d + c < 16 (N >= 32)
__device__ __forceinline__ int tile_offset(int f, int o, int N) {
    const int d = f - o;
    return d >= N - 4 ? d - N : d;
}

// tiles touched along one axis by a stencil of width w starting at cell lo (mod N)
__device__ __forceinline__ int axis_tiles(int lo, int w, int N, int nt, int t[2]) {
    t[0] = lo / kT;
    int hi = lo + w - 1;
    hi -= (hi >= N) ? N : 0;
    t[1] = hi / kT;
    return t[1] == t[0] ? 1 : 2;
}

// first_and_h for both grids from one FP64 product and sum, v = N p + 1 (the
// reference's two roundings; FP64 is a slow pipe on this part).  The shifted
// grid's v - 1/2 is exact, and floor(v), v - floor(v) and its half-cell
// variants are read from v's bits as integers, exactly; each offset then takes
// the single FP32 rounding first_and_h gives it, so cells and offsets are
// bit-identical to it.  v outside [1, 2^20) (positions outside [0, 1]) takes
// first_and_h.
__device__ __forceinline__ void first_cells(double p, int N, int nintp, bool interlaced, int &f0, float &h0, int &f1,
                                            float &h1) {
    const double v = __dadd_rn(__dmul_rn((double)N, p), 1.0);  // two roundings, as in assign.cu
    if (!(v >= 1.0 && v < 1048576.0)) {
        first_and_h(p, N, nintp, false, !interlaced, f0, h0);
        if (interlaced) first_and_h(p, N, nintp, true, false, f1, h1);
        else { f1 = f0; h1 = 0.f; }
        return;
    }
    const long long bits = __double_as_longlong(v);
    const int sh = 52 - ((int)(bits >> 52) - 1023);  // fraction bits of v: 33..52
    const long long mant = (bits & 0xFFFFFFFFFFFFFLL) | (1LL << 52);
    const long long one = 1LL << sh, half = one >> 1;
    const int iv = (int)(mant >> sh);                 // floor(v)
    const long long fr = mant & (one - 1);            // (v - floor(v)) 2^sh
    const bool up = fr >= half;                       // v - floor(v) >= 1/2
    const float scale = __int_as_float((127 - sh) << 23);  // 2^-sh
    auto off = [&](long long x) { return __ll2float_rn(x) * scale; };
    auto cell = [&](int t) {
        int f = wrap_cell(t, N);
        if (f < 0) f += N;
        return (f < 0 || f >= N) ? 0 : f;
    };
    const int ivs = up ? iv : iv - 1;                 // floor(v - 1/2)
    const long long frs = up ? fr - half : fr + half;  // (v - 1/2 - floor(v - 1/2)) 2^sh
    if (nintp == 4) {
        f0 = cell(iv - 2); h0 = off(fr);
        f1 = cell(ivs - 2); h1 = off(frs);
    } else if (nintp == 3) {
        // nint(v) = floor(v) + up; nint(v - 1/2) = floor(v)
        f0 = cell(iv + (up ? 1 : 0) - 2); h0 = off(up ? fr - one : fr);
        f1 = cell(iv - 2); h1 = off(fr - half);
    } else if (nintp == 2) {
        f0 = cell(iv); h0 = off((!interlaced && up) ? fr - one : fr);
        f1 = cell(ivs); h1 = off(frs);
    } else {
        f0 = cell(iv + (up ? 1 : 0) - 1); h0 = 0.f;
        f1 = cell(iv - 1); h1 = 0.f;
    }
    if (!interlaced) { f1 = f0; h1 = 0.f; }
}

__device__ __forceinline__ PRec make_rec(const double *__restrict__ pos, int64_t stride, int64_t i, int N, int nintp,
                                         int interlaced, int lo[3]) {
    PRec r;
    int f[2][3];
    for (int c = 0; c < 3; c++) {
        const double p = pos[(size_t)c * stride + i];
        first_cells(p, N, nintp, interlaced != 0, f[0][c], r.h[0][c], f[1][c], r.h[1][c]);
        // the shifted grid starts at the same cell or one below (circularly)
        lo[c] = (interlaced && f[1][c] == (f[0][c] == 0 ? N - 1 : f[0][c] - 1)) ? f[1][c] : f[0][c];
    }
    r.f[0] = pack3(f[0][0], f[0][1], f[0][2]);
    r.f[1] = pack3(f[1][0], f[1][1], f[1][2]);
    return r;
}

// Tile of stencil slot s (steps a = s & 1 in x, b = s >> 1 & 1 in y, c = s >> 2 in z)
// of a particle whose stencil spans nx x ny x nz tiles; -1 when it has no such slot.
__device__ __forceinline__ int slot_tile(int s, const int tx[2], const int ty[2], const int tz[2], int nx, int ny,
                                         int nz, int nt) {
    const int a = s & 1, b = (s >> 1) & 1, c = s >> 2;
    if (a >= nx || b >= ny || c >= nz) return -1;
    return (tz[c] * nt + ty[b]) * nt + tx[a];
}

template <bool IND>
__global__ void owner_count_kernel(int N, int nintp, int interlaced, int64_t npart, int64_t stride,
                                   const BoxPar *__restrict__ bp, const double *__restrict__ pos_arg, int nt,
                                   const OwnerPtrs ov, const OwnerPtrs *__restrict__ op) {
    // the captured form reads the box's position slot from its BoxPar
    const double *__restrict__ pos = (IND && bp) ? bp->pos : pos_arg;
    PRec *__restrict__ rec = IND ? op->rec : ov.rec;
    unsigned int *__restrict__ count = IND ? op->count : ov.count;
    const int w = nintp + (interlaced ? 1 : 0);  // cells spanned from the lowest first cell
    const int64_t n = bp ? bp->npart : npart;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int lo[3];
        const PRec r = make_rec(pos, stride, i, N, nintp, interlaced, lo);
        rec[i] = r;
        int tx[2], ty[2], tz[2];
        const int nx = axis_tiles(lo[0], w, N, nt, tx), ny = axis_tiles(lo[1], w, N, nt, ty),
                  nz = axis_tiles(lo[2], w, N, nt, tz);
        // slot by slot, one atomic per distinct tile of the warp (neighbouring
        // particles of a catalogue share their tiles and their tile crossings)
        const unsigned act = __activemask();
        const int lane = (int)(threadIdx.x & 31);
#pragma unroll
        for (int sl = 0; sl < 8; sl++) {
            const int t = slot_tile(sl, tx, ty, tz, nx, ny, nz, nt);
            if (!__any_sync(act, t >= 0)) continue;
            const unsigned same = __match_any_sync(act, t);
            if (t >= 0 && lane == __ffs(same) - 1) atomicAdd(count + t, (unsigned)__popc(same));
        }
    }
}

template <bool IND>
__global__ void owner_scan_kernel(int ntiles, const OwnerPtrs ov, const OwnerPtrs *__restrict__ op) {
    const unsigned int *__restrict__ count = IND ? op->count : ov.count;
    unsigned int *__restrict__ start = IND ? op->start : ov.start, *__restrict__ cursor = IND ? op->cursor : ov.cursor;
    __shared__ unsigned int warp_tot[32];
    __shared__ unsigned int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int base = 0; base < ntiles; base += blockDim.x) {
        const int i = base + threadIdx.x;
        const unsigned v = i < ntiles ? count[i] : 0u;
        unsigned x = v;
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_tot[wid] = x;
        __syncthreads();
        if (wid == 0) {
            unsigned t = lane < (int)(blockDim.x >> 5) ? warp_tot[lane] : 0u;
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned y = __shfl_up_sync(0xffffffffu, t, o);
                if (lane >= o) t += y;
            }
            warp_tot[lane] = t;
        }
        __syncthreads();
        const unsigned excl = carry + x - v + (wid ? warp_tot[wid - 1] : 0u);
        if (i < ntiles) { start[i] = excl; cursor[i] = excl; }
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry = excl + v;
        __syncthreads();
    }
    if (threadIdx.x == 0) start[ntiles] = carry;
}

// Offset d of a stencil's first cell from a tile origin on one axis (tile_offset)
// and the mask of its NI cells d .. d + NI - 1 that fall inside the tile.
__device__ __forceinline__ unsigned axis_mask(int d, int NI) {
    const int lo = max(0, -d), hi = min(NI - 1, kT - 1 - d);
    return lo <= hi ? ((2u << hi) - 1u) & ~((1u << lo) - 1u) : 0u;
}

__device__ __forceinline__ int cell_pack(unsigned f, int ox, int oy, int oz, int N, int NI) {
    const int dx = tile_offset((int)(f & 2047), ox, N), dy = tile_offset((int)((f >> 11) & 2047), oy, N);
    const int dz = tile_offset((int)(f >> 22), oz, N);
    const unsigned mx = axis_mask(dx, NI), my = axis_mask(dy, NI), mz = axis_mask(dz, NI);
    if (!mx || !my || !mz) return 0;
    return (dz * kPz + dy * kPy + dx + kBias) | (int)(mx << kMX | my << kMY | mz << kMZ);
}

template <bool IND>
__global__ void owner_scatter_kernel(int N, int nintp, int interlaced, int64_t npart, const BoxPar *__restrict__ bp,
                                     int nt, const OwnerPtrs ov, const OwnerPtrs *__restrict__ op,
                                     const double *__restrict__ weight) {
    const PRec *__restrict__ rec = IND ? op->rec : ov.rec;
    unsigned int *__restrict__ cursor = IND ? op->cursor : ov.cursor;
    PTile *__restrict__ sorted = IND ? op->sorted : ov.sorted;
    float *__restrict__ wsorted = weight ? (IND ? op->wsorted : ov.wsorted) : nullptr;
    const int w = nintp + (interlaced ? 1 : 0);
    const int64_t n = bp ? bp->npart : npart;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const PRec r = rec[i];
        int lo[3];
        for (int c = 0; c < 3; c++) {
            const unsigned f0 = (r.f[0] >> (11 * c)) & 2047, f1 = (r.f[1] >> (11 * c)) & 2047;
            lo[c] = (interlaced && (int)f1 == ((int)f0 == 0 ? N - 1 : (int)f0 - 1)) ? (int)f1 : (int)f0;
        }
        int tx[2], ty[2], tz[2];
        const int nx = axis_tiles(lo[0], w, N, nt, tx), ny = axis_tiles(lo[1], w, N, nt, ty),
                  nz = axis_tiles(lo[2], w, N, nt, tz);
        const float wt = weight ? (float)weight[i] : 1.f;
        // slot by slot (as owner_count_kernel counts them): one atomic per distinct
        // tile of the warp, the lanes that share it take consecutive places in lane order
        const unsigned act = __activemask();
        const int lane = (int)(threadIdx.x & 31);
#pragma unroll
        for (int sl = 0; sl < 8; sl++) {
            const int t = slot_tile(sl, tx, ty, tz, nx, ny, nz, nt);
            if (!__any_sync(act, t >= 0)) continue;
            const unsigned same = __match_any_sync(act, t);
            const int lead = __ffs(same) - 1;
            unsigned d = 0;
            if (t >= 0 && lane == lead) d = atomicAdd(cursor + t, (unsigned)__popc(same));
            d = __shfl_sync(same, d, lead) + (unsigned)__popc(same & ((1u << lane) - 1u));
            if (t >= 0) {
                const int ox = tx[sl & 1] * kT, oy = ty[(sl >> 1) & 1] * kT, oz = tz[sl >> 2] * kT;
                PTile o;
#pragma unroll
                for (int g = 0; g < 2; g++) {
                    o.g[g].pack = (g == 0 || interlaced) ? cell_pack(r.f[g], ox, oy, oz, N, nintp) : 0;
                    o.g[g].h[0] = r.h[g][0];
                    o.g[g].h[1] = r.h[g][1];
                    o.g[g].h[2] = r.h[g][2];
                }
                sorted[d] = o;
                if (wsorted) wsorted[d] = wt;
            }
        }
    }
}

// PCS records in columns: a half-warp takes one (particle, grid) pair of a
// record, lane (j, i) = (l >> 2 & 3, l & 3) of it the z column of cells
// (i, j, 0..3).  The x and y weights and their product are formed once per
// column, the z weights per cell, in the same order as the cell mapping,
// ((w_x w_y) w_z) weight, so every q is the same integer.  Two grids: the
// halves take grids 0 and 1 of one record; one grid: two records.  Each
// half-warp's 16 cells of a z step fall on 16 distinct bank pairs (2 i + 8 j).
// Read-only loads of the sorted records (their pointers come from the pointer
// block, so the compiler cannot infer that the kernel never writes them).
__device__ __forceinline__ PCell ld_cell(const PCell *p) {
    const int4 v = __ldg(reinterpret_cast<const int4 *>(p));
    PCell c;
    c.pack = v.x;
    c.h[0] = __int_as_float(v.y);
    c.h[1] = __int_as_float(v.z);
    c.h[2] = __int_as_float(v.w);
    return c;
}
__device__ __forceinline__ PTile ld_tile(const PTile *p) {
    PTile t;
    t.g[0] = ld_cell(&p->g[0]);
    t.g[1] = ld_cell(&p->g[1]);
    return t;
}

template <int G, bool W>
__device__ __forceinline__ void pcs_columns(unsigned b, unsigned e, int warp, int nwarps, int lane, float scale,
                                            const PTile *__restrict__ sorted, const float *__restrict__ wsorted,
                                            unsigned long long *acc64) {
    const int half = lane >> 4, ci = lane & 3, cj = (lane >> 2) & 3;
    const int g = G == 2 ? half : 0;
    const float4 px = axis_poly<4>(ci), py = axis_poly<4>(cj);
    float4 pz[4];
#pragma unroll
    for (int l = 0; l < 4; l++) {
        const float4 zc = axis_poly<4>(l);
        pz[l] = make_float4(zc.x * scale, zc.y * scale, zc.z * scale, zc.w * scale);
    }
    const int need = (1 << (kMX + ci)) | (1 << (kMY + cj));  // the column's x and y cells
    const int loff = g * kTCP + cj * kPy + ci - kBias;  // the column's cell offset less the bias
    constexpr int RPW = G == 2 ? 1 : 2;  // records per warp step
    const unsigned step = (unsigned)(RPW * nwarps), off = G == 2 ? 0u : (unsigned)half;
    // the next record of the half-warp is loaded while this one is added
    PCell cn = {};
    float wn = 1.f;
    if (b + (unsigned)(RPW * warp) + off < e) {
        cn = ld_cell(&sorted[b + (unsigned)(RPW * warp) + off].g[g]);
        if (W) wn = __ldg(&wsorted[b + (unsigned)(RPW * warp) + off]);
    }
    for (unsigned k = b + (unsigned)(RPW * warp) + off; k - off < e; k += step) {
        const PCell c = cn;
        const float wt = wn;
        if (k + step < e) {
            cn = ld_cell(&sorted[k + step].g[g]);
            if (W) wn = __ldg(&wsorted[k + step]);
        }
        // k >= e (the second record of a one-grid step past the end): pack 0
        const int pk = k < e ? c.pack : 0;
        const bool okxy = (pk & need) == need;
        const float wxy = horner(px, c.h[0]) * horner(py, c.h[1]);
        unsigned long long *col = acc64 + (loff + (pk & ((1 << kMX) - 1)));
#pragma unroll
        for (int l = 0; l < 4; l++) {
            float wv = wxy * horner(pz[l], c.h[2]);
            if (W) wv *= wt;
            const int q = __float2int_rn(wv);
            if (okxy && (pk >> (kMZ + l) & 1)) atomicAdd(col + l * kPz, (unsigned long long)(long long)q);
        }
    }
}

// Tile kernel, specialised on the stencil width NI (1..4), the number of
// grids G (2 when interlaced) and the presence of particle weights W: below
// PCS a warp takes one record (particle, tile) and its lanes take the
// G * NI^3 (grid, cell) pairs, so the cell indices and the weight polynomials
// fold to constants and shifts; PCS takes the column mapping above.  The
// fixed-point scale 2^S rides in the z polynomial (a power of two: the
// products are the same bits as scaling at the end).
template <int NI, int G, bool W, bool IND>
__global__ void __launch_bounds__(kThreads, 2) owner_tile_kernel(int N, int nt, const OwnerPtrs ov,
                                                               const OwnerPtrs *__restrict__ op, float scale,
                                                               float inv_scale, float *__restrict__ out1,
                                                               float *__restrict__ out2) {
    constexpr int NC = NI * NI * NI;
    extern __shared__ unsigned long long acc64[];  // [G][kTCP]
    const int ntiles = nt * nt * nt;
    const unsigned int *__restrict__ start = IND ? op->start : ov.start;
    const PTile *__restrict__ sorted = IND ? op->sorted : ov.sorted;
    const float *__restrict__ wsorted = W ? (IND ? op->wsorted : ov.wsorted) : nullptr;
    unsigned int *next_tile = (IND ? op->count : ov.count) + ntiles + 1;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    __shared__ int s_tile;
    // tiles are handed out dynamically (their particle loads differ by orders of
    // magnitude in clustered boxes); the counter is zeroed before the launch
    for (;;) {
        if (threadIdx.x == 0) s_tile = (int)atomicAdd(next_tile, 1u);
        __syncthreads();
        const int tile = s_tile;
        if (tile >= ntiles) break;
        const int tx = tile % nt, ty = (tile / nt) % nt, tz = tile / (nt * nt);
        const int ox = tx * kT, oy = ty * kT, oz = tz * kT;
        for (int c = threadIdx.x; c < G * kTCP; c += blockDim.x) acc64[c] = 0ull;
        __syncthreads();
        const unsigned b = __ldg(&start[tile]), e = __ldg(&start[tile + 1]);
        if constexpr (NI == 4) {
            pcs_columns<G, W>(b, e, warp, nwarps, lane, scale, sorted, wsorted, acc64);
        } else {
            // per-lane stencil cells of one grid: NIT steps of 32 cells; the (i, j, l)
            // of a lane, its cell offset, its bit pattern and its weight polynomials
            // are the same for every record
            constexpr int NIT = (NC + 31) / 32;
            int need[NIT], loff[NIT];
            float4 px[NIT], py[NIT], pz[NIT];
#pragma unroll
            for (int it = 0; it < NIT; it++) {
                const int c = it * 32 + lane;
                const int ci = c % NI, cj = (c / NI) % NI, cl = c < NC ? c / (NI * NI) : 0;
                // no cell for this lane at this step: a bit no pack has
                need[it] = c < NC ? (1 << (kMX + ci)) | (1 << (kMY + cj)) | (1 << (kMZ + cl)) : (1 << 30);
                loff[it] = cl * kPz + cj * kPy + ci - kBias;
                px[it] = axis_poly<NI>(ci);
                py[it] = axis_poly<NI>(cj);
                const float4 zc = axis_poly<NI>(cl);
                pz[it] = make_float4(zc.x * scale, zc.y * scale, zc.z * scale, zc.w * scale);
            }
            // the next record of the warp is loaded while this one is added
            PTile rn;
            float wn = 1.f;
            if (b + warp < e) {
                rn = ld_tile(&sorted[b + warp]);
                if (W) wn = __ldg(&wsorted[b + warp]);
            }
            for (unsigned k = b + warp; k < e; k += nwarps) {
                const PTile r = rn;
                const float wt = wn;
                if (k + nwarps < e) {
                    rn = ld_tile(&sorted[k + nwarps]);
                    if (W) wn = __ldg(&wsorted[k + nwarps]);
                }
                int cell[G][NIT];
                int q[G][NIT];
                bool ok[G][NIT];
#pragma unroll
                for (int g = 0; g < G; g++) {
                    const int pk = r.g[g].pack;
                    const float hx = r.g[g].h[0], hy = r.g[g].h[1], hz = r.g[g].h[2];
#pragma unroll
                    for (int it = 0; it < NIT; it++) {
                        ok[g][it] = (pk & need[it]) == need[it];
                        // the reference's product order: ((w_x w_y) w_z) weight; wv * 2^S is exact in
                        // FP32 (a power-of-two scale) and |wv| 2^S < 2^30, so q is one 32-bit integer
                        float wv = horner(px[it], hx) * horner(py[it], hy) * horner(pz[it], hz);
                        if (W) wv *= wt;
                        q[g][it] = __float2int_rn(wv);
                        cell[g][it] = (pk & ((1 << kMX) - 1)) + loff[it];
                    }
                }
                // 64-bit fixed-point adds of the sign-extended q (exact mod 2^64)
#pragma unroll
                for (int g = 0; g < G; g++)
#pragma unroll
                    for (int it = 0; it < NIT; it++)
                        if (ok[g][it])
                            atomicAdd(acc64 + g * kTCP + cell[g][it], (unsigned long long)(long long)q[g][it]);
            }
        }
        __syncthreads();
        for (int c = threadIdx.x; c < G * kTC; c += blockDim.x) {
            const int g = c / kTC, cc = c % kTC;
            const int x = cc % kT, y = (cc / kT) % kT, z = cc / (kT * kT);
            const int pc = z * kPz + y * kPy + x;
            const long long v = (long long)acc64[g * kTCP + pc];
            float *out = g ? out2 : out1;
            out[((size_t)(oz + z) * N + (oy + y)) * N + (ox + x)] = (float)v * inv_scale;
        }
        __syncthreads();
    }
}

template <int NI, int G, bool W, bool IND>
static int launch_tile_w(int N, int nt, const OwnerPtrs &ov, const OwnerPtrs *op, int bits, float *out1, float *out2,
                         cudaStream_t st) {
    const size_t smem = sizeof(unsigned long long) * G * kTCP;
    auto kern = owner_tile_kernel<NI, G, W, IND>;
    PBI4G_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int ntiles = nt * nt * nt;
    int per_sm = 0;
    PBI4G_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, smem));
    const int grid = std::min(ntiles, 152 * std::max(1, per_sm));
    kern<<<grid, kThreads, smem, st>>>(N, nt, ov, op, ldexpf(1.0f, bits), ldexpf(1.0f, -bits), out1, out2);
    PBI4G_LAUNCH_CHECK();
    return PBI4G_OK;
}

template <int NI, int G>
static int launch_tile(int N, int nt, const OwnerPtrs &ov, const OwnerPtrs *op, bool weighted, int bits, float *out1,
                       float *out2, cudaStream_t st) {
    // the captured form takes no weights
    if (op) return launch_tile_w<NI, G, false, true>(N, nt, ov, op, bits, out1, out2, st);
    return weighted ? launch_tile_w<NI, G, true, false>(N, nt, ov, op, bits, out1, out2, st)
                    : launch_tile_w<NI, G, false, false>(N, nt, ov, op, bits, out1, out2, st);
}

// zero the tile counts and the tile counter (through the pointer block)
__global__ void owner_zero_kernel(const OwnerPtrs *__restrict__ op, int n) {  // the captured form
    unsigned int *count = op->count;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) count[i] = 0u;
}

__global__ void owner_wmax_kernel(int64_t n, const double *__restrict__ w, unsigned long long *__restrict__ out) {
    double m = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double a = fabs(w[i]);
        if (!(a <= 1e300)) a = 1e308;
        m = fmax(m, a);
    }
    for (int o = 16; o; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(m));
}

}  // namespace

bool owner_supported(int N) { return N % kT == 0 && N >= 2 * kT && N <= 2048; }

bool OwnerWork::fits(int N, int64_t npart) const {
    const int nt = N / kT;
    const size_t ntiles = (size_t)nt * nt * nt;
    const size_t n = (size_t)(npart > 0 ? npart : 1);
    return count.p && count.bytes >= (ntiles + 2) * 4 && start.bytes >= (ntiles + 1) * 4 &&
           cursor.bytes >= (ntiles + 1) * 4 && rec.bytes >= n * sizeof(PRec) && sorted.bytes >= 8 * n * sizeof(PTile) &&
           wsorted.bytes >= 8 * n * 4 && wmax.bytes >= 8;
}

int OwnerWork::ensure(int N, int64_t npart) {
    if (fixed) {
        if (fits(N, npart)) return PBI4G_OK;
        return set_error(PBI4G_ERR_RANGE, "shared assignment scratch too small for grid %d, %lld particles", N,
                         (long long)npart);
    }
    const int nt = N / kT;
    const size_t ntiles = (size_t)nt * nt * nt;
    const size_t n = (size_t)(npart > 0 ? npart : 1);
    PBI4G_CHECK(count.ensure((ntiles + 2) * 4));  // + the tile kernel's work counter
    PBI4G_CHECK(start.ensure((ntiles + 1) * 4));
    PBI4G_CHECK(cursor.ensure((ntiles + 1) * 4));
    PBI4G_CHECK(rec.ensure(n * sizeof(PRec)));
    // a record per (particle, touched tile): at most 8 per particle
    PBI4G_CHECK(sorted.ensure(8 * n * sizeof(PTile)));
    PBI4G_CHECK(wsorted.ensure(8 * n * 4));
    PBI4G_CHECK(wmax.ensure(8));
    return PBI4G_OK;
}

void OwnerWork::release() {
    for (DevBuf *b : {&count, &start, &cursor, &key, &rec, &sorted, &wsorted, &wmax}) b->release();
}

size_t OwnerWork::footprint(int N, int64_t npart) {
    const size_t nt = (size_t)(N / kT);
    return 3 * (nt * nt * nt + 2) * 4 + (size_t)npart * (sizeof(PRec) + 8 * (sizeof(PTile) + 4)) + 64;
}

void owner_ptrs_host(const OwnerWork &wk, unsigned char (&block)[kOwnerPtrBytes]) {
    OwnerPtrs o;
    o.count = wk.count.as<unsigned int>();
    o.start = wk.start.as<unsigned int>();
    o.cursor = wk.cursor.as<unsigned int>();
    o.rec = static_cast<PRec *>(wk.rec.p);
    o.sorted = static_cast<PTile *>(wk.sorted.p);
    o.wsorted = wk.wsorted.as<float>();
    memset(block, 0, kOwnerPtrBytes);
    memcpy(block, &o, sizeof(o));
}

int assign_owner(OwnerWork &wk, const void *d_ptrs, int N, int nintp, bool interlaced, int64_t npart,
                 const double *d_pos, const double *d_weight, float *out, cudaStream_t st, int64_t *launches,
                 int64_t stride, const BoxPar *bp, Prof *prof, int tile_stage, int sort_stage) {
    Prof none;
    Prof &pf = prof ? *prof : none;
    if (stride <= 0) stride = npart;
    if (!owner_supported(N)) return set_error(PBI4G_ERR_UNSUPPORTED, "owner assignment needs grid %% 16 == 0");
    if (nintp < 1 || nintp > 4 || npart < 1 || !d_pos || !d_ptrs)
        return set_error(PBI4G_ERR_INVALID, "assign: nintp=%d npart=%lld", nintp, (long long)npart);
    if (npart >= (int64_t)0x1fffffffLL) return set_error(PBI4G_ERR_RANGE, "assign: npart >= 2^29");
    // the caller has sized wk (and, for the captured form, written its pointers to d_ptrs)
    if (!wk.fits(N, npart)) return set_error(PBI4G_ERR_INVALID, "assign: work buffers not sized for this box");
    unsigned char blk[kOwnerPtrBytes];
    owner_ptrs_host(wk, blk);
    OwnerPtrs ov;
    memcpy(&ov, blk, sizeof(ov));
    const OwnerPtrs *op = bp ? static_cast<const OwnerPtrs *>(d_ptrs) : nullptr;  // the captured form
    double wmax = 1.0;
    if (d_weight && bp) return set_error(PBI4G_ERR_UNSUPPORTED, "captured assignment takes no weights");
    if (d_weight) {
        PBI4G_CUDA(cudaMemsetAsync(wk.wmax.p, 0, 8, st));
        owner_wmax_kernel<<<grid_blocks(npart, 256, 152 * 8), 256, 0, st>>>(npart, d_weight,
                                                                            wk.wmax.as<unsigned long long>());
        PBI4G_LAUNCH_CHECK();
        ++*launches;
        unsigned long long bitsw = 0;
        PBI4G_CUDA(cudaMemcpyAsync(&bitsw, wk.wmax.p, 8, cudaMemcpyDeviceToHost, st));
        PBI4G_CUDA(cudaStreamSynchronize(st));
        memcpy(&wmax, &bitsw, 8);
    }
    int bits;
    PBI4G_CHECK(fixed_point_bits(npart, wmax, &bits));
    // each contribution is one 32-bit integer: |w_x w_y w_z weight| 2^S <= 3.375 wmax 2^S < 2^30
    // (the 64-bit tile sums still hold the total); 2^-28 resolution for unit weights
    bits = std::min(bits, (int)floor(30.0 - log2(4.0 * (wmax > 0 ? wmax : 1.0))));
    if (bits < 8) return set_error(PBI4G_ERR_RANGE, "assign: particle weights up to %g", wmax);
    const int nt = N / kT, ntiles = nt * nt * nt;
    pf.begin(sort_stage, st);
    // counts and the tile counter
    if (op) {
        owner_zero_kernel<<<grid_blocks(ntiles + 2, 256, 152 * 4), 256, 0, st>>>(op, ntiles + 2);
        PBI4G_LAUNCH_CHECK();
        ++*launches;
        owner_count_kernel<true><<<grid_blocks(npart, 256), 256, 0, st>>>(N, nintp, interlaced, npart, stride, bp,
                                                                          d_pos, nt, ov, op);
        PBI4G_LAUNCH_CHECK();
        owner_scan_kernel<true><<<1, 1024, 0, st>>>(ntiles, ov, op);
        PBI4G_LAUNCH_CHECK();
        owner_scatter_kernel<true><<<grid_blocks(npart, 256), 256, 0, st>>>(N, nintp, interlaced, npart, bp, nt, ov,
                                                                            op, d_weight);
    } else {
        PBI4G_CUDA(cudaMemsetAsync(wk.count.p, 0, (size_t)(ntiles + 2) * 4, st));
        owner_count_kernel<false><<<grid_blocks(npart, 256), 256, 0, st>>>(N, nintp, interlaced, npart, stride, bp,
                                                                           d_pos, nt, ov, op);
        PBI4G_LAUNCH_CHECK();
        owner_scan_kernel<false><<<1, 1024, 0, st>>>(ntiles, ov, op);
        PBI4G_LAUNCH_CHECK();
        owner_scatter_kernel<false><<<grid_blocks(npart, 256), 256, 0, st>>>(N, nintp, interlaced, npart, bp, nt, ov,
                                                                             op, d_weight);
    }
    PBI4G_LAUNCH_CHECK();
    const size_t FC = full_cells(N);
    const bool wt = d_weight != nullptr;
    float *o2 = interlaced ? out + FC : nullptr;
    pf.end(st);
    pf.begin(tile_stage, st);
    int rc = PBI4G_OK;
    switch (nintp * 2 + (interlaced ? 1 : 0)) {
        case 2: rc = launch_tile<1, 1>(N, nt, ov, op, wt, bits, out, o2, st); break;
        case 3: rc = launch_tile<1, 2>(N, nt, ov, op, wt, bits, out, o2, st); break;
        case 4: rc = launch_tile<2, 1>(N, nt, ov, op, wt, bits, out, o2, st); break;
        case 5: rc = launch_tile<2, 2>(N, nt, ov, op, wt, bits, out, o2, st); break;
        case 6: rc = launch_tile<3, 1>(N, nt, ov, op, wt, bits, out, o2, st); break;
        case 7: rc = launch_tile<3, 2>(N, nt, ov, op, wt, bits, out, o2, st); break;
        case 8: rc = launch_tile<4, 1>(N, nt, ov, op, wt, bits, out, o2, st); break;
        default: rc = launch_tile<4, 2>(N, nt, ov, op, wt, bits, out, o2, st); break;
    }
    pf.end(st);
    PBI4G_CHECK(rc);
    *launches += 4;
    return PBI4G_OK;
}

}  // namespace pbi4g
