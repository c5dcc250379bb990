// mapfft.cu -- pruned inverse transform of the FP32 shell maps (see mapfft.cuh).
//
// The maps are the "real-space shell" fields of bispectrumI4.f90 (the C2R of
// the shell-masked delta(k), bispectrumI4.f90:120-158 and 430-474 for the
// multipole sets); the same maps as build_map_spectra + a full C2R, with the
// zero parts of the shell spectra never stored or transformed.
//
// Every pass runs tiles of 32 one-dimensional transforms (lanes = transforms,
// warps = butterflies) through an in-place mixed-radix DIF FFT in shared memory
// ([point][transform], pitch 33 float2): no ping-pong buffer, so four CTAs of
// 256 threads fit on an SM for the 200-point transforms of the 256^3 workload.
#include "mapfft.cuh"

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <math.h>

#include <algorithm>

namespace pbi4g {

namespace {

constexpr int kP = 33;        // shared pitch (float2) between the points of a tile
constexpr int kThreads = 256;
// CTAs per SM each pass is compiled for (registers per thread = 65536 / (256 x this)); build-time
// tuning macros, the defaults measured best
#ifndef PBI4G_ZPASS_MINB
#define PBI4G_ZPASS_MINB 4
#endif
#ifndef PBI4G_YPASS_MINB
#define PBI4G_YPASS_MINB 4
#endif
#ifndef PBI4G_XPASS_MINB
#define PBI4G_XPASS_MINB 4
#endif
// column loads the y pass keeps in flight per thread (8: 8% faster than 1 at 256^3)
#ifndef PBI4G_YPASS_BATCH
#define PBI4G_YPASS_BATCH 8
#endif

__device__ __forceinline__ float2 czero() { return make_float2(0.f, 0.f); }

// copy the packed plan tables (twiddles | entries | positions) into shared memory
__device__ __forceinline__ void load_tables(const unsigned char *__restrict__ tab, const fftd::FftDesc &fd,
                                            float2 *tw, int2 *ent, int *perm) {
    const float2 *t = reinterpret_cast<const float2 *>(tab);
    const int2 *e = reinterpret_cast<const int2 *>(t + fd.n);
    const int *p = reinterpret_cast<const int *>(e + fd.nent);
    for (int i = threadIdx.x; i < fd.n; i += blockDim.x) {
        tw[i] = t[i];
        perm[i] = p[i];
    }
    for (int i = threadIdx.x; i < fd.nent; i += blockDim.x) ent[i] = e[i];
}

// the plan's stages, last to first, over the 32 transforms of a tile whose
// points sit at the permuted positions (ends with a barrier); natural-order output.
// R20: the plan may hold radix-20 stages (plans built with allow20)
template <bool R20>
__device__ __forceinline__ void run_dit(const fftd::FftDesc &fd, float2 *buf, const int2 *ent, const float2 *tw,
                                        int warp, int nw, int lane) {
    for (int s = fd.nst - 1; s >= 0; s--) {
        const int R = fd.rad[s], ls = fd.ls[s], nbf = fd.n / R;
        const int2 *e = ent + fd.eoff[s];
        if (R20 && R == 20) {
            for (int j = warp; j < nbf; j += nw) fftd::dit_butterfly<20>(buf, kP, lane, e[j].x, ls, e[j].y, tw);
            __syncthreads();
            continue;
        }
        switch (R) {
            case 10:
                for (int j = warp; j < nbf; j += nw) fftd::dit_butterfly<10>(buf, kP, lane, e[j].x, ls, e[j].y, tw);
                break;
            case 8:
                for (int j = warp; j < nbf; j += nw) fftd::dit_butterfly<8>(buf, kP, lane, e[j].x, ls, e[j].y, tw);
                break;
            case 4:
                for (int j = warp; j < nbf; j += nw) fftd::dit_butterfly<4>(buf, kP, lane, e[j].x, ls, e[j].y, tw);
                break;
            case 2:
                for (int j = warp; j < nbf; j += nw) fftd::dit_butterfly<2>(buf, kP, lane, e[j].x, ls, e[j].y, tw);
                break;
            case 3:
                for (int j = warp; j < nbf; j += nw) fftd::dit_butterfly<3>(buf, kP, lane, e[j].x, ls, e[j].y, tw);
                break;
            case 5:
                for (int j = warp; j < nbf; j += nw) fftd::dit_butterfly<5>(buf, kP, lane, e[j].x, ls, e[j].y, tw);
                break;
            default:
                for (int j = warp; j < nbf; j += nw) fftd::dit_butterfly<7>(buf, kP, lane, e[j].x, ls, e[j].y, tw);
                break;
        }
        __syncthreads();
    }
}

size_t table_smem(const fftd::FftDesc &fd) {
    return sizeof(float2) * fd.n + sizeof(int2) * fd.nent + sizeof(int) * fd.n;
}

struct ZArgs {
    int N, NH, Nm, nb;
    const float2 *src[3];
    int fac[3];
    float los[3];
    double *powsum;
    int pow_mask;
    const int2 *cols;
    const MapInfo *info;
    const int2 *tiles;
    int ntiles;
    const unsigned char *tab;
    fftd::FftDesc fd;
    float2 *T;
};

// z pass: tile = (map m, 32 columns (kx, ky) of its shell).  Point i of a
// column is kz = kfreq0(i, Nm); a mode is in the shell when k2lo <= |k|^2 <=
// k2hi (the shell's |k|^2 range, contiguous).  The mask, multipole factor and
// kx = 0 symmetrisation of build_map_spectra; the multipole factor in FP32.
__global__ void __launch_bounds__(kThreads, PBI4G_ZPASS_MINB) map_zpass_kernel(const ZArgs a) {
    extern __shared__ __align__(16) unsigned char zsm[];
    const fftd::FftDesc &fd = a.fd;
    const int Nm = a.Nm, N = a.N, nb = a.nb;
    float2 *tw = reinterpret_cast<float2 *>(zsm);
    int2 *ent = reinterpret_cast<int2 *>(tw + fd.n);
    int *perm = reinterpret_cast<int *>(ent + fd.nent);
    float2 *buf = reinterpret_cast<float2 *>(perm + fd.n);
    double *spow = reinterpret_cast<double *>(buf + (size_t)Nm * kP);
    load_tables(a.tab, fd, tw, ent, perm);
    if (a.powsum)
        for (int b = threadIdx.x; b < 3 * nb; b += blockDim.x) spow[b] = 0.0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int tile = blockIdx.x; tile < a.ntiles; tile += gridDim.x) {
        const int2 tl = a.tiles[tile];
        const int m = tl.x, c0 = tl.y;
        const MapInfo mi = a.info[m];
        const int s = m / nb, b = mi.shell + 1;
        const int c = c0 + lane;
        const bool valid = c < mi.ncol;
        const int2 kk = valid ? a.cols[mi.col0 + c] : make_int2(0, 0);
        const int kx = kk.x, ky = kk.y, r2 = kx * kx + ky * ky;
        // kz^2 range of the shell on this column (empty for a padding lane)
        const int lo2 = valid ? mi.k2lo - r2 : 1, hi2 = valid ? mi.k2hi - r2 : 0;
        const float2 *src = a.src[s];
        const int fac = a.fac[s];
        const int yN = ky < 0 ? ky + N : ky;
        const float lxy = a.los[0] * (float)kx + a.los[1] * (float)ky;
        const float wpow = kx == 0 ? 1.f : 2.f;  // the kx > 0 modes stand for their mirror too
        float pacc = 0.f;
        for (int i = warp; i < Nm; i += nw) {
            const int kz = kfreq0(i, Nm), kz2 = kz * kz;
            float2 v = czero();
            if (kz2 >= lo2 && kz2 <= hi2) {
                const int zN = kz < 0 ? kz + N : kz;
                v = src[((size_t)zN * N + yN) * a.NH + kx];
                if (kx == 0) {
                    const float2 w = src[((size_t)kneg0(zN, N) * N + kneg0(yN, N)) * a.NH];
                    v.x = (v.x + w.x) * 0.5f;
                    v.y = (v.y - w.y) * 0.5f;
                }
                if (fac) {
                    const float lk = lxy + a.los[2] * (float)kz;
                    const int k2 = r2 + kz2;
                    const float mu2 = k2 > 0 ? lk * lk / (float)k2 : 0.f;
                    const float L = fac == 2 ? -0.5f + 1.5f * mu2 : 0.375f + mu2 * (-3.75f + 4.375f * mu2);
                    v.x *= L;
                    v.y *= L;
                }
                pacc += wpow * (v.x * v.x + v.y * v.y);
            }
            buf[perm[i] * kP + lane] = v;
        }
        if (a.powsum && (a.pow_mask >> s & 1)) {
            double pw = (double)pacc;
#pragma unroll
            for (int o = 16; o; o >>= 1) pw += __shfl_xor_sync(0xffffffffu, pw, o);
            if (lane == 0 && pw != 0.0) atomicAdd(&spow[s * nb + b - 1], pw);
        }
        __syncthreads();
        run_dit<true>(fd, buf, ent, tw, warp, nw, lane);
        // column c0 + l -> T[tbase + (c0 + l) Nm + z], z along the lanes
        for (int l = warp; l < 32; l += nw) {
            if (c0 + l >= mi.ncol) break;
            float2 *o = a.T + mi.tbase + (size_t)(c0 + l) * Nm;
            for (int z = lane; z < Nm; z += 32) o[z] = buf[z * kP + l];
        }
        __syncthreads();
    }
    if (a.powsum) {
        for (int b = threadIdx.x; b < 3 * nb; b += blockDim.x)
            if (spow[b] != 0.0) atomicAdd(a.powsum + b, spow[b]);
    }
}

struct YArgs {
    int Nm;
    const MapInfo *info;
    const int2 *kxr;
    const int *gmap;
    int z0, nz;        // the z-slab [z0, z0 + nz)
    int nflat;         // transforms: kxtot nz
    const unsigned char *tab;
    fftd::FftDesc fd;
    const float2 *T;
    float2 *U;
};

// y pass of one z-slab: tile = 32 consecutive flat transforms f = g nz + z - z0
// (g = kxc + kx: the flat kx index over all maps, so a tile may span maps); a
// lane reads column kx of its map, ky in [-r(kx), r(kx)], from T and the
// transform lands in U[f][y].
__global__ void __launch_bounds__(kThreads, PBI4G_YPASS_MINB) map_ypass_kernel(const YArgs a) {
    extern __shared__ __align__(16) unsigned char ysm[];
    const fftd::FftDesc &fd = a.fd;
    const int Nm = a.Nm;
    float2 *tw = reinterpret_cast<float2 *>(ysm);
    int2 *ent = reinterpret_cast<int2 *>(tw + fd.n);
    int *perm = reinterpret_cast<int *>(ent + fd.nent);
    float2 *buf = reinterpret_cast<float2 *>(perm + fd.n);
    load_tables(a.tab, fd, tw, ent, perm);
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int ntiles = (a.nflat + 31) / 32;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int t0 = tile * 32;
        const int f = t0 + lane;
        const bool valid = f < a.nflat;
        const int g = valid ? f / a.nz : 0, z = a.z0 + (valid ? f - g * a.nz : 0);
        const int m = a.gmap[g];
        const MapInfo &mi = a.info[m];
        const int kx = g - mi.kxc;
        const int2 rc = valid ? a.kxr[mi.kx0 + kx] : make_int2(-1, 0);  // (r, first column)
        const float2 *in = a.T + mi.tbase + (size_t)(rc.y + rc.x) * Nm + z;  // column ky = 0
        // PBI4G_YPASS_BATCH column loads in flight per thread before their shared stores
        for (int i0 = warp; i0 < Nm; i0 += PBI4G_YPASS_BATCH * nw) {
            float2 v[PBI4G_YPASS_BATCH];
#pragma unroll
            for (int u = 0; u < PBI4G_YPASS_BATCH; u++) {
                const int i = i0 + u * nw, ky = kfreq0(i, Nm);
                v[u] = (i < Nm && ky >= -rc.x && ky <= rc.x) ? __ldcs(in + (ptrdiff_t)ky * Nm) : czero();
            }
#pragma unroll
            for (int u = 0; u < PBI4G_YPASS_BATCH; u++) {
                const int i = i0 + u * nw;
                if (i < Nm) buf[perm[i] * kP + lane] = v[u];
            }
        }
        __syncthreads();
        run_dit<true>(fd, buf, ent, tw, warp, nw, lane);
        for (int l = warp; l < 32; l += nw) {
            if (t0 + l >= a.nflat) break;
            float2 *o = a.U + (size_t)(t0 + l) * Nm;
            for (int y = lane; y < Nm; y += 32) o[y] = buf[y * kP + l];
        }
        __syncthreads();
    }
}

struct XArgs {
    int Nm, count, kxmax, oform, nb;
    const MapInfo *info;
    const unsigned char *tab;
    fftd::FftDesc fd;   // M = Nm / 2 points
    const float2 *xtw;  // e^{2 pi i k / Nm}
    const float2 *U;
    float *out;         // oform -1: dense FP32 maps
    void *bhi, *blo;    // oform 0 / 1 / 2: operand planes (MapPlanes)
    float2 *a32;
    const int *mexp;
    long long npts;     // points of the slab (the per-map stride of the dense maps)
    int row_lo, nrows;  // the slab's (z, y) rows: [row_lo, row_lo + nrows), row = z Nm + y
    float inv_nm;
};

template <int P>
__device__ __forceinline__ void store_words(void *dst, const unsigned (&w)[P]) {
    if constexpr (P == 2) *reinterpret_cast<uint2 *>(dst) = make_uint2(w[0], w[1]);
    else *reinterpret_cast<uint4 *>(dst) = make_uint4(w[0], w[1], w[2], w[3]);
}

template <int P>
__device__ __forceinline__ void store_floats(float *dst, const float2 (&v)[P]) {
#pragma unroll
    for (int i = 0; i < P; i += 2)
        *reinterpret_cast<float4 *>(dst + 2 * i) = make_float4(v[i].x, v[i].y, v[i + 1].x, v[i + 1].y);
}

// The x pass's operand-plane stores of one tile of map m: lane = W consecutive
// points of a row (the z values z[j] .. z[j + W/2 - 1] of row l), written as one
// W-element store per plane at ((chunk maps + m) 64 + point % 64).
template <int W>
__device__ __forceinline__ void store_planes(const XArgs &a, const float2 *buf, int m, int nrows, int npt, size_t c0,
                                             float sb, float sa, int warp, int nw, int lane) {
    constexpr int P = W / 2;
    const int Nm = a.Nm;
    for (int pl = 32 * W * warp + W * lane; pl < npt; pl += 32 * W * nw) {
        int l = (int)(((float)pl + 0.5f) * a.inv_nm);
        l -= l * Nm > pl ? 1 : 0;
        l += (l + 1) * Nm <= pl ? 1 : 0;
        const int j = (pl - l * Nm) >> 1;
        float2 z[P], v[P];
#pragma unroll
        for (int i = 0; i < P; i++) {
            z[i] = buf[(j + i) * kP + l];
            v[i] = fftd::cscale(z[i], sb);
        }
        const size_t ck = c0 + (pl >> 6), t = pl & 63;
        const size_t ib = (ck * a.count + m) * 64 + t;  // element index in the B planes
        if (a.oform == 1) {
            unsigned hw[P], lw[P];
#pragma unroll
            for (int i = 0; i < P; i++) {
                const __half2 h = __float22half2_rn(v[i]);
                const __half2 g = __float22half2_rn(fftd::csub(v[i], __half22float2(h)));
                hw[i] = *reinterpret_cast<const unsigned *>(&h);
                lw[i] = *reinterpret_cast<const unsigned *>(&g);
            }
            store_words<P>(reinterpret_cast<__half *>(a.bhi) + ib, hw);
            store_words<P>(reinterpret_cast<__half *>(a.blo) + ib, lw);
        } else if (a.oform == 2) {
            unsigned hw[P];
#pragma unroll
            for (int i = 0; i < P; i++) {
                const __nv_bfloat162 h = __float22bfloat162_rn(v[i]);
                hw[i] = *reinterpret_cast<const unsigned *>(&h);
            }
            store_words<P>(reinterpret_cast<__nv_bfloat16 *>(a.bhi) + ib, hw);
        } else {
            float2 h[P], lo[P];
#pragma unroll
            for (int i = 0; i < P; i++) {
                h[i] = make_float2(__uint_as_float(__float_as_uint(v[i].x) & 0xFFFFE000u),
                                   __uint_as_float(__float_as_uint(v[i].y) & 0xFFFFE000u));
                lo[i] = fftd::csub(v[i], h[i]);
            }
            store_floats<P>(reinterpret_cast<float *>(a.bhi) + ib, h);
            store_floats<P>(reinterpret_cast<float *>(a.blo) + ib, lo);
        }
        if (m < a.nb) {
#pragma unroll
            for (int i = 0; i < P; i++) z[i] = fftd::cscale(z[i], sa);
            store_floats<P>(reinterpret_cast<float *>(a.a32) + (ck * a.nb + m) * 64 + t, z);
        }
    }
}

// x pass: tile = (map m, 32 consecutive rows (z, y)).  With M = Nm / 2,
// Z[k] = (X[k] + conj X[M-k]) + i (X[k] - conj X[M-k]) e^{2 pi i k / Nm} and
// z = IDFT_M(Z) give the C2R output x[2j] = Re z[j], x[2j+1] = Im z[j].  The
// raw coefficients (kx < kxmax) stay in their own buffer while the pairs
// (k, M - k) are formed into the permuted positions of the FFT buffer.  PF:
// coefficient rows a warp prefetches into registers for the next tile
// (kxmax <= PF * warps).
template <int PF>
__global__ void __launch_bounds__(kThreads, PF <= 9 ? PBI4G_XPASS_MINB : 2) map_xpass_kernel(const XArgs a) {
    extern __shared__ __align__(16) unsigned char xsm[];
    const fftd::FftDesc &fd = a.fd;
    const int Nm = a.Nm, M = fd.n, KX = a.kxmax;
    float2 *tw = reinterpret_cast<float2 *>(xsm);
    int2 *ent = reinterpret_cast<int2 *>(tw + fd.n);
    int *perm = reinterpret_cast<int *>(ent + fd.nent);
    float2 *xt = reinterpret_cast<float2 *>(perm + fd.n);  // [Nm]
    float2 *xr = xt + Nm;                                  // [KX][kP] raw coefficients
    float2 *buf = xr + (size_t)KX * kP;                    // [M][kP]
    load_tables(a.tab, fd, tw, ent, perm);
    for (int i = threadIdx.x; i < Nm; i += blockDim.x) xt[i] = a.xtw[i];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int row_hi = a.row_lo + a.nrows, tpm = (a.nrows + 31) / 32, ntiles = tpm * a.count;
    float2 pre[PF];
    // U holds the slab: column kx of map m, row (z, y) at ((kxc + kx) nrows + row - row_lo)
    auto fetch = [&](int m, int row0) {
        const bool ok = row0 + lane < row_hi;
        const MapInfo &mi = a.info[m];
        const int kxn = mi.kxn;
        const float2 *src = a.U + (size_t)mi.kxc * a.nrows + (row0 - a.row_lo) + lane;
#pragma unroll
        for (int i = 0; i < PF; i++) {
            const int k = warp + i * nw;
            pre[i] = (k < kxn && ok) ? __ldcs(src + (size_t)k * a.nrows) : czero();
        }
    };
    // (map, tile within the map) of this CTA's tiles, advanced without divisions
    int m = blockIdx.x / tpm, r = blockIdx.x - m * tpm;
    const int gm = gridDim.x / tpm, gr = gridDim.x - gm * tpm;
    auto advance = [&](int &mm, int &rr) {
        mm += gm;
        rr += gr;
        if (rr >= tpm) { rr -= tpm; mm++; }
    };
    if (blockIdx.x < ntiles) fetch(m, a.row_lo + r * 32);
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int row0 = a.row_lo + r * 32;
        const int nrows = min(32, row_hi - row0);
        int mn = m, rn = r;
        advance(mn, rn);
        const int kxn = a.info[m].kxn;  // X[k] = 0 for k >= kxn
        __syncthreads();
#pragma unroll
        for (int i = 0; i < PF; i++) {
            const int k = warp + i * nw;
            if (k < kxn) xr[k * kP + lane] = pre[i];
        }
        if (tile + (int)gridDim.x < ntiles) fetch(mn, a.row_lo + rn * 32);
        __syncthreads();
        for (int k = warp; k <= M / 2; k += nw) {
            const int kc = M - k;
            if (k >= kxn && kc >= kxn) {  // X[k] = X[M - k] = 0 (k is warp-uniform)
                buf[perm[k] * kP + lane] = czero();
                if (k > 0 && kc != k) buf[perm[kc] * kP + lane] = czero();
                continue;
            }
            const float2 xk = k < kxn ? xr[k * kP + lane] : czero();
            const float2 xc = (k > 0 && kc < kxn) ? xr[kc * kP + lane] : czero();  // X[M - k]
            const float2 ck = make_float2(xc.x, -xc.y), cc = make_float2(xk.x, -xk.y);
            const float2 o1 = fftd::cmul(fftd::csub(xk, ck), xt[k]);
            buf[perm[k] * kP + lane] = fftd::cadd_i(fftd::cadd(xk, ck), o1);
            if (k > 0 && kc != k) {
                const float2 o2 = fftd::cmul(fftd::csub(xc, cc), xt[kc]);
                buf[perm[kc] * kP + lane] = fftd::cadd_i(fftd::cadd(xc, cc), o2);
            }
        }
        __syncthreads();
        run_dit<false>(fd, buf, ent, tw, warp, nw, lane);
        if (a.oform < 0) {
            // dense FP32 maps: one warp per row, x[2j], x[2j+1] = z[j]
            for (int l = warp; l < nrows; l += nw) {
                float2 *o =
                    reinterpret_cast<float2 *>(a.out + (size_t)m * a.npts + ((size_t)(row0 - a.row_lo) + l) * Nm);
                for (int j = lane; j < M; j += 32) o[j] = buf[j * kP + l];
            }
        } else {
            // operand planes, chunk-major: the tile's rows are whole chunks of 64 points
            // (32 Nm or 16 Nm points, Nm % 4 == 0), so a warp writes two chunk rows of a
            // plane per instruction
            const float sb = a.oform == 1 ? exp2f((float)a.mexp[m]) : 1.f;  // B planes: x 2^e
            const float sa = sb * (a.oform == 1 ? 1.f / 128.f : 1.f);       // pair factors: x 2^(e-7)
            const int npt = nrows * Nm;
            const size_t c0 = ((size_t)(row0 - a.row_lo) * Nm) >> 6;
            // a lane takes W consecutive points of one row (Nm % W == 0), 64 / W lanes a chunk row
            if (Nm % 8 == 0)
                store_planes<8>(a, buf, m, nrows, npt, c0, sb, sa, warp, nw, lane);
            else
                store_planes<4>(a, buf, m, nrows, npt, c0, sb, sa, warp, nw, lane);
        }
        m = mn;
        r = rn;
    }
}

int upload(DevBuf &d, const void *h, size_t bytes) {
    PBI4G_CHECK(d.ensure(bytes > 0 ? bytes : 8));
    if (bytes) PBI4G_CUDA(cudaMemcpy(d.p, h, bytes, cudaMemcpyHostToDevice));
    return PBI4G_OK;
}

int upload_plan(DevBuf &d, const fftd::FftPlan &p) {
    std::vector<unsigned char> h(p.bytes());
    p.pack(h.data());
    return upload(d, h.data(), h.size());
}

int grid_for(const void *kern, int threads, size_t smem, int work) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem) != cudaSuccess) per_sm = 1;
    return std::max(1, std::min(work, 152 * std::max(1, per_sm)));
}

}  // namespace

int MapTransform::build(const Shells &s, int nm) {
    Nm = s.Nm;
    nmaps = nm;
    nb = s.nb;
    // radix 20 in the z / y passes only: the x pass keeps its prefetched
    // coefficients live across the transform and has no registers to spare
    if (Nm % 4 || !pz.build(Nm, true) || !px.build(Nm / 2, false))
        return set_error(PBI4G_ERR_UNSUPPORTED, "map transform: map grid %d", Nm);
    // per shell: largest k^2, the kx range and the (kx, ky) columns
    std::vector<int> k2hi(nb, -1), k2lo(nb, -1);
    for (int k2 = 0; k2 <= s.k2max && k2 < (int)s.lut_h.size(); k2++) {
        const int b = s.lut_h[k2];
        if (b < 1 || b > nb) continue;
        if (k2lo[b - 1] < 0) k2lo[b - 1] = k2;
        k2hi[b - 1] = std::max(k2hi[b - 1], k2);
    }
    // the z pass tests shell membership as k2lo <= |k|^2 <= k2hi: every shell's
    // |k|^2 values must form one range (they do: shells are intervals of |k|)
    for (int b = 0; b < nb; b++)
        for (int k2 = std::max(k2lo[b], 0); k2 <= k2hi[b]; k2++)
            if (s.lut_h[k2] != b + 1)
                return set_error(PBI4G_ERR_UNSUPPORTED, "map transform: shell %d is not one |k|^2 range", b + 1);
    std::vector<int2> cols_h, kxr_h;
    std::vector<int> kxn(nb), ncol(nb), col0(nb), kx0(nb);
    auto isqrt = [](int v) {
        int r = (int)std::sqrt((double)v);
        while (r * r > v) r--;
        while ((r + 1) * (r + 1) <= v) r++;
        return r;
    };
    kxmax = 0;
    for (int b = 0; b < nb; b++) {
        col0[b] = (int)cols_h.size();
        kx0[b] = (int)kxr_h.size();
        kxn[b] = k2hi[b] >= 0 ? isqrt(k2hi[b]) + 1 : 0;
        if (kxn[b] > Nm / 2) return set_error(PBI4G_ERR_UNSUPPORTED, "map transform: shell %d above Nm/2", b + 1);
        for (int kx = 0; kx < kxn[b]; kx++) {
            const int r = isqrt(k2hi[b] - kx * kx);
            kxr_h.push_back(make_int2(r, (int)cols_h.size() - col0[b]));
            for (int ky = -r; ky <= r; ky++) cols_h.push_back(make_int2(kx, ky));
        }
        ncol[b] = (int)cols_h.size() - col0[b];
        kxmax = std::max(kxmax, kxn[b]);
    }
    info_h.assign(nm, MapInfo{});
    std::vector<int2> zt;
    std::vector<int> gm;
    long long tb = 0, ub = 0;
    for (int m = 0; m < nm; m++) {
        const int b = m % nb;
        MapInfo &mi = info_h[m];
        mi.shell = b;
        mi.kxn = kxn[b];
        mi.ncol = ncol[b];
        mi.col0 = col0[b];
        mi.kx0 = kx0[b];
        mi.k2lo = k2lo[b];
        mi.k2hi = k2hi[b];
        mi.kxc = (int)gm.size();
        mi.tbase = tb;
        mi.ubase = ub;
        tb += (long long)ncol[b] * Nm;
        ub += (long long)kxn[b] * Nm * Nm;
        for (int c = 0; c < ncol[b]; c += 32) zt.push_back(make_int2(m, c));
        for (int kx = 0; kx < kxn[b]; kx++) gm.push_back(m);
    }
    tsize = tb;
    usize = ub;
    nzt = (int)zt.size();
    kxtot = (int)gm.size();
    if ((long long)kxtot * Nm >= (1LL << 31))
        return set_error(PBI4G_ERR_UNSUPPORTED, "map transform: %d kx columns of grid %d", kxtot, Nm);
    std::vector<float2> xt(Nm);
    for (int k = 0; k < Nm; k++) xt[k] = make_float2((float)cos(2 * M_PI * k / Nm), (float)sin(2 * M_PI * k / Nm));
    PBI4G_CHECK(upload_plan(tab_z, pz));
    PBI4G_CHECK(upload_plan(tab_x, px));
    PBI4G_CHECK(upload(xtw, xt.data(), sizeof(float2) * Nm));
    PBI4G_CHECK(upload(cols, cols_h.data(), sizeof(int2) * cols_h.size()));
    PBI4G_CHECK(upload(kxr, kxr_h.data(), sizeof(int2) * kxr_h.size()));
    PBI4G_CHECK(upload(info, info_h.data(), sizeof(MapInfo) * info_h.size()));
    PBI4G_CHECK(upload(ztiles, zt.data(), sizeof(int2) * zt.size()));
    PBI4G_CHECK(upload(gmap, gm.data(), sizeof(int) * gm.size()));
    return PBI4G_OK;
}

int map_zpass(const Shells &sh, const MapTransform &mt, const float2 *const src[3], const int fac[3],
              const double los[3], float2 *work, double *powsum, int pow_mask, cudaStream_t st, int64_t *launches) {
    if (mt.nzt == 0) return PBI4G_OK;
    ZArgs a;
    a.N = sh.N;
    a.NH = sh.N / 2 + 1;
    a.Nm = mt.Nm;
    a.nb = mt.nb;
    for (int s = 0; s < 3; s++) {
        a.src[s] = src[s];
        a.fac[s] = fac[s];
        a.los[s] = los ? (float)los[s] : 0.f;
    }
    a.powsum = powsum;
    a.pow_mask = pow_mask;
    a.cols = mt.cols.as<int2>();
    a.info = mt.info.as<MapInfo>();
    a.tiles = mt.ztiles.as<int2>();
    a.ntiles = mt.nzt;
    a.tab = static_cast<const unsigned char *>(mt.tab_z.p);
    a.fd = mt.pz.d;
    a.T = work;
    const size_t smem = table_smem(mt.pz.d) + sizeof(float2) * (size_t)mt.Nm * kP + sizeof(double) * 3 * mt.nb;
    PBI4G_CUDA(cudaFuncSetAttribute(map_zpass_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    map_zpass_kernel<<<grid_for((const void *)map_zpass_kernel, kThreads, smem, mt.nzt), kThreads, smem, st>>>(a);
    PBI4G_LAUNCH_CHECK();
    ++*launches;
    return PBI4G_OK;
}

int map_ypass(const MapTransform &mt, float2 *work, cudaStream_t st, int64_t *launches, int z0, int z1) {
    if (z1 < 0) z1 = mt.Nm;
    if (z0 < 0 || z1 > mt.Nm || z0 >= z1)
        return set_error(PBI4G_ERR_INVALID, "y pass: slab [%d, %d) of grid %d", z0, z1, mt.Nm);
    if (mt.kxtot == 0) return PBI4G_OK;
    YArgs a;
    a.Nm = mt.Nm;
    a.info = mt.info.as<MapInfo>();
    a.kxr = mt.kxr.as<int2>();
    a.gmap = mt.gmap.as<int>();
    a.z0 = z0;
    a.nz = z1 - z0;
    a.nflat = mt.kxtot * a.nz;
    a.tab = static_cast<const unsigned char *>(mt.tab_z.p);
    a.fd = mt.pz.d;
    a.T = work;
    a.U = work + mt.tsize;
    const int ntiles = (a.nflat + 31) / 32;
    const size_t smem = table_smem(mt.pz.d) + sizeof(float2) * (size_t)mt.Nm * kP;
    PBI4G_CUDA(cudaFuncSetAttribute(map_ypass_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    map_ypass_kernel<<<grid_for((const void *)map_ypass_kernel, kThreads, smem, ntiles), kThreads, smem, st>>>(a);
    PBI4G_LAUNCH_CHECK();
    ++*launches;
    return PBI4G_OK;
}

int map_xpass(const MapTransform &mt, const float2 *work, float *out, const MapPlanes *planes, cudaStream_t st,
              int64_t *launches, int z0, int z1) {
    if (mt.nmaps == 0) return PBI4G_OK;
    if (z1 < 0) z1 = mt.Nm;
    if (z0 < 0 || z1 > mt.Nm || z0 >= z1)
        return set_error(PBI4G_ERR_INVALID, "x pass: slab [%d, %d) of grid %d", z0, z1, mt.Nm);
    XArgs a;
    a.Nm = mt.Nm;
    a.count = mt.nmaps;
    a.kxmax = mt.kxmax;
    a.oform = planes ? planes->form : -1;
    a.nb = mt.nb;
    a.info = mt.info.as<MapInfo>();
    a.tab = static_cast<const unsigned char *>(mt.tab_x.p);
    a.fd = mt.px.d;
    a.xtw = mt.xtw.as<float2>();
    a.U = work + mt.tsize;
    a.out = out;
    a.bhi = planes ? planes->bhi : nullptr;
    a.blo = planes ? planes->blo : nullptr;
    a.a32 = planes ? reinterpret_cast<float2 *>(planes->a32) : nullptr;
    a.mexp = planes ? planes->mexp : nullptr;
    a.npts = (long long)(z1 - z0) * mt.Nm * mt.Nm;
    a.row_lo = z0 * mt.Nm;
    a.nrows = (z1 - z0) * mt.Nm;
    a.inv_nm = 1.0f / (float)mt.Nm;
    // planes: whole 64-point chunks per slab
    if (planes && (planes->form < 0 || planes->form > 2 || (planes->form == 1 && !planes->mexp) ||
                   planes->npts != a.npts || planes->nmaps != mt.nmaps || a.npts % MapPlanes::kChunk))
        return set_error(PBI4G_ERR_INVALID, "x pass: operand planes do not match the maps");
    const int M = mt.Nm / 2, warps = kThreads / 32, pf = (mt.kxmax + warps - 1) / warps;
    const size_t smem =
        table_smem(mt.px.d) + sizeof(float2) * ((size_t)mt.Nm + (size_t)mt.kxmax * kP + (size_t)M * kP);
    const long long ntiles = ((long long)a.nrows + 31) / 32 * mt.nmaps;
    if (ntiles >= (1LL << 31)) return set_error(PBI4G_ERR_UNSUPPORTED, "x pass: %lld tiles", ntiles);
    const int work_tiles = (int)ntiles;
    auto launch = [&](auto kern) -> int {
        PBI4G_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        kern<<<grid_for((const void *)kern, kThreads, smem, work_tiles), kThreads, smem, st>>>(a);
        PBI4G_LAUNCH_CHECK();
        return PBI4G_OK;
    };
    if (pf <= 4) PBI4G_CHECK(launch(map_xpass_kernel<4>));
    else if (pf <= 9) PBI4G_CHECK(launch(map_xpass_kernel<9>));
    else if (pf <= 16) PBI4G_CHECK(launch(map_xpass_kernel<16>));
    else if (pf <= 32) PBI4G_CHECK(launch(map_xpass_kernel<32>));
    else return set_error(PBI4G_ERR_UNSUPPORTED, "x pass: %d coefficient rows", mt.kxmax);
    ++*launches;
    return PBI4G_OK;
}

int fft_plan_host_check(int n, int batch, const float *in, float *out) {
    fftd::FftPlan p;
    if (!p.build(n, true)) return set_error(PBI4G_ERR_UNSUPPORTED, "fft plan: %d points", n);
    std::vector<float2> buf((size_t)n);
    for (int t = 0; t < batch; t++) {
        for (int i = 0; i < n; i++)
            buf[p.perm[i]] = make_float2(in[2 * ((size_t)t * n + i)], in[2 * ((size_t)t * n + i) + 1]);
        fftd::run_plan_host(p, buf.data(), 1, 0);
        for (int k = 0; k < n; k++) {
            const float2 v = buf[k];
            out[2 * ((size_t)t * n + k)] = v.x;
            out[2 * ((size_t)t * n + k) + 1] = v.y;
        }
    }
    return PBI4G_OK;
}

}  // namespace pbi4g
