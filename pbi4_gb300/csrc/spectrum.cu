// spectrum.cu -- Fourier-space kernels of the density stage and P(k) binning.
//
//  * fcomb_half   : interlacing combine + window deconvolution + 1/npart, fused
//                   into one pass over the R2C half spectra (powerI4.f90:251-378).
//  * fcomb_full   : the same routine on a full complex grid (f2py drop-in).
//  * pk_measure   : P(k) / P_l binning (powerI4.f90:510-594, 596-693) with the
//                   constant-LOS multipole factors applied per mode, which equals
//                   compute_density_multipoles (pbi4.py:343-388 + compute_q2k/q4k)
//                   without its 22 full FFTs:
//                   FFT(delta(x) l_i l_j) = l_i l_j delta(k) by linearity, and
//                   sum_{ij} fac l_i l_j k_i k_j / k^2 = (l.k)^2 / k^2.
//  * q2k_full, q4k_full, reduce_full : f2py drop-ins on full grids.
#include "spectrum.cuh"

#include <float.h>
#include <math.h>
#include <mutex>
#include <vector>

namespace pbi4g {

void window_table(int N, int nintp, double *tW) {
    const double tpiN = (double)kTwoPiF / (double)N;
    tW[0] = 1.0;
    for (int i = 2; i <= N / 2 + 1; i++) {
        double rk = tpiN * (double)(i - 1);
        double s = sin(rk / 2.0) / (rk / 2.0), r = 1.0;
        for (int k = 0; k < nintp; k++) r *= s;
        tW[i - 1] = r;
    }
}

double fcomb_kF3(float box) {
    volatile float t = kTwoPiF * kTwoPiF;  // real(4) arithmetic, powerI4.f90:271
    t = t * kTwoPiF;
    t = t / box;
    t = t / box;
    t = t / box;
    return (double)t;
}

// ------------------------------------------------------------ complex ops ---
template <class C> __device__ __forceinline__ C cmk(double r, double i) { C c; c.x = r; c.y = i; return c; }
template <class C> __device__ __forceinline__ C cmul(C a, C b) {
    C c; c.x = a.x * b.x - a.y * b.y; c.y = a.x * b.y + a.y * b.x; return c;
}
template <class C> __device__ __forceinline__ C cadd(C a, C b) { C c; c.x = a.x + b.x; c.y = a.y + b.y; return c; }
template <class C> __device__ __forceinline__ C csub(C a, C b) { C c; c.x = a.x - b.x; c.y = a.y - b.y; return c; }
template <class C> __device__ __forceinline__ C cconj(C a) { C c; c.x = a.x; c.y = -a.y; return c; }
template <class C, class S> __device__ __forceinline__ C cscale(C a, S s) { C c; c.x = a.x * s; c.y = a.y * s; return c; }

__device__ __forceinline__ void sincos_t(float a, float *s, float *c) { sincosf(a, s, c); }
__device__ __forceinline__ void sincos_t(double a, double *s, double *c) { sincos(a, s, c); }

// The orbit {ix,icx} x {iy,icy} x {iz,icz} of one iteration of fcomb's
// interlaced loop, with the reference's write order (powerI4.f90:325-342)
// applied to an 8-entry local copy.  Where ix == icx (etc.) the two slots are
// one location and later writes win, exactly as in the Fortran.  DISTINCT: the
// caller has checked that no two slots coincide (ix != icx, iy != icy, iz != icz),
// so every index is static and the copy stays in registers.
template <class R, bool DISTINCT = false>
struct Orbit {
    using C = typename Cx<R>::T;
    C v[8];
    int ex = 0, ey = 0, ez = 0;
    __device__ __forceinline__ int key(int xs, int ys, int zs) const {
        if constexpr (DISTINCT) return xs | (ys << 1) | (zs << 2);
        return (ex ? 0 : xs) | ((ey ? 0 : ys) << 1) | ((ez ? 0 : zs) << 2);
    }
    __device__ __forceinline__ void combine(R xa, R ya, R za, R cfac) {
        // phases xrec = exp(-i pi (ix-1)/N) etc. as angles xa, ya, za
        R sx, cxr, sy, cyr, sz, czr;
        sincos_t(xa, &sx, &cxr);
        sincos_t(ya, &sy, &cyr);
        sincos_t(za, &sz, &czr);
        const C xr = cmk<C>(cxr, sx), yr = cmk<C>(cyr, sy), zr = cmk<C>(czr, sz);
        const C ci = cmk<C>(0, 1), c1 = cmk<C>(1, 0);
        const C cma = cmul(cmul(cmul(ci, xr), yr), zr);
        const C cmb = cmul(cmul(cmul(ci, xr), yr), cconj(zr));
        const C cmc = cmul(cmul(cmul(ci, xr), cconj(yr)), zr);
        const C cmd = cmul(cmul(ci, xr), cconj(cmul(yr, zr)));
        const C c000 = cadd(cmul(v[key(0, 0, 0)], csub(c1, cma)), cmul(cconj(v[key(1, 1, 1)]), cadd(c1, cma)));
        const C c001 = cadd(cmul(v[key(0, 0, 1)], csub(c1, cmb)), cmul(cconj(v[key(1, 1, 0)]), cadd(c1, cmb)));
        const C c010 = cadd(cmul(v[key(0, 1, 0)], csub(c1, cmc)), cmul(cconj(v[key(1, 0, 1)]), cadd(c1, cmc)));
        const C c011 = cadd(cmul(v[key(0, 1, 1)], csub(c1, cmd)), cmul(cconj(v[key(1, 0, 0)]), cadd(c1, cmd)));
        v[key(0, 0, 0)] = cscale(c000, cfac);
        v[key(0, 0, 1)] = cscale(c001, cfac);
        v[key(0, 1, 0)] = cscale(c010, cfac);
        v[key(0, 1, 1)] = cscale(c011, cfac);
        v[key(1, 0, 0)] = cconj(v[key(0, 1, 1)]);
        v[key(1, 0, 1)] = cconj(v[key(0, 1, 0)]);
        v[key(1, 1, 0)] = cconj(v[key(0, 0, 1)]);
        v[key(1, 1, 1)] = cconj(v[key(0, 0, 0)]);
    }
};

// ------------------------------------------------- fcomb on half spectra ---
// d(k) = F1(k) + i F2(k) is the FFT of the complex grid the reference builds
// (Re = grid 1, Im = interlaced grid); outside the stored half it is
// conj(F1(-k)) + i conj(F2(-k)).
template <class R>
__device__ __forceinline__ typename Cx<R>::T dsample(const typename Cx<R>::T *__restrict__ F1,
                                                     const typename Cx<R>::T *__restrict__ F2, int N, int X, int Y,
                                                     int Z) {
    using C = typename Cx<R>::T;
    const int NH = N / 2 + 1;
    if (X <= N / 2) {
        const size_t o = ((size_t)Z * N + Y) * NH + X;
        const C f1 = F1[o], f2 = F2[o];
        return cmk<C>(f1.x - f2.y, f1.y + f2.x);
    }
    const size_t o = ((size_t)kneg0(Z, N) * N + kneg0(Y, N)) * NH + (N - X);
    const C f1 = F1[o], f2 = F2[o];
    return cmk<C>(f1.x + f2.y, f2.x - f1.y);
}

// orbits t < NH^3 <= 1025^3 < 2^32: 32-bit index arithmetic; ang[i] = the
// reference's phase angle -pi i / N (powerI4.f90:325-342) rounded to R
template <class R>
__global__ void fcomb_interlaced_half_kernel(int N, const typename Cx<R>::T *__restrict__ spec,
                                             typename Cx<R>::T *__restrict__ delta, const R *__restrict__ iW,
                                             const R *__restrict__ ang, R cf, const BoxPar *__restrict__ bp) {
    const int NH = N / 2 + 1;
    if (bp) cf = (R)bp->fcomb_cf;
    const size_t HC = (size_t)N * N * NH;
    const typename Cx<R>::T *F1 = spec, *F2 = spec + HC;
    const unsigned total = (unsigned)NH * NH * NH;
    for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
        const unsigned q = t / NH;
        const int ox = (int)(t - q * NH), oy = (int)(q % NH), oz = (int)(q / NH);
        const int cx = kneg0(ox, N), cy = kneg0(oy, N), cz = kneg0(oz, N);
        // orbits without coinciding points (all but the kx, ky, kz = 0 and Nyquist planes)
        // take the register path
        auto run = [&](auto o) {
            o.ex = ox == cx; o.ey = oy == cy; o.ez = oz == cz;
            // the orbit's points (ox or cx, oy or cy, oz or cz) read the four half-spectrum
            // cells (ox, oy or cy, oz or cz): (ox, Y, Z) directly, (cx, Y, Z) as the mirror
            // of (ox, -Y, -Z) (dsample's two branches), so each cell is loaded once
            using C = typename Cx<R>::T;
            C f1[2][2], f2[2][2];
#pragma unroll
            for (int c = 0; c < 4; c++) {
                const int ys = c & 1, zs = c >> 1;
                const size_t off = ((size_t)(zs ? cz : oz) * N + (ys ? cy : oy)) * NH + ox;
                f1[ys][zs] = F1[off];
                f2[ys][zs] = F2[off];
            }
#pragma unroll
            for (int s = 0; s < 8; s++) {
                const int xs = s & 1, ys = (s >> 1) & 1, zs = s >> 2;
                if (xs && o.ex) continue;  // ox = cx: the same points as xs = 0
                if (!xs) {
                    const C a = f1[ys][zs], b = f2[ys][zs];
                    o.v[o.key(0, ys, zs)] = cmk<C>(a.x - b.y, a.y + b.x);
                } else {
                    const C a = f1[1 - ys][1 - zs], b = f2[1 - ys][1 - zs];
                    o.v[o.key(1, ys, zs)] = cmk<C>(a.x + b.y, b.x - a.y);
                }
            }
            const R cfac = cf * iW[ox] * iW[oy] * iW[oz];
            o.combine(ang[ox], ang[oy], ang[oz], cfac);
            // store the orbit's locations inside the half (x = ox; x = cx only if equal)
#pragma unroll
            for (int s = 0; s < 4; s++) {
                const int ys = s & 1, zs = s >> 1;
                if ((ys && o.ey) || (zs && o.ez)) continue;
                const int Y = ys ? cy : oy, Z = zs ? cz : oz;
                delta[((size_t)Z * N + Y) * NH + ox] = o.v[o.key(0, ys, zs)];
            }
        };
        if (ox != cx && oy != cy && oz != cz) run(Orbit<R, true>{});
        else run(Orbit<R, false>{});
    }
}

// I: the cell index type (32-bit when the half spectrum has < 2^31 cells)
template <class R, class I>
__global__ void fcomb_plain_half_kernel(int N, const typename Cx<R>::T *__restrict__ spec,
                                        typename Cx<R>::T *__restrict__ delta, const R *__restrict__ iW, R cf,
                                        const BoxPar *__restrict__ bp) {
    const int NH = N / 2 + 1;
    if (bp) cf = (R)bp->fcomb_cf;
    const I HC = (I)N * N * NH;
    for (I c = blockIdx.x * (I)blockDim.x + threadIdx.x; c < HC; c += (I)gridDim.x * blockDim.x) {
        const I q = c / NH;
        const int x = (int)(c - q * NH), y = (int)(q % N), z = (int)(q / N);
        const R f = cf * iW[x] * iW[kabs0(y, N)] * iW[kabs0(z, N)];
        delta[c] = cscale(spec[c], f);
    }
}

double fcomb_cf(bool interlaced, float box, double norm) {
    const double kF3 = fcomb_kF3(box);
    return (interlaced ? 1.0 / (4.0 * kF3) : 1.0 / kF3) / norm;
}

template <class R>
int fcomb_half(int N, int nintp, bool interlaced, float box, double norm, const typename Cx<R>::T *spec,
               typename Cx<R>::T *delta, WinCache &wcache, cudaStream_t st, int64_t *launches, const BoxPar *bp) {
    const int NH = N / 2 + 1;
    std::vector<double> tW(NH);
    window_table(N, nintp, tW.data());
    // 1/W, then the interlacing phase angles -pi i / N
    const double tpiN = (double)kTwoPiF / (double)N;
    std::vector<R> iW(2 * NH);
    for (int i = 0; i < NH; i++) {
        iW[i] = (R)(1.0 / tW[i]);
        iW[NH + i] = (R)((-tpiN / 2.0) * (double)i);
    }
    // the tables are tiny; they live in the caller's buffer and are rebuilt only
    // when (N, nintp, precision) changes
    if (wcache.N != N || wcache.nintp != nintp || wcache.rsize != (int)sizeof(R) || !wcache.buf.p) {
        PBI4G_CHECK(wcache.buf.ensure(sizeof(R) * 2 * NH));
        PBI4G_CUDA(cudaMemcpyAsync(wcache.buf.p, iW.data(), sizeof(R) * 2 * NH, cudaMemcpyHostToDevice, st));
        PBI4G_CUDA(cudaStreamSynchronize(st));
        wcache.N = N;
        wcache.nintp = nintp;
        wcache.rsize = (int)sizeof(R);
    }
    DevBuf &cache = wcache.buf;
    const double cf = fcomb_cf(interlaced, box, norm);
    if (interlaced) {
        const size_t total = (size_t)NH * NH * NH;
        fcomb_interlaced_half_kernel<R><<<grid_blocks(total, 256), 256, 0, st>>>(
            N, spec, delta, cache.as<R>(), cache.as<R>() + NH, (R)cf, bp);
    } else if (half_cells(N) < ((size_t)1 << 31)) {
        fcomb_plain_half_kernel<R, unsigned><<<grid_blocks(half_cells(N), 256), 256, 0, st>>>(
            N, spec, delta, cache.as<R>(), (R)cf, bp);
    } else {
        fcomb_plain_half_kernel<R, size_t><<<grid_blocks(half_cells(N), 256), 256, 0, st>>>(
            N, spec, delta, cache.as<R>(), (R)cf, bp);
    }
    PBI4G_LAUNCH_CHECK();
    ++*launches;
    return PBI4G_OK;
}

template int fcomb_half<float>(int, int, bool, float, double, const float2 *, float2 *, WinCache &, cudaStream_t,
                               int64_t *, const BoxPar *);
template int fcomb_half<double>(int, int, bool, float, double, const double2 *, double2 *, WinCache &, cudaStream_t,
                                int64_t *, const BoxPar *);

// ------------------------------------------------ fcomb on full grids (FP64) ---
__global__ void fcomb_interlaced_full_kernel(int N, const double2 *in, double2 *out, const double *__restrict__ tW,
                                             double cf, double piN) {
    const int NH = N / 2 + 1;
    const size_t total = (size_t)NH * NH * NH;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        const int ox = (int)(t % NH), oy = (int)((t / NH) % NH), oz = (int)(t / ((size_t)NH * NH));
        const int cx = kneg0(ox, N), cy = kneg0(oy, N), cz = kneg0(oz, N);
        Orbit<double> o;
        o.ex = ox == cx; o.ey = oy == cy; o.ez = oz == cz;
#pragma unroll
        for (int s = 0; s < 8; s++) {
            const int xs = s & 1, ys = (s >> 1) & 1, zs = s >> 2;
            const int X = xs ? cx : ox, Y = ys ? cy : oy, Z = zs ? cz : oz;
            o.v[o.key(xs, ys, zs)] = in[((size_t)Z * N + Y) * N + X];
        }
        const double cfac = cf / (tW[ox] * tW[oy] * tW[oz]);
        // the reference accumulates xrec = recx^(ix-1); the direct angle differs only by rounding
        o.combine(piN * ox, piN * oy, piN * oz, cfac);
#pragma unroll
        for (int s = 0; s < 8; s++) {
            const int xs = s & 1, ys = (s >> 1) & 1, zs = s >> 2;
            if ((xs && o.ex) || (ys && o.ey) || (zs && o.ez)) continue;
            const int X = xs ? cx : ox, Y = ys ? cy : oy, Z = zs ? cz : oz;
            out[((size_t)Z * N + Y) * N + X] = o.v[o.key(xs, ys, zs)];
        }
    }
}

__global__ void fcomb_plain_full_kernel(int N, const double2 *in, double2 *out, const double *__restrict__ tW,
                                        double cf) {
    const size_t n = (size_t)N * N * N;
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
        const int x = (int)(c % N), y = (int)((c / N) % N), z = (int)(c / ((size_t)N * N));
        double2 v = in[c];
        if (x <= N / 2) {
            const double cfac = cf / (tW[x] * tW[kabs0(y, N)] * tW[kabs0(z, N)]);
            v.x *= cfac;
            v.y *= cfac;
        }
        out[c] = v;
    }
}

int fcomb_full(int N, int nintp, bool interlaced, float box, const double2 *in, double2 *out, cudaStream_t st) {
    const int NH = N / 2 + 1;
    std::vector<double> tW(NH);
    window_table(N, nintp, tW.data());
    DevBuf dW;
    PBI4G_CHECK(dW.ensure(sizeof(double) * NH));
    PBI4G_CUDA(cudaMemcpyAsync(dW.p, tW.data(), sizeof(double) * NH, cudaMemcpyHostToDevice, st));
    const double kF3 = fcomb_kF3(box);
    if (interlaced) {
        const double tpiN = (double)kTwoPiF / (double)N;
        const size_t total = (size_t)NH * NH * NH;
        fcomb_interlaced_full_kernel<<<grid_blocks(total, 128), 128, 0, st>>>(N, in, out, dW.as<double>(),
                                                                              1.0 / (4.0 * kF3), -tpiN / 2.0);
    } else {
        fcomb_plain_full_kernel<<<grid_blocks(full_cells(N), 256), 256, 0, st>>>(N, in, out, dW.as<double>(),
                                                                                 1.0 / kF3);
    }
    PBI4G_LAUNCH_CHECK();
    PBI4G_CUDA(cudaStreamSynchronize(st));
    return PBI4G_OK;
}

// ------------------------------------------------------------ P(k) bins ---
struct PkExact {
    double kF, dk, kck;
};

// Bin index with the reference's FP64 operation sequence (powerI4.f90:549-566);
// explicit _rn intrinsics keep the compiler from contracting into FMAs.
__device__ __forceinline__ int pk_bin_exact(const PkExact &e, int kx, int ky, int kz) {
    const double rkx = __dmul_rn(e.kF, (double)kx), rky = __dmul_rn(e.kF, (double)ky), rkz = __dmul_rn(e.kF, (double)kz);
    const double s = __dadd_rn(__dadd_rn(__dmul_rn(rkx, rkx), __dmul_rn(rky, rky)), __dmul_rn(rkz, rkz));
    const double rk = __dsqrt_rn(s);
    const double t = __dsub_rn(__dsub_rn(__ddiv_rn(rk, e.dk), e.kck), DBL_MIN);
    return (int)llround(t) + 1;
}

__device__ __forceinline__ double pk_rk_exact(const PkExact &e, int kx, int ky, int kz) {
    const double rkx = __dmul_rn(e.kF, (double)kx), rky = __dmul_rn(e.kF, (double)ky), rkz = __dmul_rn(e.kF, (double)kz);
    return __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(rkx, rkx), __dmul_rn(rky, rky)), __dmul_rn(rkz, rkz)));
}

// half-space mode selection of powerI4.f90:563
__device__ __forceinline__ bool pk_keep(int x, int ky, int kz) { return x != 0 || ky > 0 || (ky == 0 && kz > 0); }

__global__ void pk_bins_kernel(int N, int nbins, PkExact e, unsigned long long *__restrict__ co,
                               double *__restrict__ sumk) {
    const int NH = N / 2 + 1;
    const size_t HC = (size_t)N * N * NH;
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < HC; c += (size_t)gridDim.x * blockDim.x) {
        const int x = (int)(c % NH), ky = kfreq0((int)((c / NH) % N), N), kz = kfreq0((int)(c / ((size_t)NH * N)), N);
        if (!pk_keep(x, ky, kz)) continue;
        const int b = pk_bin_exact(e, x, ky, kz);
        if (b < 1 || b > nbins) continue;
        atomicAdd(co + (b - 1), 1ull);
        atomicAdd(sumk + (b - 1), pk_rk_exact(e, x, ky, kz));
    }
}

__global__ void pk_bins_finish_kernel(int nbins, const unsigned long long *co, double *avgk_co) {
    for (int b = threadIdx.x; b < nbins; b += blockDim.x) avgk_co[nbins + b] = (double)co[b];
}

int PkBins::build(int N_, float box_, float kbin_, float kcenter_, int nbins_, cudaStream_t st, int64_t *launches) {
    if (N == N_ && box == box_ && kbin == kbin_ && kcenter == kcenter_ && nbins == nbins_ && lut.p) return PBI4G_OK;
    if (nbins_ < 1 || nbins_ > 65536 || !(kbin_ > 0)) return set_error(PBI4G_ERR_INVALID, "P bins: nbins=%d kbin=%g", nbins_, kbin_);
    N = N_; box = box_; kbin = kbin_; kcenter = kcenter_; nbins = nbins_;
    kF = (double)(kTwoPiF / box);
    kF3 = kF * kF * kF;
    dk = (double)kbin * kF;
    const double kck = (double)(kcenter / kbin);
    k2max = 3 * (N / 2) * (N / 2);
    std::vector<int> h(k2max + 1);
    for (int k2 = 0; k2 <= k2max; k2++) {
        double t = sqrt((double)k2) / (double)kbin - kck;
        double f = t - floor(t);
        if (fabs(f - 0.5) < 1e-7) { h[k2] = -1; continue; }
        long long b = llround(t) + 1;
        h[k2] = (b >= 1 && b <= nbins) ? (int)b : 0;
    }
    PBI4G_CHECK(lut.ensure(sizeof(int) * (k2max + 1)));
    PBI4G_CUDA(cudaMemcpyAsync(lut.p, h.data(), sizeof(int) * (k2max + 1), cudaMemcpyHostToDevice, st));
    PBI4G_CHECK(avgk_co.ensure(sizeof(double) * 2 * nbins + sizeof(unsigned long long) * nbins));
    double *sumk = avgk_co.as<double>();
    unsigned long long *co = reinterpret_cast<unsigned long long *>(sumk + 2 * nbins);
    PBI4G_CUDA(cudaMemsetAsync(avgk_co.p, 0, avgk_co.bytes, st));
    PkExact e{kF, dk, kck};
    pk_bins_kernel<<<grid_blocks(half_cells(N), 256), 256, 0, st>>>(N, nbins, e, co, sumk);
    PBI4G_LAUNCH_CHECK();
    pk_bins_finish_kernel<<<1, 256, 0, st>>>(nbins, co, sumk);
    PBI4G_LAUNCH_CHECK();
    *launches += 2;
    blocks = grid_blocks(half_cells(N), 256, 152 * 4);
    PBI4G_CHECK(partial.ensure(sizeof(double) * 3 * nbins * blocks));
    return PBI4G_OK;
}

template <class R> struct AccOf { using T = float; };
template <> struct AccOf<double> { using T = double; };

template <class R, int MODE>
__global__ void __launch_bounds__(256, sizeof(R) == 4 ? 4 : 2) pk_accum_kernel(int N, int nbins, const int *__restrict__ lut, PkExact e, double l0, double l1,
                                double l2, const typename Cx<R>::T *__restrict__ a,
                                const typename Cx<R>::T *__restrict__ b, const typename Cx<R>::T *__restrict__ c,
                                double *__restrict__ partial) {
    using A = typename AccOf<R>::T;
    extern __shared__ unsigned char smem_raw[];
    A *s = reinterpret_cast<A *>(smem_raw);
    const int nq = MODE == 0 ? 1 : 3;
    for (int i = threadIdx.x; i < nq * nbins; i += blockDim.x) s[i] = 0;
    __syncthreads();
    const int NH = N / 2 + 1;
    const int lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
    const int nwarps = gridDim.x * wpb;
    const A lf0 = (A)l0, lf1 = (A)l1, lf2 = (A)l2;
    // one warp per (y, z) row; a lane takes 4 consecutive x, along which |k| and so
    // the bin never decrease: the sums stay in registers until the bin changes.  A
    // lane's table and spectrum loads are issued together before its modes are added;
    // when N/2 would start a 128-wide step of its own (N = 256), the last lane takes
    // that Nyquist-plane mode as a fifth, after its four.
    const bool nyq_tail = N / 2 > 0 && (N / 2) % 128 == 0;
    const int xend = nyq_tail ? NH - 1 : NH;
    for (int row = blockIdx.x * wpb + (threadIdx.x >> 5); row < N * N; row += nwarps) {
        const int ky = kfreq0(row % N, N), kz = kfreq0(row / N, N);
        const int r2 = ky * ky + kz * kz;
        const size_t off = (size_t)row * NH;
        int cur = 0;
        A s0 = 0, s1 = 0, s2 = 0;
        auto flush = [&]() {
            if (cur < 1) return;
            atomicAdd(&s[cur - 1], s0);
            if (MODE != 0) {
                atomicAdd(&s[nbins + cur - 1], s1);
                atomicAdd(&s[2 * nbins + cur - 1], s2);
            }
        };
        using C = typename Cx<R>::T;
        auto add = [&](int x, int bin, C va, C vb, C vc) {
            if (bin < 1 || bin > nbins) return;
            if (bin != cur) {
                flush();
                cur = bin;
                s0 = s1 = s2 = 0;
            }
            if (MODE == 0) {
                s0 += (A)(va.x * vb.x + va.y * vb.y);
            } else if (MODE == 1) {
                const int k2 = x * x + r2;
                const A p = (A)(va.x * va.x + va.y * va.y);
                const A lk = lf0 * (A)x + lf1 * (A)ky + lf2 * (A)kz;
                const A mu2 = lk * lk / (A)k2;
                s0 += p;
                s1 += p * ((A)-0.5 + (A)1.5 * mu2);
                s2 += p * ((A)0.375 + mu2 * ((A)-3.75 + (A)4.375 * mu2));
            } else {
                s0 += (A)(va.x * va.x + va.y * va.y);
                s1 += (A)(va.x * vb.x + va.y * vb.y);
                s2 += (A)(va.x * vc.x + va.y * vc.y);
            }
        };
        auto bin_of = [&](int x) {
            if (!pk_keep(x, ky, kz)) return 0;
            int bin = lut[x * x + r2];
            if (bin < 0) bin = pk_bin_exact(e, x, ky, kz);
            return bin;
        };
        for (int x0 = 4 * lane; x0 < xend; x0 += 128) {
            int bin[4];
            C va[4], vb[4], vc[4];
#pragma unroll
            for (int t = 0; t < 4; t++) {
                const int x = x0 + t;
                const bool in = x < xend;
                bin[t] = in ? bin_of(x) : 0;
                va[t] = in ? a[off + x] : C{};
                vb[t] = (in && MODE != 1) ? b[off + x] : C{};
                vc[t] = (in && MODE == 2) ? c[off + x] : C{};
            }
#pragma unroll
            for (int t = 0; t < 4; t++) add(x0 + t, bin[t], va[t], vb[t], vc[t]);
        }
        if (nyq_tail && lane == 31) {
            const int x = NH - 1;
            add(x, bin_of(x), a[off + x], MODE != 1 ? b[off + x] : C{}, MODE == 2 ? c[off + x] : C{});
        }
        flush();
    }
    __syncthreads();
    double *out = partial + (size_t)blockIdx.x * 3 * nbins;
    for (int i = threadIdx.x; i < 3 * nbins; i += blockDim.x) out[i] = i < nq * nbins ? (double)s[i] : 0.0;
}

// Deterministic reduction over blocks (one warp per bin, fixed lane order and
// shuffle tree) + the output rows of measure_pk / measure_pk_multipoles
// (pout Fortran (5, nbins)).
__global__ void pk_finalize_kernel(int nbins, int blocks, int mode, double kF3, const double *__restrict__ partial,
                                   const double *__restrict__ avgk_co, double *__restrict__ pout) {
    const int lane = threadIdx.x & 31;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    for (int bi = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; bi < nbins; bi += warps) {
        double s0 = 0, s2 = 0, s4 = 0;
        for (int k = lane; k < blocks; k += 32) {
            const double *p = partial + (size_t)k * 3 * nbins;
            s0 += p[bi];
            s2 += p[nbins + bi];
            s4 += p[2 * nbins + bi];
        }
        for (int o = 16; o; o >>= 1) {
            s0 += __shfl_xor_sync(0xffffffffu, s0, o);
            s2 += __shfl_xor_sync(0xffffffffu, s2, o);
            s4 += __shfl_xor_sync(0xffffffffu, s4, o);
        }
        if (lane) continue;
        const double co = avgk_co[nbins + bi], avgk = avgk_co[bi];
        double *o = pout + 5 * (size_t)bi;
        o[0] = avgk / co;
        o[1] = s0 * kF3 / co;
        if (mode == 0) {
            o[2] = co;
            o[3] = 0.0;
            o[4] = 0.0;
        } else {
            o[2] = 5.0 * s2 * kF3 / co;
            o[3] = 9.0 * s4 * kF3 / co;
            o[4] = co;
        }
    }
}

template <class R>
int pk_measure(PkBins &bins, int mode, const double los[3], const typename Cx<R>::T *a, const typename Cx<R>::T *b,
               const typename Cx<R>::T *c, double *d_pout, cudaStream_t st, int64_t *launches) {
    using A = typename AccOf<R>::T;
    const int nbins = bins.nbins, N = bins.N;
    const size_t smem = sizeof(A) * (mode == 0 ? 1 : 3) * nbins;
    if (smem > 200 * 1024) return set_error(PBI4G_ERR_INVALID, "too many P bins (%d)", nbins);
    PkExact e{bins.kF, bins.dk, (double)(bins.kcenter / bins.kbin)};
    const double l0 = los ? los[0] : 0, l1 = los ? los[1] : 0, l2 = los ? los[2] : 0;
    const int blocks = bins.blocks;
    if (mode == 0) {
        auto k = pk_accum_kernel<R, 0>;
        if (smem > 48 * 1024) PBI4G_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k<<<blocks, 256, smem, st>>>(N, nbins, bins.lut.as<int>(), e, l0, l1, l2, a, b ? b : a, c,
                                     bins.partial.as<double>());
    } else if (mode == 1) {
        auto k = pk_accum_kernel<R, 1>;
        if (smem > 48 * 1024) PBI4G_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k<<<blocks, 256, smem, st>>>(N, nbins, bins.lut.as<int>(), e, l0, l1, l2, a, b, c, bins.partial.as<double>());
    } else {
        auto k = pk_accum_kernel<R, 2>;
        if (smem > 48 * 1024) PBI4G_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k<<<blocks, 256, smem, st>>>(N, nbins, bins.lut.as<int>(), e, l0, l1, l2, a, b, c, bins.partial.as<double>());
    }
    PBI4G_LAUNCH_CHECK();
    pk_finalize_kernel<<<(nbins * 32 + 255) / 256, 256, 0, st>>>(nbins, blocks, mode == 0 ? 0 : 1, bins.kF3,
                                                            bins.partial.as<double>(), bins.avgk_co.as<double>(),
                                                            d_pout);
    PBI4G_LAUNCH_CHECK();
    *launches += 2;
    return PBI4G_OK;
}

template int pk_measure<float>(PkBins &, int, const double *, const float2 *, const float2 *, const float2 *, double *,
                               cudaStream_t, int64_t *);
template int pk_measure<double>(PkBins &, int, const double *, const double2 *, const double2 *, const double2 *,
                                double *, cudaStream_t, int64_t *);

// --------------------------------------------------- q2k / q4k / reduce ---
__global__ void qlk_full_kernel(int N, double kF, const double2 *__restrict__ in, int nidx, int i0, int i1, int i2,
                                int i3, double2 *__restrict__ out) {
    const size_t n = (size_t)N * N * N;
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
        const int x = (int)(c % N), y = (int)((c / N) % N), z = (int)(c / ((size_t)N * N));
        double2 q = in[c];
        if (x <= N / 2) {
            if (x + y + z > 0) {
                const double v[3] = {kF * (double)kfreq0(x, N), kF * (double)kfreq0(y, N), kF * (double)kfreq0(z, N)};
                double rk2 = __dadd_rn(__dadd_rn(__dmul_rn(v[0], v[0]), __dmul_rn(v[1], v[1])), __dmul_rn(v[2], v[2]));
                if (nidx == 4) rk2 = rk2 * rk2;
                const int idx[4] = {i0, i1, i2, i3};
                for (int k = 0; k < nidx; k++) {
                    q.x = q.x * v[idx[k]];
                    q.y = q.y * v[idx[k]];
                }
                q.x = q.x / rk2;
                q.y = q.y / rk2;
            } else {
                q = make_double2(0.0, 0.0);
            }
        }
        out[c] = q;
    }
}

int q2k_full(int N, float box, const double2 *in, int i, int j, double2 *out, cudaStream_t st) {
    if (i < 1 || i > 3 || j < 1 || j > 3) return set_error(PBI4G_ERR_INVALID, "compute_q2k: index out of 1..3");
    qlk_full_kernel<<<grid_blocks(full_cells(N), 256), 256, 0, st>>>(N, (double)(kTwoPiF / box), in, 2, i - 1, j - 1,
                                                                      0, 0, out);
    PBI4G_LAUNCH_CHECK();
    return PBI4G_OK;
}

int q4k_full(int N, float box, const double2 *in, int i, int j, int l, int k, double2 *out, cudaStream_t st) {
    if (i < 1 || i > 3 || j < 1 || j > 3 || l < 1 || l > 3 || k < 1 || k > 3)
        return set_error(PBI4G_ERR_INVALID, "compute_q4k: index out of 1..3");
    qlk_full_kernel<<<grid_blocks(full_cells(N), 256), 256, 0, st>>>(N, (double)(kTwoPiF / box), in, 4, i - 1, j - 1,
                                                                      l - 1, k - 1, out);
    PBI4G_LAUNCH_CHECK();
    return PBI4G_OK;
}

// powerI4.f90:380-407, one thread per (ix, iy, iz) in [1, grid/2+1]^3; the four
// writes keep their order so aliased locations end with the last one.
__global__ void reduce_full_kernel(int L, const double2 *__restrict__ din, int N, double2 *__restrict__ dout) {
    const int NH = N / 2 + 1;
    const size_t total = (size_t)NH * NH * NH;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        const int x = (int)(t % NH), y = (int)((t / NH) % NH), z = (int)(t / ((size_t)NH * NH));
        const int icz = kneg0(z, L), jcz = kneg0(z, N), icy = kneg0(y, L), jcy = kneg0(y, N);
        const size_t LL = (size_t)L;
        auto src = [&](int yy, int zz) { return din[((size_t)zz * LL + yy) * LL + x]; };
        auto dst = [&](int yy, int zz) -> double2 & { return dout[((size_t)zz * N + yy) * N + x]; };
        dst(y, z) = src(y, z);
        dst(jcy, z) = src(icy, z);
        dst(y, jcz) = src(y, icz);
        dst(jcy, jcz) = src(icy, icz);
    }
}

int reduce_full(int L, const double2 *din, int N, double2 *dout, cudaStream_t st) {
    const int NH = N / 2 + 1;
    reduce_full_kernel<<<grid_blocks((size_t)NH * NH * NH, 256), 256, 0, st>>>(L, din, N, dout);
    PBI4G_LAUNCH_CHECK();
    return PBI4G_OK;
}


// ------------------------------------------- allocation-free P(k) variant ---
// Scratch of pbi4g_measure_pk_multipoles_noalloc lives in this file-scope
// device array instead of device allocations: the |k|^2 -> bin table, the
// per-bin mode counts and |k| sums, and the per-block partial sums.
constexpr int kNoAllocMaxGrid = 512;
constexpr int kNoAllocMaxBins = 512;
constexpr int kNoAllocBlocks = 304;
constexpr size_t kNoAllocLutBytes =
    ((sizeof(int) * (3 * (kNoAllocMaxGrid / 2) * (kNoAllocMaxGrid / 2) + 1) + 255) / 256) * 256;
constexpr size_t kNoAllocBinBytes = 24 * kNoAllocMaxBins;  // sum|k|, count (double), count (uint64)
constexpr size_t kNoAllocPartialBytes = sizeof(double) * 3 * kNoAllocMaxBins * kNoAllocBlocks;
constexpr size_t kNoAllocScratchBytes = kNoAllocLutBytes + kNoAllocBinBytes + kNoAllocPartialBytes;  // 4.3 MiB

static __device__ __align__(256) unsigned char g_pk_noalloc_scratch[kNoAllocScratchBytes];

// The host-side name of g_pk_noalloc_scratch is not a device address; its
// device address is looked up with the device current.  Outside stream capture
// every call looks it up again (a device reset or a new primary context gives
// the array a new address); inside a capture the call uses the address the
// last call on that device found, so the first call on a device must come
// before any capture.
static std::mutex g_noalloc_mutex;
static void *g_noalloc_ptr[128];

static int noalloc_scratch(cudaStream_t st, void **out) {
    int dev = -1;
    PBI4G_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 128) return set_error(PBI4G_ERR_UNSUPPORTED, "device index %d out of range", dev);
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    PBI4G_CUDA(cudaStreamIsCapturing(st, &cs));
    std::lock_guard<std::mutex> g(g_noalloc_mutex);
    if (cs == cudaStreamCaptureStatusNone || !g_noalloc_ptr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_pk_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return set_error(PBI4G_ERR_CUDA, "cudaGetSymbolAddress(scratch) failed: %s", cudaGetErrorString(e));
        g_noalloc_ptr[dev] = p;
    }
    *out = g_noalloc_ptr[dev];
    return PBI4G_OK;
}

// |k|^2 -> P bin table on the device (same rule as PkBins::build on the host).
__global__ void pk_lut_kernel(int k2max, double kbin, double kck, int nbins, int *__restrict__ lut) {
    for (int k2 = blockIdx.x * blockDim.x + threadIdx.x; k2 <= k2max; k2 += gridDim.x * blockDim.x) {
        const double t = sqrt((double)k2) / kbin - kck;
        const double f = t - floor(t);
        int b;
        if (fabs(f - 0.5) < 1e-7) {
            b = -1;
        } else {
            const long long bb = llround(t) + 1;
            b = (bb >= 1 && bb <= nbins) ? (int)bb : 0;
        }
        lut[k2] = b;
    }
}

}  // namespace pbi4g

extern "C" int pbi4g_measure_pk_multipoles_noalloc(int32_t grid, float box, float kbin, float kcenter, int32_t nbins,
                                                   const void *d_dcl_half, const void *d_dcl2_half,
                                                   const void *d_dcl4_half, double *d_pout, void *stream) {
    using namespace pbi4g;
    if (grid < 4 || (grid & 1)) return set_error(PBI4G_ERR_INVALID, "noalloc P(k): grid must be even and >= 4");
    if (grid > kNoAllocMaxGrid)
        return set_error(PBI4G_ERR_RANGE, "noalloc P(k): grid %d exceeds the scratch limit of %d", grid,
                         kNoAllocMaxGrid);
    if (nbins < 1 || nbins > kNoAllocMaxBins)
        return set_error(PBI4G_ERR_RANGE, "noalloc P(k): nbins %d outside 1..%d (scratch limit)", nbins,
                         kNoAllocMaxBins);
    if (!(kbin > 0) || !(box > 0)) return set_error(PBI4G_ERR_INVALID, "noalloc P(k): kbin and box must be > 0");
    if (!d_dcl_half || !d_dcl2_half || !d_dcl4_half || !d_pout)
        return set_error(PBI4G_ERR_INVALID, "noalloc P(k): null device pointer");
    cudaStream_t st = (cudaStream_t)stream;
    void *scratch = nullptr;
    PBI4G_CHECK(noalloc_scratch(st, &scratch));
    unsigned char *base = static_cast<unsigned char *>(scratch);
    int *lut = reinterpret_cast<int *>(base);
    double *sumk = reinterpret_cast<double *>(base + kNoAllocLutBytes);  // [2][nbins]: sum|k|, count
    unsigned long long *co = reinterpret_cast<unsigned long long *>(sumk + 2 * nbins);
    double *partial = reinterpret_cast<double *>(base + kNoAllocLutBytes + kNoAllocBinBytes);
    const int k2max = 3 * (grid / 2) * (grid / 2);
    const double kF = (double)(kTwoPiF / box);
    PkExact e{kF, (double)kbin * kF, (double)(kcenter / kbin)};
    // the array keeps the previous call's contents: clear the accumulators
    PBI4G_CUDA(cudaMemsetAsync(sumk, 0, kNoAllocBinBytes, st));
    pk_lut_kernel<<<grid_blocks((size_t)k2max + 1, 256, 152 * 4), 256, 0, st>>>(k2max, (double)kbin, e.kck, nbins,
                                                                                 lut);
    PBI4G_LAUNCH_CHECK();
    pk_bins_kernel<<<grid_blocks(half_cells(grid), 256), 256, 0, st>>>(grid, nbins, e, co, sumk);
    PBI4G_LAUNCH_CHECK();
    pk_bins_finish_kernel<<<1, 256, 0, st>>>(nbins, co, sumk);
    PBI4G_LAUNCH_CHECK();
    const size_t smem = sizeof(double) * 3 * nbins;
    pk_accum_kernel<double, 2><<<kNoAllocBlocks, 256, smem, st>>>(
        grid, nbins, lut, e, 0.0, 0.0, 0.0, static_cast<const double2 *>(d_dcl_half),
        static_cast<const double2 *>(d_dcl2_half), static_cast<const double2 *>(d_dcl4_half), partial);
    PBI4G_LAUNCH_CHECK();
    pk_finalize_kernel<<<(nbins * 32 + 255) / 256, 256, 0, st>>>(nbins, kNoAllocBlocks, 1, kF * kF * kF, partial,
                                                                 sumk, d_pout);
    PBI4G_LAUNCH_CHECK();
    return PBI4G_OK;
}
