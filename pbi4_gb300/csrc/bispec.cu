// bispec.cu -- shell tables, shell-filtered k-maps, CUDA-core triangle sums,
// exact triangle counts and the bispectrum output rows.
//
// Reference: bispectrumI4.f90 measure_bk (1-198), measure_bk_multipoles
// (200-516), measure_bk_cross (518-761), count_triangles (763-915).
//
// k-maps: the reference expands the kx >= 0 half spectrum to a full Hermitian
// grid, zeroes the imaginary part at the 8 self-conjugate points, and keeps the
// real part of a complex FFT of each shell-masked copy (:116-157).  The real
// part of a complex FFT equals the FFT of the input's Hermitian part, so here
// the masked half spectrum is Hermitian-symmetrised on the kx = 0 and kx = N/2
// planes and transformed with one batched C2R (cuFFT).  The reference's
// FORWARD transform and its x<->z transposed layout map x -> -x and permute
// axes; every output is a sum over all x, which neither changes.
#include "bispec.cuh"

#include <float.h>
#include <math.h>
#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

namespace pbi4g {

constexpr int kTP = 4;   // pairs per thread tile
constexpr int kTQ = 8;   // q maps per thread tile
constexpr int kGroupThreads = 256;

// ------------------------------------------------------------- Shells ---
// Smallest multiple of 4 above 3 kmax that the map transform handles fast
// (5-smooth, or 7-smooth when that is more than 5% smaller), else N.
int map_grid_for_kmax(int N, int kmax) {
    auto smooth = [](int n, int fmax) {
        for (int f : {2, 3, 5, 7})
            if (f <= fmax)
                while (n % f == 0) n /= f;
        return n == 1;
    };
    int n5 = 0, n7 = 0;
    for (int n = 4; n < N && (!n5 || !n7); n += 4) {
        if (n <= 3 * kmax) continue;
        if (!n7 && smooth(n, 7)) n7 = n;
        if (!n5 && smooth(n, 5)) n5 = n;
    }
    if (n5) return (n7 && n7 < 0.95 * n5) ? n7 : n5;
    return n7 ? n7 : N;
}

int shell_map_grid(int N, float kbin, float kcenter, int nb) {
    const double kck = (double)(kcenter / kbin);
    const int h = N / 2, k2max = 3 * h * h;
    int kmax = 0;
    for (int k2 = 0; k2 <= k2max; k2++) {
        const long long b = llround(sqrt((double)k2) / (double)kbin - kck - (double)FLT_MIN) + 1;
        if (b >= 1 && b <= nb) kmax = std::max(kmax, (int)floor(sqrt((double)k2)));
    }
    return map_grid_for_kmax(N, kmax);
}

int Shells::build(int N_, float kbin_, float kcenter_, int nb_, int iopen_, int cross_, cudaStream_t st) {
    if (N == N_ && kbin == kbin_ && kcenter == kcenter_ && nb == nb_ && iopen == iopen_ && cross == cross_ && lut.p)
        return PBI4G_OK;
    if (nb_ < 1 || nb_ > 4096 || !(kbin_ > 0) || N_ < 4 || (N_ & 1))
        return set_error(PBI4G_ERR_INVALID, "shells: grid=%d nbins=%d kbin=%g", N_, nb_, kbin_);
    N = N_; kbin = kbin_; kcenter = kcenter_; nb = nb_; iopen = iopen_; cross = cross_;
    counts.clear();
    const double kck = (double)(kcenter / kbin);
    const int h = N / 2;
    k2max = 3 * h * h;
    lut_h.assign(k2max + 1, 0);
    for (int k2 = 0; k2 <= k2max; k2++) {
        // idist = nint(dsqrt(di*di+dj*dj+dl*dl)/kbin - kcenter/kbin - tiny) + 1
        // (bispectrumI4.f90:73); di^2+dj^2+dl^2 is exact, so idist depends on k2 only.
        long long b = llround(sqrt((double)k2) / (double)kbin - kck - (double)FLT_MIN) + 1;
        lut_h[k2] = (b >= 1 && b <= nb) ? (int)b : 0;
    }
    // full-grid modes per shell: multiplicity of |k_axis| = d is 1 for d in {0, N/2}, else 2
    nmodes.assign(nb, 0);
    for (int dz = 0; dz <= h; dz++)
        for (int dy = 0; dy <= h; dy++)
            for (int dx = 0; dx <= h; dx++) {
                int b = lut_h[dx * dx + dy * dy + dz * dz];
                if (!b) continue;
                int m = (dx == 0 || dx == h ? 1 : 2) * (dy == 0 || dy == h ? 1 : 2) * (dz == 0 || dz == h ? 1 : 2);
                nmodes[b - 1] += m;
            }
    // Map grid: every shell mode has |k_axis| <= kmax, so the per-axis sum of
    // three of them lies in [-3 kmax, 3 kmax].  On any grid Nm > 3 kmax the
    // condition q1+q2+q3 = 0 (mod Nm) holds only for exact triangles; when
    // 3 kmax < N the reference's N grid has no aliased triangles either, and the
    // sum over x of three maps on the Nm grid equals the reference's sum times
    // (Nm/N)^3.  Otherwise the maps stay on the N grid.
    kmax = 0;
    for (int k2 = 0; k2 <= k2max; k2++)
        if (lut_h[k2]) kmax = std::max(kmax, (int)floor(sqrt((double)k2)));
    Nm = map_grid_for_kmax(N, kmax);
    ishift = (int)(kcenter / kbin) + (iopen ? 1 : 0);  // bispectrumI4.f90:38-42
    tri.clear();
    for (int l = 1; l <= nb; l++)
        for (int j = 1; j <= l; j++) {
            int imax = cross ? std::min(nb, j + l - 1 + ishift) : j;
            for (int i = std::max(1, l - j + 1 - ishift); i <= imax; i++) {
                tri.push_back(l);
                tri.push_back(j);
                tri.push_back(i);
            }
        }
    itot = (int64_t)tri.size() / 3;
    PBI4G_CHECK(lut.ensure(sizeof(int) * (k2max + 1)));
    PBI4G_CUDA(cudaMemcpyAsync(lut.p, lut_h.data(), sizeof(int) * (k2max + 1), cudaMemcpyHostToDevice, st));
    std::vector<double> nm(nb);
    for (int b = 0; b < nb; b++) nm[b] = (double)nmodes[b];
    PBI4G_CHECK(tri_d.ensure(sizeof(int) * std::max<size_t>(3, tri.size())));
    PBI4G_CUDA(cudaMemcpyAsync(tri_d.p, tri.data(), sizeof(int) * tri.size(), cudaMemcpyHostToDevice, st));
    PBI4G_CHECK(nmodes_d.ensure(sizeof(double) * nb));
    PBI4G_CUDA(cudaMemcpyAsync(nmodes_d.p, nm.data(), sizeof(double) * nb, cudaMemcpyHostToDevice, st));
    PBI4G_CUDA(cudaStreamSynchronize(st));
    return PBI4G_OK;
}

// ------------------------------------------------------------ TriPlan ---
// Output slot (m, s) = m * nsets + s.  Non-cross: S = sum M_i M_j Q_{s,l}, pair
// (i, j) of set-0 maps, q = map s*nb + l-1.  Cross: S = sum Q_i M_j M_l, pair
// (j, l) of set-0 maps, q = map qset*nb + i-1.
int TriPlan::build(const Shells &sh, int nsets_, int cross_, int max_pairs, int qoff) {
    nsets = nsets_;
    cross = cross_;
    const int nb = sh.nb;
    std::map<std::pair<int, int>, int> pidx;  // pair -> index in first-appearance order
    std::vector<int2> plist;
    std::vector<int> qlist;
    std::map<int, int> qidx;
    struct E { int p, q, slot; };
    std::vector<E> ents;
    for (int64_t m = 0; m < sh.itot; m++) {
        const int l = sh.tri[3 * m], j = sh.tri[3 * m + 1], i = sh.tri[3 * m + 2];
        for (int s = 0; s < nsets; s++) {
            int pa, pb, qm;
            if (!cross) { pa = i - 1; pb = j - 1; qm = qoff + s * nb + l - 1; }
            else { pa = j - 1; pb = l - 1; qm = cross * nb + i - 1; }  // cross = set index of the q field
            auto pk = std::make_pair(pb, pa);
            auto it = pidx.find(pk);
            int p;
            if (it == pidx.end()) { p = (int)plist.size(); pidx[pk] = p; plist.push_back(make_int2(pa, pb)); }
            else p = it->second;
            qidx[qm] = 0;
            ents.push_back({p, qm, (int)(m * nsets + s)});
        }
    }
    // q order: sorted map index
    for (auto &kv : qidx) { kv.second = (int)qlist.size(); qlist.push_back(kv.first); }
    for (auto &e : ents) e.q = qidx[e.q];
    np = (int)plist.size();
    nq = (int)qlist.size();
    nslots = (int)(sh.itot * nsets);
    // tiles
    std::map<std::pair<int, int>, int> tidx;
    std::vector<int4> tl;
    std::vector<int> stab;
    for (auto &e : ents) {
        auto key = std::make_pair(e.p / kTP, e.q / kTQ);
        auto it = tidx.find(key);
        int t;
        if (it == tidx.end()) {
            t = (int)tl.size();
            tidx[key] = t;
            tl.push_back(make_int4(key.first * kTP, key.second * kTQ, 0, t * kTP * kTQ));
            stab.resize(stab.size() + kTP * kTQ, -1);
        } else t = it->second;
        stab[(size_t)t * kTP * kTQ + (e.p % kTP) * kTQ + (e.q % kTQ)] = e.slot;
    }
    // Pair blocks of <= max_pairs consecutive pairs; inside a block tiles are
    // ordered (q tile, pair tile) so the threads of a warp share a q tile.
    // Groups are runs of <= kGroupThreads tiles of one block.
    std::vector<int> order(tl.size());
    for (size_t k = 0; k < order.size(); k++) order[k] = (int)k;
    const int pblk = std::max(kTP, (max_pairs / kTP) * kTP);
    std::sort(order.begin(), order.end(), [&](int a, int b) {
        const int ba = tl[a].x / pblk, bb = tl[b].x / pblk;
        if (ba != bb) return ba < bb;
        return tl[a].y != tl[b].y ? tl[a].y < tl[b].y : tl[a].x < tl[b].x;
    });
    std::vector<int4> tiles_sorted;
    std::vector<int> stab_sorted;
    std::vector<int4> gl;
    size_t k = 0;
    while (k < order.size()) {
        const int blk = tl[order[k]].x / pblk;
        size_t e = k;
        while (e < order.size() && tl[order[e]].x / pblk == blk) e++;
        for (size_t g0 = k; g0 < e; g0 += kGroupThreads) {
            const size_t g1 = std::min(e, g0 + (size_t)kGroupThreads);
            int pmin = 1 << 30, pmax = 0;
            for (size_t u = g0; u < g1; u++) {
                pmin = std::min(pmin, tl[order[u]].x);
                pmax = std::max(pmax, tl[order[u]].x + kTP);
            }
            const int t0 = (int)tiles_sorted.size();
            for (size_t u = g0; u < g1; u++) {
                int4 t = tl[order[u]];
                const int ns = (int)tiles_sorted.size();
                stab_sorted.insert(stab_sorted.end(), stab.begin() + (size_t)t.w,
                                   stab.begin() + (size_t)t.w + kTP * kTQ);
                t.z = (int)gl.size();
                t.w = ns * kTP * kTQ;
                tiles_sorted.push_back(t);
            }
            gl.push_back(make_int4(t0, (int)tiles_sorted.size(), pmin, pmax));
        }
        k = e;
    }
    ntiles = (int)tiles_sorted.size();
    ngroups = (int)gl.size();
    max_group_pairs = 0;
    for (auto &g : gl) max_group_pairs = std::max(max_group_pairs, g.w - g.z);
    // pad pair list to a multiple of kTP with a harmless pair (0,0)
    while ((int)plist.size() % kTP) plist.push_back(make_int2(0, 0));
    while ((int)qlist.size() % kTQ) qlist.push_back(qlist.empty() ? 0 : qlist[0]);
    PBI4G_CHECK(pairs.ensure(sizeof(int2) * plist.size()));
    PBI4G_CUDA(cudaMemcpy(pairs.p, plist.data(), sizeof(int2) * plist.size(), cudaMemcpyHostToDevice));
    PBI4G_CHECK(qmap.ensure(sizeof(int) * qlist.size()));
    PBI4G_CUDA(cudaMemcpy(qmap.p, qlist.data(), sizeof(int) * qlist.size(), cudaMemcpyHostToDevice));
    PBI4G_CHECK(tiles.ensure(sizeof(int4) * std::max<size_t>(1, tiles_sorted.size())));
    PBI4G_CUDA(cudaMemcpy(tiles.p, tiles_sorted.data(), sizeof(int4) * tiles_sorted.size(), cudaMemcpyHostToDevice));
    PBI4G_CHECK(slots.ensure(sizeof(int) * std::max<size_t>(1, stab_sorted.size())));
    PBI4G_CUDA(cudaMemcpy(slots.p, stab_sorted.data(), sizeof(int) * stab_sorted.size(), cudaMemcpyHostToDevice));
    PBI4G_CHECK(groups.ensure(sizeof(int4) * std::max<size_t>(1, gl.size())));
    PBI4G_CUDA(cudaMemcpy(groups.p, gl.data(), sizeof(int4) * gl.size(), cudaMemcpyHostToDevice));
    return PBI4G_OK;
}

// ------------------------------------------------------- map spectra ---
template <class C> __device__ __forceinline__ C czero() { C c; c.x = 0; c.y = 0; return c; }

constexpr int kMapChunk = 8;  // maps per block row: each block writes 8 contiguous map regions

template <class R>
__global__ void build_map_spectra_kernel(int N, int Nm, int nb, int k2max, const int *__restrict__ lut, int count,
                                         const typename Cx<R>::T *__restrict__ s0,
                                         const typename Cx<R>::T *__restrict__ s1,
                                         const typename Cx<R>::T *__restrict__ s2, int f0, int f1, int f2, double l0,
                                         double l1, double l2, typename Cx<R>::T *__restrict__ out,
                                         double *__restrict__ powsum, int pow_mask) {
    using C = typename Cx<R>::T;
    extern __shared__ double spow[];  // [3][nb] powers sum |H|^2 over the full grid, per set and shell
    if (powsum)
        for (int b = threadIdx.x; b < 3 * nb; b += blockDim.x) spow[b] = 0.0;
    __syncthreads();
    const int NH = N / 2 + 1, NHm = Nm / 2 + 1;
    const size_t HCm = (size_t)Nm * Nm * NHm;
    const int j0 = blockIdx.y * kMapChunk, j1 = min(count, j0 + kMapChunk);
    for (size_t cell = blockIdx.x * (size_t)blockDim.x + threadIdx.x; cell < HCm;
         cell += (size_t)gridDim.x * blockDim.x) {
        const int x = (int)(cell % NHm), y = (int)((cell / NHm) % Nm), z = (int)(cell / ((size_t)NHm * Nm));
        const int ky = kfreq0(y, Nm), kz = kfreq0(z, Nm);
        const int k2 = x * x + ky * ky + kz * kz;
        const int sb = k2 <= k2max ? lut[k2] : 0;
        bool any = false;
        for (int j = j0; j < j1; j++) any |= (j % nb + 1 == sb);
        if (!any) {
            for (int j = j0; j < j1; j++) out[(size_t)j * HCm + cell] = czero<C>();
            continue;
        }
        // source cell on the N grid (same signed frequency), and its mirror -k
        const int yN = ky < 0 ? ky + N : ky, zN = kz < 0 ? kz + N : kz;
        const size_t sc = ((size_t)zN * N + yN) * NH + x;
        const bool herm = (x == 0 || x == Nm / 2);
        const size_t mc = ((size_t)kneg0(zN, N) * N + kneg0(yN, N)) * NH + x;
        const double lk = l0 * x + l1 * ky + l2 * kz;
        const R mu2 = k2 > 0 ? (R)(lk * lk / (double)k2) : (R)0;
        const double wfull = herm ? 1.0 : 2.0;
        for (int j = j0; j < j1; j++) {
            const int s = j / nb, b = j % nb + 1;
            if (b != sb) {
                out[(size_t)j * HCm + cell] = czero<C>();
                continue;
            }
            const C *src = s == 0 ? s0 : (s == 1 ? s1 : s2);
            const int fac = s == 0 ? f0 : (s == 1 ? f1 : f2);
            C v = src[sc];
            if (herm) {
                const C w = src[mc];
                v.x = (v.x + w.x) * (R)0.5;
                v.y = (v.y - w.y) * (R)0.5;
            }
            R L = 1;
            if (fac == 2) L = (R)-0.5 + (R)1.5 * mu2;
            else if (fac == 4) L = (R)0.375 + mu2 * ((R)-3.75 + (R)4.375 * mu2);
            v.x *= L;
            v.y *= L;
            out[(size_t)j * HCm + cell] = v;
            if (powsum && (pow_mask >> s & 1))
                atomicAdd(&spow[s * nb + b - 1], wfull * ((double)v.x * v.x + (double)v.y * v.y));
        }
    }
    if (powsum) {
        __syncthreads();
        for (int b = threadIdx.x; b < 3 * nb; b += blockDim.x)
            if (spow[b] != 0.0) atomicAdd(powsum + b, spow[b]);
    }
}

template <class R>
int build_map_spectra(const Shells &sh, int count, const typename Cx<R>::T *const src[3], const int fac[3],
                      const double los[3], typename Cx<R>::T *out, double *powsum, int pow_mask, cudaStream_t st,
                      int64_t *launches) {
    const size_t smem = powsum ? sizeof(double) * 3 * sh.nb : 0;
    const dim3 grid(grid_blocks(half_cells(sh.Nm), 256, 152 * 2), (count + kMapChunk - 1) / kMapChunk);
    build_map_spectra_kernel<R><<<grid, 256, smem, st>>>(
        sh.N, sh.Nm, sh.nb, sh.k2max, sh.lut.as<int>(), count, src[0], src[1], src[2], fac[0], fac[1], fac[2],
        los ? los[0] : 0, los ? los[1] : 0, los ? los[2] : 0, out, powsum, pow_mask);
    PBI4G_LAUNCH_CHECK();
    ++*launches;
    return PBI4G_OK;
}

template int build_map_spectra<float>(const Shells &, int, const float2 *const[3], const int[3], const double[3],
                                      float2 *, double *, int, cudaStream_t, int64_t *);

template int build_map_spectra<double>(const Shells &, int, const double2 *const[3], const int[3], const double[3],
                                       double2 *, double *, int, cudaStream_t, int64_t *);

template <class R>
__global__ void build_indicator_kernel(int N, int k2max, const int *__restrict__ lut, int m0, int count,
                                       typename Cx<R>::T *__restrict__ out) {
    using C = typename Cx<R>::T;
    const int NH = N / 2 + 1;
    const size_t HC = (size_t)N * N * NH;
    for (size_t cell = blockIdx.x * (size_t)blockDim.x + threadIdx.x; cell < HC;
         cell += (size_t)gridDim.x * blockDim.x) {
        const int x = (int)(cell % NH), ay = kabs0((int)((cell / NH) % N), N),
                  az = kabs0((int)(cell / ((size_t)NH * N)), N);
        const int k2 = x * x + ay * ay + az * az;
        const int sb = k2 <= k2max ? lut[k2] : 0;
        for (int j = 0; j < count; j++) {
            C v = czero<C>();
            if (sb == m0 + j + 1) v.x = 1;
            out[(size_t)j * HC + cell] = v;
        }
    }
}

template <class R>
int build_indicator_spectra(const Shells &sh, int m0, int count, typename Cx<R>::T *out, cudaStream_t st,
                            int64_t *launches) {
    build_indicator_kernel<R><<<grid_blocks(half_cells(sh.Nm), 256, 152 * 8), 256, 0, st>>>(
        sh.Nm, sh.k2max, sh.lut.as<int>(), m0, count, out);
    PBI4G_LAUNCH_CHECK();
    ++*launches;
    return PBI4G_OK;
}
template int build_indicator_spectra<float>(const Shells &, int, int, float2 *, cudaStream_t, int64_t *);
template int build_indicator_spectra<double>(const Shells &, int, int, double2 *, cudaStream_t, int64_t *);

// ------------------------------------------------------ triangle sums ---
// CUDA-core form (FP32 plain / FP64).  Each CTA owns a group of register
// tiles (kTP pairs x kTQ q maps per thread) and a contiguous range of the
// contraction (grid points).  Per chunk of kc points inside one grid row the
// CTA stages the q maps and the pair-source maps in shared memory (k
// contiguous), forms the pair products, then every thread runs its tile.
// FP32 chunk sums are folded into Kahan-compensated running sums.
template <class T> struct VecOf;
template <> struct VecOf<float> { static constexpr int W = 4; using V = float4; using V2 = float2; };
template <> struct VecOf<double> { static constexpr int W = 2; using V = double2; using V2 = double2; };

template <class T> __device__ __forceinline__ void vload(const T *p, T v[VecOf<T>::W]);
template <> __device__ __forceinline__ void vload<float>(const float *p, float v[4]) {
    const float4 a = *reinterpret_cast<const float4 *>(p);
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
}
template <> __device__ __forceinline__ void vload<double>(const double *p, double v[2]) {
    const double2 a = *reinterpret_cast<const double2 *>(p);
    v[0] = a.x; v[1] = a.y;
}

// Accumulation of one chunk into the running sum: Kahan-compensated for FP32.
template <class T> struct Runner {
    T sum = 0, comp = 0;
    __device__ __forceinline__ void add(T v) {
        T y = v - comp;
        T t = sum + y;
        comp = (t - sum) - y;
        sum = t;
    }
};
template <> struct Runner<double> {
    double sum = 0, comp = 0;
    __device__ __forceinline__ void add(double v) { sum += v; }
};

constexpr int kKCmax = 64;

// Shared layout (k-major, the tile index contiguous): sQ[k][q], sP[k][p], so a
// warp whose threads share one q tile reads it by broadcast and reads its
// consecutive pair tiles as one contiguous 512-byte row segment.
template <class T>
__global__ void __launch_bounds__(kGroupThreads) trisum_kernel(
    int N, int kc, const T *__restrict__ maps, size_t mstride, int rs, int nb, int nq, const int *__restrict__ qmap,
    const int2 *__restrict__ pairs, const int4 *__restrict__ tiles, const int4 *__restrict__ groups,
    const int *__restrict__ slots, int ngroups, int ksplit, long long K, int nslots, double *__restrict__ partial,
    int qrow, int prow) {
    using V2 = typename VecOf<T>::V2;
    constexpr int ARS = kKCmax + (sizeof(T) == 4 ? 4 : 2);  // sA row stride (k contiguous)
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int g = blockIdx.x % ngroups, split = blockIdx.x / ngroups;
    const int4 G = groups[g];
    const int ntile = G.y - G.x, p0g = G.z, npg = G.w - G.z;
    T *sQ = reinterpret_cast<T *>(smem_raw);  // [kKCmax][qrow]
    T *sP = sQ + (size_t)kKCmax * qrow;       // [kKCmax][prow]
    T *sA = sP + (size_t)kKCmax * prow;       // [nb][ARS]
    const int my = threadIdx.x;
    int4 tile = make_int4(0, 0, 0, 0);
    if (my < ntile) tile = tiles[G.x + my];
    const int tp = tile.x - p0g, tq = tile.y;

    const long long nchunks = K / kc;
    const long long cb = nchunks * split / ksplit, ce = nchunks * (split + 1) / ksplit;

    T acc[kTP][kTQ];
    Runner<T> run[kTP][kTQ];
#pragma unroll
    for (int a = 0; a < kTP; a++)
#pragma unroll
        for (int b = 0; b < kTQ; b++) acc[a][b] = 0;

    const int hv = kc / 2;  // vec2 loads per staged row
    for (long long ch = cb; ch < ce; ch++) {
        const long long k0 = ch * kc;
        for (int idx = threadIdx.x; idx < (nq + nb) * hv; idx += blockDim.x) {
            const int m = idx / hv, c = idx - m * hv;
            const int map = m < nq ? qmap[m] : m - nq;
            // N is even, so a pair of points never straddles a grid row
            const long long p = k0 + 2 * c;
            const V2 v = *reinterpret_cast<const V2 *>(maps + (size_t)map * mstride + (size_t)(p / N) * rs +
                                                       (size_t)(p % N));
            if (m < nq) {
                sQ[(size_t)(2 * c) * qrow + m] = v.x;
                sQ[(size_t)(2 * c + 1) * qrow + m] = v.y;
            } else {
                T *dst = sA + (size_t)(m - nq) * ARS + 2 * c;
                dst[0] = v.x;
                dst[1] = v.y;
            }
        }
        __syncthreads();
        for (int idx = threadIdx.x; idx < npg * kc; idx += blockDim.x) {
            const int pp = idx % npg, k = idx / npg;
            const int2 pr = pairs[p0g + pp];
            sP[(size_t)k * prow + pp] = sA[(size_t)pr.x * ARS + k] * sA[(size_t)pr.y * ARS + k];
        }
        __syncthreads();
        if (my < ntile) {
#pragma unroll 4
            for (int kk = 0; kk < kc; kk++) {
                T av[kTP], qv[kTQ];
                vload<T>(sP + (size_t)kk * prow + tp, av);
                if (VecOf<T>::W == 2) vload<T>(sP + (size_t)kk * prow + tp + 2, av + 2);
#pragma unroll
                for (int b = 0; b < kTQ; b += VecOf<T>::W) vload<T>(sQ + (size_t)kk * qrow + tq + b, qv + b);
#pragma unroll
                for (int a = 0; a < kTP; a++)
#pragma unroll
                    for (int b = 0; b < kTQ; b++) acc[a][b] = fma(av[a], qv[b], acc[a][b]);
            }
#pragma unroll
            for (int a = 0; a < kTP; a++)
#pragma unroll
                for (int b = 0; b < kTQ; b++) {
                    run[a][b].add(acc[a][b]);
                    acc[a][b] = 0;
                }
        }
        __syncthreads();
    }
    if (my < ntile) {
        const int *st = slots + tile.w;
#pragma unroll
        for (int a = 0; a < kTP; a++)
#pragma unroll
            for (int b = 0; b < kTQ; b++) {
                const int s = st[a * kTQ + b];
                if (s >= 0) partial[(size_t)split * nslots + s] = (double)run[a][b].sum - (double)run[a][b].comp;
            }
    }
}

__global__ void reduce_partial_kernel(int nslots, int ksplit, const double *__restrict__ partial,
                                      double *__restrict__ S, int accumulate) {
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nslots; s += gridDim.x * blockDim.x) {
        double v = 0;
        for (int k = 0; k < ksplit; k++) v += partial[(size_t)k * nslots + s];
        S[s] = accumulate ? S[s] + v : v;
    }
}

int reduce_partials(int nslots, int ksplit, const double *partial, double *S, bool accumulate, cudaStream_t st) {
    reduce_partial_kernel<<<(nslots + 255) / 256, 256, 0, st>>>(nslots, ksplit, partial, S, accumulate ? 1 : 0);
    PBI4G_LAUNCH_CHECK();
    return PBI4G_OK;
}

template <class T>
int triangle_sums(const Shells &sh, const TriPlan &tp, const T *maps, size_t mstride, int rowlen, int rs,
                  long long K, DevBuf &partial, double *S, bool accumulate, cudaStream_t st, int64_t *launches) {
    const int N = rowlen;
    int kc = kKCmax;
    while (kc > 4 && K % kc) kc /= 2;
    if (K < 1 || K % kc || (N & 1) || (rs & 1) || (mstride & 1))
        return set_error(PBI4G_ERR_UNSUPPORTED, "triangle sums: %lld points in rows of %d have no even chunk width",
                         K, N);
    const int qpad = ((tp.nq + kTQ - 1) / kTQ) * kTQ;  // q tiles read up to 8 columns per tile
    const int gpad = ((tp.max_group_pairs + kTP - 1) / kTP) * kTP;
    const int qrow = qpad + 4, prow = gpad + 4;          // 16-B aligned rows, staggered banks
    const int ARS = kKCmax + (sizeof(T) == 4 ? 4 : 2);
    const size_t smem = sizeof(T) * ((size_t)kKCmax * (qrow + prow) + (size_t)sh.nb * ARS);
    if (smem > 220 * 1024) return set_error(PBI4G_ERR_UNSUPPORTED, "triangle sums: %zu B shared memory", smem);
    const int target = 152 * 2;
    int ksplit = std::max(1, target / std::max(1, tp.ngroups));
    ksplit = (int)std::min<long long>(ksplit, std::max<long long>(1, K / kc / 8));
    PBI4G_CHECK(partial.ensure(sizeof(double) * (size_t)ksplit * tp.nslots));
    auto kern = trisum_kernel<T>;
    PBI4G_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kern<<<tp.ngroups * ksplit, kGroupThreads, smem, st>>>(
        N, kc, maps, mstride, rs, sh.nb, qpad, tp.qmap.as<int>(), tp.pairs.as<int2>(), tp.tiles.as<int4>(),
        tp.groups.as<int4>(), tp.slots.as<int>(), tp.ngroups, ksplit, K, tp.nslots, partial.as<double>(), qrow, prow);
    PBI4G_LAUNCH_CHECK();
    PBI4G_CHECK(reduce_partials(tp.nslots, ksplit, partial.as<double>(), S, accumulate, st));
    *launches += 2;
    return PBI4G_OK;
}

template int triangle_sums<float>(const Shells &, const TriPlan &, const float *, size_t, int, int, long long,
                                  DevBuf &, double *, bool, cudaStream_t, int64_t *);
template int triangle_sums<double>(const Shells &, const TriPlan &, const double *, size_t, int, int, long long,
                                   DevBuf &, double *, bool, cudaStream_t, int64_t *);

// ------------------------------------------------------------ outputs ---
__global__ void bk_finalize_kernel(int64_t itot, int nb, int nsets, int cross, const int *__restrict__ tri,
                                   const double *__restrict__ S, const double *__restrict__ powsum,
                                   const double *__restrict__ nmodes, double kf3, double powSN, double gridD,
                                   double kcenter, double kbin, const float *__restrict__ counts,
                                   double *__restrict__ bout, double sfac, const BoxPar *__restrict__ bp) {
    if (bp) powSN = bp->pow_sn;
    const double powSN2 = powSN * powSN;
    for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < itot; m += (int64_t)gridDim.x * blockDim.x) {
        const int l = tri[3 * m], j = tri[3 * m + 1], i = tri[3 * m + 2];
        const double c = (double)counts[m];
        const double tl = kcenter + (double)(l - 1) * kbin, tj = kcenter + (double)(j - 1) * kbin,
                     ti = kcenter + (double)(i - 1) * kbin;
        if (cross) {
            double *o = bout + 5 * m;
            o[0] = tl; o[1] = tj; o[2] = ti;
            o[3] = kf3 * (sfac * S[m * nsets]) / c;
            o[4] = (double)(float)(c / gridD);
            continue;
        }
        // pow(i) = kf3*avg/dble(gridd)/dble(nmodes) - powSN, avg = sum_x m^2 = gridD * sum_k |H|^2
        auto pw = [&](int b) { return kf3 * (gridD * powsum[b - 1]) / gridD / nmodes[b - 1] - powSN; };
        const double pl = pw(l), pj = pw(j), pi = pw(i);
        const double bispSN = (pi + pj + pl) * powSN + powSN2;
        const int rows = nsets == 3 ? 11 : 9;
        double *o = bout + (size_t)rows * m;
        o[0] = tl; o[1] = tj; o[2] = ti;
        o[3] = pl; o[4] = pj; o[5] = pi;
        o[6] = kf3 * (sfac * S[m * nsets]) / c + bispSN;
        o[7] = bispSN;
        o[8] = (double)(float)(c / gridD);
        if (nsets == 3) {
            o[9] = 5 * kf3 * (sfac * S[m * nsets + 1]) / c;
            o[10] = 9 * kf3 * (sfac * S[m * nsets + 2]) / c;
        }
    }
}

double bk_pow_sn(float kf, int64_t npart) {
    const float kf3f = kf * kf * kf;
    return 1.0 / (double)npart / (double)kf3f;
}

int bk_finalize(const Shells &sh, int nsets, int cross, const double *S, const double *powsum, float kf,
                int64_t npart, const float *counts_f32, double *bout, cudaStream_t st, int64_t *launches,
                const BoxPar *bp) {
    const float kf3f = kf * kf * kf;
    const double kf3 = (double)kf3f;
    const double powSN = bk_pow_sn(kf, npart);
    const double gridD = (double)sh.N * sh.N * sh.N;
    bk_finalize_kernel<<<grid_blocks(sh.itot, 128), 128, 0, st>>>(
        sh.itot, sh.nb, nsets, cross, sh.tri_d.as<int>(), S, powsum, sh.nmodes_d.as<double>(), kf3, powSN, gridD,
        (double)sh.kcenter, (double)sh.kbin, counts_f32, bout,
        // the sums were taken over the Nm^3 map grid: the reference sums over N^3
        ((double)sh.N / sh.Nm) * ((double)sh.N / sh.Nm) * ((double)sh.N / sh.Nm), bp);
    PBI4G_LAUNCH_CHECK();
    ++*launches;
    return PBI4G_OK;
}

// ------------------------------------------------------------- counts ---
// Counts depend only on (grid, kbin, kcenter, nbins, iopen, cross): one
// process-wide copy per binning serves every plan that uses it.
static std::mutex g_counts_mutex;
static std::map<std::tuple<int, float, float, int, int, int>, std::vector<int64_t>> g_counts_cache;

static int upload_counts(Shells &sh) {
    const double gridD = (double)sh.N * sh.N * sh.N;
    std::vector<float> c32(sh.itot);
    for (int64_t m = 0; m < sh.itot; m++) c32[m] = (float)(gridD * (double)sh.counts[m]);
    PBI4G_CHECK(sh.counts_f32.ensure(sizeof(float) * std::max<int64_t>(1, sh.itot)));
    PBI4G_CUDA(cudaMemcpy(sh.counts_f32.p, c32.data(), sizeof(float) * sh.itot, cudaMemcpyHostToDevice));
    return PBI4G_OK;
}

// Orbit representatives of the map grid under the cube group (the 48 axis
// permutations and sign flips, x_a -> -x_a mod Nm).  A shell indicator map
// I_b(x) = sum over the shell's modes of e^{2 pi i k.x / Nm} is invariant under
// the group (the shell is a set of |k|, and Nm / 2 is no shell frequency since
// Nm > 3 kmax), so sum_x I_l I_j I_i = sum over representatives (a <= b <= c,
// each in [0, Nm/2]) of |orbit| I_l I_j I_i, with |orbit| = 2 per coordinate
// outside {0, Nm/2} times the distinct permutations of (a, b, c) (6, 3 or 1).
// Representatives are packed a | b << 11 | c << 22 and padded with weight-0
// points to a multiple of 64.
static int orbit_points(int Nm, std::vector<unsigned> &pts, long long &nrep) {
    const int h = Nm / 2;
    pts.clear();
    long long wsum = 0;
    for (int a = 0; a <= h; a++)
        for (int b = a; b <= h; b++)
            for (int c = b; c <= h; c++) {
                pts.push_back((unsigned)a | ((unsigned)b << 11) | ((unsigned)c << 22));
                const int sg = (a == 0 || a == h ? 1 : 2) * (b == 0 || b == h ? 1 : 2) * (c == 0 || c == h ? 1 : 2);
                const int pm = (a == b && b == c) ? 1 : ((a == b || b == c) ? 3 : 6);
                wsum += (long long)sg * pm;
            }
    nrep = (long long)pts.size();
    if (wsum != (long long)Nm * Nm * Nm)
        return set_error(PBI4G_ERR_UNSUPPORTED, "orbit weights of grid %d sum to %lld", Nm, wsum);
    while (pts.size() % 64) pts.push_back(0u);
    return PBI4G_OK;
}

__device__ __forceinline__ double orbit_weight(unsigned pk, int h) {
    const int a = pk & 2047, b = (pk >> 11) & 2047, c = pk >> 22;
    const int sg = (a == 0 || a == h ? 1 : 2) * (b == 0 || b == h ? 1 : 2) * (c == 0 || c == h ? 1 : 2);
    const int pm = (a == b && b == c) ? 1 : ((a == b || b == c) ? 3 : 6);
    return (double)(sg * pm);
}

// maps [m0, m0 + count) of the in-place C2R output (map j at real + j * 2 HC,
// point (a, b, c) at (a Nm + b) (2 NH) + c) at the representatives:
// out[m][p] = I_m(rep p), out[nb + m][p] = |orbit p| I_m(rep p)
__global__ void orbit_gather_kernel(int Nm, int nb, int m0, int count, long long nrep, long long npad,
                                    const unsigned *__restrict__ pts, const double *__restrict__ real,
                                    double *__restrict__ out) {
    const int NH = Nm / 2 + 1;
    const size_t HC2 = 2 * (size_t)Nm * Nm * NH;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npad;
         p += (long long)gridDim.x * blockDim.x) {
        const unsigned pk = pts[p];
        const bool real_pt = p < nrep;
        const double w = real_pt ? orbit_weight(pk, Nm / 2) : 0.0;
        const size_t off = ((size_t)(pk & 2047) * Nm + ((pk >> 11) & 2047)) * (2 * NH) + (pk >> 22);
        for (int j = 0; j < count; j++) {
            const double v = real_pt ? real[(size_t)j * HC2 + off] : 0.0;
            out[(size_t)(m0 + j) * npad + p] = v;
            out[(size_t)(nb + m0 + j) * npad + p] = w * v;
        }
    }
}

int triangle_counts(Shells &sh, cudaStream_t st, int64_t *launches) {
    if (!sh.counts.empty()) return PBI4G_OK;
    const auto ckey = std::make_tuple(sh.N, sh.kbin, sh.kcenter, sh.nb, sh.iopen, sh.cross);
    {
        std::lock_guard<std::mutex> g(g_counts_mutex);
        auto it = g_counts_cache.find(ckey);
        if (it != g_counts_cache.end()) {
            sh.counts = it->second;
            return upload_counts(sh);
        }
    }
    const int N = sh.Nm, nb = sh.nb, NH = N / 2 + 1;  // indicator maps on the map grid
    if (N > 2046) return set_error(PBI4G_ERR_UNSUPPORTED, "counts: map grid %d", N);
    const size_t HC = half_cells(N);
    std::vector<unsigned> hpts;
    long long nrep = 0;
    PBI4G_CHECK(orbit_points(N, hpts, nrep));
    const long long npad = (long long)hpts.size();
    DevBuf pts, rep, spec, partial, S;
    PBI4G_CHECK(pts.ensure(sizeof(unsigned) * hpts.size()));
    PBI4G_CUDA(cudaMemcpyAsync(pts.p, hpts.data(), sizeof(unsigned) * hpts.size(), cudaMemcpyHostToDevice, st));
    PBI4G_CHECK(rep.ensure(sizeof(double) * 2 * (size_t)nb * npad));
    // indicator spectra and their FP64 C2R in batches of at most 4 GiB
    const int bsz = (int)std::max<size_t>(1, std::min<size_t>((size_t)nb, ((size_t)4 << 30) / (sizeof(double2) * HC)));
    PBI4G_CHECK(spec.ensure(sizeof(double2) * HC * bsz));
    int n[3] = {N, N, N}, inembed[3] = {N, N, NH}, onembed[3] = {N, N, 2 * NH};
    cufftHandle plan = 0;
    int plan_batch = 0;
    int rc = PBI4G_OK;
    for (int m0 = 0; m0 < nb && rc == PBI4G_OK; m0 += bsz) {
        const int cnt = std::min(bsz, nb - m0);
        if ((rc = build_indicator_spectra<double>(sh, m0, cnt, spec.as<double2>(), st, launches))) break;
        if (plan_batch != cnt) {
            if (plan) cufftDestroy(plan);
            plan = 0;
            if (cufftPlanMany(&plan, 3, n, inembed, 1, (int)HC, onembed, 1, (int)(2 * HC), CUFFT_Z2D, cnt) !=
                CUFFT_SUCCESS) {
                plan = 0;
                rc = set_error(PBI4G_ERR_CUFFT, "counts: cufftPlanMany (%d maps of grid %d)", cnt, N);
                break;
            }
            plan_batch = cnt;
        }
        cufftSetStream(plan, st);
        const cufftResult r = cufftExecZ2D(plan, spec.as<cufftDoubleComplex>(), spec.as<cufftDoubleReal>());
        if (r != CUFFT_SUCCESS) {
            rc = set_error(PBI4G_ERR_CUFFT, "counts: cufftExecZ2D failed (%d)", (int)r);
            break;
        }
        orbit_gather_kernel<<<grid_blocks((size_t)npad, 256, 152 * 8), 256, 0, st>>>(
            N, nb, m0, cnt, nrep, npad, pts.as<unsigned>(), spec.as<double>(), rep.as<double>());
        if (cudaPeekAtLastError() != cudaSuccess) {
            rc = set_error(PBI4G_ERR_CUDA, "counts: gather launch: %s", cudaGetErrorString(cudaGetLastError()));
            break;
        }
        ++*launches;
    }
    if (plan) {
        cudaStreamSynchronize(st);
        cufftDestroy(plan);
    }
    PBI4G_CHECK(rc);
    spec.release();
    // all three factors are indicator maps of the same set (also for the cross
    // enumeration, bispectrumI4.f90:887-896), so the non-cross pair layout
    // applies: pairs from the plain copies [0, nb), q from the weighted copies
    TriPlan tp;
    PBI4G_CHECK(tp.build(sh, 1, 0, 128, nb));
    PBI4G_CHECK(S.ensure(sizeof(double) * tp.nslots));
    PBI4G_CHECK(triangle_sums<double>(sh, tp, rep.as<double>(), (size_t)npad, 64, 64, npad, partial, S.as<double>(),
                                      false, st, launches));
    std::vector<double> Sh(tp.nslots);
    PBI4G_CUDA(cudaMemcpyAsync(Sh.data(), S.p, sizeof(double) * tp.nslots, cudaMemcpyDeviceToHost, st));
    PBI4G_CUDA(cudaStreamSynchronize(st));
    const double gridD = (double)N * N * N;
    sh.counts.resize(sh.itot);
    double maxdev = 0;
    for (int64_t m = 0; m < sh.itot; m++) {
        double v = Sh[m] / gridD;
        long long c = llround(v);
        maxdev = std::max(maxdev, fabs(v - (double)c));
        sh.counts[m] = c;
    }
    if (maxdev > 0.25) {
        sh.counts.clear();
        return set_error(PBI4G_ERR_RANGE, "triangle counts not resolved to integers (max deviation %g)", maxdev);
    }
    {
        std::lock_guard<std::mutex> g(g_counts_mutex);
        g_counts_cache[ckey] = sh.counts;
    }
    return upload_counts(sh);
}

}  // namespace pbi4g
