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
    // smallest multiple of 4 above 3 kmax that cuFFT handles fast: 5-smooth,
    // or 7-smooth when that is more than 5% smaller
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
    Nm = N;
    if (n5) Nm = (n7 && n7 < 0.95 * n5) ? n7 : n5;
    else if (n7) Nm = n7;
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
int TriPlan::build(const Shells &sh, int nsets_, int cross_, int max_pairs) {
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
            if (!cross) { pa = i - 1; pb = j - 1; qm = s * nb + l - 1; }
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

// ---------------------------------------------- pruned map spectra (FP32) ---
// The spectra of all maps as planes [m][kx][z][y] with kx < KX: every mode of
// every shell has kx <= kmax < KX, so the planes kx >= KX (and the Nyquist
// plane) are zero and are neither stored nor transformed.  The same mask,
// multipole factor, Hermitian symmetrisation and shell powers as
// build_map_spectra_kernel.  Threads run along y, so the writes are coalesced;
// the reads of delta(k) (one N-grid half spectrum) stay in L2.
__global__ void build_map_cols_kernel(int N, int Nm, int KX, int nb, int k2max, const int *__restrict__ lut, int count,
                                      const float2 *__restrict__ s0, const float2 *__restrict__ s1,
                                      const float2 *__restrict__ s2, int f0, int f1, int f2, double l0, double l1,
                                      double l2, float2 *__restrict__ out, double *__restrict__ powsum, int pow_mask) {
    extern __shared__ double spow[];  // [3][nb]
    if (powsum)
        for (int b = threadIdx.x; b < 3 * nb; b += blockDim.x) spow[b] = 0.0;
    __syncthreads();
    const int NH = N / 2 + 1;
    const size_t plane = (size_t)Nm * Nm, cells = plane * KX;
    const int j0 = blockIdx.y * kMapChunk, j1 = min(count, j0 + kMapChunk);
    for (size_t cell = blockIdx.x * (size_t)blockDim.x + threadIdx.x; cell < cells;
         cell += (size_t)gridDim.x * blockDim.x) {
        const int x = (int)(cell / plane);
        const size_t row = cell - (size_t)x * plane;  // z * Nm + y
        const int y = (int)(row % Nm), z = (int)(row / Nm);
        const int ky = kfreq0(y, Nm), kz = kfreq0(z, Nm);
        const int k2 = x * x + ky * ky + kz * kz;
        const int sb = k2 <= k2max ? lut[k2] : 0;
        float2 *o = out + (size_t)x * plane + row;  // + j * KX * plane for map j
        const size_t mstr = (size_t)KX * plane;
        bool any = false;
        for (int j = j0; j < j1; j++) any |= (j % nb + 1 == sb);
        if (!any) {
            for (int j = j0; j < j1; j++) o[(size_t)j * mstr] = make_float2(0.f, 0.f);
            continue;
        }
        const int yN = ky < 0 ? ky + N : ky, zN = kz < 0 ? kz + N : kz;
        const size_t sc = ((size_t)zN * N + yN) * NH + x;
        const bool herm = x == 0;
        const size_t mc = ((size_t)kneg0(zN, N) * N + kneg0(yN, N)) * NH + x;
        const double lk = l0 * x + l1 * ky + l2 * kz;
        const float mu2 = k2 > 0 ? (float)(lk * lk / (double)k2) : 0.f;
        const double wfull = herm ? 1.0 : 2.0;
        for (int j = j0; j < j1; j++) {
            const int s = j / nb, b = j % nb + 1;
            if (b != sb) {
                o[(size_t)j * mstr] = make_float2(0.f, 0.f);
                continue;
            }
            const float2 *src = s == 0 ? s0 : (s == 1 ? s1 : s2);
            const int fac = s == 0 ? f0 : (s == 1 ? f1 : f2);
            float2 v = src[sc];
            if (herm) {
                const float2 w = src[mc];
                v.x = (v.x + w.x) * 0.5f;
                v.y = (v.y - w.y) * 0.5f;
            }
            float L = 1.f;
            if (fac == 2) L = -0.5f + 1.5f * mu2;
            else if (fac == 4) L = 0.375f + mu2 * (-3.75f + 4.375f * mu2);
            v.x *= L;
            v.y *= L;
            o[(size_t)j * mstr] = v;
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

int build_map_cols(const Shells &sh, int count, int KX, const float2 *const src[3], const int fac[3],
                   const double los[3], float2 *out, double *powsum, int pow_mask, cudaStream_t st,
                   int64_t *launches) {
    const size_t smem = powsum ? sizeof(double) * 3 * sh.nb : 0;
    const dim3 grid(grid_blocks((size_t)sh.Nm * sh.Nm * KX, 256, 152 * 2), (count + kMapChunk - 1) / kMapChunk);
    build_map_cols_kernel<<<grid, 256, smem, st>>>(sh.N, sh.Nm, KX, sh.nb, sh.k2max, sh.lut.as<int>(), count, src[0],
                                                   src[1], src[2], fac[0], fac[1], fac[2], los ? los[0] : 0,
                                                   los ? los[1] : 0, los ? los[2] : 0, out, powsum, pow_mask);
    PBI4G_LAUNCH_CHECK();
    ++*launches;
    return PBI4G_OK;
}

// The last (x) pass of the inverse 3D transform, after the (z, y) passes, on
// planes kx < KX of Hermitian rows: x[n] = sum_k X[k] e^{+2 pi i k n / Nm} with
// X[Nm - k] = conj X[k] (cuFFT's C2R convention).  With M = Nm / 2,
// E[k] = X[k] + conj X[M-k] and O[k] = (X[k] - conj X[M-k]) e^{2 pi i k / Nm},
// z = IDFT_M(E + i O) gives x[2m] = Re z[m], x[2m+1] = Im z[m].  A CTA takes 32
// rows (one map, 32 consecutive (y, z)): it loads their KX coefficients with
// coalesced reads along y, runs a mixed-radix Stockham FFT of the 32 rows
// together in shared memory ([k][row], rows fastest), and writes each row with
// one warp.
namespace {
__constant__ float2 c_roots[9][8];  // e^{2 pi i t / R} for R = 2..8
constexpr int kXRows = 32;
constexpr int kXPitch = kXRows + 1;  // padded [k][row] pitch of the shared tiles

__device__ __forceinline__ float2 cadd2(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub2(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul2(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 itimes(float2 a) { return make_float2(-a.y, a.x); }  // i a

// inverse (e^{+2 pi i q r / R}) DFT of R points in place
template <int R>
__device__ __forceinline__ void dft_small(float2 (&v)[8]) {
    if constexpr (R == 2) {
        const float2 a = v[0], b = v[1];
        v[0] = cadd2(a, b);
        v[1] = csub2(a, b);
    } else if constexpr (R == 3) {
        const float c = -0.5f, sn = 0.8660254037844386f;
        const float2 b = cadd2(v[1], v[2]), d = csub2(v[1], v[2]);
        const float2 t = make_float2(v[0].x + c * b.x, v[0].y + c * b.y);
        const float2 u = itimes(make_float2(sn * d.x, sn * d.y));
        v[0] = cadd2(v[0], b);
        v[1] = cadd2(t, u);
        v[2] = csub2(t, u);
    } else if constexpr (R == 4) {
        const float2 s02 = cadd2(v[0], v[2]), d02 = csub2(v[0], v[2]);
        const float2 s13 = cadd2(v[1], v[3]), d13 = itimes(csub2(v[1], v[3]));
        v[0] = cadd2(s02, s13);
        v[2] = csub2(s02, s13);
        v[1] = cadd2(d02, d13);
        v[3] = csub2(d02, d13);
    } else if constexpr (R == 5) {
        const float c1 = 0.30901699437494745f, c2 = -0.8090169943749475f;
        const float s1 = 0.9510565162951535f, s2 = 0.5877852522924731f;
        const float2 b1 = cadd2(v[1], v[4]), b2 = cadd2(v[2], v[3]);
        const float2 d1 = csub2(v[1], v[4]), d2 = csub2(v[2], v[3]);
        const float2 t1 = make_float2(v[0].x + c1 * b1.x + c2 * b2.x, v[0].y + c1 * b1.y + c2 * b2.y);
        const float2 t2 = make_float2(v[0].x + c2 * b1.x + c1 * b2.x, v[0].y + c2 * b1.y + c1 * b2.y);
        const float2 u1 = itimes(make_float2(s1 * d1.x + s2 * d2.x, s1 * d1.y + s2 * d2.y));
        const float2 u2 = itimes(make_float2(s2 * d1.x - s1 * d2.x, s2 * d1.y - s1 * d2.y));
        v[0] = cadd2(v[0], cadd2(b1, b2));
        v[1] = cadd2(t1, u1);
        v[4] = csub2(t1, u1);
        v[2] = cadd2(t2, u2);
        v[3] = csub2(t2, u2);
    } else {
        float2 o[R];
#pragma unroll
        for (int q = 0; q < R; q++) {
            float2 acc = v[0];
#pragma unroll
            for (int r = 1; r < R; r++) acc = cadd2(acc, cmul2(v[r], c_roots[R][(q * r) % R]));
            o[q] = acc;
        }
#pragma unroll
        for (int q = 0; q < R; q++) v[q] = o[q];
    }
}

// one Stockham stage over the 32 rows of the tile: warp w takes butterflies
// j = w, w + nwarps, ..., its lanes the rows (uniform j, twiddles broadcast)
template <int R>
__device__ __forceinline__ void stockham_stage(const float2 *__restrict__ b0, float2 *__restrict__ b1,
                                               const float2 *__restrict__ tw, int M, int Ns, int warp, int nw,
                                               int lane) {
    const int nj = M / R, tstep = 2 * (M / (Ns * R));  // twiddle e^{2 pi i jn r / (Ns R)} = tw[jn r tstep]
    for (int j = warp; j < nj; j += nw) {
        float2 v[8];
        const int jq = j / Ns, jn = j - jq * Ns;
#pragma unroll
        for (int r = 0; r < R; r++) {
            const float2 a = b0[(j + r * nj) * kXPitch + lane];
            v[r] = r > 0 ? cmul2(a, tw[jn * r * tstep]) : a;
        }
        dft_small<R>(v);
        const int base = jq * Ns * R + jn;
#pragma unroll
        for (int r = 0; r < R; r++) b1[(base + r * Ns) * kXPitch + lane] = v[r];
    }
}
}  // namespace

struct XPassPlan {
    int M = 0, nst = 0, rad[12] = {0};
};

// PF: rows of X a warp prefetches into registers for the next tile (KX <= PF * warps)
template <int PF>
__global__ void c2r_rows_kernel(const float2 *__restrict__ cols, float *__restrict__ out,
                                const float2 *__restrict__ tw_g, XPassPlan xp, int Nm, int KX, int count,
                                int dense) {
    extern __shared__ float2 sx[];  // [Nm] twiddles | [M][kXPitch] x 2 buffers
    const int M = xp.M;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const long long plane = (long long)Nm * Nm;
    const long long tiles_per_map = (plane + kXRows - 1) / kXRows, ntiles = tiles_per_map * count;
    float2 *tw = sx, *b0 = sx + Nm, *b1 = b0 + (size_t)M * kXPitch;
    for (int t = threadIdx.x; t < Nm; t += blockDim.x) tw[t] = tw_g[t];
    // the next tile's coefficients are loaded into registers while this tile computes
    float2 pre[PF];
    auto fetch = [&](long long tile) {
        const int m = (int)(tile / tiles_per_map);
        const long long row0 = (tile - (long long)m * tiles_per_map) * kXRows;
        const bool ok = row0 + lane < plane;
        const float2 *src = cols + (size_t)m * KX * plane + row0 + lane;
#pragma unroll
        for (int i = 0; i < PF; i++) {
            const int k = warp + i * nw;
            pre[i] = (k < KX && ok) ? __ldcs(src + (size_t)k * plane) : make_float2(0.f, 0.f);
        }
    };
    if (blockIdx.x < ntiles) fetch(blockIdx.x);
    for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int m = (int)(tile / tiles_per_map);
        const long long row0 = (tile - (long long)m * tiles_per_map) * kXRows;
        const int nrows = (int)((plane - row0) < kXRows ? (plane - row0) : kXRows);
        __syncthreads();
        // raw coefficients X[k][row] for k < KX into b1, then prefetch the next tile
#pragma unroll
        for (int i = 0; i < PF; i++) {
            const int k = warp + i * nw;
            if (k < KX) b1[k * kXPitch + lane] = pre[i];
        }
        if (tile + gridDim.x < ntiles) fetch(tile + gridDim.x);
        __syncthreads();
        // Z = E + i O into b0
        for (int k = warp; k < M; k += nw) {
            const float2 xk = k < KX ? b1[k * kXPitch + lane] : make_float2(0.f, 0.f);
            const int kc = M - k;
            float2 xc = make_float2(0.f, 0.f);
            if (kc < KX) {
                xc = b1[kc * kXPitch + lane];
                xc.y = -xc.y;
            }
            const float2 o = cmul2(csub2(xk, xc), tw[k]);
            b0[k * kXPitch + lane] = cadd2(cadd2(xk, xc), itimes(o));
        }
        __syncthreads();
        int Ns = 1;
        float2 *in = b0, *ou = b1;
        for (int s = 0; s < xp.nst; s++) {
            const int R = xp.rad[s];
            switch (R) {
                case 2: stockham_stage<2>(in, ou, tw, M, Ns, warp, nw, lane); break;
                case 3: stockham_stage<3>(in, ou, tw, M, Ns, warp, nw, lane); break;
                case 4: stockham_stage<4>(in, ou, tw, M, Ns, warp, nw, lane); break;
                case 5: stockham_stage<5>(in, ou, tw, M, Ns, warp, nw, lane); break;
                default: stockham_stage<7>(in, ou, tw, M, Ns, warp, nw, lane); break;
            }
            __syncthreads();
            float2 *t = in;
            in = ou;
            ou = t;
            Ns *= R;
        }
        // x[2mm] = Re z[mm], x[2mm+1] = Im z[mm]; one warp per row
        for (int l = warp; l < nrows; l += nw) {
            const long long row = row0 + l;
            float *o = dense ? out + (size_t)m * plane * Nm + (size_t)row * Nm
                             : out + ((size_t)row * count + m) * Nm;
            for (int mm = lane; mm < M; mm += 32) reinterpret_cast<float2 *>(o)[mm] = in[mm * kXPitch + l];
        }
    }
}

int c2r_rows(const Shells &sh, int count, int KX, const float2 *cols, float *out, bool dense, DevBuf &tw,
             cudaStream_t st, int64_t *launches) {
    const int Nm = sh.Nm, M = Nm / 2;
    XPassPlan xp;
    xp.M = M;
    int rest = M;
    for (int r : {4, 2, 3, 5, 7})
        while (rest % r == 0 && xp.nst < 12) {
            xp.rad[xp.nst++] = r;
            rest /= r;
        }
    if (rest != 1 || KX > M) return set_error(PBI4G_ERR_UNSUPPORTED, "x pass: Nm=%d (KX=%d)", Nm, KX);
    static std::once_flag roots_once;
    static int roots_rc = 0;
    std::call_once(roots_once, [] {
        float2 h[9][8] = {};
        for (int R = 2; R <= 8; R++)
            for (int t = 0; t < R; t++) h[R][t] = make_float2((float)cos(2 * M_PI * t / R), (float)sin(2 * M_PI * t / R));
        roots_rc = cudaMemcpyToSymbol(c_roots, h, sizeof(h)) == cudaSuccess ? 0 : 1;
    });
    if (roots_rc) return set_error(PBI4G_ERR_CUDA, "x pass: constant roots upload failed");
    if (tw.bytes < sizeof(float2) * Nm) {
        std::vector<float2> h(Nm);
        for (int t = 0; t < Nm; t++) h[t] = make_float2((float)cos(2 * M_PI * t / Nm), (float)sin(2 * M_PI * t / Nm));
        PBI4G_CHECK(tw.ensure(sizeof(float2) * Nm));
        PBI4G_CUDA(cudaMemcpy(tw.p, h.data(), sizeof(float2) * Nm, cudaMemcpyHostToDevice));
    }
    const size_t smem = sizeof(float2) * (Nm + 2 * (size_t)M * kXPitch);
    const int warps = 8, pf = (KX + warps - 1) / warps;
    auto launch = [&](auto kern) -> int {
        PBI4G_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        int per_sm = 0;
        PBI4G_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, warps * 32, smem));
        kern<<<152 * std::max(1, per_sm), warps * 32, smem, st>>>(cols, out, tw.as<float2>(), xp, Nm, KX, count,
                                                                   dense ? 1 : 0);
        PBI4G_LAUNCH_CHECK();
        return PBI4G_OK;
    };
    if (pf <= 4) PBI4G_CHECK(launch(c2r_rows_kernel<4>));
    else if (pf <= 9) PBI4G_CHECK(launch(c2r_rows_kernel<9>));
    else if (pf <= 16) PBI4G_CHECK(launch(c2r_rows_kernel<16>));
    else if (pf <= 32) PBI4G_CHECK(launch(c2r_rows_kernel<32>));
    else return set_error(PBI4G_ERR_UNSUPPORTED, "x pass: KX=%d", KX);
    ++*launches;
    return PBI4G_OK;
}

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
                                      double *__restrict__ S) {
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nslots; s += gridDim.x * blockDim.x) {
        double v = 0;
        for (int k = 0; k < ksplit; k++) v += partial[(size_t)k * nslots + s];
        S[s] = v;
    }
}

int reduce_partials(int nslots, int ksplit, const double *partial, double *S, cudaStream_t st) {
    reduce_partial_kernel<<<(nslots + 255) / 256, 256, 0, st>>>(nslots, ksplit, partial, S);
    PBI4G_LAUNCH_CHECK();
    return PBI4G_OK;
}

template <class T>
int triangle_sums(const Shells &sh, const TriPlan &tp, const T *maps, size_t mstride, int rs, DevBuf &partial,
                  double *S, cudaStream_t st, int64_t *launches) {
    const int N = sh.Nm;  // maps live on the map grid
    const long long K = (long long)N * N * N;
    int kc = kKCmax;
    while (kc > 4 && K % kc) kc /= 2;
    if (K % kc || (N & 1) || (rs & 1) || (mstride & 1))
        return set_error(PBI4G_ERR_UNSUPPORTED, "triangle sums: grid %d has no even chunk width", N);
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
    reduce_partial_kernel<<<(tp.nslots + 255) / 256, 256, 0, st>>>(tp.nslots, ksplit, partial.as<double>(), S);
    PBI4G_LAUNCH_CHECK();
    *launches += 2;
    return PBI4G_OK;
}

template int triangle_sums<float>(const Shells &, const TriPlan &, const float *, size_t, int, DevBuf &, double *,
                                  cudaStream_t, int64_t *);
template int triangle_sums<double>(const Shells &, const TriPlan &, const double *, size_t, int, DevBuf &, double *,
                                   cudaStream_t, int64_t *);

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
    const size_t HC = half_cells(N);
    DevBuf maps, partial, S;
    PBI4G_CHECK(maps.ensure(sizeof(double2) * HC * nb));
    PBI4G_CHECK(build_indicator_spectra<double>(sh, 0, nb, maps.as<double2>(), st, launches));
    cufftHandle plan;
    int n[3] = {N, N, N}, inembed[3] = {N, N, NH}, onembed[3] = {N, N, 2 * NH};
    PBI4G_CUFFT(cufftPlanMany(&plan, 3, n, inembed, 1, (int)HC, onembed, 1, (int)(2 * HC), CUFFT_Z2D, nb));
    cufftSetStream(plan, st);
    cufftResult r = cufftExecZ2D(plan, maps.as<cufftDoubleComplex>(), maps.as<cufftDoubleReal>());
    cufftDestroy(plan);
    if (r != CUFFT_SUCCESS) return set_error(PBI4G_ERR_CUFFT, "counts: cufftExecZ2D failed (%d)", (int)r);
    // all three factors are indicator maps of the same set (also for the cross
    // enumeration, bispectrumI4.f90:887-896), so the non-cross pair layout applies
    TriPlan tp;
    PBI4G_CHECK(tp.build(sh, 1, 0, 128));
    PBI4G_CHECK(S.ensure(sizeof(double) * tp.nslots));
    PBI4G_CHECK(triangle_sums<double>(sh, tp, maps.as<double>(), 2 * HC, 2 * NH, partial, S.as<double>(), st, launches));
    std::vector<double> Sh(tp.nslots);
    PBI4G_CUDA(cudaMemcpyAsync(Sh.data(), S.p, sizeof(double) * tp.nslots, cudaMemcpyDeviceToHost, st));
    PBI4G_CUDA(cudaStreamSynchronize(st));
    const double gridD = (double)N * N * N;
    sh.counts.resize(sh.itot);
    std::vector<float> c32(sh.itot);
    double maxdev = 0;
    for (int64_t m = 0; m < sh.itot; m++) {
        double v = Sh[m] / gridD;
        long long c = llround(v);
        maxdev = std::max(maxdev, fabs(v - (double)c));
        sh.counts[m] = c;
        c32[m] = (float)(gridD * (double)c);
    }
    if (maxdev > 0.25) {
        sh.counts.clear();
        return set_error(PBI4G_ERR_RANGE, "triangle counts not resolved to integers (max deviation %g)", maxdev);
    }
    {
        std::lock_guard<std::mutex> g(g_counts_mutex);
        g_counts_cache[ckey] = sh.counts;
    }
    (void)c32;
    return upload_counts(sh);
}

}  // namespace pbi4g
