// bispec.cuh -- host interface of the bispectrum kernels (bispec.cu):
// shell tables, shell-filtered k-maps, triangle sums, exact triangle counts.
#pragma once
#include <vector>

#include <cufft.h>

#include "common.cuh"
#include "spectrum.cuh"

namespace pbi4g {

// Input-independent shell binning and triangle enumeration (cached per plan).
struct Shells {
    int N = 0, nb = 0, iopen = 0, cross = 0, ishift = 0;
    int Nm = 0;  // grid of the shell maps (the smallest alias-free size, at most N)
    int kmax = 0;  // largest |k_axis| of any shell mode (columns kx > kmax of every map are zero)
    float kbin = 0, kcenter = 0;
    int k2max = 0;
    std::vector<int> lut_h;          // shell of |k|^2 (1..nb), 0 outside
    std::vector<int64_t> nmodes;     // full-grid modes per shell
    std::vector<int> tri;            // (l, j, i) per triangle, reference order
    int64_t itot = 0;
    DevBuf lut;                      // int32 [k2max+1]
    DevBuf nmodes_d;                 // double [nb]
    DevBuf tri_d;                    // int32 [itot][3] = (l, j, i)
    std::vector<int64_t> counts;     // exact integer triangle counts (empty until computed)
    DevBuf counts_f32;               // float [itot] = float32(N^3 * count), the reference's `counts`
    int build(int N, float kbin, float kcenter, int nb, int iopen, int cross, cudaStream_t st);
};

// Grid of the shell maps for shells whose modes reach |k_axis| <= kmax (the
// smallest FFT-friendly multiple of 4 above 3 kmax, at most N), and the same
// from the binning (what Shells::build sets as Nm), host only.
int map_grid_for_kmax(int N, int kmax);
int shell_map_grid(int N, float kbin, float kcenter, int nb);

// Sparse "pair x q" contraction S[slot] = sum_x P_a(x) P_b(x) Q(x) arranged as
// register tiles; built once per (shells, number of q sets).
struct TriPlan {
    int nsets = 1;       // q sets (1: B0; 3: B0, B2, B4; cross: 1 with q from the second field)
    int cross = 0;
    int np = 0, nq = 0;  // pairs, q maps
    int nslots = 0;      // itot * nsets
    int ngroups = 0;
    DevBuf pairs;        // int2 [np]: source maps of each pair (within the pair set)
    DevBuf qmap;         // int [nq]: map index of each q (within all maps)
    DevBuf tiles;        // int4 [ntiles]: (pair0, q0, group, slot table offset)
    DevBuf slots;        // int [ntiles][TP][TQ]: output slot or -1
    DevBuf groups;       // int4 [ngroups]: (tile0, tile1, pair0, pair1)
    std::vector<int> group_tiles;
    int ntiles = 0, max_group_pairs = 0;
    // qoff: added to the map index of every non-cross q (a second copy of the maps)
    int build(const Shells &sh, int nsets, int cross, int max_pairs = 256, int qoff = 0);
};

// Build the half spectra of all `count` maps on the map grid Nm into `out`
// (count x Nm*Nm*(Nm/2+1) complex R, the in-place C2R layout).  Map m belongs
// to set m / nb and shell m % nb + 1.  Set s reads src[s] (a half spectrum on the
// N grid) times the multipole factor fac[s] (0: 1, 2: L2(mu), 4: L4(mu)); the
// kx = 0 (and Nyquist) planes are Hermitian-symmetrised.  When powsum != null,
// the full-grid sum of |H|^2 of every shell of each set in pow_mask is added
// into powsum[s * nb + shell - 1] (double).
template <class R>
int build_map_spectra(const Shells &sh, int count, const typename Cx<R>::T *const src[3], const int fac[3],
                      const double los[3], typename Cx<R>::T *out, double *powsum, int pow_mask, cudaStream_t st,
                      int64_t *launches);

// Indicator half spectra of shells [m0, m0+count) (count_triangles, bispectrumI4.f90:862-869).
template <class R>
int build_indicator_spectra(const Shells &sh, int m0, int count, typename Cx<R>::T *out, cudaStream_t st,
                            int64_t *launches);

// Triangle sums on CUDA cores: S[slot] for all slots of tp over K points,
// maps FP32/FP64 laid out as rows of `rowlen` points with row stride rs
// (rowlen + 2 for padded C2R output).  maps: base of all maps, map m at
// maps + m * mstride.  Result S (double, nslots) on device; with accumulate the
// sums are added to S (a contraction streamed in point ranges).
template <class T>
int triangle_sums(const Shells &sh, const TriPlan &tp, const T *maps, size_t mstride, int rowlen, int rs,
                  long long K, DevBuf &partial, double *S, bool accumulate, cudaStream_t st, int64_t *launches);

// Output rows of measure_bk (9), measure_bk_multipoles (11), measure_bk_cross (5).
// With bp the shot-noise factor is read from bp->pow_sn (graph-captured form).
int bk_finalize(const Shells &sh, int nsets, int cross, const double *S, const double *powsum, float kf,
                int64_t npart, const float *counts_f32, double *bout, cudaStream_t st, int64_t *launches,
                const BoxPar *bp = nullptr);
// 1 / npart / kf^3 with kf^3 in real(4), as bk_finalize uses it
double bk_pow_sn(float kf, int64_t npart);

// Exact integer triangle counts (FP64 indicator maps + FP64 sums over the
// cube-group orbit representatives of the map grid, rounded).
int triangle_counts(Shells &sh, cudaStream_t st, int64_t *launches);

}  // namespace pbi4g
