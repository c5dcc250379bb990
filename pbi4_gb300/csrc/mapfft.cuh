// mapfft.cuh -- pruned inverse transform of the FP32 shell maps (mapfft.cu).
//
// The maps of the bispectrum are I_b(x) = sum over the modes k of shell b of
// delta(k) e^{ikx} (times a multipole factor), i.e. a C2R of a half spectrum
// that is zero outside one spherical shell.  The transform runs as three
// passes of in-place FFTs over batches of 32 one-dimensional transforms, each
// pass skipping what the shell leaves zero:
//   z pass: the (kx >= 0, ky) columns with kx^2 + ky^2 <= k2hi(b) only; the
//           spectrum is built on the fly from delta(k) (shell mask, multipole
//           factor, Hermitian symmetrisation of the kx = 0 plane, shell power)
//           -> T[m][column][z];
//   y pass: per (kx < kxn(b), z), input ky in [-r(kx), r(kx)] -> U[m][kx][z][y];
//   x pass: per (z, y) row, the Hermitian C2R from kx < kxn(b) -> the real map,
//           written dense FP32 [m][z][y][x] or as the tensor-core operand planes.
#pragma once

#include "bispec.cuh"
#include "fft_small.cuh"

namespace pbi4g {

struct MapInfo {
    int shell;        // 0-based shell of the map (map m: set m / nb, shell m % nb)
    int kxn;          // columns kx < kxn hold modes of the shell
    int ncol;         // (kx, ky) columns of the z pass
    int col0;         // first column of the shell in MapTransform::cols
    int kx0;          // first (shell, kx) entry in MapTransform::kxr
    int k2lo, k2hi;   // the shell's modes are exactly those with k2lo <= |k|^2 <= k2hi
    int kxc;          // first flat kx index of the map (sum of kxn over the maps before it)
    long long tbase;  // first float2 of the map in T ([column][z])
    long long ubase;  // first float2 of the map in U of the whole grid ([kx][z][y]) = kxc Nm^2
};

// Tensor-core operands of the maps ("planes"), written by the x pass for the
// tensor-core forms.  Points are grouped in chunks of 64 consecutive points
// (point = (z Nm + y) Nm + x, counted from the first point of the z-slab the
// planes hold; the slab's point count is a multiple of 64), and every array is
// chunk-major, [chunk][map][64 points], so the operand tile of a chunk (64 maps
// x 64 points) is one contiguous block:
//   form 1 (FP16 hi+lo): bhi, blo FP16 with v 2^mexp[m] = hi + lo (|v 2^mexp| <= 2^14);
//   form 2 (BF16):       bhi BF16 of v;
//   form 0 (TF32 hi+lo): bhi FP32 = v with the 13 low mantissa bits cleared, blo = v - bhi;
// and a32 [chunk][nb][64] = the set-0 maps in FP32, times 2^(mexp[m] - 7) for
// form 1 (the pair factors: their products are the A operand, |A| <= 2^14, with
// no further scaling).
struct MapPlanes {
    static constexpr int kChunk = 64;
    int form = -1;
    long long npts = 0, nchunks = 0;
    int nmaps = 0, nb = 0;
    void *bhi = nullptr, *blo = nullptr;
    float *a32 = nullptr;
    const int *mexp = nullptr;
    static size_t bytes(int form, long long npts, int nmaps, int nb) {
        const size_t b = form == 0 ? 8 : (form == 1 ? 4 : 2);  // B bytes per point and map
        return b * (size_t)npts * nmaps + 4 * (size_t)npts * nb;
    }
    void carve(int form_, long long npts_, int nmaps_, int nb_, void *base, const int *mexp_) {
        form = form_;
        npts = npts_;
        nchunks = npts / kChunk;
        nmaps = nmaps_;
        nb = nb_;
        mexp = mexp_;
        const size_t half = (form == 0 ? 4 : 2) * (size_t)npts * nmaps;  // bytes of one of hi / lo
        unsigned char *p = static_cast<unsigned char *>(base);
        bhi = p;
        blo = form == 2 ? nullptr : p + half;
        a32 = reinterpret_cast<float *>(p + (form == 2 ? half : 2 * half));
    }
};

struct MapTransform {
    int Nm = 0, nmaps = 0, nb = 0, kxmax = 0;
    fftd::FftPlan pz;    // Nm points (z and y passes; radix 20 allowed)
    fftd::FftPlan px;    // Nm / 2 points (x pass)
    DevBuf tab_z, tab_x;  // packed plan tables (twiddles, butterfly entries, output positions)
    DevBuf xtw;           // e^{2 pi i k / Nm}, k < Nm (the x pass's even/odd split)
    DevBuf cols;          // int2 [sum ncol]: (kx, ky) of every column of every shell
    DevBuf kxr;           // int2 [sum kxn]: (r(kx), first column of kx) per shell
    DevBuf info;          // MapInfo [nmaps]
    DevBuf ztiles;        // int2 (map, first column) per 32-wide z-pass tile
    DevBuf gmap;          // int [kxtot]: map of each flat kx index
    int nzt = 0, kxtot = 0;
    long long tsize = 0, usize = 0;  // float2 elements of T and of U for the whole grid (kxtot Nm^2)
    std::vector<MapInfo> info_h;
    int build(const Shells &sh, int nmaps);
    // T + U for z-slabs of zs planes (U holds one slab: kxtot zs Nm elements)
    size_t work_bytes(int zs) const { return sizeof(float2) * (size_t)(tsize + (long long)kxtot * zs * Nm); }
    size_t work_bytes() const { return work_bytes(Nm); }
};

// z pass (shell spectra + z transform) of all maps into work[0, tsize).
// src[s] / fac[s] / los / powsum / pow_mask as for build_map_spectra.
int map_zpass(const Shells &sh, const MapTransform &mt, const float2 *const src[3], const int fac[3],
              const double los[3], float2 *work, double *powsum, int pow_mask, cudaStream_t st, int64_t *launches);
// y pass of the z-slab [z0, z1) (z1 < 0: Nm): work[0, tsize) -> U at
// work[tsize, ...) = [kx flat][z - z0][y], i.e. float2 index
// ((kxc + kx) (z1 - z0) + z - z0) Nm + y for map m, column kx of it.
int map_ypass(const MapTransform &mt, float2 *work, cudaStream_t st, int64_t *launches, int z0 = 0, int z1 = -1);
// x pass: real maps from the U that map_ypass wrote for the same z-slab
// [z0, z1) (z1 < 0: Nm): dense FP32 [m][z][y][x] into `out` when planes is
// null, else the tensor-core operand planes, as if the grid held the slab's
// points alone (map stride (z1 - z0) Nm^2 for the dense maps; planes->npts =
// that count, a multiple of 64).
int map_xpass(const MapTransform &mt, const float2 *work, float *out, const MapPlanes *planes, cudaStream_t st,
              int64_t *launches, int z0 = 0, int z1 = -1);

// Host check of the in-place FFT plan: n-point inverse DFTs of `batch`
// transforms in[t][n] -> out[t][k] on the CPU with the kernels' butterflies.
int fft_plan_host_check(int n, int batch, const float *in, float *out);

}  // namespace pbi4g
