// spectrum.cuh -- host interface of the Fourier-space kernels (spectrum.cu):
// interlacing combine / window deconvolution, P(k) binning, multipole factors.
#pragma once
#include "common.cuh"

namespace pbi4g {

template <class R> struct Cx;
template <> struct Cx<float> { using T = float2; };
template <> struct Cx<double> { using T = double2; };

// Input-independent P(k) binning of one configuration (cached per plan).
struct PkBins {
    int N = 0, nbins = 0;
    float box = 0, kbin = 0, kcenter = 0;
    double kF = 0, kF3 = 0, dk = 0;
    int k2max = 0;
    DevBuf lut;     // int32 [k2max+1]: bin 1..nbins, 0 outside, -1 tie -> exact FP64 per cell
    DevBuf avgk_co; // double [2][nbins]: sum of |k| and mode count per bin (reference loop semantics)
    DevBuf partial; // double [blocks][3][nbins]
    int blocks = 0;
    int build(int N, float box, float kbin, float kcenter, int nbins, cudaStream_t st, int64_t *launches);
};

// Device copy of the 1/W window table used by fcomb_half.
struct WinCache {
    DevBuf buf;
    int N = -1, nintp = -1, rsize = -1;
};

// fcomb on the R2C half spectra of one (non-interlaced) or two (interlaced)
// real grids: spec [G][N][N][N/2+1] -> delta [N][N][N/2+1], including the
// 1/norm normalisation (dcl /= npart, pbi4.py:336); with bp the factor is read
// from bp->fcomb_cf (graph-captured form).
// normalisation factor of fcomb_half for `norm` particles
double fcomb_cf(bool interlaced, float box, double norm);

template <class R>
int fcomb_half(int N, int nintp, bool interlaced, float box, double norm, const typename Cx<R>::T *spec,
               typename Cx<R>::T *delta, WinCache &wcache, cudaStream_t st, int64_t *launches, const BoxPar *bp = nullptr);

// Full-grid fcomb (drop-in, FP64), in place allowed.
int fcomb_full(int N, int nintp, bool interlaced, float box, const double2 *in, double2 *out, cudaStream_t st);

// P(k) accumulation on a half spectrum.  mode 0: sum Re(conj(a) b) (b may equal a);
// mode 1: multipoles of an auto spectrum from the constant-LOS factor
// (-1/2 + 3/2 mu^2, 3/8 - 30/8 mu^2 + 35/8 mu^4) applied to a;
// mode 2: multipoles from explicit delta_2 (b) and delta_4 (c) half spectra.
// Writes pout (5, nbins) Fortran order on the device.
template <class R>
int pk_measure(PkBins &bins, int mode, const double los[3], const typename Cx<R>::T *a,
               const typename Cx<R>::T *b, const typename Cx<R>::T *c, double *d_pout, cudaStream_t st,
               int64_t *launches);

// Drop-in helpers on full FP64 grids.
int q2k_full(int N, float box, const double2 *in, int i, int j, double2 *out, cudaStream_t st);
int q4k_full(int N, float box, const double2 *in, int i, int j, int l, int k, double2 *out, cudaStream_t st);
int reduce_full(int L, const double2 *din, int N, double2 *dout, cudaStream_t st);

// Host-side window table tW(1..N/2+1) of powerI4.f90:278-292.
void window_table(int N, int nintp, double *tW);
double fcomb_kF3(float box);  // the real(4) kF3 of powerI4.f90:271

}  // namespace pbi4g
