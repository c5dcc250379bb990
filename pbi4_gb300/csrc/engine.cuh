// engine.cuh -- bispectrum engine shared by the plan and the drop-in entry points.
#pragma once
#include "bispec.cuh"
#include "mapfft.cuh"
#include "trisum_tm.cuh"

namespace pbi4g {

// Triangle-sum form of a PBI4G_PREC_* precision: 0 CUDA cores (FP32 / FP64),
// 1 FP16 hi+lo, 2 BF16, 3 TF32 hi+lo (tensor cores).
inline int tc_mode_of(int precision) {
    switch (precision) {
        case PBI4G_PREC_FP16SPLIT: return 1;
        case PBI4G_PREC_BF16: return 2;
        case PBI4G_PREC_TF32SPLIT: return 3;
        default: return 0;
    }
}

// Resident state of the bispectrum stage for one (grid, binning, sets) layout.
struct BkEngine {
    Shells sh;
    TriPlan tp;
    int tp_nsets = -1, tp_cross = -1, tp_fp64 = -1;
    int nsets = 1, cross = 0;  // cross: 1 => q maps from the second field
    DevBuf maps;               // FP64: [nmaps][N][N][N/2+1] half spectra, padded real maps after the C2R;
                               // FP32: the pruned transform's intermediates (T, and U of one slab)
    DevBuf dense;              // plain FP32: real maps [m][point]; tensor-core forms: the operand planes
    MapPlanes planes;          // tensor-core forms: the layout of `dense`
    // FP32 forms: upper bound on the bytes of the slab-sized map buffers (the y
    // pass's output in `maps` and the real maps in `dense`; 0: none).  When the
    // whole grid's exceed it, the y pass, the x pass and the triangle sums stream
    // over z-slabs of slab_z planes, the sums of each slab added to the last.
    size_t map_budget = 0;
    int slab_z = 0, nslabs = 0;  // of the last run
    cufftHandle inv = 0;       // FP64 maps: batched Z2D
    int inv_batch = 0, inv_N = 0;
    MapTransform mt;           // FP32 maps: pruned z / y / x passes
    int mt_nmaps = -1;
    DevBuf powsum, S, partial;
    // tensor-core form: 0 off (CUDA cores), 1 FP16 hi+lo, 2 BF16, 3 TF32 hi+lo
    int tc_mode = 0;
    TmPlan tmp;
    int tmp_nsets = -1;
    ~BkEngine() {
        if (inv) cufftDestroy(inv);
    }
    int nmaps() const { return cross ? 2 * sh.nb : nsets * sh.nb; }
    static size_t footprint(int N, float kbin, float kcenter, int nb, int nsets, int cross, int precision,
                            size_t map_budget = 0);
    // z-planes per slab on map grid Nm for `per_plane` bytes of slab buffers a z-plane
    static int slab_planes(int Nm, size_t per_plane, size_t budget);
    // PBI4G_ERR_TIMEOUT if a bounded wait of a tensor-core launch gave up (synchronises st)
    int check(cudaStream_t st);

    // src[s]: half spectra (N, N, N/2+1) of set s; fac[s]: 0 none, 2/4 the
    // multipole factor from `los`.  counts_f32: device float counts[itot].
    template <class R>
    int run(const typename Cx<R>::T *const src[3], const int fac[3], const double los[3], float kf, int64_t npart,
            const float *counts_f32, double *d_bout, cudaStream_t st, int64_t *launches, Prof *prof = nullptr,
            const BoxPar *bp = nullptr);
};

}  // namespace pbi4g
