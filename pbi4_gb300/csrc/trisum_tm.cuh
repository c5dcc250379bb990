// trisum_tm.cuh -- host interface of the tensor-core triangle sums (trisum_tm.cu).
#pragma once
#include "bispec.cuh"
#include "mapfft.cuh"

namespace pbi4g {

// Unit layout of the tcgen05 contraction for one (shells, q sets) layout:
// units of one 128-pair M tile and one 64-map N tile; q = map index (set-major).
struct TmPlan {
    int nsets = 1, npairs = 0, nslots = 0, nunits = 0, nA = 0;
    DevBuf units, prow, slots, err;
    DevBuf mexp;     // FP16 form: per-map power-of-two exponents
    DevBuf kahan;    // per-CTA running sums when they do not fit in TMEM beside the accumulators
    uint32_t wait_limit = 0;  // diagnostic: polls before a main-loop wait gives up (0: the default)
    int build(const Shells &sh, int nsets);
};

bool tm_supported(const Shells &sh);

// FP16 form: the per-map power-of-two exponents into tp.mexp, before the x
// pass writes the scaled operand planes.  powsum[s*nb + b] is the full-grid sum
// of |H|^2 per set and shell (sets in pow_mask), which with the shell's mode
// count bounds max |M|; lfac[s] bounds |L_l| for sets without their own power.
int tm_map_exponents(const Shells &sh, TmPlan &tp, int nmaps, const double *powsum, int pow_mask,
                     const double lfac[3], cudaStream_t st, int64_t *launches);

// S[slot] for every (triangle, set) slot on the tensor cores, from the operand
// planes the x pass wrote (pl.form: 0 TF32 hi+lo, 1 FP16 hi+lo with pl.mexp ==
// tp.mexp, 2 BF16).  The planes may hold one slab of the map grid's points
// (pl.npts <= Nm^3); with accumulate the slab's sums are added to S.
int triangle_sums_tm(const Shells &sh, TmPlan &tp, const MapPlanes &pl, DevBuf &partial, double *S,
                     bool accumulate, cudaStream_t st, int64_t *launches);
// PBI4G_ERR_TIMEOUT if a bounded wait inside the last launch gave up (synchronises st).
int tm_check_error(TmPlan &tp, cudaStream_t st);

// deterministic reduction of [ksplit][nslots] partial sums into S (added to S
// with accumulate) (bispec.cu)
int reduce_partials(int nslots, int ksplit, const double *partial, double *S, bool accumulate, cudaStream_t st);

}  // namespace pbi4g
