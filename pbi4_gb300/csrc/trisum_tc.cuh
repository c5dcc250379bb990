// trisum_tc.cuh -- host interface of the tensor-core triangle sums (trisum_tc.cu).
#pragma once
#include "bispec.cuh"

namespace pbi4g {

// Unit layout of the tcgen05 contraction for one (shells, q sets) layout:
// units of up to two 128-pair M tiles sharing one 64-map N tile.
struct TcPlan {
    int nsets = 1, npairs = 0, nslots = 0, nunits = 0, umax = 0;
    double useful = 0;  // fraction of the computed (pair, q) products that are triangles
    DevBuf units, umaps, psrc, pmap, qsrc, qmap, slots, pexp, qexp, err;
    int build(const Shells &sh, int nsets);
};

// S[slot] for every (triangle, set) slot.  maps: FP32 maps on the map grid
// (padded C2R rows, row stride rs floats, map stride mstride floats);
// powsum[s*nb + b]: full-grid sum of |H|^2 per set and shell (sets in pow_mask),
// which with the shell's mode count bounds max |M| and sets each map's fp16
// scale; lfac[s] bounds |L_l| for sets without their own power.
// split: FP16 hi+lo (3 products) when true, single BF16 product when false.
int triangle_sums_tc(const Shells &sh, TcPlan &tp, bool split, const float *maps, size_t mstride, int rs,
                     const double *powsum, int pow_mask, const double lfac[3], DevBuf &mexp, DevBuf &partial, double *S,
                     cudaStream_t st, int64_t *launches);
// PBI4G_ERR_TIMEOUT if a bounded wait inside the last launch gave up (synchronises st).
int tc_check_error(TcPlan &tp, cudaStream_t st);

// deterministic reduction of [ksplit][nslots] partial sums (bispec.cu)
int reduce_partials(int nslots, int ksplit, const double *partial, double *S, cudaStream_t st);

}  // namespace pbi4g
