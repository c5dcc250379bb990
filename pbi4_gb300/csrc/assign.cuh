// assign.cuh -- host interface of the mass-assignment kernels (assign.cu).
#pragma once
#include "common.cuh"

namespace pbi4g {

// Device scratch of the assignment: fixed-point grids and the tile sort.
struct AssignWork {
    DevBuf grids;  // uint64 [G][N^3], G = 2 when interlaced
    DevBuf tile_count, tile_start, tile_cursor, ptile, order, wmax;
    int ensure(int N, int64_t npart, bool interlaced);
    static size_t footprint(int N, int64_t npart, bool interlaced);
};

// Number of fraction bits S of the fixed-point grid for npart particles of
// weight at most wmax (sum of |contributions| stays below 2^62).
int fixed_point_bits(int64_t npart, double wmax, int *bits);

// Scatter npart particles (d_pos: (3, npart) float64 SoA on device, d_weight
// optional) into wk.grids.  Weights/products in FP64 when fp64_weights, else FP32.
int assign_fixed(AssignWork &wk, int N, int nintp, bool interlaced, bool fp64_weights, int64_t npart,
                 const double *d_pos, const double *d_weight, int *bits_out, cudaStream_t st, int64_t *launches);

// Fixed-point grids -> real grids (float or double), [G][N^3] contiguous.
int fixed_to_real(const AssignWork &wk, int N, bool interlaced, int bits, bool fp64, void *out, cudaStream_t st,
                  int64_t *launches);
// Interlaced fixed-point grids -> complex128 (Re grid 1, Im grid 2).
int fixed_to_complex(const AssignWork &wk, int N, int bits, double2 *out, cudaStream_t st, int64_t *launches);

}  // namespace pbi4g
