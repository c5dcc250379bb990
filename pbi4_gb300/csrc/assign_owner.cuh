// assign_owner.cuh -- owner-computes tiled assignment into FP32 grids (assign_owner.cu).
#pragma once
#include "assign.cuh"

namespace pbi4g {

struct OwnerWork {
    DevBuf count, start, cursor, key, rec, sorted, wsorted, wmax;
    bool fixed = false;  // a shared scratch: sized once, never reallocated (ensure fails instead)
    int ensure(int N, int64_t npart);
    bool fits(int N, int64_t npart) const;
    void release();
    static size_t footprint(int N, int64_t npart);
};

bool owner_supported(int N);

// The owner kernels read the buffers of their OwnerWork from a device block of
// kOwnerPtrBytes bytes, which the caller fills from owner_ptrs_host whenever the
// buffers or the OwnerWork in use change (stream-ordered, outside any capture):
// a captured graph then follows its plan to another OwnerWork.
constexpr size_t kOwnerPtrBytes = 64;
void owner_ptrs_host(const OwnerWork &wk, unsigned char (&block)[kOwnerPtrBytes]);

// Assign npart particles (device (3, npart) float64, optional device weights)
// into FP32 real grids out[G][N^3] (G = 2 when interlaced), fixed-point exact sums.
// stride: distance between the x, y, z rows of d_pos (npart when <= 0).  bp:
// when set, the particle count is read from bp->npart (npart is then the
// capacity that sizes the launches: the graph-captured form).
// prof: when set, the counting sort is timed as stage sort_stage and the tile
// kernel as stage tile_stage.
// wk must fit (N, npart) and d_ptrs hold its pointers (owner_ptrs_host).
int assign_owner(OwnerWork &wk, const void *d_ptrs, int N, int nintp, bool interlaced, int64_t npart,
                 const double *d_pos, const double *d_weight, float *out, cudaStream_t st, int64_t *launches,
                 int64_t stride = 0, const BoxPar *bp = nullptr, Prof *prof = nullptr, int tile_stage = 0,
                 int sort_stage = 0);

}  // namespace pbi4g
