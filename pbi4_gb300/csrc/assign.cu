// assign.cu -- mass assignment (NGP/CIC/TSC/PCS, optional interlacing) into
// 64-bit fixed-point grids.
//
// Follows powerI4.f90:68-140 (assign_single_grid) and :142-249
// (assign_double_grid): the same cell indices (including the +1 cell shift of
// CIC relative to TSC/PCS and the -1/2 cell shift of the interlaced grid) and
// the same per-axis weights, with one deliberate difference: every contribution
// w_x w_y w_z weight is rounded once to a 64-bit integer at scale 2^S and added
// with integer atomics, so the grid does not depend on particle order or on
// thread scheduling (bit-reproducible), unlike an FP sum.
//
// Two kernels:
//  * assign_tiled  -- particles are counting-sorted into cubic cell tiles; one
//    CTA accumulates a tile (plus its stencil halo) in shared memory with
//    shared 64-bit atomics, then flushes the halo-extended tile to the global
//    grid with one global atomic per touched cell.  Used for dense boxes.
//  * assign_direct -- one global atomic per contribution (small / sparse inputs).
#include "common.cuh"
#include "assign.cuh"

#include <math.h>
#include <string.h>

namespace pbi4g {

// Per-axis stencil of one particle coordinate p in [0,1]: first cell index
// (0-based, not yet wrapped) and the nintp weights.  `cic_nint` selects the
// single-grid CIC offset h = v - nint(v) (powerI4.f90:120) instead of
// h = v - int(v) (double grid, powerI4.f90:216-217).
template <class W>
__device__ __forceinline__ void axis_stencil(double p, int N, int nintp, bool shifted, bool cic_nint, int &first,
                                             W w[4]) {
    // vr = dble(Nv)*pos + 1 with the product and the sum rounded separately (no FMA
    // contraction), as the oracle's ISO C and an FMA-free Fortran build compute it
    double v = __dadd_rn(__dmul_rn((double)N, p), 1.0);
    if (shifted) v = v - 0.5;       // vt = vr - 0.5
    double h;
    if (nintp == 4) {
        long long iv = (long long)v;           // int(vr)
        first = (int)((iv - 2) % N);            // mod(ivr - 3 + 1 + N, N)
        h = v - (double)iv;
        W hh = (W)h, h2 = hh * hh;
        w[0] = ((W)1 - hh) * ((W)1 - hh) * ((W)1 - hh) / (W)6;
        w[1] = (W)4 / (W)6 + ((W)0.5 * hh - (W)1) * h2;
        w[3] = h2 * hh / (W)6;
        w[2] = (W)1 - w[0] - w[1] - w[3];
    } else if (nintp == 3) {
        long long iv = llround(v);             // nint(vr)
        first = (int)((iv - 2) % N);
        h = v - (double)iv;
        W hh = (W)h, h2 = hh * hh;
        w[0] = (W)0.5 * ((W)0.5 - hh) * ((W)0.5 - hh);
        w[1] = (W)0.75 - h2;
        w[2] = (W)1 - w[0] - w[1];
        w[3] = 0;
    } else if (nintp == 2) {
        long long iv = (long long)v;           // int(vr)
        first = (int)(iv % N);                  // mod(ivr - 1 + 1 + N, N)
        h = cic_nint ? v - (double)llround(v) : v - (double)iv;
        w[0] = (W)1 - (W)h;
        w[1] = (W)h;
        w[2] = w[3] = 0;
    } else {
        long long iv = llround(v);             // nint(vr)
        first = (int)((iv - 1) % N);            // mod(ivr - 1 + N, N)
        w[0] = 1;
        w[1] = w[2] = w[3] = 0;
    }
    // Negative or non-finite coordinates are outside the reference's domain;
    // keep the index in range so no access leaves the grid.
    if (first < 0) first += N;
    if (first < 0 || first >= N) first = 0;
}

template <class W>
__device__ __forceinline__ long long to_fixed(W c, double scale) {
    return __double2ll_rn((double)c * scale);
}

// ---------------------------------------------------------------- direct ---
template <class W>
__global__ void assign_direct_kernel(int N, int nintp, int64_t npart, const double *__restrict__ pos,
                                     const double *__restrict__ weight, double scale, int interlaced,
                                     unsigned long long *__restrict__ g1, unsigned long long *__restrict__ g2) {
    const size_t NN = (size_t)N * N;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < npart;
         i += (int64_t)gridDim.x * blockDim.x) {
        const double p0 = pos[i], p1 = pos[npart + i], p2 = pos[2 * npart + i];
        const W wt = weight ? (W)weight[i] : (W)1;
        for (int g = 0; g < (interlaced ? 2 : 1); g++) {
            int f0, f1, f2;
            W wx[4], wy[4], wz[4];
            const bool shifted = g == 1, cic_nint = !interlaced;
            axis_stencil<W>(p0, N, nintp, shifted, cic_nint, f0, wx);
            axis_stencil<W>(p1, N, nintp, shifted, cic_nint, f1, wy);
            axis_stencil<W>(p2, N, nintp, shifted, cic_nint, f2, wz);
            unsigned long long *grid = g ? g2 : g1;
            for (int a = 0; a < nintp; a++) {
                int x = f0 + a; x -= (x >= N) ? N : 0;
                for (int b = 0; b < nintp; b++) {
                    int y = f1 + b; y -= (y >= N) ? N : 0;
                    W wxy = wx[a] * wy[b];
                    for (int c = 0; c < nintp; c++) {
                        int z = f2 + c; z -= (z >= N) ? N : 0;
                        long long q = to_fixed<W>(wxy * wz[c] * wt, scale);
                        atomicAdd(grid + (size_t)z * NN + (size_t)y * N + x, (unsigned long long)q);
                    }
                }
            }
        }
    }
}

// ----------------------------------------------------------------- tiled ---
// Tile of TS^3 cells; the stencil of a particle whose first cell lies in the
// tile reaches at most nintp-1 cells further, so the shared accumulator covers
// (TS+3)^3 cells.  Particles are binned by the tile of their first cell
// (grid 1; the interlaced grid's first cell is the same or one cell lower,
// which the halo covers by starting the accumulator one cell early).
constexpr int kTile = 8;
constexpr int kHalo = 4;                   // 1 cell below + up to 3 above
constexpr int kAcc = kTile + kHalo;        // 12
constexpr int kAccCells = kAcc * kAcc * kAcc;  // 1728 x 8 B = 13.8 KB per grid

__device__ __forceinline__ int tile_of(double p, int N, int nintp, int ntile_axis) {
    int f;
    float w[4];
    axis_stencil<float>(p, N, nintp, false, false, f, w);
    return f / kTile < ntile_axis ? f / kTile : ntile_axis - 1;
}

__global__ void tile_count_kernel(int N, int nintp, int64_t npart, const double *__restrict__ pos, int nt,
                                  unsigned int *__restrict__ tile_count, unsigned int *__restrict__ ptile) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < npart;
         i += (int64_t)gridDim.x * blockDim.x) {
        int tx = tile_of(pos[i], N, nintp, nt);
        int ty = tile_of(pos[npart + i], N, nintp, nt);
        int tz = tile_of(pos[2 * npart + i], N, nintp, nt);
        unsigned int t = (unsigned)((tz * nt + ty) * nt + tx);
        ptile[i] = t;
        atomicAdd(tile_count + t, 1u);
    }
}

// exclusive scan of tile counts by a single CTA (number of tiles <= 2^21)
__global__ void tile_scan_kernel(int ntiles, const unsigned int *__restrict__ count, unsigned int *__restrict__ start,
                                 unsigned int *__restrict__ cursor) {
    __shared__ unsigned int warp_tot[32];
    __shared__ unsigned int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int base = 0; base < ntiles; base += blockDim.x) {
        int i = base + threadIdx.x;
        unsigned int v = i < ntiles ? count[i] : 0u, x = v;
        for (int o = 1; o < 32; o <<= 1) {
            unsigned int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_tot[wid] = x;
        __syncthreads();
        if (wid == 0) {
            unsigned int t = lane < (int)(blockDim.x >> 5) ? warp_tot[lane] : 0u;
            for (int o = 1; o < 32; o <<= 1) {
                unsigned int y = __shfl_up_sync(0xffffffffu, t, o);
                if (lane >= o) t += y;
            }
            warp_tot[lane] = t;
        }
        __syncthreads();
        unsigned int excl = carry + x - v + (wid ? warp_tot[wid - 1] : 0u);
        if (i < ntiles) { start[i] = excl; cursor[i] = excl; }
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry = excl + v;
        __syncthreads();
    }
    if (threadIdx.x == 0) start[ntiles] = carry;
}

__global__ void tile_scatter_kernel(int64_t npart, const unsigned int *__restrict__ ptile,
                                    unsigned int *__restrict__ cursor, unsigned int *__restrict__ order) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < npart;
         i += (int64_t)gridDim.x * blockDim.x)
        order[atomicAdd(cursor + ptile[i], 1u)] = (unsigned int)i;
}

template <class W>
__global__ void __launch_bounds__(256) assign_tiled_kernel(int N, int nintp, int64_t npart,
                                                           const double *__restrict__ pos,
                                                           const double *__restrict__ weight, double scale,
                                                           int interlaced, int nt,
                                                           const unsigned int *__restrict__ start,
                                                           const unsigned int *__restrict__ order,
                                                           unsigned long long *__restrict__ g1,
                                                           unsigned long long *__restrict__ g2) {
    __shared__ unsigned long long acc[2][kAccCells];
    const size_t NN = (size_t)N * N;
    const int ntiles = nt * nt * nt;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const unsigned int b = start[tile], e = start[tile + 1];
        if (b == e) continue;
        const int tx = tile % nt, ty = (tile / nt) % nt, tz = tile / (nt * nt);
        // accumulator origin: one cell below the tile (interlaced grid reaches it)
        const int ox = tx * kTile - 1, oy = ty * kTile - 1, oz = tz * kTile - 1;
        for (int c = threadIdx.x; c < kAccCells * 2; c += blockDim.x) (&acc[0][0])[c] = 0ull;
        __syncthreads();
        for (unsigned int k = b + threadIdx.x; k < e; k += blockDim.x) {
            const unsigned int i = order[k];
            const double p0 = pos[i], p1 = pos[npart + i], p2 = pos[2 * (size_t)npart + i];
            const W wt = weight ? (W)weight[i] : (W)1;
            for (int g = 0; g < (interlaced ? 2 : 1); g++) {
                int f0, f1, f2;
                W wx[4], wy[4], wz[4];
                const bool shifted = g == 1, cic_nint = !interlaced;
                axis_stencil<W>(p0, N, nintp, shifted, cic_nint, f0, wx);
                axis_stencil<W>(p1, N, nintp, shifted, cic_nint, f1, wy);
                axis_stencil<W>(p2, N, nintp, shifted, cic_nint, f2, wz);
                // local coordinates; a first cell that wrapped below 0 maps to N-1
                int lx = f0 - ox, ly = f1 - oy, lz = f2 - oz;
                if (lx < 0) lx += N; if (ly < 0) ly += N; if (lz < 0) lz += N;
                if (lx >= N) lx -= N; if (ly >= N) ly -= N; if (lz >= N) lz -= N;
                const bool inside = lx + nintp <= kAcc && ly + nintp <= kAcc && lz + nintp <= kAcc;
                for (int a = 0; a < nintp; a++)
                    for (int bb = 0; bb < nintp; bb++) {
                        W wxy = wx[a] * wy[bb];
                        for (int c = 0; c < nintp; c++) {
                            long long q = to_fixed<W>(wxy * wz[c] * wt, scale);
                            if (inside) {
                                atomicAdd(&acc[g][((lz + c) * kAcc + (ly + bb)) * kAcc + (lx + a)],
                                          (unsigned long long)q);
                            } else {  // cannot happen for tiles built by tile_of; kept as a safe path
                                int x = f0 + a; x -= (x >= N) ? N : 0;
                                int y = f1 + bb; y -= (y >= N) ? N : 0;
                                int z = f2 + c; z -= (z >= N) ? N : 0;
                                unsigned long long *grid = g ? g2 : g1;
                                atomicAdd(grid + (size_t)z * NN + (size_t)y * N + x, (unsigned long long)q);
                            }
                        }
                    }
            }
        }
        __syncthreads();
        for (int g = 0; g < (interlaced ? 2 : 1); g++) {
            unsigned long long *grid = g ? g2 : g1;
            for (int c = threadIdx.x; c < kAccCells; c += blockDim.x) {
                unsigned long long v = acc[g][c];
                if (v == 0ull) continue;
                int lx = c % kAcc, ly = (c / kAcc) % kAcc, lz = c / (kAcc * kAcc);
                int x = (ox + lx + N) % N, y = (oy + ly + N) % N, z = (oz + lz + N) % N;
                atomicAdd(grid + (size_t)z * NN + (size_t)y * N + x, v);
            }
        }
        __syncthreads();
    }
}

// --------------------------------------------------------------- helpers ---
__global__ void weight_absmax_kernel(int64_t n, const double *__restrict__ w, unsigned long long *__restrict__ out) {
    double m = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double a = fabs(w[i]);
        if (!(a <= 1e300)) a = 1e308;  // NaN/inf -> flagged by the host
        m = fmax(m, a);
    }
    for (int o = 16; o; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(m));
}

template <class R>
__global__ void fixed_to_real_kernel(size_t n, const unsigned long long *__restrict__ g, R inv_scale,
                                     R *__restrict__ out) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = (R)(long long)g[i] * inv_scale;
}

// double grid -> interleaved complex128 (Re = grid 1, Im = grid 2)
__global__ void fixed_to_complex_kernel(size_t n, const unsigned long long *__restrict__ g1,
                                        const unsigned long long *__restrict__ g2, double inv_scale,
                                        double2 *__restrict__ out) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = make_double2((double)(long long)g1[i] * inv_scale, (double)(long long)g2[i] * inv_scale);
}

// ------------------------------------------------------------ host side ---
int fixed_point_bits(int64_t npart, double wmax, int *bits) {
    if (!(wmax >= 0.0) || wmax > 1e300) return set_error(PBI4G_ERR_RANGE, "non-finite particle weight");
    double bound = (double)(npart > 0 ? npart : 1) * (wmax > 0 ? wmax : 1.0) * 4.0;  // |w_x w_y w_z| <= 3.375
    int s = (int)floor(62.0 - log2(bound));
    if (s > 50) s = 50;
    if (s < 12)
        return set_error(PBI4G_ERR_RANGE, "fixed-point range exceeded: npart*max|weight| = %g", bound / 4);
    *bits = s;
    return PBI4G_OK;
}

int AssignWork::ensure(int N, int64_t npart, bool interlaced) {
    const size_t cells = full_cells(N);
    PBI4G_CHECK(grids.ensure(cells * sizeof(unsigned long long) * (interlaced ? 2 : 1)));
    const int nt = (N + kTile - 1) / kTile;
    const size_t ntiles = (size_t)nt * nt * nt;
    PBI4G_CHECK(tile_count.ensure((ntiles + 1) * sizeof(unsigned int)));
    PBI4G_CHECK(tile_start.ensure((ntiles + 1) * sizeof(unsigned int)));
    PBI4G_CHECK(tile_cursor.ensure((ntiles + 1) * sizeof(unsigned int)));
    PBI4G_CHECK(ptile.ensure((size_t)(npart > 0 ? npart : 1) * sizeof(unsigned int)));
    PBI4G_CHECK(order.ensure((size_t)(npart > 0 ? npart : 1) * sizeof(unsigned int)));
    PBI4G_CHECK(wmax.ensure(sizeof(unsigned long long)));
    return PBI4G_OK;
}

size_t AssignWork::footprint(int N, int64_t npart, bool interlaced) {
    const int nt = (N + kTile - 1) / kTile;
    const size_t ntiles = (size_t)nt * nt * nt;
    return full_cells(N) * 8 * (interlaced ? 2 : 1) + 3 * (ntiles + 1) * 4 + 2 * (size_t)npart * 4 + 64;
}

int assign_fixed(AssignWork &wk, int N, int nintp, bool interlaced, bool fp64_weights, int64_t npart,
                 const double *d_pos, const double *d_weight, int *bits_out, cudaStream_t st, int64_t *launches) {
    if (N < 2 || nintp < 1 || nintp > 4 || npart < 0)
        return set_error(PBI4G_ERR_INVALID, "assign: bad grid=%d nintp=%d npart=%lld", N, nintp, (long long)npart);
    if (npart > 0 && !d_pos) return set_error(PBI4G_ERR_INVALID, "assign: null positions");
    if (npart >= (int64_t)0xffffffffLL) return set_error(PBI4G_ERR_RANGE, "assign: npart >= 2^32");
    PBI4G_CHECK(wk.ensure(N, npart, interlaced));
    const size_t cells = full_cells(N);
    unsigned long long *g1 = wk.grids.as<unsigned long long>();
    unsigned long long *g2 = interlaced ? g1 + cells : nullptr;
    PBI4G_CUDA(cudaMemsetAsync(g1, 0, cells * 8 * (interlaced ? 2 : 1), st));
    double wmax = 1.0;
    if (d_weight && npart > 0) {
        PBI4G_CUDA(cudaMemsetAsync(wk.wmax.p, 0, 8, st));
        weight_absmax_kernel<<<grid_blocks(npart, 256, 152 * 8), 256, 0, st>>>(npart, d_weight,
                                                                                wk.wmax.as<unsigned long long>());
        PBI4G_LAUNCH_CHECK();
        ++*launches;
        unsigned long long bitsw = 0;
        PBI4G_CUDA(cudaMemcpyAsync(&bitsw, wk.wmax.p, 8, cudaMemcpyDeviceToHost, st));
        PBI4G_CUDA(cudaStreamSynchronize(st));
        memcpy(&wmax, &bitsw, 8);
    }
    int bits;
    PBI4G_CHECK(fixed_point_bits(npart, wmax, &bits));
    *bits_out = bits;
    if (npart == 0) return PBI4G_OK;
    const double scale = ldexp(1.0, bits);
    const int nt = (N + kTile - 1) / kTile;
    const int ntiles = nt * nt * nt;
    // Tiling pays when tiles hold several particles on average.
    const bool tiled = N >= 2 * kTile && npart >= (int64_t)ntiles * 2;
    if (!tiled) {
        if (fp64_weights)
            assign_direct_kernel<double><<<grid_blocks(npart, 256), 256, 0, st>>>(N, nintp, npart, d_pos, d_weight,
                                                                                 scale, interlaced, g1, g2);
        else
            assign_direct_kernel<float><<<grid_blocks(npart, 256), 256, 0, st>>>(N, nintp, npart, d_pos, d_weight,
                                                                                scale, interlaced, g1, g2);
        PBI4G_LAUNCH_CHECK();
        ++*launches;
        return PBI4G_OK;
    }
    unsigned int *cnt = wk.tile_count.as<unsigned int>();
    PBI4G_CUDA(cudaMemsetAsync(cnt, 0, (size_t)(ntiles + 1) * 4, st));
    tile_count_kernel<<<grid_blocks(npart, 256), 256, 0, st>>>(N, nintp, npart, d_pos, nt, cnt,
                                                               wk.ptile.as<unsigned int>());
    PBI4G_LAUNCH_CHECK();
    tile_scan_kernel<<<1, 1024, 0, st>>>(ntiles, cnt, wk.tile_start.as<unsigned int>(),
                                         wk.tile_cursor.as<unsigned int>());
    PBI4G_LAUNCH_CHECK();
    tile_scatter_kernel<<<grid_blocks(npart, 256), 256, 0, st>>>(npart, wk.ptile.as<unsigned int>(),
                                                                 wk.tile_cursor.as<unsigned int>(),
                                                                 wk.order.as<unsigned int>());
    PBI4G_LAUNCH_CHECK();
    const int blocks = ntiles < 152 * 8 ? ntiles : 152 * 8;
    if (fp64_weights)
        assign_tiled_kernel<double><<<blocks, 256, 0, st>>>(N, nintp, npart, d_pos, d_weight, scale, interlaced, nt,
                                                           wk.tile_start.as<unsigned int>(),
                                                           wk.order.as<unsigned int>(), g1, g2);
    else
        assign_tiled_kernel<float><<<blocks, 256, 0, st>>>(N, nintp, npart, d_pos, d_weight, scale, interlaced, nt,
                                                          wk.tile_start.as<unsigned int>(),
                                                          wk.order.as<unsigned int>(), g1, g2);
    PBI4G_LAUNCH_CHECK();
    *launches += 4;
    return PBI4G_OK;
}

int fixed_to_real(const AssignWork &wk, int N, bool interlaced, int bits, bool fp64, void *out, cudaStream_t st,
                  int64_t *launches) {
    const size_t n = full_cells(N) * (interlaced ? 2 : 1);
    if (fp64)
        fixed_to_real_kernel<double><<<grid_blocks(n, 256), 256, 0, st>>>(
            n, wk.grids.as<unsigned long long>(), ldexp(1.0, -bits), static_cast<double *>(out));
    else
        fixed_to_real_kernel<float><<<grid_blocks(n, 256), 256, 0, st>>>(
            n, wk.grids.as<unsigned long long>(), ldexpf(1.0f, -bits), static_cast<float *>(out));
    PBI4G_LAUNCH_CHECK();
    ++*launches;
    return PBI4G_OK;
}

int fixed_to_complex(const AssignWork &wk, int N, int bits, double2 *out, cudaStream_t st, int64_t *launches) {
    const size_t n = full_cells(N);
    const unsigned long long *g = wk.grids.as<unsigned long long>();
    fixed_to_complex_kernel<<<grid_blocks(n, 256), 256, 0, st>>>(n, g, g + n, ldexp(1.0, -bits), out);
    PBI4G_LAUNCH_CHECK();
    ++*launches;
    return PBI4G_OK;
}

}  // namespace pbi4g
