// dropin.cu -- the f2py drop-in entry points (host buffers in/out), one per
// routine that the reference's pbi4.py imports from powerI4 / bispectrumI4
// (pbi4.py:12-14).  Each copies its inputs to the current device, runs the
// GPU kernels and copies the outputs back; Fortran-ordered grids throughout.
#include "assign.cuh"
#include "engine.cuh"

#include <math.h>
#include <string.h>
#include <algorithm>
#include <memory>
#include <vector>

using namespace pbi4g;

namespace {

int g_dropin_precision = PBI4G_PREC_FP32;

// kx >= 0 half (x in [0, N/2]) of a Fortran-ordered full complex grid -> device [z][y][x]
int upload_half(int N, const double *host_full, DevBuf &out, cudaStream_t st) {
    const int NH = N / 2 + 1;
    PBI4G_CHECK(out.ensure(sizeof(double2) * half_cells(N)));
    PBI4G_CUDA(cudaMemcpy2DAsync(out.p, sizeof(double2) * NH, host_full, sizeof(double2) * N, sizeof(double2) * NH,
                                 (size_t)N * N, cudaMemcpyHostToDevice, st));
    return PBI4G_OK;
}

__global__ void d2f_kernel(size_t n, const double2 *__restrict__ in, float2 *__restrict__ out) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = make_float2((float)in[i].x, (float)in[i].y);
}

int check_grid(int N) {
    if (N < 2 || N > 2048) return set_error(PBI4G_ERR_INVALID, "grid out of range: %d", N);
    return PBI4G_OK;
}

int assign_common(int32_t grid, int32_t nintp, int64_t npart, const double *pos, const double *weight, bool interlaced,
                  double *out) {
    PBI4G_CHECK(check_grid(grid));
    if (nintp < 1 || nintp > 4) return set_error(PBI4G_ERR_INVALID, "nintp must be 1..4");
    if (!out || (npart > 0 && (!pos || !weight))) return set_error(PBI4G_ERR_INVALID, "null argument");
    cudaStream_t st = 0;
    int64_t launches = 0;
    AssignWork aw;
    DevBuf dpos, dw, dout;
    if (npart > 0) {
        PBI4G_CHECK(dpos.ensure(sizeof(double) * 3 * (size_t)npart));
        PBI4G_CHECK(dw.ensure(sizeof(double) * (size_t)npart));
        PBI4G_CUDA(cudaMemcpyAsync(dpos.p, pos, sizeof(double) * 3 * (size_t)npart, cudaMemcpyHostToDevice, st));
        PBI4G_CUDA(cudaMemcpyAsync(dw.p, weight, sizeof(double) * (size_t)npart, cudaMemcpyHostToDevice, st));
    }
    int bits = 0;
    PBI4G_CHECK(assign_fixed(aw, grid, nintp, interlaced, true, npart, dpos.as<double>(), dw.as<double>(), &bits, st,
                             &launches));
    const size_t FC = full_cells(grid);
    PBI4G_CHECK(dout.ensure(FC * (interlaced ? 16 : 8)));
    if (interlaced)
        PBI4G_CHECK(fixed_to_complex(aw, grid, bits, dout.as<double2>(), st, &launches));
    else
        PBI4G_CHECK(fixed_to_real(aw, grid, false, bits, true, dout.p, st, &launches));
    PBI4G_CUDA(cudaMemcpyAsync(out, dout.p, FC * (interlaced ? 16 : 8), cudaMemcpyDeviceToHost, st));
    PBI4G_CUDA(cudaStreamSynchronize(st));
    return PBI4G_OK;
}

// Bispectrum drop-ins: nsrc half spectra uploaded, set layout per routine.
int bk_common(int32_t nbins, int32_t grid, float kbin, float kcenter, int32_t iopen, float kf, int64_t itot,
              int64_t npart, const float *counts, const double *const *fulls, int nsrc, int nsets, int cross,
              int rows, double *bout) {
    PBI4G_CHECK(check_grid(grid));
    if (grid < 4 || (grid & 1)) return set_error(PBI4G_ERR_INVALID, "grid must be even");
    if (!bout || !counts) return set_error(PBI4G_ERR_INVALID, "null argument");
    if (npart < 1) return set_error(PBI4G_ERR_INVALID, "npart must be >= 1");
    cudaStream_t st = 0;
    int64_t launches = 0;
    std::unique_ptr<BkEngine> bk(new BkEngine());
    PBI4G_CHECK(bk->sh.build(grid, kbin, kcenter, nbins, iopen, cross, st));
    if (bk->sh.itot != itot)
        return set_error(PBI4G_ERR_INVALID, "itot=%lld does not match the triangle enumeration (%lld)",
                         (long long)itot, (long long)bk->sh.itot);
    bk->nsets = nsets;
    bk->cross = cross;
    bk->tc_mode = tc_mode_of(g_dropin_precision);
    DevBuf h[3], hf[3], dcounts, dbout;
    for (int s = 0; s < nsrc; s++) {
        if (!fulls[s]) return set_error(PBI4G_ERR_INVALID, "null grid");
        PBI4G_CHECK(upload_half(grid, fulls[s], h[s], st));
    }
    PBI4G_CHECK(dcounts.ensure(sizeof(float) * itot));
    PBI4G_CUDA(cudaMemcpyAsync(dcounts.p, counts, sizeof(float) * itot, cudaMemcpyHostToDevice, st));
    PBI4G_CHECK(dbout.ensure(sizeof(double) * rows * itot));
    const int fac[3] = {0, 0, 0};  // explicit delta_2 / delta_4 grids
    const double los[3] = {0, 0, 1};
    if (g_dropin_precision == PBI4G_PREC_FP64) {
        const double2 *src[3] = {h[0].as<double2>(), h[nsrc > 1 ? 1 : 0].as<double2>(),
                                 h[nsrc > 2 ? 2 : 0].as<double2>()};
        PBI4G_CHECK(bk->run<double>(src, fac, los, kf, npart, dcounts.as<float>(), dbout.as<double>(), st, &launches));
    } else {
        const size_t HC = half_cells(grid);
        for (int s = 0; s < nsrc; s++) {
            PBI4G_CHECK(hf[s].ensure(sizeof(float2) * HC));
            d2f_kernel<<<grid_blocks(HC, 256), 256, 0, st>>>(HC, h[s].as<double2>(), hf[s].as<float2>());
            PBI4G_LAUNCH_CHECK();
            h[s].release();
        }
        const float2 *src[3] = {hf[0].as<float2>(), hf[nsrc > 1 ? 1 : 0].as<float2>(), hf[nsrc > 2 ? 2 : 0].as<float2>()};
        PBI4G_CHECK(bk->run<float>(src, fac, los, kf, npart, dcounts.as<float>(), dbout.as<double>(), st, &launches));
    }
    PBI4G_CUDA(cudaMemcpyAsync(bout, dbout.p, sizeof(double) * rows * itot, cudaMemcpyDeviceToHost, st));
    PBI4G_CUDA(cudaStreamSynchronize(st));
    return bk->check(st);
}

}  // namespace

extern "C" {

int pbi4g_set_dropin_precision(int32_t precision) {
    if (precision < PBI4G_PREC_FP32 || precision > PBI4G_PREC_TF32SPLIT)
        return set_error(PBI4G_ERR_INVALID, "unknown precision %d", precision);
    g_dropin_precision = precision;
    return PBI4G_OK;
}

int pbi4g_assign_single_grid(int32_t grid, int32_t nintp, int64_t npart, const double *pos, const double *weight,
                             double *dtl) {
    return assign_common(grid, nintp, npart, pos, weight, false, dtl);
}

int pbi4g_assign_double_grid(int32_t grid, int32_t nintp, int64_t npart, const double *pos, const double *weight,
                             double *dcl) {
    return assign_common(grid, nintp, npart, pos, weight, true, dcl);
}

int pbi4g_fcomb(int32_t grid, int32_t nintp, int32_t interlacing, float box, const double *fdcl, double *dcl) {
    PBI4G_CHECK(check_grid(grid));
    if ((grid & 1) || !fdcl || !dcl) return set_error(PBI4G_ERR_INVALID, "fcomb: even grid and non-null grids required");
    if (nintp < 1 || nintp > 4) return set_error(PBI4G_ERR_INVALID, "nintp must be 1..4");
    DevBuf d;
    const size_t bytes = full_cells(grid) * 16;
    PBI4G_CHECK(d.ensure(bytes));
    PBI4G_CUDA(cudaMemcpy(d.p, fdcl, bytes, cudaMemcpyHostToDevice));
    PBI4G_CHECK(fcomb_full(grid, nintp, interlacing != 0, box, d.as<double2>(), d.as<double2>(), 0));
    PBI4G_CUDA(cudaMemcpy(dcl, d.p, bytes, cudaMemcpyDeviceToHost));
    return PBI4G_OK;
}

int pbi4g_reduce_array(int32_t L, const double *din, int32_t grid, double *dout) {
    PBI4G_CHECK(check_grid(grid));
    PBI4G_CHECK(check_grid(L));
    if (L < grid || !din || !dout) return set_error(PBI4G_ERR_INVALID, "reduce_array needs L >= grid (L=%d grid=%d)", L, grid);
    DevBuf a, b;
    PBI4G_CHECK(a.ensure(full_cells(L) * 16));
    PBI4G_CHECK(b.ensure(full_cells(grid) * 16));
    PBI4G_CUDA(cudaMemcpy(a.p, din, full_cells(L) * 16, cudaMemcpyHostToDevice));
    PBI4G_CUDA(cudaMemset(b.p, 0, full_cells(grid) * 16));
    PBI4G_CHECK(reduce_full(L, a.as<double2>(), grid, b.as<double2>(), 0));
    PBI4G_CUDA(cudaMemcpy(dout, b.p, full_cells(grid) * 16, cudaMemcpyDeviceToHost));
    return PBI4G_OK;
}

static int qlk_common(int32_t grid, float box, const double *in, int n, const int *idx, double *out) {
    PBI4G_CHECK(check_grid(grid));
    if (!in || !out) return set_error(PBI4G_ERR_INVALID, "null grid");
    DevBuf a, b;
    const size_t bytes = full_cells(grid) * 16;
    PBI4G_CHECK(a.ensure(bytes));
    PBI4G_CHECK(b.ensure(bytes));
    PBI4G_CUDA(cudaMemcpy(a.p, in, bytes, cudaMemcpyHostToDevice));
    if (n == 2)
        PBI4G_CHECK(q2k_full(grid, box, a.as<double2>(), idx[0], idx[1], b.as<double2>(), 0));
    else
        PBI4G_CHECK(q4k_full(grid, box, a.as<double2>(), idx[0], idx[1], idx[2], idx[3], b.as<double2>(), 0));
    PBI4G_CUDA(cudaMemcpy(out, b.p, bytes, cudaMemcpyDeviceToHost));
    return PBI4G_OK;
}

int pbi4g_compute_q2k(int32_t grid, float box, const double *deltak, int32_t i, int32_t j, double *q2k) {
    const int idx[2] = {i, j};
    return qlk_common(grid, box, deltak, 2, idx, q2k);
}

int pbi4g_compute_q4k(int32_t grid, float box, const double *deltak, int32_t i, int32_t j, int32_t l, int32_t k,
                      double *q4k) {
    const int idx[4] = {i, j, l, k};
    return qlk_common(grid, box, deltak, 4, idx, q4k);
}

static int pk_common(int32_t grid, float box, float kbin, float kcenter, int32_t nbins, const double *a,
                     const double *b, const double *c, int mode, double *pout) {
    PBI4G_CHECK(check_grid(grid));
    if ((grid & 1) || !a || !b || (mode == 2 && !c) || !pout)
        return set_error(PBI4G_ERR_INVALID, "measure_pk: even grid and non-null arrays required");
    cudaStream_t st = 0;
    int64_t launches = 0;
    PkBins bins;
    PBI4G_CHECK(bins.build(grid, box, kbin, kcenter, nbins, st, &launches));
    DevBuf ha, hb, hc, dp;
    PBI4G_CHECK(upload_half(grid, a, ha, st));
    PBI4G_CHECK(upload_half(grid, b, hb, st));
    if (mode == 2) PBI4G_CHECK(upload_half(grid, c, hc, st));
    PBI4G_CHECK(dp.ensure(sizeof(double) * 5 * nbins));
    PBI4G_CHECK(pk_measure<double>(bins, mode, nullptr, ha.as<double2>(), hb.as<double2>(),
                                   mode == 2 ? hc.as<double2>() : nullptr, dp.as<double>(), st, &launches));
    PBI4G_CUDA(cudaMemcpyAsync(pout, dp.p, sizeof(double) * 5 * nbins, cudaMemcpyDeviceToHost, st));
    PBI4G_CUDA(cudaStreamSynchronize(st));
    return PBI4G_OK;
}

int pbi4g_measure_pk(int32_t grid, float box, float kbin, float kcenter, int32_t nbins, const double *dcl1,
                     const double *dcl2, double *pout) {
    return pk_common(grid, box, kbin, kcenter, nbins, dcl1, dcl2, nullptr, 0, pout);
}

int pbi4g_measure_pk_multipoles(int32_t grid, float box, float kbin, float kcenter, int32_t nbins, const double *dcl,
                                const double *dcl2, const double *dcl4, double *pout) {
    return pk_common(grid, box, kbin, kcenter, nbins, dcl, dcl2, dcl4, 2, pout);
}

int pbi4g_count_triangles(int32_t nbins, int32_t grid, float kbin, float kcenter, int32_t iopen, int32_t cross,
                          int32_t npool, int64_t itot, double *counts) {
    (void)npool;
    PBI4G_CHECK(check_grid(grid));
    if (!counts) return set_error(PBI4G_ERR_INVALID, "null counts");
    Shells sh;
    PBI4G_CHECK(sh.build(grid, kbin, kcenter, nbins, iopen, cross, 0));
    if (sh.itot != itot)
        return set_error(PBI4G_ERR_INVALID, "itot=%lld does not match the triangle enumeration (%lld)",
                         (long long)itot, (long long)sh.itot);
    int64_t launches = 0;
    PBI4G_CHECK(triangle_counts(sh, 0, &launches));
    const double gridD = (double)grid * grid * grid;
    for (int64_t m = 0; m < itot; m++) counts[m] = gridD * (double)sh.counts[m];
    return PBI4G_OK;
}

int pbi4g_measure_bk(int32_t nbins, int32_t grid, float kbin, float kcenter, int32_t iopen, float kf, int32_t npool,
                     int64_t itot, int64_t npart, const float *counts, const double *dcl, double *bout) {
    (void)npool;
    const double *f[1] = {dcl};
    return bk_common(nbins, grid, kbin, kcenter, iopen, kf, itot, npart, counts, f, 1, 1, 0, 9, bout);
}

int pbi4g_measure_bk_multipoles(int32_t nbins, int32_t grid, float kbin, float kcenter, int32_t iopen, float kf,
                                int32_t npool, int64_t itot, int64_t npart, const float *counts, const double *dcl,
                                const double *dcl2, const double *dcl4, double *bout) {
    (void)npool;
    const double *f[3] = {dcl, dcl2, dcl4};
    return bk_common(nbins, grid, kbin, kcenter, iopen, kf, itot, npart, counts, f, 3, 3, 0, 11, bout);
}

int pbi4g_measure_bk_cross(int32_t nbins, int32_t grid, float kbin, float kcenter, int32_t iopen, float kf,
                           int32_t npool, int64_t itot, int64_t npart, const float *counts, const double *dcl1,
                           const double *dcl2, double *bout) {
    (void)npool;
    const double *f[2] = {dcl1, dcl2};
    return bk_common(nbins, grid, kbin, kcenter, iopen, kf, itot, npart, counts, f, 2, 1, 1, 5, bout);
}

}  // extern "C"
