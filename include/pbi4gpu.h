/*
 * pbi4gpu.h -- C ABI of the GB300 (sm_103a) PBI4 estimator library (libpbi4gpu.so).
 *
 * Two groups of entry points:
 *
 *  1. Drop-ins for the f2py routines the reference's pbi4/pbi4.py imports
 *     (`from powerI4 import ...`, `from bispectrumI4 import ...`, pbi4.py:12-14).
 *     Same arguments, same meaning, host buffers in and out, Fortran-ordered
 *     3-D grids (a(ix,iy,iz) with ix fastest), complex grids as interleaved
 *     (re, im) float64.  Outputs are fully written (f2py zero-fills them).
 *     The computation runs on the current CUDA device; copies are inside.
 *
 *  2. A device-resident estimator plan (the throughput path): positions in
 *     HBM -> density -> P(k) multipoles -> bispectrum, with FFT plans, shell
 *     tables and triangle counts kept resident between boxes.
 *
 * Every function returns PBI4G_OK (0) or a PBI4G_ERR_* code and never exits the
 * process; pbi4g_last_error() gives the message of the calling thread's last
 * failure.  Scalar kinds follow the Fortran interfaces: `real` -> float,
 * `real(kind=8)` -> double, `integer` -> int32_t, `integer(kind=8)` -> int64_t,
 * `logical` -> int32_t (0/1).
 */
#ifndef PBI4GPU_H
#define PBI4GPU_H

#include <stdint.h>

#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define PBI4G_OK 0
#define PBI4G_ERR_INVALID 1     /* bad argument (sizes, ranges, null pointers) */
#define PBI4G_ERR_CUDA 2        /* CUDA runtime error */
#define PBI4G_ERR_NOMEM 3       /* device allocation failed */
#define PBI4G_ERR_CUFFT 4       /* cuFFT error */
#define PBI4G_ERR_TIMEOUT 5     /* a bounded device wait gave up */
#define PBI4G_ERR_UNSUPPORTED 6 /* option not supported by this build / device */
#define PBI4G_ERR_RANGE 7       /* input outside the documented range (e.g. fixed-point bound) */

/* Arithmetic of the shell maps and triangle sums (and of the FFTs for FP64). */
#define PBI4G_PREC_FP32 0      /* plain form: FP32 FFTs, maps and products, FP64 bin reductions */
#define PBI4G_PREC_FP64 1      /* FP64 everywhere (GPU oracle form) */
#define PBI4G_PREC_FP16SPLIT 2 /* mixed: maps as FP16 hi+lo, tensor-core sums, FP32 accumulate */
#define PBI4G_PREC_BF16 3      /* mixed: maps as BF16, tensor-core sums, FP32 accumulate */
#define PBI4G_PREC_TF32SPLIT 4 /* mixed: maps and pair products as TF32 hi+lo, tensor-core sums, FP32 accumulate */

const char *pbi4g_last_error(void);
int pbi4g_version(void);
/* Precision used by the drop-in bispectrum entry points (default FP32); the
 * tensor-core forms apply to measure_bk and measure_bk_multipoles (cross
 * spectra use the CUDA-core FP32 form). */
int pbi4g_set_dropin_precision(int32_t precision);

/* ---------------- 1. f2py drop-ins: powerI4 ---------------- */

/* replaces powerI4.f90:68-140 assign_single_grid.  pos: (3, npart) float64,
 * C order (pos[c*npart + i]); weight: npart float64; dtl: grid^3 float64.
 * Accumulation is 64-bit fixed point, so dtl is bit-reproducible. */
int pbi4g_assign_single_grid(int32_t grid, int32_t nintp, int64_t npart, const double *pos,
                             const double *weight, double *dtl);
/* replaces powerI4.f90:142-249 assign_double_grid; dcl: grid^3 complex128,
 * Re = grid at x, Im = grid at x - 1/2 cell. */
int pbi4g_assign_double_grid(int32_t grid, int32_t nintp, int64_t npart, const double *pos,
                             const double *weight, double *dcl);
/* replaces powerI4.f90:251-378 fcomb (interlacing combine + window deconvolution
 * of a full complex FFT); fdcl and dcl: grid^3 complex128 (may alias). */
int pbi4g_fcomb(int32_t grid, int32_t nintp, int32_t interlacing, float box, const double *fdcl,
                double *dcl);
/* replaces powerI4.f90:380-407 reduce_array; din: L^3, dout: grid^3 complex128. */
int pbi4g_reduce_array(int32_t L, const double *din, int32_t grid, double *dout);
/* replaces powerI4.f90:409-458 compute_q2k (1-based i, j). */
int pbi4g_compute_q2k(int32_t grid, float box, const double *deltak, int32_t i, int32_t j, double *q2k);
/* replaces powerI4.f90:460-508 compute_q4k (1-based i, j, l, k). */
int pbi4g_compute_q4k(int32_t grid, float box, const double *deltak, int32_t i, int32_t j, int32_t l,
                      int32_t k, double *q4k);
/* replaces powerI4.f90:510-594 measure_pk; pout: (5, nbins) float64, Fortran order. */
int pbi4g_measure_pk(int32_t grid, float box, float kbin, float kcenter, int32_t nbins, const double *dcl1,
                     const double *dcl2, double *pout);
/* replaces powerI4.f90:596-693 measure_pk_multipoles. */
int pbi4g_measure_pk_multipoles(int32_t grid, float box, float kbin, float kcenter, int32_t nbins,
                                const double *dcl, const double *dcl2, const double *dcl4, double *pout);

/* P(k) multipoles like pbi4g_measure_pk_multipoles, but for callers that may
 * not allocate device memory: applications that hand all device memory out
 * through their own pool, or pipelines that forbid allocation after start-up.
 * It has no counterpart in the reference.  Inputs are device arrays: the kx >= 0
 * halves of dcl, dcl2, dcl4 as complex128 (N, N, N/2+1), C order [z][y][x]
 * (x = ix-1 fastest); d_pout is a device (5, nbins) float64 array, Fortran
 * order.  Work is queued on `stream` (a cudaStream_t, NULL = legacy default);
 * the call returns without synchronising.  No cudaMalloc/cudaFree: its scratch
 * is a fixed 4.3 MiB device array inside the library, held by every device that
 * loads the library until exit, sized for grid <= 512 and nbins <= 512; larger
 * sizes return PBI4G_ERR_RANGE.  Each call outside stream capture looks up the
 * array's device address on the current device (so a device reset is
 * harmless); a call inside a capture reuses the address the previous call on
 * that device found, so make the first call on a device before any capture.
 * All calls share the one array: calls that overlap on the GPU (other streams,
 * other host threads) race and must be serialised by the caller. */
int pbi4g_measure_pk_multipoles_noalloc(int32_t grid, float box, float kbin, float kcenter, int32_t nbins,
                                        const void *d_dcl_half, const void *d_dcl2_half, const void *d_dcl4_half,
                                        double *d_pout, void *stream);

/* ---------------- 1. f2py drop-ins: bispectrumI4 ---------------- */

/* replaces bispectrumI4.f90:763-915 count_triangles; counts: itot float64
 * (= grid^3 x exact integer triangle count). npool is accepted and ignored. */
int pbi4g_count_triangles(int32_t nbins, int32_t grid, float kbin, float kcenter, int32_t iopen,
                          int32_t cross, int32_t npool, int64_t itot, double *counts);
/* replaces bispectrumI4.f90:1-198 measure_bk; bout: (9, itot) float64 Fortran order. */
int pbi4g_measure_bk(int32_t nbins, int32_t grid, float kbin, float kcenter, int32_t iopen, float kf,
                     int32_t npool, int64_t itot, int64_t npart, const float *counts, const double *dcl,
                     double *bout);
/* replaces bispectrumI4.f90:200-516 measure_bk_multipoles; bout: (11, itot). */
int pbi4g_measure_bk_multipoles(int32_t nbins, int32_t grid, float kbin, float kcenter, int32_t iopen,
                                float kf, int32_t npool, int64_t itot, int64_t npart, const float *counts,
                                const double *dcl, const double *dcl2, const double *dcl4, double *bout);
/* replaces bispectrumI4.f90:518-761 measure_bk_cross; bout: (5, itot). */
int pbi4g_measure_bk_cross(int32_t nbins, int32_t grid, float kbin, float kcenter, int32_t iopen, float kf,
                           int32_t npool, int64_t itot, int64_t npart, const float *counts,
                           const double *dcl1, const double *dcl2, double *bout);

/* ---------------- 2. device-resident estimator plan ---------------- */

/* One estimator configuration: the params dict of pbi4.py (IO.derived_params,
 * pbi4.py:86-119) reduced to what the hot path reads.  P and B may use
 * different binnings (the reference shares kbin/kcenter; pass equal values to
 * reproduce it). */
typedef struct pbi4g_config {
    int32_t grid;        /* N */
    float box;           /* L in Mpc/h (real(4), as the reference passes it) */
    int32_t nintp;       /* 1 NGP, 2 CIC, 3 TSC, 4 PCS */
    int32_t interlacing; /* 0/1 */
    int32_t multipoles;  /* 0: P0 / B0 (real space); 1: P0,P2,P4 / B0,B2,B4 */
    double los[3];       /* params['los'] after derived_params: los / (los . los) */
    float kbin_ps, kcenter_ps;
    int32_t nbins_ps;
    int32_t do_bispectrum; /* 0: P only */
    float kbin_bs, kcenter_bs;
    int32_t nbins_bs;
    int32_t iopen;
    int32_t precision;   /* PBI4G_PREC_* of the shell maps / triangle sums */
    int32_t map_budget_mb; /* FP32 forms: MiB the real-space shell maps may hold at
                            * once (0: no bound).  Above it the maps are made and
                            * contracted z-slab by z-slab (same results up to the
                            * order of the FP64 slab additions). */
    int32_t reserved[6]; /* must be zero */
} pbi4g_config;

typedef struct pbi4g_plan pbi4g_plan;

/* Device bytes a plan for cfg needs for boxes of up to npart_max particles
 * (admission control).  Does not allocate. */
int pbi4g_plan_footprint(const pbi4g_config *cfg, int64_t npart_max, int64_t *bytes);
/* Create a plan on the current device (allocates its buffers, cuFFT plans,
 * bin/shell tables; triangle counts are computed on first use and cached). */
int pbi4g_plan_create(const pbi4g_config *cfg, pbi4g_plan **out);
int pbi4g_plan_destroy(pbi4g_plan *plan);
/* Work of the plan is issued on this stream (a cudaStream_t; NULL = legacy default). */
int pbi4g_plan_set_stream(pbi4g_plan *plan, void *stream);

/* Shared assignment scratch.  The FP32 and tensor-core forms count-sort the
 * particles into per-tile records (up to 8 per particle: 3.2 GB at 10^7
 * particles) in buffers each plan owns, and the captured form holds `batch` position
 * slots of its capacity.  Plans that run one after another on one stream (a
 * serving slot) can share one scratch instead: pbi4g_plan_use_scratch points the
 * plan's assignment at it and frees the plan's own buffers (and its position slots
 * when the scratch holds `boxes` >= the plan's batch of at least its capacity), and
 * NULL returns the plan to its own.  The plan must be idle; its captured graphs
 * follow the binding (the kernels read the record addresses from a per-plan device
 * block, rewritten on the plan's stream when the binding changes, and each box's
 * position slot from its per-launch parameters).  A scratch never grows: a box
 * above its grid or particle count fails with PBI4G_ERR_RANGE.  Plans sharing a
 * scratch must not run concurrently.  The FP64 form has no such buffers
 * (use_scratch is a no-op).  destroy fails while plans still use it.  Binding,
 * destroying a bound plan and destroying a scratch keep a count of its plans:
 * call them from one host thread.  Replaces nothing in the reference (its
 * Fortran assignment needs no scratch). */
typedef struct pbi4g_scratch pbi4g_scratch;
int pbi4g_scratch_footprint(int32_t grid_max, int64_t npart_max, int32_t boxes, int64_t *bytes);
int pbi4g_scratch_create(int32_t grid_max, int64_t npart_max, int32_t boxes, pbi4g_scratch **out);
int pbi4g_scratch_destroy(pbi4g_scratch *scratch);
int pbi4g_plan_use_scratch(pbi4g_plan *plan, pbi4g_scratch *scratch);
/* Output sizes: pout is (5, nbins_ps), bout is (brows, itot), Fortran order. */
int pbi4g_plan_shape(const pbi4g_plan *plan, int32_t *nbins_ps, int64_t *itot, int32_t *brows);

/* Grid of the bispectrum shell maps (the smallest FFT-friendly size above
 * 3 kmax, at most `grid`; 0 without a bispectrum) and the number of maps per
 * box (nbins_bs, x3 with multipoles).  Sums on it are scaled by (grid/map_grid)^3. */
int pbi4g_plan_map_grid(const pbi4g_plan *plan, int32_t *map_grid, int32_t *nmaps);
/* Complex FP32 elements of the pruned map transform's two intermediates (the
 * z-transformed shell columns and the (z, y)-transformed kx planes) of the
 * FP32 forms, as sized by the first bispectrum run (0 before it, and for FP64). */
int pbi4g_plan_map_work(const pbi4g_plan *plan, int64_t *zcols, int64_t *yplanes);
/* z-planes per slab of the map grid and slabs per box of the last bispectrum
 * run (one slab of map_grid planes without a map budget; 0, 0 before a run). */
int pbi4g_plan_map_slabs(const pbi4g_plan *plan, int32_t *slab_planes, int32_t *nslabs);
/* Tensor-core triangle sums of the last bispectrum run: units (one 128-pair x
 * 64-map tile of the contraction each) and MMA products per K step (3 for the
 * hi+lo split forms, 1 for BF16); 0, 0 for the CUDA-core forms and before a run.
 * The executed tensor work per box is units * (map grid)^3 * 128 * 64 * 2 *
 * products flops, against 2 (map grid)^3 itot sets useful ones. */
int pbi4g_plan_tensor_units(const pbi4g_plan *plan, int32_t *units, int32_t *products);
/* Exact integer triangle counts of the plan's binning (computed once, cached). */
int pbi4g_plan_triangle_counts(pbi4g_plan *plan, int64_t *counts_host);

/* Density stage (pbi4.py:290-341 + 343-388): positions (3, npart) float64 in
 * [0,1) on the device (pos[c*npart+i]); weight device float64 or NULL (ones).
 * Leaves delta(k) on the kx >= 0 half resident in the plan. */
int pbi4g_plan_density(pbi4g_plan *plan, int64_t npart, const double *d_pos, const double *d_weight);
/* P(k) stage (pbi4.py:405-461): d_pout device (5, nbins_ps) float64: rows avgk,
 * P0 (not shot-noise subtracted, as measure_pk*), P2, P4, Nmodes. */
int pbi4g_plan_powerspectrum(pbi4g_plan *plan, double *d_pout);
/* B stage (pbi4.py:478-553): d_bout device (brows, itot) float64, rows as
 * measure_bk (9) / measure_bk_multipoles (11). */
int pbi4g_plan_bispectrum(pbi4g_plan *plan, double *d_bout);
/* Whole box on device buffers: density + P (+ B when configured). */
int pbi4g_plan_run_device(pbi4g_plan *plan, int64_t npart, const double *d_pos, const double *d_weight,
                          double *d_pout, double *d_bout);
/* Whole box from host buffers (pinned or pageable): copies in, runs, copies
 * pout/bout back, synchronises the plan's stream. */
int pbi4g_plan_run_host(pbi4g_plan *plan, int64_t npart, const double *pos, const double *weight,
                        double *pout, double *bout);
/* Captured form (serving): `batch` box slots of at most npart_cap particles
 * held by the plan.  Runs one direct box to size every buffer and build the
 * lazy tables (synchronous).  Needs an FP32-family precision, grid % 16 == 0,
 * a stream set with pbi4g_plan_set_stream (not the legacy default stream);
 * boxes carry no weights. */
int pbi4g_plan_graph_build(pbi4g_plan *plan, int32_t batch, int64_t npart_cap);
/* nboxes (1..batch) boxes through one CUDA graph launch on the plan's stream:
 * copies pos[b] ((3, npart[b]) float64 host) into the slots, launches the graph
 * captured for nboxes boxes (captured on first use; the particle counts and
 * their normalisation factors are read from device memory, so one graph serves
 * any counts up to npart_cap), copies pout[b] ((5, nbins_ps)) and bout[b]
 * ((brows, itot)) out.  Asynchronous with pinned host buffers, which must stay
 * alive until the plan's stream completes (pbi4g_plan_check). */
int pbi4g_plan_graph_run_host(pbi4g_plan *plan, int32_t nboxes, const int64_t *npart, const double *const *pos,
                              double *const *pout, double *const *bout);
/* Synchronise the plan's stream and report PBI4G_ERR_TIMEOUT if a bounded wait
 * inside a tensor-core launch of this plan gave up (the device launches of
 * pbi4g_plan_run_device are asynchronous; run_host checks by itself). */
int pbi4g_plan_check(pbi4g_plan *plan);
/* Copy the resident delta(k) half spectrum (N, N, N/2+1) complex128, C order
 * [z][y][x], to host memory. */
int pbi4g_plan_get_delta_half(pbi4g_plan *plan, double *host_half);
/* Replace the resident delta(k) half spectrum, (N, N, N/2+1) complex128 C order
 * [z][y][x], e.g. a density read back from disk (pbi4.py:257-288); npart is the
 * particle count the shot-noise terms use. */
int pbi4g_plan_set_delta_half(pbi4g_plan *plan, int64_t npart, const double *host_half);
/* Use these triangle counts (itot float64, grid^3 x count as count_triangles
 * returns, e.g. read from a counts file, pbi4.py:466-470) instead of computing
 * them; they are cast to float32 as the reference does (bispectrumI4.f90:8). */
int pbi4g_plan_set_counts(pbi4g_plan *plan, const double *counts_host);
/* Launches of this library's kernels issued by this plan since creation. */
int64_t pbi4g_plan_kernel_launches(const pbi4g_plan *plan);

/* Stage timing with CUDA events on the plan's stream (off by default).
 * Stages: 0 assign, 1 grid convert, 2 forward FFT, 3 fcomb, 4 P(k) binning,
 * 5 triangle counts, 6 shell maps z (shell spectra; FP32 forms with their z
 * transform), 7 shell maps y (FP32 forms: y transform; FP64: the batched C2R),
 * 8 triangle sums, 9 output rows, 10 shell maps x (FP32 forms: the real maps),
 * 11 the FP32 forms' counting sort of the particles into owner tiles (stage 0
 * is then the tile accumulation alone).  pbi4g_plan_stage_times synchronises the stream, writes the
 * summed milliseconds and the number of timed calls per stage since the last
 * query (arrays of PBI4G_NSTAGES) and resets them. */
#define PBI4G_NSTAGES 12
int pbi4g_plan_enable_timing(pbi4g_plan *plan, int32_t enable);
int pbi4g_plan_stage_times(pbi4g_plan *plan, double *ms, int64_t *calls);

/* Catalogue step of IO.read_catalogues (pbi4.py:121-245) on the device: d_pos
 * (npart, 3) row-major catalogue positions in Mpc/h, float32 (is_double = 0) or
 * float64, optional d_vel (npart, 3) of the same type with the RSD shift along
 * los[3]: rsd_mode 1 pos += vel * los / hz * (1 + z) (Gadget, Rockstar, Quijote),
 * rsd_mode 0 pos += vel * los (Minerva), the shift in float64 and rounded to the
 * catalogue type as numpy does; then the wrap (pos + box) % box and pos / box in
 * the catalogue type, clipped at 1.0, into d_out (3, npart) float64: the
 * positions the assignment reads.  Asynchronous on `stream` (a cudaStream_t). */
int pbi4g_catalog_positions(int64_t npart, const void *d_pos, const void *d_vel, int32_t is_double,
                            const double *los, int32_t rsd_mode, double hz, double z, double box, double *d_out,
                            void *stream);

/* Diagnostics.  Device allocations (cudaMalloc) this library has made for its
 * own buffers since it was loaded (cuFFT's plan work areas are not counted). */
int64_t pbi4g_device_allocs(void);
/* Host-side failure hook for tests of the callers' error paths: with k > 0 the
 * k-th next device allocation of this library returns PBI4G_ERR_NOMEM (no
 * cudaMalloc is issued for it), once; 0 disarms.  No device fault is involved. */
int pbi4g_debug_fail_alloc(int32_t k);

/* Diagnostic limit of the plan's tensor-core triangle sums: after `polls`
 * polls (non-blocking) a main-loop barrier wait gives up, so that the waits run
 * out on healthy work and the launch takes its abort path (every role stops,
 * the copies and tensor-core work in flight are waited for with the normal
 * limit, tensor memory is freed) and the call returns PBI4G_ERR_TIMEOUT.  0
 * restores the normal limit (about 4 million polls).  For tests of the callers'
 * error handling; no device fault is involved. */
int pbi4g_plan_debug_wait_limit(pbi4g_plan *plan, int64_t polls);

/* Host check of the shell maps' FFT plans (no device work): `batch` inverse
 * DFTs of n points, X[k] = sum_j x[j] e^{+2 pi i j k / n}, of interleaved
 * complex FP32 rows in[t][n][2] -> out[t][n][2], computed on the CPU with the
 * same plan tables and butterflies the z / y / x pass kernels run.  n must be
 * 7-smooth (else PBI4G_ERR_UNSUPPORTED). */
int pbi4g_fft_plan_check(int32_t n, int32_t batch, const float *in, float *out);

#ifdef __cplusplus
}
#endif

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif

#endif /* PBI4GPU_H */
