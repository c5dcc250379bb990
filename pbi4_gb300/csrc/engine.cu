// engine.cu -- the plan (device-resident estimator) and the bispectrum engine.
//
// Density   : assign (fixed point) -> real grids -> batched R2C -> fcomb_half
//             (pbi4.py:290-341, powerI4.f90:68-378)
// P(k)      : pk_measure on the half spectrum, multipoles by the per-mode
//             constant-LOS factors (pbi4.py:343-461, powerI4.f90:596-693)
// B(k)      : shell spectra -> one batched C2R -> triangle sums -> output rows
//             (pbi4.py:478-553, bispectrumI4.f90)
#include "engine.cuh"
#include "assign.cuh"
#include "assign_owner.cuh"

#include <stdarg.h>
#include <stdio.h>
#include <string.h>
#include <math.h>
#include <algorithm>
#include <vector>

namespace pbi4g {

static thread_local char g_err[1024] = "";

int set_error(int code, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
    return code;
}

Prof::~Prof() {
    for (auto e : pool) cudaEventDestroy(e);
    for (auto &r : recs) { cudaEventDestroy(r.a); cudaEventDestroy(r.b); }
}

cudaEvent_t Prof::get() {
    if (!pool.empty()) {
        cudaEvent_t e = pool.back();
        pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

void Prof::begin(int stage, cudaStream_t st) {
    if (!on) return;
    cur_a = get();
    cur_stage = stage;
    cudaEventRecord(cur_a, st);
}

void Prof::end(cudaStream_t st) {
    if (!on || cur_stage < 0) return;
    cudaEvent_t b = get();
    cudaEventRecord(b, st);
    recs.push_back({cur_stage, cur_a, b});
    cur_stage = -1;
}

size_t BkEngine::footprint(int N, float kbin, float kcenter, int nb, int nsets, int cross, int precision,
                           size_t budget) {
    const bool fp64 = precision == PBI4G_PREC_FP64;
    const int Nm = shell_map_grid(N, kbin, kcenter, nb);  // the maps' grid, as the plan will choose it
    const size_t HC = half_cells(Nm), FC = full_cells(Nm);
    const int nm = cross ? 2 * nb : nsets * nb;
    const size_t cs = fp64 ? 16 : 8;
    // FP64: half spectra + a cuFFT work area of about one batch of the same size;
    // FP32 forms: the pruned transform's intermediates (at most two half-spectrum
    // sets) + the real maps or operand planes of one slab (upper estimates)
    const size_t maps = (size_t)nm * HC * cs;
    const int tc = tc_mode_of(precision);
    const size_t per_point = tc == 3 ? 8 : (tc == 2 ? 2 : 4);  // bytes per map and point
    const size_t dense = (size_t)nm * FC * per_point + (tc ? (size_t)nb * FC * 4 : 0);
    return 2 * maps + (fp64 ? 0 : (budget ? std::min(dense, budget) : dense)) + (size_t)nb * 8 +
           ((size_t)1 << 26);
}

int BkEngine::slab_planes(int Nm, size_t per_plane, size_t budget) {
    // a slab holds whole 64-point chunks: q z-planes with q Nm^2 a multiple of 64
    const long long plane = (long long)Nm * Nm;
    int q = 1;
    while ((q * plane) % 64) q *= 2;
    if (!budget) return Nm;
    long long zs = (long long)(budget / per_plane);
    zs = std::max<long long>(q, zs / q * q);
    return (int)std::min<long long>(Nm, zs);
}

int BkEngine::check(cudaStream_t st) {
    if (tmp_nsets >= 0) PBI4G_CHECK(tm_check_error(tmp, st));
    return PBI4G_OK;
}

template <class R>
int BkEngine::run(const typename Cx<R>::T *const src[3], const int fac[3], const double los[3], float kf,
                  int64_t npart, const float *counts_f32, double *d_bout, cudaStream_t st, int64_t *launches,
                  Prof *prof, const BoxPar *bp) {
    using C = typename Cx<R>::T;
    Prof dummy;
    Prof &pf = prof ? *prof : dummy;
    const int N = sh.Nm, NH = N / 2 + 1, nb = sh.nb;  // maps live on the map grid Nm
    const size_t HC = half_cells(N);
    const int nm = nmaps();
    const bool fp64 = sizeof(R) == 8;
    if (tp_nsets != nsets || tp_cross != cross || tp_fp64 != (int)fp64) {
        PBI4G_CHECK(tp.build(sh, cross ? 1 : nsets, cross, fp64 ? 128 : 256));
        tp_nsets = nsets;
        tp_cross = cross;
        tp_fp64 = fp64;
    }
    PBI4G_CHECK(powsum.ensure(sizeof(double) * 3 * nb));
    PBI4G_CHECK(S.ensure(sizeof(double) * std::max(1, tp.nslots)));
    const bool tc = tc_mode != 0 && !fp64 && !cross;
    const int form = tc_mode == 1 ? 1 : (tc_mode == 2 ? 2 : 0);  // trisum_tm forms
    if (tc && !tm_supported(sh))
        return set_error(PBI4G_ERR_UNSUPPORTED, "tensor-core triangle sums: map grid %d with %d shells", N, nb);
    // set 0 always (shell powers); the other sets only when the FP16 scale bound
    // needs their own power (explicit delta_2 / delta_4 grids)
    int pow_mask = 1;
    if (tc) {
        if (tmp_nsets != nsets) {
            PBI4G_CHECK(tmp.build(sh, nsets));
            tmp_nsets = nsets;
        }
        PBI4G_CHECK(S.ensure(sizeof(double) * std::max(1, tmp.nslots)));
        if (form == 1)
            for (int s = 1; s < nsets; s++)
                if (fac[s] == 0) pow_mask |= 1 << s;
    }
    const size_t FCm = (size_t)N * N * N;
    // FP64: in-place C2R (padded rows); plain FP32: dense FP32 maps; tensor-core
    // forms: the operand planes of the form (MapPlanes), of one z-slab of the grid
    PBI4G_CUDA(cudaMemsetAsync(powsum.p, 0, sizeof(double) * 3 * nb, st));
    if (fp64) {
        PBI4G_CHECK(maps.ensure(sizeof(C) * HC * nm));
        pf.begin(6, st);
        PBI4G_CHECK(build_map_spectra<R>(sh, nm, src, fac, los, maps.as<C>(), powsum.as<double>(), pow_mask, st,
                                         launches));
        pf.end(st);
        if (!inv || inv_batch != nm || inv_N != N) {
            if (inv) cufftDestroy(inv);
            inv = 0;
            int n[3] = {N, N, N}, inembed[3] = {N, N, NH}, onembed[3] = {N, N, 2 * NH};
            PBI4G_CUFFT(cufftPlanMany(&inv, 3, n, inembed, 1, (int)HC, onembed, 1, (int)(2 * HC), CUFFT_Z2D, nm));
            inv_batch = nm;
            inv_N = N;
        }
        PBI4G_CUFFT(cufftSetStream(inv, st));
        pf.begin(7, st);
        PBI4G_CUFFT(cufftExecZ2D(inv, maps.as<cufftDoubleComplex>(), maps.as<cufftDoubleReal>()));
        pf.end(st);
    } else {
        // pruned inverse transform: z pass (with the shell spectra), y pass, x pass
        if (mt_nmaps != nm || mt.Nm != N) {
            PBI4G_CHECK(mt.build(sh, nm));
            mt_nmaps = nm;
        }
        // per z-plane of a slab: the y pass's output U and the real maps (dense
        // FP32 or the operand planes of the form)
        const size_t per_point = tc ? MapPlanes::bytes(form, 1, nm, nb) : sizeof(float) * nm;
        const size_t per_plane = per_point * (size_t)N * N + sizeof(float2) * (size_t)mt.kxtot * N;
        const int zs = slab_planes(N, per_plane, map_budget);
        slab_z = zs;
        nslabs = (N + zs - 1) / zs;
        PBI4G_CHECK(dense.ensure(per_point * (size_t)zs * N * N));
        PBI4G_CHECK(maps.ensure(mt.work_bytes(zs)));
        const float2 *const *fsrc = reinterpret_cast<const float2 *const *>(src);
        pf.begin(6, st);
        PBI4G_CHECK(map_zpass(sh, mt, fsrc, fac, los, maps.as<float2>(), powsum.as<double>(), pow_mask, st,
                              launches));
        pf.end(st);
        if (tc && form == 1) {
            // largest |L_l(mu)| over mu^2 in [0, |los|^2]: bounds the delta_2 / delta_4 maps by the delta map
            double lfac[3] = {1.0, 1.0, 1.0};
            const double l2max = los ? los[0] * los[0] + los[1] * los[1] + los[2] * los[2] : 1.0;
            for (int s = 1; s < nsets; s++) {
                if (fac[s] == 0) continue;
                double mx = 0;
                for (int k = 0; k <= 2000; k++) {
                    const double m2 = l2max * k / 2000.0;
                    const double L = fac[s] == 2 ? -0.5 + 1.5 * m2 : 0.375 + m2 * (-3.75 + 4.375 * m2);
                    mx = std::max(mx, fabs(L));
                }
                lfac[s] = mx * 1.01;
            }
            PBI4G_CHECK(tm_map_exponents(sh, tmp, nm, powsum.as<double>(), pow_mask, lfac, st, launches));
        }
        // y pass, x pass and triangle sums slab by slab (one slab: the whole grid)
        for (int z0 = 0; z0 < N; z0 += zs) {
            const int z1 = std::min(N, z0 + zs);
            const long long spts = (long long)(z1 - z0) * N * N;
            pf.begin(7, st);
            PBI4G_CHECK(map_ypass(mt, maps.as<float2>(), st, launches, z0, z1));
            pf.end(st);
            pf.begin(10, st);
            if (tc) {
                planes.carve(form, spts, nm, nb, dense.p, form == 1 ? tmp.mexp.as<int>() : nullptr);
                PBI4G_CHECK(map_xpass(mt, maps.as<float2>(), nullptr, &planes, st, launches, z0, z1));
            } else {
                PBI4G_CHECK(map_xpass(mt, maps.as<float2>(), dense.as<float>(), nullptr, st, launches, z0, z1));
            }
            pf.end(st);
            pf.begin(8, st);
            if (tc)
                PBI4G_CHECK(triangle_sums_tm(sh, tmp, planes, partial, S.as<double>(), z0 > 0, st, launches));
            else
                PBI4G_CHECK(triangle_sums<float>(sh, tp, dense.as<float>(), (size_t)spts, N, N, spts, partial,
                                                 S.as<double>(), z0 > 0, st, launches));
            pf.end(st);
        }
    }
    if (fp64) {
        pf.begin(8, st);
        PBI4G_CHECK(triangle_sums<R>(sh, tp, maps.as<R>(), 2 * HC, N, 2 * NH, (long long)FCm, partial,
                                     S.as<double>(), false, st, launches));
        pf.end(st);
    }
    pf.begin(9, st);
    PBI4G_CHECK(bk_finalize(sh, cross ? 1 : nsets, cross, S.as<double>(), powsum.as<double>(), kf, npart, counts_f32,
                            d_bout, st, launches, bp));
    pf.end(st);
    return PBI4G_OK;
}

template int BkEngine::run<float>(const float2 *const[3], const int[3], const double[3], float, int64_t, const float *,
                                  double *, cudaStream_t, int64_t *, Prof *, const BoxPar *);
template int BkEngine::run<double>(const double2 *const[3], const int[3], const double[3], float, int64_t,
                                   const float *, double *, cudaStream_t, int64_t *, Prof *, const BoxPar *);

}  // namespace pbi4g

using namespace pbi4g;

// ================================================================ plan ===
// Assignment buffers shared by the plans that run on one stream (a serving slot).
struct pbi4g_scratch {
    OwnerWork wk;
    DevBuf pos;         // graph position slots: [boxes][3][cap] float64
    int boxes = 0;
    int64_t cap = 0;
    int bound = 0;      // plans using it
};

struct pbi4g_plan {
    pbi4g_config cfg;
    cudaStream_t st = 0;
    int64_t launches = 0;
    bool fp64 = false;
    int N = 0, G = 1;
    AssignWork aw;
    OwnerWork ow;               // the plan's own assignment buffers
    OwnerWork *ow_cur = &ow;    // the buffers in use: ow or a shared scratch (pbi4g_plan_use_scratch)
    DevBuf optr;                // the owner kernels' pointer block (owner_ptrs_host of *ow_cur)
    unsigned char optr_host[kOwnerPtrBytes] = {};
    bool optr_valid = false;
    pbi4g_scratch *scratch = nullptr;  // the shared scratch in use, if any
    DevBuf real_grids, spec, delta;
    DevBuf pos_stage, w_stage, pout_d, bout_d;
    cufftHandle fwd = 0;
    PkBins pk;
    WinCache win;
    BkEngine bk;
    bool have_delta = false;
    int64_t npart = 0;
    Prof prof;
    // captured form (pbi4g_plan_graph_*): `batch` box slots of at most `cap` particles
    struct Graphs {
        int batch = 0;
        int64_t cap = 0;
        DevBuf pos, pout, bout, par;           // [batch][3][cap], [batch][pout], [batch][bout], [batch] BoxPar
        std::vector<cudaGraphExec_t> exec;     // exec[b - 1] runs boxes 0..b-1
        std::vector<int64_t> exec_launches;    // kernels of this library in exec[b - 1]
        std::vector<BoxPar> hpar;
        size_t pout_n = 0, bout_n = 0;         // doubles per box
        ~Graphs() {
            for (auto e : exec)
                if (e) cudaGraphExecDestroy(e);
        }
    } g;
    ~pbi4g_plan() {
        if (fwd) cufftDestroy(fwd);
    }
};

static int check_config(const pbi4g_config *c) {
    if (!c) return set_error(PBI4G_ERR_INVALID, "null config");
    if (c->grid < 4 || (c->grid & 1) || c->grid > 2048)
        return set_error(PBI4G_ERR_INVALID, "grid must be even and in [4, 2048] (got %d)", c->grid);
    if (c->nintp < 1 || c->nintp > 4) return set_error(PBI4G_ERR_INVALID, "interpolation must be 1..4");
    if (!(c->box > 0)) return set_error(PBI4G_ERR_INVALID, "box must be > 0");
    if (c->nbins_ps < 1 || !(c->kbin_ps > 0)) return set_error(PBI4G_ERR_INVALID, "bad P binning");
    if (c->do_bispectrum && (c->nbins_bs < 1 || !(c->kbin_bs > 0)))
        return set_error(PBI4G_ERR_INVALID, "bad B binning");
    if (c->precision < PBI4G_PREC_FP32 || c->precision > PBI4G_PREC_TF32SPLIT)
        return set_error(PBI4G_ERR_INVALID, "unknown precision %d", c->precision);
    if (c->map_budget_mb < 0) return set_error(PBI4G_ERR_INVALID, "map budget must be >= 0");
    for (int k = 0; k < 6; k++)
        if (c->reserved[k]) return set_error(PBI4G_ERR_INVALID, "reserved config fields must be zero");
    return PBI4G_OK;
}

extern "C" {

const char *pbi4g_last_error(void) { return g_err; }

int pbi4g_fft_plan_check(int32_t n, int32_t batch, const float *in, float *out) {
    if (n < 2 || batch < 0 || (batch > 0 && (!in || !out)))
        return set_error(PBI4G_ERR_INVALID, "fft plan check: n=%d batch=%d", n, batch);
    return fft_plan_host_check(n, batch, in, out);
}
int pbi4g_version(void) { return 100; }

int64_t pbi4g_device_allocs(void) { return (int64_t)pbi4g::g_dev_allocs.load(); }

int pbi4g_debug_fail_alloc(int32_t k) {
    if (k < 0) return pbi4g::set_error(PBI4G_ERR_INVALID, "debug_fail_alloc: k must be >= 0");
    pbi4g::g_fail_alloc_in.store(k);
    return PBI4G_OK;
}

int pbi4g_plan_footprint(const pbi4g_config *cfg, int64_t npart_max, int64_t *bytes) {
    PBI4G_CHECK(check_config(cfg));
    if (!bytes || npart_max < 0) return set_error(PBI4G_ERR_INVALID, "bad footprint arguments");
    const int N = cfg->grid, G = cfg->interlacing ? 2 : 1;
    const bool fp64 = cfg->precision == PBI4G_PREC_FP64;
    const size_t rs = fp64 ? 8 : 4, cs = 2 * rs, HC = half_cells(N), FC = full_cells(N);
    size_t b = (fp64 ? AssignWork::footprint(N, npart_max, cfg->interlacing) : OwnerWork::footprint(N, npart_max)) +
               G * FC * rs + G * HC * cs + HC * cs;
    b += 2 * G * HC * cs;  // cuFFT work area (upper estimate)
    b += (size_t)npart_max * 32 + 5 * (size_t)cfg->nbins_ps * 8 * 1300;
    if (cfg->do_bispectrum) {
        b += BkEngine::footprint(N, cfg->kbin_bs, cfg->kcenter_bs, cfg->nbins_bs, cfg->multipoles ? 3 : 1, 0,
                                 cfg->precision, (size_t)cfg->map_budget_mb << 20);
        b += (size_t)FC * 8 * (size_t)0;  // counts use a temporary FP64 map set, freed after the first box
    }
    *bytes = (int64_t)b;
    return PBI4G_OK;
}

int pbi4g_plan_create(const pbi4g_config *cfg, pbi4g_plan **out) {
    PBI4G_CHECK(check_config(cfg));
    if (!out) return set_error(PBI4G_ERR_INVALID, "null out");
    pbi4g_plan *p = new pbi4g_plan();
    p->cfg = *cfg;
    p->N = cfg->grid;
    p->G = cfg->interlacing ? 2 : 1;
    p->fp64 = cfg->precision == PBI4G_PREC_FP64;
    int rc = PBI4G_OK;
    do {
        const int N = p->N;
        const size_t rs = p->fp64 ? 8 : 4, HC = half_cells(N), FC = full_cells(N);
        if ((rc = p->real_grids.ensure(p->G * FC * rs))) break;
        if ((rc = p->spec.ensure(p->G * HC * 2 * rs))) break;
        if ((rc = p->delta.ensure(HC * 2 * rs))) break;
        int n[3] = {N, N, N};
        cufftResult r = cufftPlanMany(&p->fwd, 3, n, nullptr, 1, (int)FC, nullptr, 1, (int)HC,
                                      p->fp64 ? CUFFT_D2Z : CUFFT_R2C, p->G);
        if (r != CUFFT_SUCCESS) { rc = set_error(PBI4G_ERR_CUFFT, "R2C plan failed (%d)", (int)r); p->fwd = 0; break; }
        if ((rc = p->pk.build(N, cfg->box, cfg->kbin_ps, cfg->kcenter_ps, cfg->nbins_ps, p->st, &p->launches))) break;
        if (cfg->do_bispectrum) {
            if ((rc = p->bk.sh.build(N, cfg->kbin_bs, cfg->kcenter_bs, cfg->nbins_bs, cfg->iopen, 0, p->st))) break;
            p->bk.nsets = cfg->multipoles ? 3 : 1;
            p->bk.cross = 0;
            p->bk.tc_mode = tc_mode_of(cfg->precision);
            p->bk.map_budget = (size_t)cfg->map_budget_mb << 20;
        }
        cudaError_t e = cudaStreamSynchronize(p->st);
        if (e != cudaSuccess) { rc = set_error(PBI4G_ERR_CUDA, "plan create: %s", cudaGetErrorString(e)); break; }
    } while (0);
    if (rc) {
        delete p;
        return rc;
    }
    *out = p;
    return PBI4G_OK;
}

int pbi4g_plan_destroy(pbi4g_plan *plan) {
    if (plan && plan->scratch) plan->scratch->bound--;
    delete plan;
    return PBI4G_OK;
}

int pbi4g_scratch_footprint(int32_t grid_max, int64_t npart_max, int32_t boxes, int64_t *bytes) {
    if (!bytes || npart_max < 1 || boxes < 0 || boxes > 64 || !owner_supported(grid_max))
        return set_error(PBI4G_ERR_INVALID,
                         "scratch footprint: grid %d (a multiple of 16 in [32, 2048]), %lld particles, %d boxes",
                         grid_max, (long long)npart_max, boxes);
    *bytes = (int64_t)(OwnerWork::footprint(grid_max, npart_max) + sizeof(double) * 3 * (size_t)npart_max * boxes);
    return PBI4G_OK;
}

int pbi4g_scratch_create(int32_t grid_max, int64_t npart_max, int32_t boxes, pbi4g_scratch **out) {
    int64_t b = 0;
    PBI4G_CHECK(pbi4g_scratch_footprint(grid_max, npart_max, boxes, &b));
    if (!out) return set_error(PBI4G_ERR_INVALID, "null scratch handle");
    auto *sc = new (std::nothrow) pbi4g_scratch();
    if (!sc) return set_error(PBI4G_ERR_NOMEM, "scratch object");
    int rc = sc->wk.ensure(grid_max, npart_max);
    if (rc == PBI4G_OK && boxes > 0) rc = sc->pos.ensure(sizeof(double) * 3 * (size_t)npart_max * boxes);
    if (rc != PBI4G_OK) {
        delete sc;
        return rc;
    }
    sc->wk.fixed = true;
    sc->boxes = boxes;
    sc->cap = npart_max;
    *out = sc;
    return PBI4G_OK;
}

int pbi4g_scratch_destroy(pbi4g_scratch *scratch) {
    if (!scratch) return PBI4G_OK;
    if (scratch->bound > 0)
        return set_error(PBI4G_ERR_INVALID, "scratch still in use by %d plan(s)", scratch->bound);
    delete scratch;
    return PBI4G_OK;
}

static int owner_bind(pbi4g_plan *p, int64_t npart);

// Whether the plan's scratch holds its graph position slots (batch boxes of cap particles).
static bool scratch_holds_slots(const pbi4g_plan *p) {
    return p->scratch && p->g.batch > 0 && p->scratch->boxes >= p->g.batch && p->scratch->cap >= p->g.cap;
}

// The graph position slots in use: the scratch's, or the plan's own (allocated on demand).
static int pos_slots(pbi4g_plan *p, double **slots) {
    if (scratch_holds_slots(p)) {
        *slots = p->scratch->pos.as<double>();
        return PBI4G_OK;
    }
    PBI4G_CHECK(p->g.pos.ensure(sizeof(double) * 3 * (size_t)p->g.cap * p->g.batch));
    *slots = p->g.pos.as<double>();
    return PBI4G_OK;
}

int pbi4g_plan_use_scratch(pbi4g_plan *plan, pbi4g_scratch *scratch) {
    if (!plan) return set_error(PBI4G_ERR_INVALID, "null plan");
    if (plan->fp64 || !owner_supported(plan->N)) return PBI4G_OK;  // no owner-computes assignment in this form
    if (scratch == plan->scratch && plan->optr_valid) return PBI4G_OK;
    OwnerWork *w = scratch ? &scratch->wk : &plan->ow;
    const int64_t cap = std::max<int64_t>(1, plan->g.cap);
    if (scratch && !w->fits(plan->N, cap))
        return set_error(PBI4G_ERR_RANGE, "scratch too small for grid %d and %lld particles", plan->N,
                         (long long)cap);
    OwnerWork *prev = plan->ow_cur;
    plan->ow_cur = w;
    const int rc = owner_bind(plan, cap);
    if (rc != PBI4G_OK) {  // keep the previous binding; the next run writes its block again
        plan->ow_cur = prev;
        plan->optr_valid = false;
        return rc;
    }
    if (plan->scratch) plan->scratch->bound--;
    plan->scratch = scratch;
    if (scratch) {
        scratch->bound++;
        plan->ow.release();  // the plan's own buffers (idle plan: the caller's contract)
        if (scratch_holds_slots(plan)) plan->g.pos.release();
    }
    return PBI4G_OK;
}

int pbi4g_plan_set_stream(pbi4g_plan *plan, void *stream) {
    if (!plan) return set_error(PBI4G_ERR_INVALID, "null plan");
    plan->st = (cudaStream_t)stream;
    return PBI4G_OK;
}

int pbi4g_plan_shape(const pbi4g_plan *plan, int32_t *nbins_ps, int64_t *itot, int32_t *brows) {
    if (!plan) return set_error(PBI4G_ERR_INVALID, "null plan");
    if (nbins_ps) *nbins_ps = plan->cfg.nbins_ps;
    if (itot) *itot = plan->cfg.do_bispectrum ? plan->bk.sh.itot : 0;
    if (brows) *brows = plan->cfg.do_bispectrum ? (plan->cfg.multipoles ? 11 : 9) : 0;
    return PBI4G_OK;
}

int pbi4g_plan_map_grid(const pbi4g_plan *plan, int32_t *map_grid, int32_t *nmaps) {
    if (!plan) return set_error(PBI4G_ERR_INVALID, "null plan");
    const bool bk = plan->cfg.do_bispectrum != 0;
    if (map_grid) *map_grid = bk ? plan->bk.sh.Nm : 0;
    if (nmaps) *nmaps = bk ? (plan->cfg.multipoles ? 3 : 1) * plan->bk.sh.nb : 0;
    return PBI4G_OK;
}

int pbi4g_plan_map_work(const pbi4g_plan *plan, int64_t *zcols, int64_t *yplanes) {
    if (!plan) return set_error(PBI4G_ERR_INVALID, "null plan");
    const bool built = plan->cfg.do_bispectrum && plan->bk.mt_nmaps >= 0;
    if (zcols) *zcols = built ? plan->bk.mt.tsize : 0;
    if (yplanes) *yplanes = built ? plan->bk.mt.usize : 0;
    return PBI4G_OK;
}

int pbi4g_plan_map_slabs(const pbi4g_plan *plan, int32_t *slab_planes, int32_t *nslabs) {
    if (!plan) return set_error(PBI4G_ERR_INVALID, "null plan");
    const bool bk = plan->cfg.do_bispectrum != 0;
    if (slab_planes) *slab_planes = bk ? plan->bk.slab_z : 0;
    if (nslabs) *nslabs = bk ? plan->bk.nslabs : 0;
    return PBI4G_OK;
}

int pbi4g_plan_tensor_units(const pbi4g_plan *plan, int32_t *units, int32_t *products) {
    if (!plan) return set_error(PBI4G_ERR_INVALID, "null plan");
    const BkEngine &bk = plan->bk;
    const bool tc = plan->cfg.do_bispectrum && bk.tc_mode != 0 && bk.tmp_nsets >= 0;
    if (units) *units = tc ? bk.tmp.nunits : 0;
    if (products) *products = tc ? (bk.tc_mode == 2 ? 1 : 3) : 0;
    return PBI4G_OK;
}

int64_t pbi4g_plan_kernel_launches(const pbi4g_plan *plan) { return plan ? plan->launches : -1; }

int pbi4g_plan_triangle_counts(pbi4g_plan *plan, int64_t *counts_host) {
    if (!plan || !plan->cfg.do_bispectrum) return set_error(PBI4G_ERR_INVALID, "plan has no bispectrum");
    PBI4G_CHECK(triangle_counts(plan->bk.sh, plan->st, &plan->launches));
    if (counts_host) memcpy(counts_host, plan->bk.sh.counts.data(), sizeof(int64_t) * plan->bk.sh.itot);
    return PBI4G_OK;
}

// Size the plan's assignment buffers in use (*ow_cur) for npart particles and
// point its pointer block at them (a stream-ordered copy, only when they changed).
static int owner_bind(pbi4g_plan *p, int64_t npart) {
    PBI4G_CHECK(p->ow_cur->ensure(p->N, npart));
    unsigned char blk[kOwnerPtrBytes];
    owner_ptrs_host(*p->ow_cur, blk);
    if (p->optr_valid && memcmp(blk, p->optr_host, kOwnerPtrBytes) == 0) return PBI4G_OK;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    PBI4G_CUDA(cudaStreamIsCapturing(p->st, &cs));
    if (cs != cudaStreamCaptureStatusNone)
        return set_error(PBI4G_ERR_INVALID, "assignment buffers changed during a capture");
    PBI4G_CHECK(p->optr.ensure(kOwnerPtrBytes));
    memcpy(p->optr_host, blk, kOwnerPtrBytes);
    // the copy reads optr_host before the call returns (pageable source)
    PBI4G_CUDA(cudaMemcpyAsync(p->optr.p, p->optr_host, kOwnerPtrBytes, cudaMemcpyHostToDevice, p->st));
    p->optr_valid = true;
    return PBI4G_OK;
}

// One box's density.  bp == nullptr: npart particles at d_pos (rows of npart).
// bp != nullptr (captured form): npart is the slot capacity (rows of npart), the
// particle count and the normalisation come from bp on the device.
static int density_impl(pbi4g_plan *p, int64_t npart, const double *d_pos, const double *d_weight, const BoxPar *bp) {
    const int N = p->N;
    int bits;
    if (!p->fp64 && owner_supported(N)) {
        // FP32 grids straight from the owner-computes tiles (fixed-point sums in shared memory);
        // a captured box uses the binding made before the capture
        if (!bp) PBI4G_CHECK(owner_bind(p, npart));
        if (!p->optr_valid) return set_error(PBI4G_ERR_INVALID, "assignment buffers not bound before capture");
        PBI4G_CHECK(assign_owner(*p->ow_cur, p->optr.p, N, p->cfg.nintp, p->G == 2, npart, d_pos, d_weight,
                                 p->real_grids.as<float>(), p->st, &p->launches, npart, bp, &p->prof, 0, 11));
    } else {
        if (bp) return set_error(PBI4G_ERR_UNSUPPORTED, "captured form needs the owner-computes assignment");
        p->prof.begin(0, p->st);
        PBI4G_CHECK(assign_fixed(p->aw, N, p->cfg.nintp, p->G == 2, p->fp64, npart, d_pos, d_weight, &bits, p->st,
                                 &p->launches));
        p->prof.end(p->st);
        p->prof.begin(1, p->st);
        PBI4G_CHECK(fixed_to_real(p->aw, N, p->G == 2, bits, p->fp64, p->real_grids.p, p->st, &p->launches));
        p->prof.end(p->st);
    }
    PBI4G_CUFFT(cufftSetStream(p->fwd, p->st));
    p->prof.begin(2, p->st);
    if (p->fp64)
        PBI4G_CUFFT(cufftExecD2Z(p->fwd, p->real_grids.as<cufftDoubleReal>(), p->spec.as<cufftDoubleComplex>()));
    else
        PBI4G_CUFFT(cufftExecR2C(p->fwd, p->real_grids.as<cufftReal>(), p->spec.as<cufftComplex>()));
    p->prof.end(p->st);
    p->prof.begin(3, p->st);
    if (p->fp64)
        PBI4G_CHECK(fcomb_half<double>(N, p->cfg.nintp, p->G == 2, p->cfg.box, (double)npart, p->spec.as<double2>(),
                                       p->delta.as<double2>(), p->win, p->st, &p->launches, bp));
    else
        PBI4G_CHECK(fcomb_half<float>(N, p->cfg.nintp, p->G == 2, p->cfg.box, (double)npart, p->spec.as<float2>(),
                                      p->delta.as<float2>(), p->win, p->st, &p->launches, bp));
    p->prof.end(p->st);
    p->have_delta = true;
    p->npart = npart;
    return PBI4G_OK;
}

int pbi4g_plan_density(pbi4g_plan *p, int64_t npart, const double *d_pos, const double *d_weight) {
    if (!p) return set_error(PBI4G_ERR_INVALID, "null plan");
    if (npart < 1) return set_error(PBI4G_ERR_INVALID, "npart must be >= 1");
    return density_impl(p, npart, d_pos, d_weight, nullptr);
}

int pbi4g_plan_powerspectrum(pbi4g_plan *p, double *d_pout) {
    if (!p || !d_pout) return set_error(PBI4G_ERR_INVALID, "null plan/output");
    if (!p->have_delta) return set_error(PBI4G_ERR_INVALID, "powerspectrum before density");
    const int mode = p->cfg.multipoles ? 1 : 0;
    p->prof.begin(4, p->st);
    int rc;
    if (p->fp64)
        rc = pk_measure<double>(p->pk, mode, p->cfg.los, p->delta.as<double2>(), p->delta.as<double2>(), nullptr,
                                d_pout, p->st, &p->launches);
    else
        rc = pk_measure<float>(p->pk, mode, p->cfg.los, p->delta.as<float2>(), p->delta.as<float2>(), nullptr, d_pout,
                               p->st, &p->launches);
    p->prof.end(p->st);
    return rc;
}

static int bispectrum_impl(pbi4g_plan *p, double *d_bout, const BoxPar *bp);

int pbi4g_plan_bispectrum(pbi4g_plan *p, double *d_bout) { return bispectrum_impl(p, d_bout, nullptr); }

static int bispectrum_impl(pbi4g_plan *p, double *d_bout, const BoxPar *bp) {
    if (!p || !d_bout) return set_error(PBI4G_ERR_INVALID, "null plan/output");
    if (!p->cfg.do_bispectrum) return set_error(PBI4G_ERR_INVALID, "plan has no bispectrum");
    if (!p->have_delta) return set_error(PBI4G_ERR_INVALID, "bispectrum before density");
    if (p->bk.sh.counts.empty()) {
        p->prof.begin(5, p->st);
        PBI4G_CHECK(triangle_counts(p->bk.sh, p->st, &p->launches));
        p->prof.end(p->st);
    }
    // the reference passes kf = 2 pi / box as real(4) (pbi4.py:100, bispectrumI4.f90:8)
    const float kf = (float)(2.0 * 3.14159265358979323846 / (double)p->cfg.box);
    const int fac[3] = {0, 2, 4};
    if (p->fp64) {
        const double2 *src[3] = {p->delta.as<double2>(), p->delta.as<double2>(), p->delta.as<double2>()};
        return p->bk.run<double>(src, fac, p->cfg.los, kf, p->npart, p->bk.sh.counts_f32.as<float>(), d_bout, p->st,
                                 &p->launches, &p->prof, bp);
    }
    const float2 *src[3] = {p->delta.as<float2>(), p->delta.as<float2>(), p->delta.as<float2>()};
    return p->bk.run<float>(src, fac, p->cfg.los, kf, p->npart, p->bk.sh.counts_f32.as<float>(), d_bout, p->st,
                            &p->launches, &p->prof, bp);
}

// ------------------------------------------------------- captured form ---
static float plan_kf(const pbi4g_plan *p) { return (float)(2.0 * 3.14159265358979323846 / (double)p->cfg.box); }

int pbi4g_plan_graph_build(pbi4g_plan *p, int32_t batch, int64_t npart_cap) {
    if (!p || batch < 1 || batch > 64 || npart_cap < 1) return set_error(PBI4G_ERR_INVALID, "bad graph arguments");
    if (p->fp64 || !owner_supported(p->N))
        return set_error(PBI4G_ERR_UNSUPPORTED, "captured form needs an FP32-family plan with grid %% 16 == 0");
    if (p->st == 0) return set_error(PBI4G_ERR_INVALID, "captured form needs a non-default stream");
    auto &g = p->g;
    for (auto e : g.exec)
        if (e) cudaGraphExecDestroy(e);
    g.exec.assign(batch, nullptr);
    g.exec_launches.assign(batch, 0);
    g.batch = batch;
    g.cap = npart_cap;
    g.pout_n = (size_t)5 * p->cfg.nbins_ps;
    g.bout_n = p->cfg.do_bispectrum ? (size_t)(p->cfg.multipoles ? 11 : 9) * p->bk.sh.itot : 0;
    PBI4G_CHECK(g.pout.ensure(sizeof(double) * g.pout_n * batch));
    PBI4G_CHECK(g.bout.ensure(sizeof(double) * std::max<size_t>(1, g.bout_n) * batch));
    PBI4G_CHECK(g.par.ensure(sizeof(BoxPar) * batch));
    g.hpar.assign(batch, BoxPar{1, fcomb_cf(p->G == 2, p->cfg.box, 1.0), bk_pow_sn(plan_kf(p), 1), nullptr});
    if (!p->fp64 && owner_supported(p->N)) PBI4G_CHECK(owner_bind(p, npart_cap));
    double *slots = nullptr;  // the scratch's position slots, or the plan's own
    PBI4G_CHECK(pos_slots(p, &slots));
    // positions at 0 (valid, in [0, 1)); one direct box sizes every buffer and
    // builds the lazy tables (windows, shells, triangle counts, cuFFT plans)
    PBI4G_CUDA(cudaMemsetAsync(slots, 0, sizeof(double) * 3 * (size_t)npart_cap, p->st));
    PBI4G_CHECK(pbi4g_plan_run_device(p, 1, slots, nullptr, g.pout.as<double>(),
                                      g.bout_n ? g.bout.as<double>() : nullptr));
    PBI4G_CUDA(cudaStreamSynchronize(p->st));
    return p->cfg.do_bispectrum ? p->bk.check(p->st) : PBI4G_OK;
}

static int graph_capture(pbi4g_plan *p, int nboxes) {
    auto &g = p->g;
    double *slots = nullptr;  // (the captured assignment reads each box's slot from its BoxPar)
    PBI4G_CHECK(pos_slots(p, &slots));
    const bool prof_on = p->prof.on;
    p->prof.on = false;  // no timing events inside a graph
    cudaGraph_t graph = nullptr;
    const int64_t l0 = p->launches;
    PBI4G_CUDA(cudaStreamBeginCapture(p->st, cudaStreamCaptureModeRelaxed));
    int rc = PBI4G_OK;
    for (int b = 0; b < nboxes && rc == PBI4G_OK; b++) {
        const BoxPar *bp = g.par.as<BoxPar>() + b;
        const double *pos = slots + (size_t)b * 3 * g.cap;
        double *po = g.pout.as<double>() + (size_t)b * g.pout_n;
        double *bo = g.bout.as<double>() + (size_t)b * g.bout_n;
        rc = density_impl(p, g.cap, pos, nullptr, bp);
        if (rc == PBI4G_OK) rc = pbi4g_plan_powerspectrum(p, po);
        if (rc == PBI4G_OK && p->cfg.do_bispectrum) rc = bispectrum_impl(p, bo, bp);
    }
    const cudaError_t e = cudaStreamEndCapture(p->st, &graph);
    p->prof.on = prof_on;
    const int64_t captured = p->launches - l0;
    p->launches = l0;
    if (rc != PBI4G_OK) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
    }
    if (e != cudaSuccess) return set_error(PBI4G_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
    cudaGraphExec_t exec = nullptr;
    const cudaError_t ei = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ei != cudaSuccess) return set_error(PBI4G_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(ei));
    g.exec[nboxes - 1] = exec;
    g.exec_launches[nboxes - 1] = captured;
    return PBI4G_OK;
}

int pbi4g_plan_graph_run_host(pbi4g_plan *p, int32_t nboxes, const int64_t *npart, const double *const *pos,
                              double *const *pout, double *const *bout) {
    if (!p || !npart || !pos || !pout) return set_error(PBI4G_ERR_INVALID, "null argument");
    auto &g = p->g;
    if (g.batch == 0) return set_error(PBI4G_ERR_INVALID, "pbi4g_plan_graph_build first");
    if (nboxes < 1 || nboxes > g.batch) return set_error(PBI4G_ERR_INVALID, "nboxes %d outside 1..%d", nboxes, g.batch);
    if (g.bout_n && !bout) return set_error(PBI4G_ERR_INVALID, "null bout");
    const float kf = plan_kf(p);
    for (int b = 0; b < nboxes; b++) {
        if (npart[b] < 1 || npart[b] > g.cap)
            return set_error(PBI4G_ERR_RANGE, "box %d: npart %lld outside 1..%lld", b, (long long)npart[b],
                             (long long)g.cap);
        g.hpar[b] = BoxPar{(long long)npart[b], fcomb_cf(p->G == 2, p->cfg.box, (double)npart[b]),
                           bk_pow_sn(kf, npart[b]), nullptr};
    }
    // the assignment's pointer block holds the buffers in use (rebound after a failed change)
    if (!p->fp64 && owner_supported(p->N)) PBI4G_CHECK(owner_bind(p, g.cap));
    if (!g.exec[nboxes - 1]) PBI4G_CHECK(graph_capture(p, nboxes));
    double *slots = nullptr;  // the scratch's position slots, or the plan's own
    PBI4G_CHECK(pos_slots(p, &slots));
    for (int b = 0; b < nboxes; b++) {
        g.hpar[b].pos = slots + (size_t)b * 3 * g.cap;
        PBI4G_CUDA(cudaMemcpy2DAsync(slots + (size_t)b * 3 * g.cap, sizeof(double) * g.cap, pos[b],
                                     sizeof(double) * npart[b], sizeof(double) * npart[b], 3, cudaMemcpyHostToDevice,
                                     p->st));
    }
    PBI4G_CUDA(cudaMemcpyAsync(g.par.p, g.hpar.data(), sizeof(BoxPar) * nboxes, cudaMemcpyHostToDevice, p->st));
    PBI4G_CUDA(cudaGraphLaunch(g.exec[nboxes - 1], p->st));
    p->launches += g.exec_launches[nboxes - 1];
    for (int b = 0; b < nboxes; b++) {
        PBI4G_CUDA(cudaMemcpyAsync(pout[b], g.pout.as<double>() + (size_t)b * g.pout_n, sizeof(double) * g.pout_n,
                                   cudaMemcpyDeviceToHost, p->st));
        if (g.bout_n)
            PBI4G_CUDA(cudaMemcpyAsync(bout[b], g.bout.as<double>() + (size_t)b * g.bout_n, sizeof(double) * g.bout_n,
                                       cudaMemcpyDeviceToHost, p->st));
    }
    p->npart = npart[nboxes - 1];
    return PBI4G_OK;
}

int pbi4g_plan_run_device(pbi4g_plan *p, int64_t npart, const double *d_pos, const double *d_weight, double *d_pout,
                          double *d_bout) {
    PBI4G_CHECK(pbi4g_plan_density(p, npart, d_pos, d_weight));
    PBI4G_CHECK(pbi4g_plan_powerspectrum(p, d_pout));
    if (p->cfg.do_bispectrum) PBI4G_CHECK(pbi4g_plan_bispectrum(p, d_bout));
    return PBI4G_OK;
}

int pbi4g_plan_run_host(pbi4g_plan *p, int64_t npart, const double *pos, const double *weight, double *pout,
                        double *bout) {
    if (!p || !pos || !pout) return set_error(PBI4G_ERR_INVALID, "null argument");
    if (p->cfg.do_bispectrum && !bout) return set_error(PBI4G_ERR_INVALID, "null bout");
    PBI4G_CHECK(p->pos_stage.ensure(sizeof(double) * 3 * (size_t)npart));
    PBI4G_CUDA(cudaMemcpyAsync(p->pos_stage.p, pos, sizeof(double) * 3 * (size_t)npart, cudaMemcpyHostToDevice, p->st));
    const double *dw = nullptr;
    if (weight) {
        PBI4G_CHECK(p->w_stage.ensure(sizeof(double) * (size_t)npart));
        PBI4G_CUDA(cudaMemcpyAsync(p->w_stage.p, weight, sizeof(double) * (size_t)npart, cudaMemcpyHostToDevice, p->st));
        dw = p->w_stage.as<double>();
    }
    const size_t pb = sizeof(double) * 5 * p->cfg.nbins_ps;
    const size_t bb = p->cfg.do_bispectrum ? sizeof(double) * (p->cfg.multipoles ? 11 : 9) * p->bk.sh.itot : 0;
    PBI4G_CHECK(p->pout_d.ensure(pb));
    if (bb) PBI4G_CHECK(p->bout_d.ensure(bb));
    PBI4G_CHECK(pbi4g_plan_run_device(p, npart, p->pos_stage.as<double>(), dw, p->pout_d.as<double>(),
                                      bb ? p->bout_d.as<double>() : nullptr));
    PBI4G_CUDA(cudaMemcpyAsync(pout, p->pout_d.p, pb, cudaMemcpyDeviceToHost, p->st));
    if (bb) PBI4G_CUDA(cudaMemcpyAsync(bout, p->bout_d.p, bb, cudaMemcpyDeviceToHost, p->st));
    PBI4G_CUDA(cudaStreamSynchronize(p->st));
    return p->cfg.do_bispectrum ? p->bk.check(p->st) : PBI4G_OK;
}

int pbi4g_plan_check(pbi4g_plan *p) {
    if (!p) return set_error(PBI4G_ERR_INVALID, "null plan");
    PBI4G_CUDA(cudaStreamSynchronize(p->st));
    return p->cfg.do_bispectrum ? p->bk.check(p->st) : PBI4G_OK;
}

int pbi4g_plan_debug_wait_limit(pbi4g_plan *p, int64_t polls) {
    if (!p || polls < 0) return set_error(PBI4G_ERR_INVALID, "debug_wait_limit: null plan or negative limit");
    p->bk.tmp.wait_limit = polls > 0xFFFFFFFFLL ? 0u : (uint32_t)polls;
    return PBI4G_OK;
}

int pbi4g_plan_enable_timing(pbi4g_plan *p, int32_t enable) {
    if (!p) return set_error(PBI4G_ERR_INVALID, "null plan");
    p->prof.on = enable != 0;
    return PBI4G_OK;
}

int pbi4g_plan_stage_times(pbi4g_plan *p, double *ms, int64_t *calls) {
    if (!p || !ms) return set_error(PBI4G_ERR_INVALID, "null argument");
    PBI4G_CUDA(cudaStreamSynchronize(p->st));
    for (int s = 0; s < PBI4G_NSTAGES; s++) {
        ms[s] = 0;
        if (calls) calls[s] = 0;
    }
    for (auto &r : p->prof.recs) {
        float t = 0;
        PBI4G_CUDA(cudaEventElapsedTime(&t, r.a, r.b));
        ms[r.stage] += t;
        if (calls) calls[r.stage] += 1;
        p->prof.pool.push_back(r.a);
        p->prof.pool.push_back(r.b);
    }
    p->prof.recs.clear();
    return PBI4G_OK;
}

int pbi4g_plan_set_delta_half(pbi4g_plan *p, int64_t npart, const double *host_half) {
    if (!p || !host_half || npart < 1) return set_error(PBI4G_ERR_INVALID, "bad arguments");
    const size_t HC = half_cells(p->N);
    if (p->fp64) {
        PBI4G_CUDA(cudaMemcpyAsync(p->delta.p, host_half, HC * 16, cudaMemcpyHostToDevice, p->st));
    } else {
        std::vector<float2> tmp(HC);
        for (size_t i = 0; i < HC; i++) tmp[i] = make_float2((float)host_half[2 * i], (float)host_half[2 * i + 1]);
        PBI4G_CUDA(cudaMemcpyAsync(p->delta.p, tmp.data(), HC * 8, cudaMemcpyHostToDevice, p->st));
        PBI4G_CUDA(cudaStreamSynchronize(p->st));
    }
    p->have_delta = true;
    p->npart = npart;
    return PBI4G_OK;
}

int pbi4g_plan_set_counts(pbi4g_plan *p, const double *counts_host) {
    if (!p || !counts_host) return set_error(PBI4G_ERR_INVALID, "bad arguments");
    if (!p->cfg.do_bispectrum) return set_error(PBI4G_ERR_INVALID, "plan has no bispectrum");
    Shells &sh = p->bk.sh;
    const double gridD = (double)p->N * p->N * p->N;
    sh.counts.assign(sh.itot, 0);
    std::vector<float> c32(sh.itot);
    for (int64_t m = 0; m < sh.itot; m++) {
        c32[m] = (float)counts_host[m];
        sh.counts[m] = llround(counts_host[m] / gridD);
    }
    PBI4G_CHECK(sh.counts_f32.ensure(sizeof(float) * std::max<int64_t>(1, sh.itot)));
    PBI4G_CUDA(cudaMemcpy(sh.counts_f32.p, c32.data(), sizeof(float) * sh.itot, cudaMemcpyHostToDevice));
    return PBI4G_OK;
}

int pbi4g_plan_get_delta_half(pbi4g_plan *p, double *host_half) {
    if (!p || !host_half) return set_error(PBI4G_ERR_INVALID, "null argument");
    if (!p->have_delta) return set_error(PBI4G_ERR_INVALID, "no density yet");
    const size_t HC = half_cells(p->N);
    if (p->fp64) {
        PBI4G_CUDA(cudaMemcpyAsync(host_half, p->delta.p, HC * 16, cudaMemcpyDeviceToHost, p->st));
        PBI4G_CUDA(cudaStreamSynchronize(p->st));
        return PBI4G_OK;
    }
    std::vector<float2> tmp(HC);
    PBI4G_CUDA(cudaMemcpyAsync(tmp.data(), p->delta.p, HC * 8, cudaMemcpyDeviceToHost, p->st));
    PBI4G_CUDA(cudaStreamSynchronize(p->st));
    for (size_t i = 0; i < HC; i++) {
        host_half[2 * i] = tmp[i].x;
        host_half[2 * i + 1] = tmp[i].y;
    }
    return PBI4G_OK;
}

}  // extern "C"
