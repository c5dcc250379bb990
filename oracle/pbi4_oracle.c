/*
 * pbi4_oracle.c -- CPU restatement (FP64, serial) of the PBI4 estimator routines.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle: tests/, the smoke
 * check in __graft_entry__.py and the cpu_baseline leg of bench.py load it as the
 * checker.  The product path (pbi4_gb300/) never links, imports or calls it.
 *
 * Each function restates one Fortran-90 routine of the reference
 * (pbi4/F90_modules/powerI4.f90 and pbi4/F90_modules/bispectrumI4.f90) with the
 * same arithmetic kinds:
 *   - `real, parameter :: twopi = 6.28319` is a float32 constant;
 *   - box, kbin, kcenter, kf and counts are real(4) (float) arguments;
 *   - Fortran nint() rounds half away from zero (C lround), int() truncates;
 *   - arrays keep Fortran semantics: a(ix,iy,iz) with 1-based indices and the
 *     first index fastest in memory.
 * Complex arrays are interleaved (re, im) doubles, like numpy complex128.
 * The FFTs the reference takes from FFTW / scipy are done by the Python side of
 * the oracle (oracle/pbi4_oracle.py) with scipy.fft in FP64.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <float.h>

#define TWOPI_F 6.28319f

/* Fortran a(ix,iy,iz), 1-based, first index fastest. */
#define F3(ix, iy, iz, n) ((size_t)((ix) - 1) + (size_t)(n) * ((size_t)((iy) - 1) + (size_t)(n) * (size_t)((iz) - 1)))

static inline long f_nint(double x) { return lround(x); }     /* round half away from zero */
static inline long f_int(double x) { return (long)x; }        /* truncation toward zero   */
static inline long f_mod(long a, long p) { return a % p; }    /* sign of a, like Fortran mod */

static double powi_d(double x, int n) {
    double r = 1.0;
    for (int k = 0; k < n; k++) r *= x;
    return r;
}

/* powerI4.f90:68-140  assign_single_grid.  pos is numpy (3, npart) C-order:
 * pos(c,i) -> pos[(c-1)*npart + (i-1)].  dtl is zero-filled by the caller
 * (f2py zero-fills intent(out) arrays). */
void or_assign_single_grid(int grid, int nintp, int64_t npart, const double *pos,
                           const double *weight, double *dtl) {
    const int nintph = (nintp >= 3) ? 3 : 1;
    const long Nv = grid;
    double w[3][4];
    long iv[3][4];
    memset(w, 0, sizeof w);
    for (int64_t i = 0; i < npart; i++) {
        double vr[3];
        long ivr[3];
        for (int c = 0; c < 3; c++) vr[c] = (double)Nv * pos[(size_t)c * npart + i] + 1.0;
        if (nintp == 4) {
            for (int c = 0; c < 3; c++) ivr[c] = f_int(vr[c]);
            for (int j = 1; j <= 4; j++)
                for (int c = 0; c < 3; c++) iv[c][j - 1] = f_mod(ivr[c] - nintph + j + Nv, Nv) + 1;
            for (int c = 0; c < 3; c++) {
                double h = vr[c] - (double)f_int(vr[c]);
                double h2 = h * h;
                w[c][0] = (1.0 - h) * (1.0 - h) * (1.0 - h) / 6.0;
                w[c][1] = 4.0 / 6.0 + (0.5 * h - 1.0) * h2;
                w[c][3] = h2 * h / 6.0;
                w[c][2] = 1.0 - w[c][0] - w[c][1] - w[c][3];
            }
        }
        if (nintp == 3) {
            for (int c = 0; c < 3; c++) ivr[c] = f_nint(vr[c]);
            for (int j = 1; j <= 3; j++)
                for (int c = 0; c < 3; c++) iv[c][j - 1] = f_mod(ivr[c] - nintph + j + Nv, Nv) + 1;
            for (int c = 0; c < 3; c++) {
                double h = vr[c] - (double)f_nint(vr[c]);
                double h2 = h * h;
                w[c][0] = 0.5 * (0.5 - h) * (0.5 - h);
                w[c][1] = 0.75 - h2;
                w[c][2] = 1.0 - w[c][0] - w[c][1];
            }
        }
        if (nintp == 2) { /* CIC: index from int(), offset from nint() (powerI4.f90:115,120) */
            for (int c = 0; c < 3; c++) ivr[c] = f_int(vr[c]);
            for (int j = 1; j <= 2; j++)
                for (int c = 0; c < 3; c++) iv[c][j - 1] = f_mod(ivr[c] - nintph + j + Nv, Nv) + 1;
            for (int c = 0; c < 3; c++) {
                double h = vr[c] - (double)f_nint(vr[c]);
                w[c][0] = 1.0 - h;
                w[c][1] = h;
            }
        }
        if (nintp == 1) {
            for (int c = 0; c < 3; c++)
                for (int j = 0; j < 4; j++) w[c][j] = 1.0;
            for (int c = 0; c < 3; c++) {
                ivr[c] = f_nint(vr[c]);
                iv[c][0] = f_mod(ivr[c] - 1 + Nv, Nv) + 1;
            }
        }
        for (int ix = 0; ix < nintp; ix++)
            for (int iy = 0; iy < nintp; iy++)
                for (int iz = 0; iz < nintp; iz++)
                    dtl[F3(iv[0][ix], iv[1][iy], iv[2][iz], grid)] += w[0][ix] * w[1][iy] * w[2][iz] * weight[i];
    }
}

/* powerI4.f90:142-249  assign_double_grid: Re = grid at vr, Im = grid at vr-0.5. */
void or_assign_double_grid(int grid, int nintp, int64_t npart, const double *pos,
                           const double *weight, double *dcl) {
    const int nintph = (nintp >= 3) ? 3 : 1;
    const long Nv = grid;
    double w1[3][4], w2[3][4];
    long iv[3][4], jv[3][4];
    memset(w1, 0, sizeof w1);
    memset(w2, 0, sizeof w2);
    for (int64_t i = 0; i < npart; i++) {
        double vr[3], vt[3];
        long ivr[3], ivt[3];
        for (int c = 0; c < 3; c++) {
            vr[c] = (double)Nv * pos[(size_t)c * npart + i] + 1.0;
            vt[c] = vr[c] - 0.5;
        }
        if (nintp == 4) {
            for (int c = 0; c < 3; c++) { ivr[c] = f_int(vr[c]); ivt[c] = f_int(vt[c]); }
            for (int j = 1; j <= 4; j++)
                for (int c = 0; c < 3; c++) {
                    iv[c][j - 1] = f_mod(ivr[c] - nintph + j + Nv, Nv) + 1;
                    jv[c][j - 1] = f_mod(ivt[c] - nintph + j + Nv, Nv) + 1;
                }
            for (int c = 0; c < 3; c++) {
                double h1 = vr[c] - (double)f_int(vr[c]);
                double h2 = vt[c] - (double)f_int(vt[c]);
                double h1sq = h1 * h1, h2sq = h2 * h2;
                w1[c][0] = (1.0 - h1) * (1.0 - h1) * (1.0 - h1) / 6.0;
                w1[c][1] = 4.0 / 6.0 + (0.5 * h1 - 1.0) * h1sq;
                w1[c][3] = h1sq * h1 / 6.0;
                w1[c][2] = 1.0 - w1[c][0] - w1[c][1] - w1[c][3];
                w2[c][0] = (1.0 - h2) * (1.0 - h2) * (1.0 - h2) / 6.0;
                w2[c][1] = 4.0 / 6.0 + (0.5 * h2 - 1.0) * h2sq;
                w2[c][3] = h2sq * h2 / 6.0;
                w2[c][2] = 1.0 - w2[c][0] - w2[c][1] - w2[c][3];
            }
        }
        if (nintp == 3) {
            for (int c = 0; c < 3; c++) { ivr[c] = f_nint(vr[c]); ivt[c] = f_nint(vt[c]); }
            for (int j = 1; j <= 3; j++)
                for (int c = 0; c < 3; c++) {
                    iv[c][j - 1] = f_mod(ivr[c] - nintph + j + Nv, Nv) + 1;
                    jv[c][j - 1] = f_mod(ivt[c] - nintph + j + Nv, Nv) + 1;
                }
            for (int c = 0; c < 3; c++) {
                double h1 = vr[c] - (double)f_nint(vr[c]);
                double h2 = vt[c] - (double)f_nint(vt[c]);
                double h1sq = h1 * h1, h2sq = h2 * h2;
                w1[c][0] = 0.5 * (0.5 - h1) * (0.5 - h1);
                w1[c][1] = 0.75 - h1sq;
                w1[c][2] = 1.0 - w1[c][0] - w1[c][1];
                w2[c][0] = 0.5 * (0.5 - h2) * (0.5 - h2);
                w2[c][1] = 0.75 - h2sq;
                w2[c][2] = 1.0 - w2[c][0] - w2[c][1];
            }
        }
        if (nintp == 2) { /* double-grid CIC uses int() for both (powerI4.f90:209-223) */
            for (int c = 0; c < 3; c++) { ivr[c] = f_int(vr[c]); ivt[c] = f_int(vt[c]); }
            for (int j = 1; j <= 2; j++)
                for (int c = 0; c < 3; c++) {
                    iv[c][j - 1] = f_mod(ivr[c] - nintph + j + Nv, Nv) + 1;
                    jv[c][j - 1] = f_mod(ivt[c] - nintph + j + Nv, Nv) + 1;
                }
            for (int c = 0; c < 3; c++) {
                double h1 = vr[c] - (double)f_int(vr[c]);
                double h2 = vt[c] - (double)f_int(vt[c]);
                w1[c][0] = 1.0 - h1;
                w1[c][1] = h1;
                w2[c][0] = 1.0 - h2;
                w2[c][1] = h2;
            }
        }
        if (nintp == 1) {
            for (int c = 0; c < 3; c++)
                for (int j = 0; j < 4; j++) { w1[c][j] = 1.0; w2[c][j] = 1.0; }
            for (int c = 0; c < 3; c++) {
                ivr[c] = f_nint(vr[c]);
                ivt[c] = f_nint(vt[c]);
                iv[c][0] = f_mod(ivr[c] - 1 + Nv, Nv) + 1;
                jv[c][0] = f_mod(ivt[c] - 1 + Nv, Nv) + 1;
            }
        }
        for (int ix = 0; ix < nintp; ix++)
            for (int iy = 0; iy < nintp; iy++)
                for (int iz = 0; iz < nintp; iz++) {
                    size_t a = F3(iv[0][ix], iv[1][iy], iv[2][iz], grid);
                    dcl[2 * a] += w1[0][ix] * w1[1][iy] * w1[2][iz] * weight[i];
                    size_t b = F3(jv[0][ix], jv[1][iy], jv[2][iz], grid);
                    dcl[2 * b + 1] += w2[0][ix] * w2[1][iy] * w2[2][iz] * weight[i];
                }
    }
}

/* ---- small complex helpers (Fortran complex(8) arithmetic) ---- */
typedef struct { double re, im; } cplx;
static inline cplx cmk(double r, double i) { cplx c = {r, i}; return c; }
static inline cplx cmul(cplx a, cplx b) { return cmk(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re); }
static inline cplx cadd(cplx a, cplx b) { return cmk(a.re + b.re, a.im + b.im); }
static inline cplx csub(cplx a, cplx b) { return cmk(a.re - b.re, a.im - b.im); }
static inline cplx cconj(cplx a) { return cmk(a.re, -a.im); }
static inline cplx cscale(cplx a, double s) { return cmk(a.re * s, a.im * s); }
static inline cplx cget(const double *a, size_t k) { return cmk(a[2 * k], a[2 * k + 1]); }
static inline void cset(double *a, size_t k, cplx v) { a[2 * k] = v.re; a[2 * k + 1] = v.im; }

/* sinc^nintp window table, powerI4.f90:278-292 */
static void window_table(int grid, int nintp, double *tW) {
    const double tpiN = (double)TWOPI_F / (double)grid;
    tW[0] = 1.0;
    for (int i = 2; i <= grid / 2 + 1; i++) {
        double rk = tpiN * (double)(i - 1);
        tW[i - 1] = powi_d(sin(rk / 2.0) / (rk / 2.0), nintp);
    }
}

/* powerI4.f90:251-378  fcomb, in place on dcl (the caller passes a copy of fdcl). */
void or_fcomb(int grid, int nintp, int interlacing, float box, double *dcl) {
    const int N = grid, Nnyq = grid / 2 + 1;
    const double tpiN = (double)TWOPI_F / (double)grid;
    float kf3f = TWOPI_F * TWOPI_F;
    kf3f = kf3f * TWOPI_F;
    kf3f = kf3f / box;
    kf3f = kf3f / box;
    kf3f = kf3f / box;
    const double kF3 = (double)kf3f;
    double *tW = (double *)malloc(sizeof(double) * (size_t)Nnyq);
    window_table(grid, nintp, tW);
    if (interlacing) {
        const double cf = 1.0 / (4.0 * kF3);
        const double piN = -tpiN / 2.0;
        const cplx rec = cmk(cos(piN), sin(piN));
        const cplx c1 = cmk(1.0, 0.0), ci = cmk(0.0, 1.0);
        cplx zrec = c1;
        for (int iz = 1; iz <= Nnyq; iz++) {
            int icz = (int)f_mod(N - iz + 1, N) + 1;
            double Wkz = tW[iz - 1];
            cplx yrec = c1;
            for (int iy = 1; iy <= Nnyq; iy++) {
                int icy = (int)f_mod(N - iy + 1, N) + 1;
                double Wky = tW[iy - 1];
                cplx xrec = c1;
                for (int ix = 1; ix <= Nnyq; ix++) {
                    int icx = (int)f_mod(N - ix + 1, N) + 1;
                    double Wkx = tW[ix - 1];
                    double cfac = cf / (Wkx * Wky * Wkz);
                    cplx cma = cmul(cmul(cmul(ci, xrec), yrec), zrec);
                    cplx cmb = cmul(cmul(cmul(ci, xrec), yrec), cconj(zrec));
                    cplx cmc = cmul(cmul(cmul(ci, xrec), cconj(yrec)), zrec);
                    cplx cmd = cmul(cmul(ci, xrec), cconj(cmul(yrec, zrec)));
                    cplx c000 = cadd(cmul(cget(dcl, F3(ix, iy, iz, N)), csub(c1, cma)),
                                     cmul(cconj(cget(dcl, F3(icx, icy, icz, N))), cadd(c1, cma)));
                    cplx c001 = cadd(cmul(cget(dcl, F3(ix, iy, icz, N)), csub(c1, cmb)),
                                     cmul(cconj(cget(dcl, F3(icx, icy, iz, N))), cadd(c1, cmb)));
                    cplx c010 = cadd(cmul(cget(dcl, F3(ix, icy, iz, N)), csub(c1, cmc)),
                                     cmul(cconj(cget(dcl, F3(icx, iy, icz, N))), cadd(c1, cmc)));
                    cplx c011 = cadd(cmul(cget(dcl, F3(ix, icy, icz, N)), csub(c1, cmd)),
                                     cmul(cconj(cget(dcl, F3(icx, iy, iz, N))), cadd(c1, cmd)));
                    cset(dcl, F3(ix, iy, iz, N), cscale(c000, cfac));
                    cset(dcl, F3(ix, iy, icz, N), cscale(c001, cfac));
                    cset(dcl, F3(ix, icy, iz, N), cscale(c010, cfac));
                    cset(dcl, F3(ix, icy, icz, N), cscale(c011, cfac));
                    cset(dcl, F3(icx, iy, iz, N), cconj(cget(dcl, F3(ix, icy, icz, N))));
                    cset(dcl, F3(icx, iy, icz, N), cconj(cget(dcl, F3(ix, icy, iz, N))));
                    cset(dcl, F3(icx, icy, iz, N), cconj(cget(dcl, F3(ix, iy, icz, N))));
                    cset(dcl, F3(icx, icy, icz, N), cconj(cget(dcl, F3(ix, iy, iz, N))));
                    xrec = cmul(xrec, rec);
                }
                yrec = cmul(yrec, rec);
            }
            zrec = cmul(zrec, rec);
        }
    } else {
        const double cf = 1.0 / kF3;
        for (int iz = 1; iz <= Nnyq; iz++) {
            int icz = (int)f_mod(N - iz + 1, N) + 1;
            double Wkz = tW[iz - 1];
            for (int iy = 1; iy <= Nnyq; iy++) {
                int icy = (int)f_mod(N - iy + 1, N) + 1;
                double Wky = tW[iy - 1];
                for (int ix = 1; ix <= Nnyq; ix++) {
                    double Wkx = tW[ix - 1];
                    double cfac = cf / (Wkx * Wky * Wkz);
                    size_t a;
                    a = F3(ix, iy, iz, N); cset(dcl, a, cscale(cget(dcl, a), cfac));
                    if (iz != icz) { a = F3(ix, iy, icz, N); cset(dcl, a, cscale(cget(dcl, a), cfac)); }
                    if (iy != icy) { a = F3(ix, icy, iz, N); cset(dcl, a, cscale(cget(dcl, a), cfac)); }
                    if (iz != icz && iy != icy) { a = F3(ix, icy, icz, N); cset(dcl, a, cscale(cget(dcl, a), cfac)); }
                }
            }
        }
    }
    free(tW);
}

/* powerI4.f90:380-407  reduce_array: din is an L^3 grid, dout a grid^3 grid
 * (zero-filled by the caller). */
void or_reduce_array(int L, const double *din, int grid, double *dout) {
    for (int iz = 1; iz <= grid / 2 + 1; iz++) {
        int icz = (int)f_mod(L - iz + 1, L) + 1;
        int jcz = (int)f_mod(grid - iz + 1, grid) + 1;
        for (int iy = 1; iy <= grid / 2 + 1; iy++) {
            int icy = (int)f_mod(L - iy + 1, L) + 1;
            int jcy = (int)f_mod(grid - iy + 1, grid) + 1;
            for (int ix = 1; ix <= grid / 2 + 1; ix++) {
                cset(dout, F3(ix, iy, iz, grid), cget(din, F3(ix, iy, iz, L)));
                cset(dout, F3(ix, jcy, iz, grid), cget(din, F3(ix, icy, iz, L)));
                cset(dout, F3(ix, iy, jcz, grid), cget(din, F3(ix, iy, icz, L)));
                cset(dout, F3(ix, jcy, jcz, grid), cget(din, F3(ix, icy, icz, L)));
            }
        }
    }
}

/* signed frequency of 1-based index i on an n grid, Nyquist -> +n/2 (powerI4.f90:435) */
static inline int kfreq(int i, int n) { return (int)f_mod(i + n / 2 - 2, n) - n / 2 + 1; }

/* powerI4.f90:409-458 compute_q2k (Q2k = deltak, then the kx>=0 half rescaled). */
void or_compute_q2k(int grid, float box, const double *deltak, int i, int j, double *Q2k) {
    const int N = grid;
    const double kF = (double)(TWOPI_F / box);
    memcpy(Q2k, deltak, sizeof(double) * 2 * (size_t)N * N * N);
    for (int iz = 1; iz <= N; iz++) {
        double v3 = kF * (double)kfreq(iz, N);
        for (int iy = 1; iy <= N; iy++) {
            double v2 = kF * (double)kfreq(iy, N);
            for (int ix = 1; ix <= N / 2 + 1; ix++) {
                double v1 = kF * (double)kfreq(ix, N);
                double v[3] = {v1, v2, v3};
                size_t a = F3(ix, iy, iz, N);
                if (ix + iy + iz > 3) {
                    double rk2 = v1 * v1 + v2 * v2 + v3 * v3;
                    cplx q = cget(Q2k, a);
                    q = cscale(q, v[i - 1]);
                    q = cscale(q, v[j - 1]);
                    q = cmk(q.re / rk2, q.im / rk2);
                    cset(Q2k, a, q);
                } else {
                    cset(Q2k, a, cmk(0.0, 0.0));
                }
            }
        }
    }
}

/* powerI4.f90:460-508 compute_q4k */
void or_compute_q4k(int grid, float box, const double *deltak, int i, int j, int l, int k, double *Q4k) {
    const int N = grid;
    const double kF = (double)(TWOPI_F / box);
    memcpy(Q4k, deltak, sizeof(double) * 2 * (size_t)N * N * N);
    for (int iz = 1; iz <= N; iz++) {
        double v3 = kF * (double)kfreq(iz, N);
        for (int iy = 1; iy <= N; iy++) {
            double v2 = kF * (double)kfreq(iy, N);
            for (int ix = 1; ix <= N / 2 + 1; ix++) {
                double v1 = kF * (double)kfreq(ix, N);
                double v[3] = {v1, v2, v3};
                size_t a = F3(ix, iy, iz, N);
                if (ix + iy + iz > 3) {
                    double d = v1 * v1 + v2 * v2 + v3 * v3;
                    double rk2 = d * d;
                    cplx q = cget(Q4k, a);
                    q = cscale(q, v[i - 1]);
                    q = cscale(q, v[j - 1]);
                    q = cscale(q, v[l - 1]);
                    q = cscale(q, v[k - 1]);
                    q = cmk(q.re / rk2, q.im / rk2);
                    cset(Q4k, a, q);
                } else {
                    cset(Q4k, a, cmk(0.0, 0.0));
                }
            }
        }
    }
}

/* P-side bin index, powerI4.f90:565-566 (and 654-655). */
static inline long pk_bin(double rk, double dk, float kcenter, float kbin) {
    return f_nint(rk / dk - (double)(kcenter / kbin) - DBL_MIN) + 1;
}

/* powerI4.f90:510-594 measure_pk.  pout is Fortran pout(5,nbins): pout[(r-1) + 5*(b-1)]. */
void or_measure_pk(int grid, float box, float kbin, float kcenter, int nbins,
                   const double *dcl1, const double *dcl2, double *pout) {
    const int N = grid;
    const double kF = (double)(TWOPI_F / box);
    const double kF3 = kF * kF * kF;
    const double dk = (double)kbin * kF;
    double *avgk = calloc((size_t)nbins, sizeof(double));
    double *avgP = calloc((size_t)nbins, sizeof(double));
    double *co = calloc((size_t)nbins, sizeof(double));
    for (int iz = 1; iz <= N; iz++) {
        int ikz = kfreq(iz, N);
        double rkz = kF * (double)(float)ikz;
        for (int iy = 1; iy <= N; iy++) {
            int iky = kfreq(iy, N);
            double rky = kF * (double)(float)iky;
            for (int ix = 1; ix <= N / 2 + 1; ix++) {
                int ikx = kfreq(ix, N);
                double rkx = kF * (double)(float)ikx;
                if (ix != 1 || (ix == 1 && iky > 0) || (ix == 1 && iky == 0 && ikz > 0)) {
                    double rk = sqrt(rkx * rkx + rky * rky + rkz * rkz);
                    long imk = pk_bin(rk, dk, kcenter, kbin);
                    if (imk <= nbins && imk > 0) {
                        co[imk - 1] += 1.0;
                        avgk[imk - 1] += rk;
                        cplx ct1 = cget(dcl1, F3(ix, iy, iz, N));
                        cplx ct2 = cget(dcl2, F3(ix, iy, iz, N));
                        cplx pk = cmul(cconj(ct1), ct2);
                        avgP[imk - 1] += pk.re;
                    }
                }
            }
        }
    }
    for (int b = 0; b < nbins; b++) {
        for (int r = 0; r < 5; r++) pout[r + 5 * b] = 0.0;
        pout[0 + 5 * b] = avgk[b] / co[b];
        pout[1 + 5 * b] = avgP[b] * kF3 / co[b];
        pout[2 + 5 * b] = co[b];
    }
    free(avgk); free(avgP); free(co);
}

/* powerI4.f90:596-693 measure_pk_multipoles */
void or_measure_pk_multipoles(int grid, float box, float kbin, float kcenter, int nbins,
                              const double *dcl, const double *dcl2, const double *dcl4, double *pout) {
    const int N = grid;
    const double kF = (double)(TWOPI_F / box);
    const double kF3 = kF * kF * kF;
    const double dk = (double)kbin * kF;
    double *avgk = calloc((size_t)nbins, sizeof(double));
    double *avgP = calloc((size_t)nbins, sizeof(double));
    double *avgP2 = calloc((size_t)nbins, sizeof(double));
    double *avgP4 = calloc((size_t)nbins, sizeof(double));
    double *co = calloc((size_t)nbins, sizeof(double));
    for (int iz = 1; iz <= N; iz++) {
        int ikz = kfreq(iz, N);
        double rkz = kF * (double)(float)ikz;
        for (int iy = 1; iy <= N; iy++) {
            int iky = kfreq(iy, N);
            double rky = kF * (double)(float)iky;
            for (int ix = 1; ix <= N / 2 + 1; ix++) {
                int ikx = kfreq(ix, N);
                double rkx = kF * (double)(float)ikx;
                if (ix != 1 || (ix == 1 && iky > 0) || (ix == 1 && iky == 0 && ikz > 0)) {
                    double rk = sqrt(rkx * rkx + rky * rky + rkz * rkz);
                    long imk = pk_bin(rk, dk, kcenter, kbin);
                    if (imk <= nbins && imk > 0) {
                        size_t a = F3(ix, iy, iz, N);
                        co[imk - 1] += 1.0;
                        avgk[imk - 1] += rk;
                        cplx ct = cget(dcl, a), ct2 = cget(dcl2, a), ct4 = cget(dcl4, a);
                        double ab = hypot(ct.re, ct.im);
                        avgP[imk - 1] += ab * ab;
                        avgP2[imk - 1] += cmul(cconj(ct), ct2).re;
                        avgP4[imk - 1] += cmul(cconj(ct), ct4).re;
                    }
                }
            }
        }
    }
    for (int b = 0; b < nbins; b++) {
        pout[0 + 5 * b] = avgk[b] / co[b];
        pout[1 + 5 * b] = avgP[b] * kF3 / co[b];
        pout[2 + 5 * b] = 5. * avgP2[b] * kF3 / co[b];
        pout[3 + 5 * b] = 9. * avgP4[b] * kF3 / co[b];
        pout[4 + 5 * b] = co[b];
    }
    free(avgk); free(avgP); free(avgP2); free(avgP4); free(co);
}

/* Shell index of every full-grid mode, bispectrumI4.f90:66-77 (measure_bk*) and
 * :809-820 (count_triangles).  Output in the same traversal order as the
 * reference (i slowest, l fastest): shell[(l) + N*(j + N*i)] for i,j,l in [0,N).
 * tiny_double selects tiny(real(8)) (count_triangles uses tiny(rmax)) over
 * tiny(real(4)) (measure_bk* use tiny(kf)); both are far below one ulp of the
 * operand, kept for fidelity. */
void or_shell_index(int grid, float kbin, float kcenter, int tiny_double, int32_t *shell) {
    const double tiny = tiny_double ? DBL_MIN : (double)FLT_MIN;
    const double kck = (double)(kcenter / kbin);
    size_t m = 0;
    for (int i = 0; i < grid; i++)
        for (int j = 0; j < grid; j++)
            for (int l = 0; l < grid; l++) {
                double di = (double)(i < grid - i ? i : grid - i);
                double dj = (double)(j < grid - j ? j : grid - j);
                double dl = (double)(l < grid - l ? l : grid - l);
                shell[m++] = (int32_t)(f_nint(sqrt(di * di + dj * dj + dl * dl) / (double)kbin - kck - tiny) + 1);
            }
}

/* ishift, bispectrumI4.f90:38-42 */
static int bk_ishift(float kbin, float kcenter, int iopen) {
    int s = (int)f_int((double)(kcenter / kbin));
    return iopen ? s + 1 : s;
}

/* Triangle enumeration (bispectrumI4.f90:165-167, :733-735, :885-892). */
int64_t or_count_itot(int nbins, float kbin, float kcenter, int iopen, int cross) {
    int ishift = bk_ishift(kbin, kcenter, iopen);
    int64_t m = 0;
    for (int l = 1; l <= nbins; l++)
        for (int j = 1; j <= l; j++) {
            int imin = l - j + 1 - ishift; if (imin < 1) imin = 1;
            int imax = cross ? ((j + l - 1 + ishift) < nbins ? (j + l - 1 + ishift) : nbins) : j;
            for (int i = imin; i <= imax; i++) m++;
        }
    return m;
}

/* The "Last sum" loops of the four routines below visit the triangles in the
 * reference's order (l outer, j, then i); every triangle's sum is an independent
 * serial loop over the grid, so the routines take a row range [m0, m1) of that
 * order and compute only those rows: a caller may split the rows over threads
 * and gets the same bits as one serial pass.  The plain-named routines are the
 * whole range. */
#define TRI_LOOP_BEGIN(CROSS)                                                                   \
    int ishift = bk_ishift(kbin, kcenter, iopen);                                               \
    int64_t m = 0;                                                                              \
    for (int l = 1; l <= nbins && m < m1; l++)                                                  \
        for (int j = 1; j <= l && m < m1; j++) {                                                \
            int imin = l - j + 1 - ishift; if (imin < 1) imin = 1;                              \
            int imax = (CROSS) ? ((j + l - 1 + ishift) < nbins ? (j + l - 1 + ishift) : nbins) : j; \
            for (int i = imin; i <= imax; i++, m++) {                                           \
                if (m < m0) continue;                                                           \
                if (m >= m1) break;
#define TRI_LOOP_END }}

/* count_triangles "Last sum" (bispectrumI4.f90:884-908): maps are FP64
 * [nbins][gridD].  counts[m] = sum_n map_i map_j map_l. */
void or_triangle_counts_sum_rows(int nbins, float kbin, float kcenter, int iopen, int cross,
                                 int64_t gridD, const double *maps, double *counts, int64_t m0, int64_t m1) {
    TRI_LOOP_BEGIN(cross)
        const double *mi = maps + (size_t)(i - 1) * gridD;
        const double *mj = maps + (size_t)(j - 1) * gridD;
        const double *ml = maps + (size_t)(l - 1) * gridD;
        double sum = 0.0;
        for (int64_t n = 0; n < gridD; n++) sum = sum + mi[n] * mj[n] * ml[n];
        counts[m] = sum;
    TRI_LOOP_END
}

void or_triangle_counts_sum(int nbins, float kbin, float kcenter, int iopen, int cross,
                            int64_t gridD, const double *maps, double *counts) {
    or_triangle_counts_sum_rows(nbins, kbin, kcenter, iopen, cross, gridD, maps, counts, 0, INT64_MAX);
}

/* measure_bk "Last sum" (bispectrumI4.f90:160-193), bout(9,itot) Fortran order.
 * maps: FP64 [nbins][gridD]; pow[nbins] already shot-noise subtracted. */
void or_bk_last_sum_rows(int nbins, float kbin, float kcenter, int iopen, float kf, int64_t npart,
                         int64_t gridD, const float *counts, const double *maps, const double *pow_,
                         double *bout, int64_t m0, int64_t m1) {
    float kf3f = kf * kf * kf;
    double kf3 = (double)kf3f;
    double powSN = 1.0 / (double)npart / kf3;
    double powSN2 = powSN * powSN;
    TRI_LOOP_BEGIN(0)
        const double *mi = maps + (size_t)(i - 1) * gridD;
        const double *mj = maps + (size_t)(j - 1) * gridD;
        const double *ml = maps + (size_t)(l - 1) * gridD;
        double sum = 0.0;
        for (int64_t n = 0; n < gridD; n++) sum = sum + mi[n] * mj[n] * ml[n];
        double bispSN = (pow_[i - 1] + pow_[j - 1] + pow_[l - 1]) * powSN + powSN2;
        double *o = bout + 9 * m;
        o[0] = (double)kcenter + (double)(l - 1) * (double)kbin;
        o[1] = (double)kcenter + (double)(j - 1) * (double)kbin;
        o[2] = (double)kcenter + (double)(i - 1) * (double)kbin;
        o[3] = pow_[l - 1];
        o[4] = pow_[j - 1];
        o[5] = pow_[i - 1];
        o[6] = kf3 * sum / (double)counts[m] + bispSN;
        o[7] = bispSN;
        o[8] = (double)(float)((double)counts[m] / (double)gridD);
    TRI_LOOP_END
}

void or_bk_last_sum(int nbins, float kbin, float kcenter, int iopen, float kf, int64_t npart,
                    int64_t gridD, const float *counts, const double *maps, const double *pow_,
                    double *bout) {
    or_bk_last_sum_rows(nbins, kbin, kcenter, iopen, kf, npart, gridD, counts, maps, pow_, bout, 0, INT64_MAX);
}

/* measure_bk_multipoles "Last sum" (bispectrumI4.f90:476-511), bout(11,itot). */
void or_bk_multipoles_last_sum_rows(int nbins, float kbin, float kcenter, int iopen, float kf, int64_t npart,
                                    int64_t gridD, const float *counts, const double *maps,
                                    const double *maps2, const double *maps4, const double *pow_,
                                    double *bout, int64_t m0, int64_t m1) {
    float kf3f = kf * kf * kf;
    double kf3 = (double)kf3f;
    double powSN = 1.0 / (double)npart / kf3;
    double powSN2 = powSN * powSN;
    TRI_LOOP_BEGIN(0)
        const double *mi = maps + (size_t)(i - 1) * gridD;
        const double *mj = maps + (size_t)(j - 1) * gridD;
        const double *ml = maps + (size_t)(l - 1) * gridD;
        const double *m2l = maps2 + (size_t)(l - 1) * gridD;
        const double *m4l = maps4 + (size_t)(l - 1) * gridD;
        double sum = 0.0, sum2 = 0.0, sum4 = 0.0;
        for (int64_t n = 0; n < gridD; n++) {
            sum = sum + mi[n] * mj[n] * ml[n];
            sum2 = sum2 + mi[n] * mj[n] * m2l[n];
            sum4 = sum4 + mi[n] * mj[n] * m4l[n];
        }
        double bispSN = (pow_[i - 1] + pow_[j - 1] + pow_[l - 1]) * powSN + powSN2;
        double *o = bout + 11 * m;
        o[0] = (double)kcenter + (double)(l - 1) * (double)kbin;
        o[1] = (double)kcenter + (double)(j - 1) * (double)kbin;
        o[2] = (double)kcenter + (double)(i - 1) * (double)kbin;
        o[3] = pow_[l - 1];
        o[4] = pow_[j - 1];
        o[5] = pow_[i - 1];
        o[6] = kf3 * sum / (double)counts[m] + bispSN;
        o[7] = bispSN;
        o[8] = (double)(float)((double)counts[m] / (double)gridD);
        o[9] = 5 * kf3 * sum2 / (double)counts[m];
        o[10] = 9 * kf3 * sum4 / (double)counts[m];
    TRI_LOOP_END
}

void or_bk_multipoles_last_sum(int nbins, float kbin, float kcenter, int iopen, float kf, int64_t npart,
                               int64_t gridD, const float *counts, const double *maps,
                               const double *maps2, const double *maps4, const double *pow_,
                               double *bout) {
    or_bk_multipoles_last_sum_rows(nbins, kbin, kcenter, iopen, kf, npart, gridD, counts, maps, maps2, maps4,
                                   pow_, bout, 0, INT64_MAX);
}

/* measure_bk_cross "Last sum" (bispectrumI4.f90:732-756), bout(5,itot):
 * S = sum mapkB_i mapk_j mapk_l with i up to min(nbins, j+l-1+ishift). */
void or_bk_cross_last_sum_rows(int nbins, float kbin, float kcenter, int iopen, float kf,
                               int64_t gridD, const float *counts, const double *maps,
                               const double *mapsB, double *bout, int64_t m0, int64_t m1) {
    float kf3f = kf * kf * kf;
    double kf3 = (double)kf3f;
    TRI_LOOP_BEGIN(1)
        const double *bi = mapsB + (size_t)(i - 1) * gridD;
        const double *mj = maps + (size_t)(j - 1) * gridD;
        const double *ml = maps + (size_t)(l - 1) * gridD;
        double sum = 0.0;
        for (int64_t n = 0; n < gridD; n++) sum = sum + bi[n] * mj[n] * ml[n];
        double *o = bout + 5 * m;
        o[0] = (double)kcenter + (double)(l - 1) * (double)kbin;
        o[1] = (double)kcenter + (double)(j - 1) * (double)kbin;
        o[2] = (double)kcenter + (double)(i - 1) * (double)kbin;
        o[3] = kf3 * sum / (double)counts[m];
        o[4] = (double)(float)((double)counts[m] / (double)gridD);
    TRI_LOOP_END
}

void or_bk_cross_last_sum(int nbins, float kbin, float kcenter, int iopen, float kf,
                          int64_t gridD, const float *counts, const double *maps,
                          const double *mapsB, double *bout) {
    or_bk_cross_last_sum_rows(nbins, kbin, kcenter, iopen, kf, gridD, counts, maps, mapsB, bout, 0, INT64_MAX);
}
