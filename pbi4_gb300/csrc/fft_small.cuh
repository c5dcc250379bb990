// fft_small.cuh -- building blocks of the shell-map inverse transforms
// (mapfft.cu): complex helpers, inverse DFTs of 2, 3, 4, 5, 7, 8 and 10 points, and
// the host-side plan of an in-place mixed-radix decimation-in-frequency FFT
// (radices 2, 3, 4, 5, 7, 8, 10 and 20).
//
// Sign convention: every transform here is an inverse DFT,
//   X[k] = sum_n x[n] e^{+2 pi i n k / N}   (no 1/N: cuFFT's CUFFT_INVERSE / C2R).
//
// In-place DIF over a batch of transforms held as buf[n * pitch + t] (t the
// transform, n the point): with N = R_1 R_2 ... R_s and L_1 = N, stage t
// (radix R = R_t, Ls = L_t / R) runs N / R butterflies j = b Ls + n1 over the
// points base + Ls r (base = b L_t + n1, r < R): an R-point DFT, then output q
// times e^{2 pi i n1 q / L_t}, stored back in place; L_{t+1} = Ls.  The result
// X[k] ends at the digit-reversed position perm[k]: for k = q + R_1 k1,
// perm_N(k) = q N / R_1 + perm_{N/R_1}(k1).
//
// The kernels run the transpose of that factorisation (the DFT matrix is
// symmetric, and so is every stage's block of R-point DFTs and its diagonal of
// twiddles): x[n] is placed at perm[n], the stages run last to first, each
// butterfly multiplies its inputs by the twiddles before the R-point DFT, and
// X[k] comes out at position k.  The permutation then falls on the side where
// the lanes run over transforms (conflict-free in shared memory) and the
// natural-order output is read along the points.
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <vector>

namespace pbi4g {
namespace fftd {

constexpr int kMaxRadix = 20;

// Complex helpers.  Device code forms additions, subtractions and products by
// a real number with the packed FP32 pair instructions (each element rounded as
// the scalar operation rounds it: about a third fewer FP instructions in the
// DFTs below); host code (the plan check) uses scalar arithmetic.
__host__ __device__ __forceinline__ float2 cadd(float2 a, float2 b) {
#ifdef __CUDA_ARCH__
    return __fadd2_rn(a, b);
#else
    return make_float2(a.x + b.x, a.y + b.y);
#endif
}
__host__ __device__ __forceinline__ float2 csub(float2 a, float2 b) {
#ifdef __CUDA_ARCH__
    return __ffma2_rn(b, make_float2(-1.f, -1.f), a);  // a - b, one rounding
#else
    return make_float2(a.x - b.x, a.y - b.y);
#endif
}
__host__ __device__ __forceinline__ float2 cscale(float2 a, float s) {
#ifdef __CUDA_ARCH__
    return __fmul2_rn(a, make_float2(s, s));
#else
    return make_float2(s * a.x, s * a.y);
#endif
}
// a + c b for a real c (one rounding per element)
__host__ __device__ __forceinline__ float2 caxpy(float c, float2 b, float2 a) {
#ifdef __CUDA_ARCH__
    return __ffma2_rn(make_float2(c, c), b, a);
#else
    return make_float2(std::fma(c, b.x, a.x), std::fma(c, b.y, a.y));
#endif
}
__host__ __device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ __forceinline__ float2 itimes(float2 a) { return make_float2(-a.y, a.x); }  // i a
// a + i w and a - i w (the rotation swaps components: scalar)
__host__ __device__ __forceinline__ float2 cadd_i(float2 a, float2 w) { return make_float2(a.x - w.y, a.y + w.x); }
__host__ __device__ __forceinline__ float2 csub_i(float2 a, float2 w) { return make_float2(a.x + w.y, a.y - w.x); }

// inverse DFT of R points in place: v[q] <- sum_r v[r] e^{+2 pi i q r / R}
template <int R>
__host__ __device__ __forceinline__ void dft_small(float2 (&v)[kMaxRadix]) {
    if constexpr (R == 2) {
        const float2 a = v[0], b = v[1];
        v[0] = cadd(a, b);
        v[1] = csub(a, b);
    } else if constexpr (R == 3) {
        const float c = -0.5f, sn = 0.8660254037844386f;
        const float2 b = cadd(v[1], v[2]), d = csub(v[1], v[2]);
        const float2 t = caxpy(c, b, v[0]);
        const float2 w = cscale(d, sn);
        v[0] = cadd(v[0], b);
        v[1] = cadd_i(t, w);
        v[2] = csub_i(t, w);
    } else if constexpr (R == 4) {
        const float2 s02 = cadd(v[0], v[2]), d02 = csub(v[0], v[2]);
        const float2 s13 = cadd(v[1], v[3]), d13 = csub(v[1], v[3]);
        v[0] = cadd(s02, s13);
        v[2] = csub(s02, s13);
        v[1] = cadd_i(d02, d13);
        v[3] = csub_i(d02, d13);
    } else if constexpr (R == 5) {
        const float c1 = 0.30901699437494745f, c2 = -0.8090169943749475f;
        const float s1 = 0.9510565162951535f, s2 = 0.5877852522924731f;
        const float2 b1 = cadd(v[1], v[4]), b2 = cadd(v[2], v[3]);
        const float2 d1 = csub(v[1], v[4]), d2 = csub(v[2], v[3]);
        const float2 t1 = caxpy(c2, b2, caxpy(c1, b1, v[0]));
        const float2 t2 = caxpy(c1, b2, caxpy(c2, b1, v[0]));
        const float2 w1 = caxpy(s2, d2, cscale(d1, s1));
        const float2 w2 = caxpy(-s1, d2, cscale(d1, s2));
        v[0] = cadd(v[0], cadd(b1, b2));
        v[1] = cadd_i(t1, w1);
        v[4] = csub_i(t1, w1);
        v[2] = cadd_i(t2, w2);
        v[3] = csub_i(t2, w2);
    } else if constexpr (R == 7) {
        // pairs (r, 7 - r): X[q] = v0 + sum_k cos(2 pi k q / 7) b_k + i sum_k sin(2 pi k q / 7) d_k
        const float c1 = 0.6234898018587336f, c2 = -0.22252093395631434f, c3 = -0.900968867902419f;
        const float s1 = 0.7818314824680298f, s2 = 0.9749279121818236f, s3 = 0.43388373911755823f;
        const float2 b1 = cadd(v[1], v[6]), b2 = cadd(v[2], v[5]), b3 = cadd(v[3], v[4]);
        const float2 d1 = csub(v[1], v[6]), d2 = csub(v[2], v[5]), d3 = csub(v[3], v[4]);
        const float2 x0 = v[0];
        const float2 t1 = caxpy(c3, b3, caxpy(c2, b2, caxpy(c1, b1, x0)));
        const float2 t2 = caxpy(c1, b3, caxpy(c3, b2, caxpy(c2, b1, x0)));
        const float2 t3 = caxpy(c2, b3, caxpy(c1, b2, caxpy(c3, b1, x0)));
        const float2 w1 = caxpy(s3, d3, caxpy(s2, d2, cscale(d1, s1)));
        const float2 w2 = caxpy(-s1, d3, caxpy(-s3, d2, cscale(d1, s2)));
        const float2 w3 = caxpy(s2, d3, caxpy(-s1, d2, cscale(d1, s3)));
        v[0] = cadd(x0, cadd(b1, cadd(b2, b3)));
        v[1] = cadd_i(t1, w1);
        v[6] = csub_i(t1, w1);
        v[2] = cadd_i(t2, w2);
        v[5] = csub_i(t2, w2);
        v[3] = cadd_i(t3, w3);
        v[4] = csub_i(t3, w3);
    } else if constexpr (R == 10) {
        // prime-factor split 10 = 2 x 5 (no twiddles): n = (5 n1 + 2 n2) mod 10,
        // X[k] with k = k1 (mod 2), k = k2 (mod 5): 2-point DFTs over n1, then
        // 5-point DFTs over n2; X[k2 even/odd partner] read back by the CRT map
        float2 a[kMaxRadix], b[kMaxRadix];
#pragma unroll
        for (int n2 = 0; n2 < 5; n2++) {
            const float2 x0 = v[(2 * n2) % 10], x1 = v[(5 + 2 * n2) % 10];
            a[n2] = cadd(x0, x1);  // k1 = 0
            b[n2] = csub(x0, x1);  // k1 = 1
        }
        dft_small<5>(a);
        dft_small<5>(b);
        // k = 5 k1 + 6 k2 (mod 10): k mod 2 = k1, k mod 5 = k2
#pragma unroll
        for (int k2 = 0; k2 < 5; k2++) {
            v[(6 * k2) % 10] = a[k2];
            v[(5 + 6 * k2) % 10] = b[k2];
        }
    } else if constexpr (R == 20) {
        // prime-factor split 20 = 4 x 5 (no twiddles): n = (5 n1 + 4 n2) mod 20,
        // 4-point DFTs over n1, then 5-point DFTs over n2; X[k] for k = k1 (mod 4),
        // k = k2 (mod 5) sits at k = (5 k1 + 16 k2) mod 20
        float2 c[5][kMaxRadix];
#pragma unroll
        for (int n2 = 0; n2 < 5; n2++) {
#pragma unroll
            for (int n1 = 0; n1 < 4; n1++) c[n2][n1] = v[(5 * n1 + 4 * n2) % 20];
            dft_small<4>(c[n2]);
        }
#pragma unroll
        for (int k1 = 0; k1 < 4; k1++) {
            float2 d[kMaxRadix];
#pragma unroll
            for (int n2 = 0; n2 < 5; n2++) d[n2] = c[n2][k1];
            dft_small<5>(d);
#pragma unroll
            for (int k2 = 0; k2 < 5; k2++) v[(5 * k1 + 16 * k2) % 20] = d[k2];
        }
    } else {
        static_assert(R == 8, "radix");
        // one radix-2 step (n, n + 4) then two 4-point DFTs: even outputs from the
        // sums, odd outputs from the differences times e^{2 pi i r / 8}
        const float h = 0.7071067811865476f;
        float2 a[4], b[4];
#pragma unroll
        for (int r = 0; r < 4; r++) {
            a[r] = cadd(v[r], v[r + 4]);
            b[r] = csub(v[r], v[r + 4]);
        }
        b[1] = make_float2(h * (b[1].x - b[1].y), h * (b[1].x + b[1].y));    // (1 + i) / sqrt 2
        b[2] = itimes(b[2]);                                                // i
        b[3] = make_float2(-h * (b[3].x + b[3].y), h * (b[3].x - b[3].y));  // (-1 + i) / sqrt 2
        float2 e[kMaxRadix], o[kMaxRadix];
#pragma unroll
        for (int r = 0; r < 4; r++) {
            e[r] = a[r];
            o[r] = b[r];
        }
        dft_small<4>(e);
        dft_small<4>(o);
#pragma unroll
        for (int q = 0; q < 4; q++) {
            v[2 * q] = e[q];
            v[2 * q + 1] = o[q];
        }
    }
}

// The transposed (decimation-in-time) butterfly: inputs r times tw[r * tstep],
// then the R-point DFT, in place.
template <int R>
__host__ __device__ __forceinline__ void dit_butterfly(float2 *buf, int pitch, int t, int base, int ls, int tstep,
                                                       const float2 *tw) {
    float2 v[kMaxRadix];
    v[0] = buf[base * pitch + t];
    if (tstep) {
#pragma unroll
        for (int r = 1; r < R; r++) v[r] = cmul(buf[(base + ls * r) * pitch + t], tw[r * tstep]);
    } else {
#pragma unroll
        for (int r = 1; r < R; r++) v[r] = buf[(base + ls * r) * pitch + t];
    }
    dft_small<R>(v);
#pragma unroll
    for (int q = 0; q < R; q++) buf[(base + ls * q) * pitch + t] = v[q];
}

constexpr int kMaxStages = 10;

// Device-side description of an in-place DIF plan; its tables (stage entries,
// perm, twiddles) live in one device buffer laid out as FftPlan::pack writes it.
struct FftDesc {
    int n = 0, nst = 0;
    int rad[kMaxStages] = {0}, ls[kMaxStages] = {0}, eoff[kMaxStages] = {0};
    int nent = 0;  // stage entries in total
};

// Host plan: radices, per-stage butterfly entries (base, tstep), output perm, twiddles.
struct FftPlan {
    FftDesc d;
    std::vector<int2> ent;   // [nent]: (base, tstep) per butterfly, stage by stage
    std::vector<int> perm;   // [n]: position of X[k]
    std::vector<float2> tw;  // [n]: e^{2 pi i s / n}

    // false when n has a prime factor above 7 (or needs too many stages).  Radices
    // are taken greedily from {10, 8, 4, 2, 3, 5, 7}; with allow20 the factorisation
    // that starts with 20 is used instead when it has fewer stages (each stage is a
    // round trip of every point through shared memory).
    bool build(int n, bool allow20 = false) {
        auto factor = [&](bool with20, FftDesc &o) {
            o = FftDesc();
            o.n = n;
            int rest = n;
            if (with20)
                while (rest % 20 == 0) {
                    if (o.nst == kMaxStages) return false;
                    o.rad[o.nst++] = 20;
                    rest /= 20;
                }
            for (int r : {10, 8, 4, 2, 3, 5, 7})
                while (rest % r == 0) {
                    if (o.nst == kMaxStages) return false;
                    o.rad[o.nst++] = r;
                    rest /= r;
                }
            return rest == 1 && n >= 2;
        };
        FftDesc alt;
        if (!factor(false, d)) return false;
        if (allow20 && factor(true, alt) && alt.nst < d.nst) d = alt;
        ent.clear();
        int L = n;
        for (int s = 0; s < d.nst; s++) {
            const int R = d.rad[s], Ls = L / R;
            d.ls[s] = Ls;
            d.eoff[s] = (int)ent.size();
            for (int j = 0; j < n / R; j++) {
                const int b = j / Ls, n1 = j % Ls;
                ent.push_back(make_int2(b * L + n1, n1 * (n / L)));
            }
            L = Ls;
        }
        d.nent = (int)ent.size();
        perm.assign(n, 0);
        for (int k = 0; k < n; k++) {
            int pos = 0, kk = k, len = n;
            for (int s = 0; s < d.nst; s++) {
                const int R = d.rad[s], sub = len / R;
                pos += (kk % R) * sub;
                kk /= R;
                len = sub;
            }
            perm[k] = pos;
        }
        tw.resize(n);
        for (int s = 0; s < n; s++)
            tw[s] = make_float2((float)std::cos(2.0 * M_PI * s / n), (float)std::sin(2.0 * M_PI * s / n));
        return true;
    }

    // bytes of the packed tables: twiddles, entries, perm
    size_t bytes() const { return sizeof(float2) * tw.size() + sizeof(int2) * ent.size() + sizeof(int) * perm.size(); }
    void pack(unsigned char *dst) const {
        size_t o = 0;
        for (const float2 &t : tw) { *reinterpret_cast<float2 *>(dst + o) = t; o += sizeof(float2); }
        for (const int2 &e : ent) { *reinterpret_cast<int2 *>(dst + o) = e; o += sizeof(int2); }
        for (int p : perm) { *reinterpret_cast<int *>(dst + o) = p; o += sizeof(int); }
    }
};

// Run the transposed plan over transform t of buf on one thread, input already
// at the permuted positions (the host check of the plan and butterflies; the
// kernels run the same butterflies across warps).
inline void run_plan_host(const FftPlan &p, float2 *buf, int pitch, int t) {
    for (int s = p.d.nst - 1; s >= 0; s--) {
        for (int j = 0; j < p.d.n / p.d.rad[s]; j++) {
            const int2 e = p.ent[p.d.eoff[s] + j];
            switch (p.d.rad[s]) {
                case 2: dit_butterfly<2>(buf, pitch, t, e.x, p.d.ls[s], e.y, p.tw.data()); break;
                case 3: dit_butterfly<3>(buf, pitch, t, e.x, p.d.ls[s], e.y, p.tw.data()); break;
                case 4: dit_butterfly<4>(buf, pitch, t, e.x, p.d.ls[s], e.y, p.tw.data()); break;
                case 5: dit_butterfly<5>(buf, pitch, t, e.x, p.d.ls[s], e.y, p.tw.data()); break;
                case 7: dit_butterfly<7>(buf, pitch, t, e.x, p.d.ls[s], e.y, p.tw.data()); break;
                case 8: dit_butterfly<8>(buf, pitch, t, e.x, p.d.ls[s], e.y, p.tw.data()); break;
                case 20: dit_butterfly<20>(buf, pitch, t, e.x, p.d.ls[s], e.y, p.tw.data()); break;
                default: dit_butterfly<10>(buf, pitch, t, e.x, p.d.ls[s], e.y, p.tw.data()); break;
            }
        }
    }
}

}  // namespace fftd
}  // namespace pbi4g
