// catalog.cu -- catalogue positions to the [0, 1] positions the assignment
// reads, on the device (IO.read_catalogues, pbi4.py:121-245).
//
// The reference (numpy) does, for a catalogue of dtype T (float32 or float64):
//   pos[:] += Vel[:] * los / Hz * (1 + z)      (pbi4.py:158, 170, 214; Minerva
//                                               pbi4.py:184: pos += Vel * los)
//   pos = (pos + box) % box                     (pbi4.py:242)
//   pos = np.minimum(1 - nextafter(0, 1), pos / box)   (pbi4.py:243)
// with numpy's promotion rules: Vel * los is float64 (los is a float64 array), so
// the shift is computed in float64 and rounded once into T by the in-place add;
// box is a Python float, so the wrap and the division run in T; the clip
// compares with a float64 scalar (1 - 5e-324 == 1.0), so the result is float64.
// np.remainder for floats is fmod plus b where fmod's sign differs from b's.
#include <math.h>

#include "common.cuh"

namespace pbi4g {

namespace {

template <class T>
__device__ __forceinline__ T remainder_np(T a, T b) {
    T m = fmod(a, b);
    if (m != (T)0 && ((b < (T)0) != (m < (T)0))) m += b;
    return m;
}

template <class T>
__global__ void catalog_positions_kernel(int64_t n, const T *__restrict__ pos, const T *__restrict__ vel, double l0,
                                         double l1, double l2, double hz, double opz, int mode, double box,
                                         double *__restrict__ out) {
    const T b = (T)box;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
#pragma unroll
        for (int d = 0; d < 3; d++) {
            T p = pos[3 * i + d];
            if (vel) {
                const double ld = d == 0 ? l0 : (d == 1 ? l1 : l2);
                // one rounding per numpy operation (no contraction into FMAs)
                double t = __dmul_rn((double)vel[3 * i + d], ld);
                if (mode == 1) t = __dmul_rn(__ddiv_rn(t, hz), opz);
                p = (T)__dadd_rn((double)p, t);
            }
            p = remainder_np<T>(p + b, b);
            const double q = (double)(p / b);
            out[(size_t)d * n + i] = (q < 1.0 || isnan(q)) ? q : 1.0;  // np.minimum keeps NaN
        }
    }
}

}  // namespace

}  // namespace pbi4g

using namespace pbi4g;

extern "C" {

int pbi4g_catalog_positions(int64_t npart, const void *d_pos, const void *d_vel, int32_t is_double,
                            const double *los, int32_t rsd_mode, double hz, double z, double box, double *d_out,
                            void *stream) {
    if (npart < 0 || (npart > 0 && (!d_pos || !d_out)) || !(box > 0) || (d_vel && !los) ||
        (d_vel && (rsd_mode < 0 || rsd_mode > 1)) || (d_vel && rsd_mode == 1 && !(hz != 0)))
        return set_error(PBI4G_ERR_INVALID, "catalogue positions: npart=%lld box=%g rsd_mode=%d hz=%g",
                         (long long)npart, box, rsd_mode, hz);
    if (npart == 0) return PBI4G_OK;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const double l0 = d_vel ? los[0] : 0, l1 = d_vel ? los[1] : 0, l2 = d_vel ? los[2] : 0;
    const double opz = 1.0 + z;
    const int blocks = grid_blocks((size_t)npart, 256);
    if (is_double)
        catalog_positions_kernel<double><<<blocks, 256, 0, st>>>(npart, static_cast<const double *>(d_pos),
                                                                 static_cast<const double *>(d_vel), l0, l1, l2, hz,
                                                                 opz, rsd_mode, box, d_out);
    else
        catalog_positions_kernel<float><<<blocks, 256, 0, st>>>(npart, static_cast<const float *>(d_pos),
                                                                static_cast<const float *>(d_vel), l0, l1, l2, hz,
                                                                opz, rsd_mode, box, d_out);
    PBI4G_LAUNCH_CHECK();
    return PBI4G_OK;
}

}  // extern "C"
