// Shared device helpers for the FIt-SNE GB300 kernels.
//
// Precision scheme of the fast (FP32) form:
//  * embedding coordinates are kept as double-float pairs (hi + lo, two FP32 values,
//    about 48 significant bits) so that box-local offsets and neighbour differences are
//    exact to FP32 relative precision however far a point sits from the origin;
//  * everything downstream of those differences (Lagrange weights, spread, FFT, gather,
//    attraction) runs in FP32;
//  * reductions that feed a global scalar (Z, KL, the mean of Y) accumulate in FP64.
// The plain form instantiates the same kernels with double everywhere.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#define FITSNE_HD __host__ __device__ __forceinline__
#define FITSNE_D __device__ __forceinline__

namespace fitsne {

// ---------------------------------------------------------------------------------
// complex helpers
template <typename T>
struct Cx;
template <>
struct Cx<float> {
    typedef float2 t;
};
template <>
struct Cx<double> {
    typedef double2 t;
};

FITSNE_HD float2 mkc(float a, float b) { return make_float2(a, b); }
FITSNE_HD double2 mkc(double a, double b) { return make_double2(a, b); }
template <typename C>
FITSNE_HD C cadd(C a, C b) { return mkc(a.x + b.x, a.y + b.y); }
template <typename C>
FITSNE_HD C csub(C a, C b) { return mkc(a.x - b.x, a.y - b.y); }
template <typename C>
FITSNE_HD C cmul(C a, C b) { return mkc(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
template <typename C>
FITSNE_HD C cconj(C a) { return mkc(a.x, -a.y); }
// multiply by -i (forward) or +i (inverse)
template <typename C>
FITSNE_HD C cmul_mi(C a) { return mkc(a.y, -a.x); }
template <typename C>
FITSNE_HD C cmul_pi(C a) { return mkc(-a.y, a.x); }
template <typename C, typename T>
FITSNE_HD C cscale(C a, T s) { return mkc(a.x * s, a.y * s); }

// ---------------------------------------------------------------------------------
// double-float arithmetic (Knuth two-sum / Dekker with FMA)
struct df32 {
    float hi, lo;
};

FITSNE_HD df32 two_sum(float a, float b) {
    float s = a + b;
    float bb = s - a;
    float e = (a - (s - bb)) + (b - bb);
    return {s, e};
}
FITSNE_HD df32 quick_two_sum(float a, float b) {
    float s = a + b;
    float e = b - (s - a);
    return {s, e};
}
FITSNE_HD df32 df_add(df32 a, df32 b) {
    df32 s = two_sum(a.hi, b.hi);
    float e = s.lo + a.lo + b.lo;
    return quick_two_sum(s.hi, e);
}
FITSNE_HD df32 df_add_f(df32 a, float b) {
    df32 s = two_sum(a.hi, b);
    float e = s.lo + a.lo;
    return quick_two_sum(s.hi, e);
}
FITSNE_HD df32 df_neg(df32 a) { return {-a.hi, -a.lo}; }
FITSNE_HD df32 df_from_double(double x) {
    float h = (float) x;
    float l = (float) (x - (double) h);
    return {h, l};
}
FITSNE_HD double df_to_double(df32 a) { return (double) a.hi + (double) a.lo; }
// (a - b) rounded to float, accurate to float precision of the difference
FITSNE_HD float df_diff(df32 a, df32 b) { return (a.hi - b.hi) + (a.lo - b.lo); }
#ifdef __CUDACC__
FITSNE_D df32 two_prod(float a, float b) {
    float p = a * b;
    float e = __fmaf_rn(a, b, -p);
    return {p, e};
}
#endif

// ---------------------------------------------------------------------------------
// scalar helpers
template <typename T>
FITSNE_HD T sgn(T x) {
    return x == T(0) ? T(0) : (x < T(0) ? T(-1) : T(1));
}

constexpr int kMaxInterp = 8;  // largest n_interpolation_points supported on the device

}  // namespace fitsne
