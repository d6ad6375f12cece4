// FP32 evaluation of the perplexity calibration's entropy H(beta) with an error bound,
// shared by the bisection (affinity.cu) and the warm-started search (calib_mlp.cu).
#pragma once
#include <cuda_runtime.h>

namespace fitsne {

// FP32 value of H(beta) on the row's shifted distances s[m * sstride] = (float)(d[m] - d0),
//   H = beta sum(d e) / sum(e) + log sum(e) = beta sum(t e') / sum(e') + log sum(e'),
// with t = d - d0 and e' = exp(-beta t): both terms are non-negative (sum(e') >= 1), so no
// cancellation occurs.  Returns H and, in *E, a bound on its error.  With u = 2^-24, each e'
// carries 3u |x| + 4u relative error (x = -beta t, with beta and t rounded to FP32 and
// their product rounded; expf within 2 ulp); the sums are compensated (2u); so, with
// h1 = beta <t>, h2 = beta^2 <t^2> (weights e'):
//   |dB| / B <= 3u h1 + 6u,  |dA| / A <= 3u h2 / h1 + 7u,
//   |dH| <= 3u h2 + 3u h1^2 + 19u h1 + 2u log B + u H + 6u   (first order);
// the bound used is twice that, plus 1e-9 for the FP64 value's own rounding.  *t1 and *t2
// (may be null) receive <t> and <t^2> for a Newton step.
static __device__ __forceinline__ float screen_value(const float *__restrict__ s, int sstride, int K, double beta,
                                                     double *E, float *t1 = nullptr, float *t2 = nullptr) {
    const float bf = (float) beta;
    float B = 0.f, cB = 0.f, A = 0.f, cA = 0.f, A2 = 0.f;
    for (int m = 0; m < K; ++m) {
        const float t = s[(size_t) m * sstride];
        const float e = expf(-bf * t);
        float y = e - cB;
        float z = B + y;
        cB = (z - B) - y;
        B = z;
        const float te = t * e;
        y = te - cA;
        z = A + y;
        cA = (z - A) - y;
        A = z;
        A2 = fmaf(t * t, e, A2);
    }
    const float mt = A / B, m2 = A2 / B;
    const float h1 = bf * mt, lb = logf(B);
    const float h = h1 + lb;
    const double u = 5.9604644775390625e-8;
    const double dh1 = h1, dh2 = (double) bf * bf * m2;
    *E = 2.0 * u * (3.0 * dh2 + 3.0 * dh1 * dh1 + 19.0 * dh1 + 2.0 * lb + fabs((double) h) + 6.0) + 1e-9;
    if (t1) *t1 = mt;
    if (t2) *t2 = m2;
    return h;
}

}  // namespace fitsne
