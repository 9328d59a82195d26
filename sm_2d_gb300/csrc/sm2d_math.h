/* sm2d_math.h -- single-precision exp, log, sin, cos and erf written with
 * IEEE basic operations only (add, subtract, multiply, divide, compare and
 * integer moves of the bit pattern).
 *
 * The transport kernels (nvcc --fmad=false) and the C oracle
 * (gcc -ffp-contract=off) both call these, so every per-bin quantity -- and
 * with it every angle bin, energy bin, block id and slot decision -- comes
 * out bit-identical on the GPU and on the host.  Results differ from CUDA's
 * and glibc's own functions by about one ulp, as those two differ from each
 * other.
 *
 * Methods (constants derived from exact values by sm2d_math_coeffs.py):
 *   exp  Cody-Waite reduction x = k ln2 + r (W. J. Cody, W. Waite, Software
 *        Manual for the Elementary Functions, 1980), Taylor series of e^r on
 *        |r| <= ln2/2, exact scaling by 2^k;                  max 1.1 ulp
 *   log  x = m 2^e with m in [sqrt(1/2), sqrt(2)), log m = 2 atanh(s),
 *        s = (m-1)/(m+1), by its series;                      max 1.9 ulp
 *   sin, cos  reduction by pi/2 in three parts, Taylor series on
 *        |r| <= pi/4; arguments |x| < 1e4;                    max 1.7 ulp
 *   erf  Chebyshev least-squares fits on [0,1] (as x + x R(x^2)), [1,2],
 *        [2,4]; 1 beyond 4;                                   max 1.2 ulp
 * (errors over dense samples of the ranges the transport uses, against
 * double-precision libm). */
#pragma once
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define SM2D_MF __host__ __device__ __forceinline__
#else
#define SM2D_MF static inline
#endif

SM2D_MF uint32_t sm2d_fbits(float x) {
    uint32_t u;
    memcpy(&u, &x, 4);
    return u;
}
SM2D_MF float sm2d_bitsf(uint32_t u) {
    float x;
    memcpy(&x, &u, 4);
    return x;
}
/* floor of a float known to lie well inside the int range */
SM2D_MF int sm2d_ifloor(float y) {
    int i = (int)y;
    return ((float)i > y) ? i - 1 : i;
}
/* 2^k, exact, for -149 <= k <= 127 */
SM2D_MF float sm2d_pow2i(int k) {
    return k >= -126 ? sm2d_bitsf((uint32_t)(k + 127) << 23) : sm2d_bitsf(1u << (k + 149));
}

SM2D_MF float sm2d_expf(float x) {
    if (x != x) return x;
    if (x > 88.72283935546875f) return sm2d_bitsf(0x7f800000u);
    if (x < -103.97208404541016f) return 0.0f;
    const int k = sm2d_ifloor(x * 1.4426950216293335f + 0.5f);
    const float kf = (float)k;
    const float r = (x - kf * 0.693145751953125f) - kf * 1.428606765330187e-06f;
    float p = 0.00019841270113829523f;
    p = p * r + 0.0013888889225199819f;
    p = p * r + 0.008333333767950535f;
    p = p * r + 0.0416666679084301f;
    p = p * r + 0.1666666716337204f;
    p = p * r + 0.5f;
    p = p * r + 1.0f;
    p = p * r + 1.0f;
    if (k > 127) return (p * sm2d_pow2i(127)) * sm2d_pow2i(k - 127);
    if (k < -126) return (p * sm2d_pow2i(-126)) * sm2d_pow2i(k + 126);
    return p * sm2d_pow2i(k);
}

SM2D_MF float sm2d_logf(float x) {
    if (x != x) return x;
    if (x < 0.0f) return sm2d_bitsf(0x7fc00000u);
    if (x == 0.0f) return sm2d_bitsf(0xff800000u);
    uint32_t u = sm2d_fbits(x);
    if (u >= 0x7f800000u) return x;
    int e = 0;
    if (u < 0x00800000u) {   /* subnormal: scale into the normal range */
        x = x * 8388608.0f;
        u = sm2d_fbits(x);
        e = -23;
    }
    e += (int)(u >> 23) - 127;
    float m = sm2d_bitsf((u & 0x007fffffu) | 0x3f800000u);
    if (m > 1.4142135381698608f) {
        m = m * 0.5f;
        e += 1;
    }
    const float f = m - 1.0f;
    const float s = f / (2.0f + f);
    const float t = s * s;
    float p = 0.07692307978868484f;
    p = p * t + 0.09090909361839294f;
    p = p * t + 0.1111111119389534f;
    p = p * t + 0.1428571492433548f;
    p = p * t + 0.20000000298023224f;
    p = p * t + 0.3333333432674408f;
    p = p * t;
    const float s2 = s + s;
    const float lm = s2 + s2 * p;
    const float ef = (float)e;
    return ef * 0.693145751953125f + (lm + ef * 1.428606765330187e-06f);
}

/* r = x - k pi/2 and the quadrant k mod 4 */
SM2D_MF float sm2d_reduce_pi2(float x, int* q) {
    const int k = sm2d_ifloor(x * 0.6366197466850281f + 0.5f);
    const float kf = (float)k;
    *q = k & 3;
    return ((x - kf * 1.57080078125f) - kf * -4.453584551811218e-06f) - kf * -8.705515752716053e-10f;
}
SM2D_MF float sm2d_sin_poly(float r) {
    const float t = r * r;
    float p = -2.5052107943679403e-08f;
    p = p * t + 2.7557318844628753e-06f;
    p = p * t + -0.00019841270113829523f;
    p = p * t + 0.008333333767950535f;
    p = p * t + -0.1666666716337204f;
    return r + (r * t) * p;
}
SM2D_MF float sm2d_cos_poly(float r) {
    const float t = r * r;
    float p = 2.0876755879584152e-09f;
    p = p * t + -2.755731998149713e-07f;
    p = p * t + 2.4801587642286904e-05f;
    p = p * t + -0.0013888889225199819f;
    p = p * t + 0.0416666679084301f;
    p = p * t + -0.5f;
    return 1.0f + t * p;
}
SM2D_MF float sm2d_sinf(float x) {
    int q;
    const float r = sm2d_reduce_pi2(x, &q);
    const float v = (q & 1) ? sm2d_cos_poly(r) : sm2d_sin_poly(r);
    return (q & 2) ? -v : v;
}
SM2D_MF float sm2d_cosf(float x) {
    int q;
    const float r = sm2d_reduce_pi2(x, &q);
    const float v = (q & 1) ? sm2d_sin_poly(r) : sm2d_cos_poly(r);
    return ((q + 1) & 2) ? -v : v;
}

SM2D_MF float sm2d_erff(float x) {
    if (x != x) return x;
    const float a = x < 0.0f ? -x : x;
    float y;
    if (a < 1.0f) {
        const float t = a * a;
        float p = 8.00684210844338e-05f;
        p = p * t + -0.0008053741184994578f;
        p = p * t + 0.005192956887185574f;
        p = p * t + -0.026856068521738052f;
        p = p * t + 0.11283634603023529f;
        p = p * t + -0.3761262893676758f;
        p = p * t + 0.12837916612625122f;
        y = a + a * p;
    } else if (a < 2.0f) {
        const float u = a - 1.5f;
        float p = -4.159687887295149e-05f;
        p = p * u + 0.0015482403105124831f;
        p = p * u + -0.0023760374169796705f;
        p = p * u + -0.00470518134534359f;
        p = p * u + 0.019327789545059204f;
        p = p * u + -0.01487016398459673f;
        p = p * u + -0.04459894821047783f;
        p = p * u + 0.13875216245651245f;
        p = p * u + -0.17839543521404266f;
        p = p * u + 0.11893028765916824f;
        y = p * u + 0.9661051630973816f;
    } else if (a < 4.0f) {
        const float u = a - 3.0f;
        float p = 1.501270503467822e-06f;
        p = p * u + -9.547827175993007e-06f;
        p = p * u + 1.7624568499741144e-05f;
        p = p * u + 1.2103173503419384e-05f;
        p = p * u + -0.00013608112931251526f;
        p = p * u + 0.00039168717921711504f;
        p = p * u + -0.0007376078865490854f;
        p = p * u + 0.0010162255493924022f;
        p = p * u + -0.0010444661602377892f;
        p = p * u + 0.0007891395362094045f;
        p = p * u + -0.0004177551600150764f;
        p = p * u + 0.00013925172970630229f;
        y = p * u + 0.9999778866767883f;
        if (y > 1.0f) y = 1.0f;
    } else {
        y = 1.0f;
    }
    return x < 0.0f ? -y : y;
}
