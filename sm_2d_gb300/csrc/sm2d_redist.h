/* sm2d_redist.h -- redistribution weights of the expectation form of the
 * transport step, shared by the CUDA kernels and the C oracle.
 *
 * The reference's K2/K3 draw one hashed Gaussian MCS angle and (K3) one
 * hashed Vavilov straggling loss per local bin and step, then re-bin the
 * sampled component: the angle onto the nearest bin centre with a frac^2
 * share to the neighbour towards the sample (variance preserving,
 * device_bucket.cuh:450-478), the energy onto the bin containing it (with
 * this build's energy split: a mean-preserving pair of neighbouring centres).
 * The expectation form replaces each draw by its distribution and emits the
 * expected result of that re-binning instead of one sample of it:
 *
 *   theta  distance t = 0..7 bins from the incoming bin centre c, mass Mt[t]
 *          (t >= 1: half of it to c - t, half to c + t), for an offset
 *          u ~ N(0, s^2) in units of the bin width, s = sigma_theta / dtheta:
 *          E[ (1 - r^2) at round(u), r^2 at the neighbour towards u ] with
 *          r = u - round(u); distances beyond 6 fold into t = 7.
 *   energy offset e = 0..emax below the window top j (bin j - e, centre
 *          cen[e]), mass Me[e], for E' ~ N(E_mean, sigma_E^2): the expected
 *          mean-preserving split of E' between the two centres around it;
 *          E' above cen[0] folds into e = 0, below cen[emax] into emax.  The
 *          window's top is the second bin centre above E_mean, at most the
 *          incoming bin (E' above the incoming energy folds into it, as the
 *          reference clamps a negative straggling loss to zero).
 *
 * Both masses come from closed forms in the standard normal CDF and density
 * (integrals of (u - a)^2 phi and of linear ramps times phi over bin
 * intervals).  The table of a component is T[t + 8 e] = Mt[t] Me[e]: the 8
 * theta x 4 E layout the learned surrogate predicts.  Parts lighter than the
 * split threshold fold into the centre angle / the major energy (the energy
 * split's rule for light minor parts).
 *
 * The includer may define SM2D_RD_DOUBLE to evaluate in double with the C
 * library (the FP64 oracle); otherwise float with sm2d_math.h, so that the
 * kernels (nvcc --fmad=false) and the float oracle (gcc -ffp-contract=off)
 * agree bit for bit. */
#pragma once
#include "sm2d_math.h"

#ifdef SM2D_RD_DOUBLE
#include <math.h>
typedef double sm2d_rd_t;
#define SM2D_RD_C(x) (x)
#define SM2D_RD_ERF erf
#define SM2D_RD_EXP exp
#else
typedef float sm2d_rd_t;
#define SM2D_RD_C(x) (x##f)
#define SM2D_RD_ERF sm2d_erff
#define SM2D_RD_EXP sm2d_expf
#endif

#define SM2D_RD_NT 8    /* angular distances 0..7      */
#define SM2D_RD_NE 4    /* energy offsets 0..3 below j */
#define SM2D_RD_KIDS 15 /* angular children per energy offset: c, c-1, c+1, ..., c-7, c+7 */

/* standard normal CDF and density; exactly 1/0 and 0 beyond 8 */
SM2D_MF sm2d_rd_t sm2d_rd_Phi(sm2d_rd_t v) {
    if (v > SM2D_RD_C(8.0)) return SM2D_RD_C(1.0);
    if (v < SM2D_RD_C(-8.0)) return SM2D_RD_C(0.0);
    return SM2D_RD_C(0.5) * (SM2D_RD_C(1.0) + SM2D_RD_ERF(v * SM2D_RD_C(0.70710678118654752)));
}
SM2D_MF sm2d_rd_t sm2d_rd_phi(sm2d_rd_t v) {
    if (v > SM2D_RD_C(8.0) || v < SM2D_RD_C(-8.0)) return SM2D_RD_C(0.0);
    return SM2D_RD_C(0.39894228040143268) * SM2D_RD_EXP(SM2D_RD_C(-0.5) * (v * v));
}

/* integral over u in [kl/2, kh/2] of (u - a)^2 phi_s(u) (points given as
 * half-integer indices with their standardised CDF and density values) */
SM2D_MF sm2d_rd_t sm2d_rd_sq(sm2d_rd_t s, int kl, int kh, sm2d_rd_t a, const sm2d_rd_t* P, const sm2d_rd_t* p) {
    const sm2d_rd_t L = ((sm2d_rd_t)kl * SM2D_RD_C(0.5)) / s, H = ((sm2d_rd_t)kh * SM2D_RD_C(0.5)) / s, A = a / s;
    const sm2d_rd_t v = (SM2D_RD_C(1.0) + A * A) * (P[kh] - P[kl]) - (H * p[kh] - L * p[kl]) +
                        SM2D_RD_C(2.0) * A * (p[kh] - p[kl]);
    return (s * s) * v;
}

/* angular masses Mt[0..7] for s = sigma_theta / dtheta */
SM2D_MF void sm2d_rd_theta(sm2d_rd_t s, sm2d_rd_t* Mt) {
    for (int t = 0; t < SM2D_RD_NT; ++t) Mt[t] = SM2D_RD_C(0.0);
    if (!(s > SM2D_RD_C(1e-6))) {
        Mt[0] = SM2D_RD_C(1.0);
        return;
    }
    sm2d_rd_t P[15], p[15];   /* at u = k / 2, k = 0..14 */
    for (int k = 0; k < 15; ++k) {
        const sm2d_rd_t v = ((sm2d_rd_t)k * SM2D_RD_C(0.5)) / s;
        P[k] = sm2d_rd_Phi(v);
        p[k] = sm2d_rd_phi(v);
    }
    /* offset 0: samples in [-1/2, 1/2] keep 1 - r^2, samples in the inner
     * halves of bins -1 and +1 send (u +- 1)^2 back */
    const sm2d_rd_t in0 = (P[1] - P[0]) + (P[1] - P[0]);
    const sm2d_rd_t sq0 = sm2d_rd_sq(s, 0, 1, SM2D_RD_C(0.0), P, p) + sm2d_rd_sq(s, 0, 1, SM2D_RD_C(0.0), P, p);
    sm2d_rd_t m0 = (in0 - sq0) + (sm2d_rd_sq(s, 1, 2, SM2D_RD_C(1.0), P, p) + sm2d_rd_sq(s, 1, 2, SM2D_RD_C(1.0), P, p));
    Mt[0] = m0 > SM2D_RD_C(0.0) ? m0 : SM2D_RD_C(0.0);
    sm2d_rd_t sum = Mt[0];
    for (int m = 1; m < SM2D_RD_NT - 1; ++m) {
        /* one side: bin m keeps 1 - r^2, bin m-1's outer half sends r^2 up,
         * bin m+1's inner half sends r^2 down */
        const sm2d_rd_t a = (P[2 * m + 1] - P[2 * m - 1]) - sm2d_rd_sq(s, 2 * m - 1, 2 * m + 1, (sm2d_rd_t)m, P, p);
        const sm2d_rd_t b = sm2d_rd_sq(s, 2 * m - 2, 2 * m - 1, (sm2d_rd_t)(m - 1), P, p);
        const sm2d_rd_t c = sm2d_rd_sq(s, 2 * m + 1, 2 * m + 2, (sm2d_rd_t)(m + 1), P, p);
        sm2d_rd_t side = (a + b) + c;
        side = side > SM2D_RD_C(0.0) ? side : SM2D_RD_C(0.0);
        Mt[m] = side + side;
        sum = sum + Mt[m];
    }
    const sm2d_rd_t tail = SM2D_RD_C(1.0) - sum;
    Mt[SM2D_RD_NT - 1] = tail > SM2D_RD_C(0.0) ? tail : SM2D_RD_C(0.0);
    /* the rounding of the sums lands on the centre mass */
    sm2d_rd_t off = SM2D_RD_C(0.0);
    for (int t = SM2D_RD_NT - 1; t >= 1; --t) off = off + Mt[t];
    Mt[0] = SM2D_RD_C(1.0) - off;
}

/* energy masses Me[0..emax] for E' ~ N(Em, sE^2) over the centres cen[0] >
 * cen[1] > ... > cen[emax] (emax <= 3); returns the represented energy
 * sum Me[e] cen[e] */
SM2D_MF sm2d_rd_t sm2d_rd_energy(sm2d_rd_t Em, sm2d_rd_t sE, const sm2d_rd_t* cen, int emax, sm2d_rd_t* Me) {
    for (int e = 0; e < SM2D_RD_NE; ++e) Me[e] = SM2D_RD_C(0.0);
    if (emax <= 0) {
        Me[0] = SM2D_RD_C(1.0);
        return cen[0];
    }
    if (!(sE > SM2D_RD_C(1e-9))) {   /* no spread: the split of Em itself */
        if (Em >= cen[0]) Me[0] = SM2D_RD_C(1.0);
        else if (Em <= cen[emax]) Me[emax] = SM2D_RD_C(1.0);
        else {
            int e = 0;
            while (e < emax - 1 && Em < cen[e + 1]) ++e;
            const sm2d_rd_t fh = (Em - cen[e + 1]) / (cen[e] - cen[e + 1]);
            Me[e] = fh;
            Me[e + 1] = SM2D_RD_C(1.0) - fh;
        }
    } else {
        sm2d_rd_t P[SM2D_RD_NE], p[SM2D_RD_NE];
        for (int e = 0; e <= emax; ++e) {
            const sm2d_rd_t v = (cen[e] - Em) / sE;
            P[e] = sm2d_rd_Phi(v);
            p[e] = sm2d_rd_phi(v);
        }
        Me[0] = SM2D_RD_C(1.0) - P[0];
        Me[emax] = P[emax];
        for (int e = 0; e < emax; ++e) {
            /* E' in [cen[e+1], cen[e]]: share (E' - cen[e+1]) / width to e */
            const sm2d_rd_t prob = P[e] - P[e + 1];
            const sm2d_rd_t wid = cen[e] - cen[e + 1];
            sm2d_rd_t up = ((Em - cen[e + 1]) * prob + sE * (p[e + 1] - p[e])) / wid;
            up = up < SM2D_RD_C(0.0) ? SM2D_RD_C(0.0) : (up > prob ? prob : up);
            Me[e] = Me[e] + up;
            Me[e + 1] = Me[e + 1] + (prob - up);
        }
        int em = 0;
        for (int e = 0; e <= emax; ++e) {
            if (Me[e] < SM2D_RD_C(0.0)) Me[e] = SM2D_RD_C(0.0);
            if (Me[e] > Me[em]) em = e;
        }
        /* the rounding of the sums lands on the largest mass */
        sm2d_rd_t off = SM2D_RD_C(0.0);
        for (int e = 0; e <= emax; ++e)
            if (e != em) off = off + Me[e];
        Me[em] = SM2D_RD_C(1.0) - off;
    }
    sm2d_rd_t Er = SM2D_RD_C(0.0);
    for (int e = 0; e <= emax; ++e) Er = Er + Me[e] * cen[e];
    return Er;
}

/* light angular parts (w * mass < minw) fold into the centre angle; the
 * energy masses are never folded (a light component whose lower energy
 * share folded into its current bin would keep its energy step after step
 * and never stop); returns the represented energy */
SM2D_MF sm2d_rd_t sm2d_rd_fold(sm2d_rd_t w, sm2d_rd_t minw, sm2d_rd_t* Mt, sm2d_rd_t* Me, const sm2d_rd_t* cen,
                               int emax) {
    for (int t = 1; t < SM2D_RD_NT; ++t)
        if (Mt[t] > SM2D_RD_C(0.0) && w * Mt[t] < minw) {
            Mt[0] = Mt[0] + Mt[t];
            Mt[t] = SM2D_RD_C(0.0);
        }
    sm2d_rd_t Er = SM2D_RD_C(0.0);
    for (int e = 0; e <= emax; ++e) Er = Er + Me[e] * cen[e];
    return Er;
}

/* child k = 0..14 of an energy offset: angular distance and side
 * (k = 0: c; 2t - 1: c - t; 2t: c + t) */
SM2D_MF int sm2d_rd_kid_t(int k) { return (k + 1) >> 1; }
SM2D_MF int sm2d_rd_kid_side(int k) { return k == 0 ? 0 : ((k & 1) ? -1 : 1); }
/* the weight of child k of energy offset e of a component of weight w */
SM2D_MF sm2d_rd_t sm2d_rd_kid_w(sm2d_rd_t w, const sm2d_rd_t* Mt, const sm2d_rd_t* Me, int k, int e) {
    const int t = sm2d_rd_kid_t(k);
    const sm2d_rd_t mt = t == 0 ? Mt[0] : Mt[t] * SM2D_RD_C(0.5);
    return (w * mt) * Me[e];
}
