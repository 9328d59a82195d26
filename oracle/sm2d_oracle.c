/*
 * sm2d_oracle.c -- CPU oracle (test infrastructure) for the SM_2D K1..K6
 * transport step.  See sm2d_oracle.h for the scope and the pinning.
 *
 * Reference files are cited by their path inside the SM_2D project.  The
 * float build reproduces the reference arithmetic order (no FMA contraction:
 * build with -ffp-contract=off) and takes exp/log/sin/cos/erf of the
 * transport physics from the library's sm2d_math.h, the functions the CUDA
 * kernels call, so that its per-bin results equal the kernels' bit for bit
 * (host-side tables keep the C library, as the reference's host code does);
 * the double build (-DORC_FP64) evaluates the same method in FP64.
 */
#include "sm2d_oracle.h"
#include "sm2d_math.h"
#ifdef ORC_FP64
#define SM2D_RD_DOUBLE
#endif
#include "sm2d_redist.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#ifdef ORC_FP64
#define RL(x) (x)
#define r_log log
#define r_exp exp
#define r_sqrt sqrt
#define r_cos cos
#define r_sin sin
#define r_erf erf
#define r_fabs fabs
#define r_floor floor
#define r_ceil ceil
#define r_max fmax
#define r_min fmin
#else
#define RL(x) (x##f)
#define r_log sm2d_logf
#define r_exp sm2d_expf
#define r_sqrt sqrtf
#define r_cos sm2d_cosf
#define r_sin sm2d_sinf
#define r_erf sm2d_erff
#define r_fabs fabsf
#define r_floor floorf
#define r_ceil ceilf
#define r_max fmaxf
#define r_min fminf
#endif

typedef orc_real real;

/* ------------------------------------------------------------------------- */
/* constants                                                                  */
/* ------------------------------------------------------------------------- */
/* device_physics.cuh:38-42 */
#define M_P_MEV RL(938.272)
#define M_E_MEV RL(0.511)
#define X0_WATER RL(360.8)
#define K_VAV RL(0.307)
#define Z_A_WATER RL(0.555)
/* k3_finetransport.cu:37-41, 56-58 */
#define E_CUTOFF RL(0.1)
#define K3_PRUNE RL(1e-15)
#define K2_PRUNE RL(1e-12)          /* k2_coarsetransport.cu:50 */
#define BOUNDARY_SAFETY RL(1.001)
#define SEED_A 2654435761u
#define SEED_B 2246822519u
#define SEED_C 3266489917u
/* k2_coarsetransport.cu:54-56 */
#define UNRES_BASE RL(0.04)
#define UNRES_SLOPE RL(0.003)
#define UNRES_MAX RL(0.35)
/* K3 in-transport lateral sigma (k3_finetransport.cu:353) */
#define K3_SIGMA_TRANSPORT RL(0.001)
#define SPREAD_CELLS 11

enum { FACE_ZP = 0, FACE_ZM = 1, FACE_XP = 2, FACE_XM = 3 };

/* ------------------------------------------------------------------------- */
/* context                                                                    */
/* ------------------------------------------------------------------------- */
typedef struct bucket {           /* DeviceOutflowBucket, device_bucket.cuh:48-57 */
    uint32_t* bid;                /* [Kb] (the reference: 32 = DEVICE_Kb_out) */
    uint16_t* count;              /* [Kb] */
    real* val;                    /* [Kb * L] */
} bucket;

typedef struct rlut {             /* DeviceRLUT, device_lut.cuh:16-26 */
    int N;
    float Emin, Emax;
    real *R, *S, *logE, *logR, *logS;
    const real* edges;
    int precise;                  /* precision form: invert in double below R_prec = R(10 MeV) */
    real R_prec;
} rlut;

typedef struct psi_buf {
    uint32_t* bid;                /* [Nc*Kb] */
    real* val;                    /* [Nc*Kb*L] */
    uint8_t* occ;                 /* per cell: any slot claimed */
} psi_buf;

struct orc_ctx {
    orc_config cfg;
    int L, Nc, Kb;
    int N_theta, N_E;
    real* th_edges;               /* [N_theta+1] */
    real* E_edges;                /* [N_E+1] */
    rlut lut;
    float *fe_A, *fe_B, *fe_sigma;
    /* density of each depth row (slab phantom; NULL: water) and the
     * water-equivalent depth of each row's upper face */
    float *rho, *wet;
    psi_buf buf[2];
    int in_idx;                   /* which buffer is psi_in */
    uint8_t *mask, *mask_prev;
    uint32_t *active, *coarse;
    int n_active, n_coarse;
    /* cumulative tallies (K1K6PipelineState, k1k6_pipeline.cuh:174-188) */
    double *edep, *e_cut, *e_nuc, *e_bnd;
    float *w_cut, *w_nuc, *w_bnd;
    double *p_edep, *p_e_cut, *p_e_nuc, *p_e_bnd;
    float *p_w_cut, *p_w_nuc, *p_w_bnd;
    float *dw_cut, *dw_nuc, *dw_bnd;   /* this iteration's weight increments (precision form) */
    /* bucket scratch for the current batch */
    bucket* buckets;
    int n_buckets_cap;
    int* cell_to_bucket;          /* [Nc], -1 when not in batch */
    /* drop counters of the current iteration (k2/k3/k4 __device__ symbols) */
    double k2_slot_w, k2_slot_e, k2_bkt_w, k2_bkt_e, k2_prune_w, k2_prune_e;
    double k3_slot_w, k3_slot_e, k3_bkt_w, k3_bkt_e, k3_prune_w, k3_prune_e;
    double k4_slot_w, k4_slot_e;
    /* the same, summed over the iterations since create: [K2, K3, K4][slot, bucket, prune] */
    double cum_drop_w[3][3], cum_drop_e[3][3];
    /* run state */
    double transport_drop_w, transport_drop_e, audit_residual;
    float src_inj_w, src_oog_w, src_slot_w;
    double src_inj_e, src_oog_e, src_slot_e, src_rep_loss;
    int iter;
    int finished;
    double cell_steps, slots_in, slots_out;
    orc_audit audit;
    /* claim-demand diagnostic (off unless orc_track_claims enabled it):
     * distinct block ids aimed at each container (psi_out cell or bucket)
     * within one iteration, and the largest such count seen */
    int track_claims;
    struct claim_key { const uint32_t* ids; uint32_t want; } *ck;
    struct claim_cnt { const uint32_t* ids; int n; } *cc;
    size_t ck_cap, cc_cap, ck_n, cc_n;
    int claim_demand_max, claim_batch;
    /* the learned surrogate's network (orc_set_surrogate), NULL: none */
    struct orc_net* net;
};

static inline psi_buf* psi_in(orc_ctx* c) { return &c->buf[c->in_idx]; }
static inline psi_buf* psi_out(orc_ctx* c) { return &c->buf[1 - c->in_idx]; }

/* ------------------------------------------------------------------------- */
/* encodings: block_encoding.hpp:21-30, local_bins.hpp:62-146                */
/* ------------------------------------------------------------------------- */
static inline uint32_t enc_block(uint32_t b_theta, uint32_t b_E) {
    return (b_theta & 0xFFFu) | ((b_E & 0xFFFu) << 12);
}
static inline int enc_lidx(const orc_ctx* c, int t, int e, int x, int z) {
    return t + c->cfg.nt_local * (e + c->cfg.ne_local * (x + c->cfg.nx_sub * z));
}
static inline void dec_lidx(const orc_ctx* c, int l, int* t, int* e, int* x, int* z) {
    *t = l % c->cfg.nt_local;
    int r = l / c->cfg.nt_local;
    *e = r % c->cfg.ne_local;
    r /= c->cfg.ne_local;
    *x = r % c->cfg.nx_sub;
    *z = r / c->cfg.nx_sub;
}
/* sub-cell centre offsets; for 8 x-bins this is dx*(-0.4375+0.125*x), for
 * 4 z-bins dz*(-0.375+0.25*z) -- identical values in float (all exact). */
static inline real sub_offset(int s, int n, real d) {
    return d * ((RL(0.5) + (real)s) / (real)n - RL(0.5));
}
static inline int sub_bin(real off, real d, int n) {
    real norm = (off / d) + RL(0.5);
    int b = (int)(norm * (real)n);
    if (b < 0) b = 0;
    if (b >= n) b = n - 1;
    return b;
}

/* ------------------------------------------------------------------------- */
/* grids: grids.cpp:6-149                                                    */
/* ------------------------------------------------------------------------- */
int orc_energy_grid_log(float E_min, float E_max, int N, float* edges, float* rep) {
    float lmin = logf(E_min), lmax = logf(E_max);
    float d = (lmax - lmin) / N;
    for (int i = 0; i <= N; ++i) edges[i] = expf(lmin + i * d);
    for (int i = 0; i < N; ++i) rep[i] = sqrtf(edges[i] * edges[i + 1]);
    return N;
}

int orc_energy_grid_piecewise(int ng, const float* g, float* edges, float* rep) {
    int total = 0;
    for (int k = 0; k < ng; ++k) total += (int)((g[3 * k + 1] - g[3 * k]) / g[3 * k + 2] + 0.5f);
    if (!edges) return total;
    int off = 0;
    for (int k = 0; k < ng; ++k) {
        float a = g[3 * k], b = g[3 * k + 1], res = g[3 * k + 2];
        int n = (int)((b - a) / res + 0.5f);
        for (int i = 0; i <= n; ++i) edges[off + i] = a + i * res;
        for (int i = 0; i < n; ++i) rep[off + i] = sqrtf(edges[off + i] * edges[off + i + 1]);
        off += n;
    }
    edges[total] = g[3 * (ng - 1) + 1];
    return total;
}

void orc_angular_grid(float th_min, float th_max, int N, float* edges, float* rep) {
    float d = (th_max - th_min) / N;
    for (int i = 0; i <= N; ++i) edges[i] = th_min + i * d;
    for (int i = 0; i < N; ++i) rep[i] = 0.5f * (edges[i] + edges[i + 1]);
}

/* ------------------------------------------------------------------------- */
/* PSTAR water table (public NIST data; nist_loader.cpp:26-46 and           */
/* src/data/nist/pstar_water.txt hold the same 19 rows)                      */
/* ------------------------------------------------------------------------- */
static const float PSTAR[19][3] = {
    {0.001f, 133.7f, 0.000006319f}, {0.01f, 422.9f, 0.00003599f}, {0.1f, 814.5f, 0.0001607f},
    {0.5f, 412.8f, 0.0008869f},     {1.0f, 260.6f, 0.002458f},    {2.0f, 158.6f, 0.007555f},
    {5.0f, 79.11f, 0.03623f},       {10.0f, 45.64f, 0.1230f},     {20.0f, 26.05f, 0.4260f},
    {30.0f, 18.76f, 0.8853f},       {50.0f, 12.45f, 2.227f},      {70.0f, 9.555f, 4.080f},
    {80.0f, 8.622f, 5.184f},        {90.0f, 7.884f, 6.398f},      {100.0f, 7.286f, 7.718f},
    {150.0f, 5.443f, 15.77f},       {200.0f, 4.491f, 25.96f},     {250.0f, 3.910f, 37.94f},
    {300.0f, 3.519f, 51.45f}};

/* GenerateRLUT(grid), r_lut.cpp:69-129 (always float, like the host code) */
void orc_generate_rlut(int N_E, const float* rep, float* R, float* S,
                       float* logE, float* logR, float* logS) {
    const float to_mm = 10.0f / 1.0f;
    for (int i = 0; i < N_E; ++i) {
        float E = rep[i];
        int it = 0;                        /* lower_bound on energy */
        while (it < 19 && PSTAR[it][0] < E) ++it;
        if (it == 0) {
            R[i] = PSTAR[0][2] * to_mm;
            S[i] = PSTAR[0][1];
        } else if (it == 19) {
            R[i] = PSTAR[18][2] * to_mm;
            S[i] = PSTAR[18][1];
        } else {
            float E0 = PSTAR[it - 1][0], E1 = PSTAR[it][0];
            float R0 = PSTAR[it - 1][2] * to_mm, R1 = PSTAR[it][2] * to_mm;
            float S0 = PSTAR[it - 1][1], S1 = PSTAR[it][1];
            float lr = logf(R0) + (logf(R1) - logf(R0)) * (logf(E) - logf(E0)) / (logf(E1) - logf(E0));
            R[i] = expf(lr);
            float ls = logf(S0) + (logf(S1) - logf(S0)) * (logf(E) - logf(E0)) / (logf(E1) - logf(E0));
            S[i] = expf(ls);
        }
        logE[i] = logf(rep[i]);
        logR[i] = logf(R[i]);
        logS[i] = logf(S[i]);
    }
}

/* host-side LUT (RLUT::lookup_*, r_lut.cpp:131-204) used by the FE precompute */
typedef struct hlut {
    int N;
    float Emin, Emax;
    float edges[257], rep[256], R[256], S[256], logE[256], logR[256], logS[256];
} hlut;

static int host_find_bin(const hlut* h, float E) {     /* grids.cpp:99-113 */
    if (E < h->edges[0]) return 0;
    if (E >= h->edges[h->N]) return h->N - 1;
    int lo = 0, hi = h->N;
    while (lo < hi) {
        int mid = (lo + hi) / 2;
        if (h->edges[mid + 1] <= E) lo = mid + 1; else hi = mid;
    }
    return lo;
}
static float host_lookup_R(const hlut* h, float E) {
    float Ec = fmaxf(h->Emin, fminf(E, h->Emax));
    int b = host_find_bin(h, Ec);
    if (b == h->N - 1 || Ec >= h->Emax) return h->R[h->N - 1];
    float le = logf(Ec);
    float lr = h->logR[b] + (h->logR[b + 1] - h->logR[b]) * (le - h->logE[b]) / (h->logE[b + 1] - h->logE[b]);
    return expf(lr);
}
static float host_lookup_E_inverse(const hlut* h, float Rin) {
    if (Rin <= 0.0f) return h->Emin;
    if (Rin >= h->R[h->N - 1]) return h->Emax;
    if (Rin <= h->R[0]) return h->Emin;
    int it = 0;
    while (it < h->N && h->R[it] < Rin) ++it;     /* lower_bound */
    int b = it;
    if (b > h->N - 2) b = h->N - 2;
    if (b < 0) b = 0;
    float lr = logf(Rin);
    float dlr = h->logR[b + 1] - h->logR[b];
    if (fabsf(dlr) < 1e-10f) return expf(h->logE[b]);
    float le = h->logE[b] + (h->logE[b + 1] - h->logE[b]) * (lr - h->logR[b]) / dlr;
    return expf(le);
}
/* step_control.hpp:81-92 */
static float host_energy_deposition(const hlut* h, float E, float step) {
    float Rn = host_lookup_R(h, E) - step;
    float En = (Rn <= 0.0f) ? 0.0f : host_lookup_E_inverse(h, Rn);
    return E - En;
}
/* highland_sigma, highland.hpp:59-80 (host) == device_physics.cuh:50-71 */
static float highland_f(float E, float ds) {
    float gamma = (E + 938.272f) / 938.272f;
    float beta = sqrtf(fmaxf(1.0f - 1.0f / (gamma * gamma), 0.0f));
    float p = sqrtf(fmaxf((E + 938.272f) * (E + 938.272f) - 938.272f * 938.272f, 0.0f));
    float t = ds / 360.8f;
    if (t < 1e-6f) return 0.0f;
    float br = 1.0f + 0.038f * logf(t);
    br = fmaxf(br, 0.25f);
    return (13.6f * 1.0f / (beta * p)) * sqrtf(t) * br;
}

/* Fermi-Eyges precompute of A(z), B(z), sigma_total(z): k1k6_pipeline.cu:1061-1176.
 * With a density per row (rho, NULL: water) each row's energy loss and
 * scattering thickness are its water-equivalent path rho dz. */
void orc_fe_precompute_density(float E0, int Nz, float dz, float sx0, const float* rho, float* A, float* B,
                               float* sig) {
    for (int i = 0; i < Nz; ++i) { A[i] = 0.0f; B[i] = 0.0f; sig[i] = sx0; }
    if (!(E0 > 0.0f)) {
        for (int i = 0; i < Nz; ++i) sig[i] = 0.0f;
        return;
    }
    static hlut h;                     /* GenerateRLUT(0.1, 300, 256) */
    static int h_ready = 0;
    if (!h_ready) {
        h.N = 256; h.Emin = 0.1f; h.Emax = 300.0f;
        orc_energy_grid_log(0.1f, 300.0f, 256, h.edges, h.rep);
        orc_generate_rlut(256, h.rep, h.R, h.S, h.logE, h.logR, h.logS);
        h_ready = 1;
    }
    float Ec = E0, Aa = 0.0f, Ba = 0.0f;
    for (int iz = 0; iz < Nz; ++iz) {
        A[iz] = Aa;
        B[iz] = Ba;
        if (Ec <= 0.5f) break;
        const float rw = (rho ? rho[iz] : 1.0f) * dz;
        float dE = host_energy_deposition(&h, Ec, rw);
        dE = fminf(dE, Ec - 0.1f);
        float Em = Ec - 0.5f * dE;
        if (Em < 0.5f) Em = 0.5f;
        float s = highland_f(Em, rw);
        float T = s * s / dz;
        float Ao = Aa;
        Aa = Ao + T * dz;
        Ba = Ba + Ao * dz + 0.5f * T * dz * dz;
        Ec -= dE;
        if (Ec < 0.1f) Ec = 0.1f;
    }
    /* sigma_total: the corrected second pass (k1k6_pipeline.cu:1149-1176) */
    float Et = E0, At = 0.0f, Bt = 0.0f, C = sx0 * sx0;
    for (int iz = 0; iz < Nz; ++iz) {
        sig[iz] = sqrtf(fmaxf(0.0f, C));
        if (Et <= 0.5f) {
            for (int j = iz + 1; j < Nz; ++j) sig[j] = sig[iz];
            break;
        }
        const float rw = (rho ? rho[iz] : 1.0f) * dz;
        float dE = host_energy_deposition(&h, Et, rw);
        dE = fminf(dE, Et - 0.1f);
        float Em = fmaxf(0.5f, Et - 0.5f * dE);
        float s = highland_f(Em, rw);
        float T = s * s / dz;
        float dC = 2.0f * Bt * dz + At * dz * dz + T * dz * dz * dz / 3.0f;
        C += dC;
        float Ao = At;
        At = Ao + T * dz;
        Bt = Bt + Ao * dz + 0.5f * T * dz * dz;
        Et -= dE;
        if (Et < 0.1f) Et = 0.1f;
    }
}

void orc_fe_precompute(float E0, int Nz, float dz, float sx0, float* A, float* B, float* sig) {
    orc_fe_precompute_density(E0, Nz, dz, sx0, NULL, A, B, sig);
}

/* Post-process lateral convolution: gpu_transport_wrapper.cu:551-616 */
void orc_postprocess(const double* in, const float* sig, float sx0, int Nx, int Nz, float dx, double* out) {
    memcpy(out, in, sizeof(double) * (size_t)Nx * Nz);
    double* row = (double*)malloc(sizeof(double) * Nx);
    double* ker = (double*)malloc(sizeof(double) * (Nx + 1));
    float s0sq = sx0 * sx0;
    for (int iz = 0; iz < Nz; ++iz) {
        float st = sig[iz];
        float msq = st * st - s0sq;
        if (msq <= 1e-6f) continue;
        float sm = sqrtf(msq);
        float sc = sm / dx;
        int hk = (int)ceilf(3.0f * sc);
        if (hk > Nx / 2) hk = Nx / 2;
        if (hk < 1) hk = 1;
        double ksum = 0.0;
        for (int k = -hk; k <= hk; ++k) {
            double v = exp(-0.5 * ((double)k * k) / ((double)sc * sc));
            ker[k + hk] = v;
            ksum += v;
        }
        for (int k = 0; k < 2 * hk + 1; ++k) ker[k] /= ksum;
        for (int ix = 0; ix < Nx; ++ix) row[ix] = out[(size_t)iz * Nx + ix];
        for (int ix = 0; ix < Nx; ++ix) {
            double acc = 0.0;
            for (int k = -hk; k <= hk; ++k) {
                int j = ix + k;
                if (j >= 0 && j < Nx) acc += row[j] * ker[k + hk];
            }
            out[(size_t)iz * Nx + ix] = acc;
        }
    }
    free(row);
    free(ker);
}

/* ------------------------------------------------------------------------- */
/* device LUT lookups: device_lut.cuh:34-214                                 */
/* ------------------------------------------------------------------------- */
static inline int find_bin_edges(const real* e, int N, real E) {
    if (E <= e[0]) return 0;
    if (E >= e[N]) return N - 1;
    int lo = 0, hi = N;
    while (lo < hi) {
        int mid = (lo + hi) / 2;
        if (e[mid + 1] <= E) lo = mid + 1; else hi = mid;
    }
    return lo;
}
static real lut_R(const rlut* l, real E) {
    real Ec = r_max((real)l->Emin, r_min(E, (real)l->Emax));
    int b = find_bin_edges(l->edges, l->N, Ec);
    if (b == l->N - 1 || Ec >= (real)l->Emax) return l->R[l->N - 1];
    real le = r_log(Ec);
    real lr = l->logR[b] + (l->logR[b + 1] - l->logR[b]) * (le - l->logE[b]) / (l->logE[b + 1] - l->logE[b]);
    return r_exp(lr);
}
static real lut_E_inverse(const rlut* l, real Rin) {
    if (Rin <= RL(0.0)) return (real)l->Emin;
    int lo = 0, hi = l->N;
    while (lo < hi) {
        int mid = (lo + hi) / 2;
        if (l->R[mid] < Rin) lo = mid + 1; else hi = mid;
    }
    int b = lo;
    if (b > l->N - 2) b = l->N - 2;
    if (b < 0) b = 0;
    if (l->precise && Rin < l->R_prec) {   /* precision form: the interpolation in double */
        const double dl = (double)l->logR[b + 1] - (double)l->logR[b];
        if (fabs(dl) < 1e-10) return (real)(float)exp((double)l->logE[b]);
        const double le = (double)l->logE[b] +
                          ((double)l->logE[b + 1] - (double)l->logE[b]) * (log((double)Rin) - (double)l->logR[b]) / dl;
        return (real)(float)exp(le);
    }
    real lr = r_log(Rin);
    real dlr = l->logR[b + 1] - l->logR[b];
    if (r_fabs(dlr) < RL(1e-10)) return r_exp(l->logE[b]);
    real le = l->logE[b] + (l->logE[b + 1] - l->logE[b]) * (lr - l->logR[b]) / dlr;
    return r_exp(le);
}
static real lut_energy_deposition(const rlut* l, real E, real step) {
    real Rn = lut_R(l, E) - step;
    real En = (Rn <= 0) ? (real)l->Emin : lut_E_inverse(l, Rn);
    return E - En;
}
static real max_step(const rlut* l, real E) {
    real R = lut_R(l, E);
    real d = RL(0.01) * R;
    real smin;
    if (E < RL(2.0)) smin = RL(0.1);
    else if (E < RL(20.0)) smin = RL(0.25);
    else if (E < RL(100.0)) smin = RL(0.5);
    else smin = RL(1.0);
    d = r_max(d, smin);
    if (E < RL(0.5)) d = r_min(d, RL(0.05));
    else if (E < RL(5.0)) d = r_min(d, RL(0.2));
    else if (E < RL(20.0)) d = r_min(d, RL(0.5));
    return d;
}

/* ------------------------------------------------------------------------- */
/* physics: device_physics.cuh:50-437                                        */
/* ------------------------------------------------------------------------- */
static real highland(real E, real ds) {
    real gamma = (E + M_P_MEV) / M_P_MEV;
    real beta2 = RL(1.0) - RL(1.0) / (gamma * gamma);
    real beta = r_sqrt(r_max(beta2, RL(0.0)));
    real p = r_sqrt(r_max((E + M_P_MEV) * (E + M_P_MEV) - M_P_MEV * M_P_MEV, RL(0.0)));
    real t = ds / X0_WATER;
    if (t < RL(1e-6)) return RL(0.0);
    real br = RL(1.0) + RL(0.038) * r_log(t);
    br = r_max(br, RL(0.25));
    return (RL(13.6) * RL(1.0) / (beta * p)) * r_sqrt(t) * br;
}
static real gauss_sample(unsigned* seed) {
    *seed = 1664525u * *seed + 1013904223u;
    real u1 = (real)(*seed >> 16) / RL(65536.0);
    *seed = 1664525u * *seed + 1013904223u;
    real u2 = (real)(*seed >> 16) / RL(65536.0);
    u1 = r_max(u1, RL(1e-6));
    return r_sqrt(RL(-2.0) * r_log(u1)) * r_cos(RL(2.0) * (real)3.14159265358979323846f * u2);
}
static real vav_xi(real beta, real rho, real ds_cm) {
    return (K_VAV / RL(2.0)) * Z_A_WATER * (RL(1.0) * RL(1.0) / (beta * beta)) * rho * ds_cm;
}
static real bohr_sigma(real E, real ds, real rho) {
    real gamma = (E + M_P_MEV) / M_P_MEV;
    real beta2 = RL(1.0) - RL(1.0) / (gamma * gamma);
    real beta = r_sqrt(r_max(beta2, RL(0.01)));
    return RL(0.156) * r_sqrt(rho * ds) / beta;
}
static real straggling_sigma(real E, real ds, real rho) {
    real gamma = (E + M_P_MEV) / M_P_MEV;
    real beta2 = RL(1.0) - RL(1.0) / (gamma * gamma);
    real beta = r_sqrt(r_max(beta2, RL(0.0)));
    real ds_cm = ds / RL(10.0);
    real xi = vav_xi(beta, rho, ds_cm);
    real mr = M_E_MEV / M_P_MEV;
    real num = RL(2.0) * M_E_MEV * beta * beta * gamma * gamma;
    real den = RL(1.0) + RL(2.0) * gamma * mr + mr * mr;
    real tmax = num / r_max(den, RL(1e-10));
    real kappa = xi / r_max(tmax, RL(1e-10));
    kappa = r_max(kappa, RL(1e-6));
    if (kappa > RL(10.0)) return bohr_sigma(E, ds, rho);
    real g2 = (E + M_P_MEV) / M_P_MEV;
    real b2 = r_sqrt(r_max(RL(1.0) - RL(1.0) / (g2 * g2), RL(0.0)));
    real xi2 = vav_xi(b2, rho, ds / RL(10.0));
    real landau = RL(4.0) * xi2 / RL(2.355);
    if (kappa < RL(0.01)) return landau;
    real sb = bohr_sigma(E, ds, rho);
    real w = RL(1.0) / (RL(1.0) + kappa);
    return w * landau + (RL(1.0) - w) * sb;
}
static real nuclear_xs(real E) {
    if (E < RL(5.0)) return RL(0.0);
    if (E >= RL(20.0)) {
        real f = RL(1.0) - RL(0.15) * r_log(E / RL(100.0));
        return RL(0.0012) * r_max(f, RL(0.4));
    }
    return RL(0.0016) * ((E - RL(5.0)) / RL(15.0));
}
static real nuclear_atten(real w, real E, real step, real* w_rem, real* E_rem) {
    real s = nuclear_xs(E);
    real surv = r_exp(-s * step);
    real wn = w * surv;
    real wr = w - wn;
    *w_rem = wr;
    *E_rem = wr * E;
    return wn;
}
static real gcdf(real x, real mu, real sigma) {
    if (sigma < RL(1e-10)) return (x >= mu) ? RL(1.0) : RL(0.0);
    real arg = (x - mu) / sigma * RL(0.70710678);
    real cdf = RL(0.5) * (RL(1.0) + r_erf(arg));
    return r_min(RL(1.0), r_max(RL(0.0), cdf));
}
static void spread_weights(real* w, real xm, real sigma, real dx, int N) {
    sigma = r_max(sigma, RL(1e-6));
    real xmin = xm - RL(0.5) * (real)N * dx;
    real prev = gcdf(xmin, xm, sigma);
    for (int i = 0; i < N; ++i) {
        real xb = xmin + (real)(i + 1) * dx;
        real cur = gcdf(xb, xm, sigma);
        w[i] = cur - prev;
        prev = cur;
    }
    real s = 0;
    for (int i = 0; i < N; ++i) s += w[i];
    if (s > RL(1e-10)) {
        for (int i = 0; i < N; ++i) w[i] /= s;
    } else {
        for (int i = 0; i < N; ++i) w[i] = (i == N / 2) ? RL(1.0) : RL(0.0);
    }
}
static void spread_weights_subcell(real* w, real xm, real sigma, real dx, int N) {
    sigma = r_max(sigma, RL(1e-6));
    real dxs = dx / (real)N;
    real xmin = -dx * RL(0.5);
    real prev = gcdf(xmin, xm, sigma);
    for (int i = 0; i < N; ++i) {
        real xb = xmin + (real)(i + 1) * dxs;
        real cur = gcdf(xb, xm, sigma);
        w[i] = cur - prev;
        prev = cur;
    }
    real s = 0;
    for (int i = 0; i < N; ++i) s += w[i];
    if (s > RL(1e-10)) {
        for (int i = 0; i < N; ++i) w[i] /= s;
    } else {
        for (int i = 0; i < N; ++i) w[i] = (i == N / 2) ? RL(1.0) : RL(0.0);
    }
}
/* scattering power per geometric mm in a medium of density rho: Highland
 * angle of the water-equivalent thickness rho ds */
static real scattering_T(real E, real ds, real rho) {
    real th = highland(E, rho * ds);
    if (ds < RL(1e-6)) return RL(0.0);
    return th * th / ds;
}
static real rho_of(const orc_ctx* c, int iz) { return c->rho ? (real)c->rho[iz] : RL(1.0); }

/* ------------------------------------------------------------------------- */
/* slot tables: device_psic.cuh:163-292, device_bucket.cuh:61-128           */
/* ------------------------------------------------------------------------- */
static inline int bid_distance(uint32_t a, uint32_t b) {
    int ta = (int)(a & 0xFFFu), ea = (int)((a >> 12) & 0xFFFu);
    int tb = (int)(b & 0xFFFu), eb = (int)((b >> 12) & 0xFFFu);
    return abs(ea - eb) * 8 + abs(ta - tb);
}
/* find exact / claim empty / fall back to nearest occupied slot */
static int slot_with_fallback_n(uint32_t* ids, int n, int n_claim, uint32_t want, uint32_t* sel) {
    *sel = want;
    for (int s = 0; s < n; ++s) if (ids[s] == want) return s;
    for (int s = 0; s < n_claim; ++s) {
        if (ids[s] == ORC_EMPTY) { ids[s] = want; return s; }
        if (ids[s] == want) return s;
    }
    if (n_claim < 0) return -1;    /* light deposit of the split method: no merge */
    int best = -1, bd = 0x7fffffff;
    uint32_t bb = ORC_EMPTY;
    for (int s = 0; s < n; ++s) {
        if (ids[s] == ORC_EMPTY) continue;
        int d = bid_distance(ids[s], want);
        if (d < bd) { bd = d; best = s; bb = ids[s]; }
    }
    if (best >= 0) *sel = bb;
    return best;
}
static int remap_lidx(const orc_ctx* c, int l, uint32_t src, uint32_t dst) {
    if (src == dst) return l;
    int t, e, x, z;
    dec_lidx(c, l, &t, &e, &x, &z);
    int tg = (int)(src & 0xFFFu) * c->cfg.nt_local + t;
    int eg = (int)((src >> 12) & 0xFFFu) * c->cfg.ne_local + e;
    int td = tg - (int)(dst & 0xFFFu) * c->cfg.nt_local;
    int ed = eg - (int)((dst >> 12) & 0xFFFu) * c->cfg.ne_local;
    if (td < 0) td = 0;
    if (td > c->cfg.nt_local - 1) td = c->cfg.nt_local - 1;
    if (ed < 0) ed = 0;
    if (ed > c->cfg.ne_local - 1) ed = c->cfg.ne_local - 1;
    return enc_lidx(c, td, ed, x, z);
}
static int slot_with_fallback(uint32_t* ids, int n, uint32_t want, uint32_t* sel) {
    return slot_with_fallback_n(ids, n, n, want, sel);
}
/* ---- claim-demand diagnostic: open-addressing sets, cleared per iteration */
static size_t ck_hash(const void* p, uint32_t w) {
    uint64_t h = (uint64_t)(uintptr_t)p * 0x9E3779B97F4A7C15ull ^ (uint64_t)w * 0xC2B2AE3D27D4EB4Full;
    return (size_t)(h ^ (h >> 29));
}
static void claims_reset(orc_ctx* c) {
    if (c->ck) memset(c->ck, 0, sizeof(*c->ck) * c->ck_cap);
    if (c->cc) memset(c->cc, 0, sizeof(*c->cc) * c->cc_cap);
    c->ck_n = c->cc_n = 0;
}
static void claims_grow(orc_ctx* c) {
    size_t ncap = c->ck_cap ? 2 * c->ck_cap : (1u << 16);
    struct claim_key* old = c->ck;
    size_t ocap = c->ck_cap;
    c->ck = calloc(ncap, sizeof(*c->ck));
    c->ck_cap = ncap;
    for (size_t i = 0; i < ocap; ++i)
        if (old[i].ids) {
            size_t h = ck_hash(old[i].ids, old[i].want) & (ncap - 1);
            while (c->ck[h].ids) h = (h + 1) & (ncap - 1);
            c->ck[h] = old[i];
        }
    free(old);
    struct claim_cnt* oc = c->cc;
    size_t occ = c->cc_cap;
    c->cc = calloc(ncap, sizeof(*c->cc));
    c->cc_cap = ncap;
    for (size_t i = 0; i < occ; ++i)
        if (oc[i].ids) {
            size_t h = ck_hash(oc[i].ids, 0) & (ncap - 1);
            while (c->cc[h].ids) h = (h + 1) & (ncap - 1);
            c->cc[h] = oc[i];
        }
    free(oc);
}
static void claims_note(orc_ctx* c, const uint32_t* ids, uint32_t want) {
    if (!c->track_claims) return;
    /* a bucket's storage is reused by the next batch of the iteration: key
     * bucket claims by batch as well */
    const psi_buf* po = &c->buf[1 - c->in_idx];
    if (ids < po->bid || ids >= po->bid + (size_t)c->Nc * c->Kb)
        ids = (const uint32_t*)((uintptr_t)ids ^ ((uintptr_t)c->claim_batch << 56));
    if (2 * (c->ck_n + 1) > c->ck_cap) claims_grow(c);
    size_t m = c->ck_cap - 1, h = ck_hash(ids, want) & m;
    while (c->ck[h].ids) {
        if (c->ck[h].ids == ids && c->ck[h].want == want) return;
        h = (h + 1) & m;
    }
    c->ck[h].ids = ids;
    c->ck[h].want = want;
    c->ck_n++;
    h = ck_hash(ids, 0) & m;
    while (c->cc[h].ids && c->cc[h].ids != ids) h = (h + 1) & m;
    if (!c->cc[h].ids) { c->cc[h].ids = ids; c->cc_n++; }
    if (++c->cc[h].n > c->claim_demand_max) c->claim_demand_max = c->cc[h].n;
}
void orc_track_claims(orc_ctx* c, int on) { c->track_claims = on; }
/* the expectation form's masses (sm2d_redist.h) in this build's precision */
void orc_redist_masses(double s, double Em, double sE, const double* cen, int emax, double* Mt, double* Me) {
    real c4[SM2D_RD_NE] = {0}, mt[SM2D_RD_NT], me[SM2D_RD_NE];
    for (int e = 0; e <= emax && e < SM2D_RD_NE; ++e) c4[e] = (real)cen[e];
    sm2d_rd_theta((real)s, mt);
    sm2d_rd_energy((real)Em, (real)sE, c4, emax, me);
    for (int t = 0; t < SM2D_RD_NT; ++t) Mt[t] = (double)mt[t];
    for (int e = 0; e < SM2D_RD_NE; ++e) Me[e] = (double)me[e];
}
int orc_claim_demand(const orc_ctx* c) { return c->claim_demand_max; }

/* number of slots a deposit of weight w may claim */
static inline int claimable(const orc_ctx* c, int n, double w) {
    return (c->cfg.claim_reserve_weight > 0.0f && w < (double)c->cfg.claim_reserve_weight) ? n - 8 : n;
}
/* slot claim of a deposit of weight w: light deposits of the split method
 * claim among the first 24 slots and are dropped (not merged) when those
 * are taken; heavy ones use all 32 and the nearest-block fallback */
static int claim_w(const orc_ctx* c, uint32_t* ids, int n, uint32_t want, uint32_t* sel, double w) {
    claims_note((orc_ctx*)c, ids, want);
    int nc = claimable(c, n, w);
    if (nc < n) {
        *sel = want;
        for (int s = 0; s < n; ++s) if (ids[s] == want) return s;
        for (int s = 0; s < nc; ++s) {
            if (ids[s] == ORC_EMPTY) { ids[s] = want; return s; }
            if (ids[s] == want) return s;
        }
        return -1;
    }
    return slot_with_fallback_n(ids, n, n, want, sel);
}
/* psi_out slot claim marks the cell occupied */
static int psi_slot(orc_ctx* c, psi_buf* p, int cell, uint32_t want, uint32_t* sel, double w) {
    int s = claim_w(c, &p->bid[(size_t)cell * c->Kb], c->Kb, want, sel, w);
    if (s >= 0) p->occ[cell] = 1;
    return s;
}

/* ------------------------------------------------------------------------- */
/* energy binning of an emitted component                                    */
/* ------------------------------------------------------------------------- */
typedef struct eparts { int n; int bin[2]; real frac[2]; real Erep; } eparts;

static inline real e_center(const orc_ctx* c, int b) {
    return c->E_edges[b] + RL(0.5) * (c->E_edges[b + 1] - c->E_edges[b]);
}
/* reference: one bin, the one containing E (device_find_bin_edges).
 * energy_split: mean-preserving split between the two neighbouring bin
 * centres (method extension needed on coarse log grids). */
static eparts bin_energy(const orc_ctx* c, real E, real w) {
    eparts p;
    int k = find_bin_edges(c->E_edges, c->N_E, E);
    p.n = 1; p.bin[0] = k; p.frac[0] = RL(1.0); p.bin[1] = k; p.frac[1] = RL(0.0);
    p.Erep = e_center(c, k);
    if (!c->cfg.energy_split) return p;
    real ck = e_center(c, k);
    int lo, hi;
    if (E >= ck) { lo = k; hi = k + 1; } else { lo = k - 1; hi = k; }
    if (lo < 0 || hi > c->N_E - 1) return p;
    real cl = e_center(c, lo), ch = e_center(c, hi);
    real fh = (E - cl) / (ch - cl);
    if (fh <= RL(0.0)) { p.bin[0] = lo; p.Erep = cl; return p; }
    if (fh >= RL(1.0)) { p.bin[0] = hi; p.Erep = ch; return p; }
    if (w * r_min(fh, RL(1.0) - fh) < (real)c->cfg.split_min_weight) {
        /* light minor part: keep the whole component in the nearer centre */
        if (fh >= RL(0.5)) { p.bin[0] = hi; p.Erep = ch; } else { p.bin[0] = lo; p.Erep = cl; }
        return p;
    }
    p.n = 2;
    p.bin[0] = lo; p.frac[0] = RL(1.0) - fh;
    p.bin[1] = hi; p.frac[1] = fh;
    p.Erep = p.frac[0] * cl + p.frac[1] * ch;
    return p;
}

/* expectation form: the children of one component (sm2d_redist.h); c and j
 * are its incoming angle and energy bins */
typedef struct kids {
    int c, j, emax;
    real Mt[SM2D_RD_NT], Me[SM2D_RD_NE];
    real Erep;
    int tab;                               /* 1: the weights are the table T */
    real T[SM2D_RD_NT * SM2D_RD_NE];       /* T[t + 8 e] */
} kids;
/* energy window: its top is the second centre above the step's mean energy
 * Em, at most the incoming bin jin */
static void make_kids(const orc_ctx* c, int tb, int jin, real s, real Em, real sE, real w, kids* k) {
    real Ec = r_max(c->E_edges[0], r_min(Em, c->E_edges[c->N_E]));
    int b = find_bin_edges(c->E_edges, c->N_E, Ec);
    int up = Ec >= e_center(c, b) ? b + 1 : b;
    int Eb = up + 1 < jin ? up + 1 : jin;
    k->c = tb;
    k->j = Eb;
    k->tab = 0;
    k->emax = Eb < SM2D_RD_NE - 1 ? Eb : SM2D_RD_NE - 1;
    real cen[SM2D_RD_NE];
    for (int e = 0; e <= k->emax; ++e) cen[e] = e_center(c, Eb - e);
    sm2d_rd_theta(s, k->Mt);
    sm2d_rd_energy(Em, sE, cen, k->emax, k->Me);
    k->Erep = sm2d_rd_fold(w, (real)c->cfg.split_min_weight, k->Mt, k->Me, cen, k->emax);
}
/* The surrogate's features of a component (the GPU's surr_features): s =
 * sigma_theta / dtheta; u, where Em lies between the centres around it; r =
 * sigma_E / their spacing; cap = 1 when the window's top is the incoming
 * bin.  0: outside the table's domain (a window of fewer than four centres or
 * of uneven spacing), which keeps the closed forms. */
static int surr_features(const orc_ctx* c, int jin, real s, real Em, real sE, real* f) {
    real Ec = r_max(c->E_edges[0], r_min(Em, c->E_edges[c->N_E]));
    int b = find_bin_edges(c->E_edges, c->N_E, Ec);
    int up = Ec >= e_center(c, b) ? b + 1 : b;
    int jt = up + 1 < jin ? up + 1 : jin;
    if (up < 1 || up > c->N_E - 1 || jt < SM2D_RD_NE - 1) return 0;
    real ch = e_center(c, up), cl = e_center(c, up - 1), D = ch - cl;
    for (int e = 0; e < SM2D_RD_NE - 1; ++e) {
        real de = e_center(c, jt - e) - e_center(c, jt - e - 1);
        if (r_fabs(de - D) > RL(1e-3) * D) return 0;
    }
    f[0] = s;
    f[1] = r_min(r_max((Em - cl) / D, RL(0.0)), (real)0.99999994f);
    f[2] = sE / D;
    f[3] = jt == up ? RL(1.0) : RL(0.0);
    return 1;
}
/* the plain table of a feature row (the GPU's plain_table) */
static void plain_table(const real* f, real* out) {
    const real cap1[4] = {RL(1.0), RL(0.0), RL(-1.0), RL(-2.0)}, cap0[4] = {RL(2.0), RL(1.0), RL(0.0), RL(-1.0)};
    real Mt[SM2D_RD_NT], Me[SM2D_RD_NE];
    sm2d_rd_theta(r_max(f[0], RL(0.0)), Mt);
    sm2d_rd_energy(f[1], r_max(f[2], RL(0.0)), f[3] > RL(0.5) ? cap1 : cap0, SM2D_RD_NE - 1, Me);
    for (int e = 0; e < SM2D_RD_NE; ++e)
        for (int t = 0; t < SM2D_RD_NT; ++t) out[t + 8 * e] = Mt[t] * Me[e];
}
/* children from a table row (the GPU's make_kids_t): the window is complete
 * (emax 3); as in the closed forms (sm2d_rd_fold), an angular distance whose
 * total mass over the energy offsets is light folds into the centre angle;
 * the represented energy counts each offset's whole mass */
static void make_kids_tab(const orc_ctx* c, int tb, int jin, real Em, real w, const real* row, kids* k) {
    real Ec = r_max(c->E_edges[0], r_min(Em, c->E_edges[c->N_E]));
    int b = find_bin_edges(c->E_edges, c->N_E, Ec);
    int up = Ec >= e_center(c, b) ? b + 1 : b;
    int j = up + 1 < jin ? up + 1 : jin;
    k->c = tb;
    k->j = j;
    k->tab = 1;
    k->emax = SM2D_RD_NE - 1;
    for (int i = 0; i < SM2D_RD_NT * SM2D_RD_NE; ++i) k->T[i] = r_max(row[i], RL(0.0));
    real Er = RL(0.0);
    for (int e = 0; e < SM2D_RD_NE; ++e) {
        real me = RL(0.0);
        for (int t = 0; t < SM2D_RD_NT; ++t) me = me + k->T[t + 8 * e];
        Er = Er + me * e_center(c, j - e);
    }
    k->Erep = Er;
    const real minw = (real)c->cfg.split_min_weight;
    for (int t = 1; t < SM2D_RD_NT; ++t) {
        real mt = RL(0.0);
        for (int e = 0; e < SM2D_RD_NE; ++e) mt = mt + k->T[t + 8 * e];
        if (mt > RL(0.0) && w * mt < minw) {
            for (int e = 0; e < SM2D_RD_NE; ++e) {
                k->T[8 * e] = k->T[8 * e] + k->T[t + 8 * e];
                k->T[t + 8 * e] = RL(0.0);
            }
        }
    }
}
/* The learned surrogate's network (sm2d_surrogate.cu) restated: 4 features
 * scaled to [-1, 1] as bf16 pairs (value, 128 x remainder), 16 -> 128 -> 128 ->
 * 32 with ReLU, every GEMM operand rounded to bf16 (the first layer's
 * remainder columns weighted by bf16(W1) / 128), sums in double; softmax,
 * weights below 2^-12 zero, the largest taking 1 - the others.  A row whose
 * calibrated region error exceeds the tolerance falls back to the closed
 * forms.  Parameter layout: W1[128][16] W2[128][128] W3[32][128] b1 b2 b3. */
typedef struct orc_net {
    float W1[128 * 16], W2[128 * 128], W3[32 * 128], b1[128], b2[128], b3[32];
    float region_err[4096];
    float tol;
    long long rows, fallback;   /* rows asked for, rows that fell back */
} orc_net;
static float bf16r(float x) {
    uint32_t u;
    memcpy(&u, &x, 4);
    u = ((u + 0x7FFFu + ((u >> 16) & 1u)) >> 16) << 16;
    float y;
    memcpy(&y, &u, 4);
    return y;
}
static int net_region(const float* f) {
    int ia = (int)(sqrtf(fmaxf(f[0], 0.0f) / 8.0f) * 16.0f), ib = (int)(f[1] * 16.0f);
    int ic = (int)(sqrtf(fmaxf(f[2], 0.0f) / 4.0f) * 8.0f), id = f[3] > 0.5f ? 1 : 0;
    ia = ia < 0 ? 0 : (ia > 15 ? 15 : ia);
    ib = ib < 0 ? 0 : (ib > 15 ? 15 : ib);
    ic = ic < 0 ? 0 : (ic > 7 ? 7 : ic);
    return ((ia * 16 + ib) * 8 + ic) * 2 + id;
}
/* 1: the network's table of feature row f into out[32]; 0: the row falls back */
static int net_table(orc_net* n, const real* fr, real* out) {
    float f[4] = {(float)fr[0], (float)fr[1], (float)fr[2], (float)fr[3]};
    n->rows++;
    if (n->region_err[net_region(f)] > n->tol) {
        n->fallback++;
        return 0;
    }
    const float s = fminf(fmaxf(f[0], 0.0f), 8.0f), r = fminf(fmaxf(f[2], 0.0f), 4.0f);
    const float u[4] = {2.0f * s / 8.0f - 1.0f, 2.0f * f[1] - 1.0f, 2.0f * r / 4.0f - 1.0f, 2.0f * f[3] - 1.0f};
    float x[16] = {0};
    for (int i = 0; i < 4; ++i) {
        x[i] = bf16r(u[i]);
        x[4 + i] = bf16r((u[i] - x[i]) * 128.0f);
    }
    float h1[128], h2[128];
    double z[32];
    for (int o = 0; o < 128; ++o) {
        double a = (double)n->b1[o];
        for (int i = 0; i < 4; ++i) {
            const float w = bf16r(n->W1[o * 16 + i]);
            a += (double)x[i] * w + (double)x[4 + i] * (double)(w / 128.0f);
        }
        h1[o] = bf16r((float)(a > 0.0 ? a : 0.0));
    }
    for (int o = 0; o < 128; ++o) {
        double a = (double)n->b2[o];
        for (int i = 0; i < 128; ++i) a += (double)h1[i] * bf16r(n->W2[o * 128 + i]);
        h2[o] = bf16r((float)(a > 0.0 ? a : 0.0));
    }
    double m = -1e300;
    int am = 0;
    for (int o = 0; o < 32; ++o) {
        double a = (double)n->b3[o];
        for (int i = 0; i < 128; ++i) a += (double)h2[i] * bf16r(n->W3[o * 128 + i]);
        z[o] = a;
        if (a > m) { m = a; am = o; }
    }
    double sum = 0.0, rest = 0.0;
    for (int o = 0; o < 32; ++o) { z[o] = exp(z[o] - m); sum += z[o]; }
    for (int o = 0; o < 32; ++o) {
        z[o] /= sum;
        if (z[o] < 1.0 / 4096.0) z[o] = 0.0;
        if (o != am) rest += z[o];
    }
    z[am] = 1.0 - rest;
    for (int o = 0; o < 32; ++o) out[o] = (real)z[o];
    return 1;
}
void orc_set_surrogate(orc_ctx* c, const float* params, const float* region_err, float tol) {
    free(c->net);
    c->net = NULL;
    if (!params) return;
    orc_net* n = (orc_net*)malloc(sizeof(orc_net));
    memcpy(n->W1, params, sizeof n->W1);
    memcpy(n->W2, params + 128 * 16, sizeof n->W2);
    memcpy(n->W3, params + 128 * 16 + 128 * 128, sizeof n->W3);
    memcpy(n->b1, params + 128 * 16 + 128 * 128 + 32 * 128, sizeof n->b1);
    memcpy(n->b2, params + 128 * 16 + 128 * 128 + 32 * 128 + 128, sizeof n->b2);
    memcpy(n->b3, params + 128 * 16 + 128 * 128 + 32 * 128 + 256, sizeof n->b3);
    memcpy(n->region_err, region_err, sizeof n->region_err);
    n->tol = tol;
    n->rows = n->fallback = 0;
    c->net = n;
}
void orc_surrogate_counts(const orc_ctx* c, long long* out2) {
    out2[0] = c->net ? c->net->rows : 0;
    out2[1] = c->net ? c->net->fallback : 0;
}
static inline int kid_live(const kids* k, int t, int e) {
    return k->tab ? k->T[t + 8 * e] > RL(0.0) : (k->Me[e] > RL(0.0) && k->Mt[t] > RL(0.0));
}
static inline real kid_weight(const kids* k, real w, int kk, int e) {
    if (!k->tab) return sm2d_rd_kid_w(w, k->Mt, k->Me, kk, e);
    const int t = sm2d_rd_kid_t(kk);
    const real m = k->T[t + 8 * e];
    return w * (t == 0 ? m : m * RL(0.5));
}
static inline int kid_tbin(const orc_ctx* c, const kids* k, int kk) {
    int tb = k->c + sm2d_rd_kid_side(kk) * sm2d_rd_kid_t(kk);
    if (tb < 0) tb = 0;
    if (tb > c->N_theta - 1) tb = c->N_theta - 1;
    return tb;
}

/* ------------------------------------------------------------------------- */
/* bucket emission: device_bucket.cuh:431-533 (4-D, theta 2-bin split)       */
/* ------------------------------------------------------------------------- */
/* energy-bin index of local bin l of block bid */
static inline int ebin_of(const orc_ctx* c, uint32_t bid, int l) {
    return (int)((bid >> 12) & 0xFFFu) * c->cfg.ne_local + (l / c->cfg.nt_local) % c->cfg.ne_local;
}
/* The split method keeps energy when a saturated slot table re-bins a part
 * into another block: the shift (intended - stored centre) * w goes to *eshift. */
/* the children of a component (expectation form), in child order */
static real emit_kids_to_bucket(orc_ctx* c, bucket* bk, const kids* kd, real weight, int xs, int zs, double* eshift) {
    if (weight <= RL(0.0)) return RL(0.0);
    real dropped = RL(0.0);
    for (int e = 0; e <= kd->emax; ++e) {
        int Eb = kd->j - e;
        int El = Eb % c->cfg.ne_local;
        uint32_t bE = (uint32_t)(Eb / c->cfg.ne_local);
        for (int k = 0; k < SM2D_RD_KIDS; ++k) {
            if (!kid_live(kd, sm2d_rd_kid_t(k), e)) continue;
            real wk = kid_weight(kd, weight, k, e);
            int tbin = kid_tbin(c, kd, k);
            uint32_t want = enc_block((uint32_t)(tbin / c->cfg.nt_local), bE);
            int l = enc_lidx(c, tbin % c->cfg.nt_local, El, xs, zs);
            uint32_t sel;
            int s = claim_w(c, bk->bid, c->Kb, want, &sel, (double)wk);
            if (s < 0) { dropped += wk; continue; }
            int le = (sel == want) ? l : remap_lidx(c, l, want, sel);
            if (sel != want && eshift) *eshift += (double)((e_center(c, Eb) - e_center(c, ebin_of(c, sel, le))) * wk);
            bk->val[(size_t)s * c->L + le] += wk;
            bk->count[s]++;
        }
    }
    return dropped;
}
static real emit_to_bucket(orc_ctx* c, bucket* bk, real theta, real E, real weight, int xs, int zs, double* eshift) {
    if (weight <= RL(0.0)) return RL(0.0);
    real tmin = c->th_edges[0], tmax = c->th_edges[c->N_theta];
    real dth = (tmax - tmin) / (real)c->N_theta;
    real tc = r_max(tmin, r_min(theta, tmax));
    real c0 = tmin + RL(0.5) * dth;
    real cont = (tc - c0) / dth;
    int bc = (int)r_floor(cont + RL(0.5));
    if (bc < 0) bc = 0;
    if (bc > c->N_theta - 1) bc = c->N_theta - 1;
    real tcen = c0 + (real)bc * dth;
    real dlt = tc - tcen;
    int tb[2] = {bc, bc};
    real tw[2] = {RL(1.0), RL(0.0)};
    if (dlt > RL(0.0) && bc < c->N_theta - 1) tb[1] = bc + 1;
    else if (dlt < RL(0.0) && bc > 0) tb[1] = bc - 1;
    if (tb[1] != tb[0]) {
        real f = r_min(RL(1.0), r_fabs(dlt) / dth);
        tw[1] = f * f;
        tw[0] = RL(1.0) - tw[1];
        if (c->cfg.energy_split && weight * tw[1] < (real)c->cfg.split_min_weight) {
            tw[1] = RL(0.0);
            tw[0] = RL(1.0);
        }
    }
    real Ec = r_max(c->E_edges[0], r_min(E, c->E_edges[c->N_E]));
    eparts ep = bin_energy(c, Ec, weight);
    real dropped = RL(0.0);
    for (int ei = 0; ei < ep.n; ++ei) {
        int Eb = ep.bin[ei];
        int El = Eb % c->cfg.ne_local;
        uint32_t bE = (uint32_t)(Eb / c->cfg.ne_local);
        for (int ti = 0; ti < 2; ++ti) {
            real wt = tw[ti];
            if (wt <= RL(0.0)) continue;
            real we = weight * wt;
            if (c->cfg.energy_split) we = we * ep.frac[ei];
            int tbin = tb[ti];
            uint32_t want = enc_block((uint32_t)(tbin / c->cfg.nt_local), bE);
            int l = enc_lidx(c, tbin % c->cfg.nt_local, El, xs, zs);
            uint32_t sel;
            int s = claim_w(c, bk->bid, c->Kb, want, &sel, (double)we);
            if (s < 0) { dropped += we; continue; }
            int le = (sel == want) ? l : remap_lidx(c, l, want, sel);
            if (sel != want && c->cfg.energy_split && eshift)
                *eshift += (double)((e_center(c, Eb) - e_center(c, ebin_of(c, sel, le))) * we);
            bk->val[(size_t)s * c->L + le] += we;
            bk->count[s]++;
        }
    }
    return dropped;
}

static inline int bucket_index(const orc_ctx* c, int cell, int face) {
    int base = c->cell_to_bucket[cell];
    return base < 0 ? -1 : base + face;
}

static int exit_face(real x, real z, real dx, real dz) {   /* device_bucket.cuh:783-807 */
    const real eps = RL(0.001);
    real hz = dz * RL(0.5), hx = dx * RL(0.5);
    if (z >= hz - eps) return FACE_ZP;
    if (z <= -hz + eps) return FACE_ZM;
    if (x >= hx - eps) return FACE_XP;
    if (x <= -hx + eps) return FACE_XM;
    return -1;
}
static int neighbor(int cell, int face, int Nx, int Nz) {
    int ix = cell % Nx, iz = cell / Nx;
    switch (face) {
        case FACE_ZP: return iz + 1 >= Nz ? -1 : cell + Nx;
        case FACE_ZM: return iz <= 0 ? -1 : cell - Nx;
        case FACE_XP: return ix + 1 >= Nx ? -1 : cell + 1;
        case FACE_XM: return ix <= 0 ? -1 : cell - 1;
    }
    return -1;
}

/* +z emission with N-cell lateral Gaussian split: device_bucket.cuh:857-987 */
static real emit_lateral_spread(orc_ctx* c, int src, int tz, real theta, real E, const kids* kd, real weight,
                                real xoff, real sigma, real* boundary_w, double* eshift) {
    if (weight <= RL(0.0)) return RL(0.0);
    real dropped = RL(0.0);
    sigma = r_max(sigma, RL(1e-6));
    const int N = SPREAD_CELLS;
    real w[SPREAD_CELLS];
    spread_weights(w, xoff, sigma, (real)c->cfg.dx, N);
    real s = 0;
    for (int i = 0; i < N; ++i) { w[i] = r_max(RL(0.0), w[i]); s += w[i]; }
    if (s < RL(1e-12)) {
        for (int i = 0; i < N; ++i) w[i] = RL(0.0);
        w[N / 2] = RL(1.0);
    } else {
        for (int i = 0; i < N; ++i) w[i] /= s;
    }
    int Nx = c->cfg.Nx, Nz = c->cfg.Nz;
    int ixs = src % Nx, izs = src / Nx;
    for (int i = 0; i < N; ++i) {
        real wf = w[i];
        if (wf <= RL(0.0)) continue;
        int off = -(N / 2) + i;
        int ixt = ixs + off;
        if (ixt < 0 || ixt >= Nx || tz < 0 || tz >= Nz) { *boundary_w += weight * wf; continue; }
        int emit_cell = ixt + izs * Nx;
        int bi = bucket_index(c, emit_cell, FACE_ZP);
        if (bi < 0) { dropped += weight * wf; continue; }
        int xt = off < 0 ? c->cfg.nx_sub - 1 : (off > 0 ? 0 : c->cfg.nx_sub / 2);
        dropped += kd ? emit_kids_to_bucket(c, &c->buckets[bi], kd, weight * wf, xt, 0, eshift)
                      : emit_to_bucket(c, &c->buckets[bi], theta, E, weight * wf, xt, 0, eshift);
    }
    return dropped;
}

/* ------------------------------------------------------------------------- */
/* per-cell transport                                                         */
/* ------------------------------------------------------------------------- */
typedef struct tally {
    double edep, e_cut, e_nuc, e_bnd;
    float w_cut, w_nuc, w_bnd;
} tally;

static inline unsigned iter_salt(const orc_ctx* c) {
    return c->cfg.seed_iteration_salt ? (unsigned)(c->iter - 1) * 0x9E3779B9u : 0u;
}

static int seed_slot(const orc_ctx* c, const uint32_t* ids, int slot) {
    if (c->cfg.seed_slot_mode == 0) return slot;
    int r = 0;
    for (int s = 0; s < c->Kb; ++s)
        if (ids[s] != ORC_EMPTY && ids[s] < ids[slot]) ++r;
    return r;
}

/* Stay-in-cell emission shared by K2 and K3 (k2_coarsetransport.cu:471-690,
 * k3_finetransport.cu:516-746).  Returns 0 when the component was dropped by
 * slot saturation (the caller's per-bin `continue`). */
static int emit_stay(orc_ctx* c, int k3, int cell, real theta_new, real E_new, real w_new,
                     real x_new, real z_new, real sig_sub, real sig_cell, tally* t) {
    psi_buf* po = psi_out(c);
    const int Nx = c->cfg.Nx;
    const real dx = (real)c->cfg.dx, dz = (real)c->cfg.dz;
    real tmin = c->th_edges[0], tmax = c->th_edges[c->N_theta];
    real dth = (tmax - tmin) / (real)c->N_theta;
    int tbn = (int)((theta_new - tmin) / dth);
    tbn = (int)r_max(RL(0.0), r_min((real)tbn, (real)(c->N_theta - 1)));
    eparts ep = bin_energy(c, E_new, w_new);
    int nxs = c->cfg.nx_sub;
    real w[64];
    spread_weights_subcell(w, x_new, sig_sub, dx, nxs);
    int ix = cell % Nx;
    int zst = sub_bin(z_new, dz, c->cfg.nz_sub);
    real lb = -dx * RL(0.5), rb = dx * RL(0.5);
    real win = gcdf(rb, x_new, sig_cell) - gcdf(lb, x_new, sig_cell);
    real wcf = r_min(RL(1.0), r_max(RL(0.0), win));
    real wsum = 0;
    for (int i = 0; i < nxs; ++i) { w[i] = r_max(RL(0.0), w[i]); wsum += w[i]; }
    if (wsum < RL(1e-12)) {
        for (int i = 0; i < nxs; ++i) w[i] = RL(0.0);
        w[nxs / 2] = RL(1.0);
        wsum = RL(1.0);
    }
    real E_emit = ep.Erep;
    for (int ei = 0; ei < ep.n; ++ei) {
        int Eb = ep.bin[ei];
        uint32_t want = ((uint32_t)(Eb / c->cfg.ne_local) << 12) | ((uint32_t)(tbn / c->cfg.nt_local) & 0xFFFu);
        uint32_t sel;
        real wpart = c->cfg.energy_split ? w_new * ep.frac[ei] : w_new;
        int os = psi_slot(c, po, cell, want, &sel, (double)wpart);
        if (os < 0) {
            double *cw = k3 ? &c->k3_slot_w : &c->k2_slot_w, *ce = k3 ? &c->k3_slot_e : &c->k2_slot_e;
            *cw += (double)wpart;
            *ce += (double)(E_new * wpart);
            if (!c->cfg.energy_split) return 0;
            continue;
        }
        int tbe = tbn, Ebe = Eb;
        if (sel != want) {
            int bt = (int)(sel & 0xFFFu), be = (int)((sel >> 12) & 0xFFFu);
            int t0 = bt * c->cfg.nt_local, e0 = be * c->cfg.ne_local;
            if (tbe < t0) tbe = t0;
            if (tbe > t0 + c->cfg.nt_local - 1) tbe = t0 + c->cfg.nt_local - 1;
            if (Ebe < e0) Ebe = e0;
            if (Ebe > e0 + c->cfg.ne_local - 1) Ebe = e0 + c->cfg.ne_local - 1;
        }
        if (!c->cfg.energy_split) E_emit = e_center(c, Ebe);
        else if (Ebe != Eb) t->edep += (double)((e_center(c, Eb) - e_center(c, Ebe)) * wpart * wcf);
        int tl = tbe % c->cfg.nt_local, El = Ebe % c->cfg.ne_local;
        for (int xs = 0; xs < nxs; ++xs) {
            real wf = (w[xs] / wsum) * wcf;
            if (wf <= RL(0.0)) continue;
            int l = enc_lidx(c, tl, El, xs, zst);
            po->val[((size_t)cell * c->Kb + os) * c->L + l] += wpart * wf;
        }
    }
    real wl = RL(0.0), wr = RL(0.0);
    if (wcf < RL(1.0) - RL(1e-6)) {
        real wlr = r_max(RL(0.0), gcdf(lb, x_new, sig_cell));
        real wrr = r_max(RL(0.0), RL(1.0) - gcdf(rb, x_new, sig_cell));
        real tt = r_max(RL(0.0), RL(1.0) - wcf);
        real ts = wlr + wrr;
        if (tt > RL(0.0) && ts > RL(1e-12)) {
            real sc = tt / ts;
            wl = wlr * sc;
            wr = wrr * sc;
        }
        double *bw = k3 ? &c->k3_bkt_w : &c->k2_bkt_w, *be = k3 ? &c->k3_bkt_e : &c->k2_bkt_e;
        if (wl > RL(0.0)) {
            real ws = w_new * wl;
            if (ix > 0) {
                int bi = bucket_index(c, cell, FACE_XM);
                if (bi < 0) {
                    *bw += (double)ws;
                    *be += (double)(E_new * ws);
                    return 1;
                }
                real d = emit_to_bucket(c, &c->buckets[bi], theta_new, E_new, ws, nxs - 1,
                                        sub_bin(z_new, dz, c->cfg.nz_sub), &t->edep);
                if (d > RL(0.0)) { *bw += (double)d; *be += (double)(E_new * d); }
            } else {
                t->w_bnd += (float)ws;
                t->e_bnd += (double)(E_new * ws);
            }
        }
        if (wr > RL(0.0)) {
            real ws = w_new * wr;
            if (ix < Nx - 1) {
                int bi = bucket_index(c, cell, FACE_XP);
                if (bi < 0) {
                    *bw += (double)ws;
                    *be += (double)(E_new * ws);
                    return 1;
                }
                real d = emit_to_bucket(c, &c->buckets[bi], theta_new, E_new, ws, 0,
                                        sub_bin(z_new, dz, c->cfg.nz_sub), &t->edep);
                if (d > RL(0.0)) { *bw += (double)d; *be += (double)(E_new * d); }
            } else {
                t->w_bnd += (float)ws;
                t->e_bnd += (double)(E_new * ws);
            }
        }
    }
    /* energy fold of the re-binned weight: K3 always (k3_finetransport.cu:738-745);
     * K2 only under the energy split. */
    if (k3 || c->cfg.energy_split) {
        real rf = wcf;
        if (ix > 0) rf += wl;
        if (ix < Nx - 1) rf += wr;
        rf = r_min(RL(1.0), r_max(RL(0.0), rf));
        real rw = w_new * rf;
        if (rw > RL(0.0)) t->edep += (double)((E_new - E_emit) * rw);
    }
    return 1;
}

/* Expectation form of emit_stay: the children stay in the cell, each spread
 * over the x sub-bins; the Gaussian tails past the cell edges go to the
 * lateral buckets as children; the mean energy minus the children's
 * represented energy is folded into the deposit. */
static void emit_stay_kids(orc_ctx* c, int k3, int cell, const kids* kd, real E_new, real w_new,
                           real x_new, real z_new, real sig_sub, real sig_cell, tally* t) {
    psi_buf* po = psi_out(c);
    const int Nx = c->cfg.Nx;
    const real dx = (real)c->cfg.dx, dz = (real)c->cfg.dz;
    int nxs = c->cfg.nx_sub;
    real w[64];
    spread_weights_subcell(w, x_new, sig_sub, dx, nxs);
    int ix = cell % Nx;
    int zst = sub_bin(z_new, dz, c->cfg.nz_sub);
    real lb = -dx * RL(0.5), rb = dx * RL(0.5);
    real win = gcdf(rb, x_new, sig_cell) - gcdf(lb, x_new, sig_cell);
    real wcf = r_min(RL(1.0), r_max(RL(0.0), win));
    real wsum = 0;
    for (int i = 0; i < nxs; ++i) { w[i] = r_max(RL(0.0), w[i]); wsum += w[i]; }
    if (wsum < RL(1e-12)) {
        for (int i = 0; i < nxs; ++i) w[i] = RL(0.0);
        w[nxs / 2] = RL(1.0);
        wsum = RL(1.0);
    }
    for (int e = 0; e <= kd->emax; ++e) {
        int Eb = kd->j - e;
        for (int k = 0; k < SM2D_RD_KIDS; ++k) {
            if (!kid_live(kd, sm2d_rd_kid_t(k), e)) continue;
            real wk = kid_weight(kd, w_new, k, e);
            int tbn = kid_tbin(c, kd, k);
            uint32_t want = ((uint32_t)(Eb / c->cfg.ne_local) << 12) | ((uint32_t)(tbn / c->cfg.nt_local) & 0xFFFu);
            uint32_t sel;
            int os = psi_slot(c, po, cell, want, &sel, (double)wk);
            if (os < 0) {
                double *cw = k3 ? &c->k3_slot_w : &c->k2_slot_w, *ce = k3 ? &c->k3_slot_e : &c->k2_slot_e;
                *cw += (double)wk;
                *ce += (double)(E_new * wk);
                continue;
            }
            int tbe = tbn, Ebe = Eb;
            if (sel != want) {
                int t0 = (int)(sel & 0xFFFu) * c->cfg.nt_local, e0 = (int)((sel >> 12) & 0xFFFu) * c->cfg.ne_local;
                if (tbe < t0) tbe = t0;
                if (tbe > t0 + c->cfg.nt_local - 1) tbe = t0 + c->cfg.nt_local - 1;
                if (Ebe < e0) Ebe = e0;
                if (Ebe > e0 + c->cfg.ne_local - 1) Ebe = e0 + c->cfg.ne_local - 1;
            }
            if (Ebe != Eb) t->edep += (double)((e_center(c, Eb) - e_center(c, Ebe)) * wk * wcf);
            int tl = tbe % c->cfg.nt_local, El = Ebe % c->cfg.ne_local;
            for (int xs = 0; xs < nxs; ++xs) {
                real wf = (w[xs] / wsum) * wcf;
                if (wf <= RL(0.0)) continue;
                int l = enc_lidx(c, tl, El, xs, zst);
                po->val[((size_t)cell * c->Kb + os) * c->L + l] += wk * wf;
            }
        }
    }
    real wl = RL(0.0), wr = RL(0.0);
    if (wcf < RL(1.0) - RL(1e-6)) {
        real wlr = r_max(RL(0.0), gcdf(lb, x_new, sig_cell));
        real wrr = r_max(RL(0.0), RL(1.0) - gcdf(rb, x_new, sig_cell));
        real tt = r_max(RL(0.0), RL(1.0) - wcf);
        real ts = wlr + wrr;
        if (tt > RL(0.0) && ts > RL(1e-12)) {
            real sc = tt / ts;
            wl = wlr * sc;
            wr = wrr * sc;
        }
        double *bw = k3 ? &c->k3_bkt_w : &c->k2_bkt_w, *be = k3 ? &c->k3_bkt_e : &c->k2_bkt_e;
        if (wl > RL(0.0)) {
            real ws = w_new * wl;
            if (ix > 0) {
                real d = emit_kids_to_bucket(c, &c->buckets[bucket_index(c, cell, FACE_XM)], kd, ws, nxs - 1, zst,
                                             &t->edep);
                if (d > RL(0.0)) { *bw += (double)d; *be += (double)(E_new * d); }
            } else {
                t->w_bnd += (float)ws;
                t->e_bnd += (double)(E_new * ws);
            }
        }
        if (wr > RL(0.0)) {
            real ws = w_new * wr;
            if (ix < Nx - 1) {
                real d = emit_kids_to_bucket(c, &c->buckets[bucket_index(c, cell, FACE_XP)], kd, ws, 0, zst, &t->edep);
                if (d > RL(0.0)) { *bw += (double)d; *be += (double)(E_new * d); }
            } else {
                t->w_bnd += (float)ws;
                t->e_bnd += (double)(E_new * ws);
            }
        }
    }
    real rf = wcf;
    if (ix > 0) rf += wl;
    if (ix < Nx - 1) rf += wr;
    rf = r_min(RL(1.0), r_max(RL(0.0), rf));
    real rw = w_new * rf;
    if (rw > RL(0.0)) t->edep += (double)((E_new - kd->Erep) * rw);
}

/* Crossing a face: k2_coarsetransport.cu:363-459, k3_finetransport.cu:380-503;
 * kd: the component's children in the expectation form (NULL: re-bin the
 * sampled angle and energy) */
static void emit_cross(orc_ctx* c, int k3, int cell, int face, real theta_new, real E_new, const kids* kd, real w_new,
                       real x_new, real z_new, real sig_tr, tally* t) {
    const int Nx = c->cfg.Nx, Nz = c->cfg.Nz;
    const real dx = (real)c->cfg.dx, dz = (real)c->cfg.dz;
    double *bw = k3 ? &c->k3_bkt_w : &c->k2_bkt_w, *be = k3 ? &c->k3_bkt_e : &c->k2_bkt_e;
    int nb = neighbor(cell, face, Nx, Nz);
    if (nb < 0) {
        t->w_bnd += (float)w_new;
        t->e_bnd += (double)(E_new * w_new);
        return;
    }
    real E_emit_tr = kd ? kd->Erep : bin_energy(c, E_new, w_new).Erep;
    int fold = k3 || c->cfg.energy_split;
    if (face == FACE_ZP) {
        int tz = cell / Nx + 1;
        real lbw = RL(0.0);
        real d = emit_lateral_spread(c, cell, tz, theta_new, E_new, kd, w_new, x_new, sig_tr, &lbw, &t->edep);
        if (lbw > RL(0.0)) {
            t->w_bnd += (float)lbw;
            t->e_bnd += (double)(E_new * lbw);
        }
        if (d > RL(0.0)) { *bw += (double)d; *be += (double)(E_new * d); }
        if (fold) {
            real tw = r_max(RL(0.0), w_new - lbw - d);
            if (tw > RL(0.0)) t->edep += (double)((E_new - E_emit_tr) * tw);
        }
        return;
    }
    real xo = (face == FACE_XP) ? -dx * RL(0.5) : (face == FACE_XM ? dx * RL(0.5) : x_new);
    int xsn = sub_bin(xo, dx, c->cfg.nx_sub);
    real zo = (face == FACE_ZM) ? (k3 ? dz * RL(0.5) - dz * RL(0.125) : -dz * RL(0.5) + dz * RL(0.125)) : z_new;
    int zsn = sub_bin(zo, dz, c->cfg.nz_sub);
    if (face == FACE_ZP) zsn = 0;
    else if (face == FACE_ZM) zsn = c->cfg.nz_sub - 1;
    int bi = bucket_index(c, cell, face);
    if (bi < 0) {
        *bw += (double)w_new;
        *be += (double)(E_new * w_new);
        return;
    }
    real d = kd ? emit_kids_to_bucket(c, &c->buckets[bi], kd, w_new, xsn, zsn, &t->edep)
                : emit_to_bucket(c, &c->buckets[bi], theta_new, E_new, w_new, xsn, zsn, &t->edep);
    if (d > RL(0.0)) { *bw += (double)d; *be += (double)(E_new * d); }
    if (fold) {
        real tw = r_max(RL(0.0), w_new - d);
        if (tw > RL(0.0)) t->edep += (double)((E_new - E_emit_tr) * tw);
    }
}

static void commit_tally(orc_ctx* c, int cell, const tally* t) {
    c->dw_cut[cell] += t->w_cut;
    c->dw_nuc[cell] += t->w_nuc;
    c->dw_bnd[cell] += t->w_bnd;
    c->edep[cell] += t->edep;
    c->w_cut[cell] += t->w_cut;
    c->e_cut[cell] += t->e_cut;
    c->w_nuc[cell] += t->w_nuc;
    c->e_nuc[cell] += t->e_nuc;
    c->w_bnd[cell] += t->w_bnd;
    c->e_bnd[cell] += t->e_bnd;
}

/* K2_CoarseTransport for one cell: k2_coarsetransport.cu:76-704 */
static void k2_cell(orc_ctx* c, int cell) {
    psi_buf* pi = psi_in(c);
    const int Nx = c->cfg.Nx;
    const real dx = (real)c->cfg.dx, dz = (real)c->cfg.dz;
    const rlut* lut = &c->lut;
    tally t = {0};
    real cstep = r_min((real)c->cfg.step_coarse, r_min(dx, dz));
    const uint32_t* ids = &pi->bid[(size_t)cell * c->Kb];
    for (int slot = 0; slot < c->Kb; ++slot) {
        uint32_t bid = ids[slot];
        if (bid == ORC_EMPTY) continue;
        uint32_t bt = bid & 0xFFFu, bE = (bid >> 12) & 0xFFFu;
        int sslot = seed_slot(c, ids, slot);
        for (int l = 0; l < c->L; ++l) {
            real w = pi->val[((size_t)cell * c->Kb + slot) * c->L + l];
            if (w <= RL(0.0)) continue;
            int tl, El, xs, zs;
            dec_lidx(c, l, &tl, &El, &xs, &zs);
            int tbin = (int)bt * c->cfg.nt_local + tl;
            int Ebin = (int)bE * c->cfg.ne_local + El;
            real tmin = c->th_edges[0], tmax = c->th_edges[c->N_theta];
            real dth = (tmax - tmin) / (real)c->N_theta;
            real theta = tmin + ((real)tbin + RL(0.5)) * dth;
            real E = c->E_edges[Ebin] + RL(1.0) * ((c->E_edges[Ebin + 1] - c->E_edges[Ebin]) * RL(0.5));
            if (w < (c->cfg.prune_coarse > 0.0f ? (real)c->cfg.prune_coarse : K2_PRUNE)) {
                c->k2_prune_w += (double)w;
                c->k2_prune_e += (double)(E * w);
                continue;
            }
            if (E <= E_CUTOFF) {
                t.w_cut += (float)w;
                t.e_cut += (double)(E * w);
                continue;
            }
            real xc = sub_offset(xs, c->cfg.nx_sub, dx);
            real zc = sub_offset(zs, c->cfg.nz_sub, dz);
            real hz = dz * RL(0.5), hx = dx * RL(0.5);
            real step_lim = cstep;
            real rstep = step_lim;
            int split = 0;
            real Efo = (real)c->cfg.E_fine_on;
            const int iz = cell / Nx;
            const real rho = rho_of(c, iz);
            if (E > Efo + RL(1e-6)) {
                real Rc = lut_R(lut, E);
                real Rf = lut_R(lut, r_max(Efo, (real)lut->Emin));
                real rtf = (Rc - Rf) / rho;   /* geometric distance to the fine threshold */
                if (rtf > RL(0.0) && rtf < rstep) {
                    rstep = rtf;
                    step_lim = rstep;
                    split = 1;
                }
            }
            real dE = lut_energy_deposition(lut, E, rho * rstep);
            dE = r_min(dE, E);
            real E_new = E - dE;
            real edep = dE * w;
            real w_rem, E_rem;
            real w_new = nuclear_atten(w, E, rho * rstep, &w_rem, &E_rem);
            if (split && E_new > Efo) {
                real ex = E_new - Efo;
                if (ex > RL(0.0) && w_new > RL(0.0)) edep += ex * w_new;
                E_new = Efo;
            }
            real path0 = r_max(RL(0.0), (real)iz * dz + (zc + RL(0.5) * dz));
            /* scattering accumulated over the water-equivalent depth */
            real path0w = c->rho ? r_max(RL(0.0), (real)c->wet[iz] + rho * (zc + RL(0.5) * dz)) : path0;
            real step_mm = r_max(rstep, RL(0.0));
            real sts = RL(0.0);
            if (path0 > RL(0.0)) sts = highland(E, path0w);
            real A_old = sts * sts;
            real B_old = RL(0.5) * A_old * path0;
            real sx0 = (real)c->cfg.sigma_x_initial;
            real C_old = sx0 * sx0 + (A_old * path0 * path0) / RL(3.0);
            real E_mid = r_max(E - RL(0.5) * dE, (real)lut->Emin);
            real T = scattering_T(E_mid, step_mm, rho);
            /* device_fermi_eyges_step */
            real A_new = A_old + T * step_mm;
            real C_new = C_old + RL(2.0) * B_old * step_mm + A_old * step_mm * step_mm
                         + (RL(1.0) / RL(3.0)) * T * step_mm * step_mm * step_mm;
            A_new = r_max(A_new, RL(0.0));
            C_new = r_max(C_new, RL(0.0));
            real sig_th = r_sqrt(r_max(A_new - A_old, RL(0.0)));
            real dC = r_max(C_new - C_old, RL(0.0));
            real uf = r_min(UNRES_MAX, UNRES_BASE + UNRES_SLOPE * path0);
            real C_eff = dC + uf * C_old;
            real sig_x = r_max(r_sqrt(r_max(C_eff, RL(0.0))), RL(0.01));
            real sig_tr = r_max(r_sin(r_min(sig_th, RL(1.57))) * step_mm / RL(1.7320508), RL(0.01));
            unsigned pseed = (unsigned)r_min(path0 * RL(1000.0), RL(4294967295.0));
            unsigned ts = ((unsigned)(cell + 1) * SEED_A) ^ ((unsigned)(sslot + 1) * SEED_B) ^
                          ((unsigned)(l + 1) * SEED_C) ^ (unsigned)(Ebin + 17) ^ (pseed * 747796405u) ^ iter_salt(c);
            /* expectation form: the MCS distribution instead of a draw, the
             * step along the incoming angle */
            real scat = c->cfg.expectation ? RL(0.0) : ((sig_th <= RL(0.0)) ? RL(0.0) : gauss_sample(&ts) * sig_th);
            real theta_new = theta + scat;
            theta_new = r_max(c->th_edges[0], r_min(theta_new, c->th_edges[c->N_theta]));
            real mu = r_cos(theta_new), eta = r_sin(theta_new);
            real x_new = xc + eta * step_lim;
            real z_new = zc + mu * step_lim;
            int face = exit_face(x_new, z_new, dx, dz);
            x_new = r_max(-hx, r_min(x_new, hx));
            z_new = r_max(-hz, r_min(z_new, hz));
            t.edep += (double)edep;
            t.w_nuc += (float)w_rem;
            t.e_nuc += (double)E_rem;
            if (E_new <= E_CUTOFF || ((c->cfg.energy_split || c->cfg.floor_cutoff) && E_new <= e_center(c, 0))) {
                t.w_cut += (float)w_new;
                t.e_cut += (double)(E_new * w_new);
                continue;
            }
            if (c->cfg.expectation) {
                kids kd;
                int tc = tbin < 0 ? 0 : (tbin > c->N_theta - 1 ? c->N_theta - 1 : tbin);
                int ec = Ebin < 0 ? 0 : (Ebin > c->N_E - 1 ? c->N_E - 1 : Ebin);
                make_kids(c, tc, ec, sig_th / dth, E_new, RL(0.0), w_new, &kd);
                if (face >= 0) emit_cross(c, 0, cell, face, theta_new, E_new, &kd, w_new, x_new, z_new, sig_tr, &t);
                else emit_stay_kids(c, 0, cell, &kd, E_new, w_new, x_new, z_new, sig_x, sig_x, &t);
                continue;
            }
            if (face >= 0) emit_cross(c, 0, cell, face, theta_new, E_new, NULL, w_new, x_new, z_new, sig_tr, &t);
            else emit_stay(c, 0, cell, theta_new, E_new, w_new, x_new, z_new, sig_x, sig_x, &t);
        }
    }
    commit_tally(c, cell, &t);
}

/* K3_FineTransport for one cell: k3_finetransport.cu:94-760 */
static void k3_cell(orc_ctx* c, int cell) {
    psi_buf* pi = psi_in(c);
    const int Nx = c->cfg.Nx, Nz = c->cfg.Nz;
    const real dx = (real)c->cfg.dx, dz = (real)c->cfg.dz;
    const rlut* lut = &c->lut;
    tally t = {0};
    const uint32_t* ids = &pi->bid[(size_t)cell * c->Kb];
    for (int slot = 0; slot < c->Kb; ++slot) {
        uint32_t bid = ids[slot];
        if (bid == ORC_EMPTY) continue;
        uint32_t bt = bid & 0xFFFu, bE = (bid >> 12) & 0xFFFu;
        int sslot = seed_slot(c, ids, slot);
        for (int l = 0; l < c->L; ++l) {
            real w = pi->val[((size_t)cell * c->Kb + slot) * c->L + l];
            if (w <= RL(0.0)) continue;
            int tl, El, xs, zs;
            dec_lidx(c, l, &tl, &El, &xs, &zs);
            int tbin = (int)bt * c->cfg.nt_local + tl;
            int Ebin = (int)bE * c->cfg.ne_local + El;
            if (tbin < 0) tbin = 0;
            if (tbin > c->N_theta - 1) tbin = c->N_theta - 1;
            if (Ebin < 0) Ebin = 0;
            if (Ebin > c->N_E - 1) Ebin = c->N_E - 1;
            real El_ = c->E_edges[Ebin], Eu_ = c->E_edges[Ebin + 1];
            real E = El_ + RL(1.0) * ((Eu_ - El_) * RL(0.5));
            if (w < (c->cfg.prune_fine > 0.0f ? (real)c->cfg.prune_fine : K3_PRUNE)) {
                c->k3_prune_w += (double)w;
                c->k3_prune_e += (double)(E * w);
                continue;
            }
            real tmin = c->th_edges[0], tmax = c->th_edges[c->N_theta];
            real dth = (tmax - tmin) / (real)c->N_theta;
            real theta = c->th_edges[tbin] + RL(0.5) * dth;
            if (E <= E_CUTOFF) {
                t.w_cut += (float)w;
                t.e_cut += (double)(E * w);
                continue;
            }
            real xc = sub_offset(xs, c->cfg.nx_sub, dx);
            real zc = sub_offset(zs, c->cfg.nz_sub, dz);
            real mu0 = r_cos(theta), eta0 = r_sin(theta);
            real hz = dz * RL(0.5), hx = dx * RL(0.5);
            real szp = (mu0 > 0) ? (hz - zc) / mu0 : RL(1e30);
            real szm = (mu0 < 0) ? (-hz - zc) / mu0 : RL(1e30);
            real sxp = (eta0 > 0) ? (hx - xc) / eta0 : RL(1e30);
            real sxm = (eta0 < 0) ? (-hx - xc) / eta0 : RL(1e30);
            real sb = r_min(r_min(szp, szm), r_min(sxp, sxm));
            sb = r_max(sb, RL(0.0));
            const int iz = cell / Nx;
            const real rho = rho_of(c, iz);
            real sphys = max_step(lut, E) / rho;   /* the water-equivalent limit as a geometric step */
            real step = r_min(sphys, sb * BOUNDARY_SAFETY);
            real mean_dE = lut_energy_deposition(lut, E, rho * step);
            real dE, sE = RL(0.0);
            if (c->cfg.expectation) {   /* the straggling distribution instead of a draw */
                dE = mean_dE;
                if (c->cfg.enable_straggling) sE = straggling_sigma(E, step, rho);
            } else if (c->cfg.enable_straggling) {
                unsigned seed = ((unsigned)(cell * 7 + sslot * 13 + l * 17) ^ 0xDEECE66Du) ^ iter_salt(c);
                real sE = straggling_sigma(E, step, rho);
                if (sE <= RL(0.0)) dE = mean_dE;
                else {
                    real z = gauss_sample(&seed);
                    dE = r_max(mean_dE + z * sE, RL(0.0));
                }
            } else {
                dE = mean_dE;
            }
            dE = r_min(dE, E);
            real E_new = E - dE;
            real edep = dE * w;
            real w_rem = RL(0.0), E_rem = RL(0.0), w_new = w;
            if (c->cfg.enable_nuclear) w_new = nuclear_atten(w, E, rho * step, &w_rem, &E_rem);
            real step_mm = r_max(step, RL(0.0));
            real Ap = (c->fe_A && iz >= 0 && iz < Nz) ? (real)c->fe_A[iz] : RL(0.0);
            real Bp = (c->fe_B && iz >= 0 && iz < Nz) ? (real)c->fe_B[iz] : RL(0.0);
            real E_mid = r_max(E - RL(0.5) * dE, (real)lut->Emin);
            real T = scattering_T(E_mid, step_mm, rho);
            real sig_th = r_sqrt(r_max(T * step_mm, RL(0.0)));
            real dC = RL(2.0) * Bp * step_mm + Ap * step_mm * step_mm + T * step_mm * step_mm * step_mm / RL(3.0);
            dC = r_max(dC, RL(0.0));
            real sig_x = r_max(r_sqrt(dC), RL(0.01));
            unsigned pseed = (unsigned)r_min((real)iz * dz * RL(1000.0), RL(4294967295.0));
            unsigned ts = ((unsigned)(cell + 1) * SEED_A) ^ ((unsigned)(sslot + 1) * SEED_B) ^
                          ((unsigned)(l + 1) * SEED_C) ^ (unsigned)(Ebin + 17) ^ (pseed * 747796405u) ^ iter_salt(c);
            real scat = c->cfg.expectation ? RL(0.0) : ((sig_th <= RL(0.0)) ? RL(0.0) : gauss_sample(&ts) * sig_th);
            real theta_new = theta + scat;
            theta_new = r_max(c->th_edges[0], r_min(theta_new, c->th_edges[c->N_theta]));
            real mu = r_cos(theta_new), eta = r_sin(theta_new);
            real x_new = xc + eta * step;
            real z_new = zc + mu * step;
            int face = exit_face(x_new, z_new, dx, dz);
            x_new = r_max(-hx, r_min(x_new, hx));
            z_new = r_max(-hz, r_min(z_new, hz));
            t.edep += (double)edep;
            t.w_nuc += (float)w_rem;
            t.e_nuc += (double)E_rem;
            if (E_new <= E_CUTOFF || ((c->cfg.energy_split || c->cfg.floor_cutoff) && E_new <= e_center(c, 0))) {
                t.w_cut += (float)w_new;
                t.e_cut += (double)(E_new * w_new);
                continue;
            }
            if (c->cfg.expectation) {
                kids kd;
                real f[4], row[SM2D_RD_NT * SM2D_RD_NE];
                int tab = c->cfg.surrogate_tables && surr_features(c, Ebin, sig_th / dth, E_new, sE, f);
                if (tab && c->cfg.surrogate_tables == 2)   /* the network, or the closed forms on fallback */
                    tab = c->net && net_table(c->net, f, row);
                else if (tab)
                    plain_table(f, row);   /* the table path with the method's own table */
                if (tab) {
                    make_kids_tab(c, tbin, Ebin, E_new, w_new, row, &kd);
                } else {
                    make_kids(c, tbin, Ebin, sig_th / dth, E_new, sE, w_new, &kd);
                }
                if (face >= 0)
                    emit_cross(c, 1, cell, face, theta_new, E_new, &kd, w_new, x_new, z_new, K3_SIGMA_TRANSPORT, &t);
                else emit_stay_kids(c, 1, cell, &kd, E_new, w_new, x_new, z_new, K3_SIGMA_TRANSPORT, sig_x, &t);
                continue;
            }
            if (face >= 0) emit_cross(c, 1, cell, face, theta_new, E_new, NULL, w_new, x_new, z_new, K3_SIGMA_TRANSPORT, &t);
            else emit_stay(c, 1, cell, theta_new, E_new, w_new, x_new, z_new, K3_SIGMA_TRANSPORT, sig_x, &t);
        }
    }
    commit_tally(c, cell, &t);
}

/* ------------------------------------------------------------------------- */
/* K4_BucketTransfer: k4_transfer.cu:174-333 (gather per destination cell)  */
/* ------------------------------------------------------------------------- */
static void k4(orc_ctx* c) {
    psi_buf* po = psi_out(c);
    const int Nx = c->cfg.Nx, Nz = c->cfg.Nz;
    for (int cell = 0; cell < c->Nc; ++cell) {
        int ix = cell % Nx, iz = cell / Nx;
        for (int face = 0; face < 4; ++face) {
            int src = -1, sf = -1;
            if (face == 0 && iz > 0) { src = cell - Nx; sf = 0; }
            if (face == 1 && iz + 1 < Nz) { src = cell + Nx; sf = 1; }
            if (face == 2 && ix > 0) { src = cell - 1; sf = 2; }
            if (face == 3 && ix + 1 < Nx) { src = cell + 1; sf = 3; }
            if (src < 0) continue;
            int base = c->cell_to_bucket[src];
            if (base < 0) continue;
            bucket* bk = &c->buckets[base + sf];
            for (int s = 0; s < c->Kb; ++s) {
                uint32_t bid = bk->bid[s];
                if (bid == ORC_EMPTY) continue;
                uint32_t bE = (bid >> 12) & 0xFFFu;
                uint32_t sel;
                const real* v = &bk->val[(size_t)s * c->L];
                double wsl = 0.0;
                for (int l = 0; l < c->L; ++l) wsl += (double)v[l];
                int os = psi_slot(c, po, cell, bid, &sel, wsl);
                if (os < 0) {
                    double dw = 0.0, de = 0.0;
                    for (int l = 0; l < c->L; ++l) {
                        if (v[l] > RL(0.0)) {
                            int t_, e_, x_, z_;
                            dec_lidx(c, l, &t_, &e_, &x_, &z_);
                            int Eb = (int)bE * c->cfg.ne_local + e_;
                            if (Eb < 0) Eb = 0;
                            if (Eb > c->N_E - 1) Eb = c->N_E - 1;
                            real E = c->E_edges[Eb] + RL(1.0) * (RL(0.5) * (c->E_edges[Eb + 1] - c->E_edges[Eb]));
                            dw += (double)v[l];
                            de += (double)E * (double)v[l];
                        }
                    }
                    c->k4_slot_w += dw;
                    c->k4_slot_e += de;
                    continue;
                }
                for (int l = 0; l < c->L; ++l) {
                    if (v[l] > RL(0.0)) {
                        int le = (sel != bid) ? remap_lidx(c, l, bid, sel) : l;
                        /* split method: the re-binning shift is booked at the
                           bucket's cell (the emitting side, like the bucket-level
                           shift), so both K4 forms book it at a listed cell */
                        if (sel != bid && c->cfg.energy_split)
                            c->edep[src] += (double)((e_center(c, ebin_of(c, bid, l)) -
                                                      e_center(c, ebin_of(c, sel, le))) * v[l]);
                        po->val[((size_t)cell * c->Kb + os) * c->L + le] += v[l];
                    }
                }
            }
        }
    }
}

/* ------------------------------------------------------------------------- */
/* K1_ActiveMask (k1_activemask.cu:6-48) and the list compaction            */
/* (k1k6_pipeline.cu:589-665) in ascending cell order                        */
/* ------------------------------------------------------------------------- */
static void k1_and_lists(orc_ctx* c, int b_on, int b_off) {
    psi_buf* pi = psi_in(c);
    c->n_active = 0;
    c->n_coarse = 0;
    for (int cell = 0; cell < c->Nc; ++cell) {
        if (!pi->occ[cell]) { c->mask[cell] = 0; continue; }
        float W = 0.0f;
        int on = 0, off = 0, has_w = 0;
        const uint32_t* ids = &pi->bid[(size_t)cell * c->Kb];
        for (int s = 0; s < c->Kb; ++s) {
            if (ids[s] == ORC_EMPTY) continue;
            uint32_t bE = (ids[s] >> 12) & 0xFFFu;
            if (bE <= (uint32_t)b_on) on = 1;
            if (bE <= (uint32_t)b_off) off = 1;
            const real* v = &pi->val[((size_t)cell * c->Kb + s) * c->L];
            for (int l = 0; l < c->L; ++l) {
                W += (float)v[l];
                if (v[l] > RL(0.0)) has_w = 1;
            }
        }
        int prev = c->mask_prev[cell] != 0;
        int fine = on || (prev && off);
        c->mask[cell] = (fine && W > c->cfg.weight_active_min) ? 1 : 0;
        if (c->mask[cell] == 1) c->active[c->n_active++] = (uint32_t)cell;
        else if (has_w) c->coarse[c->n_coarse++] = (uint32_t)cell;
    }
}

static int e_bin_threshold(const orc_ctx* c, float E) {   /* compute_b_E_threshold */
    /* EnergyGrid::FindBin on the float edges */
    const real* e = c->E_edges;
    int N = c->N_E, b;
    if ((real)E < e[0]) b = 0;
    else if ((real)E >= e[N]) b = N - 1;
    else {
        int lo = 0, hi = N;
        while (lo < hi) {
            int mid = (lo + hi) / 2;
            if (e[mid + 1] <= (real)E) lo = mid + 1; else hi = mid;
        }
        b = lo;
    }
    return b / c->cfg.ne_local;
}

/* psi W/E totals (k1k6_pipeline.cu:706-768) */
static void psi_totals(const orc_ctx* c, const psi_buf* p, double* W, double* E) {
    *W = 0.0;
    *E = 0.0;
    for (int cell = 0; cell < c->Nc; ++cell) {
        if (!p->occ[cell]) continue;
        for (int s = 0; s < c->Kb; ++s) {
            uint32_t bid = p->bid[(size_t)cell * c->Kb + s];
            if (bid == ORC_EMPTY) continue;
            int bE = (int)((bid >> 12) & 0xFFFu);
            for (int l = 0; l < c->L; ++l) {
                real w = p->val[((size_t)cell * c->Kb + s) * c->L + l];
                if (w <= RL(0.0)) continue;
                int El = (l / c->cfg.nt_local) % c->cfg.ne_local;
                int Eb = bE * c->cfg.ne_local + El;
                if (Eb < 0) Eb = 0;
                if (Eb > c->N_E - 1) Eb = c->N_E - 1;
                real Ec = c->E_edges[Eb] + RL(0.5) * (c->E_edges[Eb + 1] - c->E_edges[Eb]);
                *W += (double)w;
                *E += (double)w * (double)Ec;
            }
        }
    }
}

/* K5_ConservationAudit: k5_audit.cu:22-167 */
static void k5(orc_ctx* c, float drop_w, double drop_e, int include_source) {
    orc_audit* r = &c->audit;
    memset(r, 0, sizeof(*r));
    psi_buf *pi = psi_in(c), *po = psi_out(c);
    for (int cell = 0; cell < c->Nc; ++cell) {
        double Wi = 0, Wo = 0, Ei = 0, Eo = 0;
        for (int pass = 0; pass < 2; ++pass) {
            psi_buf* p = pass ? po : pi;
            if (!p->occ[cell]) continue;
            for (int s = 0; s < c->Kb; ++s) {
                uint32_t bid = p->bid[(size_t)cell * c->Kb + s];
                if (bid == ORC_EMPTY) continue;
                uint32_t bE = (bid >> 12) & 0xFFFu;
                for (int l = 0; l < c->L; ++l) {
                    real w = p->val[((size_t)cell * c->Kb + s) * c->L + l];
                    if (w <= RL(0.0)) continue;
                    int El = (l / c->cfg.nt_local) % c->cfg.ne_local;
                    int Eb = (int)bE * c->cfg.ne_local + El;
                    if (Eb < 0) Eb = 0;
                    if (Eb > c->N_E - 1) Eb = c->N_E - 1;
                    real Ec = c->E_edges[Eb] + RL(1.0) * (RL(0.5) * (c->E_edges[Eb + 1] - c->E_edges[Eb]));
                    if (pass) { Wo += (double)w; Eo += (double)w * (double)Ec; }
                    else { Wi += (double)w; Ei += (double)w * (double)Ec; }
                }
            }
        }
        const int pf = c->cfg.precision_form;
        float Wc = fmaxf(0.0f, pf ? c->dw_cut[cell] : c->w_cut[cell] - c->p_w_cut[cell]);
        float Wn = fmaxf(0.0f, pf ? c->dw_nuc[cell] : c->w_nuc[cell] - c->p_w_nuc[cell]);
        float Wb = fmaxf(0.0f, pf ? c->dw_bnd[cell] : c->w_bnd[cell] - c->p_w_bnd[cell]);
        double Ed = fmax(0.0, c->edep[cell] - c->p_edep[cell]);
        double En = fmax(0.0, c->e_nuc[cell] - c->p_e_nuc[cell]);
        double Eb = fmax(0.0, c->e_bnd[cell] - c->p_e_bnd[cell]);
        double Ecut = fmax(0.0, c->e_cut[cell] - c->p_e_cut[cell]);
        r->W_in_total += (float)Wi;
        r->W_out_total += (float)Wo;
        r->W_cutoff_total += Wc;
        r->W_nuclear_total += Wn;
        r->W_boundary_total += Wb;
        r->E_in_total += Ei;
        r->E_out_total += Eo;
        r->E_dep_total += Ed;
        r->E_cutoff_total += Ecut;
        r->E_nuclear_total += En;
        r->E_boundary_total += Eb;
    }
    r->W_transport_drop_total += fmaxf(0.0f, drop_w);
    r->E_transport_drop_total += fmax(0.0, drop_e);
    if (include_source) {
        float wso = fmaxf(0.0f, c->src_oog_w), wss = fmaxf(0.0f, c->src_slot_w);
        double eso = fmax(0.0, c->src_oog_e), ess = fmax(0.0, c->src_slot_e);
        r->W_in_total += wso + wss;
        r->E_in_total += eso + ess;
        r->W_source_out_of_grid_total += wso;
        r->W_source_slot_drop_total += wss;
        r->E_source_out_of_grid_total += eso;
        r->E_source_slot_drop_total += ess;
    }
    r->processed_cells = c->Nc;
    float Wr = r->W_out_total + r->W_cutoff_total + r->W_nuclear_total + r->W_boundary_total +
               r->W_transport_drop_total + r->W_source_out_of_grid_total + r->W_source_slot_drop_total;
    float Wabs = fabsf(r->W_in_total - Wr);
    float Wrel = Wabs / fmaxf(r->W_in_total, 1e-20f);
    r->W_error = Wrel;
    r->W_pass = (isfinite(Wrel) && Wrel < 1e-6f) ? 1 : 0;
    double Er = r->E_out_total + r->E_dep_total + r->E_cutoff_total + r->E_nuclear_total +
                r->E_boundary_total + r->E_transport_drop_total + r->E_source_out_of_grid_total +
                r->E_source_slot_drop_total;
    double Eabs = fabs(r->E_in_total - Er);
    float Erel = (float)(Eabs / fmax(r->E_in_total, 1e-20));
    r->E_error = Erel;
    r->E_pass = (isfinite(Erel) && Erel < 1e-5f) ? 1 : 0;
    double resid = r->E_in_total - Er;
    if (isfinite(resid)) c->audit_residual += resid;
}

/* ------------------------------------------------------------------------- */
/* buffers                                                                   */
/* ------------------------------------------------------------------------- */
static void psi_clear(orc_ctx* c, psi_buf* p) {
    for (int cell = 0; cell < c->Nc; ++cell) {
        if (!p->occ[cell]) continue;
        for (int s = 0; s < c->Kb; ++s) {
            size_t k = (size_t)cell * c->Kb + s;
            if (p->bid[k] != ORC_EMPTY) {
                memset(&p->val[k * c->L], 0, sizeof(real) * c->L);
                p->bid[k] = ORC_EMPTY;
            }
        }
        /* values of a slot are only ever written after its claim, so
         * zeroing the claimed slots clears the cell */
        p->occ[cell] = 0;
    }
}

static void prepare_buckets(orc_ctx* c, const uint32_t* list, int n) {
    c->claim_batch++;
    for (int i = 0; i < c->Nc; ++i) c->cell_to_bucket[i] = -1;
    if (n * 4 > c->n_buckets_cap) {
        for (int i = 0; i < c->n_buckets_cap; ++i) {
            free(c->buckets[i].val);
            free(c->buckets[i].bid);
            free(c->buckets[i].count);
        }
        free(c->buckets);
        c->n_buckets_cap = n * 4;
        c->buckets = (bucket*)calloc((size_t)c->n_buckets_cap, sizeof(bucket));
        for (int i = 0; i < c->n_buckets_cap; ++i) {
            c->buckets[i].val = (real*)calloc((size_t)c->Kb * c->L, sizeof(real));
            c->buckets[i].bid = (uint32_t*)calloc((size_t)c->Kb, sizeof(uint32_t));
            c->buckets[i].count = (uint16_t*)calloc((size_t)c->Kb, sizeof(uint16_t));
        }
    }
    for (int i = 0; i < n; ++i) c->cell_to_bucket[list[i]] = i * 4;
    for (int b = 0; b < n * 4; ++b) {
        for (int s = 0; s < c->Kb; ++s) { c->buckets[b].bid[s] = ORC_EMPTY; c->buckets[b].count[s] = 0; }
        memset(c->buckets[b].val, 0, sizeof(real) * c->Kb * c->L);
    }
}

static size_t count_slots(const orc_ctx* c, const psi_buf* p, int cell) {
    size_t n = 0;
    for (int s = 0; s < c->Kb; ++s) if (p->bid[(size_t)cell * c->Kb + s] != ORC_EMPTY) ++n;
    return n;
}

/* one pipeline iteration, k1k6_pipeline.cu:1606-2038 */
int orc_step(orc_ctx* c) {
    if (c->finished) return 0;
    c->iter++;
    memcpy(c->mask_prev, c->mask, (size_t)c->Nc);
    int b_on = e_bin_threshold(c, c->cfg.E_fine_on);
    int b_off = e_bin_threshold(c, c->cfg.E_fine_off);
    k1_and_lists(c, b_on, b_off);
    int light = 0;
    if (c->cfg.stop_weight_fraction > 0.0f && c->iter > 1) {
        double W, E;
        psi_totals(c, psi_in(c), &W, &E);
        light = W < (double)c->cfg.stop_weight_fraction * (double)c->src_inj_w;
    }
    if ((c->n_active == 0 && c->n_coarse == 0) || light) {
        double W, E;
        psi_totals(c, psi_in(c), &W, &E);
        if (W > 0.0 || E > 0.0) { c->transport_drop_w += W; c->transport_drop_e += E; }
        c->finished = 1;
        c->iter--;   /* the terminating pass does no transport */
        return 0;
    }
    psi_clear(c, psi_out(c));
    if (c->track_claims) claims_reset(c);
    c->k2_slot_w = c->k2_slot_e = c->k2_bkt_w = c->k2_bkt_e = c->k2_prune_w = c->k2_prune_e = 0.0;
    c->k3_slot_w = c->k3_slot_e = c->k3_bkt_w = c->k3_bkt_e = c->k3_prune_w = c->k3_prune_e = 0.0;
    c->k4_slot_w = c->k4_slot_e = 0.0;
    psi_buf* pi = psi_in(c);
    for (int i = 0; i < c->n_coarse; ++i) c->slots_in += (double)count_slots(c, pi, (int)c->coarse[i]);
    for (int i = 0; i < c->n_active; ++i) c->slots_in += (double)count_slots(c, pi, (int)c->active[i]);
    c->cell_steps += c->n_active + c->n_coarse;
    if (c->n_coarse > 0) {
        prepare_buckets(c, c->coarse, c->n_coarse);
        for (int i = 0; i < c->n_coarse; ++i) k2_cell(c, (int)c->coarse[i]);
        k4(c);
    }
    if (c->n_active > 0) {
        prepare_buckets(c, c->active, c->n_active);
        for (int i = 0; i < c->n_active; ++i) k3_cell(c, (int)c->active[i]);
        k4(c);
    }
    psi_buf* po = psi_out(c);
    for (int cell = 0; cell < c->Nc; ++cell) if (po->occ[cell]) c->slots_out += (double)count_slots(c, po, cell);
    double dw = c->k2_slot_w + c->k2_bkt_w + c->k3_slot_w + c->k3_bkt_w + c->k4_slot_w + c->k2_prune_w + c->k3_prune_w;
    double de = c->k2_slot_e + c->k2_bkt_e + c->k3_slot_e + c->k3_bkt_e + c->k4_slot_e + c->k2_prune_e + c->k3_prune_e;
    {
        const double cw[3][3] = {{c->k2_slot_w, c->k2_bkt_w, c->k2_prune_w},
                                 {c->k3_slot_w, c->k3_bkt_w, c->k3_prune_w},
                                 {c->k4_slot_w, 0.0, 0.0}};
        const double ce[3][3] = {{c->k2_slot_e, c->k2_bkt_e, c->k2_prune_e},
                                 {c->k3_slot_e, c->k3_bkt_e, c->k3_prune_e},
                                 {c->k4_slot_e, 0.0, 0.0}};
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                c->cum_drop_w[a][b] += cw[a][b];
                c->cum_drop_e[a][b] += ce[a][b];
            }
    }
    c->transport_drop_w += dw;
    c->transport_drop_e += de;
    k5(c, (float)dw, de, c->iter == 1);
    memcpy(c->p_w_cut, c->w_cut, sizeof(float) * c->Nc);
    memset(c->dw_cut, 0, sizeof(float) * c->Nc);
    memset(c->dw_nuc, 0, sizeof(float) * c->Nc);
    memset(c->dw_bnd, 0, sizeof(float) * c->Nc);
    memcpy(c->p_e_cut, c->e_cut, sizeof(double) * c->Nc);
    memcpy(c->p_w_nuc, c->w_nuc, sizeof(float) * c->Nc);
    memcpy(c->p_w_bnd, c->w_bnd, sizeof(float) * c->Nc);
    memcpy(c->p_edep, c->edep, sizeof(double) * c->Nc);
    memcpy(c->p_e_nuc, c->e_nuc, sizeof(double) * c->Nc);
    memcpy(c->p_e_bnd, c->e_bnd, sizeof(double) * c->Nc);
    c->in_idx = 1 - c->in_idx;      /* K6 */
    psi_clear(c, psi_out(c));
    return 1;
}

int orc_run(orc_ctx* c, int max_it) {
    int n = 0;
    while (n < max_it && orc_step(c)) ++n;
    return n;
}

/* ------------------------------------------------------------------------- */
/* source injection                                                          */
/* ------------------------------------------------------------------------- */
/* device_psic_inject_source: device_psic.cuh:347-450 */
static int inject_one(orc_ctx* c, int cell, real theta, real E, real weight, real x, real z) {
    if (weight <= RL(0.0)) return 0;
    if (cell < 0 || cell >= c->Nc) return 0;
    real dx = (real)c->cfg.dx, dz = (real)c->cfg.dz;
    x = r_max(RL(0.0), r_min(x, dx));
    z = r_max(RL(0.0), r_min(z, dz));
    int xs = sub_bin(x - dx * RL(0.5), dx, c->cfg.nx_sub);
    int zs = sub_bin(z - dz * RL(0.5), dz, c->cfg.nz_sub);
    real tmin = c->th_edges[0], tmax = c->th_edges[c->N_theta];
    real Emin = c->E_edges[0], Emax = c->E_edges[c->N_E];
    theta = r_max(tmin, r_min(theta, tmax));
    E = r_max(Emin, r_min(E, Emax));
    real dth = (tmax - tmin) / (real)c->N_theta;
    real cont = (theta - tmin) / dth;
    int tb = (int)cont;
    real ft = cont - (real)tb;
    int Eb;
    if (E <= c->E_edges[0]) Eb = 0;
    else if (E >= c->E_edges[c->N_E]) Eb = c->N_E - 1;
    else {
        int lo = 0, hi = c->N_E;
        while (lo < hi) {
            int mid = (lo + hi) / 2;
            if (c->E_edges[mid + 1] <= E) lo = mid + 1; else hi = mid;
        }
        Eb = lo;
    }
    real Elo = c->E_edges[Eb], Ehi = c->E_edges[Eb + 1];
    real fE = (Ehi - Elo) > RL(1e-10) ? (E - Elo) / (Ehi - Elo) : RL(0.0);
    if (tb >= c->N_theta - 1) { tb = c->N_theta - 1; ft = RL(0.0); }
    if (Eb >= c->N_E - 1) { Eb = c->N_E - 1; fE = RL(0.0); }
    if (ft >= RL(0.5) && tb < c->N_theta - 1) tb++;
    if (fE >= RL(0.5) && Eb < c->N_E - 1) Eb++;
    uint32_t want = enc_block((uint32_t)(tb / c->cfg.nt_local), (uint32_t)(Eb / c->cfg.ne_local));
    int l = enc_lidx(c, tb % c->cfg.nt_local, Eb % c->cfg.ne_local, xs, zs);
    psi_buf* p = psi_in(c);
    uint32_t* ids = &p->bid[(size_t)cell * c->Kb];
    int slot = -1;
    for (int s = 0; s < c->Kb; ++s) {            /* device_psic_find_or_allocate_slot */
        if (ids[s] == ORC_EMPTY) { ids[s] = want; slot = s; break; }
        if (ids[s] == want) { slot = s; break; }
    }
    if (slot < 0) return 0;
    p->occ[cell] = 1;
    p->val[((size_t)cell * c->Kb + slot) * c->L + l] += weight;
    return 1;
}

/* gaussian_sample of the source kernel: k1k6_pipeline.cu:433-447 */
static float src_gauss(unsigned* seed) {
    *seed = 1664525u * *seed + 1013904223u;
    float u1 = (float)(*seed >> 16) / 65536.0f;
    *seed = 1664525u * *seed + 1013904223u;
    float u2 = (float)(*seed >> 16) / 65536.0f;
    float r = sqrtf(-2.0f * logf(fmaxf(u1, 1e-10f)));
    float th = (float)(2.0f * 3.14159265358979323846 * (double)u2);
    return r * cosf(th);
}

void orc_inject(orc_ctx* c, float x0, float z0, float theta0, float E0, float W,
                float sx, float sth, float sE, int n_samples, unsigned seed) {
    int gaussian = (n_samples > 1) || (sx > 0.0f) || (sth > 0.0f);   /* wrapper.cu:246 */
    float dx = c->cfg.dx, dz = c->cfg.dz, x_min = c->cfg.x_min, z_min = c->cfg.z_min;
    int Nx = c->cfg.Nx, Nz = c->cfg.Nz;
    c->src_inj_w = gaussian ? 0.0f : W;
    c->src_oog_w = c->src_slot_w = 0.0f;
    c->src_inj_e = (double)E0 * (double)c->src_inj_w;
    c->src_oog_e = c->src_slot_e = 0.0;
    if (!gaussian) {                                   /* inject_source_kernel pencil branch */
        float xr = x0 - x_min, zr = z0 - z_min;
        int sx_ = (int)(xr / dx), sz_ = (int)(zr / dz);
        sx_ = sx_ < 0 ? 0 : (sx_ >= Nx ? Nx - 1 : sx_);
        sz_ = sz_ < 0 ? 0 : (sz_ >= Nz ? Nz - 1 : sz_);
        inject_one(c, sz_ * Nx + sx_, (real)theta0, (real)E0, (real)W,
                   (real)(xr - sx_ * dx), (real)(zr - sz_ * dz));
    } else {                                           /* inject_gaussian_source_kernel */
        for (int i = 0; i < n_samples; ++i) {
            unsigned s = seed + (unsigned)i;
            float xs = x0 + sx * src_gauss(&s);
            float ts = theta0 + sth * src_gauss(&s);
            float Es = E0 + sE * src_gauss(&s);
            Es = fmaxf((float)c->E_edges[0], fminf(Es, (float)c->E_edges[c->N_E]));
            ts = fmaxf((float)c->th_edges[0], fminf(ts, (float)c->th_edges[c->N_theta]));
            float xr = xs - x_min, zr = z0 - z_min;
            int ix = (int)(xr / dx), iz = (int)(zr / dz);
            float ws = W / n_samples;
            if (ix < 0 || ix >= Nx || iz < 0 || iz >= Nz) {
                c->src_oog_w += ws;
                c->src_oog_e += (double)(Es * ws);
                continue;
            }
            int ok = inject_one(c, iz * Nx + ix, (real)ts, (real)Es, (real)ws,
                                (real)(xr - ix * dx), (real)(zr - iz * dz));
            if (ok) { c->src_inj_w += ws; c->src_inj_e += (double)(Es * ws); }
            else { c->src_slot_w += ws; c->src_slot_e += (double)(Es * ws); }
        }
    }
    double W_rep, E_rep;
    psi_totals(c, psi_in(c), &W_rep, &E_rep);
    double loss = c->src_inj_e - E_rep;
    if (fabs(loss) < 1e-12) loss = 0.0;
    c->src_rep_loss = loss;
}

/* inject_source_kernel with its spreads (k1k6_pipeline.cu:300-427), one
 * thread, in its loop order: the 7 angle nodes (k1k6_pipeline.cu:316-318)
 * when sigma_theta > 1e-4, and for each the cells within +-4 sigma_x of x0,
 * weighted by the Gaussian at their centres over the float sum of those
 * weights.  Without spreads it is the pencil branch.  Accounting as the
 * wrapper books a non-Gaussian source (W and E0 W injected). */
static const float kGhAbscissa[7] = {-2.65f, -1.67f, -0.82f, 0.0f, 0.82f, 1.67f, 2.65f};
static const float kGhWeight[7] = {0.0105f, 0.0769f, 0.2448f, 0.3357f, 0.2448f, 0.0769f, 0.0105f};

void orc_inject_quadrature(orc_ctx* c, float x0, float z0, float theta0, float sth, float E0, float W, float sx) {
    int ang = sth > 0.0001f, spat = sx > 0.01f;
    if (!ang && !spat) {
        orc_inject(c, x0, z0, theta0, E0, W, 0.0f, 0.0f, 0.0f, 1, 0u);
        return;
    }
    float dx = c->cfg.dx, dz = c->cfg.dz, x_min = c->cfg.x_min, z_min = c->cfg.z_min;
    int Nx = c->cfg.Nx, Nz = c->cfg.Nz;
    c->src_inj_w = W;
    c->src_inj_e = (double)E0 * (double)W;
    c->src_oog_w = c->src_slot_w = 0.0f;
    c->src_oog_e = c->src_slot_e = 0.0;
    float lo = x0 - 4.0f * sx, hi = x0 + 4.0f * sx;
    int ix0 = (int)((lo - x_min) / dx), ix1 = (int)((hi - x_min) / dx) + 1;
    if (ix0 < 0) ix0 = 0;
    if (ix1 > Nx) ix1 = Nx;
    real total = RL(0.0);
    for (int ix = ix0; ix < ix1; ++ix) {
        real d = ((real)x_min + ((real)ix + RL(0.5)) * (real)dx) - (real)x0;
        total += r_exp(RL(-0.5) * d * d / ((real)sx * (real)sx)) * (real)dx;
    }
    if (total <= RL(0.0)) total = RL(1.0);
    float zr = z0 - z_min;
    int cz = (int)(zr / dz);
    cz = cz < 0 ? 0 : (cz >= Nz ? Nz - 1 : cz);
    for (int it = 0; it < (ang ? 7 : 1); ++it) {
        real th = ang ? (real)theta0 + (real)kGhAbscissa[it] * (real)sth : (real)theta0;
        real wt = ang ? (real)kGhWeight[it] : RL(1.0);
        for (int ix = ix0; ix < ix1; ++ix) {
            real d = ((real)x_min + ((real)ix + RL(0.5)) * (real)dx) - (real)x0;
            real wx = (r_exp(RL(-0.5) * d * d / ((real)sx * (real)sx)) * (real)dx) / total;
            inject_one(c, cz * Nx + ix, th, (real)E0, (real)W * wt * wx, (real)dx * RL(0.5),
                       (real)zr - (real)cz * (real)dz);
        }
    }
    double W_rep, E_rep;
    psi_totals(c, psi_in(c), &W_rep, &E_rep);
    double loss = c->src_inj_e - E_rep;
    if (fabs(loss) < 1e-12) loss = 0.0;
    c->src_rep_loss = loss;
}

/* ------------------------------------------------------------------------- */
/* context lifecycle and accessors                                           */
/* ------------------------------------------------------------------------- */
void orc_get_drop_channels(const orc_ctx* c, double* w9, double* e9) {
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            w9[3 * a + b] = c->cum_drop_w[a][b];
            e9[3 * a + b] = c->cum_drop_e[a][b];
        }
}

orc_ctx* orc_create(const orc_config* cfg, int N_theta, const float* th_edges, int N_E, const float* E_edges) {
    orc_ctx* c = (orc_ctx*)calloc(1, sizeof(orc_ctx));
    c->cfg = *cfg;
    c->L = cfg->nt_local * cfg->ne_local * cfg->nx_sub * cfg->nz_sub;
    c->Kb = cfg->slots_per_cell > 0 ? cfg->slots_per_cell : 32;
    c->Nc = cfg->Nx * cfg->Nz;
    c->N_theta = N_theta;
    c->N_E = N_E;
    c->th_edges = (real*)malloc(sizeof(real) * (N_theta + 1));
    c->E_edges = (real*)malloc(sizeof(real) * (N_E + 1));
    for (int i = 0; i <= N_theta; ++i) c->th_edges[i] = (real)th_edges[i];
    for (int i = 0; i <= N_E; ++i) c->E_edges[i] = (real)E_edges[i];
    /* R-LUT on the transport energy grid (gpu_transport_runner.cpp:145) */
    float *rep = (float*)malloc(sizeof(float) * N_E), *tmp = (float*)malloc(sizeof(float) * 5 * N_E);
    for (int i = 0; i < N_E; ++i) rep[i] = sqrtf(E_edges[i] * E_edges[i + 1]);
    orc_generate_rlut(N_E, rep, tmp, tmp + N_E, tmp + 2 * N_E, tmp + 3 * N_E, tmp + 4 * N_E);
    c->lut.N = N_E;
    c->lut.Emin = cfg->grid_E_min > 0.0f ? cfg->grid_E_min : E_edges[0];
    c->lut.Emax = cfg->grid_E_max > 0.0f ? cfg->grid_E_max : E_edges[N_E];
    real** dst[5] = {&c->lut.R, &c->lut.S, &c->lut.logE, &c->lut.logR, &c->lut.logS};
    for (int k = 0; k < 5; ++k) {
        *dst[k] = (real*)malloc(sizeof(real) * N_E);
        for (int i = 0; i < N_E; ++i) (*dst[k])[i] = (real)tmp[k * N_E + i];
    }
    c->lut.edges = c->E_edges;
    c->lut.precise = 0;
    c->lut.R_prec = lut_R(&c->lut, r_max(RL(10.0), (real)c->lut.Emin));
    c->lut.precise = cfg->precision_form ? 1 : 0;
    free(rep);
    free(tmp);
    c->fe_A = (float*)calloc(cfg->Nz, sizeof(float));
    c->fe_B = (float*)calloc(cfg->Nz, sizeof(float));
    c->fe_sigma = (float*)calloc(cfg->Nz, sizeof(float));
    orc_fe_precompute(cfg->E0, cfg->Nz, cfg->dz, cfg->sigma_x_initial, c->fe_A, c->fe_B, c->fe_sigma);
    size_t ns = (size_t)c->Nc * c->Kb;
    for (int b = 0; b < 2; ++b) {
        c->buf[b].bid = (uint32_t*)malloc(sizeof(uint32_t) * ns);
        memset(c->buf[b].bid, 0xFF, sizeof(uint32_t) * ns);
        c->buf[b].val = (real*)calloc(ns * c->L, sizeof(real));
        c->buf[b].occ = (uint8_t*)calloc(c->Nc, 1);
    }
    c->mask = (uint8_t*)calloc(c->Nc, 1);
    c->mask_prev = (uint8_t*)calloc(c->Nc, 1);
    c->active = (uint32_t*)calloc(c->Nc, sizeof(uint32_t));
    c->coarse = (uint32_t*)calloc(c->Nc, sizeof(uint32_t));
    c->edep = (double*)calloc(c->Nc, sizeof(double));
    c->e_cut = (double*)calloc(c->Nc, sizeof(double));
    c->e_nuc = (double*)calloc(c->Nc, sizeof(double));
    c->e_bnd = (double*)calloc(c->Nc, sizeof(double));
    c->w_cut = (float*)calloc(c->Nc, sizeof(float));
    c->w_nuc = (float*)calloc(c->Nc, sizeof(float));
    c->w_bnd = (float*)calloc(c->Nc, sizeof(float));
    c->p_edep = (double*)calloc(c->Nc, sizeof(double));
    c->p_e_cut = (double*)calloc(c->Nc, sizeof(double));
    c->p_e_nuc = (double*)calloc(c->Nc, sizeof(double));
    c->p_e_bnd = (double*)calloc(c->Nc, sizeof(double));
    c->p_w_cut = (float*)calloc(c->Nc, sizeof(float));
    c->p_w_nuc = (float*)calloc(c->Nc, sizeof(float));
    c->p_w_bnd = (float*)calloc(c->Nc, sizeof(float));
    c->dw_cut = (float*)calloc(c->Nc, sizeof(float));
    c->dw_nuc = (float*)calloc(c->Nc, sizeof(float));
    c->dw_bnd = (float*)calloc(c->Nc, sizeof(float));
    c->cell_to_bucket = (int*)malloc(sizeof(int) * c->Nc);
    for (int i = 0; i < c->Nc; ++i) c->cell_to_bucket[i] = -1;
    return c;
}

void orc_destroy(orc_ctx* c) {
    if (!c) return;
    free(c->th_edges); free(c->E_edges);
    free(c->lut.R); free(c->lut.S); free(c->lut.logE); free(c->lut.logR); free(c->lut.logS);
    free(c->fe_A); free(c->fe_B); free(c->fe_sigma);
    free(c->rho); free(c->wet);
    free(c->net);
    for (int b = 0; b < 2; ++b) { free(c->buf[b].bid); free(c->buf[b].val); free(c->buf[b].occ); }
    free(c->mask); free(c->mask_prev); free(c->active); free(c->coarse);
    free(c->edep); free(c->e_cut); free(c->e_nuc); free(c->e_bnd);
    free(c->w_cut); free(c->w_nuc); free(c->w_bnd);
    free(c->p_edep); free(c->p_e_cut); free(c->p_e_nuc); free(c->p_e_bnd);
    free(c->p_w_cut); free(c->p_w_nuc); free(c->p_w_bnd);
    free(c->dw_cut); free(c->dw_nuc); free(c->dw_bnd);
    for (int i = 0; i < c->n_buckets_cap; ++i) {
        free(c->buckets[i].val);
        free(c->buckets[i].bid);
        free(c->buckets[i].count);
    }
    free(c->buckets);
    free(c->cell_to_bucket);
    free(c->ck);
    free(c->cc);
    free(c);
}

/* K3's per-component redistribution (the surrogate's training targets):
 * energy loss over the water-equivalent path from the R-LUT
 * (lut_energy_deposition, device_lut.cuh:145-151), straggling sigma
 * (device_physics.cuh:157-216) and the Highland angle (device_physics.cuh:50-72)
 * of the step, integrated with the transport's Gaussian CDF over 8 theta bins
 * centred on the incoming direction and 4 log-energy bins below the incoming
 * energy, tails folded into the end bins. */
void orc_redistribution_table(const orc_ctx* c, int n, const float* feats, float* out) {
    (void)c;
    const real cap1[4] = {RL(1.0), RL(0.0), RL(-1.0), RL(-2.0)}, cap0[4] = {RL(2.0), RL(1.0), RL(0.0), RL(-1.0)};
    for (int i = 0; i < n; ++i) {
        const real s = feats[4 * i], u = feats[4 * i + 1], r = feats[4 * i + 2], cap = feats[4 * i + 3];
        real Mt[SM2D_RD_NT], Me[SM2D_RD_NE];
        sm2d_rd_theta(r_max(s, RL(0.0)), Mt);
        sm2d_rd_energy(u, r_max(r, RL(0.0)), cap > RL(0.5) ? cap1 : cap0, SM2D_RD_NE - 1, Me);
        for (int e = 0; e < SM2D_RD_NE; ++e)
            for (int t = 0; t < SM2D_RD_NT; ++t) out[32 * (size_t)i + t + 8 * e] = (float)(Mt[t] * Me[e]);
    }
}

int orc_local_bins(const orc_ctx* c) { return c->L; }
int orc_slots_per_cell(const orc_ctx* c) { return c->Kb; }

/* Slab phantom: density of each depth row (NULL: water again).  Recomputes
 * the Fermi-Eyges tables through the phantom. */
void orc_set_density(orc_ctx* c, const float* rho) {
    free(c->rho); free(c->wet);
    c->rho = c->wet = NULL;
    if (rho) {
        const int Nz = c->cfg.Nz;
        c->rho = (float*)malloc(sizeof(float) * Nz);
        c->wet = (float*)malloc(sizeof(float) * Nz);
        memcpy(c->rho, rho, sizeof(float) * Nz);
        float acc = 0.0f;
        for (int iz = 0; iz < Nz; ++iz) {
            c->wet[iz] = acc;
            acc += rho[iz] * c->cfg.dz;
        }
    }
    orc_fe_precompute_density(c->cfg.E0, c->cfg.Nz, c->cfg.dz, c->cfg.sigma_x_initial, c->rho, c->fe_A, c->fe_B,
                              c->fe_sigma);
}

void orc_set_psi_in(orc_ctx* c, const uint32_t* bid, const orc_real* val) {
    psi_buf* p = psi_in(c);
    size_t ns = (size_t)c->Nc * c->Kb;
    memcpy(p->bid, bid, sizeof(uint32_t) * ns);
    memcpy(p->val, val, sizeof(real) * ns * c->L);
    for (int cell = 0; cell < c->Nc; ++cell) {
        p->occ[cell] = 0;
        for (int s = 0; s < c->Kb; ++s) if (p->bid[(size_t)cell * c->Kb + s] != ORC_EMPTY) p->occ[cell] = 1;
    }
}

void orc_get_psi_in(const orc_ctx* c, uint32_t* bid, orc_real* val) {
    const psi_buf* p = &c->buf[c->in_idx];
    size_t ns = (size_t)c->Nc * c->Kb;
    memcpy(bid, p->bid, sizeof(uint32_t) * ns);
    if (val) memcpy(val, p->val, sizeof(real) * ns * c->L);
}

/* K4 on caller arrays, the checker of the raw K4 entry: nb buckets of Kb
 * ids (bbid) and Kb x L values (bval), c2b[Nc] the first of a listed cell's
 * four buckets (faces +z, -z, +x, -x; -1: not listed); the psi_out ids and
 * values are updated in place and drop2[0..1] gains the weight and energy K4
 * could not place.  The buckets and psi_out stand in for the context's own
 * while k4 runs. */
void orc_k4_raw(orc_ctx* c, int nb, const uint32_t* bbid, const orc_real* bval, const int* c2b, uint32_t* obid,
                orc_real* oval, double* drop2) {
    bucket* saved_b = c->buckets;
    int* saved_c2b = c->cell_to_bucket;
    psi_buf* po = psi_out(c);
    const psi_buf saved_po = *po;
    bucket* tmp = (bucket*)calloc((size_t)(nb > 0 ? nb : 1), sizeof(bucket));
    uint8_t* occ = (uint8_t*)calloc((size_t)c->Nc, 1);
    for (int i = 0; i < nb; ++i) {
        tmp[i].bid = (uint32_t*)(bbid + (size_t)i * c->Kb);
        tmp[i].val = (real*)(bval + (size_t)i * c->Kb * c->L);
    }
    for (int cell = 0; cell < c->Nc; ++cell)
        for (int k = 0; k < c->Kb; ++k)
            if (obid[(size_t)cell * c->Kb + k] != ORC_EMPTY) occ[cell] = 1;
    c->buckets = tmp;
    c->cell_to_bucket = (int*)c2b;
    po->bid = obid;
    po->val = oval;
    po->occ = occ;
    const double w0 = c->k4_slot_w, e0 = c->k4_slot_e;
    k4(c);
    drop2[0] += c->k4_slot_w - w0;
    drop2[1] += c->k4_slot_e - e0;
    c->k4_slot_w = w0;
    c->k4_slot_e = e0;
    *po = saved_po;
    c->buckets = saved_b;
    c->cell_to_bucket = saved_c2b;
    free(occ);
    free(tmp);
}

void orc_get_mask(const orc_ctx* c, uint8_t* m) { memcpy(m, c->mask, (size_t)c->Nc); }

int orc_get_lists(const orc_ctx* c, uint32_t* a, int* na, uint32_t* co, int* nco) {
    *na = c->n_active;
    *nco = c->n_coarse;
    if (a) memcpy(a, c->active, sizeof(uint32_t) * c->n_active);
    if (co) memcpy(co, c->coarse, sizeof(uint32_t) * c->n_coarse);
    return c->n_active + c->n_coarse;
}

void orc_get_tallies(const orc_ctx* c, double* edep, float* w_cut, double* e_cut,
                     float* w_nuc, double* e_nuc, float* w_bnd, double* e_bnd) {
    size_t n = (size_t)c->Nc;
    if (edep) memcpy(edep, c->edep, n * sizeof(double));
    if (w_cut) memcpy(w_cut, c->w_cut, n * sizeof(float));
    if (e_cut) memcpy(e_cut, c->e_cut, n * sizeof(double));
    if (w_nuc) memcpy(w_nuc, c->w_nuc, n * sizeof(float));
    if (e_nuc) memcpy(e_nuc, c->e_nuc, n * sizeof(double));
    if (w_bnd) memcpy(w_bnd, c->w_bnd, n * sizeof(float));
    if (e_bnd) memcpy(e_bnd, c->e_bnd, n * sizeof(double));
}

void orc_get_audit(const orc_ctx* c, orc_audit* out) { *out = c->audit; }

void orc_get_scalars(const orc_ctx* c, double* o) {
    o[0] = c->transport_drop_w; o[1] = c->transport_drop_e; o[2] = c->audit_residual;
    o[3] = c->src_inj_w; o[4] = c->src_inj_e; o[5] = c->src_oog_w; o[6] = c->src_oog_e;
    o[7] = c->src_slot_w; o[8] = c->src_slot_e; o[9] = c->src_rep_loss;
    o[10] = c->iter; o[11] = c->cell_steps; o[12] = c->slots_in; o[13] = c->slots_out;
}

void orc_get_fe(const orc_ctx* c, float* A, float* B, float* s) {
    memcpy(A, c->fe_A, sizeof(float) * c->cfg.Nz);
    memcpy(B, c->fe_B, sizeof(float) * c->cfg.Nz);
    memcpy(s, c->fe_sigma, sizeof(float) * c->cfg.Nz);
}

typedef struct run_job { orc_ctx** ctxs; int n, max_it, next; pthread_mutex_t mu; } run_job;

static void* run_worker(void* arg) {
    run_job* j = (run_job*)arg;
    for (;;) {
        pthread_mutex_lock(&j->mu);
        int k = j->next++;
        pthread_mutex_unlock(&j->mu);
        if (k >= j->n) break;
        orc_run(j->ctxs[k], j->max_it);
    }
    return NULL;
}

int orc_run_many(orc_ctx** ctxs, int n, int max_it, int n_threads) {
    if (n_threads < 1) n_threads = 1;
    run_job j;
    j.ctxs = ctxs; j.n = n; j.max_it = max_it; j.next = 0;
    pthread_mutex_init(&j.mu, NULL);
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * n_threads);
    for (int i = 0; i < n_threads; ++i) pthread_create(&th[i], NULL, run_worker, &j);
    for (int i = 0; i < n_threads; ++i) pthread_join(th[i], NULL);
    free(th);
    pthread_mutex_destroy(&j.mu);
    return n;
}

void orc_math(int fn, const float* x, float* y, int n) {
    for (int i = 0; i < n; ++i) {
        float v = x[i];
        y[i] = fn == 0 ? sm2d_expf(v) : fn == 1 ? sm2d_logf(v) : fn == 2 ? sm2d_sinf(v)
             : fn == 3 ? sm2d_cosf(v) : sm2d_erff(v);
    }
}
