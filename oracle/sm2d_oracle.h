/*
 * sm2d_oracle.h -- CPU oracle for the SM_2D deterministic phase-space
 * transport step (K1..K6).  TEST INFRASTRUCTURE ONLY: this code is the
 * checker that the CUDA path is compared against.  Nothing in the product
 * (sm_2d_gb300/) includes, links or calls it; only tests/, the smoke check
 * and the CPU-baseline leg of bench.py load it.
 *
 * It restates the reference kernels one function at a time, in the
 * reference's own arithmetic order, so that the float build reproduces the
 * reference GPU dumps (results/one_step_case_*) and the double build is the
 * FP64 oracle of the same method.  Every function cites the reference
 * file:line it follows.
 *
 * Pinning: the float build is checked against the reference GPU golden dumps
 * results/one_step_case_{A,B,C,D} and against fixtures generated from the
 * reference's host grid/LUT code (tests/golden/).
 */
#ifndef SM2D_ORACLE_H
#define SM2D_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#ifdef ORC_FP64
typedef double orc_real;
#else
typedef float orc_real;
#endif

#define ORC_KB 32          /* default slots per cell and per bucket (device_psic.cuh:30, device_bucket.cuh:26) */
#define ORC_EMPTY 0xFFFFFFFFu

typedef struct orc_config {
    /* spatial grid */
    int Nx, Nz;
    float dx, dz, x_min, z_min;
    /* local-bin layout: theta_local, E_local, x_sub, z_sub */
    int nt_local, ne_local, nx_sub, nz_sub;
    /* transport controls (TransportConfig, incident_particle_config.hpp:176) */
    float E_fine_on, E_fine_off, weight_active_min;
    float step_coarse;
    float sigma_x_initial;     /* beam sigma_x, used by K2 and the post-convolution */
    float E0;                  /* beam energy for the Fermi-Eyges precompute         */
    int enable_straggling, enable_nuclear;
    /* method options (0 = reference behaviour) */
    int seed_slot_mode;        /* 0: seed uses storage slot; 1: rank of bid in cell */
    int energy_split;          /* 0: single E bin + fold; 1: mean-preserving 2-bin  */
    /* EnergyGrid::E_min/E_max (the constructor arguments; DeviceRLUT takes
     * these, not edges[0]/edges[N]).  0 means "use the edges". */
    float grid_E_min, grid_E_max;
    /* weight below which K2 / K3 drop a component into the transport-drop
     * channel; 0 means the reference values 1e-12 / 1e-15 */
    float prune_coarse, prune_fine;
    /* energy-split method: a split part lighter than this stays in the major
     * bin (energy difference folded into the deposit); 0 = always split */
    float split_min_weight;
    /* stop when the in-flight weight falls below this fraction of the
     * injected weight (remainder booked as transport drop); 0 = reference
     * behaviour (stop only when no cell is listed) */
    float stop_weight_fraction;
    /* deposits lighter than this may claim only the first 24 slots of a
     * cell or bucket and otherwise merge into the nearest block, keeping 8
     * slots for heavy components; 0 = reference (all 32 claimable) */
    float claim_reserve_weight;
    /* block slots per cell (0 = 32, the reference's DEVICE_Kb) */
    int slots_per_cell;
    /* 1: a component whose new energy is below the lowest bin centre is
     * absorbed (cutoff) instead of being re-binned up to that centre, which
     * otherwise stalls it at the grid floor; 0 = reference */
    int floor_cutoff;
    /* 1: MCS / straggling seeds are salted with the iteration index
     * ((iter-1) * 0x9E3779B9, so the first iteration is unchanged); the
     * reference re-draws the same numbers for a bin every iteration */
    int seed_iteration_salt;
    /* 1: expectation form -- K2/K3 emit the expected result of re-binning
     * their MCS angle and straggling loss (sm2d_redist.h) instead of one
     * hashed draw of each; needs energy_split = 1 */
    int expectation;
    /* expectation form with the surrogate's table path (the GPU's
     * sm2d_set_surrogate with method_tables = 1): a K3 component whose energy
     * window has four centres of uniform spacing takes the plain table of its
     * features (s, u, r, cap) as its children's weights; 0 = closed forms */
    int surrogate_tables;   /* 2: the network of orc_set_surrogate instead of the plain table */
    /* precision form: the audit books each iteration's cutoff, nuclear and
     * boundary weight from the iteration's own per-cell increments, and the
     * R-LUT is inverted in double below 10 MeV; 0 = reference */
    int precision_form;
} orc_config;

typedef struct orc_audit {       /* AuditReport, k5_audit.cuh:5-27 */
    float W_error; int W_pass; float E_error; int E_pass;
    float W_in_total, W_out_total, W_cutoff_total, W_nuclear_total, W_boundary_total;
    float W_source_out_of_grid_total, W_source_slot_drop_total, W_transport_drop_total;
    double E_in_total, E_out_total, E_dep_total, E_cutoff_total, E_nuclear_total;
    double E_boundary_total, E_source_out_of_grid_total, E_source_slot_drop_total;
    double E_transport_drop_total;
    int processed_cells;
} orc_audit;

typedef struct orc_ctx orc_ctx;

/* ---- grids and tables (usable without a context) ---- */
int  orc_energy_grid_log(float E_min, float E_max, int N, float* edges, float* rep);
int  orc_energy_grid_piecewise(int n_groups, const float* groups /* 3*n */, float* edges, float* rep);
void orc_angular_grid(float th_min, float th_max, int N, float* edges, float* rep);
void orc_generate_rlut(int N_E, const float* rep, float* R, float* S,
                       float* logE, float* logR, float* logS);
void orc_fe_precompute(float E0, int Nz, float dz, float sigma_x0,
                       float* A, float* B, float* sigma_total);
/* the same through a density per depth row (rho[Nz]; NULL: water) */
void orc_fe_precompute_density(float E0, int Nz, float dz, float sigma_x0, const float* rho,
                               float* A, float* B, float* sigma_total);
void orc_postprocess(const double* edep_in, const float* sigma_total, float sigma_x0,
                     int Nx, int Nz, float dx, double* edep_out);
/* the transport's elementary functions (0 exp, 1 log, 2 sin, 3 cos, 4 erf)
 * as the oracle evaluates them on the host, for comparison with the CUDA
 * library's device results */
void orc_math(int fn, const float* x, float* y, int n);

/* ---- transport context ---- */
orc_ctx* orc_create(const orc_config* cfg, int N_theta, const float* theta_edges,
                    int N_E, const float* E_edges);
void orc_destroy(orc_ctx* c);
int  orc_local_bins(const orc_ctx* c);
int  orc_slots_per_cell(const orc_ctx* c);

/* source injection (k1k6_pipeline.cu:300-551, gpu_transport_wrapper.cu:339-460) */
void orc_inject(orc_ctx* c, float x0, float z0, float theta0, float E0, float W_total,
                float sigma_x, float sigma_theta, float sigma_E,
                int n_samples, unsigned seed);
/* inject_source_kernel with its spreads: the quadrature source
 * (k1k6_pipeline.cu:300-427) */
void orc_inject_quadrature(orc_ctx* c, float x0, float z0, float theta0, float sigma_theta, float E0,
                           float W_total, float sigma_x);
/* overwrite psi_in directly (golden inputs); values are orc_real */
void orc_set_psi_in(orc_ctx* c, const uint32_t* bid, const orc_real* val);
/* slab phantom: the density of each depth row (rho[Nz]; NULL: water).  Energy
 * loss, range limits, straggling, nuclear attenuation and scattering use the
 * water-equivalent path rho * step; the Fermi-Eyges tables are recomputed. */
void orc_set_density(orc_ctx* c, const float* rho);
void orc_get_psi_in(const orc_ctx* c, uint32_t* bid, orc_real* val);

/* one K1..K6 iteration; returns 1 if work was done, 0 if transport finished */
int  orc_step(orc_ctx* c);
int  orc_run(orc_ctx* c, int max_iterations);     /* returns iterations run */
void orc_get_mask(const orc_ctx* c, uint8_t* mask);
int  orc_get_lists(const orc_ctx* c, uint32_t* active, int* n_active,
                   uint32_t* coarse, int* n_coarse);
void orc_get_tallies(const orc_ctx* c, double* edep, float* w_cut, double* e_cut,
                     float* w_nuc, double* e_nuc, float* w_bnd, double* e_bnd);
void orc_get_audit(const orc_ctx* c, orc_audit* out);
/* the per-iteration drop channels of k2/k3/k4_get_debug_counters summed over
 * the iterations since create: w9[3 * stage + kind], stage K2, K3, K4 and
 * kind output slot, bucket, prune */
void orc_get_drop_channels(const orc_ctx* c, double* w9, double* e9);
/* scalars: [0]=transport_dropped_weight [1]=transport_dropped_energy
 * [2]=audit residual energy [3]=source_injected_weight [4]=source_injected_energy
 * [5]=source_out_of_grid_weight [6]=source_out_of_grid_energy
 * [7]=source_slot_dropped_weight [8]=source_slot_dropped_energy
 * [9]=source_representation_loss_energy [10]=iterations [11]=cell_steps
 * [12]=occupied input slots summed over cell-steps [13]=output slots summed */
void orc_get_scalars(const orc_ctx* c, double* out14);
void orc_get_fe(const orc_ctx* c, float* A, float* B, float* sigma_total);

/* The surrogate's targets: the expectation form's redistribution table of
 * each feature row (s, u, r, cap) -- s = sigma_theta / dtheta, u the mean
 * energy's position between the centres around it, r = sigma_E / their
 * spacing, cap 1 when the energy window's top is the incoming bin -- on
 * centres of uniform spacing: out[t + 8 e] = Mt[t] Me[e] (sm2d_redist.h).
 * The context is not used. */
void orc_redistribution_table(const orc_ctx* c, int n, const float* feats, float* out);

/* claim-demand diagnostic: with tracking on, the largest number of distinct
 * block ids aimed at one container (a psi_out cell, or one bucket of one
 * batch) within one iteration since tracking began */
void orc_track_claims(orc_ctx* c, int on);
/* the learned surrogate's network for surrogate_tables = 2: its fp32
 * parameters (sm2d_mlp_get_params layout), the calibrated error of each of
 * the 4096 input regions and the fallback tolerance; params NULL removes it */
void orc_set_surrogate(orc_ctx* c, const float* params, const float* region_err, float tol);
/* rows the network was asked for, rows that fell back (since orc_set_surrogate) */
void orc_surrogate_counts(const orc_ctx* c, long long* out2);
/* K4 on caller arrays (checker of the raw K4 entry): nb buckets of Kb ids
 * and Kb x L values, c2b[Nc] the first of a listed cell's four buckets (-1:
 * none); psi_out ids and values updated in place, drop2 += dropped weight
 * and energy */
void orc_k4_raw(orc_ctx* c, int nb, const uint32_t* bbid, const orc_real* bval, const int* c2b, uint32_t* obid,
                orc_real* oval, double* drop2);
/* the expectation form's angular masses Mt[8] for s = sigma_theta / dtheta
 * and energy masses Me[4] for a Gaussian (Em, sE) over the centres cen[0..emax]
 * (sm2d_redist.h), evaluated in this build's precision */
void orc_redist_masses(double s, double Em, double sE, const double* cen, int emax, double* Mt, double* Me);
int  orc_claim_demand(const orc_ctx* c);

/* run several independent contexts on n_threads host threads */
int  orc_run_many(orc_ctx** ctxs, int n, int max_iterations, int n_threads);

#ifdef __cplusplus
}
#endif
#endif
