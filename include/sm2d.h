/*
 * sm2d.h -- C ABI of the GB300 (sm_103a) SM_2D phase-space transport step.
 *
 * One handle holds one transport problem: a spatial grid of Nx x Nz cells,
 * a block-sparse phase space with 32 slots per cell (24-bit block ids
 * (b_E << 12) | b_theta, LOCAL_BINS local bins per slot), the R-LUT, the
 * per-cell tallies and the device-resident iteration state.  Every entry
 * point returns 0 on success and a negative SM2D_ERR_* code on failure;
 * sm2d_last_error() gives the message.  Plain pointers and sizes only.
 *
 * Reference interfaces each entry replaces (paths inside the SM_2D project):
 *   sm2d_create / sm2d_destroy  K1K6PipelineState::allocate/cleanup + init_pipeline_state
 *                               (src/cuda/k1k6_pipeline.cu:853-1215), device_psic_init
 *                               (src/cuda/device/device_psic.cuh:66-123), DeviceLUTWrapper::init
 *                               (src/cuda/kernels/k3_finetransport.cuh:114-150)
 *   sm2d_inject                 inject_source_kernel / inject_gaussian_source_kernel and the
 *                               source accounting (src/cuda/gpu_transport_wrapper.cu:339-460)
 *   sm2d_inject_quadrature      inject_source_kernel with its spreads (src/cuda/k1k6_pipeline.cu:300-427)
 *   sm2d_step                   one pass of the loop body (src/cuda/k1k6_pipeline.cu:1606-2038)
 *   sm2d_run                    run_k1k6_pipeline_transport(DevicePsiC*,...) (k1k6_pipeline.cuh:296)
 *   sm2d_get_dose               EdepC D2H + lateral post-convolution
 *                               (src/cuda/gpu_transport_wrapper.cu:531-623)
 *   sm2d_get_audit              get_audit_report (src/cuda/k1k6_pipeline.cu:1249-1255)
 *   sm2d_k1_active_mask         run_k1_active_mask / K1_ActiveMask (k1k6_pipeline.cu:1261-1294,
 *                               src/cuda/kernels/k1_activemask.cu:6-48)
 *   sm2d_k4_bucket_transfer     run_k4_bucket_transfer / K4_BucketTransfer (k1k6_pipeline.cu:1415-1447,
 *                               src/cuda/kernels/k4_transfer.cu:174-333)
 *   sm2d_k5_conservation_audit  run_k5_conservation_audit / K5_ConservationAudit
 *                               (k1k6_pipeline.cu:1449-1527, src/cuda/kernels/k5_audit.cu:22-167)
 *   sm2d_compact_lists          compact_active_list / compact_coarse_list (k1k6_pipeline.cu:589-665)
 */
#ifndef SM2D_H
#define SM2D_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SM2D_KB 32
#define SM2D_KB_OUT 32
#define SM2D_EMPTY 0xFFFFFFFFu

enum {
    SM2D_OK = 0,
    SM2D_ERR_ARG = -1,       /* invalid argument or configuration            */
    SM2D_ERR_CUDA = -2,      /* a CUDA runtime call failed                    */
    SM2D_ERR_ALLOC = -3,     /* device allocation failed                      */
    SM2D_ERR_STATE = -4,     /* call out of order (e.g. step before inject)   */
    SM2D_ERR_TIMEOUT = -5,   /* a bounded device wait gave up                 */
    SM2D_ERR_LAYOUT = -6     /* local-bin layout without a compiled kernel    */
};

/* Problem description.  Pointers are host arrays read during sm2d_create. */
typedef struct sm2d_problem {
    int Nx, Nz;                  /* spatial cells                              */
    float dx, dz;                /* cell size [mm]                             */
    float x_min, z_min;          /* grid origin [mm]                           */
    int N_theta;                 /* global angular bins                        */
    const float* theta_edges;    /* N_theta + 1 (AngularGrid::edges)           */
    int N_E;                     /* global energy bins                         */
    const float* E_edges;        /* N_E + 1 (EnergyGrid::edges)                */
    float E_min, E_max;          /* EnergyGrid::E_min / E_max                  */
    int nt_local, ne_local;      /* local bins per block: (4,2) or (8,4)       */
    int nx_sub, nz_sub;          /* sub-cell bins: (8,4) or (4,1)              */
    /* transport controls (TransportConfig) */
    float E_fine_on, E_fine_off; /* K1 thresholds [MeV]                        */
    float weight_active_min;
    float step_coarse;           /* K2 step [mm] (clamped to min(dx,dz))       */
    float sigma_x_initial;       /* beam sigma_x [mm]                          */
    float E0;                    /* beam energy for the Fermi-Eyges precompute */
    int enable_straggling, enable_nuclear;
    /* method options: 0 reproduces the reference */
    int seed_slot_mode;          /* 1: MCS/straggling seed uses the rank of the block id
                                    in the cell instead of the racy storage slot      */
    int energy_split;            /* 1: mean-preserving 2-bin energy re-binning          */
    int use_buckets;             /* 1: emit through DeviceOutflowBucket + K4 (reference
                                    structure); 0: fused direct neighbour scatter       */
    int max_iterations;          /* capacity of the audit history                     */
    /* production-run options (0 = reference behaviour) */
    float prune_coarse;          /* K2 drops components lighter than this (0: 1e-12)   */
    float prune_fine;            /* K3 drops components lighter than this (0: 1e-15)   */
    float split_min_weight;      /* energy split: lighter split parts stay in the major
                                    bin (energy folded into the deposit)               */
    float stop_weight_fraction;  /* stop when in-flight weight < this * injected weight */
    int floor_cutoff;            /* absorb components re-binned up to the lowest bin   */
    int seed_iteration_salt;     /* salt MCS/straggling seeds with the iteration index */
    /* engine shape */
    int lanes;                   /* spots transported together by sm2d_batch_run
                                    (0 or 1: one; at most 512; the single-spot entries
                                    use lane 0) */
    /* slab phantom (no counterpart in the reference, which transports water):
     * density of each depth row [Nz] in g/cm^3, or NULL for water.  Energy
     * loss, range limits, straggling, nuclear attenuation and the Highland
     * thickness use the water-equivalent path rho * step; the Fermi-Eyges
     * tables are integrated through the phantom. */
    const float* density_z;
    /* expectation form (no counterpart in the reference, whose K2/K3 draw one
     * hashed MCS angle and one straggling loss per bin and step): 1 emits
     * the expected result of the reference's re-binning of those draws
     * instead -- up to 15 angle bins (frac^2 split of a Gaussian angle) times
     * 4 energy bins (mean-preserving split of a Gaussian energy) per
     * component, the 8 theta x 4 E redistribution table of sm2d_redist.h.
     * Needs energy_split = 1 and the direct scatter (use_buckets = 0); the
     * result no longer depends on random seeds or on arithmetic rounding
     * through them. */
    int expectation;
    /* precision form (no counterpart in the reference): 1 books each
     * iteration's cutoff, nuclear and boundary weight in the K5 audit from the
     * iteration's own per-cell increments, instead of the difference of the
     * cumulative float tallies (whose rounding, relative to the cumulative
     * weight, otherwise enters the iteration's balance), and inverts the
     * R-LUT (range -> energy) in double below 10 MeV, where a step's energy
     * loss is a small difference of large ranges.  psi, the transport
     * arithmetic and the per-cell tallies stay as they are. */
    int precision_form;
    /* value pages per lane of an engine of several lanes (0: 32 MB of values,
     * 2^23 / L pages).  A claimed slot's L values live in a page of the lane's
     * region, handed out by the selection of its cell and returned when the
     * next classification consumes it; the ids, masks and tallies stay per
     * cell.  One lane holds the pages its occupied slots need in one
     * iteration (the widest 70 MeV spot of the 512-spot plan peaks at 4422
     * on the reference grids, about 20000 on the 256 log-E / 512 theta
     * grid); a pass that needs more stops the run with SM2D_ERR_ALLOC.  A
     * single-lane engine always has one page per slot (no counterpart in the
     * reference, whose DevicePsiC holds every slot of every cell). */
    int slot_pages_per_lane;
} sm2d_problem;

typedef struct sm2d_beam {
    float x0, z0, theta0, E0, W_total;
    float sigma_x, sigma_theta, sigma_E;
    int n_samples;
    unsigned int seed;
} sm2d_beam;

/* AuditReport (src/cuda/kernels/k5_audit.cuh:5-27), same field order. */
typedef struct sm2d_audit {
    float W_error; int W_pass; float E_error; int E_pass;
    float W_in_total, W_out_total, W_cutoff_total, W_nuclear_total, W_boundary_total;
    float W_source_out_of_grid_total, W_source_slot_drop_total, W_transport_drop_total;
    double E_in_total, E_out_total, E_dep_total, E_cutoff_total, E_nuclear_total;
    double E_boundary_total, E_source_out_of_grid_total, E_source_slot_drop_total;
    double E_transport_drop_total;
    int processed_cells;
} sm2d_audit;

/* Outcome of one spot of sm2d_batch_run (no counterpart in the reference,
 * whose runner transports one spot per call). */
typedef struct sm2d_spot_result {
    int iterations;               /* transport iterations                              */
    int finished;                 /* 1: no cell held weight any more (or stopping rule) */
    int weight_audit_failures;    /* iterations whose weight audit failed              */
    int energy_audit_failures;    /* iterations whose energy audit failed              */
    double injected_weight, injected_energy;
    double source_out_of_grid_weight, source_slot_dropped_weight;
    double transport_dropped_weight, transport_dropped_energy;
    double audit_residual_energy, representation_loss_energy;
    double cell_steps;            /* listed cells summed over iterations               */
    double slots_in, slots_out;   /* occupied psi_in / psi_out slots summed over iterations */
    sm2d_audit last;              /* audit record of the last iteration                */
} sm2d_spot_result;

/* DeviceOutflowBucket (src/cuda/device/device_bucket.cuh:48-57) for L local bins:
 *   uint32 block_id[32]; uint16 local_count[32]; float value[32][L]; float moment_A,B,C;
 * sm2d_bucket_bytes(L) is its size. */
size_t sm2d_bucket_bytes(int local_bins);

typedef struct sm2d_ctx* sm2d_handle;

const char* sm2d_last_error(void);
int sm2d_version(void);
int sm2d_create(const sm2d_problem* p, sm2d_handle* out);
int sm2d_destroy(sm2d_handle h);
int sm2d_local_bins(sm2d_handle h);

/* source injection into psi_in (pencil or LCG Gaussian beam) */
int sm2d_inject(sm2d_handle h, const sm2d_beam* beam);
/* inject_source_kernel called with its spreads (src/cuda/k1k6_pipeline.cu:300-427):
 * the quadrature source.  Uses x0, z0, theta0, E0, W_total, sigma_x and
 * sigma_theta (sigma_E, n_samples and seed are ignored).  Without spreads
 * (sigma_theta <= 1e-4, sigma_x <= 0.01) it injects the pencil; otherwise
 * each cell centre within +-4 sigma_x of x0 takes a Gaussian weight
 * normalised over those cells, on 7 angle nodes theta0 + a_k sigma_theta with
 * weights w_k when sigma_theta > 1e-4.  Needs sigma_x > 0 on that path (the
 * reference divides by sigma_x^2).  Accounting as the wrapper books a
 * non-Gaussian source: W_total and E0 W_total injected. */
int sm2d_inject_quadrature(sm2d_handle h, const sm2d_beam* beam);
/* host <-> device phase space (psi_in): bid[Nx*Nz*32], val[Nx*Nz*32*L] */
int sm2d_set_psi_in(sm2d_handle h, const uint32_t* bid, const float* val);
int sm2d_get_psi_in(sm2d_handle h, uint32_t* bid, float* val);
/* the same on device arrays of the caller (DevicePsiC::block_id / value,
 * src/cuda/device/device_psic.cuh:39-55; single-lane engines) */
int sm2d_set_psi_in_device(sm2d_handle h, const uint32_t* d_bid, const float* d_val);
int sm2d_get_psi_in_device(sm2d_handle h, uint32_t* d_bid, float* d_val);
/* source accounting of a phase space set by the caller (the
 * K1K6PipelineState::source_* fields, src/cuda/k1k6_pipeline.cuh:190-197, that
 * the first iteration's audit lifts): [0] injected weight, [1] out-of-grid
 * weight, [2] slot-dropped weight, [3] injected energy, [4] out-of-grid
 * energy, [5] slot-dropped energy, [6] representation loss energy */
int sm2d_set_source_accounting(sm2d_handle h, const double* v7);

/* one K1..K6 iteration; *n_active/*n_coarse are the listed cells (0,0 = done) */
int sm2d_step(sm2d_handle h, int* n_active, int* n_coarse);
/* iterate until no cell holds weight or max_iterations passed; the loop runs
 * on the device (one CUDA-graph launch, no host round trip per iteration) */
int sm2d_run(sm2d_handle h, int max_iterations, int* iterations_done);
/* same as sm2d_run, returning the device time of the loop (CUDA events) */
int sm2d_run_timed(sm2d_handle h, int max_iterations, int* iterations_done, float* ms);

int sm2d_get_mask(sm2d_handle h, uint8_t* mask);
int sm2d_get_lists(sm2d_handle h, uint32_t* active, int* n_active, uint32_t* coarse, int* n_coarse);
int sm2d_get_tallies(sm2d_handle h, double* edep, float* w_cut, double* e_cut,
                     float* w_nuc, double* e_nuc, float* w_bnd, double* e_bnd);
int sm2d_get_audit(sm2d_handle h, sm2d_audit* out);
int sm2d_get_audit_history(sm2d_handle h, sm2d_audit* out, int max_entries, int* n_entries);
/* scalars: [0] transport_dropped_weight [1] transport_dropped_energy
 * [2] audit residual energy [3] source_injected_weight [4] source_injected_energy
 * [5] source_out_of_grid_weight [6] source_out_of_grid_energy
 * [7] source_slot_dropped_weight [8] source_slot_dropped_energy
 * [9] source_representation_loss_energy [10] iterations [11] cell_steps
 * [12] occupied input slots summed over cell-steps [13] output slots summed
 * [14] claim-table inserts that found no free entry [15] deposits whose
 * block id had not been gathered (both 0 in a correct run; cumulative
 * since create) [16] bin-list overflows of this spot (non-zero: the run
 * stopped early; sm2d_run/sm2d_step return SM2D_ERR_ALLOC) */
int sm2d_get_scalars(sm2d_handle h, double* out17);
/* k2_get_debug_counters / k3_get_debug_counters / k4_get_debug_counters
 * (src/cuda/kernels/k2_coarsetransport.cuh:101-112, k3_finetransport.cuh:78-89,
 * k4_transfer.cuh:19-24) for stage 2, 3 or 4: [0] output-slot drops, [1]
 * bucket drops, [2] pruned components; dropped components, weight and energy
 * (after-step energy; bin centre for K4) since sm2d_reset or
 * sm2d_reset_debug_counters, summed over lanes.  K4 counts the output slots
 * the fused deposit or the bucket move could not resolve; K4 has no bucket or
 * prune drops.  Their weights add up to the transport-drop channel, less
 * what a stopping rule or an iteration limit books there at a spot's end. */
int sm2d_get_debug_counters(sm2d_handle h, int stage, unsigned long long* counts3, double* weights3,
                            double* energies3);
/* k2/k3/k4_reset_debug_counters */
int sm2d_reset_debug_counters(sm2d_handle h, int stage);
int sm2d_get_fe(sm2d_handle h, float* A, float* B, float* sigma_total);
/* EdepC after the lateral MCS post-convolution, [Nz][Nx] row-major */
int sm2d_get_dose(sm2d_handle h, double* dose);
/* per-stage device time of the last sm2d_step (ms): classify, ascending
 * lists, claim pass, slot selection, deposit pass, K4 bucket move,
 * finalize (audit + clear + swap) */
int sm2d_get_step_timing(sm2d_handle h, float* ms7);

/* ---- asynchronous spot pipeline (no host synchronisation; stream order) ---- */
/* the library's CUDA stream (cudaStream_t) */
void* sm2d_stream(sm2d_handle h);
/* clear phase space, tallies and iteration state for a new spot */
int sm2d_reset(sm2d_handle h);
/* inject from a host beam description without waiting for the device */
int sm2d_inject_async(sm2d_handle h, const sm2d_beam* beam);
/* enqueue the device loop (<= max_iterations more iterations) */
int sm2d_run_async(sm2d_handle h, int max_iterations);
/* post-convolved dose [Nz][Nx] into host memory (pinned for an async copy) */
int sm2d_dose_async(sm2d_handle h, double* host_dose);
/* replay up to n_iterations eagerly with CUDA events around every kernel;
 * ms7 receives the summed device time of the seven stages listed at
 * sm2d_get_step_timing over the *passes passes that transported (a wave of
 * lanes runs as many passes as its longest spot needs; *iterations_done is
 * lane 0's count), *launches the number of kernel launches */
int sm2d_run_profiled(sm2d_handle h, int n_iterations, int* iterations_done, float* ms7, int* launches,
                      int* passes);

/* ---- batched spots (no counterpart in the reference: its runner transports
 * one spot per call; a plan is a loop over such calls) ---- */
/* lanes of the engine: spots transported together */
int sm2d_lanes(sm2d_handle h);
/* Transport a plan of n_spots beams to completion, each spot as an engine
 * created with problem.E0 = beam.E0 and problem.sigma_x_initial =
 * beam.sigma_x would transport it alone (sm2d_inject + sm2d_run; the
 * reference hands the beam's E0 and sigma_x to its Fermi-Eyges precompute).
 * `lanes` spots are in flight; a lane whose spot finishes takes the next
 * spot of the plan inside the device loop (one graph launch for the plan).
 * dose: host [n_spots][Nz][Nx] for the post-convolved EdepC of each spot,
 * or NULL; results: host [n_spots] or NULL.  When dose is pinned host memory
 * (cudaHostAlloc, cudaHostRegister) the device writes each spot's map there as
 * the spot completes, overlapped with the other spots' transport; other
 * memory receives one copy at the end.  A spot that reaches max_iterations
 * ends there: its remaining weight is booked as a transport drop and its
 * result reads finished = 0.  Blocking. */
int sm2d_batch_run(sm2d_handle h, const sm2d_beam* beams, int n_spots, int max_iterations, double* dose,
                   sm2d_spot_result* results);
/* The three steps of sm2d_batch_run: sm2d_plan_load stages the plan on the
 * device (its Fermi-Eyges tables computed on the host threads; with_dose
 * keeps a device dose map per spot), sm2d_plan_run_async transports it on
 * the engine's stream, sm2d_plan_results waits and copies dose (NULL: none)
 * and results (NULL: none) back.  sm2d_plan_stats: device passes, refill
 * rounds and transported bins (local bins with weight) since the last
 * plan's start (or the last reset). */
int sm2d_plan_load(sm2d_handle h, const sm2d_beam* beams, int n_spots, int max_iterations, int with_dose);
int sm2d_plan_run_async(sm2d_handle h);
int sm2d_plan_results(sm2d_handle h, double* dose, sm2d_spot_result* results);
int sm2d_plan_stats(sm2d_handle h, int* passes, int* refills, double* bins);
/* Value pages of one lane (sm2d_problem.slot_pages_per_lane) and the most
 * pages one lane held at once since the last plan's start or reset (no
 * counterpart in the reference, which stores every slot densely). */
int sm2d_page_stats(sm2d_handle h, int* pages_per_lane, int* peak_pages);
/* One wave of spots, for callers that drive the loop themselves:
 * sm2d_batch_inject resets every lane and injects beams[i] into lane i
 * (lanes past n_beams stay empty; asynchronous, like sm2d_inject_async);
 * then sm2d_run / sm2d_run_async / sm2d_run_profiled transport all lanes,
 * max_iterations passes at most; sm2d_batch_results and sm2d_batch_dose
 * read the first n lanes back (blocking). */
int sm2d_batch_inject(sm2d_handle h, const sm2d_beam* beams, int n_beams);
int sm2d_batch_results(sm2d_handle h, sm2d_spot_result* results, int n);
int sm2d_batch_dose(sm2d_handle h, double* dose, int n);
/* audit record of every iteration of lane `lane`'s spot (up to the history
 * capacity, problem.max_iterations) */
int sm2d_batch_audit_history(sm2d_handle h, int lane, sm2d_audit* out, int max_entries, int* n_entries);

/* ---- launch shape and its autotuner (no counterpart in the reference, whose
 * launches are sized by the grid) ---- */
/* blocks per SM of [0] the warp-per-cell kernels (classification, slot
 * selection; default 8), [1] finalize (4), [2] the claim pass and [3] the
 * deposit pass (0: every block the SM holds at once); the kernels stride over
 * their work, so the shape changes speed, not results */
int sm2d_get_launch_shape(sm2d_handle h, int* shape4);
int sm2d_set_launch_shape(sm2d_handle h, const int* shape4);
/* coordinate descent over the launch shape on the plan that sm2d_plan_load
 * staged: each entry's candidates are timed on a run of the whole plan and the
 * fastest is kept (about 20 plan runs); shape4 and best_ms (may be NULL)
 * receive the chosen shape and its plan time */
int sm2d_autotune(sm2d_handle h, int* shape4, float* best_ms);
/* Lanes in flight of a plan (no counterpart in the reference): a plan fills
 * lanes 0 .. n-1 only (0 or n >= lanes: every lane).  Fewer lanes in flight
 * make each pass's working set smaller (claim rows, step records, pages) at
 * the price of more passes; the results do not change.
 * sm2d_tune_lanes_in_flight times every lane, 3/4, 1/2, 1/4, 1/8 and 1/16 of
 * them (at least 8) on the plan sm2d_plan_load staged and keeps the fastest
 * (sm2d_autotune does this first, then the launch shape). */
int sm2d_set_lanes_in_flight(sm2d_handle h, int n);
int sm2d_get_lanes_in_flight(sm2d_handle h, int* n);
int sm2d_tune_lanes_in_flight(sm2d_handle h, int* lanes, float* best_ms);

/* ---- host tables (no GPU needed) ---- */
/* EnergyGrid(E_min,E_max,N) log grid (grids.cpp:6-24): edges[N+1], rep[N] */
int sm2d_energy_grid_log(float E_min, float E_max, int N, float* edges, float* rep);
/* EnergyGrid::CreatePiecewise (grids.cpp:37-97); groups = {E_start,E_end,dE}*n.
 * Returns N_E; with edges == NULL only counts. */
int sm2d_energy_grid_piecewise(int n_groups, const float* groups, float* edges, float* rep);
/* AngularGrid (grids.cpp:121-137): edges[N+1], rep[N] */
int sm2d_angular_grid(float theta_min, float theta_max, int N, float* edges, float* rep);
/* GenerateRLUT(grid) (r_lut.cpp:69-129) on representative energies rep[N] */
int sm2d_range_lut(int N, const float* rep, float* R, float* S, float* logE, float* logR, float* logS);
/* Fermi-Eyges A(z), B(z), sigma_total(z) (k1k6_pipeline.cu:1061-1176) */
int sm2d_fermi_eyges(float E0, int Nz, float dz, float sigma_x0, float* A, float* B, float* sigma_total);
/* the same through a slab phantom (density_z[Nz], as in sm2d_problem) */
int sm2d_fermi_eyges_density(float E0, int Nz, float dz, float sigma_x0, const float* density_z, float* A, float* B,
                             float* sigma_total);

/* ---- the INI front end (run_simulation's configuration file) ---- */
/* One run as the reference's configuration file describes it: the problem
 * and beam GPUTransportRunner::run builds from IncidentParticleConfig
 * (src/include/core/config_loader.hpp:98-413, src/gpu/gpu_transport_runner.cpp:28-105)
 * and run_simulation's output settings.  The grids are owned by the config
 * (problem.theta_edges / E_edges point into them): release them with
 * sm2d_run_config_free. */
typedef struct sm2d_run_config {
    sm2d_problem problem;
    sm2d_beam beam;
    int max_iterations;          /* transport.max_iterations, or grid.max_steps if 0 */
    int log_level;
    int fail_fast_on_audit;      /* parsed; the engine books audit failures instead  */
    int normalize_dose, save_2d, save_pdd;
    char output_dir[1024];       /* as written; relative paths are relative to the INI */
    char dose_2d_file[256], pdd_file[256];
    float* theta_edges_buf;
    float* E_edges_buf;
} sm2d_run_config;
/* load_incident_particle_config + validate (config_loader.hpp:324-411,
 * incident_particle_config.hpp:274-399); SM2D_ERR_ARG with the reference's
 * message for an unreadable file or an invalid value */
int sm2d_load_ini(const char* ini_path, sm2d_run_config* out);
void sm2d_run_config_free(sm2d_run_config* config);
/* run_simulation's main (run_simulation.cpp:116-188): one spot from the INI,
 * dose_2d.txt and pdd.txt under its output_dir.  0 on success. */
int sm2d_run_simulation(const char* ini_path);

/* ---- depth-dose metrics and output files (host; dose[Nz][Nx] as
 * sm2d_get_dose returns it) ---- */
/* get_depth_dose (src/validation/deterministic_beam.cpp:224-236): pdd[Nz],
 * the double sum over x of each row */
int sm2d_depth_dose(const double* dose, int Nx, int Nz, double* pdd);
/* find_bragg_peak_z (deterministic_beam.cpp:207-222): the row of the largest
 * depth dose (the first of equals; 0 if none is positive) */
int sm2d_bragg_peak_row(const double* dose, int Nx, int Nz);
/* src/validation/bragg_peak.cpp: out[5] = peak depth, FWHM, R80, R20 and
 * distal falloff R20 - R80, all in mm, from float row sums */
int sm2d_bragg_metrics(const double* dose, int Nx, int Nz, float dz, float* out);
/* save_dose_2d / save_pdd (run_simulation.cpp:31-114): the reference's
 * dose_2d.txt and pdd.txt files, byte for byte, with the cell centres of its
 * runner (x = (i + 0.5) dx - Nx dx / 2, z = j dz) */
int sm2d_write_dose_2d(const char* path, const double* dose, int Nx, int Nz, float dx, float dz, int normalize);
int sm2d_write_pdd(const char* path, const double* dose, int Nx, int Nz, float dz, int normalize);

/* ---- debug dumps in the reference's CSV formats (host; built with
 * SM2D_ENABLE_DEBUG_DUMPS there), from a host copy of psi (sm2d_get_psi_in)
 * and the problem's grids ---- */
/* debug_ps_raw_iter_NN_<stage>.csv: dump_phase_space_raw_to_csv
 * (src/cuda/k1k6_pipeline.cu:195-291, precision 8) and the initial dump of
 * src/cuda/gpu_transport_wrapper.cu:22-120 (iteration 0, precision 6) */
int sm2d_write_ps_raw_csv(const char* path, const sm2d_problem* p, const uint32_t* bid, const float* val,
                          int iteration, int precision);
/* debug_cells_iter_NN_<stage>.csv: dump_nonzero_cells_to_csv (k1k6_pipeline.cu:29-193) */
int sm2d_write_cells_csv(const char* path, const sm2d_problem* p, const uint32_t* bid, const float* val);
/* debug_channels_totals_iter01.csv (k1k6_pipeline.cu:2125-2155) from the 17
 * totals of iteration 1 in the file's order; sm2d_channel_totals computes
 * them from a single-spot engine (cell sums in cell order, then its scalars) */
int sm2d_write_channel_totals_csv(const char* path, const double* totals17);
int sm2d_channel_totals(sm2d_handle h, int Nx, int Nz, double* totals17);

/* ---- raw stage entries on caller-owned device memory (stream may be 0) ---- */
int sm2d_k1_active_mask(const uint32_t* d_block_ids, const float* d_values, uint8_t* d_mask,
                        const uint8_t* d_mask_prev, int Nx, int Nz, int local_bins,
                        int b_E_fine_on, int b_E_fine_off, float weight_active_min, void* stream);
int sm2d_compact_lists(const uint8_t* d_mask, const uint32_t* d_block_ids, const float* d_values,
                       int Nx, int Nz, int local_bins, uint32_t* d_active, int* d_n_active,
                       uint32_t* d_coarse, int* d_n_coarse, void* stream);
int sm2d_k4_bucket_transfer(const void* d_buckets, const int* d_cell_to_bucket_base,
                            float* d_values_out, uint32_t* d_block_ids_out, int Nx, int Nz,
                            int local_bins, int nt_local, int ne_local, int nx_sub,
                            const float* d_E_edges, int N_E, int N_E_local,
                            double* d_drop_weight_energy /* [2], accumulated */, void* stream);
int sm2d_k5_conservation_audit(
    const uint32_t* d_bid_in, const float* d_val_in, const uint32_t* d_bid_out, const float* d_val_out,
    const double* d_EdepC, const double* d_AbsorbedEnergy_nuclear, const double* d_BoundaryLoss_energy,
    const double* d_AbsorbedEnergy_cutoff, const double* d_PrevEdepC,
    const double* d_PrevAbsorbedEnergy_nuclear, const double* d_PrevBoundaryLoss_energy,
    const double* d_PrevAbsorbedEnergy_cutoff, const float* d_AbsorbedWeight_cutoff,
    const float* d_AbsorbedWeight_nuclear, const float* d_BoundaryLoss_weight,
    const float* d_PrevAbsorbedWeight_cutoff, const float* d_PrevAbsorbedWeight_nuclear,
    const float* d_PrevBoundaryLoss_weight, float source_out_of_grid_weight,
    float source_slot_dropped_weight, double source_out_of_grid_energy,
    double source_slot_dropped_energy, float transport_dropped_weight,
    double transport_dropped_energy, int include_source_terms, const float* d_E_edges, int N_E,
    int nt_local, int N_E_local, int local_bins, sm2d_audit* d_report, int N_cells, void* stream);
/* The K5 audit above without any device allocation (no counterpart in the
 * reference; for callers that cannot call cudaMalloc).  Same arguments and
 * report; the reduction scratch is a file-scope static __device__ array of
 * 2048 x 11 doubles plus a counter (about 176 KB per device), so N_cells is
 * limited to 524288 (2048 blocks of 256 cells); larger grids are refused
 * with SM2D_ERR_ARG.  The block totals are summed in a fixed order, so the
 * report is the same on every call.  All calls share the scratch: calls
 * whose kernels overlap on the GPU (other streams or threads) race. */
int sm2d_k5_conservation_audit_static(
    const uint32_t* d_bid_in, const float* d_val_in, const uint32_t* d_bid_out, const float* d_val_out,
    const double* d_EdepC, const double* d_AbsorbedEnergy_nuclear, const double* d_BoundaryLoss_energy,
    const double* d_AbsorbedEnergy_cutoff, const double* d_PrevEdepC,
    const double* d_PrevAbsorbedEnergy_nuclear, const double* d_PrevBoundaryLoss_energy,
    const double* d_PrevAbsorbedEnergy_cutoff, const float* d_AbsorbedWeight_cutoff,
    const float* d_AbsorbedWeight_nuclear, const float* d_BoundaryLoss_weight,
    const float* d_PrevAbsorbedWeight_cutoff, const float* d_PrevAbsorbedWeight_nuclear,
    const float* d_PrevBoundaryLoss_weight, float source_out_of_grid_weight,
    float source_slot_dropped_weight, double source_out_of_grid_energy,
    double source_slot_dropped_energy, float transport_dropped_weight,
    double transport_dropped_energy, int include_source_terms, const float* d_E_edges, int N_E,
    int nt_local, int N_E_local, int local_bins, sm2d_audit* d_report, int N_cells, void* stream);

/* ---- diagnostics (no counterpart in the reference) ---- */
/* Evaluate one of the transport's elementary functions (0 exp, 1 log,
 * 2 sin, 3 cos, 4 erf; sm2d_math.h) on n host values on the device; the
 * oracle's build of the same header must agree bit for bit. */
int sm2d_math_eval(int fn, const float* x, float* y, int n);

/* ---- learned redistribution surrogate of the fine step ----
 * Replaces the closed-form redistribution weights of K3_FineTransport's
 * expectation form (the per-bin Highland-MCS / Vavilov-straggling /
 * energy-split re-binning of src/cuda/kernels/k3_finetransport.cu:263-366,
 * evaluated as expectations in sm2d_redist.h) by a 4 -> 128 -> 128 -> 32 MLP
 * (ReLU, softmax).  Inputs are float4 rows (s, u, r, cap): s = sigma_theta /
 * dtheta (the step's MCS angle in angle bins, 0..8), u in [0, 1) (where the
 * step's mean energy lies between the two energy-bin centres around it),
 * r = sigma_E / spacing of those centres (straggling in bins, 0..4), cap
 * (1: the energy window's top is the incoming bin; 0: the second centre above
 * the mean).  Outputs are 32 weights per row, index t + 8 e: angular
 * distance t = 0..7 bins (t >= 1 split between both sides) times energy
 * offset e = 0..3 below the window's top; they sum to 1.  The method's own
 * tables come from sm2d_redistribution_table (the closed forms on centres of
 * uniform spacing).  bf16 weights, fp32 accumulation on the tcgen05 tensor
 * cores, trained on the device (softmax cross-entropy, Adam).  Device arrays
 * must be 16-byte aligned.  gradients, train, forward and redistribute only
 * enqueue work on the handle's stream; sm2d_mlp_sync waits for it and reports
 * a device wait that gave up (SM2D_ERR_TIMEOUT).
 * The reference has no learned part; these entries have no counterpart. */
typedef struct sm2d_mlp* sm2d_mlp_handle;
int sm2d_mlp_param_count(void);   /* 22816 fp32: W1[128][16] W2[128][128] W3[32][128] b1 b2 b3 */
/* max_batch: the largest training batch (rounded up to 128); stream: the
 * cudaStream_t of every launch (NULL: the legacy stream).  Weights start
 * He-uniform from a fixed seed. */
int sm2d_mlp_create(int max_batch, void* stream, sm2d_mlp_handle* out);
int sm2d_mlp_destroy(sm2d_mlp_handle m);
/* host fp32 parameters in and out (setting them resets the Adam state) */
int sm2d_mlp_set_params(sm2d_mlp_handle m, const float* host_params);
int sm2d_mlp_get_params(sm2d_mlp_handle m, float* host_params);
/* mean softmax cross-entropy of n <= max_batch rows against d_target
 * [n][32] and its gradient (the fp32 parameter layout) into device arrays */
int sm2d_mlp_gradients(sm2d_mlp_handle m, const float* d_feats, const float* d_target, int n, float* d_grads,
                       float* d_loss);
/* `steps` Adam steps over consecutive batches of the set (wrapping), cosine
 * learning rate from lr0 to lr_min; per-step loss into d_loss_hist (or NULL) */
int sm2d_mlp_train(sm2d_mlp_handle m, const float* d_feats, const float* d_target, int n_total, int batch, int steps,
                   float lr0, float lr_min, float* d_loss_hist);
/* surrogate tables of n rows into d_table [n][32] */
int sm2d_mlp_forward(sm2d_mlp_handle m, const float* d_feats, int n, float* d_table);
/* n training inputs (hash of seed and row): s = 8 a^2, u uniform on [0, 1),
 * r = 4 c^2 (a, c uniform on [0, 1)), cap 0 or 1 */
int sm2d_redistribution_features(int n, uint32_t seed, float* d_feats, void* stream);
/* the method's own tables (the closed forms of sm2d_redist.h); the work runs
 * on h's stream */
int sm2d_redistribution_table(sm2d_handle h, const float* d_feats, int n, float* d_table);
/* per input region (16 sqrt(s/8) x 16 u x 8 sqrt(r/4) x 2 cap) the largest
 * absolute weight error of the surrogate rows against the plain rows;
 * optional host copy of the 4096 errors (as float bits) */
int sm2d_mlp_calibrate(sm2d_mlp_handle m, const float* d_feats, const float* d_plain, const float* d_surrogate, int n,
                       float* host_region_err);
/* surrogate tables, with the plain table of the handle's physics in the rows
 * whose calibrated region error exceeds tol (d_fallback[i] = 1 there).  The
 * work runs on the surrogate's stream after the work already enqueued on h's
 * stream (an event orders the two streams). */
int sm2d_mlp_redistribute(sm2d_mlp_handle m, sm2d_handle h, const float* d_feats, int n, float tol, float* d_table,
                          int* d_fallback);
/* wait for the handle's stream; SM2D_ERR_TIMEOUT if a kernel's bounded wait
 * gave up since the last sync (the flag is cleared once reported) */
int sm2d_mlp_sync(sm2d_mlp_handle m);
/* feature ranges and calibration regions: s_max, u_max, r_max, cap_max,
 * regions along s, u, r and cap */
int sm2d_mlp_geometry(float* out8);
/* The surrogate inside the transport of an expectation-form handle: every K3
 * bin that stays above the cutoff and whose energy window has four centres
 * of uniform spacing takes its children's weights from network m instead of
 * the closed forms of k3_finetransport.cu:263-366 (sm2d_redist.h).  The
 * claim pass writes the bin's feature row and defers its claims; the network
 * runs on the transport's stream inside the device loop; the rows' claims and
 * the deposit pass then use the row's table (network weights below 2^-12 are
 * zero and the rest sum to 1, so the weight is conserved; the energy the
 * table does not represent goes to the deposit).  A row whose calibrated
 * region error (sm2d_mlp_calibrate) exceeds tol falls back to the closed
 * forms.  max_rows: surrogate rows per pass (0: min(bin list, 4 Mi)); bins
 * beyond it keep the closed forms.  method_tables = 1 gives every row the
 * plain table of its features instead of the network's (the table path with
 * the method's own numbers; no calibration needed).  m = NULL detaches.  m
 * must stay alive while attached and run on the device of h.  A bounded wait
 * of the network that gives up sets m's error flag (sm2d_mlp_sync). */
int sm2d_set_surrogate(sm2d_handle h, sm2d_mlp_handle m, float tol, int max_rows, int method_tables);
/* since the last reset: [0] surrogate rows served, [1] rows that fell back
 * to the closed forms, [2] K3 bins beyond max_rows */
int sm2d_surrogate_stats(sm2d_handle h, double* out3);

#ifdef __cplusplus
}
#endif
#endif
