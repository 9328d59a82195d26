// sm2d_ref_types.hpp -- the types and entry points of the SM_2D transport
// path's C++ interface, for the drop-in layer (sm_2d_gb300/shim) that binds
// them to the C ABI of sm2d.h.
//
// A caller that builds with the SM_2D tree includes that tree's headers
// instead (the shim compiles against either; -DSM2D_SHIM_REFERENCE_HEADERS
// selects the tree's).  The declarations here keep the reference's names,
// member order and member types, so that objects built against either header
// exchange the same bytes:
//   EnergyGrid, AngularGrid          src/include/core/grids.hpp:7-48
//   RLUT, GenerateRLUT               src/include/lut/r_lut.hpp:5-29
//   DeviceRLUT                       src/cuda/device/device_lut.cuh:16-26
//   DevicePsiC                       src/cuda/device/device_psic.cuh:39-55
//   AuditReport                      src/cuda/kernels/k5_audit.cuh:5-28
//   TransportEnergyGroup, TransportConfig
//                                    src/include/core/incident_particle_config.hpp:157-202
//   DeviceLUTWrapper, init_device_lut, run_k1k6_pipeline_transport (wrapper)
//                                    src/include/cuda/gpu_transport_wrapper.hpp:21-92
//   K1K6PipelineConfig, K1K6PipelineState, the pipeline entry and the stage
//   entries                          src/cuda/k1k6_pipeline.cuh:36-416
//   the local-bin constants          src/include/core/local_bins.hpp:19-23
#pragma once
#include <cstdint>
#include <string>
#include <tuple>
#include <vector>

constexpr int N_theta_local = 4;
constexpr int N_E_local = 2;
constexpr int N_x_sub = 8;
constexpr int N_z_sub = 4;
constexpr int LOCAL_BINS = N_theta_local * N_E_local * N_x_sub * N_z_sub;

struct EnergyGrid {
    int N_E;
    float E_min;
    float E_max;
    std::vector<float> edges;   // N_E + 1
    std::vector<float> rep;     // N_E
    bool is_piecewise;

    EnergyGrid(float E_min, float E_max, int N_E);
    static EnergyGrid CreatePiecewise(const std::vector<std::tuple<float, float, float>>& groups);
    int GetN_E() const { return N_E; }
    float GetE_min() const { return E_min; }
    float GetE_max() const { return E_max; }
    int FindBin(float E) const;
    float GetRepEnergy(int bin) const;
};

struct AngularGrid {
    int N_theta;
    float theta_min;
    float theta_max;
    std::vector<float> edges;   // N_theta + 1
    std::vector<float> rep;     // N_theta

    AngularGrid(float theta_min, float theta_max, int N_theta);
    int FindBin(float theta) const;
    float GetRepTheta(int bin) const;
    int GetN_theta() const { return N_theta; }
    float GetTheta_min() const { return theta_min; }
    float GetTheta_max() const { return theta_max; }
};

struct RLUT {
    EnergyGrid grid;
    std::vector<float> R;
    std::vector<float> S;
    std::vector<float> log_E;
    std::vector<float> log_R;
    std::vector<float> log_S;
    float lookup_R(float E) const;
    float lookup_S(float E) const;
    float lookup_E_inverse(float R) const;
};
RLUT GenerateRLUT(float E_min, float E_max, int N_E);
RLUT GenerateRLUT(const EnergyGrid& grid);

struct DeviceRLUT {
    int N_E;
    float E_min;
    float E_max;
    const float* __restrict__ R;
    const float* __restrict__ S;
    const float* __restrict__ log_E;
    const float* __restrict__ log_R;
    const float* __restrict__ log_S;
    const float* __restrict__ E_edges;
};

struct DevicePsiC {
    int Nx;
    int Nz;
    int N_cells;
    int Kb;
    uint32_t* block_id;   // [N_cells * Kb]
    float* value;         // [N_cells * Kb * LOCAL_BINS]
};

struct DeviceOutflowBucket;   // 32 ids, 32 counts, [32][LOCAL_BINS] values, 3 moments

struct AuditReport {
    float W_error;
    int W_pass;
    float E_error;
    int E_pass;
    float W_in_total;
    float W_out_total;
    float W_cutoff_total;
    float W_nuclear_total;
    float W_boundary_total;
    float W_source_out_of_grid_total;
    float W_source_slot_drop_total;
    float W_transport_drop_total;
    double E_in_total;
    double E_out_total;
    double E_dep_total;
    double E_cutoff_total;
    double E_nuclear_total;
    double E_boundary_total;
    double E_source_out_of_grid_total;
    double E_source_slot_drop_total;
    double E_transport_drop_total;
    int processed_cells;
};

namespace sm_2d {

struct TransportEnergyGroup {
    float E_min_MeV = 0.1f;
    float E_max_MeV = 1.0f;
    float dE_MeV = 0.1f;
};

inline std::vector<TransportEnergyGroup> default_transport_energy_groups() {
    return {{0.1f, 2.0f, 0.1f}, {2.0f, 20.0f, 0.2f}, {20.0f, 100.0f, 0.25f}, {100.0f, 250.0f, 0.25f}};
}

struct TransportConfig {
    int N_theta = 36;
    int N_theta_local = ::N_theta_local;
    int N_E_local = ::N_E_local;
    std::vector<TransportEnergyGroup> energy_groups = default_transport_energy_groups();
    float E_fine_on = 10.0f;
    float E_fine_off = 11.0f;
    float E_trigger = 10.0f;
    float weight_active_min = 1e-12f;
    float E_coarse_max = 300.0f;
    float step_coarse = 5.0f;
    int n_steps_per_cell = 1;
    int fine_batch_max_cells = 0;
    int fine_halo_cells = 1;
    float preflight_vram_margin = 0.85f;
    bool validation_mode = false;
    bool fail_fast_on_audit = false;
    bool debug_dumps = true;
    int max_iterations = 0;
    int log_level = 1;
};

class DeviceLUTWrapperImpl;

class DeviceLUTWrapper {
public:
    DeviceLUTWrapper();
    ~DeviceLUTWrapper();
    DeviceLUTWrapper(const DeviceLUTWrapper&) = delete;
    DeviceLUTWrapper& operator=(const DeviceLUTWrapper&) = delete;
    const ::DeviceRLUT* get() const { return dlut_ptr; }

private:
    friend bool init_device_lut(const ::RLUT& cpu_lut, DeviceLUTWrapper& wrapper);
    DeviceLUTWrapperImpl* p_impl;
    const ::DeviceRLUT* dlut_ptr;
};

bool init_device_lut(const ::RLUT& cpu_lut, DeviceLUTWrapper& wrapper);

bool run_k1k6_pipeline_transport(float x0, float z0, float theta0, float E0, float W_total, float sigma_x,
                                 float sigma_theta, float sigma_E, int n_samples, unsigned int random_seed, int Nx,
                                 int Nz, float dx, float dz, float x_min, float z_min, int N_theta_local,
                                 int N_E_local, const AngularGrid& theta_grid, const EnergyGrid& E_grid,
                                 const ::DeviceRLUT& dlut, const TransportConfig& transport,
                                 std::vector<std::vector<double>>& edep);

std::string get_gpu_name_internal();

struct K1K6PipelineConfig {
    float E_fine_on;
    float E_fine_off;
    float weight_active_min;
    float E_coarse_max;
    float step_coarse;
    int n_steps_per_cell;
    float sigma_x_initial;
    float E0_MeV;
    int Nx, Nz;
    float dx, dz;
    int N_theta, N_E;
    int N_theta_local, N_E_local;
    int fine_batch_max_cells = 0;
    int max_iterations;
    int log_level;
    bool fail_fast_on_audit = false;
    bool debug_dumps_enabled = true;
};

struct K1K6PipelineState {
    DevicePsiC* psi_in;
    DevicePsiC* psi_out;
    uint8_t* d_ActiveMask;
    uint8_t* d_ActiveMask_prev;
    uint32_t* d_ActiveList;
    uint32_t* d_CoarseList;
    int n_active;
    int n_coarse;
    int* d_n_active;
    int* d_n_coarse;
    double* d_EdepC;
    float* d_AbsorbedWeight_cutoff;
    double* d_AbsorbedEnergy_cutoff;
    float* d_AbsorbedWeight_nuclear;
    double* d_AbsorbedEnergy_nuclear;
    float* d_BoundaryLoss_weight;
    double* d_BoundaryLoss_energy;
    float* d_prev_AbsorbedWeight_cutoff;
    double* d_prev_AbsorbedEnergy_cutoff;
    float* d_prev_AbsorbedWeight_nuclear;
    float* d_prev_BoundaryLoss_weight;
    double* d_prev_EdepC;
    double* d_prev_AbsorbedEnergy_nuclear;
    double* d_prev_BoundaryLoss_energy;
    DeviceOutflowBucket* d_BucketScratch;
    int bucket_scratch_capacity_cells;
    int* d_CellToBucketBase;
    float* d_theta_edges;
    float* d_E_edges;
    AuditReport* d_audit_report;
    double* d_weight_in;
    double* d_weight_out;
    float source_injected_weight;
    float source_out_of_grid_weight;
    float source_slot_dropped_weight;
    double source_injected_energy;
    double source_out_of_grid_energy;
    double source_slot_dropped_energy;
    double source_representation_loss_energy;
    double transport_dropped_weight;
    double transport_dropped_energy;
    double transport_audit_residual_energy;
    float* d_FE_moment_A;
    float* d_FE_moment_B;
    float* d_FE_sigma_total;
    bool owns_device_memory;

    K1K6PipelineState()
        : psi_in(nullptr), psi_out(nullptr), d_ActiveMask(nullptr), d_ActiveMask_prev(nullptr),
          d_ActiveList(nullptr), d_CoarseList(nullptr), n_active(0), n_coarse(0), d_n_active(nullptr),
          d_n_coarse(nullptr), d_EdepC(nullptr), d_AbsorbedWeight_cutoff(nullptr), d_AbsorbedEnergy_cutoff(nullptr),
          d_AbsorbedWeight_nuclear(nullptr), d_AbsorbedEnergy_nuclear(nullptr), d_BoundaryLoss_weight(nullptr),
          d_BoundaryLoss_energy(nullptr), d_prev_AbsorbedWeight_cutoff(nullptr),
          d_prev_AbsorbedEnergy_cutoff(nullptr), d_prev_AbsorbedWeight_nuclear(nullptr),
          d_prev_BoundaryLoss_weight(nullptr), d_prev_EdepC(nullptr), d_prev_AbsorbedEnergy_nuclear(nullptr),
          d_prev_BoundaryLoss_energy(nullptr), d_BucketScratch(nullptr), bucket_scratch_capacity_cells(0),
          d_CellToBucketBase(nullptr), d_theta_edges(nullptr), d_E_edges(nullptr), d_audit_report(nullptr),
          d_weight_in(nullptr), d_weight_out(nullptr), source_injected_weight(0.0f), source_out_of_grid_weight(0.0f),
          source_slot_dropped_weight(0.0f), source_injected_energy(0.0), source_out_of_grid_energy(0.0),
          source_slot_dropped_energy(0.0), source_representation_loss_energy(0.0), transport_dropped_weight(0.0),
          transport_dropped_energy(0.0), transport_audit_residual_energy(0.0), d_FE_moment_A(nullptr),
          d_FE_moment_B(nullptr), d_FE_sigma_total(nullptr), owns_device_memory(false) {}
    bool allocate(int Nx, int Nz);
    void cleanup();
    ~K1K6PipelineState() { cleanup(); }
};

bool run_k1k6_pipeline_transport(DevicePsiC* psi_in, DevicePsiC* psi_out, const ::DeviceRLUT& dlut,
                                 const EnergyGrid& e_grid, const AngularGrid& a_grid, const K1K6PipelineConfig& config,
                                 K1K6PipelineState& state);
bool run_k1_active_mask(const DevicePsiC& psi_in, uint8_t* d_ActiveMask, const uint8_t* d_ActiveMaskPrev, int Nx,
                        int Nz, int b_E_fine_on, int b_E_fine_off, float weight_active_min);
bool run_k2_coarse_transport(const DevicePsiC& psi_in, DevicePsiC& psi_out, const uint8_t* d_ActiveMask,
                             const uint32_t* d_CoarseList, int n_coarse, const ::DeviceRLUT& dlut,
                             const K1K6PipelineConfig& config, K1K6PipelineState& state);
bool run_k3_fine_transport(const DevicePsiC& psi_in, DevicePsiC& psi_out, const uint32_t* d_ActiveList, int n_active,
                           const ::DeviceRLUT& dlut, const K1K6PipelineConfig& config, K1K6PipelineState& state);
bool run_k4_bucket_transfer(DevicePsiC& psi_out, const DeviceOutflowBucket* d_OutflowBuckets,
                            const int* d_CellToBucketBase, int Nx, int Nz, const float* d_E_edges, int N_E,
                            int N_E_local);
bool run_k5_conservation_audit(const DevicePsiC& psi_in, const DevicePsiC& psi_out, const double* d_EdepC,
                               const double* d_AbsorbedEnergy_cutoff, const double* d_AbsorbedEnergy_nuclear,
                               const double* d_BoundaryLoss_energy, const double* d_prev_EdepC,
                               const double* d_prev_AbsorbedEnergy_cutoff, const double* d_prev_AbsorbedEnergy_nuclear,
                               const double* d_prev_BoundaryLoss_energy, const float* d_AbsorbedWeight_cutoff,
                               const float* d_AbsorbedWeight_nuclear, const float* d_BoundaryLoss_weight,
                               const float* d_prev_AbsorbedWeight_cutoff, const float* d_prev_AbsorbedWeight_nuclear,
                               const float* d_prev_BoundaryLoss_weight, float source_out_of_grid_weight,
                               float source_slot_dropped_weight, double source_out_of_grid_energy,
                               double source_slot_dropped_energy, float transport_dropped_weight,
                               double transport_dropped_energy, int include_source_terms, const float* d_E_edges,
                               int N_E, int N_E_local, AuditReport* d_report, int Nx, int Nz);
void run_k6_swap_buffers(DevicePsiC*& psi_in, DevicePsiC*& psi_out);
bool init_pipeline_state(const K1K6PipelineConfig& config, const EnergyGrid& e_grid, const AngularGrid& a_grid,
                         K1K6PipelineState& state);
void reset_pipeline_state(K1K6PipelineState& state, int Nx, int Nz);
AuditReport get_audit_report(const K1K6PipelineState& state, int Nx, int Nz);

}  // namespace sm_2d
