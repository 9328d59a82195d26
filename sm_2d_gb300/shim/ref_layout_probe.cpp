// ref_layout_probe.cpp -- prints the size and member offsets of every type
// the C++ drop-in layer exchanges with callers.  check_reference_abi.sh
// builds it once against include/sm2d_ref_types.hpp and once against the
// SM_2D tree's headers (-DSM2D_SHIM_REFERENCE_HEADERS); the two outputs must
// be equal.
#ifdef SM2D_SHIM_REFERENCE_HEADERS
#include "core/grids.hpp"
#include "core/incident_particle_config.hpp"
#include "cuda/gpu_transport_wrapper.hpp"
#include "k1k6_pipeline.cuh"
#include "lut/r_lut.hpp"
#else
#include "sm2d_ref_types.hpp"
#endif
#include <cstddef>
#include <cstdio>

#define SIZE(T) std::printf("sizeof %s %zu\n", #T, sizeof(T))
#define OFF(T, m) std::printf("offsetof %s.%s %zu\n", #T, #m, offsetof(T, m))

int main() {
    using sm_2d::K1K6PipelineConfig;
    using sm_2d::K1K6PipelineState;
    using sm_2d::TransportConfig;
    using sm_2d::TransportEnergyGroup;
    SIZE(EnergyGrid); OFF(EnergyGrid, N_E); OFF(EnergyGrid, E_min); OFF(EnergyGrid, E_max); OFF(EnergyGrid, edges);
    OFF(EnergyGrid, rep); OFF(EnergyGrid, is_piecewise);
    SIZE(AngularGrid); OFF(AngularGrid, N_theta); OFF(AngularGrid, theta_min); OFF(AngularGrid, theta_max);
    OFF(AngularGrid, edges); OFF(AngularGrid, rep);
    SIZE(RLUT); OFF(RLUT, grid); OFF(RLUT, R); OFF(RLUT, S); OFF(RLUT, log_E); OFF(RLUT, log_R); OFF(RLUT, log_S);
    SIZE(DeviceRLUT); OFF(DeviceRLUT, N_E); OFF(DeviceRLUT, E_min); OFF(DeviceRLUT, E_max); OFF(DeviceRLUT, R);
    OFF(DeviceRLUT, S); OFF(DeviceRLUT, log_E); OFF(DeviceRLUT, log_R); OFF(DeviceRLUT, log_S);
    OFF(DeviceRLUT, E_edges);
    SIZE(DevicePsiC); OFF(DevicePsiC, Nx); OFF(DevicePsiC, Nz); OFF(DevicePsiC, N_cells); OFF(DevicePsiC, Kb);
    OFF(DevicePsiC, block_id); OFF(DevicePsiC, value);
    SIZE(AuditReport); OFF(AuditReport, W_pass); OFF(AuditReport, W_in_total); OFF(AuditReport, W_transport_drop_total);
    OFF(AuditReport, E_in_total); OFF(AuditReport, E_transport_drop_total); OFF(AuditReport, processed_cells);
    SIZE(TransportEnergyGroup);
    SIZE(TransportConfig); OFF(TransportConfig, N_theta); OFF(TransportConfig, energy_groups);
    OFF(TransportConfig, E_fine_on); OFF(TransportConfig, E_fine_off); OFF(TransportConfig, weight_active_min);
    OFF(TransportConfig, step_coarse); OFF(TransportConfig, preflight_vram_margin);
    OFF(TransportConfig, validation_mode); OFF(TransportConfig, fail_fast_on_audit); OFF(TransportConfig, debug_dumps);
    OFF(TransportConfig, max_iterations); OFF(TransportConfig, log_level);
    SIZE(K1K6PipelineConfig); OFF(K1K6PipelineConfig, E_fine_on); OFF(K1K6PipelineConfig, step_coarse);
    OFF(K1K6PipelineConfig, sigma_x_initial); OFF(K1K6PipelineConfig, E0_MeV); OFF(K1K6PipelineConfig, Nx);
    OFF(K1K6PipelineConfig, dz); OFF(K1K6PipelineConfig, N_theta); OFF(K1K6PipelineConfig, N_E_local);
    OFF(K1K6PipelineConfig, fine_batch_max_cells); OFF(K1K6PipelineConfig, max_iterations);
    OFF(K1K6PipelineConfig, log_level); OFF(K1K6PipelineConfig, fail_fast_on_audit);
    OFF(K1K6PipelineConfig, debug_dumps_enabled);
    SIZE(K1K6PipelineState); OFF(K1K6PipelineState, psi_in); OFF(K1K6PipelineState, d_ActiveMask);
    OFF(K1K6PipelineState, n_active); OFF(K1K6PipelineState, d_EdepC); OFF(K1K6PipelineState, d_BoundaryLoss_energy);
    OFF(K1K6PipelineState, d_prev_BoundaryLoss_energy); OFF(K1K6PipelineState, d_BucketScratch);
    OFF(K1K6PipelineState, bucket_scratch_capacity_cells); OFF(K1K6PipelineState, d_CellToBucketBase);
    OFF(K1K6PipelineState, d_E_edges); OFF(K1K6PipelineState, d_audit_report); OFF(K1K6PipelineState, d_weight_out);
    OFF(K1K6PipelineState, source_injected_weight); OFF(K1K6PipelineState, source_slot_dropped_weight);
    OFF(K1K6PipelineState, source_injected_energy); OFF(K1K6PipelineState, source_representation_loss_energy);
    OFF(K1K6PipelineState, transport_audit_residual_energy); OFF(K1K6PipelineState, d_FE_moment_A);
    OFF(K1K6PipelineState, d_FE_sigma_total); OFF(K1K6PipelineState, owns_device_memory);
    SIZE(sm_2d::DeviceLUTWrapper);
    std::printf("LOCAL_BINS %d %d %d %d %d\n", N_theta_local, N_E_local, N_x_sub, N_z_sub, LOCAL_BINS);
    return 0;
}
