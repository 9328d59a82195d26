// sm2d_ref_shim.cpp -- the SM_2D transport path's C++ entry points over the
// C ABI of sm2d.h: linked in place of the reference's
// src/cuda/gpu_transport_wrapper.cu and src/cuda/k1k6_pipeline.cu, the
// reference's runner (GPUTransportRunner::run), its run_simulation command
// and code that drives the pipeline or its stages on DevicePsiC buffers call
// this library's kernels unchanged.
//
// Built against include/sm2d_ref_types.hpp, or against the SM_2D tree's own
// headers with -DSM2D_SHIM_REFERENCE_HEADERS (the same names, member order
// and types; a build recipe checks both).  Conventions kept from the
// reference: bool results with a message on stderr, the default device and
// stream, a device synchronisation before each entry returns.
//
// What differs, by design of the engine under it:
//   * K2 and K3 run as one deterministic pass (claim pass, slot selection,
//     deposit pass over both batches), so run_k2_coarse_transport and
//     run_k3_fine_transport have no stand-alone form: they report that and
//     return false.  The pipeline entry and sm2d_step run both stages.
//   * The engine builds its R-LUT on the device from the energy grid with
//     GenerateRLUT's arithmetic (r_lut.cpp:69-129); the dlut argument must be
//     the LUT of that grid, as the reference's runner passes it.
#ifdef SM2D_SHIM_REFERENCE_HEADERS
#include "core/grids.hpp"
#include "core/incident_particle_config.hpp"
#include "cuda/gpu_transport_wrapper.hpp"
#include "k1k6_pipeline.cuh"
#include "lut/r_lut.hpp"
#else
#include "sm2d_ref_types.hpp"
#endif

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <iostream>
#include <map>
#include <utility>
#include <vector>

#include "sm2d.h"

namespace {

bool say(const char* where) {
    std::cerr << where << ": " << sm2d_last_error() << std::endl;
    return false;
}
bool cuda_ok(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return true;
    std::cerr << what << ": " << cudaGetErrorString(e) << std::endl;
    return false;
}

// local-bin layout of (N_theta_local, N_E_local): the sub-cell bins that
// complete it (local_bins.hpp:19-23 for (4, 2); the 128-bin layout (8, 4)
// with 4 x sub-bins)
bool layout_of(int ntl, int nel, sm2d_problem& p) {
    if (ntl == 4 && nel == 2) {
        p.nt_local = 4; p.ne_local = 2; p.nx_sub = 8; p.nz_sub = 4;
        return true;
    }
    if (ntl == 8 && nel == 4) {
        p.nt_local = 8; p.ne_local = 4; p.nx_sub = 4; p.nz_sub = 1;
        return true;
    }
    std::cerr << "local bins " << ntl << " x " << nel << ": the engine has kernels for 4 x 2 and 8 x 4" << std::endl;
    return false;
}

sm2d_problem problem_of(int Nx, int Nz, float dx, float dz, float x_min, float z_min, const AngularGrid& a,
                        const EnergyGrid& e) {
    sm2d_problem p{};
    p.Nx = Nx; p.Nz = Nz; p.dx = dx; p.dz = dz;
    p.x_min = x_min; p.z_min = z_min;
    p.N_theta = a.N_theta; p.theta_edges = a.edges.data();
    p.N_E = e.N_E; p.E_edges = e.edges.data();
    p.E_min = e.E_min; p.E_max = e.E_max;
    p.enable_straggling = 1;
    p.enable_nuclear = 1;
    p.lanes = 1;
    return p;
}

struct Handle {   // one engine for the duration of a call
    sm2d_handle h = nullptr;
    ~Handle() {
        if (h) sm2d_destroy(h);
    }
};

// the fused K4's drop accumulator of run_k4_bucket_transfer, per device
double* k4_drops() {
    static std::map<int, double*> per_dev;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
    auto it = per_dev.find(dev);
    if (it != per_dev.end()) return it->second;
    double* p = nullptr;
    if (cudaMalloc(&p, 2 * sizeof(double)) != cudaSuccess) return nullptr;
    cudaMemset(p, 0, 2 * sizeof(double));
    per_dev[dev] = p;
    return p;
}

bool psic_clear(DevicePsiC& p) {
    const size_t n = (size_t)p.N_cells * p.Kb;
    return cuda_ok(cudaMemset(p.block_id, 0xFF, n * sizeof(uint32_t)), "psi clear") &&
           cuda_ok(cudaMemset(p.value, 0, n * LOCAL_BINS * sizeof(float)), "psi clear");
}

}  // namespace

namespace sm_2d {

// ---------------------------------------------------------------- gpu_transport_wrapper.hpp
class DeviceLUTWrapperImpl {
public:
    ::DeviceRLUT dlut{};
    std::vector<void*> bufs;
    ~DeviceLUTWrapperImpl() {
        for (void* p : bufs) cudaFree(p);
    }
    const float* upload(const std::vector<float>& v) {
        void* p = nullptr;
        if (v.empty() || cudaMalloc(&p, v.size() * sizeof(float)) != cudaSuccess) return nullptr;
        bufs.push_back(p);
        if (cudaMemcpy(p, v.data(), v.size() * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess) return nullptr;
        return static_cast<const float*>(p);
    }
};

DeviceLUTWrapper::DeviceLUTWrapper() : p_impl(new DeviceLUTWrapperImpl()), dlut_ptr(nullptr) {}
DeviceLUTWrapper::~DeviceLUTWrapper() { delete p_impl; }

// DeviceLUTWrapper::init (k3_finetransport.cuh:114-150): the host LUT's
// arrays and the grid's edges on the device
bool init_device_lut(const ::RLUT& cpu_lut, DeviceLUTWrapper& wrapper) {
    DeviceLUTWrapperImpl& m = *wrapper.p_impl;
    ::DeviceRLUT d{};
    d.N_E = cpu_lut.grid.N_E;
    d.E_min = cpu_lut.grid.E_min;
    d.E_max = cpu_lut.grid.E_max;
    d.R = m.upload(cpu_lut.R);
    d.S = m.upload(cpu_lut.S);
    d.log_E = m.upload(cpu_lut.log_E);
    d.log_R = m.upload(cpu_lut.log_R);
    d.log_S = m.upload(cpu_lut.log_S);
    d.E_edges = m.upload(cpu_lut.grid.edges);
    if (!d.R || !d.S || !d.log_E || !d.log_R || !d.log_S || !d.E_edges) {
        std::cerr << "init_device_lut: device copy of the LUT failed" << std::endl;
        return false;
    }
    m.dlut = d;
    wrapper.dlut_ptr = &m.dlut;
    return true;
}

// One spot from its beam description to the post-convolved dose
// (gpu_transport_wrapper.cu:213-640): the engine injects the pencil or the
// sampled Gaussian source, runs the device loop and convolves the deposit.
bool run_k1k6_pipeline_transport(float x0, float z0, float theta0, float E0, float W_total, float sigma_x,
                                 float sigma_theta, float sigma_E, int n_samples, unsigned int random_seed, int Nx,
                                 int Nz, float dx, float dz, float x_min, float z_min, int N_theta_local,
                                 int N_E_local, const AngularGrid& theta_grid, const EnergyGrid& e_grid,
                                 const ::DeviceRLUT& dlut, const TransportConfig& transport,
                                 std::vector<std::vector<double>>& edep) {
    (void)dlut;
    if (transport.max_iterations <= 0) {
        std::cerr << "Invalid max_iterations: " << transport.max_iterations << std::endl;
        return false;
    }
    sm2d_problem p = problem_of(Nx, Nz, dx, dz, x_min, z_min, theta_grid, e_grid);
    if (!layout_of(N_theta_local, N_E_local, p)) return false;
    p.E_fine_on = transport.E_fine_on;
    p.E_fine_off = transport.E_fine_off;
    p.weight_active_min = transport.weight_active_min;
    p.step_coarse = transport.step_coarse;
    p.sigma_x_initial = sigma_x;
    p.E0 = E0;
    p.max_iterations = transport.max_iterations;
    Handle H;
    if (sm2d_create(&p, &H.h)) return say("run_k1k6_pipeline_transport");
    const sm2d_beam b{x0, z0, theta0, E0, W_total, sigma_x, sigma_theta, sigma_E, n_samples, random_seed};
    int done = 0;
    if (sm2d_inject(H.h, &b) || sm2d_run(H.h, transport.max_iterations, &done))
        return say("run_k1k6_pipeline_transport");
    std::vector<double> dose((size_t)Nx * Nz);
    if (sm2d_get_dose(H.h, dose.data())) return say("run_k1k6_pipeline_transport");
    edep.assign(Nz, std::vector<double>(Nx, 0.0));
    for (int iz = 0; iz < Nz; ++iz)
        std::copy_n(dose.data() + (size_t)iz * Nx, Nx, edep[iz].begin());
    if (transport.log_level >= 1) {
        sm2d_audit a{};
        sm2d_get_audit(H.h, &a);
        std::cout << "  K1-K6 pipeline: " << done << " iterations, last audit W " << (a.W_pass ? "pass" : "FAIL")
                  << ", E " << (a.E_pass ? "pass" : "FAIL") << std::endl;
    }
    return true;
}

std::string get_gpu_name_internal() {
    cudaDeviceProp prop{};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&prop, dev) != cudaSuccess) return "unknown";
    return prop.name;
}

// ---------------------------------------------------------------- k1k6_pipeline.cuh: state
bool K1K6PipelineState::allocate(int Nx, int Nz) {
    const size_t n = (size_t)Nx * Nz;
    bool ok = true;
    auto A = [&](auto** p, size_t bytes, const char* name) {
        if (ok) ok = cuda_ok(cudaMalloc((void**)p, bytes ? bytes : 1), name);
    };
    A(&d_ActiveMask, n, "d_ActiveMask");
    A(&d_ActiveMask_prev, n, "d_ActiveMask_prev");
    A(&d_ActiveList, n * 4, "d_ActiveList");
    A(&d_CoarseList, n * 4, "d_CoarseList");
    A(&d_n_active, sizeof(int), "d_n_active");
    A(&d_n_coarse, sizeof(int), "d_n_coarse");
    A(&d_EdepC, n * 8, "d_EdepC");
    A(&d_AbsorbedWeight_cutoff, n * 4, "d_AbsorbedWeight_cutoff");
    A(&d_AbsorbedEnergy_cutoff, n * 8, "d_AbsorbedEnergy_cutoff");
    A(&d_AbsorbedWeight_nuclear, n * 4, "d_AbsorbedWeight_nuclear");
    A(&d_AbsorbedEnergy_nuclear, n * 8, "d_AbsorbedEnergy_nuclear");
    A(&d_BoundaryLoss_weight, n * 4, "d_BoundaryLoss_weight");
    A(&d_BoundaryLoss_energy, n * 8, "d_BoundaryLoss_energy");
    A(&d_prev_AbsorbedWeight_cutoff, n * 4, "d_prev_AbsorbedWeight_cutoff");
    A(&d_prev_AbsorbedEnergy_cutoff, n * 8, "d_prev_AbsorbedEnergy_cutoff");
    A(&d_prev_AbsorbedWeight_nuclear, n * 4, "d_prev_AbsorbedWeight_nuclear");
    A(&d_prev_BoundaryLoss_weight, n * 4, "d_prev_BoundaryLoss_weight");
    A(&d_prev_EdepC, n * 8, "d_prev_EdepC");
    A(&d_prev_AbsorbedEnergy_nuclear, n * 8, "d_prev_AbsorbedEnergy_nuclear");
    A(&d_prev_BoundaryLoss_energy, n * 8, "d_prev_BoundaryLoss_energy");
    A(&d_FE_moment_A, (size_t)Nz * 4, "d_FE_moment_A");
    A(&d_FE_moment_B, (size_t)Nz * 4, "d_FE_moment_B");
    A(&d_FE_sigma_total, (size_t)Nz * 4, "d_FE_sigma_total");
    A(&d_CellToBucketBase, n * 4, "d_CellToBucketBase");
    A(&d_audit_report, sizeof(AuditReport), "d_audit_report");
    A(&d_weight_in, n * 8, "d_weight_in");
    A(&d_weight_out, n * 8, "d_weight_out");
    owns_device_memory = true;   // what was allocated is released by cleanup
    return ok;
}

void K1K6PipelineState::cleanup() {
    if (!owns_device_memory) return;
    void* ps[] = {d_ActiveMask, d_ActiveMask_prev, d_ActiveList, d_CoarseList, d_n_active, d_n_coarse, d_EdepC,
                  d_AbsorbedWeight_cutoff, d_AbsorbedEnergy_cutoff, d_AbsorbedWeight_nuclear,
                  d_AbsorbedEnergy_nuclear, d_BoundaryLoss_weight, d_BoundaryLoss_energy,
                  d_prev_AbsorbedWeight_cutoff, d_prev_AbsorbedEnergy_cutoff, d_prev_AbsorbedWeight_nuclear,
                  d_prev_BoundaryLoss_weight, d_prev_EdepC, d_prev_AbsorbedEnergy_nuclear, d_prev_BoundaryLoss_energy,
                  d_FE_sigma_total, d_FE_moment_A, d_FE_moment_B, d_BucketScratch, d_CellToBucketBase, d_theta_edges,
                  d_E_edges, d_audit_report, d_weight_in, d_weight_out};
    for (void* p : ps)
        if (p) cudaFree(p);
    d_ActiveMask = d_ActiveMask_prev = nullptr;
    d_ActiveList = d_CoarseList = nullptr;
    d_n_active = d_n_coarse = nullptr;
    d_EdepC = d_AbsorbedEnergy_cutoff = d_AbsorbedEnergy_nuclear = d_BoundaryLoss_energy = nullptr;
    d_AbsorbedWeight_cutoff = d_AbsorbedWeight_nuclear = d_BoundaryLoss_weight = nullptr;
    d_prev_AbsorbedWeight_cutoff = d_prev_AbsorbedWeight_nuclear = d_prev_BoundaryLoss_weight = nullptr;
    d_prev_AbsorbedEnergy_cutoff = d_prev_EdepC = d_prev_AbsorbedEnergy_nuclear = d_prev_BoundaryLoss_energy = nullptr;
    d_FE_sigma_total = d_FE_moment_A = d_FE_moment_B = nullptr;
    d_BucketScratch = nullptr;
    bucket_scratch_capacity_cells = 0;
    d_CellToBucketBase = nullptr;
    d_theta_edges = d_E_edges = nullptr;
    d_audit_report = nullptr;
    d_weight_in = d_weight_out = nullptr;
    owns_device_memory = false;
}

// state arrays, grid edges on the device and the Fermi-Eyges moments of the
// configured beam (k1k6_pipeline.cu:1002-1215)
bool init_pipeline_state(const K1K6PipelineConfig& config, const EnergyGrid& e_grid, const AngularGrid& a_grid,
                         K1K6PipelineState& state) {
    if (!state.allocate(config.Nx, config.Nz)) {
        state.cleanup();
        return false;
    }
    bool ok = cuda_ok(cudaMalloc((void**)&state.d_theta_edges, (config.N_theta + 1) * sizeof(float)), "d_theta_edges") &&
              cuda_ok(cudaMalloc((void**)&state.d_E_edges, (config.N_E + 1) * sizeof(float)), "d_E_edges") &&
              cuda_ok(cudaMemcpy(state.d_theta_edges, a_grid.edges.data(), (config.N_theta + 1) * sizeof(float),
                                 cudaMemcpyHostToDevice), "copy d_theta_edges") &&
              cuda_ok(cudaMemcpy(state.d_E_edges, e_grid.edges.data(), (config.N_E + 1) * sizeof(float),
                                 cudaMemcpyHostToDevice), "copy d_E_edges");
    const int Nz = config.Nz;
    if (ok && config.E0_MeV > 0.0f) {
        std::vector<float> A(Nz), B(Nz), S(Nz);
        if (sm2d_fermi_eyges(config.E0_MeV, Nz, config.dz, config.sigma_x_initial, A.data(), B.data(), S.data()))
            ok = say("init_pipeline_state");
        ok = ok && cuda_ok(cudaMemcpy(state.d_FE_sigma_total, S.data(), Nz * 4, cudaMemcpyHostToDevice), "FE copy") &&
             cuda_ok(cudaMemcpy(state.d_FE_moment_A, A.data(), Nz * 4, cudaMemcpyHostToDevice), "FE copy") &&
             cuda_ok(cudaMemcpy(state.d_FE_moment_B, B.data(), Nz * 4, cudaMemcpyHostToDevice), "FE copy");
    } else if (ok) {
        ok = cuda_ok(cudaMemset(state.d_FE_moment_A, 0, Nz * 4), "FE clear") &&
             cuda_ok(cudaMemset(state.d_FE_moment_B, 0, Nz * 4), "FE clear") &&
             cuda_ok(cudaMemset(state.d_FE_sigma_total, 0, Nz * 4), "FE clear");
    }
    if (!ok) state.cleanup();
    return ok;
}

// k1k6_pipeline.cu:1217-1247
void reset_pipeline_state(K1K6PipelineState& state, int Nx, int Nz) {
    const size_t n = (size_t)Nx * Nz;
    cudaMemset(state.d_ActiveMask, 0, n);
    cudaMemset(state.d_ActiveMask_prev, 0, n);
    for (double* p : {state.d_EdepC, state.d_AbsorbedEnergy_cutoff, state.d_AbsorbedEnergy_nuclear,
                      state.d_BoundaryLoss_energy, state.d_prev_AbsorbedEnergy_cutoff, state.d_prev_EdepC,
                      state.d_prev_AbsorbedEnergy_nuclear, state.d_prev_BoundaryLoss_energy})
        cudaMemset(p, 0, n * 8);
    for (float* p : {state.d_AbsorbedWeight_cutoff, state.d_AbsorbedWeight_nuclear, state.d_BoundaryLoss_weight,
                     state.d_prev_AbsorbedWeight_cutoff, state.d_prev_AbsorbedWeight_nuclear,
                     state.d_prev_BoundaryLoss_weight})
        cudaMemset(p, 0, n * 4);
    cudaMemset(state.d_CellToBucketBase, 0xFF, n * 4);
    cudaMemset(state.d_n_active, 0, sizeof(int));
    cudaMemset(state.d_n_coarse, 0, sizeof(int));
    state.transport_dropped_weight = 0.0;
    state.transport_dropped_energy = 0.0;
    state.transport_audit_residual_energy = 0.0;
}

AuditReport get_audit_report(const K1K6PipelineState& state, int Nx, int Nz) {
    (void)Nx;
    (void)Nz;
    AuditReport r{};
    cudaMemcpy(&r, state.d_audit_report, sizeof(AuditReport), cudaMemcpyDeviceToHost);
    return r;
}

// ---------------------------------------------------------------- k1k6_pipeline.cuh: the loop
// The transport of the phase space in psi_in until no cell holds weight or
// config.max_iterations passed (k1k6_pipeline.cu:1540-2038).  The state
// receives what the reference's loop leaves there: the cumulative tallies
// (and their previous-iteration copies), the last audit record, the drop and
// residual sums; the source accounting fields are read from it for the first
// iteration's audit.  The final phase space is in the buffer the reference's
// pointer swaps end on (psi_in after an even number of iterations, psi_out
// after an odd one); the other buffer is cleared.
bool run_k1k6_pipeline_transport(DevicePsiC* psi_in, DevicePsiC* psi_out, const ::DeviceRLUT& dlut,
                                 const EnergyGrid& e_grid, const AngularGrid& a_grid, const K1K6PipelineConfig& config,
                                 K1K6PipelineState& state) {
    (void)dlut;
    if (config.max_iterations <= 0) {
        std::cerr << "Invalid max_iterations: " << config.max_iterations << std::endl;
        return false;
    }
    if (!psi_in || !psi_out || psi_in->Kb != 32 || psi_in->N_cells != config.Nx * config.Nz) {
        std::cerr << "run_k1k6_pipeline_transport: phase-space buffers do not match the grid" << std::endl;
        return false;
    }
    if (config.N_theta_local != N_theta_local || config.N_E_local != N_E_local) {
        std::cerr << "run_k1k6_pipeline_transport: DevicePsiC holds " << LOCAL_BINS << " local bins ("
                  << N_theta_local << " x " << N_E_local << ")" << std::endl;
        return false;
    }
    reset_pipeline_state(state, config.Nx, config.Nz);
    sm2d_problem p = problem_of(config.Nx, config.Nz, config.dx, config.dz, -(config.Nx * config.dx) / 2.0f, 0.0f,
                                a_grid, e_grid);
    layout_of(config.N_theta_local, config.N_E_local, p);
    p.E_fine_on = config.E_fine_on;
    p.E_fine_off = config.E_fine_off;
    p.weight_active_min = config.weight_active_min;
    p.step_coarse = config.step_coarse;
    p.sigma_x_initial = config.sigma_x_initial;
    p.E0 = config.E0_MeV;
    p.max_iterations = config.max_iterations;
    Handle H;
    if (sm2d_create(&p, &H.h)) return say("run_k1k6_pipeline_transport");
    const double src[7] = {state.source_injected_weight, state.source_out_of_grid_weight,
                           state.source_slot_dropped_weight, state.source_injected_energy,
                           state.source_out_of_grid_energy, state.source_slot_dropped_energy,
                           state.source_representation_loss_energy};
    int done = 0;
    if (sm2d_set_psi_in_device(H.h, psi_in->block_id, psi_in->value) || sm2d_set_source_accounting(H.h, src) ||
        sm2d_run(H.h, config.max_iterations, &done))
        return say("run_k1k6_pipeline_transport");
    // tallies, their previous-iteration copies and the last audit record
    const size_t n = (size_t)config.Nx * config.Nz;
    std::vector<double> edep(n), ecut(n), enuc(n), ebnd(n);
    std::vector<float> wcut(n), wnuc(n), wbnd(n);
    sm2d_audit a{};
    double sc[17];
    if (sm2d_get_tallies(H.h, edep.data(), wcut.data(), ecut.data(), wnuc.data(), enuc.data(), wbnd.data(),
                         ebnd.data()) ||
        sm2d_get_audit(H.h, &a) || sm2d_get_scalars(H.h, sc))
        return say("run_k1k6_pipeline_transport");
    static_assert(sizeof(sm2d_audit) == sizeof(AuditReport), "AuditReport layout");
    bool ok = true;
    auto up = [&](void* dst, const void* srcp, size_t bytes) {
        if (ok) ok = cuda_ok(cudaMemcpy(dst, srcp, bytes, cudaMemcpyHostToDevice), "state copy");
    };
    up(state.d_EdepC, edep.data(), n * 8);
    up(state.d_prev_EdepC, edep.data(), n * 8);
    up(state.d_AbsorbedEnergy_cutoff, ecut.data(), n * 8);
    up(state.d_prev_AbsorbedEnergy_cutoff, ecut.data(), n * 8);
    up(state.d_AbsorbedEnergy_nuclear, enuc.data(), n * 8);
    up(state.d_prev_AbsorbedEnergy_nuclear, enuc.data(), n * 8);
    up(state.d_BoundaryLoss_energy, ebnd.data(), n * 8);
    up(state.d_prev_BoundaryLoss_energy, ebnd.data(), n * 8);
    up(state.d_AbsorbedWeight_cutoff, wcut.data(), n * 4);
    up(state.d_prev_AbsorbedWeight_cutoff, wcut.data(), n * 4);
    up(state.d_AbsorbedWeight_nuclear, wnuc.data(), n * 4);
    up(state.d_prev_AbsorbedWeight_nuclear, wnuc.data(), n * 4);
    up(state.d_BoundaryLoss_weight, wbnd.data(), n * 4);
    up(state.d_prev_BoundaryLoss_weight, wbnd.data(), n * 4);
    up(state.d_audit_report, &a, sizeof(AuditReport));
    if (!ok) return false;
    state.transport_dropped_weight = sc[0];
    state.transport_dropped_energy = sc[1];
    state.transport_audit_residual_energy = sc[2];
    state.n_active = state.n_coarse = 0;
    DevicePsiC* fin = (done & 1) ? psi_out : psi_in;
    DevicePsiC* other = (done & 1) ? psi_in : psi_out;
    if (sm2d_get_psi_in_device(H.h, fin->block_id, fin->value)) return say("run_k1k6_pipeline_transport");
    return psic_clear(*other) && cuda_ok(cudaDeviceSynchronize(), "run_k1k6_pipeline_transport");
}

// ---------------------------------------------------------------- k1k6_pipeline.cuh: stages
bool run_k1_active_mask(const DevicePsiC& psi_in, uint8_t* d_ActiveMask, const uint8_t* d_ActiveMaskPrev, int Nx,
                        int Nz, int b_E_fine_on, int b_E_fine_off, float weight_active_min) {
    if (sm2d_k1_active_mask(psi_in.block_id, psi_in.value, d_ActiveMask, d_ActiveMaskPrev, Nx, Nz, LOCAL_BINS,
                            b_E_fine_on, b_E_fine_off, weight_active_min, nullptr))
        return say("K1 kernel launch failed");
    return cuda_ok(cudaDeviceSynchronize(), "K1");
}

bool run_k2_coarse_transport(const DevicePsiC&, DevicePsiC&, const uint8_t*, const uint32_t*, int, const ::DeviceRLUT&,
                             const K1K6PipelineConfig&, K1K6PipelineState&) {
    std::cerr << "run_k2_coarse_transport: K2 and K3 run as one deterministic pass in this library; call "
                 "run_k1k6_pipeline_transport (or sm2d_step for one iteration)" << std::endl;
    return false;
}

bool run_k3_fine_transport(const DevicePsiC&, DevicePsiC&, const uint32_t*, int, const ::DeviceRLUT&,
                           const K1K6PipelineConfig&, K1K6PipelineState&) {
    std::cerr << "run_k3_fine_transport: K2 and K3 run as one deterministic pass in this library; call "
                 "run_k1k6_pipeline_transport (or sm2d_step for one iteration)" << std::endl;
    return false;
}

bool run_k4_bucket_transfer(DevicePsiC& psi_out, const DeviceOutflowBucket* d_OutflowBuckets,
                            const int* d_CellToBucketBase, int Nx, int Nz, const float* d_E_edges, int N_E,
                            int N_E_local_) {
    double* drops = k4_drops();
    if (!drops) return cuda_ok(cudaErrorMemoryAllocation, "K4 drop accumulator");
    if (sm2d_k4_bucket_transfer(d_OutflowBuckets, d_CellToBucketBase, psi_out.value, psi_out.block_id, Nx, Nz,
                                LOCAL_BINS, N_theta_local, N_E_local, N_x_sub, d_E_edges, N_E, N_E_local_, drops,
                                nullptr))
        return say("K4 kernel launch failed");
    return cuda_ok(cudaDeviceSynchronize(), "K4");
}

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
                               int N_E, int N_E_local_, AuditReport* d_report, int Nx, int Nz) {
    if (sm2d_k5_conservation_audit(
            psi_in.block_id, psi_in.value, psi_out.block_id, psi_out.value, d_EdepC, d_AbsorbedEnergy_nuclear,
            d_BoundaryLoss_energy, d_AbsorbedEnergy_cutoff, d_prev_EdepC, d_prev_AbsorbedEnergy_nuclear,
            d_prev_BoundaryLoss_energy, d_prev_AbsorbedEnergy_cutoff, d_AbsorbedWeight_cutoff,
            d_AbsorbedWeight_nuclear, d_BoundaryLoss_weight, d_prev_AbsorbedWeight_cutoff,
            d_prev_AbsorbedWeight_nuclear, d_prev_BoundaryLoss_weight, source_out_of_grid_weight,
            source_slot_dropped_weight, source_out_of_grid_energy, source_slot_dropped_energy,
            transport_dropped_weight, transport_dropped_energy, include_source_terms, d_E_edges, N_E, N_theta_local,
            N_E_local_, LOCAL_BINS, reinterpret_cast<sm2d_audit*>(d_report), Nx * Nz, nullptr))
        return say("K5 kernel launch failed");
    return cuda_ok(cudaDeviceSynchronize(), "K5");
}

void run_k6_swap_buffers(DevicePsiC*& psi_in, DevicePsiC*& psi_out) { std::swap(psi_in, psi_out); }

}  // namespace sm_2d
