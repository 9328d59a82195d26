// shim_driver.cpp -- drives the C++ drop-in layer (libsm2d_ref.so) the way
// the reference's runner and its pipeline tests call that interface, and
// writes the results as raw doubles for tests/test_gpu_ref_shim.py.
//
//   shim_driver wrapper  OUT   run_k1k6_pipeline_transport from a beam
//                              description (the runner's call): edep [Nz][Nx]
//   shim_driver pipeline OUT   run_k1k6_pipeline_transport on DevicePsiC
//                              buffers holding an injected source, then the
//                              state: EdepC [Nc], the audit record's totals,
//                              the drop sums, the final phase space's weight
//   shim_driver stages   OUT   run_k1_active_mask on that source, and the
//                              answer of run_k2_coarse_transport
//
// Case: 40 MeV Gaussian beam (sigma_x 1.5 mm, sigma_theta 2 mrad, sigma_E
// 0.4 MeV, 400 samples, seed 11) on 40 x 80 cells of 0.5 mm, the runner's
// grids (36 theta bins on +-0.35 rad, the default piecewise energy groups).
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <string>
#include <tuple>
#include <vector>

#include "sm2d.h"
#include "sm2d_ref_types.hpp"

namespace {
constexpr int Nx = 40, Nz = 80;
constexpr float dx = 0.5f, dz = 0.5f, E0 = 40.0f, SX = 1.5f, STH = 0.002f, SE = 0.4f;
constexpr int NS = 400, MAXIT = 1000;
constexpr unsigned SEED = 11;

int write(const char* path, const std::vector<double>& v) {
    FILE* f = std::fopen(path, "wb");
    if (!f) return 1;
    std::fwrite(v.data(), sizeof(double), v.size(), f);
    std::fclose(f);
    return 0;
}
}  // namespace

int main(int argc, char** argv) {
    if (argc < 3) return 2;
    const std::string mode = argv[1];
    AngularGrid a(-0.35f, 0.35f, 36);
    EnergyGrid e = EnergyGrid::CreatePiecewise({{0.1f, 2.0f, 0.1f}, {2.0f, 20.0f, 0.2f}, {20.0f, 100.0f, 0.25f},
                                                {100.0f, 250.0f, 0.25f}});
    RLUT lut = GenerateRLUT(e);
    sm_2d::DeviceLUTWrapper w;
    if (!sm_2d::init_device_lut(lut, w)) return 3;
    const float x_min = -(Nx * dx) / 2.0f;
    if (mode == "wrapper") {
        sm_2d::TransportConfig tc;
        tc.max_iterations = MAXIT;
        tc.log_level = 0;
        std::vector<std::vector<double>> edep;
        if (!sm_2d::run_k1k6_pipeline_transport(0.0f, 0.0f, 0.0f, E0, 1.0f, SX, STH, SE, NS, SEED, Nx, Nz, dx, dz, x_min,
                                                0.0f, N_theta_local, N_E_local, a, e, *w.get(), tc, edep))
            return 4;
        std::vector<double> flat;
        for (const auto& row : edep) flat.insert(flat.end(), row.begin(), row.end());
        return write(argv[2], flat);
    }
    // a source in DevicePsiC buffers: the C ABI's injection, as the
    // reference's wrapper fills psi_in with its injection kernels
    sm2d_problem p{};
    p.Nx = Nx; p.Nz = Nz; p.dx = dx; p.dz = dz; p.x_min = x_min;
    p.N_theta = a.N_theta; p.theta_edges = a.edges.data();
    p.N_E = e.N_E; p.E_edges = e.edges.data(); p.E_min = e.E_min; p.E_max = e.E_max;
    p.nt_local = 4; p.ne_local = 2; p.nx_sub = 8; p.nz_sub = 4;
    p.E_fine_on = 10.0f; p.E_fine_off = 11.0f; p.weight_active_min = 1e-12f; p.step_coarse = 5.0f;
    p.sigma_x_initial = SX; p.E0 = E0; p.enable_straggling = 1; p.enable_nuclear = 1;
    p.max_iterations = MAXIT; p.lanes = 1;
    sm2d_handle h = nullptr;
    if (sm2d_create(&p, &h)) return 5;
    const sm2d_beam b{0.0f, 0.0f, 0.0f, E0, 1.0f, SX, STH, SE, NS, SEED};
    if (sm2d_inject(h, &b)) return 6;
    const size_t Nc = (size_t)Nx * Nz, ns = Nc * 32;
    std::vector<uint32_t> hb(ns);
    std::vector<float> hv(ns * LOCAL_BINS);
    double sc[17];
    if (sm2d_get_psi_in(h, hb.data(), hv.data()) || sm2d_get_scalars(h, sc)) return 7;
    sm2d_destroy(h);
    DevicePsiC pin{Nx, Nz, (int)Nc, 32, nullptr, nullptr}, pout = pin;
    for (DevicePsiC* q : {&pin, &pout}) {
        if (cudaMalloc(&q->block_id, ns * 4) != cudaSuccess || cudaMalloc(&q->value, ns * LOCAL_BINS * 4) != cudaSuccess)
            return 8;
        cudaMemset(q->block_id, 0xFF, ns * 4);
        cudaMemset(q->value, 0, ns * LOCAL_BINS * 4);
    }
    cudaMemcpy(pin.block_id, hb.data(), ns * 4, cudaMemcpyHostToDevice);
    cudaMemcpy(pin.value, hv.data(), ns * LOCAL_BINS * 4, cudaMemcpyHostToDevice);
    if (mode == "stages") {
        uint8_t *m = nullptr, *mp = nullptr;
        cudaMalloc(&m, Nc);
        cudaMalloc(&mp, Nc);
        cudaMemset(mp, 0, Nc);
        const int bon = e.FindBin(10.0f) / N_E_local, boff = e.FindBin(11.0f) / N_E_local;
        if (!sm_2d::run_k1_active_mask(pin, m, mp, Nx, Nz, bon, boff, 1e-12f)) return 9;
        std::vector<uint8_t> hm(Nc);
        cudaMemcpy(hm.data(), m, Nc, cudaMemcpyDeviceToHost);
        sm_2d::K1K6PipelineConfig cfg{};
        sm_2d::K1K6PipelineState st;
        const bool k2 = sm_2d::run_k2_coarse_transport(pin, pout, m, nullptr, 0, *w.get(), cfg, st);
        std::vector<double> out(hm.begin(), hm.end());
        out.push_back(k2 ? 1.0 : 0.0);
        return write(argv[2], out);
    }
    sm_2d::K1K6PipelineConfig cfg{};
    cfg.E_fine_on = 10.0f; cfg.E_fine_off = 11.0f; cfg.weight_active_min = 1e-12f; cfg.E_coarse_max = 300.0f;
    cfg.step_coarse = 5.0f; cfg.n_steps_per_cell = 1; cfg.sigma_x_initial = SX; cfg.E0_MeV = E0;
    cfg.Nx = Nx; cfg.Nz = Nz; cfg.dx = dx; cfg.dz = dz; cfg.N_theta = a.N_theta; cfg.N_E = e.N_E;
    cfg.N_theta_local = N_theta_local; cfg.N_E_local = N_E_local; cfg.max_iterations = MAXIT; cfg.log_level = 0;
    sm_2d::K1K6PipelineState st;
    if (!sm_2d::init_pipeline_state(cfg, e, a, st)) return 10;
    st.source_injected_weight = (float)sc[3];
    st.source_injected_energy = sc[4];
    st.source_out_of_grid_weight = (float)sc[5];
    st.source_out_of_grid_energy = sc[6];
    st.source_slot_dropped_weight = (float)sc[7];
    st.source_slot_dropped_energy = sc[8];
    st.source_representation_loss_energy = sc[9];
    if (!sm_2d::run_k1k6_pipeline_transport(&pin, &pout, *w.get(), e, a, cfg, st)) return 11;
    std::vector<double> out(Nc);
    cudaMemcpy(out.data(), st.d_EdepC, Nc * 8, cudaMemcpyDeviceToHost);
    const AuditReport r = sm_2d::get_audit_report(st, Nx, Nz);
    for (double v : {(double)r.W_in_total, (double)r.W_out_total, (double)r.W_cutoff_total, (double)r.W_nuclear_total,
                     (double)r.W_boundary_total, r.E_in_total, r.E_out_total, r.E_dep_total, r.E_cutoff_total,
                     r.E_nuclear_total, r.E_boundary_total, (double)r.W_pass, (double)r.E_pass,
                     st.transport_dropped_weight, st.transport_dropped_energy, st.transport_audit_residual_energy})
        out.push_back(v);
    // what the buffers hold at the end: weight in psi_in, weight in psi_out
    for (DevicePsiC* q : {&pin, &pout}) {
        cudaMemcpy(hv.data(), q->value, ns * LOCAL_BINS * 4, cudaMemcpyDeviceToHost);
        double s = 0.0;
        for (float v : hv) s += v;
        out.push_back(s);
    }
    return write(argv[2], out);
}
