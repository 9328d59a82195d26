// sm2d_output.cpp -- depth-dose metrics and output files of a dose grid
// dose[Nz][Nx] (the post-convolved EdepC of one spot, sm2d_get_dose), in the
// reference's text formats, so that its plotting and comparison scripts read
// them unchanged.  Host code, no GPU needed.
//
// Formats (kept alike on purpose: they are the files the reference writes):
//   dose_2d.txt  run_simulation.cpp:31-75  two '#' header lines, then per
//                row z and column x "x\tz\tdose[\tdose/max]" in fixed point
//                with 4 decimals, a blank line after each row; NaN/inf doses
//                print as 0
//   pdd.txt      run_simulation.cpp:80-114 three '#' header lines (the third
//                names the Bragg peak in default stream formatting), then
//                "depth\tdose[\tdose/peak]" per row, fixed point, 4 decimals
// Cell centres and depths are computed as the reference's runner does
// (gpu_transport_runner.cpp:52-62, float arithmetic): x = (i + 0.5) dx -
// Nx dx / 2, z = j dz.
#include <algorithm>
#include <cmath>
#include <fstream>
#include <iomanip>
#include <string>
#include <vector>

#include "sm2d.h"
#include "sm2d_tables.h"

namespace {

// sum over x of row j in double, columns in order (get_depth_dose,
// deterministic_beam.cpp:224-236)
double row_sum(const double* dose, int Nx, int j) {
    double s = 0.0;
    for (int i = 0; i < Nx; ++i) s += dose[(size_t)j * Nx + i];
    return s;
}
// the same in float, as the Bragg-peak metrics sum (bragg_peak.cpp)
float row_sum_f(const double* dose, int Nx, int j) {
    float s = 0.0f;
    for (int i = 0; i < Nx; ++i) s += static_cast<float>(dose[(size_t)j * Nx + i]);
    return s;
}
// find_bragg_peak_z (deterministic_beam.cpp:207-222): first row of the
// largest positive double row sum, 0 if none
int peak_row(const double* dose, int Nx, int Nz) {
    int best = 0;
    double mx = 0.0;
    for (int j = 0; j < Nz; ++j) {
        const double s = row_sum(dose, Nx, j);
        if (s > mx) {
            mx = s;
            best = j;
        }
    }
    return best;
}
// find_bragg_peak_position_mm (bragg_peak.cpp:6-22): depth of the first row
// of the largest positive float row sum
float peak_position(const double* dose, int Nx, int Nz, float dz) {
    float mx = 0.0f, zp = 0.0f;
    for (int j = 0; j < Nz; ++j) {
        const float s = row_sum_f(dose, Nx, j);
        if (s > mx) {
            mx = s;
            zp = j * dz;
        }
    }
    return zp;
}
// first depth beyond the peak (rows peak, peak+1, ...) whose float row sum
// falls below frac of the peak row's; the last row's depth if none
// (find_R80 / find_R20, bragg_peak.cpp:67-117)
float distal_depth(const double* dose, int Nx, int Nz, float dz, float frac) {
    const float zp = peak_position(dose, Nx, Nz, dz);
    const int pk = static_cast<int>(zp / dz);
    const float thr = row_sum_f(dose, Nx, pk) * frac;
    for (int j = pk; j < Nz; ++j)
        if (row_sum_f(dose, Nx, j) < thr) return j * dz;
    return (Nz - 1) * dz;
}
bool grid_ok(const double* dose, int Nx, int Nz) { return dose && Nx > 0 && Nz > 0; }

}  // namespace

extern "C" {

int sm2d_depth_dose(const double* dose, int Nx, int Nz, double* pdd) {
    if (!grid_ok(dose, Nx, Nz) || !pdd) return sm2d::fail(SM2D_ERR_ARG, "invalid dose grid");
    for (int j = 0; j < Nz; ++j) pdd[j] = row_sum(dose, Nx, j);
    return 0;
}

int sm2d_bragg_peak_row(const double* dose, int Nx, int Nz) {
    if (!grid_ok(dose, Nx, Nz)) return sm2d::fail(SM2D_ERR_ARG, "invalid dose grid");
    return peak_row(dose, Nx, Nz);
}

int sm2d_bragg_metrics(const double* dose, int Nx, int Nz, float dz, float* out) {
    if (!grid_ok(dose, Nx, Nz) || !out || !(dz > 0.0f)) return sm2d::fail(SM2D_ERR_ARG, "invalid dose grid");
    const float zp = peak_position(dose, Nx, Nz, dz);
    // FWHM (compute_bragg_peak_fwhm, bragg_peak.cpp:24-65): the first rows
    // below half the peak row's sum, scanning down and up from the peak
    const int pk = static_cast<int>(zp / dz);
    const float half = row_sum_f(dose, Nx, pk) * 0.5f;
    float zl = zp, zr = zp;
    for (int j = pk; j >= 0; --j)
        if (row_sum_f(dose, Nx, j) < half) {
            zl = j * dz;
            break;
        }
    for (int j = pk; j < Nz; ++j)
        if (row_sum_f(dose, Nx, j) < half) {
            zr = j * dz;
            break;
        }
    const float r80 = distal_depth(dose, Nx, Nz, dz, 0.8f), r20 = distal_depth(dose, Nx, Nz, dz, 0.2f);
    out[0] = zp;
    out[1] = zr - zl;
    out[2] = r80;
    out[3] = r20;
    out[4] = r20 - r80;   // distal falloff (compute_distal_falloff, bragg_peak.cpp:119-125)
    return 0;
}

int sm2d_write_dose_2d(const char* path, const double* dose, int Nx, int Nz, float dx, float dz, int normalize) {
    if (!path || !grid_ok(dose, Nx, Nz)) return sm2d::fail(SM2D_ERR_ARG, "invalid argument");
    std::ofstream out(path);
    if (!out.is_open()) return sm2d::fail(SM2D_ERR_ARG, "cannot open %s", path);
    double mx = 0.0;
    if (normalize)
        for (size_t k = 0; k < (size_t)Nx * Nz; ++k) mx = std::max(mx, dose[k]);
    out << "# 2D Dose Distribution\n";
    out << "# x(mm) z(mm) dose(Gy)";
    if (normalize) out << " dose_norm";
    out << "\n";
    for (int iz = 0; iz < Nz; ++iz) {
        const float z = iz * dz;
        for (int ix = 0; ix < Nx; ++ix) {
            const float x = (ix + 0.5f) * dx - (Nx * dx) / 2.0f;
            double v = dose[(size_t)iz * Nx + ix];
            if (std::isnan(v) || std::isinf(v)) v = 0.0;
            out << std::fixed << std::setprecision(4) << x << "\t" << z << "\t" << v;
            if (normalize && mx > 0) out << "\t" << (v / mx);
            out << "\n";
        }
        out << "\n";
    }
    out.close();
    return out.fail() ? sm2d::fail(SM2D_ERR_ARG, "write failed: %s", path) : 0;
}

int sm2d_write_pdd(const char* path, const double* dose, int Nx, int Nz, float dz, int normalize) {
    if (!path || !grid_ok(dose, Nx, Nz)) return sm2d::fail(SM2D_ERR_ARG, "invalid argument");
    std::ofstream out(path);
    if (!out.is_open()) return sm2d::fail(SM2D_ERR_ARG, "cannot open %s", path);
    std::vector<double> pdd(Nz);
    for (int j = 0; j < Nz; ++j) pdd[j] = row_sum(dose, Nx, j);
    const int pk = peak_row(dose, Nx, Nz);
    const double peak = pdd[pk];
    out << "# Depth-Dose Distribution (PDD)\n";
    out << "# Depth(mm) Dose(Gy)";
    if (normalize) out << " Dose_norm";
    out << "\n";
    out << "# Bragg Peak at: " << (pk * dz) << " mm, " << peak << " Gy\n";
    for (size_t i = 0; i < pdd.size(); ++i) {
        const double depth = i * dz;
        double v = pdd[i];
        if (std::isnan(v) || std::isinf(v)) v = 0.0;
        out << std::fixed << std::setprecision(4) << depth << "\t" << v;
        if (normalize && peak > 0) out << "\t" << (v / peak);
        out << "\n";
    }
    out.close();
    return out.fail() ? sm2d::fail(SM2D_ERR_ARG, "write failed: %s", path) : 0;
}

// ---------------------------------------------------------------- debug dumps
// The reference's debug CSV files (built with SM2D_ENABLE_DEBUG_DUMPS), from
// a host copy of psi (sm2d_get_psi_in: ids [cell][32], values
// [cell][32][L]) and the problem's grids.  Rows are the bins with weight
// above 1e-12, in cell, slot, local-bin order.
//   debug_ps_raw_iter_NN_<stage>.csv  dump_phase_space_raw_to_csv
//       (k1k6_pipeline.cu:195-291; 8 decimals) and dump_initial_cells_to_csv
//       (gpu_transport_wrapper.cu:22-120; 6 decimals, iteration 0)
//   debug_cells_iter_NN_<stage>.csv   dump_nonzero_cells_to_csv
//       (k1k6_pipeline.cu:29-193): per cell with weight, float sums
//   debug_channels_totals_iter01.csv  k1k6_pipeline.cu:2125-2155
int sm2d_write_ps_raw_csv(const char* path, const sm2d_problem* p, const uint32_t* bid, const float* val,
                          int iteration, int precision) {
    if (!path || !p || !bid || !val || !p->theta_edges || !p->E_edges) return sm2d::fail(SM2D_ERR_ARG, "invalid argument");
    const int NT = p->nt_local, NE = p->ne_local, NX = p->nx_sub, NZ = p->nz_sub, L = NT * NE * NX * NZ;
    if (L <= 0) return sm2d::fail(SM2D_ERR_LAYOUT, "invalid local layout");
    std::ofstream ofs(path);
    if (!ofs.is_open()) return sm2d::fail(SM2D_ERR_ARG, "cannot open %s", path);
    // sub-bin centre offsets from the cell centre (local_bins.hpp:80-107):
    // d (-1/2 + 1/(2n) + s/n), exact constants for power-of-two n
    const float cx0 = -0.5f + 0.5f / NX, cx1 = 1.0f / NX, cz0 = -0.5f + 0.5f / NZ, cz1 = 1.0f / NZ;
    ofs << "iter,cell,ix,iz,slot,bid,lidx,weight,"
        << "b_theta,b_E,theta_local,E_local,x_sub,z_sub,"
        << "theta_bin,E_bin,theta_rep,E_rep,x_offset_mm,z_offset_mm\n";
    ofs << std::fixed << std::setprecision(precision);
    const int Nc = p->Nx * p->Nz;
    for (int cell = 0; cell < Nc; ++cell) {
        const int ix = cell % p->Nx, iz = cell / p->Nx;
        for (int slot = 0; slot < 32; ++slot) {
            const uint32_t b = bid[(size_t)cell * 32 + slot];
            if (b == 0xFFFFFFFFu) continue;
            const int bt = (int)(b & 0xFFFu), be = (int)((b >> 12) & 0xFFFu);
            for (int l = 0; l < L; ++l) {
                const float w = val[((size_t)cell * 32 + slot) * L + l];
                if (w <= 1e-12f) continue;
                const int tl = l % NT, el = (l / NT) % NE, xs = (l / (NT * NE)) % NX, zs = l / (NT * NE * NX);
                const int tb = std::max(0, std::min(bt * NT + tl, p->N_theta - 1));
                const int eb = std::max(0, std::min(be * NE + el, p->N_E - 1));
                const float th = p->theta_edges[tb] + 0.5f * (p->theta_edges[tb + 1] - p->theta_edges[tb]);
                const float er = p->E_edges[eb] + 0.5f * (p->E_edges[eb + 1] - p->E_edges[eb]);
                const float xo = p->dx * (cx0 + cx1 * xs), zo = p->dz * (cz0 + cz1 * zs);
                ofs << iteration << "," << cell << "," << ix << "," << iz << "," << slot << "," << b << "," << l << ","
                    << w << "," << bt << "," << be << "," << tl << "," << el << "," << xs << "," << zs << "," << tb
                    << "," << eb << "," << th << "," << er << "," << xo << "," << zo << "\n";
            }
        }
    }
    ofs.close();
    return ofs.fail() ? sm2d::fail(SM2D_ERR_ARG, "write failed: %s", path) : 0;
}

int sm2d_write_cells_csv(const char* path, const sm2d_problem* p, const uint32_t* bid, const float* val) {
    if (!path || !p || !bid || !val || !p->theta_edges || !p->E_edges) return sm2d::fail(SM2D_ERR_ARG, "invalid argument");
    const int NT = p->nt_local, NE = p->ne_local, NX = p->nx_sub, NZ = p->nz_sub, L = NT * NE * NX * NZ;
    if (L <= 0) return sm2d::fail(SM2D_ERR_LAYOUT, "invalid local layout");
    std::ofstream ofs(path);
    if (!ofs.is_open()) return sm2d::fail(SM2D_ERR_ARG, "cannot open %s", path);
    // bin centres: uniform theta, energy at lower edge + half width
    const float t0 = p->theta_edges[0], t1 = p->theta_edges[p->N_theta];
    const float dth = (t1 - t0) / p->N_theta;
    std::vector<float> tc(p->N_theta), ec(p->N_E);
    for (int i = 0; i < p->N_theta; ++i) tc[i] = t0 + (i + 0.5f) * dth;
    for (int i = 0; i < p->N_E; ++i) ec[i] = p->E_edges[i] + 1.00f * ((p->E_edges[i + 1] - p->E_edges[i]) * 0.5f);
    ofs << "cell,ix,iz,x_mm,z_mm,total_weight,num_slots,mean_E_MeV,mean_theta_rad,min_E_MeV,max_E_MeV,min_theta_rad,"
           "max_theta_rad\n";
    ofs << std::fixed << std::setprecision(6);
    const int Nc = p->Nx * p->Nz;
    for (int cell = 0; cell < Nc; ++cell) {
        float W = 0.0f, sE = 0.0f, sT = 0.0f, Emin = 1e30f, Emax = -1e30f, Tmin = 1e30f, Tmax = -1e30f;
        int n = 0;
        for (int slot = 0; slot < 32; ++slot) {
            const uint32_t b = bid[(size_t)cell * 32 + slot];
            if (b == 0xFFFFFFFFu) continue;
            const int bt = (int)(b & 0xFFFu), be = (int)((b >> 12) & 0xFFFu);
            for (int l = 0; l < L; ++l) {
                const float w = val[((size_t)cell * 32 + slot) * L + l];
                if (!(w > 1e-12f)) continue;
                W += w;
                ++n;
                const int tl = l % NT, el = (l / NT) % NE;
                const float th = tc[std::max(0, std::min(bt * NT + tl, p->N_theta - 1))];
                const float E = ec[std::max(0, std::min(be * NE + el, p->N_E - 1))];
                sE += E * w;
                sT += th * w;
                Emin = std::min(Emin, E);
                Emax = std::max(Emax, E);
                Tmin = std::min(Tmin, th);
                Tmax = std::max(Tmax, th);
            }
        }
        if (!(W > 1e-12f)) continue;
        const int ix = cell % p->Nx, iz = cell / p->Nx;
        ofs << cell << "," << ix << "," << iz << "," << (ix + 0.5f) * p->dx << "," << (iz + 0.5f) * p->dz << "," << W
            << "," << n << "," << sE / W << "," << sT / W << "," << Emin << "," << Emax << "," << Tmin << "," << Tmax
            << "\n";
    }
    ofs.close();
    return ofs.fail() ? sm2d::fail(SM2D_ERR_ARG, "write failed: %s", path) : 0;
}

int sm2d_write_channel_totals_csv(const char* path, const double* t) {
    if (!path || !t) return sm2d::fail(SM2D_ERR_ARG, "invalid argument");
    static const char* names[17] = {"EdepC", "AbsorbedWeight_cutoff", "AbsorbedEnergy_cutoff", "AbsorbedWeight_nuclear",
                                    "AbsorbedEnergy_nuclear", "BoundaryLoss_weight", "BoundaryLoss_energy",
                                    "transport_dropped_weight", "transport_dropped_energy",
                                    "transport_audit_residual_energy", "source_injected_weight",
                                    "source_out_of_grid_weight", "source_slot_dropped_weight", "source_injected_energy",
                                    "source_out_of_grid_energy", "source_slot_dropped_energy",
                                    "source_representation_loss_energy"};
    std::ofstream ofs(path);
    if (!ofs.is_open()) return sm2d::fail(SM2D_ERR_ARG, "cannot open %s", path);
    ofs << "iter,channel,value\n";
    for (int k = 0; k < 10; ++k) ofs << "0," << names[k] << ",0\n";
    for (int k = 0; k < 17; ++k) ofs << "1," << names[k] << "," << t[k] << "\n";
    ofs.close();
    return ofs.fail() ? sm2d::fail(SM2D_ERR_ARG, "write failed: %s", path) : 0;
}

// The channel totals of a single-spot engine in the file's order: cell sums
// in cell order (k1k6_pipeline.cu:2030-2099), then the run's scalars.
int sm2d_channel_totals(sm2d_handle h, int Nx, int Nz, double* out) {
    if (!h || !out || Nx <= 0 || Nz <= 0) return sm2d::fail(SM2D_ERR_ARG, "invalid argument");
    const size_t n = (size_t)Nx * Nz;
    std::vector<double> edep(n), ecut(n), enuc(n), ebnd(n), sc(17);
    std::vector<float> wcut(n), wnuc(n), wbnd(n);
    int rc = sm2d_get_tallies(h, edep.data(), wcut.data(), ecut.data(), wnuc.data(), enuc.data(), wbnd.data(),
                              ebnd.data());
    if (!rc) rc = sm2d_get_scalars(h, sc.data());
    if (rc) return rc;
    double s[7] = {};
    for (size_t i = 0; i < n; ++i) {
        s[0] += edep[i];
        s[1] += wcut[i];
        s[2] += ecut[i];
        s[3] += wnuc[i];
        s[4] += enuc[i];
        s[5] += wbnd[i];
        s[6] += ebnd[i];
    }
    for (int k = 0; k < 7; ++k) out[k] = s[k];
    // transport drops and residual; source weights; source energies
    out[7] = sc[0]; out[8] = sc[1]; out[9] = sc[2];
    out[10] = sc[3]; out[11] = sc[5]; out[12] = sc[7];
    out[13] = sc[4]; out[14] = sc[6]; out[15] = sc[8]; out[16] = sc[9];
    return 0;
}

}  // extern "C"
