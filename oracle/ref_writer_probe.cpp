// Probe of the reference's output writers and depth-dose metrics (test
// infrastructure): links the reference's own save_dose_2d / save_pdd
// (run_simulation.cpp:31-114, its main renamed), get_depth_dose /
// find_bragg_peak_z (deterministic_beam.cpp:207-236) and the Bragg-peak
// metrics (bragg_peak.cpp), reads a dose grid, writes the reference's files
// and prints the metrics.  The transport runner is not linked: a stub stands
// in for it, since only the writers are probed.
//
// usage: ref_writer_probe <dose.bin> <out_dir>
//   dose.bin: int32 Nx, int32 Nz, float32 dx, float32 dz, float64 dose[Nz][Nx]
#include "gpu/gpu_transport_runner.hpp"
#include "validation/bragg_peak.hpp"
#include "validation/deterministic_beam.hpp"

#include <cstdio>
#include <stdexcept>
#include <string>

bool save_dose_2d(const std::string& filepath, const SimulationResult& result, bool normalize);
bool save_pdd(const std::string& filepath, const SimulationResult& result, bool normalize);

namespace sm_2d {
SimulationResult GPUTransportRunner::run(const IncidentParticleConfig&) { throw std::runtime_error("not linked"); }
}  // namespace sm_2d

int main(int argc, char** argv) {
    if (argc != 3) return 2;
    FILE* f = std::fopen(argv[1], "rb");
    if (!f) return 3;
    int hdr[2];
    float dd[2];
    if (std::fread(hdr, 4, 2, f) != 2 || std::fread(dd, 4, 2, f) != 2) return 4;
    SimulationResult r;
    r.Nx = hdr[0];
    r.Nz = hdr[1];
    r.dx = dd[0];
    r.dz = dd[1];
    r.edep.assign(r.Nz, std::vector<double>(r.Nx, 0.0));
    for (int j = 0; j < r.Nz; ++j)
        if (std::fread(r.edep[j].data(), 8, r.Nx, f) != (size_t)r.Nx) return 5;
    std::fclose(f);
    // coordinates as the GPU runner builds them (gpu_transport_runner.cpp:52-62)
    r.x_centers.resize(r.Nx);
    r.z_centers.resize(r.Nz);
    for (int i = 0; i < r.Nx; ++i) r.x_centers[i] = (i + 0.5f) * r.dx - (r.Nx * r.dx) / 2.0f;
    for (int j = 0; j < r.Nz; ++j) r.z_centers[j] = j * r.dz;
    const std::string out = argv[2];
    if (!save_dose_2d(out + "/dose_2d_norm.txt", r, true) || !save_dose_2d(out + "/dose_2d.txt", r, false) ||
        !save_pdd(out + "/pdd_norm.txt", r, true) || !save_pdd(out + "/pdd.txt", r, false))
        return 6;
    std::printf("{\"bragg_peak_row\": %d, \"peak_mm\": %.9g, \"fwhm_mm\": %.9g, \"r80_mm\": %.9g, \"r20_mm\": %.9g, "
                "\"distal_falloff_mm\": %.9g}\n",
                find_bragg_peak_z(r), (double)find_bragg_peak_position_mm(r), (double)compute_bragg_peak_fwhm(r),
                (double)find_R80(r), (double)find_R20(r), (double)compute_distal_falloff(r));
    return 0;
}
