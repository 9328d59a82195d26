// sm2d_config.cpp -- the reference's INI front end over the C ABI: the
// configuration file run_simulation reads (sections [particle] [beam]
// [energy] [spatial] [angular] [sampling] [grid] [transport] [output]), its
// mapping onto one transport problem and beam as the reference's runner
// makes it, and run_simulation's single-spot run with its output files.
//
// Parsing (ConfigLoader::load, config_loader.hpp:98-152): lines are trimmed;
// empty lines and lines starting with '#' or ';' are skipped; "[name]" opens
// a section (keys before any section go to "default"); "key = value" splits
// at the first '='; a value in matching single or double quotes loses them;
// a later key overrides an earlier one.  Numbers parse as std::stof /
// std::stoi do (a leading number, else the default); booleans are true for
// "true", "1", "yes", "on" in any case.
//
// Mapping (load_incident_particle_config, config_loader.hpp:324-411, and
// GPUTransportRunner::run, gpu_transport_runner.cpp:28-105): the angular
// grid is N_theta bins on +-0.35 rad, the energy grid the piecewise groups
// of [transport] energy_groups ("Emin:Emax:dE,..."), x_min = -Nx dx / 2,
// z_min = 0, max_iterations = 0 means grid.max_steps, the legacy E_trigger
// lifts into E_fine_on/off, and the beam passes the energy, position, angle,
// spreads, samples and seed of the file.
#include <sys/stat.h>

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "sm2d.h"
#include "sm2d_tables.h"

namespace {

using Section = std::map<std::string, std::string>;
using Ini = std::map<std::string, Section>;

std::string trim(const std::string& s) {
    size_t a = 0, b = s.size();
    while (a < b && std::isspace(static_cast<unsigned char>(s[a]))) ++a;
    while (b > a && std::isspace(static_cast<unsigned char>(s[b - 1]))) --b;
    return s.substr(a, b - a);
}

bool parse_ini(const char* path, Ini& ini) {
    std::ifstream f(path);
    if (!f.is_open()) return false;
    std::string line, sec = "default";
    while (std::getline(f, line)) {
        line = trim(line);
        if (line.empty() || line[0] == '#' || line[0] == ';') continue;
        if (line[0] == '[' && line.back() == ']') {
            sec = trim(line.substr(1, line.size() - 2));
            continue;
        }
        const size_t eq = line.find('=');
        if (eq == std::string::npos) continue;
        const std::string key = trim(line.substr(0, eq));
        std::string val = trim(line.substr(eq + 1));
        if (val.size() >= 2 && ((val.front() == '"' && val.back() == '"') || (val.front() == '\'' && val.back() == '\'')))
            val = val.substr(1, val.size() - 2);
        ini[sec][key] = val;
    }
    return true;
}

struct View {
    const Section* s;
    bool has(const char* k) const { return s && s->count(k); }
    std::string str(const char* k, const std::string& def) const { return has(k) ? s->at(k) : def; }
    float f(const char* k, float def) const {
        if (!has(k)) return def;
        try {
            return std::stof(s->at(k));
        } catch (...) {
            return def;
        }
    }
    int i(const char* k, int def) const {
        if (!has(k)) return def;
        try {
            return std::stoi(s->at(k));
        } catch (...) {
            return def;
        }
    }
    bool b(const char* k, bool def) const {
        if (!has(k)) return def;
        std::string v = s->at(k);
        std::transform(v.begin(), v.end(), v.begin(), [](unsigned char c) { return (char)std::tolower(c); });
        return v == "true" || v == "1" || v == "yes" || v == "on";
    }
};
View section(const Ini& ini, const char* name) {
    auto it = ini.find(name);
    return View{it == ini.end() ? nullptr : &it->second};
}

// "Emin:Emax:dE,..." (parse_transport_energy_groups, config_loader.hpp:235-272);
// any malformed group keeps the default groups
std::vector<float> energy_groups(const std::string& raw) {
    const std::vector<float> def = {0.1f, 2.0f, 0.1f, 2.0f, 20.0f, 0.2f, 20.0f, 100.0f, 0.25f, 100.0f, 250.0f, 0.25f};
    if (raw.empty()) return def;
    std::vector<float> g;
    std::stringstream ss(raw);
    std::string tok;
    while (std::getline(ss, tok, ',')) {
        tok = trim(tok);
        if (tok.empty()) continue;
        std::stringstream ts(tok);
        std::string p[3];
        if (!std::getline(ts, p[0], ':') || !std::getline(ts, p[1], ':') || !std::getline(ts, p[2], ':')) return def;
        try {
            for (auto& x : p) g.push_back(std::stof(trim(x)));
        } catch (...) {
            return def;
        }
    }
    return g.empty() ? def : g;
}

void copy_str(char* dst, size_t n, const std::string& s) {
    std::snprintf(dst, n, "%s", s.c_str());
}

}  // namespace

extern "C" {

void sm2d_run_config_free(sm2d_run_config* c) {
    if (!c) return;
    std::free(c->theta_edges_buf);
    std::free(c->E_edges_buf);
    c->theta_edges_buf = c->E_edges_buf = nullptr;
    c->problem.theta_edges = c->problem.E_edges = nullptr;
}

int sm2d_load_ini(const char* path, sm2d_run_config* out) {
    if (!path || !out) return sm2d::fail(SM2D_ERR_ARG, "null argument");
    std::memset(out, 0, sizeof *out);
    Ini ini;
    if (!parse_ini(path, ini)) return sm2d::fail(SM2D_ERR_ARG, "Failed to load configuration file: %s", path);
    const View beam = section(ini, "beam"), energy = section(ini, "energy"), spatial = section(ini, "spatial"),
               angular = section(ini, "angular"), sampling = section(ini, "sampling"), grid = section(ini, "grid"),
               tr = section(ini, "transport"), output = section(ini, "output");
    // values and their defaults (incident_particle_config.hpp:88-257)
    const float W = beam.f("weight", 1.0f);
    const float E0 = energy.f("mean_MeV", 150.0f), sE = energy.f("sigma_MeV", 0.0f);
    const float Emin_cut = energy.f("min_MeV", 0.0f), Emax_cut = energy.f("max_MeV", 500.0f);
    const float x0 = spatial.f("x0_mm", 0.0f), z0 = spatial.f("z0_mm", 0.0f), sx = spatial.f("sigma_x_mm", 0.0f);
    const float sz = spatial.f("sigma_z_mm", 0.0f);
    const float th0 = angular.f("theta0_rad", 0.0f), sth = angular.f("sigma_theta_rad", 0.0f);
    const int n_samples = sampling.i("n_samples", 1000);
    const unsigned seed = static_cast<unsigned>(sampling.i("random_seed", 42));
    const int Nx = grid.i("Nx", 100), Nz = grid.i("Nz", 200), max_steps = grid.i("max_steps", 100);
    const float dx = grid.f("dx_mm", 1.0f), dz = grid.f("dz_mm", 1.0f);
    const int N_theta = tr.i("N_theta", 36), ntl = tr.i("N_theta_local", 4), nel = tr.i("N_E_local", 2);
    // fine-transport thresholds with the legacy E_trigger alias
    const bool has_on = tr.has("E_fine_on_MeV") || tr.has("E_fine_on");
    const bool has_off = tr.has("E_fine_off_MeV") || tr.has("E_fine_off");
    const bool has_trig = tr.has("E_trigger_MeV") || tr.has("E_trigger");
    float on = 10.0f, off = 11.0f, trig = 10.0f;
    if (has_on) on = tr.f("E_fine_on", tr.f("E_fine_on_MeV", on));
    if (has_off) off = tr.f("E_fine_off", tr.f("E_fine_off_MeV", off));
    if (has_trig) {
        trig = tr.f("E_trigger", tr.f("E_trigger_MeV", trig));
        if (!has_on) on = trig;
    } else {
        trig = on;
    }
    if (!has_off) off = std::max(off, on);
    // the runner's lift of a customised trigger (gpu_transport_runner.cpp:71-76)
    if (std::fabs(trig - on) > 1e-6f && std::fabs(on - 10.0f) < 1e-6f && std::fabs(off - 11.0f) < 1e-6f) {
        on = trig;
        off = std::max(off, on);
    }
    const float wmin = tr.f("weight_active_min", 1e-12f);
    const float step = tr.f("step_coarse", tr.f("step_coarse_mm", 5.0f));
    const int max_it = tr.i("max_iterations", 0), log_level = tr.i("log_level", 1);
    const bool validation = tr.b("validation_mode", false);
    const bool fail_fast = tr.b("fail_fast_on_audit", false) || validation;
    const std::vector<float> groups = energy_groups(tr.str("energy_groups", ""));

    // validate() (incident_particle_config.hpp:274-399), the checks that
    // concern this path
    const char* bad = nullptr;
    if (!(E0 > 0.0f)) bad = "mean_E0 must be positive";
    else if (sE < 0.0f) bad = "sigma_E must be non-negative";
    else if (Emin_cut < 0.0f) bad = "min_E must be non-negative";
    else if (!(Emax_cut > Emin_cut)) bad = "max_E must be > min_E";
    else if (sx < 0.0f || sz < 0.0f) bad = "sigma must be non-negative";
    else if (sth < 0.0f) bad = "sigma_theta must be non-negative";
    else if (n_samples <= 0) bad = "n_samples must be positive";
    else if (!(W > 0.0f)) bad = "W_total must be positive";
    else if (Nx <= 0 || Nz <= 0) bad = "grid dimensions must be positive";
    else if (!(dx > 0.0f) || !(dz > 0.0f)) bad = "grid spacing must be positive";
    else if (max_steps <= 0) bad = "max_steps must be positive";
    else if (N_theta <= 0) bad = "transport.N_theta must be positive";
    else if (!(on > 0.0f)) bad = "transport.E_fine_on must be positive";
    else if (off < on) bad = "transport.E_fine_off must be >= transport.E_fine_on";
    else if (!(wmin > 0.0f)) bad = "transport.weight_active_min must be positive";
    else if (!(step > 0.0f)) bad = "transport.step_coarse must be positive";
    else if (max_it < 0) bad = "transport.max_iterations cannot be negative";
    else if (log_level < 0) bad = "transport.log_level cannot be negative";
    for (size_t k = 0; !bad && k < groups.size(); k += 3) {
        if (!(groups[k] > 0.0f)) bad = "transport.energy_groups E_min must be positive";
        else if (!(groups[k + 1] > groups[k])) bad = "transport.energy_groups E_max must be > E_min";
        else if (!(groups[k + 2] > 0.0f)) bad = "transport.energy_groups dE must be positive";
        else if (k > 0 && groups[k] < groups[k - 2]) bad = "transport.energy_groups must be non-overlapping and ordered";
    }
    if (bad) return sm2d::fail(SM2D_ERR_ARG, "IncidentParticleConfig: %s", bad);
    int nx_sub, nz_sub;
    if (ntl == 4 && nel == 2) { nx_sub = 8; nz_sub = 4; }
    else if (ntl == 8 && nel == 4) { nx_sub = 4; nz_sub = 1; }
    else
        return sm2d::fail(SM2D_ERR_LAYOUT, "local bins N_theta_local=%d, N_E_local=%d not compiled; use (4,2) or (8,4)",
                          ntl, nel);

    // grids
    const int n_groups = (int)groups.size() / 3;
    const int N_E = sm2d::energy_grid_piecewise(n_groups, groups.data(), nullptr, nullptr);
    if (N_E <= 1) return sm2d::fail(SM2D_ERR_ARG, "empty energy grid");
    out->theta_edges_buf = static_cast<float*>(std::malloc(sizeof(float) * (N_theta + 1)));
    out->E_edges_buf = static_cast<float*>(std::malloc(sizeof(float) * (N_E + 1)));
    std::vector<float> rep(std::max(N_theta, N_E));
    if (!out->theta_edges_buf || !out->E_edges_buf) {
        sm2d_run_config_free(out);
        return sm2d::fail(SM2D_ERR_ALLOC, "grid buffers");
    }
    sm2d::angular_grid(-0.35f, 0.35f, N_theta, out->theta_edges_buf, rep.data());
    sm2d::energy_grid_piecewise(n_groups, groups.data(), out->E_edges_buf, rep.data());

    sm2d_problem& p = out->problem;
    p.Nx = Nx; p.Nz = Nz; p.dx = dx; p.dz = dz;
    p.x_min = -(Nx * dx) / 2.0f;
    p.z_min = 0.0f;
    p.N_theta = N_theta; p.theta_edges = out->theta_edges_buf;
    p.N_E = N_E; p.E_edges = out->E_edges_buf;
    p.E_min = out->E_edges_buf[0];
    p.E_max = out->E_edges_buf[N_E];
    p.nt_local = ntl; p.ne_local = nel; p.nx_sub = nx_sub; p.nz_sub = nz_sub;
    p.E_fine_on = on; p.E_fine_off = off;
    p.weight_active_min = wmin;
    p.step_coarse = step;
    p.sigma_x_initial = sx;
    p.E0 = E0;
    p.enable_straggling = 1;
    p.enable_nuclear = 1;
    out->max_iterations = max_it > 0 ? max_it : max_steps;
    p.max_iterations = out->max_iterations;
    p.lanes = 1;
    out->beam = sm2d_beam{x0, z0, th0, E0, W, sx, sth, sE, n_samples, seed};
    out->log_level = log_level;
    out->fail_fast_on_audit = fail_fast ? 1 : 0;
    out->normalize_dose = output.b("normalize_dose", true) ? 1 : 0;
    out->save_2d = output.b("save_2d", true) ? 1 : 0;
    out->save_pdd = output.b("save_pdd", true) ? 1 : 0;
    copy_str(out->output_dir, sizeof out->output_dir, output.str("output_dir", "results"));
    copy_str(out->dose_2d_file, sizeof out->dose_2d_file, output.str("dose_2d_file", "dose_2d.txt"));
    copy_str(out->pdd_file, sizeof out->pdd_file, output.str("pdd_file", "pdd.txt"));
    return 0;
}

// run_simulation's main (run_simulation.cpp:116-188): one spot from the INI,
// its dose and the Bragg peak, the output files under output_dir (relative
// to the INI's directory).
int sm2d_run_simulation(const char* ini_path) {
    sm2d_run_config c;
    int rc = sm2d_load_ini(ini_path, &c);
    if (rc) return rc;
    std::string dir = c.output_dir;
    if (!dir.empty() && dir[0] != '/') {
        const std::string ip = ini_path;
        const size_t slash = ip.find_last_of("/\\");
        if (slash != std::string::npos) dir = ip.substr(0, slash) + "/" + dir;
    }
    struct stat st;
    if (stat(dir.c_str(), &st) != 0 && mkdir(dir.c_str(), 0755) != 0)
        std::fprintf(stderr, "Warning: Could not create output directory: %s\n", dir.c_str());
    sm2d_handle h = nullptr;
    std::vector<double> dose((size_t)c.problem.Nx * c.problem.Nz);
    int done = 0;
    rc = sm2d_create(&c.problem, &h);
    if (!rc) rc = sm2d_inject(h, &c.beam);
    if (!rc) rc = sm2d_run(h, c.max_iterations, &done);
    if (!rc) rc = sm2d_get_dose(h, dose.data());
    sm2d_destroy(h);
    if (!rc) {
        const int pk = sm2d_bragg_peak_row(dose.data(), c.problem.Nx, c.problem.Nz);
        double peak = 0.0;
        for (int i = 0; i < c.problem.Nx; ++i) peak += dose[(size_t)pk * c.problem.Nx + i];
        if (c.log_level >= 1)
            std::printf("Simulation complete: %d iterations.\n  Bragg Peak: %g mm depth, %g Gy\n", done,
                        (double)(pk * c.problem.dz), peak);
        const std::string d2 = dir + "/" + c.dose_2d_file, pd = dir + "/" + c.pdd_file;
        if (c.save_2d)
            rc = sm2d_write_dose_2d(d2.c_str(), dose.data(), c.problem.Nx, c.problem.Nz, c.problem.dx, c.problem.dz,
                                    c.normalize_dose);
        if (!rc && c.save_pdd)
            rc = sm2d_write_pdd(pd.c_str(), dose.data(), c.problem.Nx, c.problem.Nz, c.problem.dz, c.normalize_dose);
    }
    sm2d_run_config_free(&c);
    return rc;
}

}  // extern "C"
