// ref_probe.cpp -- fixture generator linked against the reference's own host
// sources (grids.cpp, r_lut.cpp, nist_loader.cpp and the header-only host
// physics).  Built by ref_build.sh into oracle/_ref/; it only prints JSON
// that tests/golden/make_golden.py stores as fixtures.  Test infrastructure.
#include "core/grids.hpp"
#include "lut/r_lut.hpp"
#include "physics/step_control.hpp"
#include "physics/highland.hpp"
#include <cmath>
#include <cstdio>
#include <tuple>
#include <vector>

static void arr(const char* name, const std::vector<float>& v, bool last = false) {
    std::printf("\"%s\": [", name);
    for (size_t i = 0; i < v.size(); ++i) std::printf("%s%.9g", i ? ", " : "", v[i]);
    std::printf("]%s\n", last ? "" : ",");
}

static void grid_block(const char* key, const EnergyGrid& g, bool with_lut) {
    std::printf("\"%s\": {\n", key);
    std::printf("\"N_E\": %d, \"E_min\": %.9g, \"E_max\": %.9g,\n", g.N_E, g.E_min, g.E_max);
    arr("edges", g.edges);
    if (with_lut) {
        RLUT lut = GenerateRLUT(g);
        arr("rep", g.rep);
        arr("R", lut.R);
        arr("S", lut.S);
        arr("logE", lut.log_E);
        arr("logR", lut.log_R);
        arr("logS", lut.log_S, true);
    } else {
        arr("rep", g.rep, true);
    }
    std::printf("},\n");
}

int main() {
    std::printf("{\n");
    EnergyGrid log250(0.1f, 250.0f, 256);
    grid_block("log_0.1_250_256", log250, true);
    EnergyGrid log300(0.1f, 300.0f, 256);
    grid_block("log_0.1_300_256", log300, true);
    std::vector<std::tuple<float, float, float>> groups = {
        {0.1f, 2.0f, 0.1f}, {2.0f, 20.0f, 0.2f}, {20.0f, 100.0f, 0.25f}, {100.0f, 250.0f, 0.25f}};
    EnergyGrid pw = EnergyGrid::CreatePiecewise(groups);
    grid_block("piecewise_default", pw, true);
    AngularGrid a36(-0.35f, 0.35f, 36), a360(-0.35f, 0.35f, 360), a512(-M_PI / 2, M_PI / 2, 512);
    std::printf("\"theta_0.35_36\": {"); arr("edges", a36.edges); arr("rep", a36.rep, true); std::printf("},\n");
    std::printf("\"theta_0.35_360\": {"); arr("edges", a360.edges); arr("rep", a360.rep, true); std::printf("},\n");
    std::printf("\"theta_pi2_512\": {"); arr("edges", a512.edges); arr("rep", a512.rep, true); std::printf("},\n");
    // host lookups used by the Fermi-Eyges precompute (LUT on the 0.1-300 log grid)
    RLUT lut = GenerateRLUT(0.1f, 300.0f, 256);
    std::vector<float> Es = {0.15f, 0.5f, 1.0f, 3.0f, 9.9f, 10.0f, 25.0f, 70.0f, 99.5f, 150.0f, 151.3f, 229.0f, 249.9f};
    std::vector<float> R, Einv, dE, hs;
    for (float E : Es) {
        float r = lut.lookup_R(E);
        R.push_back(r);
        Einv.push_back(lut.lookup_E_inverse(r));
        dE.push_back(compute_energy_deposition(lut, E, 0.5f));
        hs.push_back(highland_sigma(E, 0.5f));
    }
    std::printf("\"host_lookups\": {"); arr("E", Es); arr("R", R); arr("E_inverse", Einv);
    arr("dE_0.5mm", dE); arr("highland_0.5mm", hs, true); std::printf("}\n");
    std::printf("}\n");
    return 0;
}
