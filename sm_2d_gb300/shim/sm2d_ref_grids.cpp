// sm2d_ref_grids.cpp -- EnergyGrid, AngularGrid and RLUT of the C++ drop-in
// layer for programs built without the SM_2D tree's host code (grids.cpp,
// r_lut.cpp): the same tables from this library's host entries, which equal
// the reference's bit for bit (sm2d_tables.cpp).  A program linked with the
// reference's host objects uses those instead and leaves this file out.
#include <algorithm>
#include <cmath>
#include <vector>

#include "sm2d.h"
#include "sm2d_ref_types.hpp"

EnergyGrid::EnergyGrid(float E_min_, float E_max_, int N_E_)
    : N_E(N_E_), E_min(E_min_), E_max(E_max_), edges(N_E_ + 1), rep(N_E_), is_piecewise(false) {
    sm2d_energy_grid_log(E_min, E_max, N_E, edges.data(), rep.data());
}

EnergyGrid EnergyGrid::CreatePiecewise(const std::vector<std::tuple<float, float, float>>& groups) {
    std::vector<float> g;
    for (const auto& t : groups) {
        g.push_back(std::get<0>(t));
        g.push_back(std::get<1>(t));
        g.push_back(std::get<2>(t));
    }
    const int n = sm2d_energy_grid_piecewise((int)groups.size(), g.data(), nullptr, nullptr);
    EnergyGrid e(1.0f, 2.0f, 1);
    if (n <= 0) return e;
    e.N_E = n;
    e.edges.assign(n + 1, 0.0f);
    e.rep.assign(n, 0.0f);
    sm2d_energy_grid_piecewise((int)groups.size(), g.data(), e.edges.data(), e.rep.data());
    e.E_min = e.edges.front();
    e.E_max = e.edges.back();
    e.is_piecewise = true;
    return e;
}

int EnergyGrid::FindBin(float E) const {
    if (E <= edges[0]) return 0;
    if (E >= edges[N_E]) return N_E - 1;
    return (int)(std::upper_bound(edges.begin(), edges.end(), E) - edges.begin()) - 1;
}
float EnergyGrid::GetRepEnergy(int bin) const { return rep[std::max(0, std::min(bin, N_E - 1))]; }

AngularGrid::AngularGrid(float lo, float hi, int N)
    : N_theta(N), theta_min(lo), theta_max(hi), edges(N + 1), rep(N) {
    sm2d_angular_grid(lo, hi, N, edges.data(), rep.data());
}
int AngularGrid::FindBin(float theta) const {
    if (theta <= edges[0]) return 0;
    if (theta >= edges[N_theta]) return N_theta - 1;
    return (int)(std::upper_bound(edges.begin(), edges.end(), theta) - edges.begin()) - 1;
}
float AngularGrid::GetRepTheta(int bin) const { return rep[std::max(0, std::min(bin, N_theta - 1))]; }

RLUT GenerateRLUT(const EnergyGrid& grid) {
    RLUT l{grid, {}, {}, {}, {}, {}};
    const size_t n = (size_t)grid.N_E;
    l.R.resize(n); l.S.resize(n); l.log_E.resize(n); l.log_R.resize(n); l.log_S.resize(n);
    sm2d_range_lut(grid.N_E, grid.rep.data(), l.R.data(), l.S.data(), l.log_E.data(), l.log_R.data(), l.log_S.data());
    return l;
}
RLUT GenerateRLUT(float E_min, float E_max, int N_E) { return GenerateRLUT(EnergyGrid(E_min, E_max, N_E)); }

// log-log interpolation between the table's representative energies
static float loglog(const std::vector<float>& lx, const std::vector<float>& ly, float x) {
    const float l = std::log(x);
    if (l <= lx.front()) return std::exp(ly.front());
    if (l >= lx.back()) return std::exp(ly.back());
    const size_t i = (size_t)(std::upper_bound(lx.begin(), lx.end(), l) - lx.begin()) - 1;
    const float t = (l - lx[i]) / (lx[i + 1] - lx[i]);
    return std::exp(ly[i] + t * (ly[i + 1] - ly[i]));
}
float RLUT::lookup_R(float E) const { return loglog(log_E, log_R, E); }
float RLUT::lookup_S(float E) const { return loglog(log_E, log_S, E); }
float RLUT::lookup_E_inverse(float Rv) const { return loglog(log_R, log_E, Rv); }
