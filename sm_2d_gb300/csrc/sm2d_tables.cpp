// sm2d_tables.cpp -- host-side tables of the transport step: energy and
// angular grids, the PSTAR range LUT, the Fermi-Eyges depth moments and the
// lateral post-convolution.  Compiled with -ffp-contract=off so that the
// Arm host reproduces the reference's x86 float results.
#include "sm2d_tables.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace sm2d {

// PSTAR liquid-water table (public NIST data): energy [MeV], electronic
// stopping power [MeV cm2/g], CSDA range [g/cm2].  The reference ships the
// same 19 rows in src/data/nist/pstar_water.txt and nist_loader.cpp:26-46.
static const float kPstar[19][3] = {
    {0.001f, 133.7f, 0.000006319f}, {0.01f, 422.9f, 0.00003599f}, {0.1f, 814.5f, 0.0001607f},
    {0.5f, 412.8f, 0.0008869f},     {1.0f, 260.6f, 0.002458f},    {2.0f, 158.6f, 0.007555f},
    {5.0f, 79.11f, 0.03623f},       {10.0f, 45.64f, 0.1230f},     {20.0f, 26.05f, 0.4260f},
    {30.0f, 18.76f, 0.8853f},       {50.0f, 12.45f, 2.227f},      {70.0f, 9.555f, 4.080f},
    {80.0f, 8.622f, 5.184f},        {90.0f, 7.884f, 6.398f},      {100.0f, 7.286f, 7.718f},
    {150.0f, 5.443f, 15.77f},       {200.0f, 4.491f, 25.96f},     {250.0f, 3.910f, 37.94f},
    {300.0f, 3.519f, 51.45f}};

// EnergyGrid(E_min, E_max, N), grids.cpp:6-24: log-spaced edges, geometric-mean reps.
void energy_grid_log(float E_min, float E_max, int N, float* edges, float* rep) {
    const float a = std::log(E_min), b = std::log(E_max);
    const float step = (b - a) / N;
    for (int i = 0; i <= N; ++i) edges[i] = std::exp(a + i * step);
    for (int i = 0; i < N; ++i) rep[i] = std::sqrt(edges[i] * edges[i + 1]);
}

// EnergyGrid::CreatePiecewise, grids.cpp:37-97.
int energy_grid_piecewise(int n_groups, const float* g, float* edges, float* rep) {
    int n_total = 0;
    for (int k = 0; k < n_groups; ++k)
        n_total += static_cast<int>((g[3 * k + 1] - g[3 * k]) / g[3 * k + 2] + 0.5f);
    if (edges == nullptr) return n_total;
    int base = 0;
    for (int k = 0; k < n_groups; ++k) {
        const float lo = g[3 * k], hi = g[3 * k + 1], width = g[3 * k + 2];
        const int n = static_cast<int>((hi - lo) / width + 0.5f);
        for (int i = 0; i <= n; ++i) edges[base + i] = lo + i * width;
        for (int i = 0; i < n; ++i) rep[base + i] = std::sqrt(edges[base + i] * edges[base + i + 1]);
        base += n;
    }
    edges[n_total] = g[3 * (n_groups - 1) + 1];
    return n_total;
}

// AngularGrid, grids.cpp:121-137.
void angular_grid(float lo, float hi, int N, float* edges, float* rep) {
    const float step = (hi - lo) / N;
    for (int i = 0; i <= N; ++i) edges[i] = lo + i * step;
    for (int i = 0; i < N; ++i) rep[i] = 0.5f * (edges[i] + edges[i + 1]);
}

// GenerateRLUT(grid), r_lut.cpp:69-129: log-log interpolation of PSTAR onto
// the grid's representative energies.
void range_lut(int N, const float* rep, float* R, float* S, float* logE, float* logR, float* logS) {
    const float to_mm = 10.0f / 1.0f;
    for (int i = 0; i < N; ++i) {
        const float E = rep[i];
        int hi = 0;
        while (hi < 19 && kPstar[hi][0] < E) ++hi;
        if (hi == 0 || hi == 19) {
            const int r = hi == 0 ? 0 : 18;
            R[i] = kPstar[r][2] * to_mm;
            S[i] = kPstar[r][1];
        } else {
            const float e0 = kPstar[hi - 1][0], e1 = kPstar[hi][0];
            const float r0 = kPstar[hi - 1][2] * to_mm, r1 = kPstar[hi][2] * to_mm;
            const float s0 = kPstar[hi - 1][1], s1 = kPstar[hi][1];
            const float lr = std::log(r0) + (std::log(r1) - std::log(r0)) * (std::log(E) - std::log(e0)) /
                                                (std::log(e1) - std::log(e0));
            R[i] = std::exp(lr);
            const float ls = std::log(s0) + (std::log(s1) - std::log(s0)) * (std::log(E) - std::log(e0)) /
                                                (std::log(e1) - std::log(e0));
            S[i] = std::exp(ls);
        }
        logE[i] = std::log(rep[i]);
        logR[i] = std::log(R[i]);
        logS[i] = std::log(S[i]);
    }
}

namespace {
// Host range table on the 0.1-300 MeV 256-bin log grid that the reference's
// Fermi-Eyges precompute builds (k1k6_pipeline.cu:1068).
struct HostLut {
    int N = 256;
    float E_min = 0.1f, E_max = 300.0f;
    float edges[257], rep[256], R[256], S[256], logE[256], logR[256], logS[256];
    HostLut() {
        energy_grid_log(E_min, E_max, N, edges, rep);
        range_lut(N, rep, R, S, logE, logR, logS);
    }
    int find_bin(float E) const {  // EnergyGrid::FindBin, grids.cpp:99-113
        if (E < edges[0]) return 0;
        if (E >= edges[N]) return N - 1;
        int lo = 0, hi = N;
        while (lo < hi) {
            const int mid = (lo + hi) / 2;
            if (edges[mid + 1] <= E) lo = mid + 1; else hi = mid;
        }
        return lo;
    }
    float range(float E) const {  // RLUT::lookup_R, r_lut.cpp:131-149
        const float Ec = std::max(E_min, std::min(E, E_max));
        const int b = find_bin(Ec);
        if (b == N - 1 || Ec >= E_max) return R[N - 1];
        const float lr = logR[b] + (logR[b + 1] - logR[b]) * (std::log(Ec) - logE[b]) / (logE[b + 1] - logE[b]);
        return std::exp(lr);
    }
    float energy_of_range(float r) const {  // RLUT::lookup_E_inverse, r_lut.cpp:171-204
        if (r <= 0.0f) return E_min;
        if (r >= R[N - 1]) return E_max;
        if (r <= R[0]) return E_min;
        const int k = static_cast<int>(std::lower_bound(R, R + N, r) - R);
        const int b = std::max(0, std::min(k, N - 2));
        const float d = logR[b + 1] - logR[b];
        if (std::fabs(d) < 1e-10f) return std::exp(logE[b]);
        return std::exp(logE[b] + (logE[b + 1] - logE[b]) * (std::log(r) - logR[b]) / d);
    }
    float energy_loss(float E, float s) const {  // compute_energy_deposition, step_control.hpp:81-92
        const float r = range(E) - s;
        return E - (r <= 0.0f ? 0.0f : energy_of_range(r));
    }
};

float highland_host(float E, float ds) {  // highland.hpp:59-80
    const float mp = 938.272f;
    const float gamma = (E + mp) / mp;
    const float beta = std::sqrt(std::max(1.0f - 1.0f / (gamma * gamma), 0.0f));
    const float p = std::sqrt(std::max((E + mp) * (E + mp) - mp * mp, 0.0f));
    const float t = ds / 360.8f;
    if (t < 1e-6f) return 0.0f;
    const float bracket = std::max(1.0f + 0.038f * std::log(t), 0.25f);
    return (13.6f * 1.0f / (beta * p)) * std::sqrt(t) * bracket;
}
}  // namespace

// Fermi-Eyges moments A(z), B(z) and the total lateral sigma(z) along the
// central axis: k1k6_pipeline.cu:1061-1176 (A and B stay zero past the range,
// sigma holds its last value); through a slab phantom, each row's energy
// loss and scattering use its water-equivalent thickness.
void fermi_eyges_moments(float E0, int Nz, float dz, float sigma_x0, float* A, float* B, float* sigma, const float* rho) {
    for (int i = 0; i < Nz; ++i) { A[i] = 0.0f; B[i] = 0.0f; sigma[i] = sigma_x0; }
    if (!(E0 > 0.0f)) {
        std::fill(sigma, sigma + Nz, 0.0f);
        return;
    }
    static const HostLut lut;
    {
        float E = E0, a = 0.0f, b = 0.0f;
        for (int iz = 0; iz < Nz; ++iz) {
            A[iz] = a;
            B[iz] = b;
            if (E <= 0.5f) break;
            const float rw = (rho ? rho[iz] : 1.0f) * dz;
            float dE = std::min(lut.energy_loss(E, rw), E - 0.1f);
            float Em = E - 0.5f * dE;
            if (Em < 0.5f) Em = 0.5f;
            const float th = highland_host(Em, rw);
            const float T = th * th / dz;
            const float a_prev = a;
            a = a_prev + T * dz;
            b = b + a_prev * dz + 0.5f * T * dz * dz;
            E -= dE;
            if (E < 0.1f) E = 0.1f;
        }
    }
    float E = E0, a = 0.0f, b = 0.0f, C = sigma_x0 * sigma_x0;
    for (int iz = 0; iz < Nz; ++iz) {
        sigma[iz] = std::sqrt(std::max(0.0f, C));
        if (E <= 0.5f) {
            for (int j = iz + 1; j < Nz; ++j) sigma[j] = sigma[iz];
            break;
        }
        const float rw = (rho ? rho[iz] : 1.0f) * dz;
        const float dE = std::min(lut.energy_loss(E, rw), E - 0.1f);
        const float Em = std::max(0.5f, E - 0.5f * dE);
        const float th = highland_host(Em, rw);
        const float T = th * th / dz;
        C += 2.0f * b * dz + a * dz * dz + T * dz * dz * dz / 3.0f;
        const float a_prev = a;
        a = a_prev + T * dz;
        b = b + a_prev * dz + 0.5f * T * dz * dz;
        E -= dE;
        if (E < 0.1f) E = 0.1f;
    }
}

// Kernel of the per-row lateral convolution (gpu_transport_wrapper.cu:551-584):
// sigma_MCS(z) = sqrt(sigma_total^2 - sigma0^2) in cells, truncated at 3 sigma.
// Returns the half width (0 = row left unchanged).
int lateral_kernel(float sigma_total, float sigma_x0, float dx, int Nx, double* k) {
    const float msq = sigma_total * sigma_total - sigma_x0 * sigma_x0;
    if (msq <= 1e-6f) return 0;
    const float sc = std::sqrt(msq) / dx;
    int half = static_cast<int>(std::ceil(3.0f * sc));
    half = std::max(1, std::min(half, Nx / 2));
    double sum = 0.0;
    for (int j = -half; j <= half; ++j) {
        const double v = std::exp(-0.5 * (static_cast<double>(j) * j) / (static_cast<double>(sc) * sc));
        k[j + half] = v;
        sum += v;
    }
    for (int j = 0; j <= 2 * half; ++j) k[j] /= sum;
    return half;
}

}  // namespace sm2d
