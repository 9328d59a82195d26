// sm2d_tables.h -- host-side tables of the transport step (see sm2d_tables.cpp).
#pragma once

namespace sm2d {
// Records a formatted message for sm2d_last_error() and returns `code`.
int fail(int code, const char* fmt, ...);

void energy_grid_log(float E_min, float E_max, int N, float* edges, float* rep);
int energy_grid_piecewise(int n_groups, const float* groups, float* edges, float* rep);
void angular_grid(float lo, float hi, int N, float* edges, float* rep);
void range_lut(int N, const float* rep, float* R, float* S, float* logE, float* logR, float* logS);
// rho: density of each depth row (NULL: water); a row's energy loss and
// scattering thickness are its water-equivalent path rho dz
void fermi_eyges_moments(float E0, int Nz, float dz, float sigma_x0, float* A, float* B, float* sigma,
                         const float* rho = nullptr);
int lateral_kernel(float sigma_total, float sigma_x0, float dx, int Nx, double* k);
}  // namespace sm2d
