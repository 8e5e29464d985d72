// trail.cuh -- plasma frequency of a parametric meteor trail at a cell (FP64).
//
// n = n0(s) exp(-d^2 / r0^2): s is the position along the trail axis, d the
// distance from it; log10 n0 rises linearly from lo at s = -s_half to hi at
// s = +s_half and is held beyond.  Cell coordinates are -(N-1)/2*d + i*d along
// each axis (grid centre at the origin).  omega_p = sqrt(n QE^2 / (E0 ME))
// with the solver's constants (source/meteor-2.1.cpp:12-18).
#pragma once

#include "common.hpp"

namespace mfdtd {

struct TrailDev {
    int Nx, Ny, Nz;
    double dx, dy, dz, c[3], a[3], r0, lo, hi, sh;
};

inline TrailDev trail_dev(const Problem &P) {
    TrailDev t;
    t.Nx = P.Nx; t.Ny = P.Ny; t.Nz = P.Nz;
    t.dx = P.dx; t.dy = P.dy; t.dz = P.dz;
    for (int q = 0; q < 3; q++) { t.c[q] = P.trail.centre[q]; t.a[q] = P.trail.axis[q]; }
    t.r0 = P.trail.r0; t.lo = P.trail.log10n_lo; t.hi = P.trail.log10n_hi; t.sh = P.trail.s_half;
    return t;
}

// E0 * omega_p^2 for the FP32 form: geometry in FP64, the density's exp10/exp
// in FP32 (the map is stored in FP32; FP64 transcendentals are slow here).
__device__ __forceinline__ float trail_wq_f32(const TrailDev &t, int i, int j, int k) {
    const double kQE = 1.602177e-19, kE0 = 8.85419e-12, kME = 9.10939e-31;
    const double x = -(t.Nx - 1) / 2.0 * t.dx + t.dx * i - t.c[0];
    const double y = -(t.Ny - 1) / 2.0 * t.dy + t.dy * j - t.c[1];
    const double z = -(t.Nz - 1) / 2.0 * t.dz + t.dz * k - t.c[2];
    const double s = x * t.a[0] + y * t.a[1] + z * t.a[2];
    double d2 = x * x + y * y + z * z - s * s;
    if (d2 < 0) d2 = 0;
    double f = (s + t.sh) / (2 * t.sh);
    f = f < 0 ? 0 : (f > 1 ? 1 : f);
    const float lg = (float)(t.lo + (t.hi - t.lo) * f);
    const float n = exp10f(lg) * expf((float)(-d2 / (t.r0 * t.r0)));
    return (float)(kE0 * (kQE * kQE / (kE0 * kME))) * n;  // E0 wp^2 = n QE^2 / ME
}

__device__ __forceinline__ double trail_wp(const TrailDev &t, int i, int j, int k) {
    const double kQE = 1.602177e-19, kE0 = 8.85419e-12, kME = 9.10939e-31;
    const double x = -(t.Nx - 1) / 2.0 * t.dx + t.dx * i - t.c[0];
    const double y = -(t.Ny - 1) / 2.0 * t.dy + t.dy * j - t.c[1];
    const double z = -(t.Nz - 1) / 2.0 * t.dz + t.dz * k - t.c[2];
    const double s = x * t.a[0] + y * t.a[1] + z * t.a[2];
    double d2 = x * x + y * y + z * z - s * s;
    if (d2 < 0) d2 = 0;
    double f = (s + t.sh) / (2 * t.sh);
    f = f < 0 ? 0 : (f > 1 ? 1 : f);
    const double n = pow(10.0, t.lo + (t.hi - t.lo) * f) * exp(-d2 / (t.r0 * t.r0));
    return sqrt(n * kQE * kQE / (kE0 * kME));
}

}  // namespace mfdtd
