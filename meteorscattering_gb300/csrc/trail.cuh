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
    // FP32 copies for the FP32 form's map: cell sizes, centre, axis,
    // 1/r0^2, the log10 n0 end points, 1/(2 s_half), and E0 QE^2/(E0 ME)
    float fd[3], fc[3], fa[3], finv_r02, flo, fhi, fsh, finv_2sh, fwq;
};

inline TrailDev trail_dev(const Problem &P) {
    TrailDev t;
    t.Nx = P.Nx; t.Ny = P.Ny; t.Nz = P.Nz;
    t.dx = P.dx; t.dy = P.dy; t.dz = P.dz;
    for (int q = 0; q < 3; q++) { t.c[q] = P.trail.centre[q]; t.a[q] = P.trail.axis[q]; }
    t.r0 = P.trail.r0; t.lo = P.trail.log10n_lo; t.hi = P.trail.log10n_hi; t.sh = P.trail.s_half;
    const double kQE = 1.602177e-19, kE0 = 8.85419e-12, kME = 9.10939e-31;
    const double d[3] = {P.dx, P.dy, P.dz};
    for (int q = 0; q < 3; q++) {
        t.fd[q] = (float)d[q];
        t.fc[q] = (float)t.c[q];
        t.fa[q] = (float)t.a[q];
    }
    t.finv_r02 = (float)(1.0 / (t.r0 * t.r0));
    t.flo = (float)t.lo;
    t.fhi = (float)t.hi;
    t.fsh = (float)t.sh;
    t.finv_2sh = (float)(1.0 / (2 * t.sh));
    t.fwq = (float)(kE0 * (kQE * kQE / (kE0 * kME)));
    return t;
}

// E0 * omega_p^2 for the FP32 form (the map is stored in FP32), in FP32 on
// this part's full-rate pipes (FP64 geometry made the map of a 768x768x1536
// grid take 67 ms).  The offset from the axis is formed as r - s a rather
// than |r|^2 - s^2, which would cancel near the axis far from the centre:
// the map then agrees with the FP64 one to about 1e-5 relative.
__device__ __forceinline__ float trail_wq_f32(const TrailDev &t, int i, int j, int k) {
    const float x = ((float)i - 0.5f * (float)(t.Nx - 1)) * t.fd[0] - t.fc[0];
    const float y = ((float)j - 0.5f * (float)(t.Ny - 1)) * t.fd[1] - t.fc[1];
    const float z = ((float)k - 0.5f * (float)(t.Nz - 1)) * t.fd[2] - t.fc[2];
    const float s = x * t.fa[0] + y * t.fa[1] + z * t.fa[2];
    const float px = x - s * t.fa[0], py = y - s * t.fa[1], pz = z - s * t.fa[2];
    const float d2 = px * px + py * py + pz * pz;
    float f = (s + t.fsh) * t.finv_2sh;
    f = f < 0.f ? 0.f : (f > 1.f ? 1.f : f);
    const float lg = t.flo + (t.fhi - t.flo) * f;
    return t.fwq * (exp10f(lg) * expf(-d2 * t.finv_r02));  // E0 wp^2 = n QE^2 / ME
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
