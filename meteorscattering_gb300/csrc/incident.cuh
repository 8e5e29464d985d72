// incident.cuh -- the incident plane wave at any field node, for reading out
// scattered fields (total minus incident inside the total-field region), as
// analysis/plotMresults.m:210-234 does on the host for its movies.
//
// The total-field region of a node is the one the TF/SF corrections of the
// update imply, so that the subtraction leaves exactly the scattered field:
//   * plane wave along +x from the reference's 1-D line
//     (source/meteor-2.1.cpp:705-923, 1069-1304): the corrections are gated by
//     index ranges that ignore staggering, so E_y/E_z nodes are inside for
//     i, j, k in [b1, b2-1] and H_y/H_z nodes for i in [bx1, bx2-2],
//     j in [by1, by2-1], k in [bz1, bz2-1]; E_x and H_x have no incident part;
//   * oblique incidence (the auxiliary line of the extended inputs): a node
//     with doubled coordinates P is inside when every P[d] lies in
//     [2 b1[d], 2 (b2[d] - 1)], and sees the line at s = kr . P/2 + s0 (E) or
//     s - 1/2 (H, whose line nodes sit half a cell on), weighted by the field
//     direction ke / kh.
// Line values are those of the state being read: E^{n+1} and H^{n+1/2} after
// pass n.
#pragma once

template <class T>
struct IncidentWave {
    int oblique;
    int b1[3], b2[3];
    const T *ey, *ez, *hy, *hz;  // 1-D line along x (plane wave along +x)
    const T *eline, *hline;      // auxiliary line (oblique)
    double kr[3], s0, ke[3], kh[3];

    __device__ double line_at(const T *line, double s) const {
        const double fl = floor(s);
        const int n = (int)fl;
        const double w = s - fl;
        return (double)line[n] + w * ((double)line[n + 1] - (double)line[n]);
    }
    __device__ bool in_box2(const int P[3]) const {
        for (int d = 0; d < 3; d++)
            if (P[d] < 2 * b1[d] || P[d] > 2 * (b2[d] - 1)) return false;
        return true;
    }
    // Incident E_c (c = 0, 1, 2) at the E_c node of cell (i, j, k); 0 outside.
    __device__ double e(int c, int i, int j, int k) const {
        if (!oblique) {
            if (c == 0) return 0.0;
            if (i < b1[0] || i > b2[0] - 1 || j < b1[1] || j > b2[1] - 1 || k < b1[2] || k > b2[2] - 1)
                return 0.0;
            return (double)(c == 1 ? ey[i] : ez[i]);
        }
        const int P[3] = {2 * i + (c == 0), 2 * j + (c == 1), 2 * k + (c == 2)};
        if (!in_box2(P)) return 0.0;
        const double s = kr[0] * (0.5 * P[0]) + kr[1] * (0.5 * P[1]) + kr[2] * (0.5 * P[2]) + s0;
        return ke[c] * line_at(eline, s);
    }
    // Incident H_c at the H_c node of cell (i, j, k); 0 outside.
    __device__ double h(int c, int i, int j, int k) const {
        if (!oblique) {
            if (c == 0) return 0.0;
            if (i < b1[0] || i > b2[0] - 2 || j < b1[1] || j > b2[1] - 1 || k < b1[2] || k > b2[2] - 1)
                return 0.0;
            return (double)(c == 1 ? hy[i] : hz[i]);
        }
        const int P[3] = {2 * i + (c != 0), 2 * j + (c != 1), 2 * k + (c != 2)};
        if (!in_box2(P)) return 0.0;
        const double s = kr[0] * (0.5 * P[0]) + kr[1] * (0.5 * P[1]) + kr[2] * (0.5 * P[2]) + s0;
        return kh[c] * line_at(hline, s - 0.5);
    }
};

// One slice element of a record block (source/meteor-2.1.cpp:996-1013,
// 1322-1340): the plane (z at k = ssz, y at j = ssy, x at i = ssx), the
// component (0: y, 1: z) and the cell, from the element index q.  Returns
// false for the H entries the reference never assigns (they stay 0).
struct SliceCell {
    int i, j, k, comp;
};
__device__ __forceinline__ bool slice_cell_of(size_t q, int Nx, int Ny, int Nz, int ssx, int ssy, int ssz,
                                              bool is_h, SliceCell *c) {
    const size_t zxy = (size_t)Nx * Ny, yxz = (size_t)Nx * Nz, xyz = (size_t)Ny * Nz;
    if (q < 2 * zxy) {
        c->comp = (int)(q / zxy);
        const size_t r = q % zxy;
        c->i = (int)(r / Ny); c->j = (int)(r % Ny); c->k = ssz;
        return !(is_h && c->j >= Ny - 1);
    }
    q -= 2 * zxy;
    if (q < 2 * yxz) {
        c->comp = (int)(q / yxz);
        const size_t r = q % yxz;
        c->i = (int)(r / Nz); c->k = (int)(r % Nz); c->j = ssy;
        return !(is_h && c->k >= Nz - 1);
    }
    q -= 2 * yxz;
    c->comp = (int)(q / xyz);
    const size_t r = q % xyz;
    c->j = (int)(r / Nz); c->k = (int)(r % Nz); c->i = ssx;
    return !(is_h && (c->j >= Ny - 1 || c->k >= Nz - 1));
}
