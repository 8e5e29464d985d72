// plain_fp64.cu -- FP64 plain form of the meteor FDTD time step.
//
// This is the drop-in form: every cell performs the reference's floating-point
// operations in the reference's order (this file is compiled with
// -fmad=false, IEEE division and square root), so its fields, currents and
// running DFT sums are bit-identical to source/meteor-fork.cpp on the same
// inputs.  One thread owns one Yee cell (i,j,k) and all three components there.
//
// A time step is two kernels:
//   k_plain_h  -- J update of the previous step (source/meteor-fork.cpp:
//                 1523-1595; it only reads E, which this kernel does not
//                 write), then the H half-step with its CPML psi recursion,
//                 TF/SF face corrections and CPML corrections
//                 (source/meteor-2.1.cpp:656-937), the 1-D incident-line H
//                 update, and the E probes of the previous step.
//   k_plain_e  -- the E half-step with psi, TF/SF, plate, CPML
//                 (source/meteor-2.1.cpp:1020-1374), the 1-D incident-line E
//                 update and source injection, both halves of the running
//                 DFT on the Huygens surface (:942-992, :1388-1438), the H
//                 probes and, on record steps, the field slices (:997-1014,
//                 :1323-1340; Ez is sampled before its CPML correction).
// Lagging J by one kernel is exact: the reference updates J after every E
// cell is final, and k_plain_h of the next step sees exactly those values.
#include <cuda_runtime.h>

#include "common.hpp"
#include "incident.cuh"
#include "trail.cuh"

namespace mfdtd {
namespace {

constexpr double kE0 = 8.85419e-12;

__device__ __forceinline__ size_t cidx(const PlainArgs &a, int i, int j, int k) {
    return ((size_t)i * a.Ny + (size_t)j) * a.Nz + (size_t)k;
}
// psi slabs: x-normal [2L][Ny][Nz], y-normal [Nx][2L][Nz], z-normal [Nx][Ny][2L]
__device__ __forceinline__ size_t pxi(const PlainArgs &a, int ii, int j, int k) {
    return ((size_t)ii * a.Ny + (size_t)j) * a.Nz + (size_t)k;
}
__device__ __forceinline__ size_t pyi(const PlainArgs &a, int i, int jj, int k) {
    return ((size_t)i * (2 * a.L) + (size_t)jj) * a.Nz + (size_t)k;
}
__device__ __forceinline__ size_t pzi(const PlainArgs &a, int i, int j, int kk) {
    return ((size_t)i * a.Ny + (size_t)j) * (2 * a.L) + (size_t)kk;
}

// Slab index for the H-psi ranges [0,L) and [N-L-1, N-1); -1 if outside.
__device__ __forceinline__ int hslab(int n, int N, int L, int shift) {
    if (n < L) return n;
    if (n >= N - L - 1 && n < N - 1) return n - shift;
    return -1;
}
// Slab index for the E-psi ranges [1,L+1) and [N-L-1, N-1); -1 if outside.
__device__ __forceinline__ int eslab(int n, int N, int L, int shift) {
    if (n >= 1 && n < L + 1) return n - 1;
    if (n >= N - L - 1 && n < N - 1) return n - shift;
    return -1;
}

// ---- oblique incidence (extended inputs) ----------------------------------
// The incident field comes from a 1-D auxiliary line along k (E in Ezinc, H in
// Hyinc).  A node with doubled coordinates P sees the line at
// s = kr . P/2 + s0, E nodes at s and H nodes at s - 1/2, interpolated
// linearly.  Every curl term whose neighbour lies on the other side of the
// TF/SF box surface is corrected with the neighbour's incident value.  Same
// expression trees as the oracle, so the FP64 results are bit-identical.
__device__ __forceinline__ bool obl_in(const PlainArgs &a, const int P[3]) {
    return P[0] >= 2 * a.bx1 && P[0] <= 2 * (a.bx2 - 1) && P[1] >= 2 * a.by1 &&
           P[1] <= 2 * (a.by2 - 1) && P[2] >= 2 * a.bz1 && P[2] <= 2 * (a.bz2 - 1);
}
__device__ __forceinline__ double obl_line(const double *line, double s) {
    const double fl = floor(s);
    const int n = (int)fl;
    const double w = s - fl;
    return line[n] + w * (line[n + 1] - line[n]);
}
__device__ __forceinline__ bool obl_shell(const PlainArgs &a, int i, int j, int k) {
    return i >= a.bx1 - 1 && i <= a.bx2 && j >= a.by1 - 1 && j <= a.by2 && k >= a.bz1 - 1 &&
           k <= a.bz2 &&
           !(i > a.bx1 && i < a.bx2 - 2 && j > a.by1 && j < a.by2 - 2 && k > a.bz1 && k < a.bz2 - 2);
}
// Correction of component c of the target field (E when is_e) at (i,j,k);
// returns false when no curl-term neighbour crosses the box surface.
__device__ bool obl_corr(const PlainArgs &a, bool is_e, int c, int i, int j, int k, double *corr) {
    int P[3] = {2 * i, 2 * j, 2 * k};
    for (int q = 0; q < 3; q++)
        if (is_e ? q == c : q != c) P[q] += 1;
    const bool T = obl_in(a, P);
    const int ax[2] = {(c + 1) % 3, (c + 2) % 3};
    const int comp[2] = {(c + 2) % 3, (c + 1) % 3};
    const int sg[2] = {is_e ? 1 : -1, is_e ? -1 : 1};
    const double d[3] = {a.dx, a.dy, a.dz};
    const double *line = is_e ? a.Hyinc : a.Ezinc;  // the neighbour field's line
    double acc = 0;
    bool any = false;
    for (int term = 0; term < 2; term++)
        for (int side = 1; side >= -1; side -= 2) {
            int Q[3] = {P[0], P[1], P[2]};
            Q[ax[term]] += side;
            const bool Tn = obl_in(a, Q);
            if (Tn == T) continue;
            const double sp = ((a.kr[0] * (0.5 * Q[0]) + a.kr[1] * (0.5 * Q[1])) + a.kr[2] * (0.5 * Q[2])) + a.s0;
            const double inc = is_e ? a.kh[comp[term]] * obl_line(line, sp - 0.5)
                                    : a.ke[comp[term]] * obl_line(line, sp);
            const double v = inc / d[ax[term]];
            if (sg[term] * side * ((int)T - (int)Tn) > 0) acc = acc + v;
            else acc = acc - v;
            any = true;
        }
    *corr = acc;
    return any;
}

__device__ __forceinline__ bool in_sphere(const PlainArgs &a, int i, int j, int k) {
    double x = a.xc[i], y = a.yc[j], z = a.zc[k];
    double dist = sqrt(x * x + y * y + z * z);
    return dist < a.platesize;
}

// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_plain_h(PlainArgs a, int t) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int i = blockIdx.z;
    const int Nx = a.Nx, Ny = a.Ny, Nz = a.Nz, L = a.L;
    if (k >= Nz || j >= Ny) return;
    const size_t c = cidx(a, i, j, k);
    const size_t sI = (size_t)Ny * Nz, sJ = (size_t)Nz;

    // ---- J update of step t-1 (source/meteor-fork.cpp:1523-1595) ----
    if (t > 0 && i >= 1 && i < Nx - 1 && j >= 1 && j < Ny - 1 && k >= 1 && k < Nz - 1) {
        const size_t ij = (size_t)i * Ny + j;
        const double wpe = a.doplate ? 0.0 : a.wp3 ? a.wp3[c] : a.wp2[ij] * a.G[k];
        if (!a.doB0) {
            const double nue = a.doplate ? 0.0 : a.nu3 ? a.nu3[c] : a.nu2[ij] * a.G[k];
            const double dt = a.dt;
            const double ca = (2 - nue * dt) / (2 + nue * dt);
            const double cb = 2 * ((kE0 * wpe * wpe * dt) / (2 + nue * dt));
            a.Jx[c] = ca * a.Jx[c] + cb * a.Ex[c];
            a.Jy[c] = ca * a.Jy[c] + cb * a.Ey[c];
            a.Jz[c] = ca * a.Jz[c] + cb * a.Ez[c];
        } else {
            size_t e = a.lk_mode == LK_PER_K ? (size_t)k : a.lk_mode == LK_PER_IJ ? ij : c;
            const double *m = a.lk + e * kLkStride;
            // E averaged over two nodes as the reference does, or (extended
            // input) E at the current's own node.
            const double m0 = a.lk_colocated ? a.Ex[c] : (a.Ex[c] + a.Ex[c - sI]) / 2;
            const double m1 = a.lk_colocated ? a.Ey[c] : (a.Ey[c] + a.Ey[c - sJ]) / 2;
            const double m2 = a.lk_colocated ? a.Ez[c] : (a.Ez[c] + a.Ez[c - 1]) / 2;
            const double jx = a.Jx[c], jy = a.Jy[c], jz = a.Jz[c];
            const double q = kE0 * wpe * wpe;
            a.Jx[c] = m[0] * jx + m[1] * jy + m[2] * jz + q * (m[9] * m0 + m[10] * m1 + m[11] * m2);
            a.Jy[c] = m[3] * jx + m[4] * jy + m[5] * jz + q * (m[12] * m0 + m[13] * m1 + m[14] * m2);
            a.Jz[c] = m[6] * jx + m[7] * jy + m[8] * jz + q * (m[15] * m0 + m[16] * m1 + m[17] * m2);
        }
    }

    const bool inbx = i >= a.bx1 && i < a.bx2;
    const bool inby = j >= a.by1 && j < a.by2;
    const bool inbz = k >= a.bz1 && k < a.bz2;

    // ---- Hx (i < Nx, j < Ny-1, k < Nz-1), source/meteor-2.1.cpp:656-678, 766-819
    if (j < Ny - 1 && k < Nz - 1) {
        const double dEz = a.Ez[c + sJ] - a.Ez[c];
        const double dEy = a.Ey[c + 1] - a.Ey[c];
        double py = 0, pz = 0;
        int sy = -1, sz = -1;
        if (a.dopml) {
            sy = hslab(j, Ny, L, a.yshift);
            if (sy >= 0) {
                size_t o = pyi(a, i, sy, k);
                py = a.Bh[sy] * a.Phxy[o] + a.Ah[sy] * dEz / a.dy;
                a.Phxy[o] = py;
            }
            sz = hslab(k, Nz, L, a.zshift);
            if (sz >= 0) {
                size_t o = pzi(a, i, j, sz);
                pz = a.Bh[sz] * a.Phxz[o] + a.Ah[sz] * dEy / a.dz;
                a.Phxz[o] = pz;
            }
        }
        double h = a.c1h * a.Hx[c] - a.c2h * (dEz / a.dy - dEy / a.dz);
        if (!a.oblique) {
            if (inbx && inbz) {
                if (j == a.by1 - 1) h = h + a.c2h * a.Ezinc[i] / a.dy;
                if (j == a.by2 - 1) h = h - a.c2h * a.Ezinc[i] / a.dy;
            }
            if (inbx && inby) {
                if (k == a.bz1 - 1) h = h - a.c2h * a.Eyinc[i] / a.dz;
                if (k == a.bz2 - 1) h = h + a.c2h * a.Eyinc[i] / a.dz;
            }
        } else if (obl_shell(a, i, j, k)) {
            double corr;
            if (obl_corr(a, false, 0, i, j, k, &corr)) h = h + a.c2h * corr;
        }
        if (sy >= 0) h = h - a.c2h * (a.kappa_on ? py + a.Kh[sy] * dEz / a.dy : py);
        if (sz >= 0) h = h + a.c2h * (a.kappa_on ? pz + a.Kh[sz] * dEy / a.dz : pz);
        a.Hx[c] = h;
    }

    // ---- Hy (i < Nx-1, j < Ny, k < Nz-1), :680-717, 823-877
    if (i < Nx - 1 && k < Nz - 1) {
        const double dEx = a.Ex[c + 1] - a.Ex[c];
        const double dEz = a.Ez[c + sI] - a.Ez[c];
        double px = 0, pz = 0;
        int sx = -1, sz = -1;
        if (a.dopml) {
            sx = hslab(i, Nx, L, a.xshift);
            if (sx >= 0) {
                size_t o = pxi(a, sx, j, k);
                px = a.Bh[sx] * a.Phyx[o] + a.Ah[sx] * dEz / a.dx;
                a.Phyx[o] = px;
            }
            sz = hslab(k, Nz, L, a.zshift);
            if (sz >= 0) {
                size_t o = pzi(a, i, j, sz);
                pz = a.Bh[sz] * a.Phyz[o] + a.Ah[sz] * dEx / a.dz;
                a.Phyz[o] = pz;
            }
        }
        double h = a.c1h * a.Hy[c] - a.c2h * (dEx / a.dz - dEz / a.dx);
        if (!a.oblique) {
            if (inby && inbz) {
                if (i == a.bx1 - 1) h = h - a.c2h * a.Ezinc[a.bx1] / a.dx;
                if (i == a.bx2 - 1) h = h + a.c2h * a.Ezinc[a.bx2 - 1] / a.dx;
            }
        } else if (obl_shell(a, i, j, k)) {
            double corr;
            if (obl_corr(a, false, 1, i, j, k, &corr)) h = h + a.c2h * corr;
        }
        if (sx >= 0) h = h + a.c2h * (a.kappa_on ? px + a.Kh[sx] * dEz / a.dx : px);
        if (sz >= 0) h = h - a.c2h * (a.kappa_on ? pz + a.Kh[sz] * dEx / a.dz : pz);
        a.Hy[c] = h;
    }

    // ---- Hz (i < Nx-1, j < Ny-1, k < Nz), :719-760, 882-937
    if (i < Nx - 1 && j < Ny - 1) {
        const double dEy = a.Ey[c + sI] - a.Ey[c];
        const double dEx = a.Ex[c + sJ] - a.Ex[c];
        double px = 0, py = 0;
        int sx = -1, sy = -1;
        if (a.dopml) {
            sx = hslab(i, Nx, L, a.xshift);
            if (sx >= 0) {
                size_t o = pxi(a, sx, j, k);
                px = a.Bh[sx] * a.Phzx[o] + a.Ah[sx] * dEy / a.dx;
                a.Phzx[o] = px;
            }
            sy = hslab(j, Ny, L, a.yshift);
            if (sy >= 0) {
                size_t o = pyi(a, i, sy, k);
                py = a.Bh[sy] * a.Phzy[o] + a.Ah[sy] * dEx / a.dy;
                a.Phzy[o] = py;
            }
        }
        double h = a.c1h * a.Hz[c] - a.c2h * (dEy / a.dx - dEx / a.dy);
        if (!a.oblique) {
            if (inby && inbz) {
                if (i == a.bx1 - 1) h = h + a.c2h * a.Eyinc[a.bx1] / a.dx;
                if (i == a.bx2 - 1) h = h - a.c2h * a.Eyinc[a.bx2 - 1] / a.dx;
            }
        } else if (obl_shell(a, i, j, k)) {
            double corr;
            if (obl_corr(a, false, 2, i, j, k, &corr)) h = h + a.c2h * corr;
        }
        if (sx >= 0) h = h - a.c2h * (a.kappa_on ? px + a.Kh[sx] * dEy / a.dx : px);
        if (sy >= 0) h = h + a.c2h * (a.kappa_on ? py + a.Kh[sy] * dEx / a.dy : py);
        a.Hz[c] = h;
    }

    // ---- oblique incidence: auxiliary line, H part (nodes n = i, i + Nx, ...)
    if (a.oblique && j == 0 && k == 0) {
        const int M = a.M;
        for (int n = i; n < M - 1; n += Nx) {
            double h = a.c1h * a.Hyinc[n] - a.c2h * (a.Ezinc[n + 1] - a.Ezinc[n]) / a.dl;
            if (n >= M - L - 1) {
                const int s = n - a.ashift;
                const double p = a.Bh1[s] * a.PhyxI[s] + a.Ah1[s] * (a.Ezinc[n + 1] - a.Ezinc[n]) / a.dl;
                a.PhyxI[s] = p;
                h = h - a.c2h * p;
            }
            a.Hyinc[n] = h;
        }
    }

    // ---- 1-D incident line, H part (:705-706, 741-742, 833, 892, 863, 923)
    if (!a.oblique && j == 0 && k == 0 && i < Nx - 1) {
        const int s = (a.dopml && i >= Nx - L - 1) ? i - a.xshift : -1;
        double pyI = 0, pzI = 0;
        if (s >= 0) {
            pyI = a.Bh[s] * a.PhyxI[s] + a.Ah[s] * (a.Ezinc[i + 1] - a.Ezinc[i]) / a.dx;
            a.PhyxI[s] = pyI;
            pzI = a.Bh[s] * a.PhzxI[s] + a.Ah[s] * (a.Eyinc[i + 1] - a.Eyinc[i]) / a.dx;
            a.PhzxI[s] = pzI;
        }
        double hy = a.c1h * a.Hyinc[i] + a.c2h * (a.Ezinc[i + 1] - a.Ezinc[i]) / a.dx;
        double hz = a.c1h * a.Hzinc[i] - a.c2h * (a.Eyinc[i + 1] - a.Eyinc[i]) / a.dx;
        if (s >= 0) {
            hy = hy + a.c2h * pyI;
            hz = hz - a.c2h * pzI;
        }
        a.Hyinc[i] = hy;
        a.Hzinc[i] = hz;
    }

    // ---- E probes of step t-1 (:1443-1450); E is final for that step here
    if (t > 0 && i == 0 && j == 0 && k < a.nprobes) {
        const int ix = a.probe_ijk[3 * k], iy = a.probe_ijk[3 * k + 1], iz = a.probe_ijk[3 * k + 2];
        const size_t p = cidx(a, ix, iy, iz);
        const size_t o = (size_t)(t - 1) * a.nprobes + k, T = (size_t)a.tsteps * a.nprobes;
        a.probe[o] = 0.5 * (a.Ex[p] + a.Ex[p - sI]);
        a.probe[T + o] = 0.5 * (a.Ey[p] + a.Ey[p - sJ]);
        a.probe[2 * T + o] = 0.5 * (a.Ez[p] + a.Ez[p - 1]);
    }
}

// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_plain_e(PlainArgs a, int t, int record) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int i = blockIdx.z;
    const int Nx = a.Nx, Ny = a.Ny, Nz = a.Nz, L = a.L;
    if (k >= Nz || j >= Ny) return;
    const size_t c = cidx(a, i, j, k);
    const size_t sI = (size_t)Ny * Nz, sJ = (size_t)Nz;

    const bool sphere = a.doplate == 2 && in_sphere(a, i, j, k);
    const double c1e = sphere ? a.c1s : a.c1e0;
    const double c2e = sphere ? a.c2s : a.c2e0;
    const double c2e0 = a.c2e0;
    const bool plate_row = a.doplate == 1 && i == a.ssx;

    // ---- Ex (i < Nx-1, 1 <= j < Ny-1, 1 <= k < Nz-1), :1025-1048, 1130-1185
    double ex = a.Ex[c];
    if (i < Nx - 1 && j >= 1 && j < Ny - 1 && k >= 1 && k < Nz - 1) {
        const double dHz = a.Hz[c] - a.Hz[c - sJ];
        const double dHy = a.Hy[c] - a.Hy[c - 1];
        double py = 0, pz = 0;
        int sy = -1, sz = -1;
        if (a.dopml) {
            sy = eslab(j, Ny, L, a.yshift);
            if (sy >= 0) {
                size_t o = pyi(a, i, sy, k);
                py = a.Be[sy] * a.Pexy[o] + a.Ae[sy] * dHz / a.dy;
                a.Pexy[o] = py;
            }
            sz = eslab(k, Nz, L, a.zshift);
            if (sz >= 0) {
                size_t o = pzi(a, i, j, sz);
                pz = a.Be[sz] * a.Pexz[o] + a.Ae[sz] * dHy / a.dz;
                a.Pexz[o] = pz;
            }
        }
        double e = c1e * ex + c2e * (dHz / a.dy - dHy / a.dz) - c2e * a.Jx[c];
        if (!a.oblique) {
            if (i >= a.bx1 && i < a.bx2 - 1) {
                if (j >= a.by1 && j < a.by2) {
                    if (k == a.bz1) e = e + c2e0 * a.Hyinc[i] / a.dz;
                    if (k == a.bz2) e = e - c2e0 * a.Hyinc[i] / a.dz;
                }
                if (k >= a.bz1 && k < a.bz2) {
                    if (j == a.by1) e = e - c2e0 * a.Hzinc[i] / a.dy;
                    if (j == a.by2) e = e + c2e0 * a.Hzinc[i] / a.dy;
                }
            }
        } else if (obl_shell(a, i, j, k)) {
            double corr;
            if (obl_corr(a, true, 0, i, j, k, &corr)) e = e + c2e0 * corr;
        }
        if (sy >= 0) e = e + c2e0 * (a.kappa_on ? py + a.Ke[sy] * dHz / a.dy : py);
        if (sz >= 0) e = e - c2e0 * (a.kappa_on ? pz + a.Ke[sz] * dHy / a.dz : pz);
        ex = e;
        a.Ex[c] = e;
    }

    // ---- Ey (1 <= i < Nx-1, j < Ny, 1 <= k < Nz), :1052-1090, 1190-1244
    double ey = a.Ey[c];
    if (i >= 1 && i < Nx - 1 && k >= 1) {
        const double dHx = a.Hx[c] - a.Hx[c - 1];
        const double dHz = a.Hz[c] - a.Hz[c - sI];
        double px = 0, pz = 0;
        const int sx = a.dopml ? eslab(i, Nx, L, a.xshift) : -1;
        const int sz = a.dopml ? eslab(k, Nz, L, a.zshift) : -1;
        // psi is advanced on j < Ny-1, k < Nz-1 only; the correction below
        // also covers j = Ny-1 and k = Nz-1, where psi stays zero.
        if (sx >= 0 && j < Ny - 1 && k < Nz - 1) {
            size_t o = pxi(a, sx, j, k);
            px = a.Be[sx] * a.Peyx[o] + a.Ae[sx] * dHz / a.dx;
            a.Peyx[o] = px;
        }
        if (sz >= 0 && j < Ny - 1) {
            size_t o = pzi(a, i, j, sz);
            pz = a.Be[sz] * a.Peyz[o] + a.Ae[sz] * dHx / a.dz;
            a.Peyz[o] = pz;
        }
        double e = c1e * ey + c2e * (dHx / a.dz - dHz / a.dx) - c2e * a.Jy[c];
        if (!a.oblique) {
            if (j >= a.by1 && j < a.by2 && k >= a.bz1 && k < a.bz2) {
                if (i == a.bx1) e = e + c2e0 * a.Hzinc[a.bx1 - 1] / a.dx;
                if (i == a.bx2 - 1) e = e - c2e0 * a.Hzinc[a.bx2 - 1] / a.dx;
            }
        } else if (obl_shell(a, i, j, k)) {
            double corr;
            if (obl_corr(a, true, 1, i, j, k, &corr)) e = e + c2e0 * corr;
        }
        if (sx >= 0) e = e - c2e0 * (a.kappa_on ? px + a.Ke[sx] * dHz / a.dx : px);
        if (sz >= 0) e = e + c2e0 * (a.kappa_on ? pz + a.Ke[sz] * dHx / a.dz : pz);
        if (plate_row && j >= a.plate_lo && j < a.plate_up - 1 && k >= a.plate_lo && k < a.plate_up)
            e = 0;
        ey = e;
        a.Ey[c] = e;
    } else if (plate_row && j >= a.plate_lo && j < a.plate_up - 1 && k >= a.plate_lo &&
               k < a.plate_up) {
        ey = 0;
        a.Ey[c] = 0;
    }

    // ---- Ez (1 <= i < Nx-1, 1 <= j < Ny, k < Nz), :1095-1125, 1248-1374
    double ez = a.Ez[c];
    double ez_slice = ez;
    if (i >= 1 && i < Nx - 1 && j >= 1) {
        const double dHy = a.Hy[c] - a.Hy[c - sI];
        const double dHx = a.Hx[c] - a.Hx[c - sJ];
        double px = 0, py = 0;
        const int sx = a.dopml ? eslab(i, Nx, L, a.xshift) : -1;
        const int sy = a.dopml ? eslab(j, Ny, L, a.yshift) : -1;
        if (sx >= 0 && j < Ny - 1 && k < Nz - 1) {
            size_t o = pxi(a, sx, j, k);
            px = a.Be[sx] * a.Pezx[o] + a.Ae[sx] * dHy / a.dx;
            a.Pezx[o] = px;
        }
        if (sy >= 0 && k < Nz - 1) {
            size_t o = pyi(a, i, sy, k);
            py = a.Be[sy] * a.Pezy[o] + a.Ae[sy] * dHx / a.dy;
            a.Pezy[o] = py;
        }
        double e = c1e * ez + c2e * (dHy / a.dx - dHx / a.dy) - c2e * a.Jz[c];
        if (!a.oblique) {
            if (j >= a.by1 && j < a.by2 && k >= a.bz1 && k < a.bz2) {
                if (i == a.bx1) e = e - c2e0 * a.Hyinc[a.bx1 - 1] / a.dx;
                if (i == a.bx2 - 1) e = e + c2e0 * a.Hyinc[a.bx2 - 1] / a.dx;
            }
        } else if (obl_shell(a, i, j, k)) {
            double corr;
            if (obl_corr(a, true, 2, i, j, k, &corr)) e = e + c2e0 * corr;
        }
        if (plate_row && j >= a.plate_lo && j < a.plate_up && k >= a.plate_lo && k < a.plate_up - 1)
            e = 0;
        ez_slice = e;  // slices see Ez before its CPML correction
        if (sx >= 0) e = e + c2e0 * (a.kappa_on ? px + a.Ke[sx] * dHy / a.dx : px);
        if (sy >= 0 && k < Nz - 1) e = e - c2e0 * (a.kappa_on ? py + a.Ke[sy] * dHx / a.dy : py);
        ez = e;
        a.Ez[c] = e;
    } else if (plate_row && j >= a.plate_lo && j < a.plate_up && k >= a.plate_lo &&
               k < a.plate_up - 1) {
        ez = 0;
        ez_slice = 0;
        a.Ez[c] = 0;
    }

    // ---- 1-D incident line, E part and source (:1201, 1259, 1069-1071,
    //      1105-1107, 1227-1229, 1355-1357, 1278-1304)
    if (a.oblique && j == 0 && k == 0) {  // auxiliary line, E part, and the source
        const int M = a.M;
        for (int n = i; n < M - 1; n += Nx) {
            if (n == 0) {
                a.Ezinc[0] = a.src[2 * t];
                continue;
            }
            double e = a.c1e0 * a.Ezinc[n] - c2e0 * (a.Hyinc[n] - a.Hyinc[n - 1]) / a.dl;
            if (n >= M - L - 1) {
                const int s = n - a.ashift;
                const double p = a.Be1[s] * a.PezxI[s] + a.Ae1[s] * (a.Hyinc[n] - a.Hyinc[n - 1]) / a.dl;
                a.PezxI[s] = p;
                e = e - c2e0 * p;
            }
            a.Ezinc[n] = e;
        }
    }
    if (!a.oblique && j == 0 && k == 0) {
        if (i >= 1 && i < Nx - 1) {
            const int s = (a.dopml && i >= Nx - L - 1) ? i - a.xshift : -1;
            double pyI = 0, pzI = 0;
            if (s >= 0) {
                pyI = a.Be[s] * a.PeyxI[s] + a.Ae[s] * (a.Hzinc[i] - a.Hzinc[i - 1]) / a.dx;
                a.PeyxI[s] = pyI;
                pzI = a.Be[s] * a.PezxI[s] + a.Ae[s] * (a.Hyinc[i] - a.Hyinc[i - 1]) / a.dx;
                a.PezxI[s] = pzI;
            }
            double ey1 = a.c1e0 * a.Eyinc[i] - c2e0 * (a.Hzinc[i] - a.Hzinc[i - 1]) / a.dx;
            if (s >= 0) ey1 = ey1 - c2e0 * pyI;
            double ez1 = a.c1e0 * a.Ezinc[i] + c2e0 * (a.Hyinc[i] - a.Hyinc[i - 1]) / a.dx;
            if (s >= 0) ez1 = ez1 + c2e0 * pzI;
            a.Eyinc[i] = ey1;
            a.Ezinc[i] = ez1;
        } else if (i == 0) {
            a.Ezinc[0] = a.src[2 * t];
            a.Eyinc[0] = a.src[2 * t + 1];
        }
    }

    // ---- running DFT on the Huygens surface (:942-992 H part, :1388-1438 E part)
    {
        const int nb = a.ntfb, nf = a.nntf;
        const double *ph = a.phase + (size_t)t * nf * 2;
        const bool fr = i == nb, bk = i == Nx - nb, tp = j == Ny - nb, bt = j == nb,
                   lf = k == nb, rt = k == Nz - nb;
        if (fr || bk || tp || bt || lf || rt) {
            const size_t n2 = 2 * (size_t)nf;
            // H averages across the surface: own cell and the one below it.
            auto acc2 = [&](double *A, double *B, size_t base, double va, double vb) {
                for (int m = 0; m < nf; m++) {
                    const double s = ph[2 * m], co = ph[2 * m + 1];
                    A[base + 2 * m] += va * s;
                    A[base + 2 * m + 1] += va * co;
                    B[base + 2 * m] += vb * s;
                    B[base + 2 * m + 1] += vb * co;
                }
            };
            if (fr || bk) {
                const size_t base = ((size_t)j * Nz + k) * n2;
                const double hz = 0.5 * (a.Hz[c] + a.Hz[c - sI]);
                const double hy = 0.5 * (a.Hy[c] + a.Hy[c - sI]);
                if (fr) {  // Jy_front=+hz, Jz_front=-hy ; My_front=-Ez, Mz_front=+Ey
                    acc2(a.ntf[2], a.ntf[3], base, hz, -hy);
                    acc2(a.ntf[0], a.ntf[1], base, -ez, ey);
                }
                if (bk) {  // Jy_back=-hz, Jz_back=+hy ; My_back=+Ez, Mz_back=-Ey
                    acc2(a.ntf[6], a.ntf[7], base, -hz, hy);
                    acc2(a.ntf[4], a.ntf[5], base, ez, -ey);
                }
            }
            if (tp || bt) {
                const size_t base = ((size_t)i * Nz + k) * n2;
                const double hz = 0.5 * (a.Hz[c] + a.Hz[c - sJ]);
                const double hx = 0.5 * (a.Hx[c] + a.Hx[c - sJ]);
                if (tp) {  // Jx_top=+hz, Jz_top=-hx ; Mx_top=-Ez, Mz_top=+Ex
                    acc2(a.ntf[10], a.ntf[11], base, hz, -hx);
                    acc2(a.ntf[8], a.ntf[9], base, -ez, ex);
                }
                if (bt) {  // Jx_bot=-hz, Jz_bot=+hx ; Mx_bot=+Ez, Mz_bot=-Ex
                    acc2(a.ntf[14], a.ntf[15], base, -hz, hx);
                    acc2(a.ntf[12], a.ntf[13], base, ez, -ex);
                }
            }
            if (lf || rt) {
                const size_t base = ((size_t)i * Ny + j) * n2;
                const double hy = 0.5 * (a.Hy[c] + a.Hy[c - 1]);
                const double hx = 0.5 * (a.Hx[c] + a.Hx[c - 1]);
                if (lf) {  // Jx_left=+hy, Jy_left=-hx ; Mx_left=-Ey, My_left=+Ex
                    acc2(a.ntf[18], a.ntf[19], base, hy, -hx);
                    acc2(a.ntf[16], a.ntf[17], base, -ey, ex);
                }
                if (rt) {  // Jx_right=-hy, Jy_right=+hx ; Mx_right=+Ey, My_right=-Ex
                    acc2(a.ntf[22], a.ntf[23], base, -hy, hx);
                    acc2(a.ntf[20], a.ntf[21], base, ey, -ex);
                }
            }
        }
    }

    // ---- H probes of step t (:1452-1454); H is final for step t here
    if (i == 0 && j == 0 && k < a.nprobes) {
        const int ix = a.probe_ijk[3 * k], iy = a.probe_ijk[3 * k + 1], iz = a.probe_ijk[3 * k + 2];
        const size_t p = cidx(a, ix, iy, iz);
        const size_t o = (size_t)t * a.nprobes + k, T = (size_t)a.tsteps * a.nprobes;
        a.probe[3 * T + o] = 0.25 * (a.Hx[p] + a.Hx[p - sJ] + a.Hx[p - 1] + a.Hx[p - sJ - 1]);
        a.probe[4 * T + o] = 0.25 * (a.Hy[p] + a.Hy[p - sI] + a.Hy[p - 1] + a.Hy[p - sI - 1]);
        a.probe[5 * T + o] = 0.25 * (a.Hz[p] + a.Hz[p - sJ] + a.Hz[p - sI] + a.Hz[p - sI - sJ]);
    }

    // ---- slices on record steps (:997-1014 H, :1323-1340 E)
    if (record) {
        const size_t oz = 0, oy = 2 * (size_t)Nx * Ny, ox = oy + 2 * (size_t)Nx * Nz;
        if (k == a.ssz) {
            a.slE[oz + (size_t)i * Ny + j] = ey;
            a.slE[oz + (size_t)Nx * Ny + (size_t)i * Ny + j] = ez_slice;
            if (j < Ny - 1) {
                a.slH[oz + (size_t)i * Ny + j] = a.Hy[c];
                a.slH[oz + (size_t)Nx * Ny + (size_t)i * Ny + j] = a.Hz[c];
            }
        }
        if (j == a.ssy) {
            a.slE[oy + (size_t)i * Nz + k] = ey;
            a.slE[oy + (size_t)Nx * Nz + (size_t)i * Nz + k] = ez_slice;
            if (k < Nz - 1) {
                a.slH[oy + (size_t)i * Nz + k] = a.Hy[c];
                a.slH[oy + (size_t)Nx * Nz + (size_t)i * Nz + k] = a.Hz[c];
            }
        }
        if (i == a.ssx) {
            a.slE[ox + (size_t)j * Nz + k] = ey;
            a.slE[ox + (size_t)Ny * Nz + (size_t)j * Nz + k] = ez_slice;
            if (j < Ny - 1 && k < Nz - 1) {
                a.slH[ox + (size_t)j * Nz + k] = a.Hy[c];
                a.slH[ox + (size_t)Ny * Nz + (size_t)j * Nz + k] = a.Hz[c];
            }
        }
    }
}

// E probes of the last step (the per-step ones ride in the next k_plain_h).
__global__ void k_plain_flush(PlainArgs a, int t_last) {
    const int p = threadIdx.x;
    if (p >= a.nprobes) return;
    const size_t sI = (size_t)a.Ny * a.Nz, sJ = (size_t)a.Nz;
    const int ix = a.probe_ijk[3 * p], iy = a.probe_ijk[3 * p + 1], iz = a.probe_ijk[3 * p + 2];
    const size_t q = cidx(a, ix, iy, iz);
    const size_t o = (size_t)t_last * a.nprobes + p, T = (size_t)a.tsteps * a.nprobes;
    a.probe[o] = 0.5 * (a.Ex[q] + a.Ex[q - sI]);
    a.probe[T + o] = 0.5 * (a.Ey[q] + a.Ey[q - sJ]);
    a.probe[2 * T + o] = 0.5 * (a.Ez[q] + a.Ez[q - 1]);
}

// max |Ex| over the grid (source/meteor-2.1.cpp:1528-1537).  NaN is skipped,
// as the reference's `fabs(Ex) > Emax` test skips it.  Non-negative doubles
// order like their bit patterns, so an integer atomicMax suffices.
__global__ void __launch_bounds__(256) k_emax(const double *__restrict__ ex, size_t n,
                                              unsigned long long *out) {
    double m = 0.0;
    for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < n;
         q += (size_t)gridDim.x * blockDim.x) {
        double v = fabs(ex[q]);
        if (v > m) m = v;
    }
    for (int off = 16; off > 0; off >>= 1) {
        double o = __shfl_down_sync(0xffffffffu, m, off);
        if (o > m) m = o;
    }
    __shared__ double warp_max[8];
    if ((threadIdx.x & 31) == 0) warp_max[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); w++)
            if (warp_max[w] > m) m = warp_max[w];
        atomicMax(out, (unsigned long long)__double_as_longlong(m));
    }
}

// Field guard: flags any non-finite E component (the max|Ex| scan above skips
// NaN, so it cannot serve as the guard).
__global__ void __launch_bounds__(256) k_nonfinite(const double *__restrict__ ex,
                                                   const double *__restrict__ ey,
                                                   const double *__restrict__ ez, size_t n,
                                                   unsigned int *flag) {
    unsigned int bad = 0;
    for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < n;
         q += (size_t)gridDim.x * blockDim.x)
        bad |= !isfinite(ex[q]) | !isfinite(ey[q]) | !isfinite(ez[q]);
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(flag, 1u);
}

__global__ void k_trail_map(TrailDev t, double *out) {
    const size_t n = (size_t)t.Nx * t.Ny * t.Nz;
    for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < n;
         q += (size_t)gridDim.x * blockDim.x) {
        const int k = (int)(q % t.Nz), j = (int)((q / t.Nz) % t.Ny), i = (int)(q / ((size_t)t.Ny * t.Nz));
        out[q] = trail_wp(t, i, j, k);
    }
}

}  // namespace

void trail_map_fp64(const Problem &P, double *out, void *stream) {
    k_trail_map<<<152 * 8, 256, 0, (cudaStream_t)stream>>>(trail_dev(P), out);
}

int plain_launch_guard(const PlainArgs &a, void *stream) {
    cudaStream_t s = (cudaStream_t)stream;
    cudaMemsetAsync(a.flag, 0, sizeof(unsigned int), s);
    size_t n = (size_t)a.Nx * a.Ny * a.Nz;
    int blocks = (int)std::min<size_t>((n + 255) / 256, 152 * 8);
    k_nonfinite<<<blocks, 256, 0, s>>>(a.Ex, a.Ey, a.Ez, n, a.flag);
    return 1;
}

int plain_launch_step(const PlainArgs &a, int t, int record, void *stream, void *const *ev) {
    cudaStream_t s = (cudaStream_t)stream;
    dim3 block(32, 8, 1);
    dim3 grid((a.Nz + 31) / 32, (a.Ny + 7) / 8, a.Nx);
    if (ev) cudaEventRecord((cudaEvent_t)ev[0], s);
    k_plain_h<<<grid, block, 0, s>>>(a, t);
    if (ev) cudaEventRecord((cudaEvent_t)ev[1], s);
    k_plain_e<<<grid, block, 0, s>>>(a, t, record);
    if (ev) cudaEventRecord((cudaEvent_t)ev[2], s);
    return 2;
}

int plain_launch_flush(const PlainArgs &a, int t_last, void *stream) {
    if (a.nprobes <= 0) return 0;
    k_plain_flush<<<1, ((a.nprobes + 31) / 32) * 32, 0, (cudaStream_t)stream>>>(a, t_last);
    return 1;
}

// Slices of the current state in the record layout, optionally with the
// incident field subtracted inside the total-field region (scattered field).
__global__ void k_plain_slices(const PlainArgs a, IncidentWave<double> w, int scattered, double *E,
                               double *H, size_t n) {
    for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
        SliceCell c;
        slice_cell_of(q, a.Nx, a.Ny, a.Nz, a.ssx, a.ssy, a.ssz, false, &c);
        const size_t x = cidx(a, c.i, c.j, c.k);
        double e = c.comp == 0 ? a.Ey[x] : a.Ez[x];
        if (scattered) e -= w.e(1 + c.comp, c.i, c.j, c.k);
        E[q] = e;
        double h = 0.0;
        if (slice_cell_of(q, a.Nx, a.Ny, a.Nz, a.ssx, a.ssy, a.ssz, true, &c)) {
            h = c.comp == 0 ? a.Hy[x] : a.Hz[x];
            if (scattered) h -= w.h(1 + c.comp, c.i, c.j, c.k);
        }
        H[q] = h;
    }
}

int plain_launch_slices(const PlainArgs &a, int scattered, double *E, double *H, void *stream) {
    IncidentWave<double> w{};
    w.oblique = a.oblique;
    w.b1[0] = a.bx1; w.b1[1] = a.by1; w.b1[2] = a.bz1;
    w.b2[0] = a.bx2; w.b2[1] = a.by2; w.b2[2] = a.bz2;
    w.ey = a.Eyinc; w.ez = a.Ezinc; w.hy = a.Hyinc; w.hz = a.Hzinc;
    w.eline = a.Ezinc; w.hline = a.Hyinc;  // the auxiliary line's E and H (oblique)
    for (int d = 0; d < 3; d++) { w.kr[d] = a.kr[d]; w.ke[d] = a.ke[d]; w.kh[d] = a.kh[d]; }
    w.s0 = a.s0;
    const size_t n = 2 * ((size_t)a.Nx * a.Ny + (size_t)a.Nx * a.Nz + (size_t)a.Ny * a.Nz);
    k_plain_slices<<<152 * 4, 256, 0, (cudaStream_t)stream>>>(a, w, scattered, E, H, n);
    return 1;
}

int plain_launch_emax(const PlainArgs &a, void *stream) {
    cudaStream_t s = (cudaStream_t)stream;
    cudaMemsetAsync(a.emax, 0, sizeof(unsigned long long), s);
    size_t n = (size_t)a.Nx * a.Ny * a.Nz;
    int blocks = (int)std::min<size_t>((n + 255) / 256, 152 * 8);
    k_emax<<<blocks, 256, 0, s>>>(a.Ex, n, a.emax);
    return 1;
}

}  // namespace mfdtd
