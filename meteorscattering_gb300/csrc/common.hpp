// common.hpp -- internal types shared by the host code and the CUDA kernels.
#pragma once

#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/mfdtd.h"

namespace mfdtd {

// Largest CPML thickness the kernels' coefficient tables hold (the reference
// hard-codes 10 cells, source/meteor-2.1.cpp:343).
constexpr int kMaxPml = 32;

// Record the message mfdtd_last_error() returns on this thread (sim.cpp).
void set_last_error(const std::string &msg);

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

// How the Lee-Kalluri update matrices are indexed.  The collision frequency of
// a cell is nu2[i][j] * G[k] (source/meteor-2.1.cpp:325-326), so when nu2 is
// uniform the matrices vary with k only, and when G is identically 1 they
// vary with (i,j) only; the general case needs one entry per cell.
enum LkMode : int { LK_PER_K = 0, LK_PER_IJ = 1, LK_PER_CELL = 2 };
constexpr int kLkStride = 18;  // Ae[3][3] then Ke[3][3], row-major

// Parsed inputs plus every host-side table the time loop needs.  All derived
// values are computed on the host with the same expression trees as the
// reference (source/meteor-2.1.cpp:116-552, source/meteor-fork.cpp:226-232,
// 1546-1573) so that the device sees bit-identical coefficients.
struct Problem {
    // inputs.dat
    int dopml = 1, savefields = 0, sourcetype = 2, sourcepol = 1, tsteps = 0;
    int Nx = 0, Ny = 0, Nz = 0, mettype = 0, numfiles = 1, doplate = 0, doB0 = 0;
    int doB0_present = 0;
    double f0 = 0, fsig = 0, gridfactor = 0, dt = 0, metsize[2] = {0, 0};
    double wpmax = 0, numax = 0, metloc[3] = {0, 0, 0}, metangle = 0, platesize = 0;
    std::vector<int32_t> probex, probey, probez;
    std::vector<double> fntf;
    double B[3] = {0, 0, 0};
    std::vector<double> wp2, nu2;  // [Nx][Ny] as read

    // derived
    int L = 10, xshift = 0, yshift = 0, zshift = 0;
    int bx1 = 0, bx2 = 0, by1 = 0, by2 = 0, bz1 = 0, bz2 = 0, ntfb = 0;
    int ssx = 0, ssy = 0, ssz = 0, plate_lo = 0, plate_up = 0, record_period = 1;
    double dx = 0, dy = 0, dz = 0, c1h = 0, c2h = 0, c1e0 = 0, c2e0 = 0, c1s = 0, c2s = 0;
    double wcex = 0, wcey = 0, wcez = 0, wce0 = 0;
    std::vector<double> x, y, z;       // cell coordinates (reference quirks kept)
    std::vector<double> G;             // z-Gaussian factor per k
    std::vector<double> wp2e, nu2e;    // effective 2-D maps (zero when doplate)
    std::vector<double> src;           // [tsteps][2] : Ezinc[0], Eyinc[0]
    std::vector<double> phase;         // [tsteps][nntf][2] : sin, cos
    std::vector<double> Be, Ae, Bh, Ah;  // [2L] CPML recursion coefficients
    int lk_mode = LK_PER_K;
    std::vector<double> lk;            // L&K matrices, kLkStride per entry
    std::vector<double> srcdft;        // Eydft[2n] then Ezdft[2n] (full run)

    // Extended inputs (no counterpart in the reference's inputs.dat): CPML
    // thickness and grading, TF/SF and Huygens-surface offsets, oblique
    // plane-wave incidence, exact coordinates, per-cell plasma maps.  With
    // ext_present == 0 every derived table is the reference's.
    mfdtd_ext ext{};
    int ext_present = 0;
    std::vector<double> wp3, nu3;      // [Nx][Ny][Nz] omega_p and nu, when given
    int has_trail = 0;                 // parametric trail (replaces wp2 * G and wp3)
    mfdtd_trail trail{};               // axis normalised

    // derived, extended
    int kappa_on = 0;
    std::vector<double> Ke, Kh;        // [2L] 1/kappa - 1 at E and H grading
    int oblique = 0;
    double inc_k[3] = {1, 0, 0}, inc_e[3] = {0, 0, 1}, inc_h[3] = {0, -1, 0};
    double dl = 0;                     // auxiliary-line cell size (dispersion matched)
    double kr[3] = {0, 0, 0}, s0 = 0;  // s(r) = kr . r_cells + s0, in line cells
    int M = 0, ashift = 0;             // line nodes; psi index = n - ashift at the far end
    std::vector<double> Be1, Ae1, Bh1, Ah1;  // [2L] line CPML (high half used)

    int nprobes() const { return (int)probex.size(); }
    int nntf() const { return (int)fntf.size(); }
    size_t cells() const { return (size_t)Nx * Ny * Nz; }
    void derive();  // fills every derived member; throws Error on bad input
};

// The reference's values of every extended input (problem.cpp).
void ext_defaults(mfdtd_ext &e);

Problem problem_from_rundir(const std::string &dir);
Problem problem_from_params(const mfdtd_params &p, const double *wp2, const double *nu2,
                            const double B0[3]);

// Arguments of the FP64 plain-form kernels (passed by value).
struct PlainArgs {
    int Nx, Ny, Nz, L, xshift, yshift, zshift;
    int bx1, bx2, by1, by2, bz1, bz2, ntfb, nntf, ssx, ssy, ssz;
    int dopml, doplate, doB0, lk_mode, plate_lo, plate_up, nprobes, tsteps;
    double dx, dy, dz, c1h, c2h, c1e0, c2e0, c1s, c2s, platesize, dt;
    double Be[2 * kMaxPml], Ae[2 * kMaxPml], Bh[2 * kMaxPml], Ah[2 * kMaxPml];
    double *Ex, *Ey, *Ez, *Hx, *Hy, *Hz, *Jx, *Jy, *Jz;
    double *Phxy, *Phxz, *Phyx, *Phyz, *Phzx, *Phzy;
    double *Pexy, *Pexz, *Peyx, *Peyz, *Pezx, *Pezy;
    double *Eyinc, *Ezinc, *Hyinc, *Hzinc, *PeyxI, *PezxI, *PhyxI, *PhzxI;
    const double *wp2, *nu2, *G, *xc, *yc, *zc, *lk, *src, *phase;
    double *ntf[24];
    // extended inputs
    int kappa_on, oblique, M, ashift, lk_colocated;
    double Ke[2 * kMaxPml], Kh[2 * kMaxPml];
    double ke[3], kh[3], kr[3], s0, dl;
    double Be1[2 * kMaxPml], Ae1[2 * kMaxPml], Bh1[2 * kMaxPml], Ah1[2 * kMaxPml];
    const double *wp3, *nu3;  // per-cell maps or null
    double *probe;            // [6][tsteps][nprobes]
    const int *probe_ijk;     // [nprobes][3]
    double *slE, *slH;        // slice records (z, y, x planes, 2 comps each)
    unsigned long long *emax; // max|Ex| bits
    unsigned int *flag;       // non-finite E detected
};

// Launchers (plain_fp64.cu).  All enqueue on `stream` and return the number of
// kernels launched.
// `ev` (may be null) receives three events: before the H kernel, between the
// two kernels, after the E kernel.
int plain_launch_step(const PlainArgs &a, int t, int record, void *stream, void *const *ev);
int plain_launch_flush(const PlainArgs &a, int t_last, void *stream);
int plain_launch_emax(const PlainArgs &a, void *stream);
// Slices of the current state (record layout) into device E[n], H[n], with the
// incident field subtracted inside the total-field region when `scattered`.
int plain_launch_slices(const PlainArgs &a, int scattered, double *E, double *H, void *stream);
int plain_launch_guard(const PlainArgs &a, void *stream);

// omega_p of a parametric trail at every cell, [Nx][Ny][Nz] doubles
// (plain_fp64.cu).  The same formula in FP64 feeds the FP32 form.
void trail_map_fp64(const Problem &P, double *out, void *stream);

}  // namespace mfdtd
