/*
 * fdtd_oracle.c -- CPU restatement of the meteor FDTD time-stepping core.
 *
 * TEST INFRASTRUCTURE ONLY: this file is the parity checker for the GPU engine
 * and the CPU baseline of the benchmark.  The product never links it.
 *
 * It restates source/meteor-fork.cpp (a superset of source/meteor-2.1.cpp) block
 * by block.  Every floating-point expression keeps the reference's expression
 * tree (operand order and parenthesisation), and the file is compiled with
 * -ffp-contract=off, so on one machine it produces bit-identical output files.
 * The OpenMP layout mirrors the reference: the Yee updates and the J update are
 * parallel over the outer index, everything else is serial, and the NTF phase
 * factors are evaluated inline per element, as the reference does, so its time
 * is a faithful stand-in for the reference's.
 *
 * Line references "R21:" are to source/meteor-2.1.cpp, "RFK:" to
 * source/meteor-fork.cpp.
 *
 * Deliberate differences from the reference, none of which changes an output
 * byte on a valid input:
 *   - arrays live on the heap instead of the stack (the reference needs
 *     `ulimit -s unlimited`);
 *   - coordinates y[], z[] beyond index Nx-1 are 0 instead of uninitialised
 *     stack memory (R21:134-138 fills y, z only for i < Nx);
 *   - the source DFT sums Ezdft/Eydft start at 0 (R21:555-556 never
 *     initialises them);
 *   - the debug print of My_front[39][79] (R21:1601-1602) happens only when
 *     that index is inside the array;
 *   - sizes that make the reference divide by zero or index out of bounds are
 *     rejected with an error code.
 */
#include "fdtd_oracle.h"

#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/resource.h>
#include <sys/time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Solver constants, R21:12-18. */
#define OR_PI 3.141592653589793
#define OR_QE 1.602177e-19
#define OR_E0 8.85419e-12
#define OR_U0 1.2566e-6
#define OR_ME 9.10939e-31
#define OR_C 3.0000e8

/* Settings the reference hard-codes (R21:342-343 pmllen 10, R21:413-415 m = 4,
 * kappa = 1, alpha = 0, R21:539-552 TF/SF gap 10 and NTF gap 5).  The optional
 * ext.dat of a run directory (no counterpart in the reference) overrides
 * them; without it every value is the reference's. */
#define OR_MAXPML 32

typedef struct {
    int present, pmllen, tfsf_gap, ntf_gap, oblique, exact_coords, has_wp3, has_nu3, lk_colocated;
    double pml_m, kappa_max, alpha_max, inc_theta, inc_phi, inc_psi;
} or_ext;

typedef struct {
    int dopml, savefields, sourcetype, sourcepol, tsteps, Nx, Ny, Nz;
    int mettype, numfiles, nprobes, nntf, doplate, doB0;
    double f0, fsig, gridfactor, dt, metsize[2], wpmax, numax, metloc[3];
    double metangle, platesize;
    int *probex, *probey, *probez;
    double *fntf;
    double Bx, By, Bz;
    double *wp2, *nu2; /* [Nx][Ny], C order as read */
    or_ext ext;
    double *wp3, *nu3; /* [Nx][Ny][Nz] per-cell maps (extended inputs) or NULL */
    int has_trail;     /* trail.dat: parametric trail (extended input) */
    double trail[10];  /* centre[3], axis[3] (normalised), r0, log10n_lo, log10n_hi, s_half */
} or_in;

static double now_s(void) {
    struct timeval tv;
    gettimeofday(&tv, NULL);
    return (double)tv.tv_sec + 1e-6 * (double)tv.tv_usec;
}

static FILE *open_in(const char *dir, const char *name, const char *mode) {
    char path[4096];
    snprintf(path, sizeof path, "%s/%s", dir, name);
    return fopen(path, mode);
}

static int rd(void *dst, size_t sz, size_t n, FILE *f) {
    return fread(dst, sz, n, f) == n ? 0 : -1;
}

/* inputs.dat, R21:84-112 (+ RFK:115 doB0, absent in MATLAB-written files). */
static int read_inputs(const char *dir, or_in *p) {
    memset(p, 0, sizeof *p);
    FILE *f = open_in(dir, "inputs.dat", "rb");
    if (!f) return -1;
    int e = 0;
    e |= rd(&p->dopml, 4, 1, f);
    e |= rd(&p->savefields, 4, 1, f);
    e |= rd(&p->f0, 8, 1, f);
    e |= rd(&p->fsig, 8, 1, f);
    e |= rd(&p->sourcetype, 4, 1, f);
    e |= rd(&p->sourcepol, 4, 1, f);
    e |= rd(&p->gridfactor, 8, 1, f);
    e |= rd(&p->dt, 8, 1, f);
    e |= rd(&p->tsteps, 4, 1, f);
    e |= rd(&p->Nx, 4, 1, f);
    e |= rd(&p->Ny, 4, 1, f);
    e |= rd(&p->Nz, 4, 1, f);
    e |= rd(p->metsize, 8, 2, f);
    e |= rd(&p->wpmax, 8, 1, f);
    e |= rd(&p->numax, 8, 1, f);
    e |= rd(p->metloc, 8, 3, f);
    e |= rd(&p->metangle, 8, 1, f);
    e |= rd(&p->mettype, 4, 1, f);
    e |= rd(&p->numfiles, 4, 1, f);
    e |= rd(&p->nprobes, 4, 1, f);
    if (e || p->nprobes < 0 || p->nprobes > (1 << 20)) { fclose(f); return -2; }
    size_t np = (size_t)(p->nprobes > 0 ? p->nprobes : 1);
    p->probex = calloc(np, sizeof(int));
    p->probey = calloc(np, sizeof(int));
    p->probez = calloc(np, sizeof(int));
    e |= rd(p->probex, 4, (size_t)p->nprobes, f);
    e |= rd(p->probey, 4, (size_t)p->nprobes, f);
    e |= rd(p->probez, 4, (size_t)p->nprobes, f);
    e |= rd(&p->nntf, 4, 1, f);
    if (e || p->nntf < 1 || p->nntf > 4096) { fclose(f); return -2; }
    p->fntf = calloc((size_t)p->nntf, sizeof(double));
    e |= rd(p->fntf, 8, (size_t)p->nntf, f);
    e |= rd(&p->doplate, 4, 1, f);
    e |= rd(&p->platesize, 8, 1, f);
    if (e) { fclose(f); return -2; }
    if (fread(&p->doB0, 4, 1, f) != 1) p->doB0 = 0; /* MATLAB-written file */
    fclose(f);

    /* ext.dat: magic, 8 int32, 6 doubles (88 bytes). */
    p->ext.pmllen = 10; p->ext.tfsf_gap = 10; p->ext.ntf_gap = 5;
    p->ext.pml_m = 4.0; p->ext.kappa_max = 1.0; p->ext.alpha_max = 0.0;
    p->ext.inc_theta = OR_PI / 2;
    f = open_in(dir, "ext.dat", "rb");
    if (f) {
        char magic[8];
        int32_t iv[8];
        double dv[6];
        if (rd(magic, 1, 8, f) || memcmp(magic, "MFDTDX01", 8) || rd(iv, 4, 8, f) || rd(dv, 8, 6, f)) {
            fclose(f);
            return -2;
        }
        fclose(f);
        or_ext *x = &p->ext;
        x->present = 1;
        x->pmllen = iv[0]; x->tfsf_gap = iv[1]; x->ntf_gap = iv[2]; x->oblique = iv[3];
        x->exact_coords = iv[4]; x->has_wp3 = iv[5]; x->has_nu3 = iv[6]; x->lk_colocated = iv[7];
        x->pml_m = dv[0]; x->kappa_max = dv[1]; x->alpha_max = dv[2];
        x->inc_theta = dv[3]; x->inc_phi = dv[4]; x->inc_psi = dv[5];
        if (x->pmllen < 1 || x->pmllen > OR_MAXPML || x->tfsf_gap < 2 || x->ntf_gap < 1 ||
            x->ntf_gap > x->tfsf_gap - 2)
            return -3;
        int need = 2 * (x->pmllen + x->tfsf_gap) + 3;
        if (p->Nx < need || p->Ny < need || p->Nz < need) return -3;
    }
    {
        const int L = p->ext.pmllen;
        if (p->Nx < 2 * L + 2 || p->Ny < 2 * L + 2 || p->Nz < 2 * L + 2) return -3;
    }
    if (p->tsteps < 1 || p->numfiles < 1 || p->tsteps / p->numfiles < 1) return -3;
    for (int n = 0; n < p->nprobes; n++) {
        if (p->probex[n] < 1 || p->probex[n] >= p->Nx || p->probey[n] < 1 ||
            p->probey[n] >= p->Ny || p->probez[n] < 1 || p->probez[n] >= p->Nz)
            return -3;
    }

    /* B0.dat, RFK:219-224 */
    f = open_in(dir, "B0.dat", "rb");
    if (!f) return -1;
    e |= rd(&p->Bx, 8, 1, f);
    e |= rd(&p->By, 8, 1, f);
    e |= rd(&p->Bz, 8, 1, f);
    fclose(f);
    if (e) return -2;

    /* wp.dat, nu.dat, R21:307-315 */
    size_t n2 = (size_t)p->Nx * (size_t)p->Ny;
    p->wp2 = malloc(n2 * sizeof(double));
    p->nu2 = malloc(n2 * sizeof(double));
    f = open_in(dir, "wp.dat", "rb");
    if (!f) return -1;
    e |= rd(p->wp2, 8, n2, f);
    fclose(f);
    f = open_in(dir, "nu.dat", "rb");
    if (!f) return -1;
    e |= rd(p->nu2, 8, n2, f);
    fclose(f);
    /* trail.dat: magic then 12 doubles */
    f = open_in(dir, "trail.dat", "rb");
    if (f) {
        char magic[8];
        double tv[12];
        if (rd(magic, 1, 8, f) || memcmp(magic, "MFDTDT01", 8) || rd(tv, 8, 12, f)) {
            fclose(f);
            return -2;
        }
        fclose(f);
        double an = sqrt(tv[3] * tv[3] + tv[4] * tv[4] + tv[5] * tv[5]);
        if (!(an > 0) || !(tv[6] > 0) || !(tv[9] > 0)) return -3;
        for (int q = 0; q < 10; q++) p->trail[q] = tv[q];
        for (int q = 3; q < 6; q++) p->trail[q] = tv[q] / an;
        p->has_trail = 1;
    }
    /* per-cell maps announced by ext.dat */
    size_t n3 = n2 * (size_t)p->Nz;
    if (p->ext.has_wp3) {
        p->wp3 = malloc(n3 * sizeof(double));
        f = open_in(dir, "wp3.dat", "rb");
        if (!f) return -1;
        e |= rd(p->wp3, 8, n3, f);
        fclose(f);
    }
    if (p->ext.has_nu3) {
        p->nu3 = malloc(n3 * sizeof(double));
        f = open_in(dir, "nu3.dat", "rb");
        if (!f) return -1;
        e |= rd(p->nu3, 8, n3, f);
        fclose(f);
    }
    return e ? -2 : 0;
}

static void free_inputs(or_in *p) {
    free(p->probex); free(p->probey); free(p->probez);
    free(p->fntf); free(p->wp2); free(p->nu2); free(p->wp3); free(p->nu3);
}

static double *dalloc(size_t n) {
    double *a = calloc(n ? n : 1, sizeof(double));
    if (!a) { fprintf(stderr, "oracle: out of memory (%zu doubles)\n", n); exit(3); }
    return a;
}

/* PML coefficient tables, R21:411-526, with the grading order, kappa_max and
 * alpha_max as parameters (reference: 4, 1, 0).  Index m in [L, 2L) is the
 * high side, the low side mirrors it.  Ke/Kh hold 1/kappa - 1 for the
 * derivative term a kappa != 1 adds to the field update. */
typedef struct {
    double Be[2 * OR_MAXPML], Ae[2 * OR_MAXPML]; /* half-cell grading: E psi  */
    double Bh[2 * OR_MAXPML], Ah[2 * OR_MAXPML]; /* full-cell grading: H psi  */
    double Ke[2 * OR_MAXPML], Kh[2 * OR_MAXPML];
} or_pml;

static void pml_tables(int L, double pmlm, double kamax, double almax, double dx, double dt,
                       or_pml *t) {
    double simax = 1.5 * (double)(pmlm + 1) / (150 * OR_PI * dx);
    double s[OR_MAXPML], sm[OR_MAXPML], ka[OR_MAXPML], kam[OR_MAXPML];
    double al[OR_MAXPML], alm[OR_MAXPML];
    for (int m = 0; m < L; m++) {
        double mf = (double)m;
        s[m] = simax * pow(((mf + 0.5) / L), pmlm);
        sm[m] = simax * pow(((mf + 1) / L), pmlm);
        ka[m] = 1 + (kamax - 1) * pow(((mf + 0.5) / L), pmlm);
        kam[m] = 1 + (kamax - 1) * pow(((mf + 1) / L), pmlm);
        al[m] = almax * pow(((L - mf - 0.5) / L), pmlm);
        alm[m] = almax * pow(((L - mf - 1) / L), pmlm);
    }
    /* The reference computes these tables with E0 for both E and H psi
     * (R21:478-496); the x, y and z tables are identical. */
    for (int m = L; m < 2 * L; m++) {
        int n = m - L;
        t->Be[m] = exp(-((s[n] / ka[n]) + al[n]) * dt / OR_E0);
        t->Ae[m] = s[n] / (s[n] * ka[n] + pow(ka[n], 2) * al[n]) * (t->Be[m] - 1);
        t->Bh[m] = exp(-((sm[n] / kam[n]) + alm[n]) * dt / OR_E0);
        t->Ah[m] = sm[n] / (sm[n] * kam[n] + pow(kam[n], 2) * alm[n]) * (t->Bh[m] - 1);
        t->Ke[m] = 1 / ka[n] - 1;
        t->Kh[m] = 1 / kam[n] - 1;
    }
    for (int m = 0; m < L; m++) {
        t->Be[m] = t->Be[2 * L - 1 - m];
        t->Ae[m] = t->Ae[2 * L - 1 - m];
        t->Bh[m] = t->Bh[2 * L - 1 - m];
        t->Ah[m] = t->Ah[2 * L - 1 - m];
        t->Ke[m] = t->Ke[2 * L - 1 - m];
        t->Kh[m] = t->Kh[2 * L - 1 - m];
    }
}

/* ---- oblique plane-wave incidence (extended inputs; the reference has only
 * the +x line of R21:1278-1304) ----
 * A 1-D auxiliary Yee line along k carries the incident wave.  Its cell size
 * matches the 3-D grid's numerical wavenumber along k at f0 (matched
 * numerical dispersion, Taflove & Hagness ch. 5): both dispersion relations
 * are solved by bisection.  A node with doubled coordinates P sees the line
 * at s = kr . P/2 + s0 (line cells; linear interpolation), E nodes at integer
 * s, H nodes at s + 1/2.  TF/SF corrections are generic: every curl term whose
 * neighbour lies on the other side of the box surface gets the neighbour's
 * incident value, added on the total-field side and subtracted on the
 * scattered-field side. */
typedef struct {
    double ke[3], kh[3], kr[3], s0, dl, d[3];
    int b1[3], b2[3], M, ashift;
} or_obl;

static double yee3_wavenumber(double w, double dt, double c, const double d[3], const double u[3]) {
    const double S = sin(w * dt / 2) / (c * dt);
    const double S2 = S * S;
    double lo = 0.5 * w / c, hi = 4 * w / c;
    for (int it = 0; it < 200; it++) {
        const double mid = 0.5 * (lo + hi);
        double f = 0;
        for (int q = 0; q < 3; q++) {
            const double v = sin(mid * u[q] * d[q] / 2) / d[q];
            f = f + v * v;
        }
        if (f < S2) lo = mid;
        else hi = mid;
    }
    return 0.5 * (lo + hi);
}

static double matched_line_cell(double k, double w, double dt, double c, double dmin, double dmax) {
    const double S = sin(w * dt / 2) / (c * dt);
    double lo = 0.25 * dmin, hi = 2 * dmax;
    for (int it = 0; it < 200; it++) {
        const double mid = 0.5 * (lo + hi);
        if (sin(k * mid / 2) / mid > S) lo = mid;
        else hi = mid;
    }
    return 0.5 * (lo + hi);
}

static int obl_in(const or_obl *o, const int P[3]) {
    for (int q = 0; q < 3; q++)
        if (P[q] < 2 * o->b1[q] || P[q] > 2 * (o->b2[q] - 1)) return 0;
    return 1;
}

static double obl_line(const double *line, double s) {
    double fl = floor(s);
    int n = (int)fl;
    double w = s - fl;
    return line[n] + w * (line[n + 1] - line[n]);
}

/* Incident value of component q at doubled coordinates P: an E component when
 * the neighbour field is E (line = E line), else an H component. */
static double obl_inc(const or_obl *o, int nbr_is_e, int q, const int P[3], const double *line) {
    double s = ((o->kr[0] * (0.5 * P[0]) + o->kr[1] * (0.5 * P[1])) + o->kr[2] * (0.5 * P[2])) + o->s0;
    if (nbr_is_e) return o->ke[q] * obl_line(line, s);
    return o->kh[q] * obl_line(line, s - 0.5);
}

/* TF/SF correction of component c of the target field (E when is_e) at cell
 * (i,j,k).  Returns 1 and sets *corr when some curl-term neighbour lies on
 * the other side of the box surface; the caller then adds c2 * corr.  `line`
 * is the auxiliary line of the neighbour field (H line for E targets). */
static int obl_corr(const or_obl *o, int is_e, int c, int i, int j, int k, const double *line,
                    double *corr) {
    int P[3] = {2 * i, 2 * j, 2 * k};
    /* a target of either field is offset by half a cell along the axes other
     * than its own component for H, along its own component for E */
    for (int q = 0; q < 3; q++)
        if (is_e ? q == c : q != c) P[q] += 1;
    const int T = obl_in(o, P);
    const int ax[2] = {(c + 1) % 3, (c + 2) % 3};
    const int comp[2] = {(c + 2) % 3, (c + 1) % 3};
    const int sg[2] = {is_e ? 1 : -1, is_e ? -1 : 1};
    double acc = 0;
    int any = 0;
    for (int term = 0; term < 2; term++)
        for (int side = 1; side >= -1; side -= 2) {
            int Q[3] = {P[0], P[1], P[2]};
            Q[ax[term]] += side;
            const int Tn = obl_in(o, Q);
            if (Tn == T) continue;
            const double v = obl_inc(o, !is_e, comp[term], Q, line) / o->d[ax[term]];
            if (sg[term] * side * (T - Tn) > 0) acc = acc + v;
            else acc = acc - v;
            any = 1;
        }
    *corr = acc;
    return any;
}

static void write_all(FILE *f, const double *a, size_t n) {
    if (n) fwrite(a, sizeof(double), n, f);
}

int oracle_run_dir(const char *dir, int max_steps, int nthreads, int mirror_dead_work,
                   double *loop_seconds) {
    double tStart = now_s();
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    or_in in;
    int rc = read_inputs(dir, &in);
    if (rc) { free_inputs(&in); return rc; }

    const int Nx = in.Nx, Ny = in.Ny, Nz = in.Nz, tsteps = in.tsteps, nntf = in.nntf;
    const int L = in.ext.pmllen;
    const int obl = in.ext.oblique != 0;
    const int kappa_on = in.dopml && in.ext.kappa_max != 1.0;
    const double dt = in.dt;
    const size_t NC = (size_t)Nx * Ny * Nz;
#define I3(i, j, k) ((((size_t)(i)) * Ny + (size_t)(j)) * Nz + (size_t)(k))

    /* Grid, R21:116-138.  dx = dy = dz.  Coordinates use integer (N-1)/2 and
     * are filled for index < Nx only (see header note). */
    double lambda = OR_C / in.f0;
    double dx = lambda / in.gridfactor, dy = lambda / in.gridfactor, dz = lambda / in.gridfactor;
    int nmax = Nx > Ny ? Nx : Ny;
    if (Nz > nmax) nmax = Nz;
    double *x = dalloc((size_t)nmax), *y = dalloc((size_t)nmax), *z = dalloc((size_t)nmax);
    if (in.ext.exact_coords) { /* extended input: every axis, real division */
        for (int i = 0; i < Nx; i++) x[i] = -(Nx - 1) / 2.0 * dx + dx * i;
        for (int i = 0; i < Ny; i++) y[i] = -(Ny - 1) / 2.0 * dy + dy * i;
        for (int i = 0; i < Nz; i++) z[i] = -(Nz - 1) / 2.0 * dz + dz * i;
    } else {
        for (int i = 0; i < Nx; i++) {
            x[i] = -(Nx - 1) / 2 * dx + dx * i;
            if (i < nmax) y[i] = -(Ny - 1) / 2 * dy + dy * i;
            if (i < nmax) z[i] = -(Nz - 1) / 2 * dz + dz * i;
        }
    }
    const int ssx = (Nx + 1) / 2, ssy = (Ny + 1) / 2, ssz = (Nz + 1) / 2;

    /* Source waveforms, R21:152-175. */
    double *EsA = dalloc((size_t)tsteps), *EsB = dalloc((size_t)tsteps);
    {
        double f0 = in.f0, fsig = in.fsig;
        double rdelayA = 1.6 * sqrt(6) / OR_PI / f0;
        double rdelayB = (1.6 + 1 / sqrt(3)) * sqrt(6) / OR_PI / f0;
        const double PI = OR_PI;
        for (int t = 0; t < tsteps; t++) {
            if (in.sourcetype == 2) {
                EsA[t] = sin(2 * PI * f0 * (t - 3 * fsig) * dt) * exp(-(t - 3 * fsig) * (t - 3 * fsig) / (2 * fsig * fsig));
                EsB[t] = cos(2 * PI * f0 * (t - 3 * fsig) * dt) * exp(-(t - 3 * fsig) * (t - 3 * fsig) / (2 * fsig * fsig));
            } else if (in.sourcetype == 3) {
                EsA[t] = (1 - 2 * PI * PI * f0 * f0 * (t * dt - rdelayA) * (t * dt - rdelayA)) * exp(-PI * PI * f0 * f0 * (t * dt - rdelayA) * (t * dt - rdelayA));
                EsB[t] = (1 - 2 * PI * PI * f0 * f0 * (t * dt - rdelayB) * (t * dt - rdelayB)) * exp(-PI * PI * f0 * f0 * (t * dt - rdelayB) * (t * dt - rdelayB));
            } else { /* 1 and any other value: sinusoid */
                EsA[t] = sin(2 * PI * f0 * t * dt);
                EsB[t] = cos(2 * PI * f0 * t * dt);
            }
        }
    }

    /* Update coefficients, R21:180-210. */
    const double sigm = 0, sig = 0;
    const double c1h = (2 * OR_U0 - sigm * dt) / (2 * OR_U0 + sigm * dt);
    const double c2h = 2 * dt / (2 * OR_U0 + sigm * dt);
    const double c1e0 = (2 * OR_E0 - sig * dt) / (2 * OR_E0 + sig * dt);
    const double c2e0 = 2 * dt / (2 * OR_E0 + sig * dt);
    double *c1e = dalloc(NC), *c2e = dalloc(NC);
    const double c1s = (2 * OR_E0 - 1e7 * dt) / (2 * OR_E0 + 1e7 * dt);
    const double c2s = 2 * dt / (2 * OR_E0 + 1e7 * dt);
    for (int i = 0; i < Nx; i++)
        for (int j = 0; j < Ny; j++)
            for (int k = 0; k < Nz; k++) {
                size_t c = I3(i, j, k);
                c1e[c] = c1e0;
                c2e[c] = c2e0;
                if (in.doplate == 2) {
                    double dist = sqrt(x[i] * x[i] + y[j] * y[j] + z[k] * z[k]);
                    if (dist < in.platesize) { c1e[c] = c1s; c2e[c] = c2s; }
                }
            }

    /* Gyrofrequency, RFK:226-232. */
    const double wcex = -OR_QE * in.Bx / OR_ME;
    const double wcey = -OR_QE * in.By / OR_ME;
    const double wcez = -OR_QE * in.Bz / OR_ME;
    const double wce0 = sqrt(wcex * wcex + wcey * wcey + wcez * wcez);

    /* Fields (zero), R21:217-293. */
    double *Ex = dalloc(NC), *Ey = dalloc(NC), *Ez = dalloc(NC);
    double *Hx = dalloc(NC), *Hy = dalloc(NC), *Hz = dalloc(NC);
    double *Jx = dalloc(NC), *Jy = dalloc(NC), *Jz = dalloc(NC);
    double *Eyinc = dalloc((size_t)Nx), *Ezinc = dalloc((size_t)Nx);
    double *Hyinc = dalloc((size_t)Nx), *Hzinc = dalloc((size_t)Nx);
    const int np = in.nprobes;
    double *Prb[6];
    for (int q = 0; q < 6; q++) Prb[q] = dalloc((size_t)tsteps * (size_t)(np > 0 ? np : 1));
    double *Emag = mirror_dead_work ? dalloc(NC) : NULL;
    double *Smag = mirror_dead_work ? dalloc(NC) : NULL;

    /* Slices, R21:282-290: [2][Nx][Ny], [2][Nx][Nz], [2][Ny][Nz]. */
    const size_t szz = 2 * (size_t)Nx * Ny, szy = 2 * (size_t)Nx * Nz, szx = 2 * (size_t)Ny * Nz;
    double *ESz = dalloc(szz), *ESy = dalloc(szy), *ESx = dalloc(szx);
    double *HSz = dalloc(szz), *HSy = dalloc(szy), *HSx = dalloc(szx);
    double *JSz = dalloc(szz), *JSy = dalloc(szy), *JSx = dalloc(szx); /* never assigned */

    /* Plasma maps, R21:301-334. */
    double *wpe = dalloc(NC), *nue = dalloc(NC);
    {
        double msig0 = in.metsize[0];
        if (!in.doplate) {
            for (int i = 0; i < Nx; i++)
                for (int j = 0; j < Ny; j++)
                    for (int k = 0; k < Nz; k++) {
                        size_t c = I3(i, j, k);
                        wpe[c] = in.wp2[(size_t)i * Ny + j] * exp(-pow((z[k] - in.metloc[2]), 2) / (msig0 * msig0));
                        nue[c] = in.nu2[(size_t)i * Ny + j] * exp(-pow((z[k] - in.metloc[2]), 2) / (msig0 * msig0));
                        if (in.wp3) wpe[c] = in.wp3[c]; /* per-cell maps (extended inputs) */
                        if (in.has_trail) { /* parametric trail, exact cell coordinates */
                            const double *T = in.trail;
                            const double px = -(Nx - 1) / 2.0 * dx + dx * i - T[0];
                            const double py = -(Ny - 1) / 2.0 * dy + dy * j - T[1];
                            const double pz = -(Nz - 1) / 2.0 * dz + dz * k - T[2];
                            const double sa = px * T[3] + py * T[4] + pz * T[5];
                            double d2 = px * px + py * py + pz * pz - sa * sa;
                            if (d2 < 0) d2 = 0;
                            double fr = (sa + T[9]) / (2 * T[9]);
                            fr = fr < 0 ? 0 : (fr > 1 ? 1 : fr);
                            const double n = pow(10.0, T[7] + (T[8] - T[7]) * fr) * exp(-d2 / (T[6] * T[6]));
                            wpe[c] = sqrt(n * OR_QE * OR_QE / (OR_E0 * OR_ME));
                        }
                        if (in.nu3) nue[c] = in.nu3[c];
                    }
        }
    }

    /* CPML, R21:342-535. */
    or_pml T;
    memset(&T, 0, sizeof T);
    if (in.dopml)
        pml_tables(L, in.ext.pml_m, in.ext.kappa_max, in.ext.alpha_max, dx, dt, &T);
    const int xshift = Nx - 2 * L - 1, yshift = Ny - 2 * L - 1, zshift = Nz - 2 * L - 1;
    /* psi slabs: x-normal [2L][Ny][Nz], y-normal [Nx][2L][Nz], z-normal [Nx][Ny][2L] */
    const size_t nxs = (size_t)2 * L * Ny * Nz, nys = (size_t)Nx * 2 * L * Nz, nzs = (size_t)Nx * Ny * 2 * L;
    double *P_hxy = dalloc(nys), *P_hxz = dalloc(nzs), *P_hyx = dalloc(nxs);
    double *P_hyz = dalloc(nzs), *P_hzx = dalloc(nxs), *P_hzy = dalloc(nys);
    double *P_exy = dalloc(nys), *P_exz = dalloc(nzs), *P_eyx = dalloc(nxs);
    double *P_eyz = dalloc(nzs), *P_ezx = dalloc(nxs), *P_ezy = dalloc(nys);
    double P_eyxI[2 * OR_MAXPML] = {0}, P_ezxI[2 * OR_MAXPML] = {0};
    double P_hyxI[2 * OR_MAXPML] = {0}, P_hzxI[2 * OR_MAXPML] = {0};
#define PX(i, j, k) ((((size_t)(i)) * Ny + (size_t)(j)) * Nz + (size_t)(k))        /* [2L][Ny][Nz] */
#define PY(i, j, k) ((((size_t)(i)) * (2 * L) + (size_t)(j)) * Nz + (size_t)(k))   /* [Nx][2L][Nz] */
#define PZ(i, j, k) ((((size_t)(i)) * Ny + (size_t)(j)) * (2 * L) + (size_t)(k))   /* [Nx][Ny][2L] */
    const double *Bh = T.Bh, *Ah = T.Ah, *Be = T.Be, *Ae = T.Ae, *Ke = T.Ke, *Kh = T.Kh;
    /* A CPML correction with kappa != 1 also carries (1/kappa - 1) times the
     * derivative the psi recursion uses (extended inputs). */
#define KAP(p, K, s, diff, d) (kappa_on ? (p) + (K)[s] * (diff) / (d) : (p))

    /* TF/SF box and NTF surface, R21:539-552. */
    const int gap = in.ext.tfsf_gap;
    const int bx1 = L + gap, bx2 = Nx - L - gap;
    const int by1 = L + gap, by2 = Ny - L - gap;
    const int bz1 = L + gap, bz2 = Nz - L - gap;
    int ntfb = L + in.ext.ntf_gap;

    /* Oblique incidence set-up (extended inputs).  E1d lives in Ezinc and H1d
     * in Hyinc, which then hold M nodes; Eyinc and Hzinc stay zero. */
    or_obl O;
    memset(&O, 0, sizeof O);
    or_pml T1;
    memset(&T1, 0, sizeof T1);
    double P_e1[2 * OR_MAXPML] = {0}, P_h1[2 * OR_MAXPML] = {0};
    if (obl) {
        const double th = in.ext.inc_theta, ph = in.ext.inc_phi, ps = in.ext.inc_psi;
        double kk[3] = {sin(th) * cos(ph), sin(th) * sin(ph), cos(th)};
        const double tht[3] = {cos(th) * cos(ph), cos(th) * sin(ph), -sin(th)};
        const double phh[3] = {-sin(ph), cos(ph), 0.0};
        for (int q = 0; q < 3; q++) O.ke[q] = cos(ps) * (-tht[q]) + sin(ps) * phh[q];
        O.kh[0] = kk[1] * O.ke[2] - kk[2] * O.ke[1];
        O.kh[1] = kk[2] * O.ke[0] - kk[0] * O.ke[2];
        O.kh[2] = kk[0] * O.ke[1] - kk[1] * O.ke[0];
        const double cl = 1 / sqrt(OR_U0 * OR_E0);
        O.d[0] = dx; O.d[1] = dy; O.d[2] = dz;
        const double w = 2 * OR_PI * in.f0;
        const double k3 = yee3_wavenumber(w, dt, cl, O.d, kk);
        double dmin = dx < dy ? dx : dy, dmax = dx > dy ? dx : dy;
        if (dz < dmin) dmin = dz;
        if (dz > dmax) dmax = dz;
        O.dl = matched_line_cell(k3, w, dt, cl, dmin, dmax);
        if (!(cl * dt < O.dl)) { free_inputs(&in); return -3; }
        for (int q = 0; q < 3; q++) O.kr[q] = kk[q] * O.d[q] / O.dl;
        /* line node 0 at the grid corner the wave enters first: a wave along +x
         * sees the line at s = x index, like the reference's line */
        const int gx[2] = {0, Nx - 1}, gy[2] = {0, Ny - 1}, gz[2] = {0, Nz - 1};
        const int cx[2] = {bx1 - 1, bx2}, cy[2] = {by1 - 1, by2}, cz[2] = {bz1 - 1, bz2};
        double gmin = 1e300, pmax = -1e300;
        for (int a = 0; a < 2; a++)
            for (int b = 0; b < 2; b++)
                for (int e = 0; e < 2; e++) {
                    const double g = O.kr[0] * gx[a] + O.kr[1] * gy[b] + O.kr[2] * gz[e];
                    const double pp = O.kr[0] * cx[a] + O.kr[1] * cy[b] + O.kr[2] * cz[e];
                    if (g < gmin) gmin = g;
                    if (pp > pmax) pmax = pp;
                }
        O.s0 = -gmin;
        O.M = (int)ceil(pmax + O.s0) + 6 + L;
        O.ashift = O.M - 2 * L - 1;
        {   /* the shell's line positions must sit inside the line */
            double smin = 1e300, smax = -1e300;
            for (int a = 0; a < 2; a++)
                for (int b = 0; b < 2; b++)
                    for (int e = 0; e < 2; e++) {
                        const double sc = O.kr[0] * cx[a] + O.kr[1] * cy[b] + O.kr[2] * cz[e] + O.s0;
                        if (sc < smin) smin = sc;
                        if (sc > smax) smax = sc;
                    }
            if (!(smin >= 1.0) || !(smax + 3 <= O.M - L - 2)) { free_inputs(&in); return -3; }
        }
        O.b1[0] = bx1; O.b1[1] = by1; O.b1[2] = bz1;
        O.b2[0] = bx2; O.b2[1] = by2; O.b2[2] = bz2;
        pml_tables(L, in.ext.pml_m, 1.0, 0.0, O.dl, dt, &T1);
        if (O.M > Nx) { /* the line outgrows the reference's Nx-node arrays */
            free(Ezinc); free(Hyinc);
            Ezinc = dalloc((size_t)O.M); Hyinc = dalloc((size_t)O.M);
        }
    }
    /* the shell of cells that can carry a TF/SF correction */
#define SHELL(i, j, k) ((i) >= bx1 - 1 && (i) <= bx2 && (j) >= by1 - 1 && (j) <= by2 && \
                        (k) >= bz1 - 1 && (k) <= bz2 &&                                \
                        !((i) > bx1 && (i) < bx2 - 2 && (j) > by1 && (j) < by2 - 2 &&    \
                          (k) > bz1 && (k) < bz2 - 2))
    /* next k of the shell scan: inside an interior (i,j) column the run
     * bz1+1 .. bz2-3 holds no crossing and is skipped */
#define SHELL_NEXT(i, j, k) (((i) > bx1 && (i) < bx2 - 2 && (j) > by1 && (j) < by2 - 2 && \
                              (k) == bz1) ? bz2 - 2 : (k) + 1)

    /* NTF running sums, R21:558-610. */
    double *Ezdft = dalloc(2 * (size_t)nntf), *Eydft = dalloc(2 * (size_t)nntf);
    const size_t fbn = (size_t)Ny * Nz * 2 * nntf, tbn = (size_t)Nx * Nz * 2 * nntf, lrn = (size_t)Nx * Ny * 2 * nntf;
    double *My_front = dalloc(fbn), *Mz_front = dalloc(fbn), *Jy_front = dalloc(fbn), *Jz_front = dalloc(fbn);
    double *My_back = dalloc(fbn), *Mz_back = dalloc(fbn), *Jy_back = dalloc(fbn), *Jz_back = dalloc(fbn);
    double *Mx_top = dalloc(tbn), *Mz_top = dalloc(tbn), *Jx_top = dalloc(tbn), *Jz_top = dalloc(tbn);
    double *Mx_bot = dalloc(tbn), *Mz_bot = dalloc(tbn), *Jx_bot = dalloc(tbn), *Jz_bot = dalloc(tbn);
    double *Mx_left = dalloc(lrn), *My_left = dalloc(lrn), *Jx_left = dalloc(lrn), *Jy_left = dalloc(lrn);
    double *Mx_right = dalloc(lrn), *My_right = dalloc(lrn), *Jx_right = dalloc(lrn), *Jy_right = dalloc(lrn);
#define F2(a, b, nb, m) ((((size_t)(a)) * (nb) + (size_t)(b)) * (2 * (size_t)nntf) + (size_t)(m))

    /* log.txt header, R21:619-643. */
    FILE *lg = open_in(dir, "log.txt", "w");
    {
        struct rusage ru;
        getrusage(RUSAGE_SELF, &ru);
        double memusage = (double)ru.ru_maxrss / 1024 / 1024;
        if (lg) {
            fprintf(lg, "------------------------------------------\n");
            fprintf(lg, "3D Meteor Scattering Simulation\n");
            fprintf(lg, "------------------------------------------\n");
            fprintf(lg, "dx = %g\n", dx);
            fprintf(lg, "source type = %d\n", in.sourcetype);
            fprintf(lg, "source polarization = %d\n", in.sourcepol);
            fprintf(lg, "Time step = %g\n", dt);
            fprintf(lg, "Total time steps = %d\n", tsteps);
            fprintf(lg, "Total NTF frequencies = %d\n", nntf);
            fprintf(lg, "last NTF frequency = %g\n", in.fntf[nntf - 1]);
            fprintf(lg, "Total memory usage = %g GB\n", memusage);
            fclose(lg);
        }
    }

    const double PI = OR_PI;
    const double *fntf = in.fntf;
    const int nsteps = (max_steps >= 0 && max_steps < tsteps) ? max_steps : tsteps;
    const int rec_period = tsteps / in.numfiles;
    double tloopStart = now_s();

    for (int t = 0; t < nsteps; t++) {
        /* ---------------- H psi, R21:656-760 ---------------- */
        if (in.dopml) {
            for (int i = 0; i < Nx; i++) {
                for (int j = 0; j < L; j++)
                    for (int k = 0; k < Nz - 1; k++)
                        P_hxy[PY(i, j, k)] = Bh[j] * P_hxy[PY(i, j, k)] + Ah[j] * (Ez[I3(i, j + 1, k)] - Ez[I3(i, j, k)]) / dy;
                for (int j = Ny - L - 1; j < Ny - 1; j++)
                    for (int k = 0; k < Nz - 1; k++)
                        P_hxy[PY(i, j - yshift, k)] = Bh[j - yshift] * P_hxy[PY(i, j - yshift, k)] + Ah[j - yshift] * (Ez[I3(i, j + 1, k)] - Ez[I3(i, j, k)]) / dy;
            }
            for (int i = 0; i < Nx; i++)
                for (int j = 0; j < Ny - 1; j++) {
                    for (int k = 0; k < L; k++)
                        P_hxz[PZ(i, j, k)] = Bh[k] * P_hxz[PZ(i, j, k)] + Ah[k] * (Ey[I3(i, j, k + 1)] - Ey[I3(i, j, k)]) / dz;
                    for (int k = Nz - L - 1; k < Nz - 1; k++)
                        P_hxz[PZ(i, j, k - zshift)] = Bh[k - zshift] * P_hxz[PZ(i, j, k - zshift)] + Ah[k - zshift] * (Ey[I3(i, j, k + 1)] - Ey[I3(i, j, k)]) / dz;
                }
            for (int i = 0; i < L; i++)
                for (int j = 0; j < Ny; j++)
                    for (int k = 0; k < Nz - 1; k++)
                        P_hyx[PX(i, j, k)] = Bh[i] * P_hyx[PX(i, j, k)] + Ah[i] * (Ez[I3(i + 1, j, k)] - Ez[I3(i, j, k)]) / dx;
            for (int i = Nx - L - 1; i < Nx - 1; i++) {
                for (int j = 0; j < Ny; j++)
                    for (int k = 0; k < Nz - 1; k++)
                        P_hyx[PX(i - xshift, j, k)] = Bh[i - xshift] * P_hyx[PX(i - xshift, j, k)] + Ah[i - xshift] * (Ez[I3(i + 1, j, k)] - Ez[I3(i, j, k)]) / dx;
                if (!obl) P_hyxI[i - xshift] = Bh[i - xshift] * P_hyxI[i - xshift] + Ah[i - xshift] * (Ezinc[i + 1] - Ezinc[i]) / dx;
            }
            for (int i = 0; i < Nx - 1; i++)
                for (int j = 0; j < Ny; j++) {
                    for (int k = 0; k < L; k++)
                        P_hyz[PZ(i, j, k)] = Bh[k] * P_hyz[PZ(i, j, k)] + Ah[k] * (Ex[I3(i, j, k + 1)] - Ex[I3(i, j, k)]) / dz;
                    for (int k = Nz - L - 1; k < Nz - 1; k++)
                        P_hyz[PZ(i, j, k - zshift)] = Bh[k - zshift] * P_hyz[PZ(i, j, k - zshift)] + Ah[k - zshift] * (Ex[I3(i, j, k + 1)] - Ex[I3(i, j, k)]) / dz;
                }
            for (int i = 0; i < L; i++)
                for (int j = 0; j < Ny - 1; j++)
                    for (int k = 0; k < Nz; k++)
                        P_hzx[PX(i, j, k)] = Bh[i] * P_hzx[PX(i, j, k)] + Ah[i] * (Ey[I3(i + 1, j, k)] - Ey[I3(i, j, k)]) / dx;
            for (int i = Nx - L - 1; i < Nx - 1; i++) {
                for (int j = 0; j < Ny - 1; j++)
                    for (int k = 0; k < Nz; k++)
                        P_hzx[PX(i - xshift, j, k)] = Bh[i - xshift] * P_hzx[PX(i - xshift, j, k)] + Ah[i - xshift] * (Ey[I3(i + 1, j, k)] - Ey[I3(i, j, k)]) / dx;
                if (!obl) P_hzxI[i - xshift] = Bh[i - xshift] * P_hzxI[i - xshift] + Ah[i - xshift] * (Eyinc[i + 1] - Eyinc[i]) / dx;
            }
            for (int i = 0; i < Nx - 1; i++) {
                for (int j = 0; j < L; j++)
                    for (int k = 0; k < Nz; k++)
                        P_hzy[PY(i, j, k)] = Bh[j] * P_hzy[PY(i, j, k)] + Ah[j] * (Ex[I3(i, j + 1, k)] - Ex[I3(i, j, k)]) / dy;
                for (int j = Ny - L - 1; j < Ny - 1; j++)
                    for (int k = 0; k < Nz; k++)
                        P_hzy[PY(i, j - yshift, k)] = Bh[j - yshift] * P_hzy[PY(i, j - yshift, k)] + Ah[j - yshift] * (Ex[I3(i, j + 1, k)] - Ex[I3(i, j, k)]) / dy;
            }
        }

        /* ---------------- Hx, R21:766-819 ---------------- */
#pragma omp parallel for
        for (int i = 0; i < Nx; i++)
            for (int j = 0; j < Ny - 1; j++)
                for (int k = 0; k < Nz - 1; k++)
                    Hx[I3(i, j, k)] = c1h * Hx[I3(i, j, k)] - c2h * ((Ez[I3(i, j + 1, k)] - Ez[I3(i, j, k)]) / dy - (Ey[I3(i, j, k + 1)] - Ey[I3(i, j, k)]) / dz);
        if (!obl) {
            for (int i = bx1; i < bx2; i++)
                for (int k = bz1; k < bz2; k++) {
                    Hx[I3(i, by1 - 1, k)] = Hx[I3(i, by1 - 1, k)] + c2h * Ezinc[i] / dy;
                    Hx[I3(i, by2 - 1, k)] = Hx[I3(i, by2 - 1, k)] - c2h * Ezinc[i] / dy;
                }
            for (int i = bx1; i < bx2; i++)
                for (int j = by1; j < by2; j++) {
                    Hx[I3(i, j, bz1 - 1)] = Hx[I3(i, j, bz1 - 1)] - c2h * Eyinc[i] / dz;
                    Hx[I3(i, j, bz2 - 1)] = Hx[I3(i, j, bz2 - 1)] + c2h * Eyinc[i] / dz;
                }
        } else {
            for (int i = bx1 - 1; i <= bx2; i++)
                for (int j = by1 - 1; j <= by2; j++)
                    for (int k = bz1 - 1; k <= bz2; k = SHELL_NEXT(i, j, k)) {
                        double corr;
                        if (SHELL(i, j, k) && obl_corr(&O, 0, 0, i, j, k, Ezinc, &corr))
                            Hx[I3(i, j, k)] = Hx[I3(i, j, k)] + c2h * corr;
                    }
        }
        if (in.dopml) {
            for (int i = 0; i < Nx; i++) {
                for (int j = 0; j < L; j++)
                    for (int k = 0; k < Nz - 1; k++)
                        Hx[I3(i, j, k)] = Hx[I3(i, j, k)] - c2h * KAP(P_hxy[PY(i, j, k)], Kh, j, Ez[I3(i, j + 1, k)] - Ez[I3(i, j, k)], dy);
                for (int j = Ny - L - 1; j < Ny - 1; j++)
                    for (int k = 0; k < Nz - 1; k++)
                        Hx[I3(i, j, k)] = Hx[I3(i, j, k)] - c2h * KAP(P_hxy[PY(i, j - yshift, k)], Kh, j - yshift, Ez[I3(i, j + 1, k)] - Ez[I3(i, j, k)], dy);
            }
            for (int i = 0; i < Nx; i++)
                for (int j = 0; j < Ny - 1; j++) {
                    for (int k = 0; k < L; k++)
                        Hx[I3(i, j, k)] = Hx[I3(i, j, k)] + c2h * KAP(P_hxz[PZ(i, j, k)], Kh, k, Ey[I3(i, j, k + 1)] - Ey[I3(i, j, k)], dz);
                    for (int k = Nz - L - 1; k < Nz - 1; k++)
                        Hx[I3(i, j, k)] = Hx[I3(i, j, k)] + c2h * KAP(P_hxz[PZ(i, j, k - zshift)], Kh, k - zshift, Ey[I3(i, j, k + 1)] - Ey[I3(i, j, k)], dz);
                }
        }

        /* ---------------- Hy, R21:823-877 ---------------- */
#pragma omp parallel for
        for (int i = 0; i < Nx - 1; i++) {
            for (int j = 0; j < Ny; j++)
                for (int k = 0; k < Nz - 1; k++)
                    Hy[I3(i, j, k)] = c1h * Hy[I3(i, j, k)] - c2h * ((Ex[I3(i, j, k + 1)] - Ex[I3(i, j, k)]) / dz - (Ez[I3(i + 1, j, k)] - Ez[I3(i, j, k)]) / dx);
            if (!obl) Hyinc[i] = c1h * Hyinc[i] + c2h * (Ezinc[i + 1] - Ezinc[i]) / dx;
        }
        if (!obl) {
            for (int j = by1; j < by2; j++)
                for (int k = bz1; k < bz2; k++) {
                    Hy[I3(bx1 - 1, j, k)] = Hy[I3(bx1 - 1, j, k)] - c2h * Ezinc[bx1] / dx;
                    Hy[I3(bx2 - 1, j, k)] = Hy[I3(bx2 - 1, j, k)] + c2h * Ezinc[bx2 - 1] / dx;
                }
        } else {
            for (int i = bx1 - 1; i <= bx2; i++)
                for (int j = by1 - 1; j <= by2; j++)
                    for (int k = bz1 - 1; k <= bz2; k = SHELL_NEXT(i, j, k)) {
                        double corr;
                        if (SHELL(i, j, k) && obl_corr(&O, 0, 1, i, j, k, Ezinc, &corr))
                            Hy[I3(i, j, k)] = Hy[I3(i, j, k)] + c2h * corr;
                    }
        }
        if (in.dopml) {
            for (int i = 0; i < L; i++)
                for (int j = 0; j < Ny; j++)
                    for (int k = 0; k < Nz - 1; k++)
                        Hy[I3(i, j, k)] = Hy[I3(i, j, k)] + c2h * KAP(P_hyx[PX(i, j, k)], Kh, i, Ez[I3(i + 1, j, k)] - Ez[I3(i, j, k)], dx);
            for (int i = Nx - L - 1; i < Nx - 1; i++) {
                for (int j = 0; j < Ny; j++)
                    for (int k = 0; k < Nz - 1; k++)
                        Hy[I3(i, j, k)] = Hy[I3(i, j, k)] + c2h * KAP(P_hyx[PX(i - xshift, j, k)], Kh, i - xshift, Ez[I3(i + 1, j, k)] - Ez[I3(i, j, k)], dx);
                if (!obl) Hyinc[i] = Hyinc[i] + c2h * P_hyxI[i - xshift];
            }
            for (int i = 0; i < Nx - 1; i++)
                for (int j = 0; j < Ny; j++) {
                    for (int k = 0; k < L; k++)
                        Hy[I3(i, j, k)] = Hy[I3(i, j, k)] - c2h * KAP(P_hyz[PZ(i, j, k)], Kh, k, Ex[I3(i, j, k + 1)] - Ex[I3(i, j, k)], dz);
                    for (int k = Nz - L - 1; k < Nz - 1; k++)
                        Hy[I3(i, j, k)] = Hy[I3(i, j, k)] - c2h * KAP(P_hyz[PZ(i, j, k - zshift)], Kh, k - zshift, Ex[I3(i, j, k + 1)] - Ex[I3(i, j, k)], dz);
                }
        }

        /* ---------------- Hz, R21:882-937 ---------------- */
#pragma omp parallel for
        for (int i = 0; i < Nx - 1; i++) {
            for (int j = 0; j < Ny - 1; j++)
                for (int k = 0; k < Nz; k++)
                    Hz[I3(i, j, k)] = c1h * Hz[I3(i, j, k)] - c2h * ((Ey[I3(i + 1, j, k)] - Ey[I3(i, j, k)]) / dx - (Ex[I3(i, j + 1, k)] - Ex[I3(i, j, k)]) / dy);
            if (!obl) Hzinc[i] = c1h * Hzinc[i] - c2h * (Eyinc[i + 1] - Eyinc[i]) / dx;
        }
        if (!obl) {
            for (int j = by1; j < by2; j++)
                for (int k = bz1; k < bz2; k++) {
                    Hz[I3(bx1 - 1, j, k)] = Hz[I3(bx1 - 1, j, k)] + c2h * Eyinc[bx1] / dx;
                    Hz[I3(bx2 - 1, j, k)] = Hz[I3(bx2 - 1, j, k)] - c2h * Eyinc[bx2 - 1] / dx;
                }
        } else {
            for (int i = bx1 - 1; i <= bx2; i++)
                for (int j = by1 - 1; j <= by2; j++)
                    for (int k = bz1 - 1; k <= bz2; k = SHELL_NEXT(i, j, k)) {
                        double corr;
                        if (SHELL(i, j, k) && obl_corr(&O, 0, 2, i, j, k, Ezinc, &corr))
                            Hz[I3(i, j, k)] = Hz[I3(i, j, k)] + c2h * corr;
                    }
        }
        if (in.dopml) {
            for (int i = 0; i < L; i++)
                for (int j = 0; j < Ny - 1; j++)
                    for (int k = 0; k < Nz; k++)
                        Hz[I3(i, j, k)] = Hz[I3(i, j, k)] - c2h * KAP(P_hzx[PX(i, j, k)], Kh, i, Ey[I3(i + 1, j, k)] - Ey[I3(i, j, k)], dx);
            for (int i = Nx - L - 1; i < Nx - 1; i++) {
                for (int j = 0; j < Ny - 1; j++)
                    for (int k = 0; k < Nz; k++)
                        Hz[I3(i, j, k)] = Hz[I3(i, j, k)] - c2h * KAP(P_hzx[PX(i - xshift, j, k)], Kh, i - xshift, Ey[I3(i + 1, j, k)] - Ey[I3(i, j, k)], dx);
                if (!obl) Hzinc[i] = Hzinc[i] - c2h * P_hzxI[i - xshift];
            }
            for (int i = 0; i < Nx - 1; i++) {
                for (int j = 0; j < L; j++)
                    for (int k = 0; k < Nz; k++)
                        Hz[I3(i, j, k)] = Hz[I3(i, j, k)] + c2h * KAP(P_hzy[PY(i, j, k)], Kh, j, Ex[I3(i, j + 1, k)] - Ex[I3(i, j, k)], dy);
                for (int j = Ny - L - 1; j < Ny - 1; j++)
                    for (int k = 0; k < Nz; k++)
                        Hz[I3(i, j, k)] = Hz[I3(i, j, k)] + c2h * KAP(P_hzy[PY(i, j - yshift, k)], Kh, j - yshift, Ex[I3(i, j + 1, k)] - Ex[I3(i, j, k)], dy);
            }
        }

        /* ---------------- auxiliary line, H part (oblique incidence) ------ */
        if (obl) {
            const int M = O.M;
            for (int n = 0; n < M - 1; n++) {
                double h = c1h * Hyinc[n] - c2h * (Ezinc[n + 1] - Ezinc[n]) / O.dl;
                if (n >= M - L - 1) {
                    const int sidx = n - O.ashift;
                    P_h1[sidx] = T1.Bh[sidx] * P_h1[sidx] + T1.Ah[sidx] * (Ezinc[n + 1] - Ezinc[n]) / O.dl;
                    h = h - c2h * P_h1[sidx];
                }
                Hyinc[n] = h;
            }
        }

        /* ---------------- NTF, H part, R21:942-992 ---------------- */
        for (int j = 0; j < Ny; j++)
            for (int k = 0; k < Nz; k++)
                for (int m = 0; m < nntf; m++) {
                    double s = sin(2 * PI * fntf[m] * t * dt), c = cos(2 * PI * fntf[m] * t * dt);
                    double hzf = 0.5 * (Hz[I3(ntfb, j, k)] + Hz[I3(ntfb - 1, j, k)]);
                    double hyf = -0.5 * (Hy[I3(ntfb, j, k)] + Hy[I3(ntfb - 1, j, k)]);
                    double hzb = -0.5 * (Hz[I3(Nx - ntfb, j, k)] + Hz[I3(Nx - ntfb - 1, j, k)]);
                    double hyb = 0.5 * (Hy[I3(Nx - ntfb, j, k)] + Hy[I3(Nx - ntfb - 1, j, k)]);
                    Jy_front[F2(j, k, Nz, 2 * m)] += hzf * s;
                    Jy_front[F2(j, k, Nz, 2 * m + 1)] += hzf * c;
                    Jz_front[F2(j, k, Nz, 2 * m)] += hyf * s;
                    Jz_front[F2(j, k, Nz, 2 * m + 1)] += hyf * c;
                    Jy_back[F2(j, k, Nz, 2 * m)] += hzb * s;
                    Jy_back[F2(j, k, Nz, 2 * m + 1)] += hzb * c;
                    Jz_back[F2(j, k, Nz, 2 * m)] += hyb * s;
                    Jz_back[F2(j, k, Nz, 2 * m + 1)] += hyb * c;
                }
        for (int i = 0; i < Nx; i++)
            for (int k = 0; k < Nz; k++)
                for (int m = 0; m < nntf; m++) {
                    double s = sin(2 * PI * fntf[m] * t * dt), c = cos(2 * PI * fntf[m] * t * dt);
                    double hzt = 0.5 * (Hz[I3(i, Ny - ntfb, k)] + Hz[I3(i, Ny - ntfb - 1, k)]);
                    double hxt = -0.5 * (Hx[I3(i, Ny - ntfb, k)] + Hx[I3(i, Ny - ntfb - 1, k)]);
                    double hzb = -0.5 * (Hz[I3(i, ntfb, k)] + Hz[I3(i, ntfb - 1, k)]);
                    double hxb = 0.5 * (Hx[I3(i, ntfb, k)] + Hx[I3(i, ntfb - 1, k)]);
                    Jx_top[F2(i, k, Nz, 2 * m)] += hzt * s;
                    Jx_top[F2(i, k, Nz, 2 * m + 1)] += hzt * c;
                    Jz_top[F2(i, k, Nz, 2 * m)] += hxt * s;
                    Jz_top[F2(i, k, Nz, 2 * m + 1)] += hxt * c;
                    Jx_bot[F2(i, k, Nz, 2 * m)] += hzb * s;
                    Jx_bot[F2(i, k, Nz, 2 * m + 1)] += hzb * c;
                    Jz_bot[F2(i, k, Nz, 2 * m)] += hxb * s;
                    Jz_bot[F2(i, k, Nz, 2 * m + 1)] += hxb * c;
                }
        for (int i = 0; i < Nx; i++)
            for (int j = 0; j < Ny; j++)
                for (int m = 0; m < nntf; m++) {
                    double s = sin(2 * PI * fntf[m] * t * dt), c = cos(2 * PI * fntf[m] * t * dt);
                    double hyl = 0.5 * (Hy[I3(i, j, ntfb)] + Hy[I3(i, j, ntfb - 1)]);
                    double hxl = -0.5 * (Hx[I3(i, j, ntfb)] + Hx[I3(i, j, ntfb - 1)]);
                    double hyr = -0.5 * (Hy[I3(i, j, Nz - ntfb)] + Hy[I3(i, j, Nz - ntfb - 1)]);
                    double hxr = 0.5 * (Hx[I3(i, j, Nz - ntfb)] + Hx[I3(i, j, Nz - ntfb - 1)]);
                    Jx_left[F2(i, j, Ny, 2 * m)] += hyl * s;
                    Jx_left[F2(i, j, Ny, 2 * m + 1)] += hyl * c;
                    Jy_left[F2(i, j, Ny, 2 * m)] += hxl * s;
                    Jy_left[F2(i, j, Ny, 2 * m + 1)] += hxl * c;
                    Jx_right[F2(i, j, Ny, 2 * m)] += hyr * s;
                    Jx_right[F2(i, j, Ny, 2 * m + 1)] += hyr * c;
                    Jy_right[F2(i, j, Ny, 2 * m)] += hxr * s;
                    Jy_right[F2(i, j, Ny, 2 * m + 1)] += hxr * c;
                }

        /* ---------------- H slices, R21:997-1014 ---------------- */
        for (int i = 0; i < Nx; i++)
            for (int j = 0; j < Ny - 1; j++) {
                HSz[(size_t)i * Ny + j] = Hy[I3(i, j, ssz)];
                HSz[(size_t)Nx * Ny + (size_t)i * Ny + j] = Hz[I3(i, j, ssz)];
            }
        for (int i = 0; i < Nx; i++)
            for (int k = 0; k < Nz - 1; k++) {
                HSy[(size_t)i * Nz + k] = Hy[I3(i, ssy, k)];
                HSy[(size_t)Nx * Nz + (size_t)i * Nz + k] = Hz[I3(i, ssy, k)];
            }
        for (int j = 0; j < Ny - 1; j++)
            for (int k = 0; k < Nz - 1; k++) {
                HSx[(size_t)j * Nz + k] = Hy[I3(ssx, j, k)];
                HSx[(size_t)Ny * Nz + (size_t)j * Nz + k] = Hz[I3(ssx, j, k)];
            }

        /* ---------------- E psi, R21:1020-1125 ---------------- */
        if (in.dopml) {
            for (int i = 0; i < Nx - 1; i++) {
                for (int j = 1; j < L + 1; j++)
                    for (int k = 1; k < Nz - 1; k++)
                        P_exy[PY(i, j - 1, k)] = Be[j - 1] * P_exy[PY(i, j - 1, k)] + Ae[j - 1] * (Hz[I3(i, j, k)] - Hz[I3(i, j - 1, k)]) / dy;
                for (int j = Ny - L - 1; j < Ny - 1; j++)
                    for (int k = 1; k < Nz - 1; k++)
                        P_exy[PY(i, j - yshift, k)] = Be[j - yshift] * P_exy[PY(i, j - yshift, k)] + Ae[j - yshift] * (Hz[I3(i, j, k)] - Hz[I3(i, j - 1, k)]) / dy;
            }
            for (int i = 0; i < Nx; i++)
                for (int j = 1; j < Ny - 1; j++) {
                    for (int k = 1; k < L + 1; k++)
                        P_exz[PZ(i, j, k - 1)] = Be[k - 1] * P_exz[PZ(i, j, k - 1)] + Ae[k - 1] * (Hy[I3(i, j, k)] - Hy[I3(i, j, k - 1)]) / dz;
                    for (int k = Nz - L - 1; k < Nz - 1; k++)
                        P_exz[PZ(i, j, k - zshift)] = Be[k - zshift] * P_exz[PZ(i, j, k - zshift)] + Ae[k - zshift] * (Hy[I3(i, j, k)] - Hy[I3(i, j, k - 1)]) / dz;
                }
            for (int i = 1; i < L + 1; i++)
                for (int j = 0; j < Ny - 1; j++)
                    for (int k = 1; k < Nz - 1; k++)
                        P_eyx[PX(i - 1, j, k)] = Be[i - 1] * P_eyx[PX(i - 1, j, k)] + Ae[i - 1] * (Hz[I3(i, j, k)] - Hz[I3(i - 1, j, k)]) / dx;
            for (int i = Nx - L - 1; i < Nx - 1; i++) {
                for (int j = 0; j < Ny - 1; j++)
                    for (int k = 1; k < Nz - 1; k++)
                        P_eyx[PX(i - xshift, j, k)] = Be[i - xshift] * P_eyx[PX(i - xshift, j, k)] + Ae[i - xshift] * (Hz[I3(i, j, k)] - Hz[I3(i - 1, j, k)]) / dx;
                if (!obl) P_eyxI[i - xshift] = Be[i - xshift] * P_eyxI[i - xshift] + Ae[i - xshift] * (Hzinc[i] - Hzinc[i - 1]) / dx;
            }
            for (int i = 1; i < Nx - 1; i++)
                for (int j = 0; j < Ny - 1; j++) {
                    for (int k = 1; k < L + 1; k++)
                        P_eyz[PZ(i, j, k - 1)] = Be[k - 1] * P_eyz[PZ(i, j, k - 1)] + Ae[k - 1] * (Hx[I3(i, j, k)] - Hx[I3(i, j, k - 1)]) / dz;
                    for (int k = Nz - L - 1; k < Nz - 1; k++)
                        P_eyz[PZ(i, j, k - zshift)] = Be[k - zshift] * P_eyz[PZ(i, j, k - zshift)] + Ae[k - zshift] * (Hx[I3(i, j, k)] - Hx[I3(i, j, k - 1)]) / dz;
                }
            for (int i = 1; i < L + 1; i++)
                for (int j = 1; j < Ny - 1; j++)
                    for (int k = 0; k < Nz - 1; k++)
                        P_ezx[PX(i - 1, j, k)] = Be[i - 1] * P_ezx[PX(i - 1, j, k)] + Ae[i - 1] * (Hy[I3(i, j, k)] - Hy[I3(i - 1, j, k)]) / dx;
            for (int i = Nx - L - 1; i < Nx - 1; i++) {
                for (int j = 1; j < Ny - 1; j++)
                    for (int k = 0; k < Nz - 1; k++)
                        P_ezx[PX(i - xshift, j, k)] = Be[i - xshift] * P_ezx[PX(i - xshift, j, k)] + Ae[i - xshift] * (Hy[I3(i, j, k)] - Hy[I3(i - 1, j, k)]) / dx;
                if (!obl) P_ezxI[i - xshift] = Be[i - xshift] * P_ezxI[i - xshift] + Ae[i - xshift] * (Hyinc[i] - Hyinc[i - 1]) / dx;
            }
            for (int i = 1; i < Nx - 1; i++) {
                for (int j = 1; j < L + 1; j++)
                    for (int k = 0; k < Nz - 1; k++)
                        P_ezy[PY(i, j - 1, k)] = Be[j - 1] * P_ezy[PY(i, j - 1, k)] + Ae[j - 1] * (Hx[I3(i, j, k)] - Hx[I3(i, j - 1, k)]) / dy;
                for (int j = Ny - L - 1; j < Ny - 1; j++)
                    for (int k = 0; k < Nz - 1; k++)
                        P_ezy[PY(i, j - yshift, k)] = Be[j - yshift] * P_ezy[PY(i, j - yshift, k)] + Ae[j - yshift] * (Hx[I3(i, j, k)] - Hx[I3(i, j - 1, k)]) / dy;
            }
        }

        /* ---------------- Ex, R21:1130-1185 ---------------- */
#pragma omp parallel for
        for (int i = 0; i < Nx - 1; i++)
            for (int j = 1; j < Ny - 1; j++)
                for (int k = 1; k < Nz - 1; k++) {
                    size_t c = I3(i, j, k);
                    Ex[c] = c1e[c] * Ex[c] + c2e[c] * ((Hz[c] - Hz[I3(i, j - 1, k)]) / dy - (Hy[c] - Hy[I3(i, j, k - 1)]) / dz) - c2e[c] * Jx[c];
                }
        if (!obl) {
            for (int i = bx1; i < bx2 - 1; i++)
                for (int j = by1; j < by2; j++) {
                    Ex[I3(i, j, bz1)] = Ex[I3(i, j, bz1)] + c2e0 * Hyinc[i] / dz;
                    Ex[I3(i, j, bz2)] = Ex[I3(i, j, bz2)] - c2e0 * Hyinc[i] / dz;
                }
            for (int i = bx1; i < bx2 - 1; i++)
                for (int k = bz1; k < bz2; k++) {
                    Ex[I3(i, by1, k)] = Ex[I3(i, by1, k)] - c2e0 * Hzinc[i] / dy;
                    Ex[I3(i, by2, k)] = Ex[I3(i, by2, k)] + c2e0 * Hzinc[i] / dy;
                }
        } else {
            for (int i = bx1 - 1; i <= bx2; i++)
                for (int j = by1 - 1; j <= by2; j++)
                    for (int k = bz1 - 1; k <= bz2; k = SHELL_NEXT(i, j, k)) {
                        double corr;
                        if (SHELL(i, j, k) && obl_corr(&O, 1, 0, i, j, k, Hyinc, &corr))
                            Ex[I3(i, j, k)] = Ex[I3(i, j, k)] + c2e0 * corr;
                    }
        }
        if (in.dopml) {
            for (int i = 0; i < Nx - 1; i++) {
                for (int j = 1; j < L + 1; j++)
                    for (int k = 1; k < Nz - 1; k++)
                        Ex[I3(i, j, k)] = Ex[I3(i, j, k)] + c2e0 * KAP(P_exy[PY(i, j - 1, k)], Ke, j - 1, Hz[I3(i, j, k)] - Hz[I3(i, j - 1, k)], dy);
                for (int j = Ny - L - 1; j < Ny - 1; j++)
                    for (int k = 1; k < Nz - 1; k++)
                        Ex[I3(i, j, k)] = Ex[I3(i, j, k)] + c2e0 * KAP(P_exy[PY(i, j - yshift, k)], Ke, j - yshift, Hz[I3(i, j, k)] - Hz[I3(i, j - 1, k)], dy);
            }
            for (int i = 0; i < Nx - 1; i++)
                for (int j = 1; j < Ny - 1; j++) {
                    for (int k = 1; k < L + 1; k++)
                        Ex[I3(i, j, k)] = Ex[I3(i, j, k)] - c2e0 * KAP(P_exz[PZ(i, j, k - 1)], Ke, k - 1, Hy[I3(i, j, k)] - Hy[I3(i, j, k - 1)], dz);
                    for (int k = Nz - L - 1; k < Nz - 1; k++)
                        Ex[I3(i, j, k)] = Ex[I3(i, j, k)] - c2e0 * KAP(P_exz[PZ(i, j, k - zshift)], Ke, k - zshift, Hy[I3(i, j, k)] - Hy[I3(i, j, k - 1)], dz);
                }
        }

        /* ---------------- Ey, R21:1190-1244 ---------------- */
#pragma omp parallel for
        for (int i = 1; i < Nx - 1; i++) {
            for (int j = 0; j < Ny; j++)
                for (int k = 1; k < Nz; k++) {
                    size_t c = I3(i, j, k);
                    Ey[c] = c1e[c] * Ey[c] + c2e[c] * ((Hx[c] - Hx[I3(i, j, k - 1)]) / dz - (Hz[c] - Hz[I3(i - 1, j, k)]) / dx) - c2e[c] * Jy[c];
                }
            if (!obl) Eyinc[i] = c1e0 * Eyinc[i] - c2e0 * (Hzinc[i] - Hzinc[i - 1]) / dx;
        }
        if (!obl) {
            for (int j = by1; j < by2; j++)
                for (int k = bz1; k < bz2; k++) {
                    Ey[I3(bx1, j, k)] = Ey[I3(bx1, j, k)] + c2e0 * Hzinc[bx1 - 1] / dx;
                    Ey[I3(bx2 - 1, j, k)] = Ey[I3(bx2 - 1, j, k)] - c2e0 * Hzinc[bx2 - 1] / dx;
                }
        } else {
            for (int i = bx1 - 1; i <= bx2; i++)
                for (int j = by1 - 1; j <= by2; j++)
                    for (int k = bz1 - 1; k <= bz2; k = SHELL_NEXT(i, j, k)) {
                        double corr;
                        if (SHELL(i, j, k) && obl_corr(&O, 1, 1, i, j, k, Hyinc, &corr))
                            Ey[I3(i, j, k)] = Ey[I3(i, j, k)] + c2e0 * corr;
                    }
        }
        if (in.dopml) {
            for (int i = 1; i < L + 1; i++)
                for (int j = 0; j < Ny; j++)
                    for (int k = 1; k < Nz; k++)
                        Ey[I3(i, j, k)] = Ey[I3(i, j, k)] - c2e0 * KAP(P_eyx[PX(i - 1, j, k)], Ke, i - 1, Hz[I3(i, j, k)] - Hz[I3(i - 1, j, k)], dx);
            for (int i = Nx - L - 1; i < Nx - 1; i++) {
                for (int j = 0; j < Ny; j++)
                    for (int k = 1; k < Nz; k++)
                        Ey[I3(i, j, k)] = Ey[I3(i, j, k)] - c2e0 * KAP(P_eyx[PX(i - xshift, j, k)], Ke, i - xshift, Hz[I3(i, j, k)] - Hz[I3(i - 1, j, k)], dx);
                if (!obl) Eyinc[i] = Eyinc[i] - c2e0 * P_eyxI[i - xshift];
            }
            for (int i = 1; i < Nx - 1; i++)
                for (int j = 0; j < Ny; j++) {
                    for (int k = 1; k < L + 1; k++)
                        Ey[I3(i, j, k)] = Ey[I3(i, j, k)] + c2e0 * KAP(P_eyz[PZ(i, j, k - 1)], Ke, k - 1, Hx[I3(i, j, k)] - Hx[I3(i, j, k - 1)], dz);
                    for (int k = Nz - L - 1; k < Nz - 1; k++)
                        Ey[I3(i, j, k)] = Ey[I3(i, j, k)] + c2e0 * KAP(P_eyz[PZ(i, j, k - zshift)], Ke, k - zshift, Hx[I3(i, j, k)] - Hx[I3(i, j, k - 1)], dz);
                }
        }

        /* ---------------- Ez, R21:1248-1271 ---------------- */
#pragma omp parallel for
        for (int i = 1; i < Nx - 1; i++) {
            for (int j = 1; j < Ny; j++)
                for (int k = 0; k < Nz; k++) {
                    size_t c = I3(i, j, k);
                    Ez[c] = c1e[c] * Ez[c] + c2e[c] * ((Hy[c] - Hy[I3(i - 1, j, k)]) / dx - (Hx[c] - Hx[I3(i, j - 1, k)]) / dy) - c2e[c] * Jz[c];
                }
            if (!obl) Ezinc[i] = c1e0 * Ezinc[i] + c2e0 * (Hyinc[i] - Hyinc[i - 1]) / dx;
        }
        if (!obl) {
            for (int j = by1; j < by2; j++)
                for (int k = bz1; k < bz2; k++) {
                    Ez[I3(bx1, j, k)] = Ez[I3(bx1, j, k)] - c2e0 * Hyinc[bx1 - 1] / dx;
                    Ez[I3(bx2 - 1, j, k)] = Ez[I3(bx2 - 1, j, k)] + c2e0 * Hyinc[bx2 - 1] / dx;
                }
        } else {
            for (int i = bx1 - 1; i <= bx2; i++)
                for (int j = by1 - 1; j <= by2; j++)
                    for (int k = bz1 - 1; k <= bz2; k = SHELL_NEXT(i, j, k)) {
                        double corr;
                        if (SHELL(i, j, k) && obl_corr(&O, 1, 2, i, j, k, Hyinc, &corr))
                            Ez[I3(i, j, k)] = Ez[I3(i, j, k)] + c2e0 * corr;
                    }
        }

        /* ---------------- source, R21:1278-1304 ---------------- */
        if (obl) { /* auxiliary line, E part, then the hard source at node 0 */
            const int M = O.M;
            for (int n = 1; n < M - 1; n++) {
                double e = c1e0 * Ezinc[n] - c2e0 * (Hyinc[n] - Hyinc[n - 1]) / O.dl;
                if (n >= M - L - 1) {
                    const int sidx = n - O.ashift;
                    P_e1[sidx] = T1.Be[sidx] * P_e1[sidx] + T1.Ae[sidx] * (Hyinc[n] - Hyinc[n - 1]) / O.dl;
                    e = e - c2e0 * P_e1[sidx];
                }
                Ezinc[n] = e;
            }
            Ezinc[0] = EsA[t];
        } else {
            switch (in.sourcepol) {
            case 2: Ezinc[0] = 0; Eyinc[0] = EsA[t]; break;
            case 3: Ezinc[0] = EsA[t]; Eyinc[0] = EsA[t]; break;
            case 4: Ezinc[0] = EsA[t]; Eyinc[0] = EsB[t]; break;
            case 5: Ezinc[0] = EsB[t]; Eyinc[0] = EsA[t]; break;
            default: Ezinc[0] = EsA[t]; Eyinc[0] = 0; break; /* 1 and others */
            }
        }

        /* ---------------- plate, R21:1307-1320 ---------------- */
        if (in.doplate == 1) {
            int lo = (int)(ssy - in.platesize / 2 / dy);
            int up = (int)(ssy + in.platesize / 2 / dy);
            for (int j = lo; j < up - 1; j++)
                for (int k = lo; k < up; k++) Ey[I3(ssx, j, k)] = 0;
            for (int j = lo; j < up; j++)
                for (int k = lo; k < up - 1; k++) Ez[I3(ssx, j, k)] = 0;
        }

        /* ---------------- E slices (Ez before its PML fix), R21:1323-1340 */
        for (int i = 0; i < Nx; i++)
            for (int j = 0; j < Ny; j++) {
                ESz[(size_t)i * Ny + j] = Ey[I3(i, j, ssz)];
                ESz[(size_t)Nx * Ny + (size_t)i * Ny + j] = Ez[I3(i, j, ssz)];
            }
        for (int i = 0; i < Nx; i++)
            for (int k = 0; k < Nz; k++) {
                ESy[(size_t)i * Nz + k] = Ey[I3(i, ssy, k)];
                ESy[(size_t)Nx * Nz + (size_t)i * Nz + k] = Ez[I3(i, ssy, k)];
            }
        for (int j = 0; j < Ny; j++)
            for (int k = 0; k < Nz; k++) {
                ESx[(size_t)j * Nz + k] = Ey[I3(ssx, j, k)];
                ESx[(size_t)Ny * Nz + (size_t)j * Nz + k] = Ez[I3(ssx, j, k)];
            }

        /* ---------------- Ez PML, R21:1343-1374 ---------------- */
        if (in.dopml) {
            for (int i = 1; i < L + 1; i++)
                for (int j = 1; j < Ny; j++)
                    for (int k = 0; k < Nz; k++)
                        Ez[I3(i, j, k)] = Ez[I3(i, j, k)] + c2e0 * KAP(P_ezx[PX(i - 1, j, k)], Ke, i - 1, Hy[I3(i, j, k)] - Hy[I3(i - 1, j, k)], dx);
            for (int i = Nx - L - 1; i < Nx - 1; i++) {
                for (int j = 1; j < Ny; j++)
                    for (int k = 0; k < Nz; k++)
                        Ez[I3(i, j, k)] = Ez[I3(i, j, k)] + c2e0 * KAP(P_ezx[PX(i - xshift, j, k)], Ke, i - xshift, Hy[I3(i, j, k)] - Hy[I3(i - 1, j, k)], dx);
                if (!obl) Ezinc[i] = Ezinc[i] + c2e0 * P_ezxI[i - xshift];
            }
            for (int i = 1; i < Nx - 1; i++) {
                for (int j = 1; j < L + 1; j++)
                    for (int k = 0; k < Nz - 1; k++)
                        Ez[I3(i, j, k)] = Ez[I3(i, j, k)] - c2e0 * KAP(P_ezy[PY(i, j - 1, k)], Ke, j - 1, Hx[I3(i, j, k)] - Hx[I3(i, j - 1, k)], dy);
                for (int j = Ny - L - 1; j < Ny - 1; j++)
                    for (int k = 0; k < Nz - 1; k++)
                        Ez[I3(i, j, k)] = Ez[I3(i, j, k)] - c2e0 * KAP(P_ezy[PY(i, j - yshift, k)], Ke, j - yshift, Hx[I3(i, j, k)] - Hx[I3(i, j - 1, k)], dy);
            }
        }

        /* ---------------- source DFT, R21:1378-1383 ((t+1/2) is t) -------- */
        for (int m = 0; m < nntf; m++) {
            Ezdft[2 * m] += Ezinc[0] * sin(2 * PI * fntf[m] * (t + 1 / 2) * dt);
            Ezdft[2 * m + 1] += Ezinc[0] * cos(2 * PI * fntf[m] * (t + 1 / 2) * dt);
            Eydft[2 * m] += Eyinc[0] * sin(2 * PI * fntf[m] * (t + 1 / 2) * dt);
            Eydft[2 * m + 1] += Eyinc[0] * cos(2 * PI * fntf[m] * (t + 1 / 2) * dt);
        }

        /* ---------------- NTF, E part, R21:1388-1438 ---------------- */
        for (int j = 0; j < Ny; j++)
            for (int k = 0; k < Nz; k++)
                for (int m = 0; m < nntf; m++) {
                    double s = sin(2 * PI * fntf[m] * (t + 1 / 2) * dt), c = cos(2 * PI * fntf[m] * (t + 1 / 2) * dt);
                    double a = -Ez[I3(ntfb, j, k)], b = Ey[I3(ntfb, j, k)];
                    double cc = Ez[I3(Nx - ntfb, j, k)], d = -Ey[I3(Nx - ntfb, j, k)];
                    My_front[F2(j, k, Nz, 2 * m)] += a * s;
                    My_front[F2(j, k, Nz, 2 * m + 1)] += a * c;
                    Mz_front[F2(j, k, Nz, 2 * m)] += b * s;
                    Mz_front[F2(j, k, Nz, 2 * m + 1)] += b * c;
                    My_back[F2(j, k, Nz, 2 * m)] += cc * s;
                    My_back[F2(j, k, Nz, 2 * m + 1)] += cc * c;
                    Mz_back[F2(j, k, Nz, 2 * m)] += d * s;
                    Mz_back[F2(j, k, Nz, 2 * m + 1)] += d * c;
                }
        for (int i = 0; i < Nx; i++)
            for (int k = 0; k < Nz; k++)
                for (int m = 0; m < nntf; m++) {
                    double s = sin(2 * PI * fntf[m] * (t + 1 / 2) * dt), c = cos(2 * PI * fntf[m] * (t + 1 / 2) * dt);
                    double a = -Ez[I3(i, Ny - ntfb, k)], b = Ex[I3(i, Ny - ntfb, k)];
                    double cc = Ez[I3(i, ntfb, k)], d = -Ex[I3(i, ntfb, k)];
                    Mx_top[F2(i, k, Nz, 2 * m)] += a * s;
                    Mx_top[F2(i, k, Nz, 2 * m + 1)] += a * c;
                    Mz_top[F2(i, k, Nz, 2 * m)] += b * s;
                    Mz_top[F2(i, k, Nz, 2 * m + 1)] += b * c;
                    Mx_bot[F2(i, k, Nz, 2 * m)] += cc * s;
                    Mx_bot[F2(i, k, Nz, 2 * m + 1)] += cc * c;
                    Mz_bot[F2(i, k, Nz, 2 * m)] += d * s;
                    Mz_bot[F2(i, k, Nz, 2 * m + 1)] += d * c;
                }
        for (int i = 0; i < Nx; i++)
            for (int j = 0; j < Ny; j++)
                for (int m = 0; m < nntf; m++) {
                    double s = sin(2 * PI * fntf[m] * (t + 1 / 2) * dt), c = cos(2 * PI * fntf[m] * (t + 1 / 2) * dt);
                    double a = -Ey[I3(i, j, ntfb)], b = Ex[I3(i, j, ntfb)];
                    double cc = Ey[I3(i, j, Nz - ntfb)], d = -Ex[I3(i, j, Nz - ntfb)];
                    Mx_left[F2(i, j, Ny, 2 * m)] += a * s;
                    Mx_left[F2(i, j, Ny, 2 * m + 1)] += a * c;
                    My_left[F2(i, j, Ny, 2 * m)] += b * s;
                    My_left[F2(i, j, Ny, 2 * m + 1)] += b * c;
                    Mx_right[F2(i, j, Ny, 2 * m)] += cc * s;
                    Mx_right[F2(i, j, Ny, 2 * m + 1)] += cc * c;
                    My_right[F2(i, j, Ny, 2 * m)] += d * s;
                    My_right[F2(i, j, Ny, 2 * m + 1)] += d * c;
                }

        /* ---------------- probes, R21:1443-1455 ---------------- */
        for (int n = 0; n < np; n++) {
            int ix = in.probex[n], iy = in.probey[n], iz = in.probez[n];
            size_t o = (size_t)t * np + n;
            Prb[0][o] = 0.5 * (Ex[I3(ix, iy, iz)] + Ex[I3(ix - 1, iy, iz)]);
            Prb[1][o] = 0.5 * (Ey[I3(ix, iy, iz)] + Ey[I3(ix, iy - 1, iz)]);
            Prb[2][o] = 0.5 * (Ez[I3(ix, iy, iz)] + Ez[I3(ix, iy, iz - 1)]);
            Prb[3][o] = 0.25 * (Hx[I3(ix, iy, iz)] + Hx[I3(ix, iy - 1, iz)] + Hx[I3(ix, iy, iz - 1)] + Hx[I3(ix, iy - 1, iz - 1)]);
            Prb[4][o] = 0.25 * (Hy[I3(ix, iy, iz)] + Hy[I3(ix - 1, iy, iz)] + Hy[I3(ix, iy, iz - 1)] + Hy[I3(ix - 1, iy, iz - 1)]);
            Prb[5][o] = 0.25 * (Hz[I3(ix, iy, iz)] + Hz[I3(ix, iy - 1, iz)] + Hz[I3(ix - 1, iy, iz)] + Hz[I3(ix - 1, iy - 1, iz)]);
        }

        /* ---------------- unused |E| and |S| pass, R21:1460-1487 ---------- */
        if (mirror_dead_work) {
#pragma omp parallel for
            for (int i = 1; i < Nx - 1; i++)
                for (int j = 1; j < Ny - 1; j++)
                    for (int k = 1; k < Nz - 1; k++) {
                        size_t c = I3(i, j, k);
                        double exm = (Ex[c] + Ex[I3(i - 1, j, k)]) / 2;
                        double eym = (Ey[c] + Ey[I3(i, j - 1, k)]) / 2;
                        double ezm = (Ez[c] + Ez[I3(i, j, k - 1)]) / 2;
                        double hxm = (Hx[c] + Hx[I3(i, j - 1, k)] + Hx[I3(i, j, k - 1)] + Hx[I3(i, j - 1, k - 1)]) / 4;
                        double hym = (Hy[c] + Hy[I3(i - 1, j, k)] + Hy[I3(i, j, k - 1)] + Hy[I3(i - 1, j, k - 1)]) / 4;
                        double hzm = (Hz[c] + Hz[I3(i - 1, j, k)] + Hz[I3(i, j - 1, k)] + Hz[I3(i - 1, j - 1, k)]) / 4;
                        Emag[c] = sqrt(exm * exm + eym * eym + ezm * ezm);
                        double sx = eym * hzm - ezm * hym, sy = ezm * hxm - exm * hzm, sz = exm * hym - eym * hxm;
                        Smag[c] = sqrt(sx * sx + sy * sy + sz * sz);
                    }
        }

        /* ---------------- J update, R21:1492-1504 / RFK:1539-1595 ---------- */
        if (!in.doB0) {
#pragma omp parallel for
            for (int i = 1; i < Nx - 1; i++)
                for (int j = 1; j < Ny - 1; j++)
                    for (int k = 1; k < Nz - 1; k++) {
                        size_t c = I3(i, j, k);
                        double nu = nue[c], w = wpe[c];
                        Jx[c] = ((2 - nu * dt) / (2 + nu * dt)) * Jx[c] + 2 * ((OR_E0 * w * w * dt) / (2 + nu * dt)) * Ex[c];
                        Jy[c] = ((2 - nu * dt) / (2 + nu * dt)) * Jy[c] + 2 * ((OR_E0 * w * w * dt) / (2 + nu * dt)) * Ey[c];
                        Jz[c] = ((2 - nu * dt) / (2 + nu * dt)) * Jz[c] + 2 * ((OR_E0 * w * w * dt) / (2 + nu * dt)) * Ez[c];
                    }
        } else {
            const double cw = cos(wce0 * dt), sw = sin(wce0 * dt);
#pragma omp parallel for
            for (int i = 1; i < Nx - 1; i++)
                for (int j = 1; j < Ny - 1; j++)
                    for (int k = 1; k < Nz - 1; k++) {
                        size_t c = I3(i, j, k);
                        double nu = nue[c], w = wpe[c];
                        double Ee1 = exp(-nu * dt);
                        double Ee2 = 1 / (wce0 * wce0 + nu * nu);
                        double Se1 = sw / wce0;
                        double Ce1 = (1 - cw) / (wce0 * wce0);
                        double Ce2 = (1 - Ee1) / nu - Ee1 * nu * Ce1 - Ee1 * Se1;
                        double Ce3 = nu * (1 - Ee1 * cw) + Ee1 * wce0 * sw;
                        double Ce4 = 1 - Ee1 * cw - Ee1 * nu * Se1;
                        double A00 = Ee1 * (Ce1 * wcex * wcex + cw), A01 = Ee1 * (Ce1 * wcex * wcey - Se1 * wcez), A02 = Ee1 * (Ce1 * wcex * wcez + Se1 * wcey);
                        double A10 = Ee1 * (Ce1 * wcey * wcex + Se1 * wcez), A11 = Ee1 * (Ce1 * wcey * wcey + cw), A12 = Ee1 * (Ce1 * wcey * wcez - Se1 * wcex);
                        double A20 = Ee1 * (Ce1 * wcez * wcex - Se1 * wcey), A21 = Ee1 * (Ce1 * wcez * wcey + Se1 * wcex), A22 = Ee1 * (Ce1 * wcez * wcez + cw);
                        double K00 = Ee2 * (Ce2 * wcex * wcex + Ce3), K01 = Ee2 * (Ce2 * wcex * wcey - Ce4 * wcez), K02 = Ee2 * (Ce2 * wcex * wcez + Ce4 * wcey);
                        double K10 = Ee2 * (Ce2 * wcey * wcex + Ce4 * wcez), K11 = Ee2 * (Ce2 * wcey * wcey + Ce3), K12 = Ee2 * (Ce2 * wcey * wcez - Ce4 * wcex);
                        double K20 = Ee2 * (Ce2 * wcez * wcex - Ce4 * wcey), K21 = Ee2 * (Ce2 * wcez * wcey + Ce4 * wcex), K22 = Ee2 * (Ce2 * wcez * wcez + Ce3);
                        /* extended input lk_colocated: E at the current's own node */
                        const int colo = in.ext.lk_colocated;
                        double m0 = colo ? Ex[c] : (Ex[c] + Ex[I3(i - 1, j, k)]) / 2;
                        double m1 = colo ? Ey[c] : (Ey[c] + Ey[I3(i, j - 1, k)]) / 2;
                        double m2 = colo ? Ez[c] : (Ez[c] + Ez[I3(i, j, k - 1)]) / 2;
                        double jx = Jx[c], jy = Jy[c], jz = Jz[c];
                        Jx[c] = A00 * jx + A01 * jy + A02 * jz + OR_E0 * w * w * (K00 * m0 + K01 * m1 + K02 * m2);
                        Jy[c] = A10 * jx + A11 * jy + A12 * jz + OR_E0 * w * w * (K10 * m0 + K11 * m1 + K12 * m2);
                        Jz[c] = A20 * jx + A21 * jy + A22 * jz + OR_E0 * w * w * (K20 * m0 + K21 * m1 + K22 * m2);
                    }
        }

        /* ---------------- progress, record step, R21:1512-1571 ------------ */
        if (t == 20) {
            double runtimemin = (now_s() - tloopStart) / 60.0;
            double totaltime = runtimemin * tsteps / 20.0;
            lg = open_in(dir, "log.txt", "a");
            if (lg) {
                fprintf(lg, "t = 20, time taken = %g minutes.\n", runtimemin);
                fprintf(lg, "You can expect the total simulation to take %g minutes.\n", totaltime);
                fclose(lg);
            }
        }
        if (t % rec_period == 0) {
            double partialtime = 100 * t / tsteps;
            double Emax = 0;
            for (size_t c = 0; c < NC; c++)
                if (fabs(Ex[c]) > Emax) Emax = fabs(Ex[c]);
            lg = open_in(dir, "log.txt", "a");
            if (lg) {
                fprintf(lg, "t = %d: %g %% Done...  Maximum abs(Ex) is %g\n", t, partialtime, Emax);
                fclose(lg);
            }
            if (in.savefields) {
                FILE *f = open_in(dir, "output_E.dat", "ab");
                if (f) {
                    write_all(f, ESz, szz); write_all(f, ESy, szy); write_all(f, ESx, szx);
                    write_all(f, Eyinc, (size_t)Nx); write_all(f, Ezinc, (size_t)Nx);
                    fclose(f);
                }
                f = open_in(dir, "output_J.dat", "ab");
                if (f) {
                    write_all(f, JSz, szz); write_all(f, JSy, szy); write_all(f, JSx, szx);
                    fclose(f);
                }
                f = open_in(dir, "output_H.dat", "ab");
                if (f) {
                    write_all(f, HSz, szz); write_all(f, HSy, szy); write_all(f, HSx, szx);
                    write_all(f, Hyinc, (size_t)Nx); write_all(f, Hzinc, (size_t)Nx);
                    fclose(f);
                }
            }
        }
    }
    double tloopEnd = now_s();
    if (loop_seconds) *loop_seconds = tloopEnd - tloopStart;

    /* ---------------- final outputs, R21:1579-1636 ---------------- */
    FILE *f = open_in(dir, "output_NTF.dat", "wb");
    if (f) {
        fwrite(&nntf, sizeof(int), 1, f);
        fwrite(&ntfb, sizeof(int), 1, f);
        write_all(f, in.fntf, (size_t)nntf);
        write_all(f, Eydft, 2 * (size_t)nntf);
        write_all(f, Ezdft, 2 * (size_t)nntf);
        double *fb[8] = {My_front, Mz_front, Jy_front, Jz_front, My_back, Mz_back, Jy_back, Jz_back};
        double *tb[8] = {Mx_top, Mz_top, Jx_top, Jz_top, Mx_bot, Mz_bot, Jx_bot, Jz_bot};
        double *lr[8] = {Mx_left, My_left, Jx_left, Jy_left, Mx_right, My_right, Jx_right, Jy_right};
        for (int q = 0; q < 8; q++) write_all(f, fb[q], fbn);
        if (Ny > 39 && Nz > 79) {
            printf("My-front at y = 40, z = 80 is %g\n", My_front[F2(39, 79, Nz, 0)]);
            printf("Mz-front at y = 40, z = 80 is %g\n", Mz_front[F2(39, 79, Nz, 0)]);
        }
        for (int q = 0; q < 8; q++) write_all(f, tb[q], tbn);
        for (int q = 0; q < 8; q++) write_all(f, lr[q], lrn);
        fclose(f);
    }
    f = open_in(dir, "Probe.dat", "wb");
    if (f) {
        fwrite(&np, sizeof(int), 1, f);
        if (np) {
            fwrite(in.probex, sizeof(int), (size_t)np, f);
            fwrite(in.probey, sizeof(int), (size_t)np, f);
            fwrite(in.probez, sizeof(int), (size_t)np, f);
        }
        for (int q = 0; q < 6; q++) write_all(f, Prb[q], (size_t)tsteps * np);
        fclose(f);
    }
    lg = open_in(dir, "log.txt", "a");
    if (lg) {
        fprintf(lg, "All done!\n");
        fprintf(lg, "Total run time = %gminutes.\n", (now_s() - tStart) / 60.0);
        fclose(lg);
    }

    /* release */
    double *all[] = {x, y, z, EsA, EsB, c1e, c2e, Ex, Ey, Ez, Hx, Hy, Hz, Jx, Jy, Jz,
                     Eyinc, Ezinc, Hyinc, Hzinc, Emag, Smag, ESz, ESy, ESx, HSz, HSy, HSx,
                     JSz, JSy, JSx, wpe, nue, P_hxy, P_hxz, P_hyx, P_hyz, P_hzx, P_hzy,
                     P_exy, P_exz, P_eyx, P_eyz, P_ezx, P_ezy, Ezdft, Eydft,
                     My_front, Mz_front, Jy_front, Jz_front, My_back, Mz_back, Jy_back, Jz_back,
                     Mx_top, Mz_top, Jx_top, Jz_top, Mx_bot, Mz_bot, Jx_bot, Jz_bot,
                     Mx_left, My_left, Jx_left, Jy_left, Mx_right, My_right, Jx_right, Jy_right};
    for (size_t q = 0; q < sizeof all / sizeof all[0]; q++) free(all[q]);
    for (int q = 0; q < 6; q++) free(Prb[q]);
    free_inputs(&in);
    return 0;
#undef I3
#undef PX
#undef PY
#undef PZ
#undef F2
}

#ifdef ORACLE_MAIN
int main(int argc, char **argv) {
    const char *dir = argc > 1 ? argv[1] : ".";
    int steps = argc > 2 ? atoi(argv[2]) : -1;
    int threads = argc > 3 ? atoi(argv[3]) : 0;
    double secs = 0;
    int rc = oracle_run_dir(dir, steps, threads, 1, &secs);
    if (rc) fprintf(stderr, "oracle: error %d\n", rc);
    else fprintf(stderr, "oracle: loop %.6f s\n", secs);
    return rc ? 1 : 0;
}
#endif
