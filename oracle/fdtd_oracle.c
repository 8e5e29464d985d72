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

/* Hard-coded solver settings, R21:119, R21:342-343, R21:413-415, R21:539-552. */
#define OR_PMLLEN 10
#define OR_PMLM 4.0
#define OR_TFSF_GAP 10
#define OR_NTF_GAP 5

typedef struct {
    int dopml, savefields, sourcetype, sourcepol, tsteps, Nx, Ny, Nz;
    int mettype, numfiles, nprobes, nntf, doplate, doB0;
    double f0, fsig, gridfactor, dt, metsize[2], wpmax, numax, metloc[3];
    double metangle, platesize;
    int *probex, *probey, *probez;
    double *fntf;
    double Bx, By, Bz;
    double *wp2, *nu2; /* [Nx][Ny], C order as read */
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

    if (p->Nx < 2 * OR_PMLLEN + 2 || p->Ny < 2 * OR_PMLLEN + 2 || p->Nz < 2 * OR_PMLLEN + 2)
        return -3;
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
    return e ? -2 : 0;
}

static void free_inputs(or_in *p) {
    free(p->probex); free(p->probey); free(p->probez);
    free(p->fntf); free(p->wp2); free(p->nu2);
}

static double *dalloc(size_t n) {
    double *a = calloc(n ? n : 1, sizeof(double));
    if (!a) { fprintf(stderr, "oracle: out of memory (%zu doubles)\n", n); exit(3); }
    return a;
}

/* PML coefficient tables, R21:411-526.  Index m in [L, 2L) is the high side,
 * the low side mirrors it. */
typedef struct {
    double Be[2 * OR_PMLLEN], Ae[2 * OR_PMLLEN]; /* half-cell grading: E psi  */
    double Bh[2 * OR_PMLLEN], Ah[2 * OR_PMLLEN]; /* full-cell grading: H psi  */
} or_pml;

static void pml_tables(double dx, double dt, or_pml *t) {
    const int L = OR_PMLLEN;
    const double pmlm = OR_PMLM;
    double simax = 1.5 * (double)(pmlm + 1) / (150 * OR_PI * dx);
    double kamax = 1, almax = 0;
    double s[OR_PMLLEN], sm[OR_PMLLEN], ka[OR_PMLLEN], kam[OR_PMLLEN];
    double al[OR_PMLLEN], alm[OR_PMLLEN];
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
    }
    for (int m = 0; m < L; m++) {
        t->Be[m] = t->Be[2 * L - 1 - m];
        t->Ae[m] = t->Ae[2 * L - 1 - m];
        t->Bh[m] = t->Bh[2 * L - 1 - m];
        t->Ah[m] = t->Ah[2 * L - 1 - m];
    }
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
    const int L = OR_PMLLEN;
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
    for (int i = 0; i < Nx; i++) {
        x[i] = -(Nx - 1) / 2 * dx + dx * i;
        if (i < nmax) y[i] = -(Ny - 1) / 2 * dy + dy * i;
        if (i < nmax) z[i] = -(Nz - 1) / 2 * dz + dz * i;
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
                    }
        }
    }

    /* CPML, R21:342-535. */
    or_pml T;
    memset(&T, 0, sizeof T);
    if (in.dopml) pml_tables(dx, dt, &T);
    const int xshift = Nx - 2 * L - 1, yshift = Ny - 2 * L - 1, zshift = Nz - 2 * L - 1;
    /* psi slabs: x-normal [2L][Ny][Nz], y-normal [Nx][2L][Nz], z-normal [Nx][Ny][2L] */
    const size_t nxs = (size_t)2 * L * Ny * Nz, nys = (size_t)Nx * 2 * L * Nz, nzs = (size_t)Nx * Ny * 2 * L;
    double *P_hxy = dalloc(nys), *P_hxz = dalloc(nzs), *P_hyx = dalloc(nxs);
    double *P_hyz = dalloc(nzs), *P_hzx = dalloc(nxs), *P_hzy = dalloc(nys);
    double *P_exy = dalloc(nys), *P_exz = dalloc(nzs), *P_eyx = dalloc(nxs);
    double *P_eyz = dalloc(nzs), *P_ezx = dalloc(nxs), *P_ezy = dalloc(nys);
    double P_eyxI[2 * OR_PMLLEN] = {0}, P_ezxI[2 * OR_PMLLEN] = {0};
    double P_hyxI[2 * OR_PMLLEN] = {0}, P_hzxI[2 * OR_PMLLEN] = {0};
#define PX(i, j, k) ((((size_t)(i)) * Ny + (size_t)(j)) * Nz + (size_t)(k))        /* [2L][Ny][Nz] */
#define PY(i, j, k) ((((size_t)(i)) * (2 * L) + (size_t)(j)) * Nz + (size_t)(k))   /* [Nx][2L][Nz] */
#define PZ(i, j, k) ((((size_t)(i)) * Ny + (size_t)(j)) * (2 * L) + (size_t)(k))   /* [Nx][Ny][2L] */
    const double *Bh = T.Bh, *Ah = T.Ah, *Be = T.Be, *Ae = T.Ae;

    /* TF/SF box and NTF surface, R21:539-552. */
    const int bx1 = L + OR_TFSF_GAP, bx2 = Nx - L - OR_TFSF_GAP;
    const int by1 = L + OR_TFSF_GAP, by2 = Ny - L - OR_TFSF_GAP;
    const int bz1 = L + OR_TFSF_GAP, bz2 = Nz - L - OR_TFSF_GAP;
    int ntfb = L + OR_NTF_GAP;

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
                P_hyxI[i - xshift] = Bh[i - xshift] * P_hyxI[i - xshift] + Ah[i - xshift] * (Ezinc[i + 1] - Ezinc[i]) / dx;
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
                P_hzxI[i - xshift] = Bh[i - xshift] * P_hzxI[i - xshift] + Ah[i - xshift] * (Eyinc[i + 1] - Eyinc[i]) / dx;
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
        if (in.dopml) {
            for (int i = 0; i < Nx; i++) {
                for (int j = 0; j < L; j++)
                    for (int k = 0; k < Nz - 1; k++)
                        Hx[I3(i, j, k)] = Hx[I3(i, j, k)] - c2h * P_hxy[PY(i, j, k)];
                for (int j = Ny - L - 1; j < Ny - 1; j++)
                    for (int k = 0; k < Nz - 1; k++)
                        Hx[I3(i, j, k)] = Hx[I3(i, j, k)] - c2h * P_hxy[PY(i, j - yshift, k)];
            }
            for (int i = 0; i < Nx; i++)
                for (int j = 0; j < Ny - 1; j++) {
                    for (int k = 0; k < L; k++)
                        Hx[I3(i, j, k)] = Hx[I3(i, j, k)] + c2h * P_hxz[PZ(i, j, k)];
                    for (int k = Nz - L - 1; k < Nz - 1; k++)
                        Hx[I3(i, j, k)] = Hx[I3(i, j, k)] + c2h * P_hxz[PZ(i, j, k - zshift)];
                }
        }

        /* ---------------- Hy, R21:823-877 ---------------- */
#pragma omp parallel for
        for (int i = 0; i < Nx - 1; i++) {
            for (int j = 0; j < Ny; j++)
                for (int k = 0; k < Nz - 1; k++)
                    Hy[I3(i, j, k)] = c1h * Hy[I3(i, j, k)] - c2h * ((Ex[I3(i, j, k + 1)] - Ex[I3(i, j, k)]) / dz - (Ez[I3(i + 1, j, k)] - Ez[I3(i, j, k)]) / dx);
            Hyinc[i] = c1h * Hyinc[i] + c2h * (Ezinc[i + 1] - Ezinc[i]) / dx;
        }
        for (int j = by1; j < by2; j++)
            for (int k = bz1; k < bz2; k++) {
                Hy[I3(bx1 - 1, j, k)] = Hy[I3(bx1 - 1, j, k)] - c2h * Ezinc[bx1] / dx;
                Hy[I3(bx2 - 1, j, k)] = Hy[I3(bx2 - 1, j, k)] + c2h * Ezinc[bx2 - 1] / dx;
            }
        if (in.dopml) {
            for (int i = 0; i < L; i++)
                for (int j = 0; j < Ny; j++)
                    for (int k = 0; k < Nz - 1; k++)
                        Hy[I3(i, j, k)] = Hy[I3(i, j, k)] + c2h * P_hyx[PX(i, j, k)];
            for (int i = Nx - L - 1; i < Nx - 1; i++) {
                for (int j = 0; j < Ny; j++)
                    for (int k = 0; k < Nz - 1; k++)
                        Hy[I3(i, j, k)] = Hy[I3(i, j, k)] + c2h * P_hyx[PX(i - xshift, j, k)];
                Hyinc[i] = Hyinc[i] + c2h * P_hyxI[i - xshift];
            }
            for (int i = 0; i < Nx - 1; i++)
                for (int j = 0; j < Ny; j++) {
                    for (int k = 0; k < L; k++)
                        Hy[I3(i, j, k)] = Hy[I3(i, j, k)] - c2h * P_hyz[PZ(i, j, k)];
                    for (int k = Nz - L - 1; k < Nz - 1; k++)
                        Hy[I3(i, j, k)] = Hy[I3(i, j, k)] - c2h * P_hyz[PZ(i, j, k - zshift)];
                }
        }

        /* ---------------- Hz, R21:882-937 ---------------- */
#pragma omp parallel for
        for (int i = 0; i < Nx - 1; i++) {
            for (int j = 0; j < Ny - 1; j++)
                for (int k = 0; k < Nz; k++)
                    Hz[I3(i, j, k)] = c1h * Hz[I3(i, j, k)] - c2h * ((Ey[I3(i + 1, j, k)] - Ey[I3(i, j, k)]) / dx - (Ex[I3(i, j + 1, k)] - Ex[I3(i, j, k)]) / dy);
            Hzinc[i] = c1h * Hzinc[i] - c2h * (Eyinc[i + 1] - Eyinc[i]) / dx;
        }
        for (int j = by1; j < by2; j++)
            for (int k = bz1; k < bz2; k++) {
                Hz[I3(bx1 - 1, j, k)] = Hz[I3(bx1 - 1, j, k)] + c2h * Eyinc[bx1] / dx;
                Hz[I3(bx2 - 1, j, k)] = Hz[I3(bx2 - 1, j, k)] - c2h * Eyinc[bx2 - 1] / dx;
            }
        if (in.dopml) {
            for (int i = 0; i < L; i++)
                for (int j = 0; j < Ny - 1; j++)
                    for (int k = 0; k < Nz; k++)
                        Hz[I3(i, j, k)] = Hz[I3(i, j, k)] - c2h * P_hzx[PX(i, j, k)];
            for (int i = Nx - L - 1; i < Nx - 1; i++) {
                for (int j = 0; j < Ny - 1; j++)
                    for (int k = 0; k < Nz; k++)
                        Hz[I3(i, j, k)] = Hz[I3(i, j, k)] - c2h * P_hzx[PX(i - xshift, j, k)];
                Hzinc[i] = Hzinc[i] - c2h * P_hzxI[i - xshift];
            }
            for (int i = 0; i < Nx - 1; i++) {
                for (int j = 0; j < L; j++)
                    for (int k = 0; k < Nz; k++)
                        Hz[I3(i, j, k)] = Hz[I3(i, j, k)] + c2h * P_hzy[PY(i, j, k)];
                for (int j = Ny - L - 1; j < Ny - 1; j++)
                    for (int k = 0; k < Nz; k++)
                        Hz[I3(i, j, k)] = Hz[I3(i, j, k)] + c2h * P_hzy[PY(i, j - yshift, k)];
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
                P_eyxI[i - xshift] = Be[i - xshift] * P_eyxI[i - xshift] + Ae[i - xshift] * (Hzinc[i] - Hzinc[i - 1]) / dx;
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
                P_ezxI[i - xshift] = Be[i - xshift] * P_ezxI[i - xshift] + Ae[i - xshift] * (Hyinc[i] - Hyinc[i - 1]) / dx;
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
        if (in.dopml) {
            for (int i = 0; i < Nx - 1; i++) {
                for (int j = 1; j < L + 1; j++)
                    for (int k = 1; k < Nz - 1; k++)
                        Ex[I3(i, j, k)] = Ex[I3(i, j, k)] + c2e0 * P_exy[PY(i, j - 1, k)];
                for (int j = Ny - L - 1; j < Ny - 1; j++)
                    for (int k = 1; k < Nz - 1; k++)
                        Ex[I3(i, j, k)] = Ex[I3(i, j, k)] + c2e0 * P_exy[PY(i, j - yshift, k)];
            }
            for (int i = 0; i < Nx - 1; i++)
                for (int j = 1; j < Ny - 1; j++) {
                    for (int k = 1; k < L + 1; k++)
                        Ex[I3(i, j, k)] = Ex[I3(i, j, k)] - c2e0 * P_exz[PZ(i, j, k - 1)];
                    for (int k = Nz - L - 1; k < Nz - 1; k++)
                        Ex[I3(i, j, k)] = Ex[I3(i, j, k)] - c2e0 * P_exz[PZ(i, j, k - zshift)];
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
            Eyinc[i] = c1e0 * Eyinc[i] - c2e0 * (Hzinc[i] - Hzinc[i - 1]) / dx;
        }
        for (int j = by1; j < by2; j++)
            for (int k = bz1; k < bz2; k++) {
                Ey[I3(bx1, j, k)] = Ey[I3(bx1, j, k)] + c2e0 * Hzinc[bx1 - 1] / dx;
                Ey[I3(bx2 - 1, j, k)] = Ey[I3(bx2 - 1, j, k)] - c2e0 * Hzinc[bx2 - 1] / dx;
            }
        if (in.dopml) {
            for (int i = 1; i < L + 1; i++)
                for (int j = 0; j < Ny; j++)
                    for (int k = 1; k < Nz; k++)
                        Ey[I3(i, j, k)] = Ey[I3(i, j, k)] - c2e0 * P_eyx[PX(i - 1, j, k)];
            for (int i = Nx - L - 1; i < Nx - 1; i++) {
                for (int j = 0; j < Ny; j++)
                    for (int k = 1; k < Nz; k++)
                        Ey[I3(i, j, k)] = Ey[I3(i, j, k)] - c2e0 * P_eyx[PX(i - xshift, j, k)];
                Eyinc[i] = Eyinc[i] - c2e0 * P_eyxI[i - xshift];
            }
            for (int i = 1; i < Nx - 1; i++)
                for (int j = 0; j < Ny; j++) {
                    for (int k = 1; k < L + 1; k++)
                        Ey[I3(i, j, k)] = Ey[I3(i, j, k)] + c2e0 * P_eyz[PZ(i, j, k - 1)];
                    for (int k = Nz - L - 1; k < Nz - 1; k++)
                        Ey[I3(i, j, k)] = Ey[I3(i, j, k)] + c2e0 * P_eyz[PZ(i, j, k - zshift)];
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
            Ezinc[i] = c1e0 * Ezinc[i] + c2e0 * (Hyinc[i] - Hyinc[i - 1]) / dx;
        }
        for (int j = by1; j < by2; j++)
            for (int k = bz1; k < bz2; k++) {
                Ez[I3(bx1, j, k)] = Ez[I3(bx1, j, k)] - c2e0 * Hyinc[bx1 - 1] / dx;
                Ez[I3(bx2 - 1, j, k)] = Ez[I3(bx2 - 1, j, k)] + c2e0 * Hyinc[bx2 - 1] / dx;
            }

        /* ---------------- source, R21:1278-1304 ---------------- */
        switch (in.sourcepol) {
        case 2: Ezinc[0] = 0; Eyinc[0] = EsA[t]; break;
        case 3: Ezinc[0] = EsA[t]; Eyinc[0] = EsA[t]; break;
        case 4: Ezinc[0] = EsA[t]; Eyinc[0] = EsB[t]; break;
        case 5: Ezinc[0] = EsB[t]; Eyinc[0] = EsA[t]; break;
        default: Ezinc[0] = EsA[t]; Eyinc[0] = 0; break; /* 1 and others */
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
                        Ez[I3(i, j, k)] = Ez[I3(i, j, k)] + c2e0 * P_ezx[PX(i - 1, j, k)];
            for (int i = Nx - L - 1; i < Nx - 1; i++) {
                for (int j = 1; j < Ny; j++)
                    for (int k = 0; k < Nz; k++)
                        Ez[I3(i, j, k)] = Ez[I3(i, j, k)] + c2e0 * P_ezx[PX(i - xshift, j, k)];
                Ezinc[i] = Ezinc[i] + c2e0 * P_ezxI[i - xshift];
            }
            for (int i = 1; i < Nx - 1; i++) {
                for (int j = 1; j < L + 1; j++)
                    for (int k = 0; k < Nz - 1; k++)
                        Ez[I3(i, j, k)] = Ez[I3(i, j, k)] - c2e0 * P_ezy[PY(i, j - 1, k)];
                for (int j = Ny - L - 1; j < Ny - 1; j++)
                    for (int k = 0; k < Nz - 1; k++)
                        Ez[I3(i, j, k)] = Ez[I3(i, j, k)] - c2e0 * P_ezy[PY(i, j - yshift, k)];
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
                        double m0 = (Ex[c] + Ex[I3(i - 1, j, k)]) / 2;
                        double m1 = (Ey[c] + Ey[I3(i, j - 1, k)]) / 2;
                        double m2 = (Ez[c] + Ez[I3(i, j, k - 1)]) / 2;
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
