// problem.cpp -- input parsing and host-side set-up tables.
//
// Everything here runs once per simulation on the host.  The arithmetic keeps
// the reference's expression trees (this file is compiled with
// -ffp-contract=off) and calls the same libm functions, so the coefficients
// the device uses are bit-identical to the reference's.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <unordered_map>

#include "common.hpp"

namespace mfdtd {

namespace {

// Solver constants, source/meteor-2.1.cpp:12-18.
constexpr double kPI = 3.141592653589793;
constexpr double kQE = 1.602177e-19;
constexpr double kE0 = 8.85419e-12;
constexpr double kU0 = 1.2566e-6;
constexpr double kME = 9.10939e-31;
constexpr double kC = 3.0000e8;

struct Reader {
    std::vector<unsigned char> buf;
    size_t off = 0;
    std::string name;
    template <class T> T get() {
        if (off + sizeof(T) > buf.size())
            throw Error(MFDTD_EIO, name + ": file ends early at byte " + std::to_string(off));
        T v;
        std::memcpy(&v, buf.data() + off, sizeof(T));
        off += sizeof(T);
        return v;
    }
    bool has(size_t n) const { return off + n <= buf.size(); }
};

std::vector<unsigned char> slurp(const std::string &path) {
    FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) throw Error(MFDTD_EIO, "cannot open " + path);
    std::vector<unsigned char> b;
    unsigned char tmp[1 << 16];
    size_t n;
    while ((n = std::fread(tmp, 1, sizeof tmp, f)) > 0) b.insert(b.end(), tmp, tmp + n);
    std::fclose(f);
    return b;
}

bool file_exists(const std::string &path) {
    FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) return false;
    std::fclose(f);
    return true;
}

// Optional extended inputs of a run directory: ext.dat (88 bytes, layout in
// rundir.py write_ext) and the per-cell maps it announces.  The reference
// never writes these files, so its run directories are unaffected.
void read_ext_sidecars(const std::string &dir, Problem &P) {
    // trail.dat: 8-byte magic then 12 doubles (centre[3], axis[3], r0,
    // log10n_lo, log10n_hi, s_half, 0, 0).
    const std::string tpath = dir + "/trail.dat";
    if (file_exists(tpath)) {
        Reader r;
        r.name = tpath;
        r.buf = slurp(tpath);
        if (r.buf.size() < 8 || std::memcmp(r.buf.data(), "MFDTDT01", 8) != 0)
            throw Error(MFDTD_EIO, tpath + ": not a trail file (bad magic)");
        r.off = 8;
        mfdtd_trail t;
        for (double &v : t.centre) v = r.get<double>();
        for (double &v : t.axis) v = r.get<double>();
        t.r0 = r.get<double>();
        t.log10n_lo = r.get<double>();
        t.log10n_hi = r.get<double>();
        t.s_half = r.get<double>();
        P.trail = t;
        P.has_trail = 1;
    }
    const std::string path = dir + "/ext.dat";
    if (!file_exists(path)) return;
    Reader r;
    r.name = path;
    r.buf = slurp(path);
    if (r.buf.size() < 8 || std::memcmp(r.buf.data(), "MFDTDX01", 8) != 0)
        throw Error(MFDTD_EIO, path + ": not an extended-input file (bad magic)");
    r.off = 8;
    mfdtd_ext e;
    e.pmllen = r.get<int32_t>();
    e.tfsf_gap = r.get<int32_t>();
    e.ntf_gap = r.get<int32_t>();
    e.oblique = r.get<int32_t>();
    e.exact_coords = r.get<int32_t>();
    const int has_wp3 = r.get<int32_t>();
    const int has_nu3 = r.get<int32_t>();
    e.lk_colocated = r.get<int32_t>();
    e.pml_m = r.get<double>();
    e.kappa_max = r.get<double>();
    e.alpha_max = r.get<double>();
    e.inc_theta = r.get<double>();
    e.inc_phi = r.get<double>();
    e.inc_psi = r.get<double>();
    P.ext = e;
    P.ext_present = 1;
    if (!has_wp3 && !has_nu3) return;
    const size_t n3 = P.cells();
    for (int q = 0; q < 2; q++) {
        if (!(q == 0 ? has_wp3 : has_nu3)) continue;
        Reader w;
        w.name = dir + (q == 0 ? "/wp3.dat" : "/nu3.dat");
        w.buf = slurp(w.name);
        if (w.buf.size() < n3 * 8)
            throw Error(MFDTD_EIO, w.name + ": expected " + std::to_string(n3 * 8) + " bytes");
        std::vector<double> &dst = q == 0 ? P.wp3 : P.nu3;
        dst.resize(n3);
        std::memcpy(dst.data(), w.buf.data(), n3 * 8);
    }
}

// Numerical wavenumber of the 3-D Yee grid along the unit vector u at angular
// frequency w: the root of sum_q (sin(k u_q d_q / 2) / d_q)^2 =
// (sin(w dt / 2) / (c dt))^2 (the Yee dispersion relation), by bisection.
double yee3_wavenumber(double w, double dt, double c, const double d[3], const double u[3]) {
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

// Cell size of a 1-D Yee line whose numerical wavenumber at w equals k:
// the root of sin(k D / 2) / D = sin(w dt / 2) / (c dt), by bisection.
double matched_line_cell(double k, double w, double dt, double c, double dmin, double dmax) {
    const double S = sin(w * dt / 2) / (c * dt);
    double lo = 0.25 * dmin, hi = 2 * dmax;
    for (int it = 0; it < 200; it++) {
        const double mid = 0.5 * (lo + hi);
        if (sin(k * mid / 2) / mid > S) lo = mid;
        else hi = mid;
    }
    return 0.5 * (lo + hi);
}

// CPML recursion tables for slab index m in [L, 2L) (the low side mirrors
// it), source/meteor-2.1.cpp:411-526 with the grading order, kappa_max and
// alpha_max as parameters.  Ke/Kh (may be null) receive 1/kappa - 1.
void cpml_tables(int pmllen, double pmlm, double kamax, double almax, double dx, double dt,
                 double *Be, double *Ae, double *Bh, double *Ah, double *Ke, double *Kh) {
    double simax = 1.5 * (double)(pmlm + 1) / (150 * kPI * dx);
    for (int m = pmllen; m < 2 * pmllen; m++) {
        int n = m - pmllen;
        double mf = (double)n;
        double s = simax * pow(((mf + 0.5) / pmllen), pmlm);
        double sm = simax * pow(((mf + 1) / pmllen), pmlm);
        double ka = 1 + (kamax - 1) * pow(((mf + 0.5) / pmllen), pmlm);
        double kam = 1 + (kamax - 1) * pow(((mf + 1) / pmllen), pmlm);
        double al = almax * pow(((pmllen - mf - 0.5) / pmllen), pmlm);
        double alm = almax * pow(((pmllen - mf - 1) / pmllen), pmlm);
        Be[m] = exp(-((s / ka) + al) * dt / kE0);
        Ae[m] = s / (s * ka + pow(ka, 2) * al) * (Be[m] - 1);
        Bh[m] = exp(-((sm / kam) + alm) * dt / kE0);
        Ah[m] = sm / (sm * kam + pow(kam, 2) * alm) * (Bh[m] - 1);
        if (Ke) Ke[m] = 1 / ka - 1;
        if (Kh) Kh[m] = 1 / kam - 1;
    }
    for (int m = 0; m < pmllen; m++) {
        Be[m] = Be[2 * pmllen - 1 - m]; Ae[m] = Ae[2 * pmllen - 1 - m];
        Bh[m] = Bh[2 * pmllen - 1 - m]; Ah[m] = Ah[2 * pmllen - 1 - m];
        if (Ke) Ke[m] = Ke[2 * pmllen - 1 - m];
        if (Kh) Kh[m] = Kh[2 * pmllen - 1 - m];
    }
}

}  // namespace

void ext_defaults(mfdtd_ext &e) {
    std::memset(&e, 0, sizeof e);
    e.pmllen = 10;
    e.tfsf_gap = 10;
    e.ntf_gap = 5;
    e.pml_m = 4;
    e.kappa_max = 1;
    e.alpha_max = 0;
    e.inc_theta = kPI / 2;
}

// inputs.dat: source/meteor-2.1.cpp:84-112, doB0 source/meteor-fork.cpp:115.
Problem problem_from_rundir(const std::string &dir) {
    Problem P;
    Reader r;
    r.name = dir + "/inputs.dat";
    r.buf = slurp(r.name);
    P.dopml = r.get<int32_t>();
    P.savefields = r.get<int32_t>();
    P.f0 = r.get<double>();
    P.fsig = r.get<double>();
    P.sourcetype = r.get<int32_t>();
    P.sourcepol = r.get<int32_t>();
    P.gridfactor = r.get<double>();
    P.dt = r.get<double>();
    P.tsteps = r.get<int32_t>();
    P.Nx = r.get<int32_t>();
    P.Ny = r.get<int32_t>();
    P.Nz = r.get<int32_t>();
    P.metsize[0] = r.get<double>();
    P.metsize[1] = r.get<double>();
    P.wpmax = r.get<double>();
    P.numax = r.get<double>();
    for (double &v : P.metloc) v = r.get<double>();
    P.metangle = r.get<double>();
    P.mettype = r.get<int32_t>();
    P.numfiles = r.get<int32_t>();
    int np = r.get<int32_t>();
    if (np < 0 || !r.has((size_t)np * 12)) throw Error(MFDTD_EIO, r.name + ": bad nprobes");
    P.probex.resize(np); P.probey.resize(np); P.probez.resize(np);
    for (auto &v : P.probex) v = r.get<int32_t>();
    for (auto &v : P.probey) v = r.get<int32_t>();
    for (auto &v : P.probez) v = r.get<int32_t>();
    int nntf = r.get<int32_t>();
    if (nntf < 1 || !r.has((size_t)nntf * 8)) throw Error(MFDTD_EIO, r.name + ": bad nntf");
    P.fntf.resize(nntf);
    for (auto &v : P.fntf) v = r.get<double>();
    P.doplate = r.get<int32_t>();
    P.platesize = r.get<double>();
    if (r.has(4)) { P.doB0 = r.get<int32_t>(); P.doB0_present = 1; }
    else { P.doB0 = 0; P.doB0_present = 0; }  // MATLAB-written file: no doB0

    // B0.dat, source/meteor-fork.cpp:219-224
    Reader b;
    b.name = dir + "/B0.dat";
    b.buf = slurp(b.name);
    for (double &v : P.B) v = b.get<double>();

    if (P.Nx <= 0 || P.Ny <= 0 || P.Nz <= 0 || (size_t)P.Nx * P.Ny > (size_t)1 << 34)
        throw Error(MFDTD_EINVAL, "inputs.dat: bad grid size");
    size_t n2 = (size_t)P.Nx * P.Ny;
    for (int q = 0; q < 2; q++) {
        Reader w;
        w.name = dir + (q == 0 ? "/wp.dat" : "/nu.dat");
        w.buf = slurp(w.name);
        if (w.buf.size() < n2 * 8)
            throw Error(MFDTD_EIO, w.name + ": expected " + std::to_string(n2 * 8) + " bytes");
        std::vector<double> &dst = q == 0 ? P.wp2 : P.nu2;
        dst.resize(n2);
        std::memcpy(dst.data(), w.buf.data(), n2 * 8);
    }
    read_ext_sidecars(dir, P);
    P.derive();
    return P;
}

Problem problem_from_params(const mfdtd_params &p, const double *wp2, const double *nu2,
                            const double B0[3]) {
    Problem P;
    P.dopml = p.dopml; P.savefields = p.savefields; P.f0 = p.f0; P.fsig = p.fsig;
    P.sourcetype = p.sourcetype; P.sourcepol = p.sourcepol; P.gridfactor = p.gridfactor;
    P.dt = p.dt; P.tsteps = p.tsteps; P.Nx = p.Nx; P.Ny = p.Ny; P.Nz = p.Nz;
    P.metsize[0] = p.metsize[0]; P.metsize[1] = p.metsize[1]; P.wpmax = p.wpmax;
    P.numax = p.numax;
    for (int q = 0; q < 3; q++) P.metloc[q] = p.metloc[q];
    P.metangle = p.metangle; P.mettype = p.mettype; P.numfiles = p.numfiles;
    if (p.nprobes < 0 || (p.nprobes > 0 && (!p.probex || !p.probey || !p.probez)))
        throw Error(MFDTD_EINVAL, "probe arrays missing");
    P.probex.assign(p.probex, p.probex + p.nprobes);
    P.probey.assign(p.probey, p.probey + p.nprobes);
    P.probez.assign(p.probez, p.probez + p.nprobes);
    if (p.nntf < 1 || !p.fntf) throw Error(MFDTD_EINVAL, "nntf must be >= 1 with fntf given");
    P.fntf.assign(p.fntf, p.fntf + p.nntf);
    P.doplate = p.doplate; P.platesize = p.platesize; P.doB0 = p.doB0; P.doB0_present = 1;
    if (!B0 || !wp2 || !nu2) throw Error(MFDTD_EINVAL, "wp2/nu2/B0 must not be NULL");
    for (int q = 0; q < 3; q++) P.B[q] = B0[q];
    if (P.Nx <= 0 || P.Ny <= 0 || P.Nz <= 0) throw Error(MFDTD_EINVAL, "bad grid size");
    size_t n2 = (size_t)P.Nx * P.Ny;
    P.wp2.assign(wp2, wp2 + n2);
    P.nu2.assign(nu2, nu2 + n2);
    P.derive();
    return P;
}

void Problem::derive() {
    if (!ext_present) ext_defaults(ext);
    if (has_trail) {
        const double an = sqrt(trail.axis[0] * trail.axis[0] + trail.axis[1] * trail.axis[1] +
                               trail.axis[2] * trail.axis[2]);
        if (!(an > 0) || !(trail.r0 > 0) || !(trail.s_half > 0) || !std::isfinite(trail.log10n_lo) ||
            !std::isfinite(trail.log10n_hi) || trail.log10n_lo > 30 || trail.log10n_hi > 30)
            throw Error(MFDTD_EINVAL, "trail: need a nonzero axis, r0 > 0, s_half > 0 and "
                                      "log10 densities <= 30");
        for (double &v : trail.axis) v = v / an;
    }
    L = ext.pmllen;  // source/meteor-2.1.cpp:343 (10)
    if (ext_present) {
        if (L < 1 || L > kMaxPml) throw Error(MFDTD_EINVAL, "pmllen must be in [1, 32]");
        if (ext.tfsf_gap < 2 || ext.ntf_gap < 1 || ext.ntf_gap > ext.tfsf_gap - 2)
            throw Error(MFDTD_EINVAL, "need tfsf_gap >= 2 and 1 <= ntf_gap <= tfsf_gap - 2 "
                                      "(Huygens surface between the CPML and the TF/SF box)");
        if (!(ext.pml_m >= 0) || !(ext.kappa_max >= 1) || !(ext.alpha_max >= 0))
            throw Error(MFDTD_EINVAL, "need pml_m >= 0, kappa_max >= 1, alpha_max >= 0");
        const int need = 2 * (L + ext.tfsf_gap) + 3;
        if (Nx < need || Ny < need || Nz < need)
            throw Error(MFDTD_EINVAL, "grid must be at least " + std::to_string(need) +
                                          " cells along each axis for this CPML and TF/SF box");
        if (!wp3.empty() && wp3.size() != cells())
            throw Error(MFDTD_EINVAL, "wp3 must hold Nx*Ny*Nz values");
        if (!nu3.empty() && nu3.size() != cells())
            throw Error(MFDTD_EINVAL, "nu3 must hold Nx*Ny*Nz values");
    }
    if (Nx < 2 * L + 2 || Ny < 2 * L + 2 || Nz < 2 * L + 2)
        throw Error(MFDTD_EINVAL, "grid must be at least 22 cells along each axis "
                                  "(two 10-cell CPML slabs that do not overlap)");
    if (tsteps < 1) throw Error(MFDTD_EINVAL, "tsteps must be >= 1");
    if (numfiles < 1 || tsteps / numfiles < 1)
        throw Error(MFDTD_EINVAL, "numfiles must be in [1, tsteps] (the reference divides "
                                  "by tsteps/numfiles)");
    if (fntf.empty()) throw Error(MFDTD_EINVAL, "nntf must be >= 1");
    if (!(dt > 0) || !(f0 > 0) || !(gridfactor > 0))
        throw Error(MFDTD_EINVAL, "dt, f0 and gridfactor must be positive");
    for (size_t n = 0; n < probex.size(); n++)
        if (probex[n] < 1 || probex[n] >= Nx || probey[n] < 1 || probey[n] >= Ny ||
            probez[n] < 1 || probez[n] >= Nz)
            throw Error(MFDTD_EINVAL, "probe " + std::to_string(n) +
                                          " outside [1, N-1) (its stencil reads index-1)");
    record_period = tsteps / numfiles;

    // Grid, source/meteor-2.1.cpp:116-147.  y[] and z[] are filled for index < Nx
    // only, like the reference; entries beyond are 0 here.
    double lambda = kC / f0;
    dx = lambda / gridfactor;
    dy = lambda / gridfactor;
    dz = lambda / gridfactor;
    int nmax = std::max(Nx, std::max(Ny, Nz));
    x.assign(nmax, 0.0); y.assign(nmax, 0.0); z.assign(nmax, 0.0);
    if (ext.exact_coords) {
        for (int i = 0; i < Nx; i++) x[i] = -(Nx - 1) / 2.0 * dx + dx * i;
        for (int i = 0; i < Ny; i++) y[i] = -(Ny - 1) / 2.0 * dy + dy * i;
        for (int i = 0; i < Nz; i++) z[i] = -(Nz - 1) / 2.0 * dz + dz * i;
    } else {
        for (int i = 0; i < Nx; i++) {
            x[i] = -(Nx - 1) / 2 * dx + dx * i;
            y[i] = -(Ny - 1) / 2 * dy + dy * i;
            z[i] = -(Nz - 1) / 2 * dz + dz * i;
        }
    }
    ssx = (Nx + 1) / 2;
    ssy = (Ny + 1) / 2;
    ssz = (Nz + 1) / 2;

    // Source, source/meteor-2.1.cpp:152-175, polarisation :1278-1304.
    src.assign((size_t)tsteps * 2, 0.0);
    {
        const double PI = kPI;
        double rdelayA = 1.6 * sqrt(6) / PI / f0;
        double rdelayB = (1.6 + 1 / sqrt(3)) * sqrt(6) / PI / f0;
        for (int t = 0; t < tsteps; t++) {
            double A, B;
            if (sourcetype == 2) {
                A = sin(2 * PI * f0 * (t - 3 * fsig) * dt) * exp(-(t - 3 * fsig) * (t - 3 * fsig) / (2 * fsig * fsig));
                B = cos(2 * PI * f0 * (t - 3 * fsig) * dt) * exp(-(t - 3 * fsig) * (t - 3 * fsig) / (2 * fsig * fsig));
            } else if (sourcetype == 3) {
                A = (1 - 2 * PI * PI * f0 * f0 * (t * dt - rdelayA) * (t * dt - rdelayA)) * exp(-PI * PI * f0 * f0 * (t * dt - rdelayA) * (t * dt - rdelayA));
                B = (1 - 2 * PI * PI * f0 * f0 * (t * dt - rdelayB) * (t * dt - rdelayB)) * exp(-PI * PI * f0 * f0 * (t * dt - rdelayB) * (t * dt - rdelayB));
            } else {
                A = sin(2 * PI * f0 * t * dt);
                B = cos(2 * PI * f0 * t * dt);
            }
            double ez, ey;
            if (ext.oblique) {  // one waveform on the auxiliary line
                src[2 * t] = A;
                src[2 * t + 1] = 0;
                continue;
            }
            switch (sourcepol) {
            case 2: ez = 0; ey = A; break;
            case 3: ez = A; ey = A; break;
            case 4: ez = A; ey = B; break;
            case 5: ez = B; ey = A; break;
            default: ez = A; ey = 0; break;
            }
            src[2 * t] = ez;
            src[2 * t + 1] = ey;
        }
    }

    // Running-DFT phase factors.  The reference evaluates sin/cos(2*PI*f*t*dt)
    // inline for both halves of the step (source/meteor-2.1.cpp:947,1380,1393;
    // (t+1/2) is integer arithmetic and equals t).
    const int nf = nntf();
    phase.assign((size_t)tsteps * nf * 2, 0.0);
    {
        const double PI = kPI;
        for (int t = 0; t < tsteps; t++)
            for (int m = 0; m < nf; m++) {
                phase[((size_t)t * nf + m) * 2] = sin(2 * PI * fntf[m] * t * dt);
                phase[((size_t)t * nf + m) * 2 + 1] = cos(2 * PI * fntf[m] * t * dt);
            }
        // Source DFT (source/meteor-2.1.cpp:1378-1383): a function of the
        // injected values only, so it is summed here.  Starts at zero (the
        // reference leaves these sums uninitialised).
        srcdft.assign((size_t)4 * nf, 0.0);
        double *Eydft = srcdft.data(), *Ezdft = srcdft.data() + 2 * nf;
        for (int t = 0; t < tsteps; t++)
            for (int m = 0; m < nf; m++) {
                double s = sin(2 * PI * fntf[m] * (t + 1 / 2) * dt);
                double c = cos(2 * PI * fntf[m] * (t + 1 / 2) * dt);
                Ezdft[2 * m] += src[2 * t] * s;
                Ezdft[2 * m + 1] += src[2 * t] * c;
                Eydft[2 * m] += src[2 * t + 1] * s;
                Eydft[2 * m + 1] += src[2 * t + 1] * c;
            }
    }

    // Update coefficients, source/meteor-2.1.cpp:180-206.
    const double sigm = 0, sig = 0;
    c1h = (2 * kU0 - sigm * dt) / (2 * kU0 + sigm * dt);
    c2h = 2 * dt / (2 * kU0 + sigm * dt);
    c1e0 = (2 * kE0 - sig * dt) / (2 * kE0 + sig * dt);
    c2e0 = 2 * dt / (2 * kE0 + sig * dt);
    c1s = (2 * kE0 - 1e7 * dt) / (2 * kE0 + 1e7 * dt);
    c2s = 2 * dt / (2 * kE0 + 1e7 * dt);

    // Gyrofrequency, source/meteor-fork.cpp:228-232.
    wcex = -kQE * B[0] / kME;
    wcey = -kQE * B[1] / kME;
    wcez = -kQE * B[2] / kME;
    wce0 = sqrt(wcex * wcex + wcey * wcey + wcez * wcez);

    // Plasma maps, source/meteor-2.1.cpp:319-334: wpe = wp2[i][j] * G[k].
    G.assign(Nz, 0.0);
    {
        double msig0 = metsize[0];
        for (int k = 0; k < Nz; k++) G[k] = exp(-pow((z[k] - metloc[2]), 2) / (msig0 * msig0));
    }
    wp2e = wp2;
    nu2e = nu2;
    if (doplate) {
        std::fill(wp2e.begin(), wp2e.end(), 0.0);
        std::fill(nu2e.begin(), nu2e.end(), 0.0);
    }

    // Lee-Kalluri matrices (source/meteor-fork.cpp:1546-1573).  The reference
    // recomputes them per cell per step; they depend only on the cell's
    // collision frequency, so they are tabulated once per distinct value.
    if (doB0) {
        bool nu_uniform = true;
        bool g_one = true;
        if (!nu3.empty()) {  // per-cell map: uniform, or one entry per cell
            for (size_t q = 1; q < nu3.size(); q++)
                if (std::memcmp(&nu3[q], &nu3[0], 8) != 0) { nu_uniform = false; g_one = false; break; }
        } else {
            for (size_t q = 1; q < nu2e.size(); q++)
                if (std::memcmp(&nu2e[q], &nu2e[0], 8) != 0) { nu_uniform = false; break; }
            for (int k = 0; k < Nz; k++)
                if (!(G[k] == 1.0)) { g_one = false; break; }
        }
        if (doplate) nu_uniform = true;  // nue is exactly zero everywhere
        size_t entries;
        if (nu_uniform) { lk_mode = LK_PER_K; entries = Nz; }
        else if (g_one) { lk_mode = LK_PER_IJ; entries = (size_t)Nx * Ny; }
        else { lk_mode = LK_PER_CELL; entries = cells(); }
        if (entries > ((size_t)1 << 25))
            throw Error(MFDTD_ENOMEM, "Lee-Kalluri table would need " + std::to_string(entries) +
                                          " entries (collision frequency varies in all three axes "
                                          "on a large grid)");
        lk.assign(entries * kLkStride, 0.0);
        const double cw = cos(wce0 * dt), sw = sin(wce0 * dt);
        auto fill = [&](double *o, double nu) {
            double Ee1 = exp(-nu * dt);
            double Ee2 = 1 / (wce0 * wce0 + nu * nu);
            double Se1 = sw / wce0;
            double Ce1 = (1 - cw) / (wce0 * wce0);
            double Ce2 = (1 - Ee1) / nu - Ee1 * nu * Ce1 - Ee1 * Se1;
            double Ce3 = nu * (1 - Ee1 * cw) + Ee1 * wce0 * sw;
            double Ce4 = 1 - Ee1 * cw - Ee1 * nu * Se1;
            o[0] = Ee1 * (Ce1 * wcex * wcex + cw);
            o[1] = Ee1 * (Ce1 * wcex * wcey - Se1 * wcez);
            o[2] = Ee1 * (Ce1 * wcex * wcez + Se1 * wcey);
            o[3] = Ee1 * (Ce1 * wcey * wcex + Se1 * wcez);
            o[4] = Ee1 * (Ce1 * wcey * wcey + cw);
            o[5] = Ee1 * (Ce1 * wcey * wcez - Se1 * wcex);
            o[6] = Ee1 * (Ce1 * wcez * wcex - Se1 * wcey);
            o[7] = Ee1 * (Ce1 * wcez * wcey + Se1 * wcex);
            o[8] = Ee1 * (Ce1 * wcez * wcez + cw);
            o[9] = Ee2 * (Ce2 * wcex * wcex + Ce3);
            o[10] = Ee2 * (Ce2 * wcex * wcey - Ce4 * wcez);
            o[11] = Ee2 * (Ce2 * wcex * wcez + Ce4 * wcey);
            o[12] = Ee2 * (Ce2 * wcey * wcex + Ce4 * wcez);
            o[13] = Ee2 * (Ce2 * wcey * wcey + Ce3);
            o[14] = Ee2 * (Ce2 * wcey * wcez - Ce4 * wcex);
            o[15] = Ee2 * (Ce2 * wcez * wcex - Ce4 * wcey);
            o[16] = Ee2 * (Ce2 * wcez * wcey + Ce4 * wcex);
            o[17] = Ee2 * (Ce2 * wcez * wcez + Ce3);
        };
        // The cell value is nu2[i][j] * G[k] (one rounding), as in the reference;
        // with a plate or sphere scatterer it is exactly 0 (memset, :330-334).
        // With a per-cell map the cell value is nu3 itself.
        auto nu_at = [&](size_t ij, int k) {
            if (doplate) return 0.0;
            if (!nu3.empty()) return nu3[ij * Nz + k];
            return nu2e[ij] * G[k];
        };
        if (lk_mode == LK_PER_K) {
            for (int k = 0; k < Nz; k++) fill(&lk[(size_t)k * kLkStride], nu_at(0, k));
        } else if (lk_mode == LK_PER_IJ) {
            for (size_t q = 0; q < (size_t)Nx * Ny; q++) fill(&lk[q * kLkStride], nu_at(q, 0));
        } else {
            for (int i = 0; i < Nx; i++)
                for (int j = 0; j < Ny; j++)
                    for (int k = 0; k < Nz; k++)
                        fill(&lk[(((size_t)i * Ny + j) * Nz + k) * kLkStride],
                             nu_at((size_t)i * Ny + j, k));
        }
    }

    // CPML, source/meteor-2.1.cpp:411-526 (reference: m=4, kappa=1, alpha=0;
    // the H tables also use E0, :478-496).  kappa != 1 adds a (1/kappa - 1)
    // derivative term to each CPML correction (the reference's field update
    // has no 1/kappa factor).
    Be.assign(2 * L, 0.0); Ae.assign(2 * L, 0.0); Bh.assign(2 * L, 0.0); Ah.assign(2 * L, 0.0);
    Ke.assign(2 * L, 0.0); Kh.assign(2 * L, 0.0);
    kappa_on = dopml && ext.kappa_max != 1.0;
    if (dopml)
        cpml_tables(L, ext.pml_m, ext.kappa_max, ext.alpha_max, dx, dt, Be.data(), Ae.data(),
                    Bh.data(), Ah.data(), Ke.data(), Kh.data());
    xshift = Nx - 2 * L - 1;
    yshift = Ny - 2 * L - 1;
    zshift = Nz - 2 * L - 1;
    // TF/SF box and NTF surface, source/meteor-2.1.cpp:539-552 (gaps 10, 5).
    bx1 = L + ext.tfsf_gap; bx2 = Nx - L - ext.tfsf_gap;
    by1 = L + ext.tfsf_gap; by2 = Ny - L - ext.tfsf_gap;
    bz1 = L + ext.tfsf_gap; bz2 = Nz - L - ext.tfsf_gap;
    ntfb = L + ext.ntf_gap;

    // Oblique incidence: a 1-D auxiliary Yee line along k whose cell size dl
    // matches the 3-D grid's numerical wavenumber along k at f0 (matched
    // numerical dispersion), so the injected wave and the grid's own wave
    // travel at the same speed.  The incident field at a node of doubled
    // coordinates P is the line's value at s = kr . (P/2) + s0 (linear
    // interpolation).  The line ends in an L-cell CPML.
    oblique = ext.oblique ? 1 : 0;
    if (oblique) {
        const double th = ext.inc_theta, ph = ext.inc_phi, ps = ext.inc_psi;
        inc_k[0] = sin(th) * cos(ph); inc_k[1] = sin(th) * sin(ph); inc_k[2] = cos(th);
        const double tht[3] = {cos(th) * cos(ph), cos(th) * sin(ph), -sin(th)};
        const double phh[3] = {-sin(ph), cos(ph), 0.0};
        for (int q = 0; q < 3; q++) inc_e[q] = cos(ps) * (-tht[q]) + sin(ps) * phh[q];
        inc_h[0] = inc_k[1] * inc_e[2] - inc_k[2] * inc_e[1];
        inc_h[1] = inc_k[2] * inc_e[0] - inc_k[0] * inc_e[2];
        inc_h[2] = inc_k[0] * inc_e[1] - inc_k[1] * inc_e[0];
        const double c = 1 / sqrt(kU0 * kE0);
        const double d3[3] = {dx, dy, dz};
        const double w = 2 * kPI * f0;
        const double k3 = yee3_wavenumber(w, dt, c, d3, inc_k);
        dl = matched_line_cell(k3, w, dt, c, std::min(dx, std::min(dy, dz)), std::max(dx, std::max(dy, dz)));
        if (!(c * dt < dl))
            throw Error(MFDTD_EINVAL, "oblique incidence: the auxiliary line would be unstable "
                                      "(grid too coarse for f0)");
        for (int q = 0; q < 3; q++) kr[q] = inc_k[q] * d3[q] / dl;
        // Line node 0 sits at the grid corner the wave enters first, so a wave
        // along +x sees the line at s = x index, as the reference's line does.
        const int gx[2] = {0, Nx - 1}, gy[2] = {0, Ny - 1}, gz[2] = {0, Nz - 1};
        const int cx[2] = {bx1 - 1, bx2}, cy[2] = {by1 - 1, by2}, cz[2] = {bz1 - 1, bz2};
        double gmin = 1e300, pmax = -1e300;
        for (int a = 0; a < 2; a++)
            for (int b = 0; b < 2; b++)
                for (int e = 0; e < 2; e++) {
                    gmin = std::min(gmin, kr[0] * gx[a] + kr[1] * gy[b] + kr[2] * gz[e]);
                    pmax = std::max(pmax, kr[0] * cx[a] + kr[1] * cy[b] + kr[2] * cz[e]);
                }
        s0 = -gmin;
        M = (int)ceil(pmax + s0) + 6 + L;
        ashift = M - 2 * L - 1;
        // Every node that can carry a correction lies in the box [b1-1, b2]^3,
        // so its s lies between the extremes over that box's corners; the
        // interpolation reads line nodes floor(s - 1/2) .. floor(s) + 2.
        double smin = 1e300, smax = -1e300;
        for (int a = 0; a < 2; a++)
            for (int b = 0; b < 2; b++)
                for (int e = 0; e < 2; e++) {
                    const double sc = kr[0] * cx[a] + kr[1] * cy[b] + kr[2] * cz[e] + s0;
                    smin = std::min(smin, sc);
                    smax = std::max(smax, sc);
                }
        if (!(smin >= 1.0) || !(smax + 3 <= M - L - 2))
            throw Error(MFDTD_EINVAL, "oblique incidence: TF/SF box outside the auxiliary line");
        Be1.assign(2 * L, 0.0); Ae1.assign(2 * L, 0.0); Bh1.assign(2 * L, 0.0); Ah1.assign(2 * L, 0.0);
        cpml_tables(L, ext.pml_m, 1.0, 0.0, dl, dt, Be1.data(), Ae1.data(), Bh1.data(), Ah1.data(),
                    nullptr, nullptr);
    }
    // Plate, source/meteor-2.1.cpp:1308-1309.
    plate_lo = (int)(ssy - platesize / 2 / dy);
    plate_up = (int)(ssy + platesize / 2 / dy);
    if (doplate == 1 &&
        (plate_lo < 0 || plate_up > std::min(Ny, Nz) || plate_lo >= plate_up))
        throw Error(MFDTD_EINVAL, "plate does not fit inside the grid");
}

}  // namespace mfdtd
