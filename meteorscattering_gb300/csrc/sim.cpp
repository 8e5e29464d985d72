// sim.cpp -- device-resident simulation, output writers and the C ABI.
#include <cuda_runtime.h>
#include <sys/resource.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "common.hpp"
#include "farfield.hpp"
#include "fp32.hpp"

using mfdtd::Error;
using mfdtd::Problem;

struct mfdtd_problem {
    Problem P;
};

namespace mfdtd {
namespace {

thread_local std::string g_last_error;

void ck(cudaError_t e, const char *what) {
    if (e != cudaSuccess)
        throw Error(MFDTD_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

double wall_s() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

// One record step's output (source/meteor-2.1.cpp:1523-1568).
struct Record {
    int t = 0;
    double emax = 0;
    std::vector<double> E, H;  // slices + incident arrays, file layout
};

// Appends records to the run directory like the reference does.
struct FileSink {
    std::string dir;
    void append(const std::string &name, const void *p, size_t bytes) {
        std::string path = dir + "/" + name;
        FILE *f = std::fopen(path.c_str(), "ab");
        if (!f) throw Error(MFDTD_EIO, "cannot append to " + path);
        if (bytes && std::fwrite(p, 1, bytes, f) != bytes) {
            std::fclose(f);
            throw Error(MFDTD_EIO, "short write to " + path);
        }
        std::fclose(f);
    }
    void log(const std::string &line) {
        std::string path = dir + "/log.txt";
        FILE *f = std::fopen(path.c_str(), "a");
        if (!f) throw Error(MFDTD_EIO, "cannot append to " + path);
        std::fputs(line.c_str(), f);
        std::fclose(f);
    }
};

std::string fmt_g(double v) {
    char b[64];
    std::snprintf(b, sizeof b, "%g", v);
    return b;
}

}  // namespace

void set_last_error(const std::string &msg) { g_last_error = msg; }

}  // namespace mfdtd

struct mfdtd_batch;

struct mfdtd_sim {
    Problem P;
    mfdtd_batch *batch = nullptr;  // set while the simulation is a batch member
    mfdtd_run_opts opts{};
    int form = MFDTD_FORM_FP64_PLAIN;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::vector<void *> allocs;
    int64_t device_bytes = 0;
    mfdtd::PlainArgs pa{};
    std::unique_ptr<mfdtd::Fp32Sim> f32;
    int t = 0;
    bool flushed = false;
    std::vector<mfdtd::Record> records;
    mfdtd::FileSink *sink = nullptr;
    double loop_start = 0;
    double last_ms_per_step = 0;
    int64_t last_launches = 0;
    // opts.profile: per-kernel-class totals of the last advance
    std::vector<std::string> kname;
    std::vector<double> ktotal_ms;
    std::vector<int64_t> kcount;
    std::vector<cudaEvent_t> kev;  // event pool, (classes+1) per profiled step
    size_t slice_len = 0;  // doubles in one slice block (3 planes x 2 comps)
    // Record steps in flight, two deep: each is staged in device memory on
    // the simulation's stream, copied to pinned host memory on copy_stream,
    // and finished (log line, file appends, collection) when its slot comes
    // round again or when the advance ends -- so the host's file writes
    // overlap the following steps.
    struct RecSlot {
        double *dE = nullptr, *dH = nullptr, *hE = nullptr, *hH = nullptr;
        unsigned long long *dbits = nullptr, *hbits = nullptr;
        cudaEvent_t staged = nullptr, copied = nullptr;
        int t = -1;
        bool collect = false, busy = false;
    };
    RecSlot rslot[2];
    int rnext = 0;  // slot of the next record
    cudaStream_t copy_stream = nullptr;

    template <class T> T *dalloc(size_t n) {
        void *p = nullptr;
        size_t bytes = std::max<size_t>(n, 1) * sizeof(T);
        mfdtd::ck(cudaMalloc(&p, bytes), "cudaMalloc");
        allocs.push_back(p);
        device_bytes += (int64_t)bytes;
        mfdtd::ck(cudaMemsetAsync(p, 0, bytes, stream), "cudaMemset");
        return (T *)p;
    }
    template <class T> T *upload(const std::vector<T> &v) {
        T *d = dalloc<T>(v.size());
        if (!v.empty())
            mfdtd::ck(cudaMemcpyAsync(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, stream),
                      "cudaMemcpy H2D");
        return d;
    }

    void init(const Problem &pb, const mfdtd_run_opts *o) {
        P = pb;
        if (o) opts = *o;
        form = opts.form;
        mfdtd::ck(cudaSetDevice(opts.device), "cudaSetDevice");
        mfdtd::ck(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "cudaStreamCreate");
        mfdtd::ck(cudaEventCreate(&ev0), "cudaEventCreate");
        mfdtd::ck(cudaEventCreate(&ev1), "cudaEventCreate");
        slice_len = 2 * ((size_t)P.Nx * P.Ny + (size_t)P.Nx * P.Nz + (size_t)P.Ny * P.Nz);
        if (form == MFDTD_FORM_FP64_PLAIN) init_plain();
        else if (form == MFDTD_FORM_FP32_FUSED) {
            f32.reset(new mfdtd::Fp32Sim());
            f32->init(P, stream);
            device_bytes = f32->device_bytes();
        } else throw Error(MFDTD_EINVAL, "unknown form");
        mfdtd::ck(cudaStreamSynchronize(stream), "set-up");
    }

    void init_plain() {
        const size_t NC = P.cells();
        mfdtd::PlainArgs &a = pa;
        std::memset(&a, 0, sizeof a);
        a.Nx = P.Nx; a.Ny = P.Ny; a.Nz = P.Nz; a.L = P.L;
        a.xshift = P.xshift; a.yshift = P.yshift; a.zshift = P.zshift;
        a.bx1 = P.bx1; a.bx2 = P.bx2; a.by1 = P.by1; a.by2 = P.by2; a.bz1 = P.bz1; a.bz2 = P.bz2;
        a.ntfb = P.ntfb; a.nntf = P.nntf(); a.ssx = P.ssx; a.ssy = P.ssy; a.ssz = P.ssz;
        a.dopml = P.dopml; a.doplate = P.doplate; a.doB0 = P.doB0; a.lk_mode = P.lk_mode;
        a.plate_lo = P.plate_lo; a.plate_up = P.plate_up; a.nprobes = P.nprobes();
        a.tsteps = P.tsteps;
        a.dx = P.dx; a.dy = P.dy; a.dz = P.dz; a.c1h = P.c1h; a.c2h = P.c2h;
        a.c1e0 = P.c1e0; a.c2e0 = P.c2e0; a.c1s = P.c1s; a.c2s = P.c2s;
        a.platesize = P.platesize; a.dt = P.dt;
        for (int m = 0; m < 2 * P.L; m++) {
            a.Be[m] = P.Be[m]; a.Ae[m] = P.Ae[m]; a.Bh[m] = P.Bh[m]; a.Ah[m] = P.Ah[m];
            a.Ke[m] = P.Ke[m]; a.Kh[m] = P.Kh[m];
        }
        a.kappa_on = P.kappa_on;
        a.oblique = P.oblique;
        a.lk_colocated = P.ext.lk_colocated;
        if (P.oblique) {
            a.M = P.M; a.ashift = P.ashift; a.s0 = P.s0; a.dl = P.dl;
            for (int q = 0; q < 3; q++) { a.ke[q] = P.inc_e[q]; a.kh[q] = P.inc_h[q]; a.kr[q] = P.kr[q]; }
            for (int m = 0; m < 2 * P.L; m++) {
                a.Be1[m] = P.Be1[m]; a.Ae1[m] = P.Ae1[m]; a.Bh1[m] = P.Bh1[m]; a.Ah1[m] = P.Ah1[m];
            }
        }
        double **f[9] = {&a.Ex, &a.Ey, &a.Ez, &a.Hx, &a.Hy, &a.Hz, &a.Jx, &a.Jy, &a.Jz};
        for (auto p : f) *p = dalloc<double>(NC);
        const size_t L2 = 2 * (size_t)P.L;
        const size_t nxs = L2 * P.Ny * P.Nz, nys = (size_t)P.Nx * L2 * P.Nz, nzs = (size_t)P.Nx * P.Ny * L2;
        if (P.dopml) {
            a.Phxy = dalloc<double>(nys); a.Phxz = dalloc<double>(nzs); a.Phyx = dalloc<double>(nxs);
            a.Phyz = dalloc<double>(nzs); a.Phzx = dalloc<double>(nxs); a.Phzy = dalloc<double>(nys);
            a.Pexy = dalloc<double>(nys); a.Pexz = dalloc<double>(nzs); a.Peyx = dalloc<double>(nxs);
            a.Peyz = dalloc<double>(nzs); a.Pezx = dalloc<double>(nxs); a.Pezy = dalloc<double>(nys);
        }
        // Incident line: the reference's x-directed line has Nx nodes; the
        // oblique auxiliary line keeps its E in Ezinc and its H in Hyinc.
        const size_t nline = std::max<size_t>(P.Nx, P.oblique ? (size_t)P.M : 0);
        a.Eyinc = dalloc<double>(nline); a.Ezinc = dalloc<double>(nline);
        a.Hyinc = dalloc<double>(nline); a.Hzinc = dalloc<double>(nline);
        a.PeyxI = dalloc<double>(L2); a.PezxI = dalloc<double>(L2);
        a.PhyxI = dalloc<double>(L2); a.PhzxI = dalloc<double>(L2);
        a.wp2 = upload(P.wp2e); a.nu2 = upload(P.nu2e); a.G = upload(P.G);
        if (P.has_trail) {  // omega_p of the parametric trail, evaluated on the device
            double *w = dalloc<double>(NC);
            mfdtd::trail_map_fp64(P, w, stream);
            mfdtd::ck(cudaGetLastError(), "trail map");
            a.wp3 = w;
        } else {
            a.wp3 = P.wp3.empty() ? nullptr : upload(P.wp3);
        }
        a.nu3 = P.nu3.empty() ? nullptr : upload(P.nu3);
        a.xc = upload(P.x); a.yc = upload(P.y); a.zc = upload(P.z);
        a.lk = upload(P.lk); a.src = upload(P.src); a.phase = upload(P.phase);
        const size_t nf2 = 2 * (size_t)P.nntf();
        const size_t fb = (size_t)P.Ny * P.Nz * nf2, tb = (size_t)P.Nx * P.Nz * nf2, lr = (size_t)P.Nx * P.Ny * nf2;
        for (int q = 0; q < 24; q++) a.ntf[q] = dalloc<double>(q < 8 ? fb : q < 16 ? tb : lr);
        a.probe = dalloc<double>((size_t)6 * P.tsteps * P.nprobes());
        std::vector<int> ijk;
        for (int n = 0; n < P.nprobes(); n++) {
            ijk.push_back(P.probex[n]); ijk.push_back(P.probey[n]); ijk.push_back(P.probez[n]);
        }
        a.probe_ijk = upload(ijk);
        a.slE = dalloc<double>(slice_len);
        a.slH = dalloc<double>(slice_len);
        a.emax = dalloc<unsigned long long>(1);
        a.flag = dalloc<unsigned int>(1);
    }

    ~mfdtd_sim() {
        if (stream) cudaStreamSynchronize(stream);
        if (copy_stream) cudaStreamSynchronize(copy_stream);
        for (RecSlot &r : rslot) {
            if (r.dE) cudaFree(r.dE);
            if (r.hE) cudaFreeHost(r.hE);
            if (r.staged) cudaEventDestroy(r.staged);
            if (r.copied) cudaEventDestroy(r.copied);
        }
        if (copy_stream) cudaStreamDestroy(copy_stream);
        for (cudaEvent_t e : kev) cudaEventDestroy(e);
        f32.reset();
        for (void *p : allocs) cudaFree(p);
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        if (stream) cudaStreamDestroy(stream);
    }

    void wait() {
        if (opts.timeout_s > 0) {
            cudaEvent_t e;
            mfdtd::ck(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "cudaEventCreate");
            mfdtd::ck(cudaEventRecord(e, stream), "cudaEventRecord");
            double t0 = mfdtd::wall_s();
            for (;;) {
                cudaError_t q = cudaEventQuery(e);
                if (q == cudaSuccess) break;
                if (q != cudaErrorNotReady) { cudaEventDestroy(e); mfdtd::ck(q, "device"); }
                if (mfdtd::wall_s() - t0 > opts.timeout_s) {
                    cudaEventDestroy(e);
                    throw Error(MFDTD_ETIMEOUT, "device did not finish within timeout_s");
                }
                std::this_thread::sleep_for(std::chrono::microseconds(200));
            }
            cudaEventDestroy(e);
        } else {
            mfdtd::ck(cudaStreamSynchronize(stream), "device");
        }
    }

    // Record step: max|Ex| and the slice/incident arrays after step t.
    void do_record(int tt, bool collect) {
        const size_t Nx = P.Nx, blk = slice_len + 2 * Nx;
        if (!copy_stream) {
            mfdtd::ck(cudaStreamCreateWithFlags(&copy_stream, cudaStreamNonBlocking), "cudaStreamCreate");
            for (RecSlot &r : rslot) {
                mfdtd::ck(cudaMalloc(&r.dE, 2 * blk * 8 + 16), "cudaMalloc");
                r.dH = r.dE + blk;
                r.dbits = (unsigned long long *)(r.dH + blk);
                mfdtd::ck(cudaMallocHost(&r.hE, 2 * blk * 8 + 16), "cudaMallocHost");
                r.hH = r.hE + blk;
                r.hbits = (unsigned long long *)(r.hH + blk);
                mfdtd::ck(cudaEventCreateWithFlags(&r.staged, cudaEventDisableTiming), "cudaEventCreate");
                mfdtd::ck(cudaEventCreateWithFlags(&r.copied, cudaEventDisableTiming), "cudaEventCreate");
            }
        }
        RecSlot &r = rslot[rnext];
        rnext ^= 1;
        if (r.busy) finish_record(r);  // the older of the two in flight
        const cudaMemcpyKind d2d = cudaMemcpyDeviceToDevice;
        if (form == MFDTD_FORM_FP64_PLAIN) {
            mfdtd::plain_launch_emax(pa, stream);
            mfdtd::ck(cudaMemcpyAsync(r.dbits, pa.emax, 8, d2d, stream), "D2D");
            mfdtd::ck(cudaMemcpyAsync(r.dE, pa.slE, slice_len * 8, d2d, stream), "D2D");
            mfdtd::ck(cudaMemcpyAsync(r.dE + slice_len, pa.Eyinc, Nx * 8, d2d, stream), "D2D");
            mfdtd::ck(cudaMemcpyAsync(r.dE + slice_len + Nx, pa.Ezinc, Nx * 8, d2d, stream), "D2D");
            mfdtd::ck(cudaMemcpyAsync(r.dH, pa.slH, slice_len * 8, d2d, stream), "D2D");
            mfdtd::ck(cudaMemcpyAsync(r.dH + slice_len, pa.Hyinc, Nx * 8, d2d, stream), "D2D");
            mfdtd::ck(cudaMemcpyAsync(r.dH + slice_len + Nx, pa.Hzinc, Nx * 8, d2d, stream), "D2D");
        } else {
            f32->record_stage(r.dE, r.dH, (unsigned int *)r.dbits, stream);
        }
        mfdtd::ck(cudaEventRecord(r.staged, stream), "cudaEventRecord");
        mfdtd::ck(cudaStreamWaitEvent(copy_stream, r.staged, 0), "cudaStreamWaitEvent");
        mfdtd::ck(cudaMemcpyAsync(r.hE, r.dE, 2 * blk * 8 + 8, cudaMemcpyDeviceToHost, copy_stream), "D2H");
        mfdtd::ck(cudaEventRecord(r.copied, copy_stream), "cudaEventRecord");
        r.t = tt;
        r.collect = collect;
        r.busy = true;
    }

    // Wait (bounded by opts.timeout_s when set) for a record's copy and emit it.
    void finish_record(RecSlot &rs) {
        if (opts.timeout_s > 0) {
            const double t0 = mfdtd::wall_s();
            for (;;) {
                cudaError_t q = cudaEventQuery(rs.copied);
                if (q == cudaSuccess) break;
                if (q != cudaErrorNotReady) mfdtd::ck(q, "record copy");
                if (mfdtd::wall_s() - t0 > opts.timeout_s)
                    throw Error(MFDTD_ETIMEOUT, "record copy did not finish within timeout_s");
                std::this_thread::sleep_for(std::chrono::microseconds(200));
            }
        } else {
            mfdtd::ck(cudaEventSynchronize(rs.copied), "record copy");
        }
        rs.busy = false;
        const size_t blk = slice_len + 2 * (size_t)P.Nx;
        mfdtd::Record r;
        r.t = rs.t;
        r.E.assign(rs.hE, rs.hE + blk);
        r.H.assign(rs.hH, rs.hH + blk);
        if (form == MFDTD_FORM_FP64_PLAIN) {
            std::memcpy(&r.emax, rs.hbits, 8);
        } else {
            float f;
            std::memcpy(&f, rs.hbits, 4);  // FP32 bits of max|Ex| in the low word
            r.emax = f;
        }
        emit_record(r, rs.collect);
    }

    // Finish every record in flight, oldest first.
    void drain_records() {
        RecSlot &older = rslot[rnext], &newer = rslot[rnext ^ 1];
        if (older.busy) finish_record(older);
        if (newer.busy) finish_record(newer);
    }

    void emit_record(mfdtd::Record &r, bool collect) {
        const int tt = r.t;
        if (sink) {
            char line[256];
            double partialtime = 100 * tt / P.tsteps;
            std::snprintf(line, sizeof line, "t = %d: %s %% Done...  Maximum abs(Ex) is %s\n", tt,
                          mfdtd::fmt_g(partialtime).c_str(), mfdtd::fmt_g(r.emax).c_str());
            sink->log(line);
            if (P.savefields) {
                std::vector<double> zeros(slice_len, 0.0);  // output_J.dat: never assigned
                sink->append("output_E.dat", r.E.data(), r.E.size() * 8);
                sink->append("output_J.dat", zeros.data(), zeros.size() * 8);
                sink->append("output_H.dat", r.H.data(), r.H.size() * 8);
            }
        }
        if (collect) records.push_back(std::move(r));
    }

    int kernel_classes() const {
        return form == MFDTD_FORM_FP64_PLAIN ? 2 : mfdtd::Fp32Sim::kernel_classes();
    }

    void advance(int nsteps, bool collect) {
        if (batch) throw Error(MFDTD_ESTATE, "the simulation is a batch member (mfdtd_batch_remove first)");
        if (nsteps < 0 || t + nsteps > P.tsteps)
            throw Error(MFDTD_EINVAL, "advance past tsteps");
        int64_t launches = 0;
        const int nk = kernel_classes();
        const int prof_steps = opts.profile ? std::min(nsteps, 512) : 0;
        if (prof_steps) {
            kname.assign(nk, "");
            for (int q = 0; q < nk; q++)
                kname[q] = form == MFDTD_FORM_FP64_PLAIN ? (q == 0 ? "k_plain_h" : "k_plain_e")
                                                         : mfdtd::Fp32Sim::kernel_name(q);
            ktotal_ms.assign(nk, 0.0);
            kcount.assign(nk, 0);
            while ((int)kev.size() < (nk + 1) * prof_steps) {
                cudaEvent_t e;
                mfdtd::ck(cudaEventCreate(&e), "cudaEventCreate");
                kev.push_back(e);
            }
        }
        mfdtd::ck(cudaEventRecord(ev0, stream), "cudaEventRecord");
        const long long fast0 = f32 ? f32->fast_passes() : 0, gen0 = f32 ? f32->general_passes() : 0;
        const int t_begin = t, t_end = t + nsteps;
        for (; t < t_end; t++) {
            const bool rec = (t % P.record_period) == 0;
            const int ps = t - t_begin;
            void *const *ev = ps < prof_steps ? (void *const *)&kev[(size_t)(nk + 1) * ps] : nullptr;
            if (form == MFDTD_FORM_FP64_PLAIN) launches += mfdtd::plain_launch_step(pa, t, rec, stream, ev);
            // (an FP32 record step takes the general pass to capture the
            // slices; with nobody taking the records it is an ordinary step)
            else launches += f32->step(t, rec && (collect || sink), stream, ev);
            mfdtd::ck(cudaGetLastError(), "kernel launch");
            if (rec && (collect || sink)) {
                mfdtd::ck(cudaEventRecord(ev1, stream), "cudaEventRecord");
                do_record(t, collect);
            }
            if (t == 20 && sink) {
                wait();
                drain_records();
                double runtimemin = (mfdtd::wall_s() - loop_start) / 60.0;
                double totaltime = runtimemin * P.tsteps / 20.0;
                sink->log("t = 20, time taken = " + mfdtd::fmt_g(runtimemin) + " minutes.\n");
                sink->log("You can expect the total simulation to take " + mfdtd::fmt_g(totaltime) +
                          " minutes.\n");
            }
            if (opts.guard_period > 0 && (t + 1) % opts.guard_period == 0) guard();
        }
        if (f32) launches += f32->drain_ntf(stream);  // the DFT sums are whole after every advance
        mfdtd::ck(cudaEventRecord(ev1, stream), "cudaEventRecord");
        mfdtd::ck(cudaGetLastError(), "kernel launch");
        last_launches = launches;
        if (prof_steps && f32) {
            // Class 0 of the FP32 form is the pass with its band kernels; name
            // the pass kernel(s) that ran in this advance.
            const bool fast = f32->fast_passes() > fast0, gen = f32->general_passes() > gen0;
            const std::string fname = f32->fast_pass_name();
            kname[0] = fast && gen ? fname + "+k_fp32_step" : fast ? fname : std::string("k_fp32_step");
        }
        if (nsteps > 0) {
            wait();
            drain_records();
            if (f32) f32->check(stream);
            float ms = 0;
            mfdtd::ck(cudaEventElapsedTime(&ms, ev0, ev1), "cudaEventElapsedTime");
            last_ms_per_step = ms / nsteps;
            for (int ps = 0; ps < prof_steps; ps++)
                for (int q = 0; q < nk; q++) {
                    float kms = 0;
                    mfdtd::ck(cudaEventElapsedTime(&kms, kev[(size_t)(nk + 1) * ps + q],
                                                   kev[(size_t)(nk + 1) * ps + q + 1]),
                              "cudaEventElapsedTime");
                    ktotal_ms[q] += kms;
                    kcount[q] += 1;
                }
        }
    }

    void guard() {
        bool bad;
        if (form == MFDTD_FORM_FP64_PLAIN) {
            unsigned int flag = 0;
            mfdtd::plain_launch_guard(pa, stream);
            mfdtd::ck(cudaMemcpyAsync(&flag, pa.flag, 4, cudaMemcpyDeviceToHost, stream), "D2H");
            wait();
            bad = flag != 0;
        } else {
            bad = f32->guard(stream) != 0;
        }
        if (bad) throw Error(MFDTD_ENUMERIC, "non-finite E field after step " + std::to_string(t));
    }

    // E probes of the final step ride in the next H kernel; emit them once.
    void flush() {
        if (flushed || t == 0) return;
        if (form == MFDTD_FORM_FP64_PLAIN) mfdtd::plain_launch_flush(pa, t - 1, stream);
        else f32->flush(t - 1, stream);
        flushed = true;
    }

    int64_t ntf_size() const {
        const int64_t nf2 = 2 * (int64_t)P.nntf();
        return 2 * nf2 + 8 * ((int64_t)P.Ny * P.Nz * nf2) + 8 * ((int64_t)P.Nx * P.Nz * nf2) +
               8 * ((int64_t)P.Nx * P.Ny * nf2);
    }

    // Source DFT sums (source/meteor-2.1.cpp:1378-1383): a function of the
    // injected waveform only, over the steps run so far.  Eydft then Ezdft.
    std::vector<double> source_dft() const {
        std::vector<double> sd(4 * (size_t)P.nntf(), 0.0);
        {
            const double PI = 3.141592653589793;
            const int nf = P.nntf();
            for (int tt = 0; tt < t; tt++)
                for (int m = 0; m < nf; m++) {
                    double s = sin(2 * PI * P.fntf[m] * (tt + 1 / 2) * P.dt);
                    double c = cos(2 * PI * P.fntf[m] * (tt + 1 / 2) * P.dt);
                    sd[2 * nf + 2 * m] += P.src[2 * tt] * s;
                    sd[2 * nf + 2 * m + 1] += P.src[2 * tt] * c;
                    sd[2 * m] += P.src[2 * tt + 1] * s;
                    sd[2 * m + 1] += P.src[2 * tt + 1] * c;
                }
        }
        return sd;
    }

    void read_ntf(double *out) {
        flush();
        const size_t nf2 = 2 * (size_t)P.nntf();
        std::vector<double> sd = source_dft();
        std::memcpy(out, sd.data(), sd.size() * 8);
        double *o = out + sd.size();
        const size_t fb = (size_t)P.Ny * P.Nz * nf2, tb = (size_t)P.Nx * P.Nz * nf2, lr = (size_t)P.Nx * P.Ny * nf2;
        for (int q = 0; q < 24; q++) {
            size_t n = q < 8 ? fb : q < 16 ? tb : lr;
            if (form == MFDTD_FORM_FP64_PLAIN)
                mfdtd::ck(cudaMemcpyAsync(o, pa.ntf[q], n * 8, cudaMemcpyDeviceToHost, stream), "D2H");
            else f32->read_ntf(q, o, stream);
            o += n;
        }
        wait();
    }

    void read_probes(double *out) {
        flush();
        size_t n = (size_t)6 * P.tsteps * P.nprobes();
        if (form == MFDTD_FORM_FP64_PLAIN)
            mfdtd::ck(cudaMemcpyAsync(out, pa.probe, n * 8, cudaMemcpyDeviceToHost, stream), "D2H");
        else f32->read_probes(out, stream);
        wait();
    }

    void read_field(int comp, double *out) {
        if (comp < 0 || comp > 8) throw Error(MFDTD_EINVAL, "component must be 0..8");
        if (form == MFDTD_FORM_FP64_PLAIN) {
            double *f[9] = {pa.Ex, pa.Ey, pa.Ez, pa.Hx, pa.Hy, pa.Hz, pa.Jx, pa.Jy, pa.Jz};
            mfdtd::ck(cudaMemcpyAsync(out, f[comp], P.cells() * 8, cudaMemcpyDeviceToHost, stream), "D2H");
        } else {
            f32->read_field(comp, out, stream);
        }
        wait();
    }

    void read_slices(int scattered, double *E, double *H) {
        if (batch) throw Error(MFDTD_ESTATE, "the simulation is a batch member (mfdtd_batch_remove first)");
        if (form == MFDTD_FORM_FP64_PLAIN) {
            double *d = nullptr;
            mfdtd::ck(cudaMallocAsync(&d, 2 * slice_len * 8, stream), "cudaMallocAsync");
            mfdtd::plain_launch_slices(pa, scattered, d, d + slice_len, stream);
            mfdtd::ck(cudaMemcpyAsync(E, d, slice_len * 8, cudaMemcpyDeviceToHost, stream), "D2H");
            mfdtd::ck(cudaMemcpyAsync(H, d + slice_len, slice_len * 8, cudaMemcpyDeviceToHost, stream), "D2H");
            mfdtd::ck(cudaFreeAsync(d, stream), "cudaFreeAsync");
        } else {
            const double s0 = P.s0;
            f32->read_slices(scattered, E, H, P.kr, s0, P.inc_e, P.inc_h, stream);
        }
        wait();
    }

    void write_final(const std::string &dir) {
        mfdtd::FileSink fs{dir};
        std::vector<double> ntf((size_t)ntf_size());
        read_ntf(ntf.data());
        // output_NTF.dat, source/meteor-2.1.cpp:1579-1620
        std::string path = dir + "/output_NTF.dat";
        FILE *f = std::fopen(path.c_str(), "wb");
        if (!f) throw Error(MFDTD_EIO, "cannot write " + path);
        int32_t hdr[2] = {P.nntf(), P.ntfb};
        std::fwrite(hdr, 4, 2, f);
        std::fwrite(P.fntf.data(), 8, P.fntf.size(), f);
        std::fwrite(ntf.data(), 8, ntf.size(), f);
        std::fclose(f);
        // Probe.dat, source/meteor-2.1.cpp:1624-1636
        std::vector<double> pr((size_t)6 * P.tsteps * P.nprobes());
        read_probes(pr.data());
        path = dir + "/Probe.dat";
        f = std::fopen(path.c_str(), "wb");
        if (!f) throw Error(MFDTD_EIO, "cannot write " + path);
        int32_t np = P.nprobes();
        std::fwrite(&np, 4, 1, f);
        if (np) {
            std::fwrite(P.probex.data(), 4, np, f);
            std::fwrite(P.probey.data(), 4, np, f);
            std::fwrite(P.probez.data(), 4, np, f);
        }
        if (!pr.empty()) std::fwrite(pr.data(), 8, pr.size(), f);
        std::fclose(f);
    }
};

struct mfdtd_batch {
    std::unique_ptr<mfdtd::Fp32Batch> fb;
    std::vector<mfdtd_sim *> members;
};

namespace {

int fail(const Error &e) {
    mfdtd::g_last_error = e.what();
    return e.code;
}

template <class F> int guarded(F &&fn) {
    try {
        fn();
        return MFDTD_OK;
    } catch (const Error &e) {
        return fail(e);
    } catch (const std::bad_alloc &) {
        mfdtd::g_last_error = "host allocation failed";
        return MFDTD_ENOMEM;
    } catch (const std::exception &e) {
        mfdtd::g_last_error = e.what();
        return MFDTD_EINVAL;
    }
}

void log_header(mfdtd::FileSink &fs, const Problem &P) {
    struct rusage ru;
    getrusage(RUSAGE_SELF, &ru);
    double memusage = (double)ru.ru_maxrss / 1024 / 1024;
    std::string dir = fs.dir + "/log.txt";
    FILE *f = std::fopen(dir.c_str(), "w");
    if (!f) throw Error(MFDTD_EIO, "cannot write " + dir);
    std::fprintf(f, "------------------------------------------\n");
    std::fprintf(f, "3D Meteor Scattering Simulation\n");
    std::fprintf(f, "------------------------------------------\n");
    std::fprintf(f, "dx = %g\n", P.dx);
    std::fprintf(f, "source type = %d\n", P.sourcetype);
    std::fprintf(f, "source polarization = %d\n", P.sourcepol);
    std::fprintf(f, "Time step = %g\n", P.dt);
    std::fprintf(f, "Total time steps = %d\n", P.tsteps);
    std::fprintf(f, "Total NTF frequencies = %d\n", P.nntf());
    std::fprintf(f, "last NTF frequency = %g\n", P.fntf.back());
    std::fprintf(f, "Total memory usage = %g GB\n", memusage);
    std::fclose(f);
}

}  // namespace

extern "C" {

const char *mfdtd_version(void) { return "mfdtd-gb300 0.1"; }

int mfdtd_last_error(char *buf, size_t n) {
    if (!buf || n == 0) return MFDTD_EINVAL;
    std::snprintf(buf, n, "%s", mfdtd::g_last_error.c_str());
    return MFDTD_OK;
}

int mfdtd_problem_from_rundir(const char *dir, mfdtd_problem **out) {
    return guarded([&] {
        if (!dir || !out) throw Error(MFDTD_EINVAL, "NULL argument");
        std::unique_ptr<mfdtd_problem> p(new mfdtd_problem());
        p->P = mfdtd::problem_from_rundir(dir);
        *out = p.release();
    });
}

int mfdtd_problem_create(const mfdtd_params *prm, const double *wp2, const double *nu2,
                         const double B0[3], mfdtd_problem **out) {
    return guarded([&] {
        if (!prm || !out) throw Error(MFDTD_EINVAL, "NULL argument");
        std::unique_ptr<mfdtd_problem> p(new mfdtd_problem());
        p->P = mfdtd::problem_from_params(*prm, wp2, nu2, B0);
        *out = p.release();
    });
}

void mfdtd_problem_destroy(mfdtd_problem *pb) { delete pb; }

void mfdtd_ext_defaults(mfdtd_ext *ext) {
    if (ext) mfdtd::ext_defaults(*ext);
}

int mfdtd_problem_set_trail(mfdtd_problem *pb, const mfdtd_trail *trail) {
    return guarded([&] {
        if (!pb) throw Error(MFDTD_EINVAL, "NULL problem");
        Problem P = pb->P;
        P.has_trail = trail ? 1 : 0;
        if (trail) P.trail = *trail;
        P.derive();
        pb->P = std::move(P);
    });
}

int mfdtd_problem_set_ext(mfdtd_problem *pb, const mfdtd_ext *ext, const double *wp3,
                          const double *nu3) {
    return guarded([&] {
        if (!pb) throw Error(MFDTD_EINVAL, "NULL problem");
        Problem P = pb->P;  // validate on a copy: a rejected call leaves pb unchanged
        if (ext) P.ext = *ext;
        else mfdtd::ext_defaults(P.ext);
        P.ext_present = 1;
        const size_t n3 = P.cells();
        if (wp3) P.wp3.assign(wp3, wp3 + n3);
        else P.wp3.clear();
        if (nu3) P.nu3.assign(nu3, nu3 + n3);
        else P.nu3.clear();
        P.derive();
        pb->P = std::move(P);
    });
}

int mfdtd_problem_dims(const mfdtd_problem *pb, int64_t out[6]) {
    return guarded([&] {
        if (!pb || !out) throw Error(MFDTD_EINVAL, "NULL argument");
        const Problem &P = pb->P;
        out[0] = P.Nx; out[1] = P.Ny; out[2] = P.Nz;
        out[3] = P.tsteps; out[4] = P.nntf(); out[5] = P.nprobes();
    });
}

int mfdtd_problem_footprint(const mfdtd_problem *pb, int32_t form, int64_t *bytes) {
    return guarded([&] {
        if (!pb || !bytes) throw Error(MFDTD_EINVAL, "NULL argument");
        const Problem &P = pb->P;
        const int64_t NC = (int64_t)P.cells(), L2 = 2 * P.L;
        const int64_t psi = P.dopml ? 4 * (L2 * P.Ny * P.Nz + (int64_t)P.Nx * L2 * P.Nz + (int64_t)P.Nx * P.Ny * L2) : 0;
        const int64_t nf2 = 2 * P.nntf();
        const int64_t ntf = 8 * nf2 * ((int64_t)P.Ny * P.Nz + (int64_t)P.Nx * P.Nz + (int64_t)P.Nx * P.Ny);
        const int64_t misc = 8 * ((int64_t)P.tsteps * (2 + nf2 + 6 * P.nprobes()) + (int64_t)P.lk.size() +
                                  4 * ((int64_t)P.Nx * P.Ny + P.Nx + P.Ny + P.Nz));
        const int64_t maps = 8 * NC * ((P.wp3.empty() && !P.has_trail ? 0 : 1) + (P.nu3.empty() ? 0 : 1));
        if (form == MFDTD_FORM_FP64_PLAIN) *bytes = 8 * (9 * NC + psi) + 8 * ntf + misc + maps;
        else *bytes = mfdtd::Fp32Sim::footprint(P);
    });
}

int mfdtd_sim_create(const mfdtd_problem *pb, const mfdtd_run_opts *opts, mfdtd_sim **out) {
    return guarded([&] {
        if (!pb || !out) throw Error(MFDTD_EINVAL, "NULL argument");
        std::unique_ptr<mfdtd_sim> s(new mfdtd_sim());
        s->init(pb->P, opts);
        *out = s.release();
    });
}

void mfdtd_sim_destroy(mfdtd_sim *s) {
    if (s && s->batch) mfdtd_batch_remove(s->batch, s);  // never leave a dangling member
    delete s;
}

int mfdtd_sim_advance(mfdtd_sim *s, int32_t nsteps, int32_t collect_records) {
    return guarded([&] {
        if (!s) throw Error(MFDTD_EINVAL, "NULL sim");
        s->advance(nsteps, collect_records != 0);
    });
}

int mfdtd_sim_sync(mfdtd_sim *s) {
    return guarded([&] {
        if (!s) throw Error(MFDTD_EINVAL, "NULL sim");
        s->wait();
    });
}

int mfdtd_sim_step_index(const mfdtd_sim *s, int32_t *t) {
    return guarded([&] {
        if (!s || !t) throw Error(MFDTD_EINVAL, "NULL argument");
        *t = s->t;
    });
}

int64_t mfdtd_sim_ntf_size(const mfdtd_sim *s) { return s ? s->ntf_size() : -1; }

int mfdtd_sim_read_ntf(mfdtd_sim *s, double *out, int64_t n) {
    return guarded([&] {
        if (!s || !out) throw Error(MFDTD_EINVAL, "NULL argument");
        if (n < s->ntf_size()) throw Error(MFDTD_EINVAL, "output buffer too small");
        s->read_ntf(out);
    });
}

int mfdtd_sim_read_probes(mfdtd_sim *s, double *out, int64_t n) {
    return guarded([&] {
        if (!s || (!out && n)) throw Error(MFDTD_EINVAL, "NULL argument");
        if (n < (int64_t)6 * s->P.tsteps * s->P.nprobes()) throw Error(MFDTD_EINVAL, "output buffer too small");
        s->read_probes(out);
    });
}

int mfdtd_sim_read_field(mfdtd_sim *s, int32_t comp, double *out, int64_t n) {
    return guarded([&] {
        if (!s || !out) throw Error(MFDTD_EINVAL, "NULL argument");
        if (n < (int64_t)s->P.cells()) throw Error(MFDTD_EINVAL, "output buffer too small");
        s->read_field(comp, out);
    });
}

int mfdtd_sim_read_slices(mfdtd_sim *s, int32_t scattered, double *E, double *H, int64_t n) {
    return guarded([&] {
        if (!s || !E || !H) throw Error(MFDTD_EINVAL, "NULL argument");
        if (n < (int64_t)s->slice_len) throw Error(MFDTD_EINVAL, "output buffer too small");
        s->read_slices(scattered != 0, E, H);
    });
}

int mfdtd_sim_plasma_fraction(const mfdtd_sim *s, double *fraction) {
    return guarded([&] {
        if (!s || !fraction) throw Error(MFDTD_EINVAL, "NULL argument");
        *fraction = s->f32 ? s->f32->plasma_fraction() : 1.0;
    });
}

int mfdtd_sim_write_outputs(mfdtd_sim *s, const char *dir) {
    return guarded([&] {
        if (!s || !dir) throw Error(MFDTD_EINVAL, "NULL argument");
        mfdtd::FileSink fs{dir};
        for (auto &r : s->records) {
            char line[256];
            double partialtime = 100 * r.t / s->P.tsteps;
            std::snprintf(line, sizeof line, "t = %d: %s %% Done...  Maximum abs(Ex) is %s\n", r.t,
                          mfdtd::fmt_g(partialtime).c_str(), mfdtd::fmt_g(r.emax).c_str());
            fs.log(line);
            if (s->P.savefields) {
                std::vector<double> zeros(s->slice_len, 0.0);
                fs.append("output_E.dat", r.E.data(), r.E.size() * 8);
                fs.append("output_J.dat", zeros.data(), zeros.size() * 8);
                fs.append("output_H.dat", r.H.data(), r.H.size() * 8);
            }
        }
        s->write_final(dir);
    });
}

int mfdtd_sim_last_timing(const mfdtd_sim *s, double *ms_per_step, int64_t *launches) {
    return guarded([&] {
        if (!s) throw Error(MFDTD_EINVAL, "NULL sim");
        if (ms_per_step) *ms_per_step = s->last_ms_per_step;
        if (launches) *launches = s->last_launches;
    });
}

int mfdtd_sim_far_field(mfdtd_sim *s, int32_t ndir, const double *theta, const double *phi,
                        int32_t method, double *out) {
    return guarded([&] {
        if (!s || !theta || !phi || !out || ndir <= 0) throw Error(MFDTD_EINVAL, "bad arguments");
        if (method != 0 && method != 1) throw Error(MFDTD_EINVAL, "unknown far-field method");
        s->flush();
        std::vector<double> sd = s->source_dft();
        double *const *ntf = s->form == MFDTD_FORM_FP64_PLAIN ? s->pa.ntf : s->f32->ntf_arrays();
        mfdtd::far_field_fp64(s->P, ntf, sd.data(), ndir, theta, phi, out, s->stream, method);
    });
}

int mfdtd_sim_kernel_stats(const mfdtd_sim *s, int32_t which, char *name, size_t name_len,
                           double *avg_ms, int64_t *launches) {
    return guarded([&] {
        if (!s) throw Error(MFDTD_EINVAL, "NULL sim");
        if (which < 0 || which >= (int32_t)s->kname.size())
            throw Error(MFDTD_EINVAL, "no such kernel class (was opts.profile set?)");
        if (name && name_len) std::snprintf(name, name_len, "%s", s->kname[which].c_str());
        if (avg_ms) *avg_ms = s->kcount[which] ? s->ktotal_ms[which] / s->kcount[which] : 0.0;
        if (launches) *launches = s->kcount[which];
    });
}

int mfdtd_batch_capacity(void) { return mfdtd::Fp32Batch::capacity(); }

int mfdtd_batch_create(int32_t device, mfdtd_batch **out) {
    return guarded([&] {
        if (!out) throw Error(MFDTD_EINVAL, "NULL argument");
        std::unique_ptr<mfdtd_batch> b(new mfdtd_batch());
        b->fb.reset(new mfdtd::Fp32Batch(device));
        *out = b.release();
    });
}

void mfdtd_batch_destroy(mfdtd_batch *b) {
    if (!b) return;
    try {
        b->fb->sync();
    } catch (...) {
    }
    for (mfdtd_sim *s : b->members) s->batch = nullptr;
    delete b;
}

int mfdtd_batch_add(mfdtd_batch *b, mfdtd_sim *s) {
    return guarded([&] {
        if (!b || !s) throw Error(MFDTD_EINVAL, "NULL argument");
        if (s->batch) throw Error(MFDTD_ESTATE, "the simulation is already a batch member");
        if (s->form != MFDTD_FORM_FP32_FUSED) throw Error(MFDTD_EINVAL, "batches hold FP32 simulations");
        if (s->opts.device != b->fb->impl_device())
            throw Error(MFDTD_EINVAL, "the simulation lives on another device");
        mfdtd::ck(cudaStreamSynchronize(s->stream), "sim");
        b->fb->add(s->f32.get(), s->t);
        s->batch = b;
        b->members.push_back(s);
    });
}

int mfdtd_batch_remove(mfdtd_batch *b, mfdtd_sim *s) {
    return guarded([&] {
        if (!b || !s) throw Error(MFDTD_EINVAL, "NULL argument");
        if (s->batch != b) throw Error(MFDTD_EINVAL, "not a member of this batch");
        b->fb->sync();
        const int done = b->fb->steps_done(s->f32.get());
        if (done >= 0) s->t = done;
        b->fb->remove(s->f32.get());
        s->batch = nullptr;
        b->members.erase(std::find(b->members.begin(), b->members.end(), s));
    });
}

int mfdtd_batch_run(mfdtd_batch *b, int32_t nsteps) {
    return guarded([&] {
        if (!b || nsteps < 0) throw Error(MFDTD_EINVAL, "bad arguments");
        b->fb->run(nsteps);
    });
}

int mfdtd_batch_sync(mfdtd_batch *b) {
    return guarded([&] {
        if (!b) throw Error(MFDTD_EINVAL, "NULL batch");
        b->fb->sync();
        for (mfdtd_sim *s : b->members) {
            const int done = b->fb->steps_done(s->f32.get());
            if (done >= 0) s->t = done;
        }
    });
}

int mfdtd_batch_tune(mfdtd_batch *b, const int32_t *slab_depths, int32_t n_depths,
                     const int32_t *ctas_per_sm, int32_t n_ctas, int32_t *best_depth,
                     int32_t *best_ctas) {
    return guarded([&] {
        if (!b || !slab_depths || !ctas_per_sm || n_depths <= 0 || n_ctas <= 0)
            throw Error(MFDTD_EINVAL, "bad arguments");
        for (int q = 0; q < n_depths; q++)
            if (slab_depths[q] < 2) throw Error(MFDTD_EINVAL, "slab depth must be >= 2");
        std::vector<int> d(slab_depths, slab_depths + n_depths), c(ctas_per_sm, ctas_per_sm + n_ctas);
        b->fb->tune(d.data(), n_depths, c.data(), n_ctas);
        if (best_depth) *best_depth = b->fb->tuned_chunk();
        if (best_ctas) *best_ctas = b->fb->tuned_ctas();
    });
}

int mfdtd_batch_tile_shape(const mfdtd_batch *b, int32_t *rows, int32_t *cols) {
    return guarded([&] {
        if (!b) throw Error(MFDTD_EINVAL, "NULL batch");
        if (rows) *rows = 8;
        if (cols) *cols = b->fb->tuned_tile_cols();
    });
}

int mfdtd_run_rundir(const char *dir, const mfdtd_run_opts *opts) {
    return guarded([&] {
        if (!dir) throw Error(MFDTD_EINVAL, "NULL dir");
        double tStart = mfdtd::wall_s();
        Problem P = mfdtd::problem_from_rundir(dir);
        mfdtd::FileSink fs{dir};
        log_header(fs, P);
        std::unique_ptr<mfdtd_sim> s(new mfdtd_sim());
        s->init(P, opts);
        s->sink = &fs;
        s->loop_start = mfdtd::wall_s();
        s->advance(P.tsteps, false);
        s->write_final(dir);
        const bool quiet = opts && opts->quiet;
        if (!quiet && P.Ny > 39 && P.Nz > 79) {
            // debug print of source/meteor-2.1.cpp:1601-1602, in bounds only
            std::vector<double> ntf((size_t)s->ntf_size());
            s->read_ntf(ntf.data());
            const size_t nf2 = 2 * (size_t)P.nntf();
            const size_t at = 4 * (size_t)P.nntf() + ((size_t)39 * P.Nz + 79) * nf2;
            const size_t fb = (size_t)P.Ny * P.Nz * nf2;
            std::printf("My-front at y = 40, z = 80 is %g\n", ntf[at]);
            std::printf("Mz-front at y = 40, z = 80 is %g\n", ntf[at + fb]);
        }
        fs.log("All done!\n");
        fs.log("Total run time = " + mfdtd::fmt_g((mfdtd::wall_s() - tStart) / 60.0) + "minutes.\n");
    });
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Serving loop

namespace {

struct ServerJob {
    int64_t id = 0;
    Problem P;
    std::vector<double> theta, phi;
    std::unique_ptr<mfdtd_sim> sim;
    int64_t bytes = 0;
    int kind = -1;                 // batch key: current-update kind + 3 x batch class
    bool solo = false;             // marched alone on its own stream (kSoloCells), not in a batch
    double t_submit = 0, t_admit = 0, t_done = 0;
    int state = 0;                 // 0 queued, 1 running, 2 retired, 3 failed
    bool cancel = false;           // leave at the end of the current round
    int code = 0;
    std::string err;
    std::vector<double> result;
};

// A job of at least this many cells fills the GPU by itself: batching gains it
// nothing, and inside a batch every tick waits for it.  The server marches it
// as a single simulation (its own stream, the single-simulation kernels)
// beside the batches.
constexpr int64_t kSoloCells = int64_t(1) << 25;

}  // namespace

struct mfdtd_server {
    int device = 0;
    int64_t cap = 0;
    int steps = 100;
    std::thread worker;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    bool stop = false;
    int64_t next_id = 1, n_submitted = 0, n_retired = 0, used = 0;
    std::deque<ServerJob *> queued;
    std::map<int64_t, std::unique_ptr<ServerJob>> jobs;
    std::vector<ServerJob *> running;
    std::map<int, std::unique_ptr<mfdtd_batch>> batches;

    void loop() {
        cudaSetDevice(device);
        for (;;) {
            // admit in arrival order while memory and slots allow
            std::vector<ServerJob *> admit;
            {
                std::unique_lock<std::mutex> lk(mu);
                if (running.empty() && queued.empty() && !stop)
                    cv_work.wait_for(lk, std::chrono::milliseconds(20));
                if (stop) break;
                int64_t free_bytes = cap - used;
                // member slots are shared by every batch on the device
                int slots = mfdtd::Fp32Batch::free_slots(device);
                while (!queued.empty()) {
                    ServerJob *j = queued.front();
                    if (j->bytes > free_bytes) break;  // arrival order: no overtaking
                    if (!j->solo && slots <= 0) break;
                    queued.pop_front();
                    free_bytes -= j->bytes;
                    if (!j->solo) slots--;
                    used += j->bytes;
                    admit.push_back(j);
                }
            }
            for (ServerJob *j : admit) {
                try {
                    mfdtd_run_opts o{};
                    o.form = MFDTD_FORM_FP32_FUSED;
                    o.device = device;
                    o.quiet = 1;
                    j->sim.reset(new mfdtd_sim());
                    j->sim->init(j->P, &o);
                    if (!j->solo) {
                        auto &b = batches[j->kind];
                        if (!b) {
                            b.reset(new mfdtd_batch());
                            b->fb.reset(new mfdtd::Fp32Batch(device));
                        }
                        b->fb->add(j->sim->f32.get(), 0);
                        j->sim->batch = b.get();
                        b->members.push_back(j->sim.get());
                    }
                    std::lock_guard<std::mutex> lk(mu);
                    j->state = 1;
                    j->t_admit = mfdtd::wall_s();
                    running.push_back(j);
                } catch (const Error &e) {
                    finish_failed(j, e.code, e.what());
                } catch (const std::exception &e) {
                    finish_failed(j, MFDTD_ECUDA, e.what());
                }
            }
            if (running.empty()) continue;
            // one round: every batch advances; the batches overlap on the device
            for (auto &kv : batches)
                if (!kv.second->members.empty()) kv.second->fb->run(steps);
            // the jobs marched alone, on their own streams, while the batches run
            for (ServerJob *j : running) {
                if (!j->solo || j->code) continue;
                {
                    std::lock_guard<std::mutex> lk(mu);
                    if (j->cancel) continue;
                }
                mfdtd_sim *m = j->sim.get();
                try {
                    m->advance(std::min(steps, m->P.tsteps - m->t), false);
                } catch (const Error &e) {
                    j->code = e.code, j->err = e.what();
                } catch (const std::exception &e) {
                    j->code = MFDTD_ECUDA, j->err = e.what();
                }
            }
            for (auto &kv : batches) {
                if (kv.second->members.empty()) continue;
                try {
                    kv.second->fb->sync();
                } catch (const Error &e) {
                    for (mfdtd_sim *m : kv.second->members)
                        for (ServerJob *j : running)
                            if (j->sim.get() == m) j->code = e.code, j->err = e.what();
                }
                for (mfdtd_sim *m : kv.second->members) {
                    const int d = kv.second->fb->steps_done(m->f32.get());
                    if (d >= 0) m->t = d;
                }
            }
            // retire
            std::vector<ServerJob *> still;
            for (ServerJob *j : running) {
                mfdtd_sim *m = j->sim.get();
                bool cancel;
                {
                    std::lock_guard<std::mutex> lk(mu);
                    cancel = j->cancel;
                }
                if (j->code == 0 && !cancel && m->t < m->P.tsteps) {
                    still.push_back(j);
                    continue;
                }
                try {
                    if (j->code) throw Error(j->code, j->err);
                    if (cancel) throw Error(MFDTD_ECANCELED, "canceled");
                    if (mfdtd_batch *b = m->batch) {
                        b->fb->remove(m->f32.get());
                        b->members.erase(std::find(b->members.begin(), b->members.end(), m));
                        m->batch = nullptr;
                    }
                    const int nd = (int)j->theta.size();
                    j->result.assign((size_t)m->P.nntf() * nd * 3, 0.0);
                    m->flush();
                    std::vector<double> sd = m->source_dft();
                    mfdtd::far_field_fp64(m->P, m->f32->ntf_arrays(), sd.data(), nd, j->theta.data(),
                                          j->phi.data(), j->result.data(), m->stream, 1);
                    j->sim.reset();
                    std::lock_guard<std::mutex> lk(mu);
                    used -= j->bytes;
                    j->state = 2;
                    j->t_done = mfdtd::wall_s();
                    n_retired++;
                } catch (const Error &e) {
                    if (m && m->batch) {
                        mfdtd_batch *b = m->batch;
                        b->fb->remove(m->f32.get());
                        b->members.erase(std::find(b->members.begin(), b->members.end(), m));
                        m->batch = nullptr;
                    }
                    j->sim.reset();
                    finish_failed(j, e.code, e.what());
                }
                cv_done.notify_all();
            }
            std::lock_guard<std::mutex> lk(mu);
            running.swap(still);
        }
    }

    void finish_failed(ServerJob *j, int code, const std::string &msg) {
        std::lock_guard<std::mutex> lk(mu);
        if (j->state == 1 || j->state == 0) used -= j->bytes;
        j->state = 3;
        j->code = code;
        j->err = msg;
        j->t_done = mfdtd::wall_s();
        cv_done.notify_all();
    }

    ~mfdtd_server() {
        {
            std::lock_guard<std::mutex> lk(mu);
            stop = true;
        }
        cv_work.notify_all();
        if (worker.joinable()) worker.join();
        for (auto &kv : jobs)
            if (kv.second->sim && kv.second->sim->batch) {
                mfdtd_batch *b = kv.second->sim->batch;
                try {
                    b->fb->remove(kv.second->sim->f32.get());
                } catch (...) {
                }
                kv.second->sim->batch = nullptr;
            }
        jobs.clear();
        batches.clear();
    }
};

extern "C" {

int mfdtd_server_create(int32_t device, int64_t hbm_cap_bytes, int32_t steps_per_round,
                        mfdtd_server **out) {
    return guarded([&] {
        if (!out || hbm_cap_bytes <= 0 || steps_per_round <= 0) throw Error(MFDTD_EINVAL, "bad arguments");
        std::unique_ptr<mfdtd_server> s(new mfdtd_server());
        s->device = device;
        s->cap = hbm_cap_bytes;
        s->steps = steps_per_round;
        mfdtd::ck(cudaSetDevice(device), "cudaSetDevice");
        mfdtd_server *raw = s.get();
        s->worker = std::thread([raw] { raw->loop(); });
        *out = s.release();
    });
}

void mfdtd_server_destroy(mfdtd_server *s) { delete s; }

int mfdtd_server_submit(mfdtd_server *s, const mfdtd_problem *pb, int32_t ndir, const double *theta,
                        const double *phi, int64_t *job_id) {
    return guarded([&] {
        if (!s || !pb || !theta || !phi || ndir <= 0 || !job_id) throw Error(MFDTD_EINVAL, "bad arguments");
        std::unique_ptr<ServerJob> j(new ServerJob());
        j->P = pb->P;
        j->theta.assign(theta, theta + ndir);
        j->phi.assign(phi, phi + ndir);
        j->bytes = mfdtd::Fp32Sim::footprint(j->P);
        if (j->bytes > s->cap) throw Error(MFDTD_ENOMEM, "job footprint exceeds the server's device cap");
        // The batch key: the current update the FP32 kernel will use.
        const Problem &P = j->P;
        int kind = 0;
        if (P.doB0) {
            bool uniform = !P.lk.empty();
            for (size_t q = 18; q < P.lk.size() && uniform; q++) uniform = P.lk[q] == P.lk[q % 18];
            kind = uniform ? 1 : 2;
        }
        j->kind = kind + 3 * mfdtd::Fp32Sim::batch_class(P);  // and the batch class
        j->solo = (int64_t)P.Nx * P.Ny * P.Nz >= kSoloCells;
        j->t_submit = mfdtd::wall_s();
        std::lock_guard<std::mutex> lk(s->mu);
        j->id = s->next_id++;
        *job_id = j->id;
        s->queued.push_back(j.get());
        s->jobs[j->id] = std::move(j);
        s->n_submitted++;
        s->cv_work.notify_all();
    });
}

int mfdtd_server_poll(mfdtd_server *s, int64_t job_id, int32_t wait_ms, double *out, int64_t n_out,
                      double times[3], int32_t *done) {
    return guarded([&] {
        if (!s || !done) throw Error(MFDTD_EINVAL, "bad arguments");
        std::unique_lock<std::mutex> lk(s->mu);
        auto it = s->jobs.find(job_id);
        if (it == s->jobs.end()) throw Error(MFDTD_EINVAL, "unknown job id");
        ServerJob *j = it->second.get();
        if (j->state < 2 && wait_ms > 0)
            s->cv_done.wait_for(lk, std::chrono::milliseconds(wait_ms), [&] { return j->state >= 2; });
        *done = j->state >= 2 ? 1 : 0;
        if (j->state < 2) return;
        if (j->state == 3) {
            const int code = j->code ? j->code : MFDTD_ECUDA;
            const std::string msg = j->err;
            s->jobs.erase(it);
            throw Error(code, "job failed: " + msg);
        }
        if (out) {
            if (n_out < (int64_t)j->result.size()) throw Error(MFDTD_EINVAL, "output buffer too small");
            std::memcpy(out, j->result.data(), j->result.size() * 8);
        }
        if (times) {
            times[0] = j->t_admit - j->t_submit;
            times[1] = j->t_done - j->t_submit;
            times[2] = 0;
        }
        s->jobs.erase(it);
    });
}

int mfdtd_server_cancel(mfdtd_server *s, int64_t job_id) {
    return guarded([&] {
        if (!s) throw Error(MFDTD_EINVAL, "bad arguments");
        std::lock_guard<std::mutex> lk(s->mu);
        auto it = s->jobs.find(job_id);
        if (it == s->jobs.end()) throw Error(MFDTD_EINVAL, "unknown job id");
        ServerJob *j = it->second.get();
        if (j->state >= 2) {  // finished: drop the result
            s->jobs.erase(it);
            return;
        }
        auto q = std::find(s->queued.begin(), s->queued.end(), j);
        if (q != s->queued.end()) {  // never admitted: no device memory held
            s->queued.erase(q);
            j->state = 3;
            j->code = MFDTD_ECANCELED;
            j->err = "canceled";
            j->t_done = mfdtd::wall_s();
            s->cv_done.notify_all();
            return;
        }
        j->cancel = true;  // admitted: the worker retires it after this round
        s->cv_work.notify_all();
    });
}

int mfdtd_server_stats(mfdtd_server *s, int64_t out[5]) {
    return guarded([&] {
        if (!s || !out) throw Error(MFDTD_EINVAL, "bad arguments");
        std::lock_guard<std::mutex> lk(s->mu);
        out[0] = s->n_submitted;
        out[1] = (int64_t)s->queued.size();
        out[2] = (int64_t)s->running.size();
        out[3] = s->n_retired;
        out[4] = s->used;
    });
}

}  // extern "C"
