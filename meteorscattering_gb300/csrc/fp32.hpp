// fp32.hpp -- FP32 fused form of the time step (interface used by sim.cpp).
#pragma once

#include "common.hpp"

namespace mfdtd {

class Fp32Sim {
public:
    static int64_t footprint(const Problem &P);
    void init(const Problem &P, void *stream);
    int64_t device_bytes() const { return bytes_; }
    // Enqueue one time step; returns the number of kernels launched.  `ev`
    // (may be null) receives kernel_classes()+1 boundary events.
    int step(int t, bool record, void *stream, void *const *ev);
    static int kernel_classes();
    static const char *kernel_name(int which);
    // Record-step outputs in the reference file layout (doubles).
    void record(double *E, double *H, double *emax, void *stream);
    double guard(void *stream);
    void flush(int t_last, void *stream);
    void read_ntf(int q, double *out, void *stream);
    void read_probes(double *out, void *stream);
    void read_field(int comp, double *out, void *stream);
    // Throws if a kernel set the device error flag (a bounded wait ran out).
    void check(void *stream);
    // Device pointers of the 24 DFT arrays (output_NTF.dat order).
    double *const *ntf_arrays() const;
    ~Fp32Sim();

private:
    struct Impl;
    Impl *impl_ = nullptr;
    int64_t bytes_ = 0;
    int m_cur_ = 0;  // which ping-pong set holds the current E/H state
};

}  // namespace mfdtd
