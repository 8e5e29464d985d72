// fp32.hpp -- FP32 fused form of the time step (interface used by sim.cpp).
#pragma once

#include "common.hpp"

namespace mfdtd {

class Fp32Batch;

class Fp32Sim {
public:
    static int64_t footprint(const Problem &P);
    void init(const Problem &P, void *stream);
    int64_t device_bytes() const { return bytes_; }
    // Enqueue one time step; returns the number of kernels launched.  `ev`
    // (may be null) receives kernel_classes()+1 boundary events.
    int step(int t, bool record, void *stream, void *const *ev);
    // Add the running-DFT steps still held in the ring to the FP64 sums (the
    // caller does so at the end of every advance, before anything reads the
    // sums); returns the number of kernels launched.
    int drain_ntf(void *stream);
    static int kernel_classes();
    // Batch class of a problem's FP32 simulation: 1 when batches march it
    // with an interior path (the wide 8 x 64 one by default, or the fast 8 x
    // 32 one) and the CPML slab march (CPML band on every axis, oblique
    // incidence without a plate or sphere, no Lee-Kalluri table, an 8 x 32
    // tile interior in j and k), else 0 (general path).  A batch holds
    // simulations of one class.
    static int batch_class(const Problem &P);
    // Passes run so far by the fast form (k_fp32_step_wide with the slab
    // march, or k_fp32_step_fast with the band kernels: steps whose records
    // nobody takes) and by the general one (k_fp32_step).
    long long fast_passes() const;
    long long general_passes() const;
    // Kernel name(s) of a fast pass: "k_fp32_step_wide+k_fp32_slab" (the
    // interior pass with the slab march) or "k_fp32_step_fast" (followed by
    // the band kernels).
    const char *fast_pass_name() const;
    // Current-update kind of this simulation's kernel (0 Young DI, 1 uniform
    // Lee-Kalluri, 2 tabulated Lee-Kalluri); batches group by it.
    int current_update() const;
    static const char *kernel_name(int which);
    // Record-step outputs in the reference file layout (doubles), staged in
    // device memory without waiting: E and H blocks of slice_len + 2 Nx
    // doubles each (slices, then the two incident arrays), and bits[0] the
    // FP32 bits of max|Ex|.
    void record_stage(double *dE, double *dH, unsigned int *bits, void *stream);
    double guard(void *stream);
    void flush(int t_last, void *stream);
    void read_ntf(int q, double *out, void *stream);
    void read_probes(double *out, void *stream);
    void read_field(int comp, double *out, void *stream);
    // Slices of the current state in the record layout (E and H blocks of
    // the host arrays E[n], H[n]), minus the incident field inside the
    // total-field region when `scattered`; the oblique geometry in FP64.
    void read_slices(int scattered, double *E, double *H, const double kr[3], double s0,
                     const double ke[3], const double kh[3], void *stream);
    // Share of the pass's (plane, tile) blocks that hold plasma: J is loaded,
    // updated and stored there only.
    double plasma_fraction() const;
    // Throws if a kernel set the device error flag (a bounded wait ran out).
    void check(void *stream);
    // Device pointers of the 24 DFT arrays (output_NTF.dat order).
    double *const *ntf_arrays() const;
    ~Fp32Sim();

    struct Impl;
    Impl *impl() const { return impl_; }

private:
    friend class Fp32Batch;
    Impl *impl_ = nullptr;
    int64_t bytes_ = 0;
    int m_cur_ = 0;  // which ping-pong set holds the current E/H state
};

// Many FP32 simulations advanced together, one persistent-kernel launch per
// time step, two steps replayed as one CUDA graph (fp32_fused.cu).
class Fp32Batch {
public:
    explicit Fp32Batch(int device);
    ~Fp32Batch();
    static int capacity();
    // Member slots still free on `device`: the capacity is shared by every
    // batch on a device.
    static int free_slots(int device);
    // Join at step 0; returns the slot.  Throws when full or when the current
    // update differs from the batch's.
    int add(Fp32Sim *sim, int t0);
    void remove(Fp32Sim *sim);
    // Advance every member `nticks` steps (members at their step count idle);
    // returns kernel launches enqueued.  Asynchronous on stream().
    int run(int nticks);
    void sync();
    int steps_done(const Fp32Sim *sim) const;
    // Try every (tile shape, slab depth, CTAs per SM) on the live batch and
    // keep the fastest; returns the steps spent.  Tile shapes: 8 x 32 tiles
    // everywhere, or, for a batch of the slab class, interior tiles paired into
    // 8 x 64 tiles on the wide path (at most two CTAs per SM).
    int tune(const int *chunks, int nchunks, const int *ctas, int nctas);
    int tuned_chunk() const;
    int tuned_ctas() const;
    // Columns of the interior tiles: 32 (the fast path), or 64 (pairs on the
    // wide path; batches of the slab class only).
    int tuned_tile_cols() const;
    long long tick() const;
    void *stream() const;
    int impl_device() const;
    struct Impl;

private:
    Impl *impl_;
};

}  // namespace mfdtd
