/*
 * mfdtd.h -- C ABI of the GB300 meteor-scattering FDTD engine.
 *
 * The reference solver (source/meteor-2.1.cpp, and its magnetized variant
 * source/meteor-fork.cpp) has no library interface: its boundary is a process
 * started in a run directory (setup/writepbsfile.m:15, qsub -d in
 * setup/meteorrun.m:169) that reads inputs.dat, B0.dat, wp.dat, nu.dat and
 * writes log.txt, output_{E,H,J}.dat, output_NTF.dat and Probe.dat.  The entry
 * points below replace that process: mfdtd_run_rundir() is the whole program,
 * the finer-grained calls expose its stages (input parse, device state, time
 * stepping, output write-out) to callers that keep data in memory.
 *
 * Conventions: every call returns an mfdtd_status (0 = success); no C++
 * exception crosses this boundary; the text of the last error on the calling
 * thread is available from mfdtd_last_error().  Handles are independent: calls
 * on different handles may run concurrently from different threads; calls on
 * one handle must be serialised by the caller.  All arrays are plain host
 * pointers in C order unless a comment says otherwise.
 */
#ifndef MFDTD_H
#define MFDTD_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    MFDTD_OK = 0,
    MFDTD_EINVAL = -1,   /* invalid argument or input-file content            */
    MFDTD_EIO = -2,      /* missing or short input file, unwritable output     */
    MFDTD_ECUDA = -3,    /* CUDA runtime error                                 */
    MFDTD_ENOMEM = -4,   /* device or host allocation failed / over the limit  */
    MFDTD_ETIMEOUT = -5, /* a bounded wait ran out                             */
    MFDTD_ENUMERIC = -6, /* NaN/Inf detected by the field guard                */
    MFDTD_ESTATE = -7,   /* call not valid in the handle's current state        */
    MFDTD_ECANCELED = -8 /* the job was canceled (mfdtd_server_cancel)          */
} mfdtd_status;

/* Arithmetic form of the time stepping. */
typedef enum {
    MFDTD_FORM_FP64_PLAIN = 0, /* FP64, reference operation order, no FMA
                                  contraction: the drop-in form              */
    MFDTD_FORM_FP32_FUSED = 1  /* FP32 fields/currents/psi, FP64 DFT sums    */
} mfdtd_form;

/* Contents of inputs.dat in file order (source/meteor-2.1.cpp:84-112, plus
 * doB0 read by source/meteor-fork.cpp:115).  Pointers are borrowed for the
 * duration of the call that receives the struct. */
typedef struct {
    int32_t dopml, savefields;
    double f0, fsig;
    int32_t sourcetype, sourcepol;
    double gridfactor, dt;
    int32_t tsteps, Nx, Ny, Nz;
    double metsize[2];
    double wpmax, numax;
    double metloc[3];
    double metangle;
    int32_t mettype, numfiles, nprobes;
    const int32_t *probex, *probey, *probez; /* [nprobes] */
    int32_t nntf;
    const double *fntf;                      /* [nntf] Hz */
    int32_t doplate;
    double platesize;
    int32_t doB0;                            /* 0: Young DI J, 1: Lee-Kalluri */
} mfdtd_params;

/* Run options.  A zeroed struct (or NULL) selects the defaults shown. */
typedef struct {
    int32_t form;          /* mfdtd_form; default FP64_PLAIN                     */
    int32_t device;        /* CUDA device ordinal; default 0                     */
    int32_t guard_period;  /* >0: check max|E| for NaN/Inf every N steps and
                              stop with MFDTD_ENUMERIC; default 0 (off)          */
    int32_t quiet;         /* nonzero: no stdout lines                            */
    double timeout_s;      /* >0: bound on each host wait for the device          */
    int32_t profile;       /* nonzero: time every kernel class with CUDA events
                              on the simulation's stream (mfdtd_sim_kernel_stats) */
} mfdtd_run_opts;

/* Extended inputs.  The reference hard-codes every one of these
 * (source/meteor-2.1.cpp:343 pmllen = 10, :413-415 grading m = 4, kappa = 1,
 * alpha = 0, :539-552 TF/SF box 10 cells and Huygens surface 5 cells inside
 * the CPML, :1278-1304 a plane wave along +x, :134-138 coordinates filled
 * for index < Nx only, :319-334 a 2-D plasma map times a Gaussian in z).
 * mfdtd_ext_defaults() fills the reference's values; a problem that never
 * receives an mfdtd_ext behaves exactly like the reference.
 * In a run directory the same content is the optional file ext.dat
 * (written by meteorscattering_gb300.rundir.write_ext), with wp3.dat/nu3.dat
 * beside it when the per-cell maps are used. */
typedef struct {
    int32_t pmllen;       /* CPML thickness in cells (1..32)                   */
    int32_t tfsf_gap;     /* cells between the CPML and the TF/SF box          */
    int32_t ntf_gap;      /* cells between the CPML and the Huygens surface;
                             must be <= tfsf_gap - 2 (surface outside the box)  */
    int32_t oblique;      /* 1: plane wave along inc_theta/inc_phi through a
                             dispersion-matched auxiliary line; the waveform
                             is the sourcetype's first column; sourcepol is
                             ignored                                           */
    int32_t exact_coords; /* 1: cell coordinates -(N-1)/2*d + i*d along every
                             axis with real division                           */
    int32_t lk_colocated; /* 1: the Lee-Kalluri current update is driven by E
                             at the current's own node.  0 (the reference,
                             source/meteor-fork.cpp:1574-1576) averages E over
                             two nodes but applies J at one; that asymmetric
                             coupling grows without bound in magnetized
                             plasma, faster at higher density               */
    double pml_m;         /* polynomial grading order                           */
    double kappa_max;     /* CPML kappa at the outer face (>= 1)                */
    double alpha_max;     /* CPML alpha in the units of the reference's sigma
                             (S/m): the recursion decays as
                             exp(-(sigma/kappa + alpha) dt / E0)               */
    double inc_theta;     /* direction of k: polar angle from +z (radians)      */
    double inc_phi;       /* azimuth from +x (radians)                          */
    double inc_psi;       /* polarisation: E along cos(psi)(-theta_hat) +
                             sin(psi) phi_hat; psi = 0 is TM (E in the plane of
                             k and z), psi = pi/2 is TE                         */
} mfdtd_ext;

/* Parametric meteor trail (extended input; the reference builds trails only
 * as a 2-D map times a Gaussian in z, setup/meteorrun.m:83-104 and
 * source/meteor-2.1.cpp:319-334).  Electron density
 *     n = n0(s) exp(-d^2 / r0^2),
 * s the position along the axis through `centre` with direction `axis`, d the
 * distance from that axis; log10 n0 rises linearly from log10n_lo at
 * s = -s_half to log10n_hi at s = +s_half and is held beyond.  Positions are
 * the grid's cell coordinates -(N-1)/2*d + i*d along every axis (metres,
 * grid centre at the origin); omega_p = sqrt(n QE^2 / (E0 ME)) with the
 * solver's constants.  The engine evaluates the map on the device (FP64), so
 * no per-cell array crosses the host boundary. */
typedef struct {
    double centre[3];   /* m                                  */
    double axis[3];     /* direction; normalised by the engine */
    double r0;          /* m, > 0                              */
    double log10n_lo;   /* log10 of n0 in m^-3 at s = -s_half  */
    double log10n_hi;   /* log10 of n0 in m^-3 at s = +s_half  */
    double s_half;      /* m, > 0                              */
} mfdtd_trail;

typedef struct mfdtd_problem mfdtd_problem; /* parsed inputs + derived tables */
typedef struct mfdtd_sim mfdtd_sim;         /* device-resident state          */

/* ---- whole-program entry point ------------------------------------------
 * Replaces running the `meteor` executable with `dir` as the working
 * directory (source/meteor-2.1.cpp:42-1649; invocation setup/writepbsfile.m:15).
 * Reads the four input files, runs every step on the GPU, and writes the same
 * output files byte for byte (log.txt differs only in timing/memory lines).
 * Like the reference, output_{E,H,J}.dat are appended to; removing stale ones
 * is the job script's task (setup/writepbsfile.m:10-13). */
int mfdtd_run_rundir(const char *dir, const mfdtd_run_opts *opts);

/* ---- problem (host) -------------------------------------------------------
 * From a run directory: replaces the input parse of
 * source/meteor-2.1.cpp:51-114 and source/meteor-fork.cpp:115,219-224,
 * source/meteor-2.1.cpp:301-315.  wp.dat/nu.dat keep their on-disk order:
 * C [Nx][Ny] as the reference reads them. */
int mfdtd_problem_from_rundir(const char *dir, mfdtd_problem **out);
/* From memory: same content.  wp2/nu2 are [Nx][Ny] C-order (the byte order of
 * wp.dat/nu.dat), B0 = {Bx, By, Bz} in tesla. */
int mfdtd_problem_create(const mfdtd_params *p, const double *wp2, const double *nu2,
                         const double B0[3], mfdtd_problem **out);
void mfdtd_problem_destroy(mfdtd_problem *pb);
/* The reference's values of every extended input. */
void mfdtd_ext_defaults(mfdtd_ext *ext);
/* Apply extended inputs to a problem and re-derive its tables.  ext may be
 * NULL (reference values).  wp3/nu3 (may be NULL) are per-cell plasma
 * frequency (rad/s) and collision frequency (1/s) maps [Nx][Ny][Nz] in C
 * order; wp3 replaces wp2 * G(z), nu3 replaces nu2 * G(z).  No counterpart in
 * the reference, which cannot express these inputs. */
int mfdtd_problem_set_ext(mfdtd_problem *pb, const mfdtd_ext *ext, const double *wp3,
                          const double *nu3);
/* Use a parametric trail for the plasma frequency (replaces wp2 * G(z) and any
 * wp3 map); NULL removes it.  Run directories carry it as trail.dat. */
int mfdtd_problem_set_trail(mfdtd_problem *pb, const mfdtd_trail *trail);
/* Grid and run sizes: out[0..5] = Nx, Ny, Nz, tsteps, nntf, nprobes. */
int mfdtd_problem_dims(const mfdtd_problem *pb, int64_t out[6]);
/* Device bytes a simulation of this problem in `form` will hold. */
int mfdtd_problem_footprint(const mfdtd_problem *pb, int32_t form, int64_t *bytes);

/* ---- simulation (device) -------------------------------------------------- */
/* The FP32 form takes its device memory from the device's default
 * stream-ordered pool, which this library sets to keep up to a quarter of the
 * device's memory cached after frees: memory a destroyed simulation held
 * stays reserved by the process, for the next simulation, up to that amount
 * (cudaMemPoolTrimTo on the default pool returns it). */
int mfdtd_sim_create(const mfdtd_problem *pb, const mfdtd_run_opts *opts, mfdtd_sim **out);
void mfdtd_sim_destroy(mfdtd_sim *s);  /* leaves its batch first, if any */
/* Advance `nsteps` time steps (source/meteor-2.1.cpp:652-1574 per step).
 * Record-step side effects (max|Ex| log line, slice records) are kept in the
 * handle when `collect_records` is nonzero. Asynchronous unless a record step
 * or guard check falls in the range. */
int mfdtd_sim_advance(mfdtd_sim *s, int32_t nsteps, int32_t collect_records);
/* Wait for queued work; returns MFDTD_ETIMEOUT if opts.timeout_s elapses. */
int mfdtd_sim_sync(mfdtd_sim *s);
/* Steps completed so far. */
int mfdtd_sim_step_index(const mfdtd_sim *s, int32_t *t);
/* Near-to-far-field sums in the layout of output_NTF.dat after the two ints
 * and fntf (source/meteor-2.1.cpp:1588-1620): Eydft[2n], Ezdft[2n], then 24
 * face arrays.  `out` must hold mfdtd_sim_ntf_size() doubles. */
int64_t mfdtd_sim_ntf_size(const mfdtd_sim *s);
int mfdtd_sim_read_ntf(mfdtd_sim *s, double *out, int64_t n);
/* Probe series [6][tsteps][nprobes] (Ex,Ey,Ez,Hx,Hy,Hz; Probe.dat order). */
int mfdtd_sim_read_probes(mfdtd_sim *s, double *out, int64_t n);
/* One field component as [Nx][Ny][Nz] doubles: comp 0..8 = Ex,Ey,Ez,Hx,Hy,Hz,Jx,Jy,Jz. */
int mfdtd_sim_read_field(mfdtd_sim *s, int32_t comp, double *out, int64_t n);
/* The record slices of the current state, computed on the device: E and H
 * each hold n >= 2*(Nx*Ny + Nx*Nz + Ny*Nz) doubles in the layout of one
 * output_E.dat / output_H.dat record without its incident arrays
 * (source/meteor-2.1.cpp:996-1013, 1322-1340; Ez is the updated value).  With
 * scattered != 0 the incident field is subtracted inside the total-field
 * region, exactly where the TF/SF corrections put it -- the scattered field
 * analysis/plotMresults.m:210-234 forms on the host for its movies. */
int mfdtd_sim_read_slices(mfdtd_sim *s, int32_t scattered, double *E, double *H, int64_t n);
/* Share of the FP32 pass's (plane, 8 x 32 tile) blocks that hold plasma;
 * elsewhere J is identically zero and the pass neither loads nor stores it
 * (1 for the FP64 plain form, which updates J everywhere as the reference
 * does). */
int mfdtd_sim_plasma_fraction(const mfdtd_sim *s, double *fraction);
/* Write output_{E,H,J}.dat (collected records), output_NTF.dat, Probe.dat
 * and the log.txt record lines into `dir`. */
int mfdtd_sim_write_outputs(mfdtd_sim *s, const char *dir);
/* Mean device time per step of the last mfdtd_sim_advance (CUDA events on the
 * simulation's stream), and the number of kernels it launched. */
int mfdtd_sim_last_timing(const mfdtd_sim *s, double *ms_per_step, int64_t *launches);

/* Bistatic radar cross section from the simulation's near-to-far-field sums,
 * replacing analysis/meteorNTF.m:236-332 (which handles only the backscatter
 * direction theta = 90 deg, phi = 180 deg) for any list of directions
 * (radians; theta from +z, phi from +x).  Uses the analysis constants of
 * analysis/loadconstants.m and the incident power of the source DFT, as the
 * MATLAB does.  out[(m * ndir + d) * 3 + {0, 1, 2}] = sigma, and its two
 * polarisation parts |L_phi + eta0 N_theta|^2 and |L_theta - eta0 N_phi|^2
 * terms, in m^2, for frequency m.  method 0: FP64 on the CUDA cores.
 * method 1: the dense contraction (sums x phases) on the tensor cores in TF32
 * with a three-term split (about 21 bits per product) and FP32 accumulation;
 * the angular reduction in FP64. */
int mfdtd_sim_far_field(mfdtd_sim *s, int32_t ndir, const double *theta, const double *phi,
                        int32_t method, double *out);

/* Far field of caller-held DFT sums without allocating any device memory.
 * No counterpart in the reference (which computes the far field in MATLAB,
 * analysis/meteorNTF.m).  For callers that cannot call cudaMalloc while they
 * run -- a plugin inside a host that owns all device memory, a service that
 * reserves its memory at start-up and forbids allocation afterwards.  The
 * working memory is one fixed array of about 17 MB inside the library.  It
 * is created on a device when the library's far-field module is first used
 * there (CUDA loads modules lazily), normally by the first call of this
 * function, and held until the process exits: make one warm-up call per
 * device at start-up, before the request path and before any stream
 * capture.  Every call looks the array's device address up again (with the
 * device current), so a context reset in between is safe.  Limits: each face
 * of the Huygens box at most 2048 cells along either in-plane axis (larger
 * grids: mfdtd_sim_far_field); ntfb >= 0.  All calls share that array and see
 * what the last call left in it, so calls whose GPU work overlaps race and
 * must be serialised by the caller.
 * ntf_dev: the 24 face arrays on the current device, output_NTF.dat order and
 * layout ([a][b][2*nntf] doubles).  fntf[nntf], srcdft (Eydft[2n] then
 * Ezdft[2n]), theta/phi[ndir] and out[nntf*ndir*3] are host arrays; out has the
 * layout of mfdtd_sim_far_field.  stream may be NULL (legacy stream); the
 * call returns after its GPU work finished. */
int mfdtd_far_field_static(const double *const ntf_dev[24], int32_t Nx, int32_t Ny, int32_t Nz,
                           int32_t ntfb, int32_t nntf, const double *fntf, double dx, double dy,
                           double dz, const double *srcdft, int32_t ndir, const double *theta,
                           const double *phi, double *out, void *stream);

/* Per-kernel-class device time of the last mfdtd_sim_advance when the
 * simulation was created with opts.profile set: for class `which` (0, 1, ...)
 * its name, mean duration of one launch in ms, and launch count.  A class
 * may time consecutive launches together: the FP32 form's class 0 is the
 * pass with the work that completes it, named after the kernels that ran in
 * that advance: "k_fp32_step_wide+k_fp32_slab" (non-record steps: the interior
 * pass with two cells per thread and, on a second stream, the march over the
 * CPML slabs and domain edges), "k_fp32_step_fast" (non-record steps on grids
 * too small for the wide pass, followed by the two CPML band kernels),
 * "k_fp32_step" (record steps: the general pass and the band kernels), joined
 * by '+' when several ran.  Returns MFDTD_EINVAL when `which` is past the last
 * class. */
int mfdtd_sim_kernel_stats(const mfdtd_sim *s, int32_t which, char *name, size_t name_len,
                           double *avg_ms, int64_t *launches);

/* ---- batches (chosen form: many trails in one persistent kernel) ----------
 * No counterpart in the reference, which runs one trail per process and fans
 * trails out as separate PBS jobs (setup/meteorbatch.m, setup/writepbsfile.m).
 * A batch advances up to mfdtd_batch_capacity() FP32 simulations together
 * (a capacity shared by every batch on the same device):
 * each time step is one launch of a persistent kernel whose CTAs pull
 * (simulation, tile, x-slab) work items from a device queue, boundary tiles
 * first; two steps are replayed as one CUDA graph.  Members keep their fields
 * on the device; a member past its step count idles until removed.  Members
 * join at step 0, must share the batch's device and current update (Young DI,
 * uniform Lee-Kalluri or tabulated Lee-Kalluri), and cannot be advanced on
 * their own while in a batch.  Read a member's results only after
 * mfdtd_batch_sync. */
typedef struct mfdtd_batch mfdtd_batch;
int mfdtd_batch_capacity(void);
int mfdtd_batch_create(int32_t device, mfdtd_batch **out);
void mfdtd_batch_destroy(mfdtd_batch *b);  /* members stay valid */
int mfdtd_batch_add(mfdtd_batch *b, mfdtd_sim *s);
int mfdtd_batch_remove(mfdtd_batch *b, mfdtd_sim *s);
/* Enqueue nsteps time steps of every member (asynchronous). */
int mfdtd_batch_run(mfdtd_batch *b, int32_t nsteps);
/* Wait for the batch; updates every member's step index. */
int mfdtd_batch_sync(mfdtd_batch *b);
/* Autotuner: time every (tile shape, slab depth, CTAs per SM) on the live
 * members (they advance while being timed) and keep the fastest; best_* may
 * be NULL.  Tile shapes: 8 x 32 (j, k) tiles everywhere; and, when the
 * members qualify for the CPML slab march (oblique incidence without a plate
 * or sphere, no Lee-Kalluri table), their interior tiles paired into 8 x 64
 * tiles with two cells per thread (at most two CTAs per SM).  A CTA count a
 * shape cannot run is skipped for that shape. */
int mfdtd_batch_tune(mfdtd_batch *b, const int32_t *slab_depths, int32_t n_depths,
                     const int32_t *ctas_per_sm, int32_t n_ctas, int32_t *best_depth,
                     int32_t *best_ctas);
/* The (j, k) tile shape the batch runs its interior tiles with: 8 x 32 or
 * 8 x 64 (see mfdtd_batch_tune).  Untuned, a batch whose members qualify for
 * the slab march runs 8 x 64 at two CTAs per SM. */
int mfdtd_batch_tile_shape(const mfdtd_batch *b, int32_t *rows, int32_t *cols);

/* ---- serving loop (chosen form) ---------------------------------------------
 * No counterpart in the reference (its sweep driver is MATLAB + PBS,
 * setup/meteorbatch.m).  A server owns a worker thread on one device.  Jobs
 * (a problem plus the radar directions wanted) are queued by
 * mfdtd_server_submit and admitted in arrival order while their FP32 device
 * footprint fits under hbm_cap_bytes and their batch has a free slot; every
 * round the worker advances all admitted jobs steps_per_round steps in
 * batches (one per current-update kind, overlapping on the device), retires
 * the jobs that reached their step count -- far field computed on the device
 * (method 1: the contraction on the tensor cores), device memory freed -- and
 * admits waiting jobs into the freed space.  A job of at least 2^25 cells
 * fills the GPU by itself: it takes no batch slot and marches alone, with the
 * single-simulation kernels on its own stream, while the batches run.
 * Fields stay on the device from admission to retirement. */
typedef struct mfdtd_server mfdtd_server;
int mfdtd_server_create(int32_t device, int64_t hbm_cap_bytes, int32_t steps_per_round,
                        mfdtd_server **out);
/* Stops the worker; jobs not yet retired are dropped. */
void mfdtd_server_destroy(mfdtd_server *s);
/* Queue a job: the problem is copied; theta/phi[ndir] in radians (as for
 * mfdtd_sim_far_field).  Fails with MFDTD_ENOMEM when the job alone exceeds
 * the cap. */
int mfdtd_server_submit(mfdtd_server *s, const mfdtd_problem *pb, int32_t ndir,
                        const double *theta, const double *phi, int64_t *job_id);
/* Wait up to wait_ms for the job.  *done = 1: out[nntf*ndir*3] holds the cross
 * sections (mfdtd_sim_far_field layout), times[0..2] = seconds from submission
 * to admission, to retirement, and device seconds are not separable (0); the
 * job record is released.  *done = 0: still queued or running. */
int mfdtd_server_poll(mfdtd_server *s, int64_t job_id, int32_t wait_ms, double *out, int64_t n_out,
                      double times[3], int32_t *done);
/* out[0..4] = submitted, queued, running, retired, device bytes in use. */
int mfdtd_server_stats(mfdtd_server *s, int64_t out[5]);
/* Cancel a job.  A queued job leaves the queue at once; a running job leaves
 * its batch at the end of the worker's current round, without a far field,
 * and its device memory returns to the cap; a finished job's result is
 * discarded.  Polling a canceled job then fails with MFDTD_ECANCELED and
 * releases it (a finished job is released here).  MFDTD_EINVAL for an
 * unknown id. */
int mfdtd_server_cancel(mfdtd_server *s, int64_t job_id);

/* ---- errors ---------------------------------------------------------------- */
/* Copy the last error message of the calling thread into buf (NUL-terminated). */
int mfdtd_last_error(char *buf, size_t n);
/* Library version string. */
const char *mfdtd_version(void);

#ifdef __cplusplus
}
#endif
#endif /* MFDTD_H */
