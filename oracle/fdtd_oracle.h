/*
 * fdtd_oracle.h -- CPU restatement of the meteor FDTD solver (TEST INFRASTRUCTURE).
 *
 * This is the checker for the GPU engine, not part of the product.  Only the
 * tests, the smoke check and the benchmark's CPU-baseline leg may load it.
 *
 * Parity is pinned: tests/test_oracle_pin.py runs this restatement and the
 * reference solver (source/meteor-fork.cpp, compiled from its own sources by
 * oracle/Makefile) on the same run directories and requires byte-identical
 * output files; tests/golden/ holds the reference outputs for runs where the
 * reference binary is not available.
 */
#ifndef FDTD_ORACLE_H
#define FDTD_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Run the solver in directory `dir` exactly like the reference executable run
 * with that directory as its working directory: read inputs.dat, B0.dat,
 * wp.dat, nu.dat; write log.txt, output_{E,H,J}.dat (appended), output_NTF.dat
 * and Probe.dat.  `max_steps` >= 0 stops the time loop early (for timing
 * samples; outputs are still written).  `nthreads` > 0 sets the OpenMP thread
 * count.  `loop_seconds` (may be NULL) receives the wall time of the time loop.
 * `mirror_dead_work` != 0 also performs the reference's unused per-cell
 * |E| / Poynting-magnitude pass (source/meteor-2.1.cpp:1460-1487) so that the
 * timing matches the reference's cost; it has no effect on any output.
 * Returns 0 on success, a negative number on a missing/short input file or an
 * invalid size. */
int oracle_run_dir(const char *dir, int max_steps, int nthreads,
                   int mirror_dead_work, double *loop_seconds);

#ifdef __cplusplus
}
#endif
#endif
