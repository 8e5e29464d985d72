// meteor_main.cpp -- drop-in replacement for the reference `meteor` executable.
//
// Same contract as the reference (setup/writepbsfile.m:15): no arguments, the
// working directory is the run directory.  Optional extras for scripted use:
//   meteor [rundir] [--fp32] [--device N] [--quiet]
// The exit status is 0 on success and 1 on any error (the reference always
// returns 0 and crashes on missing files); the error text goes to stderr.
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "../../include/mfdtd.h"

int main(int argc, char **argv) {
    const char *dir = ".";
    mfdtd_run_opts opts;
    std::memset(&opts, 0, sizeof opts);
    for (int a = 1; a < argc; a++) {
        if (!std::strcmp(argv[a], "--fp32")) opts.form = MFDTD_FORM_FP32_FUSED;
        else if (!std::strcmp(argv[a], "--quiet")) opts.quiet = 1;
        else if (!std::strcmp(argv[a], "--device") && a + 1 < argc) opts.device = std::atoi(argv[++a]);
        else dir = argv[a];
    }
    int rc = mfdtd_run_rundir(dir, &opts);
    if (rc != MFDTD_OK) {
        char msg[1024];
        mfdtd_last_error(msg, sizeof msg);
        std::fprintf(stderr, "meteor: error %d: %s\n", rc, msg);
        return 1;
    }
    return 0;
}
