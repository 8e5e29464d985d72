// farfield.hpp -- near-to-far-field projection (farfield.cu).
#pragma once

#include "common.hpp"

namespace mfdtd {

// Bistatic cross sections from the 24 device-resident DFT arrays `ntf`
// (output_NTF.dat layout).  `srcdft` = Eydft[2n] then Ezdft[2n] (host).
// out[(m * ndir + d) * 3 + {0,1,2}] = sigma, sigma_a, sigma_b in m^2.
// method 0: FP64 on the CUDA cores; 1: the dense stage on the tensor cores
// (TF32 split precision, FP32 accumulation), the reduction in FP64.
void far_field_fp64(const Problem &P, double *const ntf[24], const double *srcdft, int ndir,
                    const double *theta, const double *phi, double *out, void *stream,
                    int method = 0);

}  // namespace mfdtd
