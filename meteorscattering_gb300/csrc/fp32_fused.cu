// fp32_fused.cu -- FP32 fused form of the time step.
#include <cuda_runtime.h>

#include "fp32.hpp"

namespace mfdtd {

struct Fp32Sim::Impl {};

int64_t Fp32Sim::footprint(const Problem &P) { return (int64_t)P.cells() * 76; }
void Fp32Sim::init(const Problem &, void *) {
    throw Error(MFDTD_EINVAL, "FP32 fused form is not available in this build");
}
int Fp32Sim::step(int, bool, void *, void *const *) { return 0; }
int Fp32Sim::kernel_classes() { return 1; }
const char *Fp32Sim::kernel_name(int) { return "fp32_step"; }
void Fp32Sim::record(double *, double *, double *, void *) {}
double Fp32Sim::guard(void *) { return 0; }
void Fp32Sim::flush(int, void *) {}
void Fp32Sim::read_ntf(int, double *, void *) {}
void Fp32Sim::read_probes(double *, void *) {}
void Fp32Sim::read_field(int, double *, void *) {}
Fp32Sim::~Fp32Sim() { delete impl_; }

}  // namespace mfdtd
