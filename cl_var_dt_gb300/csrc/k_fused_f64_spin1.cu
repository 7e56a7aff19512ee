// Instantiations of the fused step kernel: double, spin1 model.
#include "fused_impl.cuh"

namespace clv {
void *fused_kernel_f64_spin1(int spt, int ln, bool fast) { return fused_fn<double, CLV_MODEL_SPIN1>(spt, ln, fast); }
}  // namespace clv
