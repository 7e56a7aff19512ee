// Instantiations of the fused step kernel: float, spin1 model.
#include "fused_impl.cuh"

namespace clv {
void *fused_kernel_f32_spin1(int spt, int ln, bool fast) { return fused_fn<float, CLV_MODEL_SPIN1>(spt, ln, fast); }
}  // namespace clv
