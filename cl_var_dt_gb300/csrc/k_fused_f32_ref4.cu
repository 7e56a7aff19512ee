// Instantiations of the fused step kernel: float, ref4 model.
#include "fused_impl.cuh"

namespace clv {
void *fused_kernel_f32_ref4(int spt, int ln, bool fast) { return fused_fn<float, CLV_MODEL_REF4>(spt, ln, fast); }
}  // namespace clv
