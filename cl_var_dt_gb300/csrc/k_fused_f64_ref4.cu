// Instantiations of the fused step kernel: double, ref4 model.
#include "fused_impl.cuh"

namespace clv {
void *fused_kernel_f64_ref4(int spt, int ln, bool fast) { return fused_fn<double, CLV_MODEL_REF4>(spt, ln, fast); }
}  // namespace clv
