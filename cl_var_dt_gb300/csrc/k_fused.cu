// k_fused.cu -- launch and set-up of the fused step kernel (fused_impl.cuh);
// its instantiations live in k_fused_<precision>_<model>.cu so that they
// compile in parallel.
#include "fused_impl.cuh"

namespace clv {

template <class R>
static void *fused_kernel_of(int model, int spt, int ln, bool fast) {
    if (sizeof(R) == 4)
        return model == CLV_MODEL_REF4 ? fused_kernel_f32_ref4(spt, ln, fast) : fused_kernel_f32_spin1(spt, ln, fast);
    return model == CLV_MODEL_REF4 ? fused_kernel_f64_ref4(spt, ln, fast) : fused_kernel_f64_spin1(spt, ln, fast);
}

// The production variant (fused_step_kernel's FAST) serves launches that use
// exactly its fixed choices (both fields per CTA among them).
static bool fused_fast(const LaunchFused &L) {
    return L.ln > 0 && L.noise == CLV_NOISE_PHILOX && L.dt_rule == CLV_DT_K_OVER_MAX && L.use_tma &&
           !L.drift_out && L.mode != FUSED_MAXONLY && !L.split;
}

template <class R>
cudaError_t launch_fused(const LaunchFused &L, cudaStream_t s) {
    if (L.ntasks == 0) return cudaSuccess;
    void *fn = fused_kernel_of<R>(L.model, L.spt, L.ln, fused_fast(L));
    void *args[] = {const_cast<LaunchFused *>(&L)};
    return cudaLaunchKernel(fn, dim3(L.ntasks), dim3(256), args, L.smem_bytes, s);
}

// Allow the device's whole opt-in shared memory (minus the kernel's static
// shared memory), then report how many CTAs of L.smem_bytes fit on one SM.
template <class R>
cudaError_t setup_fused(const LaunchFused &L, int *ctas_per_sm) {
    int dev = 0, optin = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e != cudaSuccess) return e;
    void *fn = nullptr;
    for (int fast = 0; fast < (L.ln > 0 ? 2 : 1); ++fast) {
        fn = fused_kernel_of<R>(L.model, L.spt, L.ln, fast != 0);
        cudaFuncAttributes fa{};
        e = cudaFuncGetAttributes(&fa, fn);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     optin - (int)fa.sharedSizeBytes);
        if (e != cudaSuccess) return e;
    }
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas_per_sm, fn, 256, L.smem_bytes);
}

template cudaError_t launch_fused<double>(const LaunchFused &, cudaStream_t);
template cudaError_t launch_fused<float>(const LaunchFused &, cudaStream_t);
template cudaError_t setup_fused<double>(const LaunchFused &, int *);
template cudaError_t setup_fused<float>(const LaunchFused &, int *);

}  // namespace clv
