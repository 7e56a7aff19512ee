// k_kinetic.cu -- kinetic term as a real, even Fourier filter applied line by
// line along one lattice axis, in shared memory:
//
//     dst = F^-1 [ f(k) . F src ]        (one axis, all lines of all chains)
//
// The reference computes its kinetic term with batched cuFFT Z2Z transforms
// over all spatial axes, a -px^2 multiply and a normalisation pass
// (Propagator_without_cutoff.cu:410-424, 160-203; Lattice.cu:135-187).  Its
// multiplier depends on px only, so the transforms along y and z cancel and the
// same result is one filter pass along x with f(k) = -px(k)^2 / (a_x NX).  The
// exponential kinetic factor exp(-eps (k^2/2 - mu - q m^2)) of the spin-1 model
// is separable, exp(eps(mu + q m^2)) * prod_d exp(-eps k_d^2/2), so it is one
// pass per axis.  Each CTA holds a bundle of complete lines in shared memory
// and runs a Stockham autosort FFT (radix 2/3/4/5/8) forward, the filter and
// the inverse FFT there, so every element is read once and written once per
// pass.
#include "clv_internal.cuh"
#include "clv_launch.h"
#include "fft_radix.cuh"

namespace clv {

// One Stockham pass of radix R over `nl` lines of length n held in src/dst.
template <class C2, int R>
__device__ __forceinline__ void stockham_pass(const C2 *__restrict__ src, C2 *__restrict__ dst,
                                              const C2 *__restrict__ tw, int n, int nl, int Ns,
                                              int S) {
    const int nR = n / R;
    const int step = n / (Ns * R);  // twiddle index stride
    for (int b = threadIdx.x; b < nl * nR; b += blockDim.x) {
        const int w = b / nR, j = b - w * nR;
        const int k = j % Ns;
        const C2 *ls = src + w * n;
        C2 v[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            C2 x = ls[j + r * nR];
            if (r > 0 && k > 0) {
                C2 t = tw[k * r * step];
                t.y = S < 0 ? t.y : -t.y;  // table holds exp(-2 pi i k/n)
                x = cmul(x, t);
            }
            v[r] = x;
        }
        Radix<C2, R>::run(v, S);
        C2 *ld = dst + w * n + (j / Ns) * Ns * R + k;
#pragma unroll
        for (int q = 0; q < R; ++q) ld[q * Ns] = v[q];
    }
}

// Full transform of all lines in buf; returns the buffer holding the result.
template <class C2>
__device__ C2 *fft_lines(C2 *buf0, C2 *buf1, const C2 *tw, const AxisDev &ax, int nl, int S) {
    C2 *src = buf0, *dst = buf1;
    int Ns = 1;
    for (int p = 0; p < ax.nf; ++p) {
        const int R = ax.fac[p];
        switch (R) {
            case 8: stockham_pass<C2, 8>(src, dst, tw, ax.n, nl, Ns, S); break;
            case 4: stockham_pass<C2, 4>(src, dst, tw, ax.n, nl, Ns, S); break;
            case 2: stockham_pass<C2, 2>(src, dst, tw, ax.n, nl, Ns, S); break;
            case 3: stockham_pass<C2, 3>(src, dst, tw, ax.n, nl, Ns, S); break;
            default: stockham_pass<C2, 5>(src, dst, tw, ax.n, nl, Ns, S); break;
        }
        __syncthreads();
        C2 *t = src; src = dst; dst = t;
        Ns *= R;
    }
    return src;
}

template <class R>
__device__ __forceinline__ const typename Cx<R>::T *twiddles(const AxisDev &ax);
template <>
__device__ __forceinline__ const double2 *twiddles<double>(const AxisDev &ax) { return ax.tw64; }
template <>
__device__ __forceinline__ const float2 *twiddles<float>(const AxisDev &ax) { return ax.tw32; }
template <class R>
__device__ __forceinline__ const R *filter_of(const AxisDev &ax, int which);
template <>
__device__ __forceinline__ const double *filter_of<double>(const AxisDev &ax, int which) {
    return which == 0 ? ax.filt64 : ax.efilt64;
}
template <>
__device__ __forceinline__ const float *filter_of<float>(const AxisDev &ax, int which) {
    return which == 0 ? ax.filt32 : ax.efilt32;
}

// mode 0: dst = filtered(src) (times the component constant when with_const);
// mode 1: dst += filtered(src).  blockIdx.y selects the field (psi, psibar).
template <class R>
__global__ void __launch_bounds__(256)
line_filter_kernel(const ChainDev *__restrict__ chains, const LineTask *__restrict__ tasks,
                   int axis, const typename Cx<R>::T *src0, const typename Cx<R>::T *src1,
                   typename Cx<R>::T *dst0, typename Cx<R>::T *dst1, int filter, int mode,
                   int with_const) {
    using C2 = typename Cx<R>::T;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const LineTask task = tasks[blockIdx.x];
    const ChainDev &ch = chains[task.chain];
    const AxisDev &ax = ch.axis[axis];
    const int n = ax.n, inner = ax.inner, nl = task.nlines;
    C2 *buf0 = reinterpret_cast<C2 *>(smem_raw);
    C2 *buf1 = buf0 + nl * n;
    const C2 *src = (blockIdx.y == 0 ? src0 : src1) + ch.off;
    C2 *dst = (blockIdx.y == 0 ? dst0 : dst1) + ch.off;
    const int total = nl * n;
    for (int e = threadIdx.x; e < total; e += blockDim.x) {
        int w, i;
        if (inner == 1) { w = e / n; i = e - w * n; }
        else { i = e / nl; w = e - i * nl; }
        const int l = task.line0 + w;
        const long long g = (long long)(l / inner) * n * inner + (long long)i * inner + (l % inner);
        buf0[w * n + i] = src[g];
    }
    __syncthreads();
    const C2 *tw = twiddles<R>(ax);
    C2 *spec = fft_lines<C2>(buf0, buf1, tw, ax, nl, -1);
    C2 *other = spec == buf0 ? buf1 : buf0;
    const R *f = filter_of<R>(ax, filter);
    const long long slice_elems = (long long)ch.nt * ch.V;
    for (int e = threadIdx.x; e < total; e += blockDim.x) {
        const int w = e / n, k = e - w * n;
        R m = f[k];
        if (with_const) {
            const int l = task.line0 + w;
            const long long base = (long long)(l / inner) * n * inner + (l % inner);
            m *= (R)ch.comp_const[(int)(base / slice_elems)];
        }
        spec[e] = cscale(m, spec[e]);
    }
    __syncthreads();
    C2 *res = fft_lines<C2>(spec, other, tw, ax, nl, +1);
    for (int e = threadIdx.x; e < total; e += blockDim.x) {
        int w, i;
        if (inner == 1) { w = e / n; i = e - w * n; }
        else { i = e / nl; w = e - i * nl; }
        const int l = task.line0 + w;
        const long long g = (long long)(l / inner) * n * inner + (long long)i * inner + (l % inner);
        C2 v = res[w * n + i];
        if (mode == 1) v = cadd(dst[g], v);
        dst[g] = v;
    }
}

template <class R>
cudaError_t launch_line_filter(const LaunchLineFilter &L, cudaStream_t s) {
    using C2 = typename Cx<R>::T;
    if (L.ntasks == 0) return cudaSuccess;
    const size_t smem = 2 * (size_t)L.max_bundle * sizeof(C2);
    dim3 grid(L.ntasks, L.nfields);
    line_filter_kernel<R><<<grid, 256, smem, s>>>(
        L.chains, L.tasks, L.axis, (const C2 *)L.src0, (const C2 *)L.src1, (C2 *)L.dst0,
        (C2 *)L.dst1, L.filter, L.mode, L.with_const);
    return cudaGetLastError();
}

cudaError_t setup_line_filter() {
    const int bytes = 2 * kMaxBundleElems64 * (int)sizeof(double2);
    cudaError_t e = cudaFuncSetAttribute(line_filter_kernel<double>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(line_filter_kernel<float>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

template cudaError_t launch_line_filter<double>(const LaunchLineFilter &, cudaStream_t);
template cudaError_t launch_line_filter<float>(const LaunchLineFilter &, cudaStream_t);

}  // namespace clv
