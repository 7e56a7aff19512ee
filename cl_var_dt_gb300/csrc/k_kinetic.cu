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

namespace clv {

template <class C2, int R>
struct Radix;

// y_q = sum_r a_r exp(S * 2 pi i r q / R), S = -1 forward, +1 inverse.
template <class C2>
__device__ __forceinline__ C2 times_si(C2 z, int S) {  // S * i * z
    C2 r; r.x = -S * z.y; r.y = S * z.x; return r;
}

template <class C2>
struct Radix<C2, 2> {
    static __device__ __forceinline__ void run(C2 *a, int) {
        C2 t = a[0];
        a[0] = cadd(t, a[1]);
        a[1] = csub(t, a[1]);
    }
};
template <class C2>
struct Radix<C2, 4> {
    static __device__ __forceinline__ void run(C2 *a, int S) {
        C2 s02 = cadd(a[0], a[2]), d02 = csub(a[0], a[2]);
        C2 s13 = cadd(a[1], a[3]), d13 = times_si(csub(a[1], a[3]), S);
        a[0] = cadd(s02, s13);
        a[2] = csub(s02, s13);
        a[1] = cadd(d02, d13);
        a[3] = csub(d02, d13);
    }
};
template <class C2>
struct Radix<C2, 8> {
    static __device__ __forceinline__ void run(C2 *a, int S) {
        using R = decltype(a[0].x);
        const R h = (R)0.70710678118654752440;
        C2 e[4] = {a[0], a[2], a[4], a[6]};
        C2 o[4] = {a[1], a[3], a[5], a[7]};
        Radix<C2, 4>::run(e, S);
        Radix<C2, 4>::run(o, S);
        // twiddles exp(S 2 pi i q/8) for q = 1, 2, 3
        C2 w1; w1.x = h * (o[1].x - S * o[1].y); w1.y = h * (o[1].y + S * o[1].x);
        C2 w2 = times_si(o[2], S);
        C2 w3; w3.x = h * (-o[3].x - S * o[3].y); w3.y = h * (-o[3].y + S * o[3].x);
        a[0] = cadd(e[0], o[0]); a[4] = csub(e[0], o[0]);
        a[1] = cadd(e[1], w1);   a[5] = csub(e[1], w1);
        a[2] = cadd(e[2], w2);   a[6] = csub(e[2], w2);
        a[3] = cadd(e[3], w3);   a[7] = csub(e[3], w3);
    }
};
template <class C2>
struct Radix<C2, 3> {
    static __device__ __forceinline__ void run(C2 *a, int S) {
        using R = decltype(a[0].x);
        const R half = (R)0.5, s3 = (R)0.86602540378443864676;
        C2 t1 = cadd(a[1], a[2]), t2 = csub(a[1], a[2]);
        C2 m; m.x = a[0].x - half * t1.x; m.y = a[0].y - half * t1.y;
        C2 r = times_si(cscale(s3, t2), S);
        a[0] = cadd(a[0], t1);
        a[1] = cadd(m, r);
        a[2] = csub(m, r);
    }
};
template <class C2>
struct Radix<C2, 5> {
    static __device__ __forceinline__ void run(C2 *a, int S) {
        using R = decltype(a[0].x);
        const R c1 = (R)0.30901699437494742410, c2 = (R)-0.80901699437494742410;
        const R s1 = (R)0.95105651629515357212, s2 = (R)0.58778525229247312917;
        C2 t1 = cadd(a[1], a[4]), t2 = cadd(a[2], a[3]);
        C2 t3 = csub(a[1], a[4]), t4 = csub(a[2], a[3]);
        C2 b1; b1.x = a[0].x + c1 * t1.x + c2 * t2.x; b1.y = a[0].y + c1 * t1.y + c2 * t2.y;
        C2 b2; b2.x = a[0].x + c2 * t1.x + c1 * t2.x; b2.y = a[0].y + c2 * t1.y + c1 * t2.y;
        C2 q1; q1.x = s1 * t3.x + s2 * t4.x; q1.y = s1 * t3.y + s2 * t4.y;
        C2 q2; q2.x = s2 * t3.x - s1 * t4.x; q2.y = s2 * t3.y - s1 * t4.y;
        q1 = times_si(q1, S);
        q2 = times_si(q2, S);
        a[0] = cadd(a[0], cadd(t1, t2));
        a[1] = cadd(b1, q1);
        a[4] = csub(b1, q1);
        a[2] = cadd(b2, q2);
        a[3] = csub(b2, q2);
    }
};

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
