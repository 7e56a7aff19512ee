// k_plane.cu -- kinetic filter of a whole square plane (both of its axes) in one
// pass over HBM, for the tiled path's 2D slices (n x n) and the (y, z) planes of
// 3D slices (n x n at each x), n = 32, 64, 96 or 128.
//
// The spin-1 kinetic factor exp(-eps k^2/2) is a product over the axes, so the
// plane's filter is the line filter along one axis followed by the line filter
// along the other (the same operator as two axis_filter_kernel launches,
// Propagator_without_cutoff.cu:410-424 for the reference's transform sequence).
// One CTA (plane_threads(n) threads) holds one plane of one (component, tau)
// slice of one field in shared memory (n rows at an odd pitch n + 1).  Each line
// filter runs in place as a mixed-radix Cooley-Tukey transform: decimation in
// frequency forward, the filter, decimation in time back.  A butterfly reads and
// writes the same R elements, so the butterflies of a pass are independent: a
// thread streams its butterflies one after another with R values in registers,
// and one block barrier separates the passes.  The forward passes leave the
// spectrum in digit-reversed order; the middle pass multiplies each frequency by
// its filter value there, and the inverse passes take digit-reversed input back
// to natural order, so the filter needs no reordering pass.
// Butterfly b of a pass is butterfly j = b / n of line l = b % n, so the 32 lanes
// of a warp take 32 consecutive lines at one j: their addresses differ by the line
// stride (the odd pitch along rows, 1 along columns) and are free of bank
// conflicts, while the twiddle and filter reads of the warp are one broadcast.
// The first pass (along the slower axis, whose lines are columns) reads its
// butterflies straight from global memory, 32 consecutive columns a warp; the
// plane is written back from shared memory in row order.  The plane is read once
// and written once: half the traffic of the two axis launches it replaces.
#include "clv_internal.cuh"
#include "clv_launch.h"
#include "fused_impl.cuh"

namespace clv {

// Span L_p = n / (R_0 ... R_{p-1}) of forward pass p of the plan plane_fac(n, .):
// pass p transforms blocks of L_p elements, R_p strided sub-sequences of each.
__host__ __device__ constexpr int plane_span(int n, int p) {
    int L = n;
    for (int i = 0; i < p; ++i) L /= plane_fac(n, i);
    return L;
}

// Butterflies whose global loads the first pass issues together: all of a thread's
// where one CTA fills the SM (FP32 planes of 128, FP64 planes of 96), else one (the
// other resident CTAs keep loads in flight).
__host__ __device__ constexpr int plane_first_group(int n, int esz) {
    return (n == 128 && esz == 8) || (n == 96 && esz == 16) ? n * (n / plane_fac(n, 0)) / plane_threads(n) : 1;
}

// Butterflies of a pass unrolled together: all where one CTA fills the SM, else one
// at a time (streamed: the registers of several resident CTAs).
__host__ __device__ constexpr int plane_unroll(int n, int esz, int per) {
    return plane_first_group(n, esz) > 1 ? per : 1;
}

// Frequency index of the q = 0 output of middle-pass butterfly j (the output q has
// frequency mid_freq(j) + q n / R_last): position i = sum_p q_p (L_p / R_p) after the
// forward passes holds frequency sum_p q_p (R_0 ... R_{p-1}); j = i / R_last.
template <int N, int P = 0, int W = 1>
__device__ __forceinline__ int mid_freq(int rem) {
    constexpr int NF = plane_nfac(N), RL = plane_fac(N, NF - 1);
    if constexpr (P >= NF - 1) {
        return 0;
    } else {
        constexpr int S = plane_span(N, P + 1) / RL;  // place value of digit p in j
        const int q = rem / S;
        return q * W + mid_freq<N, P + 1, W * plane_fac(N, P)>(rem - q * S);
    }
}

// Forward pass p (decimation in frequency) over the n lines of the plane t (element a
// of line l at t[l * LS + a * ES]): butterfly (block, k) takes elements
// block L + k + m S (m < R, S = L / R), y_q = sum_m x_m w_R^{mq}, then y_q w_L^{qk}, in
// place.  FIRST: the inputs come from the global plane g (element a of column line l
// at g[a * n + l]) and the twiddles from the global table tw.
template <class C2, int N, int P, bool FIRST>
__device__ __forceinline__ void dif_pass(C2 *t, int LS, int ES, const C2 *tw, const C2 *g) {
    constexpr int T = plane_threads(N), R = plane_fac(N, P), L = plane_span(N, P), S = L / R;
    constexpr int NB = N * (N / R), PER = NB / T;
    constexpr int G = FIRST ? plane_first_group(N, (int)sizeof(C2)) : 1;
    static_assert(PER * T == NB && PER % G == 0, "butterflies per thread");
#pragma unroll(FIRST ? 1 : plane_unroll(N, (int)sizeof(C2), PER))
    for (int p0 = 0; p0 < PER; p0 += G) {
        C2 v[G][R];
#pragma unroll
        for (int u = 0; u < G; ++u) {
            const int b = threadIdx.x + (p0 + u) * T, l = b % N, j = b / N;
            const int a0 = (j / S) * L + j % S;
#pragma unroll
            for (int m = 0; m < R; ++m) {
                if constexpr (FIRST) v[u][m] = g[(a0 + m * S) * N + l];
                else v[u][m] = t[l * LS + (a0 + m * S) * ES];
            }
        }
#pragma unroll
        for (int u = 0; u < G; ++u) {
            const int b = threadIdx.x + (p0 + u) * T, l = b % N, j = b / N;
            const int a0 = (j / S) * L + j % S, k = j % S;
            Radix<C2, R>::template run<-1>(v[u]);
            if constexpr (S > 1) {
#pragma unroll
                for (int q = 1; q < R; ++q) v[u][q] = cmul(v[u][q], tw[q * k * (N / L)]);
            }
#pragma unroll
            for (int q = 0; q < R; ++q) t[l * LS + (a0 + q * S) * ES] = v[u][q];
        }
    }
}

// Inverse of forward pass p (decimation in time): inputs y_q at block L + k + q S
// times conj(w_L^{qk}), x_m = sum_q y_q w_R^{-mq}, in place.
template <class C2, int N, int P>
__device__ __forceinline__ void dit_pass(C2 *t, int LS, int ES, const C2 *tw) {
    constexpr int T = plane_threads(N), R = plane_fac(N, P), L = plane_span(N, P), S = L / R;
    constexpr int NB = N * (N / R), PER = NB / T;
    static_assert(PER * T == NB, "butterflies per thread");
#pragma unroll(plane_unroll(N, (int)sizeof(C2), PER))
    for (int p = 0; p < PER; ++p) {
        const int b = threadIdx.x + p * T, l = b % N, j = b / N;
        const int a0 = (j / S) * L + j % S, k = j % S;
        C2 v[R];
#pragma unroll
        for (int q = 0; q < R; ++q) {
            C2 x = t[l * LS + (a0 + q * S) * ES];
            if (S > 1 && q > 0) {
                C2 w = tw[q * k * (N / L)];
                w.y = -w.y;
                x = cmul(x, w);
            }
            v[q] = x;
        }
        Radix<C2, R>::template run<1>(v);
#pragma unroll
        for (int m = 0; m < R; ++m) t[l * LS + (a0 + m * S) * ES] = v[m];
    }
}

// The last forward pass (span R_last, no twiddles), the filter f at each output's
// frequency times cst, and the first inverse pass, in registers.
template <class C2, class RR, int N>
__device__ __forceinline__ void mid_pass(C2 *t, int LS, int ES, const RR *f, RR cst) {
    constexpr int T = plane_threads(N), NF = plane_nfac(N), R = plane_fac(N, NF - 1), nR = N / R;
    constexpr int NB = N * nR, PER = NB / T;
    static_assert(PER * T == NB, "butterflies per thread");
#pragma unroll(plane_unroll(N, (int)sizeof(C2), PER))
    for (int p = 0; p < PER; ++p) {
        const int b = threadIdx.x + p * T, l = b % N, j = b / N;
        C2 v[R];
#pragma unroll
        for (int m = 0; m < R; ++m) v[m] = t[l * LS + (j * R + m) * ES];
        Radix<C2, R>::template run<-1>(v);
        const int fj = mid_freq<N>(j);
#pragma unroll
        for (int q = 0; q < R; ++q) v[q] = cscale(f[fj + q * nR] * cst, v[q]);
        Radix<C2, R>::template run<1>(v);
#pragma unroll
        for (int m = 0; m < R; ++m) t[l * LS + (j * R + m) * ES] = v[m];
    }
}

template <class C2, int N, int P>
__device__ __forceinline__ void plane_fwd(C2 *t, int LS, int ES, const C2 *tw) {
    if constexpr (P < plane_nfac(N) - 1) {
        dif_pass<C2, N, P, false>(t, LS, ES, tw, nullptr);
        __syncthreads();
        plane_fwd<C2, N, P + 1>(t, LS, ES, tw);
    }
}

template <class C2, int N, int P>
__device__ __forceinline__ void plane_inv(C2 *t, int LS, int ES, const C2 *tw) {
    if constexpr (P >= 0) {
        dit_pass<C2, N, P>(t, LS, ES, tw);
        __syncthreads();
        plane_inv<C2, N, P - 1>(t, LS, ES, tw);
    }
}

// Filter all n lines of the plane along one axis, in place, from forward pass P0 on
// (P0 = 1: the caller ran pass 0); ends with a block barrier.
template <class C2, class RR, int N, int P0>
__device__ __forceinline__ void plane_lines_filter(C2 *t, int LS, int ES, const C2 *tw, const RR *f, RR cst) {
    constexpr int NF = plane_nfac(N);
    static_assert(NF >= 2, "two radix factors at least");
    plane_fwd<C2, N, P0>(t, LS, ES, tw);
    mid_pass<C2, RR, N>(t, LS, ES, f, cst);
    __syncthreads();
    plane_inv<C2, N, NF - 2>(t, LS, ES, tw);
}

// Resident CTAs per SM the registers are budgeted for (shared memory allows as many).
__host__ __device__ constexpr int plane_min_ctas(int n, int esz) {
    return esz == 8 ? (n == 32 ? 8 : (n == 64 ? 4 : (n == 96 ? 3 : 1))) : (n == 32 ? 4 : (n == 64 ? 3 : 1));
}

// Task: AxisTask {chain, slice = c * nt + tau, l0 = plane index within the slice
// (the x index of a 3D slice, 0 for 2D)}; blockIdx.x % 2 selects the field.
// Axes A.axis (rows, the slower one) and A.axis + 1 (columns, contiguous).
template <class R, int N>
__global__ void __launch_bounds__(plane_threads(N), plane_min_ctas(N, (int)sizeof(R) * 2))
plane_filter_kernel(const LaunchAxis A) {
    using C2 = typename Cx<R>::T;
    constexpr int T = plane_threads(N), PL = plane_pitch(N), EPT = N * N / T;
    extern __shared__ __align__(128) unsigned char smem[];
    const AxisTask task = A.tasks[blockIdx.x >> 1];
    const int field = (int)(blockIdx.x & 1);
    const ChainDev &ch = A.chains[task.chain];
    const AxisDev &axr = ch.axis[A.axis], &axc = ch.axis[A.axis + 1];
    C2 *twS = reinterpret_cast<C2 *>(smem);
    R *fr = reinterpret_cast<R *>(smem + N * sizeof(C2));
    R *fc = fr + N;
    C2 *tile = reinterpret_cast<C2 *>(smem + plane_tab_bytes(N, sizeof(C2)));
    const long long soff = ch.off + (long long)task.slice * ch.V + (long long)task.l0 * (N * N);
    const C2 *src = reinterpret_cast<const C2 *>(field ? A.src1 : A.src0) + soff;
    C2 *dst = reinterpret_cast<C2 *>(field ? A.dst1 : A.dst0) + soff;
    const C2 *tw = tw_of<R>(axc);  // both axes have n sites: one twiddle table
    // first forward pass along the columns, straight from global memory (twiddles from
    // the global table); the shared tables are filled meanwhile
    dif_pass<C2, N, 0, true>(tile, 1, PL, tw, src);
    {
        const R *f0 = filt_of<R>(axr), *f1 = filt_of<R>(axc);
        for (int i = threadIdx.x; i < N; i += T) {
            twS[i] = tw[i];
            fr[i] = f0[i];
            fc[i] = f1[i];
        }
    }
    __syncthreads();
    const int c = task.slice / ch.nt;
    const R cst = A.with_const ? (R)ch.comp_const[c] : (R)1;
    plane_lines_filter<C2, R, N, 1>(tile, 1, PL, twS, fr, (R)1);  // along the columns (the slower axis)
    plane_lines_filter<C2, R, N, 0>(tile, PL, 1, twS, fc, cst);  // along the rows (contiguous axis)
#pragma unroll
    for (int i = 0; i < EPT; ++i) {
        const int e = threadIdx.x + i * T;
        dst[threadIdx.x + i * T] = tile[(e / N) * PL + e % N];
    }
}

// FP64 planes of 128 need 264 KB of shared memory: the engine never selects them.
template <class R>
static const void *plane_kernel_ptr(int n) {
    if (n == 32) return (const void *)plane_filter_kernel<R, 32>;
    if (n == 64) return (const void *)plane_filter_kernel<R, 64>;
    if (n == 96) return (const void *)plane_filter_kernel<R, 96>;
    if constexpr (sizeof(R) == 4) {
        if (n == 128) return (const void *)plane_filter_kernel<R, 128>;
    }
    return nullptr;
}

template <class R>
cudaError_t setup_plane_filter(int n, size_t smem_bytes, int *ctas_per_sm) {
    const void *fn = plane_kernel_ptr<R>(n);
    if (!fn) return cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes);
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas_per_sm, fn, plane_threads(n), smem_bytes);
}

template <class R>
cudaError_t launch_plane_filter(const LaunchAxis &L, cudaStream_t s) {
    if (L.ntasks == 0) return cudaSuccess;
    const void *fn = plane_kernel_ptr<R>(L.n);
    if (!fn) return cudaErrorInvalidValue;
    void *args[] = {(void *)&L};
    return cudaLaunchKernel(fn, dim3(2 * L.ntasks), dim3(plane_threads(L.n)), args, L.smem_bytes, s);
}

template cudaError_t setup_plane_filter<float>(int, size_t, int *);
template cudaError_t setup_plane_filter<double>(int, size_t, int *);
template cudaError_t launch_plane_filter<float>(const LaunchAxis &, cudaStream_t);
template cudaError_t launch_plane_filter<double>(const LaunchAxis &, cudaStream_t);

}  // namespace clv
