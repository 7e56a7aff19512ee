// k_plane.cu -- kinetic filter of a whole square plane (both of its axes) in one
// pass over HBM, for the tiled path's 2D slices (n x n) and the (y, z) planes of
// 3D slices (n x n at each x), n = 32, 64, 96 or 128.
//
// The spin-1 kinetic factor exp(-eps k^2/2) is a product over the axes, so the
// plane's filter is the line filter along one axis followed by the line filter
// along the other (the same operator as two axis_filter_kernel launches,
// Propagator_without_cutoff.cu:410-424 for the reference's transform sequence).
// One CTA (plane_threads(n, esz) threads) holds one plane of one (component, tau)
// slice of one field in shared memory (n rows at an odd pitch n + 1) and filters
// its lines in place (inplace_fft.cuh: decimation in frequency, the filter at the
// digit-reversed frequencies, decimation in time; one block barrier per pass).
// The first pass (along the slower axis, whose lines are columns) reads its
// butterflies straight from global memory, 32 consecutive columns a warp; the
// plane is written back from shared memory in row order.  FP32 planes of 64 take
// one thread per line instead, the line in registers (plane_lines_in_registers).
// The plane is read once and written once: half the traffic of the two axis
// launches it replaces.
#include "clv_internal.cuh"
#include "clv_launch.h"
#include "fused_impl.cuh"
#include "inplace_fft.cuh"

namespace clv {

// Butterflies whose global loads the first pass issues together: all of a thread's
// where one CTA fills the SM (FP32 planes of 128, FP64 planes of 96), else one (the
// other resident CTAs keep loads in flight).
__host__ __device__ constexpr int plane_first_group(int n, int esz) {
    return (n == 128 && esz == 8) || (n == 96 && esz == 16) ? n * (n / plane_fac(n, 0)) / plane_threads(n, esz) : 1;
}

// Butterflies of a pass unrolled together: all of a thread's (at most 8) for the FP64
// planes of 96 (one CTA per SM), else one at a time, streamed (several resident CTAs;
// on the FP32 planes of 128 the streamed passes measured 4-6 % faster than unrolled).
__host__ __device__ constexpr int plane_unroll(int n, int esz) { return n == 96 && esz == 16 ? 8 : 1; }

// Two-radix line plans of the plane (clv_launch.h plane_fac).
struct PlanePlan {
    static __host__ __device__ constexpr int nfac(int n) { return plane_nfac(n); }
    static __host__ __device__ constexpr int fac(int n, int p) { return plane_fac(n, p); }
};

// Resident CTAs per SM the registers are budgeted for (shared memory allows as many).
__host__ __device__ constexpr int plane_min_ctas(int n, int esz) {
    return esz == 8 ? (n == 32 ? 8 : (n == 64 ? 6 : (n == 96 ? 3 : 1))) : (n == 32 ? 4 : (n == 64 ? 3 : 1));
}

// One thread per line with the whole line in registers (FP32 planes of 64): thread l
// loads column l straight from global memory (a warp: 32 consecutive columns), runs the
// 64-point transform, the filter and the inverse in registers and writes the column into
// the tile; after a barrier it does the same for row l, and the plane goes back in row
// order: 4 shared-memory accesses per element instead of the 12 of the in-place passes.
template <class R, int N>
__device__ __forceinline__ void plane_lines_in_registers(const LaunchAxis &A) {
    using C2 = typename Cx<R>::T;
    constexpr int PL = plane_pitch(N);
    extern __shared__ __align__(128) unsigned char smem[];
    const AxisTask task = A.tasks[blockIdx.x >> 1];
    const int field = (int)(blockIdx.x & 1);
    const ChainDev &ch = A.chains[task.chain];
    const AxisDev &axr = ch.axis[A.axis], &axc = ch.axis[A.axis + 1];
    R *fr = reinterpret_cast<R *>(smem + N * sizeof(C2));
    R *fc = fr + N;
    C2 *tile = reinterpret_cast<C2 *>(smem + plane_tab_bytes(N, sizeof(C2)));
    const long long soff = ch.off + (long long)task.slice * ch.V + (long long)task.l0 * (N * N);
    const C2 *src = reinterpret_cast<const C2 *>(field ? A.src1 : A.src0) + soff;
    C2 *dst = reinterpret_cast<C2 *>(field ? A.dst1 : A.dst0) + soff;
    const int l = threadIdx.x;
    const R cst = A.with_const ? (R)ch.comp_const[task.slice / ch.nt] : (R)1;
    // phase 0 along column l (the slower axis), phase 1 along row l (the contiguous axis):
    // one copy of the transforms' code for both (the unrolled transforms are large)
#pragma unroll 1
    for (int ph = 0; ph < 2; ++ph) {
        C2 v[N];
        if (ph == 0) {
#pragma unroll
            for (int a = 0; a < N; ++a) v[a] = src[a * N + l];
            fr[l] = filt_of<R>(axr)[l];
            fc[l] = filt_of<R>(axc)[l] * cst;
            __syncthreads();
        } else {
#pragma unroll
            for (int a = 0; a < N; ++a) v[a] = tile[l * PL + a];
        }
        Radix<C2, N>::template run<-1>(v);
        const R *f = ph ? fc : fr;
#pragma unroll
        for (int k = 0; k < N; ++k) v[k] = cscale(f[k], v[k]);
        Radix<C2, N>::template run<1>(v);
        const int s0 = ph ? l * PL : l, sa = ph ? 1 : PL;  // element a of the line in the tile
#pragma unroll
        for (int a = 0; a < N; ++a) tile[s0 + a * sa] = v[a];
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < N; ++i) dst[i * N + l] = tile[i * PL + l];
}

// In-place passes over the plane in shared memory (inplace_fft.cuh).
template <class R, int N>
__device__ __forceinline__ void plane_in_place(const LaunchAxis &A) {
    using C2 = typename Cx<R>::T;
    constexpr int T = plane_threads(N, (int)sizeof(C2)), PL = plane_pitch(N), EPT = N * N / T, R0 = plane_fac(N, 0);
    constexpr int PER0 = N * (N / R0) / T, G = plane_first_group(N, (int)sizeof(C2));
    using IP = InPlace<PlanePlan, N, N, T, plane_unroll(N, (int)sizeof(C2))>;
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
#pragma unroll 1
    for (int p0 = 0; p0 < PER0; p0 += G) {
        C2 v[G][R0];
        IP::template first_load<C2, G>(v, src, 1, N, p0);
        IP::template first_finish<C2, G>(v, tile, 1, PL, tw, p0);
    }
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
    IP::template filter<C2, R, 1>(tile, 1, PL, twS, fr, (R)1);  // along the columns (the slower axis)
    IP::template filter<C2, R, 0>(tile, PL, 1, twS, fc, cst);  // along the rows (contiguous axis)
#pragma unroll
    for (int i = 0; i < EPT; ++i) {
        const int e = threadIdx.x + i * T;
        dst[threadIdx.x + i * T] = tile[(e / N) * PL + e % N];
    }
}

// Task: AxisTask {chain, slice = c * nt + tau, l0 = plane index within the slice
// (the x index of a 3D slice, 0 for 2D)}; blockIdx.x % 2 selects the field.
// Axes A.axis (rows, the slower one) and A.axis + 1 (columns, contiguous).
template <class R, int N>
__global__ void __launch_bounds__(plane_threads(N, (int)sizeof(R) * 2), plane_min_ctas(N, (int)sizeof(R) * 2))
plane_filter_kernel(const LaunchAxis A) {
    if constexpr (plane_line_per_thread(N, (int)sizeof(R) * 2)) plane_lines_in_registers<R, N>(A);
    else plane_in_place<R, N>(A);
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
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas_per_sm, fn, plane_threads(n, (int)sizeof(R) * 2), smem_bytes);
}

template <class R>
cudaError_t launch_plane_filter(const LaunchAxis &L, cudaStream_t s) {
    if (L.ntasks == 0) return cudaSuccess;
    const void *fn = plane_kernel_ptr<R>(L.n);
    if (!fn) return cudaErrorInvalidValue;
    void *args[] = {(void *)&L};
    return cudaLaunchKernel(fn, dim3(2 * L.ntasks), dim3(plane_threads(L.n, (int)sizeof(R) * 2)), args, L.smem_bytes, s);
}

template cudaError_t setup_plane_filter<float>(int, size_t, int *);
template cudaError_t setup_plane_filter<double>(int, size_t, int *);
template cudaError_t launch_plane_filter<float>(const LaunchAxis &, cudaStream_t);
template cudaError_t launch_plane_filter<double>(const LaunchAxis &, cudaStream_t);

}  // namespace clv
