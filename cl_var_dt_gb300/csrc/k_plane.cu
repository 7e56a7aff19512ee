// k_plane.cu -- kinetic filter of a whole square plane (both of its axes) in one
// pass over HBM, for the tiled path's 2D slices (n x n) and the (y, z) planes of
// 3D slices (n x n at each x), n = 32, 64, 96 or 128.
//
// The spin-1 kinetic factor exp(-eps k^2/2) is a product over the axes, so the
// plane's filter is the line filter along one axis followed by the line filter
// along the other (the same operator as two axis_filter_kernel launches,
// Propagator_without_cutoff.cu:410-424 for the reference's transform sequence).
// One CTA (plane_threads(n) threads) holds one plane of one (component, tau)
// slice of one field in shared memory (n rows at an odd pitch n + 1) and runs
// every Stockham pass in place: each thread loads the inputs of its butterflies
// into registers, the block synchronises, then the thread stores its outputs.  Butterfly b of a pass is
// butterfly j = b / n of line l = b % n, so the 32 lanes of a warp take 32
// consecutive lines at one j: their addresses differ by the line stride (the odd
// pitch along rows, 1 along columns) and are free of bank conflicts, while the
// twiddle and filter reads of the warp are one broadcast.  The plane is read
// once and written once: half the traffic of the two axis launches it replaces.
#include "clv_internal.cuh"
#include "clv_launch.h"
#include "fused_impl.cuh"

namespace clv {

// In-place pass of radix R over the n lines of the plane t (element a of line l at
// t[l * LS + a * ES]): MID = false: Stockham pass with stride NS (direction S);
// MID = true: the last forward pass (NS = N / R), the filter f[k] * cst and the
// first inverse pass, in registers.
template <class C2, class RR, int N, int R, int NS, int S, bool MID>
__device__ __forceinline__ void plane_pass(C2 *t, int LS, int ES, const C2 *tw, const RR *f, RR cst) {
    constexpr int T = plane_threads(N), nR = N / R, PER = N * nR / T;
    static_assert(PER * T == N * nR, "butterflies per thread");
    constexpr int tstep = MID ? 1 : N / (NS * R);
    C2 v[PER][R];
#pragma unroll
    for (int p = 0; p < PER; ++p) {
        const int b = threadIdx.x + p * T;
        const int l = b % N, j = b / N;
        const int k = MID ? j : j % NS;
        const C2 *base = t + l * LS;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            C2 x = base[(j + r * nR) * ES];
            if ((MID || NS > 1) && r > 0) {
                C2 w = tw[k * r * tstep];
                if (!MID && S > 0) w.y = -w.y;
                x = cmul(x, w);
            }
            v[p][r] = x;
        }
    }
    __syncthreads();
#pragma unroll
    for (int p = 0; p < PER; ++p) {
        const int b = threadIdx.x + p * T;
        const int l = b % N, j = b / N;
        C2 *base = t + l * LS;
        if constexpr (MID) {
            Radix<C2, R>::template run<-1>(v[p]);
#pragma unroll
            for (int q = 0; q < R; ++q) v[p][q] = cscale(f[j + q * nR] * cst, v[p][q]);
            Radix<C2, R>::template run<1>(v[p]);
#pragma unroll
            for (int q = 0; q < R; ++q) base[(j * R + q) * ES] = v[p][q];
        } else {
            Radix<C2, R>::template run<S>(v[p]);
            const int k = j % NS, o = (j / NS) * NS * R + k;
#pragma unroll
            for (int q = 0; q < R; ++q) base[(o + q * NS) * ES] = v[p][q];
        }
    }
    __syncthreads();
}

template <class C2, class RR, int N, int P, int NS>
__device__ __forceinline__ void plane_fwd(C2 *t, int LS, int ES, const C2 *tw) {
    constexpr int NF = ax_nfac(N);
    if constexpr (P < NF - 1) {
        constexpr int R = ax_fac(N, P);
        plane_pass<C2, RR, N, R, NS, -1, false>(t, LS, ES, tw, nullptr, (RR)1);
        plane_fwd<C2, RR, N, P + 1, NS * R>(t, LS, ES, tw);
    }
}

template <class C2, class RR, int N, int P, int NS>
__device__ __forceinline__ void plane_inv(C2 *t, int LS, int ES, const C2 *tw) {
    if constexpr (P >= 0) {
        constexpr int R = ax_fac(N, P);
        plane_pass<C2, RR, N, R, NS, 1, false>(t, LS, ES, tw, nullptr, (RR)1);
        plane_inv<C2, RR, N, P - 1, NS * R>(t, LS, ES, tw);
    }
}

// Filter all n lines of the plane along one axis, in place.
template <class C2, class RR, int N>
__device__ __forceinline__ void plane_lines_filter(C2 *t, int LS, int ES, const C2 *tw, const RR *f, RR cst) {
    constexpr int NF = ax_nfac(N), RL = ax_fac(N, NF - 1);
    static_assert(NF >= 2, "two radix factors at least");
    plane_fwd<C2, RR, N, 0, 1>(t, LS, ES, tw);
    plane_pass<C2, RR, N, RL, N / RL, -1, true>(t, LS, ES, tw, f, cst);
    plane_inv<C2, RR, N, NF - 2, RL>(t, LS, ES, tw);
}

// Task: AxisTask {chain, slice = c * nt + tau, l0 = plane index within the slice
// (the x index of a 3D slice, 0 for 2D)}; blockIdx.x % 2 selects the field.
// Axes A.axis (rows, the slower one) and A.axis + 1 (columns, contiguous).
template <class R, int N>
__global__ void __launch_bounds__(plane_threads(N), (sizeof(R) == 4 && N == 64) ? 3 : 1)
plane_filter_kernel(const LaunchAxis A) {
    using C2 = typename Cx<R>::T;
    constexpr int T = plane_threads(N), PL = plane_pitch(N), EPT = N * N / T;
    static_assert(EPT % 8 == 0, "loads in groups of eight");
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
    // eight loads in flight per thread, then their stores into the tile (all of a thread's
    // loads at once measured no faster on 128 x 128 planes: the load queue throttles)
    constexpr int LB = 8;
#pragma unroll
    for (int i0 = 0; i0 < EPT; i0 += LB) {
        C2 v[LB];
#pragma unroll
        for (int i = 0; i < LB; ++i) v[i] = src[threadIdx.x + (i0 + i) * T];
#pragma unroll
        for (int i = 0; i < LB; ++i) {
            const int e = threadIdx.x + (i0 + i) * T;
            tile[(e / N) * PL + e % N] = v[i];
        }
    }
    {
        const C2 *tw = tw_of<R>(axc);
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
    plane_lines_filter<C2, R, N>(tile, PL, 1, twS, fc, cst);  // along the rows (contiguous axis)
    plane_lines_filter<C2, R, N>(tile, 1, PL, twS, fr, (R)1);  // along the columns
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
