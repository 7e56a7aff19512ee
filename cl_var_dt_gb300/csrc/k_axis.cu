// k_axis.cu -- kinetic filter along one axis for slices too large for the
// fused step kernel (2D 128 x 128, 3D 64^3, long 1D lines).
//
// The kinetic factor is separable over the axes (the reference's -px^2 filter
// acts on x only; the spin-1 factor exp(-eps k^2/2) is a product over axes), so
// the filter is one pass per axis: dst = F^-1 [f(k) . F src] along every line
// of the axis (Propagator_without_cutoff.cu:410-424, 160-203 for the
// reference's cuFFT + multiply + normalise sequence).
//
// A CTA takes a tile of up to W adjacent lines of one (component, tau) slice of
// one field (blockIdx.x / 2 the tile, blockIdx.x % 2 the field; one field per launch:
// blockIdx.x the tile).
// * FP32 lines of 64 of a strided axis (stride `inner` > 1): one thread per line with
//   the line in registers (axis_line_kernel: blockIdx.x the tile, one warp per field),
//   no shared memory.
// * Other full tiles of a strided axis with a compile-time plan: filtered in place
//   (inplace_fft.cuh); the first pass reads its butterflies straight from global
//   memory and the last pass writes them back, W consecutive lines a warp, so the
//   tile never round-trips through separate load and store phases.
// * Otherwise lines that are neighbours in memory are loaded with W-wide coalesced
//   rows and transposed into shared memory (for the innermost axis the tile is one
//   contiguous block).  For the common line lengths the whole CTA runs the Stockham
//   passes of all the tile's lines together (compile-time mixed-radix plan; the last
//   forward radix, the filter and the first inverse radix fused in registers; a
//   scratch tile), the last inverse pass writing back into the tile; other lengths
//   use a runtime plan with one warp per line.  The tile is stored with the same
//   coalesced rows.
// Tile lines are kept at an odd pitch, so line-wise reads and transposing stores are
// free of bank conflicts; every element is read once and written once per axis.
#include "clv_internal.cuh"
#include "clv_launch.h"
#include "fused_impl.cuh"
#include "inplace_fft.cuh"

namespace clv {

template <class R>
__device__ __forceinline__ const R *efilt_of(const AxisDev &ax);
template <> __device__ __forceinline__ const double *efilt_of<double>(const AxisDev &ax) { return ax.efilt64; }
template <> __device__ __forceinline__ const float *efilt_of<float>(const AxisDev &ax) { return ax.efilt32; }

// ----------------------------------------------------------- CTA-wide passes
// One Stockham pass of radix R over `nl` lines at once: butterfly b of the CTA
// is butterfly b % nR of line b / nR, so every thread works in every pass even
// when a line has fewer butterflies than a warp has lanes (lines of 64 or 128).
// Line l of the source starts at s + l * SS, of the destination at d + l * SD;
// PS/PD: padded layouts (one spare element per 16).
template <class C2, int N, int R, int NS, int S, bool PS, bool PD>
__device__ __forceinline__ void cta_pass(const C2 *s, C2 *d, int SS, int SD, int nl, const C2 *tw) {
    constexpr int nR = N / R, tstep = N / (NS * R);
    for (int b = threadIdx.x; b < nl * nR; b += blockDim.x) {
        const int l = b / nR, j = b - l * nR;
        const int k = (int)((unsigned)j % (unsigned)NS);
        const C2 *ls = s + l * SS;
        C2 *ld = d + l * SD;
        C2 v[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int idx = j + r * nR;
            C2 x = ls[PS ? padi(idx) : idx];
            if (NS > 1 && r > 0) {
                C2 t = tw[k * r * tstep];
                if (S > 0) t.y = -t.y;
                x = cmul(x, t);
            }
            v[r] = x;
        }
        Radix<C2, R>::template run<S>(v);
        const int o = (j / NS) * NS * R + k;
#pragma unroll
        for (int q = 0; q < R; ++q) {
            const int idx = o + q * NS;
            ld[PD ? padi(idx) : idx] = v[q];
        }
    }
    __syncthreads();
}

// Last forward pass, real filter f[k] * cst, first inverse pass, in registers.
template <class C2, class RR, int N, int R>
__device__ __forceinline__ void cta_mid(const C2 *s, C2 *d, int SS, int SD, int nl, const C2 *tw,
                                        const RR *f, RR cst) {
    constexpr int nR = N / R;
    for (int b = threadIdx.x; b < nl * nR; b += blockDim.x) {
        const int l = b / nR, j = b - l * nR;
        const C2 *ls = s + l * SS;
        C2 *ld = d + l * SD;
        C2 v[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            C2 x = ls[padi(j + r * nR)];
            if (nR > 1 && r > 0) x = cmul(x, tw[j * r]);
            v[r] = x;
        }
        Radix<C2, R>::template run<-1>(v);
#pragma unroll
        for (int q = 0; q < R; ++q) v[q] = cscale(f[j + q * nR] * cst, v[q]);
        Radix<C2, R>::template run<1>(v);
#pragma unroll
        for (int q = 0; q < R; ++q) ld[padi(j * R + q)] = v[q];
    }
    __syncthreads();
}

// The passes alternate between two buffers of nl lines at the same pitch P: pass
// k reads A and writes B when k is even, and the other way round when k is odd.
// The first pass reads the dense tile (A), the middle ones use the padded layout,
// and the last (pass 2 NF - 2, even) writes dense lines into B.
template <class C2, int N, int P, int NS, bool SRC_A>
__device__ __forceinline__ void cta_fwd2(C2 *A, C2 *B, int PP, int nl, const C2 *tw) {
    constexpr int NF = ax_nfac(N);
    if constexpr (P < NF - 1) {
        constexpr int R = ax_fac(N, P);
        cta_pass<C2, N, R, NS, -1, (P > 0), true>(SRC_A ? A : B, SRC_A ? B : A, PP, PP, nl, tw);
        cta_fwd2<C2, N, P + 1, NS * R, !SRC_A>(A, B, PP, nl, tw);
    }
}

template <class C2, int N, int P, int NS, bool SRC_A>
__device__ __forceinline__ void cta_inv2(C2 *A, C2 *B, int PP, int nl, const C2 *tw) {
    if constexpr (P >= 0) {
        constexpr int R = ax_fac(N, P);
        cta_pass<C2, N, R, NS, 1, true, (P > 0)>(SRC_A ? A : B, SRC_A ? B : A, PP, PP, nl, tw);
        cta_inv2<C2, N, P - 1, NS * R, !SRC_A>(A, B, PP, nl, tw);
    }
}

// Filter the nl dense lines of A (at least two radix factors); the result lands in
// B as dense lines; one block barrier per pass.
template <class C2, class RR, int N>
__device__ __forceinline__ void cta_lines_filter(C2 *A, C2 *B, int PP, int nl, const C2 *tw,
                                                 const RR *f, RR cst) {
    constexpr int NF = ax_nfac(N);
    constexpr int RL = ax_fac(N, NF - 1);
    static_assert(NF >= 2, "compile-time plans need two radix factors");
    cta_fwd2<C2, N, 0, 1, true>(A, B, PP, nl, tw);
    // the middle pass has index NF - 1: it reads A when NF - 1 is even
    constexpr bool MID_A = ((NF - 1) % 2) == 0;
    cta_mid<C2, RR, N, RL>(MID_A ? A : B, MID_A ? B : A, PP, PP, nl, tw, f, cst);
    cta_inv2<C2, N, NF - 2, RL, !MID_A>(A, B, PP, nl, tw);
}

struct AxisPlan {
    static __host__ __device__ constexpr int nfac(int n) { return ax_nfac(n); }
    static __host__ __device__ constexpr int fac(int n, int p) { return ax_fac(n, p); }
};

// N > 0: compile-time line length (32, 64, 96, 128, 256, 512): CTA-wide passes
// alternating between the tile and one scratch tile (both at a pitch that holds
// a padded line), the result in the scratch tile.  N = 0: runtime plan, one warp
// per line (per-warp scratch of two padded lines), the result back in the tile.
template <class R, int N>
__global__ void __launch_bounds__(256) axis_filter_kernel(const LaunchAxis A) {
    using C2 = typename Cx<R>::T;
    constexpr int W = axis_tile_lines<R>(N);
    constexpr int PER = N > 0 ? W * N / 256 : 1;  // elements per thread of a full tile
    extern __shared__ __align__(128) unsigned char smem[];
    const AxisTask task = A.tasks[A.nfields == 2 ? blockIdx.x >> 1 : blockIdx.x];
    const int field = A.nfields == 2 ? (int)(blockIdx.x & 1) : 0;
    const ChainDev &ch = A.chains[task.chain];
    const AxisDev &ax = ch.axis[A.axis];
    const int n = N ? N : ax.n;
    const int PL = A.pitch, inner = ax.inner, nl = task.nl, total = nl * n;
    C2 *twS = reinterpret_cast<C2 *>(smem);
    R *fS = reinterpret_cast<R *>(smem + (size_t)n * sizeof(C2));
    C2 *tile = reinterpret_cast<C2 *>(smem + axis_tab_bytes(n, sizeof(C2)));
    C2 *scr = tile + axis_tile_elems(n, PL, W);
    const long long soff = ch.off + (long long)task.slice * ch.V;
    const C2 *src = reinterpret_cast<const C2 *>(field ? A.src1 : A.src0) + soff;
    C2 *dst = reinterpret_cast<C2 *>(field ? A.dst1 : A.dst0) + soff;
    const long long base = inner == 1 ? (long long)task.l0 * n
                                      : (long long)(task.l0 / inner) * n * inner + (task.l0 % inner);
    if constexpr (N > 0) {
        if (inner > 1 && nl == W) {
            // in place: element a of tile line w at tile[w * PL + a], in global memory at
            // base + w + a * inner
            using IP = InPlace<AxisPlan, N, W, 256, 1>;
            const C2 *tw = tw_of<R>(ax);
#pragma unroll 1
            for (int p0 = 0; p0 < IP::PER0; ++p0) {
                C2 v[1][IP::R0];
                IP::template first_load<C2, 1>(v, src + base, 1, inner, p0);
                IP::template first_finish<C2, 1>(v, tile, PL, 1, tw, p0);
            }
            {
                const R *f = A.filter ? efilt_of<R>(ax) : filt_of<R>(ax);
                for (int i = threadIdx.x; i < n; i += blockDim.x) {
                    twS[i] = tw[i];
                    fS[i] = f[i];
                }
            }
            __syncthreads();
            const R cst = A.with_const ? (R)ch.comp_const[task.slice / ch.nt] : (R)1;
            IP::template fwd<C2, 1>(tile, PL, 1, twS);
            IP::template mid<C2, R>(tile, PL, 1, fS, cst);
            __syncthreads();
            IP::template inv<C2, IP::NF - 2, 1>(tile, PL, 1, twS);
            IP::template dit<C2, 0, true>(tile, PL, 1, twS, dst + base, 1, inner, A.accumulate != 0);
            return;
        }
    }
    if (N > 0 && nl == W) {
        // full tile: every load of the thread in flight before the first store
        C2 v[PER];
#pragma unroll
        for (int k = 0; k < PER; ++k) {
            const int e = threadIdx.x + 256 * k;
            v[k] = src[inner == 1 ? base + e : base + (long long)(e / W) * inner + (e % W)];
        }
#pragma unroll
        for (int k = 0; k < PER; ++k) {
            const int e = threadIdx.x + 256 * k;
            tile[inner == 1 ? (e / n) * PL + (e % n) : (e % W) * PL + e / W] = v[k];
        }
    } else if (inner == 1) {
        for (int e = threadIdx.x; e < total; e += blockDim.x) {
            const int w = e / n, a = e - w * n;
            tile[w * PL + a] = src[base + e];
        }
    } else {
        for (int e = threadIdx.x; e < total; e += blockDim.x) {
            const int a = e / nl, w = e - a * nl;
            tile[w * PL + a] = src[base + (long long)a * inner + w];
        }
    }
    {
        const C2 *tw = tw_of<R>(ax);
        const R *f = A.filter ? efilt_of<R>(ax) : filt_of<R>(ax);
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            twS[i] = tw[i];
            fS[i] = f[i];
        }
    }
    __syncthreads();
    const int c = task.slice / ch.nt;
    const R cst = A.with_const ? (R)ch.comp_const[c] : (R)1;
    const int px = padded_line(n);
    const C2 *res = tile;  // dense result lines at pitch PL
    if constexpr (N > 0) {
        cta_lines_filter<C2, R, N>(tile, scr, PL, nl, twS, fS, cst);
        res = scr;
    } else {
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
        C2 *scrX = scr + 2 * px * warp, *scrY = scrX + px;
        for (int w = warp; w < nl; w += nwarps) {
            C2 *line = tile + w * PL;
            warp_line_filter_1d<C2, R>(line, scrX, scrY, ax, twS, fS, cst, lane);
            for (int i = lane; i < n; i += 32) line[i] = scrX[i];
            __syncwarp();
        }
        __syncthreads();
    }
    const bool acc = A.accumulate != 0;
    if (inner == 1) {
        for (int e = threadIdx.x; e < total; e += blockDim.x) {
            const int w = e / n, a = e - w * n;
            const C2 v = res[w * PL + a];
            dst[base + e] = acc ? cadd(dst[base + e], v) : v;
        }
    } else if (nl == W) {
        for (int e = threadIdx.x; e < total; e += blockDim.x) {
            const int a = e / W, w = e - a * W;
            const long long g = base + (long long)a * inner + w;
            const C2 v = res[w * PL + a];
            dst[g] = acc ? cadd(dst[g], v) : v;
        }
    } else {
        for (int e = threadIdx.x; e < total; e += blockDim.x) {
            const int a = e / nl, w = e - a * nl;
            const long long g = base + (long long)a * inner + w;
            const C2 v = res[w * PL + a];
            dst[g] = acc ? cadd(dst[g], v) : v;
        }
    }
}

// FP32 lines of 64 of a strided axis: one thread per line with the whole line in
// registers.  Lane w of warp `field` takes line l0 + w of the task's tile (neighbours in
// memory, so a warp's loads and stores of one index are 32 consecutive elements), runs the
// 64-point transform, the filter and the inverse, and writes the line back: no shared
// memory and no barriers, 64 loads in flight per thread.
static_assert(axis_tile_lines<float>(64) == 32, "one lane per line of a tile");
template <int N>
__global__ void __launch_bounds__(64, 6) axis_line_kernel(const LaunchAxis A) {
    using C2 = float2;
    const AxisTask task = A.tasks[blockIdx.x];
    const int field = (int)(threadIdx.x >> 5), w = (int)(threadIdx.x & 31);
    if (w >= task.nl) return;
    const ChainDev &ch = A.chains[task.chain];
    const AxisDev &ax = ch.axis[A.axis];
    const int inner = ax.inner;
    const long long off = ch.off + (long long)task.slice * ch.V +
                          (long long)(task.l0 / inner) * N * inner + (task.l0 % inner) + w;
    const C2 *src = reinterpret_cast<const C2 *>(field ? A.src1 : A.src0) + off;
    C2 *dst = reinterpret_cast<C2 *>(field ? A.dst1 : A.dst0) + off;
    C2 v[N];
#pragma unroll
    for (int a = 0; a < N; ++a) v[a] = src[(long long)a * inner];
    const float *f = A.filter ? efilt_of<float>(ax) : filt_of<float>(ax);
    const float cst = A.with_const ? (float)ch.comp_const[task.slice / ch.nt] : 1.0f;
    Radix<C2, N>::template run<-1>(v);
#pragma unroll
    for (int k = 0; k < N; ++k) v[k] = cscale(f[k] * cst, v[k]);
    Radix<C2, N>::template run<1>(v);
    const bool acc = A.accumulate != 0;
#pragma unroll
    for (int a = 0; a < N; ++a) {
        C2 *d = dst + (long long)a * inner;
        *d = acc ? cadd(*d, v[a]) : v[a];
    }
}

template <class R>
static const void *axis_kernel_ptr(int n) {
    switch (n) {
        case 32: return (const void *)axis_filter_kernel<R, 32>;
        case 64: return (const void *)axis_filter_kernel<R, 64>;
        case 96: return (const void *)axis_filter_kernel<R, 96>;
        case 128: return (const void *)axis_filter_kernel<R, 128>;
        case 256: return (const void *)axis_filter_kernel<R, 256>;
        case 512: return (const void *)axis_filter_kernel<R, 512>;
        default: return (const void *)axis_filter_kernel<R, 0>;
    }
}

template <class R>
cudaError_t setup_axis_filter(int n, size_t smem_bytes, int *ctas_per_sm) {
    const void *fn = axis_kernel_ptr<R>(n);
    // the runtime-plan kernel serves every other line length: keep the largest request
    cudaFuncAttributes fa;
    cudaError_t e = cudaFuncGetAttributes(&fa, fn);
    if (e != cudaSuccess) return e;
    if ((int)smem_bytes > fa.maxDynamicSharedSizeBytes) {
        e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes);
        if (e != cudaSuccess) return e;
    }
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas_per_sm, fn, 256, smem_bytes);
}

template <class R>
cudaError_t launch_axis_filter(const LaunchAxis &L, cudaStream_t s) {
    if (L.ntasks == 0) return cudaSuccess;
    void *args[] = {(void *)&L};
    if (sizeof(R) == 4 && L.n == 64 && L.strided)
        return cudaLaunchKernel((const void *)axis_line_kernel<64>, dim3(L.ntasks), dim3(32 * L.nfields), args, 0, s);
    const void *fn = axis_kernel_ptr<R>(L.n);
    return cudaLaunchKernel(fn, dim3(L.nfields * L.ntasks), dim3(256), args, L.smem_bytes, s);
}

template cudaError_t setup_axis_filter<float>(int, size_t, int *);
template cudaError_t setup_axis_filter<double>(int, size_t, int *);
template cudaError_t launch_axis_filter<float>(const LaunchAxis &, cudaStream_t);
template cudaError_t launch_axis_filter<double>(const LaunchAxis &, cudaStream_t);

}  // namespace clv
