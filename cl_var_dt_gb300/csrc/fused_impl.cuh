// fused_impl.cuh -- the whole Langevin step of chains whose spatial slice fits in
// shared memory, in one kernel that streams through imaginary time.
//
// A CTA owns imaginary times [tau0, tau1) of one chain.  Field slices
// (all components of one tau, contiguous in the [c][tau][x][y][z] layout) arrive
// in shared memory by TMA bulk copies (cp.async.bulk + mbarrier), prefetched
// two slices ahead.  For every tau the CTA
//   1. applies the kinetic filter to psi(tau) and psibar(tau+1) in shared
//      memory (Stockham FFT per axis, real filter, inverse FFT);
//   2. computes the drift K(tau), Kbar(tau) of every site from the resident
//      slices psi(tau-1), psi(tau), psi(tau+1), psibar(tau), psibar(tau+1) and the
//      kinetic terms kin(tau-1), kinbar(tau+1);
//   3. adds dt K + sqrt(dt) xi (in-register Philox noise or an injected buffer)
//      and stores psi(tau), psibar(tau) of the new state into the other buffer
//      of the ping-pong pair.
// So each field is read once and written once per step (plus one halo slice per
// CTA), the kinetic term never reaches HBM, and no drift array exists.
//
// The step size depends on max|drift| over the whole chain.  Modes:
//   SPEC    : update with dt = dt_max (the K/max rule's cap) while reducing
//             |K|; the chain's last CTA computes the true dt and marks the step
//             accepted when it equals dt_max.  Otherwise an APPLY pass redoes
//             the chain from the untouched input buffer.  Results are identical
//             to the two-pass order.
//   MAXONLY : reduce only (no stores); the last CTA computes dt.
//   APPLY   : update with the dt of the chain's state (after MAXONLY, or for
//             rejected chains after SPEC).
#pragma once

#include "clv_internal.cuh"
#include "clv_launch.h"
#include "drift_math.cuh"
#include "fft_radix.cuh"

namespace clv {

// ------------------------------------------------------------ TMA / mbarrier
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}"
                 ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void tma_load_1d(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
        ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok) : "r"(smem_u32(bar)), "r"(parity) : "memory");
    return ok != 0;
}
__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// Bounded wait: gives up after 0.5 s or 2^22 polls, whichever comes first (far
// beyond any copy's latency), so a copy that never lands cannot hang the GPU.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = globaltimer_ns();
    for (int i = 0; i < (1 << 22); ++i) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((i & 255) == 255 && globaltimer_ns() - t0 > 500000000ull) return false;
    }
    return false;
}

// ------------------------------------------------------- warp line filter
// One Stockham pass of radix R over one line (length n, element stride `inner`)
// executed by the 32 lanes of a warp.  When f != nullptr (last forward pass) the
// output, in natural frequency order, is multiplied by f[k] * cst.
template <class C2, class RR, int R>
__device__ __forceinline__ void warp_pass(const C2 *s, C2 *d, int inner, int n, int Ns, int S,
                                          const C2 *tw, const RR *f, RR cst, int lane) {
    const int nR = n / R, tstep = n / (Ns * R);
    for (int j = lane; j < nR; j += 32) {
        const int k = j % Ns;
        C2 v[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            C2 x = s[(j + r * nR) * inner];
            if (r > 0 && k > 0) {
                C2 t = tw[k * r * tstep];
                if (S > 0) t.y = -t.y;  // table holds exp(-2 pi i k/n)
                x = cmul(x, t);
            }
            v[r] = x;
        }
        Radix<C2, R>::run(v, S);
        const int o = (j / Ns) * Ns * R + k;
#pragma unroll
        for (int q = 0; q < R; ++q) {
            const int idx = o + q * Ns;
            C2 val = v[q];
            if (f) val = cscale(f[idx] * cst, val);
            d[idx * inner] = val;
        }
    }
}

// Filter one line in place: forward FFT, real filter, inverse FFT along the
// line starting at buf + base.  Passes alternate buf -> tmp -> buf ...; their
// number 2*nf is even, so the result lands back in buf.  Warp-synchronous.
template <class C2, class RR>
__device__ __forceinline__ void warp_line_filter(C2 *buf, C2 *tmp, int base, const AxisDev &ax,
                                                 const C2 *tw, const RR *f, RR cst, int lane) {
    C2 *src = buf + base, *dst = tmp + base;
    for (int dir = 0; dir < 2; ++dir) {
        const int S = dir == 0 ? -1 : +1;
        int Ns = 1;
        for (int p = 0; p < ax.nf; ++p) {
            const int R = ax.fac[p];
            const RR *fp = (dir == 0 && p == ax.nf - 1) ? f : nullptr;
            switch (R) {
                case 8: warp_pass<C2, RR, 8>(src, dst, ax.inner, ax.n, Ns, S, tw, fp, cst, lane); break;
                case 4: warp_pass<C2, RR, 4>(src, dst, ax.inner, ax.n, Ns, S, tw, fp, cst, lane); break;
                case 2: warp_pass<C2, RR, 2>(src, dst, ax.inner, ax.n, Ns, S, tw, fp, cst, lane); break;
                case 3: warp_pass<C2, RR, 3>(src, dst, ax.inner, ax.n, Ns, S, tw, fp, cst, lane); break;
                default: warp_pass<C2, RR, 5>(src, dst, ax.inner, ax.n, Ns, S, tw, fp, cst, lane); break;
            }
            __syncwarp();
            C2 *t = src; src = dst; dst = t;
            Ns *= R;
        }
    }
}

// ------------------------------------------------- contiguous-line fast path
// Lines of a 1D chain are contiguous.  Intermediate layouts are padded with one
// spare element after every 16, which removes the shared-memory bank conflicts
// of the strided Stockham stores.
__device__ __forceinline__ int padi(int i) { return i + (i >> 4); }

template <class C2, int R, bool PS, bool PD>
__device__ __forceinline__ void warp_pass_1d(const C2 *s, C2 *d, int n, int Ns, int S, const C2 *tw,
                                             int lane) {
    const int nR = n / R, tstep = n / (Ns * R);
    for (int j = lane; j < nR; j += 32) {
        const int k = j % Ns;
        C2 v[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int idx = j + r * nR;
            C2 x = s[PS ? padi(idx) : idx];
            if (r > 0 && k > 0) {
                C2 t = tw[k * r * tstep];
                if (S > 0) t.y = -t.y;
                x = cmul(x, t);
            }
            v[r] = x;
        }
        Radix<C2, R>::run(v, S);
        const int o = (j / Ns) * Ns * R + k;
#pragma unroll
        for (int q = 0; q < R; ++q) {
            const int idx = o + q * Ns;
            d[PD ? padi(idx) : idx] = v[q];
        }
    }
}

// Last forward pass (radix R, Ns = n/R), real filter, first inverse pass
// (radix R, Ns = 1) in registers: lane j holds frequencies j + q n/R after the
// forward butterfly, which are exactly the inputs of its inverse butterfly.
template <class C2, class RR, int R, bool PS, bool PD>
__device__ __forceinline__ void warp_mid_1d(const C2 *s, C2 *d, int n, const C2 *tw, const RR *f,
                                            RR cst, int lane) {
    const int nR = n / R;
    for (int j = lane; j < nR; j += 32) {
        C2 v[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int idx = j + r * nR;
            C2 x = s[PS ? padi(idx) : idx];
            if (r > 0 && j > 0) x = cmul(x, tw[j * r]);
            v[r] = x;
        }
        Radix<C2, R>::run(v, -1);
#pragma unroll
        for (int q = 0; q < R; ++q) v[q] = cscale(f[j + q * nR] * cst, v[q]);
        Radix<C2, R>::run(v, +1);
#pragma unroll
        for (int q = 0; q < R; ++q) {
            const int idx = j * R + q;
            d[PD ? padi(idx) : idx] = v[q];
        }
    }
}

template <class C2, bool PS, bool PD>
__device__ __forceinline__ void pass_1d(int R, const C2 *s, C2 *d, int n, int Ns, int S,
                                        const C2 *tw, int lane) {
    switch (R) {
        case 8: warp_pass_1d<C2, 8, PS, PD>(s, d, n, Ns, S, tw, lane); break;
        case 4: warp_pass_1d<C2, 4, PS, PD>(s, d, n, Ns, S, tw, lane); break;
        case 2: warp_pass_1d<C2, 2, PS, PD>(s, d, n, Ns, S, tw, lane); break;
        case 3: warp_pass_1d<C2, 3, PS, PD>(s, d, n, Ns, S, tw, lane); break;
        default: warp_pass_1d<C2, 5, PS, PD>(s, d, n, Ns, S, tw, lane); break;
    }
}
template <class C2, class RR, bool PS, bool PD>
__device__ __forceinline__ void mid_1d(int R, const C2 *s, C2 *d, int n, const C2 *tw, const RR *f,
                                       RR cst, int lane) {
    switch (R) {
        case 8: warp_mid_1d<C2, RR, 8, PS, PD>(s, d, n, tw, f, cst, lane); break;
        case 4: warp_mid_1d<C2, RR, 4, PS, PD>(s, d, n, tw, f, cst, lane); break;
        case 2: warp_mid_1d<C2, RR, 2, PS, PD>(s, d, n, tw, f, cst, lane); break;
        case 3: warp_mid_1d<C2, RR, 3, PS, PD>(s, d, n, tw, f, cst, lane); break;
        default: warp_mid_1d<C2, RR, 5, PS, PD>(s, d, n, tw, f, cst, lane); break;
    }
}

// Filter of one contiguous line: src (dense) -> ... -> out (dense).  The 2 nf - 1
// passes alternate the padded buffers X and Y and end in X == out: out may
// alias X and Y may alias src (src is read only by the first pass).
template <class C2, class RR>
__device__ __forceinline__ void warp_line_filter_1d(const C2 *src, C2 *X, C2 *Y, const AxisDev &ax,
                                                    const C2 *tw, const RR *f, RR cst, int lane) {
    const int n = ax.n, nf = ax.nf;
    if (nf == 1) {
        mid_1d<C2, RR, false, false>(ax.fac[0], src, X, n, tw, f, cst, lane);
        __syncwarp();
        return;
    }
    int Ns = 1;
    const C2 *cur = src;
    C2 *nxt = X, *oth = Y;
    for (int p = 0; p < nf - 1; ++p) {
        if (p == 0) pass_1d<C2, false, true>(ax.fac[p], cur, nxt, n, Ns, -1, tw, lane);
        else pass_1d<C2, true, true>(ax.fac[p], cur, nxt, n, Ns, -1, tw, lane);
        __syncwarp();
        Ns *= ax.fac[p];
        cur = nxt;
        C2 *t = nxt; nxt = oth; oth = t;
    }
    const int Rl = ax.fac[nf - 1];
    mid_1d<C2, RR, true, true>(Rl, cur, nxt, n, tw, f, cst, lane);
    __syncwarp();
    cur = nxt;
    { C2 *t = nxt; nxt = oth; oth = t; }
    Ns = Rl;
    for (int p = nf - 2; p >= 0; --p) {
        if (p == 0) pass_1d<C2, true, false>(ax.fac[p], cur, nxt, n, Ns, +1, tw, lane);
        else pass_1d<C2, true, true>(ax.fac[p], cur, nxt, n, Ns, +1, tw, lane);
        __syncwarp();
        Ns *= ax.fac[p];
        cur = nxt;
        C2 *t = nxt; nxt = oth; oth = t;
    }
}

// ------------------------------------ compile-time plans for power-of-two lines
// Stockham pass with every size known at compile time (NS a power of two).
// Multiplying by the k = 0 twiddle (exactly 1) leaves values unchanged, so the
// twiddle is applied unconditionally.  PT: tw is this pass's own table
// (tw_*_off), else the length-N table exp(-2 pi i m/N).
// Addresses are a per-lane base plus compile-time offsets: padi(a + b) =
// padi(a) + padi(b) whenever (a mod 16) + (b mod 16) < 16, which holds for the
// loads j + r nR (nR a multiple of 16, or j + r nR < 16 per 16-block) and the
// stores o + q NS (o mod 16 + q NS mod 16 < 16 for power-of-two NS and R).
template <class C2, int N, int R, int NS, int S, bool PS, bool PD, bool PT>
__device__ __forceinline__ void ct_pass(const C2 *s, C2 *d, const C2 *tw, int lane) {
    constexpr int nR = N / R, tstep = N / (NS * R);
#pragma unroll 1
    for (int jj = 0; jj < (nR + 31) / 32; ++jj) {
        const int j = lane + 32 * jj;
        if (nR % 32 != 0 && j >= nR) break;
        const int k = j & (NS - 1);
        const C2 *sl = s + (PS ? padi(j) : j);
        const C2 *twl = PT ? tw + k : tw;
        C2 v[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            C2 x = sl[PS ? padi(r * nR) : r * nR];
            if (NS > 1 && r > 0) {
                C2 t;
                if constexpr (PT) {
                    t = twl[(r - 1) * NS];
                } else {
                    t = tw[k * r * tstep];
                    if (S > 0) t.y = -t.y;
                }
                x = cmul(x, t);
            }
            v[r] = x;
        }
        Radix<C2, R>::template run<S>(v);
        const int o = (j / NS) * NS * R + k;
        C2 *dl = d + (PD ? padi(o) : o);
#pragma unroll
        for (int q = 0; q < R; ++q) dl[PD ? padi(q * NS) : q * NS] = v[q];
    }
}

template <class C2, class RR, int N, int R, bool PS, bool PD, bool PT>
__device__ __forceinline__ void ct_mid(const C2 *s, C2 *d, const C2 *tw, const RR *f, RR cst,
                                       int lane) {
    constexpr int nR = N / R;
#pragma unroll 1
    for (int jj = 0; jj < (nR + 31) / 32; ++jj) {
        const int j = lane + 32 * jj;
        if (nR % 32 != 0 && j >= nR) break;
        const C2 *sl = s + (PS ? padi(j) : j);
        C2 v[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            C2 x = sl[PS ? padi(r * nR) : r * nR];
            if (nR > 1 && r > 0) x = cmul(x, PT ? tw[(r - 1) * nR + j] : tw[j * r]);
            v[r] = x;
        }
        Radix<C2, R>::template run<-1>(v);
#pragma unroll
        for (int q = 0; q < R; ++q) v[q] = cscale(f[j + q * nR] * cst, v[q]);
        Radix<C2, R>::template run<1>(v);
        C2 *dl = d + (PD ? padi(j * R) : j * R);
#pragma unroll
        for (int q = 0; q < R; ++q) dl[q] = v[q];
    }
}

template <class C2, int N, int P, int NS, bool PT>
__device__ __forceinline__ void ct_fwd(const C2 *&cur, C2 *&nxt, C2 *&oth, const C2 *tw, int lane) {
    constexpr int NF = p2_nfac(N);
    if constexpr (P < NF - 1) {
        constexpr int R = p2_fac(N, P);
        const C2 *twp = PT ? tw + tw_fwd_off(N, P) : tw;
        if constexpr (P == 0) ct_pass<C2, N, R, NS, -1, false, true, PT>(cur, nxt, twp, lane);
        else ct_pass<C2, N, R, NS, -1, true, true, PT>(cur, nxt, twp, lane);
        __syncwarp();
        cur = nxt;
        C2 *t = nxt; nxt = oth; oth = t;
        ct_fwd<C2, N, P + 1, NS * R, PT>(cur, nxt, oth, tw, lane);
    }
}

template <class C2, int N, int P, int NS, bool PT>
__device__ __forceinline__ void ct_inv(const C2 *&cur, C2 *&nxt, C2 *&oth, const C2 *tw, int lane) {
    if constexpr (P >= 0) {
        constexpr int R = p2_fac(N, P);
        const C2 *twp = PT ? tw + tw_inv_off(N, P) : tw;
        if constexpr (P == 0) ct_pass<C2, N, R, NS, 1, true, false, PT>(cur, nxt, twp, lane);
        else ct_pass<C2, N, R, NS, 1, true, true, PT>(cur, nxt, twp, lane);
        __syncwarp();
        cur = nxt;
        C2 *t = nxt; nxt = oth; oth = t;
        ct_inv<C2, N, P - 1, NS * R, PT>(cur, nxt, oth, tw, lane);
    }
}

// Same contract as warp_line_filter_1d for a compile-time length N = 2^k.  PT:
// tw holds the per-pass tables (tw_*_off), else the length-N table.
template <class C2, class RR, int N, bool PT = false>
__device__ __forceinline__ void warp_line_filter_ct(const C2 *src, C2 *X, C2 *Y, const C2 *tw,
                                                    const RR *f, RR cst, int lane) {
    constexpr int NF = p2_nfac(N);
    constexpr int RL = p2_fac(N, NF - 1);
    const C2 *twm = PT ? tw + tw_mid_off(N) : tw;
    if constexpr (NF == 1) {
        ct_mid<C2, RR, N, RL, false, false, PT>(src, X, twm, f, cst, lane);
        __syncwarp();
    } else {
        const C2 *cur = src;
        C2 *nxt = X, *oth = Y;
        ct_fwd<C2, N, 0, 1, PT>(cur, nxt, oth, tw, lane);
        ct_mid<C2, RR, N, RL, true, true, PT>(cur, nxt, twm, f, cst, lane);
        __syncwarp();
        cur = nxt;
        { C2 *t = nxt; nxt = oth; oth = t; }
        ct_inv<C2, N, NF - 2, RL, PT>(cur, nxt, oth, tw, lane);
    }
}

// 256 = 8 8 4: forward pass 1 (7 x 8), middle (3 x 64), inverse 1 (7 x 4), inverse 0 (7 x 32)
static_assert(tw_mid_off(256) == 56 && tw_inv_off(256, 1) == 248 && tw_inv_off(256, 0) == 276 &&
              tw_entries(256) == 500, "pass tables of 256");
static_assert(tw_entries(128) == 56 + 64 + 14 + 112 && tw_entries(64) == 56 + 56, "pass-table sizes");

// Contiguous-line filter: compile-time plan for the common power-of-two
// lengths, runtime plan otherwise.
template <class C2, class RR>
__device__ __forceinline__ void line_filter_1d(const C2 *src, C2 *X, C2 *Y, const AxisDev &ax,
                                               const C2 *tw, const RR *f, RR cst, int lane) {
    switch (ax.n) {
        case 64: warp_line_filter_ct<C2, RR, 64>(src, X, Y, tw, f, cst, lane); break;
        case 128: warp_line_filter_ct<C2, RR, 128>(src, X, Y, tw, f, cst, lane); break;
        case 256: warp_line_filter_ct<C2, RR, 256>(src, X, Y, tw, f, cst, lane); break;
        case 512: warp_line_filter_ct<C2, RR, 512>(src, X, Y, tw, f, cst, lane); break;
        default: warp_line_filter_1d<C2, RR>(src, X, Y, ax, tw, f, cst, lane); break;
    }
}

// ------------------------------- lines split over a group of NT = 32 G threads
// At FP64 the pipe's throughput per SM sub-partition is the bound, and one warp
// per line keeps only as many sub-partitions busy as there are lines.  A group of
// G warps shares one line of N = 4^k sites: radix-4 Stockham passes (N / 4
// butterflies each, one or more per thread), the group's threads synchronised by
// the named barrier `id` between passes.  Same contract and padded layouts as
// warp_line_filter_ct; twiddles from the length-N table exp(-2 pi i m / N).
template <int NT>
__device__ __forceinline__ void group_sync(int id) {
    if constexpr (NT == 32) __syncwarp();
    else asm volatile("bar.sync %0, %1;" ::"r"(id), "n"(NT) : "memory");
}

template <class C2, int N, int NS, int S, bool PS, bool PD, int NT>
__device__ __forceinline__ void g4_pass(const C2 *s, C2 *d, const C2 *tw, int t) {
    constexpr int nR = N / 4, tstep = N / (NS * 4);
#pragma unroll
    for (int jj = 0; jj < (nR + NT - 1) / NT; ++jj) {
        const int j = t + NT * jj;
        if (nR % NT != 0 && j >= nR) break;
        const int k = j & (NS - 1);
        const C2 *sl = s + (PS ? padi(j) : j);
        C2 v[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            C2 x = sl[PS ? padi(r * nR) : r * nR];
            if (NS > 1 && r > 0) {
                C2 w = tw[k * r * tstep];
                if (S > 0) w.y = -w.y;
                x = cmul(x, w);
            }
            v[r] = x;
        }
        Radix<C2, 4>::template run<S>(v);
        const int o = (j / NS) * NS * 4 + k;
        C2 *dl = d + (PD ? padi(o) : o);
#pragma unroll
        for (int q = 0; q < 4; ++q) dl[PD ? padi(q * NS) : q * NS] = v[q];
    }
}

template <class C2, class RR, int N, bool PS, int NT>
__device__ __forceinline__ void g4_mid(const C2 *s, C2 *d, const C2 *tw, const RR *f, RR cst, int t) {
    constexpr int nR = N / 4;
#pragma unroll
    for (int jj = 0; jj < (nR + NT - 1) / NT; ++jj) {
        const int j = t + NT * jj;
        if (nR % NT != 0 && j >= nR) break;
        const C2 *sl = s + (PS ? padi(j) : j);
        C2 v[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            C2 x = sl[PS ? padi(r * nR) : r * nR];
            if (nR > 1 && r > 0) x = cmul(x, tw[j * r]);
            v[r] = x;
        }
        Radix<C2, 4>::template run<-1>(v);
#pragma unroll
        for (int q = 0; q < 4; ++q) v[q] = cscale(f[j + q * nR] * cst, v[q]);
        Radix<C2, 4>::template run<1>(v);
        C2 *dl = d + padi(j * 4);
#pragma unroll
        for (int q = 0; q < 4; ++q) dl[q] = v[q];
    }
}

template <class C2, int N, int P, int NS, int NT>
__device__ __forceinline__ void g4_fwd(const C2 *&cur, C2 *&nxt, C2 *&oth, const C2 *tw, int t, int id) {
    if constexpr (NS * 4 < N) {  // every forward pass but the last (done by g4_mid)
        g4_pass<C2, N, NS, -1, (P > 0), true, NT>(cur, nxt, tw, t);
        group_sync<NT>(id);
        cur = nxt;
        C2 *x = nxt; nxt = oth; oth = x;
        g4_fwd<C2, N, P + 1, NS * 4, NT>(cur, nxt, oth, tw, t, id);
    }
}

template <class C2, int N, int NS, int NT>
__device__ __forceinline__ void g4_inv(const C2 *&cur, C2 *&nxt, C2 *&oth, const C2 *tw, int t, int id) {
    if constexpr (NS < N) {
        constexpr bool last = NS * 4 == N;  // writes the dense result
        g4_pass<C2, N, NS, 1, true, !last, NT>(cur, nxt, tw, t);
        group_sync<NT>(id);
        cur = nxt;
        C2 *x = nxt; nxt = oth; oth = x;
        g4_inv<C2, N, NS * 4, NT>(cur, nxt, oth, tw, t, id);
    }
}

// N = 4^k, k >= 2: src (dense, read only by the first pass) -> out = X (dense); Y scratch.
template <class C2, class RR, int N, int NT>
__device__ __forceinline__ void group_line_filter4(const C2 *src, C2 *X, C2 *Y, const C2 *tw, const RR *f,
                                                   RR cst, int t, int id) {
    static_assert(N >= 16 && (N & (N - 1)) == 0 && (N & 0x55555555) != 0, "N = 4^k");
    // passes: (k - 1) forward, the middle one, (k - 1) inverse = 2k - 1 in all, alternating
    // X, Y, X, ... from X, so the last (k - 1 odd or even) lands in X when 2k - 1 is odd
    const C2 *cur = src;
    C2 *nxt = X, *oth = Y;
    g4_fwd<C2, N, 0, 1, NT>(cur, nxt, oth, tw, t, id);
    g4_mid<C2, RR, N, true, NT>(cur, nxt, tw, f, cst, t);
    group_sync<NT>(id);
    cur = nxt;
    { C2 *x = nxt; nxt = oth; oth = x; }
    g4_inv<C2, N, 4, NT>(cur, nxt, oth, tw, t, id);
}

template <class R>
__device__ __forceinline__ const typename Cx<R>::T *tw_of(const AxisDev &ax);
template <> __device__ __forceinline__ const double2 *tw_of<double>(const AxisDev &ax) { return ax.tw64; }
template <> __device__ __forceinline__ const float2 *tw_of<float>(const AxisDev &ax) { return ax.tw32; }
template <class R>
__device__ __forceinline__ const typename Cx<R>::T *ptw_of(const AxisDev &ax);
template <> __device__ __forceinline__ const double2 *ptw_of<double>(const AxisDev &ax) { return ax.ptw64; }
template <> __device__ __forceinline__ const float2 *ptw_of<float>(const AxisDev &ax) { return ax.ptw32; }
template <class R>
__device__ __forceinline__ const R *filt_of(const AxisDev &ax);
template <> __device__ __forceinline__ const double *filt_of<double>(const AxisDev &ax) { return ax.filt64; }
template <> __device__ __forceinline__ const float *filt_of<float>(const AxisDev &ax) { return ax.filt32; }

// Kinetic filter of NJ slices (slice j in buf_j, partner tmp_j; components at
// stride cs): every warp takes whole lines, one block barrier per axis.  The
// kinetic term ends in tmp_j for 1D chains (contiguous-line path) and in buf_j
// otherwise.  twS/fS: shared tables.
template <class R, int LN>
__device__ void slices_filter(const ChainDev &ch, int ncomp, int cs, int kinetic, int NJ,
                              typename Cx<R>::T *buf0, typename Cx<R>::T *tmp0,
                              typename Cx<R>::T *buf1, typename Cx<R>::T *tmp1,
                              const typename Cx<R>::T *twS, const R *fS) {
    using C2 = typename Cx<R>::T;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
    const int V = ch.V;
    if (LN || (ch.ny == 1 && ch.nz == 1)) {
        const AxisDev &ax = ch.axis[0];
        const bool wc = kinetic == CLV_KIN_EXP;
        for (int t = warp; t < NJ * ncomp; t += nwarps) {
            const int job = t >= ncomp;
            const int c = t - job * ncomp;
            C2 *b = (job ? buf1 : buf0) + c * cs, *x = (job ? tmp1 : tmp0) + c * cs;
            const R cst = wc ? (R)ch.comp_const[c] : (R)1;
            if constexpr (LN > 0) warp_line_filter_ct<C2, R, LN>(b, x, b, twS, fS, cst, lane);
            else line_filter_1d<C2, R>(b, x, b, ax, twS, fS, cst, lane);
        }
        __syncthreads();
        return;
    }
    int toff = 0;
    bool first_axis = true;
    for (int a = 0; a < 3; ++a) {
        const AxisDev &ax = ch.axis[a];
        if (ax.n <= 1) continue;
        if (kinetic == CLV_KIN_REF_LINEAR_PX && a > 0) break;
        const int lpc = V / ax.n;
        const int per_job = ncomp * lpc;
        const bool wc = first_axis && kinetic == CLV_KIN_EXP;
        for (int t = warp; t < NJ * per_job; t += nwarps) {
            const int job = t >= per_job;
            const int L = t - job * per_job;
            const int c = L / lpc, l = L - c * lpc;
            const int base = c * cs + (l / ax.inner) * ax.n * ax.inner + (l % ax.inner);
            const R cst = wc ? (R)ch.comp_const[c] : (R)1;
            warp_line_filter<C2, R>(job ? buf1 : buf0, job ? tmp1 : tmp0, base, ax,
                                    twS + toff, fS + toff, cst, lane);
        }
        __syncthreads();
        toff += ax.n;
        first_axis = false;
    }
}

// -------------------------------------------------------------- the kernel
// SPT: lattice sites per thread (V <= 256 * SPT).  LN > 0: every chain of the
// launch is a 1D line of LN sites (compile-time sizes and plan), LN = 0: any
// slice shape.  FAST (LN > 0 only): the production variant -- K/max step rule,
// in-register Philox noise, bulk copies, no stored drift, both fields per CTA --
// with those choices fixed at compile time, so the per-tau frame carries no
// branches on them.
// Per-site state carried in registers across imaginary times: psi(tau-1),
// kin(tau-1), psibar(tau).

template <class R, int MODEL, int SPT, int LN, bool FAST = false>
// FP64 1D lines off the production variant (the reference's step rule on few CTAs):
// registers capped at two CTAs' worth, so that the programmatic update's CTAs (its
// noise drawn while this pass runs) fit beside this kernel's on every SM.
__global__ void __launch_bounds__(256, (sizeof(R) == 4 && SPT == 1) ? 3 : ((LN > 0 && !FAST) ? 2 : 1))
fused_step_kernel(const LaunchFused A) {
    using C2 = typename Cx<R>::T;
    constexpr int NC = MODEL == CLV_MODEL_REF4 ? 4 : 3;
    constexpr int NPS = MODEL == CLV_MODEL_REF4 ? 3 : 2;  // psi slots (REF4 also reads psi(tau+1))
    constexpr int NQS = 2;                                // psibar slots
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ int abort_cta;
    // a kernel launched after this one with a programmatic launch (the stored-drift
    // update) may start now; it waits for this grid's end before it reads its results
    asm volatile("griddepcontrol.launch_dependents;");
    const FusedTask task = A.tasks[blockIdx.x];
    const ChainDev &ch = A.chains[task.chain];
    // fields this CTA steps (the production variant always takes both)
    const int side = FAST ? 0 : task.side;
    const bool do_psi = side != 2, do_bar = side != 1;
    // components of this CTA (all unless the chunk is split by component halves)
    const int cmask = (FAST || task.cmask == 0) ? 0xF : task.cmask;
    auto own = [&](int c) { return ((cmask >> c) & 1) != 0; };
    ChainState *st = A.state + task.chain;
    if (A.mode == FUSED_APPLY && A.only_rejected && st->accepted) return;  // uniform per CTA

    const int V = LN ? LN : ch.V, T = ch.nt, cs = LN ? padded_line(LN) : A.comp_stride;
    const int TV = T * V;  // elements of one component of the chain
    const bool kin_in_partner = LN || (ch.ny == 1 && ch.nz == 1);  // contiguous-line FFT path
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem);  // NPS + NQS barriers
    C2 *twS = reinterpret_cast<C2 *>(smem + 64);
    R *fS = reinterpret_cast<R *>(smem + 64 + A.tab_n * sizeof(C2));
    C2 *twT = reinterpret_cast<C2 *>(smem + fused_ptw_offset(A.tab_n, (int)sizeof(C2)));  // LN > 0
    // slot geometry: compile-time for 1D lines of LN sites (the host's formulas, tables of
    // the one filtered axis), so slot addresses are constant offsets
    const int tab_bytes = LN ? fused_tab_bytes(LN, (int)sizeof(C2), LN) : A.tab_bytes;
    const int slot_stride = LN ? fused_slot_stride(NC, LN, (int)sizeof(C2)) : A.slot_stride;
    C2 *slots = reinterpret_cast<C2 *>(smem + tab_bytes);
    auto slot = [&](int i) { return slots + (size_t)i * slot_stride; };
    // slots 0..NPS-1: psi ring; NPS..NPS+NQS-1: psibar ring; then the kinetic
    // results of the two fields, two FFT scratch buffers and the noise of one tau
    C2 *part0 = slot(NPS + NQS), *part1 = slot(NPS + NQS + 1);
    C2 *ybuf0 = slot(NPS + NQS + 2), *ybuf1 = slot(NPS + NQS + 3), *nzbuf = slot(NPS + NQS + 4);
    const C2 *gpsi = reinterpret_cast<const C2 *>(A.psi_in) + ch.off;
    const C2 *gpsic = reinterpret_cast<const C2 *>(A.psic_in) + ch.off;
    C2 *opsi = reinterpret_cast<C2 *>(A.psi_out) + ch.off;
    C2 *opsic = reinterpret_cast<C2 *>(A.psic_out) + ch.off;
    static_assert(!FAST || LN > 0, "the production variant needs compile-time lines");
    const bool tma = FAST || A.use_tma != 0;
    const bool writes = FAST || A.mode != FUSED_MAXONLY;

    R dt = 0;
    uint64_t nstep = 0;
    if (A.mode == FUSED_SPEC) { dt = (R)ch.dt_max; nstep = st->step; }
    else if (A.mode == FUSED_APPLY) { dt = (R)st->dt; nstep = st->noise_step; }
    const R sd = (R)sqrt((double)dt);

    if (threadIdx.x == 0) {
        abort_cta = 0;
        for (int i = 0; i < NPS + NQS; ++i) mbar_init(&bars[i], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // shared copies of the twiddle and filter tables of the chain's filtered axes
    {
        int toff = 0;
        for (int a = 0; a < 3; ++a) {
            const AxisDev &ax = ch.axis[a];
            if (ax.n <= 1) continue;
            if (A.kinetic == CLV_KIN_REF_LINEAR_PX && a > 0) break;
            const C2 *tw = tw_of<R>(ax);
            const R *f = filt_of<R>(ax);
            for (int i = threadIdx.x; i < ax.n; i += blockDim.x) {
                twS[toff + i] = tw[i];
                fS[toff + i] = f[i];
            }
            toff += ax.n;
        }
        if constexpr (LN > 0) {
            const C2 *pt = ptw_of<R>(ch.axis[0]);
            for (int i = threadIdx.x; i < tw_entries(LN); i += blockDim.x) twT[i] = pt[i];
        }
    }
    __syncthreads();

    uint32_t phase = 0, pending = 0;
    auto issue = [&](int sl, const C2 *g, int tau) {
        // periodic wrap: the CTA reads imaginary times tau0 - 1 .. tau1 + 1 of [0, T)
        const int t = tau < 0 ? tau + T : (tau >= T ? tau - T : tau);
        if (tma) {
            if (threadIdx.x == 0) {
                mbar_expect_tx(&bars[sl], (uint32_t)(NC * V * sizeof(C2)));
                for (int c = 0; c < NC; ++c)
                    tma_load_1d(slot(sl) + c * cs, g + ((long long)c * T + t) * V,
                                (uint32_t)(V * sizeof(C2)), &bars[sl]);
            }
            pending |= 1u << sl;
        } else {
            C2 *d = slot(sl);
            for (int e = threadIdx.x; e < NC * V; e += blockDim.x) {
                const int c = e / V, s = e - c * V;
                d[c * cs + s] = g[((long long)c * T + t) * V + s];
            }
        }
    };
    // Only warp 0 polls a copy's barrier; the block barrier that follows every wait
    // orders the landed slice before the other warps' reads (the copy's completion
    // happens before warp 0 passes the wait, which happens before the block barrier).
    auto wait_slot = [&](int sl) {
        if (!(pending & (1u << sl))) return;
        if (threadIdx.x < 32 && !mbar_wait(&bars[sl], (phase >> sl) & 1u)) {
            mbar_wait(&bars[sl], (phase >> sl) & 1u);  // second bounded chance for the copy
            if (threadIdx.x == 0) {
                atomicOr(&st->flags, CLV_FLAG_TIMEOUT);
                abort_cta = 1;
            }
        }
        phase ^= 1u << sl;
        pending &= ~(1u << sl);
    };

    const int tau0 = task.tau0, tau1 = task.tau1;
    const int last_psi = MODEL == CLV_MODEL_REF4 ? tau1 : tau1 - 1;  // last psi time read
    C2 Pp[SPT][NC], Kp[SPT][NC], Qc[SPT][NC];  // psi(tau-1), kin(tau-1), psibar(tau)
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = FAST ? 8 : blockDim.x >> 5;
    // 1D chains: one warp per line (2 NC lines); the remaining warps draw the
    // Philox noise of the imaginary time into shared memory meanwhile: at FP32 every
    // component (2 % faster than leaving the third component's block to each site's
    // thread in the drift phase); at FP64, whose Box-Muller transforms are costly, the
    // first pair only (8 % faster than all three).
    constexpr int SMEM_PAIRS = (NC == 3 && sizeof(R) == 8) ? 1 : (NC + 1) / 2;
    const bool noise_smem =
        kin_in_partner && writes && (FAST || A.noise == CLV_NOISE_PHILOX) && 2 * NC < nwarps;
    const AxisDev &ax0 = ch.axis[0];
    const bool wc = A.kinetic == CLV_KIN_EXP;
    // kinetic filter of component c of a 1D slice: src (read only) -> X, scratch Y
    auto line1d = [&](const C2 *src, C2 *X, C2 *Y, int c) {
        const R cst = wc ? (R)ch.comp_const[c] : (R)1;
        if constexpr (LN > 0) warp_line_filter_ct<C2, R, LN, true>(src + c * cs, X + c * cs, Y + c * cs, twT, fS, cst, lane);
        else line_filter_1d<C2, R>(src + c * cs, X + c * cs, Y + c * cs, ax0, twS, fS, cst, lane);
    };
    // FP64 lines of 256 sites when a CTA filters at most four lines per imaginary time
    // (the chunks split by field and component halves of the few-CTA problems, e.g. the
    // reference's own 256 x 32 lattice): two warps per line, so all four SM
    // sub-partitions' FP64 pipes share the filter instead of one per line.
    constexpr bool kPairLines = sizeof(R) == 8 && LN == 256 && !FAST;
    // Filter the lines of `mask` (bit job * NC + c: job 0 = psi of src0 -> X0, job 1 =
    // psibar of src1 -> X1): warp pairs when they fit, else one warp per line.
    auto filter_lines = [&](int mask, const C2 *src0, C2 *X0, C2 *Y0, const C2 *src1, C2 *X1, C2 *Y1) {
        const int nl = __popc(mask);
        if (kPairLines && 2 * nl <= nwarps) {
            const int g = warp >> 1;
            if (g < nl) {
                int m = mask;
                for (int i = 0; i < g; ++i) m &= m - 1;
                const int bit = __ffs(m) - 1, job = bit >= NC, c = bit - job * NC;
                const R cst = wc ? (R)ch.comp_const[c] : (R)1;
                if constexpr (kPairLines)
                    group_line_filter4<C2, R, LN, 64>((job ? src1 : src0) + c * cs, (job ? X1 : X0) + c * cs,
                                                      (job ? Y1 : Y0) + c * cs, twS, fS, cst,
                                                      threadIdx.x & 63, 1 + g);
            }
            return;
        }
        if (warp < 2 * NC) {
            const int job = warp >= NC, c = warp - job * NC;
            if ((mask >> warp) & 1) line1d(job ? src1 : src0, job ? X1 : X0, job ? Y1 : Y0, c);
        }
    };

    // prologue: psi(tau0-1) and its kinetic term, psibar(tau0)
    if (A.withhold && tma && blockIdx.x == 0)
        pending |= 1u;  // test hook: the copy is never issued, so its bounded wait runs out
    else
        issue(0, gpsi, tau0 - 1);
    issue(NPS, gpsic, tau0);
    wait_slot(0);
    wait_slot(NPS);
    __syncthreads();
#pragma unroll
    for (int k = 0; k < SPT; ++k) {
        const int s = threadIdx.x + k * 256;
        if (s < V)
#pragma unroll
            for (int c = 0; c < NC; ++c) {
                Pp[k][c] = slot(0)[c * cs + s];
                Qc[k][c] = slot(NPS)[c * cs + s];
            }
    }
    if (kin_in_partner) {
        filter_lines(do_psi ? cmask & ((1 << NC) - 1) : 0, slot(0), part0, ybuf0, nullptr, nullptr, nullptr);
        __syncthreads();
    } else {
        __syncthreads();
        if (do_psi) slices_filter<R, LN>(ch, NC, cs, A.kinetic, 1, slot(0), part0, nullptr, nullptr, twS, fS);
    }
    {
        const C2 *kin0 = kin_in_partner ? part0 : slot(0);
#pragma unroll
        for (int k = 0; k < SPT; ++k) {
            const int s = threadIdx.x + k * 256;
            if (s < V)
#pragma unroll
                for (int c = 0; c < NC; ++c) Kp[k][c] = kin0[c * cs + s];
        }
    }
    __syncthreads();
    if (!abort_cta) {  // a CTA whose prologue copy timed out issues nothing more and leaves
        for (int i = 0; i < NPS; ++i)
            if (tau0 + i <= last_psi) issue(i, gpsi, tau0 + i);
        for (int i = 0; i < NQS; ++i)
            if (tau0 + 1 + i <= tau1) issue(NPS + i, gpsic, tau0 + 1 + i);
    }

    // step-rule reduction in the working precision per thread (the max is exact;
    // the REF mean sums at most SPT * (tau1 - tau0) values), FP64 across the CTA
    R mxr = 0, smr = 0;
    int bad = 0;
    const DriftConsts<R> dk(ch);
    const uint64_t seed = ch.seed;
    const int ref_rule = !FAST && A.dt_rule == CLV_DT_REF_MEANMAX;
    int ia = 0, ic = 0;  // ring positions of psi(tau) and psibar(tau+1)
    for (int tau = tau0; tau < tau1; ++tau) {
        const int sp = ia, spp = (ia + 1) % NPS, sq = NPS + ic;
        wait_slot(sp);
        if (MODEL == CLV_MODEL_REF4) wait_slot(spp);
        wait_slot(sq);
        // every thread is past the previous imaginary time's drift: its slots and
        // the kinetic buffers may be reused from here on
        __syncthreads();
        if (abort_cta) break;
        if (tau > tau0) {
            const int fp = (ia + NPS - 1) % NPS, fq = NPS + (ic + NQS - 1) % NQS;
            if (tau - 1 + NPS <= last_psi) issue(fp, gpsi, tau - 1 + NPS);
            if (tau + NQS <= tau1) issue(fq, gpsic, tau + NQS);
        }
        C2 vpc[SPT][NC], vcp[SPT][NC], vpp[SPT][NC];
        auto read_fields = [&]() {
#pragma unroll
            for (int k = 0; k < SPT; ++k) {
                const int s = threadIdx.x + k * 256;
                if (s < V)
#pragma unroll
                    for (int c = 0; c < NC; ++c) {
                        vpc[k][c] = slot(sp)[c * cs + s];
                        vcp[k][c] = slot(sq)[c * cs + s];
                        if (MODEL == CLV_MODEL_REF4) vpp[k][c] = slot(spp)[c * cs + s];
                    }
            }
        };
        if (kin_in_partner) {
            // kin(tau) -> part0, kinbar(tau+1) -> part1; the field slots stay intact
            // (kin(tau) only feeds the next imaginary time: the chunk's last skips it)
            if (warp < 2 * NC || (kPairLines && !noise_smem)) {
                const int own_lines = cmask & ((1 << NC) - 1);
                filter_lines(((do_psi && tau + 1 < tau1) ? own_lines : 0) | (do_bar ? own_lines << NC : 0),
                             slot(sp), part0, ybuf0, slot(sq), part1, ybuf1);
            } else if (noise_smem && LN > 0 && (NC & 1) && NC - 1 < 2 * SMEM_PAIRS) {
                // even lines with a lone component: site pairs (2j, 2j + 1) of the slice, the
                // pair blocks of both sites and their shared lone block drawn together (three
                // independent Philox chains per iteration, a compile-time trip count)
                const int nthr = (nwarps - 2 * NC) * 32, t = (warp - 2 * NC) * 32 + lane;
                constexpr int c = NC - 1;
#pragma unroll 1
                for (int j = t; j < LN / 2; j += nthr) {
                    const int s0 = 2 * j;
                    const uint32_t site = (uint32_t)(tau * LN + s0);
                    uint4 o0[(NC - 1) / 2], o1[(NC - 1) / 2];
#pragma unroll
                    for (int p = 0; p < (NC - 1) / 2; ++p) {
                        o0[p] = philox_block(seed, (uint32_t)task.chain, nstep, p, site);
                        o1[p] = philox_block(seed, (uint32_t)task.chain, nstep, p, site + 1);
                    }
                    const uint4 ol = philox_block(seed, (uint32_t)task.chain, nstep, c >> 1, site >> 1);
#pragma unroll
                    for (int p = 0; p < (NC - 1) / 2; ++p) {
                        nzbuf[2 * p * cs + s0] = unit_normal<R, C2>(o0[p].x, o0[p].y);
                        nzbuf[(2 * p + 1) * cs + s0] = unit_normal<R, C2>(o0[p].z, o0[p].w);
                        nzbuf[2 * p * cs + s0 + 1] = unit_normal<R, C2>(o1[p].x, o1[p].y);
                        nzbuf[(2 * p + 1) * cs + s0 + 1] = unit_normal<R, C2>(o1[p].z, o1[p].w);
                    }
                    nzbuf[c * cs + s0] = unit_normal<R, C2>(ol.x, ol.y);
                    nzbuf[c * cs + s0 + 1] = unit_normal<R, C2>(ol.z, ol.w);
                }
            } else if (noise_smem) {
                const int nthr = (nwarps - 2 * NC) * 32, t = (warp - 2 * NC) * 32 + lane;
                // component pairs: one Philox block per site
                for (int s = t; s < V; s += nthr) {
                    const uint32_t site = (uint32_t)(tau * V + s);
#pragma unroll
                    for (int c = 0; c + 1 < NC && c < 2 * SMEM_PAIRS; c += 2) {
                        const uint4 o = philox_block(seed, (uint32_t)task.chain, nstep, c >> 1, site);
                        nzbuf[c * cs + s] = unit_normal<R, C2>(o.x, o.y);
                        nzbuf[(c + 1) * cs + s] = unit_normal<R, C2>(o.z, o.w);
                    }
                }
                // the lone component of an odd count: one block per two consecutive sites
                // (noise_words); a block straddling the slice's ends serves one site here
                if constexpr ((NC & 1) && NC - 1 < 2 * SMEM_PAIRS) {
                    constexpr int c = NC - 1;
                    const int first = tau * V, last = first + V - 1;
                    for (int j = (first >> 1) + t; j <= (last >> 1); j += nthr) {
                        const uint4 o = philox_block(seed, (uint32_t)task.chain, nstep, c >> 1, (uint32_t)j);
                        const int s0 = 2 * j - first;
                        if (s0 >= 0) nzbuf[c * cs + s0] = unit_normal<R, C2>(o.x, o.y);
                        if (s0 + 1 < V) nzbuf[c * cs + s0 + 1] = unit_normal<R, C2>(o.z, o.w);
                    }
                }
            }
            __syncthreads();
            read_fields();
        } else {
            read_fields();
            __syncthreads();
            // in place: kin(tau) into the psi(tau) slot, kinbar(tau+1) into the psibar(tau+1) slot
            // (the chunk's last imaginary time needs kinbar(tau+1) only)
            const bool kin_psi = do_psi && tau + 1 < tau1;
            if (kin_psi && do_bar)
                slices_filter<R, LN>(ch, NC, cs, A.kinetic, 2, slot(sp), part0, slot(sq), part1, twS, fS);
            else if (do_bar)
                slices_filter<R, LN>(ch, NC, cs, A.kinetic, 1, slot(sq), part1, nullptr, nullptr, twS, fS);
            else if (kin_psi)
                slices_filter<R, LN>(ch, NC, cs, A.kinetic, 1, slot(sp), part0, nullptr, nullptr, twS, fS);
        }
        const C2 *kinb = kin_in_partner ? part0 : slot(sp);   // kin(tau)
        const C2 *kinq = kin_in_partner ? part1 : slot(sq);   // kinbar(tau+1)
#pragma unroll
        for (int k = 0; k < SPT; ++k) {
            const int s = threadIdx.x + k * 256;
            if (s >= V) continue;
            C2 kp[NC], K[NC], Kc[NC];
            if (!FAST && side) {
#pragma unroll
                for (int c = 0; c < NC; ++c) K[c] = Kc[c] = mk<C2>(0.0, 0.0);
            }
#pragma unroll
            for (int c = 0; c < NC; ++c) kp[c] = kinq[c * cs + s];
            if (MODEL == CLV_MODEL_REF4)
                drift_ref4_vals<R>(dk, Pp[k], vpc[k], vpp[k], Qc[k], vcp[k], Kp[k], kp, K, Kc,
                                   FAST ? 3 : (do_psi ? 1 : 0) | (do_bar ? 2 : 0), cmask);
            else
                // (recomputing the bilinears of (psibar(tau), psi(tau-1)) measured faster
                // here than carrying them: the registers cost occupancy)
                drift_spin1_vals<R>(dk, Pp[k], vpc[k], Qc[k], vcp[k], Kp[k], kp, K, Kc,
                                    FAST ? 3 : (do_psi ? 1 : 0) | (do_bar ? 2 : 0));
            if (!FAST && A.mode == FUSED_MAXONLY && A.drift_out) {
                // the apply step reads the drift instead of recomputing filter and drift
#pragma unroll
                for (int c = 0; c < NC; ++c) {
                    if (!own(c)) continue;
                    const long long gi = ((long long)c * T + tau) * V + s;
                    if (do_psi) reinterpret_cast<C2 *>(A.drift_out)[ch.off + gi] = K[c];
                    if (do_bar) reinterpret_cast<C2 *>(A.driftc_out)[ch.off + gi] = Kc[c];
                }
            }
            if (A.mode != FUSED_APPLY) {
                if (ref_rule) {
                    if (own(0)) {  // (a psibar CTA's K is zero)
                        const R a0 = hypot(K[0].x, K[0].y);
                        mxr = fmax(mxr, a0);
                        smr += a0;
                        bad |= !isfinite(a0);
                    }
                } else {
#pragma unroll
                    for (int c = 0; c < NC; ++c) {
                        if (!own(c)) continue;
                        const R m1 = abs2<R>(K[c]);
                        const R m2 = abs2<R>(Kc[c]);
                        if constexpr (sizeof(R) == 4) {
                            mxr = max_nan(mxr, max_nan(m1, m2));  // a NaN reaches the finish
                        } else {
                            mxr = fmax(mxr, fmax(m1, m2));
                            smr += m1 + m2;  // unused by the rule; carries a NaN to the finish
                        }
                    }
                }
            }
            if (writes) {
                const uint32_t site = (uint32_t)(tau * V + s);
#pragma unroll
                for (int c = 0; c < NC; c += 2) {
                    C2 z[2];
                    if (noise_smem && (c >> 1) < SMEM_PAIRS) {
                        z[0] = nzbuf[c * cs + s];
                        if (c + 1 < NC) z[1] = nzbuf[(c + 1) * cs + s];
                    } else if (FAST || A.noise == CLV_NOISE_PHILOX) {
                        if (c + 1 < NC) {
                            const uint4 o = philox_block(seed, (uint32_t)task.chain, nstep, c >> 1, site);
                            z[0] = unit_normal<R, C2>(o.x, o.y);
                            z[1] = unit_normal<R, C2>(o.z, o.w);
                        } else {
                            const uint2 w = noise_words(seed, (uint32_t)task.chain, nstep, c, NC, site);
                            z[0] = unit_normal<R, C2>(w.x, w.y);
                        }
                    } else {
#pragma unroll
                        for (int u = 0; u < 2; ++u) {
                            if (c + u >= NC) break;
                            const long long r = ch.noise_off + (((long long)(c + u) * V + s) * T + tau) * 2;
                            z[u].x = (R)A.noise_buf[r];
                            z[u].y = (R)A.noise_buf[r + 1];
                        }
                    }
#pragma unroll
                    for (int u = 0; u < 2; ++u) {
                        const int cc = c + u;
                        if (cc >= NC) break;
                        C2 zz;
                        zz.x = mul_rn<R>(sd, z[u].x);
                        zz.y = mul_rn<R>(sd, z[u].y);
                        const int gi = cc * TV + tau * V + s;  // < 2^31 (plan_fused)
                        if (!own(cc)) continue;
                        if (do_psi) opsi[gi] = langevin_update<R>(vpc[k][cc], K[cc], dt, zz, false);
                        if (do_bar) opsic[gi] = langevin_update<R>(Qc[k][cc], Kc[cc], dt, zz, true);
                    }
                }
            }
#pragma unroll
            for (int c = 0; c < NC; ++c) {
                Pp[k][c] = vpc[k][c];
                Kp[k][c] = kinb[c * cs + s];
                Qc[k][c] = vcp[k][c];
            }
        }
        ia = (ia + 1) % NPS;
        ic = (ic + 1) % NQS;
    }
    // no copy may be in flight when the CTA exits (warp 0 keeps the CTA resident)
    for (int sl = 0; sl < NPS + NQS; ++sl)
        if (pending & (1u << sl)) {
            if (threadIdx.x < 32) mbar_wait(&bars[sl], (phase >> sl) & 1u);
            phase ^= 1u << sl;
        }
    bad |= abort_cta;
    if (A.mode == FUSED_APPLY) return;

    // chain-wide reduction: partial per CTA, the last CTA of the chain finishes the step
    double mx = (double)mxr, sm = (double)smr;
    bad |= !isfinite(mx) || !isfinite(sm);
    bad = __syncthreads_or(bad);
    block_max_sum(mx, sm);
    __shared__ int am_last;
    if (threadIdx.x == 0) {
        A.partials[ch.fused_block0 + task.part] =
            make_double2(mx, bad ? __longlong_as_double(0x7ff8000000000000ll) : sm);
        __threadfence();
        const unsigned prev = atomicAdd(&st->arrive, 1u);
        am_last = prev == (unsigned)ch.fused_nblocks - 1;
    }
    __syncthreads();
    if (!am_last) return;
    __threadfence();
    mx = 0.0;
    sm = 0.0;
    bad = 0;
    for (int i = threadIdx.x; i < ch.fused_nblocks; i += blockDim.x) {
        const double2 p = __ldcg(&A.partials[ch.fused_block0 + i]);
        mx = fmax(mx, p.x);
        sm += p.y;
        bad |= !isfinite(p.y) || !isfinite(p.x);
    }
    bad = __syncthreads_or(bad);
    block_max_sum(mx, sm);
    if (threadIdx.x == 0) {
        double mean;
        const double dtn = step_rule(ch, *st, A.dt_rule, mx, sm, mean);
        if (bad || !isfinite(mx) || !isfinite(sm)) st->flags |= CLV_FLAG_NONFINITE;
        st->dt = dtn;
        st->max = mx;
        st->mean = mean;
        st->t += dtn;
        st->noise_step = st->step;
        st->step += 1;
        st->accepted = (A.mode == FUSED_SPEC && dtn == ch.dt_max) ? 1 : 0;
        if (!st->accepted) st->rejected += (A.mode == FUSED_SPEC);
        st->arrive = 0;
    }
}

// Kernel pointer of one instantiation (defined in k_fused_<precision>_<model>.cu).
void *fused_kernel_f32_ref4(int spt, int ln, bool fast);
void *fused_kernel_f32_spin1(int spt, int ln, bool fast);
void *fused_kernel_f64_ref4(int spt, int ln, bool fast);
void *fused_kernel_f64_spin1(int spt, int ln, bool fast);

template <class R, int MODEL>
void *fused_fn(int spt, int ln, bool fast) {
    switch (ln) {
        case 64: return fast ? (void *)fused_step_kernel<R, MODEL, 1, 64, true>
                             : (void *)fused_step_kernel<R, MODEL, 1, 64>;
        case 128: return fast ? (void *)fused_step_kernel<R, MODEL, 1, 128, true>
                              : (void *)fused_step_kernel<R, MODEL, 1, 128>;
        case 256: return fast ? (void *)fused_step_kernel<R, MODEL, 1, 256, true>
                              : (void *)fused_step_kernel<R, MODEL, 1, 256>;
        default: break;
    }
    if (spt == 1) return (void *)fused_step_kernel<R, MODEL, 1, 0>;
    if (spt == 2) return (void *)fused_step_kernel<R, MODEL, 2, 0>;
    return (void *)fused_step_kernel<R, MODEL, 4, 0>;
}

}  // namespace clv
