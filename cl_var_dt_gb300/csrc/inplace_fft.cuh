// inplace_fft.cuh -- in-place mixed-radix line filters over a CTA's tile of lines in
// shared memory (the plane filter and the strided-axis filter).
//
// Each line of N sites is filtered in place as a Cooley-Tukey transform: decimation in
// frequency forward, the filter, decimation in time back.  A butterfly reads and writes
// the same R elements, so the butterflies of a pass are independent: a thread streams
// its butterflies with R values in registers, and one block barrier separates the
// passes.  The forward passes leave the spectrum in digit-reversed order; the middle
// pass multiplies each frequency by its filter value there, and the inverse passes take
// digit-reversed input back to natural order, so the filter needs no reordering pass.
//
// Geometry: NL lines, element a of line l at t[l * LS + a * ES] (shared) or
// g[l * LG + a * EG] (global, first and last passes); butterfly b = tid + p T of a
// pass is butterfly j = b / NL of line l = b % NL, so consecutive lanes take
// consecutive lines at one j (conflict-free at an odd line pitch, coalesced where the
// lines are neighbours in global memory; twiddle and filter reads are broadcasts).
// Plan: Plan::nfac(N) radices Plan::fac(N, p), p = 0 first.
#pragma once

#include "fft_radix.cuh"

namespace clv {

template <class Plan, int N, int NL, int T, int U>
struct InPlace {
    static constexpr int NF = Plan::nfac(N);
    static_assert(NF >= 2, "two radix factors at least");
    // span L_p = N / (R_0 ... R_{p-1}) of forward pass p: it transforms blocks of L_p
    // elements, R_p strided sub-sequences of each
    static __host__ __device__ constexpr int span(int p) {
        int L = N;
        for (int i = 0; i < p; ++i) L /= Plan::fac(N, i);
        return L;
    }
    static constexpr int RL = Plan::fac(N, NF - 1);

    // Frequency index of the q = 0 output of middle-pass butterfly j (output q has
    // frequency mid_freq(j) + q N / R_last): position i = sum_p q_p (L_p / R_p) after
    // the forward passes holds frequency sum_p q_p (R_0 ... R_{p-1}); j = i / R_last.
    template <int P = 0, int W = 1>
    static __device__ __forceinline__ int mid_freq(int rem) {
        if constexpr (P >= NF - 1) {
            return 0;
        } else {
            constexpr int S = span(P + 1) / RL;  // place value of digit p in j
            const int q = rem / S;
            return q * W + mid_freq<P + 1, W * Plan::fac(N, P)>(rem - q * S);
        }
    }

    // Forward pass p (decimation in frequency): butterfly (block, k) takes elements
    // block L + k + m S (m < R, S = L / R), y_q = sum_m x_m w_R^{mq}, then y_q w_L^{qk}
    // (tw: the table exp(-2 pi i m / N)).
    template <class C2, int P>
    static __device__ __forceinline__ void dif(C2 *t, int LS, int ES, const C2 *tw) {
        constexpr int R = Plan::fac(N, P), L = span(P), S = L / R, NB = NL * (N / R), PER = (NB + T - 1) / T;
#pragma unroll(U)
        for (int p = 0; p < PER; ++p) {
            const int b = threadIdx.x + p * T;
            if (NB % T != 0 && b >= NB) break;
            const int l = b % NL, j = b / NL;
            const int a0 = (j / S) * L + j % S, k = j % S;
            C2 v[R];
#pragma unroll
            for (int m = 0; m < R; ++m) v[m] = t[l * LS + (a0 + m * S) * ES];
            Radix<C2, R>::template run<-1>(v);
            if constexpr (S > 1) {
#pragma unroll
                for (int q = 1; q < R; ++q) v[q] = cmul(v[q], tw[q * k * (N / L)]);
            }
#pragma unroll
            for (int q = 0; q < R; ++q) t[l * LS + (a0 + q * S) * ES] = v[q];
        }
    }

    // Inverse of forward pass p (decimation in time): inputs y_q at block L + k + q S
    // times conj(w_L^{qk}), x_m = sum_q y_q w_R^{-mq}, in place.  GLOBAL (pass 0 only):
    // the outputs go to g[l LG + a EG] instead (added to what is there when acc).
    template <class C2, int P, bool GLOBAL = false>
    static __device__ __forceinline__ void dit(C2 *t, int LS, int ES, const C2 *tw, C2 *g = nullptr,
                                               long long LG = 0, long long EG = 0, bool acc = false) {
        constexpr int R = Plan::fac(N, P), L = span(P), S = L / R, NB = NL * (N / R), PER = (NB + T - 1) / T;
        static_assert(!GLOBAL || P == 0, "the last inverse pass writes global memory");
#pragma unroll(U)
        for (int p = 0; p < PER; ++p) {
            const int b = threadIdx.x + p * T;
            if (NB % T != 0 && b >= NB) break;
            const int l = b % NL, j = b / NL;
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
            if constexpr (GLOBAL) {
#pragma unroll
                for (int m = 0; m < R; ++m) {
                    C2 *d = g + l * LG + (a0 + m * S) * EG;
                    *d = acc ? cadd(*d, v[m]) : v[m];
                }
            } else {
#pragma unroll
                for (int m = 0; m < R; ++m) t[l * LS + (a0 + m * S) * ES] = v[m];
            }
        }
    }

    // The last forward pass (span R_last, no twiddles), the filter f at each output's
    // frequency times cst, and the first inverse pass, in registers.
    template <class C2, class RR>
    static __device__ __forceinline__ void mid(C2 *t, int LS, int ES, const RR *f, RR cst) {
        constexpr int nR = N / RL, NB = NL * nR, PER = (NB + T - 1) / T;
#pragma unroll(U)
        for (int p = 0; p < PER; ++p) {
            const int b = threadIdx.x + p * T;
            if (NB % T != 0 && b >= NB) break;
            const int l = b % NL, j = b / NL;
            C2 v[RL];
#pragma unroll
            for (int m = 0; m < RL; ++m) v[m] = t[l * LS + (j * RL + m) * ES];
            Radix<C2, RL>::template run<-1>(v);
            const int fj = mid_freq(j);
#pragma unroll
            for (int q = 0; q < RL; ++q) v[q] = cscale(f[fj + q * nR] * cst, v[q]);
            Radix<C2, RL>::template run<1>(v);
#pragma unroll
            for (int m = 0; m < RL; ++m) t[l * LS + (j * RL + m) * ES] = v[m];
        }
    }

    // Pass 0 from global memory in two halves: first_load fills v with the inputs of
    // a thread's butterflies p0 .. p0 + G - 1 (element a of line l at g[l LG + a EG]),
    // first_finish runs them (twiddles from tw, which may be the global table) and
    // stores them into the tile.
    static constexpr int R0 = Plan::fac(N, 0), NB0 = NL * (N / R0), PER0 = (NB0 + T - 1) / T;
    template <class C2, int G>
    static __device__ __forceinline__ void first_load(C2 (&v)[G][R0], const C2 *g, long long LG, long long EG,
                                                      int p0) {
        constexpr int S = N / R0;
#pragma unroll
        for (int u = 0; u < G; ++u) {
            const int b = threadIdx.x + (p0 + u) * T;
            if (NB0 % T != 0 && b >= NB0) break;
            const int l = b % NL, j = b / NL;
#pragma unroll
            for (int m = 0; m < R0; ++m) v[u][m] = g[l * LG + (j + m * S) * EG];
        }
    }
    template <class C2, int G>
    static __device__ __forceinline__ void first_finish(C2 (&v)[G][R0], C2 *t, int LS, int ES, const C2 *tw,
                                                        int p0) {
        constexpr int S = N / R0;
#pragma unroll
        for (int u = 0; u < G; ++u) {
            const int b = threadIdx.x + (p0 + u) * T;
            if (NB0 % T != 0 && b >= NB0) break;
            const int l = b % NL, k = b / NL;
            Radix<C2, R0>::template run<-1>(v[u]);
#pragma unroll
            for (int q = 1; q < R0; ++q) v[u][q] = cmul(v[u][q], tw[q * k]);
#pragma unroll
            for (int q = 0; q < R0; ++q) t[l * LS + (k + q * S) * ES] = v[u][q];
        }
    }

    template <class C2, int P>
    static __device__ __forceinline__ void fwd(C2 *t, int LS, int ES, const C2 *tw) {
        if constexpr (P < NF - 1) {
            dif<C2, P>(t, LS, ES, tw);
            __syncthreads();
            fwd<C2, P + 1>(t, LS, ES, tw);
        }
    }
    // inverse passes P .. P_END (P_END = 1 when the caller writes pass 0 to global)
    template <class C2, int P, int P_END = 0>
    static __device__ __forceinline__ void inv(C2 *t, int LS, int ES, const C2 *tw) {
        if constexpr (P >= P_END) {
            dit<C2, P>(t, LS, ES, tw);
            __syncthreads();
            inv<C2, P - 1, P_END>(t, LS, ES, tw);
        }
    }

    // Filter all NL lines of the tile along their axis, in place, from forward pass P0
    // on (P0 = 1: the caller ran pass 0); ends with a block barrier.
    template <class C2, class RR, int P0>
    static __device__ __forceinline__ void filter(C2 *t, int LS, int ES, const C2 *tw, const RR *f, RR cst) {
        fwd<C2, P0>(t, LS, ES, tw);
        mid<C2, RR>(t, LS, ES, f, cst);
        __syncthreads();
        inv<C2, NF - 2>(t, LS, ES, tw);
    }
};

}  // namespace clv
