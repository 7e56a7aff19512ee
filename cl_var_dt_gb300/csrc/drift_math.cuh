// drift_math.cuh -- per-site drift of both models on register values.
//
// Inputs at one spatial site: psi(tau-1) pm, psi(tau) pc, psi(tau+1) pp,
// psibar(tau) cc, psibar(tau+1) cp, kinetic terms km = kin(tau-1) and
// kp = kinbar(tau+1).  Outputs K (psi drift) and Kc (psibar drift).
#pragma once

#include "clv_internal.cuh"

namespace clv {

// Per-chain constants of the drift in the working precision, loaded once per CTA.
template <class R>
struct DriftConsts {
    R eps, pre, g2, c0, c1, ec0, ec1;
    R mu[4];
    __device__ __forceinline__ explicit DriftConsts(const ChainDev &ch) {
        eps = (R)ch.eps;
        pre = (R)ch.a_x;
        g2 = (R)(2 * ch.G);
        c0 = (R)ch.c0;
        c1 = (R)ch.c1;
        ec0 = (R)(ch.eps * ch.c0);  // spin-1: eps c0 and eps c1 (the drift's prefactors)
        ec1 = (R)(ch.eps * ch.c1);
        mu[0] = (R)(ch.mu + ch.P + ch.Q);
        mu[1] = (R)ch.mu;
        mu[2] = (R)ch.mu;
        mu[3] = (R)(ch.mu - ch.P + ch.Q);
    }
};

// Reference 4-component model: calculate_drift_without_noise
// (Propagator_without_cutoff.cu:24-128) with factor = 1.  which: 1 = K only, 2 =
// Kbar only, 3 = both (a CTA-uniform choice of the kernels that split the fields);
// cmask: the components a whose K[a], Kc[a] are computed (bit a; CTA-uniform).
template <class R, class C2>
__device__ __forceinline__ void drift_ref4_vals(const DriftConsts<R> &k, const C2 *pm, const C2 *pc,
                                                const C2 *pp, const C2 *cc, const C2 *cp,
                                                const C2 *km, const C2 *kp, C2 *K, C2 *Kc, int which = 3,
                                                int cmask = 0xF) {
    const R *mu = k.mu;
    const R pre = k.pre, eps = k.eps, g2 = k.g2;
    if (which & 1) {
        C2 N[4], tm_[4];
#pragma unroll
        for (int a = 0; a < 4; ++a) N[a] = cmul(pm[a], cc[a]);
        if (cmask & 1) tm_[0] = cadd(cmul(cadd(cadd(N[0], N[1]), N[2]), pm[0]), cmul(cmul(pm[1], cc[3]), pm[2]));
        if (cmask & 2) tm_[1] = cadd(cmul(cadd(cadd(N[0], N[1]), N[3]), pm[1]), cmul(cmul(pm[0], cc[2]), pm[3]));
        if (cmask & 4) tm_[2] = cadd(cmul(cadd(cadd(N[0], N[2]), N[3]), pm[2]), cmul(cmul(pm[3], cc[1]), pm[0]));
        if (cmask & 8) tm_[3] = cadd(cmul(cadd(cadd(N[1], N[2]), N[3]), pm[3]), cmul(cmul(pm[2], cc[0]), pm[1]));
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            if (!((cmask >> a) & 1)) continue;
            const C2 inner = cadd(csub(cscale(mu[a], pm[a]), cscale(g2, tm_[a])), km[a]);
            K[a] = cscale(pre, cadd(csub(pm[a], pc[a]), cscale(eps, inner)));
        }
    }
    if (which & 2) {
        C2 Nc[4], tp_[4];
#pragma unroll
        for (int a = 0; a < 4; ++a) Nc[a] = cmul(pc[a], cp[a]);
        if (cmask & 1) tp_[0] = cadd(cmul(cadd(cadd(Nc[0], Nc[1]), Nc[2]), cp[0]), cmul(cmul(cp[1], pc[3]), cp[2]));
        if (cmask & 2) tp_[1] = cadd(cmul(cadd(cadd(Nc[0], Nc[1]), Nc[3]), cp[1]), cmul(cmul(cp[0], pc[2]), cp[3]));
        if (cmask & 4) tp_[2] = cadd(cmul(cadd(cadd(Nc[0], Nc[2]), Nc[3]), cp[2]), cmul(cmul(cp[3], pc[1]), cp[0]));
        if (cmask & 8) tp_[3] = cadd(cmul(cadd(cadd(Nc[1], Nc[2]), Nc[3]), cp[3]), cmul(cmul(cp[2], pc[0]), cp[1]));
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            if (!((cmask >> a) & 1)) continue;
            // the chemical-potential term of the conjugate drift multiplies psi(tau+1)
            // (Propagator_without_cutoff.cu:71,88,105,122)
            const C2 inner = cadd(csub(cscale(mu[a], pp[a]), cscale(g2, tp_[a])), kp[a]);
            Kc[a] = cscale(pre, cadd(csub(cp[a], cc[a]), cscale(eps, inner)));
        }
    }
}

// Bilinears of one (bar, ket) pair: density n = sum_m bar_m ket_m, F_z =
// bar_0 ket_0 - bar_2 ket_2 and P = F+/sqrt2 = bar_0 ket_1 + bar_1 ket_2,
// M = F-/sqrt2 = bar_1 ket_0 + bar_2 ket_1 of the spin-1 contact potential
// V = c0/2 n^2 + c1/2 (Fz^2 + F+ F-) = c0/2 n^2 + c1/2 Fz^2 + c1 P M.  The pair
// (psibar(tau+1), psi(tau)) enters both the psibar drift at tau and the psi
// drift at tau+1, so the streaming kernels compute it once and carry it.
template <class C2>
struct Spin1Bilinears {
    C2 n, Fz, P, M;
};

template <class C2, class R>
__device__ __forceinline__ Spin1Bilinears<C2> spin1_bilinears(const C2 *bar, const C2 *ket) {
    Spin1Bilinears<C2> b;
    const C2 p0 = cmul(bar[0], ket[0]), p2 = cmul(bar[2], ket[2]);
    b.n = cadd(cadd(p0, cmul(bar[1], ket[1])), p2);
    b.Fz = csub(p0, p2);
    b.P = cadd(cmul(bar[0], ket[1]), cmul(bar[1], ket[2]));
    b.M = cadd(cmul(bar[1], ket[0]), cmul(bar[2], ket[1]));
    return b;
}

// a - b z - s w for complex a, b, z, w and a real s (one rounding chain per part)
template <class C2, class R>
__device__ __forceinline__ C2 sub_cmul_scale(C2 a, C2 b, C2 z, R s, C2 w) {
    C2 r;
    r.x = a.x - b.x * z.x + b.y * z.y - s * w.x;
    r.y = a.y - b.x * z.y - b.y * z.x - s * w.y;
    return r;
}

// K_m = d_m - eps dV/dbar_m (bar, ket from the pair's bilinears; d = kin - psi):
// dV/dbar = c0 n ket + c1 s with s_0 = Fz ket_0 + M ket_1, s_1 = P ket_0 + M ket_2,
// s_2 = P ket_1 - Fz ket_2; the constants arrive as e0 = eps c0, e1 = eps c1.
template <class C2, class R>
__device__ __forceinline__ void spin1_drift_bar(R e0, R e1, const Spin1Bilinears<C2> &b, const C2 *ket,
                                                const C2 *d, C2 *K) {
    const C2 en = cscale(e0, b.n);
    const C2 s0 = cadd(cmul(b.Fz, ket[0]), cmul(b.M, ket[1]));
    const C2 s1 = cadd(cmul(b.P, ket[0]), cmul(b.M, ket[2]));
    const C2 s2 = csub(cmul(b.P, ket[1]), cmul(b.Fz, ket[2]));
    K[0] = sub_cmul_scale(d[0], en, ket[0], e1, s0);
    K[1] = sub_cmul_scale(d[1], en, ket[1], e1, s1);
    K[2] = sub_cmul_scale(d[2], en, ket[2], e1, s2);
}

// Kbar_m = d_m - eps dV/dket_m: dV/dket = c0 n bar + c1 s with s_0 = Fz bar_0 +
// P bar_1, s_1 = M bar_0 + P bar_2, s_2 = M bar_1 - Fz bar_2.
template <class C2, class R>
__device__ __forceinline__ void spin1_drift_ket(R e0, R e1, const Spin1Bilinears<C2> &b, const C2 *bar,
                                                const C2 *d, C2 *K) {
    const C2 en = cscale(e0, b.n);
    const C2 s0 = cadd(cmul(b.Fz, bar[0]), cmul(b.P, bar[1]));
    const C2 s1 = cadd(cmul(b.M, bar[0]), cmul(b.P, bar[2]));
    const C2 s2 = csub(cmul(b.M, bar[1]), cmul(b.Fz, bar[2]));
    K[0] = sub_cmul_scale(d[0], en, bar[0], e1, s0);
    K[1] = sub_cmul_scale(d[1], en, bar[1], e1, s1);
    K[2] = sub_cmul_scale(d[2], en, bar[2], e1, s2);
}

// Spin-1 model: K_m = kin_m(tau-1) - psi_m(tau) - eps dV/dbar_m(psibar(tau), psi(tau-1)),
// Kbar_m = kinbar_m(tau+1) - psibar_m(tau) - eps dV/dket_m(psibar(tau+1), psi(tau)).
// bm: bilinears of (psibar(tau), psi(tau-1)); bp: of (psibar(tau+1), psi(tau)).
template <class R, class C2>
__device__ __forceinline__ void drift_spin1_vals_b(const DriftConsts<R> &k, const Spin1Bilinears<C2> &bm,
                                                   const Spin1Bilinears<C2> &bp, const C2 *pm,
                                                   const C2 *pc, const C2 *cc, const C2 *cp,
                                                   const C2 *km, const C2 *kp, C2 *K, C2 *Kc) {
    C2 d[3], dc[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        d[a] = csub(km[a], pc[a]);
        dc[a] = csub(kp[a], cc[a]);
    }
    spin1_drift_bar<C2, R>(k.ec0, k.ec1, bm, pm, d, K);
    spin1_drift_ket<C2, R>(k.ec0, k.ec1, bp, cp, dc, Kc);
}

// which: 1 = K only, 2 = Kbar only, 3 = both.
template <class R, class C2>
__device__ __forceinline__ void drift_spin1_vals(const DriftConsts<R> &k, const C2 *pm, const C2 *pc,
                                                 const C2 *cc, const C2 *cp, const C2 *km,
                                                 const C2 *kp, C2 *K, C2 *Kc, int which = 3) {
    if (which == 3) {
        drift_spin1_vals_b<R, C2>(k, spin1_bilinears<C2, R>(cc, pm), spin1_bilinears<C2, R>(cp, pc), pm, pc,
                                  cc, cp, km, kp, K, Kc);
        return;
    }
    C2 d[3];
    if (which & 1) {
#pragma unroll
        for (int a = 0; a < 3; ++a) d[a] = csub(km[a], pc[a]);
        spin1_drift_bar<C2, R>(k.ec0, k.ec1, spin1_bilinears<C2, R>(cc, pm), pm, d, K);
    } else {
#pragma unroll
        for (int a = 0; a < 3; ++a) d[a] = csub(kp[a], cc[a]);
        spin1_drift_ket<C2, R>(k.ec0, k.ec1, spin1_bilinears<C2, R>(cp, pc), cp, d, Kc);
    }
}

template <class R> __device__ __forceinline__ R mul_rn(R a, R b);
template <> __device__ __forceinline__ double mul_rn<double>(double a, double b) { return __dmul_rn(a, b); }
template <> __device__ __forceinline__ float mul_rn<float>(float a, float b) { return __fmul_rn(a, b); }
template <class R> __device__ __forceinline__ R add_rn(R a, R b);
template <> __device__ __forceinline__ double add_rn<double>(double a, double b) { return __dadd_rn(a, b); }
template <> __device__ __forceinline__ float add_rn<float>(float a, float b) { return __fadd_rn(a, b); }

template <class R> __device__ __forceinline__ R fma_rn(R a, R b, R c);
template <> __device__ __forceinline__ double fma_rn<double>(double a, double b, double c) { return __fma_rn(a, b, c); }
template <> __device__ __forceinline__ float fma_rn<float>(float a, float b, float c) { return __fmaf_rn(a, b, c); }

// |z|^2 of a drift value for the K/max rule's reduction, rounded the same way in
// every kernel that reduces it (x x + (y y), one fused multiply-add), so that the
// kernels' step sizes agree bit for bit.
template <class R, class C2>
__device__ __forceinline__ R abs2(C2 z) {
    return fma_rn<R>(z.x, z.x, mul_rn<R>(z.y, z.y));
}

// psi + dt K + z, rounded step by step as the reference's kernels do
// (multiply_by_timestep, add_noise, summation); conj = 1 adds conj(z).  FP32,
// which has no counterpart in the reference to match bit for bit, rounds dt K + z
// once (fused multiply-add).
template <class R, class C2>
__device__ __forceinline__ C2 langevin_update(C2 p, C2 K, R dt, C2 z, bool conj) {
    C2 o;
    const R zy = conj ? -z.y : z.y;
    if constexpr (sizeof(R) == 4) {
        o.x = __fadd_rn(p.x, __fmaf_rn(K.x, dt, z.x));
        o.y = __fadd_rn(p.y, __fmaf_rn(K.y, dt, zy));
    } else {
        o.x = add_rn<R>(p.x, add_rn<R>(mul_rn<R>(K.x, dt), z.x));
        o.y = add_rn<R>(p.y, add_rn<R>(mul_rn<R>(K.y, dt), zy));
    }
    return o;
}

// Maximum that is NaN when either argument is (max.NaN.f32), so a reduction of
// |drift|^2 carries a non-finite drift to the chain's finish by itself.
__device__ __forceinline__ float max_nan(float a, float b) {
    float r;
    asm("max.NaN.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
    return r;
}

// Block-wide (max, sum) with warp shuffles; result valid in thread 0.
__device__ __forceinline__ void block_max_sum(double &mx, double &sm) {
    __shared__ double smx[32], ssm[32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        sm += __shfl_xor_sync(0xffffffffu, sm, o);
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) { smx[warp] = mx; ssm[warp] = sm; }
    __syncthreads();
    if (warp == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        mx = lane < nw ? smx[lane] : 0.0;
        sm = lane < nw ? ssm[lane] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
            sm += __shfl_xor_sync(0xffffffffu, sm, o);
        }
    }
    __syncthreads();
}

// New step of one chain from its reduction (run by one thread).  REF rule:
// compute_new_dt of Propagator_without_cutoff.cu:372-404; K/max rule:
// dt = min(dt_max, K / max|drift|) with the reduction taken over |K|^2.
__device__ __forceinline__ double step_rule(const ChainDev &ch, ChainState &st, int dt_rule,
                                            double &mx, double sm, double &mean) {
    double dt;
    mean = 0.0;
    if (dt_rule == CLV_DT_REF_MEANMAX) {
        mean = sm / (double)((long long)ch.ncomp * ch.V * ch.nt);
        if (mx <= 0.0) dt = ch.DT;
        else dt = __dmul_rn(mean / mx, ch.DT);
        if (dt < ch.dt_min) { dt = ch.dt_min; st.clamp_low++; st.flags |= CLV_FLAG_DT_CLAMPED_LOW; }
        if (dt > ch.dt_max_clamp) { dt = ch.dt_max_clamp; st.clamp_high++; st.flags |= CLV_FLAG_DT_CLAMPED_HIGH; }
        dt = __dadd_rn(__dmul_rn(1.0 - ch.alpha, ch.DT), __dmul_rn(ch.alpha, dt));
    } else {
        mx = sqrt(mx);
        dt = ch.dt_max;
        if (mx > 0.0) {
            const double t = ch.K / mx;
            if (t < dt) dt = t;
        }
    }
    return dt;
}

}  // namespace clv
