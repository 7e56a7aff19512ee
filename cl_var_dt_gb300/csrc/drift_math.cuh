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
    R eps, pre, g2, c0, c1;
    R mu[4];
    __device__ __forceinline__ explicit DriftConsts(const ChainDev &ch) {
        eps = (R)ch.eps;
        pre = (R)ch.a_x;
        g2 = (R)(2 * ch.G);
        c0 = (R)ch.c0;
        c1 = (R)ch.c1;
        mu[0] = (R)(ch.mu + ch.P + ch.Q);
        mu[1] = (R)ch.mu;
        mu[2] = (R)ch.mu;
        mu[3] = (R)(ch.mu - ch.P + ch.Q);
    }
};

// Reference 4-component model: calculate_drift_without_noise
// (Propagator_without_cutoff.cu:24-128) with factor = 1.
template <class R, class C2>
__device__ __forceinline__ void drift_ref4_vals(const DriftConsts<R> &k, const C2 *pm, const C2 *pc,
                                                const C2 *pp, const C2 *cc, const C2 *cp,
                                                const C2 *km, const C2 *kp, C2 *K, C2 *Kc) {
    C2 N[4], Nc[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) { N[a] = cmul(pm[a], cc[a]); Nc[a] = cmul(pc[a], cp[a]); }
    C2 tm_[4], tp_[4];
    tm_[0] = cadd(cmul(cadd(cadd(N[0], N[1]), N[2]), pm[0]), cmul(cmul(pm[1], cc[3]), pm[2]));
    tm_[1] = cadd(cmul(cadd(cadd(N[0], N[1]), N[3]), pm[1]), cmul(cmul(pm[0], cc[2]), pm[3]));
    tm_[2] = cadd(cmul(cadd(cadd(N[0], N[2]), N[3]), pm[2]), cmul(cmul(pm[3], cc[1]), pm[0]));
    tm_[3] = cadd(cmul(cadd(cadd(N[1], N[2]), N[3]), pm[3]), cmul(cmul(pm[2], cc[0]), pm[1]));
    tp_[0] = cadd(cmul(cadd(cadd(Nc[0], Nc[1]), Nc[2]), cp[0]), cmul(cmul(cp[1], pc[3]), cp[2]));
    tp_[1] = cadd(cmul(cadd(cadd(Nc[0], Nc[1]), Nc[3]), cp[1]), cmul(cmul(cp[0], pc[2]), cp[3]));
    tp_[2] = cadd(cmul(cadd(cadd(Nc[0], Nc[2]), Nc[3]), cp[2]), cmul(cmul(cp[3], pc[1]), cp[0]));
    tp_[3] = cadd(cmul(cadd(cadd(Nc[1], Nc[2]), Nc[3]), cp[3]), cmul(cmul(cp[2], pc[0]), cp[1]));
    const R *mu = k.mu;
    const R pre = k.pre, eps = k.eps, g2 = k.g2;
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        C2 inner = cadd(csub(cscale(mu[a], pm[a]), cscale(g2, tm_[a])), km[a]);
        K[a] = cscale(pre, cadd(csub(pm[a], pc[a]), cscale(eps, inner)));
        // the chemical-potential term of the conjugate drift multiplies psi(tau+1)
        // (Propagator_without_cutoff.cu:71,88,105,122)
        inner = cadd(csub(cscale(mu[a], pp[a]), cscale(g2, tp_[a])), kp[a]);
        Kc[a] = cscale(pre, cadd(csub(cp[a], cc[a]), cscale(eps, inner)));
    }
}

// Bilinears of one (bar, ket) pair: density n, F_z, F+ and F- of the spin-1
// contact potential V = c0/2 n^2 + c1/2 (Fz^2 + F+ F-).  The pair (psibar(tau+1),
// psi(tau)) enters both the psibar drift at tau and the psi drift at tau+1, so
// the streaming kernels compute it once and carry it to the next tau.
template <class C2>
struct Spin1Bilinears {
    C2 n, Fz, Fp, Fm;
};

template <class C2, class R>
__device__ __forceinline__ Spin1Bilinears<C2> spin1_bilinears(const C2 *bar, const C2 *ket) {
    const R r2 = (R)1.41421356237309504880;
    Spin1Bilinears<C2> b;
    b.n = cadd(cadd(cmul(bar[0], ket[0]), cmul(bar[1], ket[1])), cmul(bar[2], ket[2]));
    b.Fz = csub(cmul(bar[0], ket[0]), cmul(bar[2], ket[2]));
    b.Fp = cscale(r2, cadd(cmul(bar[0], ket[1]), cmul(bar[1], ket[2])));
    b.Fm = cscale(r2, cadd(cmul(bar[1], ket[0]), cmul(bar[2], ket[1])));
    return b;
}

// dV/dbar_m for bar = psibar, ket = psi, from the pair's bilinears.
template <class C2, class R>
__device__ __forceinline__ void spin1_dbar_b(R c0, R c1, const Spin1Bilinears<C2> &b, const C2 *ket,
                                             C2 *db) {
    const R ir2 = (R)0.70710678118654752440;
    const C2 s0 = cadd(cmul(b.Fz, ket[0]), cscale(ir2, cmul(b.Fm, ket[1])));
    const C2 s1 = cscale(ir2, cadd(cmul(b.Fp, ket[0]), cmul(b.Fm, ket[2])));
    const C2 s2 = csub(cscale(ir2, cmul(b.Fp, ket[1])), cmul(b.Fz, ket[2]));
    db[0] = cadd(cscale(c0, cmul(b.n, ket[0])), cscale(c1, s0));
    db[1] = cadd(cscale(c0, cmul(b.n, ket[1])), cscale(c1, s1));
    db[2] = cadd(cscale(c0, cmul(b.n, ket[2])), cscale(c1, s2));
}

// dV/dket_m from the pair's bilinears.
template <class C2, class R>
__device__ __forceinline__ void spin1_dket_b(R c0, R c1, const Spin1Bilinears<C2> &b, const C2 *bar,
                                             C2 *dk) {
    const R ir2 = (R)0.70710678118654752440;
    const C2 s0 = cadd(cmul(b.Fz, bar[0]), cscale(ir2, cmul(b.Fp, bar[1])));
    const C2 s1 = cscale(ir2, cadd(cmul(b.Fm, bar[0]), cmul(b.Fp, bar[2])));
    const C2 s2 = csub(cscale(ir2, cmul(b.Fm, bar[1])), cmul(b.Fz, bar[2]));
    dk[0] = cadd(cscale(c0, cmul(b.n, bar[0])), cscale(c1, s0));
    dk[1] = cadd(cscale(c0, cmul(b.n, bar[1])), cscale(c1, s1));
    dk[2] = cadd(cscale(c0, cmul(b.n, bar[2])), cscale(c1, s2));
}

template <class C2, class R>
__device__ __forceinline__ void spin1_dbar(R c0, R c1, const C2 *bar, const C2 *ket, C2 *db) {
    spin1_dbar_b<C2, R>(c0, c1, spin1_bilinears<C2, R>(bar, ket), ket, db);
}

template <class C2, class R>
__device__ __forceinline__ void spin1_dket(R c0, R c1, const C2 *bar, const C2 *ket, C2 *dk) {
    spin1_dket_b<C2, R>(c0, c1, spin1_bilinears<C2, R>(bar, ket), bar, dk);
}

// Spin-1 model: K_m = kin_m(tau-1) - psi_m(tau) - eps dV/dbar_m(psibar(tau), psi(tau-1)),
// Kbar_m = kinbar_m(tau+1) - psibar_m(tau) - eps dV/dket_m(psibar(tau+1), psi(tau)).
// bm: bilinears of (psibar(tau), psi(tau-1)); bp: of (psibar(tau+1), psi(tau)).
template <class R, class C2>
__device__ __forceinline__ void drift_spin1_vals_b(const DriftConsts<R> &k, const Spin1Bilinears<C2> &bm,
                                                   const Spin1Bilinears<C2> &bp, const C2 *pm,
                                                   const C2 *pc, const C2 *cc, const C2 *cp,
                                                   const C2 *km, const C2 *kp, C2 *K, C2 *Kc) {
    C2 dK[3], dKc[3];
    const R c0 = k.c0, c1 = k.c1, eps = k.eps;
    spin1_dbar_b<C2, R>(c0, c1, bm, pm, dK);
    spin1_dket_b<C2, R>(c0, c1, bp, cp, dKc);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        K[a] = csub(csub(km[a], pc[a]), cscale(eps, dK[a]));
        Kc[a] = csub(csub(kp[a], cc[a]), cscale(eps, dKc[a]));
    }
}

template <class R, class C2>
__device__ __forceinline__ void drift_spin1_vals(const DriftConsts<R> &k, const C2 *pm, const C2 *pc,
                                                 const C2 *cc, const C2 *cp, const C2 *km,
                                                 const C2 *kp, C2 *K, C2 *Kc) {
    drift_spin1_vals_b<R, C2>(k, spin1_bilinears<C2, R>(cc, pm), spin1_bilinears<C2, R>(cp, pc), pm, pc,
                              cc, cp, km, kp, K, Kc);
}

template <class R> __device__ __forceinline__ R mul_rn(R a, R b);
template <> __device__ __forceinline__ double mul_rn<double>(double a, double b) { return __dmul_rn(a, b); }
template <> __device__ __forceinline__ float mul_rn<float>(float a, float b) { return __fmul_rn(a, b); }
template <class R> __device__ __forceinline__ R add_rn(R a, R b);
template <> __device__ __forceinline__ double add_rn<double>(double a, double b) { return __dadd_rn(a, b); }
template <> __device__ __forceinline__ float add_rn<float>(float a, float b) { return __fadd_rn(a, b); }

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
