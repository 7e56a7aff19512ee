// k_step.cu -- drift with the on-device step rule, and the Langevin update.
//
// drift_kernel: one thread per lattice site (tau, s) of one chain computes the
//   drift K and Kbar of every component (reference model:
//   calculate_drift_without_noise, Propagator_without_cutoff.cu:1-129; spin-1
//   model: the contact terms c0/2 n^2 + c1/2 F^2 with the exponential kinetic
//   term), reduces |K| for the step rule with warp shuffles, writes one partial
//   per CTA, and the last CTA of each chain to finish reduces the partials in a
//   fixed order and writes the new dt into the chain's device state.  This
//   replaces compute_max_and_mean_drift + the host round trip of
//   get_max_and_mean_drift / compute_new_dt (:219-265, :351-404): no host sync,
//   deterministic, and capturable in a CUDA graph.
// update_kernel: psi += dt K + sqrt(dt) xi, psibar += dt Kbar + sqrt(dt) conj(xi)
//   (multiply_by_timestep, add_noise, summation: :131-157, Lattice.cu:32-36),
//   with xi from the injected buffer (reference ind_rand layout) or from an
//   in-register Philox4x32-10 stream.
#include "clv_internal.cuh"
#include "clv_launch.h"

namespace clv {

template <class R> __device__ __forceinline__ R mul_rn(R a, R b);
template <> __device__ __forceinline__ double mul_rn<double>(double a, double b) { return __dmul_rn(a, b); }
template <> __device__ __forceinline__ float mul_rn<float>(float a, float b) { return __fmul_rn(a, b); }
template <class R> __device__ __forceinline__ R add_rn(R a, R b);
template <> __device__ __forceinline__ double add_rn<double>(double a, double b) { return __dadd_rn(a, b); }
template <> __device__ __forceinline__ float add_rn<float>(float a, float b) { return __fadd_rn(a, b); }

__device__ __forceinline__ long long fidx(const ChainDev &ch, int c, int tau, int s) {
    return ch.off + ((long long)c * ch.nt + tau) * ch.V + s;
}

// ---------------------------------------------------------------- drift
template <class R>
__device__ __forceinline__ void drift_ref4(const ChainDev &ch, const typename Cx<R>::T *psi,
                                           const typename Cx<R>::T *psic,
                                           const typename Cx<R>::T *kin,
                                           const typename Cx<R>::T *kinc, int tau, int tm, int tp,
                                           int s, typename Cx<R>::T *K, typename Cx<R>::T *Kc) {
    using C2 = typename Cx<R>::T;
    C2 pm[4], pc[4], cc[4], cp[4], pp[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        pm[a] = psi[fidx(ch, a, tm, s)];
        pc[a] = psi[fidx(ch, a, tau, s)];
        pp[a] = psi[fidx(ch, a, tp, s)];
        cc[a] = psic[fidx(ch, a, tau, s)];
        cp[a] = psic[fidx(ch, a, tp, s)];
    }
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
    const R mu[4] = {(R)(ch.mu + ch.P + ch.Q), (R)ch.mu, (R)ch.mu, (R)(ch.mu - ch.P + ch.Q)};
    const R pre = (R)(ch.a_x * 1.0), eps = (R)ch.eps, g2 = (R)(2 * ch.G);
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        const C2 km = kin[fidx(ch, a, tm, s)];
        const C2 kp = kinc[fidx(ch, a, tp, s)];
        C2 inner = cadd(csub(cscale(mu[a], pm[a]), cscale(g2, tm_[a])), km);
        K[a] = cscale(pre, cadd(csub(pm[a], pc[a]), cscale(eps, inner)));
        // the chemical-potential term of the conjugate drift multiplies psi(tau+1)
        // (Propagator_without_cutoff.cu:71,88,105,122)
        inner = cadd(csub(cscale(mu[a], pp[a]), cscale(g2, tp_[a])), kp);
        Kc[a] = cscale(pre, cadd(csub(cp[a], cc[a]), cscale(eps, inner)));
    }
}

// dV/dbar (into db) and dV/dket (into dk) of V = c0/2 n^2 + c1/2 (Fz^2 + F+ F-)
// for bar = psibar, ket = psi at the split times of the drift.
template <class C2, class R>
__device__ __forceinline__ void spin1_dbar(R c0, R c1, const C2 *bar, const C2 *ket, C2 *db) {
    const R r2 = (R)1.41421356237309504880, ir2 = (R)0.70710678118654752440;
    const C2 n = cadd(cadd(cmul(bar[0], ket[0]), cmul(bar[1], ket[1])), cmul(bar[2], ket[2]));
    const C2 Fz = csub(cmul(bar[0], ket[0]), cmul(bar[2], ket[2]));
    const C2 Fp = cscale(r2, cadd(cmul(bar[0], ket[1]), cmul(bar[1], ket[2])));
    const C2 Fm = cscale(r2, cadd(cmul(bar[1], ket[0]), cmul(bar[2], ket[1])));
    const C2 s0 = cadd(cmul(Fz, ket[0]), cscale(ir2, cmul(Fm, ket[1])));
    const C2 s1 = cscale(ir2, cadd(cmul(Fp, ket[0]), cmul(Fm, ket[2])));
    const C2 s2 = csub(cscale(ir2, cmul(Fp, ket[1])), cmul(Fz, ket[2]));
    db[0] = cadd(cscale(c0, cmul(n, ket[0])), cscale(c1, s0));
    db[1] = cadd(cscale(c0, cmul(n, ket[1])), cscale(c1, s1));
    db[2] = cadd(cscale(c0, cmul(n, ket[2])), cscale(c1, s2));
}
template <class C2, class R>
__device__ __forceinline__ void spin1_dket(R c0, R c1, const C2 *bar, const C2 *ket, C2 *dk) {
    const R r2 = (R)1.41421356237309504880, ir2 = (R)0.70710678118654752440;
    const C2 n = cadd(cadd(cmul(bar[0], ket[0]), cmul(bar[1], ket[1])), cmul(bar[2], ket[2]));
    const C2 Fz = csub(cmul(bar[0], ket[0]), cmul(bar[2], ket[2]));
    const C2 Fp = cscale(r2, cadd(cmul(bar[0], ket[1]), cmul(bar[1], ket[2])));
    const C2 Fm = cscale(r2, cadd(cmul(bar[1], ket[0]), cmul(bar[2], ket[1])));
    const C2 s0 = cadd(cmul(Fz, bar[0]), cscale(ir2, cmul(Fp, bar[1])));
    const C2 s1 = cscale(ir2, cadd(cmul(Fm, bar[0]), cmul(Fp, bar[2])));
    const C2 s2 = csub(cscale(ir2, cmul(Fm, bar[1])), cmul(Fz, bar[2]));
    dk[0] = cadd(cscale(c0, cmul(n, bar[0])), cscale(c1, s0));
    dk[1] = cadd(cscale(c0, cmul(n, bar[1])), cscale(c1, s1));
    dk[2] = cadd(cscale(c0, cmul(n, bar[2])), cscale(c1, s2));
}

template <class R>
__device__ __forceinline__ void drift_spin1(const ChainDev &ch, const typename Cx<R>::T *psi,
                                            const typename Cx<R>::T *psic,
                                            const typename Cx<R>::T *kin,
                                            const typename Cx<R>::T *kinc, int tau, int tm,
                                            int tp, int s, typename Cx<R>::T *K,
                                            typename Cx<R>::T *Kc) {
    using C2 = typename Cx<R>::T;
    C2 pm[3], pc[3], cc[3], cp[3], dK[3], dKc[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        pm[a] = psi[fidx(ch, a, tm, s)];
        pc[a] = psi[fidx(ch, a, tau, s)];
        cc[a] = psic[fidx(ch, a, tau, s)];
        cp[a] = psic[fidx(ch, a, tp, s)];
    }
    const R c0 = (R)ch.c0, c1 = (R)ch.c1, eps = (R)ch.eps;
    spin1_dbar<C2, R>(c0, c1, cc, pm, dK);
    spin1_dket<C2, R>(c0, c1, cp, pc, dKc);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const C2 km = kin[fidx(ch, a, tm, s)];
        const C2 kp = kinc[fidx(ch, a, tp, s)];
        K[a] = csub(csub(km, pc[a]), cscale(eps, dK[a]));
        Kc[a] = csub(csub(kp, cc[a]), cscale(eps, dKc[a]));
    }
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

// New step from the chain's reduction (tid 0 of the chain's last CTA).
__device__ void finish_step(const ChainDev &ch, ChainState &st, int dt_rule, double mx, double sm,
                            int bad) {
    double dt, mean = 0.0;
    if (dt_rule == CLV_DT_REF_MEANMAX) {
        // Propagator_without_cutoff.cu:372-404
        mean = sm / (double)((long long)ch.ncomp * ch.V * ch.nt);
        if (mx <= 0.0) dt = ch.DT;
        else dt = __dmul_rn(mean / mx, ch.DT);
        if (dt < ch.dt_min) { dt = ch.dt_min; st.clamp_low++; st.flags |= CLV_FLAG_DT_CLAMPED_LOW; }
        if (dt > ch.dt_max_clamp) { dt = ch.dt_max_clamp; st.clamp_high++; st.flags |= CLV_FLAG_DT_CLAMPED_HIGH; }
        dt = __dadd_rn(__dmul_rn(1.0 - ch.alpha, ch.DT), __dmul_rn(ch.alpha, dt));
    } else {
        mx = sqrt(mx);  // the reduction ran over |K|^2
        dt = ch.dt_max;
        if (mx > 0.0) {
            const double t = ch.K / mx;
            if (t < dt) dt = t;
        }
    }
    if (bad || !isfinite(mx) || !isfinite(sm)) st.flags |= CLV_FLAG_NONFINITE;
    st.dt = dt;
    st.max = mx;
    st.mean = mean;
    st.t += dt;
    st.noise_step = st.step;
    st.step += 1;
}

template <class R, int MODEL, int RULE>
__global__ void __launch_bounds__(kSiteBlock)
drift_kernel(const ChainDev *__restrict__ chains, ChainState *__restrict__ state,
             const SiteTask *__restrict__ tasks, const typename Cx<R>::T *__restrict__ psi,
             const typename Cx<R>::T *__restrict__ psic, const typename Cx<R>::T *__restrict__ kin,
             const typename Cx<R>::T *__restrict__ kinc, typename Cx<R>::T *__restrict__ drift,
             typename Cx<R>::T *__restrict__ driftc, double2 *__restrict__ partials) {
    using C2 = typename Cx<R>::T;
    constexpr int NC = MODEL == CLV_MODEL_REF4 ? 4 : 3;
    const SiteTask task = tasks[blockIdx.x];
    const ChainDev &ch = chains[task.chain];
    const int site = task.site0 + threadIdx.x;
    double mx = 0.0, sm = 0.0;
    int bad = 0;
    if (site < ch.V * ch.nt) {
        const int tau = site / ch.V, s = site - tau * ch.V;
        const int tm = tau == 0 ? ch.nt - 1 : tau - 1;
        const int tp = tau == ch.nt - 1 ? 0 : tau + 1;
        C2 K[NC], Kc[NC];
        if (MODEL == CLV_MODEL_REF4)
            drift_ref4<R>(ch, psi, psic, kin, kinc, tau, tm, tp, s, K, Kc);
        else
            drift_spin1<R>(ch, psi, psic, kin, kinc, tau, tm, tp, s, K, Kc);
#pragma unroll
        for (int a = 0; a < NC; ++a) {
            drift[fidx(ch, a, tau, s)] = K[a];
            driftc[fidx(ch, a, tau, s)] = Kc[a];
        }
        if (RULE == CLV_DT_REF_MEANMAX) {
            // component 0 of the psi drift only (launch quirk of :363-366)
            const double a0 = (double)hypot(K[0].x, K[0].y);
            mx = a0;
            sm = a0;
            bad = !isfinite(a0);
        } else {
#pragma unroll
            for (int a = 0; a < NC; ++a) {
                const double m1 = (double)K[a].x * K[a].x + (double)K[a].y * K[a].y;
                const double m2 = (double)Kc[a].x * Kc[a].x + (double)Kc[a].y * Kc[a].y;
                bad |= !isfinite(m1) || !isfinite(m2);
                mx = fmax(mx, fmax(m1, m2));
            }
        }
    }
    bad = __syncthreads_or(bad);
    block_max_sum(mx, sm);
    __shared__ int am_last;
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = make_double2(mx, bad ? __longlong_as_double(0x7ff8000000000000ll) : sm);
        __threadfence();
        const unsigned prev = atomicAdd(&state[task.chain].arrive, 1u);
        am_last = prev == (unsigned)ch.site_nblocks - 1;
    }
    __syncthreads();
    if (!am_last) return;
    __threadfence();
    mx = 0.0;
    sm = 0.0;
    bad = 0;
    for (int i = threadIdx.x; i < ch.site_nblocks; i += blockDim.x) {
        const double2 p = __ldcg(&partials[ch.site_block0 + i]);
        mx = fmax(mx, p.x);
        sm += p.y;
        bad |= !isfinite(p.y) || !isfinite(p.x);
    }
    bad = __syncthreads_or(bad);
    block_max_sum(mx, sm);
    if (threadIdx.x == 0) {
        ChainState &st = state[task.chain];
        finish_step(ch, st, RULE, mx, sm, bad);
        st.arrive = 0;
    }
}

template <class R>
cudaError_t launch_drift(const LaunchSites &L, cudaStream_t s) {
    using C2 = typename Cx<R>::T;
    auto args = [&](auto kern) {
        kern<<<L.ntasks, kSiteBlock, 0, s>>>(L.chains, L.state, L.tasks, (const C2 *)L.psi,
                                             (const C2 *)L.psic, (const C2 *)L.kin,
                                             (const C2 *)L.kinc, (C2 *)L.drift, (C2 *)L.driftc,
                                             L.partials);
    };
    if (L.model == CLV_MODEL_REF4) {
        if (L.dt_rule == CLV_DT_REF_MEANMAX) args(drift_kernel<R, CLV_MODEL_REF4, CLV_DT_REF_MEANMAX>);
        else args(drift_kernel<R, CLV_MODEL_REF4, CLV_DT_K_OVER_MAX>);
    } else {
        if (L.dt_rule == CLV_DT_REF_MEANMAX) args(drift_kernel<R, CLV_MODEL_SPIN1, CLV_DT_REF_MEANMAX>);
        else args(drift_kernel<R, CLV_MODEL_SPIN1, CLV_DT_K_OVER_MAX>);
    }
    return cudaGetLastError();
}

// --------------------------------------------------------------- update
template <class R, int NOISE>
__global__ void __launch_bounds__(kSiteBlock)
update_kernel(const ChainDev *__restrict__ chains, const ChainState *__restrict__ state,
              const SiteTask *__restrict__ tasks, typename Cx<R>::T *__restrict__ psi,
              typename Cx<R>::T *__restrict__ psic, const typename Cx<R>::T *__restrict__ drift,
              const typename Cx<R>::T *__restrict__ driftc, const double *__restrict__ noise) {
    using C2 = typename Cx<R>::T;
    const SiteTask task = tasks[blockIdx.x];
    const ChainDev &ch = chains[task.chain];
    const int site = task.site0 + threadIdx.x;
    if (site >= ch.V * ch.nt) return;
    const int tau = site / ch.V, s = site - tau * ch.V;
    const double dtd = state[task.chain].dt;
    const R dt = (R)dtd, sd = (R)sqrt(dtd);
    const uint64_t nstep = state[task.chain].noise_step;
    for (int a = 0; a < ch.ncomp; ++a) {
        C2 z;
        if (NOISE == CLV_NOISE_EXTERNAL) {
            const long long r = ch.noise_off + (((long long)a * ch.V + s) * ch.nt + tau) * 2;
            z.x = (R)noise[r];
            z.y = (R)noise[r + 1];
        } else {
            const uint32_t idx = (uint32_t)(((long long)a * ch.nt + tau) * ch.V + s);
            if (sizeof(R) == 8) {
                const double2 g = philox_normal64(ch.seed, (uint32_t)task.chain, nstep, idx);
                z.x = (R)g.x; z.y = (R)g.y;
            } else {
                const float2 g = philox_normal32(ch.seed, (uint32_t)task.chain, nstep, idx);
                z.x = (R)g.x; z.y = (R)g.y;
            }
        }
        z.x = mul_rn<R>(sd, z.x);
        z.y = mul_rn<R>(sd, z.y);
        const long long i = fidx(ch, a, tau, s);
        const C2 K = drift[i], Kc = driftc[i];
        C2 p = psi[i], pc = psic[i];
        // d = dt*K; d += z; psi += d  (rounded step by step, as the reference's kernels)
        p.x = add_rn<R>(p.x, add_rn<R>(mul_rn<R>(K.x, dt), z.x));
        p.y = add_rn<R>(p.y, add_rn<R>(mul_rn<R>(K.y, dt), z.y));
        pc.x = add_rn<R>(pc.x, add_rn<R>(mul_rn<R>(Kc.x, dt), z.x));
        pc.y = add_rn<R>(pc.y, add_rn<R>(mul_rn<R>(Kc.y, dt), -z.y));
        psi[i] = p;
        psic[i] = pc;
    }
}

template <class R>
cudaError_t launch_update(const LaunchSites &L, cudaStream_t s) {
    using C2 = typename Cx<R>::T;
    if (L.noise == CLV_NOISE_EXTERNAL)
        update_kernel<R, CLV_NOISE_EXTERNAL><<<L.ntasks, kSiteBlock, 0, s>>>(
            L.chains, L.state, L.tasks, (C2 *)L.psi_w, (C2 *)L.psic_w, (const C2 *)L.drift,
            (const C2 *)L.driftc, L.noise_buf);
    else
        update_kernel<R, CLV_NOISE_PHILOX><<<L.ntasks, kSiteBlock, 0, s>>>(
            L.chains, L.state, L.tasks, (C2 *)L.psi_w, (C2 *)L.psic_w, (const C2 *)L.drift,
            (const C2 *)L.driftc, nullptr);
    return cudaGetLastError();
}

// ----------------------------------------------------------------- init
// set_value (Lattice.cu:50-81): comps 0,3 = v, comps 1,2 = (2/3) v; psibar gets conj(v).
template <class R>
__global__ void set_mean_field_kernel(const ChainDev *__restrict__ chains,
                                      const SiteTask *__restrict__ tasks,
                                      typename Cx<R>::T *__restrict__ f, int conj, double re,
                                      double im) {
    using C2 = typename Cx<R>::T;
    const SiteTask task = tasks[blockIdx.x];
    const ChainDev &ch = chains[task.chain];
    const int site = task.site0 + threadIdx.x;
    if (site >= ch.V * ch.nt) return;
    const int tau = site / ch.V, s = site - tau * ch.V;
    const double2 v = make_double2(re, conj ? -im : im);
    const double2 t = make_double2(2.0 / 3.0, 0.0);
    const double2 v23 = make_double2(t.x * v.x - t.y * v.y, t.x * v.y + t.y * v.x);
    for (int a = 0; a < ch.ncomp; ++a) {
        const double2 w = (a == 1 || a == 2) ? v23 : v;
        C2 o; o.x = (R)w.x; o.y = (R)w.y;
        f[fidx(ch, a, tau, s)] = o;
    }
}

template <class R>
cudaError_t launch_set_mean_field(const LaunchSites &L, int field, double re, double im,
                                  cudaStream_t s) {
    using C2 = typename Cx<R>::T;
    set_mean_field_kernel<R><<<L.ntasks, kSiteBlock, 0, s>>>(
        L.chains, L.tasks, (C2 *)(field == 0 ? L.psi_w : L.psic_w), field, re, im);
    return cudaGetLastError();
}

// Spin-1 start: psi = amp + sigma xi (Philox stream at step 2^64-1), psibar = conj(psi).
template <class R>
__global__ void init_spin1_kernel(const ChainDev *__restrict__ chains,
                                  const SiteTask *__restrict__ tasks,
                                  typename Cx<R>::T *__restrict__ psi,
                                  typename Cx<R>::T *__restrict__ psic, double amp, double sigma) {
    using C2 = typename Cx<R>::T;
    const SiteTask task = tasks[blockIdx.x];
    const ChainDev &ch = chains[task.chain];
    const int site = task.site0 + threadIdx.x;
    if (site >= ch.V * ch.nt) return;
    const int tau = site / ch.V, s = site - tau * ch.V;
    for (int a = 0; a < ch.ncomp; ++a) {
        const uint32_t idx = (uint32_t)(((long long)a * ch.nt + tau) * ch.V + s);
        const double2 g = philox_normal64(ch.seed, (uint32_t)task.chain, ~0ull, idx);
        C2 p; p.x = (R)(amp + sigma * g.x); p.y = (R)(sigma * g.y);
        psi[fidx(ch, a, tau, s)] = p;
        psic[fidx(ch, a, tau, s)] = cconj(p);
    }
}

template <class R>
cudaError_t launch_init_spin1(const LaunchSites &L, double amp, double sigma, cudaStream_t s) {
    using C2 = typename Cx<R>::T;
    init_spin1_kernel<R><<<L.ntasks, kSiteBlock, 0, s>>>(L.chains, L.tasks, (C2 *)L.psi_w,
                                                         (C2 *)L.psic_w, amp, sigma);
    return cudaGetLastError();
}

// --------------------------------------------------- boundary conversion
template <class R>
__global__ void convert_kernel(typename Cx<R>::T *dst, const double2 *src, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const double2 v = src[i];
        typename Cx<R>::T o; o.x = (R)v.x; o.y = (R)v.y;
        dst[i] = o;
    }
}
template <class R>
__global__ void convert_back_kernel(double2 *dst, const typename Cx<R>::T *src, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const typename Cx<R>::T v = src[i];
        dst[i] = make_double2((double)v.x, (double)v.y);
    }
}

template <class R>
cudaError_t launch_import(void *dst, const double2 *src, long long n, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const int blocks = (int)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096);
    convert_kernel<R><<<blocks, 256, 0, s>>>((typename Cx<R>::T *)dst, src, n);
    return cudaGetLastError();
}
template <class R>
cudaError_t launch_export(double2 *dst, const void *src, long long n, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const int blocks = (int)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096);
    convert_back_kernel<R><<<blocks, 256, 0, s>>>(dst, (const typename Cx<R>::T *)src, n);
    return cudaGetLastError();
}

#define CLV_INST(R)                                                                           \
    template cudaError_t launch_drift<R>(const LaunchSites &, cudaStream_t);                 \
    template cudaError_t launch_update<R>(const LaunchSites &, cudaStream_t);                \
    template cudaError_t launch_set_mean_field<R>(const LaunchSites &, int, double, double,  \
                                                  cudaStream_t);                             \
    template cudaError_t launch_init_spin1<R>(const LaunchSites &, double, double,           \
                                              cudaStream_t);                                 \
    template cudaError_t launch_import<R>(void *, const double2 *, long long, cudaStream_t); \
    template cudaError_t launch_export<R>(double2 *, const void *, long long, cudaStream_t);
CLV_INST(double)
CLV_INST(float)

}  // namespace clv
