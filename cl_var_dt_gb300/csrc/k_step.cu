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
#include "drift_math.cuh"

namespace clv {

__device__ __forceinline__ long long fidx(const ChainDev &ch, int c, int tau, int s) {
    return ch.off + ((long long)c * ch.nt + tau) * ch.V + s;
}

// New step from the chain's reduction (tid 0 of the chain's last CTA).
__device__ void finish_step(const ChainDev &ch, ChainState &st, int dt_rule, double mx, double sm,
                            int bad) {
    double mean;
    const double dt = step_rule(ch, st, dt_rule, mx, sm, mean);
    if (bad || !isfinite(mx) || !isfinite(sm)) st.flags |= CLV_FLAG_NONFINITE;
    st.dt = dt;
    st.max = mx;
    st.mean = mean;
    st.t += dt;
    st.noise_step = st.step;
    st.step += 1;
    st.accepted = 0;
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
        C2 K[NC], Kc[NC], pm[NC], pc[NC], pp[NC], cc[NC], cp[NC], km[NC], kp[NC];
#pragma unroll
        for (int a = 0; a < NC; ++a) {
            pm[a] = psi[fidx(ch, a, tm, s)];
            pc[a] = psi[fidx(ch, a, tau, s)];
            cc[a] = psic[fidx(ch, a, tau, s)];
            cp[a] = psic[fidx(ch, a, tp, s)];
            km[a] = kin[fidx(ch, a, tm, s)];
            kp[a] = kinc[fidx(ch, a, tp, s)];
            if (MODEL == CLV_MODEL_REF4) pp[a] = psi[fidx(ch, a, tp, s)];
        }
        const DriftConsts<R> dk(ch);
        if (MODEL == CLV_MODEL_REF4)
            drift_ref4_vals<R>(dk, pm, pc, pp, cc, cp, km, kp, K, Kc);
        else
            drift_spin1_vals<R>(dk, pm, pc, cc, cp, km, kp, K, Kc);
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
              const SiteTask *__restrict__ tasks, const typename Cx<R>::T *__restrict__ psi,
              const typename Cx<R>::T *__restrict__ psic, typename Cx<R>::T *__restrict__ psi_o,
              typename Cx<R>::T *__restrict__ psic_o, const typename Cx<R>::T *__restrict__ drift,
              const typename Cx<R>::T *__restrict__ driftc, const double *__restrict__ noise, int early) {
    using C2 = typename Cx<R>::T;
    const SiteTask task = tasks[blockIdx.x];
    const ChainDev &ch = chains[task.chain];
    const int site = task.site0 + threadIdx.x;
    const bool in = site < ch.V * ch.nt;
    const int tau = in ? site / ch.V : 0, s = in ? site - tau * ch.V : 0;
    // blockIdx.y: component pair; one Philox block serves both components of the pair
    const int a0 = 2 * (int)blockIdx.y, a1 = a0 + 2 < ch.ncomp ? a0 + 2 : ch.ncomp;
    // Under a programmatic launch this grid starts while the step's reduce pass still
    // runs: the unit normals, which do not depend on the step size, are drawn first,
    // for the noise step the state shows now (the reduce pass's last CTA moves it on
    // only at its very end), and checked against the state after the wait.
    const ChainState *stc = state + task.chain;
    const uint64_t pre = early ? __ldcg(&stc->step) : ~0ull;
    C2 zu[2] = {mk<C2>(0.0, 0.0), mk<C2>(0.0, 0.0)};
    auto draw = [&](uint64_t nstep) {
        if (NOISE == CLV_NOISE_EXTERNAL || !in) return;
        // a row with the lone component of an odd count shares its block with the
        // neighbouring site (noise_words)
        const uint32_t lin = (uint32_t)((long long)tau * ch.V + s);
        const bool lone = lone_component(a0, ch.ncomp);
        const uint4 o = philox_block(ch.seed, (uint32_t)task.chain, nstep, (int)blockIdx.y, lone ? lin >> 1 : lin);
        for (int a = a0; a < a1; ++a) {
            const bool hi = lone ? (lin & 1) != 0 : (a & 1) != 0;
            const uint32_t wx = hi ? o.z : o.x, wy = hi ? o.w : o.y;
            if (sizeof(R) == 8) {
                const double2 g = box_muller64(wx, wy);
                zu[a - a0].x = (R)g.x; zu[a - a0].y = (R)g.y;
            } else {
                const float2 g = box_muller32(wx, wy);
                zu[a - a0].x = (R)g.x; zu[a - a0].y = (R)g.y;
            }
        }
    };
    if (early) draw(pre);
    asm volatile("griddepcontrol.wait;" ::: "memory");  // the reduce pass is complete and visible
    if (!in) return;
    const uint64_t nstep = __ldcg(&stc->noise_step);
    if (nstep != pre) draw(nstep);
    const double dtd = __ldcg(&stc->dt);
    const R dt = (R)dtd, sd = (R)sqrt(dtd);
    for (int a = a0; a < a1; ++a) {
        C2 z;
        if (NOISE == CLV_NOISE_EXTERNAL) {
            const long long r = ch.noise_off + (((long long)a * ch.V + s) * ch.nt + tau) * 2;
            z.x = (R)noise[r];
            z.y = (R)noise[r + 1];
        } else {
            z = zu[a - a0];
        }
        z.x = mul_rn<R>(sd, z.x);
        z.y = mul_rn<R>(sd, z.y);
        const long long i = fidx(ch, a, tau, s);
        psi_o[i] = langevin_update<R>(psi[i], drift[i], dt, z, false);
        psic_o[i] = langevin_update<R>(psic[i], driftc[i], dt, z, true);
    }
}

template <class R>
cudaError_t launch_update(const LaunchSites &L, cudaStream_t s) {
    using C2 = typename Cx<R>::T;
    // one grid row per component pair (2 rows cover both models; rows past the last
    // component return at once)
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(L.ntasks, 2);
    cfg.blockDim = dim3(kSiteBlock);
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = L.pdl ? 1 : 0;
    if (L.noise == CLV_NOISE_EXTERNAL)
        return cudaLaunchKernelEx(&cfg, update_kernel<R, CLV_NOISE_EXTERNAL>, L.chains,
                                  (const ChainState *)L.state, L.tasks, (const C2 *)L.psi, (const C2 *)L.psic,
                                  (C2 *)L.psi_w, (C2 *)L.psic_w, (const C2 *)L.drift, (const C2 *)L.driftc,
                                  L.noise_buf, L.pdl);
    return cudaLaunchKernelEx(&cfg, update_kernel<R, CLV_NOISE_PHILOX>, L.chains, (const ChainState *)L.state,
                              L.tasks, (const C2 *)L.psi, (const C2 *)L.psic, (C2 *)L.psi_w, (C2 *)L.psic_w,
                              (const C2 *)L.drift, (const C2 *)L.driftc, (const double *)nullptr, L.pdl);
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
        const uint32_t idx = (uint32_t)((long long)tau * ch.V + s);
        const double2 g = philox_normal64(ch.seed, (uint32_t)task.chain, ~0ull, a, idx);
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
