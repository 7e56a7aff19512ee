// k_tiled.cu -- the Langevin step of chains whose slices are too large for the
// fused kernel, after the kinetic terms have been filtered along every axis
// (k_axis.cu writes kin = e^{-eps H_kin} psi and kinbar for all imaginary times).
//
// A CTA owns 256 consecutive spatial sites of one chain (one thread per site)
// and streams through imaginary times [tau0, tau1).  psi(tau-1), psi(tau),
// kin(tau-1) and psibar(tau) are carried in registers from the previous tau;
// each iteration loads psi(tau+1), psibar(tau+1), kin(tau) and kinbar(tau+1),
// prefetched one tau ahead, so every array is read once per step (plus one halo
// slice per CTA).  Drift (Propagator_without_cutoff.cu:1-129 for the reference
// model; the spin-1 drift otherwise), the step-rule reduction, the noise
// (in-register Philox or an injected buffer in the reference's ind_rand layout)
// and the update psi + dt K + sqrt(dt) xi (:131-157, Lattice.cu:32-36) happen
// in registers, and the new state goes to the other buffer of the ping-pong
// pair.  The step size follows the same protocol as the fused kernel:
// speculative update with dt_max and an exact redo of rejected chains (K/max
// rule), or a reduce-only pass and an apply pass (the reference's rule; at FP64
// the reduce pass stores the drift and the site-parallel update applies it).
#include "clv_internal.cuh"
#include "clv_launch.h"
#include "drift_math.cuh"

namespace clv {

template <class R, class C2>
__device__ __forceinline__ void normal_pair(uint64_t seed, uint32_t chain, uint64_t step, int pair,
                                            uint32_t site, C2 &z0, C2 &z1) {
    const uint4 o = philox_block(seed, chain, step, pair, site);
    if constexpr (sizeof(R) == 8) {
        const double2 g0 = box_muller64(o.x, o.y), g1 = box_muller64(o.z, o.w);
        z0.x = g0.x; z0.y = g0.y; z1.x = g1.x; z1.y = g1.y;
    } else {
        const float2 g0 = box_muller32(o.x, o.y), g1 = box_muller32(o.z, o.w);
        z0.x = g0.x; z0.y = g0.y; z1.x = g1.x; z1.y = g1.y;
    }
}


// One task: imaginary times [tau0, tau1) of 256 sites of one chain.
template <class R, int MODEL>
__device__ __forceinline__ void tiled_task(const LaunchTiled &A, const TileTask task) {
    using C2 = typename Cx<R>::T;
    constexpr int NC = MODEL == CLV_MODEL_REF4 ? 4 : 3;
    const ChainDev &ch = A.chains[task.chain];
    ChainState *st = A.state + task.chain;
    if (A.mode == FUSED_APPLY && A.only_rejected && st->accepted) return;  // uniform per CTA

    const int V = ch.V, T = ch.nt;
    const int s = task.site0 + threadIdx.x;
    const bool act = s < V;
    const C2 *gpsi = reinterpret_cast<const C2 *>(A.psi_in) + ch.off;
    const C2 *gpsic = reinterpret_cast<const C2 *>(A.psic_in) + ch.off;
    const C2 *gkin = reinterpret_cast<const C2 *>(A.kin) + ch.off;
    const C2 *gkinc = reinterpret_cast<const C2 *>(A.kinc) + ch.off;
    C2 *opsi = reinterpret_cast<C2 *>(A.psi_out) + ch.off;
    C2 *opsic = reinterpret_cast<C2 *>(A.psic_out) + ch.off;
    const bool writes = A.mode != FUSED_MAXONLY;

    R dt = 0;
    uint64_t nstep = 0;
    if (A.mode == FUSED_SPEC) { dt = (R)ch.dt_max; nstep = st->step; }
    else if (A.mode == FUSED_APPLY) { dt = (R)st->dt; nstep = st->noise_step; }
    const R sd = (R)sqrt((double)dt);

    auto at = [&](int c, int tau) -> long long {
        const int t = tau < 0 ? tau + T : (tau >= T ? tau - T : tau);
        return ((long long)c * T + t) * V + s;
    };
    const int tau0 = task.tau0, tau1 = task.tau1;
    // carried: psi(tau-1), kin(tau-1), psibar(tau), psi(tau)
    C2 Pp[NC], Kp[NC], Qc[NC], Pc[NC];
    Spin1Bilinears<C2> Bm;  // spin-1: bilinears of (psibar(tau), psi(tau-1)), carried
    // prefetched for the next tau: psi(tau+1), psibar(tau+1), kin(tau), kinbar(tau+1)
    C2 nP[NC], nQ[NC], nK[NC], nKc[NC];
    auto load_next = [&](int tau) {
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            nP[c] = gpsi[at(c, tau + 1)];
            nQ[c] = gpsic[at(c, tau + 1)];
            nK[c] = gkin[at(c, tau)];
            nKc[c] = gkinc[at(c, tau + 1)];
        }
    };
    if (act) {
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            Pp[c] = gpsi[at(c, tau0 - 1)];
            Kp[c] = gkin[at(c, tau0 - 1)];
            Qc[c] = gpsic[at(c, tau0)];
            Pc[c] = gpsi[at(c, tau0)];
        }
        if constexpr (MODEL == CLV_MODEL_SPIN1) Bm = spin1_bilinears<C2, R>(Qc, Pp);
        load_next(tau0);
    }

    R mxr = 0, smr = 0;
    int bad = 0;
    const DriftConsts<R> dk(ch);
    const uint64_t seed = ch.seed;
    const int ref_rule = A.dt_rule == CLV_DT_REF_MEANMAX;
    if (act) {
        for (int tau = tau0; tau < tau1; ++tau) {
            C2 vpp[NC], vcp[NC], kt[NC], kp[NC];
#pragma unroll
            for (int c = 0; c < NC; ++c) { vpp[c] = nP[c]; vcp[c] = nQ[c]; kt[c] = nK[c]; kp[c] = nKc[c]; }
            if (tau + 1 < tau1) load_next(tau + 1);
            C2 K[NC], Kc[NC];
            if constexpr (MODEL == CLV_MODEL_REF4)
                drift_ref4_vals<R>(dk, Pp, Pc, vpp, Qc, vcp, Kp, kp, K, Kc);
            else
            {
                const Spin1Bilinears<C2> Bp = spin1_bilinears<C2, R>(vcp, Pc);
                drift_spin1_vals_b<R>(dk, Bm, Bp, Pp, Pc, Qc, vcp, Kp, kp, K, Kc);
                Bm = Bp;
            }
            if (A.mode == FUSED_MAXONLY && A.drift_out) {
                // the stored-drift update reads the drift instead of a second drift pass
#pragma unroll
                for (int c = 0; c < NC; ++c) {
                    const long long gi = ((long long)c * T + tau) * V + s;
                    reinterpret_cast<C2 *>(A.drift_out)[ch.off + gi] = K[c];
                    reinterpret_cast<C2 *>(A.driftc_out)[ch.off + gi] = Kc[c];
                }
            }
            if (A.mode != FUSED_APPLY) {
                if (ref_rule) {
                    const R a0 = hypot(K[0].x, K[0].y);
                    mxr = fmax(mxr, a0);
                    smr += a0;
                    bad |= !isfinite(a0);
                } else {
#pragma unroll
                    for (int c = 0; c < NC; ++c) {
                        const R m1 = abs2<R>(K[c]);
                        const R m2 = abs2<R>(Kc[c]);
                        mxr = fmax(mxr, fmax(m1, m2));
                        smr += m1 + m2;  // unused by the rule; carries a NaN to the finish
                    }
                }
            }
            if (writes) {
                const uint32_t site = (uint32_t)(tau * V + s);
                C2 z[NC];
                if (A.noise == CLV_NOISE_PHILOX) {
#pragma unroll
                    for (int c = 0; c < NC; c += 2) {
                        if (c + 1 < NC) {
                            normal_pair<R>(seed, (uint32_t)task.chain, nstep, c >> 1, site, z[c], z[c + 1]);
                        } else {
                            const uint2 w = noise_words(seed, (uint32_t)task.chain, nstep, c, NC, site);
                            z[c] = unit_normal<R, C2>(w.x, w.y);
                        }
                    }
                } else {
#pragma unroll
                    for (int c = 0; c < NC; ++c) {
                        const long long r = ch.noise_off + (((long long)c * V + s) * T + tau) * 2;
                        z[c].x = (R)A.noise_buf[r];
                        z[c].y = (R)A.noise_buf[r + 1];
                    }
                }
#pragma unroll
                for (int c = 0; c < NC; ++c) {
                    C2 zz;
                    zz.x = mul_rn<R>(sd, z[c].x);
                    zz.y = mul_rn<R>(sd, z[c].y);
                    const long long gi = ((long long)c * T + tau) * V + s;
                    opsi[gi] = langevin_update<R>(Pc[c], K[c], dt, zz, false);
                    opsic[gi] = langevin_update<R>(Qc[c], Kc[c], dt, zz, true);
                }
            }
#pragma unroll
            for (int c = 0; c < NC; ++c) {
                Pp[c] = Pc[c];
                Pc[c] = vpp[c];
                Kp[c] = kt[c];
                Qc[c] = vcp[c];
            }
        }
    }
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

// One CTA per task.  (Persistent CTAs walking the task list measured slower:
// every task start exposes its first loads, which resident CTAs otherwise hide.)
template <class R, int MODEL>
__global__ void __launch_bounds__(256, sizeof(R) == 4 ? 2 : 1) tiled_step_kernel(const LaunchTiled A) {
    // a stored-drift update launched programmatically after this reduce pass may start
    // drawing its noise now; it waits for this grid's end before it reads the results
    asm volatile("griddepcontrol.launch_dependents;");
    tiled_task<R, MODEL>(A, A.tasks[blockIdx.x]);
}

template <class R>
cudaError_t launch_tiled(const LaunchTiled &L, cudaStream_t s) {
    if (L.ntasks == 0) return cudaSuccess;
    if (L.model == CLV_MODEL_REF4)
        tiled_step_kernel<R, CLV_MODEL_REF4><<<L.ntasks, 256, 0, s>>>(L);
    else
        tiled_step_kernel<R, CLV_MODEL_SPIN1><<<L.ntasks, 256, 0, s>>>(L);
    return cudaGetLastError();
}

template <class R>
cudaError_t setup_tiled(int model, int *ctas_per_sm) {
    const void *fn = model == CLV_MODEL_REF4 ? (const void *)tiled_step_kernel<R, CLV_MODEL_REF4>
                                             : (const void *)tiled_step_kernel<R, CLV_MODEL_SPIN1>;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas_per_sm, fn, 256, 0);
}

template cudaError_t setup_tiled<float>(int, int *);
template cudaError_t setup_tiled<double>(int, int *);
template cudaError_t launch_tiled<float>(const LaunchTiled &, cudaStream_t);
template cudaError_t launch_tiled<double>(const LaunchTiled &, cudaStream_t);

}  // namespace clv
