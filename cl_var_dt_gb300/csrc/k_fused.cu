// k_fused.cu -- the whole Langevin step of chains whose spatial slice fits in
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
// Bounded wait: gives up after 2^22 polls (far beyond any copy's latency).
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
    for (int i = 0; i < (1 << 22); ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// ----------------------------------------------------------- slice filter
// One Stockham pass of radix R along one axis, over NJ slices of ncomp*V sites.
template <class C2, int R>
__device__ __forceinline__ void slice_pass(int NJ, const C2 *s0, const C2 *s1, C2 *d0, C2 *d1,
                                           const AxisDev &ax, const C2 *__restrict__ tw, int V,
                                           int ncomp, int Ns, int S) {
    const int n = ax.n, inner = ax.inner, nR = n / R, tstep = n / (Ns * R);
    const int lpc = V / n;  // lines per component
    const int per_job = ncomp * lpc * nR;
    for (int b = threadIdx.x; b < NJ * per_job; b += blockDim.x) {
        const int job = b >= per_job;
        const int r0 = b - job * per_job;
        const int L = r0 / nR, j = r0 - L * nR;
        const int c = L / lpc, l = L - c * lpc;
        const int base = c * V + (l / inner) * n * inner + (l % inner);
        const C2 *ls = (job ? s1 : s0) + base;
        C2 *ld = (job ? d1 : d0) + base;
        const int k = j % Ns;
        C2 v[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            C2 x = ls[(j + r * nR) * inner];
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
        for (int q = 0; q < R; ++q) ld[(o + q * Ns) * inner] = v[q];
    }
}

template <class R>
__device__ __forceinline__ const typename Cx<R>::T *tw_of(const AxisDev &ax);
template <> __device__ __forceinline__ const double2 *tw_of<double>(const AxisDev &ax) { return ax.tw64; }
template <> __device__ __forceinline__ const float2 *tw_of<float>(const AxisDev &ax) { return ax.tw32; }
template <class R>
__device__ __forceinline__ const R *filt_of(const AxisDev &ax);
template <> __device__ __forceinline__ const double *filt_of<double>(const AxisDev &ax) { return ax.filt64; }
template <> __device__ __forceinline__ const float *filt_of<float>(const AxisDev &ax) { return ax.filt32; }

// Kinetic filter of NJ (1 or 2) slices: src_j is read-only, (wa_j, wb_j) are work
// buffers; *out_j receives the buffer holding kin_j.  Ends with __syncthreads.
template <class R>
__device__ void slice_filter(const ChainDev &ch, int ncomp, int kinetic, int NJ,
                             const typename Cx<R>::T *src0, const typename Cx<R>::T *src1,
                             typename Cx<R>::T *wa0, typename Cx<R>::T *wb0,
                             typename Cx<R>::T *wa1, typename Cx<R>::T *wb1,
                             typename Cx<R>::T **out0, typename Cx<R>::T **out1) {
    using C2 = typename Cx<R>::T;
    const int V = ch.V;
    const C2 *c0 = src0, *c1 = src1;
    C2 *d0 = wa0, *d1 = wa1, *e0 = wb0, *e1 = wb1;
    bool first_axis = true;
    for (int a = 0; a < 3; ++a) {
        const AxisDev &ax = ch.axis[a];
        if (ax.n <= 1) continue;
        if (kinetic == CLV_KIN_REF_LINEAR_PX && a > 0) break;
        const C2 *tw = tw_of<R>(ax);
        for (int dir = 0; dir < 2; ++dir) {
            const int S = dir == 0 ? -1 : +1;
            int Ns = 1;
            for (int p = 0; p < ax.nf; ++p) {
                const int Rr = ax.fac[p];
                switch (Rr) {
                    case 8: slice_pass<C2, 8>(NJ, c0, c1, d0, d1, ax, tw, V, ncomp, Ns, S); break;
                    case 4: slice_pass<C2, 4>(NJ, c0, c1, d0, d1, ax, tw, V, ncomp, Ns, S); break;
                    case 2: slice_pass<C2, 2>(NJ, c0, c1, d0, d1, ax, tw, V, ncomp, Ns, S); break;
                    case 3: slice_pass<C2, 3>(NJ, c0, c1, d0, d1, ax, tw, V, ncomp, Ns, S); break;
                    default: slice_pass<C2, 5>(NJ, c0, c1, d0, d1, ax, tw, V, ncomp, Ns, S); break;
                }
                __syncthreads();
                // the result becomes the next source; the other work buffer the next target
                C2 *n0 = (d0 == wa0) ? wb0 : wa0;
                C2 *n1 = (d1 == wa1) ? wb1 : wa1;
                c0 = d0; c1 = d1;
                d0 = n0; d1 = n1;
                Ns *= Rr;
            }
            if (dir == 0) {
                // real filter along this axis (with the component constant on the first axis)
                const R *f = filt_of<R>(ax);
                const int n = ax.n, inner = ax.inner;
                const bool wc = first_axis && kinetic == CLV_KIN_EXP;
                for (int e = threadIdx.x; e < NJ * ncomp * V; e += blockDim.x) {
                    const int job = e >= ncomp * V;
                    const int r = e - job * ncomp * V;
                    const int c = r / V, sidx = r - c * V;
                    R m = f[(sidx / inner) % n];
                    if (wc) m *= (R)ch.comp_const[c];
                    C2 *buf = const_cast<C2 *>(job ? c1 : c0);
                    buf[r] = cscale(m, buf[r]);
                }
                __syncthreads();
            }
        }
        first_axis = false;
        (void)e0; (void)e1;
    }
    *out0 = const_cast<C2 *>(c0);
    if (out1) *out1 = const_cast<C2 *>(c1);
}

// -------------------------------------------------------------- the kernel
template <class R, int MODEL>
__global__ void __launch_bounds__(256)
fused_step_kernel(const LaunchFused A) {
    using C2 = typename Cx<R>::T;
    constexpr int NC = MODEL == CLV_MODEL_REF4 ? 4 : 3;
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ int abort_cta;
    const FusedTask task = A.tasks[blockIdx.x];
    const ChainDev &ch = A.chains[task.chain];
    ChainState *st = A.state + task.chain;
    if (A.mode == FUSED_APPLY && A.only_rejected && st->accepted) return;  // uniform per CTA

    const int V = ch.V, T = ch.nt, SL = NC * V;
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem);  // 7 barriers: psi slots 0-3, psibar 4-6
    C2 *slots = reinterpret_cast<C2 *>(smem + 128);
    auto slot = [&](int i) { return slots + (size_t)i * A.slot_stride; };
    const C2 *gpsi = reinterpret_cast<const C2 *>(A.psi_in) + ch.off;
    const C2 *gpsic = reinterpret_cast<const C2 *>(A.psic_in) + ch.off;
    C2 *opsi = reinterpret_cast<C2 *>(A.psi_out) + ch.off;
    C2 *opsic = reinterpret_cast<C2 *>(A.psic_out) + ch.off;
    const bool tma = A.use_tma != 0;
    const bool writes = A.mode != FUSED_MAXONLY;

    // step size and noise step of this launch
    R dt = 0;
    uint64_t nstep = 0;
    if (A.mode == FUSED_SPEC) { dt = (R)ch.dt_max; nstep = st->step; }
    else if (A.mode == FUSED_APPLY) { dt = (R)st->dt; nstep = st->noise_step; }
    const R sd = (R)sqrt((double)dt);

    if (threadIdx.x == 0) {
        abort_cta = 0;
        for (int i = 0; i < 7; ++i) mbar_init(&bars[i], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    uint32_t phase = 0, pending = 0;  // per-barrier phase bits and outstanding loads
    auto issue = [&](int sl, const C2 *g, int tau) {
        const int t = ((tau % T) + T) % T;
        if (tma) {
            if (threadIdx.x == 0) {
                mbar_expect_tx(&bars[sl], (uint32_t)(SL * sizeof(C2)));
                for (int c = 0; c < NC; ++c)
                    tma_load_1d(slot(sl) + c * V, g + ((long long)c * T + t) * V,
                                (uint32_t)(V * sizeof(C2)), &bars[sl]);
            }
            pending |= 1u << sl;
        } else {
            C2 *d = slot(sl);
            for (int e = threadIdx.x; e < SL; e += blockDim.x) {
                const int c = e / V, s = e - c * V;
                d[e] = g[((long long)c * T + t) * V + s];
            }
        }
    };
    auto wait_slot = [&](int sl) {
        if (!(pending & (1u << sl))) return;
        if (!mbar_wait(&bars[sl], (phase >> sl) & 1u)) {
            // give the copy a second bounded chance to land before the CTA stops using smem
            mbar_wait(&bars[sl], (phase >> sl) & 1u);
            if (threadIdx.x == 0) {
                atomicOr(&st->flags, CLV_FLAG_TIMEOUT);
                abort_cta = 1;
            }
        }
        phase ^= 1u << sl;
        pending &= ~(1u << sl);
    };

    // slot roles: psi(tau-1), psi(tau), psi(tau+1), free psi; psibar(tau), psibar(tau+1), free psibar;
    // kinetic pool 7..11: ka = kin(tau-1), four work buffers
    int pm = 0, pc = 1, pp = 2, pf = 3, qc = 4, qp = 5, qf = 6;
    int pool[5] = {7, 8, 9, 10, 11};
    const int tau0 = task.tau0, tau1 = task.tau1;
    issue(pm, gpsi, tau0 - 1);
    issue(pc, gpsi, tau0);
    issue(pp, gpsi, tau0 + 1);
    issue(qc, gpsic, tau0);
    issue(qp, gpsic, tau0 + 1);
    wait_slot(pm);
    __syncthreads();
    C2 *ka;
    slice_filter<R>(ch, NC, A.kinetic, 1, slot(pm), nullptr, slot(pool[1]), slot(pool[2]), nullptr,
                    nullptr, &ka, nullptr);
    // keep ka's buffer out of the work set: pool[0] = ka
    {
        int ki = (ka == slot(pool[1])) ? 1 : 2;
        int t = pool[0]; pool[0] = pool[ki]; pool[ki] = t;
    }

    double mx = 0.0, sm = 0.0;
    int bad = 0;
    for (int tau = tau0; tau < tau1; ++tau) {
        if (tau + 2 <= tau1) {
            issue(pf, gpsi, tau + 2);
            issue(qf, gpsic, tau + 2);
        }
        wait_slot(pc);
        wait_slot(pp);
        wait_slot(qc);
        wait_slot(qp);
        __syncthreads();
        if (abort_cta) break;
        C2 *kb, *kq;
        slice_filter<R>(ch, NC, A.kinetic, 2, slot(pc), slot(qp), slot(pool[1]), slot(pool[2]),
                        slot(pool[3]), slot(pool[4]), &kb, &kq);
        const C2 *Spm = slot(pm), *Spc = slot(pc), *Spp = slot(pp), *Sqc = slot(qc), *Sqp = slot(qp);
        const C2 *Ska = slot(pool[0]);
        const int tauw = tau < T ? tau : tau - T;  // tau0 < T always; kept for clarity
        for (int s = threadIdx.x; s < V; s += blockDim.x) {
            C2 vpm[NC], vpc[NC], vpp[NC], vcc[NC], vcp[NC], vkm[NC], vkp[NC], K[NC], Kc[NC];
#pragma unroll
            for (int a = 0; a < NC; ++a) {
                vpm[a] = Spm[a * V + s];
                vpc[a] = Spc[a * V + s];
                vcc[a] = Sqc[a * V + s];
                vcp[a] = Sqp[a * V + s];
                vkm[a] = Ska[a * V + s];
                vkp[a] = kq[a * V + s];
                if (MODEL == CLV_MODEL_REF4) vpp[a] = Spp[a * V + s];
            }
            if (MODEL == CLV_MODEL_REF4)
                drift_ref4_vals<R>(ch, vpm, vpc, vpp, vcc, vcp, vkm, vkp, K, Kc);
            else
                drift_spin1_vals<R>(ch, vpm, vpc, vcc, vcp, vkm, vkp, K, Kc);
            if (A.mode != FUSED_APPLY) {
                if (A.dt_rule == CLV_DT_REF_MEANMAX) {
                    const double a0 = (double)hypot(K[0].x, K[0].y);
                    mx = fmax(mx, a0);
                    sm += a0;
                    bad |= !isfinite(a0);
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
            if (writes) {
                const uint32_t site = (uint32_t)(tauw * V + s);
#pragma unroll
                for (int a = 0; a < NC; a += 2) {
                    C2 z[2];
                    if (A.noise == CLV_NOISE_PHILOX) {
                        const uint4 o = philox_block(ch.seed, (uint32_t)task.chain, nstep, a >> 1, site);
                        if (sizeof(R) == 8) {
                            const double2 g0 = box_muller64(o.x, o.y), g1 = box_muller64(o.z, o.w);
                            z[0].x = (R)g0.x; z[0].y = (R)g0.y; z[1].x = (R)g1.x; z[1].y = (R)g1.y;
                        } else {
                            const float2 g0 = box_muller32(o.x, o.y), g1 = box_muller32(o.z, o.w);
                            z[0].x = (R)g0.x; z[0].y = (R)g0.y; z[1].x = (R)g1.x; z[1].y = (R)g1.y;
                        }
                    } else {
#pragma unroll
                        for (int u = 0; u < 2; ++u) {
                            const int c = a + u < NC ? a + u : a;
                            const long long r = ch.noise_off + (((long long)c * V + s) * T + tauw) * 2;
                            z[u].x = (R)A.noise_buf[r];
                            z[u].y = (R)A.noise_buf[r + 1];
                        }
                    }
#pragma unroll
                    for (int u = 0; u < 2; ++u) {
                        const int c = a + u;
                        if (c >= NC) break;
                        C2 zz;
                        zz.x = mul_rn<R>(sd, z[u].x);
                        zz.y = mul_rn<R>(sd, z[u].y);
                        const long long gi = ((long long)c * T + tauw) * V + s;
                        opsi[gi] = langevin_update<R>(vpc[c], K[c], dt, zz, false);
                        opsic[gi] = langevin_update<R>(vcc[c], Kc[c], dt, zz, true);
                    }
                }
            }
        }
        __syncthreads();
        // rotate: psi(tau) becomes psi(tau-1), ...; kin(tau) becomes kin(tau-1)
        int t = pm; pm = pc; pc = pp; pp = pf; pf = t;
        t = qc; qc = qp; qp = qf; qf = t;
        const int kbi = kb == slot(pool[1]) ? 1 : (kb == slot(pool[2]) ? 2 : (kb == slot(pool[3]) ? 3 : 4));
        t = pool[0]; pool[0] = pool[kbi]; pool[kbi] = t;
    }
    // no copy may be in flight when the CTA exits
    for (int sl = 0; sl < 7; ++sl)
        if (pending & (1u << sl)) {
            mbar_wait(&bars[sl], (phase >> sl) & 1u);
            phase ^= 1u << sl;
        }
    bad |= abort_cta;
    if (A.mode == FUSED_APPLY) return;

    // chain-wide reduction: partial per CTA, the last CTA of the chain finishes the step
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

template <class R>
static cudaError_t fused_dispatch(const LaunchFused &L, cudaStream_t s) {
    if (L.model == CLV_MODEL_REF4)
        fused_step_kernel<R, CLV_MODEL_REF4><<<L.ntasks, 256, L.smem_bytes, s>>>(L);
    else
        fused_step_kernel<R, CLV_MODEL_SPIN1><<<L.ntasks, 256, L.smem_bytes, s>>>(L);
    return cudaGetLastError();
}

template <class R>
cudaError_t launch_fused(const LaunchFused &L, cudaStream_t s) {
    if (L.ntasks == 0) return cudaSuccess;
    return fused_dispatch<R>(L, s);
}

// Allow the device's whole opt-in shared memory for both models, then report
// how many CTAs of L.smem_bytes fit on one SM.
template <class R>
cudaError_t setup_fused(const LaunchFused &L, int *ctas_per_sm) {
    int dev = 0, optin = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    // the dynamic limit excludes the kernel's static shared memory
    cudaFuncAttributes fa4{}, fa3{};
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa4, fused_step_kernel<R, CLV_MODEL_REF4>);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa3, fused_step_kernel<R, CLV_MODEL_SPIN1>);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(fused_step_kernel<R, CLV_MODEL_REF4>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 optin - (int)fa4.sharedSizeBytes);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(fused_step_kernel<R, CLV_MODEL_SPIN1>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 optin - (int)fa3.sharedSizeBytes);
    if (e != cudaSuccess) return e;
    if (L.model == CLV_MODEL_REF4)
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            ctas_per_sm, fused_step_kernel<R, CLV_MODEL_REF4>, 256, L.smem_bytes);
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        ctas_per_sm, fused_step_kernel<R, CLV_MODEL_SPIN1>, 256, L.smem_bytes);
}

template cudaError_t launch_fused<double>(const LaunchFused &, cudaStream_t);
template cudaError_t launch_fused<float>(const LaunchFused &, cudaStream_t);
template cudaError_t setup_fused<double>(const LaunchFused &, int *);
template cudaError_t setup_fused<float>(const LaunchFused &, int *);

}  // namespace clv
