// k_loop.cu -- many Langevin steps of a small problem in one cooperative launch,
// under the reference's step rule or the K/max rule (exact there without
// speculation: dt is known before any update).
//
// On the reference's own lattices (one chain of 256 x 32: 128 CTAs of one
// imaginary time each) a step of the two-kernel form -- the filter/drift/reduce
// pass, then the update with its noise -- costs more in launches, in the drift's
// round trip and in the update's wait for the reduce pass than in arithmetic.
// Here every CTA keeps its task (one imaginary time, one field, the components
// of FusedTask::cmask) for all steps of the launch and, per step,
//   1. reads the slices it needs from the current buffer set (L2-resident),
//   2. filters its lines (the fused kernel's line filters), while its idle warps
//      draw its half of the unit normals of its (imaginary time, components) and
//      store them for the partner CTA of the other field,
//   3. computes the drift of its sites and its step-rule partial,
//   -- grid barrier --
//   4. derives dt from the chain's partials (every CTA, in the order of the fused
//      kernel's last CTA; the chain's first CTA also advances ChainState),
//   5. updates its sites with dt K + sqrt(dt) xi into the other buffer set,
//   -- grid barrier --
// The results are those of the two-kernel form bit for bit: the same filters,
// drift, reduction order, noise stream (Philox block per component pair, the
// update kernel's words) and update rounding.  The grid barrier is a counter in
// global memory; every wait is bounded (0.5 s), after which the CTA raises
// CLV_FLAG_TIMEOUT and an abort flag that makes every CTA leave at its next
// barrier.  A cooperative launch guarantees that all CTAs are resident.
#include "fused_impl.cuh"

namespace clv {

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ int ld_volatile_i32(const int *p) {
    return *reinterpret_cast<const volatile int *>(p);
}

// Grid barrier number `gen` (1, 2, ...): true when every CTA has arrived.
__device__ __forceinline__ bool loop_grid_sync(const LaunchLoop &A, unsigned gen, ChainState *st) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int good = 1;
        if (A.withhold && blockIdx.x == 0 && gen == 1) {
            // test hook: this CTA leaves without arriving, so the others' waits run out
            atomicOr(&st->flags, CLV_FLAG_TIMEOUT);
            good = 0;
        } else {
            __threadfence();
            atomicAdd(A.bar, 1u);
            const unsigned target = gen * gridDim.x;
            const uint64_t t0 = globaltimer_ns();
            for (int i = 0;; ++i) {
                if (ld_acquire_u32(A.bar) >= target) break;
                if (ld_volatile_i32(A.abort) || i >= (1 << 26) ||
                    ((i & 63) == 63 && globaltimer_ns() - t0 > 500000000ull)) {
                    good = 0;
                    break;
                }
            }
            if (!good) {
                atomicExch(A.abort, 1);
                atomicOr(&st->flags, CLV_FLAG_TIMEOUT);
            }
        }
        __threadfence();
        ok = good;
    }
    __syncthreads();
    return ok != 0;
}

template <class R, int MODEL, int LN>
__global__ void __launch_bounds__(256, 1) loop_step_kernel(const LaunchLoop A) {
    using C2 = typename Cx<R>::T;
    constexpr int NC = MODEL == CLV_MODEL_REF4 ? 4 : 3;
    constexpr int CS = padded_line(LN);
    constexpr int SLOT = fused_slot_stride(NC, LN, (int)sizeof(C2));
    constexpr bool kPairLines = sizeof(R) == 8 && LN == 256;  // as the fused kernel (non-production)
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ double s_dt;

    const FusedTask task = A.tasks[blockIdx.x];
    const ChainDev &ch = A.chains[task.chain];
    ChainState *st = A.state + task.chain;
    const int side = task.side;  // 1: psi, 2: psibar (the loop needs split tasks)
    const bool do_psi = side == 1, do_bar = side == 2;
    const int cmask = task.cmask ? task.cmask : (1 << NC) - 1;
    auto own = [&](int c) { return ((cmask >> c) & 1) != 0; };
    const int tau = task.tau0, T = ch.nt, TV = T * LN;
    const int tm = tau == 0 ? T - 1 : tau - 1, tp = tau == T - 1 ? 0 : tau + 1;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, s = threadIdx.x;
    const bool leader = task.part == 0;  // advances the chain's ChainState

    C2 *twS = reinterpret_cast<C2 *>(smem + 64);
    R *fS = reinterpret_cast<R *>(smem + 64 + LN * sizeof(C2));
    C2 *twT = reinterpret_cast<C2 *>(smem + fused_ptw_offset(LN, (int)sizeof(C2)));
    C2 *slots = reinterpret_cast<C2 *>(smem + fused_tab_bytes(LN, (int)sizeof(C2), LN));
    C2 *sPm = slots, *sPc = slots + SLOT, *sPp = slots + 2 * SLOT, *sQc = slots + 3 * SLOT,
       *sQp = slots + 4 * SLOT, *sX = slots + 5 * SLOT, *sY = slots + 6 * SLOT;
    {
        const AxisDev &ax = ch.axis[0];
        const C2 *tw = tw_of<R>(ax), *pt = ptw_of<R>(ax);
        const R *f = filt_of<R>(ax);
        for (int i = threadIdx.x; i < LN; i += blockDim.x) {
            twS[i] = tw[i];
            fS[i] = f[i];
        }
        for (int i = threadIdx.x; i < tw_entries(LN); i += blockDim.x) twT[i] = pt[i];
    }
    const bool wc = A.kinetic == CLV_KIN_EXP;
    const DriftConsts<R> dk(ch);
    const uint64_t seed = ch.seed, nstep0 = __ldcg(&st->step);
    C2 *nz = reinterpret_cast<C2 *>(A.noise) + ch.off;

    // lines of this CTA (bit job * NC + c) and the warps that filter them; the others
    // draw the CTA's half of the unit normals meanwhile
    const int own_lines = cmask & ((1 << NC) - 1);
    const int mask = do_psi ? own_lines : own_lines << NC;
    const int nl = __popc(mask);
    const bool pair = kPairLines && 2 * nl <= 8;
    const int used = pair ? (1 << (2 * nl)) - 1 : (mask & 0xFF);
    const int idle = ~used & 0xFF;
    const bool noise_warp = (idle >> warp) & 1;
    const int nthr = __popc(idle) * 32, tn = __popc(idle & ((1 << warp) - 1)) * 32 + lane;
    const int n0 = do_psi ? 0 : LN / 2, n1 = do_psi ? LN / 2 : LN;

    auto draw = [&](int x, uint64_t nstep) {
        const uint32_t site = (uint32_t)(tau * LN + x);
#pragma unroll
        for (int p = 0; p < (NC + 1) / 2; ++p) {
            if (!((cmask >> (2 * p)) & 3)) continue;
            const bool lone = lone_component(2 * p, NC);  // (noise_words)
            const uint4 o = philox_block(seed, (uint32_t)task.chain, nstep, p, lone ? site >> 1 : site);
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const int c = 2 * p + u;
                if (c >= NC || !own(c)) continue;
                const bool hi = lone ? (site & 1) != 0 : u != 0;
                const uint32_t wx = hi ? o.z : o.x, wy = hi ? o.w : o.y;
                C2 z;
                if constexpr (sizeof(R) == 8) {
                    const double2 g = box_muller64(wx, wy);
                    z.x = (R)g.x; z.y = (R)g.y;
                } else {
                    const float2 g = box_muller32(wx, wy);
                    z.x = (R)g.x; z.y = (R)g.y;
                }
                nz[(c * T + tau) * LN + x] = z;
            }
        }
    };

    int buf = A.from;
    unsigned gen = 0;
    for (int k = 0; k < A.nsteps; ++k) {
        const uint64_t nstep = nstep0 + (uint64_t)k;
        const C2 *psi = reinterpret_cast<const C2 *>(A.fld[buf][0]) + ch.off;
        const C2 *psic = reinterpret_cast<const C2 *>(A.fld[buf][1]) + ch.off;
        C2 *opsi = reinterpret_cast<C2 *>(A.fld[buf ^ 1][0]) + ch.off;
        C2 *opsic = reinterpret_cast<C2 *>(A.fld[buf ^ 1][1]) + ch.off;
        // 1. slices (L2: other CTAs wrote them in the previous step)
        for (int e = threadIdx.x; e < NC * LN; e += blockDim.x) {
            const int c = e / LN, x = e - c * LN, o = c * CS + x;
            const long long b = (long long)c * TV + x;
            sPc[o] = __ldcg(&psi[b + tau * LN]);
            sQc[o] = __ldcg(&psic[b + tau * LN]);
            sQp[o] = __ldcg(&psic[b + tp * LN]);
            if (do_psi) sPm[o] = __ldcg(&psi[b + tm * LN]);
            if (MODEL == CLV_MODEL_REF4 && do_bar) sPp[o] = __ldcg(&psi[b + tp * LN]);
        }
        __syncthreads();
        // 2. kinetic term of the filtered field (psi side: kin(tau-1); psibar side:
        //    kinbar(tau+1)) into sX; unit normals by the idle warps
        {
            const C2 *src = do_psi ? sPm : sQp;
            if (pair) {
                const int g = warp >> 1;
                if (g < nl) {
                    int m = mask;
                    for (int i = 0; i < g; ++i) m &= m - 1;
                    const int bit = __ffs(m) - 1, c = bit - (bit >= NC ? NC : 0);
                    const R cst = wc ? (R)ch.comp_const[c] : (R)1;
                    if constexpr (kPairLines)
                        group_line_filter4<C2, R, LN, 64>(src + c * CS, sX + c * CS, sY + c * CS, twS, fS, cst,
                                                          threadIdx.x & 63, 1 + g);
                }
            } else if ((mask >> warp) & 1) {
                const int c = warp - (warp >= NC ? NC : 0);
                const R cst = wc ? (R)ch.comp_const[c] : (R)1;
                warp_line_filter_ct<C2, R, LN, true>(src + c * CS, sX + c * CS, sY + c * CS, twT, fS, cst, lane);
            }
            if (noise_warp)
                for (int x = n0 + tn; x < n1; x += nthr) draw(x, nstep);
        }
        if (nthr == 0)
            for (int x = n0 + threadIdx.x; x < n1; x += blockDim.x) draw(x, nstep);
        __syncthreads();
        // 3. drift of site s and the step-rule partial (the fused kernel's REF-rule code)
        C2 K[NC], Kc[NC], pc[NC], qc[NC];
        R mxr = 0, smr = 0;
        int bad = 0;
        if (s < LN) {
            C2 pm[NC], pp[NC], cp[NC], km[NC], kp[NC];
#pragma unroll
            for (int c = 0; c < NC; ++c) {
                K[c] = Kc[c] = mk<C2>(0.0, 0.0);
                pc[c] = sPc[c * CS + s];
                qc[c] = sQc[c * CS + s];
                cp[c] = sQp[c * CS + s];
                pm[c] = do_psi ? sPm[c * CS + s] : mk<C2>(0.0, 0.0);
                pp[c] = (MODEL == CLV_MODEL_REF4 && do_bar) ? sPp[c * CS + s] : mk<C2>(0.0, 0.0);
                km[c] = do_psi ? sX[c * CS + s] : mk<C2>(0.0, 0.0);
                kp[c] = do_bar ? sX[c * CS + s] : mk<C2>(0.0, 0.0);
            }
            if (MODEL == CLV_MODEL_REF4)
                drift_ref4_vals<R>(dk, pm, pc, pp, qc, cp, km, kp, K, Kc, do_psi ? 1 : 2, cmask);
            else
                drift_spin1_vals<R>(dk, pm, pc, qc, cp, km, kp, K, Kc, do_psi ? 1 : 2);
            if (A.dt_rule == CLV_DT_REF_MEANMAX) {
                if (own(0)) {  // (a psibar CTA's K is zero)
                    const R a0 = hypot(K[0].x, K[0].y);
                    mxr = fmax(mxr, a0);
                    smr += a0;
                    bad |= !isfinite(a0);
                }
            } else {
                // K/max rule: max |K|^2 over this CTA's field and components (the chain's
                // maximum is the same whichever CTA finds it); FP64 carries a NaN in the sum
#pragma unroll
                for (int c = 0; c < NC; ++c) {
                    if (!own(c)) continue;
                    const R m = abs2<R>(do_psi ? K[c] : Kc[c]);
                    if constexpr (sizeof(R) == 4) {
                        mxr = max_nan(mxr, m);
                    } else {
                        mxr = fmax(mxr, m);
                        smr += m;
                    }
                }
            }
        }
        double mx = (double)mxr, sm = (double)smr;
        bad |= !isfinite(mx) || !isfinite(sm);
        bad = __syncthreads_or(bad);
        block_max_sum(mx, sm);
        if (threadIdx.x == 0)
            A.partials[ch.fused_block0 + task.part] =
                make_double2(mx, bad ? __longlong_as_double(0x7ff8000000000000ll) : sm);
        if (!loop_grid_sync(A, ++gen, st)) return;
        // 4. dt from the chain's partials, in the fused kernel's order
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
            if (leader) {
                const double dtn = step_rule(ch, *st, A.dt_rule, mx, sm, mean);
                if (bad || !isfinite(mx) || !isfinite(sm)) st->flags |= CLV_FLAG_NONFINITE;
                st->dt = dtn;
                st->max = mx;
                st->mean = mean;
                st->t += dtn;
                st->noise_step = nstep;
                st->step = nstep + 1;
                st->accepted = 0;
                s_dt = dtn;
            } else {
                ChainState scratch{};
                s_dt = step_rule(ch, scratch, A.dt_rule, mx, sm, mean);
            }
        }
        __syncthreads();
        // 5. update (the rounding of the stored-drift update at FP64 and of the fused
        //    apply pass at FP32, whose sqrt takes the step rounded to FP32)
        const R dt = (R)s_dt, sd = (R)sqrt((double)dt);
        if (s < LN) {
#pragma unroll
            for (int c = 0; c < NC; ++c) {
                if (!own(c)) continue;
                const long long gi = (long long)c * TV + tau * LN + s;
                C2 z = __ldcg(&nz[gi]);
                z.x = mul_rn<R>(sd, z.x);
                z.y = mul_rn<R>(sd, z.y);
                if (do_psi) opsi[gi] = langevin_update<R>(pc[c], K[c], dt, z, false);
                else opsic[gi] = langevin_update<R>(qc[c], Kc[c], dt, z, true);
            }
        }
        if (!loop_grid_sync(A, ++gen, st)) return;
        buf ^= 1;
    }
}

template <class R, int MODEL>
static void *loop_kernel_of(int ln) {
    switch (ln) {
        case 64: return (void *)loop_step_kernel<R, MODEL, 64>;
        case 128: return (void *)loop_step_kernel<R, MODEL, 128>;
        case 256: return (void *)loop_step_kernel<R, MODEL, 256>;
        default: return nullptr;
    }
}
template <class R>
static void *loop_kernel(int model, int ln) {
    return model == CLV_MODEL_REF4 ? loop_kernel_of<R, CLV_MODEL_REF4>(ln) : loop_kernel_of<R, CLV_MODEL_SPIN1>(ln);
}

size_t loop_smem_bytes(int model, int ln, int esz) {
    const int nc = model == CLV_MODEL_REF4 ? 4 : 3;
    return (size_t)fused_tab_bytes(ln, esz, ln) + 7 * (size_t)fused_slot_stride(nc, ln, esz) * esz;
}

template <class R>
cudaError_t setup_loop(int model, int ln, int *ctas_per_sm) {
    *ctas_per_sm = 0;
    void *fn = loop_kernel<R>(model, ln);
    if (!fn) return cudaSuccess;
    const size_t smem = loop_smem_bytes(model, ln, (int)sizeof(typename Cx<R>::T));
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas_per_sm, fn, 256, smem);
}

template <class R>
cudaError_t launch_loop(const LaunchLoop &L, cudaStream_t s) {
    void *fn = loop_kernel<R>(L.model, L.ln);
    if (!fn) return cudaErrorInvalidValue;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(L.ntasks);
    cfg.blockDim = dim3(256);
    cfg.dynamicSmemBytes = loop_smem_bytes(L.model, L.ln, (int)sizeof(typename Cx<R>::T));
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    void *args[] = {const_cast<LaunchLoop *>(&L)};
    return cudaLaunchKernelExC(&cfg, fn, args);
}

template cudaError_t setup_loop<double>(int, int, int *);
template cudaError_t setup_loop<float>(int, int, int *);
template cudaError_t launch_loop<double>(const LaunchLoop &, cudaStream_t);
template cudaError_t launch_loop<float>(const LaunchLoop &, cudaStream_t);

}  // namespace clv
