// k_obs.cu -- observables accumulated on the device in FP64.
//
// Reference observables (Observables::evaluate, Observables_without_cutoff.cu:1155-1382):
//   F_x, F_y, F_z real-space profiles summed over tau (kernel
//   evaluate_spin_density_realspace, :456-488) and n_tot, n_11..n_22 (kernels
//   :35-101 evaluated on FFT'd fields and reduced with thrust).  The particle
//   numbers are computed in real space here: with the reference's transform
//   directions, sum_k psibar~(k) psi~(k) = V sum_x psibar(x) psi(x) (Parseval),
//   so no FFT and no host round trip is needed.  One thread per spatial site
//   loops over tau, so the profiles need no atomics; the number sums are
//   block-reduced and added with one atomic per CTA.
// Spin-1 observables: density, F_z, F^2 = Fz^2 + F+F- and energy
//   psibar (k^2/2 - q m^2) psi + c0/2 n^2 + c1/2 F^2, all with the point split
//   (psibar(tau+1), psi(tau)); one FP64 sample per evaluate call and chain,
//   reduced without atomics on the sums.
#include "clv_internal.cuh"
#include "clv_launch.h"

namespace clv {

__device__ __forceinline__ long long oidx(const ChainDev &ch, int c, int tau, int s) {
    return ch.off + ((long long)c * ch.nt + tau) * ch.V + s;
}

__device__ __forceinline__ double block_sum(double v, double *sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    double r = 0.0;
    if (warp == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        r = lane < nw ? sh[lane] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
    }
    return r;  // valid in thread 0
}

// tasks: one CTA per 256 spatial sites of one chain (site0 = s0).
template <class R>
__global__ void __launch_bounds__(256)
obs_ref_kernel(const ChainDev *__restrict__ chains, const SiteTask *__restrict__ tasks,
               const typename Cx<R>::T *__restrict__ psi, const typename Cx<R>::T *__restrict__ psic,
               double *__restrict__ accF, double *__restrict__ accN) {
    __shared__ double sh[32];
    const SiteTask task = tasks[blockIdx.x];
    const ChainDev &ch = chains[task.chain];
    const int s = task.site0 + threadIdx.x;
    double n[5] = {0, 0, 0, 0, 0};
    if (s < ch.V) {
        double fx = 0, fy = 0, fz = 0;
        for (int tau = 0; tau < ch.nt; ++tau) {
            const int tp = tau == ch.nt - 1 ? 0 : tau + 1;
            double2 pc[4], cp[4];
#pragma unroll
            for (int a = 0; a < 4; ++a) {
                const auto u = psi[oidx(ch, a, tau, s)];
                const auto v = psic[oidx(ch, a, tp, s)];
                pc[a] = make_double2(u.x, u.y);
                cp[a] = make_double2(v.x, v.y);
            }
            const double2 t20 = cmul(cp[2], pc[0]), t02 = cmul(cp[0], pc[2]);
            const double2 t31 = cmul(cp[3], pc[1]), t13 = cmul(cp[1], pc[3]);
            fx += cadd(cadd(cadd(t20, t02), t31), t13).x;
            // Re(i w) = -Im(w)
            fy += -csub(cadd(csub(t20, t02), t31), t13).y;
            fz += csub(csub(cadd(cmul(cp[0], pc[0]), cmul(cp[1], pc[1])), cmul(cp[2], pc[2])),
                       cmul(cp[3], pc[3])).x;
#pragma unroll
            for (int a = 0; a < 4; ++a) {
                const double d = cmul(cp[a], pc[a]).x * ch.a_x;
                n[0] += d;
                n[1 + a] += d;
            }
        }
        double *F = accF + ch.obs_off;
        F[s] += fx;
        F[ch.V + s] += fy;
        F[2 * ch.V + s] += fz;
    }
#pragma unroll
    for (int i = 0; i < 5; ++i) {
        const double r = block_sum(n[i], sh);
        if (threadIdx.x == 0) atomicAdd(&accN[task.chain * 5 + i], r * (double)ch.V);
    }
}

template <class R>
cudaError_t launch_obs_ref(const LaunchSites &L, double *accF, double *accN, cudaStream_t s) {
    using C2 = typename Cx<R>::T;
    obs_ref_kernel<R><<<L.ntasks, 256, 0, s>>>(L.chains, L.tasks, (const C2 *)L.psi,
                                               (const C2 *)L.psic, accF, accN);
    return cudaGetLastError();
}

// A CTA takes 256 spatial sites of one chain over imaginary times [tau0, tau1)
// (ObsTask); tpsi = (k^2/2) psi from the kinetic-energy filter.  Per-site
// products in the working precision R, summed per thread over the CTA's tau
// range, then in FP64 across the CTA (one partial of the 8 sums per CTA); the
// chain's last CTA adds its partials in CTA order (no atomics on the sums, the
// same result for every run) and writes the sample.
template <class R>
__global__ void __launch_bounds__(256)
obs_spin1_kernel(const ChainDev *__restrict__ chains, const ObsTask *__restrict__ tasks,
                 const typename Cx<R>::T *__restrict__ psi, const typename Cx<R>::T *__restrict__ psic,
                 const typename Cx<R>::T *__restrict__ tpsi, double *__restrict__ partials,
                 unsigned int *__restrict__ arrive, double *__restrict__ samples, int slot, int nchains) {
    using C2 = typename Cx<R>::T;
    __shared__ double sh[8][8];
    __shared__ int am_last;
    const ObsTask task = tasks[blockIdx.x];
    const ChainDev &ch = chains[task.chain];
    const int s = task.site0 + threadIdx.x;
    R acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (s < ch.V) {
        const R r2 = (R)1.41421356237309504880, q = (R)ch.q, c0h = (R)(0.5 * ch.c0),
                c1h = (R)(0.5 * ch.c1);
        for (int tau = task.tau0; tau < task.tau1; ++tau) {
            const int tp = tau == ch.nt - 1 ? 0 : tau + 1;
            C2 bar[3], ket[3], tk[3];
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                bar[a] = psic[oidx(ch, a, tp, s)];
                ket[a] = psi[oidx(ch, a, tau, s)];
                tk[a] = tpsi[oidx(ch, a, tau, s)];
            }
            const C2 n = cadd(cadd(cmul(bar[0], ket[0]), cmul(bar[1], ket[1])), cmul(bar[2], ket[2]));
            const C2 Fz = csub(cmul(bar[0], ket[0]), cmul(bar[2], ket[2]));
            const C2 Fp = cscale(r2, cadd(cmul(bar[0], ket[1]), cmul(bar[1], ket[2])));
            const C2 Fm = cscale(r2, cadd(cmul(bar[1], ket[0]), cmul(bar[2], ket[1])));
            const C2 F2 = cadd(cmul(Fz, Fz), cmul(Fp, Fm));
            C2 e1 = cmul(bar[1], tk[1]);  // m = 0
            e1 = cadd(e1, cmul(bar[0], csub(tk[0], cscale(q, ket[0]))));
            e1 = cadd(e1, cmul(bar[2], csub(tk[2], cscale(q, ket[2]))));
            const C2 e = cadd(cadd(e1, cscale(c0h, cmul(n, n))), cscale(c1h, F2));
            acc[0] += n.x; acc[1] += n.y; acc[2] += Fz.x; acc[3] += Fz.y;
            acc[4] += F2.x; acc[5] += F2.y; acc[6] += e.x; acc[7] += e.y;
        }
    }
    // FP64 above the thread: warp shuffles, then the CTA's 8 warps in order
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        double v = (double)acc[i];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) sh[warp][i] = v;
    }
    __syncthreads();
    if (threadIdx.x < 8) {
        double v = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += sh[w][threadIdx.x];
        partials[(size_t)blockIdx.x * 8 + threadIdx.x] = v;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        am_last = atomicAdd(&arrive[task.chain], 1u) == (unsigned)ch.obs_nblocks - 1;
    }
    __syncthreads();
    if (!am_last) return;
    __threadfence();
    if (threadIdx.x < 8) {
        double v = 0.0;
        for (int b = 0; b < ch.obs_nblocks; ++b)
            v += __ldcg(&partials[(size_t)(ch.obs_block0 + b) * 8 + threadIdx.x]);
        samples[((size_t)slot * nchains + task.chain) * 8 + threadIdx.x] = v / ((double)ch.V * ch.nt);
    }
    if (threadIdx.x == 0) arrive[task.chain] = 0u;
}

template <class R>
cudaError_t launch_obs_spin1(const LaunchObs &L, cudaStream_t s) {
    using C2 = typename Cx<R>::T;
    if (L.ntasks == 0) return cudaSuccess;
    obs_spin1_kernel<R><<<L.ntasks, 256, 0, s>>>(L.chains, L.tasks, (const C2 *)L.psi, (const C2 *)L.psic,
                                                 (const C2 *)L.tpsi, L.partials, L.arrive, L.samples,
                                                 L.slot, L.nchains);
    return cudaGetLastError();
}

template cudaError_t launch_obs_ref<double>(const LaunchSites &, double *, double *, cudaStream_t);
template cudaError_t launch_obs_ref<float>(const LaunchSites &, double *, double *, cudaStream_t);
template cudaError_t launch_obs_spin1<double>(const LaunchObs &, cudaStream_t);
template cudaError_t launch_obs_spin1<float>(const LaunchObs &, cudaStream_t);

}  // namespace clv
