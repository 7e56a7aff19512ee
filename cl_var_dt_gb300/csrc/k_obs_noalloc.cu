// k_obs_noalloc.cu -- reference observables of one field configuration,
// computed without allocating anything (clv_ref_observables_noalloc).
//
// Who needs it: callers that may not call cudaMalloc or any allocating routine
// at the point where they measure -- code running while a CUDA stream is being
// captured into a graph (an allocation there would invalidate the capture),
// code under a memory pool or budget that forbids new device allocations, and
// hosts that want a measurement without creating a clv_engine (whose set-up
// allocates).  Such a caller passes device buffers it already owns.
//
// Same arithmetic as obs_ref_kernel (Observables_without_cutoff.cu:35-101 and
// :456-488 via Observables::evaluate, :1155-1382): the F_x, F_y, F_z profiles
// summed over tau and the particle numbers n_tot, n_11, n_12, n_21, n_22 in
// real space.  The cross-CTA sum of the particle numbers needs scratch: one
// partial per CTA and observable plus an arrival counter.  The engine keeps
// such accumulators in memory it allocated; here they live in the file-scope
// device array g_noalloc_scratch below, of fixed size, so nothing is
// allocated.  The last CTA to arrive sums the partials in CTA order (the result
// does not depend on scheduling) and resets the counter.
#include <mutex>
#include <string>

#include "clv.h"
#include "clv_internal.cuh"

namespace clv {
int record_failure(int code, const std::string &msg);
}

using namespace clv;

namespace {

constexpr int kNoallocBlock = 256;
// Largest lattice (sites per time slice, V = nx*ny*nz) one call accepts: one
// CTA per 256 sites, one 5-double partial per CTA.
constexpr int kNoallocMaxBlocks = 4096;
constexpr long long kNoallocMaxSites = (long long)kNoallocMaxBlocks * kNoallocBlock;  // 1,048,576
// Layout of the scratch array: [0, 256) arrival counter (unsigned int),
// [256, 256 + 5*8*kNoallocMaxBlocks) partials part[i * kNoallocMaxBlocks + b].
constexpr size_t kScratchHeader = 256;
constexpr size_t kScratchBytes = kScratchHeader + sizeof(double) * 5 * kNoallocMaxBlocks;  // 164,096 B

// Shared by every call on a device; it keeps the contents of the last call.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
void *g_scratch_ptr[kMaxDevices] = {};

__device__ __forceinline__ double noalloc_block_sum(double v, double *sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    double r = 0.0;
    if (warp == 0) {
        r = lane < (kNoallocBlock >> 5) ? sh[lane] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
    }
    return r;  // valid in thread 0
}

__global__ void __launch_bounds__(kNoallocBlock)
obs_ref_noalloc_kernel(const double2 *__restrict__ psi, const double2 *__restrict__ psic, int V,
                       int nt, double a_x, double *__restrict__ F, double *__restrict__ n_out,
                       unsigned char *__restrict__ scratch) {
    __shared__ double sh[32];
    __shared__ bool last;
    unsigned int *arrive = reinterpret_cast<unsigned int *>(scratch);
    double *part = reinterpret_cast<double *>(scratch + kScratchHeader);
    const int s = blockIdx.x * kNoallocBlock + threadIdx.x;
    double n[5] = {0, 0, 0, 0, 0};
    if (s < V) {
        double fx = 0, fy = 0, fz = 0;
        for (int tau = 0; tau < nt; ++tau) {
            const int tp = tau == nt - 1 ? 0 : tau + 1;
            double2 pc[4], cp[4];
#pragma unroll
            for (int a = 0; a < 4; ++a) {
                pc[a] = psi[((long long)a * nt + tau) * V + s];
                cp[a] = psic[((long long)a * nt + tp) * V + s];
            }
            const double2 t20 = cmul(cp[2], pc[0]), t02 = cmul(cp[0], pc[2]);
            const double2 t31 = cmul(cp[3], pc[1]), t13 = cmul(cp[1], pc[3]);
            fx += cadd(cadd(cadd(t20, t02), t31), t13).x;
            fy += -csub(cadd(csub(t20, t02), t31), t13).y;  // Re(i w) = -Im(w)
            fz += csub(csub(cadd(cmul(cp[0], pc[0]), cmul(cp[1], pc[1])), cmul(cp[2], pc[2])),
                       cmul(cp[3], pc[3])).x;
#pragma unroll
            for (int a = 0; a < 4; ++a) {
                const double d = cmul(cp[a], pc[a]).x * a_x;
                n[0] += d;
                n[1 + a] += d;
            }
        }
        // Observables::write_F_* (:1614-1634) divides the tau sum by T.
        F[s] = fx / nt;
        F[V + s] = fy / nt;
        F[2 * V + s] = fz / nt;
    }
#pragma unroll
    for (int i = 0; i < 5; ++i) {
        const double r = noalloc_block_sum(n[i], sh);
        if (threadIdx.x == 0) part[i * kNoallocMaxBlocks + blockIdx.x] = r;
    }
    if (threadIdx.x == 0) {
        __threadfence();
        last = atomicAdd(arrive, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    // Fixed-order sum over the CTAs: thread t takes CTAs t, t+256, ... in order,
    // then the block tree; the same for every run.
    for (int i = 0; i < 5; ++i) {
        double v = 0.0;
        for (int b = threadIdx.x; b < (int)gridDim.x; b += kNoallocBlock)
            v += __ldcg(&part[i * kNoallocMaxBlocks + b]);
        const double r = noalloc_block_sum(v, sh);
        // Observables::write_n_* (:1527-1547): (sum * V) / T / V for one evaluate.
        if (threadIdx.x == 0) n_out[i] = r * (double)V / nt / (double)V;
    }
    if (threadIdx.x == 0) *arrive = 0u;
}

// Address of this device's scratch array, looked up once per device.
int scratch_for_current_device(unsigned char **out, int *device) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return record_failure(CLV_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices)
        return record_failure(CLV_ERR_ARG, "device ordinal " + std::to_string(dev) + " above 63");
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_ptr[dev]) {
        void *ptr = nullptr;
        e = cudaGetSymbolAddress((void **)&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || !ptr)
            return record_failure(CLV_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") +
                                                    cudaGetErrorString(e));
        g_scratch_ptr[dev] = ptr;
    }
    *out = static_cast<unsigned char *>(g_scratch_ptr[dev]);
    *device = dev;
    return CLV_OK;
}

}  // namespace

extern "C" int clv_ref_observables_noalloc(const void *psi, const void *psic, int nx, int ny,
                                           int nz, int nt, double a_x, double *n, double *F,
                                           void *stream) {
    if (!psi || !psic || !n || !F) return record_failure(CLV_ERR_ARG, "null buffer");
    if (nx < 1 || ny < 1 || nz < 1 || nt < 1) return record_failure(CLV_ERR_ARG, "lattice extent below 1");
    const long long V = (long long)nx * ny * nz;
    if (V > kNoallocMaxSites)
        return record_failure(CLV_ERR_ARG,
                              "clv_ref_observables_noalloc: nx*ny*nz = " + std::to_string(V) +
                                  " sites exceeds its maximum of " +
                                  std::to_string(kNoallocMaxSites) +
                                  " (fixed scratch of " + std::to_string(kNoallocMaxBlocks) +
                                  " partials); use clv_evaluate on an engine instead");
    if (((uintptr_t)psi | (uintptr_t)psic) & 15)
        return record_failure(CLV_ERR_ARG, "psi and psic must be 16-byte aligned");
    unsigned char *scratch = nullptr;
    int dev = 0;
    int rc = scratch_for_current_device(&scratch, &dev);
    if (rc) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // The counter must start at zero; a call that failed part-way could have
    // left it set.  The partials need no clearing: each CTA writes its own
    // before the counter lets the last CTA read them.
    cudaError_t e = cudaMemsetAsync(scratch, 0, sizeof(unsigned int), st);
    if (e != cudaSuccess)
        return record_failure(CLV_ERR_CUDA, std::string("cudaMemsetAsync(counter): ") + cudaGetErrorString(e));
    const int blocks = (int)((V + kNoallocBlock - 1) / kNoallocBlock);
    obs_ref_noalloc_kernel<<<blocks, kNoallocBlock, 0, st>>>(
        static_cast<const double2 *>(psi), static_cast<const double2 *>(psic), (int)V, nt, a_x, F, n,
        scratch);
    e = cudaGetLastError();
    if (e != cudaSuccess)
        return record_failure(CLV_ERR_CUDA, std::string("obs_ref_noalloc_kernel: ") + cudaGetErrorString(e));
    return CLV_OK;
}
