// ref_gpu_runner.cpp -- TEST INFRASTRUCTURE ONLY (the oracle's GPU pin and the
// reference's GPU timing).  Never linked by the product.
//
// Runs the reference's own CUDA kernels -- compiled unchanged from its sources
// into a cubin by oracle/ref_gpu_build.sh -- with the real cuFFT and cuRAND
// libraries, in the order of Propagator::propagate
// (Propagator_without_cutoff.cu:406-442), so the GPU engine can be compared per
// site with the reference's own GPU build on the same inputs, and the
// reference's step can be timed on the same GPU.
//
// The host side restates the reference's host methods (their device work is the
// reference's compiled kernels):
//   ComplexLattice: cufftPlanMany rank 1/2/3 over the spatial axes, batch C*T,
//     in place (Lattice.cu:135-156); fft/fft_inv direction by field
//     (Lattice.cu:158-180); normalize (Lattice.cu:182-187); operator+=
//     (Lattice.cu:197-202); operator= (Lattice.cu:211-214).  Launch geometry of
//     the 4-D kernels (Lattice.cu:108-125, Propagator_without_cutoff.cu:325-335).
//   Propagator: the constructor's cuRAND XORWOW generator seeded with `seed`
//     (Propagator_without_cutoff.cu:316-343); get_max_and_mean_drift with its
//     per-step cudaMalloc/cudaMemset/cudaMemcpy/cudaFree (:351-380);
//     compute_new_dt (:382-404); propagate (:406-442).
// The noise is either curandGenerateNormalDouble(gen, buf, 2CVT, 0, sqrt(dt))
// as in the reference, or injected: unit normals in the reference's ind_rand
// layout (Lattice.cu:7-11) scaled by sqrt(dt), for per-site parity.
//
// Kernels are looked up by name in the cubin (cuModuleEnumerateFunctions and
// the Itanium-mangled prefix _Z<len><name>), launched with cuLaunchKernel.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cufft.h>
#include <curand.h>

#include <cctype>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace {

enum {
    K_DRIFT, K_KINETIC, K_MUL_DT, K_ADD_NOISE, K_SUMMATION, K_NORMALIZATION, K_MAXMEAN, K_SET_VALUE,
    K_N_TOT, K_N_11, K_N_12, K_N_21, K_N_22, K_SPIN, K_COUNT
};
const char *const kNames[K_COUNT] = {
    "calculate_drift_without_noise", "compute_kinetic_part", "multiply_by_timestep", "add_noise",
    "summation", "normalization", "compute_max_and_mean_drift", "set_value",
    "evaluate_n_tot", "evaluate_n_11", "evaluate_n_12", "evaluate_n_21", "evaluate_n_22",
    "evaluate_spin_density_realspace"};

struct RefGpu {
    CUmodule mod = nullptr;
    CUfunction k[K_COUNT] = {};
    int X, Y, Z, T, C;
    int bs, bx, by, bz, bt;
    double eps, a_x, DT;
    long long n;  // C*V*T
    double2 *psi = nullptr, *psic = nullptr, *kin = nullptr, *kinc = nullptr, *drift = nullptr,
            *driftc = nullptr;
    double *rnd = nullptr;
    cufftHandle plan = 0;
    curandGenerator_t gen = nullptr;
    double dt, last_max = 0, last_mean = 0;
    char err[512] = {0};
};

thread_local char g_err[512];

int fail(RefGpu *h, const char *what, long long code) {
    std::snprintf(g_err, sizeof g_err, "%s failed (%lld)", what, code);
    if (h) std::snprintf(h->err, sizeof h->err, "%s", g_err);
    return 1;
}
#define DRV(h, x) do { CUresult r_ = (x); if (r_ != CUDA_SUCCESS) return fail(h, #x, (long long)r_); } while (0)
#define RT(h, x) do { cudaError_t r_ = (x); if (r_ != cudaSuccess) return fail(h, #x, (long long)r_); } while (0)
#define FFT(h, x) do { cufftResult r_ = (x); if (r_ != CUFFT_SUCCESS) return fail(h, #x, (long long)r_); } while (0)
#define RND(h, x) do { curandStatus_t r_ = (x); if (r_ != CURAND_STATUS_SUCCESS) return fail(h, #x, (long long)r_); } while (0)

int find_kernels(RefGpu *h) {
    unsigned int count = 0;
    DRV(h, cuModuleGetFunctionCount(&count, h->mod));
    std::vector<CUfunction> fns(count);
    DRV(h, cuModuleEnumerateFunctions(fns.data(), count, h->mod));
    for (int i = 0; i < K_COUNT; ++i) {
        const std::string pre = "_Z" + std::to_string(std::strlen(kNames[i])) + kNames[i];
        for (CUfunction f : fns) {
            const char *name = nullptr;
            if (cuFuncGetName(&name, f) != CUDA_SUCCESS || !name) continue;
            if (std::strncmp(name, pre.c_str(), pre.size()) == 0 && !std::isdigit((unsigned char)name[pre.size()])) {
                h->k[i] = f;
                break;
            }
        }
        if (!h->k[i]) {
            std::snprintf(h->err, sizeof h->err, "kernel %s not in the cubin", kNames[i]);
            std::snprintf(g_err, sizeof g_err, "%s", h->err);
            return 1;
        }
    }
    return 0;
}

// dimgrid/dimblock of the 4-D kernels (Propagator_without_cutoff.cu:325-335)
int launch4(RefGpu *h, int which, void **args, unsigned smem = 0) {
    DRV(h, cuLaunchKernel(h->k[which], h->X / h->bx, h->Y / h->by, (h->Z * h->T) / (h->bz * h->bt),
                          h->bx, h->by, h->bz * h->bt, smem, nullptr, args, nullptr));
    return 0;
}
// dimgrid2/dimblock2 of the 1-D kernels (Lattice.cu:119-122)
int launch1(RefGpu *h, int which, void **args) {
    DRV(h, cuLaunchKernel(h->k[which], (unsigned)(h->n / h->bs), 1, 1, h->bs, 1, 1, 0, nullptr, args,
                          nullptr));
    return 0;
}

// ComplexLattice::fft / fft_inv: psi uses CUFFT_INVERSE for fft(), psibar CUFFT_FORWARD
int fft(RefGpu *h, double2 *a, bool conjugated, bool inverse) {
    const int dir = (conjugated != inverse) ? CUFFT_FORWARD : CUFFT_INVERSE;
    FFT(h, cufftExecZ2Z(h->plan, (cufftDoubleComplex *)a, (cufftDoubleComplex *)a, dir));
    return 0;
}

int normalize(RefGpu *h, double2 *a, double f) {
    RT(h, cudaDeviceSynchronize());
    void *args[] = {&a, &f};
    if (launch1(h, K_NORMALIZATION, args)) return 1;
    RT(h, cudaDeviceSynchronize());
    return 0;
}

int add_into(RefGpu *h, double2 *a, double2 *b) {
    RT(h, cudaDeviceSynchronize());
    void *args[] = {&a, &b};
    if (launch1(h, K_SUMMATION, args)) return 1;
    RT(h, cudaDeviceSynchronize());
    return 0;
}

// Propagator::get_max_and_mean_drift (:351-380), its allocations included
int max_and_mean(RefGpu *h, double *mx, double *mean) {
    const int total = (int)h->n;
    double *d_max, *d_sum;
    RT(h, cudaMalloc(&d_max, sizeof(double)));
    RT(h, cudaMalloc(&d_sum, sizeof(double)));
    RT(h, cudaMemset(d_max, 0, sizeof(double)));
    RT(h, cudaMemset(d_sum, 0, sizeof(double)));
    const int block = h->bx * h->by * h->bz * h->bt;
    const int grid = (h->X / h->bx) * (h->Y / h->by) * ((h->Z * h->T) / (h->bz * h->bt));
    void *args[] = {&h->drift, (void *)&total, &d_max, &d_sum};
    DRV(h, cuLaunchKernel(h->k[K_MAXMEAN], grid, 1, 1, block, 1, 1, 2 * block * sizeof(double), nullptr, args,
                          nullptr));
    double hm, hs;
    RT(h, cudaMemcpy(&hm, d_max, sizeof(double), cudaMemcpyDeviceToHost));
    RT(h, cudaMemcpy(&hs, d_sum, sizeof(double), cudaMemcpyDeviceToHost));
    *mx = hm;
    *mean = hs / total;
    RT(h, cudaFree(d_max));
    RT(h, cudaFree(d_sum));
    return 0;
}

// Propagator::compute_new_dt (:382-404), without its console messages
double new_dt(double DT, double mean, double mx) {
    double dt = mx <= 0.0 ? DT : (mean / mx) * DT;
    if (dt < 1e-8) dt = 1e-8;
    if (dt > 0.01) dt = 0.01;
    const double alpha = 0.9;
    return (1 - alpha) * DT + alpha * dt;
}

// Propagator::propagate (:406-442).  normals: NULL -> cuRAND; else 2CVT host unit normals.
int propagate(RefGpu *h, double P, double MU, const double *normals) {
    const size_t bytes = (size_t)h->n * sizeof(double2);
    RT(h, cudaMemcpy(h->kin, h->psi, bytes, cudaMemcpyDeviceToDevice));
    RT(h, cudaMemcpy(h->kinc, h->psic, bytes, cudaMemcpyDeviceToDevice));
    if (fft(h, h->kin, false, false) || fft(h, h->kinc, true, false)) return 1;
    RT(h, cudaDeviceSynchronize());
    {
        void *args[] = {&h->kin, &h->kinc, &h->kin, &h->kinc};
        if (launch4(h, K_KINETIC, args)) return 1;
    }
    RT(h, cudaDeviceSynchronize());
    if (fft(h, h->kin, false, true) || fft(h, h->kinc, true, true)) return 1;
    const double f = 1. / double(h->a_x * h->X * h->Y * h->Z);
    if (normalize(h, h->kin, f) || normalize(h, h->kinc, f)) return 1;
    RT(h, cudaDeviceSynchronize());
    {
        double factor = 1.0;
        void *args[] = {&h->psi, &h->psic, &h->kin, &h->kinc, &h->drift, &h->driftc, &factor, &P, &MU};
        if (launch4(h, K_DRIFT, args)) return 1;
    }
    RT(h, cudaDeviceSynchronize());
    if (max_and_mean(h, &h->last_max, &h->last_mean)) return 1;
    RT(h, cudaDeviceSynchronize());
    h->dt = new_dt(h->DT, h->last_mean, h->last_max);
    const size_t nr = 2 * (size_t)h->n;
    if (normals) {
        std::vector<double> r(nr);
        const double sd = std::sqrt(h->dt);
        for (size_t i = 0; i < nr; ++i) r[i] = sd * normals[i];  // = 0 + sqrt(dt) * z, as cuRAND forms it
        RT(h, cudaMemcpy(h->rnd, r.data(), nr * sizeof(double), cudaMemcpyHostToDevice));
    } else {
        RND(h, curandGenerateNormalDouble(h->gen, h->rnd, nr, 0., std::sqrt(h->dt)));
    }
    RT(h, cudaDeviceSynchronize());
    {
        void *args[] = {&h->drift, &h->driftc, &h->dt};
        if (launch4(h, K_MUL_DT, args)) return 1;
    }
    RT(h, cudaDeviceSynchronize());
    {
        void *args[] = {&h->drift, &h->driftc, &h->rnd};
        if (launch4(h, K_ADD_NOISE, args)) return 1;
    }
    RT(h, cudaDeviceSynchronize());
    if (add_into(h, h->psi, h->drift)) return 1;
    RT(h, cudaDeviceSynchronize());
    if (add_into(h, h->psic, h->driftc)) return 1;
    RT(h, cudaDeviceSynchronize());
    return 0;
}

}  // namespace

extern "C" {

typedef struct RefGpu refgpu;

const char *refgpu_last_error(void) { return g_err; }

// dims: X, Y, Z, T, C; blocks: BLOCKSIZE, BLOCKSIZEX, BLOCKSIZEY, BLOCKSIZEZ,
// BLOCKSIZETAU; consts: EPS, a_x, DT -- the macros the cubin was built with.
int refgpu_create(const char *cubin, const int *dims, const int *blocks, const double *consts,
                  unsigned long long seed, int device, refgpu **out) {
    *out = nullptr;
    RefGpu *h = new RefGpu();
    h->X = dims[0]; h->Y = dims[1]; h->Z = dims[2]; h->T = dims[3]; h->C = dims[4];
    h->bs = blocks[0]; h->bx = blocks[1]; h->by = blocks[2]; h->bz = blocks[3]; h->bt = blocks[4];
    h->eps = consts[0]; h->a_x = consts[1]; h->DT = consts[2];
    h->dt = h->DT;
    h->n = (long long)h->C * h->X * h->Y * h->Z * h->T;
    auto bail = [&](int rc) { delete h; return rc; };
    // the launch geometry must tile the lattice exactly (the reference only warns,
    // Propagator_without_cutoff.cu:325-331; a partial tiling would index past the arrays)
    if (h->X % h->bx || h->Y % h->by || (h->Z * h->T) % (h->bz * h->bt) || h->n % h->bs ||
        h->bx * h->by * h->bz * h->bt > 1024)
        return bail(fail(nullptr, "lattice not tiled by the block sizes", 0));
    if (cudaSetDevice(device) != cudaSuccess || cudaFree(nullptr) != cudaSuccess)
        return bail(fail(nullptr, "cudaSetDevice", device));
    if (cuModuleLoad(&h->mod, cubin) != CUDA_SUCCESS) return bail(fail(nullptr, "cuModuleLoad", 0));
    if (find_kernels(h)) { cuModuleUnload(h->mod); return bail(1); }
    const size_t bytes = (size_t)h->n * sizeof(double2);
    double2 **bufs[] = {&h->psi, &h->psic, &h->kin, &h->kinc, &h->drift, &h->driftc};
    for (double2 **b : bufs)
        if (cudaMalloc(b, bytes) != cudaSuccess) return bail(fail(nullptr, "cudaMalloc", 0));
    if (cudaMalloc(&h->rnd, 2 * (size_t)h->n * sizeof(double)) != cudaSuccess)
        return bail(fail(nullptr, "cudaMalloc", 0));
    const int rank = h->Z > 1 ? 3 : (h->Y > 1 ? 2 : 1);
    int nn[3] = {h->X, h->Y, h->Z};
    if (cufftPlanMany(&h->plan, rank, nn, nullptr, 0, 0, nullptr, 0, 0, CUFFT_Z2Z, h->C * h->T) != CUFFT_SUCCESS)
        return bail(fail(nullptr, "cufftPlanMany", 0));
    if (curandCreateGenerator(&h->gen, CURAND_RNG_PSEUDO_XORWOW) != CURAND_STATUS_SUCCESS ||
        curandSetPseudoRandomGeneratorSeed(h->gen, seed) != CURAND_STATUS_SUCCESS)
        return bail(fail(nullptr, "curandCreateGenerator", 0));
    *out = h;
    return 0;
}

int refgpu_destroy(refgpu *h) {
    if (!h) return 0;
    cudaDeviceSynchronize();
    double2 *bufs[] = {h->psi, h->psic, h->kin, h->kinc, h->drift, h->driftc};
    for (double2 *b : bufs) cudaFree(b);
    cudaFree(h->rnd);
    if (h->plan) cufftDestroy(h->plan);
    if (h->gen) curandDestroyGenerator(h->gen);
    if (h->mod) cuModuleUnload(h->mod);
    delete h;
    return 0;
}

// psi, psic: host complex128 arrays (interleaved re, im) in the [c][tau][x][y][z] layout
int refgpu_set_fields(refgpu *h, const double *psi, const double *psic) {
    const size_t bytes = (size_t)h->n * sizeof(double2);
    RT(h, cudaMemcpy(h->psi, psi, bytes, cudaMemcpyHostToDevice));
    RT(h, cudaMemcpy(h->psic, psic, bytes, cudaMemcpyHostToDevice));
    return 0;
}

int refgpu_get_fields(refgpu *h, double *psi, double *psic) {
    const size_t bytes = (size_t)h->n * sizeof(double2);
    RT(h, cudaDeviceSynchronize());
    RT(h, cudaMemcpy(psi, h->psi, bytes, cudaMemcpyDeviceToHost));
    RT(h, cudaMemcpy(psic, h->psic, bytes, cudaMemcpyDeviceToHost));
    return 0;
}

// ComplexLattice::set_mean_field (Lattice.cu:189-194) on both fields
int refgpu_set_mean_field(refgpu *h, double re, double im, double P, double MU) {
    RT(h, cudaDeviceSynchronize());
    bool f = false, t = true;
    void *a1[] = {&h->psi, &re, &im, &f, &P, &MU};
    if (launch4(h, K_SET_VALUE, a1)) return 1;
    RT(h, cudaDeviceSynchronize());
    void *a2[] = {&h->psic, &re, &im, &t, &P, &MU};
    if (launch4(h, K_SET_VALUE, a2)) return 1;
    RT(h, cudaDeviceSynchronize());
    return 0;
}

// One Propagator::propagate.  normals: NULL -> the cuRAND stream; else 2CVT unit
// normals in the ind_rand layout.  out3 (may be NULL): dt, max, mean of the step.
int refgpu_propagate(refgpu *h, double P, double MU, const double *normals, double *out3) {
    if (propagate(h, P, MU, normals)) return 1;
    if (out3) { out3[0] = h->dt; out3[1] = h->last_max; out3[2] = h->last_mean; }
    return 0;
}

// nsteps propagate calls with cuRAND noise; *ms: CUDA-event time on the default
// stream (the reference's stream) over all of them, *wall_ms: host wall clock.
int refgpu_time(refgpu *h, int nsteps, double P, double MU, float *ms, double *wall_ms) {
    cudaEvent_t a, b;
    RT(h, cudaEventCreate(&a));
    RT(h, cudaEventCreate(&b));
    RT(h, cudaDeviceSynchronize());
    const auto t0 = std::chrono::steady_clock::now();
    RT(h, cudaEventRecord(a, 0));
    for (int i = 0; i < nsteps; ++i)
        if (propagate(h, P, MU, nullptr)) return 1;
    RT(h, cudaEventRecord(b, 0));
    RT(h, cudaEventSynchronize(b));
    const auto t1 = std::chrono::steady_clock::now();
    RT(h, cudaEventElapsedTime(ms, a, b));
    *wall_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return 0;
}

// The observables of Observables::evaluate for the current fields, per call
// (not cumulative): n[5] = sums of evaluate_n_tot, n_11, n_12, n_21, n_22 over
// the FFT'd fields (Observables_without_cutoff.cu:1310-1382) and F[3][V] the
// F_x, F_y, F_z profiles (:1274-1306).  Scratch is allocated per call.
int refgpu_observables(refgpu *h, double *n, double *F) {
    const long long V = (long long)h->X * h->Y * h->Z;
    const size_t bytes = (size_t)h->n * sizeof(double2);
    double *avg;
    RT(h, cudaMalloc(&avg, (size_t)(V * h->T) * sizeof(double)));
    RT(h, cudaMemcpy(h->kin, h->psi, bytes, cudaMemcpyDeviceToDevice));
    RT(h, cudaMemcpy(h->kinc, h->psic, bytes, cudaMemcpyDeviceToDevice));
    for (int i = 0; i < 3; ++i) {
        RT(h, cudaMemset(avg, 0, (size_t)V * sizeof(double)));
        int idx = i;
        void *args[] = {&h->kinc, &h->kin, &avg, &idx};
        if (launch4(h, K_SPIN, args)) return 1;
        RT(h, cudaMemcpy(F + i * V, avg, (size_t)V * sizeof(double), cudaMemcpyDeviceToHost));
    }
    if (fft(h, h->kinc, true, false) || fft(h, h->kin, false, false)) return 1;
    std::vector<double> hv((size_t)(V * h->T));
    for (int w = 0; w < 5; ++w) {
        RT(h, cudaMemset(avg, 0, (size_t)(V * h->T) * sizeof(double)));
        void *args[] = {&h->kinc, &h->kin, &avg};
        if (launch4(h, K_N_TOT + w, args)) return 1;
        RT(h, cudaMemcpy(hv.data(), avg, hv.size() * sizeof(double), cudaMemcpyDeviceToHost));
        double s = 0;
        for (double x : hv) s += x;
        n[w] = s;
    }
    RT(h, cudaFree(avg));
    return 0;
}

}  // extern "C"
