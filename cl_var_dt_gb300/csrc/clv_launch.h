// clv_launch.h -- launch descriptors shared between the host engine
// (clv_engine.cu) and the kernel translation units.
#pragma once

#include <cuda_runtime.h>

#include "clv_internal.cuh"

namespace clv {

// Elements of one line bundle held by a CTA of the line filter (two shared
// buffers of this many complex values; 64 KB at FP64).
constexpr int kMaxBundleElems64 = 2048;
constexpr int kMaxBundleElems32 = 4096;
constexpr int kMaxLine = 2048;

struct LaunchLineFilter {
    const ChainDev *chains;
    const LineTask *tasks;
    int ntasks;
    int max_bundle;   // largest nlines*n over the tasks
    int axis;
    int nfields;      // 1 = psi only, 2 = psi and psibar
    const void *src0, *src1;
    void *dst0, *dst1;
    int filter;       // 0 = kinetic filter, 1 = kinetic-energy filter
    int mode;         // 0 = overwrite, 1 = accumulate
    int with_const;   // multiply the component constant (first pass of the EXP kinetic)
};

struct LaunchSites {
    const ChainDev *chains;
    ChainState *state;
    const SiteTask *tasks;
    int ntasks;
    int model, dt_rule, noise;
    const void *psi, *psic, *kin, *kinc;
    void *psi_w, *psic_w;
    void *drift, *driftc;
    double2 *partials;        // one (max, sum) per CTA
    const double *noise_buf;  // external noise (reference ind_rand layout)
    double *acc;              // observable accumulators
    int acc_slot;
};

enum { FUSED_SPEC = 0, FUSED_MAXONLY = 1, FUSED_APPLY = 2 };

struct LaunchFused {
    const ChainDev *chains;
    ChainState *state;
    const FusedTask *tasks;
    int ntasks;
    int model, kinetic, dt_rule, noise, mode;
    int only_rejected;  // APPLY: skip chains whose speculative update was accepted
    int use_tma;        // slices arrive by cp.async.bulk (16-byte aligned rows)
    const void *psi_in, *psic_in;
    void *psi_out, *psic_out;
    double2 *partials;
    const double *noise_buf;
    int slot_stride;    // elements between shared-memory slots
    int comp_stride;    // elements between the components of one slot (padded V)
    int tab_n;          // twiddle/filter entries staged in shared memory
    int tab_bytes;      // bytes before the first slot (barriers + tables)
    int spt;            // lattice sites per thread (1, 2 or 4)
    int ln;             // every chain a 1D line of ln sites (64, 128, 256), else 0
    size_t smem_bytes;
};

cudaError_t setup_line_filter();
template <class R> cudaError_t launch_fused(const LaunchFused &L, cudaStream_t s);
template <class R> cudaError_t setup_fused(const LaunchFused &L, int *ctas_per_sm);
template <class R> cudaError_t launch_line_filter(const LaunchLineFilter &L, cudaStream_t s);
template <class R> cudaError_t launch_drift(const LaunchSites &L, cudaStream_t s);
template <class R> cudaError_t launch_update(const LaunchSites &L, cudaStream_t s);
template <class R> cudaError_t launch_set_mean_field(const LaunchSites &L, int field, double re,
                                                     double im, cudaStream_t s);
template <class R> cudaError_t launch_init_spin1(const LaunchSites &L, double amp, double sigma,
                                                 cudaStream_t s);
template <class R> cudaError_t launch_obs_ref(const LaunchSites &L, double *accF, double *accN,
                                              cudaStream_t s);
template <class R> cudaError_t launch_obs_spin1(const LaunchSites &L, const void *tpsi,
                                                double *samples, int slot, int nchains,
                                                cudaStream_t s);
// complex128 boundary layout <-> engine precision (same element order)
template <class R> cudaError_t launch_import(void *dst, const double2 *src, long long n,
                                             cudaStream_t s);
template <class R> cudaError_t launch_export(double2 *dst, const void *src, long long n,
                                             cudaStream_t s);

}  // namespace clv
