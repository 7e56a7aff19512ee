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
    int pdl;                  // update: programmatic launch (may start while the previous kernel runs)
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
    int withhold;       // failure-detection test: CTA 0 never issues its first copy
    void *drift_out, *driftc_out;  // MAXONLY: also store K, Kbar here (field layout), or null
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
    int split;          // tasks step psi and psibar in separate CTAs (FusedTask::side)
    size_t smem_bytes;
};

// Many steps of a small problem in one cooperative launch (k_loop.cu): one CTA per
// split fused task of one imaginary time.
struct LaunchLoop {
    const ChainDev *chains;
    ChainState *state;
    const FusedTask *tasks;
    int ntasks, nsteps;
    int model, kinetic, ln, dt_rule;
    void *fld[2][2];      // [buffer set][psi, psibar]
    int from;             // buffer set the first step reads
    void *noise;          // unit normals of the current step (field layout), exchanged by the CTA pairs
    double2 *partials;
    unsigned int *bar;    // grid barrier arrivals, zero at launch
    int *abort;           // set when a barrier wait gives up, zero at launch
    int withhold;         // failure-detection test: CTA 0 never arrives at the first barrier
};

// Compile-time plans of power-of-two lines: factor order 8, 8, ..., then 4 or 2
// (the order the host's table builder uses).
__host__ __device__ constexpr int p2_nfac(int n) {
    int k = 0;
    while (n % 8 == 0) { n /= 8; ++k; }
    while (n % 4 == 0) { n /= 4; ++k; }
    while (n % 2 == 0) { n /= 2; ++k; }
    return k;
}
__host__ __device__ constexpr int p2_fac(int n, int p) {
    for (int i = 0;; ++i) {
        const int r = (n % 8 == 0) ? 8 : ((n % 4 == 0) ? 4 : 2);
        if (i == p) return r;
        n /= r;
    }
}
// Compile-time plans of the tiled path's axis filter (lines of 32, 64, 96, 128,
// 256, 512): lines of 128 take 16 x 8 (three passes instead of five), others the
// factors 8, 4, 2, 3, 5 in that order.
__host__ __device__ constexpr int ax_first_radix(int n, int n0) {
    return (n0 == 128 && n == 128) ? 16
           : (n % 8 == 0 ? 8 : (n % 4 == 0 ? 4 : (n % 2 == 0 ? 2 : (n % 3 == 0 ? 3 : 5))));
}
__host__ __device__ constexpr int ax_nfac(int n) {
    int k = 0, m = n;
    while (m > 1) { m /= ax_first_radix(m, n); ++k; }
    return k;
}
__host__ __device__ constexpr int ax_fac(int n, int p) {
    int m = n;
    for (int i = 0;; ++i) {
        const int r = ax_first_radix(m, n);
        if (i == p) return r;
        m /= r;
    }
}
// Stride NS of forward pass p and of inverse pass p (the inverse runs the
// factors in reverse after the middle pass, whose radix is the last factor).
__host__ __device__ constexpr int tw_ns_fwd(int n, int p) {
    int ns = 1;
    for (int i = 0; i < p; ++i) ns *= p2_fac(n, i);
    return ns;
}
__host__ __device__ constexpr int tw_ns_inv(int n, int p) {
    const int nf = p2_nfac(n);
    int ns = p2_fac(n, nf - 1);
    for (int i = nf - 2; i > p; --i) ns *= p2_fac(n, i);
    return ns;
}
// Per-pass twiddle tables of the fused kernel's compile-time line plans (the axis
// filter keeps the length-n table: per-pass tables measured 3 % slower on its
// 64-point lines).  Pass (R, NS) reads its
// twiddles w^(k r) (w = exp(-2 pi i / (NS R)), conjugated for the inverse
// passes) at [(r - 1) NS + k], so the lanes of a warp read consecutive entries
// instead of the strided entries k r n/(NS R) of the length-n table, which
// collide in the shared-memory banks.  Order: forward passes 1 .. NF-2 (pass 0
// has NS = 1 and no twiddles), the middle pass ((RL - 1) n / RL entries,
// indexed by the butterfly j < n/RL), inverse passes NF-2 .. 0.
__host__ __device__ constexpr int tw_fwd_off(int n, int p) {
    int off = 0;
    for (int i = 1; i < p; ++i) off += (p2_fac(n, i) - 1) * tw_ns_fwd(n, i);
    return off;
}
__host__ __device__ constexpr int tw_mid_off(int n) { return tw_fwd_off(n, p2_nfac(n) - 1); }
__host__ __device__ constexpr int tw_inv_off(int n, int p) {
    const int nf = p2_nfac(n), rl = p2_fac(n, nf - 1);
    int off = tw_mid_off(n) + (rl - 1) * (n / rl);
    for (int i = nf - 2; i > p; --i) off += (p2_fac(n, i) - 1) * tw_ns_inv(n, i);
    return off;
}
__host__ __device__ constexpr int tw_entries(int n) { return n > 1 ? tw_inv_off(n, -1) : 0; }
// Entry e of the per-pass tables is w_n^m (m returned), conjugated when *conj.
__host__ __device__ inline int pass_twiddle_source(int n, int e, bool *conj) {
    const int nf = p2_nfac(n), rl = p2_fac(n, nf - 1);
    int rem = e, R = rl, NS = n / rl;
    bool found = false;
    *conj = false;
    for (int p = 1; p < nf - 1 && !found; ++p) {
        const int sz = (p2_fac(n, p) - 1) * tw_ns_fwd(n, p);
        if (rem < sz) { R = p2_fac(n, p); NS = tw_ns_fwd(n, p); found = true; }
        else rem -= sz;
    }
    if (!found) {
        const int sz = (rl - 1) * (n / rl);
        if (rem < sz) found = true;
        else rem -= sz;
    }
    for (int p = nf - 2; p >= 0 && !found; --p) {
        const int sz = (p2_fac(n, p) - 1) * tw_ns_inv(n, p);
        if (rem < sz) { R = p2_fac(n, p); NS = tw_ns_inv(n, p); *conj = true; found = true; }
        else rem -= sz;
    }
    const int r = 1 + rem / NS, k = rem % NS;
    return k * r * (n / (NS * R));
}

// Shared memory of the fused kernel before its slots: barriers (64 B), the
// twiddle and filter tables of tab_n entries, the per-pass twiddles of the
// compile-time plan of ln-site lines (ln > 0), rounded up to 128 B.
__host__ __device__ constexpr int fused_ptw_offset(int tab_n, int esz) {
    return (64 + tab_n * (esz + esz / 2) + 15) / 16 * 16;
}
__host__ __device__ constexpr int fused_tab_bytes(int tab_n, int esz, int ln) {
    return (fused_ptw_offset(tab_n, esz) + (ln > 0 ? tw_entries(ln) : 0) * esz + 127) / 128 * 128;
}

// Elements of a padded FFT scratch line of n sites (one spare element per 16, even).
__host__ __device__ constexpr int padded_line(int v) { return (v + v / 16 + 1) + ((v + v / 16 + 1) & 1); }
// Elements between the fused kernel's shared slots: ncomp padded component rows of
// slices of at most v sites, rounded to 128 bytes.
__host__ __device__ constexpr int fused_slot_stride(int ncomp, int v, int esz) {
    return (ncomp * padded_line(v) + 128 / esz - 1) / (128 / esz) * (128 / esz);
}

// Tiled path (slices too large for the fused kernel).  Axis filter: a CTA
// filters `W` adjacent lines of one (chain, component, tau) slice along one
// axis for one field (blockIdx.y), staged in shared memory as a tile.
struct AxisTask {
    int chain;
    int slice;  // c * nt + tau of the tile's first line
    int l0;     // first line of the tile (line index within that slice)
    int nl;     // lines in the tile (<= W; adjacent in memory for a strided axis; for the
                // innermost axis without a component constant they may run on into the
                // following slices, which are contiguous)
};

struct LaunchAxis {
    const ChainDev *chains;
    const AxisTask *tasks;
    int ntasks;
    int axis;
    int n;           // line length of every task of this launch
    int W;           // lines per tile
    int pitch;       // shared elements between the tile's lines (odd)
    int with_const;  // multiply the component constant (first axis of the EXP kinetic)
    const void *src0, *src1;
    void *dst0, *dst1;
    size_t smem_bytes;
    int nfields;     // 2: psi and psibar (blockIdx.x % 2), 1: src0 -> dst0 only
    int filter;      // 0: kinetic filter, 1: kinetic-energy filter k^2/2 (normalised)
    int accumulate;  // 1: dst += filtered (sum over axes of one-axis operators)
    int strided;     // every task's lines are neighbours in memory (axis stride > 1)
};

// Step over precomputed kinetic terms: a CTA streams imaginary times
// [tau0, tau1) of 256 consecutive sites of one chain.
struct TileTask {
    int chain;
    int site0;
    int tau0, tau1;
    int part;   // index of the CTA's step-rule partial within the chain
};

struct LaunchTiled {
    const ChainDev *chains;
    ChainState *state;
    const TileTask *tasks;
    int ntasks;
    int model, dt_rule, noise, mode;  // mode: FUSED_SPEC / FUSED_MAXONLY / FUSED_APPLY
    int only_rejected;
    const void *psi_in, *psic_in, *kin, *kinc;
    void *psi_out, *psic_out;
    double2 *partials;
    const double *noise_buf;
    void *drift_out, *driftc_out;  // MAXONLY: also store K, Kbar here (field layout), or null
};

template <class R> cudaError_t launch_axis_filter(const LaunchAxis &L, cudaStream_t s);
template <class R> cudaError_t setup_axis_filter(int n, size_t smem_bytes, int *ctas_per_sm);

// Plane filter (k_plane.cu): both axes of square n x n planes (n = 32, 64, 96, 128)
// in one pass; LaunchAxis with axis = the planes' slower axis, tasks {chain, slice,
// plane index, 1}.  Line plans of two radices, p = 0 first: 32 = 8 x 4, 64 = 8 x 8,
// 96 = 12 x 8, 128 = 16 x 8 (three passes over shared memory per axis).
__host__ __device__ constexpr int plane_nfac(int) { return 2; }
__host__ __device__ constexpr int plane_fac(int n, int p) {
    return p == 1 ? (n == 32 ? 4 : 8) : (n == 128 ? 16 : (n == 96 ? 12 : 8));
}
// Threads per CTA (esz: bytes of a complex element): FP32 planes of 64 take one thread
// per line (the whole line in registers); otherwise every pass of the plan gives each
// thread a whole number of butterflies; 128 takes 512 threads of 32 elements (measured
// 7 % faster than 1024 threads of 16 at the 64-register cap).  Shared memory: twiddles
// and the two axes' filters, then the plane at an odd pitch.
__host__ __device__ constexpr bool plane_line_per_thread(int n, int esz) { return n == 64 && esz == 8; }
__host__ __device__ constexpr int plane_threads(int n, int esz) {
    return plane_line_per_thread(n, esz) ? n : (n == 96 ? 384 : (n == 32 ? 128 : (n == 128 ? 512 : n * n / 16)));
}
__host__ __device__ constexpr int plane_pitch(int n) { return n + 1; }
__host__ __device__ constexpr size_t plane_tab_bytes(int n, size_t esz) { return ((size_t)n * 2 * esz + 15) / 16 * 16; }
__host__ __device__ constexpr size_t plane_smem_bytes(int n, size_t esz) {
    return plane_tab_bytes(n, esz) + (size_t)n * plane_pitch(n) * esz;
}
template <class R> cudaError_t launch_plane_filter(const LaunchAxis &L, cudaStream_t s);
template <class R> cudaError_t setup_plane_filter(int n, size_t smem_bytes, int *ctas_per_sm);
template <class R> cudaError_t launch_tiled(const LaunchTiled &L, cudaStream_t s);
template <class R> cudaError_t setup_tiled(int model, int *ctas_per_sm);
// Axis filter geometry.  Compile-time plans exist for lines of 32, 64, 96, 128,
// 256 and 512 sites.  Lines per tile (FP32; half at FP64): 64 for 32, 32 for 64,
// 16 for 96 and 128, 8 for 256, 512 and runtime plans (n = 0 here), so that a
// radix-8 pass has about a butterfly for each of the 256 threads and a tile with
// its scratch fits in a quarter of an SM's shared memory.
__host__ __device__ constexpr bool axis_compile_time_plan(int n) {
    return n == 32 || n == 64 || n == 96 || n == 128 || n == 256 || n == 512;
}
template <class R>
__host__ __device__ constexpr int axis_tile_lines(int n) {
    return (n == 32 ? 64 : (n == 64 ? 32 : ((n == 96 || n == 128) ? 16 : 8))) / (sizeof(R) == 4 ? 1 : 2);
}
// shared-memory bytes of the twiddle and filter tables for lines of n
__host__ __device__ constexpr size_t axis_tab_bytes(int n, size_t esz) { return ((size_t)n * (esz + esz / 2) + 15) / 16 * 16; }
// tile elements (W lines at pitch PL), rounded to keep the scratch 16-byte aligned
__host__ __device__ constexpr int axis_tile_elems(int n, int PL, int W) { return (W * PL + 1) / 2 * 2; }
// line pitch of the tile: odd (no bank conflicts for the transposing accesses); for
// the compile-time plans large enough to hold a padded line, since the tile is one
// of the two buffers the passes alternate between
__host__ __device__ constexpr int axis_pitch(int n, bool compile_time_plan) {
    return compile_time_plan ? (padded_line(n) | 1) : (n | 1);
}
// shared bytes of one CTA: tables, tile, scratch (one more tile for the CTA-wide
// compile-time plan, two padded lines per warp for the runtime plan)
__host__ __device__ constexpr size_t axis_smem_bytes(int n, bool compile_time_plan, int W, size_t esz) {
    return axis_tab_bytes(n, esz) +
           (compile_time_plan ? 2 * (size_t)axis_tile_elems(n, axis_pitch(n, true), W)
                              : (size_t)axis_tile_elems(n, axis_pitch(n, false), W) + 2 * 8 * padded_line(n)) *
               esz;
}

size_t loop_smem_bytes(int model, int ln, int esz);
template <class R> cudaError_t setup_loop(int model, int ln, int *ctas_per_sm);
template <class R> cudaError_t launch_loop(const LaunchLoop &L, cudaStream_t s);

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
// Spin-1 observables: CTA = 256 spatial sites of one chain x imaginary times [tau0, tau1).
struct LaunchObs {
    const ChainDev *chains;
    const ObsTask *tasks;
    int ntasks;
    const void *psi, *psic, *tpsi;
    double *partials;       // 8 per task
    unsigned int *arrive;   // per chain, zero between launches
    double *samples;        // [slot][chain][8]
    int slot, nchains;
};
template <class R> cudaError_t launch_obs_spin1(const LaunchObs &L, cudaStream_t s);
// complex128 boundary layout <-> engine precision (same element order)
template <class R> cudaError_t launch_import(void *dst, const double2 *src, long long n,
                                             cudaStream_t s);
template <class R> cudaError_t launch_export(double2 *dst, const void *src, long long n,
                                             cudaStream_t s);

}  // namespace clv
