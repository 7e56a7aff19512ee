// clv_internal.cuh -- device-side data structures and helpers shared by the
// engine's kernels (kinetic line filter, drift/step rule, update, observables).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/clv.h"

namespace clv {

constexpr int kMaxFactors = 16;
constexpr int kMaxComp = 4;

// Precision traits: R is the arithmetic type of the bulk field work.
template <class R> struct Cx;
template <> struct Cx<double> { using T = double2; };
template <> struct Cx<float> { using T = float2; };

template <class C2> __device__ __forceinline__ C2 mk(double x, double y) {
    C2 r; r.x = x; r.y = y; return r;
}
template <class C2> __device__ __forceinline__ C2 cadd(C2 a, C2 b) { C2 r; r.x = a.x + b.x; r.y = a.y + b.y; return r; }
template <class C2> __device__ __forceinline__ C2 csub(C2 a, C2 b) { C2 r; r.x = a.x - b.x; r.y = a.y - b.y; return r; }
// cuCmul ordering: (a.x b.x - a.y b.y, a.x b.y + a.y b.x)
template <class C2> __device__ __forceinline__ C2 cmul(C2 a, C2 b) {
    C2 r; r.x = a.x * b.x - a.y * b.y; r.y = a.x * b.y + a.y * b.x; return r;
}
template <class C2, class R> __device__ __forceinline__ C2 cscale(R s, C2 a) { C2 r; r.x = s * a.x; r.y = s * a.y; return r; }
template <class C2> __device__ __forceinline__ C2 cconj(C2 a) { C2 r; r.x = a.x; r.y = -a.y; return r; }

// One axis of one chain, as seen by the kinetic line filter.
struct AxisDev {
    int n;                 // line length (lattice extent along the axis)
    int inner;             // stride of the axis in elements (product of faster dims)
    int nf;                // number of radix factors
    int fac[kMaxFactors];  // radix of each Stockham pass
    const double2 *tw64;   // exp(-2 pi i k/n), k < n
    const float2 *tw32;
    const double *filt64;  // kinetic filter f[k], k < n (normalisation folded in)
    const float *filt32;
    const double *efilt64; // kinetic-energy filter k^2/2 / n (spin-1 observables)
    const float *efilt32;
    // per-pass twiddle tables of the fused kernel's power-of-two line plans
    // (layout tw_*_off, n = 64 ... 512); null for other lengths
    const double2 *ptw64;
    const float2 *ptw32;
};

// Per-chain constants (device copy, read-only during steps).
struct ChainDev {
    int nx, ny, nz, nt;
    int V;                     // nx*ny*nz
    int ncomp;
    long long off;             // element offset of the chain in the field arrays
    long long noise_off;       // element offset (doubles) in an external noise buffer
    double eps, a_x, mu, P, Q, G, DT, dt_min, dt_max_clamp, alpha;
    double c0, c1, q, K, dt_max;
    uint64_t seed;
    double comp_const[kMaxComp];   // EXP kinetic: exp(eps (mu + q m^2)) per component
    AxisDev axis[3];
    int site_block0, site_nblocks; // range of this chain's blocks in site-parallel kernels
    int fused_block0, fused_nblocks; // range of this chain's CTAs in the fused step kernel
    int obs_off;                   // offset of this chain's F-profile accumulators
    int obs_block0, obs_nblocks;   // range of this chain's CTAs in the spin-1 observables
};

// Per-chain mutable step state (device).
struct ChainState {
    double dt, max, mean, t;
    double red_max, red_sum;       // scratch of the last-block reduction
    unsigned long long step;       // Langevin steps completed
    unsigned long long noise_step; // step index used by the current noise draw
    unsigned int arrive;           // blocks of the drift kernel that have finished
    int flags;
    int clamp_low, clamp_high;
    int accepted;                  // 1: the speculative update of this step stands
    int rejected;                  // speculative updates redone so far
};

// A CTA's share of a site-parallel kernel: `count` consecutive (tau, s) sites
// of one chain starting at linear site index `site0` = tau*V + s.
struct SiteTask {
    int chain;
    int site0;
};

// A CTA's share of the fused step: imaginary times [tau0, tau1) of one chain;
// `part` indexes the CTA's step-rule partial within the chain.  Problems too small
// to give every SM a CTA split each chunk into a psi CTA (kinetic term of psi,
// drift K, update of psi) and a psibar CTA (the same for psibar), and, smaller
// still, each of those by component halves (the drift of a component needs every
// component's fields but only its own kinetic term).
struct FusedTask {
    int chain;
    int tau0, tau1;
    int part;
    int side;   // 0: both fields; 1: psi only, 2: psibar only (two CTAs per chunk)
    int cmask;  // components this CTA filters, drifts, updates and stores (bit c); 0: all
};

// A CTA's share of the spin-1 observables: 256 spatial sites from site0 of one
// chain over imaginary times [tau0, tau1).
struct ObsTask {
    int chain;
    int site0;
    int tau0, tau1;
};

// A CTA's share of the kinetic line filter: lines [line0, line0+nlines) of one
// chain along one axis, over both fields.
struct LineTask {
    int chain;
    int line0;
    int nlines;
};

// Sites per CTA of the site-parallel kernels (drift, update, initialisation): 128
// spreads the small lattices of the reference's own configurations (256 x 32) over
// twice as many SMs as 256 would.
constexpr int kSiteBlock = 128;

// ------------------------------------------------------------------ Philox
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), counter-based.
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
        const uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
        c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
        k.x += 0x9E3779B9u;
        k.y += 0xBB67AE85u;
    }
    return c;
}

// Unit complex normals from the counter-based stream.  One Philox block serves
// a component pair: counter = {site, step_lo, step_hi, chain + (c/2) 2^24},
// key = seed; words (x, y) = (o.x, o.y) for even c and (o.z, o.w) for odd c;
// Box-Muller with u1 = (x + 1/2) 2^-32 in (0,1), u2 = y 2^-32 in [0,1).
__device__ __forceinline__ uint4 philox_block(uint64_t seed, uint32_t chain, uint64_t step,
                                              int pair, uint32_t site) {
    return philox4x32_10(
        make_uint4(site, (uint32_t)step, (uint32_t)(step >> 32), chain + ((uint32_t)pair << 24)),
        make_uint2((uint32_t)seed, (uint32_t)(seed >> 32)));
}

// Step noise of component c at linear site `site` (tau V + s) of a chain of ncomp
// components: the words (x, y) of the block of its pair.  The last component of an
// odd count (spin-1's third) has no partner, so two consecutive sites share its
// block: counter site j = site / 2, words (x, y) for site 2j and (z, w) for 2j + 1
// (1.5 blocks per spin-1 site instead of 2).  The spin-1 start keeps one block per
// site and pair (philox_normal64).
__device__ __forceinline__ bool lone_component(int c, int ncomp) { return (ncomp & 1) && c == ncomp - 1; }
__device__ __forceinline__ uint2 noise_words(uint64_t seed, uint32_t chain, uint64_t step, int c, int ncomp,
                                             uint32_t site) {
    const bool lone = lone_component(c, ncomp);
    const uint4 o = philox_block(seed, chain, step, c >> 1, lone ? site >> 1 : site);
    return (lone ? (site & 1) : (c & 1)) ? make_uint2(o.z, o.w) : make_uint2(o.x, o.y);
}

__device__ __forceinline__ double2 box_muller64(uint32_t x, uint32_t y) {
    const double two_m32 = 2.3283064365386963e-10;
    const double u1 = ((double)x + 0.5) * two_m32;
    const double u2 = (double)y * two_m32;
    const double r = sqrt(-2.0 * log(u1));
    double s, c;
    sincospi(2.0 * u2, &s, &c);
    return make_double2(r * c, r * s);
}

// FP32 arithmetic on the same words as box_muller64 with the hardware logarithm,
// reciprocal square root and sine/cosine (MUFU); same realisation as
// box_muller64 to about 1e-6 absolute.  Near u1 = 1 the hardware logarithm's
// absolute error (~4e-7) would dominate the small radius, so for
// w = 1 - u1 < 2^-8 the logarithm is the Taylor series of log(1 - w) to w^4
// (truncation below w^5/5 < 2^-42), with w formed exactly from the integer word.
__device__ __forceinline__ float2 box_muller32(uint32_t x, uint32_t y) {
    const float two_m32 = 2.3283064365386963e-10f;
    const float u1 = fmaf((float)x, two_m32, 0.5f * two_m32);
    const float w = fmaf((float)(~x), two_m32, 0.5f * two_m32);  // 1 - u1
    const float series = -w * fmaf(w, fmaf(w, fmaf(w, 0.25f, 0.33333334f), 0.5f), 1.0f);
    const float v = -2.0f * (w < 0.00390625f ? series : __logf(u1));
    const float r = v > 0.0f ? v * rsqrtf(v) : 0.0f;
    // angle 2 pi u2 written as (2 pi u2 - pi) + pi to stay in [-pi, pi)
    const float th = fmaf((float)y, two_m32 * 6.283185307179586f, -3.141592653589793f);
    float s, c;
    __sincosf(th, &s, &c);
    return make_float2(-r * c, -r * s);
}

// Unit complex normal of the words (x, y) in the working precision.
template <class R, class C2>
__device__ __forceinline__ C2 unit_normal(uint32_t x, uint32_t y) {
    C2 z;
    if constexpr (sizeof(R) == 8) {
        const double2 g = box_muller64(x, y);
        z.x = (R)g.x; z.y = (R)g.y;
    } else {
        const float2 g = box_muller32(x, y);
        z.x = (R)g.x; z.y = (R)g.y;
    }
    return z;
}

__device__ __forceinline__ double2 philox_normal64(uint64_t seed, uint32_t chain, uint64_t step,
                                                   int comp, uint32_t site) {
    const uint4 o = philox_block(seed, chain, step, comp >> 1, site);
    return (comp & 1) ? box_muller64(o.z, o.w) : box_muller64(o.x, o.y);
}

}  // namespace clv
