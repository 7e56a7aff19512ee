/*
 * clv_oracle.h -- CPU restatement (FP64, C11 + OpenMP) of one complex-Langevin
 * step and its observables.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA engine
 * and the timed CPU baseline in bench.py; nothing in the product path
 * (cl_var_dt_gb300/) links, loads or calls it.
 *
 * Two models are restated:
 *  - REF4: the reference's 4-component model, following
 *      Propagator_without_cutoff.cu:1-203   (drift, dt multiply, noise, kinetic)
 *      Propagator_without_cutoff.cu:231-265,351-404 (max/mean drift, new dt)
 *      Propagator_without_cutoff.cu:406-442 (step order)
 *      Lattice.cu:2-11,32-81,135-214        (layout, elementwise kernels, FFT)
 *      Observables_without_cutoff.cu:35-101,456-488,1155-1382 (F profiles, n_ij)
 *    Parity is pinned by the golden vectors in tests/golden/, generated from the
 *    reference's own kernel sources (see oracle/ref_build.sh).
 *  - SPIN1: spin-1 Bose gas with an exponential kinetic factor, the K/max|drift|
 *    step rule and Philox noise.  The reference has no such model: parity is
 *    unpinned for it and the oracle is the project's own restatement.
 *
 * Layout of every field array (reference layout, Lattice.cu:2-5):
 *   element (c, tau, x, y, z) at ((c*NT + tau)*NX + x)*NY*NZ + y*NZ + z,
 *   complex128 interleaved (re, im).
 * Layout of an external noise buffer (reference ind_rand, Lattice.cu:7-11):
 *   ((((c*NX + x)*NY + y)*NZ + z)*NT + tau)*2 + part, unit-variance normals.
 */
#ifndef CLV_ORACLE_H
#define CLV_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_MODEL_REF4 = 0, ORC_MODEL_SPIN1 = 1 };
enum { ORC_KIN_REF_LINEAR_PX = 0, ORC_KIN_EXP = 1 };
enum { ORC_DT_REF_MEANMAX = 0, ORC_DT_K_OVER_MAX = 1 };

typedef struct orc_params {
    int nx, ny, nz, nt, ncomp;
    int model, kinetic, dt_rule;
    /* reference model (Parameters.h names) */
    double eps, a_x, G, Q, P, mu, DT, dt_min, dt_max_clamp, alpha;
    /* spin-1 model */
    double c0, c1, q, Kc, dt_max;
} orc_params;

/* One 1D DFT of length n on a strided line, in place, unnormalised.
 * sign = -1: X_k = sum_j x_j exp(-2 pi i jk/n);  sign = +1: exp(+2 pi i jk/n). */
void orc_fft_line(double *re_im, int n, long stride, int sign);

/* Kinetic term kin = K[psi] for both fields (all comps, all tau). */
void orc_kinetic(const orc_params *p, const double *psi, const double *psic,
                 double *kin, double *kinc);

/* Drift K, Kbar from fields and kinetic terms (factor = 1 in propagate). */
void orc_drift(const orc_params *p, const double *psi, const double *psic,
               const double *kin, const double *kinc, double *drift,
               double *driftc, double factor);

/* Reduction feeding the step rule.  REF rule: max and mean of |K| over the
 * first V*T entries of the psi drift, mean divided by C*V*T (reference quirk).
 * K/max rule: max over all entries of both drifts; mean = 0. */
void orc_max_mean(const orc_params *p, const double *drift, const double *driftc,
                  double *max_out, double *mean_out);

/* New Langevin step from the reduction (both rules). */
double orc_new_dt(const orc_params *p, double mean, double max, int *clamped);

/* Philox4x32-10 (Salmon et al., SC'11). */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* Unit complex normal (re, im) of the engine's Philox noise stream for a
 * given (seed, chain, step, component, site index tau*V + s). */
void orc_philox_normal(uint64_t seed, uint32_t chain, uint64_t step, int comp,
                       uint32_t site, double *re, double *im);

/* The engine's step noise of component comp of ncomp at linear site `site`: the
 * pair's block at the site, or, for the last component of an odd count, the block of
 * site / 2 shared with the neighbouring site (words by site parity). */
void orc_philox_step_normal(uint64_t seed, uint32_t chain, uint64_t step, int comp, int ncomp,
                            uint32_t site, double *re, double *im);

/* Fill a noise buffer (reference ind_rand layout, unit normals) from Philox. */
void orc_philox_noise_buffer(const orc_params *p, uint64_t seed, uint32_t chain,
                             uint64_t step, double *noise);

/* psi += dt*K + sqrt(dt)*xi, psic += dt*Kbar + sqrt(dt)*conj(xi). */
void orc_update(const orc_params *p, double *psi, double *psic,
                const double *drift, const double *driftc,
                const double *noise, double dt);

/* One full step: kinetic, drift, reduction, dt, update.  noise: external
 * buffer (reference layout); when NULL, Philox(seed, chain, step) is used.
 * Returns dt; max_out and mean_out receive the reduction values. */
double orc_step(const orc_params *p, double *psi, double *psic,
                const double *noise, uint64_t seed, uint32_t chain,
                uint64_t step, double *max_out, double *mean_out);

/* Reference observables of one evaluate() call, un-normalised per-call sums:
 * F[3*V]      : F_x, F_y, F_z real-space profiles summed over tau
 *               (Observables_without_cutoff.cu:456-488)
 * n[5]        : n_tot, n_11, n_12, n_21, n_22 sums a_x*V*sum Re(psic(tau+1) psi(tau))
 *               (the reference's k-space sums, Observables_without_cutoff.cu:35-101,1322-1382,
 *                equal to the real-space sums by Parseval). */
void orc_ref_observables(const orc_params *p, const double *psi, const double *psic,
                         double *F, double *n);

/* Spin-1 observables of one configuration, averaged over sites and tau.
 * out[8] = {density re, im, F_z re, im, F^2 re, im, energy re, im}. */
void orc_spin1_observables(const orc_params *p, const double *psi,
                           const double *psic, double *out);

/* Initial state: REF set_value (Lattice.cu:50-81) with value v (comps 0,3 = v,
 * comps 1,2 = (2/3) v, conj field gets conj(v)). */
void orc_set_mean_field(const orc_params *p, double *field, double re, double im,
                        int conjugated);

/* Spin-1 start: psi = amp + sigma (xi_re + i xi_im) from Philox at step 2^64-1,
 * psibar = conj(psi). */
void orc_spin1_init(const orc_params *p, uint64_t seed, uint32_t chain, double amp,
                    double sigma, double *psi, double *psic);

int orc_num_threads(void);
/* Threads of the OpenMP loops (test infrastructure: timing with 1 and all cores). */
void orc_set_num_threads(int n);

#ifdef __cplusplus
}
#endif
#endif
