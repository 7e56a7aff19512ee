/*
 * clv.h -- C ABI of the GB300-native complex-Langevin engine (libclv.so).
 *
 * One engine holds a batch of independent chains on one GPU.  Every chain has
 * its own lattice size, couplings, adaptive step and noise stream; one call
 * advances all of them.  Plain pointers and sizes only: no CUDA or C++ types
 * cross this boundary (a CUDA stream is passed as void*).
 *
 * Field layout at this boundary is the reference's (Lattice.cu:2-5):
 *   element (c, tau, x, y, z) of a chain at ((c*NT + tau)*NX + x)*NY*NZ + y*NZ + z,
 *   complex128 interleaved (re, im), C = 4 (reference model) or 3 (spin-1).
 * External noise layout is the reference's ind_rand (Lattice.cu:7-11):
 *   ((((c*NX + x)*NY + y)*NZ + z)*NT + tau)*2 + part, unit-variance normals;
 *   chains are concatenated in chain order.
 *
 * Every entry point returns a clv_status; clv_last_error() gives the message
 * of the last failure on the calling thread.
 */
#ifndef CLV_H
#define CLV_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CLV_API_VERSION 1

typedef struct clv_engine clv_engine;

typedef enum clv_status {
    CLV_OK = 0,
    CLV_ERR_ARG = 1,         /* invalid argument or configuration */
    CLV_ERR_CUDA = 2,        /* a CUDA runtime call failed */
    CLV_ERR_NONFINITE = 3,   /* a chain's drift became non-finite */
    CLV_ERR_TIMEOUT = 4,     /* a bounded device-side wait gave up */
    CLV_ERR_STATE = 5,       /* call not valid in the engine's current state */
    CLV_ERR_NOMEM = 6,       /* device or host allocation failed */
    CLV_ERR_IO = 7           /* checkpoint / file error */
} clv_status;

/* Physics model, kinetic factor, step rule, noise source, precision. */
enum { CLV_MODEL_REF4 = 0, CLV_MODEL_SPIN1 = 1 };
enum { CLV_KIN_REF_LINEAR_PX = 0, CLV_KIN_EXP = 1 };
enum { CLV_DT_REF_MEANMAX = 0, CLV_DT_K_OVER_MAX = 1 };
enum { CLV_NOISE_EXTERNAL = 0, CLV_NOISE_PHILOX = 1 };
enum { CLV_PREC_F64 = 0, CLV_PREC_F32 = 1 };
/* where a buffer lives; field transfers may add CLV_C64 (complex64 elements
 * instead of complex128, same layout) and CLV_ASYNC (enqueue the copies on the
 * engine's stream and return at once: the buffer must stay valid and, for a
 * get, is filled only after clv_synchronize or later work on that stream) */
enum { CLV_HOST = 0, CLV_DEVICE = 1, CLV_C64 = 2, CLV_ASYNC = 4 };
/* per-chain status flags (clv_get_chain_flags) */
enum { CLV_FLAG_NONFINITE = 1, CLV_FLAG_DT_CLAMPED_LOW = 2, CLV_FLAG_DT_CLAMPED_HIGH = 4,
       CLV_FLAG_TIMEOUT = 8 };

/* Per-chain parameters.  Reference-model names follow Parameters.h and
 * params.txt (XSIZE.., EPS, a_x, G, Q, DT; mu, P, seed). */
typedef struct clv_chain_params {
    int nx, ny, nz, nt;
    double eps;          /* imaginary-time step, beta = eps * nt */
    double a_x;          /* lattice spacing factor of the reference drift */
    double mu;           /* chemical potential */
    /* reference 4-component model */
    double P, Q, G;      /* Zeeman-like P, Q and contact coupling G */
    double DT;           /* base Langevin step */
    double dt_min, dt_max_clamp, alpha; /* 1e-8, 0.01, 0.9 in the reference */
    /* spin-1 model */
    double c0, c1, q;    /* density and spin couplings, quadratic Zeeman q */
    double K;            /* step rule dt = min(dt_max, K / max|drift|) */
    double dt_max;
    uint64_t seed;       /* Philox key of this chain's noise stream */
} clv_chain_params;

typedef struct clv_config {
    int model, kinetic, dt_rule, noise, precision;
    int device;          /* CUDA device ordinal */
    int nchains;
    const clv_chain_params *chains;
} clv_config;

/* Fill *p with the reference's defaults (Parameters.h, Propagator_without_cutoff.cu:382-404). */
void clv_default_chain_params(clv_chain_params *p);

/* Lifetime.  Replaces the allocations of main.cu:217-229
 * (new ComplexLattice x2, new Propagator, new Observables). */
int clv_create(const clv_config *cfg, clv_engine **out);
int clv_destroy(clv_engine *e);
const char *clv_last_error(void);
const char *clv_status_string(int status);
int clv_version(void);

/* Stream used for all work of the engine (default: the engine's own stream).
 * The pointer is a cudaStream_t. */
int clv_set_stream(clv_engine *e, void *stream);
int clv_synchronize(clv_engine *e);

/* Fields of one chain in the boundary layout (complex128, or complex64 with
 * where | CLV_C64: no conversion for an FP32 engine); chain = -1 moves every chain
 * at once, concatenated in chain order.  where = CLV_HOST or CLV_DEVICE.  Replaces ComplexLattice::get_pointer and
 * ComplexLatticeHost::copy_from_device / copy_to_device (Lattice.cu:217-220,460-468). */
int clv_set_fields(clv_engine *e, int chain, const void *psi, const void *psic, int where);
int clv_get_fields(clv_engine *e, int chain, void *psi, void *psic, int where);

/* ComplexLattice::set_mean_field (Lattice.cu:190-195, kernel set_value :50-81)
 * for every chain: field 0 = psi, 1 = psibar (gets the conjugate value). */
int clv_set_mean_field(clv_engine *e, int field, double re, double im);

/* Change the chemical potential mu and the Zeeman-like P of one chain (or of
 * every chain when chain = -1) between steps.  The reference passes both to
 * every Propagator::propagate(P, MU) call (Propagator_without_cutoff.cu:406). */
int clv_set_chemical_potential(clv_engine *e, int chain, double mu, double P);

/* Spin-1 start: every component of psi = amp + sigma*(xi_re + i xi_im) from the
 * chain's Philox stream, psibar = conj(psi). */
int clv_init_spin1(clv_engine *e, double amp, double sigma);

/* One Langevin step of every chain with the engine's own noise (Philox),
 * repeated nsteps times, enqueued on the engine's stream without a host
 * synchronisation: the steps are replayed from captured CUDA graphs, or, for
 * problems whose one-imaginary-time tasks all fit on the GPU at once (the
 * reference's own 256 x 32 lattice), run by one cooperative launch for up to
 * 2^16 steps (same results; the environment variable CLV_NO_LOOP=1 selects the
 * graphs).  Replaces Propagator::propagate (Propagator_without_cutoff.cu:406-442). */
int clv_step(clv_engine *e, int nsteps);

/* One step with injected standard normals in the reference's ind_rand layout,
 * all chains concatenated (float64, 2*C*V*T per chain); scaled by sqrt(dt) on
 * the device, as curandGenerateNormalDouble(gen, buf, n, 0, sqrt(dt)) does at
 * Propagator_without_cutoff.cu:432. */
int clv_step_with_noise(clv_engine *e, const double *noise, int where);

/* One Philox step with CUDA events recorded on the engine's stream between its
 * launches; phase_ms[i] receives the device time of launch i (kinetic filter
 * passes in axis order, then the drift, then the update) and *nphases their
 * number.  Used by the benchmark for the per-kernel roofline. */
int clv_step_timed(clv_engine *e, float *phase_ms, int capacity, int *nphases);

/* Last step's dt, max|drift| and mean|drift| per chain (arrays of nchains, any
 * may be NULL), Langevin time and step count.  Replaces
 * get_max_and_mean_drift / compute_new_dt (:351-404). */
int clv_get_step_info(clv_engine *e, double *dt, double *max_drift, double *mean_drift,
                      double *langevin_time, uint64_t *steps);
/* Per-chain CLV_FLAG_* bits (array of nchains); returns CLV_ERR_TIMEOUT when a
 * bounded device-side wait of some chain gave up (that chain's step is
 * incomplete; the other chains are unaffected), else CLV_ERR_NONFINITE when a
 * chain's drift became non-finite, else CLV_OK. */
int clv_get_chain_flags(clv_engine *e, int *flags);

/* Observables::evaluate (Observables_without_cutoff.cu:1155-1524): accumulate
 * the configured observables of every chain on the device. */
int clv_evaluate(clv_engine *e);
/* Number of evaluate() calls so far (Observables::get_counter, :1671-1674). */
int clv_get_counter(clv_engine *e);

/* Reference observables of one chain, normalised as Observables::write_*
 * (:1527-1547, :1614-1634): n[5] = n_tot, n_11, n_12, n_21, n_22;
 * F_x, F_y, F_z: V values each (any may be NULL). */
int clv_read_ref_observables(clv_engine *e, int chain, double *n, double *F_x,
                             double *F_y, double *F_z);

/* Spin-1 observable samples of one chain: samples[k*8 + j] for evaluate call k,
 * j = {density re, im, F_z re, im, F^2 re, im, energy re, im} (per-site
 * averages over the lattice and tau, FP64).  *count receives the number of
 * samples written (at most capacity). */
int clv_read_spin1_samples(clv_engine *e, int chain, double *samples, int capacity,
                           int *count);

/* Binary checkpoint of the fields, step state and observable accumulators. */
int clv_save_checkpoint(clv_engine *e, const char *path);
int clv_load_checkpoint(clv_engine *e, const char *path);

/* Device bytes held by the engine. */
int clv_device_bytes(clv_engine *e, size_t *bytes);

/* The kernel plan the engine chose for a step, as a NUL-terminated string
 * "<path>:<phase>,<phase>,...": path "fused" (every slice in shared memory),
 * "tiled" (axis filters, then the streaming step) or "unfused" (line filters,
 * drift, update); the phases in the order clv_step_timed reports them. */
int clv_get_plan(clv_engine *e, char *buf, int capacity);

/* Autotuner: times trial_steps steps of each candidate plan of the engine's path
 * (chunk of 1-64 imaginary times per CTA; for the fused path also bulk copies on/off
 * and the compile-time line plan on/off) and keeps the fastest.  The state
 * (fields, dt, step counters) is saved before and restored after every trial,
 * so a run continues exactly as without the call (for the reference's mean-based
 * dt rule up to the order of its sum).  Allocates a copy of the state while it
 * runs.  report (may be NULL) receives one line per candidate and the choice. */
int clv_autotune(clv_engine *e, int trial_steps, char *report, int capacity);

/* Arithmetic rates of `device` that the FP64 path's roofline is quoted against:
 * FP64 and FP32 fused multiply-add throughput in TFLOP/s (2 flops per FMA),
 * measured by independent FMA chains over 4 CTAs of 256 threads per SM, best of
 * 5 launches.  Either output may be NULL.  Takes about a millisecond; allocates
 * a small sink buffer.  No counterpart in the reference (it reports no rates). */
int clv_measure_peaks(int device, double *fp64_tflops, double *fp32_tflops);

/* Reference observables of ONE field configuration, with no engine and no
 * allocation.  No counterpart in the reference: it is for callers that must not
 * allocate device memory where they measure -- an application whose device
 * memory budget is already spent, a library routine that promises its caller
 * no allocation, or code that holds no engine.  psi, psic: device, complex128 (16-byte aligned), the boundary layout
 * above with C = 4; n: device, 5 doubles (n_tot, n_11, n_12, n_21, n_22); F:
 * device, 3*V doubles (F_x, F_y, F_z profiles), V = nx*ny*nz.  The values are
 * those clv_read_ref_observables returns after one clv_evaluate of the same
 * configuration.  Runs asynchronously on `stream` (NULL: the default stream)
 * on the calling thread's current device, which must hold the buffers.
 * Limit: V <= 1,048,576 sites; larger lattices return CLV_ERR_ARG.
 * The cross-CTA sums use a fixed 164,096-byte device array inside libclv.so,
 * shared by every call on a device and keeping the last call's contents; each
 * call clears what must start at zero.  Calls that overlap on the GPU (other
 * streams, other host threads, same device) race on that array: order them.
 * The first call on each device looks the array up (cudaGetSymbolAddress)
 * and keeps the address for the life of the process; make that first call
 * before any stream capture begins.  After cudaDeviceReset the kept address is
 * no longer valid: do not call this entry point again in that process. */
int clv_ref_observables_noalloc(const void *psi, const void *psic, int nx, int ny, int nz,
                                int nt, double a_x, double *n, double *F, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* CLV_H */
