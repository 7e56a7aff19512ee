/*
 * clv_oracle.c -- FP64 CPU restatement of the complex-Langevin step.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA engine and the CPU
 * baseline timed by bench.py.  The product path never links or loads it.
 * Every function names the reference lines it restates; the interface and
 * layouts are documented in clv_oracle.h.
 */
#include "clv_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ------------------------------------------------------------------ helpers */
typedef struct { double re, im; } cplx;

static inline cplx cmk(double r, double i) { cplx z = {r, i}; return z; }
static inline cplx cadd(cplx a, cplx b) { return cmk(a.re + b.re, a.im + b.im); }
static inline cplx csub(cplx a, cplx b) { return cmk(a.re - b.re, a.im - b.im); }
/* cuCmul ordering (cuComplex.h): (a.re b.re - a.im b.im, a.re b.im + a.im b.re) */
static inline cplx cmul(cplx a, cplx b) {
    return cmk(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
static inline cplx cscale(double s, cplx a) { return cmk(s * a.re, s * a.im); }
static inline cplx cld(const double *f, long i) { return cmk(f[2 * i], f[2 * i + 1]); }
static inline void cst(double *f, long i, cplx v) { f[2 * i] = v.re; f[2 * i + 1] = v.im; }

void orc_set_num_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

static inline long vol(const orc_params *p) { return (long)p->nx * p->ny * p->nz; }
/* ind() of Lattice.cu:2-5 with the periodic wrap of my_map (Helpers.cu:1-15). */
static inline long fidx(const orc_params *p, int c, int tau, long s) {
    int t = tau;
    if (t < 0) t += p->nt;
    else if (t >= p->nt) t -= p->nt;
    return ((long)c * p->nt + t) * vol(p) + s;
}

/* -------------------------------------------------------------------- FFT */
/* Mixed-radix Stockham autosort FFT on one line (any length; prime factors
 * handled by a direct DFT of that radix).  Unnormalised; sign selects the
 * exponent sign exactly as cuFFT's CUFFT_FORWARD (-1) / CUFFT_INVERSE (+1). */
static int factorize(int n, int *f) {
    int k = 0;
    while (n % 4 == 0) { f[k++] = 4; n /= 4; }
    while (n % 2 == 0) { f[k++] = 2; n /= 2; }
    for (int r = 3; n > 1; r += 2)
        while (n % r == 0) { f[k++] = r; n /= r; }
    return k;
}

/* w[k] = exp(sign 2 pi i k / n), k < n: every twiddle and small-DFT root of
 * the transform is one entry of this table. */
static void twiddle_table(cplx *w, int n, int sign) {
    for (int k = 0; k < n; ++k) {
        double ang = sign * 2.0 * M_PI * (double)k / (double)n;
        w[k] = cmk(cos(ang), sin(ang));
    }
}

static void fft_line_contig_tw(cplx *a, cplx *tmp, int n, const cplx *w) {
    if (n <= 1) return;
    int f[40];
    int nf = factorize(n, f);
    cplx *src = a, *dst = tmp;
    int Ns = 1;
    cplx v[64], o[64];
    for (int fi = 0; fi < nf; ++fi) {
        const int R = f[fi];
        const int nR = n / R;
        const int tstep = n / (Ns * R); /* twiddle k*r/(Ns R) of a turn */
        for (int j = 0; j < nR; ++j) {
            const int k = j % Ns;
            for (int r = 0; r < R; ++r) v[r] = cmul(src[j + r * nR], w[(k * r * tstep) % n]);
            for (int q = 0; q < R; ++q) {
                cplx acc = cmk(0.0, 0.0);
                for (int r = 0; r < R; ++r) acc = cadd(acc, cmul(v[r], w[((r * q) % R) * nR]));
                o[q] = acc;
            }
            const int idxD = (j / Ns) * Ns * R + k;
            for (int q = 0; q < R; ++q) dst[idxD + q * Ns] = o[q];
        }
        cplx *t = src; src = dst; dst = t;
        Ns *= R;
    }
    if (src != a) memcpy(a, src, sizeof(cplx) * (size_t)n);
}

static void fft_line_contig(cplx *a, cplx *tmp, int n, int sign) {
    cplx *w = (cplx *)malloc(sizeof(cplx) * (size_t)(n > 0 ? n : 1));
    twiddle_table(w, n, sign);
    fft_line_contig_tw(a, tmp, n, w);
    free(w);
}

void orc_fft_line(double *re_im, int n, long stride, int sign) {
    cplx *line = (cplx *)malloc(sizeof(cplx) * (size_t)n * 2);
    for (int i = 0; i < n; ++i) line[i] = cld(re_im, (long)i * stride);
    fft_line_contig(line, line + n, n, sign);
    for (int i = 0; i < n; ++i) cst(re_im, (long)i * stride, line[i]);
    free(line);
}

/* Full multi-dimensional transform of one [X][Y][Z] slice (cuFFT planMany
 * over rank 1/2/3, Lattice.cu:135-156; all spatial axes transformed). */
static int max_extent(const orc_params *p) {
    int m = p->nx > p->ny ? p->nx : p->ny;
    return p->nz > m ? p->nz : m;
}

/* buf: 3 * max_extent(p) complex values (line, scratch, twiddles). */
static void fft_slice(const orc_params *p, double *slice, int sign, cplx *buf) {
    const int X = p->nx, Y = p->ny, Z = p->nz, L = max_extent(p);
    cplx *line = buf, *tmp = buf + L, *w = buf + 2 * L;
    if (Z > 1) {
        twiddle_table(w, Z, sign);
        for (long xy = 0; xy < (long)X * Y; ++xy) {
            for (int z = 0; z < Z; ++z) line[z] = cld(slice, xy * Z + z);
            fft_line_contig_tw(line, tmp, Z, w);
            for (int z = 0; z < Z; ++z) cst(slice, xy * Z + z, line[z]);
        }
    }
    if (Y > 1) {
        twiddle_table(w, Y, sign);
        for (int x = 0; x < X; ++x)
            for (int z = 0; z < Z; ++z) {
                for (int y = 0; y < Y; ++y) line[y] = cld(slice, ((long)x * Y + y) * Z + z);
                fft_line_contig_tw(line, tmp, Y, w);
                for (int y = 0; y < Y; ++y) cst(slice, ((long)x * Y + y) * Z + z, line[y]);
            }
    }
    if (X > 1) {
        twiddle_table(w, X, sign);
        for (long yz = 0; yz < (long)Y * Z; ++yz) {
            for (int x = 0; x < X; ++x) line[x] = cld(slice, (long)x * Y * Z + yz);
            fft_line_contig_tw(line, tmp, X, w);
            for (int x = 0; x < X; ++x) cst(slice, (long)x * Y * Z + yz, line[x]);
        }
    }
}

/* Signed lattice momentum of compute_kinetic_part (Propagator_without_cutoff.cu:169-194). */
static inline double pmom(int j, int L) {
    if (j < L / 2 || L == 1) return 2. * M_PI * (double)j / (double)L;
    return -2. * M_PI * (double)(L - j) / (double)L;
}

/* ---------------------------------------------------------------- kinetic */
/* REF: kin = normalize(fft_inv(-px^2 * fft(psi)), 1/(a_x V))
 *   (Propagator_without_cutoff.cu:410-424, 160-203; Lattice.cu:158-187).
 *   psi's fft() is CUFFT_INVERSE, psic's is CUFFT_FORWARD; fft_inv the opposite.
 * EXP: kin_m = F^-1[ exp(-eps (k^2/2 - mu - q m^2)) F psi_m ] / V, m = 1 - c. */
void orc_kinetic(const orc_params *p, const double *psi, const double *psic,
                 double *kin, double *kinc) {
    const long V = vol(p);
    const int X = p->nx, Y = p->ny, Z = p->nz;
    const int nslices = p->ncomp * p->nt;
    const size_t bytes = sizeof(double) * 2 * (size_t)V * nslices;
    memcpy(kin, psi, bytes);
    memcpy(kinc, psic, bytes);
    const int maxl = max_extent(p);
#pragma omp parallel
    {
        cplx *buf = (cplx *)malloc(sizeof(cplx) * 3 * (size_t)maxl);
#pragma omp for schedule(static)
        for (int sl = 0; sl < 2 * nslices; ++sl) {
            const int conj = sl >= nslices;
            const int cs = conj ? sl - nslices : sl;
            const int comp = cs / p->nt;
            double *slice = (conj ? kinc : kin) + 2 * (size_t)V * cs;
            if (p->kinetic == ORC_KIN_REF_LINEAR_PX) {
                fft_slice(p, slice, conj ? -1 : +1, buf);
                for (int x = 0; x < X; ++x) {
                    double px = pmom(x, X);
                    double p2 = px * px; /* +py*py+pz*pz commented out in the reference */
                    for (long yz = 0; yz < (long)Y * Z; ++yz) {
                        long i = (long)x * Y * Z + yz;
                        cst(slice, i, cscale(-p2, cld(slice, i)));
                    }
                }
                fft_slice(p, slice, conj ? +1 : -1, buf);
                double nf = 1. / (double)(p->a_x * X * Y * Z);
                for (long i = 0; i < V; ++i) cst(slice, i, cscale(nf, cld(slice, i)));
            } else {
                const double m = (double)(1 - comp);
                fft_slice(p, slice, -1, buf);
                for (int x = 0; x < X; ++x)
                    for (int y = 0; y < Y; ++y)
                        for (int z = 0; z < Z; ++z) {
                            double kx = pmom(x, X), ky = pmom(y, Y), kz = pmom(z, Z);
                            double k2 = kx * kx + ky * ky + kz * kz;
                            double e = exp(-p->eps * (0.5 * k2 - p->mu - p->q * m * m)) / (double)V;
                            long i = ((long)x * Y + y) * Z + z;
                            cst(slice, i, cscale(e, cld(slice, i)));
                        }
                fft_slice(p, slice, +1, buf);
            }
        }
        free(buf);
    }
}

/* ------------------------------------------------------------------ drift */
/* REF4 drift: calculate_drift_without_noise, Propagator_without_cutoff.cu:1-129. */
static void drift_ref4_site(const orc_params *p, const double *psi, const double *psic,
                            const double *kin, const double *kinc, double *drift,
                            double *driftc, double factor, int tau, long s) {
    cplx pm[4], pc[4], cc[4], cp[4];
    for (int a = 0; a < 4; ++a) {
        pm[a] = cld(psi, fidx(p, a, tau - 1, s));
        pc[a] = cld(psi, fidx(p, a, tau, s));
        cc[a] = cld(psic, fidx(p, a, tau, s));
        cp[a] = cld(psic, fidx(p, a, tau + 1, s));
    }
    cplx N[4], Nc[4];
    for (int a = 0; a < 4; ++a) { N[a] = cmul(pm[a], cc[a]); Nc[a] = cmul(pc[a], cp[a]); }
    cplx tm[4], tp[4];
    tm[0] = cadd(cmul(cadd(cadd(N[0], N[1]), N[2]), pm[0]), cmul(cmul(pm[1], cc[3]), pm[2]));
    tm[1] = cadd(cmul(cadd(cadd(N[0], N[1]), N[3]), pm[1]), cmul(cmul(pm[0], cc[2]), pm[3]));
    tm[2] = cadd(cmul(cadd(cadd(N[0], N[2]), N[3]), pm[2]), cmul(cmul(pm[3], cc[1]), pm[0]));
    tm[3] = cadd(cmul(cadd(cadd(N[1], N[2]), N[3]), pm[3]), cmul(cmul(pm[2], cc[0]), pm[1]));
    tp[0] = cadd(cmul(cadd(cadd(Nc[0], Nc[1]), Nc[2]), cp[0]), cmul(cmul(cp[1], pc[3]), cp[2]));
    tp[1] = cadd(cmul(cadd(cadd(Nc[0], Nc[1]), Nc[3]), cp[1]), cmul(cmul(cp[0], pc[2]), cp[3]));
    tp[2] = cadd(cmul(cadd(cadd(Nc[0], Nc[2]), Nc[3]), cp[2]), cmul(cmul(cp[3], pc[1]), cp[0]));
    tp[3] = cadd(cmul(cadd(cadd(Nc[1], Nc[2]), Nc[3]), cp[3]), cmul(cmul(cp[2], pc[0]), cp[1]));
    const double Vpot = 0.;
    double mu[4];
    mu[0] = p->mu - Vpot + p->P + p->Q;
    mu[1] = p->mu - Vpot;
    mu[2] = p->mu - Vpot;
    mu[3] = p->mu - Vpot - p->P + p->Q;
    const double pre = p->a_x * factor;
    const cplx zero = cmk(0., 0.);
    for (int a = 0; a < 4; ++a) {
        cplx km = cld(kin, fidx(p, a, tau - 1, s));
        cplx kp = cld(kinc, fidx(p, a, tau + 1, s));
        cplx tpar = cadd(zero, cscale(mu[a], pm[a]));
        cplx tint = csub(zero, cscale(2 * p->G, tm[a]));
        cplx d = cscale(pre, cadd(csub(pm[a], pc[a]), cscale(p->eps, cadd(cadd(tpar, tint), km))));
        cst(drift, fidx(p, a, tau, s), d);
        /* Quirk kept for parity: the chemical-potential term of the conjugate
         * drift multiplies psi(tau+1), not psibar(tau+1)
         * (Propagator_without_cutoff.cu:71,88,105,122). */
        tpar = cadd(zero, cscale(mu[a], cld(psi, fidx(p, a, tau + 1, s))));
        tint = csub(zero, cscale(2 * p->G, tp[a]));
        d = cscale(pre, cadd(csub(cp[a], cc[a]), cscale(p->eps, cadd(cadd(tpar, tint), kp))));
        cst(driftc, fidx(p, a, tau, s), d);
    }
}

/* Spin-1 contact terms.  For fields bar (row vector) and ket (column vector):
 *   n = sum_m bar_m ket_m, Fz = bar_+ ket_+ - bar_- ket_-,
 *   F+ = sqrt2 (bar_+ ket_0 + bar_0 ket_-), F- = sqrt2 (bar_0 ket_+ + bar_- ket_0),
 *   V = c0/2 n^2 + c1/2 (Fz^2 + F+ F-).
 * dV/dbar_m -> out_ket[m]; dV/dket_m -> out_bar[m]. */
static void spin1_contact(double c0, double c1, const cplx *bar, const cplx *ket,
                          cplx *dbar, cplx *dket) {
    const double r2 = sqrt(2.0), ir2 = 1.0 / sqrt(2.0);
    cplx n = cadd(cadd(cmul(bar[0], ket[0]), cmul(bar[1], ket[1])), cmul(bar[2], ket[2]));
    cplx Fz = csub(cmul(bar[0], ket[0]), cmul(bar[2], ket[2]));
    cplx Fp = cscale(r2, cadd(cmul(bar[0], ket[1]), cmul(bar[1], ket[2])));
    cplx Fm = cscale(r2, cadd(cmul(bar[1], ket[0]), cmul(bar[2], ket[1])));
    if (dbar) {
        cplx s0 = cadd(cmul(Fz, ket[0]), cscale(ir2, cmul(Fm, ket[1])));
        cplx s1 = cscale(ir2, cadd(cmul(Fp, ket[0]), cmul(Fm, ket[2])));
        cplx s2 = cadd(cscale(-1.0, cmul(Fz, ket[2])), cscale(ir2, cmul(Fp, ket[1])));
        dbar[0] = cadd(cscale(c0, cmul(n, ket[0])), cscale(c1, s0));
        dbar[1] = cadd(cscale(c0, cmul(n, ket[1])), cscale(c1, s1));
        dbar[2] = cadd(cscale(c0, cmul(n, ket[2])), cscale(c1, s2));
    }
    if (dket) {
        cplx s0 = cadd(cmul(Fz, bar[0]), cscale(ir2, cmul(Fp, bar[1])));
        cplx s1 = cscale(ir2, cadd(cmul(Fm, bar[0]), cmul(Fp, bar[2])));
        cplx s2 = cadd(cscale(-1.0, cmul(Fz, bar[2])), cscale(ir2, cmul(Fm, bar[1])));
        dket[0] = cadd(cscale(c0, cmul(n, bar[0])), cscale(c1, s0));
        dket[1] = cadd(cscale(c0, cmul(n, bar[1])), cscale(c1, s1));
        dket[2] = cadd(cscale(c0, cmul(n, bar[2])), cscale(c1, s2));
    }
}

/* Spin-1 drift: K_m(tau) = kin_m(tau-1) - psi_m(tau) - eps dV/dpsibar_m(psibar(tau), psi(tau-1)),
 * Kbar_m(tau) = kinbar_m(tau+1) - psibar_m(tau) - eps dV/dpsi_m(psibar(tau+1), psi(tau)). */
static void drift_spin1_site(const orc_params *p, const double *psi, const double *psic,
                             const double *kin, const double *kinc, double *drift,
                             double *driftc, double factor, int tau, long s) {
    cplx pm[3], pc[3], cc[3], cp[3], dK[3], dKc[3];
    for (int a = 0; a < 3; ++a) {
        pm[a] = cld(psi, fidx(p, a, tau - 1, s));
        pc[a] = cld(psi, fidx(p, a, tau, s));
        cc[a] = cld(psic, fidx(p, a, tau, s));
        cp[a] = cld(psic, fidx(p, a, tau + 1, s));
    }
    spin1_contact(p->c0, p->c1, cc, pm, dK, NULL);
    spin1_contact(p->c0, p->c1, cp, pc, NULL, dKc);
    for (int a = 0; a < 3; ++a) {
        cplx km = cld(kin, fidx(p, a, tau - 1, s));
        cplx kp = cld(kinc, fidx(p, a, tau + 1, s));
        cplx d = csub(csub(km, pc[a]), cscale(p->eps, dK[a]));
        cst(drift, fidx(p, a, tau, s), cscale(factor, d));
        d = csub(csub(kp, cc[a]), cscale(p->eps, dKc[a]));
        cst(driftc, fidx(p, a, tau, s), cscale(factor, d));
    }
}

void orc_drift(const orc_params *p, const double *psi, const double *psic,
               const double *kin, const double *kinc, double *drift,
               double *driftc, double factor) {
    const long V = vol(p);
#pragma omp parallel for schedule(static)
    for (int tau = 0; tau < p->nt; ++tau)
        for (long s = 0; s < V; ++s) {
            if (p->model == ORC_MODEL_REF4)
                drift_ref4_site(p, psi, psic, kin, kinc, drift, driftc, factor, tau, s);
            else
                drift_spin1_site(p, psi, psic, kin, kinc, drift, driftc, factor, tau, s);
        }
}

/* -------------------------------------------------------------- step rule */
/* REF: compute_max_and_mean_drift over total_size = C*V*T entries but launched
 * with only V*T threads (Propagator_without_cutoff.cu:231-265,351-380), so the
 * max/sum cover drift entries [0, V*T) = component 0; mean = sum/(C*V*T). */
void orc_max_mean(const orc_params *p, const double *drift, const double *driftc,
                  double *max_out, double *mean_out) {
    const long V = vol(p);
    double mx = 0.0, sum = 0.0;
    if (p->dt_rule == ORC_DT_REF_MEANMAX) {
        const long n = V * p->nt;
        for (long i = 0; i < n; ++i) {
            double a = hypot(drift[2 * i], drift[2 * i + 1]);
            if (mx < a) mx = a;
            sum += a;
        }
        *max_out = mx;
        *mean_out = sum / (double)((long)p->ncomp * V * p->nt);
    } else {
        const long n = (long)p->ncomp * V * p->nt;
        for (long i = 0; i < n; ++i) {
            double a = hypot(drift[2 * i], drift[2 * i + 1]);
            double b = hypot(driftc[2 * i], driftc[2 * i + 1]);
            if (mx < a) mx = a;
            if (mx < b) mx = b;
        }
        *max_out = mx;
        *mean_out = 0.0;
    }
}

/* REF: compute_new_dt, Propagator_without_cutoff.cu:382-404.
 * K/max: dt = min(dt_max, K / max|drift|). */
double orc_new_dt(const orc_params *p, double mean, double max, int *clamped) {
    int cl = 0;
    double dt;
    if (p->dt_rule == ORC_DT_REF_MEANMAX) {
        if (max <= 0.0) dt = p->DT;
        else dt = (mean / max) * p->DT;
        if (dt < p->dt_min) { dt = p->dt_min; cl = 1; }
        if (dt > p->dt_max_clamp) { dt = p->dt_max_clamp; cl = 2; }
        dt = (1 - p->alpha) * p->DT + p->alpha * dt;
    } else {
        dt = p->dt_max;
        if (max > 0.0) {
            double t = p->Kc / max;
            if (t < dt) dt = t;
        }
    }
    if (clamped) *clamped = cl;
    return dt;
}

/* ------------------------------------------------------------------ noise */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c1 ^ k0, n1 = lo1, n2 = hi0 ^ c3 ^ k1, n3 = lo0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* Box-Muller (Box & Muller 1958).  One Philox block serves a component pair:
 * counter = {site, step_lo, step_hi, chain + (c/2) 2^24}, key = seed; words
 * (x0, x1) give component 2k, (x2, x3) component 2k+1, with
 * u1 = (x + 1/2) 2^-32 in (0,1), u2 = y 2^-32 in [0,1). */
void orc_philox_normal(uint64_t seed, uint32_t chain, uint64_t step, int comp, uint32_t site,
                       double *re, double *im) {
    uint32_t ctr[4] = {site, (uint32_t)step, (uint32_t)(step >> 32),
                       chain + ((uint32_t)(comp >> 1) << 24)};
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    uint32_t o[4];
    orc_philox4x32_10(ctr, key, o);
    const uint32_t x = (comp & 1) ? o[2] : o[0];
    const uint32_t y = (comp & 1) ? o[3] : o[1];
    const double two_m32 = 2.3283064365386963e-10;
    double u1 = ((double)x + 0.5) * two_m32;
    double u2 = (double)y * two_m32;
    double r = sqrt(-2.0 * log(u1));
    double th = 2.0 * M_PI * u2;
    *re = r * cos(th);
    *im = r * sin(th);
}

/* Step noise of component c at linear site `site` (tau V + s): the pair's block at
 * that site, except for the last component of an odd count (spin-1's third), whose
 * block is shared by the sites 2j and 2j + 1 (counter site j, words (x0, x1) for 2j
 * and (x2, x3) for 2j + 1) -- the engine's noise_words (clv_internal.cuh). */
void orc_philox_step_normal(uint64_t seed, uint32_t chain, uint64_t step, int comp, int ncomp,
                            uint32_t site, double *re, double *im) {
    if ((ncomp & 1) && comp == ncomp - 1)
        orc_philox_normal(seed, chain, step, (comp & ~1) | (int)(site & 1), site >> 1, re, im);
    else
        orc_philox_normal(seed, chain, step, comp, site, re, im);
}

void orc_philox_noise_buffer(const orc_params *p, uint64_t seed, uint32_t chain,
                             uint64_t step, double *noise) {
    const long V = vol(p);
#pragma omp parallel for schedule(static)
    for (int c = 0; c < p->ncomp; ++c)
        for (int tau = 0; tau < p->nt; ++tau)
            for (long s = 0; s < V; ++s) {
                uint32_t site = (uint32_t)((long)tau * V + s);
                double re, im;
                orc_philox_step_normal(seed, chain, step, c, p->ncomp, site, &re, &im);
                long r = (((long)c * V + s) * p->nt + tau) * 2;
                noise[r] = re;
                noise[r + 1] = im;
            }
}

/* ----------------------------------------------------------------- update */
/* multiply_by_timestep, add_noise, summation (Propagator_without_cutoff.cu:131-157,
 * Lattice.cu:32-36): d = dt*K; d += sqrt(dt) (z0 + i z1); psi += d;
 * dbar = dt*Kbar; dbar += sqrt(dt) (z0 - i z1); psibar += dbar. */
void orc_update(const orc_params *p, double *psi, double *psic, const double *drift,
                const double *driftc, const double *noise, double dt) {
    const long V = vol(p);
    const double sd = sqrt(dt);
#pragma omp parallel for schedule(static)
    for (int c = 0; c < p->ncomp; ++c)
        for (int tau = 0; tau < p->nt; ++tau)
            for (long s = 0; s < V; ++s) {
                long i = fidx(p, c, tau, s);
                long r = (((long)c * V + s) * p->nt + tau) * 2;
                double z0 = sd * noise[r], z1 = sd * noise[r + 1];
                cplx d = cmul(cld(drift, i), cmk(dt, 0.0));
                d = cadd(d, cmk(z0, z1));
                cst(psi, i, cadd(cld(psi, i), d));
                cplx dc = cmul(cld(driftc, i), cmk(dt, 0.0));
                dc = cadd(dc, cmk(z0, -z1));
                cst(psic, i, cadd(cld(psic, i), dc));
            }
}

double orc_step(const orc_params *p, double *psi, double *psic, const double *noise,
                uint64_t seed, uint32_t chain, uint64_t step, double *max_out,
                double *mean_out) {
    const size_t n = 2 * (size_t)p->ncomp * p->nt * vol(p);
    double *kin = (double *)malloc(sizeof(double) * n);
    double *kinc = (double *)malloc(sizeof(double) * n);
    double *drift = (double *)malloc(sizeof(double) * n);
    double *driftc = (double *)malloc(sizeof(double) * n);
    double *nz = NULL;
    orc_kinetic(p, psi, psic, kin, kinc);
    orc_drift(p, psi, psic, kin, kinc, drift, driftc, 1.0);
    double mx, mean;
    orc_max_mean(p, drift, driftc, &mx, &mean);
    double dt = orc_new_dt(p, mean, mx, NULL);
    if (!noise) {
        nz = (double *)malloc(sizeof(double) * n);
        orc_philox_noise_buffer(p, seed, chain, step, nz);
        noise = nz;
    }
    orc_update(p, psi, psic, drift, driftc, noise, dt);
    if (max_out) *max_out = mx;
    if (mean_out) *mean_out = mean;
    free(kin); free(kinc); free(drift); free(driftc); free(nz);
    return dt;
}

/* ------------------------------------------------------------ observables */
/* evaluate_spin_density_realspace (Observables_without_cutoff.cu:456-488) and
 * evaluate_n_tot / evaluate_n_11..22 (:35-101) reduced as in evaluate (:1322-1382). */
void orc_ref_observables(const orc_params *p, const double *psi, const double *psic,
                         double *F, double *n) {
    const long V = vol(p);
    memset(F, 0, sizeof(double) * 3 * (size_t)V);
    double nn[5] = {0, 0, 0, 0, 0};
    for (long s = 0; s < V; ++s) {
        double fx = 0, fy = 0, fz = 0;
        for (int tau = 0; tau < p->nt; ++tau) {
            cplx pc[4], cp[4];
            for (int a = 0; a < 4; ++a) {
                pc[a] = cld(psi, fidx(p, a, tau, s));
                cp[a] = cld(psic, fidx(p, a, tau + 1, s));
            }
            cplx t20 = cmul(cp[2], pc[0]), t02 = cmul(cp[0], pc[2]);
            cplx t31 = cmul(cp[3], pc[1]), t13 = cmul(cp[1], pc[3]);
            fx += cadd(cadd(cadd(t20, t02), t31), t13).re;
            cplx w = csub(cadd(csub(t20, t02), t31), t13);
            fy += cmul(cmk(0.0, 1.0), w).re;
            fz += csub(csub(cadd(cmul(cp[0], pc[0]), cmul(cp[1], pc[1])), cmul(cp[2], pc[2])),
                       cmul(cp[3], pc[3])).re;
            for (int a = 0; a < 4; ++a) {
                double d = cmul(cp[a], pc[a]).re * p->a_x;
                nn[0] += d;
                nn[1 + a] += d;
            }
        }
        F[s] = fx;
        F[V + s] = fy;
        F[2 * V + s] = fz;
    }
    for (int i = 0; i < 5; ++i) n[i] = nn[i] * (double)V;
}

/* Spin-1 observables with the point split (psibar(tau+1), psi(tau)); the
 * kinetic energy uses k^2/2 in Fourier space; one-body energy k^2/2 - q m^2. */
void orc_spin1_observables(const orc_params *p, const double *psi, const double *psic,
                           double *out) {
    const long V = vol(p);
    const int X = p->nx, Y = p->ny, Z = p->nz;
    const size_t n = 2 * (size_t)p->ncomp * p->nt * V;
    double *tk = (double *)malloc(sizeof(double) * n);
    memcpy(tk, psi, sizeof(double) * n);
    cplx *buf = (cplx *)malloc(sizeof(cplx) * 3 * (size_t)max_extent(p));
    for (int sl = 0; sl < p->ncomp * p->nt; ++sl) {
        double *slice = tk + 2 * (size_t)V * sl;
        fft_slice(p, slice, -1, buf);
        for (int x = 0; x < X; ++x)
            for (int y = 0; y < Y; ++y)
                for (int z = 0; z < Z; ++z) {
                    double kx = pmom(x, X), ky = pmom(y, Y), kz = pmom(z, Z);
                    double e = 0.5 * (kx * kx + ky * ky + kz * kz) / (double)V;
                    long i = ((long)x * Y + y) * Z + z;
                    cst(slice, i, cscale(e, cld(slice, i)));
                }
        fft_slice(p, slice, +1, buf);
    }
    free(buf);
    cplx dens = cmk(0, 0), fz = cmk(0, 0), f2 = cmk(0, 0), en = cmk(0, 0);
    const double r2 = sqrt(2.0);
    for (int tau = 0; tau < p->nt; ++tau)
        for (long s = 0; s < V; ++s) {
            cplx bar[3], ket[3], tket[3];
            for (int a = 0; a < 3; ++a) {
                bar[a] = cld(psic, fidx(p, a, tau + 1, s));
                ket[a] = cld(psi, fidx(p, a, tau, s));
                tket[a] = cld(tk, fidx(p, a, tau, s));
            }
            cplx nloc = cadd(cadd(cmul(bar[0], ket[0]), cmul(bar[1], ket[1])), cmul(bar[2], ket[2]));
            cplx Fz = csub(cmul(bar[0], ket[0]), cmul(bar[2], ket[2]));
            cplx Fp = cscale(r2, cadd(cmul(bar[0], ket[1]), cmul(bar[1], ket[2])));
            cplx Fm = cscale(r2, cadd(cmul(bar[1], ket[0]), cmul(bar[2], ket[1])));
            cplx F2 = cadd(cmul(Fz, Fz), cmul(Fp, Fm));
            cplx e1 = cmk(0, 0);
            for (int a = 0; a < 3; ++a) {
                double m = (double)(1 - a);
                e1 = cadd(e1, cmul(bar[a], csub(tket[a], cscale(p->q * m * m, ket[a]))));
            }
            cplx e = cadd(cadd(e1, cscale(0.5 * p->c0, cmul(nloc, nloc))), cscale(0.5 * p->c1, F2));
            dens = cadd(dens, nloc);
            fz = cadd(fz, Fz);
            f2 = cadd(f2, F2);
            en = cadd(en, e);
        }
    free(tk);
    const double inv = 1.0 / ((double)V * p->nt);
    out[0] = dens.re * inv; out[1] = dens.im * inv;
    out[2] = fz.re * inv;   out[3] = fz.im * inv;
    out[4] = f2.re * inv;   out[5] = f2.im * inv;
    out[6] = en.re * inv;   out[7] = en.im * inv;
}

/* Spin-1 start of the engine: psi = amp + sigma xi from the chain's Philox
 * stream at step 2^64-1, psibar = conj(psi). */
void orc_spin1_init(const orc_params *p, uint64_t seed, uint32_t chain, double amp,
                    double sigma, double *psi, double *psic) {
    const long V = vol(p);
    for (int c = 0; c < p->ncomp; ++c)
        for (int tau = 0; tau < p->nt; ++tau)
            for (long s = 0; s < V; ++s) {
                uint32_t site = (uint32_t)((long)tau * V + s);
                double re, im;
                orc_philox_normal(seed, chain, ~(uint64_t)0, c, site, &re, &im);
                long i = fidx(p, c, tau, s);
                cst(psi, i, cmk(amp + sigma * re, sigma * im));
                cst(psic, i, cmk(amp + sigma * re, -(sigma * im)));
            }
}

/* set_value (Lattice.cu:50-81). */
void orc_set_mean_field(const orc_params *p, double *field, double re, double im,
                        int conjugated) {
    const long V = vol(p);
    cplx v = conjugated ? cmk(re, -im) : cmk(re, im);
    for (int c = 0; c < p->ncomp; ++c)
        for (int tau = 0; tau < p->nt; ++tau)
            for (long s = 0; s < V; ++s) {
                long i = fidx(p, c, tau, s);
                if (c == 0 || c == 3) cst(field, i, v);
                else if (c == 1 || c == 2) cst(field, i, cmul(cmk(2.0 / 3.0, 0.), v));
            }
}
