// clv_engine.cu -- host side of the engine and the C ABI declared in include/clv.h.
//
// An engine owns, on one GPU, the fields of a batch of chains (packed one after
// another, each chain in the reference layout [c][tau][x][y][z]), the scratch
// for the kinetic term and the drift, per-chain constant tables (FFT twiddles,
// kinetic filters), per-chain device step state, and the work tables that map
// CTAs to (chain, lines) and (chain, sites).  A Langevin step is a fixed
// sequence of launches on one stream with no host synchronisation; repeated
// steps replay a captured CUDA graph.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "clv_internal.cuh"
#include "clv_launch.h"

using namespace clv;

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string &msg) {
    g_last_error = msg;
    return code;
}

#define CK(call)                                                                          \
    do {                                                                                  \
        cudaError_t _e = (call);                                                          \
        if (_e != cudaSuccess)                                                            \
            return fail(CLV_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e)); \
    } while (0)

// Signed momentum of compute_kinetic_part (Propagator_without_cutoff.cu:169-194).
double pmom(int j, int L) {
    if (j < L / 2 || L == 1) return 2. * M_PI * double(j) / double(L);
    return -2. * M_PI * double(L - j) / double(L);
}

bool factorize(int n, int *fac, int &nf) {
    nf = 0;
    while (n % 8 == 0 && nf < kMaxFactors) { fac[nf++] = 8; n /= 8; }
    while (n % 4 == 0 && nf < kMaxFactors) { fac[nf++] = 4; n /= 4; }
    while (n % 2 == 0 && nf < kMaxFactors) { fac[nf++] = 2; n /= 2; }
    while (n % 3 == 0 && nf < kMaxFactors) { fac[nf++] = 3; n /= 3; }
    while (n % 5 == 0 && nf < kMaxFactors) { fac[nf++] = 5; n /= 5; }
    return n == 1;
}

}  // namespace

namespace clv {
// Sets the message clv_last_error() returns, for entry points defined in other
// translation units.
int record_failure(int code, const std::string &msg) { return fail(code, msg); }
}  // namespace clv

struct clv_engine {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int model = 0, kinetic = 0, dt_rule = 0, noise = 0, precision = 0, ncomp = 4;
    std::vector<clv_chain_params> params;
    std::vector<ChainDev> chains_h;
    ChainDev *chains_d = nullptr;
    ChainState *state_d = nullptr;
    size_t elem_bytes = 16;
    long long total_elems = 0;  // per field, all chains
    long long max_chain_elems = 0;
    long long noise_total = 0;  // doubles of an external noise buffer, all chains
    void *fld[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};  // [buffer set][psi, psibar]
    int cur = 0;                    // buffer set holding the current state
    void *kin = nullptr, *kinc = nullptr;
    void *drift = nullptr, *driftc = nullptr;
    // fused path (every chain's slice fits in shared memory)
    bool fused = false, speculate = true, use_tma = true;
    bool withhold_copy = false;  // CLV_TEST_WITHHOLD_COPY: exercise the bounded-wait timeout
    // two-pass (reference dt rule) fused steps: the reduce pass stores the drift and a
    // streaming update applies it, instead of a second filter + drift pass
    bool store_drift = false;
    std::vector<FusedTask> fused_tasks_h;
    FusedTask *fused_tasks = nullptr;
    double2 *fused_partials = nullptr;
    int slot_stride = 0, comp_stride = 0;
    int fused_tab_n = 0, fused_tab_bytes = 0, fused_spt = 1, fused_ln = 0;
    size_t fused_smem = 0;
    int fused_ctas_per_sm = 0;
    int num_sms = 0;
    bool fused_split = false;  // psi and psibar in separate CTAs (build_fused_tasks)
    // step loop (k_loop.cu): resident CTAs of the loop kernel per SM (0: not available)
    int loop_per_sm = 0;
    unsigned int *loop_sync = nullptr;  // grid barrier counter and abort flag
    void *loop_noise = nullptr;         // a step's unit normals (field layout), allocated for problems it fits
    // tiled path (slices too large for the fused kernel): per-axis filter
    // launches grouped by (axis, line length), then the tau-streaming step
    struct AxisGroup {
        int axis, n, pitch, with_const;
        int W;          // lines per tile
        int plane = 0;  // 1: square planes over axes (axis, axis + 1) by the plane filter
        int strided = 1;  // every chain's lines of this axis are neighbours in memory (stride > 1)
        size_t smem;
        std::vector<AxisTask> tasks;
        AxisTask *d = nullptr;
    };
    bool tiled = false;
    std::vector<AxisGroup> axis_groups;
    bool energy_axis = false;             // kinetic energy of the observables by axis filters
    std::vector<AxisGroup> energy_groups;
    // plan knobs (heuristic defaults, CLV_* overrides, or chosen by clv_autotune)
    int chunk = 0;               // imaginary times per CTA of the step kernel
    int fused_ln_static = 0;     // compile-time line length available to the fused path
    bool fused_aligned = false;  // rows 16-byte aligned: bulk copies possible
    size_t task_capacity = 0;    // task/partial slots allocated (finest chunking)
    std::string tune_report;
    std::vector<TileTask> tile_tasks_h;
    TileTask *tile_tasks = nullptr;
    double2 *stage = nullptr;     // complex128 staging (2 * max_chain_elems)
    double2 *stage_all = nullptr; // staging for all-chain copies, allocated on first use
    long long stage_all_elems = 0;
    double *noise_d = nullptr;
    std::vector<SiteTask> site_tasks_h, obs_tasks_h;
    SiteTask *site_tasks = nullptr, *obs_tasks = nullptr;
    std::vector<ObsTask> s1obs_tasks_h;   // spin-1 observables
    ObsTask *s1obs_tasks = nullptr;
    double *s1obs_partials = nullptr;
    unsigned int *s1obs_arrive = nullptr;
    std::vector<LineTask> line_tasks_h[3];
    LineTask *line_tasks[3] = {nullptr, nullptr, nullptr};
    int max_bundle[3] = {0, 0, 0};
    double2 *partials = nullptr;
    double *accF = nullptr, *accN = nullptr;
    int acc_F_total = 0;
    int counter = 0;
    double *samples = nullptr;
    int sample_cap = 1024, sample_count = 0;
    std::vector<double> sample_spill;  // [k][chain][8] samples moved to the host
    int sample_spilled = 0;
    std::vector<void *> allocs;
    size_t dev_bytes = 0;
    cudaGraphExec_t graph_exec[2] = {nullptr, nullptr};  // keyed by the starting buffer set
    cudaGraph_t graph[2] = {nullptr, nullptr};
    // kStepBlock steps in one graph (an even count: the buffer set returns to its start)
    cudaGraphExec_t block_exec[2] = {nullptr, nullptr};
    cudaGraph_t block_graph[2] = {nullptr, nullptr};

    void *psi() const { return fld[cur][0]; }
    void *psic() const { return fld[cur][1]; }
    void drop_graphs() {
        for (int i = 0; i < 2; ++i) {
            if (graph_exec[i]) cudaGraphExecDestroy(graph_exec[i]);
            if (graph[i]) cudaGraphDestroy(graph[i]);
            if (block_exec[i]) cudaGraphExecDestroy(block_exec[i]);
            if (block_graph[i]) cudaGraphDestroy(block_graph[i]);
            graph_exec[i] = block_exec[i] = nullptr;
            graph[i] = block_graph[i] = nullptr;
        }
    }

    template <class T>
    int alloc(T **p, size_t bytes) {
        void *q = nullptr;
        if (bytes == 0) bytes = 16;
        cudaError_t e = cudaMalloc(&q, bytes);
        if (e != cudaSuccess)
            return fail(CLV_ERR_NOMEM, std::string("cudaMalloc(") + std::to_string(bytes) +
                                           "): " + cudaGetErrorString(e));
        allocs.push_back(q);
        dev_bytes += bytes;
        *p = (T *)q;
        return CLV_OK;
    }

    LaunchSites sites(bool obs = false) const {
        LaunchSites L{};
        L.chains = chains_d;
        L.state = state_d;
        L.tasks = obs ? obs_tasks : site_tasks;
        L.ntasks = obs ? (int)obs_tasks_h.size() : (int)site_tasks_h.size();
        L.model = model;
        L.dt_rule = dt_rule;
        L.noise = noise;
        L.psi = psi(); L.psic = psic(); L.kin = kin; L.kinc = kinc;
        L.psi_w = psi(); L.psic_w = psic();
        L.drift = drift; L.driftc = driftc;
        L.partials = partials;
        L.noise_buf = noise_d;
        return L;
    }
};

namespace {

int build_tables(clv_engine *e) {
    const int nch = (int)e->params.size();
    e->chains_h.resize(nch);
    long long off = 0, noff = 0;
    int obs_off = 0;
    // host staging for every table, uploaded at once
    struct Pending { void **dst; std::vector<unsigned char> bytes; };
    std::vector<Pending> pend;
    auto table = [&](auto **dst, auto &&vec) {
        Pending p;
        p.dst = (void **)dst;
        p.bytes.resize(vec.size() * sizeof(vec[0]));
        std::memcpy(p.bytes.data(), vec.data(), p.bytes.size());
        pend.push_back(std::move(p));
    };
    for (int c = 0; c < nch; ++c) {
        const clv_chain_params &p = e->params[c];
        ChainDev &d = e->chains_h[c];
        std::memset(&d, 0, sizeof d);
        d.nx = p.nx; d.ny = p.ny; d.nz = p.nz; d.nt = p.nt;
        d.V = p.nx * p.ny * p.nz;
        d.ncomp = e->ncomp;
        d.off = off;
        d.noise_off = noff;
        d.eps = p.eps; d.a_x = p.a_x; d.mu = p.mu; d.P = p.P; d.Q = p.Q; d.G = p.G;
        d.DT = p.DT; d.dt_min = p.dt_min; d.dt_max_clamp = p.dt_max_clamp; d.alpha = p.alpha;
        d.c0 = p.c0; d.c1 = p.c1; d.q = p.q; d.K = p.K; d.dt_max = p.dt_max;
        d.seed = p.seed;
        for (int a = 0; a < kMaxComp; ++a) {
            const double m = 1.0 - a;
            d.comp_const[a] = std::exp(p.eps * (p.mu + p.q * m * m));
        }
        const long long elems = (long long)e->ncomp * p.nt * d.V;
        off += elems;
        noff += 2 * elems;
        e->max_chain_elems = std::max(e->max_chain_elems, elems);
        d.obs_off = obs_off;
        obs_off += 3 * d.V;
        const int dims[3] = {p.nx, p.ny, p.nz};
        const int inner[3] = {p.ny * p.nz, p.nz, 1};
        for (int a = 0; a < 3; ++a) {
            AxisDev &ax = d.axis[a];
            ax.n = dims[a];
            ax.inner = inner[a];
            if (dims[a] <= 1) continue;
            if (!factorize(dims[a], ax.fac, ax.nf))
                return fail(CLV_ERR_ARG, "lattice extent " + std::to_string(dims[a]) +
                                             " has a prime factor other than 2, 3, 5");
            const int n = dims[a];
            std::vector<double2> tw64(n);
            std::vector<float2> tw32(n);
            const long double twopi = 2.0L * acosl(-1.0L);
            for (int k = 0; k < n; ++k) {
                const long double ang = -twopi * (long double)k / (long double)n;
                tw64[k] = make_double2((double)cosl(ang), (double)sinl(ang));
                tw32[k] = make_float2((float)cosl(ang), (float)sinl(ang));
            }
            std::vector<double> f64(n, 0.0), e64(n);
            for (int k = 0; k < n; ++k) {
                const double pk = pmom(k, n);
                if (e->kinetic == CLV_KIN_REF_LINEAR_PX) {
                    // -px^2 (py, pz terms are commented out in the reference) with the
                    // normalisation 1/(a_x NX) of the x-only transform pair
                    f64[k] = a == 0 ? -(pk * pk) / (p.a_x * n) : 1.0 / n;
                } else {
                    f64[k] = std::exp(-p.eps * 0.5 * pk * pk) / n;
                }
                e64[k] = 0.5 * pk * pk / n;
            }
            std::vector<float> f32(f64.begin(), f64.end()), e32(e64.begin(), e64.end());
            table(&ax.tw64, tw64);
            table(&ax.tw32, tw32);
            table(&ax.filt64, f64);
            table(&ax.filt32, f32);
            table(&ax.efilt64, e64);
            table(&ax.efilt32, e32);
            // per-pass twiddles of the fused kernel's compile-time line plans, from the
            // same rounded values
            if (n == 64 || n == 128 || n == 256 || n == 512) {
                const int ne = tw_entries(n);
                std::vector<double2> p64(ne);
                std::vector<float2> p32(ne);
                for (int i = 0; i < ne; ++i) {
                    bool conj = false;
                    const int m = pass_twiddle_source(n, i, &conj);
                    p64[i] = tw64[m];
                    p32[i] = tw32[m];
                    if (conj) { p64[i].y = -p64[i].y; p32[i].y = -p32[i].y; }
                }
                table(&ax.ptw64, p64);
                table(&ax.ptw32, p32);
            }
        }
        // site tasks: kSiteBlock consecutive (tau, s) sites per CTA
        const int nsites = d.V * p.nt;
        d.site_block0 = (int)e->site_tasks_h.size();
        d.site_nblocks = (nsites + kSiteBlock - 1) / kSiteBlock;
        for (int b = 0; b < d.site_nblocks; ++b) e->site_tasks_h.push_back({c, b * kSiteBlock});
        for (int b = 0; b < (d.V + 255) / 256; ++b) e->obs_tasks_h.push_back({c, b * 256});
        // spin-1 observables: 256 sites x chunks of at most 16 imaginary times
        {
            const int nchunk = (p.nt + 15) / 16;
            d.obs_block0 = (int)e->s1obs_tasks_h.size();
            for (int k = 0; k < nchunk; ++k)
                for (int b = 0; b < (d.V + 255) / 256; ++b)
                    e->s1obs_tasks_h.push_back({c, b * 256, (int)((long long)p.nt * k / nchunk),
                                                (int)((long long)p.nt * (k + 1) / nchunk)});
            d.obs_nblocks = (int)e->s1obs_tasks_h.size() - d.obs_block0;
        }
        // line tasks per axis
        const int budget = e->precision == CLV_PREC_F64 ? kMaxBundleElems64 : kMaxBundleElems32;
        for (int a = 0; a < 3; ++a) {
            const int n = dims[a];
            if (n <= 1) continue;
            if (n > kMaxLine) return fail(CLV_ERR_ARG, "lattice extent above 2048");
            const int lines = e->ncomp * p.nt * (d.V / n);
            int W = std::max(1, budget / n);
            W = std::min(W, lines);
            for (int l0 = 0; l0 < lines; l0 += W) {
                const int nl = std::min(W, lines - l0);
                e->line_tasks_h[a].push_back({c, l0, nl});
                e->max_bundle[a] = std::max(e->max_bundle[a], nl * n);
            }
        }
    }
    e->total_elems = off;
    e->noise_total = noff;
    e->acc_F_total = obs_off;
    // upload tables; device pointers are patched into the host chain copies
    for (auto &p : pend) {
        void *dptr = nullptr;
        int rc = e->alloc(&dptr, p.bytes.size());
        if (rc) return rc;
        CK(cudaMemcpy(dptr, p.bytes.data(), p.bytes.size(), cudaMemcpyHostToDevice));
        *p.dst = dptr;
    }
    return CLV_OK;
}

// Optional event trail of a step: an event is recorded after every launch.
struct EventTrail {
    std::vector<cudaEvent_t> ev;
    cudaError_t mark(cudaStream_t s) {
        cudaEvent_t e;
        cudaError_t r = cudaEventCreate(&e);
        if (r != cudaSuccess) return r;
        ev.push_back(e);
        return cudaEventRecord(e, s);
    }
    ~EventTrail() { for (auto e : ev) cudaEventDestroy(e); }
};

template <class R>
int run_kinetic(clv_engine *e, const void *s0, const void *s1, void *d0, void *d1, int filter,
                int nfields, EventTrail *trail = nullptr) {
    bool first = true;
    for (int a = 0; a < 3; ++a) {
        if (e->line_tasks_h[a].empty()) continue;
        if (e->kinetic == CLV_KIN_REF_LINEAR_PX && filter == 0 && a > 0) break;
        LaunchLineFilter L{};
        L.chains = e->chains_d;
        L.tasks = e->line_tasks[a];
        L.ntasks = (int)e->line_tasks_h[a].size();
        L.max_bundle = e->max_bundle[a];
        L.axis = a;
        L.nfields = nfields;
        L.filter = filter;
        if (filter == 0) {
            // kinetic: product over axes, first pass reads the fields
            L.src0 = first ? s0 : d0;
            L.src1 = first ? s1 : d1;
            L.mode = 0;
            L.with_const = first && e->kinetic == CLV_KIN_EXP;
        } else {
            // kinetic energy: sum over axes of the one-axis operators
            L.src0 = s0;
            L.src1 = s1;
            L.mode = first ? 0 : 1;
            L.with_const = 0;
        }
        L.dst0 = d0;
        L.dst1 = d1;
        CK(launch_line_filter<R>(L, e->stream));
        if (trail) CK(trail->mark(e->stream));
        first = false;
    }
    return CLV_OK;
}

LaunchFused fused_launch(const clv_engine *e, int from, int mode, bool ext) {
    LaunchFused L{};
    L.chains = e->chains_d;
    L.state = e->state_d;
    L.tasks = e->fused_tasks;
    L.ntasks = (int)e->fused_tasks_h.size();
    L.model = e->model;
    L.kinetic = e->kinetic;
    L.dt_rule = e->dt_rule;
    L.noise = ext ? CLV_NOISE_EXTERNAL : CLV_NOISE_PHILOX;
    L.mode = mode;
    L.only_rejected = 0;
    L.use_tma = e->use_tma;
    L.withhold = e->withhold_copy && mode != FUSED_APPLY;
    L.drift_out = (mode == FUSED_MAXONLY && e->store_drift) ? e->drift : nullptr;
    L.driftc_out = (mode == FUSED_MAXONLY && e->store_drift) ? e->driftc : nullptr;
    L.psi_in = e->fld[from][0];
    L.psic_in = e->fld[from][1];
    L.psi_out = e->fld[from ^ 1][0];
    L.psic_out = e->fld[from ^ 1][1];
    L.partials = e->fused_partials;
    L.noise_buf = e->noise_d;
    L.slot_stride = e->slot_stride;
    L.comp_stride = e->comp_stride;
    L.tab_n = e->fused_tab_n;
    L.tab_bytes = e->fused_tab_bytes;
    L.spt = e->fused_spt;
    L.ln = e->fused_ln;
    L.split = e->fused_split ? 1 : 0;
    L.smem_bytes = e->fused_smem;
    return L;
}

LaunchTiled tiled_launch(const clv_engine *e, int from, int mode, bool ext) {
    LaunchTiled L{};
    L.chains = e->chains_d;
    L.state = e->state_d;
    L.tasks = e->tile_tasks;
    L.ntasks = (int)e->tile_tasks_h.size();
    L.model = e->model;
    L.dt_rule = e->dt_rule;
    L.noise = ext ? CLV_NOISE_EXTERNAL : CLV_NOISE_PHILOX;
    L.mode = mode;
    L.only_rejected = 0;
    L.psi_in = e->fld[from][0];
    L.psic_in = e->fld[from][1];
    L.kin = e->kin;
    L.kinc = e->kinc;
    L.psi_out = e->fld[from ^ 1][0];
    L.psic_out = e->fld[from ^ 1][1];
    L.partials = e->fused_partials;
    L.noise_buf = e->noise_d;
    L.drift_out = (mode == FUSED_MAXONLY && e->store_drift) ? e->drift : nullptr;
    L.driftc_out = (mode == FUSED_MAXONLY && e->store_drift) ? e->driftc : nullptr;
    return L;
}

// Tiled step: kinetic filter axis by axis into kin/kinbar, then the streaming
// drift/noise/update kernel (speculative dt with redo, or reduce then apply).
template <class R>
int enqueue_tiled(clv_engine *e, bool external_noise, EventTrail *trail, int from) {
    for (const auto &g : e->axis_groups) {
        LaunchAxis A{};
        A.chains = e->chains_d;
        A.tasks = g.d;
        A.ntasks = (int)g.tasks.size();
        A.axis = g.axis;
        A.n = g.n;
        A.W = g.W;
        A.pitch = g.pitch;
        A.with_const = g.with_const;
        A.src0 = g.axis == 0 ? e->fld[from][0] : e->kin;
        A.src1 = g.axis == 0 ? e->fld[from][1] : e->kinc;
        A.dst0 = e->kin;
        A.dst1 = e->kinc;
        A.smem_bytes = g.smem;
        A.nfields = 2;
        A.filter = 0;
        A.accumulate = 0;
        A.strided = g.strided;
        if (g.plane) CK(launch_plane_filter<R>(A, e->stream));
        else CK(launch_axis_filter<R>(A, e->stream));
        if (trail) CK(trail->mark(e->stream));
    }
    if (e->speculate && e->dt_rule == CLV_DT_K_OVER_MAX) {
        CK(launch_tiled<R>(tiled_launch(e, from, FUSED_SPEC, external_noise), e->stream));
        if (trail) CK(trail->mark(e->stream));
        LaunchTiled L = tiled_launch(e, from, FUSED_APPLY, external_noise);
        L.only_rejected = 1;
        CK(launch_tiled<R>(L, e->stream));
    } else {
        CK(launch_tiled<R>(tiled_launch(e, from, FUSED_MAXONLY, external_noise), e->stream));
        if (trail) CK(trail->mark(e->stream));
        if (e->store_drift) {
            // the stored drift applied by the site-parallel update, which draws its noise
            // while the reduce pass runs (programmatic launch)
            LaunchSites L = e->sites();
            L.psi = e->fld[from][0];
            L.psic = e->fld[from][1];
            L.psi_w = e->fld[from ^ 1][0];
            L.psic_w = e->fld[from ^ 1][1];
            L.noise = external_noise ? CLV_NOISE_EXTERNAL : CLV_NOISE_PHILOX;
            L.pdl = !std::getenv("CLV_NO_PDL");
            CK(launch_update<R>(L, e->stream));
        } else {
            CK(launch_tiled<R>(tiled_launch(e, from, FUSED_APPLY, external_noise), e->stream));
        }
    }
    if (trail) CK(trail->mark(e->stream));
    return CLV_OK;
}

// Small problems run many steps per cooperative launch (k_loop.cu) when every split
// task of the fused plan covers one imaginary time and all of them fit on the GPU at
// once; the trajectory is the two-kernel form's bit for bit (CLV_NO_LOOP=1 keeps the
// two-kernel form).
bool use_loop(const clv_engine *e) {
    if (!e->fused || e->fused_ln <= 0 || !e->fused_split || !e->loop_noise) return false;
    if (e->loop_per_sm < 1 || (long long)e->fused_tasks_h.size() > (long long)e->loop_per_sm * e->num_sms)
        return false;
    for (const auto &t : e->fused_tasks_h)
        if (t.tau1 - t.tau0 != 1 || t.side == 0) return false;
    return !std::getenv("CLV_NO_LOOP");
}

// nsteps Philox steps by the step loop, in launches of at most 2^16 steps.  A
// cooperative launch the GPU refuses (the grid cannot be resident now, e.g. beside
// other work on a shared GPU) turns the loop off for this engine: *done tells the
// caller how many steps ran, and kLoopRefused that the rest is its to run.
constexpr int kLoopRefused = -1000;
template <class R>
int enqueue_loop(clv_engine *e, int nsteps, EventTrail *trail, int *done = nullptr) {
    if (done) *done = 0;
    while (nsteps > 0) {
        const int n = std::min(nsteps, 1 << 16);
        CK(cudaMemsetAsync(e->loop_sync, 0, 2 * sizeof(unsigned int), e->stream));
        if (trail) CK(trail->mark(e->stream));
        LaunchLoop L{};
        L.chains = e->chains_d;
        L.state = e->state_d;
        L.tasks = e->fused_tasks;
        L.ntasks = (int)e->fused_tasks_h.size();
        L.nsteps = n;
        L.model = e->model;
        L.kinetic = e->kinetic;
        L.ln = e->fused_ln;
        L.dt_rule = e->dt_rule;
        for (int b = 0; b < 2; ++b)
            for (int f = 0; f < 2; ++f) L.fld[b][f] = e->fld[b][f];
        L.from = e->cur;
        L.noise = e->loop_noise;
        L.partials = e->fused_partials;
        L.bar = e->loop_sync;
        L.abort = reinterpret_cast<int *>(e->loop_sync + 1);
        L.withhold = e->withhold_copy;
        const cudaError_t le = launch_loop<R>(L, e->stream);
        if (le == cudaErrorCooperativeLaunchTooLarge) {
            (void)cudaGetLastError();  // a launch-configuration error: nothing ran
            if (trail) {               // (the mark before the refused launch)
                cudaEventDestroy(trail->ev.back());
                trail->ev.pop_back();
            }
            e->loop_per_sm = 0;
            return kLoopRefused;
        }
        CK(le);
        if (trail) CK(trail->mark(e->stream));
        if (n & 1) e->cur ^= 1;
        nsteps -= n;
        if (done) *done += n;
    }
    return CLV_OK;
}

int enqueue_loop_any(clv_engine *e, int nsteps, EventTrail *trail, int *done = nullptr) {
    return e->precision == CLV_PREC_F64 ? enqueue_loop<double>(e, nsteps, trail, done)
                                        : enqueue_loop<float>(e, nsteps, trail, done);
}

// One step reading buffer set `from` and writing set `from ^ 1`.
template <class R>
int enqueue_step(clv_engine *e, bool external_noise, EventTrail *trail, int from) {
    if (e->tiled) return enqueue_tiled<R>(e, external_noise, trail, from);
    if (e->fused) {
        if (e->speculate && e->dt_rule == CLV_DT_K_OVER_MAX) {
            // update with dt = dt_max; chains whose true dt differs are redone
            CK(launch_fused<R>(fused_launch(e, from, FUSED_SPEC, external_noise), e->stream));
            if (trail) CK(trail->mark(e->stream));
            LaunchFused L = fused_launch(e, from, FUSED_APPLY, external_noise);
            L.only_rejected = 1;
            CK(launch_fused<R>(L, e->stream));
        } else {
            CK(launch_fused<R>(fused_launch(e, from, FUSED_MAXONLY, external_noise), e->stream));
            if (trail) CK(trail->mark(e->stream));
            if (e->store_drift) {
                LaunchSites L = e->sites();
                L.psi = e->fld[from][0];
                L.psic = e->fld[from][1];
                L.psi_w = e->fld[from ^ 1][0];
                L.psic_w = e->fld[from ^ 1][1];
                L.noise = external_noise ? CLV_NOISE_EXTERNAL : CLV_NOISE_PHILOX;
                // its noise is drawn while the reduce pass runs (the pass releases its
                // dependents at its start; the update waits for its end before it reads)
                L.pdl = e->dt_rule == CLV_DT_REF_MEANMAX && !std::getenv("CLV_NO_PDL");
                CK(launch_update<R>(L, e->stream));
            } else {
                CK(launch_fused<R>(fused_launch(e, from, FUSED_APPLY, external_noise), e->stream));
            }
        }
        if (trail) CK(trail->mark(e->stream));
        return CLV_OK;
    }
    int rc = run_kinetic<R>(e, e->fld[from][0], e->fld[from][1], e->kin, e->kinc, 0, 2, trail);
    if (rc) return rc;
    LaunchSites L = e->sites();
    L.psi = e->fld[from][0];
    L.psic = e->fld[from][1];
    L.psi_w = e->fld[from ^ 1][0];
    L.psic_w = e->fld[from ^ 1][1];
    L.noise = external_noise ? CLV_NOISE_EXTERNAL : CLV_NOISE_PHILOX;
    CK(launch_drift<R>(L, e->stream));
    if (trail) CK(trail->mark(e->stream));
    CK(launch_update<R>(L, e->stream));
    if (trail) CK(trail->mark(e->stream));
    return CLV_OK;
}

int enqueue_step_any(clv_engine *e, bool ext, EventTrail *trail, int from) {
    return e->precision == CLV_PREC_F64 ? enqueue_step<double>(e, ext, trail, from)
                                        : enqueue_step<float>(e, ext, trail, from);
}

// Choose the fused path when every chain's slice fits the shared-memory plan,
// and split each chain's imaginary times into chunks that fill the GPU.
// Fused tasks for chunks of L imaginary times; sets each chain's CTA range.
// Fused step tasks: chunks of L imaginary times.  Under the reference's step rule
// (two passes on the generic kernel), when the chunks are fewer than the SMs (the
// reference's own 256 x 32 lattice: 32 chunks), each chunk becomes a psi CTA and a
// psibar CTA, so twice as many SMs share the FFT and drift work; under the K/max
// rule the production variant on whole chunks measured faster (one 1D 256 x 128
// chain at FP64: 0.086 against 0.129 ms).  CLV_FUSED_SPLIT=0/1 overrides.
void build_fused_tasks(clv_engine *e, int L) {
    e->chunk = L;
    e->fused_tasks_h.clear();
    long long chunks = 0;
    for (auto &d : e->chains_h) chunks += std::max(1, (d.nt + L - 1) / L);
    bool split = e->dt_rule == CLV_DT_REF_MEANMAX && chunks < e->num_sms;
    // under the K/max rule too when the step loop takes the problem: chunks of one
    // imaginary time whose split tasks are all resident at once (the FP64 single chain
    // of 64 sites x 64 imaginary times)
    if (e->dt_rule == CLV_DT_K_OVER_MAX && L == 1 && e->fused_ln > 0 && e->loop_per_sm > 0 &&
        2 * chunks <= (long long)e->loop_per_sm * e->num_sms && !std::getenv("CLV_NO_LOOP"))
        split = true;
    if (const char *sp = std::getenv("CLV_FUSED_SPLIT")) split = sp[0] == '1';
    // fewer still (the reference's 256 x 32 lattice: 64 split CTAs on 152 SMs) and the
    // FP64 pipe the bound: each field's CTA splits again into component halves, so a
    // CTA filters two lines and drifts two components, on 1D lines of the 4-component
    // model (CLV_FUSED_CSPLIT=0/1 overrides)
    bool csplit = split && e->ncomp == 4 && e->precision == CLV_PREC_F64 && 4 * chunks <= e->num_sms;
    for (auto &d : e->chains_h)
        if (d.ny != 1 || d.nz != 1) csplit = false;
    if (const char *cs = std::getenv("CLV_FUSED_CSPLIT")) csplit = split && e->ncomp == 4 && cs[0] == '1';
    e->fused_split = split;
    const int per_chunk = split ? (csplit ? 4 : 2) : 1;
    for (int c = 0; c < (int)e->chains_h.size(); ++c) {
        ChainDev &d = e->chains_h[c];
        const int nchunk = std::max(1, (d.nt + L - 1) / L);
        d.fused_block0 = (int)e->fused_tasks_h.size();
        d.fused_nblocks = per_chunk * nchunk;
        for (int k = 0; k < nchunk; ++k) {
            const int t0 = (int)((long long)d.nt * k / nchunk);
            const int t1 = (int)((long long)d.nt * (k + 1) / nchunk);
            if (csplit) {
                for (int f = 1; f <= 2; ++f)
                    for (int h = 0; h < 2; ++h)
                        e->fused_tasks_h.push_back({c, t0, t1, 4 * k + 2 * (f - 1) + h, f, h ? 0xC : 0x3});
            } else if (split) {
                e->fused_tasks_h.push_back({c, t0, t1, 2 * k, 1, 0});
                e->fused_tasks_h.push_back({c, t0, t1, 2 * k + 1, 2, 0});
            } else {
                e->fused_tasks_h.push_back({c, t0, t1, k, 0, 0});
            }
        }
    }
}

// Tiled step tasks: 256 sites x chunks of L imaginary times.
void build_tiled_tasks(clv_engine *e, int L) {
    e->chunk = L;
    e->tile_tasks_h.clear();
    for (int c = 0; c < (int)e->chains_h.size(); ++c) {
        ChainDev &d = e->chains_h[c];
        const int ntile = (d.V + 255) / 256;
        const int nchunk = std::max(1, (d.nt + L - 1) / L);
        d.fused_block0 = (int)e->tile_tasks_h.size();
        d.fused_nblocks = ntile * nchunk;
        int part = 0;
        for (int k = 0; k < nchunk; ++k) {
            const int t0 = (int)((long long)d.nt * k / nchunk);
            const int t1 = (int)((long long)d.nt * (k + 1) / nchunk);
            for (int t = 0; t < ntile; ++t) e->tile_tasks_h.push_back({c, t * 256, t0, t1, part++});
        }
    }
}

int plan_fused(clv_engine *e) {
    const char *env = std::getenv("CLV_FUSED");
    if (env && env[0] == '0') return CLV_OK;
    const size_t esz = e->elem_bytes;
    int vmax = 0;
    bool aligned = true;
    for (auto &d : e->chains_h) {
        vmax = std::max(vmax, d.V);
        if ((d.V * esz) % 16 != 0) aligned = false;
        if (d.nt < 2) return CLV_OK;
        if ((long long)e->ncomp * d.nt * d.V >= (1LL << 31)) return CLV_OK;  // 32-bit element indices
    }
    // component regions padded (one element per 16) for the FFT's padded layouts,
    // even so that every component row stays 16-byte aligned for the bulk copies
    const int cs = padded_line(vmax);
    const int stride = fused_slot_stride(e->ncomp, vmax, (int)esz);
    const int spt = vmax <= 256 ? 1 : (vmax <= 512 ? 2 : (vmax <= 1024 ? 4 : 0));
    if (spt == 0) return CLV_OK;
    // compile-time plan when every chain is a 1D line of one common length
    int ln = e->chains_h[0].nx;
    for (auto &d : e->chains_h)
        if (d.ny != 1 || d.nz != 1 || d.nx != ln) ln = 0;
    if (ln != 64 && ln != 128 && ln != 256) ln = 0;
    if (std::getenv("CLV_NO_STATIC_PLAN")) ln = 0;
    // shared tables: twiddles and filters of the filtered axes of the largest chain
    int tab_n = 0;
    for (auto &d : e->chains_h) {
        int n = 0;
        for (int a = 0; a < 3; ++a) {
            if (d.axis[a].n <= 1) continue;
            if (e->kinetic == CLV_KIN_REF_LINEAR_PX && a > 0) break;
            n += d.axis[a].n;
        }
        tab_n = std::max(tab_n, n);
    }
    const int tab_bytes = fused_tab_bytes(tab_n, (int)esz, ln);
    const int nslots = (e->model == CLV_MODEL_REF4 ? 3 : 2) + 2 + 5;
    const size_t smem = tab_bytes + (size_t)nslots * stride * esz;
    int dev_smem = 0, nsm = 0;
    CK(cudaDeviceGetAttribute(&dev_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, e->device));
    CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, e->device));
    e->num_sms = nsm;
    if (smem + 2048 > (size_t)dev_smem) return CLV_OK;  // room for the kernel's static shared memory
    // the compile-time-line kernels derive the same geometry from ln alone
    if (ln > 0 && (tab_n != ln || stride != fused_slot_stride(e->ncomp, ln, (int)esz)))
        return fail(CLV_ERR_STATE, "fused slot geometry of the line kernels");
    e->slot_stride = stride;
    e->comp_stride = cs;
    e->fused_smem = smem;
    e->fused_tab_n = tab_n;
    e->fused_tab_bytes = tab_bytes;
    e->fused_spt = spt;
    e->fused_ln = ln;
    e->use_tma = aligned && !(std::getenv("CLV_NO_TMA"));
    e->speculate = !(std::getenv("CLV_NO_SPECULATE"));
    LaunchFused probe{};
    probe.model = e->model;
    probe.spt = spt;
    probe.ln = ln;
    probe.smem_bytes = smem;
    int per_sm = 0;
    if (e->precision == CLV_PREC_F64) CK(setup_fused<double>(probe, &per_sm));
    else CK(setup_fused<float>(probe, &per_sm));
    if (per_sm < 1) return CLV_OK;
    e->fused_ctas_per_sm = per_sm;
    // chunk length: about two waves of CTAs; a batch too small to fill the GPU takes
    // one imaginary time per CTA (its halo work runs on otherwise idle SMs)
    long long total_slices = 0;
    for (auto &d : e->chains_h) total_slices += d.nt;
    const long long target = 2LL * per_sm * nsm;
    int L = (int)std::max<long long>(1, (total_slices + target - 1) / target);
    if (const char *cl = std::getenv("CLV_CHUNK")) L = std::max(1, atoi(cl));
    e->fused_ln_static = std::getenv("CLV_NO_STATIC_PLAN") ? 0 : ln;
    e->withhold_copy = std::getenv("CLV_TEST_WITHHOLD_COPY") != nullptr;
    // FP64 arithmetic is scarce on this part: store the drift rather than recompute it
    e->store_drift = e->dt_rule == CLV_DT_REF_MEANMAX && e->precision == CLV_PREC_F64;
    if (const char *sd = std::getenv("CLV_STORE_DRIFT"))
        e->store_drift = e->dt_rule == CLV_DT_REF_MEANMAX && sd[0] == '1';
    e->fused_aligned = aligned;
    e->task_capacity = 4 * (size_t)total_slices;  // chunks of one imaginary time, split twice
    e->fused = true;
    // the step loop's resident CTAs per SM (1D lines of a compile-time length)
    if (ln > 0) {
        int coop = 0;
        CK(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, e->device));
        if (coop) {
            if (e->precision == CLV_PREC_F64) CK(setup_loop<double>(e->model, ln, &e->loop_per_sm));
            else CK(setup_loop<float>(e->model, ln, &e->loop_per_sm));
        }
    }
    build_fused_tasks(e, L);
    return CLV_OK;
}

// Tiled path for the chains the fused kernel cannot hold: every filtered axis
// needs lines of at most 512 sites and shared memory for a tile of up to W
// adjacent lines and its FFT scratch (axis_tile_lines, axis_smem_bytes).
// Otherwise the engine keeps the separate line-filter / drift / update kernels.
// Axis-filter launch groups, one per (axis, line length): kinetic (energy =
// false: the step's filter, every filtered axis, the component constant on the
// first) or kinetic energy (energy = true: k_a^2/2 on every axis, summed).  False
// when a line is longer than 512 sites or a tile does not fit shared memory.
int build_axis_groups(clv_engine *e, bool energy, std::vector<clv_engine::AxisGroup> &groups, bool &ok) {
    ok = false;
    groups.clear();
    const size_t esz = e->elem_bytes;
    int dev_smem = 0;
    CK(cudaDeviceGetAttribute(&dev_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, e->device));
    for (int c = 0; c < (int)e->chains_h.size(); ++c) {
        const ChainDev &d = e->chains_h[c];
        // square planes of side 32 to 128 (a 2D slice, or the (y, z) planes of a 3D
        // slice) under the exponential kinetic factor, a product over the axes: one
        // plane-filter launch instead of two axis launches
        int pa = -1;
        if (!energy && e->kinetic == CLV_KIN_EXP && !std::getenv("CLV_NO_PLANE")) {
            const int n1 = d.axis[1].n, n2 = d.axis[2].n;
            pa = n2 <= 1 ? (d.axis[0].n == n1 ? 0 : -1) : (n1 == n2 ? 1 : -1);
            const int pn = pa >= 0 ? d.axis[pa].n : 0;
            int occ = 0;
            if (pn == 32 || pn == 64 || pn == 96 || pn == 128) {
                const size_t sm = plane_smem_bytes(pn, esz);
                if (sm + 1024 <= (size_t)dev_smem) {
                    if (e->precision == CLV_PREC_F64) CK(setup_plane_filter<double>(pn, sm, &occ));
                    else CK(setup_plane_filter<float>(pn, sm, &occ));
                }
            }
            if (occ < 1) pa = -1;
        }
        for (int a = 0; a < 3; ++a) {
            const AxisDev &ax = d.axis[a];
            if (ax.n <= 1) continue;
            if (!energy && e->kinetic == CLV_KIN_REF_LINEAR_PX && a > 0) break;
            if (pa >= 0 && a == pa + 1) continue;  // filtered with axis pa
            if (pa >= 0 && a == pa) {
                const int n = ax.n;
                int gi = -1;
                for (int g = 0; g < (int)groups.size(); ++g)
                    if (groups[g].plane && groups[g].axis == a && groups[g].n == n) gi = g;
                if (gi < 0) {
                    clv_engine::AxisGroup g;
                    g.axis = a;
                    g.n = n;
                    g.pitch = plane_pitch(n);
                    g.W = 1;
                    g.plane = 1;
                    g.with_const = a == 0;
                    g.smem = plane_smem_bytes(n, esz);
                    groups.push_back(std::move(g));
                    gi = (int)groups.size() - 1;
                }
                const int planes = d.V / (n * n);
                for (int sl = 0; sl < d.ncomp * d.nt; ++sl)
                    for (int x = 0; x < planes; ++x) groups[gi].tasks.push_back({c, sl, x, 1});
                continue;
            }
            const int n = ax.n, lines = d.V / n;
            if (n > 512) return CLV_OK;
            const bool ct = axis_compile_time_plan(n);
            const int W = esz == 8 ? axis_tile_lines<float>(ct ? n : 0) : axis_tile_lines<double>(ct ? n : 0);
            int gi = -1;
            for (int g = 0; g < (int)groups.size(); ++g)
                if (!groups[g].plane && groups[g].axis == a && groups[g].n == n) gi = g;
            if (gi < 0) {
                clv_engine::AxisGroup g;
                g.axis = a;
                g.n = n;
                g.pitch = axis_pitch(n, ct);
                g.W = W;
                g.with_const = !energy && e->kinetic == CLV_KIN_EXP && a == 0;
                g.smem = axis_smem_bytes(n, ct, W, esz);
                if (g.smem + 1024 > (size_t)dev_smem) return CLV_OK;
                int occ = 0;
                if (e->precision == CLV_PREC_F64) CK(setup_axis_filter<double>(n, g.smem, &occ));
                else CK(setup_axis_filter<float>(n, g.smem, &occ));
                if (occ < 1) return CLV_OK;
                groups.push_back(std::move(g));
                gi = (int)groups.size() - 1;
            }
            groups[gi].strided &= ax.inner > 1;
            if (ax.inner == 1 && !groups[gi].with_const) {
                // contiguous lines run on across slices: tiles of W consecutive lines of
                // the chain (1D chains: W imaginary-time slices per tile)
                const int total = d.ncomp * d.nt * lines;
                for (int gl = 0; gl < total; gl += W)
                    groups[gi].tasks.push_back({c, gl / lines, gl % lines, std::min(W, total - gl)});
            } else {
                // tiles of W lines of one slice, never across an outer block of a strided axis
                for (int sl = 0; sl < d.ncomp * d.nt; ++sl)
                    for (int l0 = 0; l0 < lines;) {
                        const int nl = ax.inner == 1 ? std::min(W, lines - l0)
                                                     : std::min(W, ax.inner - l0 % ax.inner);
                        groups[gi].tasks.push_back({c, sl, l0, nl});
                        l0 += nl;
                    }
            }
        }
    }
    std::stable_sort(groups.begin(), groups.end(),
                     [](const clv_engine::AxisGroup &x, const clv_engine::AxisGroup &y) { return x.axis < y.axis; });
    ok = true;
    return CLV_OK;
}

int plan_tiled(clv_engine *e) {
    if (e->fused) return CLV_OK;
    const char *env = std::getenv("CLV_TILED");
    if (env && env[0] == '0') return CLV_OK;
    int nsm = 0;
    CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, e->device));
    std::vector<clv_engine::AxisGroup> groups;
    for (auto &d : e->chains_h)
        if (d.nt < 2) return CLV_OK;
    bool ok = false;
    if (int rc = build_axis_groups(e, false, groups, ok)) return rc;
    if (!ok) return CLV_OK;
    int occ = 0;
    if (e->precision == CLV_PREC_F64) CK(setup_tiled<double>(e->model, &occ));
    else CK(setup_tiled<float>(e->model, &occ));
    if (occ < 1) return CLV_OK;
    // imaginary-time chunk: about one wave of CTAs, 8..64 times per CTA (longer
    // chunks amortise the halo slice and the prologue; clv_autotune refines it);
    // fewer for problems too small to fill the GPU
    long long tile_taus = 0;
    for (auto &d : e->chains_h) tile_taus += (long long)((d.V + 255) / 256) * d.nt;
    const long long Lw = tile_taus / ((long long)occ * nsm);
    int L = (int)(Lw >= 8 ? std::min<long long>(64, Lw) : std::max<long long>(1, Lw));
    if (const char *cl = std::getenv("CLV_CHUNK")) L = std::max(1, atoi(cl));
    e->task_capacity = (size_t)tile_taus;  // chunks of one imaginary time
    build_tiled_tasks(e, L);
    e->axis_groups = std::move(groups);
    e->speculate = !(std::getenv("CLV_NO_SPECULATE"));
    // reference rule at FP64, where arithmetic is scarce: the reduce pass stores the drift
    // and the update applies it, instead of a second drift pass
    e->store_drift = e->dt_rule == CLV_DT_REF_MEANMAX && e->precision == CLV_PREC_F64;
    if (const char *sd = std::getenv("CLV_STORE_DRIFT"))
        e->store_drift = e->dt_rule == CLV_DT_REF_MEANMAX && sd[0] == '1';
    e->tiled = true;
    return CLV_OK;
}

int check_chain(clv_engine *e, int chain) {
    if (!e) return fail(CLV_ERR_ARG, "null engine");
    if (chain < 0 || chain >= (int)e->params.size()) return fail(CLV_ERR_ARG, "chain out of range");
    return CLV_OK;
}

cudaMemcpyKind kind_of(int where, bool to_device) {
    if (where & CLV_DEVICE) return cudaMemcpyDeviceToDevice;
    return to_device ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost;
}

}  // namespace

extern "C" {

int clv_version(void) { return CLV_API_VERSION; }

const char *clv_last_error(void) { return g_last_error.c_str(); }

const char *clv_status_string(int s) {
    switch (s) {
        case CLV_OK: return "ok";
        case CLV_ERR_ARG: return "invalid argument";
        case CLV_ERR_CUDA: return "CUDA error";
        case CLV_ERR_NONFINITE: return "non-finite drift";
        case CLV_ERR_TIMEOUT: return "device wait timed out";
        case CLV_ERR_STATE: return "invalid state";
        case CLV_ERR_NOMEM: return "out of memory";
        case CLV_ERR_IO: return "i/o error";
        default: return "unknown status";
    }
}

void clv_default_chain_params(clv_chain_params *p) {
    std::memset(p, 0, sizeof *p);
    // Parameters.h
    p->nx = 256; p->ny = 1; p->nz = 1; p->nt = 32;
    p->eps = 0.01; p->a_x = 1.0; p->G = 0.1; p->Q = 0.0; p->DT = 0.002;
    // compute_new_dt (Propagator_without_cutoff.cu:391-402)
    p->dt_min = 1e-8; p->dt_max_clamp = 0.01; p->alpha = 0.9;
    // params.txt
    p->mu = -1.5; p->P = 0.0; p->seed = 7342951900870119ull;
    p->c0 = 0.5; p->c1 = -0.1; p->q = 0.05; p->K = 0.05; p->dt_max = 1e-3;
}

int clv_create(const clv_config *cfg, clv_engine **out) {
    if (!cfg || !out) return fail(CLV_ERR_ARG, "null argument");
    *out = nullptr;
    if (cfg->nchains <= 0 || !cfg->chains) return fail(CLV_ERR_ARG, "nchains must be positive");
    if (cfg->model != CLV_MODEL_REF4 && cfg->model != CLV_MODEL_SPIN1)
        return fail(CLV_ERR_ARG, "unknown model");
    if (cfg->kinetic != CLV_KIN_REF_LINEAR_PX && cfg->kinetic != CLV_KIN_EXP)
        return fail(CLV_ERR_ARG, "unknown kinetic term");
    if (cfg->dt_rule != CLV_DT_REF_MEANMAX && cfg->dt_rule != CLV_DT_K_OVER_MAX)
        return fail(CLV_ERR_ARG, "unknown step rule");
    if (cfg->noise != CLV_NOISE_EXTERNAL && cfg->noise != CLV_NOISE_PHILOX)
        return fail(CLV_ERR_ARG, "unknown noise source");
    if (cfg->precision != CLV_PREC_F64 && cfg->precision != CLV_PREC_F32)
        return fail(CLV_ERR_ARG, "unknown precision");
    long long total_sites = 0;
    for (int c = 0; c < cfg->nchains; ++c) {
        const clv_chain_params &p = cfg->chains[c];
        if (p.nx < 2 || p.ny < 1 || p.nz < 1 || p.nt < 2)
            return fail(CLV_ERR_ARG, "chain " + std::to_string(c) + ": need nx >= 2, nt >= 2");
        const long long sites = (long long)p.nx * p.ny * p.nz * p.nt;
        const int ncomp = cfg->model == CLV_MODEL_REF4 ? 4 : 3;
        if (sites * ncomp >= (1ll << 31))
            return fail(CLV_ERR_ARG, "chain " + std::to_string(c) + ": lattice too large");
        if (!(p.eps > 0) || !std::isfinite(p.eps)) return fail(CLV_ERR_ARG, "eps must be positive");
        if (cfg->model == CLV_MODEL_REF4 && !(p.a_x != 0)) return fail(CLV_ERR_ARG, "a_x must be nonzero");
        total_sites += sites;
    }
    if (total_sites >= (1ll << 40)) return fail(CLV_ERR_ARG, "batch too large");
    CK(cudaSetDevice(cfg->device));
    int nsm = 0;
    CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, cfg->device));
    clv_engine *e = new clv_engine();
    e->device = cfg->device;
    e->num_sms = nsm;
    e->model = cfg->model;
    e->kinetic = cfg->kinetic;
    e->dt_rule = cfg->dt_rule;
    e->noise = cfg->noise;
    e->precision = cfg->precision;
    e->ncomp = cfg->model == CLV_MODEL_REF4 ? 4 : 3;
    e->elem_bytes = cfg->precision == CLV_PREC_F64 ? 16 : 8;
    e->params.assign(cfg->chains, cfg->chains + cfg->nchains);
    if (const char *cap = std::getenv("CLV_SAMPLE_CAPACITY")) e->sample_cap = std::max(1, atoi(cap));
    auto bail = [&](int rc) { clv_destroy(e); return rc; };
    cudaError_t ce = cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking);
    if (ce != cudaSuccess) return bail(fail(CLV_ERR_CUDA, cudaGetErrorString(ce)));
    e->own_stream = true;
    ce = setup_line_filter();
    if (ce != cudaSuccess) return bail(fail(CLV_ERR_CUDA, cudaGetErrorString(ce)));
    int rc = build_tables(e);
    if (rc) return bail(rc);
    if ((rc = plan_fused(e))) return bail(rc);
    if ((rc = plan_tiled(e))) return bail(rc);

    if (e->model == CLV_MODEL_SPIN1 && !(std::getenv("CLV_TILED") && std::getenv("CLV_TILED")[0] == '0')) {
        bool ok = false;
        if ((rc = build_axis_groups(e, true, e->energy_groups, ok))) return bail(rc);
        e->energy_axis = ok;
        if (!ok) e->energy_groups.clear();
    }
    const size_t fb = e->total_elems * e->elem_bytes;
    const size_t fb_scratch = e->fused ? 16 : fb;  // the fused path needs no kinetic/drift arrays
    // drift arrays: the separate-kernel path, and the fused and tiled two-pass paths when they
    // store the drift
    const size_t fb_drift =
        ((e->fused && e->dt_rule != CLV_DT_REF_MEANMAX) || (e->tiled && !e->store_drift)) ? 16 : fb;
    const size_t nparts = std::max<size_t>(1, e->task_capacity);
    const int nch = cfg->nchains;
    if ((rc = e->alloc(&e->fld[0][0], fb)) || (rc = e->alloc(&e->fld[0][1], fb)) ||
        (rc = e->alloc(&e->fld[1][0], fb)) || (rc = e->alloc(&e->fld[1][1], fb)) ||
        (rc = e->alloc(&e->kin, fb)) || (rc = e->alloc(&e->kinc, fb_scratch)) ||
        (rc = e->alloc(&e->drift, fb_drift)) || (rc = e->alloc(&e->driftc, fb_drift)) ||
        (rc = e->alloc(&e->fused_tasks, (e->fused ? nparts : 1) * sizeof(FusedTask))) ||
        (rc = e->alloc(&e->fused_partials, nparts * sizeof(double2))) ||
        (rc = e->alloc(&e->tile_tasks, (e->tiled ? nparts : 1) * sizeof(TileTask))) ||
        (rc = e->alloc(&e->stage, 2 * e->max_chain_elems * sizeof(double2))) ||
        (rc = e->alloc(&e->chains_d, nch * sizeof(ChainDev))) ||
        (rc = e->alloc(&e->state_d, nch * sizeof(ChainState))) ||
        (rc = e->alloc(&e->site_tasks, e->site_tasks_h.size() * sizeof(SiteTask))) ||
        (rc = e->alloc(&e->obs_tasks, e->obs_tasks_h.size() * sizeof(SiteTask))) ||
        (rc = e->alloc(&e->partials, e->site_tasks_h.size() * sizeof(double2))) ||
        (rc = e->alloc(&e->s1obs_tasks, std::max<size_t>(1, e->s1obs_tasks_h.size()) * sizeof(ObsTask))) ||
        (rc = e->alloc(&e->s1obs_partials, std::max<size_t>(1, e->s1obs_tasks_h.size()) * 8 * sizeof(double))) ||
        (rc = e->alloc(&e->s1obs_arrive, nch * sizeof(unsigned int))) ||
        (rc = e->alloc(&e->accF, std::max(1, e->acc_F_total) * sizeof(double))) ||
        (rc = e->alloc(&e->accN, nch * 5 * sizeof(double))) ||
        (rc = e->alloc(&e->samples, (size_t)e->sample_cap * nch * 8 * sizeof(double))) ||
        (rc = e->alloc(&e->loop_sync, 2 * sizeof(unsigned int))))
        return bail(rc);
    {
        // the step loop's normals: for problems whose split tasks of one imaginary time
        // can all be resident at once (the only ones the loop takes)
        long long slices = 0;
        for (auto &d : e->chains_h) slices += d.nt;
        if (e->fused && e->fused_ln > 0 && e->loop_per_sm > 0 &&
            2 * slices <= (long long)e->loop_per_sm * e->num_sms && (rc = e->alloc(&e->loop_noise, fb)))
            return bail(rc);
    }
    for (int a = 0; a < 3; ++a)
        if (!e->line_tasks_h[a].empty() &&
            (rc = e->alloc(&e->line_tasks[a], e->line_tasks_h[a].size() * sizeof(LineTask))))
            return bail(rc);
    for (auto &g : e->axis_groups)
        if ((rc = e->alloc(&g.d, g.tasks.size() * sizeof(AxisTask)))) return bail(rc);
    for (auto &g : e->energy_groups)
        if ((rc = e->alloc(&g.d, g.tasks.size() * sizeof(AxisTask)))) return bail(rc);
    auto up = [&](void *d, const void *h, size_t b) {
        return cudaMemcpy(d, h, b, cudaMemcpyHostToDevice);
    };
    if (e->fused &&
        (ce = up(e->fused_tasks, e->fused_tasks_h.data(), e->fused_tasks_h.size() * sizeof(FusedTask))) != cudaSuccess)
        return bail(fail(CLV_ERR_CUDA, cudaGetErrorString(ce)));
    if (e->tiled &&
        (ce = up(e->tile_tasks, e->tile_tasks_h.data(), e->tile_tasks_h.size() * sizeof(TileTask))) != cudaSuccess)
        return bail(fail(CLV_ERR_CUDA, cudaGetErrorString(ce)));
    for (auto *gs : {&e->axis_groups, &e->energy_groups})
        for (auto &g : *gs)
            if ((ce = up(g.d, g.tasks.data(), g.tasks.size() * sizeof(AxisTask))) != cudaSuccess)
                return bail(fail(CLV_ERR_CUDA, cudaGetErrorString(ce)));
    if ((ce = up(e->chains_d, e->chains_h.data(), nch * sizeof(ChainDev))) != cudaSuccess ||
        (ce = up(e->site_tasks, e->site_tasks_h.data(), e->site_tasks_h.size() * sizeof(SiteTask))) != cudaSuccess ||
        (ce = up(e->obs_tasks, e->obs_tasks_h.data(), e->obs_tasks_h.size() * sizeof(SiteTask))) != cudaSuccess ||
        (ce = up(e->s1obs_tasks, e->s1obs_tasks_h.data(), e->s1obs_tasks_h.size() * sizeof(ObsTask))) != cudaSuccess ||
        (ce = cudaMemset(e->s1obs_arrive, 0, nch * sizeof(unsigned int))) != cudaSuccess)
        return bail(fail(CLV_ERR_CUDA, cudaGetErrorString(ce)));
    for (int a = 0; a < 3; ++a)
        if (!e->line_tasks_h[a].empty() &&
            (ce = up(e->line_tasks[a], e->line_tasks_h[a].data(),
                     e->line_tasks_h[a].size() * sizeof(LineTask))) != cudaSuccess)
            return bail(fail(CLV_ERR_CUDA, cudaGetErrorString(ce)));
    std::vector<ChainState> st(nch);
    std::memset(st.data(), 0, nch * sizeof(ChainState));
    for (int c = 0; c < nch; ++c) {
        st[c].dt = e->model == CLV_MODEL_REF4 ? e->params[c].DT : e->params[c].dt_max;
    }
    if ((ce = up(e->state_d, st.data(), nch * sizeof(ChainState))) != cudaSuccess)
        return bail(fail(CLV_ERR_CUDA, cudaGetErrorString(ce)));
    const size_t fbz = e->total_elems * e->elem_bytes;
    if ((ce = cudaMemset(e->fld[0][0], 0, fbz)) != cudaSuccess || (ce = cudaMemset(e->fld[0][1], 0, fbz)) != cudaSuccess ||
        (ce = cudaMemset(e->fld[1][0], 0, fbz)) != cudaSuccess || (ce = cudaMemset(e->fld[1][1], 0, fbz)) != cudaSuccess ||
        (ce = cudaMemset(e->accF, 0, std::max(1, e->acc_F_total) * sizeof(double))) != cudaSuccess ||
        (ce = cudaMemset(e->accN, 0, nch * 5 * sizeof(double))) != cudaSuccess ||
        (ce = cudaMemset(e->samples, 0, (size_t)e->sample_cap * nch * 8 * sizeof(double))) != cudaSuccess)
        return bail(fail(CLV_ERR_CUDA, cudaGetErrorString(ce)));
    *out = e;
    return CLV_OK;
}

int clv_destroy(clv_engine *e) {
    if (!e) return CLV_OK;
    cudaSetDevice(e->device);
    if (e->stream) cudaStreamSynchronize(e->stream);
    e->drop_graphs();
    for (void *p : e->allocs) cudaFree(p);
    if (e->noise_d) cudaFree(e->noise_d);
    if (e->stage_all) cudaFree(e->stage_all);
    if (e->own_stream && e->stream) cudaStreamDestroy(e->stream);
    delete e;
    return CLV_OK;
}

int clv_set_stream(clv_engine *e, void *stream) {
    if (!e) return fail(CLV_ERR_ARG, "null engine");
    CK(cudaSetDevice(e->device));
    CK(cudaStreamSynchronize(e->stream));
    if (e->own_stream) cudaStreamDestroy(e->stream);
    e->stream = (cudaStream_t)stream;
    e->own_stream = false;
    e->drop_graphs();
    return CLV_OK;
}

int clv_synchronize(clv_engine *e) {
    if (!e) return fail(CLV_ERR_ARG, "null engine");
    CK(cudaSetDevice(e->device));
    CK(cudaStreamSynchronize(e->stream));
    return CLV_OK;
}

// Copies between the boundary layout (complex128) and the engine's buffers for
// chains [c0, c1), whose boundary arrays are concatenated in chain order.  The
// chains are contiguous in the engine's buffers too, so every field moves with
// one copy (and, at FP32, one conversion kernel) through a staging buffer sized
// for the range, allocated on first use.
static int copy_fields(clv_engine *e, int c0, int c1, const void *const src_in[2],
                       void *const dst_in[2], int where, bool to_engine) {
    const long long off = e->chains_h[c0].off;
    const ChainDev &last = e->chains_h[c1 - 1];
    const long long n = last.off + (long long)e->ncomp * last.nt * last.V - off;
    // complex64 boundary buffers (CLV_C64): moved as they are at FP32, converted
    // through the staging buffer at FP64; complex128 the other way round
    const bool c64 = (where & CLV_C64) != 0;
    const size_t ub = c64 ? 8 : 16;  // bytes per element of the caller's buffers
    const bool direct = c64 == (e->precision != CLV_PREC_F64);
    double2 *stage = e->stage;
    if (!direct && n > e->max_chain_elems) {
        if (e->stage_all_elems < n) {
            if (e->stage_all) cudaFree(e->stage_all);
            e->stage_all = nullptr;
            e->stage_all_elems = 0;
            void *q = nullptr;
            CK(cudaMalloc(&q, n * sizeof(double2)));
            e->stage_all = (double2 *)q;
            e->stage_all_elems = n;
        }
        stage = e->stage_all;
    }
    for (int f = 0; f < 2; ++f) {
        char *eng = (char *)e->fld[e->cur][f] + off * e->elem_bytes;
        if (to_engine) {
            if (!src_in[f]) continue;
            if (direct) {
                CK(cudaMemcpyAsync(eng, src_in[f], n * ub, kind_of(where, true), e->stream));
            } else {
                CK(cudaMemcpyAsync(stage, src_in[f], n * ub, kind_of(where, true), e->stream));
                if (c64) CK(launch_export<float>((double2 *)eng, stage, n, e->stream));
                else CK(launch_import<float>(eng, stage, n, e->stream));
            }
        } else {
            if (!dst_in[f]) continue;
            if (direct) {
                CK(cudaMemcpyAsync(dst_in[f], eng, n * ub, kind_of(where, false), e->stream));
            } else {
                if (c64) CK(launch_import<float>(stage, (const double2 *)eng, n, e->stream));
                else CK(launch_export<float>(stage, eng, n, e->stream));
                CK(cudaMemcpyAsync(dst_in[f], stage, n * ub, kind_of(where, false), e->stream));
            }
        }
    }
    if (!(where & CLV_ASYNC)) CK(cudaStreamSynchronize(e->stream));
    return CLV_OK;
}

int clv_set_fields(clv_engine *e, int chain, const void *psi, const void *psic, int where) {
    if (!e) return fail(CLV_ERR_ARG, "null engine");
    if (where & ~(CLV_DEVICE | CLV_C64 | CLV_ASYNC))
        return fail(CLV_ERR_ARG, "where: CLV_HOST or CLV_DEVICE, optionally | CLV_C64 | CLV_ASYNC");
    if (chain != -1) {
        int rc = check_chain(e, chain);
        if (rc) return rc;
    }
    CK(cudaSetDevice(e->device));
    const void *src[2] = {psi, psic};
    void *const dst[2] = {nullptr, nullptr};
    return chain == -1 ? copy_fields(e, 0, (int)e->params.size(), src, dst, where, true)
                       : copy_fields(e, chain, chain + 1, src, dst, where, true);
}

int clv_get_fields(clv_engine *e, int chain, void *psi, void *psic, int where) {
    if (!e) return fail(CLV_ERR_ARG, "null engine");
    if (where & ~(CLV_DEVICE | CLV_C64 | CLV_ASYNC))
        return fail(CLV_ERR_ARG, "where: CLV_HOST or CLV_DEVICE, optionally | CLV_C64 | CLV_ASYNC");
    if (chain != -1) {
        int rc = check_chain(e, chain);
        if (rc) return rc;
    }
    CK(cudaSetDevice(e->device));
    const void *const src[2] = {nullptr, nullptr};
    void *dst[2] = {psi, psic};
    return chain == -1 ? copy_fields(e, 0, (int)e->params.size(), src, dst, where, false)
                       : copy_fields(e, chain, chain + 1, src, dst, where, false);
}

int clv_set_mean_field(clv_engine *e, int field, double re, double im) {
    if (!e) return fail(CLV_ERR_ARG, "null engine");
    if (field != 0 && field != 1) return fail(CLV_ERR_ARG, "field must be 0 or 1");
    CK(cudaSetDevice(e->device));
    LaunchSites L = e->sites();
    if (e->precision == CLV_PREC_F64) CK(launch_set_mean_field<double>(L, field, re, im, e->stream));
    else CK(launch_set_mean_field<float>(L, field, re, im, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    return CLV_OK;
}

int clv_set_chemical_potential(clv_engine *e, int chain, double mu, double P) {
    if (!e) return fail(CLV_ERR_ARG, "null engine");
    if (chain != -1) {
        int rc = check_chain(e, chain);
        if (rc) return rc;
    }
    if (!std::isfinite(mu) || !std::isfinite(P)) return fail(CLV_ERR_ARG, "mu and P must be finite");
    CK(cudaSetDevice(e->device));
    const int c0 = chain == -1 ? 0 : chain, c1 = chain == -1 ? (int)e->params.size() : chain + 1;
    for (int c = c0; c < c1; ++c) {
        e->params[c].mu = mu;
        e->params[c].P = P;
        ChainDev &d = e->chains_h[c];
        d.mu = mu;
        d.P = P;
        for (int a = 0; a < kMaxComp; ++a) {
            const double m = 1.0 - a;
            d.comp_const[a] = std::exp(d.eps * (mu + d.q * m * m));
        }
    }
    // stream-ordered update of the device copies; captured graphs read them at run time
    CK(cudaMemcpyAsync(e->chains_d + c0, e->chains_h.data() + c0, (c1 - c0) * sizeof(ChainDev),
                       cudaMemcpyHostToDevice, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    return CLV_OK;
}

int clv_init_spin1(clv_engine *e, double amp, double sigma) {
    if (!e) return fail(CLV_ERR_ARG, "null engine");
    CK(cudaSetDevice(e->device));
    LaunchSites L = e->sites();
    if (e->precision == CLV_PREC_F64) CK(launch_init_spin1<double>(L, amp, sigma, e->stream));
    else CK(launch_init_spin1<float>(L, amp, sigma, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    return CLV_OK;
}

// Steps per block graph: long step sequences replay graphs of kStepBlock steps, so
// small lattices (the reference's own 256 x 32) pay one graph launch per block
// instead of one per step.
constexpr int kStepBlock = 16;
static_assert(kStepBlock % 2 == 0, "a block must return to its starting buffer set");

static int capture_steps(clv_engine *e, int from, int n, cudaGraph_t *g_out, cudaGraphExec_t *x_out) {
    CK(cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
    int rc = CLV_OK;
    for (int i = 0; i < n && rc == CLV_OK; ++i) rc = enqueue_step_any(e, false, nullptr, from ^ (i & 1));
    cudaGraph_t g = nullptr;
    cudaError_t ce = cudaStreamEndCapture(e->stream, &g);
    if (rc) { if (g) cudaGraphDestroy(g); return rc; }
    if (ce != cudaSuccess) return fail(CLV_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(ce));
    *g_out = g;
    CK(cudaGraphInstantiate(x_out, g, 0));
    return CLV_OK;
}

int clv_step(clv_engine *e, int nsteps) {
    if (!e) return fail(CLV_ERR_ARG, "null engine");
    if (nsteps < 0) return fail(CLV_ERR_ARG, "nsteps must be >= 0");
    CK(cudaSetDevice(e->device));
    if (nsteps == 0) return CLV_OK;
    if (use_loop(e)) {
        int done = 0;
        const int rc = enqueue_loop_any(e, nsteps, nullptr, &done);
        if (rc != kLoopRefused) return rc;
        nsteps -= done;  // the graphs take the rest
    }
    // graphs need a capturable stream (not the legacy default stream)
    if (nsteps == 1 || e->stream == nullptr || std::getenv("CLV_NO_GRAPH")) {
        for (int i = 0; i < nsteps; ++i) {
            int rc = enqueue_step_any(e, false, nullptr, e->cur);
            if (rc) return rc;
            e->cur ^= 1;
        }
        return CLV_OK;
    }
    while (nsteps >= kStepBlock) {
        const int from = e->cur;
        if (!e->block_exec[from]) {
            int rc = capture_steps(e, from, kStepBlock, &e->block_graph[from], &e->block_exec[from]);
            if (rc) return rc;
        }
        CK(cudaGraphLaunch(e->block_exec[from], e->stream));
        nsteps -= kStepBlock;
    }
    for (int i = 0; i < nsteps; ++i) {
        const int from = e->cur;
        if (!e->graph_exec[from]) {
            int rc = capture_steps(e, from, 1, &e->graph[from], &e->graph_exec[from]);
            if (rc) return rc;
        }
        CK(cudaGraphLaunch(e->graph_exec[from], e->stream));
        e->cur ^= 1;
    }
    return CLV_OK;
}

int clv_step_timed(clv_engine *e, float *phase_ms, int capacity, int *nphases) {
    if (!e) return fail(CLV_ERR_ARG, "null engine");
    CK(cudaSetDevice(e->device));
    EventTrail trail;
    int rc;
    if (use_loop(e) && (rc = enqueue_loop_any(e, 1, &trail)) != kLoopRefused) {
        if (rc) return rc;  // (two marks, bracketing the launch)
    } else {
        CK(trail.mark(e->stream));
        rc = enqueue_step_any(e, false, &trail, e->cur);
        if (rc) return rc;
        e->cur ^= 1;
    }
    CK(cudaStreamSynchronize(e->stream));
    const int n = (int)trail.ev.size() - 1;
    for (int i = 0; i < n && i < capacity; ++i) {
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, trail.ev[i], trail.ev[i + 1]));
        if (phase_ms) phase_ms[i] = ms;
    }
    if (nphases) *nphases = n;
    return CLV_OK;
}

int clv_step_with_noise(clv_engine *e, const double *noise, int where) {
    if (!e) return fail(CLV_ERR_ARG, "null engine");
    if (!noise) return fail(CLV_ERR_ARG, "null noise");
    if (where != CLV_HOST && where != CLV_DEVICE) return fail(CLV_ERR_ARG, "where: CLV_HOST or CLV_DEVICE");
    CK(cudaSetDevice(e->device));
    if (!e->noise_d) {
        void *p = nullptr;
        CK(cudaMalloc(&p, e->noise_total * sizeof(double)));
        e->noise_d = (double *)p;
    }
    CK(cudaMemcpyAsync(e->noise_d, noise, e->noise_total * sizeof(double), kind_of(where, true),
                       e->stream));
    int rc = enqueue_step_any(e, true, nullptr, e->cur);
    if (rc) return rc;
    e->cur ^= 1;
    if (where == CLV_HOST) CK(cudaStreamSynchronize(e->stream));
    return CLV_OK;
}

int clv_get_step_info(clv_engine *e, double *dt, double *max_drift, double *mean_drift,
                      double *langevin_time, uint64_t *steps) {
    if (!e) return fail(CLV_ERR_ARG, "null engine");
    CK(cudaSetDevice(e->device));
    const int nch = (int)e->params.size();
    std::vector<ChainState> st(nch);
    CK(cudaMemcpyAsync(st.data(), e->state_d, nch * sizeof(ChainState), cudaMemcpyDeviceToHost,
                       e->stream));
    CK(cudaStreamSynchronize(e->stream));
    for (int c = 0; c < nch; ++c) {
        if (dt) dt[c] = st[c].dt;
        if (max_drift) max_drift[c] = st[c].max;
        if (mean_drift) mean_drift[c] = st[c].mean;
        if (langevin_time) langevin_time[c] = st[c].t;
        if (steps) steps[c] = st[c].step;
    }
    return CLV_OK;
}

int clv_get_chain_flags(clv_engine *e, int *flags) {
    if (!e || !flags) return fail(CLV_ERR_ARG, "null argument");
    CK(cudaSetDevice(e->device));
    const int nch = (int)e->params.size();
    std::vector<ChainState> st(nch);
    CK(cudaMemcpyAsync(st.data(), e->state_d, nch * sizeof(ChainState), cudaMemcpyDeviceToHost,
                       e->stream));
    CK(cudaStreamSynchronize(e->stream));
    int any = 0;
    for (int c = 0; c < nch; ++c) {
        flags[c] = st[c].flags;
        any |= st[c].flags;
    }
    if (any & CLV_FLAG_TIMEOUT)
        return fail(CLV_ERR_TIMEOUT, "a bounded device-side wait gave up (a chain's step is incomplete)");
    return (any & CLV_FLAG_NONFINITE) ? fail(CLV_ERR_NONFINITE, "a chain's drift became non-finite") : CLV_OK;
}

int clv_evaluate(clv_engine *e) {
    if (!e) return fail(CLV_ERR_ARG, "null engine");
    CK(cudaSetDevice(e->device));
    const int nch = (int)e->params.size();
    if (e->model == CLV_MODEL_REF4) {
        LaunchSites L = e->sites(true);
        if (e->precision == CLV_PREC_F64) CK(launch_obs_ref<double>(L, e->accF, e->accN, e->stream));
        else CK(launch_obs_ref<float>(L, e->accF, e->accN, e->stream));
    } else {
        if (e->sample_count == e->sample_cap) {
            // move the full sample buffer to the host and start over
            const size_t n = (size_t)e->sample_cap * nch * 8;
            const size_t old = e->sample_spill.size();
            e->sample_spill.resize(old + n);
            CK(cudaMemcpyAsync(e->sample_spill.data() + old, e->samples, n * sizeof(double),
                               cudaMemcpyDeviceToHost, e->stream));
            CK(cudaMemsetAsync(e->samples, 0, n * sizeof(double), e->stream));
            CK(cudaStreamSynchronize(e->stream));
            e->sample_spilled += e->sample_cap;
            e->sample_count = 0;
        }
        if (e->energy_axis) {
            // kinetic energy sum_a (k_a^2/2) psi: the first axis writes, the others add
            for (const auto &g : e->energy_groups) {
                LaunchAxis A{};
                A.chains = e->chains_d;
                A.tasks = g.d;
                A.ntasks = (int)g.tasks.size();
                A.axis = g.axis;
                A.n = g.n;
                A.W = g.W;
                A.pitch = g.pitch;
                A.with_const = 0;
                A.src0 = e->psi();
                A.dst0 = e->kin;
                A.smem_bytes = g.smem;
                A.nfields = 1;
                A.filter = 1;
                A.accumulate = g.axis > 0;
                A.strided = g.strided;
                if (e->precision == CLV_PREC_F64) CK(launch_axis_filter<double>(A, e->stream));
                else CK(launch_axis_filter<float>(A, e->stream));
            }
        } else {
            int rc = e->precision == CLV_PREC_F64
                         ? run_kinetic<double>(e, e->psi(), nullptr, e->kin, nullptr, 1, 1)
                         : run_kinetic<float>(e, e->psi(), nullptr, e->kin, nullptr, 1, 1);
            if (rc) return rc;
        }
        LaunchObs L{};
        L.chains = e->chains_d;
        L.tasks = e->s1obs_tasks;
        L.ntasks = (int)e->s1obs_tasks_h.size();
        L.psi = e->psi();
        L.psic = e->psic();
        L.tpsi = e->kin;
        L.partials = e->s1obs_partials;
        L.arrive = e->s1obs_arrive;
        L.samples = e->samples;
        L.slot = e->sample_count;
        L.nchains = nch;
        if (e->precision == CLV_PREC_F64) CK(launch_obs_spin1<double>(L, e->stream));
        else CK(launch_obs_spin1<float>(L, e->stream));
        e->sample_count++;
    }
    e->counter++;
    return CLV_OK;
}

int clv_get_counter(clv_engine *e) { return e ? e->counter : 0; }

int clv_read_ref_observables(clv_engine *e, int chain, double *n, double *F_x, double *F_y,
                             double *F_z) {
    int rc = check_chain(e, chain);
    if (rc) return rc;
    if (e->model != CLV_MODEL_REF4) return fail(CLV_ERR_STATE, "reference observables need the REF4 model");
    if (e->counter == 0) return fail(CLV_ERR_STATE, "evaluate() has not been called");
    CK(cudaSetDevice(e->device));
    const ChainDev &d = e->chains_h[chain];
    std::vector<double> F(3 * d.V), N(5);
    CK(cudaMemcpyAsync(F.data(), e->accF + d.obs_off, 3 * d.V * sizeof(double),
                       cudaMemcpyDeviceToHost, e->stream));
    CK(cudaMemcpyAsync(N.data(), e->accN + chain * 5, 5 * sizeof(double), cudaMemcpyDeviceToHost,
                       e->stream));
    CK(cudaStreamSynchronize(e->stream));
    // Observables::write_n_* (:1527-1547): /T /counter /V ; write_F_* (:1614-1634): /T /counter
    const double T = d.nt, cnt = e->counter, V = d.V;
    if (n)
        for (int i = 0; i < 5; ++i) n[i] = N[i] / T / cnt / V;
    double *outs[3] = {F_x, F_y, F_z};
    for (int k = 0; k < 3; ++k)
        if (outs[k])
            for (int s = 0; s < d.V; ++s) outs[k][s] = F[k * d.V + s] / T / cnt;
    return CLV_OK;
}

int clv_read_spin1_samples(clv_engine *e, int chain, double *samples, int capacity, int *count) {
    int rc = check_chain(e, chain);
    if (rc) return rc;
    if (e->model != CLV_MODEL_SPIN1) return fail(CLV_ERR_STATE, "spin-1 samples need the SPIN1 model");
    CK(cudaSetDevice(e->device));
    const int nch = (int)e->params.size();
    const int total = e->sample_spilled + e->sample_count;
    // only this chain's rows of the device buffer ([k][chain][8]), and only what fits
    const int want = samples ? std::min(capacity, total) : 0;
    const int ndev = std::max(0, want - e->sample_spilled);
    std::vector<double> dev((size_t)ndev * 8);
    if (ndev > 0) {
        CK(cudaMemcpy2DAsync(dev.data(), 8 * sizeof(double), e->samples + (size_t)chain * 8,
                             (size_t)nch * 8 * sizeof(double), 8 * sizeof(double), ndev,
                             cudaMemcpyDeviceToHost, e->stream));
        CK(cudaStreamSynchronize(e->stream));
    }
    for (int k = 0; k < want; ++k) {
        const double *src = k < e->sample_spilled ? &e->sample_spill[((size_t)k * nch + chain) * 8]
                                                  : &dev[(size_t)(k - e->sample_spilled) * 8];
        std::memcpy(samples + (size_t)k * 8, src, 8 * sizeof(double));
    }
    if (count) *count = samples ? want : total;
    return CLV_OK;
}

// Re-plan with explicit knobs (chunk length; fused path: bulk copies, compile-time
// line length) and upload the new task tables; the captured graphs are dropped.
static int apply_plan(clv_engine *e, int L, int tma, int ln, int sd) {
    auto up = [&](void *d, const void *h, size_t b) {
        return cudaMemcpyAsync(d, h, b, cudaMemcpyHostToDevice, e->stream);
    };
    if (e->fused) {
        build_fused_tasks(e, L);
        e->use_tma = tma && e->fused_aligned;
        e->store_drift = sd && e->dt_rule == CLV_DT_REF_MEANMAX;
        if (ln != e->fused_ln) {
            LaunchFused probe{};
            probe.model = e->model;
            probe.spt = e->fused_spt;
            probe.ln = ln;
            probe.smem_bytes = e->fused_smem;
            int per_sm = 0;
            if (e->precision == CLV_PREC_F64) CK(setup_fused<double>(probe, &per_sm));
            else CK(setup_fused<float>(probe, &per_sm));
            if (per_sm < 1) return fail(CLV_ERR_ARG, "fused plan variant does not fit");
            e->fused_ln = ln;
        }
        CK(up(e->fused_tasks, e->fused_tasks_h.data(), e->fused_tasks_h.size() * sizeof(FusedTask)));
    } else if (e->tiled) {
        build_tiled_tasks(e, L);
        CK(up(e->tile_tasks, e->tile_tasks_h.data(), e->tile_tasks_h.size() * sizeof(TileTask)));
    }
    CK(up(e->chains_d, e->chains_h.data(), e->chains_h.size() * sizeof(ChainDev)));
    CK(cudaStreamSynchronize(e->stream));
    e->drop_graphs();
    return CLV_OK;
}

int clv_autotune(clv_engine *e, int trial_steps, char *report, int capacity) {
    if (!e) return fail(CLV_ERR_ARG, "null engine");
    CK(cudaSetDevice(e->device));
    trial_steps = std::max(1, trial_steps);
    std::string rep;
    if (!e->fused && !e->tiled) {
        rep = "no tunable plan (separate line-filter, drift and update kernels)";
    } else {
        struct Cand { int L, tma, ln, sd; float ms; };
        std::vector<Cand> cands;
        int tmax = 0;
        for (auto &d : e->chains_h) tmax = std::max(tmax, d.nt);
        std::vector<int> Ls = {e->chunk};
        for (int L : {1, 2, 4, 8, 16, 32, 64})
            if (L <= tmax && L != e->chunk) Ls.push_back(L);
        for (int L : Ls) {
            if (e->fused) {
                for (int tma : {1, 0}) {
                    if (tma && !e->fused_aligned) continue;
                    for (int ln : {e->fused_ln_static, 0}) {
                        for (int sd : {0, 1}) {
                            if (sd && e->dt_rule != CLV_DT_REF_MEANMAX) continue;
                            cands.push_back({L, tma, ln, sd, 0.f});
                        }
                        if (e->fused_ln_static == 0) break;
                    }
                }
            } else {
                cands.push_back({L, 0, 0, 0, 0.f});
            }
        }
        // the trials run real steps: keep the state and restore it after each
        const size_t fb = (size_t)e->total_elems * e->elem_bytes;
        const int nch = (int)e->params.size();
        void *save[2] = {nullptr, nullptr};
        std::vector<ChainState> st(nch);
        const int cur0 = e->cur;
        cudaEvent_t ev0 = nullptr, ev1 = nullptr;
        auto cleanup = [&]() {
            for (void *p : save) if (p) cudaFree(p);
            if (ev0) cudaEventDestroy(ev0);
            if (ev1) cudaEventDestroy(ev1);
        };
        auto restore = [&]() -> cudaError_t {
            cudaError_t r;
            for (int f = 0; f < 2; ++f)
                if ((r = cudaMemcpyAsync(e->fld[cur0][f], save[f], fb, cudaMemcpyDeviceToDevice, e->stream)) != cudaSuccess)
                    return r;
            if ((r = cudaMemcpyAsync(e->state_d, st.data(), nch * sizeof(ChainState), cudaMemcpyHostToDevice,
                                     e->stream)) != cudaSuccess)
                return r;
            e->cur = cur0;
            return cudaStreamSynchronize(e->stream);
        };
        cudaError_t ce = cudaSuccess;
        for (int f = 0; f < 2 && ce == cudaSuccess; ++f) {
            ce = cudaMalloc(&save[f], fb);
            if (ce == cudaSuccess)
                ce = cudaMemcpyAsync(save[f], e->fld[cur0][f], fb, cudaMemcpyDeviceToDevice, e->stream);
        }
        if (ce == cudaSuccess)
            ce = cudaMemcpyAsync(st.data(), e->state_d, nch * sizeof(ChainState), cudaMemcpyDeviceToHost, e->stream);
        if (ce == cudaSuccess) ce = cudaStreamSynchronize(e->stream);
        if (ce == cudaSuccess) ce = cudaEventCreate(&ev0);
        if (ce == cudaSuccess) ce = cudaEventCreate(&ev1);
        if (ce != cudaSuccess) {
            cleanup();
            return fail(CLV_ERR_NOMEM, std::string("autotune state copy: ") + cudaGetErrorString(ce));
        }
        int best = -1;
        for (int i = 0; i < (int)cands.size(); ++i) {
            Cand &c = cands[i];
            int rc = apply_plan(e, c.L, c.tma, c.ln, c.sd);
            if (rc == CLV_OK && (ce = restore()) != cudaSuccess) rc = fail(CLV_ERR_CUDA, cudaGetErrorString(ce));
            if (rc == CLV_OK) rc = clv_step(e, 2);  // captures the graphs of both parities
            if (rc == CLV_OK) {
                cudaEventRecord(ev0, e->stream);
                rc = clv_step(e, trial_steps);
                cudaEventRecord(ev1, e->stream);
                if ((ce = cudaEventSynchronize(ev1)) != cudaSuccess) rc = fail(CLV_ERR_CUDA, cudaGetErrorString(ce));
            }
            if (rc != CLV_OK) {
                cleanup();
                return rc;
            }
            cudaEventElapsedTime(&c.ms, ev0, ev1);
            c.ms /= trial_steps;
            if (best < 0 || c.ms < cands[best].ms) best = i;
            char line[128];
            std::snprintf(line, sizeof line, "chunk=%d tma=%d static_line=%d stored_drift=%d: %.4f ms/step\n",
                          c.L, c.tma, c.ln, c.sd, c.ms);
            rep += line;
        }
        const Cand &b = cands[best];
        int rc = apply_plan(e, b.L, b.tma, b.ln, b.sd);
        if (rc == CLV_OK && (ce = restore()) != cudaSuccess) rc = fail(CLV_ERR_CUDA, cudaGetErrorString(ce));
        cleanup();
        if (rc) return rc;
        char line[128];
        std::snprintf(line, sizeof line, "chosen: chunk=%d tma=%d static_line=%d stored_drift=%d", b.L, b.tma,
                      b.ln, b.sd);
        rep += line;
    }
    e->tune_report = rep;
    if (report && capacity > 0) {
        const size_t n = std::min(rep.size(), (size_t)capacity - 1);
        std::memcpy(report, rep.data(), n);
        report[n] = 0;
    }
    return CLV_OK;
}

int clv_get_plan(clv_engine *e, char *buf, int capacity) {
    if (!e || !buf || capacity < 1) return fail(CLV_ERR_ARG, "null argument");
    std::string p;
    if (e->fused) {
        if (use_loop(e)) p = "fused:loop_step";
        else if (e->speculate && e->dt_rule == CLV_DT_K_OVER_MAX) p = "fused:fused_step,fused_redo";
        else if (e->store_drift) p = "fused:fused_reduce,stored_drift_update";
        else p = "fused:fused_reduce,fused_apply";
    } else if (e->tiled) {
        p = "tiled:";
        for (const auto &g : e->axis_groups)
            p += (g.plane ? "plane" + std::to_string(g.axis) + std::to_string(g.axis + 1) : "axis" + std::to_string(g.axis)) +
                 "_n" + std::to_string(g.n) + ",";
        p += (e->speculate && e->dt_rule == CLV_DT_K_OVER_MAX) ? "tiled_step,tiled_redo"
             : e->store_drift ? "tiled_reduce,stored_drift_update" : "tiled_reduce,tiled_apply";
    } else {
        p = "unfused:";
        for (int a = 0; a < 3; ++a) {
            if (e->line_tasks_h[a].empty()) continue;
            if (e->kinetic == CLV_KIN_REF_LINEAR_PX && a > 0) break;
            p += "kinetic_axis" + std::to_string(a) + ",";
        }
        p += "drift,update";
    }
    if ((int)p.size() >= capacity) return fail(CLV_ERR_ARG, "buffer too small for the plan");
    std::memcpy(buf, p.c_str(), p.size() + 1);
    return CLV_OK;
}

int clv_device_bytes(clv_engine *e, size_t *bytes) {
    if (!e || !bytes) return fail(CLV_ERR_ARG, "null argument");
    *bytes = e->dev_bytes + (e->noise_d ? e->noise_total * sizeof(double) : 0);
    return CLV_OK;
}

// ------------------------------------------------------------- checkpoint
// File: magic "CLVCKPT1", int32 header {version, model, precision, ncomp, nchains},
// per chain {nx, ny, nz, nt}, ChainState[nchains], int32 counter, sample state,
// then per chain psi, psibar (complex128, boundary layout), F accumulators,
// N accumulators and the spin-1 samples.
int clv_save_checkpoint(clv_engine *e, const char *path) {
    if (!e || !path) return fail(CLV_ERR_ARG, "null argument");
    CK(cudaSetDevice(e->device));
    const int nch = (int)e->params.size();
    FILE *f = std::fopen(path, "wb");
    if (!f) return fail(CLV_ERR_IO, std::string("cannot open ") + path);
    bool ok = true;
    auto W = [&](const void *p, size_t b) { ok = ok && std::fwrite(p, 1, b, f) == b; };
    W("CLVCKPT1", 8);
    const int hdr[5] = {CLV_API_VERSION, e->model, e->precision, e->ncomp, nch};
    W(hdr, sizeof hdr);
    for (auto &p : e->params) { const int dims[4] = {p.nx, p.ny, p.nz, p.nt}; W(dims, sizeof dims); }
    std::vector<ChainState> st(nch);
    cudaError_t ce = cudaMemcpyAsync(st.data(), e->state_d, nch * sizeof(ChainState),
                                     cudaMemcpyDeviceToHost, e->stream);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(e->stream);
    if (ce != cudaSuccess) { std::fclose(f); return fail(CLV_ERR_CUDA, cudaGetErrorString(ce)); }
    W(st.data(), nch * sizeof(ChainState));
    const int counters[3] = {e->counter, e->sample_count, e->sample_spilled};
    W(counters, sizeof counters);
    std::vector<double2> a(e->max_chain_elems), b(e->max_chain_elems);
    for (int c = 0; c < nch && ok; ++c) {
        int rc = clv_get_fields(e, c, a.data(), b.data(), CLV_HOST);
        if (rc) { std::fclose(f); return rc; }
        const long long n = (long long)e->ncomp * e->chains_h[c].nt * e->chains_h[c].V;
        W(a.data(), n * 16);
        W(b.data(), n * 16);
    }
    std::vector<double> F(std::max(1, e->acc_F_total)), N(nch * 5);
    std::vector<double> S((size_t)e->sample_count * nch * 8);
    ce = cudaMemcpy(F.data(), e->accF, F.size() * sizeof(double), cudaMemcpyDeviceToHost);
    if (ce == cudaSuccess) ce = cudaMemcpy(N.data(), e->accN, N.size() * sizeof(double), cudaMemcpyDeviceToHost);
    if (ce == cudaSuccess && !S.empty())
        ce = cudaMemcpy(S.data(), e->samples, S.size() * sizeof(double), cudaMemcpyDeviceToHost);
    if (ce != cudaSuccess) { std::fclose(f); return fail(CLV_ERR_CUDA, cudaGetErrorString(ce)); }
    W(F.data(), F.size() * sizeof(double));
    W(N.data(), N.size() * sizeof(double));
    W(S.data(), S.size() * sizeof(double));
    W(e->sample_spill.data(), e->sample_spill.size() * sizeof(double));
    if (std::fclose(f) != 0) ok = false;
    return ok ? CLV_OK : fail(CLV_ERR_IO, std::string("short write to ") + path);
}

int clv_load_checkpoint(clv_engine *e, const char *path) {
    if (!e || !path) return fail(CLV_ERR_ARG, "null argument");
    CK(cudaSetDevice(e->device));
    const int nch = (int)e->params.size();
    FILE *f = std::fopen(path, "rb");
    if (!f) return fail(CLV_ERR_IO, std::string("cannot open ") + path);
    bool ok = true;
    auto R = [&](void *p, size_t b) { ok = ok && std::fread(p, 1, b, f) == b; };
    char magic[8];
    int hdr[5];
    R(magic, 8);
    R(hdr, sizeof hdr);
    if (!ok || std::memcmp(magic, "CLVCKPT1", 8) != 0 || hdr[1] != e->model ||
        hdr[2] != e->precision || hdr[3] != e->ncomp || hdr[4] != nch) {
        std::fclose(f);
        return fail(CLV_ERR_IO, "checkpoint does not match this engine");
    }
    for (auto &p : e->params) {
        int dims[4];
        R(dims, sizeof dims);
        if (!ok || dims[0] != p.nx || dims[1] != p.ny || dims[2] != p.nz || dims[3] != p.nt) {
            std::fclose(f);
            return fail(CLV_ERR_IO, "checkpoint lattice sizes do not match");
        }
    }
    std::vector<ChainState> st(nch);
    R(st.data(), nch * sizeof(ChainState));
    int counters[3];
    R(counters, sizeof counters);
    if (!ok || counters[1] < 0 || counters[1] > e->sample_cap || counters[2] < 0) {
        std::fclose(f);
        return fail(CLV_ERR_IO, "truncated checkpoint");
    }
    std::vector<double2> a(e->max_chain_elems), b(e->max_chain_elems);
    for (int c = 0; c < nch && ok; ++c) {
        const long long n = (long long)e->ncomp * e->chains_h[c].nt * e->chains_h[c].V;
        R(a.data(), n * 16);
        R(b.data(), n * 16);
        if (!ok) break;
        int rc = clv_set_fields(e, c, a.data(), b.data(), CLV_HOST);
        if (rc) { std::fclose(f); return rc; }
    }
    std::vector<double> F(std::max(1, e->acc_F_total)), N(nch * 5);
    std::vector<double> S((size_t)counters[1] * nch * 8);
    std::vector<double> spill((size_t)counters[2] * nch * 8);
    R(F.data(), F.size() * sizeof(double));
    R(N.data(), N.size() * sizeof(double));
    R(S.data(), S.size() * sizeof(double));
    R(spill.data(), spill.size() * sizeof(double));
    std::fclose(f);
    if (!ok) return fail(CLV_ERR_IO, "truncated checkpoint");
    for (auto &s : st) s.arrive = 0;
    CK(cudaMemcpy(e->state_d, st.data(), nch * sizeof(ChainState), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(e->accF, F.data(), F.size() * sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(e->accN, N.data(), N.size() * sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaMemset(e->samples, 0, (size_t)e->sample_cap * nch * 8 * sizeof(double)));
    if (!S.empty()) CK(cudaMemcpy(e->samples, S.data(), S.size() * sizeof(double), cudaMemcpyHostToDevice));
    e->counter = counters[0];
    e->sample_count = counters[1];
    e->sample_spilled = counters[2];
    e->sample_spill = std::move(spill);
    return CLV_OK;
}

}  // extern "C"
