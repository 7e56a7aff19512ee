// ref_shim_post.cpp -- C entry points that run the reference's kernels on the
// host with the launch geometry the reference uses.  TEST INFRASTRUCTURE ONLY.
//
// Geometry (Propagator_without_cutoff.cu:332-335, Lattice.cu:114-122):
//   4-D kernels: block (BLOCKSIZEX, BLOCKSIZEY, BLOCKSIZEZ*BLOCKSIZETAU),
//                grid  (XSIZE/BLOCKSIZEX, YSIZE/BLOCKSIZEY, ZSIZE*TAUSIZE/(BLOCKSIZEZ*BLOCKSIZETAU))
//   1-D kernels: block BLOCKSIZE, grid length/BLOCKSIZE.

double sdata[1 << 15];  // backing store of `extern __shared__ double sdata[]`

static void emu_launch(dim3 g, dim3 b, const std::function<void()> &f) {
    for (unsigned bz = 0; bz < g.z; ++bz)
        for (unsigned by = 0; by < g.y; ++by)
            for (unsigned bx = 0; bx < g.x; ++bx)
                for (unsigned tz = 0; tz < b.z; ++tz)
                    for (unsigned ty = 0; ty < b.y; ++ty)
                        for (unsigned tx = 0; tx < b.x; ++tx) {
                            gridDim = g;
                            blockDim = b;
                            blockIdx = make_uint3(bx, by, bz);
                            threadIdx = make_uint3(tx, ty, tz);
                            f();
                        }
}

// Blocks run one after another; inside a block every CUDA thread is a
// std::thread so that __syncthreads() keeps its meaning.
static void emu_launch_sync(dim3 g, dim3 b, const std::function<void()> &f) {
    const unsigned nthr = b.x * b.y * b.z;
    for (unsigned bz = 0; bz < g.z; ++bz)
        for (unsigned by = 0; by < g.y; ++by)
            for (unsigned bx = 0; bx < g.x; ++bx) {
                std::barrier<> bar(nthr);
                g_block_barrier = &bar;
                std::vector<std::thread> th;
                th.reserve(nthr);
                for (unsigned t = 0; t < nthr; ++t)
                    th.emplace_back([&, t] {
                        gridDim = g;
                        blockDim = b;
                        blockIdx = make_uint3(bx, by, bz);
                        threadIdx = make_uint3(t % b.x, (t / b.x) % b.y, t / (b.x * b.y));
                        f();
                    });
                for (auto &x : th) x.join();
                g_block_barrier = nullptr;
            }
}

static dim3 blk4() { return dim3(BLOCKSIZEX, BLOCKSIZEY, BLOCKSIZEZ * BLOCKSIZETAU); }
static dim3 grd4() {
    return dim3(XSIZE / BLOCKSIZEX, YSIZE / BLOCKSIZEY, ZSIZE * TAUSIZE / (BLOCKSIZEZ * BLOCKSIZETAU));
}
static const int kLen = COMPONENTS * XSIZE * YSIZE * ZSIZE * TAUSIZE;

extern "C" {

void ref_config(int *out) {
    out[0] = XSIZE; out[1] = YSIZE; out[2] = ZSIZE; out[3] = TAUSIZE; out[4] = COMPONENTS;
}

void ref_compute_kinetic_part(cuDoubleComplex *psi, cuDoubleComplex *psic,
                              cuDoubleComplex *res, cuDoubleComplex *resc) {
    emu_launch(grd4(), blk4(), [&] { compute_kinetic_part(psi, psic, res, resc); });
}

void ref_normalization(cuDoubleComplex *data, double factor) {
    emu_launch(dim3(kLen / BLOCKSIZE), dim3(BLOCKSIZE), [&] { normalization(data, factor); });
}

void ref_drift(cuDoubleComplex *psi, cuDoubleComplex *psic, cuDoubleComplex *kin,
               cuDoubleComplex *kinc, cuDoubleComplex *drift, cuDoubleComplex *driftc,
               double factor, double P, double MU) {
    emu_launch(grd4(), blk4(), [&] {
        calculate_drift_without_noise(psi, psic, kin, kinc, drift, driftc, factor, P, MU);
    });
}

// get_max_and_mean_drift (Propagator_without_cutoff.cu:351-380): the same
// launch (grid = V*T/blocksize blocks) over the same total_size.
void ref_max_and_mean_drift(cuDoubleComplex *drift, double *max_out, double *mean_out) {
    const int total_size = kLen;
    const dim3 b = blk4(), g = grd4();
    const int blockSize = b.x * b.y * b.z;
    const int gridSize = g.x * g.y * g.z;
    double d_max = 0.0, d_sum = 0.0;
    emu_launch_sync(dim3(gridSize), dim3(blockSize), [&] {
        compute_max_and_mean_drift(drift, total_size, &d_max, &d_sum);
    });
    *max_out = d_max;
    *mean_out = d_sum / total_size;
}

// Propagator::compute_new_dt (:382-404) only reads its arguments and DT.
double ref_compute_new_dt(double mean, double max) {
    alignas(Propagator) unsigned char raw[sizeof(Propagator)];
    Propagator *self = reinterpret_cast<Propagator *>(raw);
    double dt = 0.0;
    self->compute_new_dt(mean, max, &dt);
    return dt;
}

void ref_multiply_by_timestep(cuDoubleComplex *d, cuDoubleComplex *dc, double dt) {
    emu_launch(grd4(), blk4(), [&] { multiply_by_timestep(d, dc, dt); });
}

void ref_add_noise(cuDoubleComplex *d, cuDoubleComplex *dc, double *random) {
    emu_launch(grd4(), blk4(), [&] { add_noise(d, dc, random); });
}

void ref_summation(cuDoubleComplex *a, cuDoubleComplex *b) {
    emu_launch(dim3(kLen / BLOCKSIZE), dim3(BLOCKSIZE), [&] { summation(a, b); });
}

void ref_set_value(cuDoubleComplex *data, double re, double im, int conjug, double P, double MU) {
    emu_launch(grd4(), blk4(), [&] { set_value(data, re, im, conjug != 0, P, MU); });
}

// evaluate_spin_density_realspace into V bins (atomicAdd is sequential here).
void ref_spin_density(cuDoubleComplex *psic, cuDoubleComplex *psi, double *bins, int spin_index) {
    std::memset(bins, 0, sizeof(double) * XSIZE * YSIZE * ZSIZE);
    emu_launch(grd4(), blk4(), [&] { evaluate_spin_density_realspace(psic, psi, bins, spin_index); });
}

// evaluate_n_tot (which = 0) / evaluate_n_11..22 (which = 1..4) into V*T values.
void ref_n_kernel(cuDoubleComplex *psic, cuDoubleComplex *psi, double *avg, int which) {
    emu_launch(grd4(), blk4(), [&] {
        switch (which) {
            case 0: evaluate_n_tot(psic, psi, avg); break;
            case 1: evaluate_n_11(psic, psi, avg); break;
            case 2: evaluate_n_12(psic, psi, avg); break;
            case 3: evaluate_n_21(psic, psi, avg); break;
            default: evaluate_n_22(psic, psi, avg); break;
        }
    });
}

}  // extern "C"
