// ref_shim_pre.hpp -- host-side execution shim for the reference's CUDA kernels.
//
// TEST INFRASTRUCTURE ONLY (oracle pinning).  oracle/ref_build.sh streams the
// reference's own kernel sources (Helpers.cu, Lattice.cu,
// Propagator_without_cutoff.cu and the observable kernels of
// Observables_without_cutoff.cu) between this prelude and ref_shim_post.cpp
// into g++, so that the reference's kernel bodies run on the host, one thread
// at a time (or one std::thread per CUDA thread where the kernel synchronises).
// The lattice configuration normally taken from Parameters.h comes from -D
// flags (see ref_build.sh).  Kernel launches in the reference's host methods are
// stripped by the build filter; those methods are compiled but never called.
#include <cuda_runtime_api.h>
#include <cuComplex.h>
#include <cufft.h>
#include <curand.h>

#include <atomic>
#include <barrier>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <filesystem>
#include <fstream>
#include <functional>
#include <iostream>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <sys/stat.h>
#include <thread>
#include <vector>
using namespace std;

#undef __global__
#undef __device__
#undef __host__
#undef __shared__
#define __global__
#define __device__
#define __host__
#define __shared__

// CUDA built-in variables, per emulated thread.
thread_local uint3 threadIdx;
thread_local uint3 blockIdx;
thread_local dim3 blockDim;
thread_local dim3 gridDim;

static std::mutex g_atomic_mu;
static std::barrier<> *g_block_barrier = nullptr;

static inline void __syncthreads() {
    if (g_block_barrier) g_block_barrier->arrive_and_wait();
}
static inline unsigned long long atomicCAS(unsigned long long *a, unsigned long long cmp,
                                           unsigned long long val) {
    std::lock_guard<std::mutex> g(g_atomic_mu);
    unsigned long long old = *a;
    if (old == cmp) *a = val;
    return old;
}
static inline double atomicAdd(double *a, double v) {
    std::lock_guard<std::mutex> g(g_atomic_mu);
    double old = *a;
    *a = old + v;
    return old;
}
static inline long long __double_as_longlong(double d) {
    long long r;
    std::memcpy(&r, &d, sizeof r);
    return r;
}
static inline double __longlong_as_double(long long l) {
    double r;
    std::memcpy(&r, &l, sizeof r);
    return r;
}
