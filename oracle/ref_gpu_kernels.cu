// ref_gpu_kernels.cu -- TEST INFRASTRUCTURE ONLY (the oracle's GPU pin).
//
// The reference's own CUDA sources compiled as they stand, in the order and
// header context of the reference's main.cu (main.cu:1-34), for sm_103a device
// code only (nvcc -cubin).  Nothing is copied: oracle/ref_gpu_build.sh passes
// the directory that holds the reference sources as an include path and a
// generated header of Parameters.h macros, one cubin per lattice configuration.
// oracle/ref_gpu_runner.cpp loads the cubin with the CUDA driver API and drives
// its kernels in the order of Propagator::propagate
// (Propagator_without_cutoff.cu:406-442) with cuFFT and cuRAND.
#include <thrust/device_vector.h>
#include <thrust/host_vector.h>
#include <thrust/reduce.h>
#include <thrust/functional.h>
#include <thrust/iterator/transform_iterator.h>
#include <thrust/iterator/counting_iterator.h>
#include <thrust/iterator/discard_iterator.h>
#include <thrust/extrema.h>
#include <thrust/execution_policy.h>
#include <curand.h>
#include <cuComplex.h>
#include <cufft.h>
#include <iostream>
#include <ctime>
#include <stdio.h>
#include <complex>
#include <sys/stat.h>
#include <sys/types.h>
#include <string>
#include <sstream>
#include <fstream>
#include <errno.h>
#include <filesystem>
#include <map>
using namespace std;

// the lattice configuration (Parameters.h macros), written by ref_gpu_build.sh;
// included after the library headers, as main.cu includes Parameters.h
#include CLV_REF_PARAMETERS
#include "Helpers.cu"
#include "Lattice.cu"
#include "Propagator_without_cutoff.cu"
#include "Observables_without_cutoff.cu"
