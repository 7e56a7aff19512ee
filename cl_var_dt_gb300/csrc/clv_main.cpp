// clv_main.cpp -- drop-in replacement of the reference's main.cu (main.cu:53-162)
// on the GB300 engine: the same inputs (params.txt keys mu, P, seed, seed2 and
// the Parameters.h macros, read at run time from ./Parameters.h or the file
// named by CLV_PARAMETERS_H), the same loop (snapshot at step 1, every
// SNAPSHOT_TRIGGER steps and at the end; observables every EVALUATE_TRIGGER
// steps) and the same output files.
//
// usage: clv_main [device]
#include <cstdlib>
#include <ctime>
#include <iostream>

#include "clv_compat.hpp"

using namespace clv_compat;

int main(int argc, char **argv) {
    int devnum = 0;
    if (argc > 1) devnum = atoi(argv[1]);
    cudaSetDevice(devnum);
    const double timer = time(NULL);
    try {
        const char *hdr = std::getenv("CLV_PARAMETERS_H");
        use_parameters(Parameters::from_header(hdr ? hdr : "Parameters.h"));
    } catch (const Error &e) {
        std::cerr << e.what() << std::endl;
        return 1;
    }
    const Parameters &p = current_parameters();

    which_observables which;
    which.n_tot = true;
    which.n_11 = true; which.n_12 = true; which.n_21 = true; which.n_22 = true;
    which.F_x = true; which.F_y = true; which.F_z = true;

    auto params = read_params("params.txt");
    double MU = 0.0, P = 0.0;
    try {
        MU = params.at("mu");
        P = params.at("P");
    } catch (const std::out_of_range &) {
        std::cerr << "params.txt incomplete (mu or P missing)" << std::endl;
        return 1;
    }
    const unsigned long long seedvalue = static_cast<unsigned long long>(params["seed"]);
    const unsigned long long seedvalue2 = static_cast<unsigned long long>(params["seed2"]);

    try {
        ComplexLattice *fields = new ComplexLattice(false);
        ComplexLattice *fields_conjug = new ComplexLattice(true);
        ComplexLattice *drift = new ComplexLattice(false);
        ComplexLattice *drift_conjug = new ComplexLattice(true);
        Propagator *prop = new Propagator(fields, fields_conjug, drift, drift_conjug, seedvalue, seedvalue2);
        Observables *obs = new Observables(fields, fields_conjug, which);
        SaveResults *save = new SaveResults(obs, seedvalue);
        if (!save->make_directory(P, MU)) return 1;
        save->save_parameters(P, MU);
        save->make_directory_rawdata();

        fields->set_mean_field(0., 0., P, MU);
        fields_conjug->set_mean_field(0., 0., P, MU);

        std::cout << "Started simulation with parameters" << std::endl
                  << "T " << 1. / (p.TAUSIZE * p.EPS) << std::endl
                  << "mu " << MU << std::endl
                  << "g " << p.G << std::endl
                  << "M " << p.M << std::endl
                  << "SIGMA " << p.SIGMA << std::endl
                  << "D " << p.D << std::endl
                  << "OMEGAX " << p.OMEGAX << std::endl
                  << "OMEGAY " << p.OMEGAY << std::endl
                  << "OMEGAZ " << p.OMEGAZ << std::endl
                  << "P " << P << std::endl
                  << "components " << p.COMPONENTS << std::endl
                  << "lattice " << p.XSIZE << "x" << p.YSIZE << "x" << p.ZSIZE << "x" << p.TAUSIZE << std::endl
                  << "dt " << p.DT << std::endl
                  << "steps " << p.STEPS << std::endl
                  << "seed " << seedvalue << std::endl;

        for (long long i = 0; i < p.STEPS; i++) {
            const bool is_snapshot_step = ((i % p.SNAPSHOT_TRIGGER) == 0) && i != 0 && i != p.STEPS - 1;
            if (is_snapshot_step || i == 1) save->save_snapshot(P, MU);
            prop->propagate(P, MU);
            if (i % p.EVALUATE_TRIGGER == 0) obs->evaluate(P, MU);
        }
        save->save_snapshot(P, MU);
    } catch (const Error &e) {
        std::cerr << e.what() << std::endl;
        return 1;
    }
    std::cout << "Finished simulation after computation time of " << time(NULL) - timer
              << " seconds." << std::endl;
    return 0;
}
