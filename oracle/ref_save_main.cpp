// ref_save_main.cpp -- drives the reference's SaveResults (host build) with the
// fake observables: make_directory, save_parameters, make_directory_rawdata and
// two snapshots, in the order main.cu uses them.  TEST INFRASTRUCTURE ONLY.
// usage: <binary> <output dir> <mu> <P> <seed>
#include <unistd.h>
int main(int argc, char **argv) {
    if (argc < 5) return 2;
    if (chdir(argv[1]) != 0) return 3;
    const double MU = atof(argv[2]), P = atof(argv[3]);
    const unsigned long long seed = strtoull(argv[4], nullptr, 10);
    struct which_observables which {};
    which.n_tot = true;
    which.n_11 = true; which.n_12 = true; which.n_21 = true; which.n_22 = true;
    which.F_x = true; which.F_y = true; which.F_z = true;
    Observables obs(which, XSIZE * YSIZE * ZSIZE);
    SaveResults save(&obs, seed);
    if (!save.make_directory(P, MU)) return 1;
    save.save_parameters(P, MU);
    save.make_directory_rawdata();
    obs.vals.counter = 1;
    save.save_snapshot(P, MU);
    obs.vals.counter = 7;
    save.save_snapshot(P, MU);
    return 0;
}
