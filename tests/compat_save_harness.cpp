// compat_save_harness.cpp -- writes the reference's output files with the
// engine's writer (clv_compat::SaveResultsT) for the deterministic observable
// values of oracle/ref_save_fake.hpp, so tests/test_compat_layout.py can compare
// them byte for byte with what the reference's SaveResults.cu wrote.
// usage: <binary> <output dir> <Parameters.h> <mu> <P> <seed>
#include <unistd.h>

#include "clv_compat.hpp"

namespace {
struct FakeObservableValues {
    int counter = 1;
    double n(int i) const { return (1.5 + 0.25 * i) / counter + 1e-7 * i; }
    double F(int k, int i) const { return 0.1 * i - 0.3 * k + 0.01 * counter + 1.0 / (3.0 + i); }
};

struct FakeObs {
    clv_compat::which_observables w;
    FakeObservableValues vals;
    long long V;
    clv_compat::which_observables get_which() { return w; }
    int get_counter() { return vals.counter; }
    long long volume() const { return V; }
    void write_n_tot(double *x) { *x = vals.n(0); }
    void write_n_11(double *x) { *x = vals.n(1); }
    void write_n_12(double *x) { *x = vals.n(2); }
    void write_n_21(double *x) { *x = vals.n(3); }
    void write_n_22(double *x) { *x = vals.n(4); }
    void write_F_x(double *x) { for (long long i = 0; i < V; ++i) x[i] = vals.F(0, (int)i); }
    void write_F_y(double *x) { for (long long i = 0; i < V; ++i) x[i] = vals.F(1, (int)i); }
    void write_F_z(double *x) { for (long long i = 0; i < V; ++i) x[i] = vals.F(2, (int)i); }
};
}  // namespace

int main(int argc, char **argv) {
    if (argc < 6) return 2;
    clv_compat::use_parameters(clv_compat::Parameters::from_header(argv[2]));
    if (chdir(argv[1]) != 0) return 3;
    const double MU = atof(argv[3]), P = atof(argv[4]);
    const unsigned long long seed = strtoull(argv[5], nullptr, 10);
    FakeObs obs;
    obs.w.n_tot = obs.w.n_11 = obs.w.n_12 = obs.w.n_21 = obs.w.n_22 = true;
    obs.w.F_x = obs.w.F_y = obs.w.F_z = true;
    obs.V = clv_compat::current_parameters().volume();
    clv_compat::SaveResultsT<FakeObs> save(&obs, seed);
    if (!save.make_directory(P, MU)) return 1;
    save.save_parameters(P, MU);
    save.make_directory_rawdata();
    obs.vals.counter = 1;
    save.save_snapshot(P, MU);
    obs.vals.counter = 7;
    save.save_snapshot(P, MU);
    return 0;
}
