// ref_save_fake.hpp -- deterministic stand-in for the reference's Observables
// class, with the methods SaveResults.cu calls.  TEST INFRASTRUCTURE ONLY: it
// lets the reference's own SaveResults.cu write its files on the host so that
// the engine's writer (include/clv_compat.hpp) can be compared byte for byte.
// The same values are produced by tests/compat_save_harness.cpp.
#pragma once

struct FakeObservableValues {
    int counter = 1;
    double n(int i) const { return (1.5 + 0.25 * i) / counter + 1e-7 * i; }
    double F(int k, int i) const { return 0.1 * i - 0.3 * k + 0.01 * counter + 1.0 / (3.0 + i); }
};

class Observables {
  public:
    explicit Observables(struct which_observables w, int V) : which_(w), V_(V) {}
    struct which_observables get_which() { return which_; }
    int get_counter() { return vals.counter; }
    void write_n_tot(double *w) { *w = vals.n(0); }
    void write_n_11(double *w) { *w = vals.n(1); }
    void write_n_12(double *w) { *w = vals.n(2); }
    void write_n_21(double *w) { *w = vals.n(3); }
    void write_n_22(double *w) { *w = vals.n(4); }
    void write_P2(double *w) { *w = 0.0; }
    void write_jrot2(double *) {}
    void write_spectrum(double *) {}
    void write_spectrum_tot(double *) {}
    void write_density_tot(double *) {}
    void write_density_11(double *) {}
    void write_density_12(double *) {}
    void write_density_21(double *) {}
    void write_density_22(double *) {}
    void write_F_x(double *w) { for (int i = 0; i < V_; ++i) w[i] = vals.F(0, i); }
    void write_F_y(double *w) { for (int i = 0; i < V_; ++i) w[i] = vals.F(1, i); }
    void write_F_z(double *w) { for (int i = 0; i < V_; ++i) w[i] = vals.F(2, i); }
    void write_anomalous_spectrum(double *) {}
    void write_dd(double *) {}
    void write_dispersion(double *) {}
    void write_drift(int *) {}
    FakeObservableValues vals;

  private:
    struct which_observables which_;
    int V_;
};
