// clv_compat.hpp -- the reference's host interface (ComplexLattice, Propagator,
// Observables, SaveResults, read_params) on top of the C ABI of libclv.so, so
// that main.cu's update loop (main.cu:217-281) compiles and runs unchanged in
// shape, with the compile-time Parameters.h macros read at run time instead.
//
// Differences from the reference, all deliberate:
//  - sizes and couplings come from a Parameters.h file parsed at run time
//    (use_parameters / Parameters::from_header), not from macros;
//  - the noise of propagate() is the engine's Philox stream keyed by `seed`
//    (the reference uses cuRAND XORWOW); inject_noise() reproduces the
//    reference's update for a given buffer of normals;
//  - the Propagator owns the fields on the device; ComplexLattice objects are
//    handles to them (before a Propagator exists they hold host values);
//  - errors throw clv_compat::Error instead of being ignored.
#pragma once

#include <cuComplex.h>
#include <cuda_runtime_api.h>

#include <cmath>
#include <cstdlib>
#include <complex>
#include <cstdio>
#include <filesystem>
#include <fstream>
#include <iostream>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <sys/stat.h>
#include <vector>

#include "clv.h"

namespace clv_compat {

struct Error : std::runtime_error {
    int status;
    Error(int s, const std::string &m) : std::runtime_error(m), status(s) {}
};

inline void check(int rc) {
    if (rc != CLV_OK) throw Error(rc, std::string("clv: ") + clv_last_error());
}

// Parameters.h values (Parameters.h:1-53), read at run time.
struct Parameters {
    int COMPONENTS = 4, XSIZE = 256, YSIZE = 1, ZSIZE = 1, TAUSIZE = 32;
    double EPS = 0.01, a_x = 1.0, G = 0.1, M = 0.0, SIGMA = 0.0, D = 0.27735;
    double OMEGAX = 0.0, OMEGAY = 0.0, OMEGAZ = 0.0, Q = 0.0;
    long long STEPS = 8000000, SNAPSHOT_TRIGGER = 500000, EVALUATE_TRIGGER = 100;
    double DT = 0.002;

    // Reads every `#define NAME value` line; names not listed above are ignored.
    static Parameters from_header(const std::string &path) {
        Parameters p;
        std::ifstream in(path);
        if (!in) throw Error(CLV_ERR_IO, "cannot open " + path);
        std::string line;
        while (std::getline(in, line)) {
            std::istringstream ss(line);
            std::string def, name;
            double v;
            if (!(ss >> def >> name) || def != "#define") continue;
            if (!(ss >> v)) continue;
            p.set(name, v);
        }
        return p;
    }
    void set(const std::string &n, double v) {
        if (n == "COMPONENTS") COMPONENTS = (int)v;
        else if (n == "XSIZE") XSIZE = (int)v;
        else if (n == "YSIZE") YSIZE = (int)v;
        else if (n == "ZSIZE") ZSIZE = (int)v;
        else if (n == "TAUSIZE") TAUSIZE = (int)v;
        else if (n == "EPS") EPS = v;
        else if (n == "a_x") a_x = v;
        else if (n == "G") G = v;
        else if (n == "M") M = v;
        else if (n == "SIGMA") SIGMA = v;
        else if (n == "D") D = v;
        else if (n == "OMEGAX") OMEGAX = v;
        else if (n == "OMEGAY") OMEGAY = v;
        else if (n == "OMEGAZ") OMEGAZ = v;
        else if (n == "Q") Q = v;
        else if (n == "STEPS") STEPS = (long long)v;
        else if (n == "DT") DT = v;
        else if (n == "SNAPSHOT_TRIGGER") SNAPSHOT_TRIGGER = (long long)v;
        else if (n == "EVALUATE_TRIGGER") EVALUATE_TRIGGER = (long long)v;
    }
    long long volume() const { return (long long)XSIZE * YSIZE * ZSIZE; }
    long long length() const { return (long long)COMPONENTS * volume() * TAUSIZE; }
};

inline Parameters &current_parameters() {
    static Parameters p;
    return p;
}
inline void use_parameters(const Parameters &p) { current_parameters() = p; }

// params.txt reader with the semantics of read_params (main.cu:38-51): one
// `key=value` per line, unparsable lines skipped.
inline std::map<std::string, double> read_params(const std::string &filename) {
    std::map<std::string, double> params;
    std::ifstream infile(filename);
    std::string line;
    while (std::getline(infile, line)) {
        std::istringstream iss(line);
        std::string key;
        double value;
        if (std::getline(iss, key, '=') && iss >> value) params[key] = value;
    }
    return params;
}

// struct which_observables (Observables_without_cutoff.cu:1-31).  The engine
// evaluates n_tot, n_11..n_22 and F_x/F_y/F_z; requesting any other observable
// throws when Observables is constructed.
struct which_observables {
    bool n_tot = false, n_11 = false, n_12 = false, n_21 = false, n_22 = false;
    bool P2 = false, jrot2 = false;
    bool spectrum = false, anomalous_spectrum = false, dd = false, dispersion = false;
    bool spectrum_tot = false, density_tot = false;
    bool density_11 = false, density_12 = false, density_21 = false, density_22 = false;
    bool F_x = false, F_y = false, F_z = false;
    bool drift = false;
    double min_drift = 0, max_drift = 0;
    int drift_bins = 0;
    double max_momentum = 0;
    int bins = 0;
};

// One simulation's engine (REF4 model, FP64, reference kinetic term and step rule).
// propagate() only counts a step; the counted steps run, as graphs of several steps,
// before anything reads or changes the state (handle()), or once kMaxPending have
// accumulated.  The sequence of steps, and so every result, is the one the
// reference's loop makes; only the moment of the launches moves, and an error of
// a step surfaces at the call that runs it.
struct Engine {
    static constexpr int kMaxPending = 256;
    clv_engine *e = nullptr;
    Parameters p;
    int pending = 0;
    clv_engine *handle() {
        if (pending) {
            const int n = pending;
            pending = 0;
            check(clv_step(e, n));
        }
        return e;
    }
    void count_step() {
        if (++pending >= kMaxPending) handle();
    }
    ~Engine() {
        if (e) {
            if (pending) clv_step(e, pending);
            clv_destroy(e);
        }
    }
};

class ComplexLattice {
  public:
    explicit ComplexLattice(bool conjug)
        : conjugated_(conjug), host_(current_parameters().length(), std::complex<double>(0, 0)) {}

    // set_value (Lattice.cu:50-81): comps 0,3 = v, comps 1,2 = (2/3) v; the
    // conjugate lattice stores conj(v).
    void set_mean_field(double re, double im, double P = 0.0, double MU = 0.0) {
        (void)P; (void)MU;
        if (engine_) {
            check(clv_set_mean_field(engine_->handle(), conjugated_ ? 1 : 0, re, im));
            return;
        }
        const Parameters &p = current_parameters();
        const std::complex<double> v(re, conjugated_ ? -im : im);
        const long long n = p.volume() * p.TAUSIZE;
        for (int c = 0; c < p.COMPONENTS; ++c)
            for (long long i = 0; i < n; ++i)
                host_[c * n + i] = (c == 1 || c == 2) ? std::complex<double>(2.0 / 3.0, 0.0) * v : v;
    }

    // Device pointer of the field in the reference layout (Lattice.cu:217-220):
    // a device copy of the engine's current state, refreshed at every call (the
    // engine keeps the state in a ping-pong pair that moves every step).
    cuDoubleComplex *get_pointer() {
        if (!engine_) return nullptr;
        if (!dev_ptr_) {
            void *q = nullptr;
            if (cudaMalloc(&q, host_.size() * sizeof(cuDoubleComplex)) != cudaSuccess)
                throw Error(CLV_ERR_NOMEM, "cudaMalloc for get_pointer");
            dev_ptr_ = (cuDoubleComplex *)q;
        }
        check(clv_get_fields(engine_->handle(), 0, conjugated_ ? nullptr : (void *)dev_ptr_,
                             conjugated_ ? (void *)dev_ptr_ : nullptr, CLV_DEVICE));
        return dev_ptr_;
    }
    ~ComplexLattice() {
        if (dev_ptr_) cudaFree(dev_ptr_);
    }
    ComplexLattice(const ComplexLattice &) = delete;
    ComplexLattice &operator=(const ComplexLattice &) = delete;

    // Host copy of the field (ComplexLatticeHost::copy_from_device, Lattice.cu:460-463).
    std::vector<std::complex<double>> to_host() const {
        if (!engine_) return host_;
        std::vector<std::complex<double>> out(host_.size());
        check(clv_get_fields(engine_->handle(), 0, conjugated_ ? nullptr : out.data(),
                             conjugated_ ? out.data() : nullptr, CLV_HOST));
        return out;
    }
    void from_host(const std::vector<std::complex<double>> &v) {
        if (!engine_) { host_ = v; return; }
        check(clv_set_fields(engine_->handle(), 0, conjugated_ ? nullptr : v.data(),
                             conjugated_ ? v.data() : nullptr, CLV_HOST));
    }
    bool conjugated() const { return conjugated_; }

  private:
    friend class Propagator;
    friend class Observables;
    void bind(std::shared_ptr<Engine> eng) {
        engine_ = std::move(eng);
        check(clv_set_fields(engine_->e, 0, conjugated_ ? nullptr : host_.data(),
                             conjugated_ ? host_.data() : nullptr, CLV_HOST));
    }
    bool conjugated_;
    std::vector<std::complex<double>> host_;
    std::shared_ptr<Engine> engine_;
    cuDoubleComplex *dev_ptr_ = nullptr;
};

class Propagator {
  public:
    // Propagator(fields, fields_conjug, drift, drift_conjug, seed, seed2)
    // (Propagator_without_cutoff.cu:316-343).  The drift lattices are scratch in
    // the reference; the engine keeps no drift array, so they stay unused.
    Propagator(ComplexLattice *fields, ComplexLattice *fields_conjug, ComplexLattice *drift,
               ComplexLattice *drift_conjug, unsigned long long seed, unsigned long long seed2 = 0)
        : fields_(fields), fields_conjug_(fields_conjug) {
        (void)drift; (void)drift_conjug; (void)seed2;
        const Parameters &p = current_parameters();
        if (p.COMPONENTS != 4) throw Error(CLV_ERR_ARG, "the reference model has COMPONENTS = 4");
        clv_chain_params c;
        clv_default_chain_params(&c);
        c.nx = p.XSIZE; c.ny = p.YSIZE; c.nz = p.ZSIZE; c.nt = p.TAUSIZE;
        c.eps = p.EPS; c.a_x = p.a_x; c.G = p.G; c.Q = p.Q; c.DT = p.DT;
        c.mu = 0.0; c.P = 0.0; c.seed = seed;
        // plain FP64 as the reference; CLV_PRECISION=f32 selects the FP32-mixed engine
        const char *prec = std::getenv("CLV_PRECISION");
        const int precision = (prec && std::string(prec) == "f32") ? CLV_PREC_F32 : CLV_PREC_F64;
        int device = 0;
        cudaGetDevice(&device);
        clv_config cfg{CLV_MODEL_REF4, CLV_KIN_REF_LINEAR_PX, CLV_DT_REF_MEANMAX,
                       CLV_NOISE_PHILOX, precision, device, 1, &c};
        engine_ = std::make_shared<Engine>();
        engine_->p = p;
        check(clv_create(&cfg, &engine_->e));
        fields_->bind(engine_);
        fields_conjug_->bind(engine_);
    }

    // One Langevin step (Propagator_without_cutoff.cu:406-442); it runs with the
    // next batch of counted steps (Engine::handle).
    void propagate(double P, double MU) {
        set_couplings(P, MU);
        engine_->count_step();
    }

    // One step with the reference's noise buffer layout (ind_rand, unit normals).
    void inject_noise(double P, double MU, const double *normals) {
        set_couplings(P, MU);
        check(clv_step_with_noise(engine_->handle(), normals, CLV_HOST));
    }

    double last_dt() const {
        double dt = 0;
        check(clv_get_step_info(engine_->handle(), &dt, nullptr, nullptr, nullptr, nullptr));
        return dt;
    }
    std::shared_ptr<Engine> engine() const { return engine_; }

  private:
    void set_couplings(double P, double MU) {
        if (!have_ || P != P_ || MU != MU_) {
            check(clv_set_chemical_potential(engine_->handle(), 0, MU, P));
            P_ = P; MU_ = MU; have_ = true;
        }
    }
    ComplexLattice *fields_, *fields_conjug_;
    std::shared_ptr<Engine> engine_;
    bool have_ = false;
    double P_ = 0, MU_ = 0;
};

class Observables {
  public:
    // Observables(fields, fields_conjug, which) (Observables_without_cutoff.cu:809).
    // The lattices must already be bound to a Propagator.
    Observables(ComplexLattice *fields, ComplexLattice *fields_conjug, which_observables which)
        : which_(which), fields_(fields) {
        (void)fields_conjug;
        if (which.P2 || which.jrot2 || which.spectrum || which.anomalous_spectrum || which.dd ||
            which.dispersion || which.spectrum_tot || which.density_tot || which.density_11 ||
            which.density_12 || which.density_21 || which.density_22 || which.drift)
            throw Error(CLV_ERR_ARG, "only n_tot, n_11..n_22 and F_x/F_y/F_z are evaluated");
    }
    which_observables get_which() const { return which_; }
    void evaluate(double P, double MU) {
        (void)P; (void)MU;
        check(clv_evaluate(eng()));
    }
    int get_counter() const { return clv_get_counter(const_cast<Observables *>(this)->eng()); }
    // write_* (Observables_without_cutoff.cu:1527-1547, 1614-1634)
    void write_n_tot(double *w) { *w = scalar(0); }
    void write_n_11(double *w) { *w = scalar(1); }
    void write_n_12(double *w) { *w = scalar(2); }
    void write_n_21(double *w) { *w = scalar(3); }
    void write_n_22(double *w) { *w = scalar(4); }
    void write_F_x(double *w) { check(clv_read_ref_observables(eng(), 0, nullptr, w, nullptr, nullptr)); }
    void write_F_y(double *w) { check(clv_read_ref_observables(eng(), 0, nullptr, nullptr, w, nullptr)); }
    void write_F_z(double *w) { check(clv_read_ref_observables(eng(), 0, nullptr, nullptr, nullptr, w)); }
    long long volume() const { return current_parameters().volume(); }

  private:
    clv_engine *eng() {
        if (!engine_) {
            // the Propagator bound the lattice to its engine
            engine_ = bound_engine(fields_);
        }
        return engine_->handle();
    }
    static std::shared_ptr<Engine> bound_engine(ComplexLattice *l) {
        if (!l->engine_) throw Error(CLV_ERR_STATE, "construct the Propagator before evaluating");
        return l->engine_;
    }
    double scalar(int i) {
        double n[5];
        check(clv_read_ref_observables(eng(), 0, n, nullptr, nullptr, nullptr));
        return n[i];
    }
    which_observables which_;
    ComplexLattice *fields_;
    std::shared_ptr<Engine> engine_;
};

// folder_exists (SaveResults.cu:2-18)
inline bool folder_exists(const std::string &name) {
    struct stat st;
    return stat(name.c_str(), &st) == 0 && S_ISDIR(st.st_mode);
}

// Output writer with the reference's directory and file layout
// (SaveResults.cu:22-607): ./DATA/BoseCL_Sim_mu_<MU>_P_<P>/Run<r>/{Parameters.txt,
// rawdata/, F_x.txt, F_y.txt, F_z.txt} and the shared ./DATA/BoseCL_Sim_mu_<MU>_P_<P>/Skalars.txt.
// Obs provides get_which, get_counter, write_n_*, write_F_* and volume().
template <class Obs>
class SaveResultsT {
  public:
    SaveResultsT(Obs *observables, unsigned long long seedval)
        : obs_(observables), which_(observables->get_which()), seed_(seedval) {}

    bool make_directory(double P, double MU) {
        std::stringstream dirname;
        dirname << "./DATA/BoseCL_Sim_mu_" << MU << "_P_" << P << "/Run";
        for (int r = 1; r < 1000; r++) {
            if (!folder_exists(dirname.str() + std::to_string(r))) {
                dirname << r;
                break;
            }
        }
        std::filesystem::path dir = dirname.str();
        try {
            if (std::filesystem::create_directories(dir)) {
                std::cout << "Directory created successfully: " << dir << std::endl;
                directory_ = dirname.str();
                return true;
            }
            std::cout << "Directory already exists: " << dir << std::endl;
            return false;
        } catch (const std::filesystem::filesystem_error &e) {
            std::cerr << "Error: " << e.what() << std::endl;
            return false;
        }
    }

    bool make_directory_rawdata() {
        rawdata_ = directory_ + "/rawdata";
        if (mkdir(rawdata_.c_str(), 0755) < 0) {
            std::cout << "Directory for raw data could not be created!" << std::endl;
            return false;
        }
        std::cout << "Directory for raw data was successfully created" << std::endl;
        return true;
    }

    void save_parameters(double P, double MU) {
        const Parameters &p = current_parameters();
        std::fstream out;
        out.open(directory_ + "/Parameters.txt", std::fstream::out);
        out << "T\t" << 1. / (p.TAUSIZE * p.EPS) << std::endl
            << "mu\t" << MU << std::endl
            << "g\t" << p.G << std::endl
            << "M\t" << p.M << std::endl
            << "SIGMA\t" << p.SIGMA << std::endl
            << "D\t" << p.D << std::endl
            << "OMEGAX\t" << p.OMEGAX << std::endl
            << "OMEGAY\t" << p.OMEGAY << std::endl
            << "OMEGAZ\t" << p.OMEGAZ << std::endl
            << "P\t" << P << std::endl
            << "Q\t" << p.Q << std::endl
            << "components\t" << p.COMPONENTS << std::endl
            << "lattice\t" << p.XSIZE << "x" << p.YSIZE << "x" << p.ZSIZE << "x" << p.TAUSIZE << std::endl
            << "dt\t" << p.DT << std::endl
            << "steps\t" << p.STEPS << std::endl
            << "SNAPSHOT_TRIGGER\t" << p.SNAPSHOT_TRIGGER << std::endl
            << "EVALUATE_TRIGGER\t" << p.EVALUATE_TRIGGER << std::endl
            << "seed\t" << seed_;
        out.close();
        std::cout << "Saved parameters" << std::endl;
    }

    void save_snapshot(double P, double MU) {
        const int number = obs_->get_counter();
        {
            std::stringstream dir;
            dir << "./DATA/BoseCL_Sim_mu_" << MU << "_P_" << P;
            std::fstream out;
            out.open(dir.str() + "/Skalars.txt", std::fstream::app);
            std::string line;
            double v;
            // a disabled n_tot starts the line with two tabs; every other disabled
            // column appends two tabs (SaveResults.cu:208-256)
            if (which_.n_tot) { obs_->write_n_tot(&v); line = line + std::to_string(v) + "\t"; }
            else line = "\t\t";
            if (which_.n_11) { obs_->write_n_11(&v); line = line + std::to_string(v) + "\t"; }
            else line = line + "\t\t";
            if (which_.n_12) { obs_->write_n_12(&v); line = line + std::to_string(v) + "\t"; }
            else line = line + "\t\t";
            if (which_.n_21) { obs_->write_n_21(&v); line = line + std::to_string(v) + "\t"; }
            else line = line + "\t\t";
            if (which_.n_22) { obs_->write_n_22(&v); line = line + std::to_string(v) + "\t"; }
            else line = line + "\t\t";
            line = line + "\t\t";  // P2 is not evaluated
            out << line << std::endl;
            if (out.good()) std::cout << "Saved scalars at time " << number << std::endl;
            else std::cout << "Saving scalars at time " << number << " failed" << std::endl;
            out.close();
        }
        profile("F_x", which_.F_x, number, [&](double *w) { obs_->write_F_x(w); });
        profile("F_y", which_.F_y, number, [&](double *w) { obs_->write_F_y(w); });
        profile("F_z", which_.F_z, number, [&](double *w) { obs_->write_F_z(w); });
    }

    const std::string &directory() const { return directory_; }

  private:
    template <class F>
    void profile(const char *name, bool on, int number, F &&write) {
        if (!on) return;
        std::fstream out;
        out.open(directory_ + "/" + name + ".txt", std::fstream::app);
        std::vector<double> v(obs_->volume());
        write(v.data());
        for (double x : v) out << x << "\t";
        out << std::endl;
        if (out.good()) std::cout << "Saved real-space " << name << " at time " << number << std::endl;
        else std::cout << "Saving real-space " << name << " at time " << number << " failed" << std::endl;
        out.close();
    }
    Obs *obs_;
    which_observables which_;
    unsigned long long seed_;
    std::string directory_, rawdata_;
};

using SaveResults = SaveResultsT<Observables>;

}  // namespace clv_compat
