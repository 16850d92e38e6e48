// C++20 host layer over the C ABI: the reference's plugin classes
// (Potential, Propagator, Thermostat, BosonicExchangeBase, Simulation, Params)
// with the reference's names and call structure, each holding every bead of
// the ring polymer on the GPU instead of one MPI rank's bead.
//
//   Params              include/params.h:19-53, src/params.cpp:8-260
//   Potential family    include/potentials/*.h (constructor signatures kept)
//   BosonicExchange     include/bosonic_exchange/bosonic_exchange_base.h:16-54
//   Propagator          include/propagators/propagator.h:7-18
//   Thermostat          include/thermostats/thermostat.h:9-19
//   Simulation          include/simulation.h:20-131, src/simulation.cpp
//
// Errors surface as the reference's exception types: std::invalid_argument
// (configuration), std::overflow_error (non-finite exchange potential),
// std::runtime_error (CUDA).
#pragma once

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <filesystem>
#include <format>
#include <fstream>
#include <functional>
#include <limits>
#include <memory>
#include <random>
#include <stdexcept>
#include <string>
#include <vector>

#include "pimdb_gb300.h"
#include "units.hpp"

namespace pimdb_host {

// Run-control keys of config.ini that the hot path does not use.
struct RunParams {
    long steps = 100000;
    long sfreq = 1000;
    double threshold = 0.1;
    std::string init_pos_type = "random", init_pos_spec;
    std::string init_vel_type = "random", init_vel_spec;
    std::string output_positions = "off", output_velocities = "off", output_forces = "off";
    // [observables]: output unit of each observable group, or "off"
    std::string obs_energy = "kelvin", obs_classical = "off", obs_bosonic = "off", obs_gsf = "off";
};

// Reads config.ini (schema and messages of src/params.cpp:8-260); throws
// std::invalid_argument.
void read_params(const std::string& path, int ndim, pimdb_config& cfg, RunParams& run);

// "grid" initial positions (src/simulation.cpp:133-193) of one bead.
inline void grid_positions(const pimdb_config& cfg, double* pos) {
    const int N = cfg.natoms, D = cfg.ndim;
    const double L = cfg.size;
    const double volume = std::pow(L, D);
    const double side = std::pow((1.0 * N / volume), -1.0 / (1.0 * D));
    int total = 1;
    int num[3];
    double sz[3];
    for (int i = 0; i < D; i++) {
        num[i] = (int)std::ceil((L / side) - 1.0E-7);
        num[i] = std::max(num[i], 1);
        sz[i] = L / (1.0 * num[i]);
        total *= num[i];
    }
    if (total < N) throw std::runtime_error("Number of grid boxes is less than the number of particles");
    for (int n = 0; n < N; n++) {
        for (int i = 0; i < D; i++) {
            int scale = 1;
            for (int j = i + 1; j < D; j++) scale *= num[j];
            const int gi = (n / scale) % num[i];
            double v = (gi + 0.5) * sz[i] - 0.5 * L;
            if (cfg.pbc) v -= L * std::floor(v / L + 0.5);
            pos[(size_t)n * D + i] = v;
        }
    }
}

// loadTrajectories / loadMomenta (src/common.cpp:49-136): an xyz file
// (count, comment, "symbol x y z" in angstrom) or a LAMMPS-style velocity
// file (count, comment, "id type vx vy vz" in angstrom/ps, times the mass).
inline void load_xyz(const std::string& name, int N, int D, double* out) {
    std::ifstream in(name);
    if (!in.is_open()) throw std::runtime_error(std::format("Cannot open the xyz file named {}.", name));
    int n = 0;
    in >> n;
    if (n != N)
        throw std::runtime_error(
            std::format("The number of atoms in the xyz file ({}) does not match the requested number of atoms.", name));
    in.ignore(std::numeric_limits<std::streamsize>::max(), '\n');
    std::string line;
    std::getline(in, line, '\n');
    for (int i = 0; i < N; ++i) {
        std::string symbol;
        in >> symbol;
        for (int a = 0; a < D; ++a) {
            in >> out[(size_t)i * D + a];
            out[(size_t)i * D + a] = Units::convertToInternal("length", "angstrom", out[(size_t)i * D + a]);
        }
    }
}

inline void load_momenta(const std::string& name, double mass, int N, int D, double* out) {
    std::ifstream in(name);
    if (!in.is_open()) throw std::runtime_error(std::format("Cannot open the velocity file named {}.", name));
    int n = 0;
    in >> n;
    if (n != N)
        throw std::runtime_error(std::format(
            "The number of atoms in the velocity file ({}) does not match the requested number of atoms.", name));
    in.ignore(std::numeric_limits<std::streamsize>::max(), '\n');
    std::string line;
    std::getline(in, line, '\n');
    for (int i = 0; i < N; ++i) {
        std::string id, type;
        in >> id >> type;
        for (int a = 0; a < D; ++a) {
            in >> out[(size_t)i * D + a];
            out[(size_t)i * D + a] = mass * Units::convertToInternal("velocity", "angstrom/ps", out[(size_t)i * D + a]);
        }
    }
}

// A file-name specification with "{}" names one file per bead: the bead
// index starts at 1 when the file for index 0 does not exist
// (src/params.cpp:62-91, simulation.cpp:709-721).
inline std::string formatted_bead_file(const std::string& spec, int bead) {
    const int dummy = 0;
    const std::string first = std::vformat(spec, std::make_format_args(dummy));
    if (first == spec) return spec;  // not a format: the same file for every bead
    const int arg = bead + (std::filesystem::exists(first) ? 0 : 1);
    return std::vformat(spec, std::make_format_args(arg));
}

// Initial conditions as the reference draws them: bead b uses
// std::mt19937(seed + b) (src/simulation.cpp:58); random positions uniform in
// [-L/2, L/2] (:118-126), the grid (:133-193) or xyz files (:709-721);
// Maxwell-Boltzmann momenta from a fresh std::normal_distribution per draw
// (:200-217) or velocity files (:737-748).  With zero_com, random momenta
// lose their centre-of-mass momentum the way Simulation::zeroMomentum does
// it (:581-603, :750-751); loaded momenta are kept as they are.
inline void initial_state(const pimdb_config& cfg, const RunParams& run, std::vector<double>& x0,
                          std::vector<double>& p0, bool zero_com = false) {
    const int P = cfg.nbeads, N = cfg.natoms, D = cfg.ndim;
    x0.assign((size_t)P * N * D, 0.0);
    p0.assign((size_t)P * N * D, 0.0);
    const double beta = 1.0 / (1.0 * cfg.temperature);
    const double thermo_beta = beta / P;
    for (int b = 0; b < P; ++b) {
        std::mt19937 gen((unsigned)(cfg.seed + b));
        double* x = &x0[(size_t)b * N * D];
        double* p = &p0[(size_t)b * N * D];
        if (run.init_pos_type == "grid") {
            grid_positions(cfg, x);
        } else if (run.init_pos_type == "random") {
            std::uniform_real_distribution<double> u(-0.5 * cfg.size, 0.5 * cfg.size);
            for (int i = 0; i < N * D; ++i) x[i] = u(gen);
        } else {
            load_xyz(formatted_bead_file(run.init_pos_spec, b), N, D, x);
        }
        if (run.init_vel_type == "random") {
            for (int i = 0; i < N * D; ++i) {
                std::normal_distribution<double> nd(0.0, 1 / std::sqrt(thermo_beta * cfg.mass));
                p[i] = cfg.mass * nd(gen);
            }
        } else {
            const std::string name = run.init_vel_spec.empty() ? std::format("init/vel_{:02}.dat", b + 1)
                                                                : formatted_bead_file(run.init_vel_spec, b);
            load_momenta(name, cfg.mass, N, D, p);
        }
    }
    if (zero_com && run.init_vel_type == "random") {
        double cm[3] = {0.0, 0.0, 0.0};
        for (int b = 0; b < P; ++b) {
            double per[3] = {0.0, 0.0, 0.0};
            for (int i = 0; i < N; ++i)
                for (int a = 0; a < D; ++a) per[a] += p0[((size_t)b * N + i) * D + a];
            for (int a = 0; a < D; ++a) cm[a] += per[a] / (N * P);
        }
        for (size_t i = 0; i < (size_t)P * N; ++i)
            for (int a = 0; a < D; ++a) p0[i * D + a] -= cm[a];
    }
}

// The per-bead state dumps (src/states/{position,velocity,force}.cpp):
// output/position_<b>.xyz, velocity_<b>.dat, force_<b>.dat, appended at the
// start of every sfreq-th step, in the configured units ("on", "true" and
// "none" mean atomic units).
class StateWriter {
public:
    StateWriter(const pimdb_config& c, const RunParams& run, const std::string& dir) : c_(c) {
        auto unit = [](const std::string& u) { return (u == "on" || u == "true" || u == "none") ? std::string("atomic_unit") : u; };
        auto on = [](const std::string& u) { return u != "off" && u != "false"; };
        if (on(run.output_positions)) open(files_[0], dir, "position_{}.xyz", unit(run.output_positions), units_[0]);
        if (on(run.output_velocities)) open(files_[1], dir, "velocity_{}.dat", unit(run.output_velocities), units_[1]);
        if (on(run.output_forces)) open(files_[2], dir, "force_{}.dat", unit(run.output_forces), units_[2]);
    }
    bool enabled() const { return !files_[0].empty() || !files_[1].empty() || !files_[2].empty(); }
    bool wants(int k) const { return !files_[k].empty(); }
    // x, p, f: [bead][particle][axis]; any may be empty when not written
    void output(long step, const std::vector<double>& x, const std::vector<double>& p, const std::vector<double>& f) {
        const int N = c_.natoms, D = c_.ndim;
        static const char* family[3] = {"length", "velocity", "force"};
        const std::vector<double>* src[3] = {&x, &p, &f};
        for (int k = 0; k < 3; ++k) {
            if (files_[k].empty()) continue;
            for (int b = 0; b < c_.nbeads; ++b) {
                std::ofstream& o = *files_[k][b];
                o << std::format("{}\n", N) << std::format("Step {}\n", step);
                for (int i = 0; i < N; ++i) {
                    if (k == 0) o << "1";
                    else o << (i + 1) << " 1";
                    for (int a = 0; a < D; ++a) {
                        double v = (*src[k])[((size_t)b * N + i) * D + a];
                        if (k == 1) v /= c_.mass;
                        o << std::format(" {:^20.12e}", Units::convertToUser(family[k], units_[k], v));
                    }
                    if (D == 1) o << " 0.0 0.0";
                    else if (D == 2) o << " 0.0";
                    o << "\n";
                }
            }
        }
    }

private:
    void open(std::vector<std::unique_ptr<std::ofstream>>& v, const std::string& dir, const char* pattern,
              const std::string& unit, std::string& unit_out) {
        Units::convertToUser(pattern[0] == 'p' ? "length" : (pattern[0] == 'v' ? "velocity" : "force"), unit, 1.0);
        unit_out = unit;
        for (int b = 0; b < c_.nbeads; ++b) {
            const int bead = b;
            v.push_back(std::make_unique<std::ofstream>(dir + "/" + std::vformat(pattern, std::make_format_args(bead)),
                                                        std::ios::out | std::ios::app));
        }
    }
    pimdb_config c_;
    std::vector<std::unique_ptr<std::ofstream>> files_[3];
    std::string units_[3];
};

inline void check(int st, pimdb_handle* h = nullptr) {
    if (st == PIMDB_OK) return;
    char buf[512];
    pimdb_last_error(h, buf, sizeof buf);
    const std::string msg = std::string(pimdb_status_string(st)) + ": " + buf;
    if (st == PIMDB_ERR_CONFIG || st == PIMDB_ERR_PARSE || st == PIMDB_ERR_ARG) throw std::invalid_argument(msg);
    if (st == PIMDB_ERR_NONFINITE_VB) throw std::overflow_error(msg);
    throw std::runtime_error(msg);
}

// ObservablesLogger (src/observables/observable.cpp:61-116): the header and
// the rows of simulation.out, with the columns the reference's observables
// declare (energy.cpp:11-19, classical.cpp:11-19, bosonic.cpp:9-12,
// gsf_action.cpp:10-13) in their output units; the file is appended to.
class ObservablesLogger {
public:
    ObservablesLogger(const pimdb_config& c, const RunParams& run, const std::string& path) {
        using O = pimdb_observables;
        auto energy = [](const std::string& u) {
            return [u](double v) { return u == "none" ? v : Units::convertToUser("energy", u, v); };
        };
        auto plain = [](double v) { return v; };
        auto add = [&](const char* key, double O::*m, std::function<double(double)> conv) {
            cols_.push_back({key, m, conv});
        };
        if (run.obs_energy != "off") {
            const auto e = energy(run.obs_energy);
            const bool ext_free = c.ext_kind == PIMDB_POT_FREE, int_free = c.int_kind == PIMDB_POT_FREE;
            add("kinetic", &O::kinetic, e);
            if (!(ext_free && int_free)) {
                add("potential", &O::potential, e);
                if (!ext_free && !int_free) {
                    add("ext_pot", &O::ext_pot, e);
                    add("int_pot", &O::int_pot, e);
                }
                add("virial", &O::virial, e);
            }
        }
        if (run.obs_classical != "off") {
            const auto e = energy(run.obs_classical);
            add("temperature", &O::temperature, plain);
            add("cl_kinetic", &O::cl_kinetic, e);
            add("cl_spring", &O::cl_spring, e);
            if (c.thermostat >= PIMDB_THERMO_NOSE_HOOVER) add("nh_energy", &O::nh_energy, e);
        }
        if (c.bosonic && run.obs_bosonic != "off") {
            add("prob_dist", &O::prob_dist, plain);
            add("prob_all", &O::prob_all, plain);
        }
        if (run.obs_gsf != "off") {
            add("w_gsf", &O::w_gsf, plain);
            add("pot_gsf", &O::pot_gsf, energy(run.obs_gsf));
        }
        if (cols_.empty()) return;
        file_.open(path, std::ios::out | std::ios::app);
        if (!file_.is_open()) throw std::runtime_error("Failed to open " + path + ".");
        file_ << std::format("{:^16s}", "step");
        for (const auto& col : cols_) file_ << std::format(" {:^16s}", col.key);
        file_ << '\n';
    }
    bool enabled() const { return !cols_.empty(); }
    void log(long step, const pimdb_observables& o) {
        file_ << std::format("{:^16.8e}", static_cast<double>(step));
        for (const auto& col : cols_) file_ << std::format(" {:^16.8e}", col.conv(o.*(col.member)));
        file_ << '\n';
    }

private:
    struct Column {
        const char* key;
        double pimdb_observables::*member;
        std::function<double(double)> conv;
    };
    std::vector<Column> cols_;
    std::ofstream file_;
};

}  // namespace pimdb_host

namespace pimdb_gb300 {

using pimdb_host::check;

class Params {
public:
    explicit Params(const std::string& filename, int ndim = 3) { pimdb_host::read_params(filename, ndim, config, run); }
    pimdb_config config{};
    pimdb_host::RunParams run;
};

// ----------------------------------------------------------------- potentials
// The GPU evaluates the potentials; these objects carry their parameters
// (constructor signatures as in the reference).
class Potential {
public:
    virtual ~Potential() = default;
    virtual int kind() const { return PIMDB_POT_FREE; }
    virtual std::array<double, 3> params() const { return {0.0, 0.0, 0.0}; }
};
class HarmonicPotential : public Potential {  // harmonic.cpp:3-5
public:
    HarmonicPotential(double mass, double omega) : mass(mass), omega(omega) {}
    int kind() const override { return PIMDB_POT_HARMONIC; }
    std::array<double, 3> params() const override { return {omega, 0.0, 0.0}; }
    double mass, omega;
};
class DoubleWellPotential : public Potential {  // double_well.cpp:3-4
public:
    DoubleWellPotential(double mass, double strength, double loc) : mass(mass), strength(strength), loc(loc) {}
    int kind() const override { return PIMDB_POT_DOUBLE_WELL; }
    std::array<double, 3> params() const override { return {strength, loc, 0.0}; }
    double mass, strength, loc;
};
class CosinePotential : public Potential {  // cosine.cpp:4-7
public:
    CosinePotential(double amplitude, double wavelength, double phase)
        : amplitude(amplitude), wavelength(wavelength), phase(phase) {}
    int kind() const override { return PIMDB_POT_COSINE; }
    std::array<double, 3> params() const override { return {amplitude, phase, 0.0}; }
    double amplitude, wavelength, phase;
};
class DipolePotential : public Potential {  // dipole.cpp:3
public:
    explicit DipolePotential(double strength) : strength(strength) {}
    int kind() const override { return PIMDB_POT_DIPOLE; }
    std::array<double, 3> params() const override { return {strength, 0.0, 0.0}; }
    double strength;
};
class AzizPotential : public Potential {  // aziz.cpp:3-16
public:
    int kind() const override { return PIMDB_POT_AZIZ; }
};

// The device state shared by the plugins of one simulation.
class Engine {
public:
    explicit Engine(const pimdb_config& cfg, void* stream = nullptr) : cfg_(cfg) { check(pimdb_create(&cfg_, stream, &h_)); }
    ~Engine() {
        if (h_) pimdb_destroy(h_);
    }
    Engine(const Engine&) = delete;
    Engine& operator=(const Engine&) = delete;
    pimdb_handle* handle() const { return h_; }
    const pimdb_config& config() const { return cfg_; }

private:
    pimdb_config cfg_;
    pimdb_handle* h_ = nullptr;
};

// ------------------------------------------------------------ bosonic exchange
class BosonicExchangeBase {
public:
    explicit BosonicExchangeBase(Engine& e) : e_(e) {}
    virtual ~BosonicExchangeBase() = default;
    BosonicExchangeBase(const BosonicExchangeBase&) = delete;
    BosonicExchangeBase& operator=(const BosonicExchangeBase&) = delete;

    // exterior spring force of bead 1 (first = true) or bead P, [particle][axis]
    void exteriorSpringForce(std::vector<double>& f, bool first) const { f = first ? f_first_ : f_last_; }
    virtual void prepare() = 0;
    virtual double effectivePotential() = 0;
    virtual double primEstimator() = 0;
    virtual double getDistinctProbability() = 0;
    virtual double getLongestProbability() = 0;

protected:
    Engine& e_;
    std::vector<double> f_first_, f_last_;
};

// Both algorithms run on the GPU behind pimdb_exchange; the engine's
// configuration (pimdb_config::exchange) selects which.
class DeviceBosonicExchange : public BosonicExchangeBase {
public:
    explicit DeviceBosonicExchange(Engine& e) : BosonicExchangeBase(e) {}
    void prepare() override {
        const auto& c = e_.config();
        f_first_.assign((size_t)c.natoms * c.ndim, 0.0);
        f_last_.assign((size_t)c.natoms * c.ndim, 0.0);
        check(pimdb_exchange(e_.handle(), scal_.data(), f_first_.data(), f_last_.data()), e_.handle());
    }
    double effectivePotential() override { return scal_[0]; }
    double primEstimator() override { return scal_[1]; }
    double getDistinctProbability() override { return scal_[2]; }
    double getLongestProbability() override { return scal_[3]; }

private:
    std::array<double, 4> scal_{};
};
// Feldman-Hirshberg (quadratic_bosonic_exchange.cpp)
class BosonicExchange final : public DeviceBosonicExchange {
public:
    using DeviceBosonicExchange::DeviceBosonicExchange;
};
// Sum over all N! permutations (factorial_bosonic_exchange.cpp); its
// getDistinctProbability and getLongestProbability are 0 as there.
class FactorialBosonicExchange final : public DeviceBosonicExchange {
public:
    using DeviceBosonicExchange::DeviceBosonicExchange;
};

// ------------------------------------------------------ propagator, thermostat
class Propagator {
public:
    explicit Propagator(Engine& e) : e_(e) {}
    virtual ~Propagator() = default;
    virtual void step() { check(pimdb_propagate(e_.handle()), e_.handle()); }

protected:
    Engine& e_;
};
class VelocityVerletPropagator final : public Propagator {
public:
    using Propagator::Propagator;
};
class NormalModesPropagator final : public Propagator {
public:
    using Propagator::Propagator;
};

class Thermostat {
public:
    Thermostat(Engine& e, bool normal_modes) : e_(e), normal_modes_(normal_modes) {}
    virtual ~Thermostat() = default;
    // substep 0 / 1: first / second O-step of the current MD step
    void step(int substep) { check(pimdb_thermostat_step(e_.handle(), substep), e_.handle()); }
    virtual double getAdditionToH() { return 0.0; }

protected:
    Engine& e_;
    bool normal_modes_;
};
class LangevinThermostat final : public Thermostat {
public:
    using Thermostat::Thermostat;
};
// Nose-Hoover chains (nose_hoover.cpp): the chain state lives on the GPU;
// getAdditionToH is the nh_energy the observables report.
class NoseHooverThermostat : public Thermostat {
public:
    using Thermostat::Thermostat;
    double getAdditionToH() override {
        pimdb_observables o{};
        check(pimdb_compute_observables(e_.handle(), &o), e_.handle());
        return o.nh_energy;
    }
};
class NoseHooverNpThermostat final : public NoseHooverThermostat {
public:
    using NoseHooverThermostat::NoseHooverThermostat;
};
class NoseHooverNpDimThermostat final : public NoseHooverThermostat {
public:
    using NoseHooverThermostat::NoseHooverThermostat;
};

// ----------------------------------------------------------------- simulation
// Simulation::Simulation / run (src/simulation.cpp:16-101, :236-260) for all
// beads at once; the initial state is pimdb_host::initial_state's.
class Simulation {
public:
    explicit Simulation(Params& params, void* stream = nullptr) : cfg(params.config), run_params(params.run) {
        engine = std::make_unique<Engine>(cfg, stream);
        // Simulation::initializeExchangeAlgorithm (src/simulation.cpp:687-698)
        if (cfg.bosonic && cfg.nbeads > 1) {
            if (cfg.exchange == PIMDB_EXCHANGE_FACTORIAL)
                bosonic_exchange = std::make_unique<FactorialBosonicExchange>(*engine);
            else
                bosonic_exchange = std::make_unique<BosonicExchange>(*engine);
        }
        if (cfg.propagator == PIMDB_PROP_NORMAL_MODES) propagator = std::make_unique<NormalModesPropagator>(*engine);
        else propagator = std::make_unique<VelocityVerletPropagator>(*engine);
        // Simulation::initializeThermostat (src/simulation.cpp:667-684)
        if (cfg.thermostat == PIMDB_THERMO_LANGEVIN)
            thermostat = std::make_unique<LangevinThermostat>(*engine, cfg.nmthermostat);
        else if (cfg.thermostat == PIMDB_THERMO_NOSE_HOOVER)
            thermostat = std::make_unique<NoseHooverThermostat>(*engine, cfg.nmthermostat);
        else if (cfg.thermostat == PIMDB_THERMO_NOSE_HOOVER_NP)
            thermostat = std::make_unique<NoseHooverNpThermostat>(*engine, cfg.nmthermostat);
        else if (cfg.thermostat == PIMDB_THERMO_NOSE_HOOVER_NP_DIM)
            thermostat = std::make_unique<NoseHooverNpDimThermostat>(*engine, cfg.nmthermostat);
        else thermostat = std::make_unique<Thermostat>(*engine, cfg.nmthermostat);
        initialize_state();
    }

    // One MD step through the plugins (src/simulation.cpp:246-259).
    void plugin_step() {
        thermostat->step(0);
        if (cfg.fixcom) zeroMomentum();
        propagator->step();
        thermostat->step(1);
        if (cfg.fixcom) zeroMomentum();
        check(pimdb_set_step(engine->handle(), ++md_step), engine->handle());
    }
    // The same step with the fused device schedule.
    void fast_step(int n = 1) {
        check(pimdb_step(engine->handle(), n), engine->handle());
        md_step += n;
    }
    void zeroMomentum() { check(pimdb_zero_momentum(engine->handle()), engine->handle()); }
    void updateForces() { check(pimdb_compute_forces(engine->handle()), engine->handle()); }
    void get_state(std::vector<double>& x, std::vector<double>& p, std::vector<double>& f) const {
        const size_t n = (size_t)cfg.nbeads * cfg.natoms * cfg.ndim;
        x.resize(n);
        p.resize(n);
        f.resize(n);
        check(pimdb_get_state(engine->handle(), x.data(), p.data(), f.data()), engine->handle());
    }
    long getStep() const { return md_step; }
    void observables(pimdb_observables& o) { check(pimdb_compute_observables(engine->handle(), &o), engine->handle()); }

    // Simulation::run (src/simulation.cpp:236-280): steps+1 MD steps.  At
    // the start of every sfreq-th step the states are dumped; from the
    // thermalization threshold on, the observables of every sfreq-th step
    // (at its end) go to the logger.  The fused schedule runs the steps in
    // between as one call.
    void run(bool plugin, pimdb_host::ObservablesLogger* logger, pimdb_host::StateWriter* states = nullptr) {
        const long steps = run_params.steps, sfreq = std::max(1L, run_params.sfreq);
        const double threshold = run_params.threshold * steps;
        auto advance = [&](long n) {
            while (n > 0) {
                const int k = (int)std::min<long>(n, 1L << 30);
                if (plugin) {
                    for (int q = 0; q < k; ++q) plugin_step();
                } else {
                    fast_step(k);
                }
                n -= k;
            }
        };
        long s = 0;
        while (s <= steps) {
            if (s % sfreq == 0) {
                if (states && states->enabled()) {
                    std::vector<double> x, p, f;
                    get_state(x, p, f);
                    states->output(s, x, p, f);
                }
                advance(1);
                if (logger && logger->enabled() && s >= threshold) {
                    pimdb_observables o{};
                    observables(o);
                    logger->log(s, o);
                }
                s += 1;
            } else {
                const long next = (s / sfreq + 1) * sfreq;
                const long n = std::min(next, steps + 1) - s;
                advance(n);
                s += n;
            }
        }
    }

    pimdb_config cfg;
    pimdb_host::RunParams run_params;
    std::unique_ptr<Engine> engine;
    std::unique_ptr<BosonicExchangeBase> bosonic_exchange;
    std::unique_ptr<Propagator> propagator;
    std::unique_ptr<Thermostat> thermostat;
    std::vector<double> x0, p0;  // initial state [bead][particle][axis]

private:
    void initialize_state() {
        pimdb_host::initial_state(cfg, run_params, x0, p0);
        check(pimdb_set_state(engine->handle(), x0.data(), p0.data()), engine->handle());
        if (run_params.init_vel_type == "random") zeroMomentum();
    }

    long md_step = 0;
};

}  // namespace pimdb_gb300
