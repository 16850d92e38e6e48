// pimdb_gb300: command-line driver in the shape of the reference's main
// (src/pimdb.cpp:31-68): reads config.ini, builds the simulation with every
// bead on one GPU, runs steps+1 MD steps (src/simulation.cpp:236) and writes
// the observables to output/simulation.out in the reference's format.
//
//   pimdb_gb300 [-in config.ini] [--dim N] [--check] [--plugin-steps]
//               [--steps K] [--positions out.xyz] [--factorial] [--bosonic_alg]
//               [--ranmars]
//
//   --check          parse and validate the configuration only (no GPU)
//   --plugin-steps   drive the step through the plugin objects one call at a
//                    time instead of the fused device schedule
//   --steps K        override [simulation] steps
//   --positions F    write the final positions of every bead (xyz, angstrom)
//   --initial F      with --check: write the initial positions and momenta
//                    (raw doubles, [bead][particle][axis], atomic units)
//   --factorial      bosonic exchange by the sum over all N! permutations
//                    (the reference's FACTORIAL_BOSONIC_ALGORITHM build)
//                    instead of the Feldman-Hirshberg recursion
//   --bosonic_alg    print which bosonic algorithm is selected and exit
//                    (src/pimdb.cpp:12-17)
//   --ranmars        Langevin noise from the reference's RanMars streams
//                    (seed + bead, drawn per particle and axis) instead of the
//                    counter-based Philox stream: with the reference's initial
//                    state this follows the reference's own trajectory
//
// Configuration errors are printed as "[X] Invalid argument error: ..." and,
// as in the reference, the process still exits 0; CUDA errors exit 1.
#include <chrono>
#include <cstdio>
#include <cstring>
#include <filesystem>
#include <iostream>
#include <fstream>
#include <string>
#include <vector>

#include "pimdb_host.hpp"

int main(int argc, char** argv) {
    std::string config = "config.ini", positions, initial;
    int ndim = 3;
    bool check_only = false, plugin = false, factorial = false, show_alg = false, ranmars = false;
    long steps_override = -1;
    for (int i = 1; i < argc; ++i) {
        if (!std::strcmp(argv[i], "-in") && i + 1 < argc) config = argv[++i];
        else if (!std::strcmp(argv[i], "--dim") && i + 1 < argc) ndim = std::atoi(argv[++i]);
        else if (!std::strcmp(argv[i], "--check")) check_only = true;
        else if (!std::strcmp(argv[i], "--plugin-steps")) plugin = true;
        else if (!std::strcmp(argv[i], "--steps") && i + 1 < argc) steps_override = std::atol(argv[++i]);
        else if (!std::strcmp(argv[i], "--positions") && i + 1 < argc) positions = argv[++i];
        else if (!std::strcmp(argv[i], "--initial") && i + 1 < argc) initial = argv[++i];
        else if (!std::strcmp(argv[i], "--factorial")) factorial = true;
        else if (!std::strcmp(argv[i], "--bosonic_alg")) show_alg = true;
        else if (!std::strcmp(argv[i], "--ranmars")) ranmars = true;
    }
    if (show_alg) {
        std::cout << (factorial ? "Running with naive bosonic algorithm.\n" : "Running with quadratic bosonic algorithm.\n");
        return 0;
    }
    try {
        std::cout << "[*] Initializing the simulation parameters\n";
        pimdb_gb300::Params params(config, ndim);
        if (steps_override >= 0) params.run.steps = steps_override;
        if (factorial) params.config.exchange = PIMDB_EXCHANGE_FACTORIAL;
        if (ranmars) params.config.rng = PIMDB_RNG_RANMAR;
        if (check_only) {
            const auto& c = params.config;
            std::printf("[*] natoms=%d nbeads=%d ndim=%d bosonic=%d propagator=%d thermostat=%d steps=%ld exchange=%s\n",
                        c.natoms, c.nbeads, c.ndim, c.bosonic, c.propagator, c.thermostat, params.run.steps,
                        c.exchange == PIMDB_EXCHANGE_FACTORIAL ? "factorial" : "feldman_hirshberg");
            if (!initial.empty()) {
                std::vector<double> x, p;
                pimdb_host::initial_state(params.config, params.run, x, p, true);
                std::ofstream out(initial, std::ios::binary);
                out.write(reinterpret_cast<const char*>(x.data()), (std::streamsize)(x.size() * sizeof(double)));
                out.write(reinterpret_cast<const char*>(p.data()), (std::streamsize)(p.size() * sizeof(double)));
            }
            return 0;
        }
        pimdb_gb300::Simulation sim(params);
        std::filesystem::create_directories("output");
        pimdb_host::ObservablesLogger logger(params.config, params.run, "output/simulation.out");
        pimdb_host::StateWriter states(params.config, params.run, "output");
        std::cout << "[*] Running the simulation\n";
        const auto t0 = std::chrono::steady_clock::now();
        sim.run(plugin, &logger, &states);
        const double wall = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        const double bs = (double)params.config.natoms * params.config.nbeads * (params.run.steps + 1) / wall;
        std::printf("[*] Simulation finished running successfully (Runtime = %.3g sec, %.4g bead-steps/s)\n", wall, bs);
        if (!positions.empty()) {
            std::vector<double> x, p, f;
            sim.get_state(x, p, f);
            std::ofstream out(positions);
            const auto& c = params.config;
            for (int b = 0; b < c.nbeads; ++b) {
                out << c.natoms << "\nbead " << b << "\n";
                for (int i = 0; i < c.natoms; ++i) {
                    out << "1";
                    for (int a = 0; a < c.ndim; ++a) {
                        char buf[64];
                        std::snprintf(buf, sizeof buf, " %.17g", x[((size_t)b * c.natoms + i) * c.ndim + a] / 1.8897261);
                        out << buf;
                    }
                    out << "\n";
                }
            }
        }
    } catch (const std::invalid_argument& ex) {
        std::cout << "[X] Invalid argument error: " << ex.what() << "\n";
    } catch (const std::overflow_error& ex) {
        std::cout << "[X] Overflow error: " << ex.what() << "\n";
    } catch (const std::exception& ex) {
        std::cout << "[X] Error: " << ex.what() << "\n";
        return 1;
    }
    return 0;
}
