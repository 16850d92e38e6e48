// Probe driver for the compiled, unmodified PIMD-B++ reference (test
// infrastructure only; it links the reference's own object files).
//
// For a given config.ini and ring-polymer configuration (all P beads), it
// builds one reference `Simulation` per bead (rank = bead, single process),
// overwrites the bead's `coord`, `prev_coord` and `next_coord`
// (include/simulation.h:59-60) and calls the reference's own force and
// exchange routines:
//   Simulation::updateForces          src/simulation.cpp:353-374
//   Simulation::updateSpringForces    src/simulation.cpp:394-420
//   Simulation::updatePhysicalForces  src/simulation.cpp:428-455
//   BosonicExchange::effectivePotential / primEstimator /
//     getDistinctProbability / getLongestProbability
//                                     src/bosonic_exchange/quadratic_bosonic_exchange.cpp:130-279
//   Simulation::classicalSpringEnergy src/simulation.cpp:464-486
//
// Usage: ref_probe <config.ini> <coords.bin> <out.bin>
//   coords.bin: P*N*NDIM doubles, layout [bead][particle][axis], atomic units.
//   out.bin:    per bead: total forces, spring forces, physical forces
//               (each N*NDIM doubles) then 8 scalars:
//               [V_B, primEstimator, P_distinct, P_longest, classicalSpringEnergy,
//                ext V, pair V (within cutoff), is_bosonic_bead]
#include <malloc.h>

#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <vector>

#include "mpi.h"
#include "params.h"
#include "simulation.h"

static void pregrow_heap() {
    // The reference's BosonicExchange constructor evaluates the recursion
    // before `coord` is sized (src/simulation.cpp:67 vs :70).  Make the memory
    // it reads past the end of the 1-row vector zero-filled heap instead of
    // unmapped or arbitrary memory.
    mallopt(M_MMAP_THRESHOLD, 1 << 30);
    mallopt(M_TRIM_THRESHOLD, 1 << 30);
    const size_t bytes = 256u << 20;
    void* p = malloc(bytes);
    if (p) {
        std::memset(p, 0, bytes);
        free(p);
    }
}

int main(int argc, char** argv) {
    if (argc != 4) {
        std::fprintf(stderr, "usage: %s config.ini coords.bin out.bin\n", argv[0]);
        return 2;
    }
    pregrow_heap();
    MPI_Init(&argc, &argv);
    int rc = 0;
    try {
        Params params(argv[1], 0);
        int P = std::get<int>(params.sim["nbeads"]);
        int N = std::get<int>(params.sys["natoms"]);
        const size_t per_bead = (size_t)N * NDIM;

        std::vector<double> coords((size_t)P * per_bead);
        {
            std::ifstream in(argv[2], std::ios::binary);
            in.read(reinterpret_cast<char*>(coords.data()), (std::streamsize)(coords.size() * sizeof(double)));
            if (!in) throw std::runtime_error("cannot read coordinates");
        }
        std::ofstream out(argv[3], std::ios::binary);

        for (int b = 0; b < P; ++b) {
            Simulation sim(b, 1, params, 1u);
            const int bp = (b - 1 + P) % P;
            const int bn = (b + 1) % P;
            for (size_t i = 0; i < per_bead; ++i) {
                sim.coord[i] = coords[(size_t)b * per_bead + i];
                sim.prev_coord[i] = coords[(size_t)bp * per_bead + i];
                sim.next_coord[i] = coords[(size_t)bn * per_bead + i];
            }
            sim.updateForces();
            dVec spring(N), phys(N);
            sim.updateSpringForces(spring);
            sim.updatePhysicalForces(phys);

            double scal[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            if (sim.is_bosonic_bead) {
                sim.bosonic_exchange->prepare();
                scal[0] = sim.bosonic_exchange->effectivePotential();
                scal[1] = sim.bosonic_exchange->primEstimator();
                scal[2] = sim.bosonic_exchange->getDistinctProbability();
                scal[3] = sim.bosonic_exchange->getLongestProbability();
                scal[7] = 1.0;
            }
            scal[4] = sim.classicalSpringEnergy();
            scal[5] = sim.ext_potential->V(sim.coord);
            double pair_v = 0.0;
            if (sim.int_pot_cutoff != 0.0) {
                for (int i = 0; i < N; ++i)
                    for (int j = i + 1; j < N; ++j) {
                        dVec diff = sim.getSeparation(i, j, MINIM);
                        double r = diff.norm();
                        if (r < sim.int_pot_cutoff || sim.int_pot_cutoff < 0.0) pair_v += sim.int_potential->V(diff);
                    }
            }
            scal[6] = pair_v;

            out.write(reinterpret_cast<const char*>(sim.forces.data()), (std::streamsize)(per_bead * sizeof(double)));
            out.write(reinterpret_cast<const char*>(spring.data()), (std::streamsize)(per_bead * sizeof(double)));
            out.write(reinterpret_cast<const char*>(phys.data()), (std::streamsize)(per_bead * sizeof(double)));
            out.write(reinterpret_cast<const char*>(scal), sizeof(scal));
        }
    } catch (const std::exception& ex) {
        std::fprintf(stderr, "[ref_probe] %s\n", ex.what());
        rc = 1;
    }
    MPI_Finalize();
    return rc;
}
