// Reference harness: drives the reference's own library code (LinkedCells,
// LJ12_6, ATM / ATM_NOLIST, FENE, Limit, Integrator and the sensors) from a
// custom main and dumps its state as text, so that the CPU oracle and the
// CUDA engine can be checked against the reference itself.
//
// TEST INFRASTRUCTURE ONLY.  Built by oracle/ref/Makefile from the reference
// sources where they lie; the binary goes to oracle/_ref/ and is never part
// of the product.
//
// It mirrors Simulation::run (src/Simulation.cpp:10-80) without plugins and,
// unless KOMD_HARNESS_THERMOSTAT=1, without the always-on velocity-scaling
// thermostat, so that dynamics are NVE:
//   step 0 : updateContainer, forces            [+ temperature, VelocityScaling]
//   step k : integrate0, updateContainer, forces, integrate1   [+ the same]
// and after every requested step writes
//   R / V / F      per-site positions, velocities, forces   (%.17g)
//   CELLS          every cell of the (nd+2)^3 grid incl. halo copies
//   NCOUNT         per-site neighbour count inside the cutoff, read off the
//                  reference's own pair list with LJ12_6_Force's test
//   TEMP, UPOT, PRESSURE, RDF  sensor outputs (when enabled in the input)
//   LJHIST         the LJ sensor's U(r) and F(r) histograms of this step's
//                  measure alone (sums of u, sums of f, counts of u, counts
//                  of f per bin; Potential_Sensor's views, zeroed first)
//
// usage: komd_ref_harness <input.dat> <out.txt> <n_steps> [dump steps...]
//        functors are chosen from the input exactly as src/main.cpp:57-66 does.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <set>
#include <string>

#include "Registry.h"
#include "IO/Logging.h"
#include "IO/FileInput.h"
#include "IO/CheckpointIO.h"
#include "util/PhasespaceGenerator.h"
#include "potentials/LJ12_6.h"
#include "potentials/FENE.h"
#include "potentials/Limit.h"
#include "potentials/ATM.h"
#include "potentials/ATM_NOLIST.h"
#include "potentials/ATM2B.h"
#include "thermostats/VelocityScaling.h"
#include "plugins/IBI/IBI_ForceFunctor.h"
#include "plugins/IBI/RDF_Profiler.h"
#include "sensors/PressureSensor.h"
#include "sensors/LJ12_6_Sensor.h"
#include "sensors/RDFSensor.h"
#include "sensors/TemperatureSensor.h"
#include "container/LinkedCells.h"
#include "Kokkos_Core.hpp"

// the LJ sensor with its histogram views reachable: Potential_Sensor::measure
// adds every measure into the views (they are never cleared), so the harness
// zeroes them before a measure to dump that measure's histograms alone
struct LJSensorDump : public LJ12_6_Sensor {
    void clear_hist() {
        Kokkos::deep_copy(p_data_u, 0.0);
        Kokkos::deep_copy(p_data_f, 0.0);
        Kokkos::deep_copy(p_count_u, 0);
        Kokkos::deep_copy(p_count_f, 0);
    }
    void dump_hist(FILE* out) {
        fprintf(out, "LJHIST %llu\n", (unsigned long long)p_bins);
        for (uint64_t k = 0; k < p_bins; k++)
            fprintf(out, "%.17g %.17g %llu %llu\n", p_data_u[k], p_data_f[k], (unsigned long long)p_count_u[k],
                    (unsigned long long)p_count_f[k]);
    }
};

static void dump_vec(FILE* out, const char* key, KW::vec_t<math::d3>& a, uint64_t n) {
    fprintf(out, "%s %llu\n", key, (unsigned long long)n);
    for (uint64_t i = 0; i < n; i++) fprintf(out, "%.17g %.17g %.17g\n", a[i].x(), a[i].y(), a[i].z());
}

int main(int argc, char** argv) {
    if (argc < 4) {
        fprintf(stderr, "usage: %s <input.dat> <out.txt> <n_steps> [dump steps...]\n", argv[0]);
        return 2;
    }
    Kokkos::initialize(argc, argv);
    {
        Registry::instance = std::make_unique<Registry>();
        Registry::instance->configuration_ptr() = std::make_shared<Configuration>();
        Registry::instance->vtkWriter_ptr() = std::make_shared<VTKWriter>();
        Log::init();
        if (!FileInput::readFile(argv[1])) { fprintf(stderr, "input rejected\n"); return 3; }
        auto config = Registry::instance->configuration();
        Registry::instance->moleculeContainer_ptr() = std::make_shared<LinkedCells>();

        // force functors as src/main.cpp:57-66
        const bool atm2b = config->enable_3b_approx;
        Registry::instance->forceFunctors().push_back(std::make_shared<FENE>());
        Registry::instance->forceFunctors().push_back(std::make_shared<Limit>());
        if (config->enable_3b) {
            if (config->enable_3b_direct) Registry::instance->forceFunctors3b().push_back(std::make_shared<ATM_NOLIST>());
            else Registry::instance->forceFunctors3b().push_back(std::make_shared<ATM>());
        }
        Registry::instance->integrators().push_back(std::make_unique<Integrator>());
        CheckpointIO::loadCheckpoint();
        PhasespaceGenerator::generate();   // ps_gen_region entries, as main.cpp:70-71
        // ATM2B reads the molecule count in its constructor.  main.cpp:57 builds
        // it before CheckpointIO::loadCheckpoint (main.cpp:70), where the count is
        // still 0 and the factor comes out as exactly 1; here it is built after the
        // checkpoint is loaded so that the factor formula itself is exercised.  It
        // goes first in the functor list as in main.cpp:57-58.
        // KOMD_HARNESS_IBI_TABLE=<file>: IBI_ForceFunctor<IBI_Default> with that
        // force table (FunctionPL::read; defaults 1e6 below, 0 above as
        // IBI::derivativeOfPotential sets them) takes the LJ functor's place, as
        // the IBI plugin swaps it in (IBI.cpp:52-54); the RDF_Profiler histogram
        // is dumped as IBIRDF
        const char* ibi_table = getenv("KOMD_HARNESS_IBI_TABLE");
        std::shared_ptr<ForceFunctor> first;
        if (ibi_table && *ibi_table) {
            auto ibi = std::make_shared<IBI_ForceFunctor<IBI_Default>>();
            ibi->getForceFunction().read(ibi_table);
            ibi->getForceFunction().setLowerDefault(1e+6);
            ibi->getForceFunction().setUpperDefault(0.0);
            first = ibi;
        } else if (atm2b) {
            first = std::make_shared<ATM2B>();
        } else {
            first = std::make_shared<LJ12_6>();
        }
        Registry::instance->forceFunctors().insert(Registry::instance->forceFunctors().begin(), first);
        std::unique_ptr<RDF_Profiler> profiler;
        if (ibi_table && *ibi_table) profiler = std::make_unique<RDF_Profiler>();

        auto temp = std::make_shared<TemperatureSensor>();
        // KOMD_HARNESS_THERMOSTAT=1: the always-on VelocityScaling of main.cpp:95
        // and Simulation.cpp:42,72 (after the initial forces and after every step)
        const char* th = getenv("KOMD_HARNESS_THERMOSTAT");
        std::unique_ptr<VelocityScaling> thermostat;
        if (th && atoi(th) != 0) {
            Registry::instance->temperature_sensor_ptr() = temp;
            thermostat = std::make_unique<VelocityScaling>();
        }
        std::shared_ptr<LJSensorDump> pot;
        std::shared_ptr<PressureSensor> pres;
        std::shared_ptr<RDFSensor> rdf;
        if (config->enable_sensor_lj) pot = std::make_shared<LJSensorDump>();
        if (config->enable_sensor_pres) pres = std::make_shared<PressureSensor>();
        auto container = Registry::instance->moleculeContainer();
        container->init();
        if (config->enable_sensor_rdf) rdf = std::make_shared<RDFSensor>();

        const int n_steps = atoi(argv[3]);
        std::set<int> dumps;
        for (int a = 4; a < argc; a++) dumps.insert(atoi(argv[a]));
        if (dumps.empty()) dumps.insert(n_steps);

        FILE* out = fopen(argv[2], "w");
        if (!out) { fprintf(stderr, "cannot write %s\n", argv[2]); return 4; }
        const double cutoff2 = std::pow(config->cutoff, 2);

        for (int step = 0; step <= n_steps; step++) {
            if (step > 0) for (auto& it : Registry::instance->integrators()) it->integrate0();
            container->updateContainer();
            for (auto& p : Registry::instance->forceFunctors()) (*p)();
            if (config->enable_3b) for (auto& p : Registry::instance->forceFunctors3b()) (*p)();
            if (step > 0) for (auto& it : Registry::instance->integrators()) it->integrate1();
            if (thermostat) { temp->measure(); thermostat->apply(); }
            if (!dumps.count(step)) continue;

            SOA& soa = container->getSOA();
            const uint64_t n = soa.size();
            fprintf(out, "STEP %d\n", step);
            dump_vec(out, "R", soa.r(), n);
            dump_vec(out, "V", soa.v(), n);
            dump_vec(out, "F", soa.f(), n);

            // cell lists, LCCellIterator order (x fastest), halo cells included
            uint64_t ncell = 0;
            for (auto it = container->iteratorCell(); it->isValid(); ++(*it)) ncell++;
            fprintf(out, "CELLS %llu\n", (unsigned long long)ncell);
            for (auto it = container->iteratorCell(); it->isValid(); ++(*it)) {
                Cell& c = it->cell();
                fprintf(out, "%llu", (unsigned long long)c.getNumIndices());
                for (uint64_t k = 0; k < c.getNumIndices(); k++) fprintf(out, " %llu", (unsigned long long)c.indices()[k]);
                fprintf(out, "\n");
            }

            // neighbour counts from the reference's own pair list
            PairList& pl = container->getPairList();
            auto pairs = pl.getPairs();
            auto offs = pl.getOffsets();
            std::vector<uint64_t> cnt(n, 0);
            for (uint64_t p = 0; p < pl.size(); p++) {
                const uint64_t s0 = pairs(p, 0), s1 = pairs(p, 1);
                if (soa.id()[s0] == soa.id()[s1]) continue;
                const math::d3 sh0 = offs(p, 0), sh1 = offs(p, 1);
                const math::d3 dr = (soa.r()[s0] + sh0) - (soa.r()[s1] + sh1);
                if (dr.dot(dr) > cutoff2) continue;
                if (sh0 == 0) cnt[s0]++;
                if (sh1 == 0) cnt[s1]++;
            }
            fprintf(out, "NCOUNT %llu\n", (unsigned long long)n);
            for (uint64_t i = 0; i < n; i++) fprintf(out, "%llu\n", (unsigned long long)cnt[i]);
            fprintf(out, "NPAIRS %llu\n", (unsigned long long)pl.size());

            temp->measure();
            fprintf(out, "TEMP %.17g\n", temp->getTemperature());
            if (pot) {
                pot->clear_hist();
                pot->measure();
                fprintf(out, "UPOT %.17g\n", pot->getCurrentPotential());
                pot->dump_hist(out);
            }
            if (pres) {
                pres->measure();
                const auto& t = pres->getPressureTensor();
                fprintf(out, "PRESSURE 6\n");
                for (int k = 0; k < 6; k++) fprintf(out, "%.17g\n", t[k]);
            }
            if (profiler) {
                profiler->reset();
                profiler->measure();
                KW::vec_t<double> g("IBIRDF", profiler->getBufferSize());
                profiler->getRDF(g);
                fprintf(out, "IBIRDF %llu\n", (unsigned long long)profiler->getBufferSize());
                for (uint64_t k = 0; k < profiler->getBufferSize(); k++) fprintf(out, "%.17g\n", g[k]);
            }
            if (rdf) {
                rdf->measure();
                rdf->write(step);   // rdf_<step>.txt in the working directory
            }
        }
        fclose(out);
    }
    Registry::instance = nullptr;
    Log::finalize();
    Kokkos::finalize();
    return 0;
}
