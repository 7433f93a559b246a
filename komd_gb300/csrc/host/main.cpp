// main.cpp -- the `komd` executable: KoMD's stock main (src/main.cpp:37-99)
// on the GB300 engine.  Usage: komd <input file> [--fused | --phasespace <out.ps>]
//   --fused   advance write_freq steps per engine call (CUDA graph replay with
//             the thermostat on the device); log lines at write steps only
//   --phasespace <out.ps>   write the initial phase space (checkpoint files and
//             ps_gen_region molecules) with 17 significant digits and stop,
//             before any GPU work
// Input files are KoMD's; the phase space comes from checkpoint_file entries
// and ps_gen_region entries (PhasespaceGenerator, as main.cpp:70-71 orders
// them).  The IBI and IBI_Reload plugins run (ibi.h); AdResS and the
// FENE and displacement sensors are not available and are reported, not
// silently skipped.
#include <cstdio>
#include <cstring>
#include <iostream>
#include <stdexcept>

#include "gpu_adapters.h"
#include "ibi.h"

using namespace komd;

int main(int argc, char **argv) {
    if (argc <= 1) {
        std::cout << "Run program with: komd <input file> [--fused]" << std::endl;
        return 0;
    }
    bool fused = false;
    const char *ps_out = nullptr;
    for (int a = 2; a < argc; a++) {
        if (std::strcmp(argv[a], "--fused") == 0) fused = true;
        if (std::strcmp(argv[a], "--phasespace") == 0 && a + 1 < argc) ps_out = argv[++a];
    }
    try {
        Registry::instance = std::make_unique<Registry>();
        Registry::instance->configuration_ptr() = std::make_shared<Configuration>();
        if (!FileInput::readFile(argv[1])) return 0;
        auto cfg = Registry::instance->configuration();
        if (cfg->enable_one_cell) throw std::runtime_error("not supported anymore");
        if (cfg->ADR_enable) throw std::runtime_error("the AdResS plugin is not available in this engine");
        const bool plugins = cfg->IBI_enable || cfg->IBI_reload_enable;
        if (plugins && fused)
            throw std::runtime_error("--fused advances whole write intervals on the device; the IBI plugins need "
                                     "their per-step hooks");
        if (plugins && cfg->gpu_skin > 0)
            throw std::runtime_error("the IBI plugins' tabulated force runs on per-step cell lists: set gpu_skin 0");
        auto container = std::make_shared<GpuLinkedCells>();
        container->device_thermostat = fused;
        Registry::instance->moleculeContainer_ptr() = container;
        Registry::instance->simulation_ptr() = std::make_shared<Simulation>();

        // force functors (main.cpp:57-66): LJ12_6 or ATM2B, FENE, Limit and ATM
        // are terms of one engine call
        Registry::instance->forceFunctors().push_back(std::make_shared<GpuForces>());
        if (cfg->enable_3b) Registry::instance->forceFunctors3b().push_back(std::make_shared<GpuATM>());
        Registry::instance->integrators().push_back(std::make_unique<GpuIntegrator>());
        if (!CheckpointIO::loadCheckpoint()) return 0;
        PhasespaceGenerator::generate();
        if (ps_out) {   // the .ps layout of CheckpointIO::writeCheckpoint, full precision
            FILE *f = std::fopen(ps_out, "w");
            if (!f) throw std::runtime_error(std::string("cannot write ") + ps_out);
            bool first = true;
            for (const Molecule &m : container->molecules())
                for (size_t q = 0; q < m.r.size(); q++) {
                    std::fprintf(f, "%s%llu\t%.17g %.17g %.17g\t%.17g %.17g %.17g\t%.17g %.17g %.17g", first ? "" : "\n",
                                 (unsigned long long)m.id, m.r[q][0], m.r[q][1], m.r[q][2], m.v[q][0], m.v[q][1],
                                 m.v[q][2], m.mass[q], m.eps[q], m.sig[q]);
                    first = false;
                }
            std::fclose(f);
            Registry::instance = nullptr;
            return 0;
        }
        container->init();

        // measurements (main.cpp:74-85)
        auto temp = std::make_shared<GpuTemperatureSensor>();
        Registry::instance->temperature_sensor_ptr() = temp;
        Registry::instance->sensors().push_back(temp);
        if (cfg->enable_sensor_lj) {
            auto pot = std::make_shared<GpuLJSensor>();
            Registry::instance->potential_sensor_ptr() = pot;
            Registry::instance->sensors().push_back(pot);
        }
        if (cfg->enable_sensor_rdf) Registry::instance->sensors().push_back(std::make_shared<GpuRDFSensor>());
        if (cfg->enable_sensor_pres) Registry::instance->sensors().push_back(std::make_shared<GpuPressureSensor>());
        if (cfg->enable_sensor_visc) Registry::instance->sensors().push_back(std::make_shared<GpuViscositySensor>());
        if (cfg->enable_sensor_fene || cfg->enable_sensor_disp)
            std::cerr << "note: the FENE and displacement sensors are not available" << std::endl;
        // plugins (main.cpp:89-91)
        if (cfg->IBI_enable) Registry::instance->plugins().push_back(std::make_unique<GpuIBI>());
        if (cfg->IBI_reload_enable) Registry::instance->plugins().push_back(std::make_unique<GpuIBIReload>());
        Registry::instance->thermostats().push_back(std::make_unique<GpuVelocityScaling>());

        Registry::instance->simulation()->run(fused);
    } catch (const std::exception &e) {
        std::cerr << "komd: " << e.what() << std::endl;
        Registry::instance = nullptr;
        return 1;
    }
    Registry::instance = nullptr;
    return 0;
}
