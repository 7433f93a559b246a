// Builds KoMD's own start-up (src/main.cpp:37-99) with the GB300 adapters of
// komd_gb300/csrc/komd_adapters/GpuKoMD.h in place of LinkedCells, the force
// functors, Integrator, TemperatureSensor and VelocityScaling, compiled
// against the reference's headers and linked with its library objects and
// libkomd_gpu.so.  TEST INFRASTRUCTURE ONLY (oracle/ref/Makefile, target
// `adapters`; tests/test_adapters_ref.py).
//
// usage: komd_adapters_check <input.dat> [steps]
// With a GPU it runs Simulation::run for the input's timesteps through the
// adapters and prints the final temperature; without one the engine's
// creation fails and the adapter reports it as KoMD reports errors (a
// std::runtime_error carrying komd_gpu_last_error()): exit code 3.
#include <cstdio>
#include <cstring>
#include <memory>
#include <stdexcept>

#include "GpuKoMD.h"
#include "IO/CheckpointIO.h"
#include "IO/FileInput.h"
#include "IO/Logging.h"
#include "Registry.h"
#include "Simulation.h"
#include "Kokkos_Core.hpp"

int main(int argc, char **argv) {
    if (argc < 2) {
        std::fprintf(stderr, "usage: %s <input.dat>\n", argv[0]);
        return 2;
    }
    int rc = 0;
    Kokkos::initialize(argc, argv);
    {
        Registry::instance = std::make_unique<Registry>();
        Registry::instance->configuration_ptr() = std::make_shared<Configuration>();
        Registry::instance->vtkWriter_ptr() = std::make_shared<VTKWriter>();
        Log::init();
        if (!FileInput::readFile(argv[1])) {
            std::fprintf(stderr, "input rejected\n");
            return 4;
        }
        auto container = std::make_shared<GpuLinkedCells>();
        Registry::instance->moleculeContainer_ptr() = container;
        Registry::instance->forceFunctors().push_back(std::make_shared<GpuForces>());
        Registry::instance->integrators().push_back(std::make_unique<GpuIntegrator>());
        Registry::instance->temperature_sensor_ptr() = std::make_shared<GpuTemperatureSensor>();
        Registry::instance->sensors().push_back(std::dynamic_pointer_cast<Sensor>(Registry::instance->temperature_sensor()));
        Registry::instance->thermostats().push_back(std::make_unique<GpuVelocityScaling>());
        CheckpointIO::loadCheckpoint();
        Registry::instance->simulation_ptr() = std::make_shared<Simulation>();
        try {
            container->init();
            Registry::instance->simulation()->run();
            std::printf("adapters ran: T=%.17g\n", Registry::instance->temperature_sensor()->getTemperature());
        } catch (const std::runtime_error &e) {
            std::printf("engine error: %s\n", e.what());
            rc = 3;
        }
    }
    Registry::instance = nullptr;
    Log::finalize();
    Kokkos::finalize();
    return rc;
}
