// GpuKoMD.h -- adapters that put the GB300 engine behind KoMD's own plugin
// interfaces, for compiling inside KoMD's build (they include the
// reference's headers: container/MoleculeContainer.h, potentials/
// ForceFunctor.h, integrators/Integrator.h, sensors/TemperatureSensor.h,
// thermostats/VelocityScaling.h).  Not built by komd_gb300/build.py, which
// has no KoMD checkout; oracle/ref/Makefile builds them against one
// (target `adapters`) and tests/test_adapters_ref.py runs that build.
//
// Registration in KoMD's main.cpp (src/main.cpp:57-95):
//   Registry::instance->moleculeContainer_ptr() = std::make_shared<GpuLinkedCells>();
//   Registry::instance->forceFunctors().push_back(std::make_shared<GpuForces>());     // LJ12_6 + FENE + Limit (+ ATM)
//   Registry::instance->integrators().push_back(std::make_unique<GpuIntegrator>());
//   Registry::instance->temperature_sensor_ptr() = std::make_shared<GpuTemperatureSensor>();
//   Registry::instance->thermostats().push_back(std::make_unique<GpuVelocityScaling>());
// in place of LinkedCells, LJ12_6 / FENE / Limit / ATM(_NOLIST), Integrator,
// TemperatureSensor and VelocityScaling; Simulation::run is unchanged.
#pragma once

#include <memory>
#include <stdexcept>

#include "container/MoleculeContainer.h"
#include "integrators/Integrator.h"
#include "potentials/ForceFunctor.h"
#include "sensors/TemperatureSensor.h"
#include "thermostats/VelocityScaling.h"

#include "komd_gpu.h"

namespace komd_gb300 {

// KOMD_ERR_* -> the std::runtime_error KoMD throws for invariants (Registry.cpp:10)
inline void check(int rc) {
    if (rc != KOMD_OK) throw std::runtime_error(komd_gpu_last_error());
}

// the engine's configuration from KoMD's Configuration (IO/Configuration.h),
// with the defaults that reproduce the reference (one cutoff for LJ and ATM,
// the reference's ATM sign, triplet set and virial, FP32 pair arithmetic)
komd_config engine_config();

}  // namespace komd_gb300

// Replaces LinkedCells (container/LinkedCells.cpp:11-572): the engine owns
// positions, cells and lists on the device; the SOA is filled at init
// (constructSOAs) and refreshed from the device only when a CPU reader needs
// it (syncSOA).
class GpuLinkedCells : public MoleculeContainer {
public:
    GpuLinkedCells() = default;
    ~GpuLinkedCells() override;
    void init() override;               // LinkedCells.cpp:47-63
    void updateContainer() override;    // LinkedCells.cpp:65-81
    // cell iteration is the engine's (komd_gpu_get_cells); the CPU iterators
    // of LinkedCells serve functors that this adapter replaces
    std::unique_ptr<CellIterator> iteratorCell() override;
    std::unique_ptr<CellPairIterator> iteratorC08() override;
    std::unique_ptr<CellTripletIterator> iteratorTripletC08() override;
    // the device state (r, v, f) into the SOA, for sensors and IO on the host
    void syncSOA();
    komd_gpu *handle() const { return h_; }
private:
    komd_gpu *h_ = nullptr;
};

// One functor for LJ12_6 + FENE + Limit (+ ATM when enable_3b): the engine
// runs the 2-body terms, then the 3-body term, as Simulation::run orders them
// (ForceFunctor.cpp:10-14 calls handlePairList with the container's list).
class GpuForces : public ForceFunctor {
protected:
    void handlePairList(PairList &) override;   // potentials/ForceFunctor.h:27
};

// Velocity Verlet on the device (integrators/Integrator.cpp:10-37).
class GpuIntegrator : public Integrator {
public:
    void integrate0() override;   // integrators/Integrator.h:49-61
    void integrate1() override;
};

// TemperatureSensor on the synced SOA: the reference's own measurement
// (TemperatureSensor.cpp:22-43) of the engine's velocities.
class GpuTemperatureSensor : public TemperatureSensor {
public:
    void measure() override;
};

// VelocityScaling (VelocityScaling.cpp:12-25) applied to the engine's velocities.
class GpuVelocityScaling : public VelocityScaling {
public:
    void apply() override;
};
