// gpu_adapters.h -- the reference's plugin interfaces implemented on the
// GB300 engine (include/komd_gpu.h).  One engine handle, owned by the
// container, is shared by the functors, the integrator, the sensors and the
// thermostat through the Registry, as the reference shares its SOA.
#pragma once

#include <stdexcept>
#include <string>
#include <vector>

#include "komd_host.h"

namespace komd {

inline void gpu_check(int rc) {
    if (rc != KOMD_OK) throw std::runtime_error(komd_gpu_last_error());
}

// LinkedCells (container/LinkedCells.{h,cpp}): COM, periodic wrap, binning,
// halo copies and the force terms' neighbour search all run in the engine.
class GpuLinkedCells : public MoleculeContainer {
public:
    ~GpuLinkedCells() override;
    void init() override;                      // LinkedCells::init: engine + upload
    void updateContainer() override;           // LinkedCells::updateContainer
    void syncHost() override;
    void advance(uint64_t n) override { gpu_check(komd_gpu_step(h_, (int64_t)n)); }
    komd_gpu *handle() const { return h_; }
    // engine configuration derived from the Registry's Configuration
    static komd_config engineConfig(const Configuration &c, bool device_thermostat);
    bool device_thermostat = false;            // set before init(): thermostat inside komd_gpu_step
private:
    komd_gpu *h_ = nullptr;
};

komd_gpu *engine();   // the container's handle (throws before init)

// LJ12_6 or ATM2B, FENE and Limit (main.cpp:57-61): one engine call computes
// every configured term, so a single functor stands for the three
class GpuForces : public ForceFunctor {
protected:
    void handlePairList() override { gpu_check(komd_gpu_forces(engine())); }
};

// ATM / ATM_NOLIST (main.cpp:63-66): the engine adds the triplet term inside
// komd_gpu_forces when enable_3b is set, so the 3-body pass has nothing left
class GpuATM : public ForceFunctor3B {
protected:
    void handleTripleList() override {}
};

class GpuIntegrator : public Integrator {
public:
    void integrate0() override { gpu_check(komd_gpu_integrate0(engine())); }
    void integrate1() override { gpu_check(komd_gpu_integrate1(engine())); }
};

class GpuTemperatureSensor : public TemperatureSensor {
public:
    void measure() override;
    void write(uint64_t) override {}           // TemperatureSensor::write writes nothing
};

// LJ12_6_Sensor + Potential_Sensor: total potential, U(r) / F(r) histograms
class GpuLJSensor : public PotentialSensor {
public:
    GpuLJSensor();
    void measure() override;
    void write(uint64_t simstep) override;     // pot_LJ12_6_<step>.txt, pot_history_LJ12_6_<step>.txt
private:
    std::vector<double> u_, f_, cu_, cf_, hist_, pot_hist_;
};

class GpuRDFSensor : public Sensor {
public:
    GpuRDFSensor();
    void measure() override;
    void write(uint64_t simstep) override;     // rdf_<step>.txt as RDFSensor::write
private:
    std::vector<double> bins_;
    uint64_t samples_ = 0;
};

class GpuPressureSensor : public Sensor {
public:
    GpuPressureSensor() : Sensor("PressureSensor") {}
    void measure() override;
    void write(uint64_t simstep) override;     // pressures_<step>.txt as PressureSensor::write
    const double *tensor() const { return p_; }
private:
    double p_[6] = {0, 0, 0, 0, 0, 0};
};

// ViscositySensor (sensors/ViscositySensor.cpp): the pressure tensor / V of
// every measure; at write, Green-Kubo integrals of the bulk (XX YY ZZ) and
// shear (XY XZ YZ) autocorrelations, averaged over the components
class GpuViscositySensor : public Sensor {
public:
    GpuViscositySensor() : Sensor("Viscosity") {}
    void measure() override;
    void write(uint64_t simstep) override;     // viscosity_<step>.txt
    // TensorEvaluator::integrate for the components `dims` of the recorded series
    static double integrate(const std::vector<std::vector<double>> &series, const int *dims, int ndims, double dt,
                            bool origin_free);
private:
    std::vector<std::vector<double>> series_ = std::vector<std::vector<double>>(6);
};

// VelocityScaling (thermostats/VelocityScaling.cpp:12-25)
class GpuVelocityScaling : public Thermostat {
public:
    void apply() override;
};

}  // namespace komd
