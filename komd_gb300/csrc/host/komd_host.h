// komd_host.h -- KoMD's host-side plugin API over the GB300 engine.
//
// The same Registry / Configuration / FileInput / CheckpointIO and the same
// plugin interfaces (ForceFunctor, ForceFunctor3B, Integrator, Sensor,
// Thermostat, Plugin, MoleculeContainer) with the reference's method names
// (src/Registry.h, src/IO/*.h, src/potentials/ForceFunctor*.h,
// src/integrators/Integrator.h, src/sensors/Sensor.h,
// src/thermostats/Thermostat.h, src/plugins/Plugin.h,
// src/container/MoleculeContainer.h).  The particle data live in the engine
// (include/komd_gpu.h); the container keeps a host copy of the sites only
// for input and checkpoint output.  Errors are std::runtime_error, as in the
// reference; FileInput::readFile returns false after printing the reason.
#pragma once

#include <array>
#include <cmath>
#include <cstdint>
#include <limits>
#include <memory>
#include <string>
#include <tuple>
#include <utility>
#include <vector>

#include "komd_gpu.h"

namespace komd {

using d3 = std::array<double, 3>;

// unit conversion J -> internal energy (u A^2 / ps^2), util/constants.h:20
constexpr double kConvJtoInternal = 6.022140754e22;

// IO/Configuration.h with the defaults of util/defaults.h; the engine keys
// (precision and physics modes) are additions under gpu_*.
struct Configuration {
    double temperature = 300;
    double delta_t = 0.001;
    uint64_t timesteps = 1;
    double cutoff = 2.5;
    double cell_size = 3.0;
    double density = 0.1;
    double max_epsilon = std::numeric_limits<double>::min();
    double max_sigma = std::numeric_limits<double>::min();
    double stiffness_factor = 30;
    double limit_factor = 20;
    double energy_3b = 1;
    int pair_steps = 4;
    int triple_steps = 8;
    d3 domainLow{0, 0, 0};
    d3 domainHigh{10, 10, 10};
    std::vector<std::pair<std::string, d3>> checkpoint_files;
    uint64_t write_freq = 10;
    std::vector<std::tuple<d3, d3, uint32_t>> phasespace_gen_regions;
    bool storeCheckpoint = false;
    bool enable_3b_approx = false;
    bool enable_3b = false;
    bool enable_3b_direct = true;
    bool enable_sensor_lj = false;
    bool enable_sensor_fene = false;
    bool enable_sensor_rdf = false;
    bool enable_sensor_disp = false;
    bool enable_sensor_pres = false;
    bool enable_sensor_visc = false;
    uint64_t sensor_lj_bins = 100;
    uint64_t sensor_fene_bins = 100;
    double sensor_rdf_max = 5.0;
    double sensor_rdf_dr = 0.1;
    int sensor_visc_window = 1000;
    bool sensor_visc_no_orig = false;
    bool IBI_enable = false;
    uint64_t IBI_bins = 100;
    double IBI_alpha = 0.2;
    int IBI_steps_equil = 1000000;
    int IBI_steps_measure = 100000;
    double IBI_conv_threshold = 0.99;
    std::string IBI_conv_mode = "integral";
    std::string IBI_conv_stop = "worse";
    int IBI_conv_window = 10;
    bool IBI_reload_enable = false;
    std::string IBI_reload_fpath, IBI_reload_ppath;
    d3 IBI_exclusion_low{0, 0, 0};
    d3 IBI_exclusion_high{0, 0, 0};
    bool ADR_enable = false;
    bool enable_one_cell = false;
    // engine keys (no reference counterpart)
    int gpu_precision = KOMD_FP32;                  // gpu_precision fp32|fp64
    int gpu_atm_sign = KOMD_ATM_SIGN_REFERENCE;     // gpu_atm_sign reference|physical
    int gpu_atm_enum = KOMD_ATM_ENUM_COMPAT;        // gpu_atm_enum compat|full
    int gpu_virial = KOMD_VIRIAL_COMPAT;            // gpu_virial compat|correct
    double gpu_skin = 0.0;                          // gpu_skin <float>
    int gpu_device = 0;                             // gpu_device <int>
    bool gpu_atm2b_physical = false;                // gpu_atm2b physical: ATM2B factor from the loaded density
    bool gpu_vtk = false;                           // gpu_vtk 1: VTK_Output_<step>.vtu as a USE_VTK build writes
    double gpu_switch_width = 0.0;                  // gpu_switch_width <float>: the labelled switched-cutoff
                                                    // option (komd_config::switch_width); 0 = the reference's
                                                    // truncated potentials
};

struct SiteDesc {
    double epsilon, sigma, mass;
    d3 r;
};
struct Component {
    std::vector<SiteDesc> sites;
    void addSite(double eps, double sig, double mass, const d3 &r) { sites.push_back({eps, sig, mass, r}); }
};

struct Molecule {
    uint64_t id = 0;
    std::vector<d3> r, v;
    std::vector<double> mass, eps, sig;
    void addSite(double e, double s, double m, const d3 &pos, const d3 &vel) {
        eps.push_back(e); sig.push_back(s); mass.push_back(m); r.push_back(pos); v.push_back(vel);
    }
    d3 centerOfMass() const;
};

// SciValue (math/SciValue.{h,cpp}): mantissa normalised into (0.1, 10) by /10
// and *10 steps, products renormalised, converted as m * pow(10, e).  The
// loops are bounded (no finite double needs 400 steps; zero, NaN and inf come
// back at once) where the reference's would not end on an infinite mantissa.
struct Sci {
    double m;
    long long e;
    Sci(double mm, long long ee) : m(mm), e(ee) { norm(); }
    explicit Sci(double v) : m(v), e(0) { if (v != 0.0) norm(); }
    void norm() {
        double a = std::fabs(m);
        if (!(a <= 1.7976931348623157e308) || a == 0.0) return;
        for (int k = 0; k < 400 && a >= 10.0; k++) { m /= 10.0; e += 1; a = std::fabs(m); }
        for (int k = 0; k < 400 && a <= 0.1; k++) { m *= 10.0; e -= 1; a = std::fabs(m); }
    }
    Sci operator*(const Sci &o) const { return Sci(m * o.m, e + o.e); }
    Sci operator/(const Sci &o) const { return Sci(m / o.m, e - o.e); }
    Sci operator*(double o) const { return *this * Sci(o); }
    double value() const { return m * std::pow(10, e); }
};

// Molecule::NEXT_ID of the reference (molecule/Molecule.cpp:8-10): every
// default-constructed molecule takes the next id (0 went to Molecule::INVALID);
// the checkpoint loader takes ids as KoMD's does and then sets the file's,
// the phase-space generator keeps them.
uint64_t next_molecule_id();

// PhasespaceGenerator (util/PhasespaceGenerator.cpp:27-95): molecules of the
// ps_gen_region entries' components on a grid of spacing L / (rho V)^(1/3)
// from begin + 0.5, each rotated by random Euler angles (uniform in [0, 2 pi),
// default_random_engine seeded 43) and given one Maxwell-Boltzmann velocity
// (normal draws from a default_random_engine seeded 42, std dev
// sqrt(T / M kB / Da) in A/ps).  Both engines are static, as in the reference:
// they run on across calls.
namespace PhasespaceGenerator {
void generate();
}

// --- plugin interfaces ------------------------------------------------------
class MoleculeContainer {
public:
    virtual ~MoleculeContainer() = default;
    virtual void init() = 0;              // after all molecules are added
    virtual void updateContainer() = 0;
    void addMolecule(const Molecule &m);  // throws if the COM is outside the domain
    uint64_t getNumMolecules() const { return molecules_.size(); }
    uint64_t getNumSites() const;
    const std::vector<Molecule> &molecules() const { return molecules_; }
    // host copy of the sites (molecule order), refreshed by syncHost()
    virtual void syncHost() = 0;
    // n whole steps (integrate0, updateContainer, forces, integrate1 and the
    // thermostat when the container runs it) without host round trips
    virtual void advance(uint64_t n) = 0;
    std::vector<d3> r, v, f;
protected:
    std::vector<Molecule> molecules_;
};

class ForceFunctor {
public:
    virtual ~ForceFunctor() = default;
    void operator()() { handlePairList(); }
protected:
    virtual void handlePairList() = 0;
};

class ForceFunctor3B {
public:
    virtual ~ForceFunctor3B() = default;
    void operator()() { handleTripleList(); }
protected:
    virtual void handleTripleList() = 0;
};

class Integrator {
public:
    virtual ~Integrator() = default;
    virtual void integrate0() = 0;
    virtual void integrate1() = 0;
};

class Sensor {
public:
    explicit Sensor(std::string name) : name_(std::move(name)) {}
    virtual ~Sensor() = default;
    virtual void measure() = 0;
    virtual void write(uint64_t simstep) = 0;
    const std::string &name() const { return name_; }
private:
    std::string name_;
};

class TemperatureSensor : public Sensor {
public:
    TemperatureSensor() : Sensor("Temperature") {}
    double getTemperature() const { return temperature_; }
protected:
    double temperature_ = 0.0;
};

class PotentialSensor : public Sensor {
public:
    using Sensor::Sensor;
    double getCurrentPotential() const { return potential_; }
protected:
    double potential_ = 0.0;
};

class Thermostat {
public:
    virtual ~Thermostat() = default;
    virtual void apply() = 0;
};

class Plugin {
public:
    explicit Plugin(std::string name) : name_(std::move(name)) {}
    virtual ~Plugin() = default;
    virtual void pre_main_loop() {}
    virtual void post_main_loop() {}
    virtual void begin_loop() {}
    virtual void end_loop() {}
    virtual void post_forces() {}
    virtual void pre_container_update() {}
    virtual void post_container_update() {}
    virtual void init() {}
    virtual void finalize() {}
    const std::string &name() const { return name_; }
private:
    std::string name_;
};

class Simulation {
public:
    // Simulation::run (Simulation.cpp:10-80); fused = one komd_gpu_step per
    // write interval (device thermostat, log lines at write steps only)
    void run(bool fused = false);
    void stop() { max_step_ = simstep_; }
    uint64_t simstep() const { return simstep_; }
private:
    uint64_t simstep_ = 0, max_step_ = 0;
};

class Registry {
public:
    static std::unique_ptr<Registry> instance;
    std::shared_ptr<Configuration> &configuration_ptr() { return configuration_; }
    std::shared_ptr<Configuration> configuration() { return configuration_; }
    std::vector<Component> &components() { return components_; }
    std::shared_ptr<MoleculeContainer> &moleculeContainer_ptr() { return container_; }
    std::shared_ptr<MoleculeContainer> moleculeContainer() { return container_; }
    std::vector<std::shared_ptr<ForceFunctor>> &forceFunctors() { return functors_; }
    std::vector<std::shared_ptr<ForceFunctor3B>> &forceFunctors3b() { return functors3b_; }
    std::vector<std::unique_ptr<Integrator>> &integrators() { return integrators_; }
    std::vector<std::shared_ptr<Sensor>> &sensors() { return sensors_; }
    std::vector<std::unique_ptr<Thermostat>> &thermostats() { return thermostats_; }
    std::vector<std::unique_ptr<Plugin>> &plugins() { return plugins_; }
    std::shared_ptr<TemperatureSensor> &temperature_sensor_ptr() { return temp_; }
    std::shared_ptr<TemperatureSensor> temperature_sensor() { return temp_; }
    std::shared_ptr<PotentialSensor> &potential_sensor_ptr() { return pot_; }
    std::shared_ptr<PotentialSensor> potential_sensor() { return pot_; }
    std::shared_ptr<Simulation> &simulation_ptr() { return simulation_; }
    std::shared_ptr<Simulation> simulation() { return simulation_; }
private:
    std::shared_ptr<Configuration> configuration_;
    std::vector<Component> components_;
    std::shared_ptr<MoleculeContainer> container_;
    std::vector<std::shared_ptr<ForceFunctor>> functors_;
    std::vector<std::shared_ptr<ForceFunctor3B>> functors3b_;
    std::vector<std::unique_ptr<Integrator>> integrators_;
    std::vector<std::shared_ptr<Sensor>> sensors_;
    std::vector<std::unique_ptr<Thermostat>> thermostats_;
    std::vector<std::unique_ptr<Plugin>> plugins_;
    std::shared_ptr<TemperatureSensor> temp_;
    std::shared_ptr<PotentialSensor> pot_;
    std::shared_ptr<Simulation> simulation_;
};

namespace FileInput {
// IO/FileInput.cpp:13-121: the same keys, checks and messages; false on error
bool readFile(const std::string &filename);
}

namespace VTKWriter {
// IO/VTKWriter.cpp:21-123: one .vtu per call (<name>_<4-digit iteration>.vtu),
// sites in molecule order with mass, velocity, force, id, cid as Float32 /
// Int32 point data; the reference writes only when built with USE_VTK, here
// only with gpu_vtk 1
void write(const std::string &filename, uint64_t iteration);
}

namespace CheckpointIO {
// IO/CheckpointIO.cpp: ckpt_<step>.ps, "id\tx y z\tvx vy vz\tm eps sig", no trailing newline
void writeCheckpoint(uint64_t simstep);
// every checkpoint_file of the configuration (with its offset) into the container
bool loadCheckpoint();
}

}  // namespace komd
