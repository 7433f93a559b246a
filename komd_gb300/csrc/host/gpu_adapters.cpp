// gpu_adapters.cpp -- plugin interfaces on the engine (see gpu_adapters.h).
#include "gpu_adapters.h"

#include <cmath>
#include <fstream>
#include <iostream>
#include <sstream>

namespace komd {

namespace {
double volume() {
    const auto c = Registry::instance->configuration();
    return (c->domainHigh[0] - c->domainLow[0]) * (c->domainHigh[1] - c->domainLow[1]) *
           (c->domainHigh[2] - c->domainLow[2]);
}
}  // namespace

komd_gpu *engine() {
    auto c = std::dynamic_pointer_cast<GpuLinkedCells>(Registry::instance->moleculeContainer());
    if (!c || !c->handle()) throw std::runtime_error("the GPU container is not initialised");
    return c->handle();
}

GpuLinkedCells::~GpuLinkedCells() {
    if (h_) komd_gpu_destroy(h_);
}

komd_config GpuLinkedCells::engineConfig(const Configuration &c, bool device_thermostat) {
    komd_config k{};
    for (int d = 0; d < 3; d++) {
        k.domain_low[d] = c.domainLow[d];
        k.domain_high[d] = c.domainHigh[d];
    }
    k.cell_size = c.cell_size;
    k.cutoff = c.cutoff;
    k.cutoff_3b = c.cutoff;                      // one cutoff, as the reference
    k.nu = c.energy_3b * 1e+9 * kConvJtoInternal;  // ATM.cpp:11-14
    k.delta_t = c.delta_t;
    k.stiffness = c.stiffness_factor;
    k.limit = c.limit_factor;
    k.terms = KOMD_TERM_LJ | KOMD_TERM_FENE | KOMD_TERM_LIMIT;
    if (c.enable_3b) k.terms |= KOMD_TERM_ATM;
    // main.cpp builds ATM2B before the checkpoint is loaded, where its factor
    // evaluates to exactly 1 (plain LJ forces); gpu_atm2b physical applies the
    // factor with the loaded density
    if (c.enable_3b_approx && c.gpu_atm2b_physical) k.terms |= KOMD_TERM_ATM2B;
    k.precision = c.gpu_precision;
    k.atm_sign = c.gpu_atm_sign;
    k.atm_enum = c.gpu_atm_enum;
    k.virial_mode = c.gpu_virial;
    k.atm_direct = c.enable_3b_direct ? 1 : 0;
    k.max_sigma = c.max_sigma;
    k.lj_bins = (int32_t)c.sensor_lj_bins;
    if (c.enable_sensor_rdf) {
        k.rdf_max = c.sensor_rdf_max;
        k.rdf_dr = c.sensor_rdf_dr;
    }
    k.skin = c.gpu_skin;
    k.temperature_target = c.temperature;
    k.thermostat = device_thermostat ? 1 : 0;
    if (c.gpu_switch_width > 0) {
        // the switched-cutoff option covers LJ and exact ATM: the always-registered
        // FENE and Limit functors must have nothing to do (one site per molecule,
        // an inactive limit), and are left out of the engine's terms
        for (const Component &comp : Registry::instance->components())
            if (comp.sites.size() > 1)
                throw std::runtime_error("gpu_switch_width needs single-site components (FENE acts on multi-site ones)");
        if (c.limit_factor < 1e29) throw std::runtime_error("gpu_switch_width needs an inactive Limit (limit >= 1e29)");
        k.terms &= ~(KOMD_TERM_FENE | KOMD_TERM_LIMIT);
        k.switch_width = c.gpu_switch_width;
    }
    return k;
}

void GpuLinkedCells::init() {
    const auto cfg = Registry::instance->configuration();
    const komd_config k = engineConfig(*cfg, device_thermostat);
    gpu_check(komd_gpu_create(&k, cfg->gpu_device, &h_));
    const uint64_t n = getNumSites();
    std::vector<double> rr(3 * n), vv(3 * n), m(n), e(n), s(n);
    std::vector<uint64_t> id(n);
    uint64_t i = 0;
    for (const Molecule &mol : molecules_)
        for (size_t q = 0; q < mol.r.size(); q++, i++) {
            for (int d = 0; d < 3; d++) {
                rr[3 * i + d] = mol.r[q][d];
                vv[3 * i + d] = mol.v[q][d];
            }
            m[i] = mol.mass[q];
            e[i] = mol.eps[q];
            s[i] = mol.sig[q];
            id[i] = mol.id;
        }
    gpu_check(komd_gpu_upload_sites(h_, (int64_t)n, rr.data(), vv.data(), m.data(), e.data(), s.data(), id.data()));
    r.assign(n, d3{0, 0, 0});
    v.assign(n, d3{0, 0, 0});
    f.assign(n, d3{0, 0, 0});
}

void GpuLinkedCells::updateContainer() { gpu_check(komd_gpu_update_container(h_)); }

void GpuLinkedCells::syncHost() {
    const uint64_t n = getNumSites();
    std::vector<double> rr(3 * n), vv(3 * n), ff(3 * n);
    gpu_check(komd_gpu_download(h_, rr.data(), vv.data(), ff.data()));
    for (uint64_t i = 0; i < n; i++)
        for (int d = 0; d < 3; d++) {
            r[i][d] = rr[3 * i + d];
            v[i][d] = vv[3 * i + d];
            f[i][d] = ff[3 * i + d];
        }
}

void GpuTemperatureSensor::measure() {
    komd_observables o{};
    gpu_check(komd_gpu_measure(engine(), KOMD_MEASURE_TEMPERATURE, &o, nullptr, nullptr));
    temperature_ = o.temperature;
}

GpuLJSensor::GpuLJSensor() : PotentialSensor("LJ12_6") {
    const size_t b = Registry::instance->configuration()->sensor_lj_bins;
    u_.assign(b, 0.0); f_.assign(b, 0.0); cu_.assign(b, 0.0); cf_.assign(b, 0.0);
    hist_.assign(4 * b, 0.0);
}

void GpuLJSensor::measure() {
    komd_observables o{};
    gpu_check(komd_gpu_measure(engine(), KOMD_MEASURE_ENERGY | KOMD_MEASURE_LJ_HIST, &o, nullptr, hist_.data()));
    potential_ = o.u_lj;
    const size_t b = u_.size();
    for (size_t k = 0; k < b; k++) {   // histograms accumulate over measures (Potential_Sensor::measure)
        u_[k] += hist_[k];
        f_[k] += hist_[b + k];
        cu_[k] += hist_[2 * b + k];
        cf_[k] += hist_[3 * b + k];
    }
    pot_hist_.push_back(potential_);
}

void GpuLJSensor::write(uint64_t simstep) {
    {   // Potential_Sensor::write (Potential_Sensor.cpp:31-49)
        std::stringstream name;
        name << "pot_" << this->name() << "_" << simstep << ".txt";
        std::ofstream file(name.str());
        if (!file.is_open()) { std::cerr << "Could not write file: " << name.str() << std::endl; return; }
        double rr = 0;
        const double width = 3.0 * Registry::instance->configuration()->max_sigma / (double)u_.size();
        for (size_t k = 0; k < u_.size(); k++) {
            file << rr << "\t\t" << f_[k] / cf_[k] << "\t\t" << u_[k] / cu_[k] << "\n";
            rr += width;
        }
    }
    std::stringstream name;
    name << "pot_history_" << this->name() << "_" << simstep << ".txt";
    std::ofstream file(name.str());
    if (!file.is_open()) { std::cerr << "Could not write file: " << name.str() << std::endl; return; }
    for (double p : pot_hist_) file << p << " ";
}

GpuRDFSensor::GpuRDFSensor() : Sensor("RDF") {
    bins_.assign((size_t)komd_gpu_rdf_bins(engine()), 0.0);
}

void GpuRDFSensor::measure() {
    komd_observables o{};
    std::vector<double> b(bins_.size());
    gpu_check(komd_gpu_measure(engine(), KOMD_MEASURE_RDF, &o, b.data(), nullptr));
    for (size_t k = 0; k < b.size(); k++) bins_[k] += b[k];
    samples_++;
}

void GpuRDFSensor::write(uint64_t simstep) {
    // RDFSensor::write (RDFSensor.cpp:37-60): g(r) from the running mean of the bins
    std::stringstream name;
    name << "rdf_" << simstep << ".txt";
    std::ofstream file(name.str());
    if (!file.is_open()) { std::cerr << "Could not write file: " << name.str() << std::endl; return; }
    const auto cfg = Registry::instance->configuration();
    const double dr = cfg->sensor_rdf_dr;
    const double v_total = volume();
    const double n = (double)Registry::instance->moleculeContainer()->getNumMolecules();
    const double n_total = n * (n - 1);
    double rr = dr / 2.0;
    const double half = rr;
    for (size_t k = 0; k < bins_.size(); k++) {
        const double n_bin = bins_[k] / (double)samples_;
        const double v_bin = 4.0 / 3.0 * M_PI * (std::pow(rr + half, 3) - std::pow(rr - half, 3));
        const double g = (n_bin * v_total) / (v_bin * n_total);
        file << rr << "\t" << g << "\t" << n_bin << "\t" << v_bin << "\t" << n_total << "\t" << v_total << "\t"
             << (n_bin * v_total) << "\t" << (v_bin * n_total) << "\n";
        rr += dr;
    }
}

void GpuPressureSensor::measure() {
    komd_observables o{};
    gpu_check(komd_gpu_measure(engine(), KOMD_MEASURE_PRESSURE, &o, nullptr, nullptr));
    for (int k = 0; k < 6; k++) p_[k] = o.pressure[k];
}

void GpuPressureSensor::write(uint64_t simstep) {
    // PressureSensor::write (PressureSensor.cpp:35-70): tensor / V in Pa with
    // factor = Da->kg / (ps->s^2 * A->m), which SciValue evaluates as the
    // normalised mantissa 1.66053906892 times 10^7
    std::stringstream name;
    name << "pressures_" << simstep << ".txt";
    std::ofstream file(name.str());
    if (!file.is_open()) { std::cerr << "Could not write file: " << name.str() << std::endl; return; }
    const double factor = 1.66053906892 * 1e7;
    const double vol = volume();
    int next = 1, count = 0;
    for (int k = 0; k < 6; k++) {
        file << p_[k] / vol * factor;
        if (++count == next) {
            count = 0;
            next++;
            file << std::endl;
        } else {
            file << " ";
        }
    }
}

void GpuViscositySensor::measure() {
    komd_observables o{};
    gpu_check(komd_gpu_measure(engine(), KOMD_MEASURE_PRESSURE, &o, nullptr, nullptr));
    const double vol = volume();
    for (int k = 0; k < 6; k++) series_[k].push_back(o.pressure[k] / vol);   // TensorEvaluator::eval
}

double GpuViscositySensor::integrate(const std::vector<std::vector<double>> &series, const int *dims, int ndims,
                                     double dt, bool origin_free) {
    // TensorEvaluator::integrate (ViscositySensor.cpp:118-149): per component the
    // autocorrelation c(k) = mean over origins of (p(t) - s)(p(t + k) - s), with
    // s the mean of p when origin_free, then (c(0) + c(n-1) + sum of the inner
    // c(k)) * dt / 2, and the mean over the components
    double sum = 0.0;
    for (int q = 0; q < ndims; q++) {
        const std::vector<double> &p = series[dims[q]];
        const int n = (int)p.size();
        if (n == 0) continue;
        double shift = 0.0;
        if (origin_free) {
            for (double x : p) shift += x;
            shift /= n;
        }
        std::vector<double> c(n, 0.0);
        for (int k = 0; k < n; k++) {
            double t = 0.0;
            for (int o = 0; o < n - k; o++) t += (p[o] - shift) * (p[o + k] - shift);
            c[k] = t / (n - k);
        }
        double integral = c[0] + c[n - 1];
        for (int k = 1; k < n - 1; k++) integral += c[k];
        sum += integral * (dt / 2.0);
    }
    return sum / ndims;
}

void GpuViscositySensor::write(uint64_t simstep) {
    // ViscositySensor::write (ViscositySensor.cpp:37-89): factor =
    // (Da_kg^2 * A_m / ps_s^3) * (V / (kB * T)) in SciValue arithmetic
    const auto cfg = Registry::instance->configuration();
    const Sci da(1.66053906892, -27), a_m(1.0, -10), ps_s(1.0, -12), kB(1.380649, -23);
    const Sci conv = (da * da * a_m) / (ps_s * ps_s * ps_s);
    const double V = volume();
    const double kBT = (kB * cfg->temperature).value();
    const double factor = (conv * (V / kBT)).value();
    static const int bulk[3] = {0, 2, 5}, shear[3] = {1, 3, 4};   // XX YY ZZ, XY XZ YZ
    std::stringstream name;
    name << "viscosity_" << simstep << ".txt";
    std::ofstream file(name.str());
    if (!file.is_open()) { std::cerr << "Could not write file: " << name.str() << std::endl; return; }
    file << "b: " << integrate(series_, bulk, 3, cfg->delta_t, cfg->sensor_visc_no_orig) * factor << std::endl;
    file << "s: " << integrate(series_, shear, 3, cfg->delta_t, cfg->sensor_visc_no_orig) * factor << std::endl;
}

void GpuVelocityScaling::apply() {
    const double target = Registry::instance->configuration()->temperature;
    const double current = Registry::instance->temperature_sensor()->getTemperature();
    gpu_check(komd_gpu_scale_velocities(engine(), std::sqrt(target / current)));
}

}  // namespace komd
