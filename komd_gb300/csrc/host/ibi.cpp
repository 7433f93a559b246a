// ibi.cpp -- IBI and IBI_ReloadForce plugins (see ibi.h), restated from the
// reference's behaviour in plugins/IBI/{IBI,IBI_Math,RDF_Profiler,IBI_ReloadForce}.cpp.
#include "ibi.h"

#include <algorithm>
#include <cmath>
#include <fstream>
#include <iostream>
#include <sstream>
#include <stdexcept>

#include "gpu_adapters.h"

namespace komd {

// ---------------------------------------------------------------------------
// FunctionPL (IBI_Math.cpp:21-76)
// ---------------------------------------------------------------------------
void FunctionPL::derivative(FunctionPL &t) const {
    const size_t n = y.size();
    t.x = x;
    t.y.assign(n, 0.0);
    if (n < 2) return;
    t.y[0] = (y[1] - y[0]) / (x[1] - x[0]);
    t.y[n - 1] = (y[n - 1] - y[n - 2]) / (x[n - 1] - x[n - 2]);
    for (size_t k = 1; k + 1 < n; k++) t.y[k] = (y[k + 1] - y[k - 1]) / (x[k + 1] - x[k - 1]);
}

FunctionPL &FunctionPL::operator*=(double v) {
    for (double &q : y) q *= v;
    return *this;
}

void FunctionPL::read(const std::string &path) {
    std::ifstream in(path);
    if (!in) throw std::runtime_error("Failed to open file: " + path);
    std::vector<double> xs, ys;
    double a, b;
    while (in >> a >> b) {
        xs.push_back(a);
        ys.push_back(b);
    }
    x = std::move(xs);
    y = std::move(ys);
}

void FunctionPL::write(const std::string &path) const {
    std::ofstream out(path);
    if (!out) throw std::runtime_error("Failed to open file: " + path);
    for (size_t k = 0; k < x.size(); k++) {
        if (k) out << "\n";
        out << x[k] << "\t" << y[k];
    }
}

// ---------------------------------------------------------------------------
// RDF_Profiler (RDF_Profiler.cpp:8-77) over the engine's pair histogram
// ---------------------------------------------------------------------------
GpuRDFProfiler::GpuRDFProfiler() {
    const auto c = Registry::instance->configuration();
    const size_t nb = c->IBI_bins;
    if (nb == 0) throw std::runtime_error("IBI_bins must be > 0");
    max_r_ = c->cutoff;
    dr_ = max_r_ / (double)nb;
    bins_.assign(nb, 0.0);
    nodes_.resize(nb);
    for (size_t k = 0; k < nb; k++) nodes_[k] = ((double)k + 0.5) * dr_;
}

void GpuRDFProfiler::measure() {
    gpu_check(komd_gpu_rdf_profile(engine(), max_r_, (int32_t)bins_.size(), bins_.data()));
    samples_ += 1.0;
}

void GpuRDFProfiler::reset() {
    std::fill(bins_.begin(), bins_.end(), 0.0);
    samples_ = 0.0;
}

void GpuRDFProfiler::getRDF(std::vector<double> &buffer) const {
    const auto c = Registry::instance->configuration();
    const double N = (double)Registry::instance->moleculeContainer()->getNumMolecules();
    const double V = (c->domainHigh[0] - c->domainLow[0]) * (c->domainHigh[1] - c->domainLow[1]) *
                     (c->domainHigh[2] - c->domainLow[2]);
    buffer.resize(bins_.size());
    for (size_t k = 0; k < bins_.size(); k++) {
        const double lo = (double)k * dr_, hi = (double)(k + 1) * dr_;
        const double shell = (4.0 / 3.0) * M_PI * (hi * hi * hi - lo * lo * lo);
        const double ideal = N * (N - 1.0) * shell / V;
        double g = bins_[k];
        g /= samples_;
        g /= ideal;
        buffer[k] = g;
    }
}

// ---------------------------------------------------------------------------
// the functor swap
// ---------------------------------------------------------------------------
void use_tabulated_force(const FunctionPL &force) {
    komd_gpu *h = engine();
    gpu_check(komd_gpu_set_terms(h, KOMD_TERM_TABULATED));
    gpu_check(komd_gpu_set_pair_table(h, (int32_t)force.x.size(), force.x.data(), force.y.data(), force.lower,
                                      force.upper));
    Registry &R = *Registry::instance;
    R.forceFunctors().clear();
    R.forceFunctors().push_back(std::make_shared<GpuForces>());
    R.forceFunctors3b().clear();
}

namespace {
// linear continuation of y below index k0 with the slope of (k0, k0 + 1)
void continue_below(std::vector<double> &y, int k0) {
    if (k0 < 0) return;
    const double dy = (size_t)k0 + 1 < y.size() ? y[k0 + 1] - y[k0] : 0.0;
    double v = y[k0];
    for (int k = k0; k >= 0; k--) {
        y[k] = v;
        v -= dy;
    }
}
}  // namespace

// ---------------------------------------------------------------------------
// IBI (IBI.cpp)
// ---------------------------------------------------------------------------
GpuIBI::GpuIBI() : Plugin("IBI") {
    const auto c = Registry::instance->configuration();
    const size_t nb = c->IBI_bins;
    reference_rdf_ = FunctionPL(nb, 0.0, 1.0);
    reference_potential_ = FunctionPL(nb, 1e+6, 0.0);
    update_function_ = FunctionPL(nb, 0.0, 0.0);
    update_function_.x = profiler_.getRNodes();
    alpha_ = c->IBI_alpha;
    T_ = c->temperature;
    steps_equil_ = c->IBI_steps_equil;
    steps_measure_ = c->IBI_steps_measure;
    conv_.init(c->IBI_conv_threshold, c->IBI_conv_mode, c->IBI_conv_stop, c->IBI_conv_window);
}

std::string GpuIBI::createFilepath(const std::string &prefix) const {
    std::stringstream p;
    p << prefix << "_" << iteration_ << ".txt";
    return p.str();
}

void GpuIBI::post_forces() {
    current_steps_++;
    switch (phase_) {
    case FIRST_INIT: {
        if (current_steps_ < steps_measure_) { profiler_.measure(); break; }
        phase_ = EQUILIBRATE;
        current_steps_ = 0;
        iteration_ = 0;
        profiler_.getRDF(reference_rdf_.y);
        reference_rdf_.x = profiler_.getRNodes();
        reference_rdf_.write(createFilepath("rdf"));
        profiler_.reset();
        initializePotentialValues();
        potential_ = reference_potential_;
        derivativeOfPotential();
        std::cout << "[IBI] Transitioning from first initialization to equilibration with PMF" << std::endl;
        break;
    }
    case EQUILIBRATE: {
        if (current_steps_ < steps_equil_) break;
        phase_ = MEASURE;
        current_steps_ = 0;
        std::cout << "[IBI] Transitioning from equilibration to measurement" << std::endl;
        break;
    }
    case MEASURE: {
        if (current_steps_ < steps_measure_) { profiler_.measure(); break; }
        phase_ = EQUILIBRATE;
        current_steps_ = 0;
        addPotentialCorrection();
        iteration_++;
        potential_.write(createFilepath("pot"));
        derivativeOfPotential();
        writeRDF();
        profiler_.getRDF(update_function_.y);
        const auto c = conv_(reference_rdf_, update_function_.y);
        std::cout << "[IBI] Convergence: target_reached=" << c.first << " value=" << c.second << std::endl;
        if (conv_.shouldStop()) {
            std::cout << "[IBI] Convergence: stopping criterion reached. Stopping now." << std::endl;
            Registry::instance->simulation()->stop();
            break;
        }
        std::cout << "[IBI] Transitioning from measurement to equilibration" << std::endl;
        profiler_.reset();
        break;
    }
    }
}

void GpuIBI::finalize() {
    // the reference dereferences its tabulated functor here even when the
    // first RDF was never completed; nothing is written in that case
    if (have_functor_) potential_.write("final_pot.txt");
    std::cout << "[IBI] Convergence steps: " << conv_.values() << std::endl;
}

void GpuIBI::initializePotentialValues() {
    reference_potential_.x = reference_rdf_.x;
    reference_potential_.y = reference_rdf_.y;
    auto &u = reference_potential_.y;
    for (double &q : u) q = -T_ * std::log(q);
    int k0 = -1;
    for (size_t k = 0; k < u.size(); k++)
        if (std::isfinite(u[k])) { k0 = (int)k; break; }
    continue_below(u, k0);
    reference_potential_.write("pot_0.txt");
}

void GpuIBI::addPotentialCorrection() {
    profiler_.getRDF(update_function_.y);
    auto &pot = potential_.y;
    auto &up = update_function_.y;
    for (size_t k = 0; k < pot.size(); k++) {
        const double d = alpha_ * T_ * std::log(up[k] / reference_rdf_.y[k]);
        if (std::isfinite(d)) {
            pot[k] += d;
            up[k] = d;
        } else {
            up[k] = 0;
        }
    }
    update_function_.write(createFilepath("update"));
    int k0 = -1;
    for (size_t k = 0; k < reference_rdf_.y.size(); k++)
        if (reference_rdf_.y[k] != 0.0) { k0 = (int)k; break; }
    continue_below(pot, k0);
}

void GpuIBI::derivativeOfPotential() {
    potential_.derivative(force_);
    force_.lower = 1e+6;
    force_.upper = 0.0;
    force_ *= -1;
    force_.write(createFilepath("force"));
    use_tabulated_force(force_);
    have_functor_ = true;
}

void GpuIBI::writeRDF() {
    profiler_.getRDF(update_function_.y);
    update_function_.write(createFilepath("rdf"));
}

// ---------------------------------------------------------------------------
// IBI::Convergence (IBI.cpp:200-281)
// ---------------------------------------------------------------------------
void GpuIBI::Convergence::init(double th, const std::string &m, const std::string &s, int w) {
    mode = m == "l2" ? L2 : INTEGRAL;
    stopping = s == "worse" ? ON_WORSE : WINDOW;
    threshold = th;
    window = w;
}

std::pair<bool, double> GpuIBI::Convergence::operator()(const FunctionPL &ref, const std::vector<double> &gi) {
    const auto &g0 = ref.y;
    double v;
    if (mode == L2) {
        v = 0.0;
        for (size_t k = 0; k < g0.size(); k++) {
            const double d = g0[k] - gi[k];
            v += d * d;
        }
    } else {
        const auto &x = ref.x;
        double diff = 0.0, sum = 0.0;
        for (size_t k = 0; k + 1 < x.size(); k++) {
            const double dx = x[k + 1] - x[k];
            diff += dx * (std::abs(gi[k + 1] - g0[k + 1]) + std::abs(gi[k] - g0[k])) / 2.0;
        }
        for (size_t k = 0; k + 1 < x.size(); k++) {
            const double dx = x[k + 1] - x[k];
            sum += dx * (std::abs(gi[k + 1] + g0[k + 1]) + std::abs(gi[k] + g0[k])) / 2.0;
        }
        if (sum == 0) sum = 1e-15;
        v = 1.0 - diff / sum;
    }
    conv_values.push_back(v);
    return {v <= threshold, v};
}

bool GpuIBI::Convergence::shouldStop() const {
    const size_t n = conv_values.size();
    if (stopping == ON_WORSE) {
        if (n < 2) return false;
        const double prev = conv_values[n - 2], last = conv_values[n - 1];
        if (mode == INTEGRAL) return !(prev < threshold) && !(prev <= last);
        return !(prev > threshold) && !(prev >= last);
    }
    if (n < (size_t)window) return false;
    bool all = true;
    for (int k = 0; k < window; k++) {
        const double v = conv_values[n - 1 - k];
        all &= mode == INTEGRAL ? v >= threshold : v <= threshold;
    }
    return all;
}

std::string GpuIBI::Convergence::values() const {
    std::stringstream s;
    for (double v : conv_values) s << v << " ";
    return s.str();
}

// ---------------------------------------------------------------------------
// IBI_ReloadForce (IBI_ReloadForce.cpp:11-58)
// ---------------------------------------------------------------------------
GpuIBIReload::GpuIBIReload() : Plugin("IBI-Reload") {
    const auto c = Registry::instance->configuration();
    if (c->IBI_enable) throw std::runtime_error("Cannot have IBI and IBI_Reload at the same time!");
    FunctionPL force(c->IBI_bins, 1e+6, 0.0), pot(c->IBI_bins, 1e+6, 0.0);
    force.read(c->IBI_reload_fpath);
    pot.read(c->IBI_reload_ppath);
    const double vol = (c->IBI_exclusion_high[0] - c->IBI_exclusion_low[0]) *
                       (c->IBI_exclusion_high[1] - c->IBI_exclusion_low[1]) *
                       (c->IBI_exclusion_high[2] - c->IBI_exclusion_low[2]);
    if (vol != 0)
        throw std::runtime_error("IBI_reload with an exclusion zone (ExclusionLJ / ExclusionATM) is not available");
    use_tabulated_force(force);
}

}  // namespace komd
