// ibi.h -- KoMD's Iterative Boltzmann Inversion plugins on the engine.
//
// plugins/IBI/IBI.{h,cpp}: an RDF g0(r) is sampled with the configured
// potentials, then the force functors are replaced by a tabulated pair force
// F = -dU/dr with U0 = -T ln g0, and U is corrected from the sampled RDF of
// each iteration (U += alpha T ln(g_i / g0)) until the convergence criterion
// stops the run.  plugins/IBI/IBI_ReloadForce.cpp: the tabulated force of a
// finished run read back from its files.
//
// The sampling (RDF_Profiler) and the tabulated force (IBI_ForceFunctor) run
// in the engine (komd_gpu_rdf_profile, KOMD_TERM_TABULATED through
// komd_gpu_set_terms / komd_gpu_set_pair_table); the function algebra, the
// files and the iteration state machine are host work, as in the reference.
#pragma once

#include <string>
#include <utility>
#include <vector>

#include "komd_host.h"

namespace komd {

// FunctionPL (plugins/IBI/IBI_Math.{h,cpp}): y(x) on ascending nodes, linear in
// between, lower/upper defaults outside
class FunctionPL {
public:
    explicit FunctionPL(size_t n = 0, double def_low = 0.0, double def_high = 0.0)
        : x(n, 0.0), y(n, 0.0), lower(def_low), upper(def_high) {}
    // forward difference at the first node, backward at the last, central between
    void derivative(FunctionPL &target) const;
    FunctionPL &operator*=(double v);   // y only; the defaults are kept
    // "x y" pairs, whitespace separated; resizes to the file's length; throws if unreadable
    void read(const std::string &path);
    // "x\ty" lines, default stream format, no trailing newline; throws if unwritable
    void write(const std::string &path) const;
    std::vector<double> x, y;
    double lower, upper;
};

// RDF_Profiler (plugins/IBI/RDF_Profiler.cpp): ordered COM pairs up to the
// cutoff in IBI_bins bins, accumulated over measure() calls
class GpuRDFProfiler {
public:
    GpuRDFProfiler();
    void measure();
    void reset();
    // normalised RDF (counts / samples / (N (N-1) V_shell / V)), one value per node
    void getRDF(std::vector<double> &buffer) const;
    const std::vector<double> &getRNodes() const { return nodes_; }
private:
    double max_r_, dr_;
    std::vector<double> bins_, nodes_;
    double samples_ = 0.0;
};

class GpuIBI : public Plugin {
public:
    GpuIBI();
    void post_forces() override;
    void finalize() override;

    // IBI::Convergence: "integral" (1 - int|g_i - g0| / int|g_i + g0|, trapezoid)
    // or "l2" (sum (g0 - g_i)^2); stopping "worse" or "window"
    struct Convergence {
        void init(double threshold, const std::string &mode, const std::string &stop, int window);
        std::pair<bool, double> operator()(const FunctionPL &ref, const std::vector<double> &g_i);
        bool shouldStop() const;
        std::string values() const;
        std::vector<double> conv_values;
        enum { INTEGRAL, L2 } mode = L2;
        enum { ON_WORSE, WINDOW } stopping = ON_WORSE;
        double threshold = 0.0;
        int window = 10;
    };
    const Convergence &convergence() const { return conv_; }

private:
    void initializePotentialValues();   // U0 = -T ln g0, linear continuation below r_min
    void addPotentialCorrection();      // U += alpha T ln(g_i / g0)
    void derivativeOfPotential();       // F = -dU/dr into the engine's table
    void writeRDF();
    std::string createFilepath(const std::string &prefix) const;

    FunctionPL reference_rdf_, reference_potential_, update_function_;
    FunctionPL potential_, force_;      // the tabulated functor's functions
    bool have_functor_ = false;
    GpuRDFProfiler profiler_;
    double alpha_, T_;
    int iteration_ = 0, steps_equil_, steps_measure_, current_steps_ = 0;
    enum { FIRST_INIT, EQUILIBRATE, MEASURE } phase_ = FIRST_INIT;
    Convergence conv_;
};

// IBI_ReloadForce: the tabulated force (and potential) of a finished run as the
// only pair functor; the exclusion-zone variant (ExclusionLJ / ExclusionATM
// inside a box) is not available and is reported
class GpuIBIReload : public Plugin {
public:
    GpuIBIReload();
};

// the Registry's functors replaced by the engine's tabulated pair term only
// (IBI.cpp:50-54): LJ / ATM2B, FENE, Limit and ATM are dropped
void use_tabulated_force(const FunctionPL &force);

}  // namespace komd
