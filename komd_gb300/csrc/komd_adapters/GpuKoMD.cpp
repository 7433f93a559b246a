// GpuKoMD.cpp -- see GpuKoMD.h.
#include "GpuKoMD.h"

#include <cmath>
#include <vector>

#include "Registry.h"
#include "util/constants.h"

namespace komd_gb300 {

komd_config engine_config() {
    auto c = Registry::instance->configuration();
    komd_config k{};
    for (int d = 0; d < 3; d++) {
        k.domain_low[d] = c->domainLow[d];
        k.domain_high[d] = c->domainHigh[d];
    }
    k.cell_size = c->cell_size;
    k.cutoff = c->cutoff;
    k.cutoff_3b = c->cutoff;                                   // one cutoff, as the reference
    k.nu = c->energy_3b * 1e+9 * Constants::conv_J_Ei;         // ATM.cpp:11-14
    k.delta_t = c->delta_t;
    k.stiffness = c->stiffness_factor;
    k.limit = c->limit_factor;
    k.terms = KOMD_TERM_LJ | KOMD_TERM_FENE | KOMD_TERM_LIMIT | (c->enable_3b ? KOMD_TERM_ATM : 0u);
    k.precision = KOMD_FP32;
    k.atm_sign = KOMD_ATM_SIGN_REFERENCE;
    k.atm_enum = KOMD_ATM_ENUM_COMPAT;
    k.virial_mode = KOMD_VIRIAL_COMPAT;
    k.atm_direct = c->enable_3b_direct ? 1 : 0;
    k.max_sigma = c->max_sigma;
    k.lj_bins = (int32_t)c->sensor_lj_bins;
    k.rdf_max = c->sensor_rdf_max;
    k.rdf_dr = c->sensor_rdf_dr;
    k.temperature_target = c->temperature;
    return k;
}

static komd_gpu *engine() {
    auto c = std::dynamic_pointer_cast<GpuLinkedCells>(Registry::instance->moleculeContainer());
    if (!c || !c->handle()) throw std::runtime_error("the GPU adapters need GpuLinkedCells as the container, initialised");
    return c->handle();
}

}  // namespace komd_gb300

using komd_gb300::check;

GpuLinkedCells::~GpuLinkedCells() {
    if (h_) komd_gpu_destroy(h_);
}

void GpuLinkedCells::init() {
    // the SOA as LinkedCells::init fills it (LinkedCells.cpp:47-51): molecules
    // (from the checkpoint) -> site arrays
    uint64_t num_sites = 0;
    for (auto &molecule : p_molecules) num_sites += molecule.getSites().size();
    p_soa.createBuffers(num_sites);
    constructSOAs();
    const komd_config k = komd_gb300::engine_config();
    check(komd_gpu_create(&k, 0, &h_));
    const uint64_t n = p_soa.size();
    std::vector<double> r(3 * n), v(3 * n), m(n), eps(n), sig(n);
    std::vector<uint64_t> id(n);
    for (uint64_t i = 0; i < n; i++) {
        for (int d = 0; d < 3; d++) {
            r[3 * i + d] = p_soa.r()[i][d];
            v[3 * i + d] = p_soa.v()[i][d];
        }
        m[i] = p_soa.mass()[i];
        eps[i] = p_soa.epsilon()[i];
        sig[i] = p_soa.sigma()[i];
        id[i] = p_soa.id()[i];
    }
    check(komd_gpu_upload_sites(h_, (int64_t)n, r.data(), v.data(), m.data(), eps.data(), sig.data(), id.data()));
}

void GpuLinkedCells::updateContainer() { check(komd_gpu_update_container(h_)); }

std::unique_ptr<MoleculeContainer::CellIterator> GpuLinkedCells::iteratorCell() {
    throw std::logic_error("GpuLinkedCells: cell lists live on the device (komd_gpu_get_cells)");
}
std::unique_ptr<MoleculeContainer::CellPairIterator> GpuLinkedCells::iteratorC08() {
    throw std::logic_error("GpuLinkedCells: the pair sweep runs on the device (komd_gpu_forces)");
}
std::unique_ptr<MoleculeContainer::CellTripletIterator> GpuLinkedCells::iteratorTripletC08() {
    throw std::logic_error("GpuLinkedCells: the triplet sweep runs on the device (komd_gpu_forces)");
}

void GpuLinkedCells::syncSOA() {
    const uint64_t n = p_soa.size();
    std::vector<double> r(3 * n), v(3 * n), f(3 * n);
    check(komd_gpu_download(h_, r.data(), v.data(), f.data()));
    for (uint64_t i = 0; i < n; i++)
        for (int d = 0; d < 3; d++) {
            p_soa.r()[i][d] = r[3 * i + d];
            p_soa.v()[i][d] = v[3 * i + d];
            p_soa.f()[i][d] = f[3 * i + d];
        }
}

void GpuForces::handlePairList(PairList &) { check(komd_gpu_forces(komd_gb300::engine())); }

void GpuIntegrator::integrate0() { check(komd_gpu_integrate0(komd_gb300::engine())); }
void GpuIntegrator::integrate1() { check(komd_gpu_integrate1(komd_gb300::engine())); }

void GpuTemperatureSensor::measure() {
    std::dynamic_pointer_cast<GpuLinkedCells>(Registry::instance->moleculeContainer())->syncSOA();
    TemperatureSensor::measure();
}

void GpuVelocityScaling::apply() {
    const double t = Registry::instance->temperature_sensor()->getTemperature();
    const double beta = std::sqrt(Registry::instance->configuration()->temperature / t);
    check(komd_gpu_scale_velocities(komd_gb300::engine(), beta));
}
