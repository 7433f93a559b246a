// host_core.cpp -- Registry, FileInput, CheckpointIO and Simulation::run of
// the host layer (komd_host.h), restated from the reference's behaviour.
#include <cmath>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <random>
#include <sstream>
#include <stdexcept>

#include "komd_host.h"

namespace komd {

std::unique_ptr<Registry> Registry::instance;

d3 Molecule::centerOfMass() const {
    // Molecule::getCenterOfMass: sum m r / sum m
    d3 c{0, 0, 0};
    double M = 0;
    for (size_t q = 0; q < r.size(); q++) {
        for (int d = 0; d < 3; d++) c[d] += r[q][d] * mass[q];
        M += mass[q];
    }
    for (int d = 0; d < 3; d++) c[d] /= M;
    return c;
}

void MoleculeContainer::addMolecule(const Molecule &m) {
    // MoleculeContainer::addMolecule (MoleculeContainer.cpp:13-22)
    const auto cfg = Registry::instance->configuration();
    const d3 p = m.centerOfMass();
    for (int d = 0; d < 3; d++)
        if (!(p[d] >= cfg->domainLow[d] && p[d] <= cfg->domainHigh[d]))
            throw std::runtime_error("Inserting Molecule at invalid position.");
    molecules_.push_back(m);
}

uint64_t MoleculeContainer::getNumSites() const {
    uint64_t n = 0;
    for (const Molecule &m : molecules_) n += m.r.size();
    return n;
}

// ---------------------------------------------------------------------------
// FileInput::readFile (IO/FileInput.cpp:13-121)
// ---------------------------------------------------------------------------
namespace {
template <typename T>
void rd(std::istream &in, T &x) { in >> x; }
void rd3(std::istream &in, d3 &x) { in >> x[0] >> x[1] >> x[2]; }
void rdb(std::istream &in, bool &x) {
    int v = 0;
    in >> v;
    x = v != 0;
}
int mode(const std::string &v, const char *a, int va, const char *b, int vb, bool &ok) {
    if (v == a) return va;
    if (v == b) return vb;
    ok = false;
    return va;
}
}  // namespace

bool FileInput::readFile(const std::string &filename) {
    std::ifstream file(filename);
    if (!file.is_open()) {
        std::cerr << "Could not open the file: " << filename << std::endl;
        return false;
    }
    Configuration &c = *Registry::instance->configuration();
    auto &components = Registry::instance->components();
    std::string var;
    while (file >> var) {
        if (var[0] == '#') {
            std::string rest;
            std::getline(file, rest);
            continue;
        }
        if (var == "temperature") rd(file, c.temperature);
        else if (var == "delta_t") rd(file, c.delta_t);
        else if (var == "cutoff") rd(file, c.cutoff);
        else if (var == "cell_size") rd(file, c.cell_size);
        else if (var == "density") rd(file, c.density);
        else if (var == "stiffness") rd(file, c.stiffness_factor);
        else if (var == "limit") rd(file, c.limit_factor);
        else if (var == "energy_3b") rd(file, c.energy_3b);
        else if (var == "pair_steps") rd(file, c.pair_steps);
        else if (var == "triple_steps") rd(file, c.triple_steps);
        else if (var == "domain_low") rd3(file, c.domainLow);
        else if (var == "domain_high") rd3(file, c.domainHigh);
        else if (var == "timesteps") rd(file, c.timesteps);
        else if (var == "write_freq") rd(file, c.write_freq);
        else if (var == "enable_3b_approx") rdb(file, c.enable_3b_approx);
        else if (var == "enable_3b") rdb(file, c.enable_3b);
        else if (var == "enable_3b_direct") rdb(file, c.enable_3b_direct);
        else if (var == "enable_sensor_lj") rdb(file, c.enable_sensor_lj);
        else if (var == "enable_sensor_fene") rdb(file, c.enable_sensor_fene);
        else if (var == "enable_sensor_rdf") rdb(file, c.enable_sensor_rdf);
        else if (var == "enable_sensor_disp") rdb(file, c.enable_sensor_disp);
        else if (var == "enable_sensor_pres") rdb(file, c.enable_sensor_pres);
        else if (var == "enable_sensor_visc") rdb(file, c.enable_sensor_visc);
        else if (var == "sensor_lj_bins") rd(file, c.sensor_lj_bins);
        else if (var == "sensor_fene_bins") rd(file, c.sensor_fene_bins);
        else if (var == "sensor_rdf_max") rd(file, c.sensor_rdf_max);
        else if (var == "sensor_rdf_dr") rd(file, c.sensor_rdf_dr);
        else if (var == "sensor_visc_window") rd(file, c.sensor_visc_window);
        else if (var == "sensor_visc_no_orig") rdb(file, c.sensor_visc_no_orig);
        else if (var == "store_checkpoint") rdb(file, c.storeCheckpoint);
        else if (var == "ADR_enable") rdb(file, c.ADR_enable);
        else if (var == "IBI_enable") rdb(file, c.IBI_enable);
        else if (var == "IBI_bins") rd(file, c.IBI_bins);
        else if (var == "IBI_alpha") rd(file, c.IBI_alpha);
        else if (var == "IBI_steps_equil") { double t = 0; file >> t; c.IBI_steps_equil = (int)t; }
        else if (var == "IBI_steps_measure") { double t = 0; file >> t; c.IBI_steps_measure = (int)t; }
        else if (var == "IBI_conv_threshold") rd(file, c.IBI_conv_threshold);
        else if (var == "IBI_conv_mode") rd(file, c.IBI_conv_mode);
        else if (var == "IBI_conv_stop") rd(file, c.IBI_conv_stop);
        else if (var == "IBI_conv_window") rd(file, c.IBI_conv_window);
        else if (var == "IBI_reload") rdb(file, c.IBI_reload_enable);
        else if (var == "IBI_reload_fpath") rd(file, c.IBI_reload_fpath);
        else if (var == "IBI_reload_ppath") rd(file, c.IBI_reload_ppath);
        else if (var == "IBI_exclusion_low") rd3(file, c.IBI_exclusion_low);
        else if (var == "IBI_exclusion_high") rd3(file, c.IBI_exclusion_high);
        else if (var == "enable_one_cell") rdb(file, c.enable_one_cell);
        else if (var == "ps_gen_region") {
            d3 b, e;
            int cid;
            file >> b[0] >> b[1] >> b[2] >> e[0] >> e[1] >> e[2] >> cid;
            if (cid < 0) { std::cerr << "negative component id not allowed" << std::endl; return false; }
            c.phasespace_gen_regions.emplace_back(b, e, (uint32_t)cid);
        } else if (var == "checkpoint_file") {
            std::string path;
            d3 off;
            file >> path >> off[0] >> off[1] >> off[2];
            c.checkpoint_files.emplace_back(path, off);
        } else if (var == "COMP") {
            int cid;
            double eps, sig, mass;
            d3 r;
            file >> cid >> eps >> sig >> mass >> r[0] >> r[1] >> r[2];
            if (cid < 0) { std::cerr << "negative component id not allowed" << std::endl; return false; }
            if ((int)components.size() <= cid) components.resize(cid + 1);
            components[cid].addSite(eps, sig, mass, r);
            if (eps > c.max_epsilon) c.max_epsilon = eps;
            if (sig > c.max_sigma) c.max_sigma = sig;
        } else if (var.rfind("gpu_", 0) == 0) {
            std::string v;
            file >> v;
            bool ok = true;
            if (var == "gpu_precision") c.gpu_precision = mode(v, "fp32", KOMD_FP32, "fp64", KOMD_FP64, ok);
            else if (var == "gpu_atm_sign")
                c.gpu_atm_sign = mode(v, "reference", KOMD_ATM_SIGN_REFERENCE, "physical", KOMD_ATM_SIGN_PHYSICAL, ok);
            else if (var == "gpu_atm_enum")
                c.gpu_atm_enum = mode(v, "compat", KOMD_ATM_ENUM_COMPAT, "full", KOMD_ATM_ENUM_FULL, ok);
            else if (var == "gpu_virial")
                c.gpu_virial = mode(v, "compat", KOMD_VIRIAL_COMPAT, "correct", KOMD_VIRIAL_CORRECT, ok);
            else if (var == "gpu_atm2b") c.gpu_atm2b_physical = mode(v, "compat", 0, "physical", 1, ok) != 0;
            else if (var == "gpu_skin") c.gpu_skin = std::stod(v);
            else if (var == "gpu_device") c.gpu_device = std::stoi(v);
            else if (var == "gpu_vtk") c.gpu_vtk = std::stoi(v) != 0;
            else if (var == "gpu_switch_width") c.gpu_switch_width = std::stod(v);
            if (!ok) { std::cerr << "invalid value for " << var << ": " << v << std::endl; return false; }
        }
        // unknown tokens are skipped, as in the reference
    }
    if (components.empty()) { std::cerr << "no components defined" << std::endl; return false; }
    if (c.max_epsilon == std::numeric_limits<double>::min()) { std::cerr << "invalid epsilon specified" << std::endl; return false; }
    if (c.max_sigma == std::numeric_limits<double>::min()) { std::cerr << "invalid sigma specified" << std::endl; return false; }
    if (c.phasespace_gen_regions.empty() && c.checkpoint_files.empty()) {
        std::cerr << "No phasespace data specified" << std::endl;
        return false;
    }
    for (auto &reg : c.phasespace_gen_regions)
        if (std::get<2>(reg) >= components.size()) {
            std::cerr << "phasespace gen region uses unknown component" << std::endl;
            return false;
        }
    if (c.cell_size < c.cutoff) {
        std::cerr << "cell size must be larger or equal to cutoff radius" << std::endl;
        return false;
    }
    return true;
}

// ---------------------------------------------------------------------------
// CheckpointIO (IO/CheckpointIO.cpp)
// ---------------------------------------------------------------------------
void CheckpointIO::writeCheckpoint(uint64_t simstep) {
    auto container = Registry::instance->moleculeContainer();
    container->syncHost();
    std::stringstream name;
    name << "ckpt_" << simstep << ".ps";
    std::ofstream file(name.str());
    if (!file.is_open()) {
        std::cerr << "Could not write checkpoint file: " << name.str() << std::endl;
        return;
    }
    bool first = true;
    size_t i = 0;
    for (const Molecule &m : container->molecules())
        for (size_t q = 0; q < m.r.size(); q++, i++) {
            if (!first) file << "\n";
            first = false;
            const d3 &r = container->r[i], &v = container->v[i];
            file << m.id << "\t" << r[0] << " " << r[1] << " " << r[2] << "\t" << v[0] << " " << v[1] << " " << v[2]
                 << "\t" << m.mass[q] << " " << m.eps[q] << " " << m.sig[q];
        }
}

void VTKWriter::write(const std::string &filename, uint64_t iteration) {
    if (!Registry::instance->configuration()->gpu_vtk) return;
    auto container = Registry::instance->moleculeContainer();
    container->syncHost();
    std::stringstream name;
    name << filename << "_" << std::setfill('0') << std::setw(4) << iteration << ".vtu";
    std::ofstream file(name.str());
    if (!file.is_open()) {
        std::cerr << "Could not write VTK file: " << name.str() << std::endl;
        return;
    }
    const auto &mols = container->molecules();
    const uint64_t n = container->getNumSites();
    file << std::setprecision(std::numeric_limits<float>::max_digits10);
    auto array = [&](const char *type, const char *nm, int comps, auto &&emit) {
        file << "      <DataArray type=\"" << type << "\" Name=\"" << nm << "\" NumberOfComponents=\"" << comps
             << "\" format=\"ascii\">";
        emit();
        file << "</DataArray>\n";
    };
    auto sites3 = [&](const std::vector<d3> &a) {
        for (uint64_t i = 0; i < n; i++) file << (float)a[i][0] << " " << (float)a[i][1] << " " << (float)a[i][2] << " ";
    };
    file << "<?xml version=\"1.0\" encoding=\"UTF-8\"?>\n"
         << "<VTKFile type=\"UnstructuredGrid\" version=\"0.1\" byte_order=\"LittleEndian\">\n"
         << "  <UnstructuredGrid>\n"
         << "    <Piece NumberOfPoints=\"" << n << "\" NumberOfCells=\"0\">\n"
         << "    <PointData>\n";
    array("Float32", "mass", 1, [&]() {
        for (const Molecule &m : mols)
            for (double q : m.mass) file << (float)q << " ";
    });
    array("Float32", "velocity", 3, [&]() { sites3(container->v); });
    array("Float32", "force", 3, [&]() { sites3(container->f); });
    array("Int32", "id", 1, [&]() {
        for (const Molecule &m : mols)
            for (size_t q = 0; q < m.r.size(); q++) file << (int32_t)m.id << " ";
    });
    array("Int32", "cid", 1, [&]() {   // checkpoint-loaded molecules carry no component id
        for (uint64_t i = 0; i < n; i++) file << 0 << " ";
    });
    file << "    </PointData>\n    <CellData/>\n    <Points>\n";
    array("Float32", "points", 3, [&]() { sites3(container->r); });
    file << "    </Points>\n    <Cells>\n";
    array("Float32", "types", 0, [&]() {});
    file << "    </Cells>\n    </Piece>\n  </UnstructuredGrid>\n</VTKFile>\n";
}

bool CheckpointIO::loadCheckpoint() {
    auto cfg = Registry::instance->configuration();
    auto container = Registry::instance->moleculeContainer();
    for (const auto &[path, offset] : cfg->checkpoint_files) {
        std::ifstream file(path);
        if (!file.is_open()) {
            std::cerr << "Could not open checkpoint file: " << path << std::endl;
            return false;
        }
        // one site per line; consecutive lines with one id form a molecule.
        // A trailing newline ends the file like none (the reference re-reads
        // the last site in that case); partial lines are ignored.
        Molecule mol;
        next_molecule_id();   // the reference's loader default-constructs one molecule per file
        bool have = false;
        std::string line;
        while (std::getline(file, line)) {
            std::istringstream in(line);
            uint64_t id;
            d3 r, v;
            double m, e, s;
            if (!(in >> id >> r[0] >> r[1] >> r[2] >> v[0] >> v[1] >> v[2] >> m >> e >> s)) continue;
            if (have && id != mol.id) {
                container->addMolecule(mol);
                mol = Molecule();
                next_molecule_id();   // ... and one per further molecule (then sets the file's id)
            }
            mol.id = id;
            have = true;
            for (int d = 0; d < 3; d++) r[d] += offset[d];
            mol.addSite(e, s, m, r, v);
        }
        if (have) container->addMolecule(mol);
    }
    return true;
}

uint64_t next_molecule_id() {
    static uint64_t next = 1;   // id 0 went to the reference's Molecule::INVALID
    return next++;
}

namespace {
// the Euler rotation of the generator (PhasespaceGenerator.cpp:12-24), term by
// term in the reference's order, so that positions round alike
d3 euler_rotate(double a, double b, double g, const d3 &q) {
    const double ca = std::cos(a), sa = std::sin(a), cb = std::cos(b), sb = std::sin(b), cg = std::cos(g),
                 sg = std::sin(g);
    d3 out;
    out[0] = cb * cg * q[0] + (sa * sb * cg - ca * sg) * q[1] + (ca * sb * cg + sa * sg) * q[2];
    out[1] = cb * sg * q[0] + (sa * sb * sg + ca * cg) * q[1] + (ca * sb * sg - sa * cg) * q[2];
    out[2] = -sb * q[0] + sa * cb * q[1] + ca * cb * q[2];
    return out;
}

// one Maxwell-Boltzmann velocity for a molecule of mass m at temperature T (K)
// (PhasespaceGenerator.cpp:85-95): three standard normal draws, each call with
// a fresh distribution on the static engine seeded 42, times
// sqrt(T / m * kB / Da) (m/s) * 1e-2 (A/ps), the constants in SciValue arithmetic
d3 maxwell_boltzmann(double T, double m) {
    static std::default_random_engine rng(42);
    static const double kb_over_da = (Sci(1.380649, -23) / Sci(1.66053906892, -27)).value();
    double sd = std::sqrt((T / m) * kb_over_da);
    sd *= Sci(1.0, -2).value();
    std::normal_distribution<double> normal(0, 1);
    d3 v;
    v[0] = normal(rng);
    v[1] = normal(rng);
    v[2] = normal(rng);
    for (int d = 0; d < 3; d++) v[d] *= sd;
    return v;
}
}  // namespace

void PhasespaceGenerator::generate() {
    auto cfg = Registry::instance->configuration();
    auto container = Registry::instance->moleculeContainer();
    auto &components = Registry::instance->components();
    d3 size;
    for (int d = 0; d < 3; d++) size[d] = cfg->domainHigh[d] - cfg->domainLow[d];
    const double num = cfg->density * (size[0] * size[1] * size[2]);
    const double per_dim = std::pow(num, 1. / 3.);
    d3 spacing;
    for (int d = 0; d < 3; d++) spacing[d] = size[d] / per_dim;
    static std::default_random_engine rng(43);
    std::uniform_real_distribution<double> uniform(0, M_PI * 2);
    const double j_to_internal = Sci(6.022140754, 22).value();   // Constants::conv_J_Ei
    for (const auto &[begin, end, cid] : cfg->phasespace_gen_regions) {
        const Component &comp = components[cid];
        for (double z = begin[2] + 0.5; z < end[2]; z += spacing[2])
            for (double y = begin[1] + 0.5; y < end[1]; y += spacing[1])
                for (double x = begin[0] + 0.5; x < end[0]; x += spacing[0]) {
                    Molecule mol;
                    mol.id = next_molecule_id();
                    const double alpha = uniform(rng), beta = uniform(rng), gamma = uniform(rng);
                    double total_mass = 0;
                    for (const SiteDesc &site : comp.sites) total_mass += site.mass;
                    const d3 v = maxwell_boltzmann(cfg->temperature, total_mass);
                    for (const SiteDesc &site : comp.sites) {
                        const d3 q = euler_rotate(alpha, beta, gamma, site.r);
                        const d3 pos{x + q[0], y + q[1], z + q[2]};
                        mol.addSite(site.epsilon * j_to_internal, site.sigma, site.mass, pos, v);
                    }
                    container->addMolecule(mol);
                }
    }
}

// ---------------------------------------------------------------------------
// Simulation::run (Simulation.cpp:10-80)
// ---------------------------------------------------------------------------
void Simulation::run(bool fused) {
    Registry &R = *Registry::instance;
    auto config = R.configuration();
    auto container = R.moleculeContainer();
    auto temp = R.temperature_sensor();
    auto pot = R.potential_sensor();
    auto &plugins = R.plugins();

    for (auto &p : plugins) p->init();
    const double dt = config->delta_t;
    const uint64_t write_freq = config->write_freq;
    for (auto &p : plugins) p->pre_container_update();
    container->updateContainer();
    for (auto &p : plugins) p->post_container_update();
    VTKWriter::write("VTK_Output", 0);
    for (auto &f : R.forceFunctors()) (*f)();
    if (config->enable_3b)
        for (auto &f : R.forceFunctors3b()) (*f)();
    for (auto &p : plugins) p->post_forces();
    temp->measure();
    std::cout << "Initial temperature T=" << temp->getTemperature() << std::endl;
    if (pot) {
        pot->measure();
        std::cout << "Initial potential u=" << pot->getCurrentPotential() << std::endl;
    }
    for (auto &t : R.thermostats()) t->apply();
    for (auto &p : plugins) p->pre_main_loop();

    double t = 0;
    max_step_ = config->timesteps;
    if (fused) {
        // one graph-replayed chunk per write interval; the thermostat runs on the
        // device after every step; sensors are read at the write steps
        while (simstep_ < max_step_) {
            const uint64_t chunk = std::min<uint64_t>(write_freq - simstep_ % write_freq, max_step_ - simstep_);
            container->advance(chunk);
            simstep_ += chunk;
            t += dt * (double)chunk;
            for (auto &s : R.sensors()) s->measure();
            std::cout << "Simstep=" << simstep_ - 1 << " t=" << t - dt << " T=" << temp->getTemperature();
            if (pot) std::cout << " u=" << pot->getCurrentPotential();
            std::cout << std::endl;
            if (simstep_ % write_freq == 0) VTKWriter::write("VTK_Output", simstep_);
            if (simstep_ % write_freq == 0)
                for (auto &s : R.sensors()) s->write(simstep_);
        }
    } else {
        while (simstep_ < max_step_) {
            for (auto &p : plugins) p->begin_loop();
            for (auto &i : R.integrators()) i->integrate0();
            for (auto &p : plugins) p->pre_container_update();
            container->updateContainer();
            for (auto &p : plugins) p->post_container_update();
            for (auto &f : R.forceFunctors()) (*f)();
            if (config->enable_3b)
                for (auto &f : R.forceFunctors3b()) (*f)();
            for (auto &p : plugins) p->post_forces();
            for (auto &i : R.integrators()) i->integrate1();
            for (auto &s : R.sensors()) s->measure();
            std::cout << "Simstep=" << simstep_ << " t=" << t << " T=" << temp->getTemperature();
            if (pot) std::cout << " u=" << pot->getCurrentPotential();
            std::cout << std::endl;
            t += dt;
            simstep_++;
            if (simstep_ % write_freq == 0) VTKWriter::write("VTK_Output", simstep_);
            if (simstep_ % write_freq == 0)
                for (auto &s : R.sensors()) s->write(simstep_);
            for (auto &th : R.thermostats()) th->apply();
            for (auto &p : plugins) p->end_loop();
        }
    }
    for (auto &p : plugins) p->post_main_loop();
    for (auto &s : R.sensors()) s->write(simstep_);
    if (config->storeCheckpoint) CheckpointIO::writeCheckpoint(simstep_);
    for (auto &p : plugins) p->finalize();
}

}  // namespace komd
