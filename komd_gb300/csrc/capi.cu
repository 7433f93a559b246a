// capi.cu -- the C ABI of include/komd_gpu.h: engine lifetime, buffers,
// the per-step launch sequence, CUDA-graph replay, sensors and parity dumps.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "engine.cuh"
#include "kernels.cuh"
#include "surrogate.cuh"

using namespace komd;

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string &msg) {
    g_last_error = msg;
    return code;
}

#define CK(call)                                                                                       \
    do {                                                                                               \
        cudaError_t _e = (call);                                                                       \
        if (_e != cudaSuccess)                                                                         \
            return fail(_e == cudaErrorMemoryAllocation ? KOMD_ERR_NOMEM : KOMD_ERR_CUDA,              \
                        std::string(#call) + ": " + cudaGetErrorString(_e));                          \
    } while (0)

template <typename T>
void dfree(T *&p) {
    if (p) cudaFree(p);
    p = nullptr;
}

template <typename T>
cudaError_t dalloc(T *&p, size_t count) {
    dfree(p);
    if (count == 0) count = 1;
    return cudaMalloc(reinterpret_cast<void **>(&p), sizeof(T) * count);
}

// TemperatureSensor's conversion (TemperatureSensor.cpp:44-47), restated in engine.cuh
double temperature_from(double mv2, double n_in_box) { return sci_temperature(mv2, n_in_box); }

// ---------------------------------------------------------------------------
// profiling: event pairs per kernel family
// ---------------------------------------------------------------------------
const char *kFamilies[] = {"container", "pair", "bonded", "limit", "atm", "integrate", "measure", "surrogate",
                           "probe", "list_rebuilds"};
constexpr int kNumFamilies = 10;   // the last is a counter (launches = Verlet-list builds), not timed
enum Fam { F_CONTAINER = 0, F_PAIR, F_BONDED, F_LIMIT, F_ATM, F_INTEGRATE, F_MEASURE, F_SURROGATE, F_PROBE };

}  // namespace

namespace komd {
// lets other translation units of the library report through komd_gpu_last_error()
void set_last_error(const std::string &msg) { g_last_error = msg; }
}  // namespace komd

// learned three-body term (surrogate.cu)
struct Surrogate {
    bool loaded = false, fallback = false;
    float *x = nullptr, *mom = nullptr, *dedx = nullptr, *esite = nullptr, *fsur = nullptr;
    __nv_bfloat16 *w1 = nullptr, *w1t = nullptr, *w2 = nullptr, *w2t = nullptr;
    float *b1 = nullptr, *b2 = nullptr, *w3 = nullptr, *fmean = nullptr, *fstd = nullptr;
    float b3 = 0.f, e_scale = 1.f, e_shift = 0.f;
    int probe_every = 0;
    double probe_threshold = 0.0, last_rmse = -1.0, max_rmse = 0.0;
    int64_t probes = 0, steps = 0, fallback_step = -1;
    double *fprobe = nullptr, *fsur_d = nullptr, *probe_acc = nullptr;
};

struct komd_gpu {
    Engine e;
    Surrogate sur;
    double *f_scratch = nullptr;
    double *acc = nullptr;            // R_NSLOTS
    double *thermo_acc = nullptr;     // R_NSLOTS, the device thermostat's kinetic sums
    int partial_cap = 0;
    bool want_posd = false;
    bool pageable_access = false;     // kernels may dereference any host pointer (host page tables)
    // the terms given at creation: the sensors evaluate these whatever the step's
    // force terms are (the reference's sensors do not go through the functor list)
    uint32_t sensor_terms = 0;
    double *prof = nullptr;           // komd_gpu_rdf_profile's device histogram
    int prof_cap = 0;
    // profiling
    std::vector<cudaEvent_t> pool;
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> pending;
    int64_t launches[kNumFamilies] = {0};
    double ms[kNumFamilies] = {0};
    int64_t graph_steps = 0;
    uint64_t graph_epoch = 0;         // step graphs captured so far
    int *flags_h = nullptr;           // pinned landing buffer of the error flags
    // komd_gpu_step_host's one-step graph (the step graph with the caller's
    // buffers bound), valid for one capture of the step graph and one set of buffers
    cudaGraphExec_t hgraph = nullptr;
    uint64_t hgraph_epoch = 0;
    const void *hkey[3] = {nullptr, nullptr, nullptr};
};

namespace {

cudaEvent_t take_event(komd_gpu *h) {
    if (!h->pool.empty()) {
        cudaEvent_t ev = h->pool.back();
        h->pool.pop_back();
        return ev;
    }
    cudaEvent_t ev;
    cudaEventCreate(&ev);
    return ev;
}

struct ProfScope {
    komd_gpu *h;
    int fam;
    cudaEvent_t a = nullptr, b = nullptr;
    ProfScope(komd_gpu *h_, int fam_) : h(h_), fam(fam_) {
        if (!h->e.profiling) return;
        a = take_event(h);
        b = take_event(h);
        cudaEventRecord(a, h->e.stream);
    }
    ~ProfScope() {
        if (!a) return;
        cudaEventRecord(b, h->e.stream);
        h->pending.push_back({fam, {a, b}});
    }
};

void collect_profile(komd_gpu *h) {
    if (h->pending.empty()) return;
    cudaStreamSynchronize(h->e.stream);
    for (auto &p : h->pending) {
        float t = 0.f;
        cudaEventElapsedTime(&t, p.second.first, p.second.second);
        h->launches[p.first] += 1;
        h->ms[p.first] += t;
        h->pool.push_back(p.second.first);
        h->pool.push_back(p.second.second);
    }
    h->pending.clear();
}

int check_launch(const char *what) {
    const cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return fail(KOMD_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(err));
    return KOMD_OK;
}

int ensure_partials(komd_gpu *h) {
    Engine &e = h->e;
    int need = e.g.ncell;                      // pair kernels write at most one partial row per cell
    need = std::max(need, atm_grid(e));
    need = std::max(need, kinetic_grid(e));
    if (need > h->partial_cap) {
        CK(dalloc(e.partials, (size_t)need * R_NSLOTS));
        h->partial_cap = need;
    }
    return KOMD_OK;
}

SurParams sur_params(komd_gpu *h) {
    Engine &e = h->e;
    Surrogate &u = h->sur;
    SurParams p;
    p.n = (int)e.n;
    p.rc = (float)e.cfg.cutoff_3b;
    p.nl = e.nl;
    p.nl_count = e.nl_count;
    p.nl_cap = e.nl_cap;
    p.fmean = u.fmean;
    p.fstd = u.fstd;
    p.x = u.x;
    p.mom = u.mom;
    p.dedx = u.dedx;
    p.e_site = u.esite;
    p.fsur = u.fsur;
    p.w1 = u.w1; p.w1t = u.w1t; p.w2 = u.w2; p.w2t = u.w2t;
    p.b1 = u.b1; p.b2 = u.b2; p.w3 = u.w3;
    p.b3 = u.b3; p.e_scale = u.e_scale; p.e_shift = u.e_shift;
    p.num_sms = e.num_sms;
    return p;
}

bool surrogate_on(komd_gpu *h) {
    return (h->e.cfg.terms & KOMD_TERM_ATM_SURROGATE) && h->sur.loaded && !h->sur.fallback;
}

// surrogate three-body forces: into f (fout == nullptr) or written to fout
void enqueue_surrogate(komd_gpu *h, double *fout) {
    Engine &e = h->e;
    SurParams p = sur_params(h);
    launch_sur_desc(p, e.stream);
    launch_sur_mlp(p, e.stream);
    launch_sur_force(p, e.stream);
    launch_sur_apply(p, e.slot_site, e.f, fout, e.stream);
}

bool fused_lj_atm(komd_gpu *h, bool measure) {
    const Engine &e = h->e;
    return !measure && !surrogate_on(h) && e.atm_acc != nullptr && e.verlet && (e.cfg.terms & KOMD_TERM_ATM);
}

// the force sequence of Simulation::run: 2-body functors (LJ / FENE, bonded,
// Limit), then the 3-body functor (ATM, exact or learned)
// returns true when integrate1 was fused into the last force kernel (with_step1)
bool enqueue_forces(komd_gpu *h, bool measure, double *lj_hist, bool with_step1 = false) {
    Engine &e = h->e;
    cudaStream_t st = e.stream;
    bool fused = false;
    int pair_blocks;
    // a force-only pass whose ATM list goes only to the once-per-triplet kernel
    // needs the neighbours above each site only
    // force-only FP32 FULL ATM on the Verlet path: the LJ pass sweeps each site's
    // triplets itself (k_lj_atm) and the ATM list never goes to memory
    const bool lj_atm = fused_lj_atm(h, measure);
    if (lj_atm) {
        ProfScope ps(h, F_PAIR);
        launch_lj_atm(e, st);   // writes f (first writer); ATM sums to the fixed-point accumulators
        pair_blocks = 0;
    } else if (measure || (e.cfg.terms & (KOMD_TERM_LJ | KOMD_TERM_FENE | KOMD_TERM_ATM))) {
        ProfScope ps(h, F_PAIR);
        pair_blocks = launch_pair(e, st, measure, lj_hist);   // the pair pass writes f (first writer)
    } else {
        pair_blocks = 0;
        cudaMemsetAsync(e.f, 0, sizeof(double) * 3 * e.n, st);
    }
    if (measure) launch_sum_partials(st, pair_blocks, e.partials, h->acc);
    if (e.cfg.terms & KOMD_TERM_TABULATED) {   // in the LJ functor's place (IBI.cpp:52-54), before Limit
        ProfScope ps(h, F_PAIR);
        launch_pair_table(e, st);
    }
    if ((e.cfg.terms & KOMD_TERM_BONDED) && (e.n_bonds > 0 || e.n_angles > 0)) {
        ProfScope ps(h, F_BONDED);
        launch_bonded(e, st, measure, h->acc);
    }
    if (e.cfg.terms & KOMD_TERM_LIMIT) {
        ProfScope ps(h, F_LIMIT);
        launch_limit(e, st);
    }
    if (surrogate_on(h)) {
        {
            ProfScope ps(h, F_SURROGATE);
            enqueue_surrogate(h, nullptr);
        }
        if (measure) launch_sum_sites((int)e.n, h->sur.esite, h->acc + R_UATM, st);
    } else if (e.cfg.terms & KOMD_TERM_ATM) {
        {
            ProfScope ps(h, F_ATM);
            fused = lj_atm ? launch_atm_flush(e, st, with_step1, lj_atm_half(e)) : launch_atm(e, st, measure, with_step1);
        }
        if (measure) launch_sum_partials(st, atm_grid(e), e.partials, h->acc);
    }
    return fused;
}

void enqueue_step(komd_gpu *h) {
    Engine &e = h->e;
    // host-buffer step with a pinned position buffer: the drift kernel keeps r on
    // the device and a copy-engine copy on the side stream writes it back while
    // the container and force kernels run (joined before the step ends)
    double *r_async = nullptr;
    if (e.hout_r && e.hout_r_async && e.side && e.ev_fork && e.ev_join) {
        r_async = e.hout_r;
        e.hout_r = nullptr;
    }
    {
        ProfScope ps(h, F_INTEGRATE);
        launch_step0(e, e.stream, true);
    }
    bool forked = false;
    if (r_async)
        forked = cudaEventRecord(e.ev_fork, e.stream) == cudaSuccess &&
                 cudaStreamWaitEvent(e.side, e.ev_fork, 0) == cudaSuccess &&
                 cudaMemcpyAsync(r_async, e.r, sizeof(double) * 3 * (size_t)e.n, cudaMemcpyDeviceToHost,
                                 e.side) == cudaSuccess &&
                 cudaEventRecord(e.ev_join, e.side) == cudaSuccess;
    {
        ProfScope ps(h, F_CONTAINER);
        launch_container(e, e.stream);
    }
    // the step's integrate1 rides on the ATM flush when the once-per-triplet path runs
    if (!enqueue_forces(h, false, nullptr, true)) {
        ProfScope ps(h, F_INTEGRATE);
        launch_step1(e, e.stream);
    }
    if (e.cfg.thermostat) {   // Simulation.cpp:72, after the step's sensors
        ProfScope ps(h, F_INTEGRATE);
        cudaMemsetAsync(h->thermo_acc, 0, sizeof(double) * R_NSLOTS, e.stream);
        launch_kinetic(e, e.stream, 0);
        launch_sum_partials(e.stream, kinetic_grid(e), e.partials, h->thermo_acc);
        launch_velocity_scale(e, e.stream, h->thermo_acc, 1.0);
    }
    if (r_async) {
        // joined before the step ends; if the side stream could not take the
        // copy, it runs here on the engine's stream instead
        if (!forked || cudaStreamWaitEvent(e.stream, e.ev_join, 0) != cudaSuccess)
            cudaMemcpyAsync(r_async, e.r, sizeof(double) * 3 * (size_t)e.n, cudaMemcpyDeviceToHost, e.stream);
        e.hout_r = r_async;
    }
}

int read_flags(komd_gpu *h, int flags[E_NFLAGS], bool clear) {
    Engine &e = h->e;
    int *land = h->flags_h ? h->flags_h : flags;   // a pinned landing buffer copies without staging
    CK(cudaMemcpyAsync(land, e.err, sizeof(int) * E_NFLAGS, cudaMemcpyDeviceToHost, e.stream));
    if (clear) CK(cudaMemsetAsync(e.err, 0, sizeof(int) * E_NFLAGS, e.stream));
    CK(cudaStreamSynchronize(e.stream));
    if (land != flags) std::memcpy(flags, land, sizeof(int) * E_NFLAGS);
    return KOMD_OK;
}

int alloc_atm_list(komd_gpu *h, int cap) {
    Engine &e = h->e;
    e.nl_cap = cap;
    if (e.cfg.terms & KOMD_TERM_ATM) {
        const size_t entry = e.cfg.precision == KOMD_FP64 ? 32 : 16;
        float4 *p = nullptr;
        dfree(e.nl);
        CK(cudaMalloc(reinterpret_cast<void **>(&p), entry * (size_t)cap * (size_t)std::max<int64_t>(e.n, 1)));
        e.nl = p;
        CK(dalloc(e.nl_count, e.n));
        set_kernel_attributes(e);
    }
    if (e.graph) { cudaGraphExecDestroy(e.graph); e.graph = nullptr; }
    e.graph_valid = false;
    return KOMD_OK;
}

int ensure_posd(komd_gpu *h) {
    Engine &e = h->e;
    if (e.posd) return KOMD_OK;
    CK(dalloc(e.posd, 3 * (size_t)e.n));
    CK(dalloc(e.seps_d, e.n));
    CK(dalloc(e.sig_d, e.n));
    if (e.graph) { cudaGraphExecDestroy(e.graph); e.graph = nullptr; }
    e.graph_valid = false;
    return KOMD_OK;
}

int alloc_verlet(komd_gpu *h, int cap) {
    Engine &e = h->e;
    e.vl_cap = cap;
    CK(dalloc(e.bias, 3 * (size_t)e.n));
    CK(dalloc(e.ref4, e.n));
    CK(dalloc(e.slot_cell, e.n));
    CK(dalloc(e.zkey, e.n));
    CK(dalloc(e.vl, (size_t)cap * (size_t)e.n));
    CK(dalloc(e.vl_count, e.n));
    if (e.graph) { cudaGraphExecDestroy(e.graph); e.graph = nullptr; }
    e.graph_valid = false;
    return KOMD_OK;
}

// forces a rebuild of cells (and, on the Verlet path, of the list) now
void launch_rebuild(komd_gpu *h) {
    Engine &e = h->e;
    if (e.verlet) cudaMemsetAsync(e.rebuild, 0x01, sizeof(int), e.stream);
    launch_container(e, e.stream);
    if (e.verlet) cudaMemsetAsync(e.rebuild, 0, sizeof(int), e.stream);
}

// The Verlet path keeps a neighbour list across steps; it is used only where
// the results do not depend on the cells of the current step: FP32 forces,
// no FENE (same-cell semantics), the FULL triplet set and the CORRECT virial.
bool uses_verlet(const komd_config &c) {
    return c.skin > 0 && c.precision == KOMD_FP32 && !(c.terms & KOMD_TERM_FENE) &&
           (!(c.terms & KOMD_TERM_ATM) || c.atm_enum == KOMD_ATM_ENUM_FULL) && c.virial_mode == KOMD_VIRIAL_CORRECT;
}

int validate(const komd_config *c, Grid &g) {
    if (!c) return fail(KOMD_ERR_ARG, "null config");
    if (!(c->cell_size > 0)) return fail(KOMD_ERR_ARG, "cell_size must be > 0");
    const bool lj = (c->terms & KOMD_TERM_LJ) != 0, atm = (c->terms & KOMD_TERM_ATM) != 0;
    if (lj && !(c->cutoff > 0)) return fail(KOMD_ERR_ARG, "cutoff must be > 0");
    if (c->thermostat && !(c->temperature_target > 0)) return fail(KOMD_ERR_ARG, "thermostat needs temperature_target > 0");
    if ((c->terms & KOMD_TERM_ATM2B) && !lj) return fail(KOMD_ERR_ARG, "KOMD_TERM_ATM2B scales the LJ term: set KOMD_TERM_LJ");
    if ((c->terms & KOMD_TERM_TABULATED) && c->skin > 0)
        return fail(KOMD_ERR_ARG, "the tabulated pair term runs on per-step cell lists (skin 0)");
    if (c->cell_size < c->cutoff)
        return fail(KOMD_ERR_ARG, "cell size must be larger or equal to cutoff radius");
    if (atm && (!(c->cutoff_3b > 0) || c->cell_size < c->cutoff_3b))
        return fail(KOMD_ERR_ARG, "cutoff_3b must be > 0 and <= cell_size");
    if (!(c->delta_t > 0)) return fail(KOMD_ERR_ARG, "delta_t must be > 0");
    if (c->precision != KOMD_FP32 && c->precision != KOMD_FP64) return fail(KOMD_ERR_ARG, "bad precision");
    if (c->skin < 0) return fail(KOMD_ERR_ARG, "skin must be >= 0");
    if (c->switch_width < 0) return fail(KOMD_ERR_ARG, "switch_width must be >= 0");
    if (c->switch_width > 0) {
        // the labelled switched-cutoff option lives on the half-list Verlet path
        if (!uses_verlet(*c))
            return fail(KOMD_ERR_ARG, "switch_width > 0 needs the Verlet path (skin > 0, FP32, FULL ATM, CORRECT virial, no FENE)");
        // with the learned three-body term the LJ pair pass carries the switch
        // (the learned energy vanishes smoothly at its cutoff by construction)
        if (c->terms & (KOMD_TERM_LIMIT | KOMD_TERM_FENE | KOMD_TERM_ATM2B | KOMD_TERM_TABULATED | KOMD_TERM_BONDED))
            return fail(KOMD_ERR_ARG, "switch_width > 0 covers LJ, exact ATM and the learned term only (no Limit, FENE, ATM2B, tabulated or bonded terms)");
        if ((lj && !(c->switch_width < c->cutoff)) || (atm && !(c->switch_width < c->cutoff_3b)))
            return fail(KOMD_ERR_ARG, "switch_width must be below each cutoff");
    }
    if (uses_verlet(*c)) {
        const double rl = std::max(lj ? c->cutoff : 0.0, atm ? c->cutoff_3b : 0.0) + c->skin;
        if (c->cell_size < rl)
            return fail(KOMD_ERR_ARG, "with a Verlet skin the cell size must be >= cutoff + skin");
    }
    g.cs = c->cell_size;
    g.ncell = 1;
    for (int d = 0; d < 3; d++) {
        g.low[d] = c->domain_low[d];
        g.high[d] = c->domain_high[d];
        g.L[d] = c->domain_high[d] - c->domain_low[d];
        const double q = std::floor(g.L[d] / c->cell_size);   // math::ufloor (LinkedCells.cpp:19)
        if (!(q >= 3.0))
            return fail(KOMD_ERR_ARG, "need at least 3 domain cells per dimension (floor(L / cell_size) >= 3)");
        if (q > 1 << 20) return fail(KOMD_ERR_ARG, "too many cells");
        g.nd[d] = (int)q;
        g.ncell *= g.nd[d];
    }
    return KOMD_OK;
}

// the launches of a measure on the engine's stream, and the copies of the
// sums (acc_h, R_NSLOTS doubles), the RDF and the LJ histograms to the host
// buffers given (asynchronous: valid once the stream has synchronised)
int measure_enqueue(komd_gpu *h, uint32_t mask, double *acc_h, double *rdf, double *lj_hist) {
    Engine &e = h->e;
    cudaStream_t st = e.stream;
    ProfScope ps(h, F_MEASURE);
    CK(cudaMemsetAsync(h->acc, 0, sizeof(double) * R_NSLOTS, st));
    const bool need_forces = (mask & (KOMD_MEASURE_ENERGY | KOMD_MEASURE_PRESSURE | KOMD_MEASURE_LJ_HIST)) != 0;
    if (need_forces) {
        // re-evaluate the force terms into a scratch force buffer (the sensors of
        // the reference re-run their functors as well); f itself is untouched
        if (mask & KOMD_MEASURE_LJ_HIST) CK(cudaMemsetAsync(e.lj_hist, 0, sizeof(double) * 4 * e.cfg.lj_bins, st));
        double *keep = e.f;
        const uint32_t force_terms = e.cfg.terms;
        CK(cudaMemsetAsync(h->f_scratch, 0, sizeof(double) * 3 * e.n, st));
        e.f = h->f_scratch;
        e.cfg.terms = h->sensor_terms;
        enqueue_forces(h, true, (mask & KOMD_MEASURE_LJ_HIST) ? e.lj_hist : nullptr);
        e.cfg.terms = force_terms;
        e.f = keep;
    }
    const int n_terms = e.cfg.virial_mode == KOMD_VIRIAL_COMPAT ? (int)e.n_mol : (int)e.n;
    launch_kinetic(e, st, n_terms);
    launch_sum_partials(st, kinetic_grid(e), e.partials, h->acc);
    if ((mask & KOMD_MEASURE_RDF) && e.rdf_bins > 0) {
        if (e.verlet) launch_rebuild(h);   // the cells of the last rebuild may be stale
        CK(cudaMemsetAsync(e.rdf, 0, sizeof(double) * e.rdf_bins, st));
        double minw = 1e300;
        for (int d = 0; d < 3; d++) minw = std::min(minw, e.cfg.cell_size);
        launch_rdf(e, st, e.rdf, e.cfg.rdf_max <= minw);
    }
    int rc = check_launch("measure");
    if (rc) return rc;
    CK(cudaMemcpyAsync(acc_h, h->acc, sizeof(double) * R_NSLOTS, cudaMemcpyDeviceToHost, st));
    if (rdf && (mask & KOMD_MEASURE_RDF) && e.rdf_bins > 0)
        CK(cudaMemcpyAsync(rdf, e.rdf, sizeof(double) * e.rdf_bins, cudaMemcpyDeviceToHost, st));
    if (lj_hist && (mask & KOMD_MEASURE_LJ_HIST))
        CK(cudaMemcpyAsync(lj_hist, e.lj_hist, sizeof(double) * 4 * e.cfg.lj_bins, cudaMemcpyDeviceToHost, st));
    return KOMD_OK;
}

void measure_fill(const double *acc, komd_observables *obs) {
    std::memset(obs, 0, sizeof(*obs));
    obs->mv2 = acc[R_MV2];
    obs->n_in_box = acc[R_NBOX];
    obs->temperature = acc[R_NBOX] > 0 ? temperature_from(acc[R_MV2], acc[R_NBOX]) : 0.0;
    obs->u_lj = acc[R_ULJ];
    obs->u_atm = acc[R_UATM];
    obs->u_bonded = acc[R_UBOND];
    for (int k = 0; k < 6; k++) {
        obs->kinetic[k] = acc[R_K0 + k];
        obs->virial[k] = acc[R_W0 + k];
        obs->pressure[k] = obs->kinetic[k] + obs->virial[k];
    }
    obs->pairs_in_cutoff = (int64_t)std::llround(acc[R_PAIRS]);
    obs->triplets = (int64_t)std::llround(acc[R_TRIPS]);
}

}  // namespace

extern "C" {

const char *komd_gpu_last_error(void) { return g_last_error.c_str(); }
int komd_gpu_abi_version(void) { return KOMD_GPU_ABI_VERSION; }

double komd_sci_temperature(double mv2, double n_in_box) { return temperature_from(mv2, n_in_box); }

int komd_gpu_create(const komd_config *cfg, int device, komd_gpu **out) {
    if (!out) return fail(KOMD_ERR_ARG, "null output handle");
    *out = nullptr;
    Grid g;
    const int rc = validate(cfg, g);
    if (rc) return rc;
    CK(cudaSetDevice(device));
    komd_gpu *h = new komd_gpu();
    Engine &e = h->e;
    e.cfg = *cfg;
    h->sensor_terms = cfg->terms;
    if (e.cfg.lj_bins <= 0) e.cfg.lj_bins = 100;
    if (!(e.cfg.max_sigma > 0)) e.cfg.max_sigma = 1.0;
    e.g = g;
    e.device = device;
    {
        int sms = 0;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) == cudaSuccess && sms > 0)
            e.num_sms = sms;
    }
    {
        int pa = 0, pt = 0;
        cudaDeviceGetAttribute(&pa, cudaDevAttrPageableMemoryAccess, device);
        cudaDeviceGetAttribute(&pt, cudaDevAttrPageableMemoryAccessUsesHostPageTables, device);
        h->pageable_access = pa != 0 && pt != 0;
    }
    if (cudaStreamCreateWithFlags(&e.stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete h;
        return fail(KOMD_ERR_CUDA, "stream creation failed");
    }
    e.own_stream = true;
    if (cudaStreamCreateWithFlags(&e.side, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&e.ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&e.ev_join, cudaEventDisableTiming) != cudaSuccess) {
        komd_gpu_destroy(h);
        return fail(KOMD_ERR_CUDA, "stream creation failed");
    }
    if (dalloc(e.cell_count, g.ncell) || dalloc(e.cell_start, g.ncell + 1) || dalloc(e.cell_mcount, g.ncell) ||
        dalloc(e.cell_mstart, g.ncell + 1) || dalloc(e.err, E_NFLAGS) || dalloc(h->acc, R_NSLOTS) || dalloc(h->thermo_acc, R_NSLOTS)) {
        komd_gpu_destroy(h);
        return fail(KOMD_ERR_NOMEM, "device allocation failed");
    }
    cudaMemset(e.err, 0, sizeof(int) * E_NFLAGS);
    if (cudaHostAlloc(reinterpret_cast<void **>(&h->flags_h), sizeof(int) * E_NFLAGS, cudaHostAllocDefault) != cudaSuccess) {
        cudaGetLastError();
        h->flags_h = nullptr;   // read_flags then copies into the caller's array
    }
    cudaMemset(e.cell_count, 0, sizeof(int) * g.ncell);    // the binning's counters start at zero
    cudaMemset(e.cell_mcount, 0, sizeof(int) * g.ncell);
    if (e.cfg.rdf_dr > 0 && e.cfg.rdf_max > 0) {
        e.rdf_bins = (int64_t)(uint64_t)(e.cfg.rdf_max / e.cfg.rdf_dr);   // RDFSensor.cpp:18
        if (e.rdf_bins > 0 && dalloc(e.rdf, e.rdf_bins)) { komd_gpu_destroy(h); return fail(KOMD_ERR_NOMEM, "rdf"); }
    }
    if (dalloc(e.lj_hist, 4 * (size_t)e.cfg.lj_bins)) { komd_gpu_destroy(h); return fail(KOMD_ERR_NOMEM, "hist"); }
    {
        // home-relative centre offsets of the 3 neighbour cells per dimension,
        // in FP64 once and rounded to FP32 (the FP32 kernels never touch FP64)
        std::vector<float> tab;
        for (int d = 0; d < 3; d++)
            for (int k = 0; k < g.nd[d]; k++)
                for (int dd = -1; dd <= 1; dd++) {
                    int q = k + dd;
                    double shift = 0.0;
                    if (q < 0) { q += g.nd[d]; shift = -g.L[d]; }
                    else if (q >= g.nd[d]) { q -= g.nd[d]; shift = g.L[d]; }
                    tab.push_back((float)((cell_centre(g, d, q) + shift) - cell_centre(g, d, k)));
                }
        if (dalloc(e.offtab, tab.size()) ||
            cudaMemcpy(e.offtab, tab.data(), sizeof(float) * tab.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
            komd_gpu_destroy(h);
            return fail(KOMD_ERR_NOMEM, "offset table");
        }
    }
    e.verlet = uses_verlet(e.cfg);
    if (e.verlet) {
        // per cell and neighbour: home-relative centre offset (FP64 -> FP32), w = periodic image
        std::vector<float4> nb((size_t)g.ncell * 27);
        for (int c = 0; c < g.ncell; c++) {
            int cx, cy, cz;
            cell_coords(g, c, cx, cy, cz);
            const int cc[3] = {cx, cy, cz};
            for (int k = 0; k < 27; k++) {
                const int dd[3] = {k % 3 - 1, (k / 3) % 3 - 1, k / 9 - 1};
                double o[3];
                bool img = false;
                for (int d = 0; d < 3; d++) {
                    int q = cc[d] + dd[d];
                    double shift = 0.0;
                    if (q < 0) { q += g.nd[d]; shift = -g.L[d]; img = true; }
                    else if (q >= g.nd[d]) { q -= g.nd[d]; shift = g.L[d]; img = true; }
                    o[d] = (cell_centre(g, d, q) + shift) - cell_centre(g, d, cc[d]);
                }
                nb[(size_t)c * 27 + k] = make_float4((float)o[0], (float)o[1], (float)o[2], img ? 1.f : 0.f);
            }
        }
        if (dalloc(e.nboff, nb.size()) || dalloc(e.rebuild, 1) || dalloc(e.rebuild_count, 1) || dalloc(e.vb_next, 1) ||
            cudaMemset(e.rebuild_count, 0, sizeof(int)) != cudaSuccess ||
            cudaMemcpy(e.nboff, nb.data(), sizeof(float4) * nb.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemset(e.rebuild, 0, sizeof(int)) != cudaSuccess) {
            komd_gpu_destroy(h);
            return fail(KOMD_ERR_NOMEM, "Verlet tables");
        }
    }
    h->want_posd = e.cfg.precision == KOMD_FP64 || (e.cfg.terms & KOMD_TERM_TABULATED);
    *out = h;
    return KOMD_OK;
}

int komd_gpu_destroy(komd_gpu *h) {
    if (!h) return KOMD_OK;
    Engine &e = h->e;
    cudaSetDevice(e.device);
    if (e.stream) cudaStreamSynchronize(e.stream);
    if (e.graph) cudaGraphExecDestroy(e.graph);
    if (h->hgraph) cudaGraphExecDestroy(h->hgraph);
    if (h->flags_h) cudaFreeHost(h->flags_h);
    dfree(e.r); dfree(e.v); dfree(e.f); dfree(e.m); dfree(e.eps); dfree(e.sig);
    dfree(e.key); dfree(e.site_mol); dfree(e.site_slot);
    dfree(e.mol_off); dfree(e.mol_cell); dfree(e.mol_rank); dfree(e.com);
    dfree(e.cell_count); dfree(e.cell_start); dfree(e.cell_mcount); dfree(e.cell_mstart); dfree(e.cell_mols);
    dfree(e.slot_site); dfree(e.skey); dfree(e.pos4); dfree(e.seps); dfree(e.posd); dfree(e.seps_d); dfree(e.sig_d);
    dfree(e.nl); dfree(e.nl_count); dfree(e.bonds); dfree(e.angles); dfree(e.partials); dfree(e.err);
    dfree(e.tab_x); dfree(e.tab_y); dfree(e.tab_s); dfree(e.atm_acc); dfree(e.fown);
    dfree(e.rdf); dfree(e.lj_hist); dfree(e.counts); dfree(h->f_scratch); dfree(h->prof); dfree(h->acc); dfree(h->thermo_acc); dfree(e.offtab);
    dfree(e.nboff); dfree(e.vb_next); dfree(e.rebuild); dfree(e.bias); dfree(e.ref4); dfree(e.slot_cell); dfree(e.zkey); dfree(e.vl); dfree(e.vl_count);
    dfree(e.rebuild_count); dfree(e.hdtm); dfree(e.exact_com);
    {
        Surrogate &u = h->sur;
        dfree(u.x); dfree(u.mom); dfree(u.dedx); dfree(u.esite); dfree(u.fsur); dfree(u.w1); dfree(u.w1t);
        dfree(u.w2); dfree(u.w2t); dfree(u.b1); dfree(u.b2); dfree(u.w3); dfree(u.fmean); dfree(u.fstd);
        dfree(u.fprobe); dfree(u.fsur_d); dfree(u.probe_acc);
    }
    for (auto &p : h->pending) { h->pool.push_back(p.second.first); h->pool.push_back(p.second.second); }
    for (auto ev : h->pool) cudaEventDestroy(ev);
    if (e.own_stream && e.stream) cudaStreamDestroy(e.stream);
    if (e.side) cudaStreamDestroy(e.side);
    if (e.ev_fork) cudaEventDestroy(e.ev_fork);
    if (e.ev_join) cudaEventDestroy(e.ev_join);
    delete h;
    return KOMD_OK;
}

int komd_gpu_set_stream(komd_gpu *h, void *stream) {
    if (!h) return fail(KOMD_ERR_ARG, "null handle");
    Engine &e = h->e;
    CK(cudaStreamSynchronize(e.stream));
    if (e.own_stream) cudaStreamDestroy(e.stream);
    if (stream) {
        e.stream = (cudaStream_t)stream;
        e.own_stream = false;
    } else {
        CK(cudaStreamCreateWithFlags(&e.stream, cudaStreamNonBlocking));
        e.own_stream = true;
    }
    if (e.graph) { cudaGraphExecDestroy(e.graph); e.graph = nullptr; }
    e.graph_valid = false;
    return KOMD_OK;
}

int komd_gpu_grid_dims(komd_gpu *h, int64_t nd[3]) {
    if (!h || !nd) return fail(KOMD_ERR_ARG, "null argument");
    for (int d = 0; d < 3; d++) nd[d] = h->e.g.nd[d];
    return KOMD_OK;
}

int64_t komd_gpu_num_sites(komd_gpu *h) { return h ? h->e.n : -1; }

int komd_gpu_upload_sites(komd_gpu *h, int64_t n, const double *r, const double *v, const double *m,
                          const double *eps, const double *sig, const uint64_t *mol_id) {
    if (!h || n <= 0 || !r || !v || !m || !eps || !sig || !mol_id) return fail(KOMD_ERR_ARG, "bad site arrays");
    if (n >= (int64_t)1 << 31) return fail(KOMD_ERR_ARG, "too many sites");
    Engine &e = h->e;
    CK(cudaSetDevice(e.device));
    if ((e.cfg.terms & KOMD_TERM_ATM) && n > kMaxAtmSlot)
        return fail(KOMD_ERR_ARG, "ATM supports at most 2^25 - 1 sites per system");
    // molecules: consecutive equal IDs (CheckpointIO.cpp:55-72); dense keys keep ID equality
    std::vector<int> off, key(n), site_mol(n);
    std::unordered_map<uint64_t, int> dense;
    dense.reserve((size_t)n);
    for (int64_t s = 0; s < n; s++) {
        if (s == 0 || mol_id[s] != mol_id[s - 1]) off.push_back((int)s);
        site_mol[s] = (int)off.size() - 1;
        auto it = dense.find(mol_id[s]);
        if (it == dense.end()) it = dense.emplace(mol_id[s], (int)dense.size()).first;
        key[s] = it->second;
        if (!(m[s] > 0)) return fail(KOMD_ERR_ARG, "site masses must be > 0");
    }
    off.push_back((int)n);
    e.n = n;
    e.n_mol = (int64_t)off.size() - 1;
    CK(dalloc(e.r, 3 * n)); CK(dalloc(e.v, 3 * n)); CK(dalloc(e.f, 3 * n)); CK(dalloc(h->f_scratch, 3 * n));
    CK(dalloc(e.m, n)); CK(dalloc(e.eps, n)); CK(dalloc(e.sig, n));
    CK(dalloc(e.key, n)); CK(dalloc(e.site_mol, n)); CK(dalloc(e.site_slot, n));
    CK(dalloc(e.mol_off, e.n_mol + 1)); CK(dalloc(e.mol_cell, e.n_mol)); CK(dalloc(e.mol_rank, e.n_mol));
    CK(dalloc(e.com, 3 * e.n_mol)); CK(dalloc(e.cell_mols, e.n_mol));
    CK(dalloc(e.slot_site, n)); CK(dalloc(e.skey, n)); CK(dalloc(e.pos4, n)); CK(dalloc(e.seps, n));
    CK(dalloc(e.counts, n));
    dfree(e.posd); dfree(e.seps_d); dfree(e.sig_d);
    if (h->want_posd) {
        CK(dalloc(e.posd, 3 * (size_t)n)); CK(dalloc(e.seps_d, n)); CK(dalloc(e.sig_d, n));
    }
    CK(cudaMemcpy(e.r, r, sizeof(double) * 3 * n, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(e.v, v, sizeof(double) * 3 * n, cudaMemcpyHostToDevice));
    CK(cudaMemset(e.f, 0, sizeof(double) * 3 * n));
    CK(cudaMemcpy(e.m, m, sizeof(double) * n, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(e.eps, eps, sizeof(double) * n, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(e.sig, sig, sizeof(double) * n, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(e.key, key.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(e.site_mol, site_mol.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(e.mol_off, off.data(), sizeof(int) * off.size(), cudaMemcpyHostToDevice));
    {
        // (dt * 0.5) / m per site, the reference's dtInv2m, and the exact-COM flags
        std::vector<double> hdtm(n);
        const double dt_half = e.cfg.delta_t * 0.5;
        for (int64_t s = 0; s < n; s++) hdtm[s] = dt_half / m[s];
        std::vector<unsigned char> exact(e.n_mol);
        for (int64_t k = 0; k < e.n_mol; k++) {
            int ex = 0;
            const double mk = m[off[k]];
            exact[k] = (off[k + 1] - off[k] == 1 && std::frexp(mk, &ex) == 0.5) ? 1 : 0;
        }
        CK(dalloc(e.hdtm, n));
        CK(dalloc(e.exact_com, e.n_mol));
        CK(cudaMemcpy(e.hdtm, hdtm.data(), sizeof(double) * n, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(e.exact_com, exact.data(), e.n_mol, cudaMemcpyHostToDevice));
        e.fused_drift = e.verlet && e.n_mol == n;
        for (int64_t k = 0; k < e.n_mol && e.fused_drift; k++) e.fused_drift = exact[k] != 0;
        e.uniform = true;
        for (int64_t s = 1; s < n && e.uniform; s++) e.uniform = eps[s] == eps[0] && sig[s] == sig[0];
        e.eps0 = (float)eps[0];
        e.sig0 = (float)sig[0];
        e.lj_fscale = 1.0;
        if (e.cfg.terms & KOMD_TERM_ATM2B) {
            // ATM2B::ATM2B (ATM2B.cpp:9-20): 1 - 2 nu rho / (3 eps sigma^6), number density of molecules
            const double rho = (double)e.n_mol / (e.g.L[0] * e.g.L[1] * e.g.L[2]);
            const double sig6 = std::pow(sig[0], 6);
            e.lj_fscale = 1.0 - ((2 * e.cfg.nu * rho) / (3 * eps[0] * sig6));
        }
    }
    // ATM list capacity: 1.6x the mean neighbour count inside cutoff_3b + 16
    int cap = e.cfg.atm_list_cap;
    if (cap <= 0) {
        const double vol = e.g.L[0] * e.g.L[1] * e.g.L[2];
        const double rc = e.cfg.cutoff_3b;
        const double mean = (double)n / vol * 4.18879 * rc * rc * rc;
        cap = (int)std::ceil(1.6 * mean + 16);
        cap = std::max(32, std::min(1024, (cap + 7) / 8 * 8));
    }
    int rc = alloc_atm_list(h, cap);
    if (rc) return rc;
    dfree(e.atm_acc);
    dfree(e.fown);
    if ((e.cfg.terms & KOMD_TERM_ATM) && e.cfg.precision == KOMD_FP32 && e.cfg.atm_enum == KOMD_ATM_ENUM_FULL) {
        // fixed-point force sums of the once-per-triplet kernel (kept at zero between launches)
        CK(dalloc(e.atm_acc, 3 * (size_t)n));
        CK(cudaMemset(e.atm_acc, 0, sizeof(unsigned long long) * 3 * n));
        CK(dalloc(e.fown, (size_t)n));
    }
    if (e.verlet) {
        if (n > kMaxVerletSlot) return fail(KOMD_ERR_ARG, "the Verlet path supports at most 2^26 - 1 sites");
        const double vol = e.g.L[0] * e.g.L[1] * e.g.L[2];
        const bool lj = (e.cfg.terms & KOMD_TERM_LJ) != 0, atm = (e.cfg.terms & KOMD_TERM_ATM) != 0;
        const double rl = std::max(lj ? e.cfg.cutoff : 0.0, atm ? e.cfg.cutoff_3b : 0.0) + e.cfg.skin;
        const double mean = (double)n / vol * 4.18879 * rl * rl * rl;
        rc = alloc_verlet(h, std::max(64, std::min(2048, ((int)std::ceil(1.5 * mean + 32) + 31) / 32 * 32)));
        if (rc) return rc;
    }
    rc = ensure_partials(h);
    if (rc) return rc;
    e.have_sites = true;
    e.have_cells = e.have_forces = false;
    if (e.graph) { cudaGraphExecDestroy(e.graph); e.graph = nullptr; }
    e.graph_valid = false;
    return KOMD_OK;
}

int komd_gpu_set_state(komd_gpu *h, const double *r, const double *v) {
    if (!h || !h->e.have_sites) return fail(KOMD_ERR_STATE, "no sites uploaded");
    Engine &e = h->e;
    if (r) CK(cudaMemcpyAsync(e.r, r, sizeof(double) * 3 * e.n, cudaMemcpyHostToDevice, e.stream));
    if (v) CK(cudaMemcpyAsync(e.v, v, sizeof(double) * 3 * e.n, cudaMemcpyHostToDevice, e.stream));
    CK(cudaStreamSynchronize(e.stream));
    if (r) e.have_cells = e.have_forces = false;
    return KOMD_OK;
}

int komd_gpu_set_topology(komd_gpu *h, int64_t n_bonds, const int64_t *bonds, int64_t n_angles,
                          const int64_t *angles) {
    if (!h || !h->e.have_sites) return fail(KOMD_ERR_STATE, "no sites uploaded");
    Engine &e = h->e;
    std::vector<int> b(2 * std::max<int64_t>(n_bonds, 0)), a(3 * std::max<int64_t>(n_angles, 0));
    for (int64_t k = 0; k < 2 * n_bonds; k++) {
        if (bonds[k] < 0 || bonds[k] >= e.n) return fail(KOMD_ERR_ARG, "bond index out of range");
        b[k] = (int)bonds[k];
    }
    for (int64_t k = 0; k < 3 * n_angles; k++) {
        if (angles[k] < 0 || angles[k] >= e.n) return fail(KOMD_ERR_ARG, "angle index out of range");
        a[k] = (int)angles[k];
    }
    CK(dalloc(e.bonds, b.size()));
    CK(dalloc(e.angles, a.size()));
    if (!b.empty()) CK(cudaMemcpy(e.bonds, b.data(), sizeof(int) * b.size(), cudaMemcpyHostToDevice));
    if (!a.empty()) CK(cudaMemcpy(e.angles, a.data(), sizeof(int) * a.size(), cudaMemcpyHostToDevice));
    e.n_bonds = std::max<int64_t>(n_bonds, 0);
    e.n_angles = std::max<int64_t>(n_angles, 0);
    if (e.graph) { cudaGraphExecDestroy(e.graph); e.graph = nullptr; }
    e.graph_valid = false;
    return KOMD_OK;
}

int komd_gpu_download(komd_gpu *h, double *r, double *v, double *f) {
    if (!h || !h->e.have_sites) return fail(KOMD_ERR_STATE, "no sites uploaded");
    Engine &e = h->e;
    if (r) CK(cudaMemcpyAsync(r, e.r, sizeof(double) * 3 * e.n, cudaMemcpyDeviceToHost, e.stream));
    if (v) CK(cudaMemcpyAsync(v, e.v, sizeof(double) * 3 * e.n, cudaMemcpyDeviceToHost, e.stream));
    if (f) CK(cudaMemcpyAsync(f, e.f, sizeof(double) * 3 * e.n, cudaMemcpyDeviceToHost, e.stream));
    CK(cudaStreamSynchronize(e.stream));
    return KOMD_OK;
}

int komd_gpu_update_container(komd_gpu *h) {
    if (!h || !h->e.have_sites) return fail(KOMD_ERR_STATE, "no sites uploaded");
    Engine &e = h->e;
    for (int attempt = 0; attempt < 6; attempt++) {
        {
            ProfScope ps(h, F_CONTAINER);
            launch_rebuild(h);
        }
        CK(cudaMemsetAsync(e.f, 0, sizeof(double) * 3 * e.n, e.stream));   // FReset_Kernel
        int rc = check_launch("update_container");
        if (rc) return rc;
        int flags[E_NFLAGS];
        rc = read_flags(h, flags, false);
        if (rc) return rc;
        if (!flags[E_VL_OVERFLOW]) break;
        CK(cudaMemsetAsync(e.err, 0, sizeof(int) * E_NFLAGS, e.stream));
        if (e.vl_cap >= 2048) return fail(KOMD_ERR_OVERFLOW, "Verlet list exceeds 2048 entries per site");
        rc = alloc_verlet(h, std::min(2048, e.vl_cap * 2));   // grow and rebuild
        if (rc) return rc;
    }
    e.have_cells = true;
    e.have_forces = false;
    return KOMD_OK;
}

int komd_gpu_forces(komd_gpu *h) {
    if (!h || !h->e.have_cells) return fail(KOMD_ERR_STATE, "update_container must run before forces");
    Engine &e = h->e;
    for (int attempt = 0; attempt < 6; attempt++) {
        enqueue_forces(h, false, nullptr);
        int rc = check_launch("forces");
        if (rc) return rc;
        int flags[E_NFLAGS];
        rc = read_flags(h, flags, true);
        if (rc) return rc;
        if (!flags[E_ATM_OVERFLOW]) {
            e.have_forces = true;
            return KOMD_OK;
        }
        if (e.nl_cap >= 1024) break;
        rc = alloc_atm_list(h, std::min(1024, e.nl_cap * 2));   // grow and recompute
        if (rc) return rc;
    }
    return fail(KOMD_ERR_OVERFLOW, "ATM neighbour list exceeds 1024 entries per site");
}

int komd_gpu_integrate0(komd_gpu *h) {
    if (!h || !h->e.have_sites) return fail(KOMD_ERR_STATE, "no sites uploaded");
    {
        ProfScope ps(h, F_INTEGRATE);
        launch_step0(h->e, h->e.stream);
    }
    int rc = check_launch("integrate0");
    if (rc) return rc;
    CK(cudaStreamSynchronize(h->e.stream));
    h->e.have_cells = h->e.have_forces = false;
    return KOMD_OK;
}

int komd_gpu_integrate1(komd_gpu *h) {
    if (!h || !h->e.have_sites) return fail(KOMD_ERR_STATE, "no sites uploaded");
    {
        ProfScope ps(h, F_INTEGRATE);
        launch_step1(h->e, h->e.stream);
    }
    int rc = check_launch("integrate1");
    if (rc) return rc;
    CK(cudaStreamSynchronize(h->e.stream));
    return KOMD_OK;
}

static int finish_steps(komd_gpu *h) {
    int flags[E_NFLAGS];
    int rc = read_flags(h, flags, true);
    if (rc) return rc;
    if (flags[E_ATM_OVERFLOW])
        return fail(KOMD_ERR_OVERFLOW, "ATM neighbour list overflowed during the steps (raise atm_list_cap)");
    if (flags[E_VL_OVERFLOW])
        return fail(KOMD_ERR_OVERFLOW, "Verlet list overflowed during the steps (density rose; call update_container)");
    if (flags[E_NONFINITE]) return fail(KOMD_ERR_NONFINITE, "non-finite velocity after a step");
    return KOMD_OK;
}

// exact-ATM probe of the learned term at the current state (the ATM list of
// this step is current): relative force RMSE; a breach switches to exact ATM
static int run_probe(komd_gpu *h) {
    Engine &e = h->e;
    Surrogate &u = h->sur;
    ProfScope ps(h, F_PROBE);
    double *keep = e.f;
    CK(cudaMemsetAsync(u.fprobe, 0, sizeof(double) * 3 * e.n, e.stream));
    e.f = u.fprobe;
    launch_atm(e, e.stream, false);
    e.f = keep;
    enqueue_surrogate(h, u.fsur_d);
    CK(cudaMemsetAsync(u.probe_acc, 0, 2 * sizeof(double), e.stream));
    launch_sur_probe((int)e.n, u.fsur_d, u.fprobe, u.probe_acc, e.stream);
    double acc[2];
    CK(cudaMemcpyAsync(acc, u.probe_acc, sizeof(acc), cudaMemcpyDeviceToHost, e.stream));
    CK(cudaStreamSynchronize(e.stream));
    u.probes++;
    u.last_rmse = acc[1] > 0 ? std::sqrt(acc[0] / acc[1]) : 0.0;
    u.max_rmse = std::max(u.max_rmse, u.last_rmse);
    if (!(u.last_rmse <= u.probe_threshold)) {
        u.fallback = true;
        u.fallback_step = u.steps;
        if (e.graph) { cudaGraphExecDestroy(e.graph); e.graph = nullptr; }
        e.graph_valid = false;
    }
    return KOMD_OK;
}

// one step captured into *out (replacing it)
static int capture_step(komd_gpu *h, cudaGraphExec_t *out) {
    Engine &e = h->e;
    cudaGraph_t graph;
    CK(cudaStreamBeginCapture(e.stream, cudaStreamCaptureModeThreadLocal));
    enqueue_step(h);
    CK(cudaStreamEndCapture(e.stream, &graph));
    if (*out) cudaGraphExecDestroy(*out);
    *out = nullptr;
    const cudaError_t ie = cudaGraphInstantiate(out, graph, 0);
    cudaGraphDestroy(graph);
    if (ie != cudaSuccess) {
        *out = nullptr;
        return fail(KOMD_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ie));
    }
    return KOMD_OK;
}

// the step graph of the current configuration; every change that invalidates
// it (buffers, terms, list capacities ...) also retires graphs of its epoch
static int ensure_graph(komd_gpu *h) {
    Engine &e = h->e;
    if (e.graph_valid && e.graph) return KOMD_OK;
    const int rc = capture_step(h, &e.graph);
    if (rc) return rc;
    e.graph_valid = true;
    h->graph_epoch++;
    return KOMD_OK;
}

static int run_steps(komd_gpu *h, int64_t n_steps) {
    Engine &e = h->e;
    if (e.profiling) {
        for (int64_t k = 0; k < n_steps; k++) enqueue_step(h);
        return check_launch("step");
    }
    const int rc = ensure_graph(h);
    if (rc) return rc;
    for (int64_t k = 0; k < n_steps; k++) CK(cudaGraphLaunch(e.graph, e.stream));
    h->graph_steps += n_steps;
    return KOMD_OK;
}

int komd_gpu_step(komd_gpu *h, int64_t n_steps) {
    if (!h || !h->e.have_sites) return fail(KOMD_ERR_STATE, "no sites uploaded");
    Engine &e = h->e;
    if (!e.have_forces) return fail(KOMD_ERR_STATE, "call update_container and forces before step");
    if (n_steps <= 0) return KOMD_OK;
    Surrogate &u = h->sur;
    int64_t done = 0;
    while (done < n_steps) {
        int64_t chunk = n_steps - done;
        const bool probing = surrogate_on(h) && u.probe_every > 0;
        if (probing) chunk = std::min<int64_t>(chunk, u.probe_every - (u.steps % u.probe_every));
        const bool learned = surrogate_on(h);
        int rc = run_steps(h, chunk);
        if (rc) return rc;
        done += chunk;
        if (learned) u.steps += chunk;
        if (probing && u.steps % u.probe_every == 0) {
            rc = run_probe(h);
            if (rc) return rc;
        }
    }
    return finish_steps(h);
}

}  // extern "C"

namespace {
// the device address of a host buffer, if kernels can reach it: pinned (mapped)
// memory, or any host memory on a system whose GPU walks the host page tables
// (NVLink-C2C with address translation, as on Grace)
const double *device_view(komd_gpu *h, const double *p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type == cudaMemoryTypeHost && a.devicePointer) return static_cast<const double *>(a.devicePointer);
    if (a.type == cudaMemoryTypeUnregistered && h->pageable_access) return p;
    return nullptr;
}

// komd_gpu_step_host without copy-engine transfers: the step's drift kernel reads
// r and v from the caller's buffers and writes the new r back, and the flush
// that ends the step writes f and v, so the host traffic runs inside those
// kernels (and in both directions at once) instead of before and after the
// step.  Only for the step graph's fused path (Verlet list, single-site
// molecules, FULL FP32 ATM ending the step, no device thermostat, no learned
// term); *applies = false (nothing done) otherwise.
int step_host_direct(komd_gpu *h, int64_t n_steps, double *r, double *v, double *f, bool *applies) {
    Engine &e = h->e;
    *applies = false;
    if (!(e.verlet && e.fused_drift && e.atm_acc && (e.cfg.terms & KOMD_TERM_ATM) && !e.cfg.thermostat &&
          !surrogate_on(h) && e.have_forces && r && v && f))
        return KOMD_OK;
    const double *rin = device_view(h, r), *vin = device_view(h, v), *fo = device_view(h, f);
    if (!rin || !vin || !fo) return KOMD_OK;
    *applies = true;
    cudaPointerAttributes pa;
    const bool r_pinned = cudaPointerGetAttributes(&pa, r) == cudaSuccess && pa.type == cudaMemoryTypeHost;
    e.hout_r_async = r_pinned;
    double *rout = const_cast<double *>(rin), *vout = const_cast<double *>(vin), *fout = const_cast<double *>(fo);
    if (n_steps == 1) {
        // one launch per call: the step with these buffers bound, captured once
        // per step graph and set of buffers
        int rc = ensure_graph(h);
        if (rc) return rc;
        if (!(h->hgraph && h->hgraph_epoch == h->graph_epoch && h->hkey[0] == rin && h->hkey[1] == vin &&
              h->hkey[2] == fo)) {
            e.hin_r = rin;
            e.hin_v = vin;
            e.hout_r = rout; e.hout_v = vout; e.hout_f = fout;
            rc = capture_step(h, &h->hgraph);
            e.hin_r = e.hin_v = nullptr;
            e.hout_r = e.hout_v = e.hout_f = nullptr;
            if (rc) return rc;
            h->hgraph_epoch = h->graph_epoch;
            h->hkey[0] = rin;
            h->hkey[1] = vin;
            h->hkey[2] = fo;
        }
        CK(cudaGraphLaunch(h->hgraph, e.stream));
        h->graph_steps += 1;
        return finish_steps(h);
    }
    e.hin_r = rin;
    e.hin_v = vin;
    enqueue_step(h);
    e.hin_r = e.hin_v = nullptr;
    e.hout_r = e.hout_v = e.hout_f = nullptr;
    int rc = check_launch("step_host");
    if (!rc && n_steps > 2) rc = run_steps(h, n_steps - 2);
    if (!rc && n_steps > 1) {
        e.hout_r = rout; e.hout_v = vout; e.hout_f = fout;
        enqueue_step(h);
        e.hout_r = e.hout_v = e.hout_f = nullptr;
        rc = check_launch("step_host");
    }
    if (rc) return rc;
    return finish_steps(h);
}
}  // namespace

extern "C" {

int komd_gpu_step_host(komd_gpu *h, int64_t n_steps, double *r, double *v, double *f) {
    if (!h || !h->e.have_sites) return fail(KOMD_ERR_STATE, "no sites uploaded");
    Engine &e = h->e;
    if (n_steps > 0 && !e.profiling) {
        bool applies = false;
        const int rc = step_host_direct(h, n_steps, r, v, f, &applies);
        if (applies) return rc;
    }
    if (r) CK(cudaMemcpyAsync(e.r, r, sizeof(double) * 3 * e.n, cudaMemcpyHostToDevice, e.stream));
    if (v) CK(cudaMemcpyAsync(e.v, v, sizeof(double) * 3 * e.n, cudaMemcpyHostToDevice, e.stream));
    int rc = komd_gpu_step(h, n_steps);
    if (rc) return rc;
    return komd_gpu_download(h, r, v, f);
}

int komd_gpu_set_pair_table(komd_gpu *h, int32_t n, const double *x, const double *y, double below,
                            double above) {
    if (!h || !x || !y) return fail(KOMD_ERR_ARG, "null argument");
    Engine &e = h->e;
    if (!(e.cfg.terms & KOMD_TERM_TABULATED)) return fail(KOMD_ERR_ARG, "the engine was created without KOMD_TERM_TABULATED");
    if (n < 2) return fail(KOMD_ERR_ARG, "a table needs at least two nodes");
    for (int32_t k = 1; k < n; k++)
        if (!(x[k] > x[k - 1])) return fail(KOMD_ERR_ARG, "table nodes must be strictly ascending");
    CK(cudaStreamSynchronize(e.stream));
    if (n != e.tab_n) {
        CK(dalloc(e.tab_x, n));
        CK(dalloc(e.tab_y, n));
        CK(dalloc(e.tab_s, n));
        e.tab_n = n;
        if (e.graph) { cudaGraphExecDestroy(e.graph); e.graph = nullptr; }
        e.graph_valid = false;
    }
    // same-size tables are replaced in place: graphs already captured read the new values
    CK(cudaMemcpy(e.tab_x, x, sizeof(double) * n, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(e.tab_y, y, sizeof(double) * n, cudaMemcpyHostToDevice));
    // segment slopes, the quotient FunctionPL::evaluateAt forms (IBI_Math.h:30-44)
    std::vector<double> sl(n, 0.0);
    for (int32_t k = 0; k + 1 < n; k++) sl[k] = (y[k + 1] - y[k]) / (x[k + 1] - x[k]);
    CK(cudaMemcpy(e.tab_s, sl.data(), sizeof(double) * n, cudaMemcpyHostToDevice));
    if (e.tab_lo != below || e.tab_hi != above) {
        e.tab_lo = below;
        e.tab_hi = above;
        if (e.graph) { cudaGraphExecDestroy(e.graph); e.graph = nullptr; }
        e.graph_valid = false;
    }
    return KOMD_OK;
}

int komd_gpu_set_terms(komd_gpu *h, uint32_t terms) {
    if (!h) return fail(KOMD_ERR_ARG, "null handle");
    Engine &e = h->e;
    if (terms & ~(h->sensor_terms | KOMD_TERM_TABULATED))
        return fail(KOMD_ERR_ARG, "only KOMD_TERM_TABULATED can be added to the terms given at creation");
    if ((terms & KOMD_TERM_TABULATED) && e.verlet)
        return fail(KOMD_ERR_ARG, "the tabulated pair term runs on per-step cell lists (skin 0)");
    if ((terms & KOMD_TERM_ATM2B) && !(terms & KOMD_TERM_LJ))
        return fail(KOMD_ERR_ARG, "KOMD_TERM_ATM2B scales the LJ term: set KOMD_TERM_LJ");
    if ((terms & KOMD_TERM_ATM_SURROGATE) && !(terms & KOMD_TERM_ATM))
        return fail(KOMD_ERR_ARG, "the learned three-body term needs KOMD_TERM_ATM");
    if (terms == e.cfg.terms) return KOMD_OK;
    CK(cudaStreamSynchronize(e.stream));
    if ((terms & KOMD_TERM_TABULATED) && !e.posd) {
        h->want_posd = true;
        if (e.have_sites) {
            int rc = ensure_posd(h);
            if (rc) return rc;
            // fill the FP64 slot-ordered positions of the current cells; the
            // container pass is idempotent on wrapped positions and leaves f alone
            if (e.have_cells) launch_rebuild(h);
            rc = check_launch("set_terms");
            if (rc) return rc;
        }
    }
    e.cfg.terms = terms;
    if (e.graph) { cudaGraphExecDestroy(e.graph); e.graph = nullptr; }
    e.graph_valid = false;
    return KOMD_OK;
}

int komd_gpu_rdf_profile(komd_gpu *h, double max_r, int32_t nbins, double *bins) {
    if (!h || !bins || nbins <= 0 || !(max_r > 0)) return fail(KOMD_ERR_ARG, "bad argument");
    Engine &e = h->e;
    if (!e.have_cells) return fail(KOMD_ERR_STATE, "update_container must run first");
    cudaStream_t st = e.stream;
    if (e.verlet) launch_rebuild(h);   // the cells of the last rebuild may be stale
    if (nbins > h->prof_cap) {   // kept across calls: a profiler samples every step
        h->prof_cap = 0;
        if (dalloc(h->prof, nbins) != cudaSuccess) {
            h->prof = nullptr;
            return fail(KOMD_ERR_NOMEM, "rdf_profile histogram");
        }
        h->prof_cap = nbins;
    }
    double *d = h->prof;
    CK(cudaMemsetAsync(d, 0, sizeof(double) * nbins, st));
    const double dr = max_r / (double)nbins;   // RDF_Profiler.cpp:8
    launch_rdf_bins(e, st, d, max_r <= e.cfg.cell_size, max_r, dr, nbins);
    int rc = check_launch("rdf_profile");
    std::vector<double> hb(nbins);
    if (!rc) {
        const cudaError_t ce = cudaMemcpyAsync(hb.data(), d, sizeof(double) * nbins, cudaMemcpyDeviceToHost, st);
        const cudaError_t se = cudaStreamSynchronize(st);
        if (ce != cudaSuccess || se != cudaSuccess) rc = fail(KOMD_ERR_CUDA, "rdf_profile copy");
    }
    if (rc) return rc;
    for (int32_t k = 0; k < nbins; k++) bins[k] += hb[k];
    return KOMD_OK;
}

int komd_gpu_scale_velocities(komd_gpu *h, double beta) {
    if (!h || !h->e.have_sites) return fail(KOMD_ERR_STATE, "no sites uploaded");
    if (!std::isfinite(beta)) return fail(KOMD_ERR_ARG, "non-finite scaling factor");
    launch_velocity_scale(h->e, h->e.stream, nullptr, beta);
    int rc = check_launch("scale_velocities");
    if (rc) return rc;
    CK(cudaStreamSynchronize(h->e.stream));
    return KOMD_OK;
}

int64_t komd_gpu_rdf_bins(komd_gpu *h) { return h ? h->e.rdf_bins : -1; }

int komd_gpu_measure(komd_gpu *h, uint32_t mask, komd_observables *obs, double *rdf, double *lj_hist) {
    if (!h || !obs) return fail(KOMD_ERR_ARG, "null argument");
    if (!h->e.have_cells) return fail(KOMD_ERR_STATE, "update_container must run before measure");
    std::memset(obs, 0, sizeof(*obs));
    double acc[R_NSLOTS];
    int rc = measure_enqueue(h, mask, acc, rdf, lj_hist);
    if (rc) return rc;
    CK(cudaStreamSynchronize(h->e.stream));
    int flags[E_NFLAGS];
    rc = read_flags(h, flags, true);
    if (rc) return rc;
    if (flags[E_ATM_OVERFLOW]) return fail(KOMD_ERR_OVERFLOW, "ATM neighbour list overflow during measure");
    measure_fill(acc, obs);
    return KOMD_OK;
}

int komd_gpu_get_cells(komd_gpu *h, int64_t *count, int64_t ncell, int64_t *idx, int64_t cap, int64_t *total) {
    if (!h || !h->e.have_cells) return fail(KOMD_ERR_STATE, "update_container must run first");
    Engine &e = h->e;
    const int nx = e.g.nd[0] + 2, ny = e.g.nd[1] + 2, nz = e.g.nd[2] + 2;
    const int64_t nall = (int64_t)nx * ny * nz;
    std::vector<int> start(e.g.ncell + 1), slot_site(e.n);
    CK(cudaMemcpy(start.data(), e.cell_start, sizeof(int) * (e.g.ncell + 1), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(slot_site.data(), e.slot_site, sizeof(int) * e.n, cudaMemcpyDeviceToHost));
    int64_t need = 0, w = 0;
    for (int z = 0; z < nz; z++)
        for (int y = 0; y < ny; y++)
            for (int x = 0; x < nx; x++) {
                // halo layer 0 copies domain cell nd, layer nd+1 copies cell 1 (LinkedCells.cpp:105-120)
                auto src = [](int c, int nd) { return c == 0 ? nd - 1 : (c == nd + 1 ? 0 : c - 1); };
                const int dc = src(x, e.g.nd[0]) + e.g.nd[0] * (src(y, e.g.nd[1]) + e.g.nd[1] * src(z, e.g.nd[2]));
                const int64_t lin = x + (int64_t)nx * (y + (int64_t)ny * z);
                const int s0 = start[dc], s1 = start[dc + 1];
                if (count && lin < ncell) count[lin] = s1 - s0;
                for (int s = s0; s < s1; s++) {
                    if (idx && w < cap) idx[w] = slot_site[s];
                    w++;
                }
                need += s1 - s0;
            }
    if (total) *total = need;
    if (count && ncell < nall) return fail(KOMD_ERR_ARG, "count array too small for (nd+2)^3 cells");
    return KOMD_OK;
}

int komd_gpu_neighbour_counts(komd_gpu *h, int64_t *counts) {
    if (!h || !counts) return fail(KOMD_ERR_ARG, "null argument");
    Engine &e = h->e;
    if (!e.have_cells) return fail(KOMD_ERR_STATE, "update_container must run first");
    if (!e.posd) {
        h->want_posd = true;
        int rc = ensure_posd(h);
        if (rc) return rc;
    }
    launch_rebuild(h);   // cells and FP64 positions of the current state (positions are already wrapped)
    launch_counts(e, e.stream);
    int rc = check_launch("neighbour_counts");
    if (rc) return rc;
    CK(cudaMemcpyAsync(counts, e.counts, sizeof(int64_t) * e.n, cudaMemcpyDeviceToHost, e.stream));
    CK(cudaStreamSynchronize(e.stream));
    return KOMD_OK;
}

int komd_gpu_surrogate_load(komd_gpu *h, const float *params, const float *fmean, const float *fstd,
                            double e_scale, double e_shift, int32_t probe_every, double probe_threshold) {
    if (!h || !params || !fmean || !fstd) return fail(KOMD_ERR_ARG, "null argument");
    Engine &e = h->e;
    if (!e.have_sites) return fail(KOMD_ERR_STATE, "no sites uploaded");
    if (!(e.cfg.terms & KOMD_TERM_ATM)) return fail(KOMD_ERR_ARG, "the learned three-body term needs KOMD_TERM_ATM");
    if (e.cfg.precision != KOMD_FP32) return fail(KOMD_ERR_ARG, "the learned three-body term runs in FP32 mode");
    Surrogate &u = h->sur;
    const int H = kSurH, F = kSurNF;
    const float *W1 = params, *b1 = W1 + H * F, *W2 = b1 + H, *b2 = W2 + H * H, *w3 = b2 + H, *b3 = w3 + H;
    // BF16 weights in the MMA B-fragment order of surrogate.cu (load_frag):
    // element (n, k) of an N x K matrix given by at(n, k)
    auto frag = [](int N, int K, auto at) {
        std::vector<__nv_bfloat16> out((size_t)N * K);
        const int S = K / 16;
        for (int t = 0; t < N / 8; t++)
            for (int s = 0; s < S; s++)
                for (int lane = 0; lane < 32; lane++) {
                    const int n = 8 * t + lane / 4, k0 = 16 * s + 2 * (lane % 4);
                    __nv_bfloat16 *o = out.data() + ((size_t)(t * S + s) * 32 + lane) * 4;
                    o[0] = __float2bfloat16(at(n, k0));
                    o[1] = __float2bfloat16(at(n, k0 + 1));
                    o[2] = __float2bfloat16(at(n, k0 + 8));
                    o[3] = __float2bfloat16(at(n, k0 + 9));
                }
        return out;
    };
    const std::vector<__nv_bfloat16> w1 = frag(H, F, [&](int n, int k) { return W1[n * F + k]; });
    const std::vector<__nv_bfloat16> w1t = frag(F, H, [&](int n, int k) { return W1[k * F + n]; });
    const std::vector<__nv_bfloat16> w2 = frag(H, H, [&](int n, int k) { return W2[n * H + k]; });
    const std::vector<__nv_bfloat16> w2t = frag(H, H, [&](int n, int k) { return W2[k * H + n]; });
    CK(dalloc(u.w1, w1.size())); CK(dalloc(u.w1t, w1t.size())); CK(dalloc(u.w2, w2.size())); CK(dalloc(u.w2t, w2t.size()));
    CK(dalloc(u.b1, H)); CK(dalloc(u.b2, H)); CK(dalloc(u.w3, H)); CK(dalloc(u.fmean, F)); CK(dalloc(u.fstd, F));
    CK(cudaMemcpy(u.w1, w1.data(), sizeof(__nv_bfloat16) * w1.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(u.w1t, w1t.data(), sizeof(__nv_bfloat16) * w1t.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(u.w2, w2.data(), sizeof(__nv_bfloat16) * w2.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(u.w2t, w2t.data(), sizeof(__nv_bfloat16) * w2t.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(u.b1, b1, sizeof(float) * H, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(u.b2, b2, sizeof(float) * H, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(u.w3, w3, sizeof(float) * H, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(u.fmean, fmean, sizeof(float) * F, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(u.fstd, fstd, sizeof(float) * F, cudaMemcpyHostToDevice));
    u.b3 = b3[0];
    u.e_scale = (float)e_scale;
    u.e_shift = (float)e_shift;
    CK(dalloc(u.x, (size_t)e.n * kSurNF)); CK(dalloc(u.mom, (size_t)e.n * kSurNC * 9));
    CK(dalloc(u.dedx, (size_t)e.n * kSurNF)); CK(dalloc(u.esite, e.n)); CK(dalloc(u.fsur, 4 * (size_t)e.n));
    CK(dalloc(u.fprobe, 3 * (size_t)e.n)); CK(dalloc(u.fsur_d, 3 * (size_t)e.n)); CK(dalloc(u.probe_acc, 2));
    CK(cudaMemset(u.fsur, 0, sizeof(float) * 4 * e.n));
    u.probe_every = probe_every;
    u.probe_threshold = probe_threshold;
    u.loaded = true;
    u.fallback = false;
    u.steps = u.probes = 0;
    u.last_rmse = -1.0;
    u.max_rmse = 0.0;
    u.fallback_step = -1;
    if (e.graph) { cudaGraphExecDestroy(e.graph); e.graph = nullptr; }
    e.graph_valid = false;
    return KOMD_OK;
}

int komd_gpu_surrogate_sample(komd_gpu *h, float *features, double *e3, double *f3) {
    if (!h) return fail(KOMD_ERR_ARG, "null handle");
    Engine &e = h->e;
    if (!e.have_cells) return fail(KOMD_ERR_STATE, "update_container must run first");
    if (!(e.cfg.terms & KOMD_TERM_ATM) || e.cfg.precision != KOMD_FP32)
        return fail(KOMD_ERR_ARG, "samples need KOMD_TERM_ATM in FP32 mode");
    Surrogate &u = h->sur;
    if (!u.x) {
        CK(dalloc(u.x, (size_t)e.n * kSurNF)); CK(dalloc(u.mom, (size_t)e.n * kSurNC * 9));
        CK(dalloc(u.fprobe, 3 * (size_t)e.n));
    }
    double *e3d = nullptr;
    CK(dalloc(e3d, e.n));
    CK(cudaMemsetAsync(e3d, 0, sizeof(double) * e.n, e.stream));
    double *keep = e.f;
    e.f = u.fprobe;
    launch_pair(e, e.stream, false, nullptr);                  // ATM neighbour list of this state
    CK(cudaMemsetAsync(u.fprobe, 0, sizeof(double) * 3 * e.n, e.stream));
    e.atm_esite = e3d;
    launch_atm(e, e.stream, true);                             // exact forces and per-site energies
    e.atm_esite = nullptr;
    e.f = keep;
    SurParams p = sur_params(h);
    p.fmean = nullptr;
    p.fstd = nullptr;                                          // raw features
    launch_sur_desc(p, e.stream);
    int rc = check_launch("surrogate_sample");
    if (rc) { dfree(e3d); return rc; }
    std::vector<float> xs((size_t)e.n * kSurNF);
    std::vector<int> slot_site(e.n);
    CK(cudaMemcpyAsync(xs.data(), u.x, sizeof(float) * xs.size(), cudaMemcpyDeviceToHost, e.stream));
    CK(cudaMemcpyAsync(slot_site.data(), e.slot_site, sizeof(int) * e.n, cudaMemcpyDeviceToHost, e.stream));
    if (e3) CK(cudaMemcpyAsync(e3, e3d, sizeof(double) * e.n, cudaMemcpyDeviceToHost, e.stream));
    if (f3) CK(cudaMemcpyAsync(f3, u.fprobe, sizeof(double) * 3 * e.n, cudaMemcpyDeviceToHost, e.stream));
    CK(cudaStreamSynchronize(e.stream));
    dfree(e3d);
    if (features)
        for (int64_t slot = 0; slot < e.n; slot++)
            std::memcpy(features + (size_t)slot_site[slot] * kSurNF, xs.data() + (size_t)slot * kSurNF,
                        sizeof(float) * kSurNF);
    int flags[E_NFLAGS];
    rc = read_flags(h, flags, true);
    if (rc) return rc;
    if (flags[E_ATM_OVERFLOW]) return fail(KOMD_ERR_OVERFLOW, "ATM neighbour list overflow");
    return KOMD_OK;
}

int komd_gpu_surrogate_forces(komd_gpu *h, double *f3, double *e3) {
    if (!h) return fail(KOMD_ERR_ARG, "null handle");
    Engine &e = h->e;
    Surrogate &u = h->sur;
    if (!u.loaded) return fail(KOMD_ERR_STATE, "komd_gpu_surrogate_load first");
    if (!e.have_cells) return fail(KOMD_ERR_STATE, "update_container must run first");
    double *keep = e.f;
    e.f = u.fprobe;
    launch_pair(e, e.stream, false, nullptr);                  // ATM neighbour list of this state
    e.f = keep;
    CK(cudaMemsetAsync(u.fsur_d, 0, sizeof(double) * 3 * e.n, e.stream));
    enqueue_surrogate(h, u.fsur_d);
    int rc = check_launch("surrogate_forces");
    if (rc) return rc;
    std::vector<float> es(e.n);
    std::vector<int> slot_site(e.n);
    if (f3) CK(cudaMemcpyAsync(f3, u.fsur_d, sizeof(double) * 3 * e.n, cudaMemcpyDeviceToHost, e.stream));
    CK(cudaMemcpyAsync(es.data(), u.esite, sizeof(float) * e.n, cudaMemcpyDeviceToHost, e.stream));
    CK(cudaMemcpyAsync(slot_site.data(), e.slot_site, sizeof(int) * e.n, cudaMemcpyDeviceToHost, e.stream));
    CK(cudaStreamSynchronize(e.stream));
    if (e3)
        for (int64_t slot = 0; slot < e.n; slot++) e3[slot_site[slot]] = es[slot];
    return KOMD_OK;
}

int komd_gpu_surrogate_status(komd_gpu *h, komd_surrogate_status *st) {
    if (!h || !st) return fail(KOMD_ERR_ARG, "null argument");
    const Surrogate &u = h->sur;
    st->steps = u.steps;
    st->probes = u.probes;
    st->last_rmse = u.last_rmse;
    st->max_rmse = u.max_rmse;
    st->fallback = u.fallback ? 1 : 0;
    st->fallback_step = u.fallback_step;
    return KOMD_OK;
}

namespace {
struct TrainBuffers {
    float *X = nullptr, *y = nullptr, *params = nullptr, *grad = nullptr, *m = nullptr, *v = nullptr, *work = nullptr;
    ~TrainBuffers() { dfree(X); dfree(y); dfree(params); dfree(grad); dfree(m); dfree(v); dfree(work); }
};

int train_setup(TrainBuffers &b, TrainParams &t, const float *X, const float *y, int64_t n, const float *params,
                int batch) {
    if (n <= 0 || n > (1LL << 31) - 1 || batch <= 0) return fail(KOMD_ERR_ARG, "bad sample or batch count");
    const int stride = kSurNF + 4 * kSurH + 2;
    CK(dalloc(b.X, (size_t)n * kSurNF)); CK(dalloc(b.y, n)); CK(dalloc(b.params, kSurNParam));
    CK(dalloc(b.grad, kSurNParam + 1)); CK(dalloc(b.m, kSurNParam)); CK(dalloc(b.v, kSurNParam));
    CK(dalloc(b.work, (size_t)batch * stride));
    CK(cudaMemcpy(b.X, X, sizeof(float) * (size_t)n * kSurNF, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(b.y, y, sizeof(float) * n, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(b.params, params, sizeof(float) * kSurNParam, cudaMemcpyHostToDevice));
    CK(cudaMemset(b.m, 0, sizeof(float) * kSurNParam));
    CK(cudaMemset(b.v, 0, sizeof(float) * kSurNParam));
    t.X = b.X; t.y = b.y; t.n = (int)n; t.batch = batch; t.params = b.params; t.grad = b.grad;
    t.m = b.m; t.v = b.v; t.work = b.work; t.lr = 0.f; t.seed = 0; t.fixed_batch = 0; t.grad_only = 0;
    return KOMD_OK;
}
}  // namespace

int komd_mlp_train(const float *X, const float *y, int64_t n, float *params, int32_t epochs, int32_t batch, float lr,
                   uint64_t seed, float *loss) {
    if (!X || !y || !params || epochs < 0) return fail(KOMD_ERR_ARG, "null argument");
    TrainBuffers b;
    TrainParams t;
    int rc = train_setup(b, t, X, y, n, params, batch);
    if (rc) return rc;
    t.lr = lr;
    t.seed = (uint32_t)(seed ^ (seed >> 32));
    const int64_t steps_per_epoch = std::max<int64_t>(1, n / batch);
    int step = 0;
    for (int ep = 0; ep < epochs; ep++) {
        double sq = 0.0;
        for (int64_t k = 0; k < steps_per_epoch; k++) {
            launch_train_step(t, step++, nullptr);
            if (loss && k == steps_per_epoch - 1) {
                // the last batch's squared error stands for the epoch (one readback per epoch)
                float s2 = 0.f;
                CK(cudaMemcpy(&s2, b.grad + kSurNParam, sizeof(float), cudaMemcpyDeviceToHost));
                sq = s2;
            }
        }
        rc = check_launch("mlp_train");
        if (rc) return rc;
        if (loss) loss[ep] = (float)(sq / batch);
    }
    CK(cudaMemcpy(params, b.params, sizeof(float) * kSurNParam, cudaMemcpyDeviceToHost));
    return KOMD_OK;
}

int komd_mlp_loss_grad(const float *X, const float *y, int64_t n, const float *params, float *grad, float *loss) {
    if (!X || !y || !params || !grad) return fail(KOMD_ERR_ARG, "null argument");
    TrainBuffers b;
    TrainParams t;
    int rc = train_setup(b, t, X, y, n, params, (int)n);
    if (rc) return rc;
    t.fixed_batch = 1;
    t.grad_only = 1;
    launch_train_step(t, 0, nullptr);
    rc = check_launch("mlp_loss_grad");
    if (rc) return rc;
    std::vector<float> g(kSurNParam + 1);
    CK(cudaMemcpy(g.data(), b.grad, sizeof(float) * g.size(), cudaMemcpyDeviceToHost));
    std::memcpy(grad, g.data(), sizeof(float) * kSurNParam);
    if (loss) *loss = g[kSurNParam] / (float)n;
    return KOMD_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// force-matched training: snapshot dataset on the device (sur_train.cu)
// ---------------------------------------------------------------------------
struct komd_sur_data {
    int device = 0;
    int cap = 0, n_site = 0;
    float rc = 0.f;
    int64_t n_snap = 0, snap_cap = 0;
    float4 *nl = nullptr;
    int *count = nullptr, *site = nullptr, *err = nullptr;
    float *x = nullptr, *mom = nullptr, *e3 = nullptr, *f3 = nullptr;
    ~komd_sur_data() {
        cudaSetDevice(device);
        dfree(nl); dfree(count); dfree(site); dfree(err); dfree(x); dfree(mom); dfree(e3); dfree(f3);
    }
};

namespace {
template <typename T>
cudaError_t dgrow(T *&p, size_t old_count, size_t new_count) {
    T *q = nullptr;
    cudaError_t rc = cudaMalloc(reinterpret_cast<void **>(&q), sizeof(T) * new_count);
    if (rc != cudaSuccess) return rc;
    if (p && old_count) rc = cudaMemcpy(q, p, sizeof(T) * old_count, cudaMemcpyDeviceToDevice);
    if (p) cudaFree(p);
    p = q;
    return rc;
}

int data_reserve(komd_sur_data *d, int64_t snaps) {
    if (snaps <= d->snap_cap) return KOMD_OK;
    const int64_t cap = std::max<int64_t>(snaps, 2 * d->snap_cap);
    const size_t o = (size_t)d->snap_cap * d->n_site, n = (size_t)cap * d->n_site;
    CK(dgrow(d->nl, o * d->cap, n * d->cap));
    CK(dgrow(d->count, o, n)); CK(dgrow(d->site, o, n));
    CK(dgrow(d->x, o * kSurNF, n * kSurNF)); CK(dgrow(d->mom, o * kSurNC * 9, n * kSurNC * 9));
    CK(dgrow(d->e3, o, n)); CK(dgrow(d->f3, 3 * o, 3 * n));
    d->snap_cap = cap;
    return KOMD_OK;
}

struct FitBuffers {
    int *snaps = nullptr;
    float *params = nullptr, *grad = nullptr, *m = nullptr, *v = nullptr, *fmean = nullptr, *fstd = nullptr;
    float *E = nullptr, *g = nullptr, *fs = nullptr, *w = nullptr, *rec = nullptr;
    double *loss = nullptr;
    __nv_bfloat16 *wf = nullptr;
    ~FitBuffers() {
        dfree(snaps); dfree(params); dfree(grad); dfree(m); dfree(v); dfree(fmean); dfree(fstd);
        dfree(E); dfree(g); dfree(fs); dfree(w); dfree(rec); dfree(loss); dfree(wf);
    }
};

int fit_setup(komd_sur_data *d, FitBuffers &b, FitParams &p, const float *params, const float *fmean,
              const float *fstd, double e_scale, double e_shift, double f2, float lam_e, float lam_f, int64_t n_snaps,
              int batch_snaps, int precision) {
    if (!d || !params || !fmean || !fstd) return fail(KOMD_ERR_ARG, "null argument");
    if (precision != KOMD_FIT_BF16 && precision != KOMD_FIT_FP32) return fail(KOMD_ERR_ARG, "unknown precision");
    if (d->n_snap <= 0) return fail(KOMD_ERR_STATE, "the dataset holds no snapshots");
    if (!(e_scale > 0.0) || !(f2 > 0.0)) return fail(KOMD_ERR_ARG, "e_scale and f2 must be positive");
    CK(cudaSetDevice(d->device));
    const int64_t nb = (int64_t)batch_snaps * d->n_site;
    if (nb > (1LL << 30)) return fail(KOMD_ERR_ARG, "batch too large");
    CK(dalloc(b.snaps, n_snaps)); CK(dalloc(b.params, kSurNParam)); CK(dalloc(b.grad, kSurNParam));
    CK(dalloc(b.m, kSurNParam)); CK(dalloc(b.v, kSurNParam)); CK(dalloc(b.fmean, kSurNF)); CK(dalloc(b.fstd, kSurNF));
    CK(dalloc(b.E, nb)); CK(dalloc(b.g, nb * kSurNF)); CK(dalloc(b.fs, 3 * nb)); CK(dalloc(b.w, nb * kSurNF));
    CK(dalloc(b.rec, nb * kFitRec)); CK(dalloc(b.loss, 2)); CK(dalloc(b.wf, kFitWf));
    CK(cudaMemcpy(b.params, params, sizeof(float) * kSurNParam, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(b.fmean, fmean, sizeof(float) * kSurNF, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(b.fstd, fstd, sizeof(float) * kSurNF, cudaMemcpyHostToDevice));
    CK(cudaMemset(b.m, 0, sizeof(float) * kSurNParam));
    CK(cudaMemset(b.v, 0, sizeof(float) * kSurNParam));
    CK(cudaMemset(b.loss, 0, sizeof(double) * 2));
    p.nl = d->nl; p.nl_count = d->count; p.cap = d->cap; p.n_site = d->n_site; p.nb = (int)nb; p.rc = d->rc;
    p.x = d->x; p.mom = d->mom; p.e3 = d->e3; p.f3 = d->f3; p.snaps = b.snaps;
    p.params = b.params; p.fmean = b.fmean; p.fstd = b.fstd;
    p.e_scale = (float)e_scale; p.e_shift = (float)e_shift;
    p.lam_e = lam_e; p.lam_f = lam_f; p.inv_f2 = (float)(1.0 / f2);
    p.E = b.E; p.g = b.g; p.fs = b.fs; p.w = b.w; p.rec = b.rec; p.loss = b.loss;
    p.wf = b.wf; p.tc = precision == KOMD_FIT_BF16 ? 1 : 0;
    return KOMD_OK;
}

uint64_t splitmix(uint64_t &s) {
    uint64_t z = (s += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
}  // namespace

extern "C" {

int komd_sur_data_create(int32_t device, int32_t nl_cap, komd_sur_data **out) {
    if (!out || nl_cap <= 0 || nl_cap > 4096) return fail(KOMD_ERR_ARG, "bad argument");
    CK(cudaSetDevice(device));
    komd_sur_data *d = new komd_sur_data();
    d->device = device;
    d->cap = nl_cap;
    if (cudaMalloc(reinterpret_cast<void **>(&d->err), sizeof(int)) != cudaSuccess) {
        delete d;
        return fail(KOMD_ERR_NOMEM, "device allocation failed");
    }
    cudaMemset(d->err, 0, sizeof(int));
    *out = d;
    return KOMD_OK;
}

void komd_sur_data_destroy(komd_sur_data *d) { delete d; }

int64_t komd_sur_data_snapshots(const komd_sur_data *d) { return d ? d->n_snap : -1; }
int32_t komd_sur_data_sites(const komd_sur_data *d) { return d ? d->n_site : -1; }

int komd_gpu_surrogate_capture(komd_gpu *h, komd_sur_data *d) {
    if (!h || !d) return fail(KOMD_ERR_ARG, "null argument");
    Engine &e = h->e;
    if (!e.have_cells) return fail(KOMD_ERR_STATE, "update_container must run first");
    if (!(e.cfg.terms & KOMD_TERM_ATM) || e.cfg.precision != KOMD_FP32)
        return fail(KOMD_ERR_ARG, "captures need KOMD_TERM_ATM in FP32 mode");
    if (e.device != d->device) return fail(KOMD_ERR_ARG, "dataset and engine live on different devices");
    if (e.n > (1 << 24)) return fail(KOMD_ERR_ARG, "snapshots are limited to 2^24 sites");
    if (d->n_snap == 0) {
        d->n_site = (int)e.n;
        d->rc = (float)e.cfg.cutoff_3b;
    } else if (d->n_site != (int)e.n || d->rc != (float)e.cfg.cutoff_3b) {
        return fail(KOMD_ERR_ARG, "all snapshots of a dataset need the same site count and three-body cutoff");
    }
    int rc = data_reserve(d, d->n_snap + 1);
    if (rc) return rc;
    Surrogate &u = h->sur;
    if (!u.x) {
        CK(dalloc(u.x, (size_t)e.n * kSurNF)); CK(dalloc(u.mom, (size_t)e.n * kSurNC * 9));
        CK(dalloc(u.fprobe, 3 * (size_t)e.n));
    }
    double *e3d = nullptr;
    CK(dalloc(e3d, e.n));
    CK(cudaMemsetAsync(e3d, 0, sizeof(double) * e.n, e.stream));
    double *keep = e.f;
    e.f = u.fprobe;
    launch_pair(e, e.stream, false, nullptr);                  // ATM neighbour list of this state
    CK(cudaMemsetAsync(u.fprobe, 0, sizeof(double) * 3 * e.n, e.stream));
    e.atm_esite = e3d;
    launch_atm(e, e.stream, true);                             // exact forces and per-site energies
    e.atm_esite = nullptr;
    e.f = keep;
    SurParams p = sur_params(h);
    p.fmean = nullptr;
    p.fstd = nullptr;
    launch_sur_desc(p, e.stream);
    const size_t o = (size_t)d->n_snap * d->n_site;
    launch_fit_capture((int)e.n, e.nl, e.nl_count, e.nl_cap, u.x, u.mom, e3d, u.fprobe, e.slot_site,
                       d->nl + o * d->cap, d->count + o, d->cap, d->x + o * kSurNF, d->mom + o * kSurNC * 9,
                       d->e3 + o, d->f3 + 3 * o, d->site + o, d->err, e.stream);
    rc = check_launch("surrogate_capture");
    int derr = 0;
    if (!rc) {
        CK(cudaMemcpyAsync(&derr, d->err, sizeof(int), cudaMemcpyDeviceToHost, e.stream));
        CK(cudaStreamSynchronize(e.stream));
    }
    dfree(e3d);
    if (rc) return rc;
    int flags[E_NFLAGS];
    rc = read_flags(h, flags, true);
    if (rc) return rc;
    if (flags[E_ATM_OVERFLOW]) return fail(KOMD_ERR_OVERFLOW, "ATM neighbour list overflow");
    if (derr) {
        cudaMemset(d->err, 0, sizeof(int));
        return fail(KOMD_ERR_OVERFLOW, "a site has more neighbours than the dataset's nl_cap");
    }
    d->n_snap++;
    return KOMD_OK;
}

int komd_sur_data_get(komd_sur_data *d, int64_t snap, float *features, float *e3, float *f3, int32_t *site) {
    if (!d) return fail(KOMD_ERR_ARG, "null dataset");
    if (snap >= d->n_snap) return fail(KOMD_ERR_ARG, "snapshot index out of range");
    CK(cudaSetDevice(d->device));
    const size_t o = snap < 0 ? 0 : (size_t)snap * d->n_site;
    const size_t n = snap < 0 ? (size_t)d->n_snap * d->n_site : (size_t)d->n_site;
    if (features) CK(cudaMemcpy(features, d->x + o * kSurNF, sizeof(float) * n * kSurNF, cudaMemcpyDeviceToHost));
    if (e3) CK(cudaMemcpy(e3, d->e3 + o, sizeof(float) * n, cudaMemcpyDeviceToHost));
    if (f3) CK(cudaMemcpy(f3, d->f3 + 3 * o, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost));
    if (site) CK(cudaMemcpy(site, d->site + o, sizeof(int) * n, cudaMemcpyDeviceToHost));
    return KOMD_OK;
}

int komd_sur_fit_grad(komd_sur_data *d, const float *params, const float *fmean, const float *fstd, double e_scale,
                      double e_shift, double f2, float lam_e, float lam_f, float *grad, double *loss,
                      int32_t precision) {
    if (!grad) return fail(KOMD_ERR_ARG, "null argument");
    FitBuffers b;
    FitParams p;
    int rc = fit_setup(d, b, p, params, fmean, fstd, e_scale, e_shift, f2, lam_e, lam_f, d ? d->n_snap : 0,
                       d ? (int)d->n_snap : 0, precision);
    if (rc) return rc;
    std::vector<int> ids((size_t)d->n_snap);
    for (int64_t k = 0; k < d->n_snap; k++) ids[k] = (int)k;
    CK(cudaMemcpy(b.snaps, ids.data(), sizeof(int) * ids.size(), cudaMemcpyHostToDevice));
    CK(cudaMemset(b.fs, 0, sizeof(float) * 3 * (size_t)p.nb));
    CK(cudaMemset(b.grad, 0, sizeof(float) * kSurNParam));
    launch_fit_step(p, b.grad, nullptr);
    rc = check_launch("sur_fit_grad");
    if (rc) return rc;
    CK(cudaMemcpy(grad, b.grad, sizeof(float) * kSurNParam, cudaMemcpyDeviceToHost));
    if (loss) CK(cudaMemcpy(loss, b.loss, sizeof(double) * 2, cudaMemcpyDeviceToHost));
    return KOMD_OK;
}

int komd_sur_fit(komd_sur_data *d, float *params, const float *fmean, const float *fstd, double e_scale,
                 double e_shift, double f2, const komd_sur_fit_opts *o, float *loss) {
    if (!o || o->epochs < 0 || o->snaps_per_batch <= 0 || !(o->lr > 0.f) || !(o->lr_end > 0.f))
        return fail(KOMD_ERR_ARG, "bad training options");
    if (!d) return fail(KOMD_ERR_ARG, "null dataset");
    const int bs = (int)std::min<int64_t>(o->snaps_per_batch, std::max<int64_t>(d->n_snap, 1));
    FitBuffers b;
    FitParams p;
    int rc = fit_setup(d, b, p, params, fmean, fstd, e_scale, e_shift, f2, o->lam_e, o->lam_f, d->n_snap, bs,
                       o->precision);
    if (rc) return rc;
    const int64_t per_epoch = d->n_snap / bs;
    const int64_t total = per_epoch * o->epochs;
    uint64_t rng = o->seed;
    std::vector<int> perm((size_t)d->n_snap);
    int64_t step = 0;
    for (int ep = 0; ep < o->epochs; ep++) {
        for (int64_t k = 0; k < d->n_snap; k++) perm[k] = (int)k;
        for (int64_t k = d->n_snap - 1; k > 0; k--) std::swap(perm[k], perm[splitmix(rng) % (uint64_t)(k + 1)]);
        CK(cudaMemcpy(b.snaps, perm.data(), sizeof(int) * perm.size(), cudaMemcpyHostToDevice));
        CK(cudaMemset(b.loss, 0, sizeof(double) * 2));
        for (int64_t k = 0; k < per_epoch; k++, step++) {
            p.snaps = b.snaps + k * bs;
            const float lr = o->lr * std::pow(o->lr_end / o->lr, total > 1 ? (float)step / (float)(total - 1) : 0.f);
            CK(cudaMemsetAsync(b.fs, 0, sizeof(float) * 3 * (size_t)p.nb, nullptr));
            CK(cudaMemsetAsync(b.grad, 0, sizeof(float) * kSurNParam, nullptr));
            launch_fit_step(p, b.grad, nullptr);
            launch_fit_adam(b.params, b.grad, b.m, b.v, lr, (int)step, nullptr);
        }
        rc = check_launch("sur_fit");
        if (rc) return rc;
        double l2[2];
        CK(cudaMemcpy(l2, b.loss, sizeof(l2), cudaMemcpyDeviceToHost));
        if (loss) {
            loss[2 * ep] = (float)(l2[0] / std::max<int64_t>(per_epoch, 1));
            loss[2 * ep + 1] = (float)(l2[1] / std::max<int64_t>(per_epoch, 1));
        }
    }
    CK(cudaMemcpy(params, b.params, sizeof(float) * kSurNParam, cudaMemcpyDeviceToHost));
    return KOMD_OK;
}

int komd_gpu_set_profiling(komd_gpu *h, int on) {
    if (!h) return fail(KOMD_ERR_ARG, "null handle");
    collect_profile(h);
    if (h->e.rebuild_count) cudaMemsetAsync(h->e.rebuild_count, 0, sizeof(int), h->e.stream);
    h->e.profiling = on != 0;
    for (int k = 0; k < kNumFamilies; k++) { h->launches[k] = 0; h->ms[k] = 0.0; }
    return KOMD_OK;
}

int komd_gpu_profile(komd_gpu *h, int max_families, int64_t *launches, double *ms, char *names, int cap) {
    if (!h) return fail(KOMD_ERR_ARG, "null handle");
    collect_profile(h);
    if (h->e.rebuild_count) {
        int rb = 0;
        CK(cudaMemcpy(&rb, h->e.rebuild_count, sizeof(int), cudaMemcpyDeviceToHost));
        h->launches[kNumFamilies - 1] = rb;
    }
    std::string s;
    for (int k = 0; k < kNumFamilies && k < max_families; k++) {
        if (launches) launches[k] = h->launches[k];
        if (ms) ms[k] = h->ms[k];
        s += kFamilies[k];
        s += '\n';
    }
    if (names && cap > 0) {
        std::strncpy(names, s.c_str(), (size_t)cap - 1);
        names[cap - 1] = 0;
    }
    return kNumFamilies;
}

// ---------------------------------------------------------------------------
// batched replicas: one CUDA graph advances every replica by steps_per_graph
// steps; replicas are spread over n_streams parallel branches of the graph
// (fork/join through events), each replica's steps in order on its branch
// ---------------------------------------------------------------------------
}  // extern "C"

struct komd_batch {
    std::vector<komd_gpu *> reps;
    int n_streams = 1, steps_per_graph = 1, device = 0;
    cudaStream_t origin = nullptr;
    bool own_origin = false;
    std::vector<cudaStream_t> branch;
    std::vector<cudaEvent_t> ev;          // [0] fork, [1..n_streams] joins
    cudaGraphExec_t graph = nullptr;
    int64_t steps = 0;
    bool packed = false;                  // one launch per stage for all replicas of a group
    std::vector<PackedStep> pk;           // the packed groups (contiguous replica ranges)
    std::vector<void *> pk_mem;           // the packed tables (device)
    double *stage = nullptr;              // pinned landing area of komd_batch_measure
    size_t stage_cap = 0;                 // in doubles
    ~komd_batch() {
        cudaSetDevice(device);
        if (stage) cudaFreeHost(stage);
        for (void *p : pk_mem) cudaFree(p);
        if (graph) cudaGraphExecDestroy(graph);
        for (auto s : branch) cudaStreamDestroy(s);
        for (auto e : ev) cudaEventDestroy(e);
        if (own_origin && origin) cudaStreamDestroy(origin);
    }
};

namespace {
// replicas that all take the step of the Verlet path with the fused drift
// and the half-list LJ + ATM pass (the benchmark's form) advance by one
// launch per stage for all of them
bool packed_ok(const komd_batch *b) {
    const Engine &e0 = b->reps[0]->e;
    for (komd_gpu *h : b->reps) {
        const Engine &e = h->e;
        if (!(e.verlet && e.fused_drift && fused_lj_atm(h, false) && lj_atm_half(e))) return false;
        if (e.cfg.thermostat || e.n_bonds > 0 || e.n_angles > 0 || (e.cfg.terms & KOMD_TERM_BONDED)) return false;
        if (e.uniform != e0.uniform || (e.cfg.switch_width > 0) != (e0.cfg.switch_width > 0)) return false;
        if (e.hin_r || e.hin_v || e.hout_r || e.hout_f || e.hout_v) return false;
    }
    return true;
}

template <typename T>
int packed_upload(komd_batch *b, const std::vector<T> &host, T *&dev) {
    T *p = nullptr;
    CK(cudaMalloc(reinterpret_cast<void **>(&p), sizeof(T) * std::max<size_t>(host.size(), 1)));
    b->pk_mem.push_back(p);
    CK(cudaMemcpy(p, host.data(), sizeof(T) * host.size(), cudaMemcpyHostToDevice));
    dev = p;
    return KOMD_OK;
}

// a stage's per-replica arguments and block ranges
template <typename T>
int packed_stage(komd_batch *b, PackedStage &s, const std::vector<T> &args, const std::vector<int> &blocks) {
    std::vector<int> start(blocks.size() + 1, 0);
    for (size_t r = 0; r < blocks.size(); r++) start[r + 1] = start[r] + blocks[r];
    T *a = nullptr;
    int rc = packed_upload(b, args, a);
    if (rc) return rc;
    s.args = a;
    rc = packed_upload(b, start, s.start);
    if (rc) return rc;
    s.blocks = start.back();
    return KOMD_OK;
}

int packed_group(komd_batch *b, PackedStep &pk, int r0, int r1, int pr) {
    const std::vector<komd_gpu *> reps(b->reps.begin() + r0, b->reps.begin() + r1);
    const int nr = r1 - r0;
    pk.nrep = nr;
    pk.uniform = reps[0]->e.uniform;
    pk.sw = reps[0]->e.cfg.switch_width > 0;
    pk.plain = true;   // cleared below by any replica with the LJ term off or an ATM2B factor
    std::vector<Step0Args> s0;
    std::vector<BinArgs> bi;
    std::vector<ScanArgs> sc;
    std::vector<ScatterArgs> sm;
    std::vector<SortArgs> so;
    std::vector<FlushArgs> fl;
    std::vector<PairParams> pp;
    std::vector<AtmParams> ap;
    std::vector<float> sa;
    std::vector<int> n, per, two, b_io, b_cont, b_sort, b_vb, b_force;
    for (komd_gpu *h : reps) {
        Engine &e = h->e;
        s0.push_back(step0_args(e));
        bi.push_back(bin_args(e));
        sc.push_back(scan_args(e));
        sm.push_back(scatter_args(e));
        so.push_back(sort_args(e));
        fl.push_back(flush_args(e, 1.0 / 4294967296.0, half_own(e)));   // the half-list pass sums force units at 2^-32
        PairParams p = pair_params(e);
        p.fown = half_own(e);
        if (!half_plain(p)) pk.plain = false;
        AtmParams a = atm_params(e);
        pp.push_back(p);
        ap.push_back(a);
        sa.push_back((float)(2.0 * a.sign * a.nu));
        n.push_back((int)e.n);
        per.push_back(pr);
        two.push_back(vbuild_two(e) ? 1 : 0);
        b_io.push_back((int)((e.n + 255) / 256));
        b_cont.push_back(packed_blocks_container(e));
        b_sort.push_back(std::max(1, std::min((e.g.ncell + kWarpsPerBlock - 1) / kWarpsPerBlock, 16)));
        b_vb.push_back(packed_blocks_vbuild(e));
        b_force.push_back((vlist_grid(e) + pr - 1) / pr);
        pk.force_smem = std::max(pk.force_smem, lj_atm_half_smem(e));
    }
    int rc = packed_stage(b, pk.step0, s0, b_io);
    if (!rc) rc = packed_stage(b, pk.bin, bi, b_cont);
    if (!rc) rc = packed_stage(b, pk.scan, sc, std::vector<int>(nr, 1));
    if (!rc) rc = packed_stage(b, pk.scatter, sm, b_cont);
    if (!rc) rc = packed_stage(b, pk.sort, so, b_sort);
    if (!rc) rc = packed_stage(b, pk.flush, fl, b_io);
    std::vector<int> dummy(nr, 0);
    if (!rc) rc = packed_stage(b, pk.vbuild, dummy, b_vb);
    if (!rc) rc = packed_stage(b, pk.force, dummy, b_force);
    if (!rc) rc = packed_upload(b, pp, pk.pp);
    if (!rc) rc = packed_upload(b, ap, pk.ap);
    if (!rc) rc = packed_upload(b, sa, pk.sa);
    if (!rc) rc = packed_upload(b, n, pk.n);
    if (!rc) rc = packed_upload(b, per, pk.per);
    if (!rc) rc = packed_upload(b, two, pk.two);
    return rc;
}

int packed_build(komd_batch *b) {
    // groups of 8 sites per block of the force pass: about eight resident waves
    // over all replicas together, each block over a contiguous range of one
    // replica's slots (the single-system rule, vlist_per, over the batch)
    long long groups = 0, atoms = 0;
    for (komd_gpu *h : b->reps) { groups += vlist_grid(h->e); atoms += h->e.n; }
    const long long target = (long long)b->reps[0]->e.num_sms * 5 * 8;
    const int pr = (int)std::max<long long>(1, (groups + target - 1) / target);
    const int nr = (int)b->reps.size();
    // one group per graph branch: a group's stage boundaries (where its
    // launch drains) overlap the other groups' work
    const int G = std::max(1, std::min(nr, (int)b->branch.size()));
    b->pk.assign(G, PackedStep());
    // contiguous ranges of about atoms / G sites each
    int r0 = 0;
    long long acc = 0;
    for (int g = 0; g < G; g++) {
        int r1 = r0 + 1;
        acc += b->reps[r0]->e.n;
        while (r1 < nr - (G - 1 - g) && (g == G - 1 || acc < atoms * (g + 1) / G)) acc += b->reps[r1++]->e.n;
        if (g == G - 1) r1 = nr;
        const int rc = packed_group(b, b->pk[g], r0, r1, pr);
        if (rc) return rc;
        r0 = r1;
    }
    return KOMD_OK;
}

int batch_capture(komd_batch *b) {
    if (b->packed) {   // per group: steps_per_graph x eight stage launches on its own branch
        CK(cudaStreamBeginCapture(b->origin, cudaStreamCaptureModeThreadLocal));
        const int G = (int)b->pk.size();
        cudaError_t ce = cudaSuccess;
        if (G == 1) {
            for (int k = 0; k < b->steps_per_graph; k++) launch_packed_step(b->pk[0], b->origin);
        } else {
            ce = cudaEventRecord(b->ev[0], b->origin);
            for (int g = 0; g < G && ce == cudaSuccess; g++) ce = cudaStreamWaitEvent(b->branch[g], b->ev[0], 0);
            for (int g = 0; g < G && ce == cudaSuccess; g++)
                for (int k = 0; k < b->steps_per_graph; k++) launch_packed_step(b->pk[g], b->branch[g]);
            for (int g = 0; g < G && ce == cudaSuccess; g++) {
                ce = cudaEventRecord(b->ev[1 + g], b->branch[g]);
                if (ce == cudaSuccess) ce = cudaStreamWaitEvent(b->origin, b->ev[1 + g], 0);
            }
        }
        cudaGraph_t graph = nullptr;
        const cudaError_t le = ce != cudaSuccess ? ce : cudaGetLastError();
        const cudaError_t ee = cudaStreamEndCapture(b->origin, &graph);
        if (le != cudaSuccess || ee != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            return fail(KOMD_ERR_CUDA, std::string("batch capture: ") + cudaGetErrorString(le != cudaSuccess ? le : ee));
        }
        const cudaError_t ie = cudaGraphInstantiate(&b->graph, graph, 0);
        cudaGraphDestroy(graph);
        if (ie != cudaSuccess) return fail(KOMD_ERR_CUDA, std::string("batch graph instantiate: ") + cudaGetErrorString(ie));
        return KOMD_OK;
    }
    CK(cudaStreamBeginCapture(b->origin, cudaStreamCaptureModeThreadLocal));
    cudaError_t ce = cudaEventRecord(b->ev[0], b->origin);
    for (int k = 0; k < b->n_streams && ce == cudaSuccess; k++) ce = cudaStreamWaitEvent(b->branch[k], b->ev[0], 0);
    if (ce == cudaSuccess) {
        for (size_t r = 0; r < b->reps.size(); r++) {
            Engine &e = b->reps[r]->e;
            cudaStream_t keep = e.stream;
            e.stream = b->branch[r % b->n_streams];
            for (int k = 0; k < b->steps_per_graph; k++) enqueue_step(b->reps[r]);
            e.stream = keep;
        }
        for (int k = 0; k < b->n_streams && ce == cudaSuccess; k++) {
            ce = cudaEventRecord(b->ev[1 + k], b->branch[k]);
            if (ce == cudaSuccess) ce = cudaStreamWaitEvent(b->origin, b->ev[1 + k], 0);
        }
    }
    cudaGraph_t graph = nullptr;
    const cudaError_t ee = cudaStreamEndCapture(b->origin, &graph);
    if (ce != cudaSuccess || ee != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return fail(KOMD_ERR_CUDA, std::string("batch capture: ") + cudaGetErrorString(ce != cudaSuccess ? ce : ee));
    }
    const cudaError_t ie = cudaGraphInstantiate(&b->graph, graph, 0);
    cudaGraphDestroy(graph);
    if (ie != cudaSuccess) return fail(KOMD_ERR_CUDA, std::string("batch graph instantiate: ") + cudaGetErrorString(ie));
    return KOMD_OK;
}
}  // namespace

extern "C" {

int komd_batch_create(komd_gpu *const *replicas, int32_t n, int32_t n_streams, int32_t steps_per_graph,
                      void *stream, komd_batch **out) {
    if (!replicas || !out || n <= 0 || n_streams <= 0 || n_streams > 128 || steps_per_graph <= 0 ||
        steps_per_graph > 1000)
        return fail(KOMD_ERR_ARG, "bad batch arguments");
    const int dev = replicas[0] ? replicas[0]->e.device : 0;
    for (int r = 0; r < n; r++) {
        komd_gpu *h = replicas[r];
        if (!h) return fail(KOMD_ERR_ARG, "null replica");
        if (h->e.device != dev) return fail(KOMD_ERR_ARG, "replicas on different devices");
        if (!h->e.have_forces) return fail(KOMD_ERR_STATE, "every replica needs update_container and forces first");
        if (surrogate_on(h)) return fail(KOMD_ERR_ARG, "replicas run the exact forces (no host-side probes)");
        if (h->e.profiling) return fail(KOMD_ERR_STATE, "switch profiling off before batching");
        for (int q = 0; q < r; q++)
            if (replicas[q] == h) return fail(KOMD_ERR_ARG, "a replica appears twice");
    }
    CK(cudaSetDevice(dev));
    komd_batch *b = new komd_batch();
    b->device = dev;
    b->reps.assign(replicas, replicas + n);
    b->n_streams = std::min<int>(n_streams, n);
    b->steps_per_graph = steps_per_graph;
    auto bail = [&](int rc) { delete b; return rc; };
    if (stream) {
        b->origin = (cudaStream_t)stream;
    } else {
        if (cudaStreamCreateWithFlags(&b->origin, cudaStreamNonBlocking) != cudaSuccess)
            return bail(fail(KOMD_ERR_CUDA, "stream creation failed"));
        b->own_origin = true;
    }
    for (int k = 0; k < b->n_streams; k++) {
        cudaStream_t s;
        if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess)
            return bail(fail(KOMD_ERR_CUDA, "stream creation failed"));
        b->branch.push_back(s);
    }
    for (int k = 0; k <= b->n_streams; k++) {
        cudaEvent_t e;
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess)
            return bail(fail(KOMD_ERR_CUDA, "event creation failed"));
        b->ev.push_back(e);
    }
    // the replicas' own queues must be drained before the batch graph runs
    for (auto h : b->reps)
        if (cudaStreamSynchronize(h->e.stream) != cudaSuccess) return bail(fail(KOMD_ERR_CUDA, "replica stream"));
    int rc = KOMD_OK;
    b->packed = packed_ok(b);
    if (b->packed) rc = packed_build(b);
    if (rc) return bail(rc);
    rc = batch_capture(b);
    if (rc) return bail(rc);
    *out = b;
    return KOMD_OK;
}

void komd_batch_destroy(komd_batch *b) { delete b; }

int komd_batch_step(komd_batch *b, int64_t n_graphs) {
    if (!b) return fail(KOMD_ERR_ARG, "null batch");
    CK(cudaSetDevice(b->device));
    for (int64_t k = 0; k < n_graphs; k++) CK(cudaGraphLaunch(b->graph, b->origin));
    CK(cudaStreamSynchronize(b->origin));
    b->steps += n_graphs * b->steps_per_graph;
    for (size_t r = 0; r < b->reps.size(); r++) {
        int rc = finish_steps(b->reps[r]);
        if (rc) return fail(rc, "replica " + std::to_string(r) + ": " + g_last_error);
    }
    return KOMD_OK;
}

// enqueue only (no synchronisation, no flag check): for timing with events on the origin stream
int komd_batch_launch(komd_batch *b, int64_t n_graphs) {
    if (!b) return fail(KOMD_ERR_ARG, "null batch");
    for (int64_t k = 0; k < n_graphs; k++) CK(cudaGraphLaunch(b->graph, b->origin));
    b->steps += n_graphs * b->steps_per_graph;
    return KOMD_OK;
}

int komd_batch_measure(komd_batch *b, uint32_t mask, komd_observables *obs, double *rdf) {
    if (!b || !obs) return fail(KOMD_ERR_ARG, "null argument");
    CK(cudaSetDevice(b->device));
    const int nr = (int)b->reps.size();
    size_t bins = 0;
    for (komd_gpu *h : b->reps) {
        if (!h->e.have_cells) return fail(KOMD_ERR_STATE, "update_container must run before measure");
        if ((mask & KOMD_MEASURE_RDF) && h->e.rdf_bins > 0) bins += (size_t)h->e.rdf_bins;
    }
    // pinned landing area: per replica the sums and the error flags, then the RDF bins
    const size_t per = R_NSLOTS + E_NFLAGS;
    const size_t need = (size_t)nr * per + bins;
    if (need > b->stage_cap) {
        if (b->stage) cudaFreeHost(b->stage);
        b->stage = nullptr;
        b->stage_cap = 0;
        CK(cudaMallocHost(reinterpret_cast<void **>(&b->stage), sizeof(double) * need));
        b->stage_cap = need;
    }
    // the measures follow the batch's graph launches on the origin stream and
    // spread over its branches; the origin waits for all of them
    CK(cudaEventRecord(b->ev[0], b->origin));
    const int nb = (int)b->branch.size();
    for (int k = 0; k < nb; k++) CK(cudaStreamWaitEvent(b->branch[k], b->ev[0], 0));
    size_t off = (size_t)nr * per;
    int rc = KOMD_OK;
    for (int r = 0; r < nr && !rc; r++) {
        Engine &e = b->reps[r]->e;
        cudaStream_t keep = e.stream;
        e.stream = b->branch[r % nb];
        double *slot = b->stage + (size_t)r * per;
        const bool with_rdf = (mask & KOMD_MEASURE_RDF) && e.rdf_bins > 0;
        rc = measure_enqueue(b->reps[r], mask, slot, with_rdf ? b->stage + off : nullptr, nullptr);
        if (!rc) {
            // the flags as read_flags reads them (read, then cleared), into the landing area
            int *fl = reinterpret_cast<int *>(slot + R_NSLOTS);
            if (cudaMemcpyAsync(fl, e.err, sizeof(int) * E_NFLAGS, cudaMemcpyDeviceToHost, e.stream) != cudaSuccess ||
                cudaMemsetAsync(e.err, 0, sizeof(int) * E_NFLAGS, e.stream) != cudaSuccess)
                rc = fail(KOMD_ERR_CUDA, "measure flags");
        }
        if (with_rdf) off += (size_t)e.rdf_bins;
        e.stream = keep;
    }
    for (int k = 0; k < nb; k++) {
        if (cudaEventRecord(b->ev[1 + k], b->branch[k]) == cudaSuccess) cudaStreamWaitEvent(b->origin, b->ev[1 + k], 0);
    }
    CK(cudaStreamSynchronize(b->origin));
    if (rc) return rc;
    off = (size_t)nr * per;
    for (int r = 0; r < nr; r++) {
        const Engine &e = b->reps[r]->e;
        const double *slot = b->stage + (size_t)r * per;
        const int *fl = reinterpret_cast<const int *>(slot + R_NSLOTS);
        if (fl[E_ATM_OVERFLOW])
            return fail(KOMD_ERR_OVERFLOW, "replica " + std::to_string(r) + ": ATM neighbour list overflow during measure");
        measure_fill(slot, obs + r);
        if ((mask & KOMD_MEASURE_RDF) && e.rdf_bins > 0) {
            if (rdf) std::memcpy(rdf, b->stage + off, sizeof(double) * (size_t)e.rdf_bins);
            if (rdf) rdf += e.rdf_bins;
            off += (size_t)e.rdf_bins;
        }
    }
    return KOMD_OK;
}

int komd_batch_form(komd_batch *b) {
    if (!b) return fail(KOMD_ERR_ARG, "null batch"), -1;
    return b->packed ? 1 : 0;
}

int komd_batch_check(komd_batch *b) {
    if (!b) return fail(KOMD_ERR_ARG, "null batch");
    CK(cudaStreamSynchronize(b->origin));
    for (size_t r = 0; r < b->reps.size(); r++) {
        int rc = finish_steps(b->reps[r]);
        if (rc) return fail(rc, "replica " + std::to_string(r) + ": " + g_last_error);
    }
    return KOMD_OK;
}

int komd_gpu_kernels_per_step(komd_gpu *h) {
    if (!h) return -1;
    const Engine &e = h->e;
    // integrate0/1; the container pass (com/wrap/bin, scan, scatter, cell sort, and
    // on the Verlet path the list build and the FP32 refresh unless the drift does it)
    int k = 2 + 4 + (e.verlet ? (e.fused_drift ? 1 : 2) : 0);
    if (e.cfg.terms & (KOMD_TERM_LJ | KOMD_TERM_FENE | KOMD_TERM_ATM)) k++;   /* pair pass (else a memset) */
    if (e.cfg.terms & KOMD_TERM_TABULATED) k++;
    if (!surrogate_on(h) && (e.cfg.terms & KOMD_TERM_ATM) && e.atm_acc) k--;   /* integrate1 fused into the ATM flush */
    if ((e.cfg.terms & KOMD_TERM_BONDED) && e.n_bonds > 0) k++;
    if ((e.cfg.terms & KOMD_TERM_BONDED) && e.n_angles > 0) k++;
    if (e.cfg.terms & KOMD_TERM_LIMIT) k++;
    if (e.cfg.thermostat) k += 3;  /* kinetic sums, partial reduction, velocity scaling */
    if (surrogate_on(h)) k += 4;   /* descriptors, MLP, forces, apply */
    else if (e.cfg.terms & KOMD_TERM_ATM)   /* once-per-triplet kernel (inside the LJ pass on the Verlet path) + flush */
        k += (e.atm_acc != nullptr) ? (fused_lj_atm(h, false) ? 1 : 2) : 1;
    return k;
}

}  // extern "C"
