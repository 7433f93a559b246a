/*
 * komd_gpu.h -- C ABI of the GB300 force engine for KoMD's hot path.
 *
 * One opaque handle owns one periodic system on one GPU (device buffers are
 * engine-owned, every host buffer is caller-owned).  Every call returns an
 * int status (0 = KOMD_OK); the message of the last failure on the calling
 * thread is komd_gpu_last_error().  Calls are synchronous from the caller's
 * view (they end with a stream synchronize), like the reference's functor
 * calls that end in Kokkos::fence (potentials/ForceFunctor.cpp:13,
 * integrators/Integrator.cpp:16,25), unless documented otherwise.
 *
 * Each entry point names the reference interface it replaces
 * (Snapex2409/KoMD, src/...).  No Kokkos, torch or other types cross the
 * boundary: plain pointers, sizes and PODs only.
 */
#ifndef KOMD_GPU_H
#define KOMD_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define KOMD_GPU_ABI_VERSION 2

/* status codes */
enum {
    KOMD_OK = 0,
    KOMD_ERR_ARG = 1,        /* invalid argument or configuration                  */
    KOMD_ERR_CUDA = 2,       /* CUDA runtime error (message has the CUDA string)   */
    KOMD_ERR_OVERFLOW = 3,   /* a device-side capacity was exceeded (flagged, not trapped) */
    KOMD_ERR_STATE = 4,      /* call out of order (e.g. no sites uploaded)         */
    KOMD_ERR_NOMEM = 5,      /* device allocation failed                           */
    KOMD_ERR_NONFINITE = 6   /* a NaN/Inf force or position was detected           */
};

/* arithmetic of the pair and triplet kernels (integration and reductions are FP64 always) */
enum { KOMD_FP32 = 0, KOMD_FP64 = 1 };
/* ATM force sign: REFERENCE reproduces potentials/ATM.cpp:55-57 (adds +grad V);
 * PHYSICAL uses F = -grad V */
enum { KOMD_ATM_SIGN_REFERENCE = 0, KOMD_ATM_SIGN_PHYSICAL = 1 };
/* ATM triplet set: COMPAT = the reference's cell-triple enumeration
 * (container/LinkedCells.h:126-152 + same-cell triples: all three cells equal
 * or all distinct); FULL = every triplet with all sides inside the cutoff */
enum { KOMD_ATM_ENUM_COMPAT = 0, KOMD_ATM_ENUM_FULL = 1 };
/* virial: COMPAT reproduces sensors/PressureSensor.cpp:143-286 (boundary pairs
 * counted per list entry, no ZZ term for ATM, direct ATM contributes nothing);
 * CORRECT counts every pair / triplet once */
enum { KOMD_VIRIAL_COMPAT = 0, KOMD_VIRIAL_CORRECT = 1 };

/* force terms (bit mask) */
#define KOMD_TERM_LJ      0x01u  /* potentials/LJ12_6.cpp:15-43                 */
#define KOMD_TERM_FENE    0x02u  /* potentials/FENE.cpp:15-43                   */
#define KOMD_TERM_LIMIT   0x04u  /* potentials/Limit.cpp:19-25                  */
#define KOMD_TERM_ATM     0x08u  /* potentials/ATM.cpp / ATM_NOLIST.cpp         */
#define KOMD_TERM_BONDED  0x10u  /* harmonic bond + angle (no reference counterpart) */
/* with KOMD_TERM_ATM: the learned three-body form (no reference counterpart)
 * replaces the exact triplet sum once komd_gpu_surrogate_load has run */
#define KOMD_TERM_ATM_SURROGATE 0x20u
/* with KOMD_TERM_LJ: ATM2B effective pair force (potentials/ATM2B.cpp:9-56,
 * main.cpp:57-58 enable_3b_approx): LJ forces times 1 - 2 nu rho / (3 eps sigma^6),
 * rho = molecules / domain volume, eps and sigma of the first uploaded site;
 * the LJ energy and virial sensors stay unscaled as in the reference */
#define KOMD_TERM_ATM2B 0x40u
/* tabulated pair force (plugins/IBI/IBI_ForceFunctor.cpp:18-37): every site pair
 * inside cutoff gets F(r) from komd_gpu_set_pair_table, FP64, in the LJ
 * functor's place before Limit (set it instead of, or with, KOMD_TERM_LJ) */
#define KOMD_TERM_TABULATED 0x80u

/* measurements (bit mask) */
#define KOMD_MEASURE_TEMPERATURE 0x01u  /* sensors/TemperatureSensor.cpp:27-48   */
#define KOMD_MEASURE_ENERGY      0x02u  /* LJ12_6_Sensor total U, ATM and bonded energy */
#define KOMD_MEASURE_PRESSURE    0x04u  /* sensors/PressureSensor.cpp:28-33        */
#define KOMD_MEASURE_RDF         0x08u  /* sensors/RDFSensor.cpp:23-34             */
#define KOMD_MEASURE_LJ_HIST     0x10u  /* Potential_Sensor U(r), F(r) histograms  */

typedef struct komd_config {
    double domain_low[3];      /* configuration()->domainLow  (IO/Configuration.h)   */
    double domain_high[3];     /* configuration()->domainHigh                        */
    double cell_size;          /* configuration()->cell_size; >= both cutoffs        */
    double cutoff;             /* LJ cutoff, configuration()->cutoff                 */
    double cutoff_3b;          /* ATM cutoff (the reference reuses cutoff)           */
    double nu;                 /* ATM coefficient in internal units (ATM.cpp:11-14)  */
    double delta_t;            /* configuration()->delta_t                           */
    double stiffness;          /* FENE stiffness factor                              */
    double limit;              /* Limit factor                                       */
    double bond_k, bond_r0;    /* harmonic bond  U = k/2 (r - r0)^2                  */
    double angle_k, angle_theta0; /* harmonic angle U = k/2 (theta - theta0)^2, radians */
    double max_sigma;          /* LJ sensor histogram range 3*max_sigma              */
    double rdf_max, rdf_dr;    /* RDF sensor range and bin width                     */
    uint32_t terms;            /* KOMD_TERM_*                                        */
    int32_t precision;         /* KOMD_FP32 | KOMD_FP64                              */
    int32_t atm_sign;          /* KOMD_ATM_SIGN_*                                    */
    int32_t atm_enum;          /* KOMD_ATM_ENUM_*                                    */
    int32_t virial_mode;       /* KOMD_VIRIAL_*                                      */
    int32_t atm_direct;        /* 1: ATM_NOLIST semantics (no ATM virial in COMPAT)  */
    int32_t lj_bins;           /* sensor_lj_bins                                     */
    int32_t atm_list_cap;      /* per-site neighbour capacity inside cutoff_3b (0 = from density) */
    double skin;               /* Verlet skin: > 0 keeps a neighbour list inside cutoff + skin and
                                  rebuilds cells and list only when a site has moved more than
                                  skin/2 (FP32, no FENE, FULL ATM, CORRECT virial); 0 rebuilds
                                  every step like LinkedCells::updateContainer.  Cells bin
                                  molecules by their centre of mass: for multi-site molecules
                                  choose cell_size >= cutoff + skin + twice a site's largest
                                  distance from its molecule's centre (only cutoff + skin is
                                  checked), so that every site pair in range is in adjacent cells */
    double temperature_target; /* VelocityScaling target in K (configuration()->temperature)   */
    int32_t thermostat;        /* 1: each step of komd_gpu_step ends with v *= sqrt(T_target / T),
                                  T measured on the device as TemperatureSensor does
                                  (VelocityScaling.cpp:12-25, Simulation.cpp:72) */
    double switch_width;       /* 0 (default): the reference's truncated LJ and ATM
                                  (potentials/LJ12_6.cpp:28, potentials/ATM.cpp:43).
                                  > 0: a labelled option with no reference counterpart --
                                  the LJ pair energy times S(r^2) and the ATM triplet
                                  energy times S over its three sides, S the C1
                                  smoothstep t^2 (3 - 2t), t = (rc^2 - x) / (rc^2 - rs^2),
                                  rs = cutoff - switch_width (cutoff_3b - switch_width for
                                  ATM); forces are the exact gradients, so the energy is
                                  conserved without the jumps of the truncation.  Needs
                                  the Verlet path (skin > 0, FP32) without Limit, FENE,
                                  ATM2B, tabulated or bonded terms; with the learned
                                  three-body term it switches the LJ pair energy (and
                                  the exact ATM of the probes) */
} komd_config;

typedef struct komd_observables {
    double temperature;        /* K, sites inside the domain only                    */
    double mv2;                /* sum m v^2 over those sites (internal units)        */
    double n_in_box;           /* number of those sites                              */
    double u_lj;               /* LJ12_6_Sensor::getCurrentPotential                 */
    double u_atm;              /* ATM energy (physical V, each triplet once)         */
    double u_bonded;           /* harmonic bond + angle energy                       */
    double kinetic[6];         /* sum m v v (XX XY YY XZ YZ ZZ), per virial_mode's site set */
    double virial[6];          /* pair + triplet (+ bonded in CORRECT) virial         */
    double pressure[6];        /* kinetic + virial, unscaled (PressureSensor::m_pressures) */
    int64_t pairs_in_cutoff;   /* LJ site pairs inside the cutoff (each once)        */
    int64_t triplets;          /* ATM triplets inside the cutoff (each once)         */
} komd_observables;

typedef struct komd_gpu komd_gpu;

/* ---- lifetime ---------------------------------------------------------- */
/* Replaces main.cpp:43-66 (container + functors from Configuration). */
int  komd_gpu_create(const komd_config *cfg, int device, komd_gpu **out);
int  komd_gpu_destroy(komd_gpu *h);
const char *komd_gpu_last_error(void);
int  komd_gpu_abi_version(void);
/* TemperatureSensor's conversion (sensors/TemperatureSensor.cpp:44-47, in
 * math/SciValue.h arithmetic): T in K from sum(m v^2) and the number of sites
 * in the box.  The same function the device thermostat evaluates inside the
 * step graph; it returns for every input (NaN and +-inf give a non-finite T,
 * zero sites give 0) -- unlike the reference's SciValue loop, which never
 * ends on an infinite mantissa. */
double komd_sci_temperature(double mv2, double n_in_box);
/* Runs the engine's work on a caller-provided cudaStream_t (NULL = engine's own). */
int  komd_gpu_set_stream(komd_gpu *h, void *cuda_stream);
/* Domain cells per dimension, floor(L / cell_size) (LinkedCells.cpp:19). */
int  komd_gpu_grid_dims(komd_gpu *h, int64_t nd[3]);

/* ---- sites -------------------------------------------------------------- */
/* Replaces MoleculeContainer::addMolecule + constructSOAs
 * (container/MoleculeContainer.cpp:13-53) and CheckpointIO::loadCheckpoint.
 * Sites in molecule order; consecutive sites with equal mol_id form one
 * molecule.  r, v: n*3 doubles (x y z per site); m, eps (internal units),
 * sig: n doubles; mol_id: n uint64. */
int  komd_gpu_upload_sites(komd_gpu *h, int64_t n, const double *r, const double *v, const double *m,
                           const double *eps, const double *sig, const uint64_t *mol_id);
/* Overwrites positions and/or velocities only (NULL keeps a field). */
int  komd_gpu_set_state(komd_gpu *h, const double *r, const double *v);
/* Harmonic topology: bonds as site-index pairs, angles as (i, vertex, k). */
int  komd_gpu_set_topology(komd_gpu *h, int64_t n_bonds, const int64_t *bonds, int64_t n_angles,
                           const int64_t *angles);
/* Copies r, v, f (n*3 doubles each, site order) to the host; NULL skips. */
int  komd_gpu_download(komd_gpu *h, double *r, double *v, double *f);
int64_t komd_gpu_num_sites(komd_gpu *h);

/* ---- hot path ----------------------------------------------------------- */
/* LinkedCells::updateContainer (LinkedCells.cpp:65-81): COM, periodic wrap,
 * f = 0, COM, counting-sort binning, cell-sorted FP32/FP64 positions. */
int  komd_gpu_update_container(komd_gpu *h);
/* All configured ForceFunctor / ForceFunctor3B terms in the reference order
 * (LJ, FENE, bonded, Limit, then ATM; Simulation.cpp:57-59); needs a prior
 * update_container. */
int  komd_gpu_forces(komd_gpu *h);
/* Integrator::integrate0 / integrate1 (integrators/Integrator.cpp:10-37). */
int  komd_gpu_integrate0(komd_gpu *h);
int  komd_gpu_integrate1(komd_gpu *h);
/* n full steps of Simulation::run's loop body without thermostat or plugins
 * (integrate0, updateContainer, forces, integrate1), replayed from one CUDA
 * graph.  Requires forces of the current positions (call update_container +
 * forces once before the first step_n). */
int  komd_gpu_step(komd_gpu *h, int64_t n_steps);
/* Same as komd_gpu_step, end to end from host buffers: takes r, v (n*3) from
 * the host, runs n_steps, returns r, v and f.  When the GPU can address the
 * buffers (pinned memory, or any host memory where the GPU walks the host page
 * tables, as over NVLink-C2C) and the step is the fused Verlet / FULL FP32 ATM
 * path without device thermostat or learned term, the first step's drift
 * kernel reads r, v and writes r back, and the last step's ATM flush writes f
 * and v, so no separate copies run; otherwise copies frame the steps.  A
 * one-step call on that path launches a graph captured for these buffers
 * (recaptured when the buffers or the step change).  The results are bitwise
 * those of komd_gpu_step. */
int  komd_gpu_step_host(komd_gpu *h, int64_t n_steps, double *r, double *v, double *f);

/* ---- sensors ------------------------------------------------------------ */
/* Sensor::measure of the selected sensors (sensors/Sensor.h:15-33).  Uses
 * the current container/forces state; rdf (may be NULL) receives the raw
 * histogram of this call (RDFSensor::m_bins for one sample), lj_hist (may be
 * NULL) 4*lj_bins doubles: U sums, F sums, U counts, F counts. */
int  komd_gpu_measure(komd_gpu *h, uint32_t mask, komd_observables *obs, double *rdf, double *lj_hist);
int64_t komd_gpu_rdf_bins(komd_gpu *h);

/* ---- parity dumps ------------------------------------------------------- */
/* Cell lists of the reference layout ((nd+2)^3 cells incl. halo copies,
 * LCCellIterator order, LinkedCells.cpp:83-121): count[ncell] and the site
 * indices of all cells concatenated (idx capacity cap; *total gets the
 * needed size). */
int  komd_gpu_get_cells(komd_gpu *h, int64_t *count, int64_t ncell, int64_t *idx, int64_t cap, int64_t *total);
/* Per-site number of LJ partners with dr2 <= cutoff^2 and a different
 * molecule ID, evaluated in FP64 with the reference's arithmetic
 * (LJ12_6.cpp:23-28), so counts are bit-exact. */
int  komd_gpu_neighbour_counts(komd_gpu *h, int64_t *counts);

/* The tabulated pair force F(r) (FunctionPL::evaluateAt, plugins/IBI/IBI_Math.h:30-44):
 * piecewise linear on n >= 2 strictly ascending nodes x with values y,
 * `below` for r < x[0], `above` for r > x[n-1].  May be replaced between
 * steps (the IBI iteration's force update, IBI.cpp:172-178). */
int  komd_gpu_set_pair_table(komd_gpu *h, int32_t n, const double *x, const double *y, double below, double above);
/* Replace the step's force terms between steps, as a plugin replaces the
 * Registry's functors (plugins/IBI/IBI.cpp:50-54 swaps LJ, FENE, Limit and
 * ATM for the tabulated force; IBI_ReloadForce.cpp:33-49).  `terms` may drop
 * any term given at creation and may add KOMD_TERM_TABULATED (per-step cell
 * lists only: skin 0); nothing else can be added.  The sensors
 * (komd_gpu_measure) keep evaluating the terms given at creation, as the
 * reference's sensors do not go through the functor list. */
int  komd_gpu_set_terms(komd_gpu *h, uint32_t terms);
/* RDF_Profiler::measure / getRDF (plugins/IBI/RDF_Profiler.cpp:18-55): ordered
 * molecule-COM pair histogram with nbins bins of max_r / nbins up to max_r
 * (added to bins, nbins doubles). */
int  komd_gpu_rdf_profile(komd_gpu *h, double max_r, int32_t nbins, double *bins);

/* VelocityScaling::apply (VelocityScaling.cpp:12-25) with the caller's
 * beta = sqrt(T_target / T_sensor): v *= beta for every site. */
int  komd_gpu_scale_velocities(komd_gpu *h, double beta);

/* ---- learned three-body term (no reference counterpart) ----------------- */
/* A 32-64-64-1 tanh MLP on per-site descriptors inside cutoff_3b (16 radial
 * Gaussians, 16 moment-tensor invariants) gives per-site three-body energies;
 * forces are the analytic gradient.  Inference runs the MLP on the tensor
 * cores (BF16 weights, FP32 accumulation). */
#define KOMD_SUR_NFEAT 32
#define KOMD_SUR_NPARAM 6337   /* W1 64x32, b1 64, W2 64x64, b2 64, w3 64, b3 1 */
typedef struct komd_surrogate_status {
    int64_t steps;             /* steps run with the learned form                 */
    int64_t probes;            /* exact-ATM probes run                            */
    double last_rmse;          /* last probe: |F_learned - F_exact| RMS / |F_exact| RMS */
    double max_rmse;
    int32_t fallback;          /* 1: a probe breached the threshold, exact ATM is used */
    int64_t fallback_step;
} komd_surrogate_status;
/* Loads weights (FP32, KOMD_SUR_NPARAM, converted to BF16), feature
 * standardisation (mean, std per feature) and energy scaling
 * (E_i = e_scale * MLP + e_shift).  Every probe_every steps of komd_gpu_step
 * the exact ATM forces are computed as well; a relative force RMSE above
 * probe_threshold switches the engine to the exact form for good. */
int  komd_gpu_surrogate_load(komd_gpu *h, const float *params, const float *fmean, const float *fstd,
                             double e_scale, double e_shift, int32_t probe_every, double probe_threshold);
/* Training sample of the current state (after update_container): raw
 * features (n*32 floats), exact per-site ATM energies V/3 per vertex (n) and
 * exact ATM forces (n*3), site order, with the configured sign and triplet set. */
int  komd_gpu_surrogate_sample(komd_gpu *h, float *features, double *e3, double *f3);
/* Learned three-body forces (n*3) and per-site energies (n) of the current state. */
int  komd_gpu_surrogate_forces(komd_gpu *h, double *f3, double *e3);
int  komd_gpu_surrogate_status(komd_gpu *h, komd_surrogate_status *st);
/* Trains the MLP on the current device by per-site energy regression
 * (mean squared error, Adam, mini-batches sampled with replacement):
 * X n*32 standardised features, y n scaled targets; params in/out;
 * loss (epochs floats, may be NULL) gets each epoch's mean batch loss. */
int  komd_mlp_train(const float *X, const float *y, int64_t n, float *params, int32_t epochs, int32_t batch,
                    float lr, uint64_t seed, float *loss);
/* Gradient of the mean squared error over all n samples (one batch) with
 * respect to the parameters, from the same kernels komd_mlp_train runs. */
int  komd_mlp_loss_grad(const float *X, const float *y, int64_t n, const float *params, float *grad, float *loss);

/* Force-matched training.  A dataset on the device holds snapshots that
 * the exact kernel produced: per site the ATM neighbour list, raw features,
 * moments, exact per-site energy and exact three-body force (slot order of
 * the capturing engine, all snapshots with one site count and one
 * cutoff_3b).  nl_cap bounds the neighbours kept per site. */
typedef struct komd_sur_data komd_sur_data;
int     komd_sur_data_create(int32_t device, int32_t nl_cap, komd_sur_data **out);
void    komd_sur_data_destroy(komd_sur_data *d);
/* Appends the engine's current state (after update_container) as a snapshot. */
int     komd_gpu_surrogate_capture(komd_gpu *h, komd_sur_data *d);
int64_t komd_sur_data_snapshots(const komd_sur_data *d);
int32_t komd_sur_data_sites(const komd_sur_data *d);   /* sites per snapshot */
/* Host copies of one snapshot (snap >= 0) or of all (snap < 0), slot order:
 * raw features (32 per site), energies, forces (3 per site), site ids. */
int     komd_sur_data_get(komd_sur_data *d, int64_t snap, float *features, float *e3, float *f3, int32_t *site);
/* arithmetic of the network's forward, reverse and weight-gradient kernels in training */
#define KOMD_FIT_BF16 0        /* tensor cores: BF16 operands, FP32 accumulation (default) */
#define KOMD_FIT_FP32 1        /* FP32 SIMT (gradient checks at FP32 tolerance)            */
typedef struct komd_sur_fit_opts {
    int32_t epochs;            /* passes over the snapshots                         */
    int32_t snaps_per_batch;   /* snapshots per Adam step                           */
    float lr, lr_end;          /* learning rate, decayed geometrically to lr_end    */
    float lam_e, lam_f;        /* weights of the energy and force terms             */
    uint64_t seed;             /* snapshot shuffling                                */
    int32_t precision;         /* KOMD_FIT_BF16 or KOMD_FIT_FP32                    */
} komd_sur_fit_opts;
/* Minimises lam_e * mean (E - (e3 - e_shift)/e_scale)^2
 *         + lam_f * mean |F - F_exact|^2 / f2      (per site, f2 = <|F_exact|^2>)
 * over the parameters (in/out) with Adam; loss (2*epochs floats, may be
 * NULL) gets each epoch's mean energy and force terms. */
int     komd_sur_fit(komd_sur_data *d, float *params, const float *fmean, const float *fstd, double e_scale,
                     double e_shift, double f2, const komd_sur_fit_opts *opts, float *loss);
/* Gradient (and the two loss terms) over all snapshots as one batch, from
 * the kernels komd_sur_fit runs with the given precision (KOMD_FIT_*). */
int     komd_sur_fit_grad(komd_sur_data *d, const float *params, const float *fmean, const float *fstd,
                          double e_scale, double e_shift, double f2, float lam_e, float lam_f, float *grad,
                          double *loss, int32_t precision);

/* ---- batched replicas (no reference counterpart) ----------------------- */
/* Independent engines (replicas of uneven sizes, each created, uploaded and
 * past update_container + forces) advance together: one CUDA graph holds
 * steps_per_graph steps of every replica, spread over n_streams parallel
 * branches (the packed form: the replicas split into n_streams contiguous
 * groups of about equal atom counts, each group one launch per stage on its
 * own branch).  stream (may be NULL) is the stream the graph is launched on.
 * Replicas must not be modified (upload, set_state, update_container) while
 * the batch exists; the exact forces run (no learned-term probes). */
typedef struct komd_batch komd_batch;
int  komd_batch_create(komd_gpu *const *replicas, int32_t n, int32_t n_streams, int32_t steps_per_graph,
                       void *stream, komd_batch **out);
void komd_batch_destroy(komd_batch *b);
/* n_graphs launches of the graph (n_graphs * steps_per_graph steps), then a
 * synchronisation and every replica's error-flag check. */
int  komd_batch_step(komd_batch *b, int64_t n_graphs);
/* Launches only (asynchronous); komd_batch_check synchronises and checks. */
int  komd_batch_launch(komd_batch *b, int64_t n_graphs);
int  komd_batch_check(komd_batch *b);
/* Every replica's observables after the batch's steps, as komd_gpu_measure
 * gives them (same mask; obs: one per replica; rdf: the replicas' RDF bins
 * one after another, komd_gpu_rdf_bins each, may be NULL).  The measures are
 * enqueued on the batch's branches behind its graph launches, with one
 * synchronisation for all; no counterpart in the reference (which has one
 * system per process). */
int  komd_batch_measure(komd_batch *b, uint32_t mask, komd_observables *obs, double *rdf);
/* 1 when the batch advances all replicas by one launch per stage of the step
 * (every replica on the Verlet path with the fused drift and the half-list
 * LJ + ATM pass: the packed form), 0 when it replays each replica's own
 * kernels on parallel graph branches; -1 for a null batch. */
int  komd_batch_form(komd_batch *b);

/* ---- profiling ---------------------------------------------------------- */
/* When enabled, every kernel launch outside komd_gpu_step's graph is
 * bracketed by CUDA events; komd_gpu_profile reports per kernel family the
 * number of launches and the summed device milliseconds since the last
 * reset.  names is a '\n'-separated list of families (<= cap bytes). */
int  komd_gpu_set_profiling(komd_gpu *h, int on);
int  komd_gpu_profile(komd_gpu *h, int max_families, int64_t *launches, double *ms, char *names, int cap);
/* Number of kernels one komd_gpu_step launches per step (for accounting). */
int  komd_gpu_kernels_per_step(komd_gpu *h);

/* ---- allocation-free variant ------------------------------------------- */
/* No counterpart in the reference.  ATM forces (FULL triplet set) of one
 * small periodic system for callers that can pass device pointers but must
 * not allocate device memory: for instance code embedded in a host
 * application whose caching allocator has reserved the device, or a time-
 * step loop that must not call cudaMalloc/cudaFree because both implicitly
 * synchronise the device.  r (n*3 doubles) and f (n*3 doubles, overwritten)
 * are device-accessible pointers; the neighbour list the kernels need lives
 * in a fixed static device array inside the library (about 6.3 MB), so this
 * call allocates nothing.  CUDA loads the library's module lazily, so the
 * array is reserved on a device by the first call there (or at context
 * creation under CUDA_MODULE_LOADING=EAGER) and held until the process exits:
 * make that first call before the host application reserves the rest of the
 * device.  Limits: n <= KOMD_NOALLOC_MAX_SITES and at most
 * KOMD_NOALLOC_NL_CAP neighbours inside cutoff_3b per site (KOMD_ERR_ARG /
 * KOMD_ERR_OVERFLOW otherwise; after KOMD_ERR_OVERFLOW f is undefined);
 * every box edge >= 2 * cutoff_3b; atm_sign is KOMD_ATM_SIGN_REFERENCE or
 * KOMD_ATM_SIGN_PHYSICAL (KOMD_ERR_ARG otherwise).  The first call on a
 * device also resolves the array's device address (set-up) and should come
 * before any stream capture on that device.  All calls share the one array:
 * calls whose GPU work overlaps race and must be serialised by the caller.
 * Synchronous on cuda_stream (NULL = legacy default stream). */
#define KOMD_NOALLOC_MAX_SITES 4096
#define KOMD_NOALLOC_NL_CAP 96
int  komd_gpu_atm_forces_noalloc(int64_t n, const double *r, double *f, const double domain_low[3],
                                 const double domain_high[3], double cutoff_3b, double nu, int32_t atm_sign,
                                 void *cuda_stream);

#ifdef __cplusplus
}
#endif
#endif
