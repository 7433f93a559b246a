/*
 * komd_oracle.h -- FP64 CPU restatement of KoMD's hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA engine
 * in komd_gb300/: tests, the smoke check and the CPU-baseline leg of bench.py
 * may call it; the product path never does.
 *
 * Every routine restates one reference function (file:line of
 * Snapex2409/KoMD cited beside each declaration) in plain C with IEEE double
 * arithmetic and no FMA contraction (built with -ffp-contract=off), so that
 * the COMPAT modes reproduce the reference's own results.  Parity of this
 * restatement is pinned against the reference itself: the reference sources
 * are compiled into a harness (oracle/ref/) whose outputs are committed as
 * fixtures under tests/golden/.
 *
 * Conventions
 *   - positions / velocities / forces are AoS double[n][3] in site order,
 *     exactly the layout of the reference's SOA::r/v/f (math::d3 views);
 *   - molecules are contiguous runs of sites: mol_off[m]..mol_off[m+1]-1;
 *   - id[s] is the molecule ID of site s (SOA::id), compared for equality only;
 *   - cell coordinates follow the reference grid: domain cells 1..nd, one
 *     halo layer (0 and nd+1) per side, linear index x + nc_x*(y + nc_y*z).
 */
#ifndef KOMD_ORACLE_H
#define KOMD_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    double low[3], high[3], L[3];
    double cs;            /* configuration()->cell_size                   */
    int64_t nd[3];        /* domain cells per dimension: floor(L / cs)    */
    int64_t nc[3];        /* nd + 2 (one halo layer per side)             */
    int64_t ncell;        /* nc_x * nc_y * nc_z                           */
    double *bl[3], *bh[3];/* per-dimension cell bounds (LinkedCells.cpp:24-44) */
} kor_grid;

typedef struct {
    int64_t ncell;
    int64_t *count;       /* entries per cell (domain + halo copies)      */
    int64_t *start;       /* exclusive prefix of count                    */
    int64_t *idx;         /* site indices, ascending within a domain cell */
    int64_t total;
} kor_cells;

/* Grid geometry: LinkedCells::LinkedCells, LinkedCells.cpp:11-45. */
int  kor_grid_init(kor_grid *g, const double low[3], const double high[3], double cell_size);
void kor_grid_free(kor_grid *g);
/* 1 if the cell at (x,y,z) is a halo cell by the reference's bound test
 * (LinkedCells.cpp:107-113: cell.low() < low or cell.high() > high). */
int  kor_is_halo(const kor_grid *g, int64_t x, int64_t y, int64_t z);

/* Per-molecule centre of mass, MoleculeContainer::updateCOM,
 * MoleculeContainer.cpp:55-75 (com += r*m; M += m; com /= M). */
void kor_com(int64_t n_mol, const int64_t *mol_off, const double *r, const double *m, double *com_mol);

/* Periodic wrap by the molecule's COM, LinkedCells::Periodic_Kernel,
 * LinkedCells.cpp:390-400 (strict < low / > high per dimension). */
void kor_wrap(const kor_grid *g, int64_t n_mol, const int64_t *mol_off, const double *com_mol, double *r);

/* Cell lists incl. halo copies, LinkedCells::writeIndices, LinkedCells.cpp:83-121. */
int  kor_bin(const kor_grid *g, int64_t n_mol, const int64_t *mol_off, const double *com_mol, kor_cells *c);
void kor_cells_free(kor_cells *c);

/* Full container update as LinkedCells::updateContainer (LinkedCells.cpp:65-81):
 * COM, wrap, zero forces, COM again, bin.  com_mol is scratch (n_mol*3). */
int  kor_update_container(const kor_grid *g, int64_t n_sites, int64_t n_mol, const int64_t *mol_off,
                          double *r, double *f, const double *m, double *com_mol, kor_cells *c);

/* Cell-pair sweep in LCC08Iterator order (LinkedCells.cpp:443-502, offsets
 * LinkedCells.h:74-86).  Writes up to cap pairs of linear cell indices and the
 * per-cell shift (3 doubles each); returns the number of cell pairs. */
int64_t kor_c08_pairs(const kor_grid *g, int64_t cap, int64_t *cells01, double *shift01);
/* Cell-triple sweep in LCTripletC08Iterator order (LinkedCells.cpp:504-572,
 * offsets LinkedCells.h:126-152). */
int64_t kor_c08_triples(const kor_grid *g, int64_t cap, int64_t *cells012, double *shift012);

/* Pair list as LinkedCells::updatePairList (LinkedCells.cpp:130-249): all
 * pairs of sites in C08 cell pairs, then same-cell pairs of domain cells.
 * pairs: 2 ints per entry; shifts: 6 doubles per entry.  Returns count (or,
 * with pairs == NULL, only counts). */
int64_t kor_pair_list(const kor_grid *g, const kor_cells *c, int64_t cap, int64_t *pairs, double *shifts);

enum { KOR_VIRIAL_COMPAT = 0, KOR_VIRIAL_CORRECT = 1 };
enum { KOR_ATM_SIGN_REFERENCE = 0, KOR_ATM_SIGN_PHYSICAL = 1 };
enum { KOR_ATM_ENUM_COMPAT = 0, KOR_ATM_ENUM_FULL = 1 };

typedef struct {
    double u_total;        /* LJ12_6_Sensor total potential (unique pairs) */
    double virial[6];      /* XX XY YY XZ YZ ZZ (PressureSensor.h:18)      */
    int64_t pairs_in_cutoff;/* entries with dr2 <= rc2 and different ids   */
} kor_lj_out;

/* LJ 12-6 force over the pair list, LJ12_6::LJ12_6_Force, LJ12_6.cpp:15-43.
 * Adds into f.  Also: the sensor potential (LJ12_6_Sensor.cpp:47-84, counting
 * entries with shift1 == 0 only), the virial (COMPAT: per list entry, as
 * PressureSensor.cpp:153-186; CORRECT: each physical pair once) and, if
 * ncount != NULL, per-site neighbour counts within the cutoff.
 * If uhist/fhist/ucnt/fcnt are non-NULL the sensor histograms over
 * 3*max_sigma with nbins bins are filled (Potential_Sensor.h:174-181). */
void kor_lj(const kor_grid *g, int64_t n_pairs, const int64_t *pairs, const double *shifts,
            const double *r, const double *eps, const double *sig, const uint64_t *id,
            double cutoff, int virial_mode, double *f, int64_t *ncount, kor_lj_out *out,
            int64_t nbins, double max_sigma, double *uhist, double *fhist, uint64_t *ucnt, uint64_t *fcnt);

typedef struct {
    double energy;         /* sum of V over counted triplets (physical V)  */
    double virial[6];
    int64_t triplets;      /* triplets inside the cutoff that were counted */
} kor_atm_out;

/* tabulated pair force (IBI_ForceFunctor): F(r) piecewise linear on ascending
 * nodes xs with values ys, lo below / hi above */
void kor_pair_table(int64_t n_pairs, const int64_t *pairs, const double *shifts, const double *r, double cutoff,
                    int64_t n_nodes, const double *xs, const double *ys, double lo, double hi, double *f);
/* ATM2B: the force factor applied by kor_lj / kor_lj_cells while set (1 = LJ12_6) */
void kor_set_lj_force_scale(double s);
/* The switched-cutoff option (no reference counterpart; width 0 = off, the
 * reference's truncated forms): LJ pair energies times S(r^2) from
 * (cutoff - lj_width)^2 to cutoff^2, ATM triplet energies times the product
 * of S over the three sides from (cutoff_3b - atm_width)^2 to cutoff_3b^2,
 * S the C1 smoothstep in the squared distance; forces are the gradients.
 * Applied by kor_lj, kor_lj_cells and kor_atm_vertex. */
void kor_set_switch(double lj_width, double atm_width);
double kor_atm2b_factor(double nu, double n_mol, double volume, double eps, double sig);
/* kor_lj without a materialised pair list: the same entries in C08 order,
 * generated from the cells (no virial, no histograms). */
void kor_lj_cells(const kor_grid *g, const kor_cells *c, const double *r, const double *eps, const double *sig,
                  const uint64_t *id, double cutoff, double *f, kor_lj_out *out);

/* ATM comp_force (ATM.h:36-69), returned as in the reference. */
double kor_atm_comp_force(double nu, double r_ab, double r_ac, double r_bc);

/* ATM in the reference's enumeration: ATM_NOLIST::handleTripleList
 * (ATM_NOLIST.cpp:20-159) -- C08 cell triples of three distinct cells
 * (halo-only triples skipped) followed by same-cell triples of domain cells;
 * forces only to sites in non-halo cells.  sign selects the reference's
 * +grad V (REFERENCE) or F = -grad V (PHYSICAL).  virial_mode COMPAT
 * reproduces ATM_Pressure (PressureSensor.cpp:223-286, no ZZ term, every
 * enumerated triplet) when with_virial is set; CORRECT counts each triplet
 * once with the physical force. */
void kor_atm_compat(const kor_grid *g, const kor_cells *c, const double *r, double nu, double cutoff,
                    int sign, int virial_mode, int with_virial, double *f, kor_atm_out *out);

/* ATM over ALL triplets with every side <= cutoff (FULL enumeration, the
 * physics reference): for each domain site the pairs of neighbours from the
 * 27 surrounding cells.  Force on the vertex only, energy and virial 1/3 per
 * vertex.  restrict_compat=1 keeps only triplets whose three cells are all
 * equal or all distinct, which must reproduce kor_atm_compat. */
void kor_atm_vertex(const kor_grid *g, const kor_cells *c, const double *r, double nu, double cutoff,
                    int sign, int restrict_compat, double *f, kor_atm_out *out);

/* ATM energy of one triplet: nu (1 + 3 cos g1 cos g2 cos g3) / (r01 r02 r12)^3. */
double kor_atm_energy(double nu, double r01, double r02, double r12);

/* FENE on same-id pairs, FENE::FENE_Force, FENE.cpp:15-43. */
void kor_fene(int64_t n_pairs, const int64_t *pairs, const double *shifts, const double *r,
              const double *eps, const double *sig, const uint64_t *id, double stiffness, double *f);

/* Per-component force clamp, Limit::Limit_Force, Limit.cpp:19-25. */
void kor_limit(int64_t n_sites, const double *eps, const double *sig, double limit_factor, double *f);

/* Harmonic bond k/2 (r - r0)^2 and angle k/2 (theta - theta0)^2 on explicit
 * topology (no reference counterpart).  Returns the bonded energy; adds
 * forces and (if virial != NULL) the pair-decomposed virial. */
double kor_bonded(int64_t n_bonds, const int64_t *bonds, double kb, double r0,
                  int64_t n_angles, const int64_t *angles, double ka, double theta0,
                  const double *r, const double *L, double *f, double *virial);

/* Velocity Verlet, Integrator::Step0 / Step1, Integrator.cpp:28-37. */
void kor_step0(int64_t n, double *r, double *v, const double *f, const double *m, double dt);
void kor_step1(int64_t n, double *v, const double *f, const double *m, double dt);

/* Temperature in K, TemperatureSensor::measure, TemperatureSensor.cpp:27-48
 * (sites inside [low, high] only, SciValue constant arithmetic reproduced). */
double kor_temperature(int64_t n, const double *r, const double *v, const double *m,
                       const double low[3], const double high[3]);

/* Kinetic tensor, PressureSensor::MomentumKernel (PressureSensor.cpp:143-151)
 * over the first n_terms sites (the reference uses getNumMolecules(), S11). */
void kor_momentum(int64_t n_terms, const double *v, const double *m, double *acc6);

/* Number of RDF bins: (uint64)(max_r / delta_r) (RDFSensor.cpp:18). */
int64_t kor_rdf_nbins(double max_r, double delta_r);
/* RDF histogram over molecule COMs, all ordered pairs, minimum image,
 * RDFSensor::RDF_Kernel (RDFSensor.cpp:61-72).  Adds into bins. */
void kor_rdf(int64_t n_mol, const double *com_mol, const double L[3], double max_r, double delta_r,
             int64_t nbins, double *bins);

/* Pressure-to-Pa conversion factor of PressureSensor::write (PressureSensor.cpp:49-51). */
double kor_pressure_factor(void);


/* ------------------------------------------------------------------------ */
/* Three-body surrogate (no reference counterpart): per-site descriptors, the */
/* 32-64-64-1 tanh MLP and the analytic forces, all in FP64.  Restates the   */
/* definition the CUDA kernels implement; parity is against this code and   */
/* finite differences (the reference has no surrogate).                      */
/* ------------------------------------------------------------------------ */
#define KOR_SUR_NR 16      /* radial Gaussians                       */
#define KOR_SUR_NC 4       /* angular channels (x4 invariants)       */
#define KOR_SUR_NF 32      /* features                               */
#define KOR_SUR_H 64       /* hidden width                           */
/* number of MLP parameters: W1 (64x32) b1 (64) W2 (64x64) b2 (64) w3 (64) b3 (1) */
#define KOR_SUR_NPARAM (KOR_SUR_H * KOR_SUR_NF + KOR_SUR_H + KOR_SUR_H * KOR_SUR_H + KOR_SUR_H + KOR_SUR_H + 1)

/* Raw features of one site from its neighbour vectors d_j = r_j - r_i
 * (n_nb x 3) inside rc: G_k = sum_j exp(-eta_r (r - mu_k)^2) fc(r), and per
 * channel c with g_c = exp(-eta_a (r - mu_c)^2) fc(r), M1 = sum g u,
 * M2 = sum g u u^T: I1 = |M1|^2, I2 = M2:M2, I3 = M1.M2.M1, I4 = tr(M2^3).
 * fc(r) = (cos(pi r / rc) + 1) / 2.  Feature order: G_0..15, I1_0..3,
 * I2_0..3, I3_0..3, I4_0..3. */
void kor_sur_features(int n_nb, const double *d, double rc, double *raw);
/* MLP on standardised features x = (raw - mean) / std: returns E (scaled
 * units) and, if dE_dx != NULL, dE/dx.  params layout as KOR_SUR_NPARAM. */
double kor_sur_mlp(const double *params, const double *x, double *dE_dx);
/* Gradient of the MLP output with respect to the parameters (same layout). */
void kor_sur_mlp_param_grad(const double *params, const double *x, double *grad);
/* Per-site energy E_i = e_scale * MLP(x_i) + e_shift and forces
 * F = -grad sum_i E_i for a periodic system, neighbour lists by all pairs
 * with the minimum image (small systems).  Returns the total energy. */
double kor_sur_energy_forces(int64_t n, const double *r, const double L[3], double rc, const double *params,
                             const double *fmean, const double *fstd, double e_scale, double e_shift,
                             double *e_site, double *f);

/* Threads used by the OpenMP loops (1 when built without OpenMP). */
int kor_num_threads(void);
void kor_set_num_threads(int n);

#ifdef __cplusplus
}
#endif
#endif
