/*
 * komd_oracle.c -- FP64 CPU restatement of KoMD's hot path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker of the CUDA engine; see komd_oracle.h).
 * Build with -ffp-contract=off: the COMPAT routines must round exactly like
 * the reference's double arithmetic (the reference build uses no FMA).
 *
 * All file:line citations refer to Snapex2409/KoMD, src/.
 */
#include "komd_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------ */
/* threads                                                                  */
/* ------------------------------------------------------------------------ */
int kor_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void kor_set_num_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

static inline void atomic_addd(double *p, double v) {
#ifdef _OPENMP
#pragma omp atomic
#endif
    *p += v;
}

/* ------------------------------------------------------------------------ */
/* grid (LinkedCells.cpp:11-45)                                             */
/* ------------------------------------------------------------------------ */
int kor_grid_init(kor_grid *g, const double low[3], const double high[3], double cs) {
    memset(g, 0, sizeof(*g));
    g->cs = cs;
    for (int d = 0; d < 3; d++) {
        g->low[d] = low[d];
        g->high[d] = high[d];
        g->L[d] = high[d] - low[d];
        const double q = floor(g->L[d] / cs);           /* math::ufloor */
        if (!(q >= 1.0)) return -1;
        g->nd[d] = (int64_t)q;
        g->nc[d] = g->nd[d] + 2;
        g->bl[d] = (double *)malloc(sizeof(double) * (size_t)g->nc[d]);
        g->bh[d] = (double *)malloc(sizeof(double) * (size_t)g->nc[d]);
        /* low starts one halo width below the domain; every cell is cs wide
         * except the last domain cell, which stretches to the domain's high */
        double lo = low[d] - cs;
        for (int64_t c = 0; c < g->nc[d]; c++) {
            const double hi = (c == g->nc[d] - 2) ? high[d] : (lo + cs);
            g->bl[d][c] = lo;
            g->bh[d][c] = hi;
            lo = hi;
        }
    }
    g->ncell = g->nc[0] * g->nc[1] * g->nc[2];
    return 0;
}

void kor_grid_free(kor_grid *g) {
    for (int d = 0; d < 3; d++) { free(g->bl[d]); free(g->bh[d]); g->bl[d] = g->bh[d] = NULL; }
}

/* per-dimension halo flag: +1 low halo, -1 high halo, 0 domain (LinkedCells.cpp:109-111) */
static inline int halo_dim(const kor_grid *g, int d, int64_t c) {
    const int check_low = g->bl[d][c] < g->low[d];
    const int check_high = g->bh[d][c] > g->high[d];
    return check_low - check_high;
}

int kor_is_halo(const kor_grid *g, int64_t x, int64_t y, int64_t z) {
    return halo_dim(g, 0, x) != 0 || halo_dim(g, 1, y) != 0 || halo_dim(g, 2, z) != 0;
}

static inline int64_t lin(const kor_grid *g, int64_t x, int64_t y, int64_t z) {
    return x + g->nc[0] * (y + g->nc[1] * z);
}

/* shift of a cell coordinate (LinkedCells.cpp:494-502): +L on the high halo
 * layer, -L on the low one */
static inline double cshift(const kor_grid *g, int d, int64_t c) {
    const int64_t cmax = g->nc[d] - 1;
    return (c >= cmax ? g->L[d] : 0.0) - (c <= 0 ? g->L[d] : 0.0);
}

/* ------------------------------------------------------------------------ */
/* COM, wrap, bin                                                           */
/* ------------------------------------------------------------------------ */
void kor_com(int64_t n_mol, const int64_t *mol_off, const double *r, const double *m, double *com) {
    for (int64_t k = 0; k < n_mol; k++) {
        double cx = 0, cy = 0, cz = 0, tm = 0;
        for (int64_t s = mol_off[k]; s < mol_off[k + 1]; s++) {
            const double ms = m[s];
            cx = cx + r[3 * s + 0] * ms;
            cy = cy + r[3 * s + 1] * ms;
            cz = cz + r[3 * s + 2] * ms;
            tm = tm + ms;
        }
        com[3 * k + 0] = cx / tm;
        com[3 * k + 1] = cy / tm;
        com[3 * k + 2] = cz / tm;
    }
}

void kor_wrap(const kor_grid *g, int64_t n_mol, const int64_t *mol_off, const double *com, double *r) {
    for (int64_t k = 0; k < n_mol; k++) {
        double off[3] = {0, 0, 0};
        for (int d = 0; d < 3; d++) {
            if (com[3 * k + d] < g->low[d]) off[d] = g->L[d];
            if (com[3 * k + d] > g->high[d]) off[d] = -g->L[d];
        }
        for (int64_t s = mol_off[k]; s < mol_off[k + 1]; s++)
            for (int d = 0; d < 3; d++) r[3 * s + d] += off[d];
    }
}

void kor_cells_free(kor_cells *c) {
    free(c->count); free(c->start); free(c->idx);
    memset(c, 0, sizeof(*c));
}

int kor_bin(const kor_grid *g, int64_t n_mol, const int64_t *mol_off, const double *com, kor_cells *c) {
    kor_cells_free(c);
    c->ncell = g->ncell;
    c->count = (int64_t *)calloc((size_t)g->ncell, sizeof(int64_t));
    c->start = (int64_t *)calloc((size_t)g->ncell + 1, sizeof(int64_t));
    int64_t *cell_of_mol = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n_mol > 0 ? n_mol : 1));
    for (int64_t k = 0; k < n_mol; k++) {
        int64_t cc[3];
        for (int d = 0; d < 3; d++) {
            const double fbin = (com[3 * k + d] - g->low[d]) / g->cs;
            int64_t b = (int64_t)fbin;
            if (b < 0) b = 0;
            if (b > g->nd[d] - 1) b = g->nd[d] - 1;
            cc[d] = b + 1;
        }
        const int64_t ci = lin(g, cc[0], cc[1], cc[2]);
        cell_of_mol[k] = ci;
        c->count[ci] += mol_off[k + 1] - mol_off[k];
    }
    /* halo cells copy their periodic source cell */
    int64_t *src = (int64_t *)malloc(sizeof(int64_t) * (size_t)g->ncell);
    for (int64_t z = 0; z < g->nc[2]; z++)
        for (int64_t y = 0; y < g->nc[1]; y++)
            for (int64_t x = 0; x < g->nc[0]; x++) {
                const int64_t ci = lin(g, x, y, z);
                const int hx = halo_dim(g, 0, x), hy = halo_dim(g, 1, y), hz = halo_dim(g, 2, z);
                if (hx == 0 && hy == 0 && hz == 0) { src[ci] = -1; continue; }
                src[ci] = lin(g, x + hx * g->nd[0], y + hy * g->nd[1], z + hz * g->nd[2]);
            }
    for (int64_t ci = 0; ci < g->ncell; ci++)
        if (src[ci] >= 0) c->count[ci] = c->count[src[ci]];
    int64_t acc = 0;
    for (int64_t ci = 0; ci < g->ncell; ci++) { c->start[ci] = acc; acc += c->count[ci]; }
    c->start[g->ncell] = acc;
    c->total = acc;
    c->idx = (int64_t *)malloc(sizeof(int64_t) * (size_t)(acc > 0 ? acc : 1));
    int64_t *fill = (int64_t *)calloc((size_t)g->ncell, sizeof(int64_t));
    for (int64_t k = 0; k < n_mol; k++) {
        const int64_t ci = cell_of_mol[k];
        for (int64_t s = mol_off[k]; s < mol_off[k + 1]; s++) c->idx[c->start[ci] + fill[ci]++] = s;
    }
    for (int64_t ci = 0; ci < g->ncell; ci++)
        if (src[ci] >= 0) memcpy(c->idx + c->start[ci], c->idx + c->start[src[ci]], sizeof(int64_t) * (size_t)c->count[ci]);
    free(fill); free(src); free(cell_of_mol);
    return 0;
}

int kor_update_container(const kor_grid *g, int64_t n_sites, int64_t n_mol, const int64_t *mol_off,
                         double *r, double *f, const double *m, double *com, kor_cells *c) {
    kor_com(n_mol, mol_off, r, m, com);
    kor_wrap(g, n_mol, mol_off, com, r);
    memset(f, 0, sizeof(double) * 3 * (size_t)n_sites);
    kor_com(n_mol, mol_off, r, m, com);
    return kor_bin(g, n_mol, mol_off, com, c);
}

/* ------------------------------------------------------------------------ */
/* C08 sweeps                                                               */
/* ------------------------------------------------------------------------ */
/* cell offsets of the pair sweep, LinkedCells.h:74-86 (o x y z xy yz xz xyz) */
static const int P_OFF[13][2][3] = {
    {{0,0,0},{0,1,0}}, {{0,1,0},{0,0,1}}, {{0,0,0},{0,0,1}}, {{0,0,0},{0,1,1}},
    {{1,0,0},{0,1,1}}, {{1,0,0},{0,1,0}}, {{1,0,0},{0,0,1}}, {{0,0,0},{1,0,0}},
    {{0,0,0},{1,1,0}}, {{1,1,0},{0,0,1}}, {{0,1,0},{1,0,1}}, {{0,0,0},{1,0,1}},
    {{0,0,0},{1,1,1}}};

#define O_ {0,0,0}
#define X_ {1,0,0}
#define Y_ {0,1,0}
#define Z_ {0,0,1}
#define XY_ {1,1,0}
#define YZ_ {0,1,1}
#define XZ_ {1,0,1}
#define XYZ_ {1,1,1}
/* cell offsets of the triplet sweep, LinkedCells.h:126-152 */
static const int T_OFF[44][3][3] = {
    {O_,X_,Y_},{O_,X_,XY_},{O_,Y_,XY_},{O_,X_,Z_},{O_,X_,XZ_},{O_,X_,YZ_},{O_,X_,XYZ_},
    {O_,Y_,Z_},{O_,Y_,XZ_},{O_,Y_,YZ_},{O_,Y_,XYZ_},{O_,XY_,Z_},{O_,XY_,XZ_},{O_,XY_,YZ_},
    {O_,XY_,XYZ_},{O_,Z_,XZ_},{O_,Z_,YZ_},{O_,Z_,XYZ_},{O_,XZ_,YZ_},{O_,XZ_,XYZ_},{O_,YZ_,XYZ_},
    {X_,Y_,XY_},{X_,Y_,Z_},{X_,Y_,XZ_},{X_,Y_,YZ_},{X_,Y_,XYZ_},{X_,XY_,Z_},{X_,XY_,YZ_},
    {Y_,XY_,Z_},{Y_,XY_,XZ_},{X_,Z_,XZ_},{Y_,Z_,XZ_},{XY_,Z_,XZ_},{X_,Z_,YZ_},{Y_,Z_,YZ_},
    {XY_,Z_,YZ_},{X_,Z_,XYZ_},{Y_,Z_,XYZ_},{XY_,Z_,XYZ_},{X_,XZ_,YZ_},{Y_,XZ_,YZ_},
    {XY_,XZ_,YZ_},{Y_,XZ_,XYZ_},{X_,YZ_,XYZ_}};
#undef O_
#undef X_
#undef Y_
#undef Z_
#undef XY_
#undef YZ_
#undef XZ_
#undef XYZ_

static inline int shift_nonzero(const double s[3]) { return s[0] != 0 || s[1] != 0 || s[2] != 0; }

/* Generic C08 sweep over bases (8 colours, stride 2, x fastest) with k cells
 * per offset entry; emits linear cell indices and shifts.  The skip rule of
 * checkState (LinkedCells.cpp:471-474, 531-534): every cell a halo -> skip. */
static int64_t c08_sweep(const kor_grid *g, int k, int nofs, const int (*ofs)[3], int64_t cap,
                         int64_t *cells, double *shifts) {
    int64_t n = 0;
    const int64_t cmx = g->nc[0] - 1, cmy = g->nc[1] - 1, cmz = g->nc[2] - 1;
    for (int color = 0; color < 8; color++) {
        const int64_t bx = color & 1, by = (color >> 1) & 1, bz = (color >> 2) & 1;
        for (int64_t z = bz;; z += 2) {
            for (int64_t y = by;; y += 2) {
                for (int64_t x = bx;; x += 2) {
                    for (int o = 0; o < nofs; o++) {
                        int64_t cc[3];
                        double sh[3][3];
                        int all_halo = 1;
                        for (int t = 0; t < k; t++) {
                            const int *of = ofs[o * k + t];
                            const int64_t cx = x + of[0], cy = y + of[1], cz = z + of[2];
                            cc[t] = lin(g, cx, cy, cz);
                            sh[t][0] = cshift(g, 0, cx);
                            sh[t][1] = cshift(g, 1, cy);
                            sh[t][2] = cshift(g, 2, cz);
                            if (!shift_nonzero(sh[t])) all_halo = 0;
                        }
                        if (all_halo) continue;
                        if (cells && n < cap) {
                            for (int t = 0; t < k; t++) {
                                cells[n * k + t] = cc[t];
                                for (int d = 0; d < 3; d++) shifts[(n * k + t) * 3 + d] = sh[t][d];
                            }
                        }
                        n++;
                    }
                    if (!(x < cmx - 2)) break;
                }
                if (!(y < cmy - 2)) break;
            }
            if (!(z < cmz - 2)) break;
        }
    }
    return n;
}

int64_t kor_c08_pairs(const kor_grid *g, int64_t cap, int64_t *cells01, double *shift01) {
    return c08_sweep(g, 2, 13, (const int (*)[3])P_OFF, cap, cells01, shift01);
}

int64_t kor_c08_triples(const kor_grid *g, int64_t cap, int64_t *cells012, double *shift012) {
    return c08_sweep(g, 3, 44, (const int (*)[3])T_OFF, cap, cells012, shift012);
}

/* list of domain cells in LCCellIterator order (x fastest) */
static int64_t domain_cells(const kor_grid *g, int64_t *out) {
    int64_t n = 0;
    for (int64_t z = 0; z < g->nc[2]; z++)
        for (int64_t y = 0; y < g->nc[1]; y++)
            for (int64_t x = 0; x < g->nc[0]; x++)
                if (!kor_is_halo(g, x, y, z)) { if (out) out[n] = lin(g, x, y, z); n++; }
    return n;
}

/* same-cell pair decode of PairListSingle_Kernel (LinkedCells.h:234-267) */
static inline void single_pair(int64_t local, int64_t *i, int64_t *j) {
    int64_t ii = (int64_t)floor((-1 + sqrt((double)(1 + 8 * local))) / 2.0);
    *j = local - ii * (ii + 1) / 2;
    *i = ii + 1;
}

int64_t kor_pair_list(const kor_grid *g, const kor_cells *c, int64_t cap, int64_t *pairs, double *shifts) {
    const int64_t ncp = kor_c08_pairs(g, 0, NULL, NULL);
    int64_t *cp = (int64_t *)malloc(sizeof(int64_t) * 2 * (size_t)ncp);
    double *sp = (double *)malloc(sizeof(double) * 6 * (size_t)ncp);
    kor_c08_pairs(g, ncp, cp, sp);
    int64_t n = 0;
    for (int64_t q = 0; q < ncp; q++) {
        const int64_t c0 = cp[2 * q], c1 = cp[2 * q + 1];
        const int64_t n0 = c->count[c0], n1 = c->count[c1];
        for (int64_t loc = 0; loc < n0 * n1; loc++) {
            if (pairs && n < cap) {
                pairs[2 * n] = c->idx[c->start[c0] + loc % n0];
                pairs[2 * n + 1] = c->idx[c->start[c1] + loc / n0];
                memcpy(shifts + 6 * n, sp + 6 * q, sizeof(double) * 6);
            }
            n++;
        }
    }
    const int64_t ndc = domain_cells(g, NULL);
    int64_t *dc = (int64_t *)malloc(sizeof(int64_t) * (size_t)ndc);
    domain_cells(g, dc);
    for (int64_t q = 0; q < ndc; q++) {
        const int64_t ci = dc[q], nn = c->count[ci];
        for (int64_t loc = 0; loc < nn * (nn - 1) / 2; loc++) {
            if (pairs && n < cap) {
                int64_t i, j;
                single_pair(loc, &i, &j);
                pairs[2 * n] = c->idx[c->start[ci] + i];
                pairs[2 * n + 1] = c->idx[c->start[ci] + j];
                memset(shifts + 6 * n, 0, sizeof(double) * 6);
            }
            n++;
        }
    }
    free(dc); free(cp); free(sp);
    return n;
}

/* ------------------------------------------------------------------------ */
/* LJ 12-6 (LJ12_6.cpp:15-43, LJ12_6_Sensor.cpp:47-84, PressureSensor.cpp:153-186) */
/* ------------------------------------------------------------------------ */
static inline uint64_t pot_bin(double r, double sigma, uint64_t bins) {
    if (r < 0) return 0;
    const double max_size = 3.0 * sigma;
    const double bin_width = max_size / (double)bins;
    uint64_t b = (uint64_t)(r / bin_width);
    if (b > bins - 1) b = bins - 1;
    return b;
}

/* FunctionPL::evaluateAt (plugins/IBI/IBI_Math.h:30-44): linear scan for the
 * first node >= x, then ya + (yb - ya) / (xb - xa) * (x - xa).  At x == x[0]
 * the reference would read x[-1]; the first segment is used instead. */
static double table_eval(double x, int64_t n, const double *xs, const double *ys, double lo, double hi) {
    if (x > xs[n - 1]) return hi;
    if (x < xs[0]) return lo;
    int64_t i = 0;
    while (x > xs[i]) {
        i++;
        if (i == n) break;
    }
    if (i < 1) i = 1;
    const double ya = ys[i - 1], yb = ys[i], xa = xs[i - 1], xb = xs[i];
    return ya + (yb - ya) / (xb - xa) * (x - xa);
}

/* IBI_ForceFunctor<IBI_Default>::IBI_Force (plugins/IBI/IBI_ForceFunctor.cpp:18-37):
 * every listed pair inside the cutoff (no same-molecule test), force =
 * (dr / r) * F(r), added to the unshifted sides in list order. */
void kor_pair_table(int64_t n_pairs, const int64_t *pairs, const double *shifts, const double *r, double cutoff,
                    int64_t n_nodes, const double *xs, const double *ys, double lo, double hi, double *f) {
    const double cutoff2 = pow(cutoff, 2);
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int64_t p = 0; p < n_pairs; p++) {
        const int64_t s0 = pairs[2 * p], s1 = pairs[2 * p + 1];
        const double *sh0 = shifts + 6 * p, *sh1 = shifts + 6 * p + 3;
        double dr[3];
        for (int d = 0; d < 3; d++) dr[d] = (r[3 * s0 + d] + sh0[d]) - (r[3 * s1 + d] + sh1[d]);
        const double dr2 = dr[0] * dr[0] + dr[1] * dr[1] + dr[2] * dr[2];
        if (dr2 > cutoff2) continue;
        const double rr = sqrt(dr2);
        const double F = table_eval(rr, n_nodes, xs, ys, lo, hi);
        double fo[3];
        for (int d = 0; d < 3; d++) fo[d] = (dr[d] / rr) * F;
        if (!shift_nonzero(sh0)) for (int d = 0; d < 3; d++) atomic_addd(&f[3 * s0 + d], fo[d]);
        if (!shift_nonzero(sh1)) for (int d = 0; d < 3; d++) atomic_addd(&f[3 * s1 + d], -fo[d]);
    }
}

/* ATM2B (potentials/ATM2B.cpp:22-47) is LJ12_6_Force with the force vector
 * multiplied by potential_factor: force = dr * fac * potential_factor.  The
 * factor applies to kor_lj and kor_lj_cells while set (1 = plain LJ). */
static double g_lj_fscale = 1.0;
void kor_set_lj_force_scale(double s) { g_lj_fscale = s; }

/* The switched-cutoff option (not in the reference; off unless set): the LJ
 * pair energy and the ATM triplet energy are multiplied by the C1 smoothstep
 * S(x) = t^2 (3 - 2 t), t = (rc^2 - x) / (rc^2 - rs^2) clamped to [0, 1], of
 * the squared distance x (for ATM the product over the three sides), with
 * rs = rc - width; forces are the exact gradients of the switched energies.
 * width 0 keeps the reference's truncated potentials. */
static double g_sw_lj = 0.0, g_sw_atm = 0.0;
void kor_set_switch(double lj_width, double atm_width) { g_sw_lj = lj_width; g_sw_atm = atm_width; }

/* S(x) and dS/dx for the switch from rs^2 to rc^2 */
static void sw_eval(double x, double rc, double width, double *S, double *dS) {
    const double rc2 = rc * rc, rs = rc - width, rs2 = rs * rs, w = rc2 - rs2;
    double t = (rc2 - x) / w;
    if (t >= 1.0) { *S = 1.0; *dS = 0.0; return; }
    if (t <= 0.0) { *S = 0.0; *dS = 0.0; return; }
    *S = t * t * (3.0 - 2.0 * t);
    *dS = -6.0 * t * (1.0 - t) / w;
}

/* ATM2B::ATM2B (ATM2B.cpp:9-20): 1 - (2 nu rho) / (3 eps sig^6) with rho =
 * molecules / volume and eps, sig of the first site of component 0 (all
 * internal units). */
double kor_atm2b_factor(double nu, double n_mol, double volume, double eps, double sig) {
    const double rho = n_mol / volume;
    const double sig6 = pow(sig, 6);
    return 1.0 - ((2 * nu * rho) / (3 * eps * sig6));
}

void kor_lj(const kor_grid *g, int64_t n_pairs, const int64_t *pairs, const double *shifts,
            const double *r, const double *eps, const double *sig, const uint64_t *id,
            double cutoff, int virial_mode, double *f, int64_t *ncount, kor_lj_out *out,
            int64_t nbins, double max_sigma, double *uhist, double *fhist, uint64_t *ucnt, uint64_t *fcnt) {
    (void)g;
    const double cutoff2 = pow(cutoff, 2);
    double u_total = 0, w[6] = {0, 0, 0, 0, 0, 0};
    int64_t inside = 0;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) reduction(+ : u_total, inside) reduction(+ : w[:6])
#endif
    for (int64_t p = 0; p < n_pairs; p++) {
        const int64_t s0 = pairs[2 * p], s1 = pairs[2 * p + 1];
        if (id[s0] == id[s1]) continue;
        const double *sh0 = shifts + 6 * p, *sh1 = shifts + 6 * p + 3;
        double dr[3];
        for (int d = 0; d < 3; d++) dr[d] = (r[3 * s0 + d] + sh0[d]) - (r[3 * s1 + d] + sh1[d]);
        const double dr2 = dr[0] * dr[0] + dr[1] * dr[1] + dr[2] * dr[2];
        if (dr2 > cutoff2) continue;
        inside++;
        const double invdr2 = 1. / dr2;
        const double sigma = (sig[s0] + sig[s1]) / 2.0;
        const double epsilon = sqrt(eps[s0] * eps[s1]);
        const double sig2 = sigma * sigma;
        const double lj6 = pow(sig2 * invdr2, 3.0);
        const double lj12 = pow(lj6, 2.0);
        double fac = 24.0 * epsilon * (2.0 * lj12 - lj6) * invdr2;
        double swS = 1.0;
        if (g_sw_lj > 0.0) {   /* switched cutoff: U S, force fac S - 2 U dS/dx */
            double dS;
            sw_eval(dr2, cutoff, g_sw_lj, &swS, &dS);
            fac = fac * swS - 2.0 * (4.0 * epsilon * (lj12 - lj6)) * dS;
        }
        double fo[3] = {dr[0] * fac, dr[1] * fac, dr[2] * fac};
        if (g_lj_fscale != 1.0)
            for (int d = 0; d < 3; d++) fo[d] = fo[d] * g_lj_fscale;
        const int dom0 = !shift_nonzero(sh0), dom1 = !shift_nonzero(sh1);
        if (dom0) for (int d = 0; d < 3; d++) atomic_addd(&f[3 * s0 + d], fo[d]);
        if (dom1) for (int d = 0; d < 3; d++) atomic_addd(&f[3 * s1 + d], -fo[d]);
        if (ncount) {
#ifdef _OPENMP
            if (dom0) {
#pragma omp atomic
                ncount[s0]++;
            }
            if (dom1) {
#pragma omp atomic
                ncount[s1]++;
            }
#else
            if (dom0) ncount[s0]++;
            if (dom1) ncount[s1]++;
#endif
        }
        /* virial */
        double wt = 1.0;
        if (virial_mode == KOR_VIRIAL_CORRECT) wt = 0.5 * (double)(dom0 + dom1);
        const double vxx = 0.5 * (dr[0] * fo[0] + dr[0] * fo[0]);
        const double vxy = 0.5 * (dr[0] * fo[1] + dr[1] * fo[0]);
        const double vyy = 0.5 * (dr[1] * fo[1] + dr[1] * fo[1]);
        const double vxz = 0.5 * (dr[0] * fo[2] + dr[2] * fo[0]);
        const double vyz = 0.5 * (dr[1] * fo[2] + dr[2] * fo[1]);
        const double vzz = 0.5 * (dr[2] * fo[2] + dr[2] * fo[2]);
        if (wt == 1.0) { w[0] += vxx; w[1] += vxy; w[2] += vyy; w[3] += vxz; w[4] += vyz; w[5] += vzz; }
        else { w[0] += wt * vxx; w[1] += wt * vxy; w[2] += wt * vyy; w[3] += wt * vxz; w[4] += wt * vyz; w[5] += wt * vzz; }
        /* sensor: ignore entries whose second side is a halo image */
        if (!shift_nonzero(sh1)) {
            const double rpos = sqrt(pow(dr[0], 2) + pow(dr[1], 2) + pow(dr[2], 2));
            const double u = 4.0 * epsilon * (lj12 - lj6) * swS;
            u_total += u;
            if (uhist) {
                const double fr = 24.0 * epsilon * (2.0 * lj12 - lj6) / rpos;
                const uint64_t b = pot_bin(rpos, max_sigma, (uint64_t)nbins);
                atomic_addd(&fhist[b], fr);
                atomic_addd(&uhist[b], u);
#ifdef _OPENMP
#pragma omp atomic
#endif
                fcnt[b]++;
#ifdef _OPENMP
#pragma omp atomic
#endif
                ucnt[b]++;
            }
        }
    }
    if (out) {
        out->u_total = u_total;
        for (int d = 0; d < 6; d++) out->virial[d] = w[d];
        out->pairs_in_cutoff = inside;
    }
}


/* LJ over the same entries as kor_lj, generated on the fly from the C08 cell
 * pairs and the same-cell pairs instead of a materialised pair list (the
 * reference's PLU kernels write that list; the arithmetic per entry is
 * identical).  Used for large systems, where the list would take GBs. */
void kor_lj_cells(const kor_grid *g, const kor_cells *c, const double *r, const double *eps, const double *sig,
                  const uint64_t *id, double cutoff, double *f, kor_lj_out *out) {
    const double cutoff2 = pow(cutoff, 2);
    const int64_t ncp = kor_c08_pairs(g, 0, NULL, NULL);
    int64_t *cp = (int64_t *)malloc(sizeof(int64_t) * 2 * (size_t)(ncp > 0 ? ncp : 1));
    double *sp = (double *)malloc(sizeof(double) * 6 * (size_t)(ncp > 0 ? ncp : 1));
    kor_c08_pairs(g, ncp, cp, sp);
    const int64_t ndc = domain_cells(g, NULL);
    int64_t *dc = (int64_t *)malloc(sizeof(int64_t) * (size_t)(ndc > 0 ? ndc : 1));
    domain_cells(g, dc);
    static const double zero6[6] = {0, 0, 0, 0, 0, 0};
    double u_total = 0;
    int64_t inside = 0;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : u_total, inside)
#endif
    for (int64_t q = 0; q < ncp + ndc; q++) {
        int64_t c0, c1;
        const double *sh;
        int single = q >= ncp;
        if (!single) { c0 = cp[2 * q]; c1 = cp[2 * q + 1]; sh = sp + 6 * q; }
        else { c0 = c1 = dc[q - ncp]; sh = zero6; }
        const int64_t n0 = c->count[c0], n1 = c->count[c1];
        const int64_t *i0 = c->idx + c->start[c0], *i1 = c->idx + c->start[c1];
        const int64_t total = single ? n0 * (n0 - 1) / 2 : n0 * n1;
        const int dom0 = !shift_nonzero(sh), dom1 = !shift_nonzero(sh + 3);
        for (int64_t loc = 0; loc < total; loc++) {
            int64_t a, b;
            if (single) single_pair(loc, &a, &b);
            else { a = loc % n0; b = loc / n0; }
            const int64_t s0 = i0[a], s1 = i1[b];
            if (id[s0] == id[s1]) continue;
            double dr[3];
            for (int d = 0; d < 3; d++) dr[d] = (r[3 * s0 + d] + sh[d]) - (r[3 * s1 + d] + sh[3 + d]);
            const double dr2 = dr[0] * dr[0] + dr[1] * dr[1] + dr[2] * dr[2];
            if (dr2 > cutoff2) continue;
            inside++;
            const double invdr2 = 1. / dr2;
            const double sigma = (sig[s0] + sig[s1]) / 2.0;
            const double epsilon = sqrt(eps[s0] * eps[s1]);
            const double sig2 = sigma * sigma;
            const double lj6 = pow(sig2 * invdr2, 3.0);
            const double lj12 = pow(lj6, 2.0);
            double fac = 24.0 * epsilon * (2.0 * lj12 - lj6) * invdr2;
            double swS = 1.0;
            if (g_sw_lj > 0.0) {   /* switched cutoff (kor_set_switch) */
                double dS;
                sw_eval(dr2, cutoff, g_sw_lj, &swS, &dS);
                fac = fac * swS - 2.0 * (4.0 * epsilon * (lj12 - lj6)) * dS;
            }
            double fo[3] = {dr[0] * fac, dr[1] * fac, dr[2] * fac};
            if (g_lj_fscale != 1.0)
                for (int d = 0; d < 3; d++) fo[d] = fo[d] * g_lj_fscale;
            if (dom0) for (int d = 0; d < 3; d++) atomic_addd(&f[3 * s0 + d], fo[d]);
            if (dom1) for (int d = 0; d < 3; d++) atomic_addd(&f[3 * s1 + d], -fo[d]);
            if (dom1) u_total += 4.0 * epsilon * (lj12 - lj6) * swS;
        }
    }
    free(dc); free(cp); free(sp);
    if (out) {
        out->u_total = u_total;
        for (int d = 0; d < 6; d++) out->virial[d] = 0.0;
        out->pairs_in_cutoff = inside;
    }
}

/* ------------------------------------------------------------------------ */
/* ATM                                                                      */
/* ------------------------------------------------------------------------ */
double kor_atm_comp_force(double nu, double r_ab, double r_ac, double r_bc) {
    /* ATM.h:36-69, term by term */
    const double r_ab2 = r_ab * r_ab, r_ab3 = r_ab2 * r_ab, r_ab4 = r_ab2 * r_ab2, r_ab6 = r_ab3 * r_ab3;
    const double r_ac2 = r_ac * r_ac, r_ac3 = r_ac2 * r_ac, r_ac5 = r_ac3 * r_ac2;
    const double r_bc2 = r_bc * r_bc, r_bc3 = r_bc2 * r_bc, r_bc5 = r_bc3 * r_bc2;
    return ((3. * nu) / (8. * r_ab)) *
           (-(8.) / (r_ab4 * r_ac3 * r_bc3)
            - (1.) / (r_ac5 * r_bc5)
            + (5. * r_ac) / (r_ab6 * r_bc5)
            + (5. * r_bc) / (r_ab6 * r_ac5)
            - (1.) / (r_ab2 * r_ac3 * r_bc5)
            - (1.) / (r_ab2 * r_ac5 * r_bc3)
            - (3.) / (r_ab4 * r_ac * r_bc5)
            - (3.) / (r_ab4 * r_ac5 * r_bc)
            - (5.) / (r_ab6 * r_ac * r_bc3)
            - (5.) / (r_ab6 * r_ac3 * r_bc)
            + (6.) / (r_ab4 * r_ac3 * r_bc3));
}

double kor_atm_energy(double nu, double a, double b, double c) {
    /* a = r01, b = r02, c = r12; cosines by the law of cosines */
    const double a2 = a * a, b2 = b * b, c2 = c * c;
    const double c0 = (a2 + b2 - c2) / (2.0 * a * b);   /* angle at 0 */
    const double c1 = (a2 + c2 - b2) / (2.0 * a * c);   /* angle at 1 */
    const double c2_ = (b2 + c2 - a2) / (2.0 * b * c);  /* angle at 2 */
    const double p = a * b * c;
    return nu * (1.0 + 3.0 * c0 * c1 * c2_) / (p * p * p);
}

/* one triplet, ATM_NOLIST_Force::operator() (ATM_NOLIST.cpp:124-159);
 * returns 1 if inside the cutoff */
static int atm_triplet(const double *r, int64_t s0, int64_t s1, int64_t s2, const double *sh0,
                       const double *sh1, const double *sh2, double nu, double cutoff2, double sgn,
                       double *f, int dom0, int dom1, int dom2, double *energy, double *w6, int vmode,
                       int with_virial) {
    double r0[3], r1[3], r2[3], d01[3], d02[3], d12[3];
    for (int d = 0; d < 3; d++) {
        r0[d] = r[3 * s0 + d] + sh0[d];
        r1[d] = r[3 * s1 + d] + sh1[d];
        r2[d] = r[3 * s2 + d] + sh2[d];
    }
    for (int d = 0; d < 3; d++) { d01[d] = r0[d] - r1[d]; d02[d] = r0[d] - r2[d]; d12[d] = r1[d] - r2[d]; }
    const double q01 = d01[0] * d01[0] + d01[1] * d01[1] + d01[2] * d01[2];
    const double q02 = d02[0] * d02[0] + d02[1] * d02[1] + d02[2] * d02[2];
    const double q12 = d12[0] * d12[0] + d12[1] * d12[1] + d12[2] * d12[2];
    if (q01 > cutoff2 || q02 > cutoff2 || q12 > cutoff2) return 0;
    const double a = sqrt(q01), b = sqrt(q02), c = sqrt(q12);
    const double v01 = kor_atm_comp_force(nu, a, b, c);
    const double v02 = kor_atm_comp_force(nu, b, a, c);
    const double v12 = kor_atm_comp_force(nu, c, a, b);
    double f0[3], f1[3], f2[3];
    for (int d = 0; d < 3; d++) {
        f0[d] = d01[d] * v01 + d02[d] * v02;
        f1[d] = d01[d] * (-v01) + d12[d] * v12;
        f2[d] = d02[d] * (-v02) + d12[d] * (-v12);
    }
    if (sgn != 1.0) for (int d = 0; d < 3; d++) { f0[d] = -f0[d]; f1[d] = -f1[d]; f2[d] = -f2[d]; }
    if (dom0) for (int d = 0; d < 3; d++) atomic_addd(&f[3 * s0 + d], f0[d]);
    if (dom1) for (int d = 0; d < 3; d++) atomic_addd(&f[3 * s1 + d], f1[d]);
    if (dom2) for (int d = 0; d < 3; d++) atomic_addd(&f[3 * s2 + d], f2[d]);
    const double wt = (vmode == KOR_VIRIAL_CORRECT) ? (double)(dom0 + dom1 + dom2) / 3.0 : 1.0;
    *energy += wt * kor_atm_energy(nu, a, b, c);
    if (with_virial) {
        /* ATM_Pressure, PressureSensor.cpp:223-286 (dVdR = -comp_force) */
        const double p01 = -v01, p02 = -v02, p12 = -v12;
        double g01[3], g02[3], g12[3];
        for (int d = 0; d < 3; d++) { g01[d] = d01[d] * p01; g02[d] = d02[d] * p02; g12[d] = d12[d] * p12; }
        double acc[6];
        acc[0] = 0.5 * (d01[0] * g01[0] + d01[0] * g01[0] + d12[0] * g12[0] + d12[0] * g12[0] + d02[0] * g02[0] + d02[0] * g02[0]);
        acc[1] = 0.5 * (d01[0] * g01[1] + d01[1] * g01[0] + d12[0] * g12[1] + d12[1] * g12[0] + d02[0] * g02[1] + d02[1] * g02[0]);
        acc[2] = 0.5 * (d01[1] * g01[1] + d01[1] * g01[1] + d12[1] * g12[1] + d12[1] * g12[1] + d02[1] * g02[1] + d02[1] * g02[1]);
        acc[3] = 0.5 * (d01[0] * g01[2] + d01[2] * g01[0] + d12[0] * g12[2] + d12[2] * g12[0] + d02[0] * g02[2] + d02[2] * g02[0]);
        acc[4] = 0.5 * (d01[1] * g01[2] + d01[2] * g01[1] + d12[1] * g12[2] + d12[2] * g12[1] + d02[1] * g02[2] + d02[2] * g02[1]);
        acc[5] = (vmode == KOR_VIRIAL_COMPAT) ? 0.0 /* no ZZ term in the reference */
                 : 0.5 * (d01[2] * g01[2] + d01[2] * g01[2] + d12[2] * g12[2] + d12[2] * g12[2] + d02[2] * g02[2] + d02[2] * g02[2]);
        for (int d = 0; d < 6; d++) w6[d] += wt * acc[d];
    }
    return 1;
}

void kor_atm_compat(const kor_grid *g, const kor_cells *c, const double *r, double nu, double cutoff,
                    int sign, int virial_mode, int with_virial, double *f, kor_atm_out *out) {
    const double cutoff2 = pow(cutoff, 2);
    const double sgn = (sign == KOR_ATM_SIGN_REFERENCE) ? 1.0 : -1.0;
    const int64_t nct = kor_c08_triples(g, 0, NULL, NULL);
    int64_t *ct = (int64_t *)malloc(sizeof(int64_t) * 3 * (size_t)(nct > 0 ? nct : 1));
    double *st = (double *)malloc(sizeof(double) * 9 * (size_t)(nct > 0 ? nct : 1));
    kor_c08_triples(g, nct, ct, st);
    double energy = 0, w[6] = {0, 0, 0, 0, 0, 0};
    int64_t ntrip = 0;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : energy, ntrip) reduction(+ : w[:6])
#endif
    for (int64_t q = 0; q < nct; q++) {
        const int64_t c0 = ct[3 * q], c1 = ct[3 * q + 1], c2 = ct[3 * q + 2];
        const double *sh0 = st + 9 * q, *sh1 = sh0 + 3, *sh2 = sh0 + 6;
        const int d0 = !shift_nonzero(sh0), d1 = !shift_nonzero(sh1), d2 = !shift_nonzero(sh2);
        const int64_t n0 = c->count[c0], n1 = c->count[c1], n2 = c->count[c2];
        const int64_t *i0 = c->idx + c->start[c0], *i1 = c->idx + c->start[c1], *i2 = c->idx + c->start[c2];
        for (int64_t loc = 0; loc < n0 * n1 * n2; loc++) {
            const int64_t a = loc % n0, b = (loc / n0) % n1, k = loc / (n0 * n1);
            ntrip += atm_triplet(r, i0[a], i1[b], i2[k], sh0, sh1, sh2, nu, cutoff2, sgn, f, d0, d1, d2, &energy, w,
                                 virial_mode, with_virial);
        }
    }
    /* same-cell triples of domain cells, ATM_NOLISTSingle_Kernel decode */
    const int64_t ndc = domain_cells(g, NULL);
    int64_t *dc = (int64_t *)malloc(sizeof(int64_t) * (size_t)(ndc > 0 ? ndc : 1));
    domain_cells(g, dc);
    int64_t maxn = 0;
    for (int64_t q = 0; q < ndc; q++) if (c->count[dc[q]] > maxn) maxn = c->count[dc[q]];
    int64_t *tri = (int64_t *)malloc(sizeof(int64_t) * (size_t)(maxn > 0 ? maxn : 1));
    for (int64_t i = 1; i < maxn + 1; i++) tri[i - 1] = i * (i + 1) * (i + 2) / 6;
    static const double zero[3] = {0, 0, 0};
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : energy, ntrip) reduction(+ : w[:6])
#endif
    for (int64_t q = 0; q < ndc; q++) {
        const int64_t ci = dc[q], n = c->count[ci];
        const int64_t *ix = c->idx + c->start[ci];
        for (int64_t loc = 0; loc < n * (n - 1) * (n - 2) / 6; loc++) {
            int64_t kidx = -1;
            for (int64_t pos = 0; pos < maxn; pos++) if (tri[pos] > loc) { kidx = pos; break; }
            const int64_t k = kidx + 2;
            int64_t tmp = loc;
            if (kidx > 0) tmp -= tri[kidx - 1];
            int64_t j = (int64_t)floor((-1 + sqrt((double)(1 + 8 * tmp))) / 2.0);
            const int64_t i = tmp - j * (j + 1) / 2;
            j += 1;
            ntrip += atm_triplet(r, ix[i], ix[j], ix[k], zero, zero, zero, nu, cutoff2, sgn, f, 1, 1, 1, &energy, w,
                                 virial_mode, with_virial);
        }
    }
    free(tri); free(dc); free(ct); free(st);
    if (out) {
        out->energy = energy;
        for (int d = 0; d < 6; d++) out->virial[d] = w[d];
        out->triplets = ntrip;
    }
}

typedef struct { int64_t s; int64_t cell; double p[3]; double d[3]; double q; } nb_t;

void kor_atm_vertex(const kor_grid *g, const kor_cells *c, const double *r, double nu, double cutoff,
                    int sign, int restrict_compat, double *f, kor_atm_out *out) {
    const double cutoff2 = pow(cutoff, 2);
    const double sgn = (sign == KOR_ATM_SIGN_REFERENCE) ? 1.0 : -1.0;
    const int64_t ndc = domain_cells(g, NULL);
    int64_t *dc = (int64_t *)malloc(sizeof(int64_t) * (size_t)(ndc > 0 ? ndc : 1));
    domain_cells(g, dc);
    double energy = 0, w[6] = {0, 0, 0, 0, 0, 0};
    int64_t nvert = 0;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 4) reduction(+ : energy, nvert) reduction(+ : w[:6])
#endif
    for (int64_t q = 0; q < ndc; q++) {
        const int64_t ci = dc[q];
        const int64_t cx = ci % g->nc[0], cy = (ci / g->nc[0]) % g->nc[1], cz = ci / (g->nc[0] * g->nc[1]);
        int64_t cap = 0;
        for (int dz = -1; dz <= 1; dz++) for (int dy = -1; dy <= 1; dy++) for (int dx = -1; dx <= 1; dx++)
            cap += c->count[lin(g, cx + dx, cy + dy, cz + dz)];
        nb_t *nb = (nb_t *)malloc(sizeof(nb_t) * (size_t)(cap > 0 ? cap : 1));
        for (int64_t a = 0; a < c->count[ci]; a++) {
            const int64_t si = c->idx[c->start[ci] + a];
            const double *ri = r + 3 * si;
            int64_t nn = 0;
            for (int dz = -1; dz <= 1; dz++) for (int dy = -1; dy <= 1; dy++) for (int dx = -1; dx <= 1; dx++) {
                const int64_t x = cx + dx, y = cy + dy, z = cz + dz, cj = lin(g, x, y, z);
                const double sh[3] = {cshift(g, 0, x), cshift(g, 1, y), cshift(g, 2, z)};
                for (int64_t b = 0; b < c->count[cj]; b++) {
                    const int64_t sj = c->idx[c->start[cj] + b];
                    if (cj == ci && sj == si) continue;
                    nb_t e;
                    e.s = sj; e.cell = cj;
                    for (int d = 0; d < 3; d++) { e.p[d] = r[3 * sj + d] + sh[d]; e.d[d] = ri[d] - e.p[d]; }
                    e.q = e.d[0] * e.d[0] + e.d[1] * e.d[1] + e.d[2] * e.d[2];
                    if (e.q > cutoff2) continue;
                    nb[nn++] = e;
                }
            }
            double fi[3] = {0, 0, 0};
            for (int64_t u = 0; u < nn; u++) {
                for (int64_t v = u + 1; v < nn; v++) {
                    if (restrict_compat) {
                        const int same = (nb[u].cell == ci) + (nb[v].cell == ci) + (nb[u].cell == nb[v].cell);
                        if (!(same == 3 || same == 0)) continue;
                    }
                    double d12[3];
                    for (int d = 0; d < 3; d++) d12[d] = nb[u].p[d] - nb[v].p[d];
                    const double q12 = d12[0] * d12[0] + d12[1] * d12[1] + d12[2] * d12[2];
                    if (q12 > cutoff2) continue;
                    const double a_ = sqrt(nb[u].q), b_ = sqrt(nb[v].q), c_ = sqrt(q12);
                    double v01 = kor_atm_comp_force(nu, a_, b_, c_);
                    double v02 = kor_atm_comp_force(nu, b_, a_, c_);
                    double v12 = kor_atm_comp_force(nu, c_, a_, b_);
                    double V = kor_atm_energy(nu, a_, b_, c_);
                    if (g_sw_atm > 0.0) {
                        /* switched: V Sa Sb Sc; (1/r) dV_sw/dr = S S S (1/r) dV/dr + V (prod of the
                         * other two S) 2 dS/dx for each side.  comp_force is (1/r) dV/dr with the
                         * reference's sign (the force adds +grad V) */
                        double Sa, dSa, Sb, dSb, Sc, dSc;
                        sw_eval(nb[u].q, cutoff, g_sw_atm, &Sa, &dSa);
                        sw_eval(nb[v].q, cutoff, g_sw_atm, &Sb, &dSb);
                        sw_eval(q12, cutoff, g_sw_atm, &Sc, &dSc);
                        v01 = Sa * Sb * Sc * v01 + V * Sb * Sc * 2.0 * dSa;
                        v02 = Sa * Sb * Sc * v02 + V * Sa * Sc * 2.0 * dSb;
                        v12 = Sa * Sb * Sc * v12 + V * Sa * Sb * 2.0 * dSc;
                        V = V * Sa * Sb * Sc;
                    }
                    for (int d = 0; d < 3; d++) fi[d] += sgn * (nb[u].d[d] * v01 + nb[v].d[d] * v02);
                    energy += V / 3.0;
                    const double p01 = -v01, p02 = -v02, p12 = -v12;
                    const double *e01 = nb[u].d, *e02 = nb[v].d;
                    w[0] += (p01 * e01[0] * e01[0] + p02 * e02[0] * e02[0] + p12 * d12[0] * d12[0]) / 3.0;
                    w[1] += (p01 * e01[0] * e01[1] + p02 * e02[0] * e02[1] + p12 * d12[0] * d12[1]) / 3.0;
                    w[2] += (p01 * e01[1] * e01[1] + p02 * e02[1] * e02[1] + p12 * d12[1] * d12[1]) / 3.0;
                    w[3] += (p01 * e01[0] * e01[2] + p02 * e02[0] * e02[2] + p12 * d12[0] * d12[2]) / 3.0;
                    w[4] += (p01 * e01[1] * e01[2] + p02 * e02[1] * e02[2] + p12 * d12[1] * d12[2]) / 3.0;
                    w[5] += (p01 * e01[2] * e01[2] + p02 * e02[2] * e02[2] + p12 * d12[2] * d12[2]) / 3.0;
                    nvert++;
                }
            }
            for (int d = 0; d < 3; d++) f[3 * si + d] += fi[d];
        }
        free(nb);
    }
    free(dc);
    if (out) {
        out->energy = energy;
        for (int d = 0; d < 6; d++) out->virial[d] = w[d];
        out->triplets = nvert / 3;
    }
}

/* ------------------------------------------------------------------------ */
/* FENE, Limit, bonded                                                      */
/* ------------------------------------------------------------------------ */
void kor_fene(int64_t n_pairs, const int64_t *pairs, const double *shifts, const double *r,
              const double *eps, const double *sig, const uint64_t *id, double stiffness, double *f) {
    for (int64_t p = 0; p < n_pairs; p++) {
        const int64_t s0 = pairs[2 * p], s1 = pairs[2 * p + 1];
        if (id[s0] != id[s1]) continue;
        if (shift_nonzero(shifts + 6 * p) || shift_nonzero(shifts + 6 * p + 3)) continue;
        double dr[3], inv[3];
        for (int d = 0; d < 3; d++) { dr[d] = r[3 * s1 + d] - r[3 * s0 + d]; inv[d] = 1.0 / dr[d]; }
        const double dr2 = dr[0] * dr[0] + dr[1] * dr[1] + dr[2] * dr[2];
        const double sigma = (sig[s0] + sig[s1]) / 2.0;
        const double R02 = pow(1.5 * sigma, 2);
        if (R02 <= dr2) {
            for (int d = 0; d < 3; d++) { f[3 * s0 + d] += inv[d] * 1e+30; f[3 * s1 + d] -= inv[d] * 1e+30; }
            continue;
        }
        const double epsilon = sqrt(eps[s0] * eps[s1]);
        const double k = stiffness * epsilon / pow(sigma, 2);
        const double fac = k / (1 - (dr2 / R02));
        for (int d = 0; d < 3; d++) { f[3 * s0 + d] += dr[d] * fac; f[3 * s1 + d] -= dr[d] * fac; }
    }
}

void kor_limit(int64_t n, const double *eps, const double *sig, double limit_factor, double *f) {
    for (int64_t s = 0; s < n; s++) {
        const double fmax = limit_factor * eps[s] / sig[s];
        for (int d = 0; d < 3; d++) {
            double x = f[3 * s + d];
            x = (fmax < x) ? fmax : x;     /* Kokkos::min(force, fmax): keeps NaN */
            x = (x < -fmax) ? -fmax : x;   /* Kokkos::max(.., -fmax)              */
            f[3 * s + d] = x;
        }
    }
}

double kor_bonded(int64_t n_bonds, const int64_t *bonds, double kb, double r0,
                  int64_t n_angles, const int64_t *angles, double ka, double theta0,
                  const double *r, const double *L, double *f, double *virial) {
    (void)L;
    double energy = 0;
    for (int64_t b = 0; b < n_bonds; b++) {
        const int64_t i = bonds[2 * b], j = bonds[2 * b + 1];
        double d[3];
        for (int k = 0; k < 3; k++) d[k] = r[3 * i + k] - r[3 * j + k];
        const double rr = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
        const double dl = rr - r0;
        energy += 0.5 * kb * dl * dl;
        const double fs = -kb * dl / rr;            /* force on i = fs * d */
        for (int k = 0; k < 3; k++) { f[3 * i + k] += fs * d[k]; f[3 * j + k] -= fs * d[k]; }
        if (virial) {
            virial[0] += fs * d[0] * d[0]; virial[1] += fs * d[0] * d[1]; virial[2] += fs * d[1] * d[1];
            virial[3] += fs * d[0] * d[2]; virial[4] += fs * d[1] * d[2]; virial[5] += fs * d[2] * d[2];
        }
    }
    for (int64_t a = 0; a < n_angles; a++) {
        const int64_t i = angles[3 * a], j = angles[3 * a + 1], k = angles[3 * a + 2];  /* j = vertex */
        double u[3], v[3];
        for (int t = 0; t < 3; t++) { u[t] = r[3 * i + t] - r[3 * j + t]; v[t] = r[3 * k + t] - r[3 * j + t]; }
        const double uu = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
        const double vv = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
        const double uv = u[0] * v[0] + u[1] * v[1] + u[2] * v[2];
        const double nu_ = sqrt(uu), nv = sqrt(vv);
        double cs = uv / (nu_ * nv);
        if (cs > 1.0) cs = 1.0;
        if (cs < -1.0) cs = -1.0;
        const double th = acos(cs);
        const double dth = th - theta0;
        energy += 0.5 * ka * dth * dth;
        double sn = sqrt(1.0 - cs * cs);
        if (sn < 1e-12) sn = 1e-12;
        /* F_i = -dU/dth * dth/dr_i,  dth/dr_i = -1/sin * dcos/dr_i */
        const double pre = ka * dth / sn;
        double fi[3], fk[3];
        for (int t = 0; t < 3; t++) {
            fi[t] = pre * (v[t] / (nu_ * nv) - cs * u[t] / uu);
            fk[t] = pre * (u[t] / (nu_ * nv) - cs * v[t] / vv);
            f[3 * i + t] += fi[t];
            f[3 * k + t] += fk[t];
            f[3 * j + t] -= fi[t] + fk[t];
        }
        if (virial) {
            virial[0] += u[0] * fi[0] + v[0] * fk[0]; virial[1] += u[0] * fi[1] + v[0] * fk[1];
            virial[2] += u[1] * fi[1] + v[1] * fk[1]; virial[3] += u[0] * fi[2] + v[0] * fk[2];
            virial[4] += u[1] * fi[2] + v[1] * fk[2]; virial[5] += u[2] * fi[2] + v[2] * fk[2];
        }
    }
    return energy;
}

/* ------------------------------------------------------------------------ */
/* integrator, sensors                                                      */
/* ------------------------------------------------------------------------ */
void kor_step0(int64_t n, double *r, double *v, const double *f, const double *m, double dt) {
    const double dt_halve = dt * 0.5;
    for (int64_t s = 0; s < n; s++) {
        const double c = dt_halve / m[s];
        for (int d = 0; d < 3; d++) v[3 * s + d] = v[3 * s + d] + f[3 * s + d] * c;
        for (int d = 0; d < 3; d++) r[3 * s + d] = r[3 * s + d] + v[3 * s + d] * dt;
    }
}

void kor_step1(int64_t n, double *v, const double *f, const double *m, double dt) {
    const double dt_halve = dt * 0.5;
    for (int64_t s = 0; s < n; s++) {
        const double c = dt_halve / m[s];
        for (int d = 0; d < 3; d++) v[3 * s + d] = v[3 * s + d] + f[3 * s + d] * c;
    }
}

/* SciValue (math/SciValue.{h,cpp}): mantissa/exponent pair normalised to
 * 0.1 < |m| < 10 by repeated /10 and *10, converted as m * pow(10, e). */
typedef struct { double m; int64_t e; } sci_t;
static sci_t sci_norm(double m, int64_t e) {
    double a = fabs(m);
    while (a >= 10.0) { m /= 10.0; e += 1; a = fabs(m); }
    while (a <= 0.1) { m *= 10.0; e -= 1; a = fabs(m); }
    sci_t s = {m, e};
    return s;
}
static sci_t sci_from(double v) { if (v == 0.0) { sci_t s = {0.0, 0}; return s; } return sci_norm(v, 0); }
static sci_t sci_mul(sci_t a, sci_t b) { return sci_norm(a.m * b.m, a.e + b.e); }
static sci_t sci_div(sci_t a, sci_t b) { return sci_norm(a.m / b.m, a.e - b.e); }
static double sci_val(sci_t a) { return a.m * pow(10, (double)a.e); }

double kor_temperature(int64_t n, const double *r, const double *v, const double *m,
                       const double low[3], const double high[3]) {
    double num = 0, mv2 = 0;
    for (int64_t s = 0; s < n; s++) {
        const double *p = r + 3 * s;
        if (!(p[0] >= low[0] && p[1] >= low[1] && p[2] >= low[2] && p[0] <= high[0] && p[1] <= high[1] && p[2] <= high[2]))
            continue;
        const double *u = v + 3 * s;
        mv2 += m[s] * (u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
        num += 1;
    }
    const sci_t kB = sci_norm(1.380649, -23), da = sci_norm(1.66053906892, -27), aps = sci_norm(1.0, 2);
    const sci_t conv = sci_div(da, kB);
    const sci_t factor = sci_mul(sci_mul(aps, aps), conv);
    num *= 3;
    return sci_val(sci_mul(factor, sci_from(mv2 / num)));
}

double kor_pressure_factor(void) {
    const sci_t da = sci_norm(1.66053906892, -27), a_m = sci_norm(1.0, -10), ps_s = sci_norm(1.0, -12);
    return sci_val(sci_div(da, sci_mul(sci_mul(ps_s, ps_s), a_m)));
}

void kor_momentum(int64_t n_terms, const double *v, const double *m, double *acc) {
    for (int64_t s = 0; s < n_terms; s++) {
        const double *u = v + 3 * s;
        acc[0] += u[0] * u[0] * m[s];
        acc[1] += u[0] * u[1] * m[s];
        acc[2] += u[1] * u[1] * m[s];
        acc[3] += u[0] * u[2] * m[s];
        acc[4] += u[1] * u[2] * m[s];
        acc[5] += u[2] * u[2] * m[s];
    }
}

int64_t kor_rdf_nbins(double max_r, double delta_r) { return (int64_t)(uint64_t)(max_r / delta_r); }

void kor_rdf(int64_t n, const double *com, const double L[3], double max_r, double delta_r, int64_t nbins, double *bins) {
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 64)
#endif
    for (int64_t a = 0; a < n; a++) {
        for (int64_t b = 0; b < n; b++) {
            if (a == b) continue;
            double dr[3];
            for (int d = 0; d < 3; d++) {
                const double delta = com[3 * a + d] - com[3 * b + d];
                dr[d] = delta - L[d] * (double)(int64_t)round(delta / L[d]);
            }
            const double rr = sqrt(pow(dr[0], 2) + pow(dr[1], 2) + pow(dr[2], 2));
            if (rr > max_r) continue;
            uint64_t bin;
            if (rr < 0) bin = (uint64_t)nbins - 1;
            else {
                bin = (uint64_t)(rr / delta_r);
                if (bin > (uint64_t)nbins - 1) bin = (uint64_t)nbins - 1;
            }
            atomic_addd(&bins[bin], 1.0);
        }
    }
}

/* ------------------------------------------------------------------------ */
/* three-body surrogate (no reference counterpart)                          */
/* ------------------------------------------------------------------------ */
static const double SUR_PI = 3.14159265358979323846;
static const double SUR_ETA_R = 50.0;
static const double SUR_ETA_A = 22.222222222222222;   /* 1 / (2 * 0.15^2) */
static const double SUR_MU_C[KOR_SUR_NC] = {1.05, 1.30, 1.55, 1.80};
static double sur_mu_r(int k) { return 0.85 + k * (1.15 / 15.0); }

typedef struct { double G[KOR_SUR_NR]; double M1[KOR_SUR_NC][3]; double M2[KOR_SUR_NC][3][3]; } sur_acc;

static void sur_accumulate(int n_nb, const double *d, double rc, sur_acc *a) {
    memset(a, 0, sizeof(*a));
    for (int j = 0; j < n_nb; j++) {
        const double *dj = d + 3 * j;
        const double r = sqrt(dj[0] * dj[0] + dj[1] * dj[1] + dj[2] * dj[2]);
        if (!(r < rc) || r == 0.0) continue;
        const double fc = 0.5 * (cos(SUR_PI * r / rc) + 1.0);
        const double u[3] = {dj[0] / r, dj[1] / r, dj[2] / r};
        for (int k = 0; k < KOR_SUR_NR; k++) {
            const double t = r - sur_mu_r(k);
            a->G[k] += exp(-SUR_ETA_R * t * t) * fc;
        }
        for (int c = 0; c < KOR_SUR_NC; c++) {
            const double t = r - SUR_MU_C[c];
            const double g = exp(-SUR_ETA_A * t * t) * fc;
            for (int p = 0; p < 3; p++) {
                a->M1[c][p] += g * u[p];
                for (int q = 0; q < 3; q++) a->M2[c][p][q] += g * u[p] * u[q];
            }
        }
    }
}

static void mat3_mul(const double A[3][3], const double B[3][3], double C[3][3]) {
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double s = 0;
            for (int k = 0; k < 3; k++) s += A[i][k] * B[k][j];
            C[i][j] = s;
        }
}

static void sur_invariants(const sur_acc *a, double *raw) {
    for (int k = 0; k < KOR_SUR_NR; k++) raw[k] = a->G[k];
    for (int c = 0; c < KOR_SUR_NC; c++) {
        const double *m1 = a->M1[c];
        double M2m1[3], M22[3][3], M23[3][3];
        for (int p = 0; p < 3; p++) M2m1[p] = a->M2[c][p][0] * m1[0] + a->M2[c][p][1] * m1[1] + a->M2[c][p][2] * m1[2];
        mat3_mul(a->M2[c], a->M2[c], M22);
        mat3_mul(M22, a->M2[c], M23);
        double i2 = 0;
        for (int p = 0; p < 3; p++) for (int q = 0; q < 3; q++) i2 += a->M2[c][p][q] * a->M2[c][p][q];
        raw[KOR_SUR_NR + c] = m1[0] * m1[0] + m1[1] * m1[1] + m1[2] * m1[2];
        raw[KOR_SUR_NR + KOR_SUR_NC + c] = i2;
        raw[KOR_SUR_NR + 2 * KOR_SUR_NC + c] = m1[0] * M2m1[0] + m1[1] * M2m1[1] + m1[2] * M2m1[2];
        raw[KOR_SUR_NR + 3 * KOR_SUR_NC + c] = M23[0][0] + M23[1][1] + M23[2][2];
    }
}

void kor_sur_features(int n_nb, const double *d, double rc, double *raw) {
    sur_acc a;
    sur_accumulate(n_nb, d, rc, &a);
    sur_invariants(&a, raw);
}

double kor_sur_mlp(const double *P, const double *x, double *dE_dx) {
    const int H = KOR_SUR_H, F = KOR_SUR_NF;
    const double *W1 = P, *b1 = W1 + H * F, *W2 = b1 + H, *b2 = W2 + H * H, *w3 = b2 + H, *b3 = w3 + H;
    double h1[KOR_SUR_H], h2[KOR_SUR_H];
    for (int o = 0; o < H; o++) {
        double z = b1[o];
        for (int i = 0; i < F; i++) z += W1[o * F + i] * x[i];
        h1[o] = tanh(z);
    }
    for (int o = 0; o < H; o++) {
        double z = b2[o];
        for (int i = 0; i < H; i++) z += W2[o * H + i] * h1[i];
        h2[o] = tanh(z);
    }
    double E = b3[0];
    for (int i = 0; i < H; i++) E += w3[i] * h2[i];
    if (dE_dx) {
        double dz2[KOR_SUR_H], dz1[KOR_SUR_H];
        for (int o = 0; o < H; o++) dz2[o] = w3[o] * (1.0 - h2[o] * h2[o]);
        for (int i = 0; i < H; i++) {
            double s = 0;
            for (int o = 0; o < H; o++) s += W2[o * H + i] * dz2[o];
            dz1[i] = s * (1.0 - h1[i] * h1[i]);
        }
        for (int i = 0; i < F; i++) {
            double s = 0;
            for (int o = 0; o < H; o++) s += W1[o * F + i] * dz1[o];
            dE_dx[i] = s;
        }
    }
    return E;
}

void kor_sur_mlp_param_grad(const double *P, const double *x, double *G) {
    const int H = KOR_SUR_H, F = KOR_SUR_NF;
    const double *W1 = P, *b1 = W1 + H * F, *W2 = b1 + H, *b2 = W2 + H * H, *w3 = b2 + H;
    double *gW1 = G, *gb1 = gW1 + H * F, *gW2 = gb1 + H, *gb2 = gW2 + H * H, *gw3 = gb2 + H, *gb3 = gw3 + H;
    double h1[KOR_SUR_H], h2[KOR_SUR_H], dz1[KOR_SUR_H], dz2[KOR_SUR_H];
    for (int o = 0; o < H; o++) {
        double z = b1[o];
        for (int i = 0; i < F; i++) z += W1[o * F + i] * x[i];
        h1[o] = tanh(z);
    }
    for (int o = 0; o < H; o++) {
        double z = b2[o];
        for (int i = 0; i < H; i++) z += W2[o * H + i] * h1[i];
        h2[o] = tanh(z);
    }
    for (int o = 0; o < H; o++) dz2[o] = w3[o] * (1.0 - h2[o] * h2[o]);
    for (int i = 0; i < H; i++) {
        double s = 0;
        for (int o = 0; o < H; o++) s += W2[o * H + i] * dz2[o];
        dz1[i] = s * (1.0 - h1[i] * h1[i]);
    }
    for (int o = 0; o < H; o++) {
        for (int i = 0; i < F; i++) gW1[o * F + i] = dz1[o] * x[i];
        gb1[o] = dz1[o];
        for (int i = 0; i < H; i++) gW2[o * H + i] = dz2[o] * h1[i];
        gb2[o] = dz2[o];
        gw3[o] = h2[o];
    }
    gb3[0] = 1.0;
}

double kor_sur_energy_forces(int64_t n, const double *r, const double L[3], double rc, const double *params,
                             const double *fmean, const double *fstd, double e_scale, double e_shift,
                             double *e_site, double *f) {
    double etot = 0;
    int cap = 256;
    double *d = (double *)malloc(sizeof(double) * 3 * (size_t)cap);
    int64_t *jj = (int64_t *)malloc(sizeof(int64_t) * (size_t)cap);
    memset(f, 0, sizeof(double) * 3 * (size_t)n);
    for (int64_t i = 0; i < n; i++) {
        int nn = 0;
        for (int64_t j = 0; j < n; j++) {
            if (j == i) continue;
            double v[3];
            for (int k = 0; k < 3; k++) {
                v[k] = r[3 * j + k] - r[3 * i + k];
                v[k] -= L[k] * round(v[k] / L[k]);
            }
            const double q = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
            if (!(q < rc * rc)) continue;
            if (nn == cap) {
                cap *= 2;
                d = (double *)realloc(d, sizeof(double) * 3 * (size_t)cap);
                jj = (int64_t *)realloc(jj, sizeof(int64_t) * (size_t)cap);
            }
            memcpy(d + 3 * nn, v, sizeof(v));
            jj[nn++] = j;
        }
        sur_acc a;
        sur_accumulate(nn, d, rc, &a);
        double raw[KOR_SUR_NF], x[KOR_SUR_NF], dx[KOR_SUR_NF];
        sur_invariants(&a, raw);
        for (int k = 0; k < KOR_SUR_NF; k++) x[k] = (raw[k] - fmean[k]) / fstd[k];
        const double e = e_scale * kor_sur_mlp(params, x, dx) + e_shift;
        if (e_site) e_site[i] = e;
        etot += e;
        double dr[KOR_SUR_NF];   /* dE_i / d raw */
        for (int k = 0; k < KOR_SUR_NF; k++) dr[k] = e_scale * dx[k] / fstd[k];
        /* coefficients of the angular chain: a_c = dE/dM1_c, B_c = dE/dM2_c */
        double ac[KOR_SUR_NC][3], Bc[KOR_SUR_NC][3][3];
        for (int c = 0; c < KOR_SUR_NC; c++) {
            const double e1 = dr[KOR_SUR_NR + c], e2 = dr[KOR_SUR_NR + KOR_SUR_NC + c];
            const double e3 = dr[KOR_SUR_NR + 2 * KOR_SUR_NC + c], e4 = dr[KOR_SUR_NR + 3 * KOR_SUR_NC + c];
            double M22[3][3];
            mat3_mul(a.M2[c], a.M2[c], M22);
            for (int p = 0; p < 3; p++) {
                double m2m1 = 0;
                for (int q = 0; q < 3; q++) m2m1 += a.M2[c][p][q] * a.M1[c][q];
                ac[c][p] = 2.0 * e1 * a.M1[c][p] + 2.0 * e3 * m2m1;
                for (int q = 0; q < 3; q++)
                    Bc[c][p][q] = 2.0 * e2 * a.M2[c][p][q] + e3 * a.M1[c][p] * a.M1[c][q] + 3.0 * e4 * M22[p][q];
            }
        }
        for (int t = 0; t < nn; t++) {
            const double *dj = d + 3 * t;
            const double rr = sqrt(dj[0] * dj[0] + dj[1] * dj[1] + dj[2] * dj[2]);
            if (!(rr < rc) || rr == 0.0) continue;
            const double u[3] = {dj[0] / rr, dj[1] / rr, dj[2] / rr};
            const double fc = 0.5 * (cos(SUR_PI * rr / rc) + 1.0);
            const double dfc = -0.5 * (SUR_PI / rc) * sin(SUR_PI * rr / rc);
            double hvec[3] = {0, 0, 0};   /* dE_i / d d_ij */
            double sr = 0;
            for (int k = 0; k < KOR_SUR_NR; k++) {
                const double tt = rr - sur_mu_r(k);
                const double ex = exp(-SUR_ETA_R * tt * tt);
                sr += dr[k] * ex * (-2.0 * SUR_ETA_R * tt * fc + dfc);
            }
            for (int p = 0; p < 3; p++) hvec[p] += sr * u[p];
            for (int c = 0; c < KOR_SUR_NC; c++) {
                const double tt = rr - SUR_MU_C[c];
                const double ex = exp(-SUR_ETA_A * tt * tt);
                const double g = ex * fc, gp = ex * (-2.0 * SUR_ETA_A * tt * fc + dfc);
                const double ua = u[0] * ac[c][0] + u[1] * ac[c][1] + u[2] * ac[c][2];
                double Bu[3];
                for (int p = 0; p < 3; p++) Bu[p] = Bc[c][p][0] * u[0] + Bc[c][p][1] * u[1] + Bc[c][p][2] * u[2];
                const double uBu = u[0] * Bu[0] + u[1] * Bu[1] + u[2] * Bu[2];
                for (int p = 0; p < 3; p++)
                    hvec[p] += gp * ua * u[p] + (g / rr) * (ac[c][p] - ua * u[p]) + gp * uBu * u[p] +
                               (2.0 * g / rr) * (Bu[p] - uBu * u[p]);
            }
            const int64_t j = jj[t];
            for (int p = 0; p < 3; p++) {
                f[3 * j + p] -= hvec[p];
                f[3 * i + p] += hvec[p];
            }
        }
    }
    free(d);
    free(jj);
    return etot;
}
