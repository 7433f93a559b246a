// engine.cuh -- device-side state and helpers of the GB300 KoMD force engine.
//
// Layout in HBM (n sites, M molecules, C = nd_x*nd_y*nd_z domain cells):
//   site order (the caller's order, molecules contiguous), FP64:
//     r, v, f          3 doubles per site (x y z), like the reference's SOA
//     m, eps, sig      1 double per site
//   per site: key (dense 32-bit molecule key: equal keys <=> equal mol IDs),
//             mol (molecule index), slot (position in cell order)
//   per molecule: off (CSR into sites), com (3 doubles), cell, rank
//   per cell:     count / start (sites, exclusive prefix), mcount / mstart
//                 (molecules), mols (molecule indices grouped by cell)
//   cell order (rebuilt every step by a counting sort, ascending site index
//   inside a cell, which is the reference's cell-list order):
//     slot_site    site index per slot
//     pos4         float4 (x, y, z relative to the cell centre, sigma/2)
//     posd         3 doubles: absolute position (FP64 kernels, exact counts)
//     skey         molecule key per slot, seps: sqrt(eps) per slot
//   ATM neighbour list: cap float4 per slot (vector r_i - r_j, packed code)
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "komd_gpu.h"

namespace komd {

// Programmatic dependent launch between consecutive kernels of a step: a
// kernel launched with launch_pdl may become resident before its
// predecessor has finished; pdl_wait (at its entry, before any memory
// access) holds it until the predecessor has completed and its writes are
// visible, and pdl_trigger lets the successor be scheduled once every block
// of this grid has started.  Both are no-ops without a programmatic launch.
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <typename... KArgs, typename... Args>
inline void launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kernel, args...);
}

constexpr int kWarpsPerBlock = 8;
constexpr int kBlock = 32 * kWarpsPerBlock;

// Grid geometry of LinkedCells (LinkedCells.cpp:11-45): nd domain cells per
// dimension of edge cs, the last one stretched to the domain's high bound.
struct Grid {
    double low[3], high[3], L[3];
    double cs;
    int nd[3];
    int ncell;
};

// Reduction slots (FP64) written per block and summed on the host side of a measure.
enum RedSlot {
    R_ULJ = 0, R_UATM, R_UBOND, R_W0, R_W1, R_W2, R_W3, R_W4, R_W5, R_PAIRS, R_TRIPS,
    R_MV2, R_NBOX, R_K0, R_K1, R_K2, R_K3, R_K4, R_K5, R_NSLOTS
};

// device error flags
enum ErrFlag { E_ATM_OVERFLOW = 0, E_NONFINITE = 1, E_VL_OVERFLOW = 2, E_NFLAGS = 4 };

// ---------------------------------------------------------------------------
// exact FP64 helpers: the reference is built without FMA contraction, so the
// binning, integration and the FP64 distance test use explicit round-to-
// nearest intrinsics that the compiler never fuses.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }

// Reference point of a cell for the FP32 cell-local coordinates.  Any fixed
// choice works as long as the sort and the force kernels agree; the centre
// keeps |local| <= half a cell so FP32 keeps ~1e-7 absolute precision.
__host__ __device__ inline double cell_centre(const Grid &g, int d, int k) {
    if (k < g.nd[d] - 1) return g.low[d] + (k + 0.5) * g.cs;
    return 0.5 * ((g.low[d] + (g.nd[d] - 1) * g.cs) + g.high[d]);
}

__host__ __device__ inline void cell_coords(const Grid &g, int c, int &x, int &y, int &z) {
    x = c % g.nd[0];
    y = (c / g.nd[0]) % g.nd[1];
    z = c / (g.nd[0] * g.nd[1]);
}

// Neighbour nb in 0..26 of a domain cell (dx fastest), wrapped periodically.
// shift[d] = +L / -L / 0 exactly like the reference's halo layers
// (LinkedCells.cpp:494-502): a neighbour beyond the high face is an image
// shifted by +L.  Returns the linear index of the wrapped domain cell.
struct NbCell {
    int cell;
    double shift[3];
    bool crosses;
};

__host__ __device__ inline NbCell neighbour_cell(const Grid &g, int cx, int cy, int cz, int nb) {
    const int dd[3] = {nb % 3 - 1, (nb / 3) % 3 - 1, nb / 9 - 1};
    const int cc[3] = {cx, cy, cz};
    int w[3];
    NbCell out;
    out.crosses = false;
    for (int d = 0; d < 3; d++) {
        int k = cc[d] + dd[d];
        out.shift[d] = 0.0;
        if (k < 0) { k += g.nd[d]; out.shift[d] = -g.L[d]; out.crosses = true; }
        else if (k >= g.nd[d]) { k -= g.nd[d]; out.shift[d] = g.L[d]; out.crosses = true; }
        w[d] = k;
    }
    out.cell = w[0] + g.nd[0] * (w[1] + g.nd[1] * w[2]);
    return out;
}

// ATM neighbour entry code: bits 0-4 neighbour-cell index (13 = home cell),
// bit 5 set when the neighbour is a periodic image, bits 6-30 neighbour slot.
__host__ __device__ inline int atm_code(int nb, bool crosses, int slot) {
    return nb | (crosses ? 32 : 0) | (slot << 6);
}
constexpr int kMaxAtmSlot = (1 << 25) - 1;

// The order in which the Verlet rows put a site's neighbours "above" it (the
// front region that the half-list pass reads): j is above i when j's z at the
// last rebuild, quantized to kZq levels over the box and compared by minimum
// image, is larger, or equal with a larger slot.  Every neighbour pair thus
// has one owner, and so does every triplet (its lowest member): on integer
// keys the relation is exactly antisymmetric, and for mutual neighbours
// (offsets far below half the box) exactly transitive.  Against the slot
// order it halves each site's neighbourhood by a plane, which balances the
// owned triplets per site (the slot order gives the first sites of a cell
// the most).
constexpr int kZq = 1 << 24;
__host__ __device__ inline bool vl_above(int zi, int zj, unsigned si, unsigned sj) {
    int d = zj - zi;
    if (d > kZq / 2) d -= kZq;
    else if (d < -kZq / 2) d += kZq;
    return d > 0 || (d == 0 && sj > si);
}

struct PairParams {
    Grid g;
    const int *cell_start;     // C+1
    const int *slot_site;
    const float4 *pos4;
    const double *posd;        // 3 per slot (FP64 kernels)
    const int *skey;
    const float *seps;         // sqrt(eps) per slot
    const double *seps_d;      // FP64 sqrt(eps) per slot
    const double *sig_d;       // FP64 sigma per slot
    double *f;                 // 3 per site, overwritten (pair terms)
    int64_t *counts;           // per site (neighbour counts), optional
    float4 *nl;                // ATM list (cap per slot)
    int *nl_count;
    int nl_cap;
    int *err;
    double *partials;          // R_NSLOTS per block
    double *lj_hist;           // 4*bins (u sums, f sums, u counts, f counts), optional
    int lj_bins;
    double max_sigma;
    double rc2, rc3sq, scan2;  // LJ cutoff^2, ATM cutoff^2, max of both
    double stiffness;
    int use_lj;
    int virial_compat;
    const float *offtab;       // per dimension nd*3 FP32 offsets centre(k+d) + shift - centre(k)
    // Verlet path
    const int *rebuild;
    unsigned *vl;
    int *vl_count;
    int vl_cap;
    double rl2;                // (cutoff + skin)^2
    const int *slot_cell;
    const int *zkey;           // per slot: quantized z at the last rebuild (the half-list order)
    int *vb_next;              // Verlet list build: next home cell to take (reset by the scan)
    const float4 *nboff;
    int *rebuild_count;
    float eps0, sig0;
    float lj_fscalef;          // ATM2B force factor (1 without ATM2B), force path only
    double lj_fscale;
    int sw;                    // switched cutoff (komd_config::switch_width > 0)
    float sw_rc2, sw_iw;       // cutoff^2 and 1 / (cutoff^2 - (cutoff - width)^2)
    float4 *fown;              // per slot, optional: the half-list pass writes each site's own FP32 force here
                               // (the flush widens it) instead of FP64 into f
};

struct AtmParams {
    int n;
    const int *slot_site;
    const float4 *nl;
    const int *nl_count;
    int nl_cap;
    double *f;
    double *partials;
    double nu;
    double rc2;
    double sign;               // +1 reference (+grad V), -1 physical
    int virial_compat;         // weights and missing ZZ of ATM_Pressure
    int atm_direct;            // COMPAT + direct: no virial contribution
    double *e_site;            // measure: per-site V/3 sums (site order), optional
    unsigned long long *acc;   // k_atm_s: 3 fixed-point force sums per slot (2^-32 units)
    int sw;                    // switched cutoff (komd_config::switch_width > 0)
    float sw_rc2, sw_iw;       // cutoff_3b^2 and 1 / (cutoff_3b^2 - (cutoff_3b - width)^2)
};

// The switched-cutoff option (komd_config::switch_width): the C1 smoothstep
// S = t^2 (3 - 2t) of the squared distance x, t = (rc^2 - x) * iw clamped to
// [0, 1] (iw = 1 / (rc^2 - rs^2)), and dS/dx = -6 t (1 - t) iw.
__host__ __device__ inline void sw_eval(float x, float rc2, float iw, float &S, float &dS) {
    float t = (rc2 - x) * iw;
    t = t < 0.f ? 0.f : (t > 1.f ? 1.f : t);
    S = t * t * (3.0f - 2.0f * t);
    dS = -6.0f * t * (1.0f - t) * iw;
}
inline void sw_params(double rc, double width, int &on, float &rc2, float &iw) {
    on = width > 0 ? 1 : 0;
    const double rs = rc - width;
    rc2 = (float)(rc * rc);
    iw = on ? (float)(1.0 / (rc * rc - rs * rs)) : 0.f;
}

// Arguments of the step kernels of the Verlet path, one struct per kernel, so
// that one launch can serve one system (the struct by value) or all replicas
// of a batch (an array of them, a block range per replica).
struct BinArgs {              // k_com_wrap_bin: COM, periodic wrap, binning
    Grid g;
    int n_mol;
    const int *mol_off;
    double *r;
    const double *m;
    double *com;
    int *mol_cell, *mol_rank, *cell_count, *cell_mcount;
    double *bias;
    const int *rebuild;
    const unsigned char *exact_com;
    int wrapped;
};
struct ScanArgs {             // k_scan2: exclusive scans of the cell counts
    int nc;
    int *a, *sa, *b, *sb;
    const int *rebuild;
    int *work;
};
struct ScatterArgs {          // k_scatter_mol: molecules into their cells
    int n_mol;
    const int *mol_cell, *mol_rank, *cell_mstart;
    int *cell_mols;
    const int *rebuild;
};
struct SortArgs {             // k_cell_sort: slots and the cell-ordered arrays
    Grid g;
    const int *mol_off, *cell_mstart, *cell_start, *cell_mols;
    const double *r, *eps, *sig;
    const int *key;
    int *slot_site, *site_slot;
    float4 *pos4;
    int *skey;
    float *seps;
    double *posd, *seps_d, *sig_d, *bias;
    float4 *ref4;
    int *slot_cell, *zkey;
    const int *rebuild;
};
struct Step0Args {            // k_step0_fused: half-kick, drift, wrap, skin test
    int n;
    double *r, *v;
    const double *f, *hdtm;
    double dt;
    Grid g;
    double *bias;
    const float4 *ref4;
    float half_skin2;
    int *rebuild;
    double *com;
    const int *site_slot;
    float4 *pos4;
    const double *r_in, *v_in;
    double *r_out;
};
struct FlushArgs {            // k_atm_flush_step1: fixed-point sums into f, half-kick
    int n;
    const int *site_slot;
    unsigned long long *acc;
    double *f;
    double scale_fix;
    double *v;
    const double *hdtm;
    int *err, *rebuild;
    double *f_out, *v_out;
    const float4 *fown;   // optional: the half-list pass's FP32 forces per slot, in place of f's
};

// TemperatureSensor's conversion (TemperatureSensor.cpp:44-47) in SciValue
// arithmetic (math/SciValue.{h,cpp}): mantissas normalised into (0.1, 10) by
// repeated /10 and *10, converted as m * 10^e.  10^e is exact for 0 <= e <= 22
// and 1 / 10^-e (one correctly rounded division) below; host and device
// evaluate the same IEEE operations, so both give the same temperature.
// The device thermostat runs this inside the step graph, so both loops are
// bounded: zero, NaN and +-inf come back unchanged at once (inf / 10 stays
// inf, and the reference's unbounded loop would never end on it), and no
// finite double needs more than 400 steps (about 10^308 to 10^-324).
constexpr int kSciMaxSteps = 400;
struct SciNum { double m; int e; };
__host__ __device__ inline SciNum sci_norm(double m, int e) {
    double a = fabs(m);
    if (!(a <= 1.7976931348623157e308) || a == 0.0) return {m, e};   // NaN, +-inf or zero
    for (int k = 0; k < kSciMaxSteps && a >= 10.0; k++) { m = m / 10.0; e += 1; a = fabs(m); }
    for (int k = 0; k < kSciMaxSteps && a <= 0.1; k++) { m = m * 10.0; e -= 1; a = fabs(m); }
    return {m, e};
}
__host__ __device__ inline double sci_pow10(int e) {
    double p = 1.0;
    const int k = e < 0 ? -e : e;
    for (int i = 0; i < k && i < 22; i++) p = p * 10.0;
    // beyond 1e22 no longer exact (not reached by finite temperatures); past
    // 1e309 the product is inf already, so the loop stops there
    for (int i = 22; i < k && i < 330; i++) p = p * 10.0;
    return e < 0 ? 1.0 / p : p;
}
__host__ __device__ inline double sci_temperature(double mv2, double n_in_box) {
    if (!(n_in_box > 0.0)) return 0.0;
    const SciNum kB = sci_norm(1.380649, -23), da = sci_norm(1.66053906892, -27), aps = sci_norm(1.0, 2);
    SciNum f = sci_norm(aps.m * aps.m, aps.e + aps.e);
    const SciNum q = sci_norm(da.m / kB.m, da.e - kB.e);
    f = sci_norm(f.m * q.m, f.e + q.e);
    const double x = mv2 / (n_in_box * 3);
    const SciNum v = x == 0.0 ? SciNum{0.0, 0} : sci_norm(x, 0);
    const SciNum t = sci_norm(f.m * v.m, f.e + v.e);
    return t.m * sci_pow10(t.e);
}

struct Engine {
    komd_config cfg;
    Grid g;
    int device = 0;
    int num_sms = 152;        // multiprocessors of the device, queried at creation (sizes resident grids)
    cudaStream_t stream = nullptr;
    bool own_stream = false;

    int64_t n = 0, n_mol = 0;
    // site arrays
    double *r = nullptr, *v = nullptr, *f = nullptr, *m = nullptr, *eps = nullptr, *sig = nullptr;
    int *key = nullptr, *site_mol = nullptr, *site_slot = nullptr;
    // molecules
    int *mol_off = nullptr, *mol_cell = nullptr, *mol_rank = nullptr;
    double *com = nullptr;
    // cells
    int *cell_count = nullptr, *cell_start = nullptr, *cell_mcount = nullptr, *cell_mstart = nullptr;
    int *cell_mols = nullptr;
    // cell order
    int *slot_site = nullptr, *skey = nullptr;
    float4 *pos4 = nullptr;
    float *seps = nullptr;
    double *posd = nullptr, *seps_d = nullptr, *sig_d = nullptr;
    float *offtab = nullptr;   // see PairParams::offtab
    // ATM list
    float4 *nl = nullptr;
    int *nl_count = nullptr;
    int nl_cap = 64;
    // topology
    int *bonds = nullptr, *angles = nullptr;
    int64_t n_bonds = 0, n_angles = 0;
    // reductions / flags
    double *partials = nullptr;
    int partial_blocks = 0;
    int *err = nullptr;
    double *rdf = nullptr;
    int64_t rdf_bins = 0;
    double *lj_hist = nullptr;
    int64_t *counts = nullptr;
    // state
    bool have_sites = false, have_cells = false, have_forces = false;
    // graph
    cudaGraphExec_t graph = nullptr;
    bool graph_valid = false;
    // profiling
    bool profiling = false;
    // Verlet list of the physics path (FP32, no FENE, FULL ATM, CORRECT virial, skin > 0)
    bool verlet = false;
    int *rebuild = nullptr;      // device flag: rebuild cells and list in this step
    // per site: bias such that (float)(r - bias) is the FP32 position relative to
    // the centre of the slot's build cell (the build cell centre plus the periodic
    // shifts applied since the build; 3 doubles)
    double *bias = nullptr;
    float4 *ref4 = nullptr;      // per site: that FP32 position at the last rebuild
    int *slot_cell = nullptr;    // per slot: its cell at the last rebuild
    int *zkey = nullptr;         // per slot: quantized z at the last rebuild (the half-list order)
    int *vb_next = nullptr;      // Verlet list build: work counter over home cells
    float4 *nboff = nullptr;     // per cell x 27: home-relative neighbour-cell offset, w = 1 for an image
    unsigned *vl = nullptr;      // vl_cap entries per slot: same-molecule bit 31 | nb << 26 | slot
    int *vl_count = nullptr;
    int vl_cap = 0;
    int *rebuild_count = nullptr;    // list builds since the last profile reset
    // per-site (dt/2)/m and per-molecule exact-COM flags (single site, power-of-two mass)
    double *hdtm = nullptr;
    unsigned char *exact_com = nullptr;
    // all sites share eps and sigma: the list kernel uses constants
    bool uniform = false;
    float eps0 = 1.f, sig0 = 1.f;
    double lj_fscale = 1.0;         // ATM2B factor (KOMD_TERM_ATM2B), else 1
    bool fused_drift = false;       // Verlet path, single-site molecules with exact COM: k_step0_fused
    // device-accessible host buffers of komd_gpu_step_host (site order, 3 doubles
    // per site), read or written directly by the step's first and last kernels;
    // nullptr outside such a step
    const double *hin_r = nullptr, *hin_v = nullptr;
    double *hout_r = nullptr, *hout_v = nullptr, *hout_f = nullptr;
    // hout_r is pinned: the step copies the drifted positions back on the copy
    // engine (side stream) while its force pass runs, instead of in the drift kernel
    bool hout_r_async = false;
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    unsigned long long *atm_acc = nullptr;   // 3 per slot, fixed-point force sums of k_atm_s (zero between steps)
    float4 *fown = nullptr;   // 1 per slot (with atm_acc): the half-list pass's own FP32 force of each site
    // tabulated pair force (KOMD_TERM_TABULATED): F(r) piecewise linear on
    // ascending nodes tab_x, values tab_y, tab_lo below / tab_hi above the nodes
    double *tab_x = nullptr, *tab_y = nullptr, *tab_s = nullptr;   // nodes, values, segment slopes
    int tab_n = 0;
    double tab_lo = 0.0, tab_hi = 0.0;
    double *atm_esite = nullptr;     // when set, measure-mode ATM writes per-site energies here
};

constexpr int kMaxVerletSlot = (1 << 26) - 1;

}  // namespace komd
