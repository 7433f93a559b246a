// kernels.cu -- hand-written sm_103a kernels of the KoMD hot path.
//
// Per step (komd_gpu_step): integrate0 -> com/wrap/bin -> scan -> scatter ->
// cell sort+gather -> pair (LJ, FENE, ATM neighbour list) -> [bonded] ->
// [limit] -> [ATM triplets] -> integrate1.  On the Verlet path with FP32
// forces the drift is one kernel (k_step0_fused), the container kernels run
// only on a rebuild, the LJ pass sweeps the triplets itself (k_lj_atm,
// pair_tile.cu) and integrate1 rides on the ATM flush.
//
// Citations are to Snapex2409/KoMD, src/.
#include <algorithm>
#include <cfloat>
#include <climits>
#include <cstdint>

#include "engine.cuh"
#include "kernels.cuh"
#include "atm_device.cuh"

namespace komd {

// ===========================================================================
// container: COM, periodic wrap, binning (LinkedCells.cpp:65-121,390-400;
// MoleculeContainer.cpp:55-75).  One thread per molecule.
// ===========================================================================
__device__ __forceinline__ void com_wrap_bin_body(const BinArgs &a, int bid, int nblk) {
    const Grid &g = a.g;
    const int n_mol = a.n_mol;
    const int *__restrict__ mol_off = a.mol_off;
    double *__restrict__ r = a.r;
    const double *__restrict__ m = a.m;
    double *__restrict__ com = a.com;
    int *__restrict__ mol_cell = a.mol_cell, *__restrict__ mol_rank = a.mol_rank;
    int *__restrict__ cell_count = a.cell_count, *__restrict__ cell_mcount = a.cell_mcount;
    double *__restrict__ bias = a.bias;
    const int *__restrict__ rebuild = a.rebuild;
    const unsigned char *__restrict__ exact_com = a.exact_com;
    if (a.wrapped && rebuild && !*rebuild) return;   // k_step0_fused wrapped this step; no rebuild
    const bool bin = !(rebuild && !*rebuild);        // no rebuild in this step: cells stay as built
    for (int k = bid * blockDim.x + threadIdx.x; k < n_mol; k += nblk * blockDim.x) {
    const int s0 = mol_off[k], s1 = mol_off[k + 1];
    // com += r * m ; M += m ; com /= M   (updateCOM, no FMA).  For a single
    // site of power-of-two mass the scaling is exact and the result is r
    // itself (up to the sign of a zero), so the FP64 division is skipped.
    double c[3] = {0.0, 0.0, 0.0}, tm = 0.0;
    if (s1 - s0 == 1 && exact_com && exact_com[k]) {
        tm = m[s0];
        for (int d = 0; d < 3; d++) c[d] = r[3 * s0 + d];
    } else {
        for (int s = s0; s < s1; s++) {
            const double ms = m[s];
            for (int d = 0; d < 3; d++) c[d] = dadd(c[d], dmul(r[3 * s + d], ms));
            tm = dadd(tm, ms);
        }
        for (int d = 0; d < 3; d++) c[d] = ddiv(c[d], tm);
    }
    // Periodic_Kernel: strict comparisons against the domain bounds
    double off[3];
    bool moved = false;
    for (int d = 0; d < 3; d++) {
        off[d] = 0.0;
        if (c[d] < g.low[d]) off[d] = g.L[d];
        if (c[d] > g.high[d]) off[d] = -g.L[d];
        moved |= (off[d] != 0.0);
    }
    if (moved) {
        double c2[3] = {0.0, 0.0, 0.0};
        for (int s = s0; s < s1; s++) {
            const double ms = m[s];
            for (int d = 0; d < 3; d++) {
                const double x = dadd(r[3 * s + d], off[d]);
                r[3 * s + d] = x;
                c2[d] = dadd(c2[d], dmul(x, ms));
            }
            if (bias)   // the cell-local position r - bias is unchanged by the wrap
                for (int d = 0; d < 3; d++)
                    if (off[d] != 0.0) bias[3 * s + d] = dadd(bias[3 * s + d], off[d]);
        }
        if (s1 - s0 == 1 && exact_com && exact_com[k]) {
            for (int d = 0; d < 3; d++) c[d] = r[3 * s0 + d];
        } else {
            for (int d = 0; d < 3; d++) c[d] = ddiv(c2[d], tm);
        }
    }
    for (int d = 0; d < 3; d++) com[3 * k + d] = c[d];
    if (!bin) continue;
    // writeIndices: (int64)((com - low) / cs) clamped to [0, nd-1]
    int b[3];
    for (int d = 0; d < 3; d++) {
        const double fbin = ddiv(dsub(c[d], g.low[d]), g.cs);
        long long q = __double2ll_rz(fbin);
        if (q < 0) q = 0;
        if (q > g.nd[d] - 1) q = g.nd[d] - 1;
        b[d] = (int)q;
    }
    const int cell = b[0] + g.nd[0] * (b[1] + g.nd[1] * b[2]);
    mol_cell[k] = cell;
    mol_rank[k] = atomicAdd(&cell_mcount[cell], 1);
    atomicAdd(&cell_count[cell], s1 - s0);
    }
}
__global__ void k_com_wrap_bin(BinArgs a) {
    pdl_trigger();
    pdl_wait();
    com_wrap_bin_body(a, blockIdx.x, gridDim.x);
}

// exclusive scan of two count arrays of length nc (one block of 1024 threads,
// each owning a contiguous chunk); the counts are zeroed once read, ready for
// the next binning (work: the Verlet list build's cell counter, reset here for
// this rebuild)
__device__ __forceinline__ void scan2_body(const ScanArgs &q) {
    __shared__ int wa[32], wb[32];
    const int nc = q.nc;
    int *__restrict__ a = q.a, *__restrict__ sa = q.sa, *__restrict__ b = q.b, *__restrict__ sb = q.sb;
    int *__restrict__ work = q.work;
    if (q.rebuild && !*q.rebuild) return;
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    if (work && t == 0) *work = 0;
    const int per = (nc + 1023) / 1024;
    const int lo = min(t * per, nc), hi = min(lo + per, nc);
    int ta = 0, tb = 0;
    for (int i = lo; i < hi; i++) { ta += a[i]; tb += b[i]; }
    // inclusive warp scan
    int xa = ta, xb = tb;
    for (int o = 1; o < 32; o <<= 1) {
        const int ya = __shfl_up_sync(0xffffffffu, xa, o), yb = __shfl_up_sync(0xffffffffu, xb, o);
        if (lane >= o) { xa += ya; xb += yb; }
    }
    if (lane == 31) { wa[w] = xa; wb[w] = xb; }
    __syncthreads();
    if (w == 0) {
        int va = wa[lane], vb = wb[lane];
        for (int o = 1; o < 32; o <<= 1) {
            const int ya = __shfl_up_sync(0xffffffffu, va, o), yb = __shfl_up_sync(0xffffffffu, vb, o);
            if (lane >= o) { va += ya; vb += yb; }
        }
        wa[lane] = va;
        wb[lane] = vb;
    }
    __syncthreads();
    int pa = xa - ta + (w > 0 ? wa[w - 1] : 0), pb = xb - tb + (w > 0 ? wb[w - 1] : 0);
    for (int i = lo; i < hi; i++) {
        sa[i] = pa; pa += a[i];
        sb[i] = pb; pb += b[i];
        a[i] = 0;
        b[i] = 0;
    }
    if (t == 1023) { sa[nc] = wa[31]; sb[nc] = wb[31]; }
}
__global__ void __launch_bounds__(1024) k_scan2(ScanArgs q) {
    pdl_trigger();
    pdl_wait();
    scan2_body(q);
}

__device__ __forceinline__ void scatter_mol_body(const ScatterArgs &a, int bid, int nblk) {
    if (a.rebuild && !*a.rebuild) return;
    for (int k = bid * blockDim.x + threadIdx.x; k < a.n_mol; k += nblk * blockDim.x)
        a.cell_mols[a.cell_mstart[a.mol_cell[k]] + a.mol_rank[k]] = k;
}
__global__ void k_scatter_mol(ScatterArgs a) {
    pdl_trigger();
    pdl_wait();
    scatter_mol_body(a, blockIdx.x, gridDim.x);
}

// One warp per domain cell: order the cell's molecules by index (ascending
// site index, the reference's cell-list order), assign slots and gather the
// cell-ordered arrays.
__device__ __forceinline__ void cell_sort_body(const SortArgs &a, int bid, int nblk) {
    const Grid &g = a.g;
    const int *__restrict__ mol_off = a.mol_off, *__restrict__ cell_mstart = a.cell_mstart;
    const int *__restrict__ cell_start = a.cell_start, *__restrict__ cell_mols = a.cell_mols;
    const double *__restrict__ r = a.r, *__restrict__ eps = a.eps, *__restrict__ sig = a.sig;
    const int *__restrict__ key = a.key;
    int *__restrict__ slot_site = a.slot_site, *__restrict__ site_slot = a.site_slot;
    float4 *__restrict__ pos4 = a.pos4;
    int *__restrict__ skey = a.skey;
    float *__restrict__ seps = a.seps;
    double *__restrict__ posd = a.posd, *__restrict__ seps_d = a.seps_d, *__restrict__ sig_d = a.sig_d;
    double *__restrict__ bias = a.bias;
    float4 *__restrict__ ref4 = a.ref4;
    int *__restrict__ slot_cell = a.slot_cell, *__restrict__ zkey = a.zkey;
    const int lane = threadIdx.x & 31;
    if (a.rebuild && !*a.rebuild) return;
    for (int cell = bid * kWarpsPerBlock + (threadIdx.x >> 5); cell < g.ncell;
         cell += nblk * kWarpsPerBlock) {
    int cx, cy, cz;
    cell_coords(g, cell, cx, cy, cz);
    const double cen[3] = {cell_centre(g, 0, cx), cell_centre(g, 1, cy), cell_centre(g, 2, cz)};
    const int ms = cell_mstart[cell], mc = cell_mstart[cell + 1] - ms;
    const int ss = cell_start[cell];
    for (int base = 0; base < mc; base += 32) {
        const int t = base + lane;
        const int mine = (t < mc) ? cell_mols[ms + t] : INT_MAX;
        int off = 0;
        for (int u = 0; u < mc; u++) {
            const int other = cell_mols[ms + u];
            if (other < mine) off += mol_off[other + 1] - mol_off[other];
        }
        if (t < mc) {
            const int s0 = mol_off[mine], s1 = mol_off[mine + 1];
            for (int s = s0; s < s1; s++) {
                const int slot = ss + off + (s - s0);
                slot_site[slot] = s;
                site_slot[s] = slot;
                const double x = r[3 * s], y = r[3 * s + 1], z = r[3 * s + 2];
                const float4 p4 = make_float4(__double2float_rn(x - cen[0]), __double2float_rn(y - cen[1]),
                                              __double2float_rn(z - cen[2]), __double2float_rn(0.5 * sig[s]));
                pos4[slot] = p4;
                skey[slot] = key[s];
                seps[slot] = __double2float_rn(sqrt(eps[s]));
                if (bias) {
                    bias[3 * s] = cen[0]; bias[3 * s + 1] = cen[1]; bias[3 * s + 2] = cen[2];
                    ref4[s] = p4;
                    slot_cell[slot] = cell;
                    // the half-list order key: z quantized over the box (see vl_above)
                    long long q = (long long)floor((z - g.low[2]) / g.L[2] * (double)kZq);
                    zkey[slot] = (int)(q < 0 ? 0 : (q >= kZq ? kZq - 1 : q));
                }
                if (posd) {
                    posd[3 * slot] = x; posd[3 * slot + 1] = y; posd[3 * slot + 2] = z;
                    seps_d[slot] = eps[s];
                    sig_d[slot] = sig[s];
                }
            }
        }
    }
    }
}
__global__ void __launch_bounds__(kBlock) k_cell_sort(SortArgs a) {
    pdl_trigger();
    pdl_wait();
    cell_sort_body(a, blockIdx.x, gridDim.x);
}

// ===========================================================================
// pair kernel: LJ 12-6 (LJ12_6.cpp:15-43), FENE (FENE.cpp:15-43), the ATM
// neighbour list inside cutoff_3b, energy / virial / histograms / counts.
//
// One warp per home cell, full shell (27 neighbour cells, periodic images by
// cell wrap), no atomics on forces: lane = (home site il, group grp); the G
// groups split each neighbour cell's sites and their partial forces are
// reduced through shared memory.  Real = float: cell-local FP32 coordinates;
// Real = double: absolute FP64 positions with the reference's exact
// dr = r_i - (r_j + shift) arithmetic.
// ===========================================================================
template <typename Real>
struct AtmEntry;
template <>
struct AtmEntry<float> { using T = float4; };
struct alignas(16) AtmEntryD { double x, y, z; long long code; };
template <>
struct AtmEntry<double> { using T = AtmEntryD; };

__device__ __forceinline__ float4 make_entry(float x, float y, float z, int code) {
    return make_float4(x, y, z, __int_as_float(code));
}
__device__ __forceinline__ AtmEntryD make_entry(double x, double y, double z, int code) {
    AtmEntryD e; e.x = x; e.y = y; e.z = z; e.code = code; return e;
}

template <typename Real, bool MEASURE, bool EMIT, bool FENE, bool COUNT>
__global__ void __launch_bounds__(kBlock) k_pair(PairParams p) {
    using Entry = typename AtmEntry<Real>::T;
    constexpr bool FP64 = sizeof(Real) == 8;
    __shared__ int s_cnt[kWarpsPerBlock][32];
    __shared__ Real s_red[kWarpsPerBlock][32][3];
    __shared__ double s_part[kWarpsPerBlock][R_NSLOTS];
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int cell = blockIdx.x * kWarpsPerBlock + wib;
    double a_u = 0.0, a_w[6] = {0, 0, 0, 0, 0, 0}, a_pairs = 0.0;
    const Real rc2 = (Real)p.rc2, rc3sq = (Real)p.rc3sq, scan2 = (Real)p.scan2;
    Entry *nl = reinterpret_cast<Entry *>(p.nl);

    if (cell < p.g.ncell) {
        int cx, cy, cz;
        cell_coords(p.g, cell, cx, cy, cz);
        const double cen[3] = {cell_centre(p.g, 0, cx), cell_centre(p.g, 1, cy), cell_centre(p.g, 2, cz)};
        const int hs = p.cell_start[cell], hn = p.cell_start[cell + 1] - hs;
        for (int base = 0; base < hn; base += 32) {
            const int hc = min(32, hn - base);
            const int G = 32 / hc;
            const int il = lane % hc, grp = lane / hc;
            const bool act = grp < G;
            const int is = hs + base + il;
            Real pix, piy, piz, sgi, epi;
            if (FP64) {
                pix = (Real)p.posd[3 * is]; piy = (Real)p.posd[3 * is + 1]; piz = (Real)p.posd[3 * is + 2];
                sgi = (Real)p.sig_d[is]; epi = (Real)p.seps_d[is];
            } else {
                const float4 q = p.pos4[is];
                pix = q.x; piy = q.y; piz = q.z; sgi = q.w; epi = p.seps[is];
            }
            const int ki = p.skey[is];
            const int site_i = p.slot_site[is];
            Real fx = 0, fy = 0, fz = 0;
            int cnt = 0;
            if (EMIT && lane < hc) s_cnt[wib][lane] = 0;
            __syncwarp();
            for (int nb = 0; nb < 27; nb++) {
                const NbCell q = neighbour_cell(p.g, cx, cy, cz, nb);
                const int js = p.cell_start[q.cell], jn = p.cell_start[q.cell + 1] - js;
                int qx, qy, qz;
                cell_coords(p.g, q.cell, qx, qy, qz);
                Real ox, oy, oz;
                if (FP64) {
                    ox = (Real)q.shift[0]; oy = (Real)q.shift[1]; oz = (Real)q.shift[2];
                } else {
                    ox = (Real)((cell_centre(p.g, 0, qx) + q.shift[0]) - cen[0]);
                    oy = (Real)((cell_centre(p.g, 1, qy) + q.shift[1]) - cen[1]);
                    oz = (Real)((cell_centre(p.g, 2, qz) + q.shift[2]) - cen[2]);
                }
                const bool vir_full = p.virial_compat && q.crosses;  // COMPAT: images counted per list entry
                if (!act) continue;
                for (int jj = grp; jj < jn; jj += G) {
                    const int j = js + jj;
                    if (j == is) continue;
                    Real dx, dy, dz, r2;
                    if (FP64) {
                        const double *pj = p.posd + 3 * j;
                        dx = (Real)dsub((double)pix, dadd(pj[0], (double)ox));
                        dy = (Real)dsub((double)piy, dadd(pj[1], (double)oy));
                        dz = (Real)dsub((double)piz, dadd(pj[2], (double)oz));
                        r2 = (Real)dadd(dadd(dmul((double)dx, (double)dx), dmul((double)dy, (double)dy)),
                                        dmul((double)dz, (double)dz));
                    } else {
                        const float4 pj = p.pos4[j];
                        dx = pix - (pj.x + ox);
                        dy = piy - (pj.y + oy);
                        dz = piz - (pj.z + oz);
                        r2 = dx * dx + dy * dy + dz * dz;
                    }
                    int kj = 0;
                    if (FENE) {
                        kj = p.skey[j];
                        if (kj == ki && !q.crosses) {
                            // FENE on same-molecule pairs, no cutoff: force on i
                            // along (r_j - r_i), overstretch -> 1e30 / (r_j - r_i)
                            const Real sgj = FP64 ? (Real)p.sig_d[j] : (Real)(2.0f * p.pos4[j].w);
                            const Real sgm = FP64 ? (sgi + sgj) / (Real)2.0 : (sgi + (Real)0.5 * sgj);
                            const Real R0 = (Real)1.5 * sgm;
                            const Real R02 = R0 * R0;
                            if (R02 <= r2) {
                                // invdr * 1e+30 with invdr = 1 / (r_j - r_i), as FENE.cpp:28-33
                                fx += ((Real)1 / (-dx)) * (Real)1e30;
                                fy += ((Real)1 / (-dy)) * (Real)1e30;
                                fz += ((Real)1 / (-dz)) * (Real)1e30;
                            } else {
                                Real e;
                                if (FP64) e = (Real)sqrt((double)epi * (double)p.seps_d[j]);
                                else e = epi * p.seps[j];
                                const Real k = (Real)p.stiffness * e / (sgm * sgm);
                                const Real fac = k / ((Real)1 - (r2 / R02));
                                fx -= dx * fac; fy -= dy * fac; fz -= dz * fac;
                            }
                        }
                    }
                    if (r2 > scan2) continue;
                    if (!FENE) kj = p.skey[j];
                    if (EMIT && r2 <= rc3sq) {
                        const int c = atomicAdd(&s_cnt[wib][il], 1);
                        if (c < p.nl_cap) nl[(size_t)is * p.nl_cap + c] = make_entry(dx, dy, dz, atm_code(nb, q.crosses, j));
                    }
                    if (!p.use_lj || r2 > rc2 || kj == ki) continue;
                    if (COUNT) { cnt++; continue; }
                    Real fac, u, ljd;
                    if (FP64) {
                        // LJ12_6_Force arithmetic in FP64 (pow(x, 3.0), pow(lj6, 2.0) as products)
                        const double inv = ddiv(1.0, (double)r2);
                        const double sgm = (p.sig_d[is] + p.sig_d[j]) / 2.0;
                        const double e = sqrt(p.seps_d[is] * p.seps_d[j]);
                        const double x = sgm * sgm * inv;
                        const double lj6 = x * x * x, lj12 = lj6 * lj6;
                        fac = (Real)(24.0 * e * (2.0 * lj12 - lj6) * inv);
                        u = (Real)(4.0 * e * (lj12 - lj6));
                        ljd = (Real)(24.0 * e * (2.0 * lj12 - lj6));
                    } else {
                        const float inv = __frcp_rn((float)r2);
                        const float sgm = (float)sgi + p.pos4[j].w;
                        const float x = sgm * sgm * inv;
                        const float lj6 = x * x * x, lj12 = lj6 * lj6;
                        const float e = (float)epi * p.seps[j];
                        ljd = 24.0f * e * (2.0f * lj12 - lj6);
                        fac = ljd * inv;
                        u = 4.0f * e * (lj12 - lj6);
                    }
                    if (!MEASURE) fac *= (Real)p.lj_fscale;   // ATM2B (1 otherwise); sensors stay unscaled
                    fx += dx * fac; fy += dy * fac; fz += dz * fac;
                    if (MEASURE) {
                        const double wt = vir_full ? 1.0 : 0.5;
                        const double gx = (double)dx * (double)fac, gy = (double)dy * (double)fac,
                                     gz = (double)dz * (double)fac;
                        a_u += 0.5 * (double)u;
                        a_pairs += 0.5;
                        a_w[0] += wt * ((double)dx * gx);
                        a_w[1] += wt * 0.5 * ((double)dx * gy + (double)dy * gx);
                        a_w[2] += wt * ((double)dy * gy);
                        a_w[3] += wt * 0.5 * ((double)dx * gz + (double)dz * gx);
                        a_w[4] += wt * 0.5 * ((double)dy * gz + (double)dz * gy);
                        a_w[5] += wt * ((double)dz * gz);
                        if (p.lj_hist) {
                            const int site_j = p.slot_site[j];
                            if (site_i < site_j) {
                                const double rp = sqrt((double)r2);
                                const double bw = 3.0 * p.max_sigma / (double)p.lj_bins;
                                unsigned long long bin = (unsigned long long)(rp / bw);
                                if (bin > (unsigned long long)(p.lj_bins - 1)) bin = p.lj_bins - 1;
                                atomicAdd(&p.lj_hist[bin], (double)u);
                                atomicAdd(&p.lj_hist[p.lj_bins + bin], (double)ljd / rp);
                                atomicAdd(&p.lj_hist[2 * p.lj_bins + bin], 1.0);
                                atomicAdd(&p.lj_hist[3 * p.lj_bins + bin], 1.0);
                            }
                        }
                    }
                }
            }
            // reduce the G partial sums of every home site
            if (COUNT) {
                s_cnt[wib][lane] = cnt;
                __syncwarp();
                if (act && grp == 0) {
                    long long c = 0;
                    for (int k = 0; k < G; k++) c += s_cnt[wib][il + k * hc];
                    p.counts[site_i] = c;
                }
                __syncwarp();
                continue;
            }
            s_red[wib][lane][0] = fx; s_red[wib][lane][1] = fy; s_red[wib][lane][2] = fz;
            __syncwarp();
            if (act && grp == 0) {
                Real sx = 0, sy = 0, sz = 0;
                for (int k = 0; k < G; k++) {
                    sx += s_red[wib][il + k * hc][0];
                    sy += s_red[wib][il + k * hc][1];
                    sz += s_red[wib][il + k * hc][2];
                }
                p.f[3 * site_i] = (double)sx;
                p.f[3 * site_i + 1] = (double)sy;
                p.f[3 * site_i + 2] = (double)sz;
            }
            if (EMIT && lane < hc) {
                const int c = s_cnt[wib][lane];
                p.nl_count[hs + base + lane] = min(c, p.nl_cap);
                if (c > p.nl_cap) atomicOr(&p.err[E_ATM_OVERFLOW], 1);
            }
            __syncwarp();
        }
    }
    if (MEASURE) {
        double vals[9] = {a_u, a_w[0], a_w[1], a_w[2], a_w[3], a_w[4], a_w[5], a_pairs, 0.0};
        for (int k = 0; k < 8; k++) {
            double x = vals[k];
            for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
            vals[k] = x;
        }
        if (lane == 0) {
            s_part[wib][R_ULJ] = vals[0];
            for (int k = 0; k < 6; k++) s_part[wib][R_W0 + k] = vals[1 + k];
            s_part[wib][R_PAIRS] = vals[7];
        }
        __syncthreads();
        if (threadIdx.x < R_NSLOTS) {
            const int t = threadIdx.x;
            double s = 0.0;
            if (t == R_ULJ || t == R_PAIRS || (t >= R_W0 && t <= R_W5))
                for (int w = 0; w < kWarpsPerBlock; w++) s += s_part[w][t];
            p.partials[(size_t)blockIdx.x * R_NSLOTS + t] = s;
        }
    }
}

// ===========================================================================
// ATM triplet kernel (ATM.cpp:22-62 / ATM_NOLIST.cpp:124-159): one warp per
// site i, every pair (a, b) of i's neighbours inside cutoff_3b with
// |r_a - r_b| inside too.  Force on i only (each triplet is visited from all
// three vertices, no atomics).  With A=|r_ia|^2, B=|r_ib|^2, C=|r_ab|^2:
//   V = nu [ (ABC)^-3/2 + 3/8 P (ABC)^-5/2 ],  P = (A+B-C)(A-B+C)(-A+B+C)
//   dV/dA = nu (ABC)^-5/2 [ -3/2 BC + 3/8 dP/dA - 15/16 P/A ]
//   F_i(physical) = -2 (dV/dA e_a + dV/dB e_b),  e_a = r_i - r_a
// which equals the reference's comp_force terms (comp_force = 2 dV/dA).
// ===========================================================================
__device__ __forceinline__ int entry_code(const float4 &e) { return __float_as_int(e.w); }
__device__ __forceinline__ int entry_code(const AtmEntryD &e) { return (int)e.code; }
__device__ __forceinline__ float rsqrt_r(float x) { return rsqrtf(x); }
__device__ __forceinline__ double rsqrt_r(double x) { return 1.0 / sqrt(x); }

template <typename Real, bool MEASURE, bool COMPAT>
__global__ void __launch_bounds__(kBlock) k_atm(AtmParams p) {
    using Entry = typename AtmEntry<Real>::T;
    struct Q2 { Real A, invA; };
    extern __shared__ float4 s_dyn[];
    __shared__ double s_part[kWarpsPerBlock][4 + 6];
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int cap = p.nl_cap;
    Entry *se = reinterpret_cast<Entry *>(s_dyn) + wib * cap;
    Q2 *sq = reinterpret_cast<Q2 *>(reinterpret_cast<Entry *>(s_dyn) + kWarpsPerBlock * cap) + wib * cap;
    const Entry *nl = reinterpret_cast<const Entry *>(p.nl);
    const int i = blockIdx.x * kWarpsPerBlock + wib;
    Real gx = 0, gy = 0, gz = 0;
    double a_e = 0.0, a_t = 0.0, a_w[6] = {0, 0, 0, 0, 0, 0};
    const Real rc2 = (Real)p.rc2;
    if (i < p.n) {
        const int ni = p.nl_count[i];
        for (int k = lane; k < ni; k += 32) {
            const Entry e = nl[(size_t)i * cap + k];
            const Real A = (Real)e.x * (Real)e.x + (Real)e.y * (Real)e.y + (Real)e.z * (Real)e.z;
            se[k] = e;
            sq[k] = Q2{A, (Real)1 / A};
        }
        __syncwarp();
        for (int a0 = 0; a0 < ni; a0 += 32) {
            const int a = a0 + lane;
            const bool av = a < ni;
            Real ax = 0, ay = 0, az = 0;
            Q2 qa{1, 1};
            int ca = 0;
            if (av) {
                const Entry ea = se[a];
                ax = (Real)ea.x; ay = (Real)ea.y; az = (Real)ea.z;
                ca = entry_code(ea);
                qa = sq[a];
            }
            const Real wa = rsqrt_r(qa.A);
            for (int d = 1; d <= ni / 2; d++) {
                if (!av || (2 * d == ni && a >= d)) continue;
                int b = a + d;
                if (b >= ni) b -= ni;
                const Entry eb = se[b];
                const Q2 qb = sq[b];
                const int cb = entry_code(eb);
                if (COMPAT) {
                    const int nba = ca & 31, nbb = cb & 31;
                    const bool ok = (nba == 13 && nbb == 13) || (nba != 13 && nbb != 13 && nba != nbb);
                    if (!ok) continue;
                }
                const Real bx = (Real)eb.x, by = (Real)eb.y, bz = (Real)eb.z;
                const Real cx = bx - ax, cy = by - ay, cz = bz - az;
                const Real C = cx * cx + cy * cy + cz * cz;
                if (C > rc2) continue;
                const Real A = qa.A, B = qb.A;
                const Real wc = rsqrt_r(C);
                const Real sv = wa * rsqrt_r(B) * wc;       // 1/(abc)
                const Real s2 = sv * sv;
                const Real s5 = s2 * s2 * sv;
                const Real t1 = A + B - C, t2 = A - B + C, t3 = B + C - A;
                const Real u = t2 * t3, v = t1 * t3, w = t1 * t2;
                const Real P = t1 * u;
                const Real vA = s5 * ((Real)-1.5 * B * C + (Real)0.375 * (u + v - w) - (Real)0.9375 * P * qa.invA);
                const Real vB = s5 * ((Real)-1.5 * A * C + (Real)0.375 * (u - v + w) - (Real)0.9375 * P * qb.invA);
                gx += vA * ax + vB * bx;
                gy += vA * ay + vB * by;
                gz += vA * az + vB * bz;
                if (MEASURE) {
                    const Real vC = s5 * ((Real)-1.5 * A * B + (Real)0.375 * (-u + v + w) - (Real)0.9375 * P * (wc * wc));
                    a_e += (double)(s2 * sv * ((Real)1 + (Real)0.375 * P * s2)) * (1.0 / 3.0);
                    a_t += 1.0 / 3.0;
                    double wt;
                    if (p.virial_compat) {
                        const int k = 1 + ((ca & 32) ? 0 : 1) + ((cb & 32) ? 0 : 1);
                        wt = p.atm_direct ? 0.0 : 1.0 / (double)k;
                    } else {
                        wt = 1.0 / 3.0;
                    }
                    // pair-decomposed virial sum_pairs P_ab d (x) d with P_ab = -2 dV/d(r_ab^2)
                    const double pa = -2.0 * (double)vA, pb = -2.0 * (double)vB, pc = -2.0 * (double)vC;
                    const double dax = ax, day = ay, daz = az, dbx = bx, dby = by, dbz = bz;
                    const double dcx = cx, dcy = cy, dcz = cz;
                    a_w[0] += wt * (pa * dax * dax + pb * dbx * dbx + pc * dcx * dcx);
                    a_w[1] += wt * (pa * dax * day + pb * dbx * dby + pc * dcx * dcy);
                    a_w[2] += wt * (pa * day * day + pb * dby * dby + pc * dcy * dcy);
                    a_w[3] += wt * (pa * dax * daz + pb * dbx * dbz + pc * dcx * dcz);
                    a_w[4] += wt * (pa * day * daz + pb * dby * dbz + pc * dcy * dcz);
                    if (!p.virial_compat) a_w[5] += wt * (pa * daz * daz + pb * dbz * dbz + pc * dcz * dcz);
                }
            }
        }
        for (int o = 16; o > 0; o >>= 1) {
            gx += __shfl_xor_sync(0xffffffffu, gx, o);
            gy += __shfl_xor_sync(0xffffffffu, gy, o);
            gz += __shfl_xor_sync(0xffffffffu, gz, o);
        }
        if (lane == 0) {
            const int site = p.slot_site[i];
            // reference sign: +2 nu (vA e_a + vB e_b); physical: the negative
            const double sc = 2.0 * (double)p.sign * p.nu;
            p.f[3 * site] += sc * (double)gx;
            p.f[3 * site + 1] += sc * (double)gy;
            p.f[3 * site + 2] += sc * (double)gz;
        }
    }
    if (MEASURE) {
        double vals[8] = {a_e, a_t, a_w[0], a_w[1], a_w[2], a_w[3], a_w[4], a_w[5]};
        for (int k = 0; k < 8; k++) {
            double x = vals[k];
            for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
            vals[k] = x;
        }
        if (lane == 0) for (int k = 0; k < 8; k++) s_part[wib][k] = vals[k];
        __syncthreads();
        if (threadIdx.x < R_NSLOTS) {
            const int t = threadIdx.x;
            double sum = 0.0;
            int src = -1;
            if (t == R_UATM) src = 0;
            else if (t == R_TRIPS) src = 1;
            else if (t >= R_W0 && t <= R_W5) src = 2 + (t - R_W0);
            if (src >= 0)
                for (int w = 0; w < kWarpsPerBlock; w++) sum += s_part[w][src];
            // nu scaling of energy and virial
            if (t == R_UATM || (t >= R_W0 && t <= R_W5)) sum *= p.nu;
            p.partials[(size_t)blockIdx.x * R_NSLOTS + t] = sum;
        }
    }
}

// FP32 ATM kernel with ballot compaction: lanes test candidate pairs (a, b)
// of the vertex's neighbour list (round-robin pairing a, a+d mod n, so each
// unordered pair is tested once) and queue the ones inside the cutoff; the
// triplet arithmetic then always runs on 32 queued pairs at a time.  All
// queued pairs share vertex i, so each lane keeps a private force sum.
template <bool MEASURE, bool COMPAT>
__global__ void __launch_bounds__(kBlock) k_atm_q(AtmParams p) {
    extern __shared__ float4 s_dyn[];
    __shared__ unsigned s_q[kWarpsPerBlock][64];
    __shared__ float s_qc[kWarpsPerBlock][64];
    __shared__ double s_part[kWarpsPerBlock][8];
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int cap = p.nl_cap;
    float4 *se = s_dyn + wib * cap;
    float4 *sq = s_dyn + kWarpsPerBlock * cap + wib * cap;   // (A, 1/A, 1/sqrt(A), -) per entry
    const int i = blockIdx.x * kWarpsPerBlock + wib;
    const float rc2 = (float)p.rc2;
    float gx = 0.f, gy = 0.f, gz = 0.f;
    float m_e = 0.f, m_w[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    int m_t = 0;   // triplet visits (each triplet is visited from its three vertices)
    unsigned lt;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lt));

    auto triplet = [&](unsigned e, float C, bool valid) {
        if (!valid) return;
        const int a = (int)(e & 0xffffu), b = (int)(e >> 16);
        const float4 ea = se[a], eb = se[b];
        const float4 qa = sq[a], qb = sq[b];
        const float A = qa.x, B = qb.x;
        const float wc = rsqrtf(C);
        const float sv = qa.z * qb.z * wc;                  // 1/(abc)
        const float s2 = sv * sv;
        const float s5 = s2 * s2 * sv;
        const float t1 = A + B - C, t2 = A - B + C, t3 = B + C - A;
        const float u = t2 * t3, v = t1 * t3, w = t1 * t2;
        const float P = t1 * u;
        float vA = s5 * (-1.5f * B * C + 0.375f * (u + v - w) - 0.9375f * P * qa.y);
        float vB = s5 * (-1.5f * A * C + 0.375f * (u - v + w) - 0.9375f * P * qb.y);
        float vC = s5 * (-1.5f * A * B + 0.375f * (-u + v + w) - 0.9375f * P * (wc * wc));
        float Vn = s2 * sv * (1.0f + 0.375f * P * s2);   // V / nu
        if (p.sw) {   // switched cutoff: V Sa Sb Sc and its derivatives in A, B, C
            float Sa, dSa, Sb, dSb, Sc, dSc;
            sw_eval(A, p.sw_rc2, p.sw_iw, Sa, dSa);
            sw_eval(B, p.sw_rc2, p.sw_iw, Sb, dSb);
            sw_eval(C, p.sw_rc2, p.sw_iw, Sc, dSc);
            const float sbc = Sb * Sc, sac = Sa * Sc, sab = Sa * Sb;
            vA = sbc * (vA * Sa + Vn * dSa);
            vB = sac * (vB * Sb + Vn * dSb);
            vC = sab * (vC * Sc + Vn * dSc);
            Vn = Vn * Sa * sbc;
        }
        gx += vA * ea.x + vB * eb.x;
        gy += vA * ea.y + vB * eb.y;
        gz += vA * ea.z + vB * eb.z;
        if (MEASURE) {
            m_e += Vn * (1.0f / 3.0f);
            m_t++;
            float wt;
            if (p.virial_compat) {
                const int ca = __float_as_int(ea.w), cb = __float_as_int(eb.w);
                const int k = 1 + ((ca & 32) ? 0 : 1) + ((cb & 32) ? 0 : 1);
                wt = p.atm_direct ? 0.0f : 1.0f / (float)k;
            } else {
                wt = 1.0f / 3.0f;
            }
            const float pa = -2.0f * vA * wt, pb = -2.0f * vB * wt, pc = -2.0f * vC * wt;
            const float cx = eb.x - ea.x, cy = eb.y - ea.y, cz = eb.z - ea.z;
            m_w[0] += pa * ea.x * ea.x + pb * eb.x * eb.x + pc * cx * cx;
            m_w[1] += pa * ea.x * ea.y + pb * eb.x * eb.y + pc * cx * cy;
            m_w[2] += pa * ea.y * ea.y + pb * eb.y * eb.y + pc * cy * cy;
            m_w[3] += pa * ea.x * ea.z + pb * eb.x * eb.z + pc * cx * cz;
            m_w[4] += pa * ea.y * ea.z + pb * eb.y * eb.z + pc * cy * cz;
            if (!p.virial_compat) m_w[5] += pa * ea.z * ea.z + pb * eb.z * eb.z + pc * cz * cz;
        }
    };

    if (i < p.n) {
        const int ni = p.nl_count[i];
        for (int k = lane; k < ni; k += 32) {
            const float4 e = p.nl[(size_t)i * cap + k];
            const float A = e.x * e.x + e.y * e.y + e.z * e.z;
            se[k] = e;
            sq[k] = make_float4(A, 1.0f / A, rsqrtf(A), 0.f);
        }
        __syncwarp();
        int qn = 0;
        const int half = ni / 2;
        for (int a0 = 0; a0 < ni; a0 += 32) {
            const int a = a0 + lane;
            const bool av = a < ni;
            float4 ea = make_float4(0.f, 0.f, 0.f, 0.f);
            if (av) ea = se[a];
            for (int d = 1; d <= half; d++) {
                bool hit = false;
                int b = 0;
                float C = 0.f;
                if (av && !(2 * d == ni && a >= d)) {
                    b = a + d;
                    if (b >= ni) b -= ni;
                    const float4 eb = se[b];
                    bool ok = true;
                    if (COMPAT) {
                        const int nba = __float_as_int(ea.w) & 31, nbb = __float_as_int(eb.w) & 31;
                        ok = (nba == 13 && nbb == 13) || (nba != 13 && nbb != 13 && nba != nbb);
                    }
                    const float cx = eb.x - ea.x, cy = eb.y - ea.y, cz = eb.z - ea.z;
                    C = cx * cx + cy * cy + cz * cz;
                    hit = ok && C <= rc2;
                }
                const unsigned m = __ballot_sync(0xffffffffu, hit);
                if (hit) {
                    const int pos = qn + __popc(m & lt);
                    s_q[wib][pos] = (unsigned)a | ((unsigned)b << 16);
                    s_qc[wib][pos] = C;
                }
                qn += __popc(m);
                if (qn >= 32) {
                    __syncwarp();
                    const unsigned e = s_q[wib][lane];
                    const float ce = s_qc[wib][lane];
                    const bool mv = lane < qn - 32;
                    const unsigned te = mv ? s_q[wib][lane + 32] : 0u;
                    const float tc = mv ? s_qc[wib][lane + 32] : 0.f;
                    __syncwarp();
                    if (mv) { s_q[wib][lane] = te; s_qc[wib][lane] = tc; }
                    __syncwarp();
                    qn -= 32;
                    triplet(e, ce, true);
                }
            }
        }
        __syncwarp();
        if (qn > 0) {
            const bool v = lane < qn;
            const unsigned e = v ? s_q[wib][lane] : 0u;
            const float ce = v ? s_qc[wib][lane] : 1.f;
            triplet(e, ce, v);
        }
        for (int o = 16; o > 0; o >>= 1) {
            gx += __shfl_xor_sync(0xffffffffu, gx, o);
            gy += __shfl_xor_sync(0xffffffffu, gy, o);
            gz += __shfl_xor_sync(0xffffffffu, gz, o);
        }
        float ev = m_e;
        if (MEASURE && p.e_site)
            for (int o = 16; o > 0; o >>= 1) ev += __shfl_xor_sync(0xffffffffu, ev, o);
        if (lane == 0) {
            const int site = p.slot_site[i];
            const double sc = 2.0 * p.sign * p.nu;   // reference: +2 nu (...); physical: -2 nu (...)
            p.f[3 * site] += sc * (double)gx;
            p.f[3 * site + 1] += sc * (double)gy;
            p.f[3 * site + 2] += sc * (double)gz;
            if (MEASURE && p.e_site) p.e_site[site] = p.nu * (double)ev;
        }
    }
    if (MEASURE) {
        // FP32 warp tree over the lanes' FP32 partials, FP64 from the warp sums on
        float vals[8] = {m_e, 0.f, m_w[0], m_w[1], m_w[2], m_w[3], m_w[4], m_w[5]};
        for (int k = 0; k < 8; k++) {
            float x = vals[k];
            for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
            vals[k] = x;
        }
        int visits = m_t;   // an exact integer count, a third of a triplet per visit
        for (int o = 16; o > 0; o >>= 1) visits += __shfl_xor_sync(0xffffffffu, visits, o);
        if (lane == 0) {
            for (int k = 0; k < 8; k++) s_part[wib][k] = (double)vals[k];
            s_part[wib][1] = (double)visits / 3.0;
        }
        __syncthreads();
        if (threadIdx.x < R_NSLOTS) {
            const int t = threadIdx.x;
            double sum = 0.0;
            int src = -1;
            if (t == R_UATM) src = 0;
            else if (t == R_TRIPS) src = 1;
            else if (t >= R_W0 && t <= R_W5) src = 2 + (t - R_W0);
            if (src >= 0)
                for (int w = 0; w < kWarpsPerBlock; w++) sum += s_part[w][src];
            if (t == R_UATM || (t >= R_W0 && t <= R_W5)) sum *= p.nu;
            p.partials[(size_t)blockIdx.x * R_NSLOTS + t] = sum;
        }
    }
}

// ===========================================================================
// bonded terms (no reference counterpart): harmonic bond and angle, FP32
// arithmetic on FP64 differences, FP64 atomic accumulation into f.
// ===========================================================================
__global__ void k_bonds(int nb, const int *__restrict__ bonds, const double *__restrict__ r, double *f, float kb,
                        float r0, double *partials, int measure) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    double e = 0.0, w[6] = {0, 0, 0, 0, 0, 0};
    if (t < nb) {
        const int i = bonds[2 * t], j = bonds[2 * t + 1];
        const float dx = (float)(r[3 * i] - r[3 * j]), dy = (float)(r[3 * i + 1] - r[3 * j + 1]),
                    dz = (float)(r[3 * i + 2] - r[3 * j + 2]);
        const float rr = sqrtf(dx * dx + dy * dy + dz * dz);
        const float dl = rr - r0;
        const float fs = -kb * dl / rr;
        atomicAdd(&f[3 * i], (double)(fs * dx)); atomicAdd(&f[3 * i + 1], (double)(fs * dy));
        atomicAdd(&f[3 * i + 2], (double)(fs * dz));
        atomicAdd(&f[3 * j], (double)(-fs * dx)); atomicAdd(&f[3 * j + 1], (double)(-fs * dy));
        atomicAdd(&f[3 * j + 2], (double)(-fs * dz));
        if (measure) {
            e = 0.5 * (double)kb * (double)dl * (double)dl;
            w[0] = fs * dx * dx; w[1] = fs * dx * dy; w[2] = fs * dy * dy;
            w[3] = fs * dx * dz; w[4] = fs * dy * dz; w[5] = fs * dz * dz;
        }
    }
    if (measure) {
        double vals[7] = {e, w[0], w[1], w[2], w[3], w[4], w[5]};
        for (int k = 0; k < 7; k++) {
            double x = vals[k];
            for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
            if ((threadIdx.x & 31) == 0) atomicAdd(&partials[k == 0 ? R_UBOND : R_W0 + k - 1], x);
        }
    }
}

__global__ void k_angles(int na, const int *__restrict__ angles, const double *__restrict__ r, double *f, float ka,
                         float th0, double *partials, int measure) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    double e = 0.0, w[6] = {0, 0, 0, 0, 0, 0};
    if (t < na) {
        const int i = angles[3 * t], j = angles[3 * t + 1], k = angles[3 * t + 2];
        float u[3], v[3];
        for (int d = 0; d < 3; d++) {
            u[d] = (float)(r[3 * i + d] - r[3 * j + d]);
            v[d] = (float)(r[3 * k + d] - r[3 * j + d]);
        }
        const float uu = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
        const float vv = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
        const float uv = u[0] * v[0] + u[1] * v[1] + u[2] * v[2];
        const float inu = rsqrtf(uu), inv_ = rsqrtf(vv);
        float cs = uv * inu * inv_;
        cs = fminf(1.0f, fmaxf(-1.0f, cs));
        const float th = acosf(cs);
        const float dth = th - th0;
        const float sn = fmaxf(sqrtf(1.0f - cs * cs), 1e-6f);
        const float pre = ka * dth / sn;
        float fi[3], fk[3];
        for (int d = 0; d < 3; d++) {
            fi[d] = pre * (v[d] * inu * inv_ - cs * u[d] * inu * inu);
            fk[d] = pre * (u[d] * inu * inv_ - cs * v[d] * inv_ * inv_);
            atomicAdd(&f[3 * i + d], (double)fi[d]);
            atomicAdd(&f[3 * k + d], (double)fk[d]);
            atomicAdd(&f[3 * j + d], -(double)(fi[d] + fk[d]));
        }
        if (measure) {
            e = 0.5 * (double)ka * (double)dth * (double)dth;
            w[0] = u[0] * fi[0] + v[0] * fk[0]; w[1] = u[0] * fi[1] + v[0] * fk[1];
            w[2] = u[1] * fi[1] + v[1] * fk[1]; w[3] = u[0] * fi[2] + v[0] * fk[2];
            w[4] = u[1] * fi[2] + v[1] * fk[2]; w[5] = u[2] * fi[2] + v[2] * fk[2];
        }
    }
    if (measure) {
        double vals[7] = {e, w[0], w[1], w[2], w[3], w[4], w[5]};
        for (int q = 0; q < 7; q++) {
            double x = vals[q];
            for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
            if ((threadIdx.x & 31) == 0) atomicAdd(&partials[q == 0 ? R_UBOND : R_W0 + q - 1], x);
        }
    }
}

// Limit_Force (Limit.cpp:19-25): clamp with Kokkos::min / max semantics
__global__ void k_limit(int n, const double *__restrict__ eps, const double *__restrict__ sig, double limit,
                        double *__restrict__ f) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const double fmax = limit * eps[s] / sig[s];
    for (int d = 0; d < 3; d++) {
        double x = f[3 * s + d];
        x = (fmax < x) ? fmax : x;
        x = (x < -fmax) ? -fmax : x;
        f[3 * s + d] = x;
    }
}

// ===========================================================================
// velocity Verlet (Integrator.cpp:28-37), FP64 without contraction
// ===========================================================================
// With a Verlet list (bias != nullptr) it also flags a rebuild when a site's
// cell-local position r - bias has moved more than skin/2 since the build.
// hdtm[s] = (dt * 0.5) / m[s], the reference's dtInv2m (Integrator.cpp:29), computed
// once at upload with the same IEEE division
__global__ void k_step0(int n, double *__restrict__ r, double *__restrict__ v, const double *__restrict__ f,
                        const double *__restrict__ hdtm, double dt, Grid g,
                        const double *__restrict__ bias, const float4 *__restrict__ ref4, float half_skin2,
                        int *__restrict__ rebuild) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const double c = hdtm[s];
    double x[3];
    for (int d = 0; d < 3; d++) {
        const double vv = dadd(v[3 * s + d], dmul(f[3 * s + d], c));
        v[3 * s + d] = vv;
        x[d] = dadd(r[3 * s + d], dmul(vv, dt));
        r[3 * s + d] = x[d];
    }
    if (bias) {
        const float4 q = ref4[s];
        const float dx = __double2float_rn(dsub(x[0], bias[3 * s])) - q.x;
        const float dy = __double2float_rn(dsub(x[1], bias[3 * s + 1])) - q.y;
        const float dz = __double2float_rn(dsub(x[2], bias[3 * s + 2])) - q.z;
        if (dx * dx + dy * dy + dz * dz > half_skin2) *rebuild = 1;
    }
}

// Verlet path with single-site molecules whose COM is exactly the position
// (power-of-two masses): integrate0, the skin test, the periodic wrap with
// its bias update and COM (k_com_wrap_bin's operations) and the FP32
// cell-local refresh (k_refresh's) in one pass over the sites.  The
// results are those of the separate kernels; on a rebuild step the cell sort
// rewrites pos4 afterwards.
// integer key with key(x) < key(y) exactly when x < y for non-NaN doubles
// (-0.0 and +0.0 share the key 0)
__device__ __forceinline__ long long dkey(double x) {
    const long long b = __double_as_longlong(x);
    const long long m = b & 0x7fffffffffffffffLL;
    return b < 0 ? -m : m;
}
// double -> float rounded to nearest (ties to even) from the bits, in integer
// instructions (GB300 converts FP64 -> FP32 on its narrow FP64 pipe): the 29
// dropped mantissa bits decide the rounding, and a carry out of the mantissa
// moves into the exponent as IEEE rounding does.  Results outside the FP32
// normal range (zero, subnormal, overflow, NaN) take the conversion
// instruction.  Bitwise equal to __double2float_rn.
__device__ __forceinline__ float d2f_rn(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int e = (int)((b >> 52) & 0x7ffu) - 1023 + 127;   // the FP32 biased exponent
    if (e < 1 || e > 254) return __double2float_rn(x);
    const unsigned long long mant = b & 0xfffffffffffffULL;
    unsigned f = ((unsigned)e << 23) | (unsigned)(mant >> 29);
    const unsigned rest = (unsigned)(mant & 0x1fffffffULL);
    f += (rest > 0x10000000u || (rest == 0x10000000u && (f & 1u))) ? 1u : 0u;
    return __uint_as_float(f | ((unsigned)(b >> 32) & 0x80000000u));
}
__device__ __forceinline__ bool dkey_nan(double x) {
    return (__double_as_longlong(x) & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL;
}

// Block-cooperative copies of a block's rows (3 doubles per site) between a
// caller's host buffer and shared memory in 16-byte pieces: over the host link
// whole contiguous lines move instead of 8-byte pieces strided by 24 bytes.
constexpr int kIoBlock = 256;   // sites per block of the kernels that do host I/O

__device__ __forceinline__ void rows_in(const double *src, double *dst_s, int base, int cnt) {
    const double *p = src + 3 * (size_t)base;
    const int m = 3 * cnt;
    if ((reinterpret_cast<uintptr_t>(p) & 15u) == 0) {
        const double2 *p2 = reinterpret_cast<const double2 *>(p);
        for (int k = threadIdx.x; k < m / 2; k += blockDim.x) {
            const double2 q = p2[k];
            dst_s[2 * k] = q.x;
            dst_s[2 * k + 1] = q.y;
        }
        if ((m & 1) && threadIdx.x == 0) dst_s[m - 1] = p[m - 1];
    } else {
        for (int k = threadIdx.x; k < m; k += blockDim.x) dst_s[k] = p[k];
    }
}

__device__ __forceinline__ void rows_out(const double *src_s, double *dst, int base, int cnt) {
    double *p = dst + 3 * (size_t)base;
    const int m = 3 * cnt;
    if ((reinterpret_cast<uintptr_t>(p) & 15u) == 0) {
        double2 *p2 = reinterpret_cast<double2 *>(p);
        for (int k = threadIdx.x; k < m / 2; k += blockDim.x) p2[k] = make_double2(src_s[2 * k], src_s[2 * k + 1]);
        if ((m & 1) && threadIdx.x == 0) p[m - 1] = src_s[m - 1];
    } else {
        for (int k = threadIdx.x; k < m; k += blockDim.x) p[k] = src_s[k];
    }
}

// r_in / v_in: where this step's positions and velocities are read (the
// engine's own arrays, or a caller's host buffers reached over the host link);
// r_out: an extra host copy of the new positions (nullptr: none).  Launched
// with kIoBlock threads per block.
__device__ __forceinline__ void step0_fused_body(const Step0Args &a, int bid) {
    __shared__ double s_r[3 * kIoBlock], s_v[3 * kIoBlock];
    const int n = a.n;
    double *r = a.r, *v = a.v;
    const double *__restrict__ f = a.f, *__restrict__ hdtm = a.hdtm;
    const double dt = a.dt;
    const Grid &g = a.g;
    double *__restrict__ bias = a.bias;
    const float4 *__restrict__ ref4 = a.ref4;
    const float half_skin2 = a.half_skin2;
    int *__restrict__ rebuild = a.rebuild;
    double *__restrict__ com = a.com;
    const int *__restrict__ site_slot = a.site_slot;
    float4 *__restrict__ pos4 = a.pos4;
    const double *r_in = a.r_in, *v_in = a.v_in;
    double *r_out = a.r_out;
    const int t = threadIdx.x;
    const int base = bid * blockDim.x, s = base + t;
    const int cnt = min((int)blockDim.x, n - base);
    const bool host_in = r_in != r;   // uniform: the whole step reads the caller's buffers
    if (host_in) {
        rows_in(r_in, s_r, base, cnt);
        rows_in(v_in, s_v, base, cnt);
        __syncthreads();
    }
    if (s < n) {
        const double c = hdtm[s];
        double x[3], b[3], vi[3], ri[3];
        for (int d = 0; d < 3; d++) {
            vi[d] = host_in ? s_v[3 * t + d] : v[3 * s + d];
            ri[d] = host_in ? s_r[3 * t + d] : r[3 * s + d];
        }
        for (int d = 0; d < 3; d++) {
            const double vv = dadd(vi[d], dmul(f[3 * s + d], c));
            v[3 * s + d] = vv;
            x[d] = dadd(ri[d], dmul(vv, dt));
            b[d] = bias[3 * s + d];
        }
        // Periodic_Kernel on the COM (= the position): strict comparisons, made on
        // order-preserving integer keys (the FP64 pipe is the bottleneck here);
        // the cell-local position x - bias is unchanged by a wrap
        double off[3];
        bool moved = false;
        for (int d = 0; d < 3; d++) {
            off[d] = 0.0;
            const long long kx = dkey(x[d]);
            if (!dkey_nan(x[d])) {
                if (kx < dkey(g.low[d])) {
                    off[d] = g.L[d];
                    moved = true;
                }
                if (kx > dkey(g.high[d])) {
                    off[d] = -g.L[d];
                    moved = true;
                }
            }
        }
        if (moved) {   // r += shift over all three components, as Periodic_Kernel
            for (int d = 0; d < 3; d++) {
                x[d] = dadd(x[d], off[d]);
                b[d] = dadd(b[d], off[d]);
                bias[3 * s + d] = b[d];
            }
        }
        float4 p = pos4[site_slot[s]];
        p.x = d2f_rn(dsub(x[0], b[0]));
        p.y = d2f_rn(dsub(x[1], b[1]));
        p.z = d2f_rn(dsub(x[2], b[2]));
        pos4[site_slot[s]] = p;
        {
            const float4 q = ref4[s];
            const float dx = p.x - q.x, dy = p.y - q.y, dz = p.z - q.z;
            if (dx * dx + dy * dy + dz * dz > half_skin2) *rebuild = 1;
        }
        for (int d = 0; d < 3; d++) {
            r[3 * s + d] = x[d];
            com[3 * s + d] = x[d];
        }
        if (r_out)   // each thread overwrites only the entries it read
            for (int d = 0; d < 3; d++) s_r[3 * t + d] = x[d];
    }
    if (r_out) {
        __syncthreads();
        rows_out(s_r, r_out, base, cnt);
    }
}
__global__ void __launch_bounds__(kIoBlock) k_step0_fused(Step0Args a) {
    pdl_trigger();
    step0_fused_body(a, blockIdx.x);
}

__global__ void k_step1(int n, double *__restrict__ v, const double *__restrict__ f, const double *__restrict__ hdtm,
                        int *__restrict__ err, int *__restrict__ rebuild) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (rebuild && s == 0) *rebuild = 0;   // every consumer of this step's flag has run
    if (s >= n) return;
    const double c = hdtm[s];
    bool bad = false;
    for (int d = 0; d < 3; d++) {
        const double vv = dadd(v[3 * s + d], dmul(f[3 * s + d], c));
        v[3 * s + d] = vv;
        bad |= !isfinite(vv);
    }
    if (bad) atomicOr(&err[E_NONFINITE], 1);
}

// Verlet path, steps without rebuild: cell-local FP32 coordinates
// (float)(r - bias) relative to each slot's build cell.
__global__ void k_refresh(int n, const int *__restrict__ slot_site, const double *__restrict__ r,
                          const double *__restrict__ bias, float4 *__restrict__ pos4, const int *__restrict__ rebuild) {
    const int slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= n || *rebuild) return;
    const int s = slot_site[slot];
    float4 p = pos4[slot];
    p.x = __double2float_rn(dsub(r[3 * s], bias[3 * s]));
    p.y = __double2float_rn(dsub(r[3 * s + 1], bias[3 * s + 1]));
    p.z = __double2float_rn(dsub(r[3 * s + 2], bias[3 * s + 2]));
    pos4[slot] = p;
}

// ===========================================================================
// sensors
// ===========================================================================
// TemperatureSensor::measure (sites inside [low, high]) + kinetic tensor
// (PressureSensor::MomentumKernel) over the first n_terms sites.
// Grid-stride over the sites (a resident grid, so each thread sums several
// sites before the fixed-tree warp and block reductions; the order is fixed,
// so the sums are deterministic).  TERMS adds the per-site kinetic tensor of
// the first n_terms sites.
template <bool TERMS>
__global__ void __launch_bounds__(kBlock) k_kinetic(Grid g, int n, int n_terms, const double *__restrict__ r,
                                                    const double *__restrict__ v, const double *__restrict__ m,
                                                    double *__restrict__ partials) {
    __shared__ double s_part[kWarpsPerBlock][8];
    constexpr int kVals = TERMS ? 8 : 2;
    double vals[kVals];
    for (int k = 0; k < kVals; k++) vals[k] = 0.0;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
        const double x = r[3 * s], y = r[3 * s + 1], z = r[3 * s + 2];
        const double vx = v[3 * s], vy = v[3 * s + 1], vz = v[3 * s + 2], ms = m[s];
        if (x >= g.low[0] && y >= g.low[1] && z >= g.low[2] && x <= g.high[0] && y <= g.high[1] && z <= g.high[2]) {
            vals[0] = dadd(vals[0], dmul(ms, dadd(dadd(dmul(vx, vx), dmul(vy, vy)), dmul(vz, vz))));
            vals[1] = dadd(vals[1], 1.0);
        }
        if constexpr (TERMS) {
            if (s < n_terms) {
                vals[2] += vx * vx * ms; vals[3] += vx * vy * ms; vals[4] += vy * vy * ms;
                vals[5] += vx * vz * ms; vals[6] += vy * vz * ms; vals[7] += vz * vz * ms;
            }
        }
    }
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    for (int k = 0; k < kVals; k++) {
        double xk = vals[k];
        for (int o = 16; o > 0; o >>= 1) xk += __shfl_xor_sync(0xffffffffu, xk, o);
        if (lane == 0) s_part[wib][k] = xk;
    }
    __syncthreads();
    if (threadIdx.x < R_NSLOTS) {
        const int t = threadIdx.x;
        double acc = 0.0;
        int src = -1;
        if (t == R_MV2) src = 0;
        else if (t == R_NBOX) src = 1;
        else if (TERMS && t >= R_K0 && t <= R_K5) src = 2 + t - R_K0;
        if (src >= 0)
            for (int w = 0; w < kWarpsPerBlock; w++) acc += s_part[w][src];
        partials[(size_t)blockIdx.x * R_NSLOTS + t] = acc;
    }
}

// RDF over molecule COMs (RDFSensor::RDF_Kernel, RDFSensor.cpp:61-72):
// minimum image delta - L*round(delta/L), bin (uint64)(r/dr) clamped.
__device__ __forceinline__ void rdf_pair(const double *ca, const double *cb, Grid g, double max_r, double dr,
                                         long long nbins, double *bins) {
    double q[3];
    for (int d = 0; d < 3; d++) {
        const double delta = dsub(ca[d], cb[d]);
        q[d] = dsub(delta, dmul(g.L[d], (double)(long long)round(ddiv(delta, g.L[d]))));
    }
    const double rr = sqrt(dadd(dadd(dmul(q[0], q[0]), dmul(q[1], q[1])), dmul(q[2], q[2])));
    if (rr > max_r) return;
    unsigned long long b = (unsigned long long)ddiv(rr, dr);
    if (b > (unsigned long long)(nbins - 1)) b = nbins - 1;
    atomicAdd(&bins[b], 1.0);
}

// Cell path (max_r <= cell edge): one warp per home cell.  The molecules of the
// 27 neighbour cells are staged in shared memory as FP32 COMs relative to the
// home cell's centre (formed in FP64, then rounded); for each home molecule
// the lanes test 32 staged molecules at a time against max_r with a 1e-4
// relative margin and queue the hits, and the queued pairs take rdf_pair's
// FP64 arithmetic, so the bin of every pair is the reference's.  The counts go
// to a per-block shared histogram of integers (hist_smem) or straight to bins,
// and the block adds its integer counts to bins at the end: the sums are
// exact, whatever the order.
constexpr int kRdfWarps = 4;
constexpr int kRdfStage = 320;
constexpr int kRdfSmemBins = 2048;   // with the staging arrays, under the 48 KB default

__device__ __forceinline__ long long rdf_pair_bin(const double *ca, const double *cb, Grid g, double max_r, double dr,
                                                  long long nbins) {
    double q[3];
    for (int d = 0; d < 3; d++) {
        const double delta = dsub(ca[d], cb[d]);
        // round(delta / L) is 0 for |delta| < 0.4 L whatever the quotient's rounding; the
        // division runs only where the minimum image can move the pair
        const double img = fabs(delta) < 0.4 * g.L[d] ? 0.0 : (double)(long long)round(ddiv(delta, g.L[d]));
        q[d] = dsub(delta, dmul(g.L[d], img));
    }
    const double rr = sqrt(dadd(dadd(dmul(q[0], q[0]), dmul(q[1], q[1])), dmul(q[2], q[2])));
    if (rr > max_r) return -1;
    unsigned long long b = (unsigned long long)ddiv(rr, dr);
    if (b > (unsigned long long)(nbins - 1)) b = nbins - 1;
    return (long long)b;
}

__global__ void __launch_bounds__(32 * kRdfWarps) k_rdf_cells(Grid g, const double *__restrict__ com,
                                                              const int *__restrict__ cell_mstart,
                                                              const int *__restrict__ cell_mols, double max_r,
                                                              double dr, long long nbins, bool hist_smem,
                                                              double *bins) {
    extern __shared__ unsigned s_hist[];   // nbins counts when hist_smem
    __shared__ float4 s_p[kRdfWarps][kRdfStage];
    __shared__ int2 s_j[kRdfWarps][kRdfStage];   // molecule, neighbour-cell index
    __shared__ double s_sh[kRdfWarps][27][3];
    __shared__ int s_st[kRdfWarps][27], s_pre[kRdfWarps][28];
    __shared__ int s_q[kRdfWarps][64];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (hist_smem)
        for (int b = threadIdx.x; b < nbins; b += blockDim.x) s_hist[b] = 0u;
    __syncthreads();
    const int cell = blockIdx.x * kRdfWarps + w;
    if (cell < g.ncell) {
        unsigned lt;
        asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lt));
        int cx, cy, cz;
        cell_coords(g, cell, cx, cy, cz);
        const double ctr[3] = {cell_centre(g, 0, cx), cell_centre(g, 1, cy), cell_centre(g, 2, cz)};
        int cnt = 0;
        if (lane < 27) {
            const NbCell q = neighbour_cell(g, cx, cy, cz, lane);
            const int s0 = cell_mstart[q.cell];
            cnt = cell_mstart[q.cell + 1] - s0;
            s_st[w][lane] = s0;
            for (int d = 0; d < 3; d++) s_sh[w][lane][d] = q.shift[d];
        }
        int inc = cnt;
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += y;
        }
        if (lane < 27) s_pre[w][lane] = inc - cnt;
        const int total = __shfl_sync(0xffffffffu, inc, 26);
        if (lane == 0) s_pre[w][27] = total;
        __syncwarp();
        const int hs = s_st[w][13], hn = s_pre[w][14] - s_pre[w][13];
        const float pre2 = (float)(max_r * max_r * (1.0 + 1e-4));
        auto rel = [&](int o, int nb) {   // FP32 COM relative to the home centre, through the periodic shift
            const double *c = com + 3 * (size_t)o;
            return make_float4((float)dsub(dadd(c[0], s_sh[w][nb][0]), ctr[0]),
                               (float)dsub(dadd(c[1], s_sh[w][nb][1]), ctr[1]),
                               (float)dsub(dadd(c[2], s_sh[w][nb][2]), ctr[2]), 0.f);
        };
        for (int sb = 0; sb < total; sb += kRdfStage) {
            const int ns = min(kRdfStage, total - sb);
            __syncwarp();
            for (int t = lane; t < ns; t += 32) {
                const int gi = sb + t;
                int a = 0, b = 27;
                while (b - a > 1) {
                    const int mid = (a + b) >> 1;
                    if (s_pre[w][mid] <= gi) a = mid;
                    else b = mid;
                }
                const int o = cell_mols[s_st[w][a] + (gi - s_pre[w][a])];
                s_p[w][t] = rel(o, a);
                s_j[w][t] = make_int2(o, a);
            }
            __syncwarp();
            for (int h = 0; h < hn; h++) {
                const int k = cell_mols[hs + h];
                const float4 hp = rel(k, 13);
                auto count = [&](int c) {
                    if (c < 0) return;
                    const long long b = rdf_pair_bin(com + 3 * (size_t)k, com + 3 * (size_t)s_j[w][c].x, g, max_r, dr,
                                                     nbins);
                    if (b < 0) return;
                    if (hist_smem) atomicAdd(&s_hist[b], 1u);
                    else atomicAdd(&bins[b], 1.0);
                };
                int qn = 0;
                for (int c0 = 0; c0 < ns; c0 += 32) {
                    const int c = c0 + lane;
                    bool hit = false;
                    if (c < ns && s_j[w][c].x != k) {
                        const float4 pj = s_p[w][c];
                        const float dx = hp.x - pj.x, dy = hp.y - pj.y, dz = hp.z - pj.z;
                        hit = dx * dx + dy * dy + dz * dz <= pre2;
                    }
                    const unsigned m = __ballot_sync(0xffffffffu, hit);
                    if (hit) s_q[w][qn + __popc(m & lt)] = c;
                    qn += __popc(m);
                    if (qn >= 32) {
                        __syncwarp();
                        count(s_q[w][lane]);
                        __syncwarp();
                        qn -= 32;
                        if (lane < qn) s_q[w][lane] = s_q[w][32 + lane];
                        __syncwarp();
                    }
                }
                __syncwarp();
                count(lane < qn ? s_q[w][lane] : -1);
                __syncwarp();
            }
        }
    }
    if (hist_smem) {
        __syncthreads();
        for (int b = threadIdx.x; b < nbins; b += blockDim.x)
            if (s_hist[b]) atomicAdd(&bins[b], (double)s_hist[b]);
    }
}

__global__ void k_rdf_all(Grid g, int n_mol, const double *__restrict__ com, double max_r, double dr,
                          long long nbins, double *bins) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n_mol) return;
    for (int o = 0; o < n_mol; o++)
        if (o != k) rdf_pair(com + 3 * k, com + 3 * o, g, max_r, dr, nbins, bins);
}

// Sums the per-block partial rows: one block of 256 threads per slot, a fixed
// thread-to-row mapping, fixed shuffle trees and a fixed order over the
// warps, so the result is deterministic.
constexpr int kSumThreads = 256;
__global__ void __launch_bounds__(kSumThreads) k_sum_partials(int nblocks, const double *__restrict__ partials,
                                                              double *__restrict__ out) {
    __shared__ double s_w[kSumThreads / 32];
    const int slot = blockIdx.x, t = threadIdx.x, lane = t & 31;
    double s = 0.0;
    for (int b = t; b < nblocks; b += kSumThreads) s += partials[(size_t)b * R_NSLOTS + slot];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) s_w[t >> 5] = s;
    __syncthreads();
    if (t == 0) {
        double y = 0.0;
        for (int w = 0; w < kSumThreads / 32; w++) y += s_w[w];
        out[slot] += y;
    }
}

// Tabulated pair force (IBI_ForceFunctor<IBI_Default>::IBI_Force,
// plugins/IBI/IBI_ForceFunctor.cpp:18-37, FunctionPL::evaluateAt,
// plugins/IBI/IBI_Math.h:30-44): for every pair inside the cutoff (no
// same-molecule exclusion) F = table(r), force = (dr / r) * F on the site.
// FP64: the exact separation and cutoff test, r = sqrt(r^2) and the table
// value as the reference forms them (the upper node is the first node >= r,
// by binary search, the node the reference's linear scan finds, and slope[k] =
// (y[k+1] - y[k]) / (x[k+1] - x[k]) is the reference's quotient, computed once
// with the same IEEE operations); dr / r as dr * (1 / r), one division per
// pair instead of three (within an ulp of the reference's quotients; the FP64
// pipe bounds this kernel).  At r == x[0] the reference reads x[-1]; here the
// first segment is used.
__device__ __forceinline__ double table_eval(double x, int n, const double *__restrict__ xs,
                                             const double *__restrict__ ys, const double *__restrict__ slope,
                                             double lo, double hi) {
    if (x > xs[n - 1]) return hi;
    if (x < xs[0]) return lo;
    int a = 0, b = n - 1;           // lower_bound: first index with xs[i] >= x
    while (a < b) {
        const int m = (a + b) >> 1;
        if (x > xs[m]) a = m + 1;
        else b = m;
    }
    const int lb = (a < 1 ? 1 : a) - 1;
    return dadd(ys[lb], dmul(slope[lb], dsub(x, xs[lb])));
}

// One warp per home cell.  The 27-cell neighbourhood is staged in shared
// memory in FP32 home-cell coordinates (cell-local position plus the
// neighbour cell's centre offset); for each home site the lanes test 32
// staged sites at a time against the cutoff with a 1e-4 relative margin (the
// FP32 separation is good to ~1e-7, so the test only drops pairs that are
// clearly outside), queue the hits by ballot, and evaluate the queue 32 pairs
// at a time in FP64 from the FP64 positions and the neighbour cell's periodic
// shift, with the exact cutoff test.  Per home site the lanes' sums are
// reduced in a fixed tree and added to f.
constexpr int kTabWarps = 4;
constexpr int kTabStage = 416;   // staged sites per round (more rounds for a larger neighbourhood)

__global__ void __launch_bounds__(32 * kTabWarps) k_pair_table(
    Grid g, const int *__restrict__ cell_start, const int *__restrict__ slot_site, const double *__restrict__ posd,
    const float4 *__restrict__ pos4, const float *__restrict__ offtab, double rc2, int n,
    const double *__restrict__ xs, const double *__restrict__ ys, const double *__restrict__ slope, double lo,
    double hi, double *__restrict__ f) {
    __shared__ float4 s_p[kTabWarps][kTabStage];
    __shared__ int2 s_j[kTabWarps][kTabStage];   // slot, neighbour-cell index
    __shared__ double s_sh[kTabWarps][27][3];
    __shared__ float s_o[kTabWarps][27][3];
    __shared__ int s_st[kTabWarps][27], s_pre[kTabWarps][28];
    __shared__ int s_q[kTabWarps][64];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int cell = blockIdx.x * kTabWarps + w;
    if (cell >= g.ncell) return;   // warp-uniform; the kernel uses no block barrier
    unsigned lt;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lt));
    int cx, cy, cz;
    cell_coords(g, cell, cx, cy, cz);
    int cnt = 0;
    if (lane < 27) {
        const NbCell q = neighbour_cell(g, cx, cy, cz, lane);
        const int s0 = cell_start[q.cell];
        cnt = cell_start[q.cell + 1] - s0;
        s_st[w][lane] = s0;
        for (int d = 0; d < 3; d++) s_sh[w][lane][d] = q.shift[d];
        s_o[w][lane][0] = offtab[cx * 3 + lane % 3];
        s_o[w][lane][1] = offtab[g.nd[0] * 3 + cy * 3 + (lane / 3) % 3];
        s_o[w][lane][2] = offtab[(g.nd[0] + g.nd[1]) * 3 + cz * 3 + lane / 9];
    }
    int inc = cnt;   // inclusive prefix of the 27 counts
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
    }
    if (lane < 27) s_pre[w][lane] = inc - cnt;
    const int total = __shfl_sync(0xffffffffu, inc, 26);
    if (lane == 0) s_pre[w][27] = total;
    __syncwarp();
    const int hs = s_st[w][13], hn = s_pre[w][14] - s_pre[w][13];   // neighbour 13 is the home cell
    const float pre2 = (float)(rc2 * (1.0 + 1e-4));
    for (int sb = 0; sb < total; sb += kTabStage) {
        const int ns = min(kTabStage, total - sb);
        __syncwarp();
        for (int t = lane; t < ns; t += 32) {
            const int gi = sb + t;
            int a = 0, b = 27;   // the neighbour cell holding staged site gi
            while (b - a > 1) {
                const int mid = (a + b) >> 1;
                if (s_pre[w][mid] <= gi) a = mid;
                else b = mid;
            }
            const int j = s_st[w][a] + (gi - s_pre[w][a]);
            float4 q = pos4[j];
            q.x += s_o[w][a][0];
            q.y += s_o[w][a][1];
            q.z += s_o[w][a][2];
            s_p[w][t] = q;
            s_j[w][t] = make_int2(j, a);
        }
        __syncwarp();
        for (int h = 0; h < hn; h++) {
            const int is = hs + h;
            const float4 hp = pos4[is];
            const double xi = posd[3 * is], yi = posd[3 * is + 1], zi = posd[3 * is + 2];
            double fx = 0.0, fy = 0.0, fz = 0.0;
            auto eval = [&](int c) {
                if (c < 0) return;
                const int2 jn = s_j[w][c];
                const double *pj = posd + 3 * (size_t)jn.x;
                const double dx = dsub(xi, dadd(pj[0], s_sh[w][jn.y][0]));
                const double dy = dsub(yi, dadd(pj[1], s_sh[w][jn.y][1]));
                const double dz = dsub(zi, dadd(pj[2], s_sh[w][jn.y][2]));
                const double r2 = dadd(dadd(dmul(dx, dx), dmul(dy, dy)), dmul(dz, dz));
                if (r2 > rc2) return;
                const double r = __dsqrt_rn(r2);
                const double F = table_eval(r, n, xs, ys, slope, lo, hi);
                const double ir = ddiv(1.0, r);
                fx = dadd(fx, dmul(dmul(dx, ir), F));
                fy = dadd(fy, dmul(dmul(dy, ir), F));
                fz = dadd(fz, dmul(dmul(dz, ir), F));
            };
            int qn = 0;
            for (int c0 = 0; c0 < ns; c0 += 32) {
                const int c = c0 + lane;
                bool hit = false;
                if (c < ns && s_j[w][c].x != is) {
                    const float4 pj = s_p[w][c];
                    const float dx = hp.x - pj.x, dy = hp.y - pj.y, dz = hp.z - pj.z;
                    hit = dx * dx + dy * dy + dz * dz <= pre2;
                }
                const unsigned m = __ballot_sync(0xffffffffu, hit);
                if (hit) s_q[w][qn + __popc(m & lt)] = c;
                qn += __popc(m);
                if (qn >= 32) {   // a full batch: one queued pair per lane
                    __syncwarp();
                    eval(s_q[w][lane]);
                    __syncwarp();
                    qn -= 32;
                    if (lane < qn) s_q[w][lane] = s_q[w][32 + lane];
                    __syncwarp();
                }
            }
            __syncwarp();
            eval(lane < qn ? s_q[w][lane] : -1);
            for (int o = 16; o > 0; o >>= 1) {
                fx = dadd(fx, __shfl_xor_sync(0xffffffffu, fx, o));
                fy = dadd(fy, __shfl_xor_sync(0xffffffffu, fy, o));
                fz = dadd(fz, __shfl_xor_sync(0xffffffffu, fz, o));
            }
            if (lane == 0) {
                const int site = slot_site[is];
                f[3 * site] = dadd(f[3 * site], fx);
                f[3 * site + 1] = dadd(f[3 * site + 1], fy);
                f[3 * site + 2] = dadd(f[3 * site + 2], fz);
            }
            __syncwarp();
        }
    }
}

// VelocityScaling (VelocityScaling.cpp:12-25): v *= beta; beta from the
// caller, or (acc != nullptr) sqrt(T_target / T) with T from the summed
// kinetic slots as TemperatureSensor computes it.  A non-finite T (an
// overflowed force upstream) leaves v unscaled and raises E_NONFINITE, which
// the host reads after the step.
__global__ void k_velocity_scale(int n, double *__restrict__ v, const double *__restrict__ acc, double t_target,
                                 double beta_in, int *__restrict__ err) {
    __shared__ double s_beta;
    if (threadIdx.x == 0) {
        double beta = beta_in;
        if (acc) {
            const double t = sci_temperature(acc[R_MV2], acc[R_NBOX]);
            if (!isfinite(t)) {
                beta = 1.0;
                if (blockIdx.x == 0 && err) atomicOr(&err[E_NONFINITE], 1);
            } else {
                beta = t > 0.0 ? __dsqrt_rn(__ddiv_rn(t_target, t)) : 1.0;
            }
        }
        s_beta = beta;
    }
    __syncthreads();
    const double beta = s_beta;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < 3 * n; k += gridDim.x * blockDim.x)
        v[k] = __dmul_rn(v[k], beta);
}

// ===========================================================================
// launchers
// ===========================================================================
static inline int nblk(long long n, int b) { return (int)((n + b - 1) / b); }

BinArgs bin_args(const Engine &e) {
    return BinArgs{e.g, (int)e.n_mol, e.mol_off, e.r, e.m, e.com, e.mol_cell, e.mol_rank, e.cell_count, e.cell_mcount,
                   e.verlet ? e.bias : nullptr, e.verlet ? e.rebuild : nullptr, e.exact_com, e.fused_drift ? 1 : 0};
}
ScanArgs scan_args(const Engine &e) {
    return ScanArgs{e.g.ncell, e.cell_count, e.cell_start, e.cell_mcount, e.cell_mstart,
                    e.verlet ? e.rebuild : nullptr, e.vb_next};
}
ScatterArgs scatter_args(const Engine &e) {
    return ScatterArgs{(int)e.n_mol, e.mol_cell, e.mol_rank, e.cell_mstart, e.cell_mols,
                       e.verlet ? e.rebuild : nullptr};
}
SortArgs sort_args(const Engine &e) {
    return SortArgs{e.g, e.mol_off, e.cell_mstart, e.cell_start, e.cell_mols, e.r, e.eps, e.sig, e.key,
                    e.slot_site, e.site_slot, e.pos4, e.skey, e.seps, e.posd, e.seps_d, e.sig_d,
                    e.verlet ? e.bias : nullptr, e.verlet ? e.ref4 : nullptr, e.verlet ? e.slot_cell : nullptr,
                    e.verlet ? e.zkey : nullptr, e.verlet ? e.rebuild : nullptr};
}
Step0Args step0_args(const Engine &e) {
    const float hs = (float)(0.5 * e.cfg.skin);
    return Step0Args{(int)e.n, e.r, e.v, e.f, e.hdtm, e.cfg.delta_t, e.g, e.bias, e.ref4, hs * hs, e.rebuild, e.com,
                     e.site_slot, e.pos4, e.hin_r ? e.hin_r : e.r, e.hin_v ? e.hin_v : e.v, e.hout_r};
}
FlushArgs flush_args(const Engine &e, double scale_fix, const float4 *own) {
    return FlushArgs{(int)e.n, e.site_slot, e.atm_acc, e.f, scale_fix, e.v, e.hdtm, e.err,
                     e.verlet ? e.rebuild : nullptr, e.hout_f, e.hout_v, own};
}

void launch_container(Engine &e, cudaStream_t st) {
    const Grid &g = e.g;
    // without a Verlet list the rebuild flag is null: the kernels rebuild unconditionally
    // the per-cell counts are zero here: zeroed at allocation, and by the scan
    // of every binning after reading them
    // grid-stride kernels on a resident grid: steps without a rebuild launch few blocks
    const int res = e.num_sms * 8;
    launch_pdl(k_com_wrap_bin, std::min(nblk(e.n_mol, 256), res), 256, 0, st, bin_args(e));
    launch_pdl(k_scan2, 1, 1024, 0, st, scan_args(e));
    launch_pdl(k_scatter_mol, std::min(nblk(e.n_mol, 256), res), 256, 0, st, scatter_args(e));
    launch_pdl(k_cell_sort, std::min(nblk(g.ncell, kWarpsPerBlock), res), kBlock, 0, st, sort_args(e));
    if (e.verlet) {
        if (!e.fused_drift)
            k_refresh<<<nblk(e.n, 256), 256, 0, st>>>((int)e.n, e.slot_site, e.r, e.bias, e.pos4, e.rebuild);
        launch_vlist_build(e, st);
    }
}

PairParams pair_params(Engine &e) {
    PairParams p;
    p.g = e.g;
    p.cell_start = e.cell_start;
    p.slot_site = e.slot_site;
    p.pos4 = e.pos4;
    p.posd = e.posd;
    p.skey = e.skey;
    p.seps = e.seps;
    p.seps_d = e.seps_d;
    p.sig_d = e.sig_d;
    p.f = e.f;
    p.counts = e.counts;
    p.nl = e.nl;
    p.nl_count = e.nl_count;
    p.nl_cap = e.nl_cap;
    p.err = e.err;
    p.partials = e.partials;
    p.lj_hist = nullptr;
    p.lj_bins = e.cfg.lj_bins;
    p.max_sigma = e.cfg.max_sigma;
    p.rc2 = e.cfg.cutoff * e.cfg.cutoff;
    p.rc3sq = e.cfg.cutoff_3b * e.cfg.cutoff_3b;
    const bool atm = (e.cfg.terms & KOMD_TERM_ATM) != 0;
    const bool lj = (e.cfg.terms & KOMD_TERM_LJ) != 0;
    p.scan2 = 0.0;
    if (lj) p.scan2 = p.rc2;
    if (atm && p.rc3sq > p.scan2) p.scan2 = p.rc3sq;
    p.stiffness = e.cfg.stiffness;
    p.use_lj = lj ? 1 : 0;
    p.lj_fscale = e.lj_fscale;
    p.lj_fscalef = (float)e.lj_fscale;
    p.virial_compat = e.cfg.virial_mode == KOMD_VIRIAL_COMPAT;
    p.offtab = e.offtab;
    p.rebuild = e.rebuild;
    p.vl = e.vl;
    p.vl_count = e.vl_count;
    p.vl_cap = e.vl_cap;
    const double rl = std::max(lj ? e.cfg.cutoff : 0.0, atm ? e.cfg.cutoff_3b : 0.0) + e.cfg.skin;
    p.rl2 = rl * rl;
    p.slot_cell = e.slot_cell;
    p.zkey = e.zkey;
    p.vb_next = e.vb_next;
    p.nboff = e.nboff;
    p.rebuild_count = e.rebuild_count;
    p.eps0 = e.eps0;
    p.sig0 = e.sig0;
    sw_params(e.cfg.cutoff, e.cfg.switch_width, p.sw, p.sw_rc2, p.sw_iw);
    p.fown = nullptr;   // set by the half-list pass's launchers (half_own)
    return p;
}

template <typename Real, bool M, bool E, bool F>
static void pair_dispatch_c(PairParams &p, int grid, cudaStream_t st) {
    k_pair<Real, M, E, F, false><<<grid, kBlock, 0, st>>>(p);
}

template <typename Real>
static void pair_dispatch(PairParams &p, bool measure, bool emit, bool fene, int grid, cudaStream_t st) {
    const int code = (measure ? 4 : 0) | (emit ? 2 : 0) | (fene ? 1 : 0);
    switch (code) {
        case 0: pair_dispatch_c<Real, false, false, false>(p, grid, st); break;
        case 1: pair_dispatch_c<Real, false, false, true>(p, grid, st); break;
        case 2: pair_dispatch_c<Real, false, true, false>(p, grid, st); break;
        case 3: pair_dispatch_c<Real, false, true, true>(p, grid, st); break;
        case 4: pair_dispatch_c<Real, true, false, false>(p, grid, st); break;
        case 5: pair_dispatch_c<Real, true, false, true>(p, grid, st); break;
        case 6: pair_dispatch_c<Real, true, true, false>(p, grid, st); break;
        default: pair_dispatch_c<Real, true, true, true>(p, grid, st); break;
    }
}

int atm_grid(const Engine &e) { return nblk(e.n, kWarpsPerBlock); }

// The FP32 force path runs the tiled kernel (pair_tile.cu, one CTA per cell);
// FP64 mode, FENE and the LJ sensor histograms use the warp-per-cell kernel
// above.  Returns the number of blocks whose partial sums were written.
int launch_pair(Engine &e, cudaStream_t st, bool measure, double *lj_hist) {
    PairParams p = pair_params(e);
    p.lj_hist = lj_hist;
    const bool emit = (e.cfg.terms & KOMD_TERM_ATM) != 0;
    const bool fene = (e.cfg.terms & KOMD_TERM_FENE) != 0;
    if (e.verlet && !lj_hist) return launch_lj_vlist(e, p, measure, emit, st);
    if (e.cfg.precision == KOMD_FP32 && !fene && !lj_hist) {
        launch_pair_tile(p, e.g.ncell, measure, emit, st);
        return e.g.ncell;
    }
    const int grid = nblk(e.g.ncell, kWarpsPerBlock);
    if (e.cfg.precision == KOMD_FP64) pair_dispatch<double>(p, measure, emit, fene, grid, st);
    else pair_dispatch<float>(p, measure, emit, fene, grid, st);
    return grid;
}

void launch_counts(Engine &e, cudaStream_t st) {
    PairParams p = pair_params(e);
    p.use_lj = 1;
    p.scan2 = p.rc2;
    k_pair<double, false, false, false, true><<<nblk(e.g.ncell, kWarpsPerBlock), kBlock, 0, st>>>(p);
}

void launch_bonded(Engine &e, cudaStream_t st, bool measure, double *acc) {
    if (e.n_bonds > 0)
        k_bonds<<<nblk(e.n_bonds, 256), 256, 0, st>>>((int)e.n_bonds, e.bonds, e.r, e.f, (float)e.cfg.bond_k,
                                                        (float)e.cfg.bond_r0, acc, measure ? 1 : 0);
    if (e.n_angles > 0)
        k_angles<<<nblk(e.n_angles, 256), 256, 0, st>>>((int)e.n_angles, e.angles, e.r, e.f, (float)e.cfg.angle_k,
                                                          (float)e.cfg.angle_theta0, acc, measure ? 1 : 0);
}

void launch_limit(Engine &e, cudaStream_t st) {
    k_limit<<<nblk(e.n, 256), 256, 0, st>>>((int)e.n, e.eps, e.sig, e.cfg.limit, e.f);
}

size_t atm_smem(const Engine &e) {
    const size_t per = e.cfg.precision == KOMD_FP64 ? (sizeof(AtmEntryD) + 2 * sizeof(double))
                                                    : (2 * sizeof(float4));
    return (size_t)kWarpsPerBlock * e.nl_cap * per;
}

// stage vertex i's neighbours above i (ballot compaction); returns their count
__device__ __forceinline__ int atm_stage(const AtmParams &p, int i, float4 *se, float4 *sq, int lane, unsigned lt) {
    const int ni = min(p.nl_count[i], p.nl_cap);
    int m = 0;
    for (int k0 = 0; k0 < ni; k0 += 32) {
        const int k = k0 + lane;
        float4 e = make_float4(0.f, 0.f, 0.f, 0.f);
        bool up = false;
        if (k < ni) {
            e = p.nl[(size_t)i * p.nl_cap + k];
            up = (__float_as_int(e.w) >> 6) > i;
        }
        const unsigned bm = __ballot_sync(0xffffffffu, up);
        if (up) {
            const int pos = m + __popc(bm & lt);
            const float A = e.x * e.x + e.y * e.y + e.z * e.z;
            se[pos] = e;
            sq[pos] = atm_stage_q(A);
        }
        m += __popc(bm);
    }
    return m;
}

// one warp per vertex: stage its neighbours above it, then the sweep
__global__ void __launch_bounds__(kBlock) k_atm_s(AtmParams p) {
    extern __shared__ float4 s_dyn[];
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int cap = p.nl_cap;
    float4 *se = s_dyn + wib * 2 * cap, *sq = se + cap;
    const int i = blockIdx.x * kWarpsPerBlock + wib;
    if (i >= p.n) return;
    unsigned lt;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lt));
    const int m = atm_stage(p, i, se, sq, lane, lt);
    __syncwarp();
    atm_vertex(p, i, se, sq, m, lane, (float)p.rc2);
}

// the same flush fused with Integrator::integrate1 of the step (ATM is the
// last force term): f[site] += ..., then v[site] += f[site] * dt/(2m) with
// k_step1's operations, its non-finite check and the rebuild-flag reset
__device__ __forceinline__ void flush_step1_body(const FlushArgs &a, int bid) {
    __shared__ double s_f[3 * kIoBlock], s_v[3 * kIoBlock];
    const int n = a.n;
    const int *__restrict__ site_slot = a.site_slot;
    unsigned long long *__restrict__ acc = a.acc;
    double *__restrict__ f = a.f, *__restrict__ v = a.v;
    const double scale_fix = a.scale_fix;
    const double *__restrict__ hdtm = a.hdtm;
    int *__restrict__ err = a.err, *__restrict__ rebuild = a.rebuild;
    double *f_out = a.f_out, *v_out = a.v_out;
    const int t = threadIdx.x;
    const int base = bid * blockDim.x, site = base + t;
    const int cnt = min((int)blockDim.x, n - base);
    if (rebuild && site == 0) *rebuild = 0;   // every consumer of this step's flag has run
    if (site < n) {
        // one thread per site (f, v, dt/2m coalesced, the accumulators
        // gathered); every load first, then the arithmetic
        const int slot = site_slot[site];
        long long q[3];
        double fo[3], vo[3];
        for (int d = 0; d < 3; d++) q[d] = (long long)acc[3 * slot + d];
        if (a.fown) {   // the half-list pass's FP32 force, widened exactly
            const float4 o = a.fown[slot];
            fo[0] = (double)o.x;
            fo[1] = (double)o.y;
            fo[2] = (double)o.z;
        } else {
            for (int d = 0; d < 3; d++) fo[d] = f[3 * site + d];
        }
        for (int d = 0; d < 3; d++) vo[d] = v[3 * site + d];
        const double c = hdtm[site];
        bool bad = false;
        for (int d = 0; d < 3; d++) {
            acc[3 * slot + d] = 0ull;
            // scale_fix = scale / 2^32 exactly: the same product as scale * (q / 2^32)
            const double fd = fo[d] + scale_fix * (double)q[d];
            f[3 * site + d] = fd;
            const double vv = dadd(vo[d], dmul(fd, c));
            v[3 * site + d] = vv;
            bad |= !isfinite(vv);
            s_f[3 * t + d] = fd;
            s_v[3 * t + d] = vv;
        }
        if (bad) atomicOr(&err[E_NONFINITE], 1);
    }
    if (f_out || v_out) {   // the caller's host buffers, in whole lines
        __syncthreads();
        if (f_out) rows_out(s_f, f_out, base, cnt);
        if (v_out) rows_out(s_v, v_out, base, cnt);
    }
}
__global__ void __launch_bounds__(kIoBlock) k_atm_flush_step1(FlushArgs a) {
    pdl_wait();
    flush_step1_body(a, blockIdx.x);
}

// f[site] += 2 sign nu g (fixed point -> FP64) and the accumulators back to 0
__global__ void k_atm_flush(int n, const int *__restrict__ slot_site, unsigned long long *__restrict__ acc,
                            double *__restrict__ f, double scale_fix, const float4 *__restrict__ own) {
    const int slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= n) return;
    const int site = slot_site[slot];
    long long q[3];
    double fo[3];
    for (int d = 0; d < 3; d++) q[d] = (long long)acc[3 * slot + d];
    if (own) {   // the half-list pass's FP32 force, widened exactly
        const float4 o = own[slot];
        fo[0] = (double)o.x;
        fo[1] = (double)o.y;
        fo[2] = (double)o.z;
    } else {
        for (int d = 0; d < 3; d++) fo[d] = f[3 * site + d];
    }
    for (int d = 0; d < 3; d++) {
        acc[3 * slot + d] = 0ull;
        f[3 * site + d] = fo[d] + scale_fix * (double)q[d];
    }
}

template <typename Real>
static void atm_dispatch(AtmParams &p, bool measure, bool compat, int grid, size_t sm, cudaStream_t st) {
    if (measure) {
        if (compat) k_atm<Real, true, true><<<grid, kBlock, sm, st>>>(p);
        else k_atm<Real, true, false><<<grid, kBlock, sm, st>>>(p);
    } else {
        if (compat) k_atm<Real, false, true><<<grid, kBlock, sm, st>>>(p);
        else k_atm<Real, false, false><<<grid, kBlock, sm, st>>>(p);
    }
}

template <>
void atm_dispatch<float>(AtmParams &p, bool measure, bool compat, int grid, size_t sm, cudaStream_t st) {
    if (measure) {
        if (compat) k_atm_q<true, true><<<grid, kBlock, sm, st>>>(p);
        else k_atm_q<true, false><<<grid, kBlock, sm, st>>>(p);
    } else {
        if (compat) k_atm_q<false, true><<<grid, kBlock, sm, st>>>(p);
        else k_atm_q<false, false><<<grid, kBlock, sm, st>>>(p);
    }
}

AtmParams atm_params(const Engine &e) {
    AtmParams p;
    p.n = (int)e.n;
    p.slot_site = e.slot_site;
    p.nl = e.nl;
    p.nl_count = e.nl_count;
    p.nl_cap = e.nl_cap;
    p.f = e.f;
    p.partials = e.partials;
    p.nu = e.cfg.nu;
    p.rc2 = e.cfg.cutoff_3b * e.cfg.cutoff_3b;
    p.sign = e.cfg.atm_sign == KOMD_ATM_SIGN_REFERENCE ? 1.0 : -1.0;
    p.virial_compat = e.cfg.virial_mode == KOMD_VIRIAL_COMPAT;
    p.atm_direct = e.cfg.atm_direct;
    p.e_site = e.atm_esite;
    p.acc = e.atm_acc;
    sw_params(e.cfg.cutoff_3b, e.cfg.switch_width, p.sw, p.sw_rc2, p.sw_iw);
    return p;
}

// the fixed-point sums of the once-per-triplet sweep into f (and, with_step1,
// integrate1 of the step); returns with_step1
bool launch_atm_flush(Engine &e, cudaStream_t st, bool with_step1, bool force_units) {
    const double sign = e.cfg.atm_sign == KOMD_ATM_SIGN_REFERENCE ? 1.0 : -1.0;
    const double scale_fix = force_units ? 1.0 / kAtmFix : 2.0 * sign * e.cfg.nu / kAtmFix;
    const float4 *own = force_units ? half_own(e) : nullptr;   // force_units: the half-list pass ran
    if (with_step1) {
        launch_pdl(k_atm_flush_step1, nblk(e.n, kIoBlock), kIoBlock, 0, st, flush_args(e, scale_fix, own));
        return true;
    }
    k_atm_flush<<<nblk(e.n, 256), 256, 0, st>>>((int)e.n, e.slot_site, e.atm_acc, e.f, scale_fix, own);
    return false;
}

bool launch_atm(Engine &e, cudaStream_t st, bool measure, bool with_step1) {
    AtmParams p = atm_params(e);
    const bool compat = e.cfg.atm_enum == KOMD_ATM_ENUM_COMPAT;
    if (!measure && !compat && e.cfg.precision == KOMD_FP32 && e.atm_acc) {
        // every triplet once (lowest slot), fixed-point scatter, then the flush into f
        k_atm_s<<<atm_grid(e), kBlock, atm_smem(e), st>>>(p);
        return launch_atm_flush(e, st, with_step1, false);
    }
    if (e.cfg.precision == KOMD_FP64) atm_dispatch<double>(p, measure, compat, atm_grid(e), atm_smem(e), st);
    else atm_dispatch<float>(p, measure, compat, atm_grid(e), atm_smem(e), st);
    return false;
}

void launch_step0(Engine &e, cudaStream_t st, bool in_step) {
    const float hs = (float)(0.5 * e.cfg.skin);
    if (in_step && e.fused_drift) {
        k_step0_fused<<<nblk(e.n, kIoBlock), kIoBlock, 0, st>>>(step0_args(e));
        return;
    }
    k_step0<<<nblk(e.n, 256), 256, 0, st>>>((int)e.n, e.r, e.v, e.f, e.hdtm, e.cfg.delta_t, e.g,
                                              e.verlet ? e.bias : nullptr, e.verlet ? e.ref4 : nullptr, hs * hs,
                                              e.rebuild);
}

void launch_step1(Engine &e, cudaStream_t st) {
    k_step1<<<nblk(e.n, 256), 256, 0, st>>>((int)e.n, e.v, e.f, e.hdtm, e.err,
                                              e.verlet ? e.rebuild : nullptr);
}

int kinetic_grid(const Engine &e) { return std::min(nblk(e.n, kBlock), e.num_sms * 2); }

void launch_pair_table(Engine &e, cudaStream_t st) {
    if (!e.tab_x || !e.tab_s || e.tab_n < 2) return;
    k_pair_table<<<nblk(e.g.ncell, kTabWarps), 32 * kTabWarps, 0, st>>>(
        e.g, e.cell_start, e.slot_site, e.posd, e.pos4, e.offtab, e.cfg.cutoff * e.cfg.cutoff, e.tab_n, e.tab_x,
        e.tab_y, e.tab_s, e.tab_lo, e.tab_hi, e.f);
}

void launch_velocity_scale(Engine &e, cudaStream_t st, const double *acc, double beta) {
    const int blocks = std::min(nblk(3 * e.n, 256), e.num_sms * 8);
    k_velocity_scale<<<blocks, 256, 0, st>>>((int)e.n, e.v, acc, e.cfg.temperature_target, beta, e.err);
}

void launch_kinetic(Engine &e, cudaStream_t st, int n_terms) {
    if (n_terms > 0) k_kinetic<true><<<kinetic_grid(e), kBlock, 0, st>>>(e.g, (int)e.n, n_terms, e.r, e.v, e.m, e.partials);
    else k_kinetic<false><<<kinetic_grid(e), kBlock, 0, st>>>(e.g, (int)e.n, 0, e.r, e.v, e.m, e.partials);
}

void launch_sum_partials(cudaStream_t st, int nblocks, const double *partials, double *out) {
    k_sum_partials<<<R_NSLOTS, kSumThreads, 0, st>>>(nblocks, partials, out);
}

void launch_rdf(Engine &e, cudaStream_t st, double *bins, bool cells) {
    launch_rdf_bins(e, st, bins, cells, e.cfg.rdf_max, e.cfg.rdf_dr, e.rdf_bins);
}

void launch_rdf_bins(Engine &e, cudaStream_t st, double *bins, bool cells, double max_r, double dr, int64_t nbins) {
    if (cells) {
        const bool hist_smem = nbins <= kRdfSmemBins;
        k_rdf_cells<<<nblk(e.g.ncell, kRdfWarps), 32 * kRdfWarps, hist_smem ? sizeof(unsigned) * nbins : 0, st>>>(
            e.g, e.com, e.cell_mstart, e.cell_mols, max_r, dr, nbins, hist_smem, bins);
    }
    else
        k_rdf_all<<<nblk(e.n_mol, 128), 128, 0, st>>>(e.g, (int)e.n_mol, e.com, max_r, dr, nbins, bins);
}

void set_kernel_attributes(Engine &e) {
    const int sm = (int)atm_smem(e);
    if (sm > 48 * 1024) cudaFuncSetAttribute(k_atm_s, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    if (sm > 48 * 1024) {
        cudaFuncSetAttribute(k_atm_q<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
        cudaFuncSetAttribute(k_atm_q<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
        cudaFuncSetAttribute(k_atm_q<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
        cudaFuncSetAttribute(k_atm_q<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
        cudaFuncSetAttribute(k_atm<double, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
        cudaFuncSetAttribute(k_atm<double, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
        cudaFuncSetAttribute(k_atm<double, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
        cudaFuncSetAttribute(k_atm<double, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    }
}

// ---- packed replicas (kernels.cuh): the container, drift and flush stages of
// every replica in one launch each
__device__ __forceinline__ int packed_rep(const int *__restrict__ start, int nrep, int b) {
    int lo = 0, hi = nrep;   // start[0] = 0 <= b < start[nrep]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (start[mid] <= b) lo = mid;
        else hi = mid;
    }
    return lo;
}
// the packed per-site stages at 32 registers (eight blocks per SM): the
// groups' stages share the SMs, and the force pass of another group needs
// the register file (6.43 against 6.46 ms per step for 512 replicas)
__global__ void __launch_bounds__(kIoBlock, 8) k_step0_fused_p(const Step0Args *a, const int *start, int nrep) {
    const int r = packed_rep(start, nrep, blockIdx.x);
    step0_fused_body(a[r], blockIdx.x - start[r]);
}
__global__ void k_com_wrap_bin_p(const BinArgs *a, const int *start, int nrep) {
    const int r = packed_rep(start, nrep, blockIdx.x);
    com_wrap_bin_body(a[r], blockIdx.x - start[r], start[r + 1] - start[r]);
}
__global__ void __launch_bounds__(1024) k_scan2_p(const ScanArgs *a) { scan2_body(a[blockIdx.x]); }
__global__ void k_scatter_mol_p(const ScatterArgs *a, const int *start, int nrep) {
    const int r = packed_rep(start, nrep, blockIdx.x);
    scatter_mol_body(a[r], blockIdx.x - start[r], start[r + 1] - start[r]);
}
__global__ void __launch_bounds__(kBlock) k_cell_sort_p(const SortArgs *a, const int *start, int nrep) {
    const int r = packed_rep(start, nrep, blockIdx.x);
    cell_sort_body(a[r], blockIdx.x - start[r], start[r + 1] - start[r]);
}
__global__ void __launch_bounds__(kIoBlock, 8) k_atm_flush_step1_p(const FlushArgs *a, const int *start, int nrep) {
    const int r = packed_rep(start, nrep, blockIdx.x);
    flush_step1_body(a[r], blockIdx.x - start[r]);
}

// blocks per replica of the container stages: on a step without a rebuild
// they exit at once; on a rebuild step a replica's blocks do its whole
// binning, so too few of them make a long tail for the launch
int packed_blocks_container(const Engine &e) { return std::max(1, std::min(nblk(e.n_mol, 256), 16)); }

// one step of every replica: the stages of enqueue_step on the Verlet path
// with the fused drift and the half-list pass, each stage one launch
void launch_packed_step(const PackedStep &pk, cudaStream_t st) {
    const int nr = pk.nrep;
    k_step0_fused_p<<<pk.step0.blocks, kIoBlock, 0, st>>>((const Step0Args *)pk.step0.args, pk.step0.start, nr);
    k_com_wrap_bin_p<<<pk.bin.blocks, 256, 0, st>>>((const BinArgs *)pk.bin.args, pk.bin.start, nr);
    k_scan2_p<<<nr, 1024, 0, st>>>((const ScanArgs *)pk.scan.args);
    k_scatter_mol_p<<<pk.scatter.blocks, 256, 0, st>>>((const ScatterArgs *)pk.scatter.args, pk.scatter.start, nr);
    k_cell_sort_p<<<pk.sort.blocks, kBlock, 0, st>>>((const SortArgs *)pk.sort.args, pk.sort.start, nr);
    launch_packed_pair_stages(pk, st, true);
    launch_packed_pair_stages(pk, st, false);
    k_atm_flush_step1_p<<<pk.flush.blocks, kIoBlock, 0, st>>>((const FlushArgs *)pk.flush.args, pk.flush.start, nr);
}


}  // namespace komd
