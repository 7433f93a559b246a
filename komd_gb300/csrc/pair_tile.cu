// pair_tile.cu -- the FP32 pair kernel of the hot path: LJ 12-6 forces
// (LJ12_6.cpp:15-43), energy and virial, and the ATM neighbour list inside
// cutoff_3b, for one home cell per CTA.
//
//   1. threads 0..26 resolve the 27 neighbour cells (periodic wrap) and their
//      home-relative offsets from a per-dimension FP32 table computed once in
//      FP64 on the host, so no FP64 instruction runs in this kernel;
//   2. the neighbourhood's sites are staged in shared memory in home-cell
//      coordinates (float4 position + slot, key, cell code, sqrt(eps));
//   3. every warp owns a subset of home sites; for a home site the 32 lanes
//      test 32 staged candidates at a time and ballot-compact the hits into a
//      per-warp queue, so the force arithmetic always runs on full warps;
//   4. each dequeued pair adds its LJ force to the home site's shared-memory
//      accumulator and, inside cutoff_3b, appends (r_i - r_j, code) to the
//      home site's ATM list in queue order (deterministic list order).
// Full shell: each site's force is summed by its own CTA, no global atomics.
//
// The Verlet path (skin > 0) has its own kernels here: the list build
// (k_vlist_build, rebuild steps only), the LJ pass over each site's list row
// (k_lj_vlist) and the LJ pass that sweeps each site's ATM triplets from
// shared memory (k_lj_atm).
#include "engine.cuh"
#include "kernels.cuh"
#include "atm_device.cuh"

namespace komd {

constexpr int kTileWarps = 4;
constexpr int kTileThreads = 32 * kTileWarps;
constexpr int kStage = 640;   // staged neighbour sites per round (more rounds if a neighbourhood is larger)
constexpr int kHome = 64;     // home sites per round
constexpr int kQ = 64;        // per-warp hit queue

__device__ __forceinline__ float rcp_approx(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// neighbour nb (dx fastest) of domain cell (cx, cy, cz), wrapped; integer only
__device__ __forceinline__ int nb_cell(const Grid &g, int cx, int cy, int cz, int nb, int &kx, int &ky, int &kz,
                                       bool &crosses) {
    kx = cx + nb % 3 - 1;
    ky = cy + (nb / 3) % 3 - 1;
    kz = cz + nb / 9 - 1;
    crosses = false;
    if (kx < 0) { kx += g.nd[0]; crosses = true; } else if (kx >= g.nd[0]) { kx -= g.nd[0]; crosses = true; }
    if (ky < 0) { ky += g.nd[1]; crosses = true; } else if (ky >= g.nd[1]) { ky -= g.nd[1]; crosses = true; }
    if (kz < 0) { kz += g.nd[2]; crosses = true; } else if (kz >= g.nd[2]) { kz -= g.nd[2]; crosses = true; }
    return kx + g.nd[0] * (ky + g.nd[1] * kz);
}

template <bool MEASURE, bool EMIT>
__global__ void __launch_bounds__(kTileThreads) k_pair_tile(PairParams p) {
    __shared__ float4 s_pos[kStage];
    __shared__ int4 s_aux[kStage];        // slot, key, code (nb | crosses << 5), sqrt(eps) bits
    __shared__ float4 s_hpos[kHome];
    __shared__ int2 s_haux[kHome];        // key, sqrt(eps) bits
    __shared__ float s_f[kHome * 3];
    __shared__ int s_cnt[kHome];
    __shared__ unsigned s_q[kTileWarps][kQ];
    __shared__ int s_nbs[27], s_nbn[27], s_nbpre[28], s_nbc[27];
    __shared__ float s_nbo[27][3];
    __shared__ double s_part[kTileWarps][8];

    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int cell = blockIdx.x;
    int cx, cy, cz;
    cell_coords(p.g, cell, cx, cy, cz);
    if (tid < 27) {
        int kx, ky, kz;
        bool cr;
        const int c = nb_cell(p.g, cx, cy, cz, tid, kx, ky, kz, cr);
        const int s0 = p.cell_start[c];
        s_nbs[tid] = s0;
        s_nbn[tid] = p.cell_start[c + 1] - s0;
        s_nbc[tid] = cr ? 32 : 0;
        // home-relative offset of the neighbour cell's centre (FP32 table, per dimension)
        s_nbo[tid][0] = p.offtab[cx * 3 + tid % 3];
        s_nbo[tid][1] = p.offtab[p.g.nd[0] * 3 + cy * 3 + (tid / 3) % 3];
        s_nbo[tid][2] = p.offtab[(p.g.nd[0] + p.g.nd[1]) * 3 + cz * 3 + tid / 9];
    }
    __syncthreads();
    if (tid == 0) {
        int acc = 0;
        for (int k = 0; k < 27; k++) { s_nbpre[k] = acc; acc += s_nbn[k]; }
        s_nbpre[27] = acc;
    }
    __syncthreads();
    const int Nn = s_nbpre[27];
    const int hs = s_nbs[13], hn = s_nbn[13];
    const float rc2 = (float)p.rc2, rc3sq = (float)p.rc3sq, scan2 = (float)p.scan2;
    float4 *nl = p.nl;
    float m_u = 0.f, m_pairs = 0.f, m_w[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};   // per-lane partials (MEASURE)

    for (int hb = 0; hb < hn; hb += kHome) {
        const int hc = min(kHome, hn - hb);
        for (int t = tid; t < hc; t += kTileThreads) {
            s_hpos[t] = p.pos4[hs + hb + t];
            s_haux[t] = make_int2(p.skey[hs + hb + t], __float_as_int(p.seps[hs + hb + t]));
            s_f[3 * t] = 0.f; s_f[3 * t + 1] = 0.f; s_f[3 * t + 2] = 0.f;
            s_cnt[t] = 0;
        }
        const int self_base = s_nbpre[13] + hb;
        for (int sb = 0; sb < Nn; sb += kStage) {
            const int ns = min(kStage, Nn - sb);
            __syncthreads();
            for (int t = tid; t < ns; t += kTileThreads) {
                const int gi = sb + t;
                int lo = 0, hi = 27;            // largest nb with s_nbpre[nb] <= gi
                while (hi - lo > 1) {
                    const int mid = (lo + hi) >> 1;
                    if (s_nbpre[mid] <= gi) lo = mid; else hi = mid;
                }
                const int nb = lo;
                const int j = s_nbs[nb] + (gi - s_nbpre[nb]);
                float4 q = p.pos4[j];
                q.x += s_nbo[nb][0];
                q.y += s_nbo[nb][1];
                q.z += s_nbo[nb][2];
                s_pos[t] = q;
                s_aux[t] = make_int4(j, p.skey[j], nb | s_nbc[nb], __float_as_int(p.seps[j]));
            }
            __syncthreads();

            // Process one queued pair per lane (valid = lane holds an entry).
            // Entries of one home site occupy contiguous lanes (the queue is
            // filled site by site), and a site belongs to exactly one warp:
            // its force is reduced over its lane group and added by the
            // group's first lane with a plain read-modify-write.
            auto process = [&](unsigned e, bool valid) {
                const int i = valid ? (int)(e >> 16) : 0;
                const int j = valid ? (int)(e & 0xffffu) : 0;
                const float4 pi = s_hpos[i];
                const float4 pj = s_pos[j];
                const int4 a = s_aux[j];
                const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
                const float r2 = dx * dx + dy * dy + dz * dz;
                const unsigned grp = __match_any_sync(0xffffffffu, valid ? i : (0x10000 | lane));
                const int first = __ffs(grp) - 1, last = 31 - __clz(grp);
                float fx = 0.f, fy = 0.f, fz = 0.f;
                if (p.use_lj && valid && r2 <= rc2 && s_haux[i].x != a.y) {
                    const float inv = rcp_approx(r2);
                    const float sg = pi.w + pj.w;
                    const float x = sg * sg * inv;
                    const float lj6 = x * x * x;
                    const float ee = __int_as_float(s_haux[i].y) * __int_as_float(a.w);
                    const float ljd = 24.0f * ee * (2.0f * lj6 * lj6 - lj6);
                    const float fac = MEASURE ? ljd * inv : ljd * inv * p.lj_fscalef;   // ATM2B factor
                    fx = dx * fac; fy = dy * fac; fz = dz * fac;
                    if (MEASURE) {
                        const float wt = (p.virial_compat && (a.z & 32)) ? 1.0f : 0.5f;
                        m_u += 2.0f * ee * (lj6 * lj6 - lj6);       // half of 4 eps (s12 - s6) per visit
                        m_pairs += 0.5f;
                        m_w[0] += wt * dx * fx;
                        m_w[1] += wt * 0.5f * (dx * fy + dy * fx);
                        m_w[2] += wt * dy * fy;
                        m_w[3] += wt * 0.5f * (dx * fz + dz * fx);
                        m_w[4] += wt * 0.5f * (dy * fz + dz * fy);
                        m_w[5] += wt * dz * fz;
                    }
                }
                for (int o = 1; o < 32; o <<= 1) {
                    const float yx = __shfl_down_sync(0xffffffffu, fx, o);
                    const float yy = __shfl_down_sync(0xffffffffu, fy, o);
                    const float yz = __shfl_down_sync(0xffffffffu, fz, o);
                    if (lane + o <= last) { fx += yx; fy += yy; fz += yz; }
                }
                const bool emit = EMIT && valid && r2 <= rc3sq;
                const unsigned em = __ballot_sync(0xffffffffu, emit) & grp;
                int base = 0;
                if (EMIT && valid && lane == first) base = s_cnt[i];
                base = __shfl_sync(0xffffffffu, base, first);
                if (valid && lane == first) {
                    s_f[3 * i] += fx;
                    s_f[3 * i + 1] += fy;
                    s_f[3 * i + 2] += fz;
                    if (EMIT) s_cnt[i] = base + __popc(em);
                }
                if (emit) {
                    const int c = base + __popc(em & lanemask_lt());
                    const int slot_i = hs + hb + i;
                    if (c < p.nl_cap)
                        nl[(size_t)slot_i * p.nl_cap + c] = make_float4(dx, dy, dz, __int_as_float(a.z | (a.x << 6)));
                }
                __syncwarp();
            };

            int qn = 0;
            for (int i = w; i < hc; i += kTileWarps) {
                const float4 pi = s_hpos[i];
                const int self = self_base + i - sb;
                for (int j0 = 0; j0 < ns; j0 += 32) {
                    const int j = j0 + lane;
                    bool hit = false;
                    if (j < ns && j != self) {
                        const float4 pj = s_pos[j];
                        const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
                        hit = dx * dx + dy * dy + dz * dz <= scan2;
                    }
                    const unsigned m = __ballot_sync(0xffffffffu, hit);
                    if (hit) s_q[w][qn + __popc(m & lanemask_lt())] = ((unsigned)i << 16) | (unsigned)j;
                    qn += __popc(m);
                    if (qn >= 32) {
                        __syncwarp();
                        const unsigned e = s_q[w][lane];
                        const unsigned tail = (lane < qn - 32) ? s_q[w][lane + 32] : 0u;
                        __syncwarp();
                        if (lane < qn - 32) s_q[w][lane] = tail;
                        __syncwarp();
                        qn -= 32;
                        process(e, true);
                    }
                }
            }
            __syncwarp();
            if (qn > 0) {
                const unsigned e = (lane < qn) ? s_q[w][lane] : 0u;
                __syncwarp();
                process(e, lane < qn);
            }
        }
        __syncthreads();
        for (int t = tid; t < hc; t += kTileThreads) {
            const int slot = hs + hb + t;
            const int site = p.slot_site[slot];
            p.f[3 * site] = (double)s_f[3 * t];
            p.f[3 * site + 1] = (double)s_f[3 * t + 1];
            p.f[3 * site + 2] = (double)s_f[3 * t + 2];
            if (EMIT) {
                const int c = s_cnt[t];
                p.nl_count[slot] = min(c, p.nl_cap);
                if (c > p.nl_cap) atomicOr(&p.err[E_ATM_OVERFLOW], 1);
            }
        }
        __syncthreads();
    }
    if (MEASURE) {
        // the lanes' FP32 partials summed over the warp in FP32 (a fixed tree:
        // GB300's FP64 pipe made an FP64 tree the bulk of this pass), FP64 from
        // the warp sums on
        float vals[8] = {m_u, m_w[0], m_w[1], m_w[2], m_w[3], m_w[4], m_w[5], m_pairs};
        for (int k = 0; k < 8; k++) {
            float x = vals[k];
            for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
            vals[k] = x;
        }
        if (lane == 0) for (int k = 0; k < 8; k++) s_part[w][k] = (double)vals[k];
        __syncthreads();
        if (tid < R_NSLOTS) {
            double s = 0.0;
            int src = -1;
            if (tid == R_ULJ) src = 0;
            else if (tid >= R_W0 && tid <= R_W5) src = 1 + tid - R_W0;
            else if (tid == R_PAIRS) src = 7;
            if (src >= 0)
                for (int k = 0; k < kTileWarps; k++) s += s_part[k][src];
            p.partials[(size_t)blockIdx.x * R_NSLOTS + tid] = s;
        }
    }
}

// ---------------------------------------------------------------------------
// Verlet list build (rebuild steps only): one warp per home cell, one lane per
// home site (groups of 32 when a cell holds more, or two homes per lane in
// the form for crowded cells).  The warp walks the 27
// neighbour cells in order and stages each one's sites (position with the
// cell's periodic offset, list word, molecule key) in warp-private shared
// memory; every lane tests them all against its site and appends the hits to
// its row.  Rows hold the pairs inside cutoff + skin by neighbour cell, then
// by slot (deterministic); bit 31 marks a same-molecule pair (no LJ).
// A row has two regions: the neighbours above the site (vl_above: larger z
// at the rebuild, ties by slot) from the front, the others from the back
// (row[cap-1] downwards); the count word holds both (above | below << 16).
// The half-list force pass reads the front region alone, full-row readers
// both (vl_entry).
// ---------------------------------------------------------------------------
constexpr int kVbWarps = 4;   // home cells per block

// appends one hit to a two-region row: the front for a neighbour above the
// site (vl_above), the back otherwise (a full row drops the hit and the count
// still grows: the caller flags the overflow)
__device__ __forceinline__ void vl_put(unsigned *row, int cap, int &chi, int &clo, unsigned word, bool up) {
    if (chi + clo < cap) row[up ? chi : cap - 1 - clo] = word;
    if (up) chi++; else clo++;
}

// the count word of a row (both regions clamped so that they never overlap)
__device__ __forceinline__ int vl_count_word(int chi, int clo, int cap) {
    const int a = min(chi, cap), b = min(clo, cap - a);
    return a | (b << 16);
}

// logical entry k of a full row (the front region, then the back region)
__device__ __forceinline__ int vl_entry(int k, int chi, int cap) { return k < chi ? k : cap - 1 - (k - chi); }

// one lane's home site in the build: position, key, row and hit count
struct VbHome {
    float4 p;
    int key, slot, c, clo, zk;
    unsigned self;
    bool active;
};

__device__ __forceinline__ void vb_home(const PairParams &p, int hs, int hn, int h, VbHome &o) {
    o.active = h < hn;
    o.slot = hs + min(h, hn - 1);
    o.p = p.pos4[o.slot];
    o.key = p.skey[o.slot];
    o.self = (13u << 26) | (unsigned)o.slot;   // the site itself, in the home cell
    o.c = 0;
    o.clo = 0;
    o.zk = p.zkey[o.slot];
}

__device__ __forceinline__ bool vb_hit(const VbHome &o, const float4 &pj, float rl2) {
    const float ax = o.p.x - pj.x, ay = o.p.y - pj.y, az = o.p.z - pj.z;
    return ax * ax + ay * ay + az * az <= rl2;
}

__device__ __forceinline__ void vb_emit(const PairParams &p, VbHome &o, const uint2 &ww, int zk) {
    if (ww.x != o.self)
        vl_put(p.vl + (size_t)o.slot * p.vl_cap, p.vl_cap, o.c, o.clo, ((int)ww.y == o.key ? 0x80000000u : 0u) | ww.x,
               vl_above(o.zk, zk, (unsigned)o.slot, ww.x & 0x3ffffffu));
}

__device__ __forceinline__ void vb_done(const PairParams &p, const VbHome &o) {
    if (o.active) {
        p.vl_count[o.slot] = vl_count_word(o.c, o.clo, p.vl_cap);
        if (o.c + o.clo > p.vl_cap) atomicOr(&p.err[E_VL_OVERFLOW], 1);
    }
}

// the 27 cells around a home cell, staged 32 sites at a time in the warp's
// shared arrays (position in the home cell's frame; list word without the
// same-molecule bit and molecule key; order key); visit(jc) tests the jc
// staged sites
template <typename Visit>
__device__ __forceinline__ void vb_walk(const PairParams &p, int cx, int cy, int cz, const float4 *nbo, float4 *sq,
                                        uint2 *sw, int *sz, int lane, Visit &&visit) {
    for (int nb = 0; nb < 27; nb++) {
        int kx, ky, kz;
        bool cr;
        const int q = nb_cell(p.g, cx, cy, cz, nb, kx, ky, kz, cr);
        const int qs = p.cell_start[q], qn = p.cell_start[q + 1] - qs;
        const float4 o = nbo[nb];
        for (int jb = 0; jb < qn; jb += 32) {
            const int jc = min(32, qn - jb);
            __syncwarp();
            if (lane < jc) {
                const int j = qs + jb + lane;
                float4 pj = p.pos4[j];
                pj.x += o.x;
                pj.y += o.y;
                pj.z += o.z;
                sq[lane] = pj;
                sw[lane] = make_uint2(((unsigned)nb << 26) | (unsigned)j, (unsigned)p.skey[j]);
                sz[lane] = p.zkey[j];
            }
            __syncwarp();
            visit(jc);
        }
    }
}

// TWO = false: a home site per lane, one walk per 32 homes (cells of up to
// about 26 sites on average); TWO = true: cells of more than 32 sites walk
// their neighbourhood once per 64 homes.  Both write the same rows.
template <bool TWO>
__device__ __forceinline__ void vlist_build_body(const PairParams &p, int bid) {
    __shared__ float4 s_q[kVbWarps][32];
    __shared__ uint2 s_w[kVbWarps][32];
    __shared__ int s_z[kVbWarps][32];
    if (!*p.rebuild) return;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (bid == 0 && threadIdx.x == 0 && p.rebuild_count) atomicAdd(p.rebuild_count, 1);
    const float rl2 = (float)p.rl2;
    float4 *sq = s_q[w];
    uint2 *sw = s_w[w];
    int *sz = s_z[w];
    // warps take home cells from a counter (reset by the scan of this rebuild):
    // cells differ in cost, and a resident grid keeps every SM busy to the end
    for (;;) {
        int cell = 0;
        if (lane == 0) cell = atomicAdd(p.vb_next, 1);
        cell = __shfl_sync(0xffffffffu, cell, 0);
        if (cell < 0 || cell >= p.g.ncell) break;
        int cx, cy, cz;
        cell_coords(p.g, cell, cx, cy, cz);
        const int hs = p.cell_start[cell], hn = p.cell_start[cell + 1] - hs;
        const float4 *nbo = p.nboff + (size_t)cell * 27;
        if (!TWO || hn <= 32) {
          for (int hb = 0; hb < hn; hb += 32) {   // one trip unless TWO is false and hn > 32
            // a home site per lane
            const int h = hb + lane;
            const bool active = h < hn;
            const int hslot = hs + min(h, hn - 1);
            const float4 hp = p.pos4[hslot];
            const int hkey = p.skey[hslot];
            const int hz = p.zkey[hslot];
            const unsigned self = (13u << 26) | (unsigned)hslot;   // the site itself, in the home cell
            unsigned *row = p.vl + (size_t)hslot * p.vl_cap;
            int c = 0, clo = 0;
            vb_walk(p, cx, cy, cz, nbo, sq, sw, sz, lane, [&](int jc) {
                if (active) {
#pragma unroll 4
                    for (int t = 0; t < jc; t++) {
                        const float4 pj = sq[t];
                        const float ax = hp.x - pj.x, ay = hp.y - pj.y, az = hp.z - pj.z;
                        if (ax * ax + ay * ay + az * az <= rl2) {   // the word is read only for hits
                            const uint2 ww = sw[t];
                            if (ww.x != self)
                                vl_put(row, p.vl_cap, c, clo, ((int)ww.y == hkey ? 0x80000000u : 0u) | ww.x,
                                       vl_above(hz, sz[t], (unsigned)hslot, ww.x & 0x3ffffffu));
                        }
                    }
                }
            });
            if (active) {
                p.vl_count[hslot] = vl_count_word(c, clo, p.vl_cap);
                if (c + clo > p.vl_cap) atomicOr(&p.err[E_VL_OVERFLOW], 1);
            }
          }
        } else {
            // up to 64 home sites per walk of the neighbourhood: lane l serves
            // homes hb + l and, while more than 32 remain, hb + 32 + l
            for (int hb = 0; hb < hn; hb += 64) {
                const bool two = hn - hb > 32;   // warp-uniform
                VbHome h0, h1;
                vb_home(p, hs, hn, hb + lane, h0);
                if (two) vb_home(p, hs, hn, hb + 32 + lane, h1);
                vb_walk(p, cx, cy, cz, nbo, sq, sw, sz, lane, [&](int jc) {
                    if (two) {   // h0 is active: hn - hb > 32
#pragma unroll 2
                        for (int t = 0; t < jc; t++) {
                            const float4 pj = sq[t];
                            const uint2 ww = sw[t];   // one read for both homes
                            if (vb_hit(h0, pj, rl2)) vb_emit(p, h0, ww, sz[t]);
                            if (h1.active && vb_hit(h1, pj, rl2)) vb_emit(p, h1, ww, sz[t]);
                        }
                    } else if (h0.active) {
#pragma unroll 4
                        for (int t = 0; t < jc; t++)
                            if (vb_hit(h0, sq[t], rl2)) vb_emit(p, h0, sw[t], sz[t]);
                    }
                });
                vb_done(p, h0);
                if (two) vb_done(p, h1);
            }
        }
    }
}
template <bool TWO>
__global__ void __launch_bounds__(32 * kVbWarps) k_vlist_build(PairParams p) {
    pdl_trigger();
    pdl_wait();
    vlist_build_body<TWO>(p, blockIdx.x);
}

// ---------------------------------------------------------------------------
// LJ forces from the Verlet list (every step of the Verlet path): one warp
// per site, one list entry per lane; the neighbour's position is its FP32
// cell-local position plus the build-cell offset of the entry's neighbour
// cell.  Inside cutoff_3b the pair is appended to the ATM list in list
// order.  No atomics: the warp owns its site.
// ---------------------------------------------------------------------------
// The LJ pass over site i's Verlet row (one warp, lanes over the entries):
// the site's LJ force to f, and inside cutoff_3b the pair appended to the ATM
// list in list order -- to the global list, or (TO_SMEM) staged in shared
// memory (se, sq) for the sweep that follows in the same warp.  Returns the
// number of ATM neighbours kept.
// U = list entries per lane in flight (independent loads for latency hiding):
// a warp covers 32 U entries of a row per pass
template <bool MEASURE, bool EMIT, bool UNIFORM, int U, bool TO_SMEM>
__device__ __forceinline__ int lj_site(const PairParams &p, int i, int lane, unsigned lt, float rc2, float rc3sq,
                                       float4 *se, float4 *sq, float &m_u, float &m_pairs, float (&m_w)[6]) {
    const int cw = p.vl_count[i];
    const int chi = cw & 0xffff, cnt = chi + (cw >> 16);   // both regions of the row
    const float4 pi = p.pos4[i];
    const float sei = UNIFORM ? 0.f : p.seps[i];
    const float4 *off = p.nboff + (size_t)p.slot_cell[i] * 27;
    const unsigned *row = p.vl + (size_t)i * p.vl_cap;
    const float sg2u = p.sig0 * p.sig0, eeu = p.eps0;
    float fx = 0.f, fy = 0.f, fz = 0.f;
    int c_atm = 0;
    for (int k0 = 0; k0 < cnt; k0 += 32 * U) {
        unsigned e[U];
        float4 o[U], pj[U];
        float sej[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int k = k0 + u * 32 + lane;
            e[u] = k < cnt ? __ldcs(row + vl_entry(k, chi, p.vl_cap)) : 0xffffffffu;   // read once per step: evict first
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
            if (e[u] != 0xffffffffu) {
                o[u] = off[(e[u] >> 26) & 31u];
                pj[u] = p.pos4[e[u] & 0x3ffffffu];
                if (!UNIFORM) sej[u] = p.seps[e[u] & 0x3ffffffu];
            }
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
            const bool valid = e[u] != 0xffffffffu;
            float dx = 0.f, dy = 0.f, dz = 0.f, r2 = 1e30f;
            if (valid) {
                dx = pi.x - (pj[u].x + o[u].x);
                dy = pi.y - (pj[u].y + o[u].y);
                dz = pi.z - (pj[u].z + o[u].z);
                r2 = dx * dx + dy * dy + dz * dz;
                if (p.use_lj && r2 <= rc2 && !(e[u] >> 31)) {
                    const float inv = rcp_approx(r2);
                    float x, ee;
                    if (UNIFORM) {
                        x = sg2u * inv;
                        ee = eeu;
                    } else {
                        const float sg = pi.w + pj[u].w;
                        x = sg * sg * inv;
                        ee = sei * sej[u];
                    }
                    const float lj6 = x * x * x;
                    float fac0 = 24.0f * ee * (2.0f * lj6 * lj6 - lj6) * inv;
                    float usw = 1.0f;
                    if (p.sw) {   // switched cutoff: U S, force fac S - 2 U dS/dx
                        float dS;
                        sw_eval(r2, p.sw_rc2, p.sw_iw, usw, dS);
                        fac0 = fac0 * usw - 8.0f * ee * (lj6 * lj6 - lj6) * dS;
                    }
                    const float fac = MEASURE ? fac0 : fac0 * p.lj_fscalef;   // ATM2B factor
                    fx += dx * fac; fy += dy * fac; fz += dz * fac;
                    if (MEASURE) {
                        const float gx = dx * fac, gy = dy * fac, gz = dz * fac;
                        m_u += 2.0f * ee * (lj6 * lj6 - lj6) * usw;
                        m_pairs += 0.5f;
                        m_w[0] += 0.5f * dx * gx;
                        m_w[1] += 0.25f * (dx * gy + dy * gx);
                        m_w[2] += 0.5f * dy * gy;
                        m_w[3] += 0.25f * (dx * gz + dz * gx);
                        m_w[4] += 0.25f * (dy * gz + dz * gy);
                        m_w[5] += 0.5f * dz * gz;
                    }
                }
            }
            if (EMIT) {
                // staged for the once-per-triplet sweep: neighbours above i only
                const bool emit = valid && r2 <= rc3sq && (!TO_SMEM || (int)(e[u] & 0x3ffffffu) > i);
                const unsigned m = __ballot_sync(0xffffffffu, emit);
                if (emit) {
                    const int pos = c_atm + __popc(m & lt);
                    const int nb = (int)((e[u] >> 26) & 31u), j = (int)(e[u] & 0x3ffffffu);
                    const int code = nb | (o[u].w != 0.f ? 32 : 0) | (j << 6);
                    if (pos < p.nl_cap) {
                        const float4 entry = make_float4(dx, dy, dz, __int_as_float(code));
                        if (TO_SMEM) {   // staged as the sweep wants it: e and (A, 1/A, 1/sqrt A)
                            se[pos] = entry;
                            sq[pos] = atm_stage_q(r2);
                        } else {
                            p.nl[(size_t)i * p.nl_cap + pos] = entry;
                        }
                    }
                }
                c_atm += __popc(m);
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        fx += __shfl_xor_sync(0xffffffffu, fx, o);
        fy += __shfl_xor_sync(0xffffffffu, fy, o);
        fz += __shfl_xor_sync(0xffffffffu, fz, o);
    }
    if (lane == 0) {
        const int site = p.slot_site[i];
        p.f[3 * site] = (double)fx;
        p.f[3 * site + 1] = (double)fy;
        p.f[3 * site + 2] = (double)fz;
        if (EMIT) {
            if (!TO_SMEM) p.nl_count[i] = min(c_atm, p.nl_cap);
            if (c_atm > p.nl_cap) atomicOr(&p.err[E_ATM_OVERFLOW], 1);
        }
    }
    return min(c_atm, p.nl_cap);
}

template <bool MEASURE, bool EMIT, bool UNIFORM, int U>
__global__ void __launch_bounds__(256, U == 3 ? 4 : 5) k_lj_vlist(PairParams p, int n, int per) {
    __shared__ double s_part[8][8];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const float rc2 = (float)p.rc2, rc3sq = (float)p.rc3sq;
    unsigned lt;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lt));
    float m_u = 0.f, m_pairs = 0.f, m_w[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    // each block walks `per` consecutive groups of 8 slots: neighbouring slots share
    // most of their neighbours, so the gathers of one group hit L1 lines of the last
    for (int it = 0; it < per; it++) {
        const int i = (blockIdx.x * per + it) * 8 + w;
        if (i < n) lj_site<MEASURE, EMIT, UNIFORM, U, false>(p, i, lane, lt, rc2, rc3sq, nullptr, nullptr, m_u, m_pairs, m_w);
    }
    if (MEASURE) {
        // the lanes' FP32 partials summed over the warp in FP32 (a fixed tree:
        // GB300's FP64 pipe made an FP64 tree the bulk of this pass), FP64 from
        // the warp sums on
        float vals[8] = {m_u, m_w[0], m_w[1], m_w[2], m_w[3], m_w[4], m_w[5], m_pairs};
        for (int k = 0; k < 8; k++) {
            float x = vals[k];
            for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
            vals[k] = x;
        }
        if (lane == 0) for (int k = 0; k < 8; k++) s_part[w][k] = (double)vals[k];
        __syncthreads();
        const int tid = threadIdx.x;
        if (tid < R_NSLOTS) {
            double s = 0.0;
            int src = -1;
            if (tid == R_ULJ) src = 0;
            else if (tid >= R_W0 && tid <= R_W5) src = 1 + tid - R_W0;
            else if (tid == R_PAIRS) src = 7;
            if (src >= 0)
                for (int k = 0; k < 8; k++) s += s_part[k][src];
            p.partials[(size_t)blockIdx.x * R_NSLOTS + tid] = s;
        }
    }
}

// LJ and ATM in one pass (FP32 forces, FULL triplets, Verlet path): each warp
// runs the LJ pass of its site, stages the site's ATM neighbours above it in
// shared memory instead of the global list, and sweeps its triplets at once.
// Warps in their latency-bound LJ phase and warps in their issue-bound sweep
// share each SM, and the ATM list never goes to memory.  The arithmetic and
// the order of every sum are those of k_lj_vlist + k_atm_s.
template <bool UNIFORM, int U>
__global__ void __launch_bounds__(256, 4) k_lj_atm(PairParams p, AtmParams a, int n, int per) {
    extern __shared__ float4 s_dyn[];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    float4 *se = s_dyn + w * 2 * p.nl_cap, *sq = se + p.nl_cap;
    const float rc2 = (float)p.rc2, rc3sq = (float)p.rc3sq, rc3f = (float)a.rc2;
    unsigned lt;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lt));
    float m_u = 0.f, m_pairs = 0.f, m_w[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int it = 0; it < per; it++) {
        const int i = (blockIdx.x * per + it) * 8 + w;
        if (i < n) {
            const int m = lj_site<false, true, UNIFORM, U, true>(p, i, lane, lt, rc2, rc3sq, se, sq, m_u, m_pairs, m_w);
            __syncwarp();
            atm_vertex(a, i, se, sq, m, lane, rc3f);
            __syncwarp();   // se / sq are refilled by the next site
        }
    }
}

// ---------------------------------------------------------------------------
// The half-list LJ + ATM pass (FP32 forces, FULL triplets, Verlet path, no
// Limit): each pair and each triplet is evaluated once, from its lowest
// member in the order vl_above.  One warp per site i walks the front region
// of i's row only (the neighbours above i, about half the row):
//   1. LJ: the force on i stays in the lanes' registers; the reaction on the
//      partner j is staged in shared memory (sr) beside the partner's slot;
//      partners inside cutoff_3b are staged for the triplet sweep as well
//      (se, sq, at the front of their arrays), LJ-only partners fill sr from
//      the back;
//   2. the triplet sweep of atm_vertex_shares leaves each ATM partner's share
//      in its owner lane;
//   3. each partner gets its LJ reaction plus its ATM share (in force units)
//      through ONE 64-bit fixed-point add per component -- integer sums, so
//      the result does not depend on the order in which warps add;
//   4. i's own force (its LJ sum plus its ATM share) is written to f; the
//      flush adds the fixed-point sums of the partners' contributions.
// Against the full-row pass this reads half the list, evaluates each LJ
// pair once instead of twice, and converts one FP32 partial per partner.
// ---------------------------------------------------------------------------
// what the half-list pass reads of a site before its arithmetic: the count
// of its front region, the region's first 64 entries (rows hold vl_cap >= 64
// entries, so both reads stay inside the row; the count masks them, and the
// entries are read without waiting for it), its position and its cell.
// (Loading this one site ahead, during the previous site's sweep, was
// measured slower: the extra live registers spill at the 64-register bound.)
struct HalfRow {
    int cnt, cell;
    unsigned e0, e1;
    float4 pi;
};

__device__ __forceinline__ void half_row_load(const PairParams &p, int i, int lane, HalfRow &h) {
    const unsigned *row = p.vl + (size_t)i * p.vl_cap;
    h.cnt = p.vl_count[i] & 0xffff;   // the neighbours above i
    h.e0 = __ldcs(row + lane);        // read once per step: evict first
    h.e1 = __ldcs(row + 32 + lane);
    h.pi = p.pos4[i];
    h.cell = p.slot_cell[i];
}

// PLAIN: the LJ term is on with no ATM2B factor (use_lj = 1, lj_fscalef = 1),
// so neither is read per pair (the products are the same: a factor of 1 is exact)
template <bool UNIFORM, bool SW, bool PLAIN>
__device__ __forceinline__ void lj_half(const PairParams &p, int i, const HalfRow &h, int lane, unsigned lt, float rc2,
                                        float rc3sq, float4 *se, float4 *sq, float4 *sr, int capa, int capr,
                                        int &m_out, int &k_out, float &fx, float &fy, float &fz) {
    const int cnt = h.cnt;
    const float4 pi = h.pi;
    const float sei = UNIFORM ? 0.f : p.seps[i];
    const float4 *off = p.nboff + (size_t)h.cell * 27;
    const unsigned *row = p.vl + (size_t)i * p.vl_cap;
    const float sg2u = p.sig0 * p.sig0, eeu = p.eps0;
    fx = fy = fz = 0.f;
    int m = 0, k = 0;
    for (int k0 = 0; k0 < cnt; k0 += 64) {
        unsigned e[2];
        float4 o[2], pj[2];
        float sej[2];
        if (k0 == 0) {   // the first 64 entries, read with the count
            e[0] = lane < cnt ? h.e0 : 0xffffffffu;
            e[1] = 32 + lane < cnt ? h.e1 : 0xffffffffu;
        } else {
#pragma unroll
            for (int u = 0; u < 2; u++) {
                const int kk = k0 + u * 32 + lane;
                e[u] = kk < cnt ? __ldcs(row + kk) : 0xffffffffu;
            }
        }
#pragma unroll
        for (int u = 0; u < 2; u++) {
            if (e[u] != 0xffffffffu) {
                o[u] = off[(e[u] >> 26) & 31u];
                pj[u] = p.pos4[e[u] & 0x3ffffffu];
                if (!UNIFORM) sej[u] = p.seps[e[u] & 0x3ffffffu];
            }
        }
#pragma unroll
        for (int u = 0; u < 2; u++) {
            const bool valid = e[u] != 0xffffffffu;
            float dx = 0.f, dy = 0.f, dz = 0.f, r2 = 1e30f;
            float gx = 0.f, gy = 0.f, gz = 0.f;
            bool lj = false;
            if (valid) {
                dx = pi.x - (pj[u].x + o[u].x);
                dy = pi.y - (pj[u].y + o[u].y);
                dz = pi.z - (pj[u].z + o[u].z);
                r2 = dx * dx + dy * dy + dz * dz;
                lj = (PLAIN || p.use_lj) && r2 <= rc2 && !(e[u] >> 31);
                if (lj) {
                    const float inv = rcp_approx(r2);
                    float x, ee;
                    if (UNIFORM) {
                        x = sg2u * inv;
                        ee = eeu;
                    } else {
                        const float sg = pi.w + pj[u].w;
                        x = sg * sg * inv;
                        ee = sei * sej[u];
                    }
                    const float lj6 = x * x * x;
                    float fac = 24.0f * ee * (2.0f * lj6 * lj6 - lj6) * inv;
                    if (!PLAIN) fac *= p.lj_fscalef;   // ATM2B factor
                    if (SW) {   // switched cutoff (no ATM2B with it): U S, force fac S - 2 U dS/dx
                        float S, dS;
                        sw_eval(r2, p.sw_rc2, p.sw_iw, S, dS);
                        fac = fac * S - 8.0f * ee * (lj6 * lj6 - lj6) * dS;
                    }
                    gx = dx * fac; gy = dy * fac; gz = dz * fac;
                    fx += gx; fy += gy; fz += gz;
                }
            }
            const bool at = valid && r2 <= rc3sq;   // a triplet partner (LJ or not)
            const bool lo = lj && !at;              // an LJ-only partner
            const unsigned ma = __ballot_sync(0xffffffffu, at), ml = __ballot_sync(0xffffffffu, lo);
            if (at || lo) {
                // the partner's slot j at bits 6-30 (j < 2^25 with ATM on): the list word
                // shifted past its cell and molecule bits.  This pass reads only
                // code >> 6 (the cell bits of atm_code are for the COMPAT filter)
                const int code = (int)(e[u] << 6);
                const float4 react = make_float4(-gx, -gy, -gz, __int_as_float(code));
                if (at) {
                    const int pos = m + __popc(ma & lt);
                    if (pos < capa) {
                        se[pos] = make_float4(dx, dy, dz, __int_as_float(code));
                        sq[pos] = atm_stage_q(r2);
                        sr[pos] = react;
                    }
                } else {
                    sr[capr - 1 - (k + __popc(ml & lt))] = react;
                }
            }
            m += __popc(ma);
            k += __popc(ml);
        }
    }
    if (lane == 0 && m > capa) atomicOr(&p.err[E_ATM_OVERFLOW], 1);
    m_out = min(m, capa);
    k_out = k;
}

template <bool UNIFORM, bool SW, bool PLAIN>
__device__ __forceinline__ void lj_atm_half_body(const PairParams &p, const AtmParams &a, float sa, int n, int per,
                                                 int bid) {
    extern __shared__ float4 s_dyn[];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int capa = p.nl_cap, capr = p.vl_cap;
    float4 *se = s_dyn + (size_t)w * (2 * capa + capr), *sq = se + capa, *sr = sq + capa;
    const float rc2 = (float)p.rc2, rc3sq = (float)p.rc3sq, rc3f = (float)a.rc2;
    const unsigned lt = lanemask_lt();
    for (int it = 0; it < per; it++) {
        const int i = (bid * per + it) * 8 + w;
        if (i >= n) break;   // warp-uniform; later groups of this block are past n too
        HalfRow cur;
        half_row_load(p, i, lane, cur);
        int m, k;
        float fx, fy, fz;
        lj_half<UNIFORM, SW, PLAIN>(p, i, cur, lane, lt, rc2, rc3sq, se, sq, sr, capa, capr, m, k, fx, fy, fz);
        __syncwarp();
        float ax, ay, az, gx, gy, gz;
        atm_vertex_shares<SW>(a, se, sq, m, lane, rc3f, sa, ax, ay, az, gx, gy, gz);
        // every partner: LJ reaction + ATM share (force units), one fixed-point add per component
        const int tot = m + k;
        for (int L = lane; L < tot; L += 32) {
            const float4 rr = sr[L < m ? L : capr - 1 - (L - m)];
            float vx = rr.x, vy = rr.y, vz = rr.z;
            if (L == lane) {   // the first trip: lane L < 32 owns partner L's share (zero for m > 32)
                vx = fmaf(sa, ax, vx);
                vy = fmaf(sa, ay, vy);
                vz = fmaf(sa, az, vz);
            }
            unsigned long long *acc = a.acc + 3 * (size_t)(__float_as_int(rr.w) >> 6);
            atm_fix_add(acc, vx);
            atm_fix_add(acc + 1, vy);
            atm_fix_add(acc + 2, vz);
        }
        // the site's own force: its LJ sum and its ATM share
        fx = fmaf(sa, gx, fx);
        fy = fmaf(sa, gy, fy);
        fz = fmaf(sa, gz, fz);
        // the warp sums of (fx, fy, fz) by the butterfly over offsets 16, 8, 4, 2, 1,
        // the lanes splitting the components on the way: after offset 16 the lanes
        // below 16 carry x and y, the others z; after offset 8 lanes 0-7 carry x,
        // 8-15 y, 16-31 z.  Every sum pairs the same partial sums as a butterfly
        // per component (FP32 addition commutes), so the totals are bitwise those
        // of 15 shuffles, with 6.
        float c0;
        {
            const bool up16 = (lane & 16) != 0, up8 = (lane & 8) != 0;
            const float r1 = __shfl_xor_sync(0xffffffffu, up16 ? fx : fz, 16);
            const float r2 = __shfl_xor_sync(0xffffffffu, fy, 16);
            c0 = (up16 ? fz : fx) + r1;   // z above 16, x below
            const float c1 = fy + r2;     // y below 16
            const float r3 = __shfl_xor_sync(0xffffffffu, (up16 || up8) ? c0 : c1, 8);
            c0 = ((up16 || !up8) ? c0 : c1) + r3;
            for (int o = 4; o > 0; o >>= 1) c0 += __shfl_xor_sync(0xffffffffu, c0, o);
        }
        if ((lane & 7) == 0) {   // lanes 0, 8, 16, 24: x, y, z and the slot's fourth word
            if (p.fown) {   // FP32 by slot, 16 bytes: the flush widens it (no FP64-pipe conversions here)
                reinterpret_cast<float *>(p.fown + i)[lane >> 3] = lane < 24 ? c0 : 0.f;
            } else if (lane < 24) {
                p.f[3 * (size_t)p.slot_site[i] + (lane >> 3)] = (double)c0;
            }
        }
        __syncwarp();   // se / sq / sr are refilled by the next site
    }
}
template <bool UNIFORM, bool SW, bool PLAIN>
__global__ void __launch_bounds__(256, 4) k_lj_atm_half(PairParams p, AtmParams a, float sa, int n, int per) {
    pdl_trigger();
    pdl_wait();
    lj_atm_half_body<UNIFORM, SW, PLAIN>(p, a, sa, n, per, blockIdx.x);
}

template <bool UNIFORM, bool SW, bool PLAIN = false>
static void launch_half(const PairParams &p, const AtmParams &a, float sa, int n, int per, int grid, size_t sm,
                        cudaStream_t st) {
    if (sm > 48 * 1024)
        cudaFuncSetAttribute(k_lj_atm_half<UNIFORM, SW, PLAIN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    launch_pdl(k_lj_atm_half<UNIFORM, SW, PLAIN>, grid, 256, sm, st, p, a, sa, n, per);
}

// shared memory of the half-list pass: per warp nl_cap staged triplet
// partners (se, sq) and vl_cap partners' reactions (sr)
size_t lj_atm_half_smem(const Engine &e) {
    return (size_t)8 * sizeof(float4) * (2 * (size_t)e.nl_cap + (size_t)e.vl_cap);
}

// the half-list pass serves the step when nothing after the pair terms reads
// or clamps the force of a site before the flush (no Limit, no FENE, no
// tabulated term) and its staging fits the shared memory of four blocks
bool lj_atm_half(const Engine &e) {
    if (e.cfg.terms & (KOMD_TERM_LIMIT | KOMD_TERM_FENE | KOMD_TERM_TABULATED)) return false;
    return lj_atm_half_smem(e) <= 56 * 1024 || e.cfg.switch_width > 0;   // the switch runs here only
}

bool half_plain(const PairParams &p) { return p.use_lj && p.lj_fscalef == 1.0f; }

// the bonded terms add to f between the force pass and the flush, so with
// them the pass writes f itself
float4 *half_own(const Engine &e) { return (e.cfg.terms & KOMD_TERM_BONDED) ? nullptr : e.fown; }

int vlist_grid(const Engine &e) { return (int)((e.n + 7) / 8); }

// groups of 8 slots per block of the force pass: about eight resident waves of
// blocks (5 per SM), each over a contiguous range of slots
int vlist_per(const Engine &e) {
    const int groups = vlist_grid(e);
    const int target = e.num_sms * 5 * 8;
    return groups <= target ? 1 : (groups + target - 1) / target;
}

// ---- packed replicas (kernels.cuh): the list build and the half-list pass of
// every replica in one launch each
__device__ __forceinline__ int packed_replica(const int *__restrict__ start, int nrep, int b) {
    int lo = 0, hi = nrep;   // start[0] = 0 <= b < start[nrep]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (start[mid] <= b) lo = mid;
        else hi = mid;
    }
    return lo;
}

__global__ void __launch_bounds__(32 * kVbWarps) k_vlist_build_p(const PairParams *__restrict__ p,
                                                                const int *__restrict__ two,
                                                                const int *__restrict__ start, int nrep) {
    const int r = packed_replica(start, nrep, blockIdx.x);
    if (two[r]) vlist_build_body<true>(p[r], blockIdx.x - start[r]);
    else vlist_build_body<false>(p[r], blockIdx.x - start[r]);
}

template <bool UNIFORM, bool SW, bool PLAIN>
__global__ void __launch_bounds__(256, 4) k_lj_atm_half_p(const PairParams *__restrict__ p,
                                                          const AtmParams *__restrict__ a,
                                                          const float *__restrict__ sa, const int *__restrict__ n,
                                                          const int *__restrict__ per, const int *__restrict__ start,
                                                          int nrep) {
    const int r = packed_replica(start, nrep, blockIdx.x);
    lj_atm_half_body<UNIFORM, SW, PLAIN>(p[r], a[r], sa[r], n[r], per[r], blockIdx.x - start[r]);
}

template <bool UNIFORM, bool SW, bool PLAIN = false>
static void launch_half_p(const PackedStep &pk, cudaStream_t st) {
    if (pk.force_smem > 48 * 1024)
        cudaFuncSetAttribute(k_lj_atm_half_p<UNIFORM, SW, PLAIN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)pk.force_smem);
    k_lj_atm_half_p<UNIFORM, SW, PLAIN><<<pk.force.blocks, 256, pk.force_smem, st>>>(pk.pp, pk.ap, pk.sa, pk.n,
                                                                                     pk.per, pk.force.start, pk.nrep);
}

void launch_packed_pair_stages(const PackedStep &pk, cudaStream_t st, bool vbuild) {
    if (vbuild) {
        k_vlist_build_p<<<pk.vbuild.blocks, 32 * kVbWarps, 0, st>>>(pk.pp, pk.two, pk.vbuild.start, pk.nrep);
        return;
    }
    if (pk.sw) {
        if (pk.uniform) launch_half_p<true, true>(pk, st);
        else launch_half_p<false, true>(pk, st);
    } else {
        if (pk.uniform && pk.plain) launch_half_p<true, false, true>(pk, st);   // the benchmark's form
        else if (pk.uniform) launch_half_p<true, false>(pk, st);
        else launch_half_p<false, false>(pk, st);
    }
}

int packed_blocks_vbuild(const Engine &e) {
    // up to 1024 warps for a rebuilding replica (a warp per home cell here);
    // the blocks of replicas without a rebuild exit at once
    return std::max(1, std::min((e.g.ncell + kVbWarps - 1) / kVbWarps, 256));
}

bool vbuild_two(const Engine &e) {
    return (double)e.n / ((double)e.g.nd[0] * e.g.nd[1] * e.g.nd[2]) > 26.0;
}

void launch_vlist_build(Engine &e, cudaStream_t st) {
    PairParams p = pair_params(e);
    // a resident grid (12 blocks of 4 warps per SM at this kernel's register count)
    const int blocks = std::min((e.g.ncell + kVbWarps - 1) / kVbWarps, e.num_sms * 12);
    // the two-home form pays off once many cells hold more than 32 sites
    if (vbuild_two(e)) launch_pdl(k_vlist_build<true>, blocks, 32 * kVbWarps, 0, st, p);
    else launch_pdl(k_vlist_build<false>, blocks, 32 * kVbWarps, 0, st, p);
}

template <bool UNIFORM>
static void lj_vlist_dispatch(PairParams &p, int n, int grid, int per, bool measure, bool emit, bool u3,
                              cudaStream_t st) {
    if (measure) {
        if (emit) k_lj_vlist<true, true, UNIFORM, 2><<<grid, 256, 0, st>>>(p, n, per);
        else k_lj_vlist<true, false, UNIFORM, 2><<<grid, 256, 0, st>>>(p, n, per);
    } else if (u3) {
        if (emit) k_lj_vlist<false, true, UNIFORM, 3><<<grid, 256, 0, st>>>(p, n, per);
        else k_lj_vlist<false, false, UNIFORM, 3><<<grid, 256, 0, st>>>(p, n, per);
    } else {
        if (emit) k_lj_vlist<false, true, UNIFORM, 2><<<grid, 256, 0, st>>>(p, n, per);
        else k_lj_vlist<false, false, UNIFORM, 2><<<grid, 256, 0, st>>>(p, n, per);
    }
}

// rows of at most 96 entries on average: one pass of 3 entries per lane
// instead of two of 2 (the row length is the number of sites within the
// list range, about density * 4/3 pi (cutoff + skin)^3)
bool vlist_u3(const Engine &e) {
    const double reach = std::max(e.cfg.cutoff, (e.cfg.terms & KOMD_TERM_ATM) ? e.cfg.cutoff_3b : 0.0) + e.cfg.skin;
    const double rho = (double)e.n / (e.g.L[0] * e.g.L[1] * e.g.L[2]);
    return rho * 4.18879020478639 * reach * reach * reach <= 88.0;
}

int launch_lj_vlist(Engine &e, PairParams &p, bool measure, bool emit, cudaStream_t st) {
    // a block's partial sums cover all its groups (the lanes' sums run across them)
    const int per = vlist_per(e);
    const int grid = (vlist_grid(e) + per - 1) / per;
    const bool u3 = vlist_u3(e);
    if (e.uniform) lj_vlist_dispatch<true>(p, (int)e.n, grid, per, measure, emit, u3, st);
    else lj_vlist_dispatch<false>(p, (int)e.n, grid, per, measure, emit, u3, st);
    return grid;
}

void launch_lj_atm(Engine &e, cudaStream_t st) {
    PairParams p = pair_params(e);
    const AtmParams a = atm_params(e);
    const int per = vlist_per(e);
    const int grid = (vlist_grid(e) + per - 1) / per;
    if (lj_atm_half(e)) {
        const size_t sm = lj_atm_half_smem(e);
        const float sa = (float)(2.0 * a.sign * a.nu);   // share units (2 sign nu) to force units
        p.fown = half_own(e);
        if (p.sw) {
            if (e.uniform) launch_half<true, true>(p, a, sa, (int)e.n, per, grid, sm, st);
            else launch_half<false, true>(p, a, sa, (int)e.n, per, grid, sm, st);
        } else {
            if (e.uniform && half_plain(p)) launch_half<true, false, true>(p, a, sa, (int)e.n, per, grid, sm, st);
            else if (e.uniform) launch_half<true, false>(p, a, sa, (int)e.n, per, grid, sm, st);
            else launch_half<false, false>(p, a, sa, (int)e.n, per, grid, sm, st);
        }
        return;
    }
    const size_t sm = (size_t)8 * 2 * sizeof(float4) * (size_t)e.nl_cap;
    const bool u3 = vlist_u3(e);
    if (e.uniform) {
        if (u3) {
            if (sm > 48 * 1024) cudaFuncSetAttribute(k_lj_atm<true, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
            k_lj_atm<true, 3><<<grid, 256, sm, st>>>(p, a, (int)e.n, per);
        } else {
            if (sm > 48 * 1024) cudaFuncSetAttribute(k_lj_atm<true, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
            k_lj_atm<true, 2><<<grid, 256, sm, st>>>(p, a, (int)e.n, per);
        }
    } else {
        if (u3) {
            if (sm > 48 * 1024) cudaFuncSetAttribute(k_lj_atm<false, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
            k_lj_atm<false, 3><<<grid, 256, sm, st>>>(p, a, (int)e.n, per);
        } else {
            if (sm > 48 * 1024) cudaFuncSetAttribute(k_lj_atm<false, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
            k_lj_atm<false, 2><<<grid, 256, sm, st>>>(p, a, (int)e.n, per);
        }
    }
}

void launch_pair_tile(PairParams &p, int ncell, bool measure, bool emit, cudaStream_t st) {
    if (measure) {
        if (emit) k_pair_tile<true, true><<<ncell, kTileThreads, 0, st>>>(p);
        else k_pair_tile<true, false><<<ncell, kTileThreads, 0, st>>>(p);
    } else {
        if (emit) k_pair_tile<false, true><<<ncell, kTileThreads, 0, st>>>(p);
        else k_pair_tile<false, false><<<ncell, kTileThreads, 0, st>>>(p);
    }
}

}  // namespace komd
