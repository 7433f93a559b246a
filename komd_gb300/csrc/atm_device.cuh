// atm_device.cuh -- device functions of the once-per-triplet ATM sweep,
// shared by k_atm_s (kernels.cu) and the fused LJ + ATM pass (pair_tile.cu).
#pragma once

#include "engine.cuh"

namespace komd {

// FP32 ATM, FULL triplet set, forces only: every triplet once, from its
// lowest member i in a total order on the sites (the slot order in k_atm_s;
// the Verlet rows' order vl_above in the half-list pass), the other two
// members being neighbours of i above it.  One warp per vertex; lane a owns
// staged neighbour a (a < m, the neighbours above i) and evaluates the
// round-robin pairs (a, a+d mod m),
// d = 1 .. m/2, directly.  Per triplet with A = |e_a|^2, B = |e_b|^2,
// C = |e_b - e_a|^2 (e = r_i - r_x) and v_X = dV/dX / nu, the forces in units
// of 2 sign nu are
//   g_i = vA e_a + vB e_b,  g_a = -vA e_a + vC (e_b - e_a),  g_b = -vB e_b - vC (e_b - e_a).
// g_i and g_a stay in the lane's registers; g_b reaches lane b by one warp
// shuffle per component (lane r pulls from lane r - d mod m).  At the end the
// per-neighbour and per-vertex sums go to 64-bit fixed-point accumulators by
// integer atomics (order-independent: the forces are bitwise reproducible);
// k_atm_flush adds them to f.
constexpr double kAtmFix = 4294967296.0;   // 2^32 fixed-point units

// staged (A, 1/A, 1/sqrt A) of a neighbour at squared distance A: the
// hardware reciprocal (about 1 ulp) and reciprocal square root; A is a squared
// distance of order one, never in the flush-to-zero range
__device__ __forceinline__ float4 atm_stage_q(float A) {
    float ia;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(ia) : "f"(A));
    return make_float4(A, ia, rsqrtf(A), 0.f);
}

// round(x * 2^32) to the nearest integer (ties to even) as int64, for finite
// |x| < 2^31, built from two 32-bit conversions: GB300 runs FP32 -> int64
// conversions on its narrow FP64 pipe, FP32 -> int32 on the wide ones.
// With a = |x|: fl = floor(a) is an integer below 2^31 (the high word), and
// a - fl is exact (Sterbenz for a >= 1, a itself below 1), so (a - fl) * 2^32
// is the exact low part in [0, 2^32 - 2^8]; it has a fraction only for
// a < 2^-9, where rounding it is rounding x * 2^32.  The sign is applied last
// (round-to-nearest-even is symmetric).  Bitwise equal to rounding x * 2^32
// to int64 directly over all finite |x| < 2^31; a NaN contributes 0.
__device__ __forceinline__ long long fix32_rn(float x) {
    const float a = fabsf(x);
    const float fl = floorf(a);
    const unsigned hi = (unsigned)__float2int_rz(fl);
    const unsigned lo = __float2uint_rn((a - fl) * 4294967296.0f);
    const long long m = (long long)(((unsigned long long)hi << 32) | lo);
    return x < 0.f ? -m : m;
}

__device__ __forceinline__ void atm_fix_add(unsigned long long *acc, float x) {
    const long long q = fix32_rn(x);
    if (q != 0) atomicAdd(acc, (unsigned long long)q);
}

struct AtmV {
    float vA, vB, vC;
};
// dV/dA, dV/dB, dV/dC over nu from the squared sides and the staged (A, 1/A, 1/sqrt(A)).
// With t1 = A + B - C, t2 = A - B + C, t3 = B + C - A (= S - 2C, S - 2B, S - 2A for
// S = A + B + C), u = t2 t3, v = t1 t3, w = t1 t2, P = t1 t2 t3 and s5 = 1/(abc)^5:
//   dV/dA = s5 (3/8 (u + v - w) - 3/2 B C - 15/16 P / A)   (B with v and A C; C with u and A B),
// written around K = 3/8 (u + v + w), which the three share.
__device__ __forceinline__ AtmV atm_derivs(float4 qa, float4 qb, float C) {
    const float A = qa.x, B = qb.x;
    const float wc = rsqrtf(C);
    const float sv = qa.z * qb.z * wc;                  // 1/(abc)
    const float s2 = sv * sv;
    const float s5 = s2 * s2 * sv;
    const float S = A + B + C;
    const float t1 = fmaf(-2.0f, C, S), t2 = fmaf(-2.0f, B, S), t3 = fmaf(-2.0f, A, S);
    const float u = t2 * t3, v = t1 * t3, w = t1 * t2;
    const float K = 0.375f * (u + v + w);
    const float nP = -0.9375f * (t1 * u);
    const float a15 = -1.5f * A;
    AtmV r;
    r.vA = s5 * fmaf(nP, qa.y, fmaf(-0.75f, w, fmaf(-1.5f * B, C, K)));
    r.vB = s5 * fmaf(nP, qb.y, fmaf(-0.75f, v, fmaf(a15, C, K)));
    r.vC = s5 * fmaf(nP, wc * wc, fmaf(-0.75f, u, fmaf(a15, B, K)));
    return r;
}

// atm_derivs under the switched cutoff (AtmParams::sw): the triplet energy
// V S(A) S(B) S(C) differentiated in the squared sides; sA / dA are S and
// dS/dx of the lane's own side A, computed once per sweep
__device__ __forceinline__ AtmV atm_derivs_sw(float4 qa, float4 qb, float C, float sA, float dA, float rc2s,
                                              float iw) {
    const float A = qa.x, B = qb.x;
    const float wc = rsqrtf(C);
    const float sv = qa.z * qb.z * wc;
    const float s2 = sv * sv;
    const float s5 = s2 * s2 * sv;
    const float S = A + B + C;
    const float t1 = fmaf(-2.0f, C, S), t2 = fmaf(-2.0f, B, S), t3 = fmaf(-2.0f, A, S);
    const float u = t2 * t3, v = t1 * t3, w = t1 * t2;
    const float K = 0.375f * (u + v + w);
    const float nP = -0.9375f * (t1 * u);
    const float a15 = -1.5f * A;
    const float vA = s5 * fmaf(nP, qa.y, fmaf(-0.75f, w, fmaf(-1.5f * B, C, K)));
    const float vB = s5 * fmaf(nP, qb.y, fmaf(-0.75f, v, fmaf(a15, C, K)));
    const float vC = s5 * fmaf(nP, wc * wc, fmaf(-0.75f, u, fmaf(a15, B, K)));
    const float Vn = s2 * sv + 0.375f * (t1 * u) * s5;   // V / nu
    float sB, dB, sC, dC;
    sw_eval(B, rc2s, iw, sB, dB);
    sw_eval(C, rc2s, iw, sC, dC);
    AtmV r;
    r.vA = sB * sC * (vA * sA + Vn * dA);
    r.vB = sA * sC * (vB * sB + Vn * dB);
    r.vC = sA * sB * (vC * sC + Vn * dC);
    return r;
}

// the round-robin sweep of one vertex: lane li = lane - gb owns staged
// neighbour li < m and plays rounds d = d_first .. d_last (at most m/2) over
// `rounds` loop trips (rounds past d_last do nothing); the lane's partial sum
// for its neighbour is returned in (ax, ay, az).  The vertex's own share is
// not summed here: per triplet g_i = -(g_a + g_b), so the vertex force is
// minus the sum of its neighbours' shares.
template <bool SW = false>
__device__ __forceinline__ void atm_sweep(const float4 *se, const float4 *sq, int m, int li, int gb, int d_first,
                                          int d_last, int rounds, float rc2, float &ax, float &ay, float &az,
                                          float4 &ea_out, float sw_iw = 0.f) {
    const bool own = li < m;
    const float4 ea = own ? se[li] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 qa = own ? sq[li] : make_float4(1.f, 1.f, 1.f, 0.f);
    ea_out = ea;
    float sA = 1.f, dA = 0.f;
    if (SW) sw_eval(qa.x, rc2, sw_iw, sA, dA);
    // the rounds this lane plays: d_first .. d_last, less the round d = m/2 for
    // the upper half of the lanes (that pair is played by the lower half)
    int t_act = own ? d_last - d_first + 1 : 0;
    if (own && (m & 1) == 0 && d_last == (m >> 1) && li >= (m >> 1)) t_act--;
    // partner b = li + d and share source li - d (mod m), stepped per round;
    // d <= m/2 keeps both within one wrap
    int b = li + d_first, src = li - d_first;
    if (b >= m) b -= m;
    if (src < 0) src += m;
    for (int t = 0; t < rounds; t++) {
        float bx = 0.f, by = 0.f, bz = 0.f;
        if (t < t_act) {
            const float4 eb = se[b];
            const float cx = eb.x - ea.x, cy = eb.y - ea.y, cz = eb.z - ea.z;
            const float C = cx * cx + cy * cy + cz * cz;
            if (C <= rc2) {
                const AtmV v = SW ? atm_derivs_sw(qa, sq[b], C, sA, dA, rc2, sw_iw) : atm_derivs(qa, sq[b], C);
                const float tx = v.vC * cx, ty = v.vC * cy, tz = v.vC * cz;
                ax += tx - v.vA * ea.x;
                ay += ty - v.vA * ea.y;
                az += tz - v.vA * ea.z;
                bx = -tx - v.vB * eb.x;
                by = -ty - v.vB * eb.y;
                bz = -tz - v.vB * eb.z;
            }
        }
        // lane li pulls the share computed, in this lane group, by the lane whose
        // partner it was.  In a round past d_last the source lane has no round
        // either and sends zero; lanes without a neighbour (li >= m) pull
        // whatever their index gives, and their sums are never used.
        const int s = src + gb;
        ax += __shfl_sync(0xffffffffu, bx, s);
        ay += __shfl_sync(0xffffffffu, by, s);
        az += __shfl_sync(0xffffffffu, bz, s);
        b = b + 1 == m ? 0 : b + 1;
        src = src == 0 ? m - 1 : src - 1;
    }
}

// vertices with more than 32 neighbours above them: a plain pair loop with a
// fixed-point atomic per contribution (rare at liquid densities); each
// contribution is scaled by sc first (1 keeps the units of 2 sign nu, and
// multiplying by 1 is exact)
template <bool SW = false>
__device__ __forceinline__ void atm_pairs_slow(const AtmParams &p, const float4 *se, const float4 *sq, int m, int lane, float rc2,
                               float &gx, float &gy, float &gz, float sc = 1.0f) {
    for (int a = lane; a < m; a += 32) {
        const float4 ea = se[a], qa = sq[a];
        float sA = 1.f, dA = 0.f;
        if (SW) sw_eval(qa.x, rc2, p.sw_iw, sA, dA);
        unsigned long long *acca = p.acc + 3 * (size_t)(__float_as_int(ea.w) >> 6);
        for (int b = a + 1; b < m; b++) {
            const float4 eb = se[b];
            const float cx = eb.x - ea.x, cy = eb.y - ea.y, cz = eb.z - ea.z;
            const float C = cx * cx + cy * cy + cz * cz;
            if (C > rc2) continue;
            const AtmV t = SW ? atm_derivs_sw(qa, sq[b], C, sA, dA, rc2, p.sw_iw) : atm_derivs(qa, sq[b], C);
            gx += t.vA * ea.x + t.vB * eb.x;
            gy += t.vA * ea.y + t.vB * eb.y;
            gz += t.vA * ea.z + t.vB * eb.z;
            unsigned long long *accb = p.acc + 3 * (size_t)(__float_as_int(eb.w) >> 6);
            atm_fix_add(acca, sc * (t.vC * cx - t.vA * ea.x));
            atm_fix_add(acca + 1, sc * (t.vC * cy - t.vA * ea.y));
            atm_fix_add(acca + 2, sc * (t.vC * cz - t.vA * ea.z));
            atm_fix_add(accb, sc * (-t.vC * cx - t.vB * eb.x));
            atm_fix_add(accb + 1, sc * (-t.vC * cy - t.vB * eb.y));
            atm_fix_add(accb + 2, sc * (-t.vC * cz - t.vB * eb.z));
        }
    }
}

__device__ __forceinline__ void atm_vertex_out(const AtmParams &p, int i, float gx, float gy, float gz) {
    atm_fix_add(p.acc + 3 * (size_t)i, gx);
    atm_fix_add(p.acc + 3 * (size_t)i + 1, gy);
    atm_fix_add(p.acc + 3 * (size_t)i + 2, gz);
}

// the sweep of one vertex whose m neighbours above it are staged in se / sq
// (e = r_i - r_x and code; |e|^2, 1/|e|^2, 1/|e|): with at most 16 the two
// half-warps split the rounds (lower and upper half of d), each delivering
// shares within itself, and their partial sums per neighbour are added; the
// neighbours' sums and the vertex's (minus their total) go to the fixed-point
// accumulators
__device__ __forceinline__ void atm_vertex(const AtmParams &p, int i, const float4 *se, const float4 *sq, int m,
                                           int lane, float rc2) {
    float gx = 0.f, gy = 0.f, gz = 0.f;
    const int half = m / 2;
    if (m <= 32) {
        float ax = 0.f, ay = 0.f, az = 0.f;
        float4 ea;
        if (m <= 16) {
            const int g = lane >> 4, li = lane & 15;
            const int h1 = (half + 1) / 2;                     // rounds of the lower half-warp
            const int d_first = g ? h1 + 1 : 1, d_last = g ? half : h1;
            atm_sweep(se, sq, m, li, 16 * g, d_first, d_last, h1, rc2, ax, ay, az, ea);
            ax += __shfl_xor_sync(0xffffffffu, ax, 16);
            ay += __shfl_xor_sync(0xffffffffu, ay, 16);
            az += __shfl_xor_sync(0xffffffffu, az, 16);
        } else {
            atm_sweep(se, sq, m, lane, 0, 1, half, half, rc2, ax, ay, az, ea);
        }
        if (lane < m) {
            unsigned long long *acc = p.acc + 3 * (size_t)(__float_as_int(ea.w) >> 6);
            atm_fix_add(acc, ax);
            atm_fix_add(acc + 1, ay);
            atm_fix_add(acc + 2, az);
            gx = -ax;
            gy = -ay;
            gz = -az;
        }
    } else {
        atm_pairs_slow(p, se, sq, m, lane, rc2, gx, gy, gz);
    }
    for (int o = 16; o > 0; o >>= 1) {
        gx += __shfl_xor_sync(0xffffffffu, gx, o);
        gy += __shfl_xor_sync(0xffffffffu, gy, o);
        gz += __shfl_xor_sync(0xffffffffu, gz, o);
    }
    if (lane == 0) atm_vertex_out(p, i, gx, gy, gz);
}

// the sweep of atm_vertex without its accumulator traffic, for the half-list
// pass that adds each neighbour's LJ reaction to its share before one
// fixed-point add per (vertex, neighbour): with m <= 32, lane li < m returns
// its neighbour's summed share in (ax, ay, az) and minus it in (gx, gy, gz)
// (the vertex's share is minus the neighbours' total); other lanes return
// zeros.  With m > 32 the plain pair loop adds every share, scaled by sc, to
// the accumulators itself, returns ax = ay = az = 0 and the lane's part of
// the vertex share in (gx, gy, gz).  Units: 2 sign nu.
template <bool SW>
__device__ __forceinline__ void atm_vertex_shares(const AtmParams &p, const float4 *se, const float4 *sq, int m, int lane,
                                                  float rc2, float sc, float &ax, float &ay, float &az, float &gx,
                                                  float &gy, float &gz) {
    ax = ay = az = gx = gy = gz = 0.f;
    const int half = m / 2;
    if (m <= 32) {
        float4 ea;
        if (m <= 16) {
            const int g = lane >> 4, li = lane & 15;
            const int h1 = (half + 1) / 2;                     // rounds of the lower half-warp
            const int d_first = g ? h1 + 1 : 1, d_last = g ? half : h1;
            atm_sweep<SW>(se, sq, m, li, 16 * g, d_first, d_last, h1, rc2, ax, ay, az, ea, p.sw_iw);
            ax += __shfl_xor_sync(0xffffffffu, ax, 16);
            ay += __shfl_xor_sync(0xffffffffu, ay, 16);
            az += __shfl_xor_sync(0xffffffffu, az, 16);
        } else {
            atm_sweep<SW>(se, sq, m, lane, 0, 1, half, half, rc2, ax, ay, az, ea, p.sw_iw);
        }
        if (lane < m) {
            gx = -ax;
            gy = -ay;
            gz = -az;
        } else {
            ax = ay = az = 0.f;
        }
    } else {
        atm_pairs_slow<SW>(p, se, sq, m, lane, rc2, gx, gy, gz, sc);
    }
}

}  // namespace komd
