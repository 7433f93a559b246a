// sur_train.cu -- force-matched training of the learned three-body term
// (no reference counterpart).
//
// Loss over a batch of nb sites (energies in the network's scaled units
// E = MLP(x), targets y = (e3 - e_shift) / e_scale; forces in physical units):
//   L = lam_e / nb * sum_b (E_b - y_b)^2 + lam_f * inv_f2 / nb * sum_b |F_b - F_exact_b|^2
// F = -grad of sum_i (e_scale E_i + e_shift), so L depends on the parameters
// through E_b and through g_b = dE_b/dx_b.  With the adjoint
//   w_b = dL/dg_b = -(2 lam_f inv_f2 / nb) (e_scale / std) * D_b,
//   D_bk = sum_j (dF_j - dF_b) . d raw_bk / d d_bj        (dF = F - F_exact)
// the parameter gradient is that of a_b E_b + w_b . g_b(theta) with a_b and w_b
// held fixed, and w . g is the forward-mode derivative of the network along w
// (a tangent pass), so one reverse sweep through value and tangent gives it.
//
// Kernels per step: k_fit_fwd (E, g), k_fit_force (learned forces, chain rule),
// k_fit_adjoint (residual, loss, w), k_fit_bwd (value + tangent reverse sweep
// into per-site records), k_fit_grad (records -> parameter gradient).
//
// Two forms of the network's part (fwd, bwd, grad).  The tensor-core form
// (FitParams::tc = 1, the default of komd_sur_fit) runs every contraction on
// mma.sync m16n8k16 with BF16 operands and FP32 accumulation: k_fit_pack
// rounds the weights to BF16 fragment order each step, k_fit_fwd_tc and
// k_fit_bwd_tc take one warp per 16 batch sites, and k_fit_grad_tc reduces the
// BF16 records over the batch as a GEMM (K = batch sites) from ldmatrix-loaded
// shared-memory tiles.  The FP32 SIMT form (thread per site) is kept for
// gradient checks at FP32 tolerance.  The descriptor chain rule (k_fit_force,
// k_fit_adjoint) is FP32 in both.
#include <cstdint>

#include "sur_device.cuh"
#include "sur_mma.cuh"
#include "surrogate.cuh"

namespace komd {

namespace {
constexpr int kOW1 = 0, kOb1 = kSurH * kSurNF, kOW2 = kOb1 + kSurH, kOb2 = kOW2 + kSurH * kSurH, kOw3 = kOb2 + kSurH,
              kOb3 = kOw3 + kSurH;
// record layout
constexpr int rX = 0, rW = 32, rH1 = 64, rHD1 = 128, rH2 = 192, rHD2 = 256, rZ1B = 320, rZD1B = 384, rZ2B = 448,
              rZD2B = 512, rA = 576;
static_assert(rA < kFitRec, "record stride");
}  // namespace

__device__ __forceinline__ size_t fit_site(const FitParams &p, int b) {
    return (size_t)p.snaps[b / p.n_site] * p.n_site + (size_t)(b % p.n_site);
}

// ---------------------------------------------------------------------------
// capture one snapshot: warp per slot; the destination pointers start at the
// snapshot's first site
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_fit_capture(int n, const float4 *__restrict__ nl, const int *__restrict__ nl_count,
                                                     int nl_cap, const float *__restrict__ x, const float *__restrict__ mom,
                                                     const double *__restrict__ e3_site, const double *__restrict__ f3_site,
                                                     const int *__restrict__ slot_site, float4 *dnl, int *dcount, int dcap,
                                                     float *dx, float *dmom, float *de3, float *df3, int *dsite, int *err) {
    const int lane = threadIdx.x & 31;
    const int i = blockIdx.x * 8 + (threadIdx.x >> 5);
    if (i >= n) return;
    const int c = nl_count[i];
    if (c > dcap && lane == 0) atomicExch(err, 1);
    const int cc = min(c, dcap);
    for (int k = lane; k < cc; k += 32) dnl[(size_t)i * dcap + k] = nl[(size_t)i * nl_cap + k];
    dx[(size_t)i * kSurNF + lane] = x[(size_t)i * kSurNF + lane];
    for (int k = lane; k < kSurNC * 9; k += 32) dmom[(size_t)i * kSurNC * 9 + k] = mom[(size_t)i * kSurNC * 9 + k];
    if (lane == 0) {
        const int s = slot_site[i];
        dcount[i] = cc;
        de3[i] = (float)e3_site[s];
        dsite[i] = s;
        for (int d = 0; d < 3; d++) df3[3 * i + d] = (float)f3_site[3 * s + d];
    }
}

// ---------------------------------------------------------------------------
// forward + input gradient, thread per batch site
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_fit_fwd(FitParams p) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    float le = 0.f;
    if (b < p.nb) {
        const size_t gs = fit_site(p, b);
        const float *W1 = p.params + kOW1, *b1 = p.params + kOb1, *W2 = p.params + kOW2, *b2 = p.params + kOb2,
                    *w3 = p.params + kOw3;
        float x[kSurNF], h1[kSurH], h2[kSurH];
        for (int k = 0; k < kSurNF; k++) x[k] = (p.x[gs * kSurNF + k] - p.fmean[k]) / p.fstd[k];
        for (int o = 0; o < kSurH; o++) {
            float z = b1[o];
            for (int k = 0; k < kSurNF; k++) z += W1[o * kSurNF + k] * x[k];
            h1[o] = tanhf(z);
        }
        float E = p.params[kOb3];
        for (int o = 0; o < kSurH; o++) {
            float z = b2[o];
            for (int k = 0; k < kSurH; k++) z += W2[o * kSurH + k] * h1[k];
            h2[o] = tanhf(z);
            E += w3[o] * h2[o];
        }
        // dE/dx = W1^T [(1 - h1^2) . W2^T [(1 - h2^2) . w3]]
        for (int o = 0; o < kSurH; o++) h2[o] = w3[o] * (1.f - h2[o] * h2[o]);
        for (int k = 0; k < kSurH; k++) {
            float s = 0.f;
            for (int o = 0; o < kSurH; o++) s += W2[o * kSurH + k] * h2[o];
            h1[k] = s * (1.f - h1[k] * h1[k]);
        }
        for (int k = 0; k < kSurNF; k++) {
            float s = 0.f;
            for (int o = 0; o < kSurH; o++) s += W1[o * kSurNF + k] * h1[o];
            p.g[(size_t)b * kSurNF + k] = s;
        }
        p.E[b] = E;
        const float y = (p.e3[gs] - p.e_shift) / p.e_scale;
        le = p.lam_e * (E - y) * (E - y) / (float)p.nb;
    }
    for (int o = 16; o > 0; o >>= 1) le += __shfl_xor_sync(0xffffffffu, le, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(&p.loss[0], (double)le);
}

// ---------------------------------------------------------------------------
// learned forces (warp per batch site), as k_sur_force
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_fit_force(FitParams p) {
    const int lane = threadIdx.x & 31;
    const int b = blockIdx.x * 8 + (threadIdx.x >> 5);
    if (b >= p.nb) return;
    const size_t gs = fit_site(p, b);
    const float drk = p.e_scale * p.g[(size_t)b * kSurNF + lane] / p.fstd[lane];
    float dr[kSurNF];
#pragma unroll
    for (int k = 0; k < kSurNF; k++) dr[k] = __shfl_sync(0xffffffffu, drk, k);
    float a[kSurNC][3], B[kSurNC][6];
    const float *mom = p.mom + gs * kSurNC * 9;
#pragma unroll
    for (int c = 0; c < kSurNC; c++)
        sur_channel_coeffs(mom + 9 * c, mom + 9 * c + 3, dr[kSurNR + c], dr[kSurNR + kSurNC + c],
                           dr[kSurNR + 2 * kSurNC + c], dr[kSurNR + 3 * kSurNC + c], a[c], B[c]);
    const int base = (b / p.n_site) * p.n_site;
    const int ni = p.nl_count[gs];
    float fx = 0.f, fy = 0.f, fz = 0.f;
    for (int k = lane; k < ni; k += 32) {
        const float4 e = p.nl[gs * p.cap + k];
        SurNb q;
        if (!sur_nb(e, p.rc, q)) continue;
        float h[3];
        sur_pair_grad(q, dr, a, B, h);
        const int j = base + (__float_as_int(e.w) >> 6);
        atomicAdd(&p.fs[3 * j], -h[0]);
        atomicAdd(&p.fs[3 * j + 1], -h[1]);
        atomicAdd(&p.fs[3 * j + 2], -h[2]);
        fx += h[0]; fy += h[1]; fz += h[2];
    }
    for (int o = 16; o > 0; o >>= 1) {
        fx += __shfl_xor_sync(0xffffffffu, fx, o);
        fy += __shfl_xor_sync(0xffffffffu, fy, o);
        fz += __shfl_xor_sync(0xffffffffu, fz, o);
    }
    if (lane == 0) {
        atomicAdd(&p.fs[3 * b], fx);
        atomicAdd(&p.fs[3 * b + 1], fy);
        atomicAdd(&p.fs[3 * b + 2], fz);
    }
}

// A:B of two symmetric matrices stored xx xy xz yy yz zz
__device__ __forceinline__ float sym_dot(const float *A, const float *B) {
    return A[0] * B[0] + A[3] * B[3] + A[5] * B[5] + 2.f * (A[1] * B[1] + A[2] * B[2] + A[4] * B[4]);
}

// ---------------------------------------------------------------------------
// residual, force loss and the adjoint w (warp per batch site)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_fit_adjoint(FitParams p) {
    const int lane = threadIdx.x & 31;
    const int b = blockIdx.x * 8 + (threadIdx.x >> 5);
    if (b >= p.nb) return;
    const size_t gs = fit_site(p, b);
    const size_t gbase = gs - (size_t)(b % p.n_site);
    const int base = (b / p.n_site) * p.n_site;
    float dFi[3];
    for (int d = 0; d < 3; d++) dFi[d] = p.fs[3 * b + d] - p.f3[3 * gs + d];
    if (lane == 0)
        atomicAdd(&p.loss[1], (double)(p.lam_f * p.inv_f2 * (dFi[0] * dFi[0] + dFi[1] * dFi[1] + dFi[2] * dFi[2]) /
                                       (float)p.nb));
    float acc[kSurNR + kSurNC * 9];      // directional derivatives: radial (16), per channel dM1 (3) + dM2 (6)
#pragma unroll
    for (int k = 0; k < kSurNR + kSurNC * 9; k++) acc[k] = 0.f;
    const int ni = p.nl_count[gs];
    for (int k = lane; k < ni; k += 32) {
        const float4 e = p.nl[gs * p.cap + k];
        SurNb q;
        if (!sur_nb(e, p.rc, q)) continue;
        const int jl = __float_as_int(e.w) >> 6;
        const int j = base + jl;
        const size_t gj = gbase + (size_t)jl;
        float dl[3];
        for (int d = 0; d < 3; d++) dl[d] = (p.fs[3 * j + d] - p.f3[3 * gj + d]) - dFi[d];
        const float *u = q.u;
        const float s = u[0] * dl[0] + u[1] * dl[1] + u[2] * dl[2];
        float G[kSurNR], dG[kSurNR];
        radial_basis(q.r, q.fc, q.dfc, G, dG);
#pragma unroll
        for (int c = 0; c < kSurNR; c++) acc[c] += dG[c] * s;
        const float pp[3] = {dl[0] - s * u[0], dl[1] - s * u[1], dl[2] - s * u[2]};
#pragma unroll
        for (int c = 0; c < kSurNC; c++) {
            const float t = q.r - sur_mu_a(c);
            const float ex = __expf(-kSurEtaA * t * t);
            const float gr = ex * q.fc * q.ir, gps = ex * (-2.f * kSurEtaA * t * q.fc + q.dfc) * s;
            float *m = acc + kSurNR + 9 * c;
            m[0] += gps * u[0] + gr * pp[0];
            m[1] += gps * u[1] + gr * pp[1];
            m[2] += gps * u[2] + gr * pp[2];
            m[3] += gps * u[0] * u[0] + gr * 2.f * pp[0] * u[0];
            m[4] += gps * u[0] * u[1] + gr * (pp[0] * u[1] + u[0] * pp[1]);
            m[5] += gps * u[0] * u[2] + gr * (pp[0] * u[2] + u[0] * pp[2]);
            m[6] += gps * u[1] * u[1] + gr * 2.f * pp[1] * u[1];
            m[7] += gps * u[1] * u[2] + gr * (pp[1] * u[2] + u[1] * pp[2]);
            m[8] += gps * u[2] * u[2] + gr * 2.f * pp[2] * u[2];
        }
    }
#pragma unroll
    for (int k = 0; k < kSurNR + kSurNC * 9; k++)
        for (int o = 16; o > 0; o >>= 1) acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], o);
    float D[kSurNF];
#pragma unroll
    for (int k = 0; k < kSurNR; k++) D[k] = acc[k];
    const float *mom = p.mom + gs * kSurNC * 9;
#pragma unroll
    for (int c = 0; c < kSurNC; c++) {
        const float *v = mom + 9 * c, *m = mom + 9 * c + 3;
        const float *dv = acc + kSurNR + 9 * c, *dm = acc + kSurNR + 9 * c + 3;
        float M[3][3], Mv[3], M2[6];
        sym_full(m, M);
        for (int x = 0; x < 3; x++) Mv[x] = M[x][0] * v[0] + M[x][1] * v[1] + M[x][2] * v[2];
        const int ix[6][2] = {{0, 0}, {0, 1}, {0, 2}, {1, 1}, {1, 2}, {2, 2}};
        for (int q = 0; q < 6; q++) {
            const int x = ix[q][0], y = ix[q][1];
            M2[q] = M[x][0] * M[0][y] + M[x][1] * M[1][y] + M[x][2] * M[2][y];
        }
        float dM[3][3];
        sym_full(dm, dM);
        float vdMv = 0.f;
        for (int x = 0; x < 3; x++)
            for (int y = 0; y < 3; y++) vdMv += v[x] * dM[x][y] * v[y];
        D[kSurNR + c] = 2.f * (v[0] * dv[0] + v[1] * dv[1] + v[2] * dv[2]);
        D[kSurNR + kSurNC + c] = 2.f * sym_dot(m, dm);
        D[kSurNR + 2 * kSurNC + c] = 2.f * (Mv[0] * dv[0] + Mv[1] * dv[1] + Mv[2] * dv[2]) + vdMv;
        D[kSurNR + 3 * kSurNC + c] = 3.f * sym_dot(M2, dm);
    }
    float dk = 0.f;
#pragma unroll
    for (int k = 0; k < kSurNF; k++)
        if (lane == k) dk = D[k];
    const float cf = 2.f * p.lam_f * p.inv_f2 / (float)p.nb;
    p.w[(size_t)b * kSurNF + lane] = -cf * (p.e_scale / p.fstd[lane]) * dk;
}

// ---------------------------------------------------------------------------
// reverse sweep through value and tangent (thread per batch site) -> record
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_fit_bwd(FitParams p) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= p.nb) return;
    const size_t gs = fit_site(p, b);
    const float *W1 = p.params + kOW1, *b1 = p.params + kOb1, *W2 = p.params + kOW2, *b2 = p.params + kOb2,
                *w3 = p.params + kOw3;
    float *rec = p.rec + (size_t)b * kFitRec;
    float x[kSurNF], w[kSurNF], h1[kSurH], hd1[kSurH], zd1[kSurH], h2[kSurH], zd2[kSurH];
    for (int k = 0; k < kSurNF; k++) {
        x[k] = (p.x[gs * kSurNF + k] - p.fmean[k]) / p.fstd[k];
        w[k] = p.w[(size_t)b * kSurNF + k];
        rec[rX + k] = x[k];
        rec[rW + k] = w[k];
    }
    for (int o = 0; o < kSurH; o++) {
        float z = b1[o], zd = 0.f;
        for (int k = 0; k < kSurNF; k++) {
            z += W1[o * kSurNF + k] * x[k];
            zd += W1[o * kSurNF + k] * w[k];
        }
        h1[o] = tanhf(z);
        zd1[o] = zd;
        hd1[o] = (1.f - h1[o] * h1[o]) * zd;
        rec[rH1 + o] = h1[o];
        rec[rHD1 + o] = hd1[o];
    }
    float E = p.params[kOb3];
    for (int o = 0; o < kSurH; o++) {
        float z = b2[o], zd = 0.f;
        for (int k = 0; k < kSurH; k++) {
            z += W2[o * kSurH + k] * h1[k];
            zd += W2[o * kSurH + k] * hd1[k];
        }
        h2[o] = tanhf(z);
        zd2[o] = zd;
        E += w3[o] * h2[o];
        rec[rH2 + o] = h2[o];
        rec[rHD2 + o] = (1.f - h2[o] * h2[o]) * zd;
    }
    const float y = (p.e3[gs] - p.e_shift) / p.e_scale;
    const float a = 2.f * p.lam_e * (E - y) / (float)p.nb;
    rec[rA] = a;
    // layer 2: z2b = s2 (a w3 - 2 h2 zd2 w3), zd2b = s2 w3  (reuse h2 for z2b, zd2 for zd2b)
    for (int o = 0; o < kSurH; o++) {
        const float s2 = 1.f - h2[o] * h2[o];
        const float z2b = s2 * (a * w3[o] - 2.f * h2[o] * zd2[o] * w3[o]);
        const float zd2b = s2 * w3[o];
        h2[o] = z2b;
        zd2[o] = zd2b;
        rec[rZ2B + o] = z2b;
        rec[rZD2B + o] = zd2b;
    }
    // layer 1
    for (int k = 0; k < kSurH; k++) {
        float h1b = 0.f, hd1b = 0.f;
        for (int o = 0; o < kSurH; o++) {
            h1b += W2[o * kSurH + k] * h2[o];
            hd1b += W2[o * kSurH + k] * zd2[o];
        }
        const float s1 = 1.f - h1[k] * h1[k];
        const float zd1b = s1 * hd1b;
        h1b -= 2.f * h1[k] * zd1[k] * hd1b;
        rec[rZ1B + k] = s1 * h1b;
        rec[rZD1B + k] = zd1b;
    }
}

// ---------------------------------------------------------------------------
// records -> parameter gradient: thread per parameter, blockIdx.y splits the
// batch into chunks of 256 sites (FP32 atomics into grad, zeroed by the caller)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_fit_grad(const float *__restrict__ rec, int nb, float *grad) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= kSurNParam) return;
    const int b0 = blockIdx.y * 256, b1 = min(nb, b0 + 256);
    float s = 0.f;
    if (q < kOb1) {
        const int o = q / kSurNF, k = q % kSurNF;
        for (int b = b0; b < b1; b++) {
            const float *r = rec + (size_t)b * kFitRec;
            s += r[rZ1B + o] * r[rX + k] + r[rZD1B + o] * r[rW + k];
        }
    } else if (q < kOW2) {
        for (int b = b0; b < b1; b++) s += rec[(size_t)b * kFitRec + rZ1B + (q - kOb1)];
    } else if (q < kOb2) {
        const int o = (q - kOW2) / kSurH, k = (q - kOW2) % kSurH;
        for (int b = b0; b < b1; b++) {
            const float *r = rec + (size_t)b * kFitRec;
            s += r[rZ2B + o] * r[rH1 + k] + r[rZD2B + o] * r[rHD1 + k];
        }
    } else if (q < kOw3) {
        for (int b = b0; b < b1; b++) s += rec[(size_t)b * kFitRec + rZ2B + (q - kOb2)];
    } else if (q < kOb3) {
        const int o = q - kOw3;
        for (int b = b0; b < b1; b++) {
            const float *r = rec + (size_t)b * kFitRec;
            s += r[rA] * r[rH2 + o] + r[rHD2 + o];
        }
    } else {
        for (int b = b0; b < b1; b++) s += rec[(size_t)b * kFitRec + rA];
    }
    atomicAdd(&grad[q], s);
}

__global__ void k_fit_adam(float *params, const float *__restrict__ grad, float *m, float *v, float lr, int step) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= kSurNParam) return;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float g = grad[q];
    const float mq = m[q] = b1 * m[q] + (1.f - b1) * g;
    const float vq = v[q] = b2 * v[q] + (1.f - b2) * g * g;
    const float mh = mq / (1.f - powf(b1, (float)(step + 1))), vh = vq / (1.f - powf(b2, (float)(step + 1)));
    params[q] -= lr * mh / (sqrtf(vh) + eps);
}


// ===========================================================================
// tensor-core form
// ===========================================================================
namespace {
// FitParams::wf: W1, W1^T, W2, W2^T as the N x K matrices of load_frag
constexpr int kWfW1 = 0, kWfW1T = kSurH * kSurNF, kWfW2 = 2 * kSurH * kSurNF, kWfW2T = kWfW2 + kSurH * kSurH;
static_assert(kWfW2T + kSurH * kSurH == kFitWf, "fragment buffer");
// BF16 record of one batch site (tensor-core form), element offsets:
//   left factors  Z1B | ZD1B (dW1), Z2B | ZD2B (dW2)
//   right factors X | W (dW1),  H1 | HD1 (dW2)
constexpr int tZ1B = 0, tZD1B = 64, tZ2B = 128, tZD2B = 192, tX = 256, tW = 288, tH1 = 320, tHD1 = 384, kRecTc = 448;
static_assert(kRecTc * 2 <= kFitRec * 4, "BF16 record inside the record stride");
constexpr int kGradChunk = 32;            // batch sites per shared-memory stage of k_fit_grad_tc
constexpr int kRecPad = kRecTc + 8;       // 912-byte rows: the 8 rows of an ldmatrix hit distinct banks
}  // namespace

// the weight matrices of the parameters, rounded to BF16, in the B-fragment
// order of load_frag (element (n, k) of an N x K matrix at
// ((t S + s) 32 + lane) 4 + j with n = 8t + lane/4, k = 16s + 2(lane%4) + (j%2) + 8(j/2))
__global__ void k_fit_pack(const float *__restrict__ params, __nv_bfloat16 *__restrict__ wf) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= kFitWf) return;
    const int which = e < kWfW1T ? 0 : e < kWfW2 ? 1 : e < kWfW2T ? 2 : 3;
    const int base = which == 0 ? kWfW1 : which == 1 ? kWfW1T : which == 2 ? kWfW2 : kWfW2T;
    const int K = which == 0 ? kSurNF : kSurH;
    const int q = e - base, j = q & 3, chunk = q >> 2, lane = chunk & 31, ts = chunk >> 5;
    const int S = K / 16, s = ts % S, t = ts / S;
    const int n = 8 * t + (lane >> 2), k = 16 * s + 2 * (lane & 3) + (j & 1) + 8 * (j >> 1);
    const float *W1 = params + kOW1, *W2 = params + kOW2;
    float v;
    if (which == 0) v = W1[n * kSurNF + k];        // W1 (64 x 32)
    else if (which == 1) v = W1[k * kSurNF + n];   // W1^T (32 x 64)
    else if (which == 2) v = W2[n * kSurH + k];    // W2
    else v = W2[k * kSurH + n];                    // W2^T
    wf[e] = __float2bfloat16(v);
}

// shared-memory copy of the BF16 weights and the FP32 biases (every block of
// the tensor-core kernels)
struct FitSmemW {
    __nv_bfloat16 w1[kSurH * kSurNF], w1t[kSurNF * kSurH], w2[kSurH * kSurH], w2t[kSurH * kSurH];
    float b1[kSurH], b2[kSurH], w3[kSurH];
};

__device__ __forceinline__ SurW fit_stage(const FitParams &p, FitSmemW &sw) {
    sur_stage(p.wf + kWfW1, p.wf + kWfW1T, p.wf + kWfW2, p.wf + kWfW2T, p.params + kOb1, p.params + kOb2,
              p.params + kOw3, sw.w1, sw.w1t, sw.w2, sw.w2t, sw.b1, sw.b2, sw.w3);
    __syncthreads();
    return SurW{sw.w1, sw.w1t, sw.w2, sw.w2t, sw.b1, sw.b2, sw.w3};
}

__device__ __forceinline__ float fit_target(const FitParams &p, int b) {
    return (p.e3[fit_site(p, b)] - p.e_shift) / p.e_scale;
}

// forward + input gradient of 16 batch sites per warp on the tensor cores:
// the tile's standardised features go to their g rows, which sur_mlp_tile
// overwrites with dE/dx
__global__ void __launch_bounds__(128) k_fit_fwd_tc(FitParams p) {
    __shared__ __align__(16) FitSmemW sw;
    const SurW W = fit_stage(p, sw);
    const int lane = threadIdx.x & 31, g = lane >> 2, tig = lane & 3;
    const int b0 = (blockIdx.x * 4 + (threadIdx.x >> 5)) * 16;
    float le = 0.f;
    if (b0 < p.nb) {
        for (int q = lane; q < 16 * kSurNF; q += 32) {
            const int b = b0 + q / kSurNF, k = q % kSurNF;
            if (b < p.nb) p.g[(size_t)b * kSurNF + k] = (p.x[fit_site(p, b) * kSurNF + k] - p.fmean[k]) / p.fstd[k];
        }
        __syncwarp();
        const int r0 = b0 + g, r1 = r0 + 8;
        const bool v0 = r0 < p.nb, v1 = r1 < p.nb;
        float *g0 = p.g + (size_t)min(r0, p.nb - 1) * kSurNF, *g1 = p.g + (size_t)min(r1, p.nb - 1) * kSurNF;
        float e0, e1;
        sur_mlp_tile(W, g0, g1, v0, v1, g0, g1, e0, e1, lane);
        if (tig == 0) {
            const float b3 = p.params[kOb3];
            if (v0) {
                const float E = e0 + b3, d = E - fit_target(p, r0);
                p.E[r0] = E;
                le += p.lam_e * d * d / (float)p.nb;
            }
            if (v1) {
                const float E = e1 + b3, d = E - fit_target(p, r1);
                p.E[r1] = E;
                le += p.lam_e * d * d / (float)p.nb;
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1) le += __shfl_xor_sync(0xffffffffu, le, o);
    if (lane == 0 && le != 0.f) atomicAdd(&p.loss[0], (double)le);
}

// sum over the 16 rows of a tile of one C-fragment column pair (rows g and
// g + 8 in q = 0, 1 and q = 2, 3): complete in the lanes with g == 0
__device__ __forceinline__ void tile_colsum(const float *c, float &s0, float &s1) {
    s0 = c[0] + c[2];
    s1 = c[1] + c[3];
#pragma unroll
    for (int o = 4; o < 32; o <<= 1) {
        s0 += __shfl_xor_sync(0xffffffffu, s0, o);
        s1 += __shfl_xor_sync(0xffffffffu, s1, o);
    }
}

__device__ __forceinline__ void st_bf16x2(__nv_bfloat16 *dst, uint32_t v) { *reinterpret_cast<uint32_t *>(dst) = v; }

// value + tangent forward and reverse sweep of 16 batch sites per warp on the
// tensor cores (the algebra of k_fit_bwd): the BF16 left and right factors of
// the weight gradients go to the records, and the gradients of the biases,
// the output weights and the output bias (column sums) straight into grad
__global__ void __launch_bounds__(128) k_fit_bwd_tc(FitParams p, float *grad) {
    __shared__ __align__(16) FitSmemW sw;
    const SurW W = fit_stage(p, sw);
    const int lane = threadIdx.x & 31, g = lane >> 2, tig = lane & 3;
    const int b0 = (blockIdx.x * 4 + (threadIdx.x >> 5)) * 16;
    if (b0 >= p.nb) return;
    const int r0 = b0 + g, r1 = r0 + 8;
    const bool v0 = r0 < p.nb, v1 = r1 < p.nb;
    const size_t s0 = v0 ? fit_site(p, r0) : 0, s1 = v1 ? fit_site(p, r1) : 0;
    __nv_bfloat16 *rec = reinterpret_cast<__nv_bfloat16 *>(p.rec);
    __nv_bfloat16 *q0 = rec + (size_t)(v0 ? r0 : 0) * kRecTc, *q1 = rec + (size_t)(v1 ? r1 : 0) * kRecTc;
    // A fragments of the standardised features and of the tangent w
    uint32_t ax[2][4], aw[2][4];
#pragma unroll
    for (int s = 0; s < 2; s++) {
        const int k = 16 * s + tig * 2;
        float x[2][4], w[2][4];   // [row][k, k + 1, k + 8, k + 9]
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const bool v = h ? v1 : v0;
            const size_t gs = h ? s1 : s0;
            const int b = h ? r1 : r0;
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const int kk = k + (u & 1) + 8 * (u >> 1);
                x[h][u] = v ? (p.x[gs * kSurNF + kk] - p.fmean[kk]) / p.fstd[kk] : 0.f;
                w[h][u] = v ? p.w[(size_t)b * kSurNF + kk] : 0.f;
            }
        }
        ax[s][0] = pack_bf16(x[0][0], x[0][1]);
        ax[s][1] = pack_bf16(x[1][0], x[1][1]);
        ax[s][2] = pack_bf16(x[0][2], x[0][3]);
        ax[s][3] = pack_bf16(x[1][2], x[1][3]);
        aw[s][0] = pack_bf16(w[0][0], w[0][1]);
        aw[s][1] = pack_bf16(w[1][0], w[1][1]);
        aw[s][2] = pack_bf16(w[0][2], w[0][3]);
        aw[s][3] = pack_bf16(w[1][2], w[1][3]);
        if (v0) {
            st_bf16x2(q0 + tX + k, ax[s][0]); st_bf16x2(q0 + tX + k + 8, ax[s][2]);
            st_bf16x2(q0 + tW + k, aw[s][0]); st_bf16x2(q0 + tW + k + 8, aw[s][2]);
        }
        if (v1) {
            st_bf16x2(q1 + tX + k, ax[s][1]); st_bf16x2(q1 + tX + k + 8, ax[s][3]);
            st_bf16x2(q1 + tW + k, aw[s][1]); st_bf16x2(q1 + tW + k + 8, aw[s][3]);
        }
    }
    // layer 1: Z1 = X W1^T + b1, ZD1 = W W1^T; H1 = tanh Z1, HD1 = (1 - H1^2) ZD1
    float h1[8][4], zd1[8][4];
#pragma unroll
    for (int t = 0; t < 8; t++) {
        const int c = t * 8 + tig * 2;
        float az[4] = {W.b1[c], W.b1[c + 1], W.b1[c], W.b1[c + 1]}, ad[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int s = 0; s < 2; s++) {
            uint32_t B0, B1;
            load_frag(W.w1, kSurNF / 16, t, s, lane, B0, B1);
            mma16816(az, ax[s], B0, B1);
            mma16816(ad, aw[s], B0, B1);
        }
#pragma unroll
        for (int q = 0; q < 4; q++) {
            h1[t][q] = tanh_fast(az[q]);
            zd1[t][q] = ad[q];
        }
    }
    uint32_t ah[4][4], ahd[4][4];
#pragma unroll
    for (int s = 0; s < 4; s++) {
#pragma unroll
        for (int u = 0; u < 2; u++) {
            const int t = 2 * s + u;
            ah[s][2 * u] = pack_bf16(h1[t][0], h1[t][1]);
            ah[s][2 * u + 1] = pack_bf16(h1[t][2], h1[t][3]);
            ahd[s][2 * u] = pack_bf16((1.f - h1[t][0] * h1[t][0]) * zd1[t][0], (1.f - h1[t][1] * h1[t][1]) * zd1[t][1]);
            ahd[s][2 * u + 1] =
                pack_bf16((1.f - h1[t][2] * h1[t][2]) * zd1[t][2], (1.f - h1[t][3] * h1[t][3]) * zd1[t][3]);
            const int c = t * 8 + tig * 2;
            if (v0) { st_bf16x2(q0 + tH1 + c, ah[s][2 * u]); st_bf16x2(q0 + tHD1 + c, ahd[s][2 * u]); }
            if (v1) { st_bf16x2(q1 + tH1 + c, ah[s][2 * u + 1]); st_bf16x2(q1 + tHD1 + c, ahd[s][2 * u + 1]); }
        }
    }
    // layer 2: Z2 = H1 W2^T + b2, ZD2 = HD1 W2^T; H2 = tanh Z2
    float h2[8][4], zd2[8][4];
#pragma unroll
    for (int t = 0; t < 8; t++) {
        const int c = t * 8 + tig * 2;
        float az[4] = {W.b2[c], W.b2[c + 1], W.b2[c], W.b2[c + 1]}, ad[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int s = 0; s < 4; s++) {
            uint32_t B0, B1;
            load_frag(W.w2, kSurH / 16, t, s, lane, B0, B1);
            mma16816(az, ah[s], B0, B1);
            mma16816(ad, ahd[s], B0, B1);
        }
#pragma unroll
        for (int q = 0; q < 4; q++) {
            h2[t][q] = tanh_fast(az[q]);
            zd2[t][q] = ad[q];
        }
    }
    // E = w3 . H2 + b3 and a = dL/dE (zero for rows past the batch)
    float e0 = 0.f, e1 = 0.f;
#pragma unroll
    for (int t = 0; t < 8; t++) {
        const int c = t * 8 + tig * 2;
        e0 += W.w3[c] * h2[t][0] + W.w3[c + 1] * h2[t][1];
        e1 += W.w3[c] * h2[t][2] + W.w3[c + 1] * h2[t][3];
    }
    e0 += __shfl_xor_sync(0xffffffffu, e0, 1);
    e0 += __shfl_xor_sync(0xffffffffu, e0, 2);
    e1 += __shfl_xor_sync(0xffffffffu, e1, 1);
    e1 += __shfl_xor_sync(0xffffffffu, e1, 2);
    const float b3 = p.params[kOb3];
    const float a0 = v0 ? 2.f * p.lam_e * (e0 + b3 - fit_target(p, r0)) / (float)p.nb : 0.f;
    const float a1 = v1 ? 2.f * p.lam_e * (e1 + b3 - fit_target(p, r1)) / (float)p.nb : 0.f;
    const float m0 = v0 ? 1.f : 0.f, m1 = v1 ? 1.f : 0.f;
    // layer 2 reverse: z2b = s2 (a w3 - 2 h2 zd2 w3), zd2b = s2 w3 (s2 = 1 - h2^2);
    // output weight gradient a h2 + s2 zd2 and b2 gradient z2b as column sums
#pragma unroll
    for (int t = 0; t < 8; t++) {
        const int c = t * 8 + tig * 2;
        float g3[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const float a = q < 2 ? a0 : a1, m = q < 2 ? m0 : m1, w3 = W.w3[c + (q & 1)];
            const float s2 = 1.f - h2[t][q] * h2[t][q];
            g3[q] = m * (a * h2[t][q] + s2 * zd2[t][q]);
            const float z2b = s2 * (a * w3 - 2.f * h2[t][q] * zd2[t][q] * w3);
            h2[t][q] = m * z2b;          // h2 now holds z2b
            zd2[t][q] = m * s2 * w3;     // zd2 now holds zd2b
        }
        float sa, sb;
        tile_colsum(g3, sa, sb);
        if (g == 0) { atomicAdd(&grad[kOw3 + c], sa); atomicAdd(&grad[kOw3 + c + 1], sb); }
        tile_colsum(h2[t], sa, sb);
        if (g == 0) { atomicAdd(&grad[kOb2 + c], sa); atomicAdd(&grad[kOb2 + c + 1], sb); }
    }
    {
        float sa = a0 + a1;
#pragma unroll
        for (int o = 4; o < 32; o <<= 1) sa += __shfl_xor_sync(0xffffffffu, sa, o);
        if (lane == 0) atomicAdd(&grad[kOb3], sa);
    }
    uint32_t az2[4][4], azd2[4][4];
#pragma unroll
    for (int s = 0; s < 4; s++) {
#pragma unroll
        for (int u = 0; u < 2; u++) {
            const int t = 2 * s + u;
            az2[s][2 * u] = pack_bf16(h2[t][0], h2[t][1]);
            az2[s][2 * u + 1] = pack_bf16(h2[t][2], h2[t][3]);
            azd2[s][2 * u] = pack_bf16(zd2[t][0], zd2[t][1]);
            azd2[s][2 * u + 1] = pack_bf16(zd2[t][2], zd2[t][3]);
            const int c = t * 8 + tig * 2;
            if (v0) { st_bf16x2(q0 + tZ2B + c, az2[s][2 * u]); st_bf16x2(q0 + tZD2B + c, azd2[s][2 * u]); }
            if (v1) { st_bf16x2(q1 + tZ2B + c, az2[s][2 * u + 1]); st_bf16x2(q1 + tZD2B + c, azd2[s][2 * u + 1]); }
        }
    }
    // layer 1 reverse: h1b = z2b W2, hd1b = zd2b W2 (B = W2^T rows);
    // z1b = s1 (h1b - 2 h1 zd1 hd1b), zd1b = s1 hd1b; b1 gradient z1b
#pragma unroll
    for (int t = 0; t < 8; t++) {
        float hb[4] = {0.f, 0.f, 0.f, 0.f}, hdb[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int s = 0; s < 4; s++) {
            uint32_t B0, B1;
            load_frag(W.w2t, kSurH / 16, t, s, lane, B0, B1);
            mma16816(hb, az2[s], B0, B1);
            mma16816(hdb, azd2[s], B0, B1);
        }
        float z1b[4], zd1b[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const float m = q < 2 ? m0 : m1;
            const float s1 = 1.f - h1[t][q] * h1[t][q];
            z1b[q] = m * s1 * (hb[q] - 2.f * h1[t][q] * zd1[t][q] * hdb[q]);
            zd1b[q] = m * s1 * hdb[q];
        }
        const int c = t * 8 + tig * 2;
        if (v0) {
            st_bf16x2(q0 + tZ1B + c, pack_bf16(z1b[0], z1b[1]));
            st_bf16x2(q0 + tZD1B + c, pack_bf16(zd1b[0], zd1b[1]));
        }
        if (v1) {
            st_bf16x2(q1 + tZ1B + c, pack_bf16(z1b[2], z1b[3]));
            st_bf16x2(q1 + tZD1B + c, pack_bf16(zd1b[2], zd1b[3]));
        }
        float sa, sb;
        tile_colsum(z1b, sa, sb);
        if (g == 0) { atomicAdd(&grad[kOb1 + c], sa); atomicAdd(&grad[kOb1 + c + 1], sb); }
    }
}

// four 8x8 BF16 matrices from shared memory, transposed (ldmatrix .trans):
// lane l gives the address of row l % 8 of matrix l / 8
__device__ __forceinline__ void ldsm_x4_t(const __nv_bfloat16 *row, uint32_t &d0, uint32_t &d1, uint32_t &d2,
                                          uint32_t &d3) {
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(row);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];"
                 : "=r"(d0), "=r"(d1), "=r"(d2), "=r"(d3)
                 : "r"(a));
}

// weight gradients from the records as a GEMM over the batch (K = sites):
//   dW1 = Z1B^T X + ZD1B^T W (64 x 32),  dW2 = Z2B^T H1 + ZD2B^T HD1 (64 x 64)
// A block stages 32 sites at a time; warp w owns the rows 16 (w / 2) .. +15
// and six 8-column tiles: W1 columns 0-31 and W2 columns 0-15 (w even) or W2
// columns 16-63 (w odd).  Each block adds its sums to grad once.
__global__ void __launch_bounds__(256) k_fit_grad_tc(const __nv_bfloat16 *__restrict__ rec, int nb, float *grad) {
    __shared__ __align__(16) __nv_bfloat16 s[kGradChunk * kRecPad];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, g = lane >> 2, tig = lane & 3;
    const int m = warp >> 1, odd = warp & 1;
    const int mi = lane >> 3, li = lane & 7;
    float acc[6][4];
#pragma unroll
    for (int j = 0; j < 6; j++)
#pragma unroll
        for (int q = 0; q < 4; q++) acc[j][q] = 0.f;
    const int nchunk = (nb + kGradChunk - 1) / kGradChunk;
    for (int ch = blockIdx.x; ch < nchunk; ch += gridDim.x) {
        __syncthreads();
        const int base = ch * kGradChunk;
        for (int e = threadIdx.x; e < kGradChunk * (kRecTc / 8); e += blockDim.x) {
            const int r = e / (kRecTc / 8), c = e % (kRecTc / 8);
            uint4 v = make_uint4(0u, 0u, 0u, 0u);
            if (base + r < nb) v = reinterpret_cast<const uint4 *>(rec + (size_t)(base + r) * kRecTc)[c];
            reinterpret_cast<uint4 *>(s + r * kRecPad)[c] = v;
        }
        __syncthreads();
#pragma unroll
        for (int kb = 0; kb < kGradChunk; kb += 16) {
            // A (this warp's rows o x sites kb..kb+15): matrices (sites +0 / +8) x (o +0 / +8)
            const int ar = kb + li + ((mi & 2) ? 8 : 0), ac = 16 * m + ((mi & 1) ? 8 : 0);
            // B (sites kb..kb+15 x 16 columns): matrices (sites +0 / +8) x (columns +0 / +8)
            const int br = kb + li + ((mi & 1) ? 8 : 0), bc = (mi & 2) ? 8 : 0;
#pragma unroll
            for (int term = 0; term < 2; term++) {
                uint32_t a[4], b[4];
                if (!odd) {
                    // W1: columns 0-31 (tiles 0-3)
                    ldsm_x4_t(s + ar * kRecPad + (term ? tZD1B : tZ1B) + ac, a[0], a[1], a[2], a[3]);
#pragma unroll
                    for (int h = 0; h < 2; h++) {
                        ldsm_x4_t(s + br * kRecPad + (term ? tW : tX) + 16 * h + bc, b[0], b[1], b[2], b[3]);
                        mma16816(acc[2 * h], a, b[0], b[1]);
                        mma16816(acc[2 * h + 1], a, b[2], b[3]);
                    }
                    // W2: columns 0-15 (tiles 4-5)
                    ldsm_x4_t(s + ar * kRecPad + (term ? tZD2B : tZ2B) + ac, a[0], a[1], a[2], a[3]);
                    ldsm_x4_t(s + br * kRecPad + (term ? tHD1 : tH1) + bc, b[0], b[1], b[2], b[3]);
                    mma16816(acc[4], a, b[0], b[1]);
                    mma16816(acc[5], a, b[2], b[3]);
                } else {
                    // W2: columns 16-63 (tiles 0-5)
                    ldsm_x4_t(s + ar * kRecPad + (term ? tZD2B : tZ2B) + ac, a[0], a[1], a[2], a[3]);
#pragma unroll
                    for (int h = 0; h < 3; h++) {
                        ldsm_x4_t(s + br * kRecPad + (term ? tHD1 : tH1) + 16 + 16 * h + bc, b[0], b[1], b[2], b[3]);
                        mma16816(acc[2 * h], a, b[0], b[1]);
                        mma16816(acc[2 * h + 1], a, b[2], b[3]);
                    }
                }
            }
        }
    }
    // C fragment: rows o = 16 m + g (+8), columns 8 j + 2 tig (+1) of the tile
#pragma unroll
    for (int j = 0; j < 6; j++) {
        int off, ld, col;
        if (!odd && j < 4) { off = kOW1; ld = kSurNF; col = 8 * j; }
        else { off = kOW2; ld = kSurH; col = odd ? 16 + 8 * j : 8 * (j - 4); }
        const int o = 16 * m + g, c = col + 2 * tig;
        atomicAdd(&grad[off + o * ld + c], acc[j][0]);
        atomicAdd(&grad[off + o * ld + c + 1], acc[j][1]);
        atomicAdd(&grad[off + (o + 8) * ld + c], acc[j][2]);
        atomicAdd(&grad[off + (o + 8) * ld + c + 1], acc[j][3]);
    }
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
void launch_fit_capture(int n, const float4 *nl, const int *nl_count, int nl_cap, const float *x, const float *mom,
                        const double *e3_site, const double *f3_site, const int *slot_site, float4 *dnl,
                        int *dcount, int dcap, float *dx, float *dmom, float *de3, float *df3, int *dsite, int *err,
                        cudaStream_t st) {
    k_fit_capture<<<(n + 7) / 8, 256, 0, st>>>(n, nl, nl_count, nl_cap, x, mom, e3_site, f3_site, slot_site, dnl,
                                               dcount, dcap, dx, dmom, de3, df3, dsite, err);
}

// fs (nb x 3) and grad (kSurNParam) must be zero on entry
void launch_fit_step(FitParams &p, float *grad, cudaStream_t st) {
    if (p.tc) {
        const int tiles = (p.nb + 15) / 16;
        const int chunks = (p.nb + kGradChunk - 1) / kGradChunk;
        k_fit_pack<<<(kFitWf + 255) / 256, 256, 0, st>>>(p.params, p.wf);
        k_fit_fwd_tc<<<(tiles + 3) / 4, 128, 0, st>>>(p);
        k_fit_force<<<(p.nb + 7) / 8, 256, 0, st>>>(p);
        k_fit_adjoint<<<(p.nb + 7) / 8, 256, 0, st>>>(p);
        k_fit_bwd_tc<<<(tiles + 3) / 4, 128, 0, st>>>(p, grad);
        k_fit_grad_tc<<<chunks < 256 ? chunks : 256, 256, 0, st>>>(reinterpret_cast<const __nv_bfloat16 *>(p.rec),
                                                                   p.nb, grad);
        return;
    }
    k_fit_fwd<<<(p.nb + 127) / 128, 128, 0, st>>>(p);
    k_fit_force<<<(p.nb + 7) / 8, 256, 0, st>>>(p);
    k_fit_adjoint<<<(p.nb + 7) / 8, 256, 0, st>>>(p);
    k_fit_bwd<<<(p.nb + 127) / 128, 128, 0, st>>>(p);
    k_fit_grad<<<dim3((kSurNParam + 127) / 128, (p.nb + 255) / 256), 128, 0, st>>>(p.rec, p.nb, grad);
}

void launch_fit_adam(float *params, const float *grad, float *m, float *v, float lr, int step, cudaStream_t st) {
    k_fit_adam<<<(kSurNParam + 127) / 128, 128, 0, st>>>(params, grad, m, v, lr, step);
}

}  // namespace komd
