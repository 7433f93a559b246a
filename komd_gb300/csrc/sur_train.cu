// sur_train.cu -- force-matched training of the learned three-body term
// (no reference counterpart).  FP32 SIMT kernels.
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
#include <cstdint>

#include "sur_device.cuh"
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
