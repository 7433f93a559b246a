// surrogate.cu -- learned three-body term (no reference counterpart): a
// 32-64-64-1 tanh MLP on per-site descriptors stands in for the ATM triplet
// sum; forces are the analytic gradient of the learned energy.
//
// Descriptors of site i from its neighbours d_j = r_j - r_i inside cutoff_3b
// (the ATM neighbour list the LJ kernel writes), with fc = (cos(pi r/rc)+1)/2:
//   G_k  = sum_j exp(-eta_r (r - mu_k)^2) fc            k = 0..15
//   per channel c = 0..3, g_c = exp(-eta_a (r - mu_c)^2) fc:
//   M1_c = sum g_c u,  M2_c = sum g_c u u^T,
//   I1 = |M1|^2, I2 = M2:M2, I3 = M1.M2.M1, I4 = tr(M2^3)
// x = (raw - mean) / std;  E_i = e_scale * MLP(x) + e_shift.
// The oracle (oracle/komd_oracle.c, kor_sur_*) states the same definition in FP64.
//
// Kernels per step: k_sur_desc (features + moments), k_sur_mlp (tensor cores:
// mma.sync m16n8k16 BF16 -> FP32, forward and input-gradient backward with the
// activations kept in registers), k_sur_force (chain rule to the pair vectors,
// neighbour forces scattered with FP32 atomics), k_sur_apply.
// Energy-only training: k_train_fwdbwd / k_train_grad / k_train_adam (FP32
// SIMT); the force-matched trainer (sur_train.cu) runs its network on the
// tensor cores.
#include <cstdint>

#include "engine.cuh"
#include "kernels.cuh"
#include "sur_device.cuh"
#include "sur_mma.cuh"
#include "surrogate.cuh"

namespace komd {

// ---------------------------------------------------------------------------
// descriptors: one thread per slot (cell order), the 52 sums in registers
// ---------------------------------------------------------------------------
// features of slot i (standardised when p.fstd is set) to xo[0..31] and its
// moments to mo[0..35] (both 16-byte aligned; mo may be null)
__device__ __forceinline__ void sur_site_desc(const SurParams &p, int i, float *xo, float *mo) {
    const int ni = min(p.nl_count[i], p.nl_cap);
    float acc[kSurNR + kSurNC * 9];   // G (16), then per channel M1 (3) + M2 (6: xx xy xz yy yz zz)
#pragma unroll
    for (int k = 0; k < kSurNR + kSurNC * 9; k++) acc[k] = 0.f;
    const float4 *row = p.nl + (size_t)i * p.nl_cap;
    for (int k = 0; k < ni; k++) {
        SurNb q;
        if (!sur_nb(row[k], p.rc, q)) continue;
        float G[kSurNR];
        radial_basis(q.r, q.fc, 0.f, G, nullptr);
#pragma unroll
        for (int c = 0; c < kSurNR; c++) acc[c] += G[c];
#pragma unroll
        for (int c = 0; c < kSurNC; c++) {
            const float t = q.r - sur_mu_a(c);
            const float g = __expf(-kSurEtaA * t * t) * q.fc;
            float *m = acc + kSurNR + 9 * c;
            const float gx = g * q.u[0], gy = g * q.u[1], gz = g * q.u[2];
            m[0] += gx; m[1] += gy; m[2] += gz;
            m[3] += gx * q.u[0]; m[4] += gx * q.u[1]; m[5] += gx * q.u[2];
            m[6] += gy * q.u[1]; m[7] += gy * q.u[2]; m[8] += gz * q.u[2];
        }
    }
    float raw[kSurNF];
#pragma unroll
    for (int k = 0; k < kSurNR; k++) raw[k] = acc[k];
#pragma unroll
    for (int c = 0; c < kSurNC; c++) {
        const float *v = acc + kSurNR + 9 * c, *m = v + 3;
        float M[3][3], Mv[3], M2[3][3];
        sym_full(m, M);
#pragma unroll
        for (int x = 0; x < 3; x++) Mv[x] = M[x][0] * v[0] + M[x][1] * v[1] + M[x][2] * v[2];
#pragma unroll
        for (int x = 0; x < 3; x++)
#pragma unroll
            for (int y = 0; y < 3; y++) M2[x][y] = M[x][0] * M[0][y] + M[x][1] * M[1][y] + M[x][2] * M[2][y];
        float i2 = 0.f, i4 = 0.f;
#pragma unroll
        for (int x = 0; x < 3; x++)
#pragma unroll
            for (int y = 0; y < 3; y++) { i2 += M[x][y] * M[x][y]; i4 += M2[x][y] * M[y][x]; }
        raw[kSurNR + c] = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
        raw[kSurNR + kSurNC + c] = i2;
        raw[kSurNR + 2 * kSurNC + c] = v[0] * Mv[0] + v[1] * Mv[1] + v[2] * Mv[2];
        raw[kSurNR + 3 * kSurNC + c] = i4;
    }
    if (p.fstd) {
#pragma unroll
        for (int k = 0; k < kSurNF; k++) raw[k] = (raw[k] - p.fmean[k]) / p.fstd[k];
    }
    float4 *x4 = reinterpret_cast<float4 *>(xo);
#pragma unroll
    for (int k = 0; k < kSurNF / 4; k++) x4[k] = make_float4(raw[4 * k], raw[4 * k + 1], raw[4 * k + 2], raw[4 * k + 3]);
    if (mo) {
        float4 *m4 = reinterpret_cast<float4 *>(mo);
#pragma unroll
        for (int k = 0; k < kSurNC * 9 / 4; k++)
            m4[k] = make_float4(acc[kSurNR + 4 * k], acc[kSurNR + 4 * k + 1], acc[kSurNR + 4 * k + 2],
                                acc[kSurNR + 4 * k + 3]);
    }
}

__global__ void __launch_bounds__(128) k_sur_desc(SurParams p) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    sur_site_desc(p, i, p.x + (size_t)i * kSurNF, p.mom ? p.mom + (size_t)i * kSurNC * 9 : nullptr);
}


__device__ __forceinline__ void sur_stage_weights(const SurParams &p, __nv_bfloat16 *sW1, __nv_bfloat16 *sW1T,
                                                  __nv_bfloat16 *sW2, __nv_bfloat16 *sW2T, float *sb1, float *sb2,
                                                  float *sw3) {
    sur_stage(p.w1, p.w1t, p.w2, p.w2t, p.b1, p.b2, p.w3, sW1, sW1T, sW2, sW2T, sb1, sb2, sw3);
}

__global__ void __launch_bounds__(128) k_sur_mlp(SurParams p) {
    __shared__ __align__(16) __nv_bfloat16 sW1[kSurH * kSurNF], sW1T[kSurNF * kSurH], sW2[kSurH * kSurH],
        sW2T[kSurH * kSurH];
    __shared__ float sb1[kSurH], sb2[kSurH], sw3[kSurH];
    sur_stage_weights(p, sW1, sW1T, sW2, sW2T, sb1, sb2, sw3);
    __syncthreads();
    const SurW W{sW1, sW1T, sW2, sW2T, sb1, sb2, sw3};
    const int lane = threadIdx.x & 31, g = lane >> 2, tig = lane & 3;
    const int warp = blockIdx.x * 4 + (threadIdx.x >> 5);
    const int nwarps = gridDim.x * 4;
    const int ntiles = (p.n + 15) / 16;
    for (int tile = warp; tile < ntiles; tile += nwarps) {
        const int r0 = tile * 16 + g, r1 = r0 + 8;
        const bool v0 = r0 < p.n, v1 = r1 < p.n;
        float e0, e1;
        sur_mlp_tile(W, p.x + (size_t)r0 * kSurNF, p.x + (size_t)r1 * kSurNF, v0, v1, p.dedx + (size_t)r0 * kSurNF,
                     p.dedx + (size_t)r1 * kSurNF, e0, e1, lane);
        if (tig == 0) {
            if (v0) p.e_site[r0] = p.e_scale * (e0 + p.b3) + p.e_shift;
            if (v1) p.e_site[r1] = p.e_scale * (e1 + p.b3) + p.e_shift;
        }
    }
}

// ---------------------------------------------------------------------------
// forces: chain rule to the pair vectors, one thread per slot; the
// neighbour's share is scattered with float4 atomics into fsur (slot order,
// xyz + pad), the centre's share is summed in registers
// ---------------------------------------------------------------------------
// forces of slot i from its dE/dx row and moment row (16-byte aligned)
__device__ __forceinline__ void sur_site_force(const SurParams &p, int i, const float *dxr, const float *mor) {
    // dE_i / d raw = e_scale * dE/dx / std
    float dr[kSurNF];
    const float4 *dx = reinterpret_cast<const float4 *>(dxr);
#pragma unroll
    for (int k = 0; k < kSurNF / 4; k++) {
        const float4 t = dx[k];
        dr[4 * k] = t.x; dr[4 * k + 1] = t.y; dr[4 * k + 2] = t.z; dr[4 * k + 3] = t.w;
    }
#pragma unroll
    for (int k = 0; k < kSurNF; k++) dr[k] *= p.e_scale / p.fstd[k];
    float a[kSurNC][3], B[kSurNC][6];
    float mom[kSurNC * 9];
    const float4 *mo = reinterpret_cast<const float4 *>(mor);
#pragma unroll
    for (int k = 0; k < kSurNC * 9 / 4; k++) {
        const float4 t = mo[k];
        mom[4 * k] = t.x; mom[4 * k + 1] = t.y; mom[4 * k + 2] = t.z; mom[4 * k + 3] = t.w;
    }
#pragma unroll
    for (int c = 0; c < kSurNC; c++)
        sur_channel_coeffs(mom + 9 * c, mom + 9 * c + 3, dr[kSurNR + c], dr[kSurNR + kSurNC + c],
                           dr[kSurNR + 2 * kSurNC + c], dr[kSurNR + 3 * kSurNC + c], a[c], B[c]);
    const int ni = min(p.nl_count[i], p.nl_cap);
    const float4 *row = p.nl + (size_t)i * p.nl_cap;
    float4 *fs = reinterpret_cast<float4 *>(p.fsur);
    float fx = 0.f, fy = 0.f, fz = 0.f;
    for (int k = 0; k < ni; k++) {
        const float4 e = row[k];
        SurNb q;
        if (!sur_nb(e, p.rc, q)) continue;
        float h[3];
        sur_pair_grad(q, dr, a, B, h);
        // dE_i/dd_ij = h:  F_j -= h, F_i += h
        const int j = __float_as_int(e.w) >> 6;
        atomicAdd(&fs[j], make_float4(-h[0], -h[1], -h[2], 0.f));
        fx += h[0]; fy += h[1]; fz += h[2];
    }
    atomicAdd(&fs[i], make_float4(fx, fy, fz, 0.f));
}

__global__ void __launch_bounds__(128) k_sur_force(SurParams p) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    sur_site_force(p, i, p.dedx + (size_t)i * kSurNF, p.mom + (size_t)i * kSurNC * 9);
}

// f[site] += fsur[slot] (then fsur = 0); with fout, the surrogate force is
// written there instead (probe comparisons)
__global__ void k_sur_apply(int n, const int *__restrict__ slot_site, float *__restrict__ fsur, double *__restrict__ f,
                            double *__restrict__ fout) {
    const int slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= n) return;
    const int s = slot_site[slot];
    float4 *f4 = reinterpret_cast<float4 *>(fsur);
    const float4 v = f4[slot];
    f4[slot] = make_float4(0.f, 0.f, 0.f, 0.f);
    const double w[3] = {(double)v.x, (double)v.y, (double)v.z};
    for (int d = 0; d < 3; d++) {
        if (fout) fout[3 * s + d] = w[d];
        else f[3 * s + d] += w[d];
    }
}

// probe: sums of |f_a - f_b|^2 and |f_b|^2 over sites
__global__ void k_sur_probe(int n, const double *__restrict__ fa, const double *__restrict__ fb, double *out2) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    double d2 = 0.0, b2 = 0.0;
    if (s < n) {
        for (int d = 0; d < 3; d++) {
            const double x = fa[3 * s + d] - fb[3 * s + d];
            d2 += x * x;
            b2 += fb[3 * s + d] * fb[3 * s + d];
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        d2 += __shfl_xor_sync(0xffffffffu, d2, o);
        b2 += __shfl_xor_sync(0xffffffffu, b2, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&out2[0], d2);
        atomicAdd(&out2[1], b2);
    }
}

__global__ void k_sum_sites(int n, const float *__restrict__ e, double *out) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    double v = s < n ? (double)e[s] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(out, v);
}

// ---------------------------------------------------------------------------
// training (FP32 SIMT): per-site energy regression, mini-batch Adam
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t hash32(uint32_t x) {
    x ^= x >> 16; x *= 0x7feb352du; x ^= x >> 15; x *= 0x846ca68bu; x ^= x >> 16;
    return x;
}

// one thread per batch sample: forward, loss gradient, backward to dz1, dz2
__global__ void k_train_fwdbwd(TrainParams t, int step) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= t.batch) return;
    const int idx = t.fixed_batch ? b : (int)(hash32((uint32_t)(t.seed * 2654435761u) ^ hash32(step * 977 + b)) % (uint32_t)t.n);
    const float *x = t.X + (size_t)idx * kSurNF;
    const float *W1 = t.params, *b1 = W1 + kSurH * kSurNF, *W2 = b1 + kSurH, *b2 = W2 + kSurH * kSurH,
                *w3 = b2 + kSurH, *b3 = w3 + kSurH;
    float xl[kSurNF], h1[kSurH], h2[kSurH];
    for (int k = 0; k < kSurNF; k++) xl[k] = x[k];
    for (int o = 0; o < kSurH; o++) {
        float z = b1[o];
        for (int k = 0; k < kSurNF; k++) z += W1[o * kSurNF + k] * xl[k];
        h1[o] = tanhf(z);
    }
    for (int o = 0; o < kSurH; o++) {
        float z = b2[o];
        for (int k = 0; k < kSurH; k++) z += W2[o * kSurH + k] * h1[k];
        h2[o] = tanhf(z);
    }
    float E = b3[0];
    for (int k = 0; k < kSurH; k++) E += w3[k] * h2[k];
    const float err = E - t.y[idx];
    const float gE = 2.f * err / (float)t.batch;      // d(mean squared error)/dE
    float *rec = t.work + (size_t)b * (kSurNF + 4 * kSurH + 2);
    float *rx = rec, *rh1 = rx + kSurNF, *rdz1 = rh1 + kSurH, *rh2 = rdz1 + kSurH, *rdz2 = rh2 + kSurH;
    for (int k = 0; k < kSurNF; k++) rx[k] = xl[k];
    float dz2[kSurH];
    for (int o = 0; o < kSurH; o++) {
        dz2[o] = gE * w3[o] * (1.f - h2[o] * h2[o]);
        rh2[o] = h2[o];
        rdz2[o] = dz2[o];
        rh1[o] = h1[o];
    }
    for (int k = 0; k < kSurH; k++) {
        float s = 0.f;
        for (int o = 0; o < kSurH; o++) s += W2[o * kSurH + k] * dz2[o];
        rdz1[k] = s * (1.f - h1[k] * h1[k]);
    }
    rec[kSurNF + 4 * kSurH] = gE;
    rec[kSurNF + 4 * kSurH + 1] = err * err;
}

// one thread per parameter: gradient summed over the batch records
__global__ void k_train_grad(TrainParams t) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q > kSurNParam) return;
    const int stride = kSurNF + 4 * kSurH + 2;
    const int ob1 = kSurH * kSurNF, oW2 = ob1 + kSurH, ob2 = oW2 + kSurH * kSurH, ow3 = ob2 + kSurH,
              ob3 = ow3 + kSurH;
    float s = 0.f;
    for (int b = 0; b < t.batch; b++) {
        const float *rec = t.work + (size_t)b * stride;
        const float *rx = rec, *rh1 = rx + kSurNF, *rdz1 = rh1 + kSurH, *rh2 = rdz1 + kSurH, *rdz2 = rh2 + kSurH;
        if (q < ob1) s += rdz1[q / kSurNF] * rx[q % kSurNF];
        else if (q < oW2) s += rdz1[q - ob1];
        else if (q < ob2) s += rdz2[(q - oW2) / kSurH] * rh1[(q - oW2) % kSurH];
        else if (q < ow3) s += rdz2[q - ob2];
        else if (q < ob3) s += rec[kSurNF + 4 * kSurH] * rh2[q - ow3];
        else if (q == ob3) s += rec[kSurNF + 4 * kSurH];
        else s += rec[kSurNF + 4 * kSurH + 1];   // q == kSurNParam: the batch's summed squared error
    }
    t.grad[q] = s;
}

__global__ void k_train_adam(TrainParams t, int step) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= kSurNParam) return;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float g = t.grad[q];
    const float m = t.m[q] = b1 * t.m[q] + (1.f - b1) * g;
    const float v = t.v[q] = b2 * t.v[q] + (1.f - b2) * g * g;
    const float mh = m / (1.f - powf(b1, (float)(step + 1))), vh = v / (1.f - powf(b2, (float)(step + 1)));
    t.params[q] -= t.lr * mh / (sqrtf(vh) + eps);
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
void launch_sur_desc(SurParams &p, cudaStream_t st) { k_sur_desc<<<(p.n + 127) / 128, 128, 0, st>>>(p); }
void launch_sur_mlp(SurParams &p, cudaStream_t st) {
    const int tiles = (p.n + 15) / 16;
    int blocks = (tiles + 3) / 4;
    const int cap = 4 * (p.num_sms > 0 ? p.num_sms : 152);
    if (blocks > cap) blocks = cap;   // persistent: weights staged once per block
    k_sur_mlp<<<blocks, 128, 0, st>>>(p);
}
void launch_sur_force(SurParams &p, cudaStream_t st) { k_sur_force<<<(p.n + 127) / 128, 128, 0, st>>>(p); }
void launch_sur_apply(SurParams &p, const int *slot_site, double *f, double *fout, cudaStream_t st) {
    k_sur_apply<<<(p.n + 255) / 256, 256, 0, st>>>(p.n, slot_site, p.fsur, f, fout);
}
void launch_sur_probe(int n, const double *fa, const double *fb, double *out2, cudaStream_t st) {
    k_sur_probe<<<(n + 255) / 256, 256, 0, st>>>(n, fa, fb, out2);
}
void launch_sum_sites(int n, const float *e, double *out, cudaStream_t st) {
    k_sum_sites<<<(n + 255) / 256, 256, 0, st>>>(n, e, out);
}
void launch_train_step(TrainParams &t, int step, cudaStream_t st) {
    k_train_fwdbwd<<<(t.batch + 127) / 128, 128, 0, st>>>(t, step);
    k_train_grad<<<(kSurNParam + 1 + 127) / 128, 128, 0, st>>>(t);
    if (!t.grad_only) k_train_adam<<<(kSurNParam + 127) / 128, 128, 0, st>>>(t, step);
}

}  // namespace komd
