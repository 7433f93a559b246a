// sur_device.cuh -- per-neighbour arithmetic of the learned three-body term,
// shared by inference (surrogate.cu) and force-matched training (sur_train.cu).
//
// Site i, neighbour d = r_j - r_i, r = |d|, u = d / r, fc = (cos(pi r/rc)+1)/2:
//   radial   G_k = exp(-eta_r (r - mu_k)^2) fc,  mu_k = 0.85 + k * 1.15/15
//   channel  g_c = exp(-eta_a (r - mu_c)^2) fc,  mu_c = 1.05 + 0.25 c
//   M1_c = sum g_c u,  M2_c = sum g_c u u^T  (symmetric, stored xx xy xz yy yz zz)
//   I1 = |M1|^2, I2 = M2:M2, I3 = M1.M2.M1, I4 = tr(M2^3)
#pragma once
#include "surrogate.cuh"

namespace komd {

__device__ __forceinline__ float sur_mu_a(int c) { return 1.05f + 0.25f * (float)c; }

// radial Gaussians by the product recurrence exp(-eta (t - D)^2) = exp(-eta t^2) exp(2 eta D t) exp(-eta D^2);
// dG (optional) is d(G_k)/dr given dfc = d(fc)/dr
__device__ __forceinline__ void radial_basis(float r, float fc, float dfc, float *G, float *dG) {
    const float D = 1.15f / 15.0f;
    float t = r - 0.85f;
    float gk = __expf(-kSurEtaR * t * t);
    float up = __expf(2.0f * kSurEtaR * D * t);
    const float c1 = __expf(-kSurEtaR * D * D), c2 = c1 * c1;
#pragma unroll
    for (int k = 0; k < kSurNR; k++) {
        G[k] = gk * fc;
        if (dG) dG[k] = gk * (-2.0f * kSurEtaR * t * fc + dfc);
        gk = gk * up * c1;
        up = up * c2;
        t -= D;
    }
}

// neighbour geometry: returns false outside the cutoff
struct SurNb {
    float r, ir, u[3], fc, dfc;
};
__device__ __forceinline__ bool sur_nb(float4 e, float rc, SurNb &q) {
    const float dx = -e.x, dy = -e.y, dz = -e.z;    // list entries hold r_i - r_j
    q.r = sqrtf(dx * dx + dy * dy + dz * dz);
    if (!(q.r < rc) || q.r == 0.f) return false;
    const float pi_rc = 3.14159265358979f / rc;
    float sn, cs;
    __sincosf(pi_rc * q.r, &sn, &cs);
    q.fc = 0.5f * (cs + 1.0f);
    q.dfc = -0.5f * pi_rc * sn;
    q.ir = 1.0f / q.r;
    q.u[0] = dx * q.ir; q.u[1] = dy * q.ir; q.u[2] = dz * q.ir;
    return true;
}

// symmetric 3x3 from 6 components
__device__ __forceinline__ void sym_full(const float *m, float M[3][3]) {
    M[0][0] = m[0]; M[0][1] = m[1]; M[0][2] = m[2];
    M[1][0] = m[1]; M[1][1] = m[3]; M[1][2] = m[4];
    M[2][0] = m[2]; M[2][1] = m[4]; M[2][2] = m[5];
}

// dE/dM1_c = a, dE/dM2_c = B (6 components) from the moments of one channel
// (v = M1, m = M2) and dE/dI1..4 = e1..e4
__device__ __forceinline__ void sur_channel_coeffs(const float *v, const float *m, float e1, float e2, float e3,
                                                   float e4, float *a, float *B) {
    float M[3][3], Mv[3], M2[3][3];
    sym_full(m, M);
    for (int x = 0; x < 3; x++) Mv[x] = M[x][0] * v[0] + M[x][1] * v[1] + M[x][2] * v[2];
    for (int x = 0; x < 3; x++)
        for (int y = 0; y < 3; y++) M2[x][y] = M[x][0] * M[0][y] + M[x][1] * M[1][y] + M[x][2] * M[2][y];
    for (int x = 0; x < 3; x++) a[x] = 2.f * e1 * v[x] + 2.f * e3 * Mv[x];
    const int ix[6][2] = {{0, 0}, {0, 1}, {0, 2}, {1, 1}, {1, 2}, {2, 2}};
    for (int q = 0; q < 6; q++) {
        const int x = ix[q][0], y = ix[q][1];
        B[q] = 2.f * e2 * M[x][y] + e3 * v[x] * v[y] + 3.f * e4 * M2[x][y];
    }
}

// h = dE_i/dd for one neighbour, given the radial coefficients dr[0..16)
// (dE/dG_k) and the channel coefficients a, B
__device__ __forceinline__ void sur_pair_grad(const SurNb &q, const float *dr, const float (*a)[3],
                                              const float (*B)[6], float *h) {
    float G[kSurNR], dG[kSurNR];
    radial_basis(q.r, q.fc, q.dfc, G, dG);
    float sr = 0.f;
#pragma unroll
    for (int k = 0; k < kSurNR; k++) sr += dr[k] * dG[k];
    h[0] = sr * q.u[0]; h[1] = sr * q.u[1]; h[2] = sr * q.u[2];
    const float *u = q.u;
#pragma unroll
    for (int c = 0; c < kSurNC; c++) {
        const float t = q.r - sur_mu_a(c);
        const float ex = __expf(-kSurEtaA * t * t);
        const float gg = ex * q.fc, gp = ex * (-2.f * kSurEtaA * t * q.fc + q.dfc);
        const float ua = u[0] * a[c][0] + u[1] * a[c][1] + u[2] * a[c][2];
        const float Bu[3] = {B[c][0] * u[0] + B[c][1] * u[1] + B[c][2] * u[2],
                             B[c][1] * u[0] + B[c][3] * u[1] + B[c][4] * u[2],
                             B[c][2] * u[0] + B[c][4] * u[1] + B[c][5] * u[2]};
        const float uBu = u[0] * Bu[0] + u[1] * Bu[1] + u[2] * Bu[2];
        const float s1 = gp * (ua + uBu) - (gg * q.ir) * (ua + 2.f * uBu);
        for (int x = 0; x < 3; x++) h[x] += s1 * u[x] + (gg * q.ir) * (a[c][x] + 2.f * Bu[x]);
    }
}

}  // namespace komd
