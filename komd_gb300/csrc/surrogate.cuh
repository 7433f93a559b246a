// surrogate.cuh -- parameters of the learned three-body term (surrogate.cu).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace komd {

constexpr int kSurNR = 16;       // radial Gaussians
constexpr int kSurNC = 4;        // angular channels (4 invariants each)
constexpr int kSurNF = 32;       // features
constexpr int kSurH = 64;        // hidden width
constexpr int kSurNParam = kSurH * kSurNF + kSurH + kSurH * kSurH + kSurH + kSurH + 1;
constexpr float kSurEtaR = 50.0f;
constexpr float kSurEtaA = 22.222222f;   // 1 / (2 * 0.15^2)

struct SurParams {
    int n;
    float rc;
    const float4 *nl;            // ATM neighbour list (r_i - r_j, code)
    const int *nl_count;
    int nl_cap;
    const float *fmean, *fstd;   // fstd == nullptr: raw features (training samples)
    float *x;                    // n x 32 features
    float *mom;                  // n x 36 moments (M1 3 + M2 6 per channel)
    float *dedx;                 // n x 32 dE/dx
    float *e_site;               // n per-site energies (physical units)
    float *fsur;                 // n x 4 surrogate forces (slot order, xyz + pad, accumulated; 16-byte aligned)
    const __nv_bfloat16 *w1, *w1t, *w2, *w2t;
    const float *b1, *b2, *w3;
    float b3, e_scale, e_shift;
    int num_sms;                 // multiprocessors of the device (persistent MLP grid)
};

struct TrainParams {
    const float *X, *y;
    int n, batch;
    float *params, *grad, *m, *v, *work;
    float lr;
    uint32_t seed;
    int fixed_batch;             // 1: the batch is samples 0..batch-1 (gradient checks)
    int grad_only;
};

// force-matched training on captured snapshots (sur_train.cu).  A dataset
// holds snapshots of n_site sites each, in the cell (slot) order of the
// engine that captured them; neighbour entries are the engine's ATM list
// entries (r_i - r_j, code) whose code >> 6 is the neighbour's slot within
// the same snapshot.  A batch is a list of snapshot ids; batch site b is
// site b % n_site of snapshot snaps[b / n_site].
struct FitParams {
    const float4 *nl;
    const int *nl_count;
    int cap, n_site, nb;
    float rc;
    const float *x, *mom, *e3, *f3;      // raw features, moments, exact energies and forces (dataset order)
    const int *snaps;
    const float *params, *fmean, *fstd;
    float e_scale, e_shift;
    float lam_e, lam_f, inv_f2;          // loss weights; 1 / <|F_exact|^2> per site
    float *E, *g, *fs, *w, *rec;         // per batch site: energy, dE/dx, learned force, tangent, record
    double *loss;                        // [0] energy term, [1] force term (accumulated)
    __nv_bfloat16 *wf;                   // the weights in BF16 fragment order (tensor-core form)
    int tc;                              // 1: the network runs on the tensor cores (BF16 operands, FP32
                                         // accumulation); 0: FP32 SIMT
};
constexpr int kFitRec = 580;             // record stride (floats; the BF16 records of the tensor-core form fit)
constexpr int kFitWf = 2 * kSurH * kSurNF + 2 * kSurH * kSurH;   // BF16 elements of FitParams::wf

void launch_fit_capture(int n, const float4 *nl, const int *nl_count, int nl_cap, const float *x, const float *mom,
                        const double *e3_site, const double *f3_site, const int *slot_site, float4 *dnl,
                        int *dcount, int dcap, float *dx, float *dmom, float *de3, float *df3, int *dsite, int *err,
                        cudaStream_t st);
void launch_fit_step(FitParams &p, float *grad, cudaStream_t st);
void launch_fit_adam(float *params, const float *grad, float *m, float *v, float lr, int step, cudaStream_t st);

void launch_sur_desc(SurParams &p, cudaStream_t st);
void launch_sur_mlp(SurParams &p, cudaStream_t st);
void launch_sur_force(SurParams &p, cudaStream_t st);
void launch_sur_apply(SurParams &p, const int *slot_site, double *f, double *fout, cudaStream_t st);
void launch_sur_probe(int n, const double *fa, const double *fb, double *out2, cudaStream_t st);
void launch_sum_sites(int n, const float *e, double *out, cudaStream_t st);
void launch_train_step(TrainParams &t, int step, cudaStream_t st);

}  // namespace komd
