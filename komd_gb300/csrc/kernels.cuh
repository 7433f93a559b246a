// kernels.cuh -- launchers of the hot-path kernels (kernels.cu).
#pragma once
#include "engine.cuh"

namespace komd {
void launch_container(Engine &e, cudaStream_t st);
int launch_pair(Engine &e, cudaStream_t st, bool measure, double *lj_hist);
void launch_pair_tile(PairParams &p, int ncell, bool measure, bool emit, cudaStream_t st);
PairParams pair_params(Engine &e);
void launch_vlist_build(Engine &e, cudaStream_t st);
int launch_lj_vlist(Engine &e, PairParams &p, bool measure, bool emit, cudaStream_t st);
int vlist_grid(const Engine &e);
void launch_counts(Engine &e, cudaStream_t st);
void launch_bonded(Engine &e, cudaStream_t st, bool measure, double *acc);
void launch_limit(Engine &e, cudaStream_t st);
// ATM forces; with_step1 (step graphs only) lets the FULL FP32 path fuse
// integrate1 into its flush: returns true when it did
bool launch_atm(Engine &e, cudaStream_t st, bool measure, bool with_step1 = false);
AtmParams atm_params(const Engine &e);
// force_units: the sums are in force units (half-list pass), else in units of 2 sign nu
bool launch_atm_flush(Engine &e, cudaStream_t st, bool with_step1, bool force_units);
// LJ forces and the once-per-triplet ATM sweep in one pass (FP32, FULL, Verlet)
void launch_lj_atm(Engine &e, cudaStream_t st);
// true when launch_lj_atm runs the half-list form, whose fixed-point sums are
// in force units (the flush scale is 2^-32) instead of units of 2 sign nu
bool lj_atm_half(const Engine &e);
// the per-slot FP32 force buffer of the half-list pass, or null where f
// receives the pass's forces directly (terms that add to f before the flush)
float4 *half_own(const Engine &e);
// LJ on and no ATM2B factor: the half-list pass reads neither per pair
bool half_plain(const PairParams &p);
// in_step (step graphs only): the fused drift path when the engine qualifies
void launch_step0(Engine &e, cudaStream_t st, bool in_step = false);
void launch_step1(Engine &e, cudaStream_t st);
void launch_kinetic(Engine &e, cudaStream_t st, int n_terms);
void launch_velocity_scale(Engine &e, cudaStream_t st, const double *acc, double beta);
void launch_pair_table(Engine &e, cudaStream_t st);
void launch_sum_partials(cudaStream_t st, int nblocks, const double *partials, double *out);
void launch_rdf(Engine &e, cudaStream_t st, double *bins, bool cells);
void launch_rdf_bins(Engine &e, cudaStream_t st, double *bins, bool cells, double max_r, double dr, int64_t nbins);
void set_kernel_attributes(Engine &e);
int atm_grid(const Engine &e);

// ---- packed replicas: one launch per stage of the step for all replicas of a
// batch.  Each stage has a device array of per-replica arguments and the
// first block of every replica (start[r] .. start[r + 1] - 1; start[nrep] is
// the stage's grid); a block runs the stage's body for its replica with its
// index inside that replica's range.
struct PackedStage {
    void *args = nullptr;     // device array of the stage's argument structs
    int *start = nullptr;     // device, nrep + 1 entries
    int blocks = 0;
};
struct PackedStep {
    int nrep = 0;
    PackedStage step0, bin, scan, scatter, sort, vbuild, force, flush;
    int *two = nullptr;       // per replica: the two-home form of the list build
    PairParams *pp = nullptr; // per replica (list build and force pass)
    AtmParams *ap = nullptr;
    float *sa = nullptr;      // per replica: 2 sign nu
    int *n = nullptr, *per = nullptr;
    size_t force_smem = 0;    // the largest replica's staging
    bool uniform = true, sw = false;
    bool plain = false;       // every replica: LJ on, no ATM2B factor (the half-list pass's PLAIN form)
};
BinArgs bin_args(const Engine &e);
ScanArgs scan_args(const Engine &e);
ScatterArgs scatter_args(const Engine &e);
SortArgs sort_args(const Engine &e);
Step0Args step0_args(const Engine &e);
FlushArgs flush_args(const Engine &e, double scale_fix, const float4 *own = nullptr);
int vlist_per(const Engine &e);
size_t lj_atm_half_smem(const Engine &e);
// the blocks a stage gives one replica (the same shapes as the single-system launches)
int packed_blocks_container(const Engine &e);
int packed_blocks_vbuild(const Engine &e);
bool vbuild_two(const Engine &e);
void launch_packed_step(const PackedStep &pk, cudaStream_t st);          // kernels.cu: all eight stages
void launch_packed_pair_stages(const PackedStep &pk, cudaStream_t st, bool vbuild);   // pair_tile.cu
int kinetic_grid(const Engine &e);
size_t atm_smem(const Engine &e);
}  // namespace komd
