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
int kinetic_grid(const Engine &e);
size_t atm_smem(const Engine &e);
}  // namespace komd
