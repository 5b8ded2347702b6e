// dvm_internal.h -- argument records shared by the kernel TU and the C-ABI TU.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "dvm_device.cuh"

namespace dvm {

constexpr int kCollideChunk = 256;  // threads per collide CTA
constexpr int kChunkSamples = 32;   // samples per chunk of one (cell, sub-integral): a warp
// A warp takes a run of consecutive chunks of one (cell, sub-integral) per visit: the runs
// are visited in a scattered order and a warp walks its run's chunks in turn, one lookup of
// the run's (cell, sub-integral) per run. Measured on the benchmark shock at fixed run
// lengths of 1, 2, 4, 8, 16, 32, 64 chunks: FP64 collide 5.44, 5.46, 5.45, 5.34, 5.25,
// 5.32, 5.58 ms; FP32 3.58, 3.58, 3.40, 3.33, 3.28, 3.31, 3.47 ms. Launches with few
// samples per warp need short runs (the cavity's FP32 collide went from 0.28 to 0.35 ms at
// 16), so k_plan picks the length per launch: as many chunks as leave each warp of the
// collide launch about kRunsPerWarp runs, between 1 and kRunChunks. It is stored in the top
// bits of the last chunk offset (chunk_off[3C] = runs | length << kRunShift).
constexpr int kRunChunks = 16;
constexpr long long kRunsPerWarp = 16;
constexpr int kRunShift = 56;
constexpr long long kRunMask = (1ll << kRunShift) - 1;

// Samples and depletion factor of each sub-integral of one cell-step
// (variance_reduction.f90:669-683, 822-835, 967-981; full_mc.f90:330-331).
struct CellPlan {
  long long num[3];
  double factor[3];
};

// A recorded collision list on the device (dvm_pairlist).
struct PairDev {
  int active;
  long long count[3];
  const int* glA[3];
  const int* glB[3];
  const double* rA[3];
  const double* rB[3];
  const double* rphi[3];
  const double* rcos[3];
};

// Scalars every collision kernel needs.
struct CollParams {
  int method;          // DVM_COLL_VR or DVM_COLL_FMC
  int samples_mode;
  long long samples_per_step;
  int num_repl;
  double mass, omega, alpha, sigma, dt, Kn, coln_rms, cdf_tolerance;
  double pi;
  uint64_t seed;
  double b3;           // mass-weighted beta3_min of compute_num_coll_pairs (host-computed)
};

cudaError_t launch_step_end(uint32_t* counter, long long* acc, const long long* total,
                            cudaStream_t s);

// Moments kept per cell for the equilibrium cache of k_cdf: dens, u, v, temp (the
// renewal test) and w (the cached equilibrium was built with it).
constexpr int kEqCache = 5;

struct CdfArgs {
  GridInfo g;
  CollParams cp;
  int ncells;
  const double* f;          // [C][nv]
  const double* props;      // [C][DVM_NPROP]
  double* eq_cache;         // [C][kEqCache] dens, u, v, temp, w of the cached equilibrium
  // [C][nv+1] cumulative sums c(p) through node p - 1, fixed point (see k_cdf), stored as
  // 2 c(p) + s(p): s(p) = 1 when node p - 1 is negative (VR: f - f_eq < 0; FMC: f < 0)
  long long* cum_eq;        // f_eq (s = 0)
  long long* cum_dev;       // |f - f_eq| (FMC: |f|)
  int2* ref_eq;             // [C][1000]
  int2* ref_dev;            // [C][1000]
  CellPlan* plan;           // [C]
  PairDev pairs;
  uint32_t* err;
};

// Per-axis remap tables (built once per grid by dvm_create). For origin o and offset
// s in [-kTabS, kTabS]: D = v[o+s] - v[o], invD = 1/D, and T = ext*(ext - int) with
// ext = v[o-s] - v[o], int = v[o+s] - v[o] -- the terms of the remap denominators
// (collisions/remapping.f90:265-368). Entries whose nodes fall off the grid are NaN.
constexpr int kTabS = 3;
constexpr int kTabW = 2 * kTabS + 1;
struct AxisEntry {
  double D[kTabW];
  double invD[kTabW];
  double T[kTabW];
};

struct CollTables {
  const AxisEntry* axis;   // [3][nmax]
  int nmax;
  const double2* gtab;     // (g, g^(2-2 omega)) by di^2+dj^2+dk^2; null unless the grid is
  int gtab_n;              //   cubic and uniform
  int gtab_smem;           // stage gtab in shared memory
  double phi_scale;        // 2*pi_used/pi: phi/pi for sincospi
  const double2* trig;     // (cos, sin) of 2*pi_used*k/kTrigN, k < kTrigN
  double two_pi;           // 2*pi_used
};

// The FP64 (g, g^(2-2 omega)) table is staged in shared memory only up to this size, which
// keeps the collide CTA small enough for several CTAs per SM; larger tables are read
// through L1. Every launch set-up decides by this one rule.
constexpr size_t kGtabSmemMaxBytes = 32 * 1024;
inline int gtab_staged(int gtab_n) {
  return (gtab_n > 0 && static_cast<size_t>(gtab_n) * sizeof(double2) <= kGtabSmemMaxBytes) ? 1
                                                                                            : 0;
}

constexpr int kTrigN = 1024;

// FP32 copies of the collision tables for the precision form.
struct AxisEntryF {
  float D[kTabW];
  float invD[kTabW];
  float T[kTabW];
};

struct CollTablesF {
  const AxisEntryF* axis;  // [3][nmax]
  const float2* gtab;      // (g, g^(2-2 omega)), as CollTables::gtab
  int gtab_smem;
  const float2* trig;      // (cos, sin) of 2*pi_used*k/kTrigN
  float two_pi;
};

struct ProjectArgs {
  GridInfo g;
  int ncells;
  double* f;               // [C][nv], FP64 state
  float* df;               // [C][nv], FP32 collision increment (zeroed on exit)
  const double* props;     // [C][DVM_NPROP], for the centring velocity
};

struct CollideArgs {
  GridInfo g;
  CollParams cp;
  CollTables t;
  int ncells;
  uint32_t step;
  const uint32_t* step_dev;  // if set, the Philox step is read here (graph replays)
  double* f;
  const long long* cum_eq;
  const long long* cum_dev;
  const int2* ref_eq;
  const int2* ref_dev;
  const CellPlan* plan;
  const long long* chunk_off;  // [3*C + 1]: run offsets; [3C] = runs | run length << kRunShift
  PairDev pairs;
  uint32_t* err;
  unsigned long long* scatter_count;  // if set, the adds into f (df) are counted here
  // FP32 copies of grid constants, filled by launch_collide / launch_collide_f32 so that
  // the kernels read them as parameters rather than hold them in registers
  float vmin[3], vfac[3];  // axis minima and nearest-node factors
  float rnx, rnxy;         // 1 / NX and 1 / (NX NY)
  uint32_t rk[20];         // Philox key schedule of cp.seed (philox_key_schedule)
};

// 2-D wall ghost slabs: one per (wall side, position along the wall).
struct WallArgs {
  GridInfo g;
  int nxs, nys;
  int base[4];              // first entry of each side, -1 if that side has no wall ghost
  int nentries;
  double acc, mass, pi;
  double wall[4][5];
  const double* f;
  double* ghost;            // [nentries][nv]
  uint32_t* err;
};

struct Convect2DArgs {
  GridInfo g;
  int nxs, nys;
  int bc_left, bc_right;
  int base[4];
  double xf, yf;            // dt/dx, dt/dy
  const float2* cfl;        // |dt/dx x_i| (nx) then |dt/dy y_j| (ny) as hi + lo pairs
  const double* f;
  const double* ghost;
  double* fconv;
};

struct Convect1DArgs {
  GridInfo g;
  int nxs;                  // cells of one row
  int rows;                 // independent rows of nxs cells, each with both ends
  int bc[2];
  double factor;            // dt/dx
  double acc, mass, pi;
  double wall[2][5];
  const double* f;
  double* fconv;
  uint32_t* err;
};

struct MomentArgs {
  GridInfo g;
  int ncells;
  double mass;
  const double* f;
  double* props;
  uint32_t* err;
  // max over cells of the relative change of n, u and T since the previous moments
  // (the convergence residual); nonnegative doubles, compared as integers
  unsigned long long* residual;
  // if set, every value of f the kernel reads is also written here (the same layout): the
  // device copy of an f read from host memory, or the host copy of the device's f
  double* mirror;
};

// Grouped launches: the instances of a batch on up to kMaxGroups velocity grids advance in
// one launch of each kernel. Each group keeps its own arguments; a CTA finds its group from
// its index (groups own consecutive CTAs) and runs that group's code path.
constexpr int kMaxGroups = 8;

struct GroupedCdf {
  int ngroups;
  int first[kMaxGroups + 1];   // first CTA (= instance) of each group; first[ngroups] = grid
  CdfArgs a[kMaxGroups];
};

struct GroupedPlan {  // one CTA per group
  int ngroups;
  int ncells[kMaxGroups];
  long long warps[kMaxGroups];  // warps of the group's share of the collide launch
  const CellPlan* plan[kMaxGroups];
  long long* chunk_off[kMaxGroups];
  long long* total[kMaxGroups];
};

struct GroupedCollide {  // persistent: group g owns CTAs first[g] .. first[g+1] - 1
  int ngroups;
  int first[kMaxGroups + 1];
  CollideArgs a[kMaxGroups];
  CollTablesF tf[kMaxGroups];  // precision form
  float* df[kMaxGroups];
};

struct GroupedProject {
  int ngroups;
  int first[kMaxGroups + 1];
  ProjectArgs a[kMaxGroups];
};

struct GroupedMoments {
  int ngroups;
  int first[kMaxGroups + 1];
  MomentArgs a[kMaxGroups];
};

// Launch wrappers (dvm_kernels.cu). Each returns the cudaGetLastError of its launch.
cudaError_t launch_cdf(const CdfArgs& a, cudaStream_t s);
// warps: the warps of the collide launch that walks this plan (sets the run length)
cudaError_t launch_plan(int ncells, const CellPlan* plan, long long* chunk_off,
                        long long* total_samples, long long warps, cudaStream_t s);
cudaError_t launch_collide(const CollideArgs& a, int grid, cudaStream_t s);
cudaError_t launch_collide_f32(const CollideArgs& a, const CollTablesF& tf, float* df, int grid,
                               cudaStream_t s);
cudaError_t launch_project(const ProjectArgs& a, cudaStream_t s);

// CTAs per SM of the FP32 collide kernel; fast: of its copy for the common configuration
// (collide_fast without the recorded-list test, which the test hooks switch per call).
int collide_f32_blocks_per_sm(const GridInfo& g, const CollTables& t, bool fast);
cudaError_t launch_wall_flux(const WallArgs& a, cudaStream_t s);
cudaError_t launch_wall_specular(const WallArgs& a, cudaStream_t s);
cudaError_t launch_convect2d(const Convect2DArgs& a, int ncells, cudaStream_t s);
cudaError_t launch_convect1d(const Convect1DArgs& a, cudaStream_t s);
cudaError_t launch_bc1d(const Convect1DArgs& a, cudaStream_t s);         // diffuse ends
cudaError_t launch_bc1d_nodes(const Convect1DArgs& a, cudaStream_t s);   // the other ends
cudaError_t launch_moments(const MomentArgs& a, cudaStream_t s);
cudaError_t launch_flush(double* buf, size_t n, cudaStream_t s);
cudaError_t launch_wait_selftest(uint32_t* err, cudaStream_t s);
cudaError_t launch_atomic_probe(double* buf, size_t n, int blocks, int per_thread,
                                cudaStream_t s);
int collide_blocks_per_sm(size_t smem);
size_t collide_smem_bytes(const GridInfo& g, const CollTables& t);

// Grouped launches (batches). cdf_threads: 256, 512 or 1024 threads per CDF CTA.
cudaError_t launch_cdf_grouped(const GroupedCdf& m, int cdf_threads, cudaStream_t s);
cudaError_t launch_plan_grouped(const GroupedPlan& m, cudaStream_t s);
// m.a[g] carry the FP32 grid constants (collide_consts); the grid is m.first[m.ngroups]
cudaError_t launch_collide_grouped(const GroupedCollide& m, bool fp32, cudaStream_t s);
cudaError_t launch_project_grouped(const GroupedProject& m, cudaStream_t s);
cudaError_t launch_moments_grouped(const GroupedMoments& m, cudaStream_t s);
// CTAs per SM of the grouped collide launch (the largest group's shared memory decides)
int collide_grouped_blocks_per_sm(const GroupedCollide& m, bool fp32);
CollideArgs collide_consts(const CollideArgs& a);

}  // namespace dvm

// Context hooks for the request server (dvm_server.cu); defined in dvm_api.cu.
struct dvm_ctx;
struct dvm_params;
struct dvm_vgrid;
namespace dvm {
// A context on its own stream; async_alloc makes its buffers stream-ordered.
int ctx_create(const dvm_params* p, const dvm_vgrid* vg, bool async_alloc, dvm_ctx** out);
void ctx_destroy(dvm_ctx* c);
cudaStream_t ctx_stream(const dvm_ctx* c);
const unsigned long long* ctx_residual(const dvm_ctx* c);
const long long* ctx_total_samples(const dvm_ctx* c);
void ctx_set_step_dev(dvm_ctx* c, const uint32_t* step);
size_t ctx_device_bytes(const dvm_ctx* c);
// Device bytes a context for (p, vg) allocates (an upper bound where the grid is cubic in
// shape but not uniform).
size_t context_bytes(const dvm_params* p, const dvm_vgrid* vg);
}  // namespace dvm
