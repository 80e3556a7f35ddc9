// wl_internal.h -- launch interfaces between the C-ABI runtime (wl_api.cpp)
// and the kernels (wl_sweep.cu, wl_loopwarp.cu, wl_misc.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "wl_types.h"

namespace wl {

// device-side status codes written to the status word of a launch
enum : int { kDevOk = 0, kDevTimeout = 1, kDevBadInstance = 2 };

// Instance-parallel sweep: one thread per (instance), one CTA per
// (instance tile, chunk of loops); the chunk's loops are streamed through a
// shared-memory ring by bulk copies and every thread walks every point.
constexpr int kSweepThreads = 128;   // instances per CTA
// resident CTAs per SM the light-profile sweep is compiled for (register cap
// 65536 / (128 * blocks)); the lattice profiles use 4
#ifndef WL_SWEEP_MIN_BLOCKS
#define WL_SWEEP_MIN_BLOCKS 6
#endif
constexpr int kSweepMinBlocks = WL_SWEEP_MIN_BLOCKS;
constexpr int kSweepStages = 4;      // shared-memory ring depth
constexpr int kSweepChunkPts = 256;  // points per bulk copy (4 KiB)

struct SweepArgs {
  const float4 *loops;  // [Nl][ppl]
  int Nl, ppl;
  int ninst;
  const float *cx, *cy;  // [ninst] centre of mass
  const float *rtT;      // [ninst] float(sqrt(T)) as the reference passes it
  const float *tqh, *tql;  // [ninst] 4 T / ppl (spin normalisation 2T/(N/2)), hi + lo
  int nF;
  float F[kMaxF];
  // double-float per-flux constants: cph = F h/3, csp = F h/3 fp_scale
  float cph_hi[kMaxF], cph_lo[kMaxF], csp_hi[kMaxF], csp_lo[kMaxF];
  FieldDev field;
  int chunk_loops;   // loops per CTA
  int n_chunks;      // Nl / chunk_loops
  double *partial;   // [n_chunks][nF][3][ninst]
  int *status;       // kDevOk / kDevTimeout
  uint32_t wait_tries;
  int kprof, fermion, nint;  // kernel selection inside the persistent batch kernel
  const float4 *bbox;        // lattice: [Nl] unit-loop (xmin, xmax, ymin, ymax)
  // optional [ninst] thread slot -> instance: lattice instances ordered by
  // proper time so that the threads of a warp sum similar numbers of images
  const int *perm;
};

// The single-job sweep runs the light profiles at 4 and 50 intervals two
// instances per thread as packed f32x2 pairs (256 per CTA of 128 threads),
// and the lattice at 4 intervals two instances per thread (their images in
// packed pairs), everything else one per thread; so do the tiles of the
// persistent batch kernel: instances per batch tile.
inline __host__ __device__ bool light_profile(int kprof) {
  return kprof == kSmooth || kprof == kStep || kprof == kQuadratic || kprof == kGaussian;
}
inline __host__ __device__ int sweep_tile_instances(int kprof, int nint) {
  return (((nint == 4 || nint == 50) && light_profile(kprof)) || (nint == 4 && kprof == kLattice))
             ? 2 * kSweepThreads
             : kSweepThreads;
}

// Persistent multi-job sweep: a queue of tiles (job, instance tile, loop
// chunk) drained by one CTA per slot; jobs differ in ensemble, profile,
// instances, flux values and loops per tile.
struct BatchTile {
  int job, tile_x, chunk, cost;
};
struct ReduceJob {  // per job: where its partial sums and outputs live
  const double *partial;
  double *out_group, *out_mean, *out_sem;
  int n_chunks, cpg, lpg, ninst, nF, first;  // first: flat (instance, F) index
};
struct BatchArgs {
  const SweepArgs *jobs;
  const BatchTile *tiles;
  int ntiles;
  int *counter;  // next tile to take
};
cudaError_t launch_batch(const BatchArgs &a, int grid, cudaStream_t s);
cudaError_t launch_batch_reduce(const ReduceJob *jobs, int njobs, int total, cudaStream_t s);
// largest number of batch-kernel CTAs resident per SM
int batch_max_ctas_per_sm();
// every profile batches; the heavy ones (periodic, spline, fixflux) are not
// instantiated in the persistent kernel (their tiles would triple its
// compilation time) and run as chunk-range launches of their own sweep
// kernel beside it, with the same partial-sum layout
bool batch_supports(int kprof, int nint);
bool batch_in_kernel(int kprof);
bool plain_supports(int kprof);

// Loop-parallel sweep: one warp per (loop, instance), lanes over groups of
// four points; per-loop results.  Used for few instances and for EV().
constexpr int kLoopWarps = 4;  // warps per CTA

struct LoopArgs {
  const float4 *loops;
  int Nl, ppl;
  int ninst;
  const float *cx, *cy, *rtT, *tqh, *tql;
  int nF;
  float F[kMaxF];
  float cph_hi[kMaxF], cph_lo[kMaxF], csp_hi[kMaxF], csp_lo[kMaxF];
  FieldDev field;
  double *partial;  // [Nl][nF][3][ninst]  (chunk = one loop)
  float4 *scal;     // optional [ninst][Nl] Wsscal of F[0]
  float4 *ferm;     // optional [ninst][Nl] Wsferm of F[0]
  const float4 *bbox;  // lattice: [Nl] unit-loop bounding boxes
};

// plain per-instance kernel (the batching baseline), light profiles only
cudaError_t launch_plain(int kprof, bool fermion, int nint, const LoopArgs &a, int inst,
                         cudaStream_t st);

// returns cudaErrorInvalidValue for an unsupported (profile, nint)
cudaError_t launch_sweep(int profile, bool fermion, int nint, const SweepArgs &a,
                         cudaStream_t s);
cudaError_t launch_loopwarp(int profile, bool fermion, int nint, const LoopArgs &a,
                            cudaStream_t s);

// partial sums -> per-group <W>, mean and SEM over groups
cudaError_t launch_group_reduce(const double *partial, int n_chunks, int chunks_per_group,
                                int loops_per_group, int ninst, int nF, double *out_group,
                                double *out_mean, double *out_sem, cudaStream_t s);

// EV(): mean over an index list of per-loop W factors (partial with
// ninst = 1, nF = 1) and the Richardson combination; writes one double.
cudaError_t launch_list_mean(const double *partial, const int *list, int n, double *out,
                             cudaStream_t s);
// the same for the ngroups lists of n consecutive loops (g n .. g n + n - 1),
// one double per group, each summed exactly as launch_list_mean sums it
cudaError_t launch_group_list_means(const double *partial, int n, int ngroups, double *out,
                                    cudaStream_t s);

// device-resident instances (cx, cy, T) -> the sweep's float arrays
// [cx | cy | rtT | tq_hi | tq_lo]; flags T <= 0 or non-finite values in *status
cudaError_t launch_instance_setup(const double *cx, const double *cy, const double *T,
                                  int ninst, int ppl, float *out, int *status,
                                  cudaStream_t s);

// pipe throughput probes: kind 0 FP32 FMA chains, 1 MUFU rcp chains;
// each thread performs iters * 8 operations
// one CTA waiting (bounded) on an mbarrier that gets its arrival or not
cudaError_t launch_wait_selftest(int *status, uint32_t max_tries, int arrive, cudaStream_t s);
cudaError_t launch_peak_probe(int kind, int blocks, int threads, int iters, float *sink,
                              cudaStream_t s);

// FP64 proper-time integral + jackknife (wl_tint.cu)
struct TintArgs {
  const double *groups;  // [nrho * nT][nF][ng]   instance i = r * nT + k
  const double *rho;     // [nrho] centre of mass x (y = 0, as rhogrand, EffAct.c:23-25)
  const double *T;       // [nT]
  const double *w;       // [nT] quadrature weights in T (dT, Simpson on ln T)
  const double *F;       // [nF]
  int nrho, nT, nF, ng, nbins;
  int profile, fermion;
  double l2, a, lmin, m2, e;
  double rimg2;   // lattice: (rimage / a)^2
  double xcm_x;   // scratch: the centre of mass of the current evaluation
  double *igrand;  // optional [nrho][nF][nT][ng]
  double *Ig;      // [nrho][nF][ng]
  double *leff, *err;  // [nrho][nF]
};
cudaError_t launch_tint(const TintArgs &a, cudaStream_t s);

// perm[0..n) = instances in decreasing rtT, then by the centre's position in
// its lattice cell (one CTA, bucketed; the order inside a bucket is arbitrary
// and changes no result)
cudaError_t launch_order_instances(const float *cx, const float *cy, const float *rtT, int n,
                                   float inv_a, int *perm, cudaStream_t s);

// 64-bit fingerprint of the (x, y) coordinates of npts float4 points (zeroes
// *out first; EV()'s check that a cached ensemble was not rewritten)
cudaError_t launch_fingerprint(const float4 *loops, size_t npts, unsigned long long *out,
                               cudaStream_t s);

// per-loop bounding boxes of an ensemble (lattice image selection)
cudaError_t launch_loop_bbox(const float4 *loops, int Nl, int ppl, float4 *out, cudaStream_t s);

// seeded unit loops
cudaError_t launch_vloops(uint64_t seed, int first, int Nl, int ppl, float4 *out,
                          cudaStream_t s);

// bytes of dynamic shared memory of the sweep kernel
constexpr int kInstArrays = 5;  // cx, cy, rtT, tq_hi, tq_lo

constexpr size_t sweep_smem_bytes() {
  return (size_t)kSweepStages * kSweepChunkPts * sizeof(float4);
}

}  // namespace wl
