// wl_batch.cu -- persistent multi-job sweep and its batched reduction.
//
// Many evaluations of uneven size (different ensembles, profiles, flux
// values, instance counts, loops per tile) run as one launch: every CTA takes
// tiles from a global queue (atomicAdd on a counter) until it is empty and
// runs the same per-tile code as the single-job sweep (sweep_tile), so a
// job's partial sums -- and its results -- do not depend on the batch.  The
// host orders tiles by decreasing cost so the queue drains evenly.
#include "wl_device.cuh"
#include "wl_internal.h"
#include "wl_sweep.cuh"

namespace wl {

namespace {

// One tile of a job: packed pairs (256 instances) for the light profiles at
// 4 and 50 intervals -- as the single-job sweep, so such a job's results match
// it bit for bit -- one instance per thread otherwise (sweep_tile_instances).
template <bool FERM, int NINT>
__device__ __forceinline__ void run_tile(int kprof, const SweepArgs &A, int tx, int chunk,
                                         const SweepShared &S, double (*sacc2)[kPairTile],
                                         float (*tot)[kSweepThreads], int &consumed) {
  if constexpr (NINT == 0) {
    switch (kprof) {
      case kSmooth: sweep_tile<kSmooth, FERM, NINT>(A, tx, chunk, S, consumed); break;
      case kGaussian: sweep_tile<kGaussian, FERM, NINT>(A, tx, chunk, S, consumed); break;
      case kStep: sweep_tile<kStep, FERM, NINT>(A, tx, chunk, S, consumed); break;
      case kQuadratic: sweep_tile<kQuadratic, FERM, NINT>(A, tx, chunk, S, consumed); break;
      case kLattice: sweep_tile<kLattice, FERM, NINT>(A, tx, chunk, S, consumed); break;
      default: break;
    }
  } else {
    switch (kprof) {
      case kSmooth:
        sweep_tile2<kSmooth, FERM, NINT>(A, tx, chunk, S.full_bar, sacc2, S.bad, S.ring,
                                         consumed);
        break;
      case kGaussian:
        sweep_tile2<kGaussian, FERM, NINT>(A, tx, chunk, S.full_bar, sacc2, S.bad, S.ring,
                                           consumed);
        break;
      case kStep:
        sweep_tile2<kStep, FERM, NINT>(A, tx, chunk, S.full_bar, sacc2, S.bad, S.ring,
                                       consumed);
        break;
      case kQuadratic:
        sweep_tile2<kQuadratic, FERM, NINT>(A, tx, chunk, S.full_bar, sacc2, S.bad, S.ring,
                                            consumed);
        break;
      case kLattice:
        if constexpr (NINT == 4)
          sweep_tile_lat<FERM, false>(A, tx, chunk, S.full_bar, sacc2, tot, S.bad, S.ring,
                                      consumed);
        break;
      default: break;
    }
  }
}

constexpr int kBatchMinBlocks = 4;

__global__ void __launch_bounds__(kSweepThreads, kBatchMinBlocks)
    batch_kernel(const __grid_constant__ BatchArgs B) {
  extern __shared__ __align__(128) float4 ring[];
  __shared__ __align__(8) uint64_t full_bar[kSweepStages];
  __shared__ int sm_bad;
  // FP64 W - 1 sums: [kMaxF * 3][kPairTile] for pair tiles, the first
  // [kMaxF * 3][kSweepThreads] of it for one-instance tiles
  __shared__ double sacc2[kMaxF * 3][kPairTile];
  __shared__ float lat_tot[kLatTotRows][kSweepThreads];  // lattice tiles' loop totals
  __shared__ __align__(16) SweepArgs job;
  __shared__ int cur[4];
  const SweepShared S = {full_bar, reinterpret_cast<double(*)[kSweepThreads]>(&sacc2[0][0]),
                         &sm_bad, ring};
  sweep_shared_init(S);
  int consumed = 0;
  for (;;) {
    if (threadIdx.x == 0) {
      const int t = atomicAdd(B.counter, 1);
      cur[0] = t;
      if (t < B.ntiles) {
        const BatchTile d = B.tiles[t];
        cur[1] = d.job;
        cur[2] = d.tile_x;
        cur[3] = d.chunk;
      }
    }
    __syncthreads();
    const int t = cur[0];
    if (t >= B.ntiles) break;
    {  // the tile's job parameters, copied word by word
      const int *src = reinterpret_cast<const int *>(B.jobs + cur[1]);
      int *dst = reinterpret_cast<int *>(&job);
      for (int w = threadIdx.x; w < (int)(sizeof(SweepArgs) / 4); w += kSweepThreads)
        dst[w] = src[w];
    }
    __syncthreads();
    const int tx = cur[2], chunk = cur[3];
    // 4 and 50 intervals (the reference's): unrolled, pairs for the light
    // profiles; any other count at run time
    const bool n50 = job.nint == 50 && light_profile(job.kprof);
    if (job.fermion) {
      if (job.nint == 4)
        run_tile<true, 4>(job.kprof, job, tx, chunk, S, sacc2, lat_tot, consumed);
      else if (n50)
        run_tile<true, 50>(job.kprof, job, tx, chunk, S, sacc2, lat_tot, consumed);
      else
        run_tile<true, 0>(job.kprof, job, tx, chunk, S, sacc2, lat_tot, consumed);
    } else {
      if (job.nint == 4)
        run_tile<false, 4>(job.kprof, job, tx, chunk, S, sacc2, lat_tot, consumed);
      else if (n50)
        run_tile<false, 50>(job.kprof, job, tx, chunk, S, sacc2, lat_tot, consumed);
      else
        run_tile<false, 0>(job.kprof, job, tx, chunk, S, sacc2, lat_tot, consumed);
    }
    if (sm_bad) break;  // a copy timed out: the status is set, stop taking tiles
    __syncthreads();    // cur[] and job are rewritten next
  }
}

// one thread per (job, instance, flux value); jobs located by binary search
__global__ void batch_reduce_kernel(const ReduceJob *__restrict__ jobs, int njobs, int total) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= total) return;
  int lo = 0, hi = njobs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) / 2;
    if (jobs[mid].first <= idx) lo = mid;
    else hi = mid - 1;
  }
  const ReduceJob J = jobs[lo];
  const int local = idx - J.first;
  const int inst = local % J.ninst, j = local / J.ninst;
  const int ng = J.n_chunks / J.cpg;
  const double inv = 1.0 / (double)J.lpg;
  double mean = 0.0;
  for (int g = 0; g < ng; ++g) {
    double s0 = 0.0, s1 = 0.0, s2 = 0.0;
    for (int c = g * J.cpg; c < (g + 1) * J.cpg; ++c) {
      const size_t b = ((size_t)(c * J.nF + j) * 3) * J.ninst + inst;
      s0 += J.partial[b];
      s1 += J.partial[b + J.ninst];
      s2 += J.partial[b + 2 * (size_t)J.ninst];
    }
    const double v = 1.0 + (8.0 / 3.0 * (s0 * inv) - 2.0 * (s1 * inv) + 1.0 / 3.0 * (s2 * inv));
    J.out_group[((size_t)inst * J.nF + j) * ng + g] = v;
    mean += v;
  }
  mean /= (double)ng;
  double ss = 0.0;
  for (int g = 0; g < ng; ++g) {
    const double v = J.out_group[((size_t)inst * J.nF + j) * ng + g];
    ss += (v - mean) * (v - mean);
  }
  J.out_mean[(size_t)inst * J.nF + j] = mean;
  J.out_sem[(size_t)inst * J.nF + j] = ng > 1 ? sqrt(ss / ((double)ng * (ng - 1.0))) : 0.0;
}

// The plain per-instance kernel: one thread per loop walking its points from
// global memory (AoS float4, strided by ppl between threads), the structure of
// the reference's ExpectValue (intEV.cu:573-582) with this library's segment
// arithmetic; one launch per instance.
template <int P, bool FERM, int NINT>
__global__ void __launch_bounds__(128) plain_kernel(const __grid_constant__ LoopArgs A, int inst) {
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= A.Nl) return;
  const float cx = A.cx[inst], cy = A.cy[inst], s = A.rtT[inst];
  const df tq = {A.tqh[inst], A.tql[inst]};
  const FieldDev &F = A.field;
  const float4 *w = A.loops + (size_t)l * A.ppl;
  ImgRange img = {0, -1, 0, -1, 1};  // lattice: this loop's images
  if constexpr (P == kLattice) img = image_range(A.bbox[l], s, cx, cy, F);
  auto pt = [&](int p, float &x, float &y) {
    const float4 v = w[p];
    x = fmaf(s, v.x, cx);
    y = fmaf(s, v.y, cy);
  };
  float ph[3] = {0.f, 0.f, 0.f}, sp[3] = {0.f, 0.f, 0.f};
  float z0x, z0y, z1x, z1y, z2x, z2y, z3x, z3y;
  pt(0, z0x, z0y);
  pt(1, z1x, z1y);
  pt(2, z2x, z2y);
  pt(3, z3x, z3y);
  seg<P, FERM, NINT>(z1x, z1y, z3x, z3y, F, img, ph[0], sp[0]);
  float zAx = z0x, zAy = z0y, zBx = z2x, zBy = z2y, zOx = z3x, zOy = z3y;
  for (int q = 1; q < A.ppl / 4; ++q) {
    float P0x, P0y, P1x, P1y, P2x, P2y, P3x, P3y;
    pt(4 * q, P0x, P0y);
    pt(4 * q + 1, P1x, P1y);
    pt(4 * q + 2, P2x, P2y);
    pt(4 * q + 3, P3x, P3y);
    seg<P, FERM, NINT>(zAx, zAy, P0x, P0y, F, img, ph[2], sp[2]);
    seg<P, FERM, NINT>(zOx, zOy, P1x, P1y, F, img, ph[0], sp[0]);
    seg<P, FERM, NINT>(zBx, zBy, P2x, P2y, F, img, ph[1], sp[1]);
    seg<P, FERM, NINT>(P1x, P1y, P3x, P3y, F, img, ph[0], sp[0]);
    zAx = P0x; zAy = P0y;
    zBx = P2x; zBy = P2y;
    zOx = P3x; zOy = P3y;
  }
  seg<P, FERM, NINT>(zOx, zOy, z1x, z1y, F, img, ph[0], sp[0]);
  seg<P, FERM, NINT>(zBx, zBy, z2x, z2y, F, img, ph[1], sp[1]);
  seg<P, FERM, NINT>(zAx, zAy, z0x, z0y, F, img, ph[2], sp[2]);
  const df G[3] = {df{ph[0], 0.f}, df{ph[1], 0.f}, df{ph[2], 0.f}};
  const df H[3] = {df{sp[0], 0.f}, df{sp[1], 0.f}, df{sp[2], 0.f}};
  loop_epilogue<FERM>(G, H, A.cph_hi, A.cph_lo, A.csp_hi, A.csp_lo, tq, A.nF,
                      [&](int j, double d0, double d1, double d2) {
                        double *o = A.partial + ((size_t)(l * A.nF + j) * 3) * A.ninst + inst;
                        o[0] = d0;
                        o[A.ninst] = d1;
                        o[2 * (size_t)A.ninst] = d2;
                      });
}

template <bool FERM, int NINT>
cudaError_t plain_dispatch(int kprof, const LoopArgs &a, int inst, cudaStream_t st) {
  const dim3 grid((a.Nl + 127) / 128);
  switch (kprof) {
    case kSmooth: plain_kernel<kSmooth, FERM, NINT><<<grid, 128, 0, st>>>(a, inst); break;
    case kGaussian: plain_kernel<kGaussian, FERM, NINT><<<grid, 128, 0, st>>>(a, inst); break;
    case kStep: plain_kernel<kStep, FERM, NINT><<<grid, 128, 0, st>>>(a, inst); break;
    case kQuadratic: plain_kernel<kQuadratic, FERM, NINT><<<grid, 128, 0, st>>>(a, inst); break;
    case kLattice: plain_kernel<kLattice, FERM, NINT><<<grid, 128, 0, st>>>(a, inst); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_plain(int kprof, bool fermion, int nint, const LoopArgs &a, int inst,
                         cudaStream_t st) {
  if (fermion)
    return nint == 4 ? plain_dispatch<true, 4>(kprof, a, inst, st)
                     : plain_dispatch<true, 0>(kprof, a, inst, st);
  return nint == 4 ? plain_dispatch<false, 4>(kprof, a, inst, st)
                   : plain_dispatch<false, 0>(kprof, a, inst, st);
}

bool batch_supports(int kprof, int nint) {
  (void)nint;
  return kprof >= kStep && kprof <= kLattice;
}

bool batch_in_kernel(int kprof) { return light_profile(kprof) || kprof == kLattice; }

bool plain_supports(int kprof) { return light_profile(kprof) || kprof == kLattice; }

// the kernel's static shared memory (the FP64 sums and the lattice totals,
// 37 KiB) and its ring (16 KiB) exceed the 48 KiB a launch gets without
// opting in; the attribute is per device, so it is set before every use
static cudaError_t batch_smem_optin() {
  return cudaFuncSetAttribute(batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)sweep_smem_bytes());
}

int batch_max_ctas_per_sm() {
  int n = 0;
  if (batch_smem_optin() != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_kernel, kSweepThreads,
                                                    sweep_smem_bytes()) != cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  return n > 0 ? n : 1;
}

cudaError_t launch_batch(const BatchArgs &a, int grid, cudaStream_t s) {
  const cudaError_t e = batch_smem_optin();
  if (e != cudaSuccess) return e;
  batch_kernel<<<grid, kSweepThreads, sweep_smem_bytes(), s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_batch_reduce(const ReduceJob *jobs, int njobs, int total, cudaStream_t s) {
  const int bs = 128;
  batch_reduce_kernel<<<(total + bs - 1) / bs, bs, 0, s>>>(jobs, njobs, total);
  return cudaGetLastError();
}

}  // namespace wl
