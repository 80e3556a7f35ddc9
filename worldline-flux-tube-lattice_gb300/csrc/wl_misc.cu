// wl_misc.cu -- profile dispatch, FP64 loop-average reductions and the
// seeded unit-loop generator.
#include <math.h>

#include "wl_device.cuh"
#include "wl_internal.h"

namespace wl {

cudaError_t launch_sweep_smooth(int, bool, int, const SweepArgs *, const LoopArgs *,
                                cudaStream_t);
cudaError_t launch_sweep_simple(int, bool, int, const SweepArgs *, const LoopArgs *,
                                cudaStream_t);
cudaError_t launch_sweep_periodic(int, bool, int, const SweepArgs *, const LoopArgs *,
                                  cudaStream_t);
cudaError_t launch_sweep_spline(int, bool, int, const SweepArgs *, const LoopArgs *,
                                cudaStream_t);
cudaError_t launch_sweep_fixflux(int, bool, int, const SweepArgs *, const LoopArgs *,
                                 cudaStream_t);
cudaError_t launch_sweep_lattice(int, bool, int, const SweepArgs *, const LoopArgs *,
                                 cudaStream_t);

static cudaError_t dispatch(int profile, bool fermion, int nint, const SweepArgs *sa,
                            const LoopArgs *la, cudaStream_t s) {
  switch (profile) {
    case kSmooth: return launch_sweep_smooth(profile, fermion, nint, sa, la, s);
    case kStep:
    case kQuadratic:
    case kGaussian: return launch_sweep_simple(profile, fermion, nint, sa, la, s);
    case kPeriodic: return launch_sweep_periodic(profile, fermion, nint, sa, la, s);
    case kSpline: return launch_sweep_spline(profile, fermion, nint, sa, la, s);
    case kFixflux:
    case kFixfluxFF: return launch_sweep_fixflux(profile, fermion, nint, sa, la, s);
    case kLattice: return launch_sweep_lattice(profile, fermion, nint, sa, la, s);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_sweep(int profile, bool fermion, int nint, const SweepArgs &a,
                         cudaStream_t s) {
  return dispatch(profile, fermion, nint, &a, nullptr, s);
}

cudaError_t launch_loopwarp(int profile, bool fermion, int nint, const LoopArgs &a,
                            cudaStream_t s) {
  return dispatch(profile, fermion, nint, nullptr, &a, s);
}

// ---------------------------------------------------------- reductions --
// One thread per (instance, flux value): group sums over the group's chunks
// in chunk order (the result of an instance does not depend on how many
// other instances share the launch), the Richardson combination
// 8/3 W_N - 2 W_N/2 + 1/3 W_N/4 (Integrand.c:400), then mean and standard
// error over the groups.  The partial sums hold W - 1 per loop; the weights
// sum to one, so <W> = 1 + the same combination of the deviations.
__global__ void group_reduce_kernel(const double *__restrict__ partial, int n_chunks,
                                    int cpg, int lpg, int ninst, int nF,
                                    double *__restrict__ out_group,
                                    double *__restrict__ out_mean,
                                    double *__restrict__ out_sem) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= ninst * nF) return;
  const int inst = idx % ninst, j = idx / ninst;
  const int ng = n_chunks / cpg;
  const double inv = 1.0 / (double)lpg;
  auto group_value = [&](int g) {
    double s0 = 0.0, s1 = 0.0, s2 = 0.0;
    for (int c = g * cpg; c < (g + 1) * cpg; ++c) {
      const size_t base = ((size_t)(c * nF + j) * 3) * ninst + inst;
      s0 += partial[base];
      s1 += partial[base + ninst];
      s2 += partial[base + 2 * (size_t)ninst];
    }
    return 1.0 + (8.0 / 3.0 * (s0 * inv) - 2.0 * (s1 * inv) + 1.0 / 3.0 * (s2 * inv));
  };
  double mean = 0.0;
  for (int g = 0; g < ng; ++g) {
    const double v = group_value(g);
    if (out_group) out_group[((size_t)inst * nF + j) * ng + g] = v;
    mean += v;
  }
  mean /= (double)ng;
  double ss = 0.0;
  for (int g = 0; g < ng; ++g) {
    const double v = out_group ? out_group[((size_t)inst * nF + j) * ng + g] : group_value(g);
    ss += (v - mean) * (v - mean);
  }
  if (out_mean) out_mean[(size_t)inst * nF + j] = mean;
  if (out_sem)
    out_sem[(size_t)inst * nF + j] = ng > 1 ? sqrt(ss / ((double)ng * (ng - 1.0))) : 0.0;
}

// ------------------------------------------------ lattice instance order --
// Key: proper time first (log2 rtT in steps of 1/8 over [-16, 16), largest
// first), then the centre's position in its lattice cell (4 x 4 bins): the
// number of images an instance sums follows both, so neighbouring threads
// get similar counts.
constexpr int kOrderTBins = 256, kOrderCellBins = 16;
constexpr int kOrderBuckets = kOrderTBins * kOrderCellBins;

__device__ __forceinline__ int order_bucket(float cx, float cy, float rtT, float inv_a) {
  const float x = log2f(fmaxf(rtT, 1e-30f)) * 8.0f;
  const int tb = kOrderTBins - 1 - min(max((int)floorf(x) + kOrderTBins / 2, 0), kOrderTBins - 1);
  const float u = cx * inv_a, v = cy * inv_a;
  const int bu = min(max((int)((u - floorf(u)) * 4.0f), 0), 3);
  const int bv = min(max((int)((v - floorf(v)) * 4.0f), 0), 3);
  return tb * kOrderCellBins + bu * 4 + bv;
}

__global__ void __launch_bounds__(1024)
    order_instances_kernel(const float *__restrict__ cx, const float *__restrict__ cy,
                           const float *__restrict__ rtT, int n, float inv_a,
                           int *__restrict__ perm) {
  __shared__ int cnt[kOrderBuckets];
  __shared__ int part[1024];
  for (int b = threadIdx.x; b < kOrderBuckets; b += blockDim.x) cnt[b] = 0;
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x)
    atomicAdd(&cnt[order_bucket(cx[i], cy[i], rtT[i], inv_a)], 1);
  __syncthreads();
  // exclusive scan of the counts: each thread scans 4 buckets, then the
  // thread totals are scanned serially by one thread
  constexpr int per = kOrderBuckets / 1024;
  const int b0 = threadIdx.x * per;
  int tot = 0;
  for (int b = b0; b < b0 + per; ++b) tot += cnt[b];
  part[threadIdx.x] = tot;
  __syncthreads();
  if (threadIdx.x == 0) {
    int run = 0;
    for (int t = 0; t < 1024; ++t) {
      const int c = part[t];
      part[t] = run;
      run += c;
    }
  }
  __syncthreads();
  int run = part[threadIdx.x];
  for (int b = b0; b < b0 + per; ++b) {
    const int c = cnt[b];
    cnt[b] = run;
    run += c;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x)
    perm[atomicAdd(&cnt[order_bucket(cx[i], cy[i], rtT[i], inv_a)], 1)] = i;
}

cudaError_t launch_order_instances(const float *cx, const float *cy, const float *rtT, int n,
                                   float inv_a, int *perm, cudaStream_t s) {
  order_instances_kernel<<<1, 1024, 0, s>>>(cx, cy, rtT, n, inv_a, perm);
  return cudaGetLastError();
}

cudaError_t launch_group_reduce(const double *partial, int n_chunks, int cpg, int lpg,
                                int ninst, int nF, double *out_group, double *out_mean,
                                double *out_sem, cudaStream_t s) {
  const int n = ninst * nF, bs = 128;
  group_reduce_kernel<<<(n + bs - 1) / bs, bs, 0, s>>>(partial, n_chunks, cpg, lpg, ninst,
                                                        nF, out_group, out_mean, out_sem);
  return cudaGetLastError();
}

// EV(): mean of the per-loop factors (stored as W - 1) over an index list,
// fixed-order tree.
constexpr int kListThreads = 128;
__global__ void __launch_bounds__(kListThreads)
    list_mean_kernel(const double *__restrict__ w, const int *__restrict__ list, int n,
                     double *__restrict__ out) {
  // list == nullptr: block b takes the consecutive loops b n .. b n + n - 1
  __shared__ double red[3][kListThreads];
  double s0 = 0.0, s1 = 0.0, s2 = 0.0;
  for (int i = threadIdx.x; i < n; i += kListThreads) {
    const int l = list ? list[i] : blockIdx.x * n + i;
    s0 += w[3 * (size_t)l];
    s1 += w[3 * (size_t)l + 1];
    s2 += w[3 * (size_t)l + 2];
  }
  red[0][threadIdx.x] = s0;
  red[1][threadIdx.x] = s1;
  red[2][threadIdx.x] = s2;
  __syncthreads();
  for (int h = kListThreads / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h)
      for (int r = 0; r < 3; ++r) red[r][threadIdx.x] += red[r][threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double inv = 1.0 / (double)n;
    out[blockIdx.x] = 1.0 + (8.0 / 3.0 * (red[0][0] * inv) - 2.0 * (red[1][0] * inv) +
                             1.0 / 3.0 * (red[2][0] * inv));
  }
}

cudaError_t launch_list_mean(const double *partial, const int *list, int n, double *out,
                             cudaStream_t s) {
  list_mean_kernel<<<1, kListThreads, 0, s>>>(partial, list, n, out);
  return cudaGetLastError();
}

cudaError_t launch_group_list_means(const double *partial, int n, int ngroups, double *out,
                                    cudaStream_t s) {
  list_mean_kernel<<<ngroups, kListThreads, 0, s>>>(partial, nullptr, n, out);
  return cudaGetLastError();
}

// instance set-up on the device: the same float conversions as the host path
// (rtT = float(sqrt(T)), tq = 4 rtT^2/ppl as a float pair hi + lo)
__global__ void instance_setup_kernel(const double *__restrict__ cx,
                                      const double *__restrict__ cy,
                                      const double *__restrict__ T, int ninst, int ppl,
                                      float *__restrict__ out, int *__restrict__ status) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ninst) return;
  const double x = cx[i], y = cy[i], t = T[i];
  const bool ok = isfinite(x) && isfinite(y) && isfinite(t) && t > 0.0;
  if (!ok) atomicExch(status, kDevBadInstance);
  const double tt = ok ? t : 1.0;
  out[i] = ok ? (float)x : 0.0f;
  out[ninst + i] = ok ? (float)y : 0.0f;
  const float rtT = (float)sqrt(tt);
  const double tq = 4.0 * ((double)rtT * (double)rtT) / (double)ppl;
  out[2 * ninst + i] = rtT;
  out[3 * ninst + i] = (float)tq;
  out[4 * ninst + i] = (float)(tq - (double)(float)tq);
}

cudaError_t launch_instance_setup(const double *cx, const double *cy, const double *T,
                                  int ninst, int ppl, float *out, int *status,
                                  cudaStream_t s) {
  const int bs = 256;
  instance_setup_kernel<<<(ninst + bs - 1) / bs, bs, 0, s>>>(cx, cy, T, ninst, ppl, out,
                                                             status);
  return cudaGetLastError();
}

// ------------------------------------------------------ bounding boxes --
// one warp per loop: (xmin, xmax, ymin, ymax) of the unit loop
__global__ void loop_bbox_kernel(const float4 *__restrict__ loops, int Nl, int ppl,
                                 float4 *__restrict__ out) {
  const int l = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (l >= Nl) return;
  const float4 *w = loops + (size_t)l * ppl;
  float x0 = INFINITY, x1 = -INFINITY, y0 = INFINITY, y1 = -INFINITY;
  for (int p = lane; p < ppl; p += 32) {
    const float4 v = w[p];
    x0 = fminf(x0, v.x);
    x1 = fmaxf(x1, v.x);
    y0 = fminf(y0, v.y);
    y1 = fmaxf(y1, v.y);
  }
  for (int off = 16; off > 0; off >>= 1) {
    x0 = fminf(x0, __shfl_xor_sync(0xffffffffu, x0, off));
    x1 = fmaxf(x1, __shfl_xor_sync(0xffffffffu, x1, off));
    y0 = fminf(y0, __shfl_xor_sync(0xffffffffu, y0, off));
    y1 = fmaxf(y1, __shfl_xor_sync(0xffffffffu, y1, off));
  }
  if (lane == 0) out[l] = make_float4(x0, x1, y0, y1);
}

// ------------------------------------------------------- fingerprint --
// Content fingerprint of an ensemble's (x, y) coordinates: the sum modulo
// 2^64 of the splitmix64 finaliser (Steele, Lea and Flood, "Fast splittable
// pseudorandom number generators", OOPSLA 2014) applied to each point's
// coordinate bits combined with its index.  Any change of a coordinate
// changes the sum except with probability ~2^-64; the sum does not depend on
// the order in which the points are added.
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

__global__ void __launch_bounds__(256)
    fingerprint_kernel(const float2 *__restrict__ pts, size_t npts,
                       unsigned long long *__restrict__ out) {
  unsigned long long acc = 0;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x; p < npts; p += stride) {
    const float2 v = pts[2 * p];  // (x, y) of the float4 point p
    const unsigned long long bits =
        (unsigned long long)__float_as_uint(v.x) |
        ((unsigned long long)__float_as_uint(v.y) << 32);
    acc += mix64(bits ^ mix64(p + 0x9e3779b97f4a7c15ull));
  }
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
  if ((threadIdx.x & 31) == 0) atomicAdd(out, acc);
}

cudaError_t launch_fingerprint(const float4 *loops, size_t npts, unsigned long long *out,
                               cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(out, 0, sizeof(*out), s);
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const size_t want = (npts + 255) / 256;
  const int grid = (int)(want < (size_t)(sms * 8) ? (want > 0 ? want : 1) : (size_t)(sms * 8));
  fingerprint_kernel<<<grid, 256, 0, s>>>(reinterpret_cast<const float2 *>(loops), npts, out);
  return cudaGetLastError();
}

cudaError_t launch_loop_bbox(const float4 *loops, int Nl, int ppl, float4 *out, cudaStream_t s) {
  const int warps = 4;
  loop_bbox_kernel<<<(Nl + warps - 1) / warps, warps * 32, 0, s>>>(loops, Nl, ppl, out);
  return cudaGetLastError();
}

// ------------------------------------------------------------ probes --
// Eight independent dependency chains per thread keep the pipe busy; the
// result is stored only if it is impossible, so the work cannot be removed.
__global__ void peak_fma_kernel(int iters, float *sink) {
  float a[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) a[k] = 1.0f + 1e-7f * (float)(threadIdx.x + k);
  const float m = 0.999999f, c = 1e-7f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = fmaf(a[k], m, c);
  }
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += a[k];
  if (s == -1.0f) sink[blockIdx.x] = s;
}

__global__ void peak_rcp_kernel(int iters, float *sink) {
  // a <- rcp(a) + tiny: the FP32 add keeps rcp(rcp(a)) from being folded and
  // costs 1/128 of an SM cycle against the reciprocal's 1/16 (MUFU-bound)
  float a[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) a[k] = 1.5f + 1e-3f * (float)(threadIdx.x + k);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = rcp_fast(a[k]) + 1e-7f;
  }
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += a[k];
  if (s == -1.0f) sink[blockIdx.x] = s;
}

// packed pairs: each fma.rn.f32x2 performs two FP32 FMAs (16 per iteration)
__global__ void peak_fma2_kernel(int iters, float *sink) {
  float2 a[8];
#pragma unroll
  for (int k = 0; k < 8; ++k)
    a[k] = make_float2(1.0f + 1e-7f * (float)(threadIdx.x + k), 1.0f - 1e-7f * (float)k);
  const float2 m = make_float2(0.999999f, 0.999998f), c = make_float2(1e-7f, 2e-7f);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = __ffma2_rn(a[k], m, c);
  }
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += a[k].x + a[k].y;
  if (s == -1.0f) sink[blockIdx.x] = s;
}

// The bounded mbarrier wait that guards every staged copy, on its own: one
// CTA initialises a barrier for one arrival and waits on its first phase
// with max_tries polls.  With arrive = 1 thread 0 arrives (the phase
// completes, nothing is written); with arrive = 0 nothing arrives, the wait
// gives up and the status word receives kDevTimeout.  No copy is issued, so
// nothing is in flight when the CTA exits.
__global__ void wait_selftest_kernel(int *status, uint32_t max_tries, int arrive) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (threadIdx.x == 0 && arrive) mbar_arrive_expect_tx(&bar, 0);
  const bool ok = mbar_wait_bounded(&bar, 0, max_tries);
  __syncthreads();
  if (threadIdx.x == 0 && !ok) atomicExch(status, kDevTimeout);
}

cudaError_t launch_wait_selftest(int *status, uint32_t max_tries, int arrive, cudaStream_t s) {
  wait_selftest_kernel<<<1, 32, 0, s>>>(status, max_tries, arrive);
  return cudaGetLastError();
}

cudaError_t launch_peak_probe(int kind, int blocks, int threads, int iters, float *sink,
                              cudaStream_t s) {
  if (kind == 0)
    peak_fma_kernel<<<blocks, threads, 0, s>>>(iters, sink);
  else if (kind == 2)
    peak_fma2_kernel<<<blocks, threads, 0, s>>>(iters, sink);
  else
    peak_rcp_kernel<<<blocks, threads, 0, s>>>(iters, sink);
  return cudaGetLastError();
}

// ------------------------------------------------------ unit-loop ensemble --
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
// easy as 1, 2, 3", SC'11): 10 rounds of the multiply-xor bijection with
// Weyl-sequence key schedule.
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    if (r > 0) {
      k.x += 0x9E3779B9u;
      k.y += 0xBB67AE85u;
    }
    const uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
    const uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
    c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
  }
  return c;
}

constexpr uint32_t kVloopTag = 0x764C6F6Fu;  // counter word 2 ("vLoo")

// four standard normals of step k of loop l (Box-Muller in FP64)
__device__ __forceinline__ void step_normals(uint2 key, int k, int lg, double n[4]) {
  const uint4 r = philox4x32_10(make_uint4((uint32_t)k, (uint32_t)lg, kVloopTag, 0u), key);
  const double two32 = 4294967296.0;
  const uint32_t v[4] = {r.x, r.y, r.z, r.w};
#pragma unroll
  for (int p = 0; p < 2; ++p) {
    const double u = ((double)v[2 * p] + 0.5) / two32;
    const double w = ((double)v[2 * p + 1] + 0.5) / two32;
    const double rad = sqrt(-2.0 * log(u));
    double sn, cs;
    sincospi(2.0 * w, &sn, &cs);
    n[2 * p] = rad * cs;
    n[2 * p + 1] = rad * sn;
  }
}

// One thread per loop.  A discrete Brownian bridge of unit proper time:
// increments N(0, 2/N) per component (the kinetic weight exp(-1/4 int xdot^2)
// of a unit loop), x_k = y_k - (k/N) y_N, then the mean is removed.  Two
// passes over the same counter-based draws avoid storing the walk.
__global__ void vloops_kernel(uint64_t seed, int first, int Nl, int ppl,
                              float4 *__restrict__ out) {
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= Nl) return;
  const uint2 key = make_uint2((uint32_t)seed, (uint32_t)(seed >> 32));
  const double sigma = sqrt(2.0 / (double)ppl);
  double y[4] = {0, 0, 0, 0}, sy[4] = {0, 0, 0, 0};
  for (int k = 0; k < ppl; ++k) {
    double n[4];
    step_normals(key, k, first + l, n);
    for (int d = 0; d < 4; ++d) {
      sy[d] += y[d];
      y[d] += sigma * n[d];
    }
  }
  // mean of x_k = (1/N) sum y_k - y_N (N-1)/(2N)
  double mean[4];
  for (int d = 0; d < 4; ++d)
    mean[d] = sy[d] / (double)ppl - y[d] * ((double)(ppl - 1) / (2.0 * ppl));
  double yy[4] = {0, 0, 0, 0};
  float4 *o = out + (size_t)l * ppl;
  for (int k = 0; k < ppl; ++k) {
    const double fk = (double)k / (double)ppl;
    o[k] = make_float4((float)(yy[0] - fk * y[0] - mean[0]), (float)(yy[1] - fk * y[1] - mean[1]),
                       (float)(yy[2] - fk * y[2] - mean[2]), (float)(yy[3] - fk * y[3] - mean[3]));
    double n[4];
    step_normals(key, k, first + l, n);
    for (int d = 0; d < 4; ++d) yy[d] += sigma * n[d];
  }
}

cudaError_t launch_vloops(uint64_t seed, int first, int Nl, int ppl, float4 *out,
                          cudaStream_t s) {
  const int bs = 64;
  vloops_kernel<<<(Nl + bs - 1) / bs, bs, 0, s>>>(seed, first, Nl, ppl, out);
  return cudaGetLastError();
}

}  // namespace wl
