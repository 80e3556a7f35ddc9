// wl_sweep.cuh -- the two Wilson-loop sweep kernels.
//
// Both compute, per (loop, instance), the reference kernel's per-loop phases
// (ExpectValue -> WilsonLoop, intEV.cu:508-582) and the EVMean factors
// (Integrand.c:352-390), and write FP64 partial sums of the W factors.
//
// sweep_kernel (instance-parallel): thread = instance (centre of mass,
//   proper time), CTA = 128 instances x a chunk of loops.  The chunk's loops
//   are streamed through a 4-stage shared-memory ring with bulk copies
//   (cp.async.bulk + mbarrier); every thread walks every point of the staged
//   loop, so each shared-memory load is a warp-wide broadcast and the loop
//   data is read from HBM once per CTA.  Within a loop the points are visited
//   in order; the three sub-loops (N/2: odd points, N/4a: i = 0 mod 4,
//   N/4b: i = 2 mod 4; intEV.cu:461-506) advance together, one group of four
//   points (four segments) at a time, and each segment adds to its sub-loop
//   in the reference's order.  Phases accumulate in FP32 with Kahan
//   compensation per block of 8 groups; W factors accumulate in FP64.
//
// loopwarp_kernel (loop-parallel): warp = (loop, instance), lanes over the
//   groups of four points; per-loop results (EV() and few-instance calls).
#pragma once

#include "wl_device.cuh"
#include "wl_internal.h"

namespace wl {

// the fixflux segment's per-warp queues assume CTAs of kFfWarps warps
static_assert(kSweepThreads == 32 * kFfWarps && kLoopWarps == kFfWarps,
              "fixflux queues: 4 warps per CTA");

// Shared-memory state of the sweep, reused by consecutive tiles of a CTA.
struct SweepShared {
  uint64_t *full_bar;                  // [kSweepStages] mbarriers
  double (*sacc)[kSweepThreads];       // [kMaxF * 3][kSweepThreads] FP64 W - 1 sums
  int *bad;                            // a stage copy timed out
  float4 *ring;                        // [kSweepStages][kSweepChunkPts]
};

__device__ __forceinline__ void sweep_shared_init(const SweepShared &S) {
  if (threadIdx.x == 0) {
    for (int st = 0; st < kSweepStages; ++st) mbar_init(&S.full_bar[st], 1);
    fence_mbar_init();
    *S.bad = 0;
  }
  __syncthreads();
}

// One tile: instances [tile_x * kSweepThreads, +kSweepThreads) of A over the
// loops of chunk `chunk`.  `consumed` counts the stage copies this CTA has
// waited for before (the ring's barrier phases continue across tiles).
// Returns false if a copy timed out (status set, nothing written).
template <int P, bool FERM, int NINT>
__device__ __forceinline__ bool sweep_tile(const SweepArgs &A, int tile_x, int chunk,
                                           const SweepShared &S, int &consumed) {
  const int tid = threadIdx.x;
  const int slot = tile_x * kSweepThreads + tid;
  const bool live = slot < A.ninst;
  const int sl = live ? slot : A.ninst - 1;
  // every per-instance read and the partial-sum write go through ic: a
  // thread's result does not depend on which slot it runs in
  const int ic = A.perm ? A.perm[sl] : sl;
  const int l0 = chunk * A.chunk_loops;
  const int nck = (A.ppl + kSweepChunkPts - 1) / kSweepChunkPts;
  const int K = A.chunk_loops * nck;
  float4 *const ring = S.ring;
  uint64_t *const full_bar = S.full_bar;

  const float cx = A.cx[ic], cy = A.cy[ic], s = A.rtT[ic];
  const FieldDev &F = A.field;
  const df tq = {A.tqh[ic], A.tql[ic]};
  const int base = consumed;

  auto issue = [&](int k) {  // chunk k -> stage (base + k) % kSweepStages
    const int st = (base + k) % kSweepStages;
    const int l = l0 + k / nck, c = k % nck;
    const int p0 = c * kSweepChunkPts;
    const int np = min(kSweepChunkPts, A.ppl - p0);
    const uint32_t bytes = (uint32_t)np * (uint32_t)sizeof(float4);
    mbar_arrive_expect_tx(&full_bar[st], bytes);
    bulk_g2s(ring + st * kSweepChunkPts, A.loops + (size_t)l * A.ppl + p0, bytes,
             &full_bar[st]);
  };
  if (tid == 0)
    for (int k = 0; k < K && k < kSweepStages; ++k) issue(k);

#pragma unroll
  for (int r = 0; r < kMaxF * 3; ++r) S.sacc[r][tid] = 0.0;

  // running sums of the current loop: phase and spin, each with compensation
  float ph[3] = {0.f, 0.f, 0.f}, pc[3] = {0.f, 0.f, 0.f};
  float sp[3] = {0.f, 0.f, 0.f}, sc[3] = {0.f, 0.f, 0.f};
  // previous point of each sub-loop and the first points (closing segments)
  float zAx = 0.f, zAy = 0.f, zBx = 0.f, zBy = 0.f, zOx = 0.f, zOy = 0.f;
  float z0x = 0.f, z0y = 0.f, z1x = 0.f, z1y = 0.f, z2x = 0.f, z2y = 0.f;
  ImgRange img = {0, -1, 0, -1, 1};  // lattice images of the current loop

  int k = 0;
  for (; k < K; ++k) {
    const int st = (base + k) % kSweepStages;
    const uint32_t par = (uint32_t)((base + k) / kSweepStages) & 1u;
    if (!mbar_wait_bounded(&full_bar[st], par, A.wait_tries)) *S.bad = 1;

    const int c = k % nck;
    const int p0 = c * kSweepChunkPts;
    const int p1 = min(A.ppl, p0 + kSweepChunkPts);
    const float2 *pts = reinterpret_cast<const float2 *>(ring + st * kSweepChunkPts);
    auto pt = [&](int p, float &x, float &y) {
      const float2 v = pts[2 * (p - p0)];  // (x, y) of the float4 point
      x = fmaf(s, v.x, cx);
      y = fmaf(s, v.y, cy);
    };

    int q = p0 >> 2;
    const int qend = p1 >> 2;
    if (c == 0) {  // first chunk of a loop: points 0..3 open the sub-loops
#pragma unroll
      for (int r = 0; r < 3; ++r) ph[r] = pc[r] = sp[r] = sc[r] = 0.f;
      if constexpr (P == kLattice) img = image_range(A.bbox[l0 + k / nck], s, cx, cy, F);
      float z3x, z3y;
      pt(0, z0x, z0y);
      pt(1, z1x, z1y);
      pt(2, z2x, z2y);
      pt(3, z3x, z3y);
      seg<P, FERM, NINT>(z1x, z1y, z3x, z3y, F, img, ph[0], sp[0]);  // N/2: 1 -> 3
      zAx = z0x; zAy = z0y;
      zBx = z2x; zBy = z2y;
      zOx = z3x; zOy = z3y;
      q = 1;
    }
    while (q < qend) {
      const int qe = min(q + 8, qend);
      float bp0 = 0.f, bp1 = 0.f, bp2 = 0.f, bs0 = 0.f, bs1 = 0.f, bs2 = 0.f;
      auto group = [&](int qq) {
        float P0x, P0y, P1x, P1y, P2x, P2y, P3x, P3y;
        pt(4 * qq, P0x, P0y);
        pt(4 * qq + 1, P1x, P1y);
        pt(4 * qq + 2, P2x, P2y);
        pt(4 * qq + 3, P3x, P3y);
        seg<P, FERM, NINT>(zAx, zAy, P0x, P0y, F, img, bp2, bs2);  // N/4a: 4q-4 -> 4q
        seg<P, FERM, NINT>(zOx, zOy, P1x, P1y, F, img, bp0, bs0);  // N/2 : 4q-1 -> 4q+1
        seg<P, FERM, NINT>(zBx, zBy, P2x, P2y, F, img, bp1, bs1);  // N/4b: 4q-2 -> 4q+2
        seg<P, FERM, NINT>(P1x, P1y, P3x, P3y, F, img, bp0, bs0);  // N/2 : 4q+1 -> 4q+3
        zAx = P0x; zAy = P0y;
        zBx = P2x; zBy = P2y;
        zOx = P3x; zOy = P3y;
      };
      if constexpr (Profile<P>::kHeavy || P == kLattice) {
#pragma unroll 1
        for (; q < qe; ++q) group(q);
      } else {
#pragma unroll 2
        for (; q < qe; ++q) group(q);
      }
      kahan_add(ph[0], pc[0], bp0);
      kahan_add(ph[1], pc[1], bp1);
      kahan_add(ph[2], pc[2], bp2);
      if (FERM) {
        kahan_add(sp[0], sc[0], bs0);
        kahan_add(sp[1], sc[1], bs1);
        kahan_add(sp[2], sc[2], bs2);
      }
    }

    if (c == nck - 1) {  // last chunk: closing segments back to points 1, 0, 2
      float tp0 = 0.f, tp1 = 0.f, tp2 = 0.f, ts0 = 0.f, ts1 = 0.f, ts2 = 0.f;
      seg<P, FERM, NINT>(zOx, zOy, z1x, z1y, F, img, tp0, ts0);  // N/2 : N-1 -> 1
      seg<P, FERM, NINT>(zBx, zBy, z2x, z2y, F, img, tp1, ts1);  // N/4b: N-2 -> 2
      seg<P, FERM, NINT>(zAx, zAy, z0x, z0y, F, img, tp2, ts2);  // N/4a: N-4 -> 0
      kahan_add(ph[0], pc[0], tp0);
      kahan_add(ph[1], pc[1], tp1);
      kahan_add(ph[2], pc[2], tp2);
      kahan_add(sp[0], sc[0], ts0);
      kahan_add(sp[1], sc[1], ts1);
      kahan_add(sp[2], sc[2], ts2);
      const df G[3] = {fast_two_sum(ph[0], -pc[0]), fast_two_sum(ph[1], -pc[1]),
                       fast_two_sum(ph[2], -pc[2])};
      const df H[3] = {fast_two_sum(sp[0], -sc[0]), fast_two_sum(sp[1], -sc[1]),
                       fast_two_sum(sp[2], -sc[2])};
      loop_epilogue<FERM>(G, H, A.cph_hi, A.cph_lo, A.csp_hi, A.csp_lo, tq, A.nF,
                          [&](int j, double w0, double w1, double w2) {
                            S.sacc[3 * j][tid] += w0;
                            S.sacc[3 * j + 1][tid] += w1;
                            S.sacc[3 * j + 2][tid] += w2;
                          });
    }

    __syncthreads();  // every thread is done with stage st
    if (*S.bad) break;
    if (tid == 0 && k + kSweepStages < K) issue(k + kSweepStages);
  }

  if (*S.bad) {
    // a copy did not arrive in time: wait (bounded) for the copies still in
    // flight so that none lands after the CTA exits, report, write nothing
    if (tid == 0) {
      const int kend = min(K, k + kSweepStages);
      for (int kk = k; kk < kend; ++kk)
        mbar_wait_bounded(&full_bar[(base + kk) % kSweepStages],
                          (uint32_t)((base + kk) / kSweepStages) & 1u, A.wait_tries);
      atomicExch(A.status, kDevTimeout);
    }
    consumed = base + K;
    return false;
  }
  consumed = base + K;

  if (live) {
    for (int r = 0; r < A.nF * 3; ++r)
      A.partial[((size_t)chunk * A.nF * 3 + r) * A.ninst + ic] = S.sacc[r][tid];
  }
  return true;
}

// instances of a packed-pair tile (two per thread)
constexpr int kPairTile = 2 * kSweepThreads;

// ------------------------------------------------ lattice, images outer --
// One segment u_i -> u_j for two images at once (packed pair; u = the loop
// point minus the image centre R, scaled): the Gaussian tube's Simpson
// integral in units of x = rho^2 / lambda^2 (exact mode), each half as
// segment_lattice evaluates one image.  Adds cross * S to ph and the spin
// integral to sp (its 1/l2 scale is applied per loop).
//
// Far nodes: at x > 18, e^-x < 1.6e-8 is below half an ulp of 1, so the
// FP32 integrand (1 - e^-x)/x is exactly 1/x; the spin integrand e^-x is
// taken as 0 there (a change below 1.6e-8 of a node's largest value,
// whichever path runs).  With VOTE, when every node of the segment, in both
// halves and on every active lane of the warp, is far, the segment takes the
// reciprocals alone -- one MUFU operation per node instead of two, and none
// of the small-x polynomial -- with results bit-identical to the full path,
// so an instance's sums still do not depend on its warp-mates.  The walks
// over blocks of staged points decide once per block instead (kLatSub).
// With MID the caller knows every node is at x >= 0.5: the integrand's
// large-x form alone (gauss_q2_big), the same bits as gauss_q2 there.
constexpr float kLatFar = 18.0f;

template <bool FERM, bool VOTE = true, bool MID = false>
__device__ __forceinline__ void lat_seg2(float2 uix, float2 uiy, float2 ujx, float2 ujy,
                                         float2 il2, float2 &ph, float2 &sp) {
  const float2 dx = add2(ujx, neg2(uix)), dy = add2(ujy, neg2(uiy));
  const float2 as = mul2(fma2(uix, uix, mul2(uiy, uiy)), il2);
  // b/l2 alone: 2b/l2, the linear coefficient, is its exact double, which
  // the node polynomial takes through exact halvings and doublings of t
  const float2 bs = mul2(fma2(uix, dx, mul2(uiy, dy)), il2);
  const float2 cs = mul2(fma2(dx, dx, mul2(dy, dy)), il2);
  const float2 cross = mul2(fma2(uix, dy, neg2(mul2(uiy, dx))), il2);
  float2 x[5];
  x[0] = as;
  x[4] = add2(fma2(bs, f2(2.0f), as), cs);  // (as + 2bs) + cs
#pragma unroll
  for (int j = 1; j < 4; j++) {
    const float t = (float)j * 0.25f;
    x[j] = fma2(fma2(cs, f2(0.5f * t), bs), f2(2.0f * t), as);  // as + t (2bs + cs t)
  }
  float xmin = fminf(x[0].x, x[0].y);
#pragma unroll
  for (int j = 1; j < 5; j++) xmin = fminf(xmin, fminf(x[j].x, x[j].y));
  if (VOTE && __all_sync(__activemask(), xmin > kLatFar)) {
    // 1/x at every node; the Simpson sum in the full path's order
    float2 r[5];
#pragma unroll
    for (int j = 0; j < 5; j++) r[j] = rcp2(x[j]);
    const float2 so = add2(r[1], r[3]);
    const float2 se = r[2];
    ph = fma2(cross, fma2(f2(4.0f), so, fma2(f2(2.0f), se, add2(r[0], r[4]))), ph);
    if (FERM) sp = add2(sp, f2(0.0f));
    return;
  }
  float2 q[5], e[5];
#pragma unroll
  for (int j = 0; j < 5; j++) {
    if (MID)  // every node at x >= 0.5 (the caller's block test); il2 > 0
      gauss_q2_big(x[j], q[j], e[j], il2.x < 0.0f ? 1.0f : -1.0f);
    else
      gauss_q2(x[j], q[j], e[j]);
    if (FERM)
      e[j] = make_float2(x[j].x > kLatFar ? 0.0f : e[j].x, x[j].y > kLatFar ? 0.0f : e[j].y);
  }
  ph = fma2(cross, fma2(f2(4.0f), add2(q[1], q[3]), fma2(f2(2.0f), q[2], add2(q[0], q[4]))), ph);
  if (FERM)
    sp = add2(sp, fma2(f2(4.0f), add2(e[1], e[3]), fma2(f2(2.0f), e[2], add2(e[0], e[4]))));
}

// The far path of lat_seg2 alone (no vote): for a walk whose every node is
// known to be far -- the same operations as lat_seg2 takes when its warp
// agrees, so the sums are bit-identical to either path of lat_seg2.  The
// spin integrand is 0 at every far node and its sum is left as it is (the
// full path would add +0 to a sum that is never -0).
__device__ __forceinline__ void lat_seg2_far(float2 uix, float2 uiy, float2 ujx, float2 ujy,
                                             float2 il2, float2 &ph) {
  const float2 dx = add2(ujx, neg2(uix)), dy = add2(ujy, neg2(uiy));
  const float2 as = mul2(fma2(uix, uix, mul2(uiy, uiy)), il2);
  const float2 bs = mul2(fma2(uix, dx, mul2(uiy, dy)), il2);
  const float2 cs = mul2(fma2(dx, dx, mul2(dy, dy)), il2);
  const float2 cross = mul2(fma2(uix, dy, neg2(mul2(uiy, dx))), il2);
  float2 r[5];
  r[0] = rcp2(as);
  r[4] = rcp2(add2(fma2(bs, f2(2.0f), as), cs));
#pragma unroll
  for (int j = 1; j < 4; j++) {
    const float t = (float)j * 0.25f;
    r[j] = rcp2(fma2(fma2(cs, f2(0.5f * t), bs), f2(2.0f * t), as));
  }
  ph = fma2(cross, fma2(f2(4.0f), add2(r[1], r[3]), fma2(f2(2.0f), r[2], add2(r[0], r[4]))), ph);
}

// A walk of an image over a block of kLatSub staged points is far when the
// block's points (and the earlier points its segments start from) lie in a
// box whose nearest point to the image centre is at x = rho^2/lambda^2 > 19:
// every Simpson node lies on a segment inside the box, and its x computed in
// FP32 stays above 18 (the rounding of rho^2 at these sizes is far below the
// 5 % margin).  Such a walk takes lat_seg2_far; any other takes the full
// path of lat_seg2 without its vote (a far node gives the same sums either
// way).  Measured on the a = 2, 5, 10 lambda lattice workloads against one
// walk per segment with a vote: boxes of 32 points with vote-free near walks
// 11-13 % faster; boxes of 64, 128, 256 points 0.5-3 % slower than 32; the
// near walk with the vote kept 4-9 % slower; unrolled by 4, 4-25 % slower.
constexpr float kLatFarChunk = 19.0f;
// A block whose box stays at x > 0.55 from the image centres has every node
// at x >= 0.5 (the same margin argument), where the integrand takes its
// large-x form: the walk skips the small-x polynomial and its selects.
constexpr float kLatMidChunk = 0.55f;
constexpr int kLatSub = 32;  // staged points per far-test box
constexpr int kLatNSub = kSweepChunkPts / kLatSub;
static_assert(kSweepChunkPts % kLatSub == 0 && kLatSub % 4 == 0, "whole groups per box");

// the rarely taken opening / closing segments as one called copy
template <bool FERM>
__device__ __noinline__ float4 lat_seg2_called(float2 uix, float2 uiy, float2 ujx, float2 ujy,
                                               float2 il2, float4 acc) {
  float2 ph = make_float2(acc.x, acc.y), sp = make_float2(acc.z, acc.w);
  lat_seg2<FERM>(uix, uiy, ujx, ujy, il2, ph, sp);
  return make_float4(ph.x, ph.y, sp.x, sp.y);
}

// Lattice tile at 4 intervals with the images outer: two instances A, B per
// thread (slots t and t + 128 of the tile's instance order, 256 per CTA).  For
// every staged chunk of a loop, the images of the two (loop, instance) pairs
// walk all of the chunk's segments two at a time as packed f32x2 pairs:
// A's image p beside B's image p while both have one, then the longer
// list's remaining images two at a time -- ceil((K_A + K_B) / 2) walks, and
// at step p the lanes of a warp hold images in the same position relative
// to similar instances.  A loop point minus an image centre is
// image-independent up to the shift, so the walk starts from the raw
// unit-loop points (reloaded from L2, the same address for every thread);
// per image pair the walk is uniform across the warp (no per-segment image
// loop, no row logic).  An instance's images are its range of image_range()
// flattened row by row (k -> m0 + k / w, n0 + k % w), its rows trimmed to
// the |R| disk where the range crosses it; an unused half is computed and
// not added.  Each image's walk
// over the chunk is summed in FP32 and added once, in image order, to its
// instance's Kahan-compensated loop totals: an instance's sums do not depend
// on its partner or on the tile's other instances.

// shared-memory rows of the lattice tile's loop totals: [instance A/B][phase,
// its compensation, spin, its compensation][sub-loop] x 128 threads (kept out
// of registers: they are touched once per image walk)
constexpr int kLatTotRows = 2 * 4 * 3;

// MIDWALK: walk the blocks between near and far with the large-x form alone
// (the single-job kernel; inside the persistent batch kernel the extra walk
// measured 3 % slower on the uneven batch, so its tiles keep two walks --
// the sums are the same bits either way)
template <bool FERM, bool MIDWALK>
__device__ __forceinline__ bool sweep_tile_lat(const SweepArgs &A, int tile_x, int chunk,
                                               uint64_t *full_bar, double (*sacc)[kPairTile],
                                               float (*tot)[kSweepThreads], int *bad,
                                               float4 *ring, int &consumed) {
  const int tid = threadIdx.x;
  // slots t and t + 128: a tile holding 128 or fewer instances gives each
  // thread at most one (the lanes of a warp still hold consecutive slots)
  const int sA = tile_x * kPairTile + tid, sB = sA + kSweepThreads;
  const bool liveA = sA < A.ninst, liveB = sB < A.ninst;
  const int slA = liveA ? sA : A.ninst - 1, slB = liveB ? sB : A.ninst - 1;
  const int iA = A.perm ? A.perm[slA] : slA, iB = A.perm ? A.perm[slB] : slB;
  const int l0 = chunk * A.chunk_loops;
  const int nck = (A.ppl + kSweepChunkPts - 1) / kSweepChunkPts;
  const int K = A.chunk_loops * nck;
  const FieldDev &F = A.field;
  const int base = consumed;

  auto issue = [&](int k) {
    const int st = (base + k) % kSweepStages;
    const int l = l0 + k / nck, c = k % nck;
    const int p0 = c * kSweepChunkPts;
    const int np = min(kSweepChunkPts, A.ppl - p0);
    const uint32_t bytes = (uint32_t)np * (uint32_t)sizeof(float4);
    mbar_arrive_expect_tx(&full_bar[st], bytes);
    bulk_g2s(ring + st * kSweepChunkPts, A.loops + (size_t)l * A.ppl + p0, bytes, &full_bar[st]);
  };
  if (tid == 0)
    for (int k = 0; k < K && k < kSweepStages; ++k) issue(k);
#pragma unroll
  for (int r = 0; r < kMaxF * 3; ++r) sacc[r][tid] = sacc[r][tid + kSweepThreads] = 0.0;

  const float2 il2 = f2(F.inv_l2);
  // per warp: the staged chunk's far-test boxes (xmin, xmax, ymin, ymax)
  __shared__ float4 lat_box[kSweepThreads / 32][kLatNSub];
  // loop totals per instance (h = 0: A, 1: B), Kahan-compensated, in tot[]
  auto T = [&](int h, int v, int r) -> float & { return tot[(h * 4 + v) * 3 + r][tid]; };
  auto tot_add = [&](int h, int r, float vp, float vs) {
    float a = T(h, 0, r), ac = T(h, 1, r);
    kahan_add(a, ac, vp);
    T(h, 0, r) = a;
    T(h, 1, r) = ac;
    if (FERM) {
      float b = T(h, 2, r), bc = T(h, 3, r);
      kahan_add(b, bc, vs);
      T(h, 2, r) = b;
      T(h, 3, r) = bc;
    }
  };

  int k = 0;
  for (; k < K; ++k) {
    const int st = (base + k) % kSweepStages;
    const uint32_t par = (uint32_t)((base + k) / kSweepStages) & 1u;
    if (!mbar_wait_bounded(&full_bar[st], par, A.wait_tries)) *bad = 1;
    const int c = k % nck;
    const int l = l0 + k / nck;
    const int p0 = c * kSweepChunkPts;
    const int p1 = min(A.ppl, p0 + kSweepChunkPts);
    const float2 *pts = reinterpret_cast<const float2 *>(ring + st * kSweepChunkPts);
    // (x, y) of loop point p: staged points from shared memory, others from L2
    const float2 *gl = reinterpret_cast<const float2 *>(A.loops + (size_t)l * A.ppl);
    auto raw = [&](int p) { return pts[2 * (p - p0)]; };
    auto graw = [&](int p) { return __ldg(&gl[2 * p]); };
    if (c == 0) {
#pragma unroll
      for (int w = 0; w < kLatTotRows; ++w) tot[w][tid] = 0.f;
    }
    const bool last = c == nck - 1;
    // bounding boxes (unit loop) of the points each block of kLatSub staged
    // points' segments touch: the block's points and the four before it (the
    // previous chunk's for the first block); each warp reduces its own copy
    {
      const int lane = tid & 31, w = tid >> 5;
#pragma unroll 1
      for (int b = 0; b < kLatNSub; ++b) {
        const int lo = max(p0 + b * kLatSub - 4, c == 0 ? p0 : p0 - 4);
        const int hi = min(p0 + (b + 1) * kLatSub, p1);
        float x0 = INFINITY, x1 = -INFINITY, y0 = INFINITY, y1 = -INFINITY;
        for (int i = lo + lane; i < hi; i += 32) {
          const float2 v = i >= p0 ? raw(i) : graw(i);
          x0 = fminf(x0, v.x);
          x1 = fmaxf(x1, v.x);
          y0 = fminf(y0, v.y);
          y1 = fmaxf(y1, v.y);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          x0 = fminf(x0, __shfl_xor_sync(0xffffffffu, x0, o));
          x1 = fmaxf(x1, __shfl_xor_sync(0xffffffffu, x1, o));
          y0 = fminf(y0, __shfl_xor_sync(0xffffffffu, y0, o));
          y1 = fmaxf(y1, __shfl_xor_sync(0xffffffffu, y1, o));
        }
        if (lane == 0) lat_box[w][b] = make_float4(x0, x1, y0, y1);
      }
      __syncwarp();
    }
    // the nearest point of block b's box, scaled and shifted as U() maps the
    // points (fma(s, w, c - R) is monotone in w), is far from the image centre
    auto block_x = [&](int b, float sc, float crx, float cry) {
      const float4 bb = lat_box[tid >> 5][b];
      const float lx = fmaf(sc, bb.x, crx), hx = fmaf(sc, bb.y, crx);
      const float ly = fmaf(sc, bb.z, cry), hy = fmaf(sc, bb.w, cry);
      const float ex = fmaxf(fmaxf(lx, -hx), 0.0f), ey = fmaxf(fmaxf(ly, -hy), 0.0f);
      return fmaf(ex, ex, ey * ey) * F.inv_l2;
    };
    // this loop's images of each instance
    const float4 bb = A.bbox[l];
    const ImgRange gA = image_range(bb, A.rtT[iA], A.cx[iA], A.cy[iA], F);
    const ImgRange gB = image_range(bb, A.rtT[iB], A.cx[iB], A.cy[iB], F);
    const int widA = max(gA.n1 - gA.n0 + 1, 1), widB = max(gB.n1 - gB.n0 + 1, 1);
    // row m of a range trimmed to the disk m^2 + n^2 <= (rimage/a)^2 (the
    // criterion image_range uses for `inside`)
    auto row = [&](const ImgRange &g, int m, int &lo, int &hi) {
      const float mm = (float)(m * m);
      int nx = (int)floorf(sqrtf(fmaxf(F.rimg2 - mm, 0.0f)));
      while (nx >= 0 && mm + (float)(nx * nx) > F.rimg2) --nx;
      while (mm + (float)((nx + 1) * (nx + 1)) <= F.rimg2) ++nx;
      lo = max(g.n0, -nx);
      hi = min(g.n1, nx);
    };
    auto count = [&](const ImgRange &g, int wid) {
      if (g.m1 < g.m0 || g.n1 < g.n0) return 0;
      if (g.inside) return (g.m1 - g.m0 + 1) * wid;
      int c = 0;
      for (int m = g.m0; m <= g.m1; ++m) {
        int lo, hi;
        row(g, m, lo, hi);
        c += max(hi - lo + 1, 0);
      }
      return c;
    };
    // a slot past the tile's instances walks nothing
    const int nA = liveA ? count(gA, widA) : 0, nB = liveB ? count(gB, widB) : 0;
    const int mn = min(nA, nB), mx = max(nA, nB);
    const int steps = mn + (mx - mn + 1) / 2;
    const int qa = c == 0 ? 1 : (p0 >> 2), qend = p1 >> 2;
    for (int p = 0; p < steps; ++p) {
      // the step's two images: (A p, B p), then the longer list two at a time
      int jx, jy;
      bool bx, by;
      if (p < mn) {
        jx = jy = p;
        bx = false;
        by = true;
      } else {
        jx = mn + 2 * (p - mn);
        jy = jx + 1;
        bx = by = nB > nA;
      }
      auto image = [&](int j, bool isB, bool &ok, float &s, float &crx, float &cry) {
        const ImgRange &g = isB ? gB : gA;
        const int wd = isB ? widB : widA, n = isB ? nB : nA;
        int jj = min(j, n - 1), m, nn;
        if (g.inside) {
          m = g.m0 + jj / wd;
          nn = g.n0 + jj % wd;
        } else {  // the rows trimmed to the disk, in order
          m = g.m0;
          nn = g.n0;
          for (int mr = g.m0; mr <= g.m1; ++mr) {
            int lo, hi;
            row(g, mr, lo, hi);
            const int cnt = max(hi - lo + 1, 0);
            if (jj < cnt) {
              m = mr;
              nn = lo + jj;
              break;
            }
            jj -= cnt;
          }
        }
        ok = j < n;
        const int ic = isB ? iB : iA;
        s = A.rtT[ic];
        crx = fmaf(-(float)m, F.a, A.cx[ic]);
        cry = fmaf(-(float)nn, F.a, A.cy[ic]);
      };
      bool okx, oky;
      float sx, sy, cxx, cxy, cyx, cyy;
      image(jx, bx, okx, sx, cxx, cyx);
      image(jy, by, oky, sy, cxy, cyy);
      const float2 s2 = make_float2(sx, sy);
      const float2 crx = make_float2(cxx, cxy), cry = make_float2(cyx, cyy);
      // point minus image centre, scaled: u = s w + (c - R)
      auto U = [&](float2 w, float2 &ux, float2 &uy) {
        ux = fma2(s2, f2(w.x), crx);
        uy = fma2(s2, f2(w.y), cry);
      };
      float2 bp[3] = {f2(0.f), f2(0.f), f2(0.f)}, bs[3] = {f2(0.f), f2(0.f), f2(0.f)};
      float2 uAx, uAy, uBx, uBy, uOx, uOy;
      if (c == 0) {  // the N/2 sub-loop's first segment 1 -> 3; sub-loops open at 0, 2, 3
        float2 u1x, u1y, u3x, u3y;
        U(raw(1), u1x, u1y);
        U(raw(3), u3x, u3y);
        const float4 r = lat_seg2_called<FERM>(u1x, u1y, u3x, u3y, il2,
                                               make_float4(0.f, 0.f, 0.f, 0.f));
        bp[0] = make_float2(r.x, r.y);
        bs[0] = make_float2(r.z, r.w);
        U(raw(0), uAx, uAy);
        U(raw(2), uBx, uBy);
        uOx = u3x;
        uOy = u3y;
      } else {  // the previous chunk's last points of each sub-loop
        U(graw(p0 - 4), uAx, uAy);
        U(graw(p0 - 2), uBx, uBy);
        U(graw(p0 - 1), uOx, uOy);
      }
      auto group4 = [&](int q, auto &&segf) {
        float2 P0x, P0y, P1x, P1y, P2x, P2y, P3x, P3y;
        U(raw(4 * q), P0x, P0y);
        U(raw(4 * q + 1), P1x, P1y);
        U(raw(4 * q + 2), P2x, P2y);
        U(raw(4 * q + 3), P3x, P3y);
        segf(uAx, uAy, P0x, P0y, 2);  // N/4a: 4q-4 -> 4q
        segf(uOx, uOy, P1x, P1y, 0);  // N/2 : 4q-1 -> 4q+1
        segf(uBx, uBy, P2x, P2y, 1);  // N/4b: 4q-2 -> 4q+2
        segf(P1x, P1y, P3x, P3y, 0);  // N/2 : 4q+1 -> 4q+3
        uAx = P0x; uAy = P0y;
        uBx = P2x; uBy = P2y;
        uOx = P3x; uOy = P3y;
      };
      auto far_seg = [&](float2 ix, float2 iy, float2 jx, float2 jy, int r) {
        lat_seg2_far(ix, iy, jx, jy, il2, bp[r]);
      };
      auto mid_seg = [&](float2 ix, float2 iy, float2 jx, float2 jy, int r) {
        lat_seg2<FERM, false, true>(ix, iy, jx, jy, il2, bp[r], bs[r]);
      };
      auto near_seg = [&](float2 ix, float2 iy, float2 jx, float2 jy, int r) {
        lat_seg2<FERM, false>(ix, iy, jx, jy, il2, bp[r], bs[r]);
      };
#pragma unroll 1
      for (int b = 0; b < kLatNSub; ++b) {
        const int q0 = max(qa, (p0 + b * kLatSub) >> 2);
        const int q1 = min(qend, (p0 + (b + 1) * kLatSub) >> 2);
        // an unused half is not added: it never holds the warp back
        const float xb = fminf(okx ? block_x(b, sx, cxx, cyx) : INFINITY,
                               oky ? block_x(b, sy, cxy, cyy) : INFINITY);
        const unsigned am = __activemask();
        if (__all_sync(am, xb > kLatFarChunk)) {
          // every node of the block's walk is far: reciprocals only, no
          // per-segment vote, four segments of straight-line work per group
#pragma unroll 2
          for (int q = q0; q < q1; ++q) group4(q, far_seg);
        } else if (MIDWALK && __all_sync(am, xb > kLatMidChunk)) {
          // no node near an image centre: the integrand's large-x form alone
#pragma unroll 2
          for (int q = q0; q < q1; ++q) group4(q, mid_seg);
        } else {
#pragma unroll 2
          for (int q = q0; q < q1; ++q) group4(q, near_seg);
        }
      }
      if (last) {  // closing segments back to points 1, 2, 0
        float2 ux, uy;
        float4 r;
        U(graw(1), ux, uy);
        r = lat_seg2_called<FERM>(uOx, uOy, ux, uy, il2,
                                  make_float4(bp[0].x, bp[0].y, bs[0].x, bs[0].y));
        bp[0] = make_float2(r.x, r.y);
        bs[0] = make_float2(r.z, r.w);
        U(graw(2), ux, uy);
        r = lat_seg2_called<FERM>(uBx, uBy, ux, uy, il2,
                                  make_float4(bp[1].x, bp[1].y, bs[1].x, bs[1].y));
        bp[1] = make_float2(r.x, r.y);
        bs[1] = make_float2(r.z, r.w);
        U(graw(0), ux, uy);
        r = lat_seg2_called<FERM>(uAx, uAy, ux, uy, il2,
                                  make_float4(bp[2].x, bp[2].y, bs[2].x, bs[2].y));
        bp[2] = make_float2(r.x, r.y);
        bs[2] = make_float2(r.z, r.w);
      }
      // each image's chunk sums into its instance's totals, in image order
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        if (okx) tot_add(bx ? 1 : 0, r, bp[r].x, bs[r].x);
        if (oky) tot_add(by ? 1 : 0, r, bp[r].y, bs[r].y);
      }
    }
    if (last) {
#pragma unroll 1
      for (int h = 0; h < 2; ++h) {  // per-loop epilogue of each instance
        const int ih = h ? iB : iA, col = tid + h * kSweepThreads;
        const df G[3] = {fast_two_sum(T(h, 0, 0), -T(h, 1, 0)),
                         fast_two_sum(T(h, 0, 1), -T(h, 1, 1)),
                         fast_two_sum(T(h, 0, 2), -T(h, 1, 2))};
        const df H[3] = {fast_two_sum(T(h, 2, 0), -T(h, 3, 0)),
                         fast_two_sum(T(h, 2, 1), -T(h, 3, 1)),
                         fast_two_sum(T(h, 2, 2), -T(h, 3, 2))};
        const df tq = {A.tqh[ih], A.tql[ih]};
        loop_epilogue<FERM>(G, H, A.cph_hi, A.cph_lo, A.csp_hi, A.csp_lo, tq, A.nF,
                            [&](int j, double d0, double d1, double d2) {
                              sacc[3 * j][col] += d0;
                              sacc[3 * j + 1][col] += d1;
                              sacc[3 * j + 2][col] += d2;
                            });
      }
    }
    __syncthreads();
    if (*bad) break;
    if (tid == 0 && k + kSweepStages < K) issue(k + kSweepStages);
  }
  if (*bad) {
    if (tid == 0) {
      const int kend = min(K, k + kSweepStages);
      for (int kk = k; kk < kend; ++kk)
        mbar_wait_bounded(&full_bar[(base + kk) % kSweepStages],
                          (uint32_t)((base + kk) / kSweepStages) & 1u, A.wait_tries);
      atomicExch(A.status, kDevTimeout);
    }
    consumed = base + K;
    return false;
  }
  consumed = base + K;
  for (int r = 0; r < A.nF * 3; ++r) {
    double *o = A.partial + ((size_t)chunk * A.nF * 3 + r) * A.ninst;
    if (liveA) o[iA] = sacc[r][tid];
    if (liveB) o[iB] = sacc[r][tid + kSweepThreads];
  }
  return true;
}

// The same tile on packed pairs: thread t runs instances t and t + 128 of a
// tile of kPairTile, every FP32 operation of the segments as one f32x2
// operation on the pair (each half rounds as the scalar sweep does); the
// per-loop epilogue runs per half.  Light profiles with a fixed interval count.
template <int P, bool FERM, int NINT>
__device__ __forceinline__ bool sweep_tile2(const SweepArgs &A, int tile_x, int chunk,
                                            uint64_t *full_bar, double (*sacc)[kPairTile],
                                            int *bad, float4 *ring, int &consumed) {
  const int tid = threadIdx.x;
  const int sA = tile_x * kPairTile + tid, sB = sA + kSweepThreads;
  const bool liveA = sA < A.ninst, liveB = sB < A.ninst;
  const int iA = liveA ? sA : A.ninst - 1, iB = liveB ? sB : A.ninst - 1;
  const int l0 = chunk * A.chunk_loops;
  const int nck = (A.ppl + kSweepChunkPts - 1) / kSweepChunkPts;
  const int K = A.chunk_loops * nck;
  const float2 cx = make_float2(A.cx[iA], A.cx[iB]), cy = make_float2(A.cy[iA], A.cy[iB]);
  const float2 s = make_float2(A.rtT[iA], A.rtT[iB]);
  const FieldDev &F = A.field;
  const int base = consumed;

  auto issue = [&](int k) {
    const int st = (base + k) % kSweepStages;
    const int l = l0 + k / nck, c = k % nck;
    const int p0 = c * kSweepChunkPts;
    const int np = min(kSweepChunkPts, A.ppl - p0);
    const uint32_t bytes = (uint32_t)np * (uint32_t)sizeof(float4);
    mbar_arrive_expect_tx(&full_bar[st], bytes);
    bulk_g2s(ring + st * kSweepChunkPts, A.loops + (size_t)l * A.ppl + p0, bytes,
             &full_bar[st]);
  };
  if (tid == 0)
    for (int k = 0; k < K && k < kSweepStages; ++k) issue(k);
#pragma unroll
  for (int r = 0; r < kMaxF * 3; ++r) sacc[r][tid] = sacc[r][tid + kSweepThreads] = 0.0;

  float2 ph[3], pc[3], sp[3], sc[3];
  float2 zAx = f2(0.f), zAy = f2(0.f), zBx = f2(0.f), zBy = f2(0.f), zOx = f2(0.f), zOy = f2(0.f);
  float2 z0x = f2(0.f), z0y = f2(0.f), z1x = f2(0.f), z1y = f2(0.f), z2x = f2(0.f), z2y = f2(0.f);
#pragma unroll
  for (int r = 0; r < 3; ++r) ph[r] = pc[r] = sp[r] = sc[r] = f2(0.f);

  int k = 0;
  for (; k < K; ++k) {
    const int st = (base + k) % kSweepStages;
    const uint32_t par = (uint32_t)((base + k) / kSweepStages) & 1u;
    if (!mbar_wait_bounded(&full_bar[st], par, A.wait_tries)) *bad = 1;
    const int c = k % nck;
    const int p0 = c * kSweepChunkPts;
    const int p1 = min(A.ppl, p0 + kSweepChunkPts);
    const float2 *pts = reinterpret_cast<const float2 *>(ring + st * kSweepChunkPts);
    auto pt = [&](int p, float2 &x, float2 &y) {
      const float2 v = pts[2 * (p - p0)];
      x = fma2(s, f2(v.x), cx);
      y = fma2(s, f2(v.y), cy);
    };
    int q = p0 >> 2;
    const int qend = p1 >> 2;
    if (c == 0) {
#pragma unroll
      for (int r = 0; r < 3; ++r) ph[r] = pc[r] = sp[r] = sc[r] = f2(0.f);
      float2 z3x, z3y;
      pt(0, z0x, z0y);
      pt(1, z1x, z1y);
      pt(2, z2x, z2y);
      pt(3, z3x, z3y);
      seg2<P, FERM, NINT>(z1x, z1y, z3x, z3y, F, ph[0], sp[0]);
      zAx = z0x; zAy = z0y;
      zBx = z2x; zBy = z2y;
      zOx = z3x; zOy = z3y;
      q = 1;
    }
    while (q < qend) {
      const int qe = min(q + 8, qend);
      float2 bp0 = f2(0.f), bp1 = f2(0.f), bp2 = f2(0.f), bs0 = f2(0.f), bs1 = f2(0.f),
             bs2 = f2(0.f);
#pragma unroll 2
      for (; q < qe; ++q) {
        float2 P0x, P0y, P1x, P1y, P2x, P2y, P3x, P3y;
        pt(4 * q, P0x, P0y);
        pt(4 * q + 1, P1x, P1y);
        pt(4 * q + 2, P2x, P2y);
        pt(4 * q + 3, P3x, P3y);
        seg2<P, FERM, NINT>(zAx, zAy, P0x, P0y, F, bp2, bs2);
        seg2<P, FERM, NINT>(zOx, zOy, P1x, P1y, F, bp0, bs0);
        seg2<P, FERM, NINT>(zBx, zBy, P2x, P2y, F, bp1, bs1);
        seg2<P, FERM, NINT>(P1x, P1y, P3x, P3y, F, bp0, bs0);
        zAx = P0x; zAy = P0y;
        zBx = P2x; zBy = P2y;
        zOx = P3x; zOy = P3y;
      }
      kahan_add2(ph[0], pc[0], bp0);
      kahan_add2(ph[1], pc[1], bp1);
      kahan_add2(ph[2], pc[2], bp2);
      if (FERM) {
        kahan_add2(sp[0], sc[0], bs0);
        kahan_add2(sp[1], sc[1], bs1);
        kahan_add2(sp[2], sc[2], bs2);
      }
    }
    if (c == nck - 1) {
      float2 tp0 = f2(0.f), tp1 = f2(0.f), tp2 = f2(0.f), ts0 = f2(0.f), ts1 = f2(0.f),
             ts2 = f2(0.f);
      seg2<P, FERM, NINT>(zOx, zOy, z1x, z1y, F, tp0, ts0);
      seg2<P, FERM, NINT>(zBx, zBy, z2x, z2y, F, tp1, ts1);
      seg2<P, FERM, NINT>(zAx, zAy, z0x, z0y, F, tp2, ts2);
      kahan_add2(ph[0], pc[0], tp0);
      kahan_add2(ph[1], pc[1], tp1);
      kahan_add2(ph[2], pc[2], tp2);
      kahan_add2(sp[0], sc[0], ts0);
      kahan_add2(sp[1], sc[1], ts1);
      kahan_add2(sp[2], sc[2], ts2);
#pragma unroll 1
      for (int h = 0; h < 2; ++h) {  // per-loop epilogue of each half
        auto lane = [h](float2 v) { return h ? v.y : v.x; };
        const int ih = h ? iB : iA, col = tid + h * kSweepThreads;
        const df G[3] = {fast_two_sum(lane(ph[0]), -lane(pc[0])),
                         fast_two_sum(lane(ph[1]), -lane(pc[1])),
                         fast_two_sum(lane(ph[2]), -lane(pc[2]))};
        const df H[3] = {fast_two_sum(lane(sp[0]), -lane(sc[0])),
                         fast_two_sum(lane(sp[1]), -lane(sc[1])),
                         fast_two_sum(lane(sp[2]), -lane(sc[2]))};
        const df tq = {A.tqh[ih], A.tql[ih]};
        loop_epilogue<FERM>(G, H, A.cph_hi, A.cph_lo, A.csp_hi, A.csp_lo, tq, A.nF,
                            [&](int j, double w0, double w1, double w2) {
                              sacc[3 * j][col] += w0;
                              sacc[3 * j + 1][col] += w1;
                              sacc[3 * j + 2][col] += w2;
                            });
      }
    }
    __syncthreads();
    if (*bad) break;
    if (tid == 0 && k + kSweepStages < K) issue(k + kSweepStages);
  }
  if (*bad) {
    if (tid == 0) {
      const int kend = min(K, k + kSweepStages);
      for (int kk = k; kk < kend; ++kk)
        mbar_wait_bounded(&full_bar[(base + kk) % kSweepStages],
                          (uint32_t)((base + kk) / kSweepStages) & 1u, A.wait_tries);
      atomicExch(A.status, kDevTimeout);
    }
    consumed = base + K;
    return false;
  }
  consumed = base + K;
  for (int r = 0; r < A.nF * 3; ++r) {
    double *o = A.partial + ((size_t)chunk * A.nF * 3 + r) * A.ninst;
    if (liveA) o[iA] = sacc[r][tid];
    if (liveB) o[iB] = sacc[r][tid + kSweepThreads];
  }
  return true;
}

template <int P, bool FERM, int NINT>
__global__ void __launch_bounds__(kSweepThreads, 4)
    sweep2_kernel(const __grid_constant__ SweepArgs A) {
  extern __shared__ __align__(128) float4 ring[];
  __shared__ __align__(8) uint64_t full_bar[kSweepStages];
  __shared__ int sm_bad;
  __shared__ double sacc[kMaxF * 3][kPairTile];
  if (threadIdx.x == 0) {
    for (int st = 0; st < kSweepStages; ++st) mbar_init(&full_bar[st], 1);
    fence_mbar_init();
    sm_bad = 0;
  }
  __syncthreads();
  int consumed = 0;
  sweep_tile2<P, FERM, NINT>(A, blockIdx.x, blockIdx.y, full_bar, sacc, &sm_bad, ring, consumed);
}

template <int P, bool FERM, int NINT>
__global__ void __launch_bounds__(kSweepThreads,
                                  (Profile<P>::kHeavy || P == kLattice) ? 4 : kSweepMinBlocks)
    sweep_kernel(const __grid_constant__ SweepArgs A) {
  extern __shared__ __align__(128) float4 ring[];  // [kSweepStages][kSweepChunkPts]
  __shared__ __align__(8) uint64_t full_bar[kSweepStages];
  __shared__ int sm_bad;
  // FP64 W-factor sums per (flux value, factor, instance): kept in shared
  // memory (touched once per loop) so they do not hold 24 registers
  __shared__ double sacc[kMaxF * 3][kSweepThreads];
  const SweepShared S = {full_bar, sacc, &sm_bad, ring};
  sweep_shared_init(S);
  int consumed = 0;
  sweep_tile<P, FERM, NINT>(A, blockIdx.x, blockIdx.y, S, consumed);
}

// the lattice at 4 intervals: images outer, two instances per thread
template <bool FERM>
__global__ void __launch_bounds__(kSweepThreads, 4)
    sweep_lat_kernel(const __grid_constant__ SweepArgs A) {
  extern __shared__ __align__(128) float4 ring[];
  __shared__ __align__(8) uint64_t full_bar[kSweepStages];
  __shared__ int sm_bad;
  __shared__ double sacc[kMaxF * 3][kPairTile];
  __shared__ float tot[kLatTotRows][kSweepThreads];
  if (threadIdx.x == 0) {
    for (int st = 0; st < kSweepStages; ++st) mbar_init(&full_bar[st], 1);
    fence_mbar_init();
    sm_bad = 0;
  }
  __syncthreads();
  int consumed = 0;
  sweep_tile_lat<FERM, true>(A, blockIdx.x, blockIdx.y, full_bar, sacc, tot, &sm_bad, ring,
                             consumed);
}

template <int P, bool FERM, int NINT>
__global__ void __launch_bounds__(kLoopWarps * 32)
    loopwarp_kernel(const __grid_constant__ LoopArgs A) {
  const int lane = threadIdx.x & 31;
  const int l = blockIdx.x * kLoopWarps + (threadIdx.x >> 5);
  const int inst = blockIdx.y;
  if (l >= A.Nl) return;  // whole warp
  const float cx = A.cx[inst], cy = A.cy[inst], s = A.rtT[inst];
  const FieldDev &F = A.field;
  const float2 *w = reinterpret_cast<const float2 *>(A.loops + (size_t)l * A.ppl);
  auto pt = [&](int p, float &x, float &y) {
    const float2 v = __ldg(&w[2 * p]);
    x = fmaf(s, v.x, cx);
    y = fmaf(s, v.y, cy);
  };
  // group q covers points 4q..4q+3 and the four segments ending there; the
  // previous points of group 0 wrap to the end of the loop (closing segments)
  const int nq = A.ppl >> 2;
  ImgRange img = {0, -1, 0, -1, 1};
  if constexpr (P == kLattice) img = image_range(A.bbox[l], s, cx, cy, F);
  float ph[3] = {0.f, 0.f, 0.f}, sp[3] = {0.f, 0.f, 0.f};
  for (int q = lane; q < nq; q += 32) {
    const int pa = (q == 0 ? A.ppl : 4 * q) - 4;
    float zAx, zAy, zBx, zBy, zOx, zOy, P0x, P0y, P1x, P1y, P2x, P2y, P3x, P3y;
    pt(pa, zAx, zAy);
    pt(pa + 2, zBx, zBy);
    pt(pa + 3, zOx, zOy);
    pt(4 * q, P0x, P0y);
    pt(4 * q + 1, P1x, P1y);
    pt(4 * q + 2, P2x, P2y);
    pt(4 * q + 3, P3x, P3y);
    seg<P, FERM, NINT>(zAx, zAy, P0x, P0y, F, img, ph[2], sp[2]);
    seg<P, FERM, NINT>(zOx, zOy, P1x, P1y, F, img, ph[0], sp[0]);
    seg<P, FERM, NINT>(zBx, zBy, P2x, P2y, F, img, ph[1], sp[1]);
    seg<P, FERM, NINT>(P1x, P1y, P3x, P3y, F, img, ph[0], sp[0]);
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      ph[r] += __shfl_xor_sync(0xffffffffu, ph[r], off);
      if (FERM) sp[r] += __shfl_xor_sync(0xffffffffu, sp[r], off);
    }
  }
  if (lane == 0) {
    const df tq = {A.tqh[inst], A.tql[inst]};
    const df G[3] = {df{ph[0], 0.f}, df{ph[1], 0.f}, df{ph[2], 0.f}};
    const df H[3] = {df{sp[0], 0.f}, df{sp[1], 0.f}, df{sp[2], 0.f}};
    loop_epilogue<FERM>(G, H, A.cph_hi, A.cph_lo, A.csp_hi, A.csp_lo, tq, A.nF,
                        [&](int j, double w0, double w1, double w2) {
                          double *o = A.partial + ((size_t)(l * A.nF + j) * 3) * A.ninst + inst;
                          o[0] = w0;
                          o[A.ninst] = w1;
                          o[2 * (size_t)A.ninst] = w2;
                        });
    // Wsscal / Wsferm of the first flux value (intEV.cu:553-561)
    const size_t o = (size_t)inst * A.Nl + l;
    auto val = [](df x) { return x.hi + x.lo; };
    const df cph0 = {A.cph_hi[0], A.cph_lo[0]};
    if (A.scal)
      A.scal[o] = make_float4(val(df_mul(cph0, G[0])), val(df_mul(cph0, G[1])),
                              val(df_mul(cph0, G[2])), 0.0f);
    if (FERM && A.ferm) {
      const df csp0 = df_mul(df{A.csp_hi[0], A.csp_lo[0]}, tq);
      A.ferm[o] = make_float4(val(df_mul(csp0, H[0])), 2.0f * val(df_mul(csp0, H[1])),
                              2.0f * val(df_mul(csp0, H[2])), 0.0f);
    }
  }
}

// instantiation + dispatch over (fermion, nint) for one profile
template <int P>
cudaError_t sweep_dispatch(bool fermion, int nint, const SweepArgs &a, cudaStream_t s) {
  const dim3 grid((a.ninst + kSweepThreads - 1) / kSweepThreads, a.n_chunks);
  const size_t smem = sweep_smem_bytes();
  const dim3 grid2((a.ninst + kPairTile - 1) / kPairTile, a.n_chunks);
  if constexpr (P == kSmooth || P == kStep || P == kQuadratic || P == kGaussian) {
    if (nint == 4) {  // packed pairs
      if (fermion)
        sweep2_kernel<P, true, 4><<<grid2, kSweepThreads, smem, s>>>(a);
      else
        sweep2_kernel<P, false, 4><<<grid2, kSweepThreads, smem, s>>>(a);
      return cudaGetLastError();
    }
  }
#ifndef WL_PAIRS50
#define WL_PAIRS50 1
#endif
  if constexpr ((P == kSmooth || P == kStep || P == kQuadratic || P == kGaussian) && WL_PAIRS50) {
    if (nint == 50) {  // the reference's interval count: packed pairs (smooth:
                       // a share of the reciprocals on the FP32 pipe); measured
                       // over one instance per thread: smooth +3 % / +7 %
                       // (scalar / spinor), Gaussian +56 % / +54 %, step
                       // +4 % / +31 %, quadratic +35 % / +24 %
      if (fermion)
        sweep2_kernel<P, true, 50><<<grid2, kSweepThreads, smem, s>>>(a);
      else
        sweep2_kernel<P, false, 50><<<grid2, kSweepThreads, smem, s>>>(a);
      return cudaGetLastError();
    }
  }
  // one instance per thread: other interval counts at run time (a
  // run-time-interval pair kernel measured 26 % slower than the unrolled
  // scalar 50), the lattice at 4 too, and the heavy profiles; the scalar 50
  // serves the loop-parallel kernel
#define WL_SWEEP_CASE(FE, NI)                                                      \
  if (fermion == FE && (NI == 0 || nint == NI)) {                                  \
    sweep_kernel<P, FE, NI><<<grid, kSweepThreads, smem, s>>>(a);                  \
    return cudaGetLastError();                                                     \
  }
  if constexpr (P == kLattice) {
    if (nint == 4) {  // images outer, two instances per thread
      // static shared memory (37 KiB) plus the ring exceeds the 48 KiB a
      // launch gets without opting in (a per-device attribute)
      auto k = fermion ? sweep_lat_kernel<true> : sweep_lat_kernel<false>;
      const cudaError_t e =
          cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
      k<<<grid2, kSweepThreads, smem, s>>>(a);
      return cudaGetLastError();
    }
  }
  if constexpr (!Profile<P>::kHeavy && P != kLattice) {
    WL_SWEEP_CASE(true, 50)
    WL_SWEEP_CASE(false, 50)
  }
  WL_SWEEP_CASE(true, 0)
  WL_SWEEP_CASE(false, 0)
#undef WL_SWEEP_CASE
  return cudaErrorInvalidValue;
}

template <int P>
cudaError_t loopwarp_dispatch(bool fermion, int nint, const LoopArgs &a, cudaStream_t s) {
  const dim3 grid((a.Nl + kLoopWarps - 1) / kLoopWarps, a.ninst);
#define WL_LOOP_CASE(FE, NI)                                                       \
  if (fermion == FE && (NI == 0 || nint == NI)) {                                  \
    loopwarp_kernel<P, FE, NI><<<grid, kLoopWarps * 32, 0, s>>>(a);                \
    return cudaGetLastError();                                                     \
  }
  if constexpr (!Profile<P>::kHeavy) {
    WL_LOOP_CASE(true, 4)
    WL_LOOP_CASE(false, 4)
  }
  if constexpr (!Profile<P>::kHeavy && P != kLattice) {
    WL_LOOP_CASE(true, 50)
    WL_LOOP_CASE(false, 50)
  }
  WL_LOOP_CASE(true, 0)
  WL_LOOP_CASE(false, 0)
#undef WL_LOOP_CASE
  return cudaErrorInvalidValue;
}

}  // namespace wl
