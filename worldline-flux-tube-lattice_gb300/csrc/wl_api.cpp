// wl_api.cpp -- C-ABI runtime of libwlgpu.so (include/wlgpu.h, wl_legacy.h).
//
// Owns contexts (device + stream + workspaces), resident loop ensembles, the
// launch planning of the sweep kernels and the legacy EV() entry point of
// intEV.cu:111-148.
#include <cuda.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/wl_legacy.h"
#include "../../include/wlgpu.h"
#include "wl_internal.h"
#include "wl_spline.h"

using wl::FieldDev;

namespace {

// ------------------------------------------------------------ helpers --
template <typename T>
struct DevBuf {  // grow-only device buffer
  T *p = nullptr;
  size_t n = 0;
  cudaError_t reserve(size_t want) {
    if (want <= n) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
    cudaError_t e = cudaMalloc((void **)&p, want * sizeof(T));
    if (e == cudaSuccess) n = want;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
};

struct Ensemble {
  float4 *dev = nullptr;
  int Nl = 0, ppl = 0;
  bool owned = false;
  float4 *bbox = nullptr;  // per-loop bounding boxes, computed on first lattice use
};

typedef CUresult (*AddressRangeFn)(CUdeviceptr *, size_t *, CUdeviceptr);

}  // namespace

struct wl_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  int num_sms = 0;
  std::map<int, Ensemble> ens;
  int next_handle = 1;
  DevBuf<float> inst;       // cx, cy, rtT, tq  (4 * ninst)
  DevBuf<double> partial;   // sweep partial sums
  DevBuf<double> out;       // group values, means, SEMs
  DevBuf<int> status;       // device status word
  DevBuf<int> list;         // EV() loop list
  DevBuf<int> perm;         // lattice: instances in decreasing proper time
  DevBuf<double> aux;       // proper-time integral inputs and outputs
  // batches: instances, partial sums, outputs, descriptors (jobs, tiles,
  // reduce jobs, queue counter)
  DevBuf<float> b_inst;
  DevBuf<double> b_part, b_out;
  DevBuf<unsigned char> b_meta;
  DevBuf<int> b_perm;
  int tune_points = 16384;  // points per tile target (autotuned)
  int tune_ctas = 0;        // persistent CTAs per SM, 0 = occupancy limit
  double last_batch_ms = 0.0;
  int last_batch_tiles = 0, last_batch_grid = 0;
  std::vector<float> h_inst;
  std::string err;
  int last_launches = 0;
  const char *last_kind = "none";
  AddressRangeFn addr_range = nullptr;
  // spline profile tables on the device, by (lambda^2, a)
  std::map<std::pair<double, double>, std::pair<float *, float4 *>> splines;
};

namespace {

int fail(wl_ctx *ctx, int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (ctx) ctx->err = buf;
  return code;
}

int cuda_fail(wl_ctx *ctx, cudaError_t e, const char *what) {
  return fail(ctx, WL_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define WL_CHECK(ctx, call)                                   \
  do {                                                        \
    cudaError_t e_ = (call);                                  \
    if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call);  \
  } while (0)

// Device memory covering [p, p + bytes) on the context's device?  Refuses
// host pointers before any kernel can dereference them.
int check_device_range(wl_ctx *ctx, const void *p, size_t bytes, const char *name) {
  if (!p) return fail(ctx, WL_ERR_INVALID, "%s is NULL", name);
  if ((uintptr_t)p % 16 != 0) return fail(ctx, WL_ERR_INVALID, "%s is not 16-byte aligned", name);
  cudaPointerAttributes at;
  cudaError_t e = cudaPointerGetAttributes(&at, p);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(ctx, WL_ERR_INVALID, "%s is not a CUDA pointer", name);
  }
  if (at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged)
    return fail(ctx, WL_ERR_INVALID, "%s is not device memory", name);
  if (at.type == cudaMemoryTypeDevice && at.device != ctx->device)
    return fail(ctx, WL_ERR_INVALID, "%s lives on device %d, context on %d", name, at.device,
                ctx->device);
  if (ctx->addr_range) {
    CUdeviceptr base = 0;
    size_t size = 0;
    if (ctx->addr_range(&base, &size, (CUdeviceptr)(uintptr_t)p) == CUDA_SUCCESS) {
      if ((uintptr_t)p + bytes > (uintptr_t)base + size)
        return fail(ctx, WL_ERR_INVALID, "%s: %zu bytes exceed its allocation", name, bytes);
    }
  }
  return WL_OK;
}

int field_to_dev(wl_ctx *ctx, const wl_field *f, int *kprofile, FieldDev *d) {
  if (!f) return fail(ctx, WL_ERR_INVALID, "field is NULL");
  int p = f->profile;
  if (!(p == WL_PROFILE_STEP || p == WL_PROFILE_SMOOTH || p == WL_PROFILE_QUADRATIC ||
        p == WL_PROFILE_GAUSSIAN || p == WL_PROFILE_PERIODIC || p == WL_PROFILE_FIXFLUX ||
        p == WL_PROFILE_LATTICE || p == WL_PROFILE_SPLINE))
    return fail(ctx, WL_ERR_INVALID, "unsupported profile %d", p);
  if (p == WL_PROFILE_LATTICE) {
    if (f->mode != WL_MODE_EXACT)
      return fail(ctx, WL_ERR_INVALID, "the lattice profile needs WL_MODE_EXACT");
    if (!(f->tubedist > 0.0) || !isfinite(f->tubedist) || !(f->rimage >= 0.0) ||
        !isfinite(f->rimage) || f->rimage / f->tubedist > 1000.0)
      return fail(ctx, WL_ERR_INVALID, "lattice: need tubedist > 0 and 0 <= rimage <= 1000 a");
  }
  if (f->nint < 2 || f->nint > 64 || f->nint % 2)
    return fail(ctx, WL_ERR_INVALID, "nint must be even in [2, 64], got %d", f->nint);
  if (f->mode != WL_MODE_REFCOMPAT && f->mode != WL_MODE_EXACT)
    return fail(ctx, WL_ERR_INVALID, "unknown mode %d", f->mode);
  if (!(f->lambda2 > 0.0) || !isfinite(f->lambda2))
    return fail(ctx, WL_ERR_INVALID, "lambda2 must be positive");
  if ((p == WL_PROFILE_PERIODIC || p == WL_PROFILE_FIXFLUX || p == WL_PROFILE_SPLINE) &&
      (!(f->tubedist > 0.0) || !isfinite(f->tubedist)))
    return fail(ctx, WL_ERR_INVALID, "tubedist must be positive");
  if (p == WL_PROFILE_FIXFLUX && !(f->tubedist > f->lmin))
    return fail(ctx, WL_ERR_INVALID, "fixflux needs tubedist > lmin");
  *kprofile = (p == WL_PROFILE_FIXFLUX && f->ff_variant) ? wl::kFixfluxFF : p;
  if (p == WL_PROFILE_LATTICE) *kprofile = wl::kLattice;
  if (p == WL_PROFILE_SPLINE) *kprofile = wl::kSpline;
  memset(d, 0, sizeof(*d));
  d->l2 = (float)f->lambda2;
  d->inv_l2 = 1.0f / d->l2;
  d->lam = sqrtf(d->l2);
  d->a = (float)f->tubedist;
  d->lmin = (float)f->lmin;
  if (p == WL_PROFILE_FIXFLUX) {
    d->lml = (d->lam - d->lmin) / (d->a - d->lmin);
    d->aml = (d->a - d->lam) / (d->a - d->lmin);
  }
  d->nint = f->nint;
  d->h = 1.0f / (float)f->nint;
  if (p == WL_PROFILE_LATTICE) {
    const double rr = f->rimage / f->tubedist;
    d->rimg2 = (float)(rr * rr * (1.0 + 1e-6));
    d->rcut = (float)(4.242640687119285 * sqrt(f->lambda2));  // sqrt(18) lambda
  }
  if (p == WL_PROFILE_SPLINE) {  // the table itself is attached per context
    d->sp_n = wl::kSplineKnots;
    d->sp_h = (float)(20.0 / wl::kSplineKnots);
    // f' argument: the reference kernel's sin(pi rho) (intEV.cu:391) or the
    // derivative of the tabulated profile, sin(pi rho / a)
    d->sp_piarg = (float)(f->mode == WL_MODE_REFCOMPAT ? M_PI : M_PI / f->tubedist);
  }
  if (f->mode == WL_MODE_REFCOMPAT) {
    d->clampA = d->clampB = d->clampC = d->clampE = 1.0e-8f;
    d->clampI = 1.0e-10f;
  } else {
    const bool divides =
        (p == WL_PROFILE_PERIODIC || p == WL_PROFILE_FIXFLUX || p == WL_PROFILE_SPLINE);
    const float fl = divides ? 1.0e-30f : -INFINITY;
    d->clampA = d->clampE = d->clampI = fl;
    d->clampB = d->clampC = -INFINITY;
  }
  return WL_OK;
}

// Double-float per-flux constants of the per-loop epilogue:
// cph = F h/3 (phase) and csp = F h/3 * fp_scale (spin, times 4T/N per
// instance on the device), fp_scale being the constant the kernels factor
// out of f' (Profile<P>::fp_scale).
template <typename Args>
void fill_flux(Args &a, const wl_field *f, int nF, const double *F) {
  const double h3 = 1.0 / (3.0 * (double)f->nint);
  double fs = 1.0;
  switch (f->profile) {
    case WL_PROFILE_SMOOTH: fs = (double)(float)f->lambda2; break;
    case WL_PROFILE_STEP:
    case WL_PROFILE_GAUSSIAN:
    case WL_PROFILE_LATTICE: fs = 1.0 / (double)(float)f->lambda2; break;
    case WL_PROFILE_QUADRATIC: fs = 2.0 / (double)(float)f->lambda2; break;
    default: fs = 1.0;
  }
  for (int j = 0; j < wl::kMaxF; ++j) {
    const double Fj = j < nF ? F[j] : 0.0;
    const double cp = Fj * h3, cs = Fj * h3 * fs;
    a.F[j] = (float)Fj;
    a.cph_hi[j] = (float)cp;
    a.cph_lo[j] = (float)(cp - (double)(float)cp);
    a.csp_hi[j] = (float)cs;
    a.csp_lo[j] = (float)(cs - (double)(float)cs);
  }
}

int lookup(wl_ctx *ctx, int handle, Ensemble *e) {
  auto it = ctx->ens.find(handle);
  if (it == ctx->ens.end()) return fail(ctx, WL_ERR_NOTFOUND, "unknown ensemble %d", handle);
  *e = it->second;
  return WL_OK;
}

int set_device(wl_ctx *ctx) {
  WL_CHECK(ctx, cudaSetDevice(ctx->device));
  return WL_OK;
}

// per-loop bounding boxes of an ensemble, computed once (lattice images)
int ensure_bbox(wl_ctx *ctx, int handle, const float4 **out) {
  auto it = ctx->ens.find(handle);
  if (it == ctx->ens.end()) return fail(ctx, WL_ERR_NOTFOUND, "unknown ensemble %d", handle);
  Ensemble &e = it->second;
  if (!e.bbox) {
    if (cudaMalloc((void **)&e.bbox, sizeof(float4) * e.Nl) != cudaSuccess) {
      cudaGetLastError();
      e.bbox = nullptr;
      return fail(ctx, WL_ERR_NOMEM, "cannot allocate loop bounding boxes");
    }
    WL_CHECK(ctx, wl::launch_loop_bbox(e.dev, e.Nl, e.ppl, e.bbox, ctx->stream));
  }
  *out = e.bbox;
  return WL_OK;
}

// the spline profile's table for (lambda^2, a) on the device, built once
int ensure_spline(wl_ctx *ctx, const wl_field *f, FieldDev *d) {
  const auto key = std::make_pair(f->lambda2, f->tubedist);
  auto it = ctx->splines.find(key);
  if (it == ctx->splines.end()) {
    const int n = wl::kSplineKnots;
    std::vector<float> rho2(n), coef(4 * (size_t)n);
    if (wl::spline_table(f->lambda2, f->tubedist, n, rho2.data(), coef.data()))
      return fail(ctx, WL_ERR_INVALID, "spline table: invalid lambda2 or tubedist");
    float *dr = nullptr;
    float4 *dc = nullptr;
    if (cudaMalloc((void **)&dr, sizeof(float) * n) != cudaSuccess ||
        cudaMalloc((void **)&dc, sizeof(float4) * n) != cudaSuccess) {
      cudaGetLastError();
      if (dr) cudaFree(dr);
      return fail(ctx, WL_ERR_NOMEM, "cannot allocate the spline table");
    }
    WL_CHECK(ctx, cudaMemcpy(dr, rho2.data(), sizeof(float) * n, cudaMemcpyHostToDevice));
    WL_CHECK(ctx, cudaMemcpy(dc, coef.data(), sizeof(float4) * n, cudaMemcpyHostToDevice));
    it = ctx->splines.emplace(key, std::make_pair(dr, dc)).first;
  }
  d->sp_rho2 = it->second.first;
  d->sp_coef = it->second.second;
  return WL_OK;
}

// stage per-instance constants: cx, cy, rtT = float(sqrt(T)) (intEV.cu:118,
// 124) and tq = 4 rtT^2/ppl (the 2T/(N/2) spin normalisation,
// intEV.cu:558-560) as a float pair hi + lo.  The kernel thus evaluates the
// instance (float(cx), float(cy), T' = float(sqrt(T))^2) exactly.
int upload_instances(wl_ctx *ctx, int ninst, const double *cx, const double *cy,
                     const double *T, int ppl) {
  for (int i = 0; i < ninst; ++i) {
    if (!isfinite(cx[i]) || !isfinite(cy[i]) || !(T[i] > 0.0) || !isfinite(T[i]))
      return fail(ctx, WL_ERR_INVALID, "instance %d: need finite centre and T > 0", i);
  }
  const int na = wl::kInstArrays;
  ctx->h_inst.resize((size_t)na * ninst);
  float *h = ctx->h_inst.data();
  for (int i = 0; i < ninst; ++i) {
    // the loops are scaled by float(sqrt(T)); the spin normalisation uses the
    // same T' = rtT^2, as the reference's rtT*rtT (intEV.cu:558)
    const float rtT = (float)sqrt(T[i]);
    const double tq = 4.0 * ((double)rtT * (double)rtT) / (double)ppl;
    h[i] = (float)cx[i];
    h[ninst + i] = (float)cy[i];
    h[2 * ninst + i] = rtT;
    h[3 * ninst + i] = (float)tq;
    h[4 * ninst + i] = (float)(tq - (double)(float)tq);
  }
  WL_CHECK(ctx, ctx->inst.reserve((size_t)na * ninst));
  // the staging vector is pageable and reused: copy synchronously
  WL_CHECK(ctx, cudaMemcpyAsync(ctx->inst.p, h, sizeof(float) * na * ninst,
                                cudaMemcpyHostToDevice, ctx->stream));
  WL_CHECK(ctx, cudaStreamSynchronize(ctx->stream));
  return WL_OK;
}

// Loops per CTA of the instance-parallel sweep: the largest divisor of the
// group size not above 8.  It depends on the ensemble's grouping only, never on
// the batch, so an instance's partial sums -- and its result, bit for bit --
// are the same whatever other instances share the launch.
int plan_chunk(int group) {
  int lc = 8;
  while (group % lc) lc /= 2;
  return lc;
}

int check_status(wl_ctx *ctx) {
  int st = 0;
  WL_CHECK(ctx, cudaMemcpyAsync(&st, ctx->status.p, sizeof(int), cudaMemcpyDeviceToHost,
                                ctx->stream));
  WL_CHECK(ctx, cudaStreamSynchronize(ctx->stream));
  if (st == wl::kDevTimeout)
    return fail(ctx, WL_ERR_TIMEOUT, "a shared-memory stage copy timed out on the device");
  if (st == wl::kDevBadInstance)
    return fail(ctx, WL_ERR_INVALID, "an instance has T <= 0 or a non-finite value");
  return WL_OK;
}

}  // namespace

namespace {
struct LegacyState {
  std::mutex mu;
  wl_field field = {WL_PROFILE_SMOOTH, 0, 50, WL_MODE_REFCOMPAT, 0, 0, 1.0, 1.0, 0.1};
  int config_gen = 1;
  wl_ctx *ctx = nullptr;
  // cache key
  bool valid = false;
  double T = 0, F = 0, l2 = 0;
  float cx = 0, cy = 0;
  const void *loops = nullptr;
  int Nl = 0, ppl = 0, fermion = 0, gen = 0;
  DevBuf<double> w;    // per-loop W factors [Nl][3]
  DevBuf<double> res;  // list mean
  // <W> of the consecutive groups g*128 .. g*128+127 at the cached (T, x_cm):
  // the groups the reference's callers pass (identity order, Tint.c:87-92),
  // computed once per (T, x_cm) so that their EV() calls need no device work
  DevBuf<double> gres;
  std::vector<double> gev;
  // fingerprint of the cached sweep's ensemble coordinates, and its scratch
  unsigned long long fp = 0;
  DevBuf<unsigned long long> fpd;
};
LegacyState &legacy() {
  static LegacyState s;
  return s;
}
}  // namespace


// ============================================================== batches ==
extern "C" {
static int eval_prologue(wl_ctx *ctx, int handle, const wl_field *field, int ninst, int nF,
                         const double *host_F, int group, Ensemble *e, int *kprof,
                         FieldDev *fd);
}

namespace {

// loops per tile of a job: the largest divisor of its group size not above
// points_per_tile / ppl (at least 1)
int batch_loops_per_tile(int points_per_tile, int ppl, int group) {
  int want = points_per_tile / ppl;
  if (want < 1) want = 1;
  int lc = want < group ? want : group;
  while (group % lc) --lc;
  return lc;
}

struct BatchPlan {
  size_t perm_total = 0;  // lattice jobs' instance orders
  std::vector<wl::SweepArgs> jobs;
  std::vector<wl::BatchTile> tiles;
  std::vector<int> side;  // heavy-profile jobs: their own sweep launch each
  std::vector<wl::ReduceJob> rjobs;
  std::vector<float> inst;
  size_t part_total = 0, out_total = 0;
  int flat_total = 0;
};

int batch_plan(wl_ctx *ctx, int njobs, const wl_job *jobs, int points, BatchPlan *P) {
  size_t inst_total = 0;
  std::vector<size_t> inst_off(njobs), part_off(njobs), out_off(njobs);
  std::vector<int> lcs(njobs), kprofs(njobs);
  std::vector<FieldDev> fds(njobs);
  for (int i = 0; i < njobs; ++i) {
    const wl_job &J = jobs[i];
    Ensemble e;
    int r = eval_prologue(ctx, J.handle, &J.field, J.ninst, J.nF, J.F, J.group, &e, &kprofs[i],
                          &fds[i]);
    if (r) return fail(ctx, r, "job %d: %s", i, ctx->err.c_str());
    if (!J.cx || !J.cy || !J.T) return fail(ctx, WL_ERR_INVALID, "job %d: NULL instance arrays", i);
    if (!wl::batch_supports(kprofs[i], J.field.nint))
      return fail(ctx, WL_ERR_INVALID, "job %d: profile %d is not supported in batches", i,
                  J.field.profile);
    lcs[i] = batch_loops_per_tile(points, e.ppl, J.group);
    inst_off[i] = inst_total;
    inst_total += (size_t)wl::kInstArrays * J.ninst;
    part_off[i] = P->part_total;
    P->part_total += (size_t)(e.Nl / lcs[i]) * J.nF * 3 * J.ninst;
    out_off[i] = P->out_total;
    P->out_total += (size_t)J.ninst * J.nF * (e.Nl / J.group + 2);
  }
  P->inst.resize(inst_total);
  P->jobs.resize(njobs);
  P->rjobs.resize(njobs);
  P->tiles.clear();
  for (int i = 0; i < njobs; ++i) {
    const wl_job &J = jobs[i];
    Ensemble e;
    lookup(ctx, J.handle, &e);
    for (int k = 0; k < J.ninst; ++k)
      if (!isfinite(J.cx[k]) || !isfinite(J.cy[k]) || !(J.T[k] > 0.0) || !isfinite(J.T[k]))
        return fail(ctx, WL_ERR_INVALID, "job %d instance %d: need finite centre and T > 0", i, k);
    float *h = P->inst.data() + inst_off[i];
    const int n = J.ninst;
    for (int k = 0; k < n; ++k) {
      const float rtT = (float)sqrt(J.T[k]);
      const double tq = 4.0 * ((double)rtT * (double)rtT) / (double)e.ppl;
      h[k] = (float)J.cx[k];
      h[n + k] = (float)J.cy[k];
      h[2 * n + k] = rtT;
      h[3 * n + k] = (float)tq;
      h[4 * n + k] = (float)(tq - (double)(float)tq);
    }
    wl::SweepArgs &a = P->jobs[i];
    memset(&a, 0, sizeof(a));
    a.loops = e.dev;
    a.Nl = e.Nl;
    a.ppl = e.ppl;
    a.ninst = n;
    // device pointers are patched in after the buffers are sized (offsets now)
    a.cx = (const float *)(uintptr_t)(inst_off[i]);
    a.nF = J.nF;
    fill_flux(a, &J.field, J.nF, J.F);
    a.field = fds[i];
    a.chunk_loops = lcs[i];
    a.n_chunks = e.Nl / lcs[i];
    a.partial = (double *)(uintptr_t)(part_off[i]);
    a.wait_tries = 1u << 22;
    a.kprof = kprofs[i];
    a.fermion = J.field.fermion != 0;
    a.nint = J.field.nint;
    if (kprofs[i] == wl::kLattice) {
      int rb = ensure_bbox(ctx, J.handle, &a.bbox);
      if (rb) return rb;
      // offset + 1 now (0 = none); patched into a device pointer later
      a.perm = (const int *)(uintptr_t)(P->perm_total + 1);
      P->perm_total += (size_t)n;
    }
    wl::ReduceJob &rj = P->rjobs[i];
    rj.n_chunks = a.n_chunks;
    rj.cpg = J.group / lcs[i];
    rj.lpg = J.group;
    rj.ninst = n;
    rj.nF = J.nF;
    rj.first = P->flat_total;
    rj.out_group = (double *)(uintptr_t)(out_off[i]);
    P->flat_total += n * J.nF;
    if (!wl::batch_in_kernel(kprofs[i])) {
      P->side.push_back(i);
      continue;
    }
    const int per_tile = wl::sweep_tile_instances(kprofs[i], J.field.nint);
    const int tiles_x = (n + per_tile - 1) / per_tile;
    const int cost = lcs[i] * e.ppl * (per_tile / wl::kSweepThreads);
    for (int c = 0; c < a.n_chunks; ++c)
      for (int t = 0; t < tiles_x; ++t) P->tiles.push_back({i, t, c, cost});
  }
  // longest tiles first: the queue then drains evenly (LPT order); ties keep
  // job order
  std::stable_sort(P->tiles.begin(), P->tiles.end(),
                   [](const wl::BatchTile &x, const wl::BatchTile &y) { return x.cost > y.cost; });
  return WL_OK;
}

int batch_run(wl_ctx *ctx, int njobs, const wl_job *jobs, int flags, int points, int ctas,
              bool copy_out) {
  BatchPlan P;
  int r = batch_plan(ctx, njobs, jobs, points, &P);
  if (r) return r;
  if (P.tiles.empty() && P.side.empty()) return fail(ctx, WL_ERR_INVALID, "empty batch");
  const size_t jobs_bytes = sizeof(wl::SweepArgs) * njobs;
  const size_t tiles_bytes = sizeof(wl::BatchTile) * P.tiles.size();
  const size_t rj_bytes = sizeof(wl::ReduceJob) * njobs;
  const size_t off_tiles = (jobs_bytes + 255) & ~(size_t)255;
  const size_t off_rj = (off_tiles + tiles_bytes + 255) & ~(size_t)255;
  const size_t off_cnt = (off_rj + rj_bytes + 255) & ~(size_t)255;
  const size_t meta_bytes = off_cnt + 256;
  if (ctx->b_inst.reserve(P.inst.size()) != cudaSuccess ||
      ctx->b_part.reserve(P.part_total) != cudaSuccess ||
      ctx->b_out.reserve(P.out_total) != cudaSuccess ||
      ctx->b_meta.reserve(meta_bytes) != cudaSuccess ||
      (P.perm_total && ctx->b_perm.reserve(P.perm_total) != cudaSuccess)) {
    cudaGetLastError();
    return fail(ctx, WL_ERR_NOMEM, "cannot allocate the batch buffers");
  }
  // patch offsets into device pointers
  for (int i = 0; i < njobs; ++i) {
    wl::SweepArgs &a = P.jobs[i];
    const size_t io = (size_t)(uintptr_t)a.cx;
    const int n = a.ninst;
    a.cx = ctx->b_inst.p + io;
    a.cy = a.cx + n;
    a.rtT = a.cx + 2 * n;
    a.tqh = a.cx + 3 * n;
    a.tql = a.cx + 4 * n;
    a.partial = ctx->b_part.p + (size_t)(uintptr_t)a.partial;
    a.status = ctx->status.p;
    if (a.perm) a.perm = ctx->b_perm.p + ((size_t)(uintptr_t)a.perm - 1);
    wl::ReduceJob &rj = P.rjobs[i];
    rj.partial = a.partial;
    const int ng = a.Nl / rj.lpg;
    rj.out_group = ctx->b_out.p + (size_t)(uintptr_t)rj.out_group;
    rj.out_mean = rj.out_group + (size_t)n * rj.nF * ng;
    rj.out_sem = rj.out_mean + (size_t)n * rj.nF;
  }
  unsigned char *meta = ctx->b_meta.p;
  WL_CHECK(ctx, cudaMemcpyAsync(ctx->b_inst.p, P.inst.data(), sizeof(float) * P.inst.size(),
                                cudaMemcpyHostToDevice, ctx->stream));
  WL_CHECK(ctx, cudaMemcpyAsync(meta, P.jobs.data(), jobs_bytes, cudaMemcpyHostToDevice, ctx->stream));
  WL_CHECK(ctx, cudaMemcpyAsync(meta + off_tiles, P.tiles.data(), tiles_bytes,
                                cudaMemcpyHostToDevice, ctx->stream));
  WL_CHECK(ctx, cudaMemcpyAsync(meta + off_rj, P.rjobs.data(), rj_bytes, cudaMemcpyHostToDevice,
                                ctx->stream));
  WL_CHECK(ctx, cudaMemsetAsync(ctx->status.p, 0, sizeof(int), ctx->stream));
  for (int i = 0; i < njobs; ++i)  // lattice jobs: instances in decreasing proper time
    if (P.jobs[i].perm)
      WL_CHECK(ctx, wl::launch_order_instances(P.jobs[i].cx, P.jobs[i].cy, P.jobs[i].rtT,
                                               P.jobs[i].ninst, 1.0f / P.jobs[i].field.a,
                                               const_cast<int *>(P.jobs[i].perm), ctx->stream));
  WL_CHECK(ctx, cudaStreamSynchronize(ctx->stream));  // host vectors are released on return

  wl::BatchArgs B;
  B.jobs = (const wl::SweepArgs *)meta;
  B.tiles = (const wl::BatchTile *)(meta + off_tiles);
  B.ntiles = (int)P.tiles.size();
  B.counter = (int *)(meta + off_cnt);
  const int occ = wl::batch_max_ctas_per_sm();
  const int per_sm = ctas > 0 && ctas <= occ ? ctas : occ;
  int grid = per_sm * ctx->num_sms;
  if (grid > B.ntiles) grid = B.ntiles;
  const wl::ReduceJob *rjd = (const wl::ReduceJob *)(meta + off_rj);
  // kernels per run: the persistent kernel, the side sweeps, the reduction
  const int launches = (B.ntiles > 0 ? 1 : 0) + (int)P.side.size() + 1;

  cudaEvent_t e0, e1;
  WL_CHECK(ctx, cudaEventCreate(&e0));
  WL_CHECK(ctx, cudaEventCreate(&e1));
  auto enqueue = [&]() -> cudaError_t {
    cudaError_t e = cudaSuccess;
    if (B.ntiles > 0) {
      e = cudaMemsetAsync(B.counter, 0, sizeof(int), ctx->stream);
      if (e == cudaSuccess) e = wl::launch_batch(B, grid, ctx->stream);
    }
    for (int i : P.side) {  // heavy profiles: their own sweep, same partial layout
      if (e != cudaSuccess) break;
      const wl::SweepArgs &a = P.jobs[i];
      e = wl::launch_sweep(a.kprof, a.fermion != 0, a.nint, a, ctx->stream);
    }
    if (e == cudaSuccess) e = wl::launch_batch_reduce(rjd, njobs, P.flat_total, ctx->stream);
    return e;
  };
  cudaError_t ce = cudaEventRecord(e0, ctx->stream);
  if (ce == cudaSuccess) {
    if (flags & WL_BATCH_GRAPH) {
      cudaGraph_t g = nullptr;
      cudaGraphExec_t ge = nullptr;
      ce = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
      if (ce == cudaSuccess) {
        cudaError_t ce2 = enqueue();
        ce = cudaStreamEndCapture(ctx->stream, &g);
        if (ce2 != cudaSuccess) ce = ce2;
      }
      if (ce == cudaSuccess) ce = cudaGraphInstantiate(&ge, g, 0);
      if (ce == cudaSuccess) ce = cudaGraphLaunch(ge, ctx->stream);
      if (ce == cudaSuccess) ce = cudaStreamSynchronize(ctx->stream);
      if (ge) cudaGraphExecDestroy(ge);
      if (g) cudaGraphDestroy(g);
    } else {
      ce = enqueue();
    }
  }
  if (ce == cudaSuccess) ce = cudaEventRecord(e1, ctx->stream);
  if (ce == cudaSuccess) ce = cudaEventSynchronize(e1);
  float ms = 0.0f;
  if (ce == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (ce != cudaSuccess) return cuda_fail(ctx, ce, "batch launch");
  ctx->last_batch_ms = ms;
  ctx->last_batch_tiles = B.ntiles;
  ctx->last_batch_grid = grid;
  ctx->last_launches = launches;
  ctx->last_kind = "persistent-batch";
  if ((r = check_status(ctx))) return r;
  if (!copy_out) return WL_OK;
  std::vector<double> host(P.out_total);
  WL_CHECK(ctx, cudaMemcpyAsync(host.data(), ctx->b_out.p, sizeof(double) * P.out_total,
                                cudaMemcpyDeviceToHost, ctx->stream));
  WL_CHECK(ctx, cudaStreamSynchronize(ctx->stream));
  for (int i = 0; i < njobs; ++i) {
    const wl_job &J = jobs[i];
    const wl::ReduceJob &rj = P.rjobs[i];
    const int ng = P.jobs[i].Nl / J.group;
    const size_t o = (size_t)(rj.out_group - ctx->b_out.p);
    const size_t ngrp = (size_t)J.ninst * J.nF * ng, nm = (size_t)J.ninst * J.nF;
    if (J.out_group) memcpy(J.out_group, host.data() + o, sizeof(double) * ngrp);
    if (J.out_mean) memcpy(J.out_mean, host.data() + o + ngrp, sizeof(double) * nm);
    if (J.out_sem) memcpy(J.out_sem, host.data() + o + ngrp + nm, sizeof(double) * nm);
  }
  return WL_OK;
}

}  // namespace

// ================================================================ C ABI ==
// Only the C entry points are exported (the build hides everything else).
#pragma GCC visibility push(default)
extern "C" {

const char *wl_version(void) { return "wlgpu 0.1 (sm_103a)"; }

const char *wl_status_string(int s) {
  switch (s) {
    case WL_OK: return "ok";
    case WL_ERR_INVALID: return "invalid argument";
    case WL_ERR_CUDA: return "CUDA error";
    case WL_ERR_NOMEM: return "out of memory";
    case WL_ERR_TIMEOUT: return "device wait timed out";
    case WL_ERR_NOTFOUND: return "unknown handle";
    case WL_ERR_ADMISSION: return "admission rejected";
    default: return "unknown status";
  }
}

int wl_ctx_create(int device, wl_ctx **out) {
  if (!out) return WL_ERR_INVALID;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) {
    cudaGetLastError();
    return WL_ERR_CUDA;
  }
  wl_ctx *ctx = new wl_ctx();
  ctx->device = device;
  if (cudaSetDevice(device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device) !=
          cudaSuccess ||
      ctx->status.reserve(1) != cudaSuccess ||
      cudaMemset(ctx->status.p, 0, sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    delete ctx;
    return WL_ERR_CUDA;
  }
  void *fn = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion("cuMemGetAddressRange", &fn, 12000, cudaEnableDefault,
                                       &q) == cudaSuccess &&
      q == cudaDriverEntryPointSuccess)
    ctx->addr_range = (AddressRangeFn)fn;
  cudaGetLastError();
  *out = ctx;
  return WL_OK;
}

int wl_ctx_destroy(wl_ctx *ctx) {
  if (!ctx) return WL_ERR_INVALID;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  for (auto &kv : ctx->ens) {
    if (kv.second.owned) cudaFree(kv.second.dev);
    if (kv.second.bbox) cudaFree(kv.second.bbox);
  }
  ctx->inst.release();
  ctx->partial.release();
  ctx->out.release();
  ctx->status.release();
  ctx->list.release();
  for (auto &kv : ctx->splines) {
    cudaFree(kv.second.first);
    cudaFree(kv.second.second);
  }
  ctx->splines.clear();
  ctx->perm.release();
  ctx->b_perm.release();
  ctx->aux.release();
  ctx->b_inst.release();
  ctx->b_part.release();
  ctx->b_out.release();
  ctx->b_meta.release();
  cudaStreamDestroy(ctx->stream);
  delete ctx;
  return WL_OK;
}

int wl_last_error(wl_ctx *ctx, char *buf, int buflen) {
  if (!ctx || !buf || buflen <= 0) return WL_ERR_INVALID;
  snprintf(buf, (size_t)buflen, "%s", ctx->err.c_str());
  return WL_OK;
}

int wl_ctx_synchronize(wl_ctx *ctx) {
  if (!ctx) return WL_ERR_INVALID;
  int r = set_device(ctx);
  if (r) return r;
  r = check_status(ctx);
  if (r != WL_OK) cudaMemsetAsync(ctx->status.p, 0, sizeof(int), ctx->stream);
  return r;
}

static int check_shape(wl_ctx *ctx, int Nl, int ppl) {
  if (Nl < 1 || ppl < 4 || ppl % 4 != 0)
    return fail(ctx, WL_ERR_INVALID, "need Nl >= 1 and ppl a positive multiple of 4 (Nl=%d ppl=%d)",
                Nl, ppl);
  if ((double)Nl * (double)ppl > 2147483647.0)
    return fail(ctx, WL_ERR_INVALID, "ensemble too large (%d x %d points)", Nl, ppl);
  return WL_OK;
}

int wl_ensemble_upload(wl_ctx *ctx, const float *host_loops, int Nl, int ppl, int *handle) {
  if (!ctx || !host_loops || !handle) return fail(ctx, WL_ERR_INVALID, "NULL argument");
  int r = check_shape(ctx, Nl, ppl);
  if (r) return r;
  if ((r = set_device(ctx))) return r;
  Ensemble e;
  e.Nl = Nl;
  e.ppl = ppl;
  e.owned = true;
  const size_t bytes = (size_t)Nl * ppl * sizeof(float4);
  if (cudaMalloc((void **)&e.dev, bytes) != cudaSuccess) {
    cudaGetLastError();
    return fail(ctx, WL_ERR_NOMEM, "cannot allocate %zu bytes for the ensemble", bytes);
  }
  cudaError_t ce = cudaMemcpyAsync(e.dev, host_loops, bytes, cudaMemcpyHostToDevice, ctx->stream);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(ctx->stream);
  if (ce != cudaSuccess) {
    cudaFree(e.dev);
    return cuda_fail(ctx, ce, "ensemble upload");
  }
  *handle = ctx->next_handle++;
  ctx->ens[*handle] = e;
  return WL_OK;
}

int wl_ensemble_wrap(wl_ctx *ctx, const float *dev_loops, int Nl, int ppl, int *handle) {
  if (!ctx || !handle) return fail(ctx, WL_ERR_INVALID, "NULL argument");
  int r = check_shape(ctx, Nl, ppl);
  if (r) return r;
  if ((r = set_device(ctx))) return r;
  if ((r = check_device_range(ctx, dev_loops, (size_t)Nl * ppl * sizeof(float4), "dev_loops")))
    return r;
  Ensemble e;
  e.dev = (float4 *)dev_loops;
  e.Nl = Nl;
  e.ppl = ppl;
  e.owned = false;
  *handle = ctx->next_handle++;
  ctx->ens[*handle] = e;
  return WL_OK;
}

int wl_ensemble_generate(wl_ctx *ctx, uint64_t seed, int first, int Nl, int ppl,
                         int *handle) {
  if (!ctx || !handle) return fail(ctx, WL_ERR_INVALID, "NULL argument");
  int r = check_shape(ctx, Nl, ppl);
  if (r) return r;
  if (first < 0) return fail(ctx, WL_ERR_INVALID, "first must be >= 0");
  if ((r = set_device(ctx))) return r;
  Ensemble e;
  e.Nl = Nl;
  e.ppl = ppl;
  e.owned = true;
  const size_t bytes = (size_t)Nl * ppl * sizeof(float4);
  if (cudaMalloc((void **)&e.dev, bytes) != cudaSuccess) {
    cudaGetLastError();
    return fail(ctx, WL_ERR_NOMEM, "cannot allocate %zu bytes for the ensemble", bytes);
  }
  cudaError_t ce = wl::launch_vloops(seed, first, Nl, ppl, e.dev, ctx->stream);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(ctx->stream);
  if (ce != cudaSuccess) {
    cudaFree(e.dev);
    return cuda_fail(ctx, ce, "loop generator");
  }
  *handle = ctx->next_handle++;
  ctx->ens[*handle] = e;
  return WL_OK;
}

int wl_ensemble_download(wl_ctx *ctx, int handle, float *host_loops) {
  if (!ctx || !host_loops) return fail(ctx, WL_ERR_INVALID, "NULL argument");
  Ensemble e;
  int r = lookup(ctx, handle, &e);
  if (r) return r;
  if ((r = set_device(ctx))) return r;
  WL_CHECK(ctx, cudaMemcpyAsync(host_loops, e.dev, (size_t)e.Nl * e.ppl * sizeof(float4),
                                cudaMemcpyDeviceToHost, ctx->stream));
  WL_CHECK(ctx, cudaStreamSynchronize(ctx->stream));
  return WL_OK;
}

int wl_ensemble_release(wl_ctx *ctx, int handle) {
  if (!ctx) return WL_ERR_INVALID;
  Ensemble e;
  int r = lookup(ctx, handle, &e);
  if (r) return r;
  if ((r = set_device(ctx))) return r;
  WL_CHECK(ctx, cudaStreamSynchronize(ctx->stream));
  if (e.owned) cudaFree(e.dev);
  if (e.bbox) cudaFree(e.bbox);
  ctx->ens.erase(handle);
  return WL_OK;
}

int wl_ensemble_info(wl_ctx *ctx, int handle, const float **dev_loops, int *Nl, int *ppl) {
  if (!ctx) return WL_ERR_INVALID;
  Ensemble e;
  int r = lookup(ctx, handle, &e);
  if (r) return r;
  if (dev_loops) *dev_loops = (const float *)e.dev;
  if (Nl) *Nl = e.Nl;
  if (ppl) *ppl = e.ppl;
  return WL_OK;
}

// Validation shared by the two eval entry points.
static int eval_prologue(wl_ctx *ctx, int handle, const wl_field *field, int ninst, int nF,
                         const double *host_F, int group, Ensemble *e, int *kprof,
                         FieldDev *fd) {
  if (!host_F) return fail(ctx, WL_ERR_INVALID, "NULL flux array");
  if (ninst < 1) return fail(ctx, WL_ERR_INVALID, "ninst must be >= 1");
  if (nF < 1 || nF > wl::kMaxF) return fail(ctx, WL_ERR_INVALID, "nF must be in [1, %d]", wl::kMaxF);
  int r = lookup(ctx, handle, e);
  if (r) return r;
  if (group < 1 || e->Nl % group != 0)
    return fail(ctx, WL_ERR_INVALID, "group %d must divide Nl = %d", group, e->Nl);
  if ((r = field_to_dev(ctx, field, kprof, fd))) return r;
  if (*kprof == wl::kSpline && (r = ensure_spline(ctx, field, fd))) return r;
  for (int j = 0; j < nF; ++j)
    if (!isfinite(host_F[j])) return fail(ctx, WL_ERR_INVALID, "F[%d] is not finite", j);
  return set_device(ctx);
}

// Sweep + reduction on the context stream; instances are already staged in
// ctx->inst as [cx | cy | rtT | tq].  Outputs are device pointers (may be
// NULL).  Returns after enqueueing.
static int run_eval(wl_ctx *ctx, const Ensemble &e, int kprof, const FieldDev &fd,
                    const float4 *bbox, const wl_field *field, int ninst, int nF,
                    const double *host_F, int group, double *dg, double *dm, double *ds) {
  const bool fermion = field->fermion != 0;
  const int nint = field->nint;
  const bool use_sweep = ninst >= 32;
  if (kprof == wl::kSpline && (!fd.sp_rho2 || !fd.sp_coef))
    return fail(ctx, WL_ERR_INVALID, "spline profile without its table");
  int n_chunks, cpg;
  if (use_sweep) {
    const int lc = plan_chunk(group);
    n_chunks = e.Nl / lc;
    if (n_chunks > 65535)
      return fail(ctx, WL_ERR_INVALID, "group %d too small for Nl = %d (grid limit)", group, e.Nl);
    cpg = group / lc;
  } else {
    n_chunks = e.Nl;
    cpg = group;
  }
  const size_t npart = (size_t)n_chunks * nF * 3 * ninst;
  if (ctx->partial.reserve(npart) != cudaSuccess) {
    cudaGetLastError();
    return fail(ctx, WL_ERR_NOMEM, "cannot allocate %zu partial sums", npart);
  }
  const float *di = ctx->inst.p;
  if (use_sweep) {
    wl::SweepArgs a;
    memset(&a, 0, sizeof(a));
    a.loops = e.dev;
    a.Nl = e.Nl;
    a.ppl = e.ppl;
    a.ninst = ninst;
    a.cx = di;
    a.cy = di + ninst;
    a.rtT = di + 2 * ninst;
    a.tqh = di + 3 * ninst;
    a.tql = di + 4 * ninst;
    a.nF = nF;
    fill_flux(a, field, nF, host_F);
    a.field = fd;
    a.chunk_loops = e.Nl / n_chunks;
    a.n_chunks = n_chunks;
    a.partial = ctx->partial.p;
    a.status = ctx->status.p;
    a.wait_tries = 1u << 22;
    a.bbox = bbox;
    if (kprof == wl::kLattice) {  // warps of similar image counts
      if (ctx->perm.reserve((size_t)ninst) != cudaSuccess) {
        cudaGetLastError();
        return fail(ctx, WL_ERR_NOMEM, "cannot allocate the instance order");
      }
      WL_CHECK(ctx, wl::launch_order_instances(a.cx, a.cy, a.rtT, ninst, 1.0f / fd.a,
                                               ctx->perm.p, ctx->stream));
      a.perm = ctx->perm.p;
    }
    WL_CHECK(ctx, wl::launch_sweep(kprof, fermion, nint, a, ctx->stream));
    ctx->last_kind = "instance-parallel";
  } else {
    wl::LoopArgs a;
    memset(&a, 0, sizeof(a));
    a.loops = e.dev;
    a.Nl = e.Nl;
    a.ppl = e.ppl;
    a.ninst = ninst;
    a.cx = di;
    a.cy = di + ninst;
    a.rtT = di + 2 * ninst;
    a.tqh = di + 3 * ninst;
    a.tql = di + 4 * ninst;
    a.nF = nF;
    fill_flux(a, field, nF, host_F);
    a.field = fd;
    a.partial = ctx->partial.p;
    a.bbox = bbox;
    WL_CHECK(ctx, wl::launch_loopwarp(kprof, fermion, nint, a, ctx->stream));
    ctx->last_kind = "loop-parallel";
  }
  WL_CHECK(ctx, wl::launch_group_reduce(ctx->partial.p, n_chunks, cpg, group, ninst, nF, dg, dm,
                                        ds, ctx->stream));
  return WL_OK;
}

int wl_eval(wl_ctx *ctx, int handle, const wl_field *field, int ninst, const double *host_cx,
            const double *host_cy, const double *host_T, int nF, const double *host_F,
            int group, double *out_group, double *out_mean, double *out_sem) {
  if (!ctx) return WL_ERR_INVALID;
  if (!host_cx || !host_cy || !host_T) return fail(ctx, WL_ERR_INVALID, "NULL instance arrays");
  Ensemble e;
  int kprof;
  FieldDev fd;
  int r = eval_prologue(ctx, handle, field, ninst, nF, host_F, group, &e, &kprof, &fd);
  if (r) return r;
  if ((r = upload_instances(ctx, ninst, host_cx, host_cy, host_T, e.ppl))) return r;
  WL_CHECK(ctx, cudaMemsetAsync(ctx->status.p, 0, sizeof(int), ctx->stream));
  const int ng = e.Nl / group;
  const size_t nout = (size_t)ninst * nF * (ng + 2);
  if (ctx->out.reserve(nout) != cudaSuccess) {
    cudaGetLastError();
    return fail(ctx, WL_ERR_NOMEM, "cannot allocate %zu outputs", nout);
  }
  double *dg = ctx->out.p, *dm = dg + (size_t)ninst * nF * ng, *ds = dm + (size_t)ninst * nF;
  const float4 *bb = nullptr;
  if (kprof == wl::kLattice && (r = ensure_bbox(ctx, handle, &bb))) return r;
  if ((r = run_eval(ctx, e, kprof, fd, bb, field, ninst, nF, host_F, group, dg, dm, ds)))
    return r;
  ctx->last_launches = 2;
  if (out_group)
    WL_CHECK(ctx, cudaMemcpyAsync(out_group, dg, sizeof(double) * ninst * nF * ng,
                                  cudaMemcpyDeviceToHost, ctx->stream));
  if (out_mean)
    WL_CHECK(ctx, cudaMemcpyAsync(out_mean, dm, sizeof(double) * ninst * nF,
                                  cudaMemcpyDeviceToHost, ctx->stream));
  if (out_sem)
    WL_CHECK(ctx, cudaMemcpyAsync(out_sem, ds, sizeof(double) * ninst * nF,
                                  cudaMemcpyDeviceToHost, ctx->stream));
  return check_status(ctx);
}

int wl_eval_device(wl_ctx *ctx, int handle, const wl_field *field, int ninst,
                   const double *dev_cx, const double *dev_cy, const double *dev_T, int nF,
                   const double *host_F, int group, double *dev_out_group, double *dev_out_mean,
                   double *dev_out_sem) {
  if (!ctx) return WL_ERR_INVALID;
  Ensemble e;
  int kprof;
  FieldDev fd;
  int r = eval_prologue(ctx, handle, field, ninst, nF, host_F, group, &e, &kprof, &fd);
  if (r) return r;
  const size_t nb = (size_t)ninst * sizeof(double);
  if ((r = check_device_range(ctx, dev_cx, nb, "dev_cx")) ||
      (r = check_device_range(ctx, dev_cy, nb, "dev_cy")) ||
      (r = check_device_range(ctx, dev_T, nb, "dev_T")))
    return r;
  const int ng = e.Nl / group;
  if (dev_out_group &&
      (r = check_device_range(ctx, dev_out_group, nb * nF * ng, "dev_out_group")))
    return r;
  if (dev_out_mean && (r = check_device_range(ctx, dev_out_mean, nb * nF, "dev_out_mean")))
    return r;
  if (dev_out_sem && (r = check_device_range(ctx, dev_out_sem, nb * nF, "dev_out_sem")))
    return r;
  WL_CHECK(ctx, ctx->inst.reserve((size_t)wl::kInstArrays * ninst));
  WL_CHECK(ctx, wl::launch_instance_setup(dev_cx, dev_cy, dev_T, ninst, e.ppl, ctx->inst.p,
                                          ctx->status.p, ctx->stream));
  const float4 *bb = nullptr;
  if (kprof == wl::kLattice && (r = ensure_bbox(ctx, handle, &bb))) return r;
  if ((r = run_eval(ctx, e, kprof, fd, bb, field, ninst, nF, host_F, group, dev_out_group,
                    dev_out_mean, dev_out_sem)))
    return r;
  ctx->last_launches = 3;
  return WL_OK;
}

int wl_spline_table(double lambda2, double tubedist, int n, float *rho2, float *coef4) {
  if (!(lambda2 > 0.0) || !(tubedist > 0.0) || n < 4 || n > (1 << 20) || !rho2 || !coef4)
    return WL_ERR_INVALID;
  return wl::spline_table(lambda2, tubedist, n, rho2, coef4) ? WL_ERR_INVALID : WL_OK;
}

int wl_selftest_wait(wl_ctx *ctx, int arrive, int max_tries, double *device_ms) {
  if (!ctx || max_tries < 1 || max_tries > (1 << 22))
    return fail(ctx, WL_ERR_INVALID, "max_tries must be in [1, 2^22]");
  int r = set_device(ctx);
  if (r) return r;
  cudaEvent_t e0, e1;
  WL_CHECK(ctx, cudaEventCreate(&e0));
  WL_CHECK(ctx, cudaEventCreate(&e1));
  WL_CHECK(ctx, cudaMemsetAsync(ctx->status.p, 0, sizeof(int), ctx->stream));
  WL_CHECK(ctx, cudaEventRecord(e0, ctx->stream));
  WL_CHECK(ctx, wl::launch_wait_selftest(ctx->status.p, (uint32_t)max_tries, arrive ? 1 : 0,
                                         ctx->stream));
  WL_CHECK(ctx, cudaEventRecord(e1, ctx->stream));
  WL_CHECK(ctx, cudaEventSynchronize(e1));
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (device_ms) *device_ms = ms;
  ctx->last_launches = 1;
  ctx->last_kind = "wait-selftest";
  return check_status(ctx);
}

int wl_peak_probe(wl_ctx *ctx, int kind, double *ops_per_s) {
  if (!ctx || !ops_per_s || kind < 0 || kind > 2) return fail(ctx, WL_ERR_INVALID, "bad probe");
  int r = set_device(ctx);
  if (r) return r;
  const int threads = 256, blocks = ctx->num_sms * 8;
  const int iters = kind == 1 ? 1024 : 4096;
  if (ctx->partial.reserve((size_t)blocks) != cudaSuccess) return fail(ctx, WL_ERR_NOMEM, "probe");
  float *sink = (float *)ctx->partial.p;
  cudaEvent_t e0, e1;
  WL_CHECK(ctx, cudaEventCreate(&e0));
  WL_CHECK(ctx, cudaEventCreate(&e1));
  WL_CHECK(ctx, wl::launch_peak_probe(kind, blocks, threads, iters, sink, ctx->stream));  // warm
  float best = 1e30f;
  for (int rep = 0; rep < 5; ++rep) {
    WL_CHECK(ctx, cudaEventRecord(e0, ctx->stream));
    WL_CHECK(ctx, wl::launch_peak_probe(kind, blocks, threads, iters, sink, ctx->stream));
    WL_CHECK(ctx, cudaEventRecord(e1, ctx->stream));
    WL_CHECK(ctx, cudaEventSynchronize(e1));
    float ms = 0.f;
    WL_CHECK(ctx, cudaEventElapsedTime(&ms, e0, e1));
    if (ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *ops_per_s = (double)blocks * threads * iters * (kind == 2 ? 16.0 : 8.0) / (best * 1e-3);
  return WL_OK;
}

// Quadrature weights in T for Simpson's rule on u = ln T (dT = T du):
// composite 1/3 rule, with the 3/8 rule on the last three intervals when the
// interval count is odd; the trapezoid rule for a single interval.
static void log_simpson_weights(const double *T, int n, double du, double *w) {
  for (int k = 0; k < n; ++k) w[k] = 0.0;
  const int m = n - 1;
  if (m == 1) {
    w[0] = w[1] = 0.5 * du;
  } else {
    const int m13 = (m % 2 == 0) ? m : m - 3;
    for (int k = 0; k < m13; k += 2) {
      w[k] += du / 3.0;
      w[k + 1] += 4.0 * du / 3.0;
      w[k + 2] += du / 3.0;
    }
    if (m13 < m) {
      const int k = m13;
      w[k] += 3.0 * du / 8.0;
      w[k + 1] += 9.0 * du / 8.0;
      w[k + 2] += 9.0 * du / 8.0;
      w[k + 3] += 3.0 * du / 8.0;
    }
  }
  for (int k = 0; k < n; ++k) w[k] *= T[k];
}

// <W> on the (rho, log T) grid, the FP64 proper-time integral per group and
// the jackknife on the device; results stay there (*ta), the caller copies
// what it needs and checks the status.
// Simpson weights (dT) of a log-spaced grid after checking it
static int log_grid_weights(wl_ctx *ctx, int nT, const double *host_T, std::vector<double> *w) {
  if (!host_T) return fail(ctx, WL_ERR_INVALID, "NULL T array");
  if (nT < 3) return fail(ctx, WL_ERR_INVALID, "need nT >= 3");
  const double du = log(host_T[1]) - log(host_T[0]);
  for (int k = 0; k < nT; ++k) {
    if (!(host_T[k] > 0.0) || !isfinite(host_T[k]))
      return fail(ctx, WL_ERR_INVALID, "T[%d] must be positive and finite", k);
    if (k > 0 && fabs((log(host_T[k]) - log(host_T[k - 1])) - du) > 1e-9 * fmax(1.0, fabs(du)))
      return fail(ctx, WL_ERR_INVALID, "T must be log-spaced (ascending, uniform in ln T)");
  }
  if (!(du > 0.0)) return fail(ctx, WL_ERR_INVALID, "T must be ascending");
  w->assign(nT, 0.0);
  log_simpson_weights(host_T, nT, du, w->data());
  return WL_OK;
}

// Nodes and weights (dT) of integrateT's rule (Tint.c:100-175): T = (1 - t)/t,
// n Simpson panels in t with the Jacobian 1/t^2.  The reference evaluates each
// panel's right end twice instead of its left end (Tint.c:127-130); summed
// over the panels that differs from Simpson's rule only by f(t = 1) - f(0),
// and both vanish (T = 0 and T = infinity), so one rule serves both modes.
static void tsub_nodes(int n, std::vector<double> *T, std::vector<double> *w) {
  const double h = 1.0 / n;
  T->clear();
  w->clear();
  for (int i = 0; i < n; ++i) {
    const double tm = h * (i + 0.5);
    T->push_back((1.0 - tm) / tm);
    w->push_back(4.0 * h / 6.0 / (tm * tm));
    if (i < n - 1) {  // t = 1 (T = 0) contributes 0
      const double tr = h * (i + 1);
      T->push_back((1.0 - tr) / tr);
      w->push_back(2.0 * h / 6.0 / (tr * tr));
    }
  }
}

static int tint_run(wl_ctx *ctx, int handle, const wl_field *field, int nrho,
                    const double *host_rho, int nT, const double *host_T, const double *host_w,
                    int nF, const double *host_F, int group, int nbins, bool want_igrand,
                    wl::TintArgs *ta_out) {
  if (!host_rho || !host_T || !host_w) return fail(ctx, WL_ERR_INVALID, "NULL rho or T array");
  if (nrho < 1 || nT < 1) return fail(ctx, WL_ERR_INVALID, "need nrho >= 1 and nT >= 1");
  Ensemble e;
  int kprof;
  FieldDev fd;
  int r = eval_prologue(ctx, handle, field, nrho * nT, nF, host_F, group, &e, &kprof, &fd);
  if (r) return r;
  const int ng = e.Nl / group;
  if (nbins < 2 || ng % nbins)
    return fail(ctx, WL_ERR_INVALID, "nbins = %d must be >= 2 and divide the %d groups", nbins, ng);
  const int ninst = nrho * nT;
  std::vector<double> cx((size_t)ninst), cy((size_t)ninst, 0.0), TT((size_t)ninst);
  for (int i = 0; i < nrho; ++i)
    for (int k = 0; k < nT; ++k) {
      cx[(size_t)i * nT + k] = host_rho[i];
      TT[(size_t)i * nT + k] = host_T[k];
    }
  if ((r = upload_instances(ctx, ninst, cx.data(), cy.data(), TT.data(), e.ppl))) return r;
  WL_CHECK(ctx, cudaMemsetAsync(ctx->status.p, 0, sizeof(int), ctx->stream));
  const size_t nout = (size_t)ninst * nF * (ng + 2);
  if (ctx->out.reserve(nout) != cudaSuccess) {
    cudaGetLastError();
    return fail(ctx, WL_ERR_NOMEM, "cannot allocate %zu outputs", nout);
  }
  double *dg = ctx->out.p;
  const float4 *bb = nullptr;
  if (kprof == wl::kLattice && (r = ensure_bbox(ctx, handle, &bb))) return r;
  if ((r = run_eval(ctx, e, kprof, fd, bb, field, ninst, nF, host_F, group, dg, nullptr,
                    nullptr)))
    return r;
  // aux: rho | T | w | F | Ig | leff | err | igrand
  const size_t n_ig = (size_t)nrho * nF * ng, n_le = (size_t)nrho * nF;
  const size_t n_igr = want_igrand ? (size_t)nrho * nF * nT * ng : 0;
  const size_t naux = (size_t)nrho + 2 * (size_t)nT + nF + n_ig + 2 * n_le + n_igr;
  if (ctx->aux.reserve(naux) != cudaSuccess) {
    cudaGetLastError();
    return fail(ctx, WL_ERR_NOMEM, "cannot allocate the proper-time buffers");
  }
  std::vector<double> h((size_t)nrho + 2 * (size_t)nT + nF);
  memcpy(h.data(), host_rho, sizeof(double) * nrho);
  memcpy(h.data() + nrho, host_T, sizeof(double) * nT);
  memcpy(h.data() + nrho + nT, host_w, sizeof(double) * nT);
  memcpy(h.data() + nrho + 2 * nT, host_F, sizeof(double) * nF);
  WL_CHECK(ctx, cudaMemcpyAsync(ctx->aux.p, h.data(), sizeof(double) * h.size(),
                                cudaMemcpyHostToDevice, ctx->stream));
  wl::TintArgs &ta = *ta_out;
  memset(&ta, 0, sizeof(ta));
  double *d = ctx->aux.p;
  ta.groups = dg;
  ta.rho = d;
  ta.T = d + nrho;
  ta.w = d + nrho + nT;
  ta.F = d + nrho + 2 * nT;
  ta.Ig = d + nrho + 2 * nT + nF;
  ta.leff = ta.Ig + n_ig;
  ta.err = ta.leff + n_le;
  ta.igrand = want_igrand ? ta.err + n_le : nullptr;
  ta.nrho = nrho;
  ta.nT = nT;
  ta.nF = nF;
  ta.ng = ng;
  ta.nbins = nbins;
  ta.profile = kprof;
  ta.fermion = field->fermion != 0;
  ta.l2 = field->lambda2;
  ta.a = field->tubedist;
  ta.lmin = field->lmin;
  ta.rimg2 = field->tubedist > 0.0 ? (field->rimage / field->tubedist) *
                                          (field->rimage / field->tubedist) : 0.0;
  ta.m2 = 1.0;         // Integrand.c:12
  ta.e = 0.30282212;   // Integrand.c:14
  WL_CHECK(ctx, wl::launch_tint(ta, ctx->stream));
  ctx->last_launches = 4;
  return WL_OK;
}

int wl_tint(wl_ctx *ctx, int handle, const wl_field *field, int nrho, const double *host_rho,
            int nT, const double *host_T, int nF, const double *host_F, int group, int nbins,
            double *out_leff, double *out_err, double *out_igrand) {
  if (!ctx) return WL_ERR_INVALID;
  if (!out_leff || !out_err) return fail(ctx, WL_ERR_INVALID, "NULL output array");
  std::vector<double> w;
  int r = log_grid_weights(ctx, nT, host_T, &w);
  if (r) return r;
  wl::TintArgs ta;
  if ((r = tint_run(ctx, handle, field, nrho, host_rho, nT, host_T, w.data(), nF, host_F, group,
                    nbins, out_igrand != nullptr, &ta)))
    return r;
  const size_t n_le = (size_t)nrho * nF, n_igr = (size_t)nrho * nF * nT * ta.ng;
  WL_CHECK(ctx, cudaMemcpyAsync(out_leff, ta.leff, sizeof(double) * n_le, cudaMemcpyDeviceToHost,
                                ctx->stream));
  WL_CHECK(ctx, cudaMemcpyAsync(out_err, ta.err, sizeof(double) * n_le, cudaMemcpyDeviceToHost,
                                ctx->stream));
  if (out_igrand)
    WL_CHECK(ctx, cudaMemcpyAsync(out_igrand, ta.igrand, sizeof(double) * n_igr,
                                  cudaMemcpyDeviceToHost, ctx->stream));
  return check_status(ctx);
}

// Classical action of the profile (EffAct.c:228-279), e = 0.30282212.
static double classical_action(int profile, double F, double l2, double a, double lmin) {
  const double e = 0.30282212, pi = M_PI;
  switch (profile) {
    case WL_PROFILE_STEP: return -2.0 * pi * F * F / (e * e * l2);
    case WL_PROFILE_SMOOTH: return -2.0 * pi * F * F / (3.0 * l2 * e * e);
    case WL_PROFILE_QUADRATIC: return -8.0 * pi * F * F / (3.0 * l2 * e * e);
    case WL_PROFILE_GAUSSIAN: return -pi * F * F / (l2 * e * e);
    case WL_PROFILE_PERIODIC: {  // EffAct.c:228-240 (the reference drops F here)
      const double l = sqrt(l2), q = 1.0 + exp(a / l);
      const double pca = 2.0 * a + 4.0 * a / (q * q * q) - l + 4.0 * l / q -
                         2.0 * (3.0 * a + 2.0 * l) / (q * q) + l * log(16.0) - 4.0 * l * log(q);
      return -pi * l / (24.0 * l2 * l2 * log(2.0) * log(2.0)) * pca;
    }
    case WL_PROFILE_SPLINE: return 1.0;  // EffAct.c:272-273 (no closed form there)
    case WL_PROFILE_FIXFLUX: {  // EffAct.c:242-253
      const double q2 = 0.0742478, q3 = 0.0187671, l = sqrt(l2);
      const double A = q3 * (a * a / (l2 * q2 * q2)), r = (l - lmin) / (a - lmin);
      const double ffca = 4.0 * A + r * ((9.0 / 4.0 * A - 9.0 / 2.0) * r - 6.0 * A + 12.0);
      return -pi * F * F / (e * e * a * a) * ffca;
    }
    default: return NAN;
  }
}

int wl_effective_action(wl_ctx *ctx, int handle, const wl_field *field, double F, int t_rule,
                        int nT, const double *host_T, int group, int nrho, double *out_action,
                        double *out_err, double *out_classical, double *out_groups) {
  if (!ctx) return WL_ERR_INVALID;
  if (!field || !out_action || !out_err) return fail(ctx, WL_ERR_INVALID, "NULL argument");
  std::vector<double> Tn, Tw;
  if (t_rule == WL_TRULE_LOG) {
    int r0 = log_grid_weights(ctx, nT, host_T, &Tw);
    if (r0) return r0;
    Tn.assign(host_T, host_T + nT);
  } else if (t_rule == WL_TRULE_SUBST) {
    if (nT < 1 || nT > 100000) return fail(ctx, WL_ERR_INVALID, "nT panels must be in [1, 1e5]");
    tsub_nodes(nT, &Tn, &Tw);
  } else {
    return fail(ctx, WL_ERR_INVALID, "unknown proper-time rule %d", t_rule);
  }
  if (nrho < 1 || nrho > 4096) return fail(ctx, WL_ERR_INVALID, "nrho must be in [1, 4096]");
  if (!isfinite(F)) return fail(ctx, WL_ERR_INVALID, "F is not finite");
  const int p = field->profile;
  if (p == WL_PROFILE_LATTICE)
    return fail(ctx, WL_ERR_INVALID, "the radial integral needs a cylindrically symmetric profile");
  const bool cell = (p == WL_PROFILE_PERIODIC || p == WL_PROFILE_FIXFLUX || p == WL_PROFILE_SPLINE);
  const bool ref = field->mode == WL_MODE_REFCOMPAT;
  // nodes and weights of the rho integral (of rho I(rho), Jacobian included)
  std::vector<double> rho, w;
  if (cell) {  // integrateRhotoa (EffAct.c:83-138): [0, a/2], n = 2 nrho intervals
    if (!(field->tubedist > 0.0)) return fail(ctx, WL_ERR_INVALID, "tubedist must be positive");
    const int n = 2 * nrho;
    const double h = field->tubedist / (2.0 * n);
    for (int k = 0; k <= n; ++k) {
      rho.push_back(h * k);
      double wk;
      if (ref) {
        // the reference adds f(0) + f(a/2) once, then every rho = h(i + 1),
        // i = 0..n-1, with weight 2 for even i and 4 for odd i -- f(a/2)
        // twice and the 2/4 weights on the opposite points of Simpson's rule
        wk = (k == 0) ? 1.0 : (((k - 1) % 2 == 0) ? 2.0 : 4.0);
        if (k == n) wk += 1.0;
      } else {
        wk = (k == 0 || k == n) ? 1.0 : (k % 2 ? 4.0 : 2.0);
      }
      w.push_back(wk * h / 3.0);
    }
  } else {  // integrateRho (EffAct.c:140-210): rho = (1 - t)/t, t in (0, 1], n panels
    const int n = nrho;
    const double h = 1.0 / n;
    // panel i: t_i = h i, t_{i+1/2}, t_{i+1}; the reference evaluates
    // f(t_{i+1}) in place of f(t_i) (rhort and rhortp1 are the same point)
    std::vector<double> wt(2 * n + 1, 0.0);  // weights on t_k = k h/2
    for (int i = 0; i < n; ++i) {
      if (ref) {
        wt[2 * i + 2] += 2.0 * h / 6.0;
      } else {
        wt[2 * i] += h / 6.0;
        wt[2 * i + 2] += h / 6.0;
      }
      wt[2 * i + 1] += 4.0 * h / 6.0;
    }
    for (int k = 1; k <= 2 * n; ++k) {  // t = 0 (rho = infinity) contributes 0
      const double t = 0.5 * h * k;
      rho.push_back((1.0 - t) / t);
      w.push_back(wt[k] / (t * t));  // d rho = dt / t^2
    }
  }
  const int nr = (int)rho.size();
  Ensemble e;
  int r = lookup(ctx, handle, &e);
  if (r) return r;
  if (group < 1 || e.Nl % group || e.Nl / group < 2)
    return fail(ctx, WL_ERR_INVALID, "group %d must divide Nl = %d into at least 2 groups", group,
                e.Nl);
  wl::TintArgs ta;
  if ((r = tint_run(ctx, handle, field, nr, rho.data(), (int)Tn.size(), Tn.data(), Tw.data(), 1,
                    &F, group, e.Nl / group, false, &ta)))
    return r;
  std::vector<double> Ig((size_t)nr * ta.ng);
  WL_CHECK(ctx, cudaMemcpyAsync(Ig.data(), ta.Ig, sizeof(double) * Ig.size(),
                                cudaMemcpyDeviceToHost, ctx->stream));
  if ((r = check_status(ctx))) return r;
  // Gamma_g = sum_k w_k rho_k I_g(rho_k), normalised as EAction (EffAct.c:289-294)
  const double norm = field->fermion ? 1.0 / (4.0 * M_PI) : -1.0 / (2.0 * M_PI);
  std::vector<double> gam(ta.ng, 0.0);
  for (int k = 0; k < nr; ++k)
    for (int g = 0; g < ta.ng; ++g) {
      double v = rho[k] * Ig[(size_t)k * ta.ng + g];
      if (isinf(v)) v = 0.0;  // EffAct.c:167-181
      gam[g] += w[k] * v;
    }
  double mean = 0.0;
  for (int g = 0; g < ta.ng; ++g) mean += (gam[g] *= norm);
  mean /= ta.ng;
  double ss = 0.0;
  for (int g = 0; g < ta.ng; ++g) ss += (gam[g] - mean) * (gam[g] - mean);
  *out_action = mean;
  *out_err = sqrt(ss / ((double)ta.ng * (ta.ng - 1.0)));
  if (out_classical)
    *out_classical = classical_action(p, F, field->lambda2, field->tubedist, field->lmin);
  if (out_groups) memcpy(out_groups, gam.data(), sizeof(double) * ta.ng);
  return WL_OK;
}

int wl_batch_eval(wl_ctx *ctx, int njobs, const wl_job *jobs, int flags) {
  if (!ctx) return WL_ERR_INVALID;
  if (njobs < 1 || !jobs) return fail(ctx, WL_ERR_INVALID, "need njobs >= 1 jobs");
  int r = set_device(ctx);
  if (r) return r;
  return batch_run(ctx, njobs, jobs, flags, ctx->tune_points, ctx->tune_ctas, true);
}

int wl_batch_autotune(wl_ctx *ctx, int njobs, const wl_job *jobs, int *points_per_tile,
                      int *ctas_per_sm) {
  if (!ctx) return WL_ERR_INVALID;
  if (njobs < 1 || !jobs) return fail(ctx, WL_ERR_INVALID, "need njobs >= 1 jobs");
  int r = set_device(ctx);
  if (r) return r;
  const int occ = wl::batch_max_ctas_per_sm();
  const int pts[5] = {4096, 8192, 16384, 32768, 65536};
  double best = 1e300;
  int bp = ctx->tune_points, bc = ctx->tune_ctas;
  for (int c = (occ > 1 ? occ - 1 : 1); c <= occ; ++c)
    for (int i = 0; i < 5; ++i) {
      // one untimed pass, then the timed one
      if ((r = batch_run(ctx, njobs, jobs, 0, pts[i], c, false))) return r;
      if ((r = batch_run(ctx, njobs, jobs, 0, pts[i], c, false))) return r;
      if (ctx->last_batch_ms < best) {
        best = ctx->last_batch_ms;
        bp = pts[i];
        bc = c;
      }
    }
  ctx->tune_points = bp;
  ctx->tune_ctas = bc;
  if (points_per_tile) *points_per_tile = bp;
  if (ctas_per_sm) *ctas_per_sm = bc;
  return WL_OK;
}

int wl_batch_stats(wl_ctx *ctx, double *device_ms, int *ntiles, int *grid, int *points_per_tile) {
  if (!ctx) return WL_ERR_INVALID;
  if (device_ms) *device_ms = ctx->last_batch_ms;
  if (ntiles) *ntiles = ctx->last_batch_tiles;
  if (grid) *grid = ctx->last_batch_grid;
  if (points_per_tile) *points_per_tile = ctx->tune_points;
  return WL_OK;
}

int wl_eval_plain(wl_ctx *ctx, int handle, const wl_field *field, int ninst, const double *host_cx,
                  const double *host_cy, const double *host_T, int nF, const double *host_F,
                  int group, double *out_group, double *out_mean, double *out_sem,
                  double *device_ms) {
  if (!ctx) return WL_ERR_INVALID;
  if (!host_cx || !host_cy || !host_T) return fail(ctx, WL_ERR_INVALID, "NULL instance arrays");
  Ensemble e;
  int kprof;
  FieldDev fd;
  int r = eval_prologue(ctx, handle, field, ninst, nF, host_F, group, &e, &kprof, &fd);
  if (r) return r;
  if (!wl::plain_supports(kprof))
    return fail(ctx, WL_ERR_INVALID, "the plain kernel covers the step, smooth, quadratic, "
                                     "gaussian and lattice profiles");
  if ((r = upload_instances(ctx, ninst, host_cx, host_cy, host_T, e.ppl))) return r;
  const int ng = e.Nl / group;
  const size_t npart = (size_t)e.Nl * nF * 3 * ninst;
  if (ctx->partial.reserve(npart) != cudaSuccess ||
      ctx->out.reserve((size_t)ninst * nF * (ng + 2)) != cudaSuccess) {
    cudaGetLastError();
    return fail(ctx, WL_ERR_NOMEM, "cannot allocate the plain-kernel buffers");
  }
  wl::LoopArgs a;
  memset(&a, 0, sizeof(a));
  a.loops = e.dev;
  a.Nl = e.Nl;
  a.ppl = e.ppl;
  a.ninst = ninst;
  a.cx = ctx->inst.p;
  a.cy = a.cx + ninst;
  a.rtT = a.cx + 2 * ninst;
  a.tqh = a.cx + 3 * ninst;
  a.tql = a.cx + 4 * ninst;
  a.nF = nF;
  fill_flux(a, field, nF, host_F);
  a.field = fd;
  a.partial = ctx->partial.p;
  if (kprof == wl::kLattice && (r = ensure_bbox(ctx, handle, &a.bbox))) return r;
  cudaEvent_t e0, e1;
  WL_CHECK(ctx, cudaEventCreate(&e0));
  WL_CHECK(ctx, cudaEventCreate(&e1));
  WL_CHECK(ctx, cudaEventRecord(e0, ctx->stream));
  for (int i = 0; i < ninst; ++i)
    WL_CHECK(ctx, wl::launch_plain(kprof, field->fermion != 0, field->nint, a, i, ctx->stream));
  WL_CHECK(ctx, cudaEventRecord(e1, ctx->stream));
  double *dg = ctx->out.p, *dm = dg + (size_t)ninst * nF * ng, *ds = dm + (size_t)ninst * nF;
  WL_CHECK(ctx, wl::launch_group_reduce(ctx->partial.p, e.Nl, group, group, ninst, nF, dg, dm, ds,
                                        ctx->stream));
  WL_CHECK(ctx, cudaEventSynchronize(e1));
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (device_ms) *device_ms = ms;
  ctx->last_launches = ninst + 1;
  ctx->last_kind = "plain-per-instance";
  if (out_group)
    WL_CHECK(ctx, cudaMemcpyAsync(out_group, dg, sizeof(double) * ninst * nF * ng,
                                  cudaMemcpyDeviceToHost, ctx->stream));
  if (out_mean)
    WL_CHECK(ctx, cudaMemcpyAsync(out_mean, dm, sizeof(double) * ninst * nF,
                                  cudaMemcpyDeviceToHost, ctx->stream));
  if (out_sem)
    WL_CHECK(ctx, cudaMemcpyAsync(out_sem, ds, sizeof(double) * ninst * nF,
                                  cudaMemcpyDeviceToHost, ctx->stream));
  return check_status(ctx);
}

int wl_ctx_stream(wl_ctx *ctx, void **stream) {
  if (!ctx || !stream) return WL_ERR_INVALID;
  *stream = (void *)ctx->stream;
  return WL_OK;
}

int wl_loops(wl_ctx *ctx, int handle, const wl_field *field, double cx, double cy, double T,
             double F, float *host_scal, float *host_ferm) {
  if (!ctx) return WL_ERR_INVALID;
  Ensemble e;
  int r = lookup(ctx, handle, &e);
  if (r) return r;
  int kprof;
  FieldDev fd;
  if ((r = field_to_dev(ctx, field, &kprof, &fd))) return r;
  if (kprof == wl::kSpline && (r = ensure_spline(ctx, field, &fd))) return r;
  if (!isfinite(F)) return fail(ctx, WL_ERR_INVALID, "F is not finite");
  if ((r = set_device(ctx))) return r;
  if ((r = upload_instances(ctx, 1, &cx, &cy, &T, e.ppl))) return r;
  if (ctx->partial.reserve((size_t)e.Nl * 3 + (size_t)e.Nl * 8) != cudaSuccess) {
    cudaGetLastError();
    return fail(ctx, WL_ERR_NOMEM, "cannot allocate per-loop outputs");
  }
  // partial: [Nl][3] doubles, then two float4 [Nl] arrays (16-byte aligned)
  float4 *ds = (float4 *)(ctx->partial.p + (((size_t)e.Nl * 3 + 1) & ~(size_t)1));
  float4 *df = ds + e.Nl;
  WL_CHECK(ctx, cudaMemsetAsync(df, 0, sizeof(float4) * e.Nl, ctx->stream));
  wl::LoopArgs a;
  memset(&a, 0, sizeof(a));
  a.loops = e.dev;
  a.Nl = e.Nl;
  a.ppl = e.ppl;
  a.ninst = 1;
  a.cx = ctx->inst.p;
  a.cy = ctx->inst.p + 1;
  a.rtT = ctx->inst.p + 2;
  a.tqh = ctx->inst.p + 3;
  a.tql = ctx->inst.p + 4;
  a.nF = 1;
  fill_flux(a, field, 1, &F);
  a.field = fd;
  a.partial = ctx->partial.p;
  if (kprof == wl::kLattice && (r = ensure_bbox(ctx, handle, &a.bbox))) return r;
  a.scal = ds;
  a.ferm = df;
  WL_CHECK(ctx, wl::launch_loopwarp(kprof, field->fermion != 0, field->nint, a, ctx->stream));
  ctx->last_launches = 1;
  ctx->last_kind = "loop-parallel";
  if (host_scal)
    WL_CHECK(ctx, cudaMemcpyAsync(host_scal, ds, sizeof(float4) * e.Nl, cudaMemcpyDeviceToHost,
                                  ctx->stream));
  if (host_ferm)
    WL_CHECK(ctx, cudaMemcpyAsync(host_ferm, df, sizeof(float4) * e.Nl, cudaMemcpyDeviceToHost,
                                  ctx->stream));
  WL_CHECK(ctx, cudaStreamSynchronize(ctx->stream));
  return WL_OK;
}

int wl_last_launches(wl_ctx *ctx, int *launches, const char **kind) {
  if (!ctx) return WL_ERR_INVALID;
  if (launches) *launches = ctx->last_launches;
  if (kind) *kind = ctx->last_kind;
  return WL_OK;
}

// ================================================================ legacy ==
// EV() keeps the reference's signature and side effects (intEV.cu:111-148):
// it computes every loop of the ensemble at (T, xcm), writes the per-loop
// phases into the caller's Wsscal_d / Wsferm_d and copies them to
// Wsscal_h / Wsferm_h, then returns the Richardson-combined mean over the
// 128 loops of WLlist.  The per-loop W factors of the last (T, xcm, field)
// stay cached on the device, so the ng calls of one Tfunc() evaluation
// (Integrand.c:249-305) cost one sweep and ng list reductions.  The cache
// also holds a 64-bit fingerprint of the ensemble's coordinates: a call for
// the first group, or for any non-consecutive list, recomputes when the
// loops were rewritten in place (the reference recomputes on every call,
// intEV.cu:123); wl_legacy_invalidate() drops the cache outright.
int wl_legacy_configure(int profile, double tubedist, double lmin, int nint, int mode) {
  LegacyState &L = legacy();
  std::lock_guard<std::mutex> lk(L.mu);
  wl_field f = L.field;
  const bool ff = profile == WL_PROFILE_FIXFLUX_FF;  // intEVff.cu's kernel
  f.profile = ff ? WL_PROFILE_FIXFLUX : profile;
  f.ff_variant = ff ? 1 : 0;
  f.tubedist = tubedist;
  f.lmin = lmin;
  f.nint = nint;
  f.mode = mode;
  f.lambda2 = 1.0;
  int kp;
  FieldDev d;
  int r = field_to_dev(nullptr, &f, &kp, &d);
  if (r) return r;
  L.field = f;
  L.config_gen++;
  L.valid = false;
  return WL_OK;
}

int wl_legacy_invalidate(void) {
  LegacyState &L = legacy();
  std::lock_guard<std::mutex> lk(L.mu);
  L.valid = false;
  return WL_OK;
}

int wl_legacy_query(int *profile, double *tubedist, double *lmin, int *nint, int *mode) {
  LegacyState &L = legacy();
  std::lock_guard<std::mutex> lk(L.mu);
  if (profile) *profile = L.field.profile;
  if (tubedist) *tubedist = L.field.tubedist;
  if (lmin) *lmin = L.field.lmin;
  if (nint) *nint = L.field.nint;
  if (mode) *mode = L.field.mode;
  return WL_OK;
}

static double legacy_fail(const char *msg) {
  fprintf(stderr, "EV(): %s\n", msg);
  return NAN;
}

double EV(double T, void *p, int *WLlist) {
  if (!p || !WLlist) return legacy_fail("NULL argument");
  const struct Wparams params = *(const struct Wparams *)p;
  LegacyState &L = legacy();
  std::lock_guard<std::mutex> lk(L.mu);
  const int groupsize = 128;  // intEV.cu:117
  if (!L.ctx) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) dev = 0;
    cudaGetLastError();
    if (wl_ctx_create(dev, &L.ctx) != WL_OK) return legacy_fail("no CUDA device");
  }
  wl_ctx *ctx = L.ctx;
  if (set_device(ctx)) return legacy_fail(ctx->err.c_str());
  if (check_shape(ctx, params.Nl, params.Nppl)) return legacy_fail(ctx->err.c_str());
  if (params.Nl < groupsize) return legacy_fail("Nl is smaller than one group of 128");
  for (int j = 0; j < groupsize; ++j)
    if (WLlist[j] < 0 || WLlist[j] >= params.Nl) return legacy_fail("WLlist index out of range");
  wl_field f = L.field;
  f.fermion = params.fermion == 1;
  f.lambda2 = params.l2;
  int kprof;
  FieldDev fd;
  if (field_to_dev(ctx, &f, &kprof, &fd)) return legacy_fail(ctx->err.c_str());
  if (kprof == wl::kSpline && ensure_spline(ctx, &f, &fd)) return legacy_fail(ctx->err.c_str());
  const size_t npts = (size_t)params.Nl * params.Nppl;
  bool hit = L.valid && L.T == T && L.F == params.F && L.l2 == params.l2 &&
             L.cx == params.xcm.x && L.cy == params.xcm.y &&
             L.loops == params.worldlines && L.Nl == params.Nl && L.ppl == params.Nppl &&
             L.fermion == f.fermion && L.gen == L.config_gen;
  // a group of consecutive loops g*128 .. g*128+127 (what Tfunc passes)
  bool consecutive = WLlist[0] % groupsize == 0;
  for (int j = 1; j < groupsize && consecutive; ++j) consecutive = WLlist[j] == WLlist[0] + j;
  if (hit && (!consecutive || WLlist[0] == 0)) {
    // the first group of a Tfunc sweep, or any other list: check that the
    // loops were not rewritten in place since the cached sweep read them
    unsigned long long fp = 0;
    cudaError_t ce = L.fpd.reserve(1);
    if (ce == cudaSuccess) ce = wl::launch_fingerprint(params.worldlines, npts, L.fpd.p, ctx->stream);
    if (ce == cudaSuccess)
      ce = cudaMemcpyAsync(&fp, L.fpd.p, sizeof(fp), cudaMemcpyDeviceToHost, ctx->stream);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(ctx->stream);
    if (ce != cudaSuccess) {
      L.valid = false;
      return legacy_fail(cudaGetErrorString(ce));
    }
    hit = fp == L.fp;
  }
  if (!hit) {
    L.valid = false;
    if (check_device_range(ctx, params.worldlines, npts * sizeof(float4), "worldlines") ||
        check_device_range(ctx, params.Wsscal_d, params.Nl * sizeof(float4), "Wsscal_d") ||
        (f.fermion &&
         check_device_range(ctx, params.Wsferm_d, params.Nl * sizeof(float4), "Wsferm_d")))
      return legacy_fail(ctx->err.c_str());
    const double cx = params.xcm.x, cy = params.xcm.y;
    if (upload_instances(ctx, 1, &cx, &cy, &T, params.Nppl)) return legacy_fail(ctx->err.c_str());
    if (L.w.reserve((size_t)params.Nl * 3) != cudaSuccess) return legacy_fail("out of memory");
    wl::LoopArgs a;
    memset(&a, 0, sizeof(a));
    a.loops = params.worldlines;
    a.Nl = params.Nl;
    a.ppl = params.Nppl;
    a.ninst = 1;
    a.cx = ctx->inst.p;
    a.cy = ctx->inst.p + 1;
    a.rtT = ctx->inst.p + 2;
    a.tqh = ctx->inst.p + 3;
    a.tql = ctx->inst.p + 4;
    a.nF = 1;
    fill_flux(a, &f, 1, &params.F);
    a.field = fd;
    a.partial = L.w.p;
    a.scal = params.Wsscal_d;
    a.ferm = f.fermion ? params.Wsferm_d : nullptr;
    unsigned long long fp = 0;
    cudaError_t ce = L.fpd.reserve(1);
    if (ce == cudaSuccess) ce = wl::launch_fingerprint(params.worldlines, npts, L.fpd.p, ctx->stream);
    if (ce == cudaSuccess)
      ce = cudaMemcpyAsync(&fp, L.fpd.p, sizeof(fp), cudaMemcpyDeviceToHost, ctx->stream);
    if (ce == cudaSuccess) ce = wl::launch_loopwarp(kprof, f.fermion != 0, f.nint, a, ctx->stream);
    if (ce == cudaSuccess && params.Wsscal_h)
      ce = cudaMemcpyAsync(params.Wsscal_h, params.Wsscal_d, params.Nl * sizeof(float4),
                           cudaMemcpyDeviceToHost, ctx->stream);
    if (ce == cudaSuccess && f.fermion && params.Wsferm_h)
      ce = cudaMemcpyAsync(params.Wsferm_h, params.Wsferm_d, params.Nl * sizeof(float4),
                           cudaMemcpyDeviceToHost, ctx->stream);
    const int ngrp = params.Nl / groupsize;
    L.gev.assign((size_t)ngrp, NAN);
    if (ce == cudaSuccess && L.gres.reserve((size_t)ngrp) != cudaSuccess) {
      cudaGetLastError();
      return legacy_fail("out of memory");
    }
    if (ce == cudaSuccess)
      ce = wl::launch_group_list_means(L.w.p, groupsize, ngrp, L.gres.p, ctx->stream);
    if (ce == cudaSuccess)
      ce = cudaMemcpyAsync(L.gev.data(), L.gres.p, sizeof(double) * ngrp,
                           cudaMemcpyDeviceToHost, ctx->stream);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(ctx->stream);
    if (ce != cudaSuccess) return legacy_fail(cudaGetErrorString(ce));
    L.T = T;
    L.F = params.F;
    L.l2 = params.l2;
    L.cx = params.xcm.x;
    L.cy = params.xcm.y;
    L.loops = params.worldlines;
    L.Nl = params.Nl;
    L.ppl = params.Nppl;
    L.fermion = f.fermion;
    L.gen = L.config_gen;
    L.fp = fp;
    L.valid = true;
  }
  // a group of consecutive loops: its mean is already on the host
  if (consecutive && (size_t)(WLlist[0] / groupsize) < L.gev.size())
    return L.gev[(size_t)(WLlist[0] / groupsize)];
  if (ctx->list.reserve(groupsize) != cudaSuccess || L.res.reserve(1) != cudaSuccess)
    return legacy_fail("out of memory");
  double ev = NAN;
  cudaError_t ce = cudaMemcpyAsync(ctx->list.p, WLlist, sizeof(int) * groupsize,
                                   cudaMemcpyHostToDevice, ctx->stream);
  if (ce == cudaSuccess) ce = wl::launch_list_mean(L.w.p, ctx->list.p, groupsize, L.res.p, ctx->stream);
  if (ce == cudaSuccess)
    ce = cudaMemcpyAsync(&ev, L.res.p, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(ctx->stream);
  if (ce != cudaSuccess) {
    L.valid = false;
    return legacy_fail(cudaGetErrorString(ce));
  }
  return ev;
}

}  // extern "C"
#pragma GCC visibility pop

static void log_simpson_weights(const double *T, int n, double du, double *w);

// Helpers shared with the allocation-free entry point (wl_noalloc.cu): the
// same field validation, flux constants and loop partition as wl_eval_device.
namespace wl {
int shared_field_to_dev(const wl_field *f, int *kprofile, FieldDev *d) {
  // the lattice needs per-loop bounding boxes and the spline profile its
  // table, both of which the library would allocate
  if (f && (f->profile == WL_PROFILE_LATTICE || f->profile == WL_PROFILE_SPLINE))
    return WL_ERR_INVALID;
  return field_to_dev(nullptr, f, kprofile, d);
}
void shared_fill_flux(SweepArgs &a, const wl_field *f, int nF, const double *F) {
  fill_flux(a, f, nF, F);
}
void shared_fill_flux(LoopArgs &a, const wl_field *f, int nF, const double *F) {
  fill_flux(a, f, nF, F);
}
int shared_plan_chunk(int group) { return plan_chunk(group); }

// for the request server (wl_server.cpp)
int rt_field(const wl_field *f, int *kprofile, FieldDev *d, std::string *err) {
  wl_ctx tmp;
  const int r = field_to_dev(&tmp, f, kprofile, d);
  if (r && err) *err = tmp.err;
  return r;
}
int rt_loops_per_tile(int points, int ppl, int group) {
  return batch_loops_per_tile(points, ppl, group);
}
void rt_log_simpson_weights(const double *T, int n, double du, double *w) {
  log_simpson_weights(T, n, du, w);
}
}  // namespace wl
