// wl_server.cpp -- continuously batched request server (include/wlgpu.h).
//
// One worker thread owns the device side.  Requests wait in arrival order
// until their HBM footprint fits the budget and a job slot is free; loop
// ensembles, keyed by (seed, Nl, ppl), are generated on the device at first
// use and stay resident until the budget needs their memory back (least
// recently used idle ensemble first).  Admitted requests are cut into tiles
// (job slot, instance tile of 128, chunk of loops) -- the tiles of the
// persistent batch kernel -- and every launch takes about one quantum of
// device time worth of tiles from all admitted requests, oldest request
// first.  Two launches are in flight at once on two streams, so a request
// that arrives while one launch runs joins the next one and its work overlaps
// the tail of the running one.  When a request's last tile has been handed
// out, its group reduction (and, for an effective-action-density request, the
// proper-time integral) follows that launch on the same stream, after the
// other stream's latest launch, and its results come back through pinned
// host memory.  A tile's partial sums do not depend on which launch or which
// neighbours it ran with, so every result equals the request evaluated alone.
#include <cuda_runtime.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/wlgpu.h"
#include "wl_internal.h"
#include "wl_spline.h"

namespace wl {
int rt_field(const wl_field *f, int *kprofile, FieldDev *d, std::string *err);
int rt_loops_per_tile(int points, int ppl, int group);
void rt_log_simpson_weights(const double *T, int n, double du, double *w);
void shared_fill_flux(SweepArgs &a, const wl_field *f, int nF, const double *F);
}  // namespace wl

namespace {

using Clock = std::chrono::steady_clock;

constexpr int kMaxQuantumTiles = 1 << 16;  // tile descriptors per launch
constexpr size_t kAlign = 256;

size_t up(size_t x) { return (x + kAlign - 1) & ~(kAlign - 1); }

// Device time of one tile-point relative to the smooth profile at 4
// intervals (the processor-sharing split and the rate estimate only): the
// node count times the profile's cost relative to the smooth one at the same
// interval count, measured on the GB300 through wl_eval (512 instances on
// Nl 1024 x ppl 1024, scalar QED) at 4, 8 and 50 intervals and interpolated
// linearly in nint between them (flat outside).
double profile_weight(int kprof, int fermion, int nint) {
  double r[3] = {1.0, 1.0, 1.0};  // at 4, 8, 50 intervals
  switch (kprof) {
    case wl::kGaussian: r[0] = 1.6; r[1] = 1.94; r[2] = 3.95; break;
    case wl::kLattice: r[0] = r[1] = r[2] = 8.0; break;
    case wl::kPeriodic: r[0] = r[1] = 30.4; r[2] = 70.8; break;
    case wl::kSpline: r[0] = r[1] = 12.6; r[2] = 29.2; break;
    case wl::kFixflux:
    case wl::kFixfluxFF: r[0] = r[1] = 180.0; r[2] = 400.0; break;
    default: break;
  }
  double w;
  if (nint <= 4) w = r[0];
  else if (nint <= 8) w = r[0] + (r[1] - r[0]) * (nint - 4) / 4.0;
  else if (nint <= 50) w = r[1] + (r[2] - r[1]) * (nint - 8) / 42.0;
  else w = r[2];
  return (fermion ? w * 1.15 : w) * (nint + 1) / 5.0;
}

struct SrvEnsemble {
  uint64_t seed = 0;
  int Nl = 0, ppl = 0;
  float4 *dev = nullptr, *bbox = nullptr;
  size_t bytes = 0;  // loops + boxes
  int users = 0;     // admitted requests on it
  uint64_t last_use = 0;
};

struct Req {
  long long ticket = 0;
  wl_request q;  // the user's request; input pointers are repointed to the copies
  std::vector<double> cx, cy, T, rho, Tg;
  int kprof = 0;
  wl::FieldDev fd;
  Clock::time_point t_submit;
  int status = WL_OK;
  bool done = false;
  // sizes
  int ninst = 0, lc = 0, n_chunks = 0, ng = 0, tiles_x = 0;
  long long ntiles = 0, next_tile = 0;
  size_t dbytes = 0, pbytes = 0;  // device / pinned footprint
  size_t o_rj = 0, o_inst = 0, o_perm = 0, o_part = 0, o_out = 0, o_aux = 0;  // device offsets
  size_t p_args = 0, p_rj = 0, p_inst = 0, p_aux = 0, n_aux_in = 0, p_out = 0, n_out = 0;
  double tile_work = 0.0, segments = 0.0;
  // admitted state
  SrvEnsemble *ens = nullptr;
  int slot = -1;
  char *dmem = nullptr, *pin = nullptr;
  wl::SweepArgs args;
  wl::ReduceJob rj;
  wl::TintArgs ta;
  cudaEvent_t done_ev = nullptr;
  bool finishing = false;
};

}  // namespace

struct wl_server {
  wl_server_config cfg;
  int num_sms = 0, grid_max = 0;
  std::thread worker;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  bool stopping = false, failed = false;
  std::string err;
  long long next_ticket = 1;
  std::deque<Req *> incoming;                       // submitted, not seen by the worker
  std::map<long long, std::unique_ptr<Req>> owned;  // every request not yet waited for
  // statistics (under mu)
  long long n_sub = 0, n_done = 0, n_rej = 0, n_fail = 0, n_launch = 0;
  std::vector<double> lat_ms;
  Clock::time_point t_first, t_last;
  double seg_done = 0.0, pub_in_use = 0.0;
  int pub_resident = 0;
  // worker state
  std::deque<Req *> pending;  // waiting for admission, in arrival order
  std::vector<Req *> running;  // admitted, in admission order
  std::vector<std::unique_ptr<SrvEnsemble>> ens;
  double in_use = 0.0;
  std::vector<int> free_slots;
  wl::SweepArgs *d_slots = nullptr;
  cudaStream_t cs = nullptr;  // allocations, generation, admission copies
  cudaStream_t st[2] = {nullptr, nullptr};
  cudaEvent_t adm_ev = nullptr;
  long long adm_seq = 0, waited_seq[2] = {0, 0};
  cudaEvent_t ev_start[2] = {nullptr, nullptr}, ev_stop[2] = {nullptr, nullptr};
  // device clock of the statistics: recorded before the first launch after a
  // reset; each retired launch adds its [start, stop] in ms from it
  cudaEvent_t ev_base = nullptr;
  bool base_recorded = false, base_reset = false;  // base_reset: under mu
  std::vector<std::pair<double, double>> spans;    // under mu
  bool busy[2] = {false, false};
  double busy_work[2] = {0.0, 0.0};
  int busy_tiles[2] = {0, 0};
  wl::BatchTile *d_tiles[2] = {nullptr, nullptr}, *h_tiles[2] = {nullptr, nullptr};
  int *d_counter = nullptr;  // [2] queue counters
  int next_stream = 0;
  double rate = 0.0;  // weighted tile work per ms of device time
  uint64_t use_clock = 0;
  std::map<size_t, std::vector<char *>> pin_cache;
  // spline profile tables by (lambda^2, tube spacing), kept until destroy
  std::map<std::pair<double, double>, std::pair<float *, float4 *>> splines;
};

namespace {

int set_err(wl_server *s, int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  std::lock_guard<std::mutex> lk(s->mu);
  s->err = buf;
  return code;
}

// ---------------------------------------------------------- validation --
int check_request(wl_server *s, const wl_request *q, Req *R) {
  if (!q) return set_err(s, WL_ERR_INVALID, "request is NULL");
  if (q->Nl < 1 || q->ppl < 4 || q->ppl % 4 || (double)q->Nl * q->ppl > 2147483647.0)
    return set_err(s, WL_ERR_INVALID, "need Nl >= 1, ppl a positive multiple of 4, Nl*ppl < 2^31");
  if (q->group < 1 || q->Nl % q->group)
    return set_err(s, WL_ERR_INVALID, "group %d must divide Nl = %d", q->group, q->Nl);
  if (q->nF < 1 || q->nF > wl::kMaxF)
    return set_err(s, WL_ERR_INVALID, "nF must be in [1, %d]", wl::kMaxF);
  for (int j = 0; j < q->nF; ++j)
    if (!isfinite(q->F[j])) return set_err(s, WL_ERR_INVALID, "F[%d] is not finite", j);
  std::string e;
  if (wl::rt_field(&q->field, &R->kprof, &R->fd, &e))
    return set_err(s, WL_ERR_INVALID, "%s", e.c_str());
  if (!wl::batch_supports(R->kprof, q->field.nint))
    return set_err(s, WL_ERR_INVALID, "profile %d is not served", q->field.profile);
  const int ng = q->Nl / q->group;
  if (q->kind == WL_REQ_W) {
    if (q->ninst < 1 || !q->cx || !q->cy || !q->T)
      return set_err(s, WL_ERR_INVALID, "need ninst >= 1 and instance arrays");
    if (!q->out_group && !q->out_mean && !q->out_sem)
      return set_err(s, WL_ERR_INVALID, "no output array");
    for (int i = 0; i < q->ninst; ++i)
      if (!isfinite(q->cx[i]) || !isfinite(q->cy[i]) || !(q->T[i] > 0.0) || !isfinite(q->T[i]))
        return set_err(s, WL_ERR_INVALID, "instance %d: need finite centre and T > 0", i);
    R->cx.assign(q->cx, q->cx + q->ninst);
    R->cy.assign(q->cy, q->cy + q->ninst);
    R->T.assign(q->T, q->T + q->ninst);
    R->ninst = q->ninst;
  } else if (q->kind == WL_REQ_LEFF) {
    if (q->nrho < 1 || q->nT < 3 || !q->rho || !q->Tgrid || !q->out_leff || !q->out_err)
      return set_err(s, WL_ERR_INVALID, "need nrho >= 1, nT >= 3, rho/T grids and outputs");
    if ((double)q->nrho * q->nT > 1e8) return set_err(s, WL_ERR_INVALID, "grid too large");
    const double du = log(q->Tgrid[1]) - log(q->Tgrid[0]);
    for (int k = 0; k < q->nT; ++k) {
      if (!(q->Tgrid[k] > 0.0) || !isfinite(q->Tgrid[k]))
        return set_err(s, WL_ERR_INVALID, "T[%d] must be positive and finite", k);
      if (k > 0 &&
          fabs((log(q->Tgrid[k]) - log(q->Tgrid[k - 1])) - du) > 1e-9 * fmax(1.0, fabs(du)))
        return set_err(s, WL_ERR_INVALID, "T must be log-spaced (ascending, uniform in ln T)");
    }
    if (!(du > 0.0)) return set_err(s, WL_ERR_INVALID, "T must be ascending");
    for (int r = 0; r < q->nrho; ++r)
      if (!isfinite(q->rho[r])) return set_err(s, WL_ERR_INVALID, "rho[%d] is not finite", r);
    if (q->nbins < 2 || ng % q->nbins)
      return set_err(s, WL_ERR_INVALID, "nbins = %d must be >= 2 and divide the %d groups",
                     q->nbins, ng);
    R->rho.assign(q->rho, q->rho + q->nrho);
    R->Tg.assign(q->Tgrid, q->Tgrid + q->nT);
    R->ninst = q->nrho * q->nT;  // instance r * nT + k: (rho_r, 0, T_k), as wl_tint
    R->cx.resize(R->ninst);
    R->cy.assign(R->ninst, 0.0);
    R->T.resize(R->ninst);
    for (int r = 0; r < q->nrho; ++r)
      for (int k = 0; k < q->nT; ++k) {
        R->cx[(size_t)r * q->nT + k] = q->rho[r];
        R->T[(size_t)r * q->nT + k] = q->Tgrid[k];
      }
  } else {
    return set_err(s, WL_ERR_INVALID, "unknown request kind %d", q->kind);
  }
  R->q = *q;
  R->q.cx = R->q.cy = R->q.T = R->q.rho = R->q.Tgrid = nullptr;  // copies above
  // sizes and footprint
  const int n = R->ninst, nF = q->nF;
  R->ng = ng;
  R->lc = wl::rt_loops_per_tile(s->cfg.points_per_tile, q->ppl, q->group);
  R->n_chunks = q->Nl / R->lc;
  const int per_tile = wl::sweep_tile_instances(R->kprof, q->field.nint);
  R->tiles_x = (n + per_tile - 1) / per_tile;
  R->ntiles = (long long)R->n_chunks * R->tiles_x;
  R->tile_work = (double)R->lc * q->ppl * per_tile *
                 profile_weight(R->kprof, q->field.fermion != 0, q->field.nint);
  R->segments = (double)n * q->Nl * q->ppl;
  const size_t n_part = (size_t)R->n_chunks * nF * 3 * n;
  const size_t n_out = (size_t)n * nF * (ng + 2);
  size_t n_aux = 0, n_aux_in = 0;
  if (q->kind == WL_REQ_LEFF) {
    n_aux_in = (size_t)q->nrho + 2 * (size_t)q->nT + nF;  // rho | T | w | F
    n_aux = n_aux_in + (size_t)q->nrho * nF * ng + 2 * (size_t)q->nrho * nF;  // Ig | leff | err
  }
  R->o_rj = up(sizeof(int));
  R->o_inst = R->o_rj + up(sizeof(wl::ReduceJob));
  R->o_perm = R->o_inst + up(sizeof(float) * wl::kInstArrays * n);
  const size_t n_perm = R->kprof == wl::kLattice ? (size_t)n : 0;
  R->o_part = R->o_perm + up(sizeof(int) * n_perm);
  R->o_out = R->o_part + up(sizeof(double) * n_part);
  R->o_aux = R->o_out + up(sizeof(double) * n_out);
  R->dbytes = R->o_aux + up(sizeof(double) * n_aux);
  // pinned staging: inputs (slot args | reduce job | instances | aux inputs), outputs
  R->p_args = 0;
  R->p_rj = up(sizeof(wl::SweepArgs));
  R->p_inst = R->p_rj + up(sizeof(wl::ReduceJob));
  R->p_aux = R->p_inst + up(sizeof(float) * wl::kInstArrays * n);
  R->n_aux_in = n_aux_in;
  R->p_out = R->p_aux + up(sizeof(double) * n_aux_in);
  if (q->kind == WL_REQ_LEFF)
    R->n_out = 2 * (size_t)q->nrho * nF;
  else
    R->n_out = q->out_group ? n_out : 2 * (size_t)n * nF;
  R->pbytes = R->p_out + up(16 + sizeof(double) * R->n_out);  // status word, then values
  return WL_OK;
}

// ------------------------------------------------------- worker helpers --
struct WorkerError {
  std::string msg;
};

void ck(cudaError_t e, const char *what) {
  if (e != cudaSuccess) throw WorkerError{std::string(what) + ": " + cudaGetErrorString(e)};
}

char *pin_get(wl_server *s, size_t bytes) {
  size_t cls = 4096;
  while (cls < bytes) cls <<= 1;
  auto &v = s->pin_cache[cls];
  if (!v.empty()) {
    char *p = v.back();
    v.pop_back();
    return p;
  }
  char *p = nullptr;
  if (cudaHostAlloc((void **)&p, cls, cudaHostAllocDefault) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return p;
}

void pin_put(wl_server *s, char *p, size_t bytes) {
  size_t cls = 4096;
  while (cls < bytes) cls <<= 1;
  s->pin_cache[cls].push_back(p);
}

// completes a request (worker side, before any device work or after its done
// event): publishes the status and statistics
void finish(wl_server *s, Req *R, int status) {
  const auto now = Clock::now();
  std::lock_guard<std::mutex> lk(s->mu);
  R->status = status;
  R->done = true;
  if (status == WL_OK) {
    ++s->n_done;
    s->lat_ms.push_back(std::chrono::duration<double, std::milli>(now - R->t_submit).count());
    s->seg_done += R->segments;
    s->t_last = now;
  } else if (status == WL_ERR_ADMISSION) {
    ++s->n_rej;
  } else {
    ++s->n_fail;
  }
  s->cv_done.notify_all();
}

SrvEnsemble *find_ens(wl_server *s, const wl_request &q) {
  for (auto &e : s->ens)
    if (e->seed == q.seed && e->Nl == q.Nl && e->ppl == q.ppl) return e.get();
  return nullptr;
}

size_t ens_need(const SrvEnsemble *e, const Req *R) {
  const size_t loops = (size_t)R->q.Nl * R->q.ppl * sizeof(float4);
  const size_t boxes = R->kprof == wl::kLattice ? (size_t)R->q.Nl * sizeof(float4) : 0;
  if (!e) return loops + boxes;
  return (boxes && !e->bbox) ? boxes : 0;
}

void evict(wl_server *s, SrvEnsemble *keep, double want) {
  while (s->in_use + want > s->cfg.hbm_budget_bytes) {
    SrvEnsemble *lru = nullptr;
    for (auto &e : s->ens)
      if (e.get() != keep && e->users == 0 && (!lru || e->last_use < lru->last_use))
        lru = e.get();
    if (!lru) return;
    ck(cudaFreeAsync(lru->dev, s->cs), "ensemble free");
    if (lru->bbox) ck(cudaFreeAsync(lru->bbox, s->cs), "bbox free");
    s->in_use -= (double)lru->bytes;
    s->ens.erase(std::find_if(s->ens.begin(), s->ens.end(),
                              [&](const std::unique_ptr<SrvEnsemble> &p) { return p.get() == lru; }));
  }
}

// Admits requests in arrival order; returns true if any was admitted or
// rejected.  Stops at the first request that must wait.
bool admit(wl_server *s) {
  bool progress = false, copied = false;
  while (!s->pending.empty()) {
    Req *R = s->pending.front();
    SrvEnsemble *E = find_ens(s, R->q);
    const size_t eneed = ens_need(E, R);
    const double need = (double)R->dbytes + (double)eneed;
    if (need > s->cfg.hbm_budget_bytes) {  // can never fit
      s->pending.pop_front();
      set_err(s, WL_ERR_ADMISSION, "request %lld needs %.0f bytes, budget %.0f", R->ticket, need,
              s->cfg.hbm_budget_bytes);
      finish(s, R, WL_ERR_ADMISSION);
      progress = true;
      continue;
    }
    if (s->free_slots.empty()) break;
    if (s->in_use + need > s->cfg.hbm_budget_bytes) evict(s, E, need);
    if (s->in_use + need > s->cfg.hbm_budget_bytes) break;  // wait for memory
    s->pending.pop_front();
    progress = true;
    char *pin = pin_get(s, R->pbytes);
    char *dmem = nullptr;
    if (!pin || cudaMallocAsync((void **)&dmem, R->dbytes, s->cs) != cudaSuccess) {
      cudaGetLastError();
      if (pin) pin_put(s, pin, R->pbytes);
      set_err(s, WL_ERR_NOMEM, "request %lld: cannot allocate its buffers", R->ticket);
      finish(s, R, WL_ERR_NOMEM);
      continue;
    }
    // the ensemble: generated once, then resident
    if (!E) {
      auto ne = std::make_unique<SrvEnsemble>();
      ne->seed = R->q.seed;
      ne->Nl = R->q.Nl;
      ne->ppl = R->q.ppl;
      ne->bytes = (size_t)R->q.Nl * R->q.ppl * sizeof(float4);
      if (cudaMallocAsync((void **)&ne->dev, ne->bytes, s->cs) != cudaSuccess) {
        cudaGetLastError();
        ck(cudaFreeAsync(dmem, s->cs), "free");
        pin_put(s, pin, R->pbytes);
        set_err(s, WL_ERR_NOMEM, "request %lld: cannot allocate its ensemble", R->ticket);
        finish(s, R, WL_ERR_NOMEM);
        continue;
      }
      ck(wl::launch_vloops(ne->seed, 0, ne->Nl, ne->ppl, ne->dev, s->cs), "loop generator");
      s->in_use += (double)ne->bytes;
      E = ne.get();
      s->ens.push_back(std::move(ne));
    }
    if (R->kprof == wl::kSpline) {  // the profile's table, once per (lambda^2, a)
      const auto key = std::make_pair(R->q.field.lambda2, R->q.field.tubedist);
      auto it = s->splines.find(key);
      if (it == s->splines.end()) {
        const int nk = wl::kSplineKnots;
        std::vector<float> rho2(nk), coef(4 * (size_t)nk);
        float *dr = nullptr;
        float4 *dc = nullptr;
        // the field was validated at submit, so the table is well defined
        wl::spline_table(R->q.field.lambda2, R->q.field.tubedist, nk, rho2.data(), coef.data());
        ck(cudaMallocAsync((void **)&dr, sizeof(float) * nk, s->cs), "spline table");
        ck(cudaMallocAsync((void **)&dc, sizeof(float4) * nk, s->cs), "spline table");
        // pageable sources: staged before the calls return
        ck(cudaMemcpyAsync(dr, rho2.data(), sizeof(float) * nk, cudaMemcpyHostToDevice, s->cs),
           "spline upload");
        ck(cudaMemcpyAsync(dc, coef.data(), sizeof(float4) * nk, cudaMemcpyHostToDevice, s->cs),
           "spline upload");
        it = s->splines.emplace(key, std::make_pair(dr, dc)).first;
      }
      R->fd.sp_rho2 = it->second.first;
      R->fd.sp_coef = it->second.second;
    }
    if (R->kprof == wl::kLattice && !E->bbox) {
      const size_t bb = (size_t)E->Nl * sizeof(float4);
      ck(cudaMallocAsync((void **)&E->bbox, bb, s->cs), "bbox allocation");
      ck(wl::launch_loop_bbox(E->dev, E->Nl, E->ppl, E->bbox, s->cs), "loop bounding boxes");
      E->bytes += bb;
      s->in_use += (double)bb;
    }
    E->users++;
    E->last_use = ++s->use_clock;
    R->ens = E;
    R->dmem = dmem;
    R->pin = pin;
    R->slot = s->free_slots.back();
    s->free_slots.pop_back();
    s->in_use += (double)R->dbytes;
    // descriptors and inputs into the pinned staging
    const int n = R->ninst, nF = R->q.nF;
    float *hi = (float *)(pin + R->p_inst);
    for (int k = 0; k < n; ++k) {  // as the batch path stages them
      const float rtT = (float)sqrt(R->T[k]);
      const double tq = 4.0 * ((double)rtT * (double)rtT) / (double)R->q.ppl;
      hi[k] = (float)R->cx[k];
      hi[n + k] = (float)R->cy[k];
      hi[2 * n + k] = rtT;
      hi[3 * n + k] = (float)tq;
      hi[4 * n + k] = (float)(tq - (double)(float)tq);
    }
    int *d_status = (int *)dmem;
    const float *d_inst = (const float *)(dmem + R->o_inst);
    double *d_part = (double *)(dmem + R->o_part), *d_out = (double *)(dmem + R->o_out);
    wl::SweepArgs &a = R->args;
    memset(&a, 0, sizeof(a));
    a.loops = E->dev;
    a.Nl = E->Nl;
    a.ppl = E->ppl;
    a.ninst = n;
    a.cx = d_inst;
    a.cy = d_inst + n;
    a.rtT = d_inst + 2 * n;
    a.tqh = d_inst + 3 * n;
    a.tql = d_inst + 4 * n;
    a.nF = nF;
    wl::shared_fill_flux(a, &R->q.field, nF, R->q.F);
    a.field = R->fd;
    a.chunk_loops = R->lc;
    a.n_chunks = R->n_chunks;
    a.partial = d_part;
    a.status = d_status;
    a.wait_tries = 1u << 22;
    a.kprof = R->kprof;
    a.fermion = R->q.field.fermion != 0;
    a.nint = R->q.field.nint;
    a.bbox = E->bbox;
    if (R->kprof == wl::kLattice) a.perm = (const int *)(dmem + R->o_perm);
    wl::ReduceJob &rj = R->rj;
    memset(&rj, 0, sizeof(rj));
    rj.partial = d_part;
    rj.out_group = d_out;
    rj.out_mean = d_out + (size_t)n * nF * R->ng;
    rj.out_sem = rj.out_mean + (size_t)n * nF;
    rj.n_chunks = R->n_chunks;
    rj.cpg = R->q.group / R->lc;
    rj.lpg = R->q.group;
    rj.ninst = n;
    rj.nF = nF;
    rj.first = 0;
    memcpy(pin + R->p_args, &a, sizeof(a));
    memcpy(pin + R->p_rj, &rj, sizeof(rj));
    if (R->q.kind == WL_REQ_LEFF) {
      const int nrho = R->q.nrho, nT = R->q.nT;
      double *h = (double *)(pin + R->p_aux);
      memcpy(h, R->rho.data(), sizeof(double) * nrho);
      memcpy(h + nrho, R->Tg.data(), sizeof(double) * nT);
      wl::rt_log_simpson_weights(R->Tg.data(), nT, log(R->Tg[1]) - log(R->Tg[0]), h + nrho + nT);
      memcpy(h + nrho + 2 * nT, R->q.F, sizeof(double) * nF);
      double *d = (double *)(dmem + R->o_aux);
      wl::TintArgs &t = R->ta;
      memset(&t, 0, sizeof(t));
      t.groups = d_out;
      t.rho = d;
      t.T = d + nrho;
      t.w = d + nrho + nT;
      t.F = d + nrho + 2 * nT;
      t.Ig = d + R->n_aux_in;
      t.leff = t.Ig + (size_t)nrho * nF * R->ng;
      t.err = t.leff + (size_t)nrho * nF;
      t.nrho = nrho;
      t.nT = nT;
      t.nF = nF;
      t.ng = R->ng;
      t.nbins = R->q.nbins;
      t.profile = R->kprof;
      t.fermion = R->q.field.fermion != 0;
      t.l2 = R->q.field.lambda2;
      t.a = R->q.field.tubedist;
      t.lmin = R->q.field.lmin;
      const double rr = R->q.field.tubedist > 0.0 ? R->q.field.rimage / R->q.field.tubedist : 0.0;
      t.rimg2 = rr * rr;
      t.m2 = 1.0;        // Integrand.c:12
      t.e = 0.30282212;  // Integrand.c:14
    }
    ck(cudaMemcpyAsync(s->d_slots + R->slot, pin + R->p_args, sizeof(wl::SweepArgs),
                       cudaMemcpyHostToDevice, s->cs), "slot upload");
    ck(cudaMemcpyAsync(dmem + R->o_rj, pin + R->p_rj, R->o_perm - R->o_rj,
                       cudaMemcpyHostToDevice, s->cs), "request upload");
    if (a.perm)  // lattice: instances in decreasing proper time
      ck(wl::launch_order_instances(a.cx, a.cy, a.rtT, n, 1.0f / a.field.a,
                                    const_cast<int *>(a.perm), s->cs),
         "instance order");
    if (R->n_aux_in)
      ck(cudaMemcpyAsync(dmem + R->o_aux, pin + R->p_aux, sizeof(double) * R->n_aux_in,
                         cudaMemcpyHostToDevice, s->cs), "grid upload");
    ck(cudaMemsetAsync(d_status, 0, sizeof(int), s->cs), "status reset");
    ck(cudaEventCreateWithFlags(&R->done_ev, cudaEventDisableTiming), "event");
    s->running.push_back(R);
    copied = true;
  }
  if (copied) {
    ck(cudaEventRecord(s->adm_ev, s->cs), "admission event");
    ++s->adm_seq;
  }
  return progress;
}

bool tiles_left(const wl_server *s) {
  for (const Req *R : s->running)
    if (R->next_tile < R->ntiles) return true;
  return false;
}

// One launch of the persistent kernel on stream k with about one quantum of
// tiles, then the reductions of the requests whose last tile it carries.
// The quantum is shared among the admitted requests with tiles left as in
// processor sharing: an even split of the budget, a request that needs less
// than its share taking all it has and leaving the rest to the others, at
// least one tile each; while tiles are left a launch gets at least one tile
// per CTA slot (oldest requests first).  A small request that arrives behind
// a large one is thus done within a few quanta instead of after it.
void launch_quantum(wl_server *s, int k) {
  cudaStream_t st = s->st[k];
  if (s->waited_seq[k] < s->adm_seq) {
    ck(cudaStreamWaitEvent(st, s->adm_ev, 0), "wait admission");
    s->waited_seq[k] = s->adm_seq;
  }
  std::vector<Req *> act;
  for (Req *R : s->running)
    if (R->next_tile < R->ntiles) act.push_back(R);
  const size_t m = act.size();
  std::vector<size_t> order(m);
  for (size_t i = 0; i < m; ++i) order[i] = i;
  auto left = [&](size_t i) { return act[i]->ntiles - act[i]->next_tile; };
  std::stable_sort(order.begin(), order.end(), [&](size_t x, size_t y) {
    return (double)left(x) * act[x]->tile_work < (double)left(y) * act[y]->tile_work;
  });
  std::vector<long long> take(m, 0);
  double budget = s->cfg.quantum_ms * s->rate;
  long long total = 0;
  for (size_t j = 0; j < m; ++j) {
    const size_t i = order[j];
    const double share = std::max(budget, 0.0) / (double)(m - j);
    long long t = (long long)ceil(share / act[i]->tile_work);
    t = std::max(1LL, std::min(t, left(i)));
    take[i] = t;
    total += t;
    budget -= (double)t * act[i]->tile_work;
  }
  for (size_t i = 0; i < m && total < s->grid_max; ++i) {  // fill every CTA slot
    const long long extra = std::min(left(i) - take[i], (long long)s->grid_max - total);
    take[i] += extra;
    total += extra;
  }
  double work = 0.0;
  int n = 0;
  long long side_tiles = 0;
  std::vector<Req *> closing;
  struct Side {  // a heavy-profile request's loop chunks [c0, c0 + nc)
    Req *R;
    int c0, nc;
  };
  std::vector<Side> side;
  wl::BatchTile *h = s->h_tiles[k];
  for (size_t i = 0; i < m && n < kMaxQuantumTiles; ++i) {
    Req *R = act[i];
    if (!wl::batch_in_kernel(R->kprof)) {
      // not in the persistent kernel: whole loop chunks, as a sweep launch
      // over them (next_tile stays a multiple of tiles_x)
      const long long tx = R->tiles_x;
      const long long t = std::min(left(i), (take[i] + tx - 1) / tx * tx);
      side.push_back({R, (int)(R->next_tile / tx), (int)(t / tx)});
      R->next_tile += t;
      side_tiles += t;
      work += (double)t * R->tile_work;
      if (R->next_tile >= R->ntiles) closing.push_back(R);
      continue;
    }
    const int cost = R->lc * R->q.ppl *
                     (wl::sweep_tile_instances(R->kprof, R->q.field.nint) / wl::kSweepThreads);
    for (long long c = 0; c < take[i] && n < kMaxQuantumTiles; ++c) {
      const long long t = R->next_tile++;
      h[n++] = {R->slot, (int)(t % R->tiles_x), (int)(t / R->tiles_x), cost};
      work += R->tile_work;
    }
    if (R->next_tile >= R->ntiles) closing.push_back(R);
  }
  // longest tiles first (LPT), ties in request order
  std::stable_sort(h, h + n, [](const wl::BatchTile &x, const wl::BatchTile &y) {
    return x.cost > y.cost;
  });
  if (n > 0) {
    ck(cudaMemcpyAsync(s->d_tiles[k], h, sizeof(wl::BatchTile) * n, cudaMemcpyHostToDevice, st),
       "tile upload");
    ck(cudaMemsetAsync(s->d_counter + k, 0, sizeof(int), st), "counter reset");
  }
  {
    bool reset;
    {
      std::lock_guard<std::mutex> lk(s->mu);
      reset = s->base_reset;
      s->base_reset = false;
    }
    if (reset || !s->base_recorded) {
      ck(cudaEventRecord(s->ev_base, st), "event");
      s->base_recorded = true;
    }
  }
  ck(cudaEventRecord(s->ev_start[k], st), "event");
  if (n > 0) {
    wl::BatchArgs B;
    B.jobs = s->d_slots;
    B.tiles = s->d_tiles[k];
    B.ntiles = n;
    B.counter = s->d_counter + k;
    ck(wl::launch_batch(B, std::min(s->grid_max, n), st), "batch launch");
  }
  for (const Side &x : side) {  // the request's own sweep over its chunk range
    const Req *R = x.R;
    wl::SweepArgs a = R->args;
    a.loops += (size_t)x.c0 * R->lc * R->q.ppl;
    a.partial += (size_t)x.c0 * R->q.nF * 3 * R->ninst;
    a.n_chunks = x.nc;
    ck(wl::launch_sweep(R->kprof, R->q.field.fermion != 0, R->q.field.nint, a, st),
       "sweep launch");
  }
  ck(cudaEventRecord(s->ev_stop[k], st), "event");
  s->busy[k] = true;
  s->busy_work[k] = work;
  s->busy_tiles[k] = n + (int)std::min<long long>(side_tiles, 1 << 30);
  if (!closing.empty()) {
    // earlier tiles of these requests may be in the other stream's launch
    ck(cudaStreamWaitEvent(st, s->ev_stop[k ^ 1], 0), "wait other stream");
    for (Req *R : closing) {
      const wl::ReduceJob *d_rj = (const wl::ReduceJob *)(R->dmem + R->o_rj);
      ck(wl::launch_batch_reduce(d_rj, 1, R->ninst * R->q.nF, st), "reduce");
      char *po = R->pin + R->p_out;
      ck(cudaMemcpyAsync(po, R->dmem, sizeof(int), cudaMemcpyDeviceToHost, st), "status read");
      const double *src;
      if (R->q.kind == WL_REQ_LEFF) {
        ck(wl::launch_tint(R->ta, st), "proper-time integral");
        src = R->ta.leff;  // leff | err contiguous
      } else {
        src = R->q.out_group ? R->rj.out_group : R->rj.out_mean;  // mean | sem contiguous
      }
      ck(cudaMemcpyAsync(po + 16, src, sizeof(double) * R->n_out, cudaMemcpyDeviceToHost, st),
         "result read");
      ck(cudaEventRecord(R->done_ev, st), "event");
      R->finishing = true;
    }
  }
  std::lock_guard<std::mutex> lk(s->mu);
  ++s->n_launch;
}

bool retire_launches(wl_server *s) {
  bool progress = false;
  for (int k = 0; k < 2; ++k) {
    if (!s->busy[k]) continue;
    const cudaError_t q = cudaEventQuery(s->ev_stop[k]);
    if (q == cudaErrorNotReady) continue;
    ck(q, "launch");
    s->busy[k] = false;
    progress = true;
    float ms = 0.0f;
    ck(cudaEventElapsedTime(&ms, s->ev_start[k], s->ev_stop[k]), "elapsed");
    float t0 = 0.0f, t1 = 0.0f;
    if (cudaEventElapsedTime(&t0, s->ev_base, s->ev_start[k]) == cudaSuccess &&
        cudaEventElapsedTime(&t1, s->ev_base, s->ev_stop[k]) == cudaSuccess) {
      std::lock_guard<std::mutex> lk(s->mu);
      // a launch issued before the base was re-recorded (t0 < 0) belongs to
      // the previous statistics
      if (!s->base_reset && t0 >= 0.0f) s->spans.emplace_back((double)t0, (double)t1);
    } else {
      cudaGetLastError();  // a launch started before the base was re-recorded
    }
    // a launch that filled every CTA slot measures the device rate
    if (s->busy_tiles[k] >= s->grid_max && ms > 0.05f) {
      const double r = s->busy_work[k] / ms;
      s->rate = s->rate > 0.0 ? 0.7 * s->rate + 0.3 * r : r;
    }
  }
  return progress;
}

bool complete_requests(wl_server *s) {
  bool progress = false;
  for (size_t i = 0; i < s->running.size();) {
    Req *R = s->running[i];
    if (!R->finishing) {
      ++i;
      continue;
    }
    const cudaError_t q = cudaEventQuery(R->done_ev);
    if (q == cudaErrorNotReady) {
      ++i;
      continue;
    }
    ck(q, "request");
    const char *po = R->pin + R->p_out;
    int dst = 0;
    memcpy(&dst, po, sizeof(int));
    const double *v = (const double *)(po + 16);
    int status = WL_OK;
    if (dst == wl::kDevTimeout) {
      status = WL_ERR_TIMEOUT;
      set_err(s, status, "request %lld: a shared-memory stage copy timed out", R->ticket);
    } else if (dst != wl::kDevOk) {
      status = WL_ERR_INVALID;
      set_err(s, status, "request %lld: device status %d", R->ticket, dst);
    }
    if (status == WL_OK) {
      const size_t nm = (size_t)R->ninst * R->q.nF;
      if (R->q.kind == WL_REQ_LEFF) {
        const size_t nl = (size_t)R->q.nrho * R->q.nF;
        memcpy(R->q.out_leff, v, sizeof(double) * nl);
        memcpy(R->q.out_err, v + nl, sizeof(double) * nl);
      } else if (R->q.out_group) {
        const size_t ngrp = nm * R->ng;
        memcpy(R->q.out_group, v, sizeof(double) * ngrp);
        if (R->q.out_mean) memcpy(R->q.out_mean, v + ngrp, sizeof(double) * nm);
        if (R->q.out_sem) memcpy(R->q.out_sem, v + ngrp + nm, sizeof(double) * nm);
      } else {
        if (R->q.out_mean) memcpy(R->q.out_mean, v, sizeof(double) * nm);
        if (R->q.out_sem) memcpy(R->q.out_sem, v + nm, sizeof(double) * nm);
      }
    }
    ck(cudaEventDestroy(R->done_ev), "event");
    R->done_ev = nullptr;
    ck(cudaFreeAsync(R->dmem, s->cs), "free");
    pin_put(s, R->pin, R->pbytes);
    R->dmem = R->pin = nullptr;
    s->free_slots.push_back(R->slot);
    s->in_use -= (double)R->dbytes;
    R->ens->users--;
    R->ens->last_use = ++s->use_clock;
    s->running.erase(s->running.begin() + i);
    finish(s, R, status);
    progress = true;
  }
  return progress;
}

void publish(wl_server *s) {
  std::lock_guard<std::mutex> lk(s->mu);
  s->pub_in_use = s->in_use;
  s->pub_resident = (int)s->ens.size();
}

void worker_main(wl_server *s) {
  try {
    ck(cudaSetDevice(s->cfg.device), "cudaSetDevice");
    for (;;) {
      {
        std::unique_lock<std::mutex> lk(s->mu);
        while (!s->incoming.empty()) {
          s->pending.push_back(s->incoming.front());
          s->incoming.pop_front();
        }
        if (s->stopping && s->pending.empty() && s->running.empty() && !s->busy[0] &&
            !s->busy[1])
          break;
      }
      bool progress = retire_launches(s);
      progress |= complete_requests(s);
      progress |= admit(s);
      if (!s->busy[0] || !s->busy[1]) {
        if (tiles_left(s)) {
          int k = s->next_stream;
          if (s->busy[k]) k ^= 1;
          launch_quantum(s, k);
          s->next_stream = k ^ 1;
          progress = true;
        }
      }
      publish(s);
      if (progress) continue;
      std::unique_lock<std::mutex> lk(s->mu);
      if (!s->incoming.empty() || s->stopping) continue;
      const bool idle = s->pending.empty() && s->running.empty() && !s->busy[0] && !s->busy[1];
      if (idle)
        s->cv_work.wait(lk, [&] { return !s->incoming.empty() || s->stopping; });
      else
        s->cv_work.wait_for(lk, std::chrono::microseconds(100));
    }
    ck(cudaStreamSynchronize(s->cs), "final sync");
  } catch (const WorkerError &e) {
    // the device state is unknown: every request still open fails
    cudaGetLastError();
    std::vector<Req *> open;
    {
      std::lock_guard<std::mutex> lk(s->mu);
      s->failed = true;
      s->err = "server worker: " + e.msg;
      for (Req *R : s->incoming) open.push_back(R);
      s->incoming.clear();
    }
    for (Req *R : s->pending) open.push_back(R);
    for (Req *R : s->running) open.push_back(R);
    s->pending.clear();
    s->running.clear();
    for (Req *R : open) finish(s, R, WL_ERR_CUDA);
  }
}

double percentile(std::vector<double> v, double p) {
  if (v.empty()) return 0.0;
  std::sort(v.begin(), v.end());
  size_t i = (size_t)ceil(p * (double)v.size());
  if (i < 1) i = 1;
  if (i > v.size()) i = v.size();
  return v[i - 1];
}

}  // namespace

#pragma GCC visibility push(default)
extern "C" {

int wl_server_create(const wl_server_config *cfg, wl_server **out) {
  if (!cfg || !out) return WL_ERR_INVALID;
  *out = nullptr;
  wl_server_config c = *cfg;
  if (c.quantum_ms <= 0.0) c.quantum_ms = 20.0;
  if (c.points_per_tile <= 0) c.points_per_tile = 16384;
  if (c.max_requests <= 0) c.max_requests = 1024;
  if (!(c.quantum_ms <= 10000.0) || c.max_requests > (1 << 20) || c.points_per_tile > (1 << 24))
    return WL_ERR_INVALID;
  if (cudaSetDevice(c.device) != cudaSuccess) {
    cudaGetLastError();
    return WL_ERR_CUDA;
  }
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
    cudaGetLastError();
    return WL_ERR_CUDA;
  }
  if (c.hbm_budget_bytes <= 0.0) c.hbm_budget_bytes = 0.8 * (double)free_b;
  std::unique_ptr<wl_server> s(new wl_server());
  s->cfg = c;
  cudaDeviceGetAttribute(&s->num_sms, cudaDevAttrMultiProcessorCount, c.device);
  const int occ = wl::batch_max_ctas_per_sm();
  const int per_sm = c.ctas_per_sm > 0 && c.ctas_per_sm <= occ ? c.ctas_per_sm : occ;
  s->grid_max = per_sm * s->num_sms;
  s->rate = 4.0e8;  // weighted tile work per ms until the first full launch is timed
  cudaError_t e = cudaStreamCreateWithFlags(&s->cs, cudaStreamNonBlocking);
  for (int k = 0; k < 2 && e == cudaSuccess; ++k) {
    e = cudaStreamCreateWithFlags(&s->st[k], cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&s->ev_start[k]);
    if (e == cudaSuccess) e = cudaEventCreate(&s->ev_stop[k]);
    if (e == cudaSuccess && !s->ev_base) e = cudaEventCreate(&s->ev_base);
    if (e == cudaSuccess) e = cudaMalloc((void **)&s->d_tiles[k], sizeof(wl::BatchTile) * kMaxQuantumTiles);
    if (e == cudaSuccess)
      e = cudaHostAlloc((void **)&s->h_tiles[k], sizeof(wl::BatchTile) * kMaxQuantumTiles,
                        cudaHostAllocDefault);
  }
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->adm_ev, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaMalloc((void **)&s->d_counter, 2 * sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc((void **)&s->d_slots, sizeof(wl::SweepArgs) * c.max_requests);
  if (e == cudaSuccess) {
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, c.device) == cudaSuccess) {
      uint64_t keep = (uint64_t)c.hbm_budget_bytes;  // keep freed blocks for reuse
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    cudaGetLastError();
  }
  if (e != cudaSuccess) {
    cudaGetLastError();
    wl_server *raw = s.release();
    raw->stopping = true;
    wl_server_destroy(raw);
    return WL_ERR_CUDA;
  }
  for (int i = c.max_requests - 1; i >= 0; --i) s->free_slots.push_back(i);
  wl_server *raw = s.release();
  raw->worker = std::thread(worker_main, raw);
  *out = raw;
  return WL_OK;
}

int wl_server_submit(wl_server *srv, const wl_request *req, long long *ticket) {
  if (!srv || !ticket) return WL_ERR_INVALID;
  *ticket = 0;
  std::unique_ptr<Req> R(new Req());
  int r = check_request(srv, req, R.get());
  if (r) return r;
  R->t_submit = Clock::now();
  std::lock_guard<std::mutex> lk(srv->mu);
  if (srv->failed) return WL_ERR_CUDA;
  if (srv->stopping) {
    srv->err = "server is stopping";
    return WL_ERR_INVALID;
  }
  R->ticket = srv->next_ticket++;
  *ticket = R->ticket;
  if (srv->n_sub == 0) srv->t_first = R->t_submit;
  ++srv->n_sub;
  srv->incoming.push_back(R.get());
  srv->owned[R->ticket] = std::move(R);
  srv->cv_work.notify_one();
  return WL_OK;
}

int wl_server_wait(wl_server *srv, long long ticket, double timeout_ms) {
  if (!srv) return WL_ERR_INVALID;
  std::unique_lock<std::mutex> lk(srv->mu);
  auto it = srv->owned.find(ticket);
  if (it == srv->owned.end()) {
    srv->err = "unknown ticket";
    return WL_ERR_NOTFOUND;
  }
  Req *R = it->second.get();
  auto ready = [&] { return R->done; };
  if (timeout_ms < 0.0) {
    srv->cv_done.wait(lk, ready);
  } else if (!srv->cv_done.wait_for(lk, std::chrono::duration<double, std::milli>(timeout_ms),
                                    ready)) {
    return WL_PENDING;
  }
  const int st = R->status;
  srv->owned.erase(it);
  return st;
}

int wl_server_get_stats(wl_server *srv, wl_server_stats *out) {
  if (!srv || !out) return WL_ERR_INVALID;
  std::lock_guard<std::mutex> lk(srv->mu);
  memset(out, 0, sizeof(*out));
  out->submitted = srv->n_sub;
  out->completed = srv->n_done;
  out->rejected = srv->n_rej;
  out->failed = srv->n_fail;
  out->p50_ms = percentile(srv->lat_ms, 0.50);
  out->p99_ms = percentile(srv->lat_ms, 0.99);
  out->p999_ms = percentile(srv->lat_ms, 0.999);
  double sum = 0.0, mx = 0.0;
  for (double v : srv->lat_ms) {
    sum += v;
    mx = std::max(mx, v);
  }
  out->mean_ms = srv->lat_ms.empty() ? 0.0 : sum / (double)srv->lat_ms.size();
  out->max_ms = mx;
  out->wall_s = srv->n_done ? std::chrono::duration<double>(srv->t_last - srv->t_first).count() : 0.0;
  out->segments = srv->seg_done;
  out->launches = srv->n_launch;
  out->resident_ensembles = srv->pub_resident;
  out->hbm_bytes_in_use = srv->pub_in_use;
  // union of the launch intervals (two streams may overlap)
  std::vector<std::pair<double, double>> sp = srv->spans;
  std::sort(sp.begin(), sp.end());
  double busy = 0.0, lo = 0.0, hi = -1.0;
  for (const auto &x : sp) {
    if (x.first > hi) {
      if (hi > lo) busy += hi - lo;
      lo = x.first;
      hi = x.second;
    } else {
      hi = std::max(hi, x.second);
    }
  }
  if (hi > lo) busy += hi - lo;
  out->device_busy_s = busy * 1e-3;
  double last = 0.0;
  for (const auto &x : sp) last = std::max(last, x.second);
  out->device_span_s = sp.empty() ? 0.0 : (last - sp.front().first) * 1e-3;
  return WL_OK;
}

int wl_server_reset_stats(wl_server *srv) {
  if (!srv) return WL_ERR_INVALID;
  std::lock_guard<std::mutex> lk(srv->mu);
  srv->n_sub = srv->n_done = srv->n_rej = srv->n_fail = srv->n_launch = 0;
  srv->lat_ms.clear();
  srv->seg_done = 0.0;
  srv->spans.clear();
  srv->base_reset = true;
  return WL_OK;
}

int wl_server_last_error(wl_server *srv, char *buf, int buflen) {
  if (!srv || !buf || buflen < 1) return WL_ERR_INVALID;
  std::lock_guard<std::mutex> lk(srv->mu);
  snprintf(buf, (size_t)buflen, "%s", srv->err.c_str());
  return WL_OK;
}

int wl_server_destroy(wl_server *srv) {
  if (!srv) return WL_ERR_INVALID;
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    srv->stopping = true;
    srv->cv_work.notify_all();
  }
  if (srv->worker.joinable()) srv->worker.join();
  cudaSetDevice(srv->cfg.device);
  if (srv->cs) cudaStreamSynchronize(srv->cs);
  for (int k = 0; k < 2; ++k) {
    if (srv->st[k]) {
      cudaStreamSynchronize(srv->st[k]);
      cudaStreamDestroy(srv->st[k]);
    }
    if (srv->ev_start[k]) cudaEventDestroy(srv->ev_start[k]);
    if (srv->ev_stop[k]) cudaEventDestroy(srv->ev_stop[k]);
    if (srv->d_tiles[k]) cudaFree(srv->d_tiles[k]);
    if (srv->h_tiles[k]) cudaFreeHost(srv->h_tiles[k]);
  }
  for (auto &e : srv->ens) {
    if (e->dev) cudaFree(e->dev);
    if (e->bbox) cudaFree(e->bbox);
  }
  for (auto &kv : srv->pin_cache)
    for (char *p : kv.second) cudaFreeHost(p);
  for (auto &kv : srv->splines) {
    cudaFree(kv.second.first);
    cudaFree(kv.second.second);
  }
  if (srv->adm_ev) cudaEventDestroy(srv->adm_ev);
  if (srv->ev_base) cudaEventDestroy(srv->ev_base);
  if (srv->d_counter) cudaFree(srv->d_counter);
  if (srv->d_slots) cudaFree(srv->d_slots);
  if (srv->cs) cudaStreamDestroy(srv->cs);
  cudaGetLastError();
  delete srv;
  return WL_OK;
}

}  // extern "C"
#pragma GCC visibility pop
