// wl_noalloc.cu -- wl_eval_noalloc: batched <W> without any allocation.
//
// Some callers cannot let a library allocate device memory: code running
// under a framework's caching allocator that owns the whole device (a
// cudaMalloc behind its back can fail or break its accounting), inside a
// region where cudaMalloc is not permitted, or on latency-critical paths where
// cudaMalloc/cudaFree would synchronise the device.  wl_eval_noalloc serves
// them: it runs the same kernels as wl_eval_device, but its scratch memory
// (the instance constants and the FP64 partial sums between the sweep and the
// reduction) is one file-scope device array of fixed size, g_noalloc_scratch,
// which every GPU that loads the library holds until the process exits.
#include <cuda.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <mutex>

#include "../../include/wlgpu.h"
#include "wl_internal.h"

namespace wl {
int shared_field_to_dev(const wl_field *f, int *kprofile, FieldDev *d);
void shared_fill_flux(SweepArgs &a, const wl_field *f, int nF, const double *F);
void shared_fill_flux(LoopArgs &a, const wl_field *f, int nF, const double *F);
int shared_plan_chunk(int group);
}  // namespace wl

namespace {

// 32 MiB: [status word | 255 bytes pad][instance floats][FP64 partial sums]
constexpr size_t kScratchBytes = (size_t)32 << 20;
__device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void *g_scratch_ptr[kMaxDevices];  // device address of g_noalloc_scratch, per device

typedef CUresult (*AddressRangeFn)(CUdeviceptr *, size_t *, CUdeviceptr);

int nfail(int code, const char *fmt, const char *a = "", long long b = 0, long long c = 0) {
  fprintf(stderr, "wl_eval_noalloc: ");
  fprintf(stderr, fmt, a, b, c);
  fprintf(stderr, "\n");
  return code;
}

// Device memory of the current device covering [p, p + bytes)?
int check_dev(const void *p, size_t bytes, const char *name, int dev) {
  if (!p) return nfail(WL_ERR_INVALID, "%s is NULL", name);
  if ((uintptr_t)p % 8 != 0) return nfail(WL_ERR_INVALID, "%s is not 8-byte aligned", name);
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return nfail(WL_ERR_INVALID, "%s is not a CUDA pointer", name);
  }
  if ((at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged) ||
      (at.type == cudaMemoryTypeDevice && at.device != dev))
    return nfail(WL_ERR_INVALID, "%s is not device memory of the current device", name);
  static AddressRangeFn range = [] {
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuMemGetAddressRange", &fn, 12000, cudaEnableDefault,
                                         &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      fn = nullptr;
    cudaGetLastError();
    return (AddressRangeFn)fn;
  }();
  if (range) {
    CUdeviceptr base = 0;
    size_t size = 0;
    if (range(&base, &size, (CUdeviceptr)(uintptr_t)p) == CUDA_SUCCESS &&
        (uintptr_t)p + bytes > (uintptr_t)base + size)
      return nfail(WL_ERR_INVALID, "%s is smaller than %lld bytes", name, (long long)bytes);
  }
  return WL_OK;
}

// The array's device address on the current device: looked up once per
// device with cudaGetSymbolAddress (host code cannot use the symbol itself).
int scratch_address(int dev, unsigned char **out) {
  if (dev < 0 || dev >= kMaxDevices) return nfail(WL_ERR_INVALID, "device %s%lld out of range", "", dev);
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_scratch_ptr[dev]) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return nfail(WL_ERR_CUDA, "cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
    g_scratch_ptr[dev] = p;
  }
  *out = (unsigned char *)g_scratch_ptr[dev];
  return WL_OK;
}

}  // namespace

#pragma GCC visibility push(default)
extern "C" int wl_eval_noalloc(const float *dev_loops, int Nl, int ppl, const wl_field *field,
                               int ninst, const double *dev_cx, const double *dev_cy,
                               const double *dev_T, int nF, const double *host_F, int group,
                               double *dev_out_group, double *dev_out_mean,
                               double *dev_out_sem, void *stream) {
  if (!field || !host_F) return nfail(WL_ERR_INVALID, "NULL field or flux array");
  if (Nl < 1 || ppl < 4 || ppl % 4 || (double)Nl * ppl > 2147483647.0)
    return nfail(WL_ERR_INVALID, "need Nl >= 1 and ppl a positive multiple of 4%s", "");
  if (ninst < 1) return nfail(WL_ERR_INVALID, "ninst must be >= 1%s", "");
  if (nF < 1 || nF > wl::kMaxF) return nfail(WL_ERR_INVALID, "nF must be in [1, 4]%s", "");
  if (group < 1 || Nl % group) return nfail(WL_ERR_INVALID, "group must divide Nl%s", "");
  for (int j = 0; j < nF; ++j)
    if (!isfinite(host_F[j])) return nfail(WL_ERR_INVALID, "F is not finite%s", "");
  int kprof;
  wl::FieldDev fd;
  if (wl::shared_field_to_dev(field, &kprof, &fd) != WL_OK)
    return nfail(WL_ERR_INVALID, "invalid field (profile, nint, mode or lambda2)%s", "");

  // the same kernel and loop partition as wl_eval_device
  const bool use_sweep = ninst >= 32;
  const int lc = use_sweep ? wl::shared_plan_chunk(group) : 1;
  const int n_chunks = Nl / lc, cpg = group / lc, ng = Nl / group;
  if (use_sweep && n_chunks > 65535) return nfail(WL_ERR_INVALID, "group too small for Nl%s", "");
  const size_t inst_off = 256;
  const size_t inst_bytes = (size_t)wl::kInstArrays * ninst * sizeof(float);
  const size_t part_off = (inst_off + inst_bytes + 255) & ~(size_t)255;
  const size_t need = part_off + (size_t)n_chunks * nF * 3 * ninst * sizeof(double);
  if (need > kScratchBytes)
    return nfail(WL_ERR_INVALID,
                 "the request needs %s%lld bytes of scratch, more than the fixed %lld "
                 "(32 MiB); split the instances into smaller batches",
                 "", (long long)need, (long long)kScratchBytes);

  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return nfail(WL_ERR_CUDA, "no current device%s", "");
  const size_t nb = (size_t)ninst * sizeof(double);
  int r;
  if ((r = check_dev(dev_loops, (size_t)Nl * ppl * 16, "dev_loops", dev)) ||
      (r = check_dev(dev_cx, nb, "dev_cx", dev)) || (r = check_dev(dev_cy, nb, "dev_cy", dev)) ||
      (r = check_dev(dev_T, nb, "dev_T", dev)))
    return r;
  if ((uintptr_t)dev_loops % 16) return nfail(WL_ERR_INVALID, "dev_loops is not 16-byte aligned%s", "");
  if (dev_out_group && (r = check_dev(dev_out_group, nb * nF * ng, "dev_out_group", dev))) return r;
  if (dev_out_mean && (r = check_dev(dev_out_mean, nb * nF, "dev_out_mean", dev))) return r;
  if (dev_out_sem && (r = check_dev(dev_out_sem, nb * nF, "dev_out_sem", dev))) return r;

  unsigned char *base;
  if ((r = scratch_address(dev, &base))) return r;
  int *status = (int *)base;
  float *inst = (float *)(base + inst_off);
  double *partial = (double *)(base + part_off);
  cudaStream_t s = (cudaStream_t)stream;

  // the array keeps the previous call's contents: only the status word must
  // start at zero (every partial sum read below is written first)
  cudaError_t ce = cudaMemsetAsync(status, 0, sizeof(int), s);
  if (ce == cudaSuccess)
    ce = wl::launch_instance_setup(dev_cx, dev_cy, dev_T, ninst, ppl, inst, status, s);
  if (ce == cudaSuccess && use_sweep) {
    wl::SweepArgs a;
    memset(&a, 0, sizeof(a));
    a.loops = (const float4 *)dev_loops;
    a.Nl = Nl;
    a.ppl = ppl;
    a.ninst = ninst;
    a.cx = inst;
    a.cy = inst + ninst;
    a.rtT = inst + 2 * ninst;
    a.tqh = inst + 3 * ninst;
    a.tql = inst + 4 * ninst;
    a.nF = nF;
    wl::shared_fill_flux(a, field, nF, host_F);
    a.field = fd;
    a.chunk_loops = lc;
    a.n_chunks = n_chunks;
    a.partial = partial;
    a.status = status;
    a.wait_tries = 1u << 22;
    ce = wl::launch_sweep(kprof, field->fermion != 0, field->nint, a, s);
  } else if (ce == cudaSuccess) {
    wl::LoopArgs a;
    memset(&a, 0, sizeof(a));
    a.loops = (const float4 *)dev_loops;
    a.Nl = Nl;
    a.ppl = ppl;
    a.ninst = ninst;
    a.cx = inst;
    a.cy = inst + ninst;
    a.rtT = inst + 2 * ninst;
    a.tqh = inst + 3 * ninst;
    a.tql = inst + 4 * ninst;
    a.nF = nF;
    wl::shared_fill_flux(a, field, nF, host_F);
    a.field = fd;
    a.partial = partial;
    ce = wl::launch_loopwarp(kprof, field->fermion != 0, field->nint, a, s);
  }
  if (ce == cudaSuccess)
    ce = wl::launch_group_reduce(partial, n_chunks, cpg, group, ninst, nF, dev_out_group,
                                 dev_out_mean, dev_out_sem, s);
  int st = 0;
  if (ce == cudaSuccess) ce = cudaMemcpyAsync(&st, status, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
  if (ce != cudaSuccess) return nfail(WL_ERR_CUDA, "%s", cudaGetErrorString(ce));
  if (st == wl::kDevTimeout) return nfail(WL_ERR_TIMEOUT, "a shared-memory stage copy timed out%s", "");
  if (st == wl::kDevBadInstance)
    return nfail(WL_ERR_INVALID, "an instance has T <= 0 or a non-finite value%s", "");
  return WL_OK;
}
#pragma GCC visibility pop
