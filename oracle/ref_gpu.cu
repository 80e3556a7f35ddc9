// ref_gpu.cu -- runs the reference's own ExpectValue kernel on the GPU.
//
// TEST INFRASTRUCTURE ONLY.  oracle/build_ref.sh compiles intEV.cu /
// intEVff.cu (unmodified, the reference's -prec-div=false -prec-sqrt=false)
// to sm_103a cubins in oracle/_ref/; this loader opens one with the CUDA
// runtime's library API and launches the reference kernel exactly as EV()
// does (intEV.cu:123-125): grid ceil(Nl/nThreads), one thread per loop.
// The reference kernel has no "inx < Nl" guard (intEV.cu:580) and relies on
// buffers padded to nBlocks*nThreads loops (EffAct.c:368-369); the loader
// refuses launches whose buffers are not padded that far.
#include <cuda_runtime.h>
#include <stdint.h>

namespace {
struct RefKernel {
  cudaLibrary_t lib;
  cudaKernel_t k;
  int ff;
};
RefKernel g_k[32];
int g_n = 0;
}  // namespace

extern "C" {

// ff = 1: the 11-argument intEVff.cu kernel (always spinor)
int refgpu_load(const char *cubin_path, int ff) {
  if (g_n >= 32) return -1;
  cudaLibrary_t lib;
  if (cudaLibraryLoadFromFile(&lib, cubin_path, nullptr, nullptr, 0, nullptr, nullptr, 0) !=
      cudaSuccess) {
    cudaGetLastError();
    return -2;
  }
  // ExpectValue(float4*, float4*, float4*, float4, float, float, float, int, int,
  //             float4*, float*[, int])  (intEV.cu:575-576, intEVff.cu:410-411)
  const char *name = ff ? "_Z11ExpectValueP6float4S0_S0_S_fffiiS0_Pf"
                        : "_Z11ExpectValueP6float4S0_S0_S_fffiiS0_Pfi";
  cudaKernel_t k;
  if (cudaLibraryGetKernel(&k, lib, name) != cudaSuccess) {
    cudaGetLastError();
    cudaLibraryUnload(lib);
    return -3;
  }
  g_k[g_n] = {lib, k, ff};
  return g_n++;
}

// Launch on the default stream and time it with CUDA events.
int refgpu_run(int handle, void *Wsscal, void *Wsferm, const void *worldlines, float xcmx,
               float xcmy, float F, float l2, float rtT, int Nl, int Nppl, int fermion,
               int nThreads, long long padded_loops, float *ms) {
  if (handle < 0 || handle >= g_n || nThreads <= 0 || Nl <= 0) return -1;
  const int nBlocks = (Nl + nThreads - 1) / nThreads;
  if ((long long)nBlocks * nThreads > padded_loops) return -4;  // no bounds guard in the kernel
  float4 xcm = make_float4(xcmx, xcmy, 0.0f, 0.0f);
  void *flcoefs = nullptr, *rho2sp = nullptr;
  void *wl = const_cast<void *>(worldlines);
  void *args[12] = {&Wsscal, &Wsferm, &wl, &xcm, &F, &l2, &rtT, &Nl, &Nppl,
                    &flcoefs, &rho2sp, &fermion};
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, 0);
  cudaError_t e = cudaLaunchKernel((const void *)g_k[handle].k, dim3(nBlocks), dim3(nThreads),
                                   args, 0, 0);
  cudaEventRecord(e1, 0);
  if (e == cudaSuccess) e = cudaEventSynchronize(e1);
  float t = 0.0f;
  cudaEventElapsedTime(&t, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (ms) *ms = t;
  if (e != cudaSuccess) {
    cudaGetLastError();
    return -5;
  }
  return 0;
}

}  // extern "C"
