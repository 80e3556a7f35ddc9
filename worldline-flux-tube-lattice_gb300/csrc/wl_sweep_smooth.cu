// wl_sweep_smooth.cu -- sweep kernel instantiations for profile(s): kSmooth
// (split by profile so that the build compiles them in parallel).
#include "wl_sweep.cuh"

namespace wl {

cudaError_t launch_sweep_smooth(int profile, bool fermion, int nint, const SweepArgs *sa,
                                 const LoopArgs *la, cudaStream_t s) {
  switch (profile) {
    case kSmooth:
      return sa ? sweep_dispatch<kSmooth>(fermion, nint, *sa, s)
                : loopwarp_dispatch<kSmooth>(fermion, nint, *la, s);
    default:
      return cudaErrorInvalidValue;
  }
}

}  // namespace wl
