// wl_sweep_periodic.cu -- sweep kernel instantiations for profile(s): kPeriodic
// (split by profile so that the build compiles them in parallel).
#include "wl_sweep.cuh"

namespace wl {

cudaError_t launch_sweep_periodic(int profile, bool fermion, int nint, const SweepArgs *sa,
                                 const LoopArgs *la, cudaStream_t s) {
  switch (profile) {
    case kPeriodic:
      return sa ? sweep_dispatch<kPeriodic>(fermion, nint, *sa, s)
                : loopwarp_dispatch<kPeriodic>(fermion, nint, *la, s);
    default:
      return cudaErrorInvalidValue;
  }
}

}  // namespace wl
