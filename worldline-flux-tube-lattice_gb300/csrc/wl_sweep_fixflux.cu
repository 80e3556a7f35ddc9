// wl_sweep_fixflux.cu -- sweep kernel instantiations for profile(s): kFixflux kFixfluxFF
// (split by profile so that the build compiles them in parallel).
#include "wl_sweep.cuh"

namespace wl {

cudaError_t launch_sweep_fixflux(int profile, bool fermion, int nint, const SweepArgs *sa,
                                 const LoopArgs *la, cudaStream_t s) {
  switch (profile) {
    case kFixflux:
      return sa ? sweep_dispatch<kFixflux>(fermion, nint, *sa, s)
                : loopwarp_dispatch<kFixflux>(fermion, nint, *la, s);
    case kFixfluxFF:
      return sa ? sweep_dispatch<kFixfluxFF>(fermion, nint, *sa, s)
                : loopwarp_dispatch<kFixfluxFF>(fermion, nint, *la, s);
    default:
      return cudaErrorInvalidValue;
  }
}

}  // namespace wl
