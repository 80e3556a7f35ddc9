// wl_sweep_simple.cu -- sweep kernel instantiations for profile(s): kStep kQuadratic kGaussian
// (split by profile so that the build compiles them in parallel).
#include "wl_sweep.cuh"

namespace wl {

cudaError_t launch_sweep_simple(int profile, bool fermion, int nint, const SweepArgs *sa,
                                 const LoopArgs *la, cudaStream_t s) {
  switch (profile) {
    case kStep:
      return sa ? sweep_dispatch<kStep>(fermion, nint, *sa, s)
                : loopwarp_dispatch<kStep>(fermion, nint, *la, s);
    case kQuadratic:
      return sa ? sweep_dispatch<kQuadratic>(fermion, nint, *sa, s)
                : loopwarp_dispatch<kQuadratic>(fermion, nint, *la, s);
    case kGaussian:
      return sa ? sweep_dispatch<kGaussian>(fermion, nint, *sa, s)
                : loopwarp_dispatch<kGaussian>(fermion, nint, *la, s);
    default:
      return cudaErrorInvalidValue;
  }
}

}  // namespace wl
