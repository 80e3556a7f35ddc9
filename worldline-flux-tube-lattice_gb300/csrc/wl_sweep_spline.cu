// wl_sweep_spline.cu -- sweep kernel instantiations for profile(s): kSpline
// (split by profile so that the build compiles them in parallel; IEEE
// division and square root, unlike the periodic and fixflux units: the
// spline's f' = e^{-sin^2(pi rho/a)/l2}/l2 takes sin of sqrt(rho^2)).
#include "wl_sweep.cuh"

namespace wl {

cudaError_t launch_sweep_spline(int profile, bool fermion, int nint, const SweepArgs *sa,
                                const LoopArgs *la, cudaStream_t s) {
  if (profile != kSpline) return cudaErrorInvalidValue;
  return sa ? sweep_dispatch<kSpline>(fermion, nint, *sa, s)
            : loopwarp_dispatch<kSpline>(fermion, nint, *la, s);
}

}  // namespace wl
