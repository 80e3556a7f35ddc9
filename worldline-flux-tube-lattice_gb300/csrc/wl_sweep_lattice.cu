// wl_sweep_lattice.cu -- sweep kernel instantiations for the square lattice of
// Gaussian tubes (image sum); split out so the build compiles it in parallel.
#include "wl_sweep.cuh"

namespace wl {

cudaError_t launch_sweep_lattice(int profile, bool fermion, int nint, const SweepArgs *sa,
                                 const LoopArgs *la, cudaStream_t s) {
  if (profile != kLattice) return cudaErrorInvalidValue;
  return sa ? sweep_dispatch<kLattice>(fermion, nint, *sa, s)
            : loopwarp_dispatch<kLattice>(fermion, nint, *la, s);
}

}  // namespace wl
