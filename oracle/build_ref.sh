#!/usr/bin/env bash
# Builds the reference's own code for the CPU into oracle/_ref/ (test
# infrastructure: golden-vector generation only).  Compiles the sources where
# they lie under the reference tree -- nothing is copied -- with the
# reconstructed configuration header in oracle/refshim/.
#
#   oracle/build_ref.sh [REFERENCE_DIR]      (default /root/reference)
#
# Outputs oracle/_ref/ref_driver_<profile> for the intEV.cu profiles and
# oracle/_ref/ref_driver_ff for intEVff.cu (fixflux, spinor),
# oracle/_ref/ref_spline (periodic.c's spline table with the GSL ODE
# stand-in of refshim/), and the GPU
# kernels oracle/_ref/ref_<case>.cubin (sm_103a device code of intEV.cu /
# intEVff.cu with the reference's own -prec-div=false -prec-sqrt=false).  Exits 0 without
# building when the reference tree is absent.
set -euo pipefail
REF=${1:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ ! -f "$REF/intEV.cu" ]; then
  echo "build_ref: no reference tree at $REF; skipped"
  exit 0
fi
mkdir -p "$OUT/obj"
NVCC=${NVCC:-nvcc}
CC=${CC:-gcc}
CUDA_INC=$(dirname "$(command -v "$NVCC")")/../include
SHIM="-I$HERE/refshim -I$HERE/../include"
# the reference's device flags (Makefile:15,17); host pass made callable
NVFLAGS="-O2 -arch sm_103a -prec-div=false -prec-sqrt=false -DWLREF_HOSTCALL -DEV=wlref_gpu_EV -w"
CFLAGS="-O2 -fcommon -D_GNU_SOURCE -w -I$CUDA_INC $SHIM"

build_one() {  # name, kernel source, profile, extra defines
  local name=$1 src=$2 prof=$3 extra=$4
  local o="$OUT/obj/$name"
  "$NVCC" -c $NVFLAGS -Dprofile=$prof $extra $SHIM "$REF/$src" -o "$o.kernel.o"
  "$CC" -c $CFLAGS -Dprofile=$prof "$REF/Integrand.c" -o "$o.integrand.o"
  "$CC" -c $CFLAGS -Dprofile=$prof "$REF/Tint.c" -o "$o.tint.o"
  "$CC" -c $CFLAGS -Dprofile=$prof $extra "$HERE/ref_driver.c" -o "$o.driver.o"
  "$NVCC" -arch sm_103a -o "$OUT/ref_driver_$name" "$o.driver.o" "$o.kernel.o" \
    "$o.integrand.o" "$o.tint.o" -lm
}

# the reference kernel itself for the GPU (device code only, its own
# fast-math flags): loaded at run time by oracle/ref_gpu.cu
build_cubin() {  # name, kernel source, profile, lattice spacing, extra defines
  local name=$1 src=$2 prof=$3 a=$4 extra=$5
  "$NVCC" -cubin -O3 -arch sm_103a -prec-div=false -prec-sqrt=false -w -Dprofile=$prof \
    -DWLREF_TUBEDIST=${a}f $extra $SHIM "$REF/$src" -o "$OUT/ref_$name.cubin"
}

# the spline-profile table builder (periodic.c) with the GSL ODE stand-in
build_spline() {
  local o="$OUT/obj/spline"
  "$CC" -c $CFLAGS "$REF/periodic.c" -o "$o.periodic.o"
  "$CC" -c $CFLAGS "$HERE/refshim/gsl_odeiv2_standin.c" -o "$o.gsl.o"
  "$CC" -c $CFLAGS "$HERE/ref_spline.c" -o "$o.driver.o"
  "$CC" -o "$OUT/ref_spline" "$o.driver.o" "$o.periodic.o" "$o.gsl.o" -lm
}

pids=()
build_spline & pids+=($!)
for prof in step smooth quadratic gaussian; do
  build_cubin "$prof" intEV.cu "$prof" 1.0 "" & pids+=($!)
done
build_cubin periodic_a1 intEV.cu periodic 1.0 "" & pids+=($!)
build_cubin periodic_a2 intEV.cu periodic 2.0 "" & pids+=($!)
build_cubin fixflux_a2 intEV.cu fixflux 2.0 "" & pids+=($!)
build_cubin ff_a2 intEVff.cu fixflux 2.0 "-DWLREF_FF" & pids+=($!)
for prof in step smooth quadratic gaussian periodic fixflux; do
  build_one "$prof" intEV.cu "$prof" "" & pids+=($!)
done
build_one ff intEVff.cu fixflux "-DWLREF_FF" & pids+=($!)
rc=0
for p in "${pids[@]}"; do wait "$p" || rc=1; done
exit $rc
