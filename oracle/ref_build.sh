#!/usr/bin/env bash
# Builds oracle/_ref/ref_harness from the reference's own, unmodified sources
# (suliaron/red.cuda mounted read-only at /root/reference, or the directory
# named by RED_REFERENCE).  Test infrastructure: the binary produces golden
# vectors for tests/golden/ on the CPU and, built on a machine with a GPU from
# the staged copy (oracle/ref_stage.sh; RED_REFERENCE=baseline/_ref/red.cuda,
# RED_REF_OUT=oracle/_ref/box), runs red's own GPU path for the parity pins
# and the plain-FP64 baseline.
#
# Two build-time shims, no source edits:
#   -DclockRate=maxThreadsPerBlock  cudaDeviceProp::clockRate was removed in
#                                   CUDA 13 (red.cuda.utility/util.cu:175)
#   -fmad=false -O2                 the reference's own flags (Makefile:17),
#                                   targeting this toolkit's sm_103a
# main.cu, options.cpp and parameter.cpp are not linked: the harness calls
# pp_disk and the integrators directly.  Only the utility copy of Tokenizer is
# linked (the two copies clash).
set -euo pipefail
REF=${RED_REFERENCE:-/root/reference}
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="${RED_REF_OUT:-$HERE/_ref}"
mkdir -p "$OUT/obj"
[ -d "$REF/src/red.cuda" ] || { echo "reference not found at $REF" >&2; exit 3; }

NVCC=${NVCC:-nvcc}
FLAGS="-O2 -fmad=false -gencode arch=compute_103a,code=sm_103a -DclockRate=maxThreadsPerBlock -w"
INC="-I$REF/red.type -I$REF/src/red.cuda.utility -I$REF/src/red.cuda"

SRCS="
$REF/src/red.cuda/pp_disk.cu
$REF/src/red.cuda/integrator.cu
$REF/src/red.cuda/int_euler.cu
$REF/src/red.cuda/int_rungekutta2.cu
$REF/src/red.cuda/int_rungekutta4.cu
$REF/src/red.cuda/int_rungekutta8.cu
$REF/src/red.cuda/analytic_gas_disk.cu
$REF/src/red.cuda/fargo_gas_disk.cu
$REF/src/red.cuda/nbody_exception.cpp
$REF/src/red.cuda.utility/tools.cpp
$REF/src/red.cuda.utility/file_util.cpp
$REF/src/red.cuda.utility/util.cu
$REF/src/red.cuda.utility/tokenizer.cpp
"
objs=()
pids=()
for s in $SRCS; do
  o="$OUT/obj/$(basename "${s%.*}").o"
  objs+=("$o")
  if [ ! -f "$o" ] || [ "$s" -nt "$o" ]; then
    $NVCC -c $FLAGS $INC -x cu -o "$o" "$s" &
    pids+=($!)
  fi
done
for p in "${pids[@]:-}"; do [ -n "$p" ] && wait "$p"; done
$NVCC $FLAGS $INC -o "$OUT/ref_harness" "$HERE/ref_harness.cu" "${objs[@]}"
echo "$OUT/ref_harness"
# red.cuda.initial's generator (golden vectors of the disk recipe), when its
# sources are there: the harness includes its main.cu with main() renamed
INIT="$REF/src/red.cuda.initial"
if [ -d "$INIT" ]; then
  iobjs=()
  for s in "$INIT/distribution.cpp" "$INIT/util_init.cpp" "$INIT/nebula.cpp"; do
    o="$OUT/obj/init_$(basename "${s%.*}").o"
    iobjs+=("$o")
    [ -f "$o" ] && [ ! "$s" -nt "$o" ] || $NVCC -c $FLAGS -I"$INIT" $INC -x cu -o "$o" "$s"
  done
  $NVCC $FLAGS -I"$INIT" $INC -o "$OUT/initial_harness" "$HERE/initial_harness.cu" "${iobjs[@]}" \
    "$OUT/obj/tools.o" "$OUT/obj/file_util.o" "$OUT/obj/util.o" "$OUT/obj/tokenizer.o"
  echo "$OUT/initial_harness"
fi
