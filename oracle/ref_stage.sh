#!/usr/bin/env bash
# Stages an unmodified copy of the reference's sources for the machine that
# has the GPU: red.type/, src/red.cuda/ and src/red.cuda.utility/ (sources and
# headers only) from /root/reference, or the directory named by RED_REFERENCE,
# into baseline/_ref/red.cuda/.  That directory is git-ignored: it is the
# reference install, not part of this project, and it exists only so that
# oracle/ref_build.sh can build red's own GPU path where the GPU is (binaries
# built here are for another CPU architecture).  Nothing is edited; the build
# shims are compiler flags in ref_build.sh.
set -euo pipefail
REF=${RED_REFERENCE:-/root/reference}
HERE="$(cd "$(dirname "$0")" && pwd)"
DST="$HERE/../baseline/_ref/red.cuda"
[ -d "$REF/src/red.cuda" ] || { echo "reference not found at $REF" >&2; exit 3; }
for d in red.type src/red.cuda src/red.cuda.utility; do
  mkdir -p "$DST/$d"
  for f in "$REF/$d"/*; do
    case "$f" in
      *.cu|*.cpp|*.h|*.cuh) cp -p "$f" "$DST/$d/" ;;
    esac
  done
done
echo "$DST"
