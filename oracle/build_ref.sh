#!/bin/sh
# Builds the UNMODIFIED reference (header-only C++) with the project-written
# shims into oracle/_ref/ref_driver. TEST INFRASTRUCTURE ONLY: the binary is a
# parity oracle and CPU timing reference for this container; it is git-ignored
# and never part of the product. Needs the reference sources: REF_DIR, by
# default the read-only checkout of this build container; without them it
# builds nothing and exits 0.
set -e
HERE="$(cd "$(dirname "$0")" && pwd)"
REF_DIR="${REF_DIR:-/root/reference}"
if [ ! -f "$REF_DIR/Source/Domain.h" ]; then
  echo "reference sources not found at $REF_DIR; skipping oracle/_ref" >&2
  exit 0
fi
mkdir -p "$HERE/_ref"
# -ffp-contract=off: no fused multiply-add, so results match the x86 build bit for bit
g++ -std=c++11 -O3 -fopenmp -fpermissive -w -ffp-contract=off \
  -I"$HERE/shim" -I"$HERE" -iquote "$REF_DIR/Source" -iquote "$REF_DIR/External" \
  "$HERE/ref_driver.cpp" -o "$HERE/_ref/ref_driver"
# where the sources were found, for the tests that read the reference's own drivers
printf '%s\n' "$REF_DIR" > "$HERE/_ref/REFERENCE_DIR"
echo "built $HERE/_ref/ref_driver"
