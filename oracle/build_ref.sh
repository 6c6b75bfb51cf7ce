#!/bin/sh
# Oracle test infrastructure: compile the reference's src/random_lcg.cpp (the
# one hot-path source of the reference that builds without cmake, HDF5,
# pugixml, fmt or xtensor) into oracle/_ref/librandom_lcg_ref.so.
# Usage: oracle/build_ref.sh [reference_root]
# The reference tree comes from the argument, else OPENMC_REF_ROOT, else the
# read-only mount /root/reference of the build container.
set -e
REF=${1:-${OPENMC_REF_ROOT:-/root/reference}}
HERE=$(cd "$(dirname "$0")" && pwd)
if [ ! -f "$REF/src/random_lcg.cpp" ]; then
  echo "reference source not found at $REF; skipping" >&2
  exit 0
fi
mkdir -p "$HERE/_ref"
${CXX:-g++} -O2 -std=c++17 -fPIC -ffp-contract=off -shared \
  -I"$REF/include" "$REF/src/random_lcg.cpp" "$HERE/ref_rng_shim.cpp" \
  -o "$HERE/_ref/librandom_lcg_ref.so"
echo "built $HERE/_ref/librandom_lcg_ref.so"
