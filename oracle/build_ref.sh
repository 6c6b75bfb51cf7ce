#!/bin/sh
# Oracle test infrastructure: compile the reference's own src/random_lcg.cpp
# and src/random_dist.cpp (the hot-path sources of the reference that build
# without cmake, HDF5, pugixml, fmt or xtensor) into
# oracle/_ref/librandom_lcg_ref.so.  random_dist.cpp includes the generated
# header openmc/version.h; it is generated here from the reference's
# include/openmc/version.h.in the way its CMake configure step does.
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
mkdir -p "$HERE/_ref/include/openmc"
sed -e 's/@OPENMC_VERSION_MAJOR@/0/' -e 's/@OPENMC_VERSION_MINOR@/15/' -e 's/@OPENMC_VERSION_PATCH@/0/' \
    -e 's/@OPENMC_DEV_STATE@/true/' -e 's/@OPENMC_COMMIT_COUNT@//' -e 's/@OPENMC_COMMIT_HASH@//' \
    "$REF/include/openmc/version.h.in" > "$HERE/_ref/include/openmc/version.h"
${CXX:-g++} -O2 -std=c++17 -fPIC -ffp-contract=off -shared \
  -I"$REF/include" -I"$HERE/_ref/include" "$REF/src/random_lcg.cpp" "$REF/src/random_dist.cpp" \
  "$HERE/ref_rng_shim.cpp" -o "$HERE/_ref/librandom_lcg_ref.so"
echo "built $HERE/_ref/librandom_lcg_ref.so"
