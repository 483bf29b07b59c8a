#!/bin/sh
# Builds the parts of the reference (Serenity) that compile standalone, from the
# sources where they lie, into oracle/_ref/ (git-ignored). Only the Lebedev
# tables qualify: everything else on the XC path needs Eigen3, libint2, xcfun
# or libxc, none of which exist in this image.
#   oracle/_ref/lebedev_dump   prints the reference's Lebedev rules
# With --table it also regenerates serenity_gb300/data/lebedev.txt.
set -e
REF=${SERENITY_REFERENCE:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
if [ ! -f "$REF/src/grid/construction/sphere_lebedev_rule.cpp" ]; then
  echo "reference sources not present; nothing to build" >&2
  exit 0
fi
mkdir -p "$HERE/_ref"
g++ -O2 -std=c++14 -I"$REF/src" "$HERE/ref_lebedev_dump.cpp" \
    "$REF/src/grid/construction/sphere_lebedev_rule.cpp" -o "$HERE/_ref/lebedev_dump"
if [ "$1" = "--table" ]; then
  "$HERE/_ref/lebedev_dump" > "$HERE/../serenity_gb300/data/lebedev.txt"
fi
