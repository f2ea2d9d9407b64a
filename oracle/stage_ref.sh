#!/bin/sh
# Test infrastructure: stages the files of the reference tree (tay10r/lbvh)
# that oracle/_ref/libref.so and the C++ header test compile from into
# baseline/_ref/ (git-ignored, never committed), so that a machine without
# the reference checkout -- the GPU host -- can compile the UNMODIFIED
# reference there and time it as the CPU baseline.
#
#   sh oracle/stage_ref.sh [SRC]     # SRC defaults to $LBVH_REF_SRC, then /root/reference
#
# A missing SRC is not an error (nothing to stage; an existing stage is kept).
# The reference is a header-only C++ library with no Python packaging, so
# `pip install --target baseline/_ref` cannot install it; this copy is the
# install step.
set -eu
SRC=${1:-${LBVH_REF_SRC:-/root/reference}}
HERE=$(cd "$(dirname "$0")" && pwd)
DST="$HERE/../baseline/_ref"
if [ ! -f "$SRC/lbvh.h" ]; then
    exit 0
fi
mkdir -p "$DST/third-party" "$DST/models"
for f in lbvh.h LICENSE third-party/tiny_obj_loader.h third-party/tiny_obj_loader.cc \
         models/monkey.obj models/teapot.obj; do
    if [ -f "$SRC/$f" ]; then
        if [ ! -f "$DST/$f" ] || ! cmp -s "$SRC/$f" "$DST/$f"; then
            rm -f "$DST/$f"
            cp "$SRC/$f" "$DST/$f"
            chmod u+w "$DST/$f"
        fi
    fi
done
