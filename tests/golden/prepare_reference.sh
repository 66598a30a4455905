#!/usr/bin/env bash
# Copies the reference ops into the git-ignored baseline/_ref/ops and applies
# the one rename nvcc 13 needs: the reference's `namespace cuda` collides with
# libcu++'s `cuda::std`, so it becomes `namespace refcuda`.  Runs where the
# reference checkout is mounted; the copy then travels with the working tree
# to the GPU machine, where make_golden.py builds and runs it.  The copy is
# never committed.
set -euo pipefail
SRC=${1:-/root/reference/ops}
ROOT=$(cd "$(dirname "$0")/../.." && pwd)
DST="$ROOT/baseline/_ref/ops"
rm -rf "$DST"
mkdir -p "$DST"
cp -r "$SRC"/. "$DST"/
find "$DST" \( -name '*.cu' -o -name '*.cuh' -o -name '*.cpp' -o -name '*.h' \) -print0 |
  xargs -0 sed -i -e 's/namespace cuda$/namespace refcuda/' -e 's/namespace cuda /namespace refcuda /' -e 's/return cuda::/return refcuda::/'
grep -rn "namespace refcuda" "$DST" | wc -l
