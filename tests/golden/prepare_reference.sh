#!/usr/bin/env bash
# Copies the reference ops into the git-ignored baseline/_ref/ops and applies
# the one rename nvcc 13 needs: the reference's `namespace cuda` collides with
# libcu++'s `cuda::std`, so it becomes `namespace refcuda`.  Also copies the
# reference's corenet.py (TemperatureSoftmin, imported by the reference's own
# LBP wrapper modules) to baseline/_ref/.  Runs where the reference checkout
# is mounted; the copy then travels with the working tree to the GPU
# machine, where make_golden.py and the reference-op tests build and run it.
# The copy is never committed.
#
# Usage: tests/golden/prepare_reference.sh <reference checkout root>
set -euo pipefail
if [ $# -ne 1 ] || [ ! -d "$1/ops" ]; then
  echo "usage: $0 <reference checkout root (the directory holding ops/ and corenet.py)>" >&2
  exit 2
fi
SRC="$1/ops"
ROOT=$(cd "$(dirname "$0")/../.." && pwd)
DST="$ROOT/baseline/_ref/ops"
rm -rf "$DST"
mkdir -p "$DST"
cp -r "$SRC"/. "$DST"/
cp "$1/corenet.py" "$ROOT/baseline/_ref/corenet.py"
find "$DST" \( -name '*.cu' -o -name '*.cuh' -o -name '*.cpp' -o -name '*.h' \) -print0 |
  xargs -0 sed -i -e 's/namespace cuda$/namespace refcuda/' -e 's/namespace cuda /namespace refcuda /' -e 's/return cuda::/return refcuda::/'
grep -rn "namespace refcuda" "$DST" | wc -l
