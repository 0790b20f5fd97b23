#!/usr/bin/env bash
# Builds the reference PyNear extension (_pynear) from its own sources, in place
# under the read-only reference checkout, into oracle/_ref/.  Used only to pin the
# oracle and to generate golden fixtures; nothing shipped links it.
#
#   PYNEAR_REFERENCE=<path of the PyNear 2.2.0 source tree> bash oracle/build_ref.sh
#
# Needs g++, OpenMP and pybind11 headers (present in the x86 build container,
# absent on the GPU host, where this script is a no-op).
set -euo pipefail
REF="${PYNEAR_REFERENCE:-}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ -z "$REF" ]; then
  echo "build_ref: PYNEAR_REFERENCE is not set; skipping" >&2
  exit 0
fi
if [ ! -d "$REF/pynear/include" ]; then
  echo "build_ref: no reference tree at $REF; skipping" >&2
  exit 0
fi
if ! python3 -c "import pybind11" 2>/dev/null; then
  echo "build_ref: pybind11 not importable; skipping" >&2
  exit 0
fi
mkdir -p "$OUT"
SUFFIX="$(python3-config --extension-suffix)"
TARGET="$OUT/_pynear$SUFFIX"
if [ -f "$TARGET" ] && [ "$TARGET" -nt "$REF/pynear/src/PythonBindings.cpp" ]; then
  exit 0
fi
ARCHFLAGS="-march=native -mavx"
case "$(uname -m)" in
  aarch64|arm64) ARCHFLAGS="-mcpu=native" ;;
esac
# Same flags the reference's setup.py passes (setup.py:67-74), minus -flto/-Wall.
g++ -O3 -std=c++17 -shared -fPIC $ARCHFLAGS -fopenmp -DENABLE_OMP_PARALLEL=1 \
    -I"$REF/pynear/include" $(python3 -m pybind11 --includes) \
    "$REF/pynear/src/PythonBindings.cpp" -o "$TARGET.tmp" -lgomp
mv "$TARGET.tmp" "$TARGET"
echo "build_ref: built $TARGET"
