#!/bin/sh
# Compiles libBICOS's own CPU backend, in place under the reference tree,
# against the project's minimal OpenCV/fmt stand-in (oracle/ref_shim) into
# oracle/_ref/libbicos_ref.so.  TEST INFRASTRUCTURE ONLY: the result is the
# checker that pins the oracle restatement and generates tests/golden/.
# Needs the reference sources at $BICOS_REF (default: a libBICOS tree named
# "reference" beside this repository's checkout); exits 0 without building
# when they are absent.
set -e
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${BICOS_REF:-$HERE/../../reference}"
if [ ! -f "$REF/src/impl/cpu.cpp" ]; then
    echo "ref_build: reference sources not found at $REF, skipping" >&2
    exit 0
fi
mkdir -p "$HERE/_ref"
# -O3 as the reference's release build (meson --buildtype release);
# -ffp-contract=off keeps a*x*x+b*x+c unfused on every host.
${CXX:-g++} -O3 -std=gnu++17 -ffp-contract=off -fPIC -shared -DBICOS_CPU \
    -I"$HERE/ref_shim" -I"$REF/include" -I"$HERE" \
    "$REF/src/impl/cpu.cpp" "$REF/src/exception.cpp" "$HERE/ref_capi.cpp" \
    -o "$HERE/_ref/libbicos_ref.so" -lpthread
echo "ref_build: built $HERE/_ref/libbicos_ref.so"
