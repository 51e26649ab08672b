#!/usr/bin/env bash
# Build the Sequoia reference's own CPU code into oracle/_ref/ (test
# infrastructure only; outputs are git-ignored).
#
# Sources are read where they lie in a checkout of the reference: the
# directory named by SEQUOIA_REF_SRC (its src/ folder), else the read-only
# checkout this project was built beside, /root/reference/src.  They are
# never copied into this repository.  The only change made on the fly is the bin count:
# `#define NUM_BINS 8` (src/builder.cpp:11) is rewritten to 16 or 32 in a
# stream fed to the compiler, which is how the 16- and 32-bin SAH
# configurations of the reference are obtained.
#
# Variants (each a shared library with the same ref_* entry points):
#   libseqref_b8.so   NUM_BINS 8,  -ffp-contract=off (IEEE per operation)
#   libseqref_b16.so  NUM_BINS 16, -ffp-contract=off
#   libseqref_b32.so  NUM_BINS 32, -ffp-contract=off
#   libseqref_mk.so   NUM_BINS 8,  the reference makefile's own flags
#                     (-march=native, default FP contraction)
#
# The reference uses x86 intrinsics (_pdep_u32, _lzcnt_u32, SSE/AVX), so this
# builds on x86-64 only; elsewhere it exits 0 without building.
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
src="${SEQUOIA_REF_SRC:-/root/reference/src}"
out="$here/_ref"
if [ ! -f "$src/builder.cpp" ]; then
  echo "build_ref: reference sources not found at $src; skipping" >&2
  exit 0
fi
case "$(uname -m)" in
  x86_64) ;;
  *) echo "build_ref: reference needs x86-64 intrinsics; skipping on $(uname -m)" >&2; exit 0 ;;
esac
mkdir -p "$out"
base="-std=c++17 -march=native -fopenmp -O3 -fPIC -w"

build_variant() {
  local name="$1" bins="$2" fp="$3"
  local dir="$out/obj_$name"
  mkdir -p "$dir"
  local flags="$base $fp -I$src"
  sed -e "s/^#define NUM_BINS 8\r\{0,1\}$/#define NUM_BINS $bins/" "$src/builder.cpp" \
    | g++ $flags -x c++ -c - -o "$dir/builder.o" &
  g++ $flags -c "$src/tracer.cpp" -o "$dir/tracer.o" &
  g++ $flags -c "$src/algorithms.cpp" -o "$dir/algorithms.o" &
  g++ $flags -Dmain=sequoia_main -c "$src/main.cpp" -o "$dir/main.o" &
  g++ $flags -c "$here/ref_shim.cpp" -o "$dir/ref_shim.o" &
  wait
  g++ $base -shared -o "$out/libseqref_$name.so" "$dir"/*.o
}

build_variant b8 8 "-ffp-contract=off" &
build_variant b16 16 "-ffp-contract=off" &
build_variant b32 32 "-ffp-contract=off" &
build_variant mk 8 "" &
wait
ls "$out"/*.so
