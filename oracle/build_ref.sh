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
# The reference uses x86 intrinsics (_pdep_u32, _lzcnt_u32, SSE/AVX2 and
# GCC's x86 move-mask builtins).  On an x86-64 host they are the compiler's
# own.  On any other host (the arm64 Grace host of a GB300) the sources are
# compiled unmodified against oracle/x86compat/immintrin.h, a portable
# restatement of those operations, which is put first on the include path
# and force-included.  On x86-64 one more variant is built that way:
#   libseqref_x8.so   as b8, but through the portable intrinsics, so the
#                     tests can check them against the x86 builds' golden
#                     outputs
# The reference's sources exist only where its checkout is; a host without
# them (a GPU machine the repository is copied to) builds nothing here.
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
src="${SEQUOIA_REF_SRC:-/root/reference/src}"
out="$here/_ref"
if [ ! -f "$src/builder.cpp" ]; then
  echo "build_ref: reference sources not found at $src; skipping" >&2
  exit 0
fi
mkdir -p "$out"
compat="-I$here/x86compat -include $here/x86compat/immintrin.h"
case "$(uname -m)" in
  x86_64) native="-march=native"; arch_flags="" ;;
  aarch64 | arm64) native="-mcpu=native"; arch_flags="$compat" ;;
  *) native=""; arch_flags="$compat" ;;
esac
base="-std=c++17 $native -fopenmp -O3 -fPIC -w"

build_variant() {
  local name="$1" bins="$2" fp="$3" extra="${4:-$arch_flags}" cpu="${5:-$base}"
  local dir="$out/obj_$name"
  mkdir -p "$dir"
  local flags="$cpu $fp $extra -I$src"
  rm -f "$dir"/*.o "$out/libseqref_$name.so"
  local pids=()
  sed -e "s/^#define NUM_BINS 8\r\{0,1\}$/#define NUM_BINS $bins/" "$src/builder.cpp" \
    | g++ $flags -x c++ -c - -o "$dir/builder.o" & pids+=($!)
  g++ $flags -c "$src/tracer.cpp" -o "$dir/tracer.o" & pids+=($!)
  g++ $flags -c "$src/algorithms.cpp" -o "$dir/algorithms.o" & pids+=($!)
  g++ $flags -Dmain=sequoia_main -c "$src/main.cpp" -o "$dir/main.o" & pids+=($!)
  g++ $flags -c "$here/ref_shim.cpp" -o "$dir/ref_shim.o" & pids+=($!)
  local ok=1
  for p in "${pids[@]}"; do wait "$p" || ok=0; done
  if [ "$ok" != 1 ]; then
    echo "build_ref: variant $name failed to compile" >&2
    return 1
  fi
  g++ $cpu -shared -Wl,--no-undefined -o "$out/libseqref_$name.so" "$dir"/*.o
}

vpids=()
build_variant b8 8 "-ffp-contract=off" & vpids+=($!)
build_variant b16 16 "-ffp-contract=off" & vpids+=($!)
build_variant b32 32 "-ffp-contract=off" & vpids+=($!)
build_variant mk 8 "" & vpids+=($!)
if [ "$(uname -m)" = x86_64 ]; then
  build_variant x8 8 "-ffp-contract=off" "$compat" "-std=c++17 -fopenmp -O3 -fPIC -w" & vpids+=($!)
fi
status=0
for p in "${vpids[@]}"; do wait "$p" || status=1; done
[ "$status" = 0 ] || exit 1
ls "$out"/*.so
