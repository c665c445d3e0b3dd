#!/usr/bin/env bash
# Builds the reference GFAz CPU CLI from its own sources, where they lie, into
# oracle/_ref/gfaz.  Test infrastructure only: the reference binary is the pin
# for the oracle restatement and the generator of the golden fixtures under
# tests/golden/.  Nothing in the product links or runs it.
#
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]
#   REFERENCE_ROOT defaults to $GFAZ_REFERENCE_ROOT.  Without either, the
#   script looks in the one place the reference checkout is mounted on the
#   build container (below); when no sources are found it builds nothing and
#   exits 3, which callers treat as "skipped".
#
# The reference normally builds with CMake against a zstd submodule; here the
# 18 CPU core sources (CMakeLists.txt:128-147) and the CLI sources are
# compiled directly with g++/OpenMP.  Two shims from oracle/ref_shim/ stand in
# for what the image lacks:
#   * zstd.h      - declarations of the public zstd calls; linked against the
#                   system runtime libzstd.so.1 (no headers in the image).
#   * cli_fix.hpp - force-included into decompress_command.cpp, which names a
#                   GPU-only constant outside its ENABLE_CUDA guard.
set -euo pipefail
REF=${1:-${GFAZ_REFERENCE_ROOT:-/root/reference}}
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
OBJ="$OUT/obj"
mkdir -p "$OBJ"

if [ ! -d "$REF/src" ]; then
  echo "reference sources not found at $REF" >&2
  exit 3
fi

ZSTD_LIB=""
for cand in /usr/lib/x86_64-linux-gnu/libzstd.so.1 /usr/lib/aarch64-linux-gnu/libzstd.so.1 \
            /usr/lib64/libzstd.so.1 /lib/x86_64-linux-gnu/libzstd.so.1; do
  if [ -e "$cand" ]; then ZSTD_LIB="$cand"; break; fi
done
if [ -z "$ZSTD_LIB" ]; then
  echo "libzstd.so.1 not found" >&2
  exit 1
fi

CORE="src/io/gfa_parser.cpp src/grammar/rule_generator.cpp src/grammar/path_encoder.cpp
src/grammar/rule_processor.cpp src/workflows/add_haplotypes_workflow.cpp
src/workflows/extraction_workflow.cpp src/workflows/compression_workflow.cpp
src/workflows/compression_debug.cpp src/workflows/decompression_workflow.cpp
src/workflows/decompression_debug.cpp src/workflows/growth_workflow.cpp
src/workflows/pav_workflow.cpp src/utils/runtime_utils.cpp src/codec/codec.cpp
src/codec/serialization.cpp src/io/gfa_writer.cpp src/io/gfa_write_utils.cpp
src/workflows/compression_utils.cpp"
CLI="src/cli/gfaz_cli.cpp src/cli/common.cpp src/cli/compress_command.cpp
src/cli/decompress_command.cpp src/cli/extract_path_command.cpp
src/cli/extract_walk_command.cpp src/cli/add_haplotypes_command.cpp
src/cli/growth_command.cpp src/cli/pav_command.cpp"

CXXFLAGS="-std=c++17 -O2 -fopenmp -w -I$REF/include -I$REF/extern/robin_hood -I$HERE/ref_shim"
pids=()
objs=()
for src in $CORE $CLI; do
  o="$OBJ/$(echo "$src" | tr '/' '_').o"
  objs+=("$o")
  extra=""
  if [ "$src" = "src/cli/decompress_command.cpp" ]; then
    extra="-include $HERE/ref_shim/cli_fix.hpp"
  fi
  if [ ! -e "$o" ] || [ "$REF/$src" -nt "$o" ]; then
    g++ $CXXFLAGS $extra -c "$REF/$src" -o "$o" &
    pids+=($!)
  fi
done
for p in "${pids[@]}"; do wait "$p"; done
g++ -fopenmp -o "$OUT/gfaz" "${objs[@]}" "$ZSTD_LIB"
echo "built $OUT/gfaz (zstd: $ZSTD_LIB)"
