#!/bin/sh
# Builds the reference's own serial FP64 solver (Pathlessbark8/C-_serial,
# header-only C++) from the sources where they lie, driven by
# oracle/ref_harness.cpp.  Output goes only to oracle/_ref/ (git-ignored).
# Test infrastructure: used to pin the C restatement and to write the golden
# fixtures; the product never runs it.  Skips quietly when the reference
# sources are not present (e.g. on a machine that only has this repository).
# This recipe is the one file that names where the reference checkout lies
# (QLSKUM_REFERENCE_DIR overrides it); it records the directory it built
# from in oracle/_ref/source_dir for the tests and the fixture script.
set -e
here=$(cd "$(dirname "$0")" && pwd)
ref=${QLSKUM_REFERENCE_DIR:-/root/reference}
if [ ! -f "$ref/q_lskum_mod.h" ]; then
    echo "build_ref: reference sources not found at $ref; skipped" >&2
    exit 0
fi
mkdir -p "$here/_ref"
# -ffp-contract=off: no FMA contraction, so the x86-64 and aarch64 builds
# evaluate every expression with the reference's own rounding sequence.
g++ -O2 -std=c++17 -ffp-contract=off -w -I"$ref" "$here/ref_harness.cpp" -o "$here/_ref/ref_harness"
printf '%s\n' "$ref" > "$here/_ref/source_dir"
echo "build_ref: built $here/_ref/ref_harness"
