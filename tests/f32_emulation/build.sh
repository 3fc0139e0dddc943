#!/bin/bash
# Builds tests/f32_emulation/_build/emulate_f32: the FP32_FIX event body compiled for the host.
# The event headers are copied into _build/src with the two inline-asm hardware approximations
# (rcp.approx, rsqrt.approx) replaced by the IEEE operations they approximate; nothing else changes.
set -euo pipefail
here=$(cd "$(dirname "$0")" && pwd)
repo=$(cd "$here/../.." && pwd)
out=$here/_build
src=$out/src
mkdir -p "$src/hydra_gb300/csrc" "$src/include"
cp "$repo/include/hps.h" "$src/include/"
for f in genbod_f32.cuh genbod.cuh rng.cuh common.h; do cp "$repo/hydra_gb300/csrc/$f" "$src/hydra_gb300/csrc/"; done
g=$src/hydra_gb300/csrc/genbod_f32.cuh
sed -i 's|asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(b));|r = 1.0f / b;|' "$g"
sed -i 's|asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));|r = 1.0f / std::sqrt(x);|' "$g"
if grep -q 'asm(' "$g"; then echo "build.sh: inline asm left in genbod_f32.cuh" >&2; exit 1; fi
${CXX:-g++} -std=c++17 -O2 -fopenmp -ffp-contract=off -I "$here" -I "$src" -o "$out/emulate_f32" "$here/emulate_f32.cpp"
echo "$out/emulate_f32"
