#!/usr/bin/env bash
# Builds oracle/ref_harness.cpp against the unmodified Hydra headers into
# oracle/_ref/ (git-ignored).  Test infrastructure only: the binaries are the
# reference implementation, used to pin the C restatement and to make the
# golden fixtures.  Needs the Hydra source tree (HYDRA_SRC, default
# /root/reference); exits 0 without building when it is absent.
#
#   ref_harness_cpp : HYDRA_DEVICE_SYSTEM=CPP, sequential, -ffp-contract=off (parity build)
#   ref_harness_omp : HYDRA_DEVICE_SYSTEM=OMP, all host threads, -ffp-contract=off
set -euo pipefail
here="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
src="${HYDRA_SRC:-/root/reference}"
out="$here/_ref"
if [ ! -f "$src/hydra/PhaseSpace.h" ]; then
    echo "build_ref.sh: Hydra sources not found at $src; skipping reference build"
    exit 0
fi
mkdir -p "$out"
if [ "$out/ref_harness_cpp" -nt "$here/ref_harness.cpp" ] && [ "$out/ref_harness_omp" -nt "$here/ref_harness.cpp" ]; then
    echo "build_ref.sh: $out up to date"
    exit 0
fi
common=(-std=c++17 -O2 -ffp-contract=off -fno-fast-math -w -I"$src" -DHYDRA_HOST_SYSTEM=CPP)
g++ "${common[@]}" -DHYDRA_DEVICE_SYSTEM=CPP "$here/ref_harness.cpp" -o "$out/ref_harness_cpp" &
g++ "${common[@]}" -fopenmp -DHYDRA_DEVICE_SYSTEM=OMP "$here/ref_harness.cpp" -o "$out/ref_harness_omp" &
wait -n && wait -n
echo "build_ref.sh: built $out/ref_harness_cpp $out/ref_harness_omp"
