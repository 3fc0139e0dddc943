#!/usr/bin/env bash
# Builds oracle/ref_harness.cpp against the unmodified Hydra headers into
# oracle/_ref/ (git-ignored).  Test infrastructure only: the binaries are the
# reference implementation, used to pin the C restatement and to make the
# golden fixtures.  Needs the Hydra source tree (HYDRA_SRC, default
# /root/reference); exits 0 without building when it is absent.
#
#   ref_harness_cpp : HYDRA_DEVICE_SYSTEM=CPP, sequential, -ffp-contract=off (parity build)
#   ref_harness_omp : HYDRA_DEVICE_SYSTEM=OMP, all host threads, -ffp-contract=off
#   ref_gpu.cubin   : the reference's DecayMother / AverageMother device code for sm_103a
#                     (oracle/ref_gpu.cu, the reference build's nvcc flags); loaded by
#                     oracle/ref_gpu.py on a GPU host, which needs no Hydra sources
set -euo pipefail
here="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
src="${HYDRA_SRC:-/root/reference}"
out="$here/_ref"
if [ ! -f "$src/hydra/PhaseSpace.h" ]; then
    echo "build_ref.sh: Hydra sources not found at $src; skipping reference build"
    exit 0
fi
mkdir -p "$out"
nvcc="${NVCC:-$(command -v nvcc || echo /usr/local/cuda/bin/nvcc)}"
pids=()
common=(-std=c++17 -O2 -ffp-contract=off -fno-fast-math -w -I"$src" -DHYDRA_HOST_SYSTEM=CPP)
if ! [ "$out/ref_harness_cpp" -nt "$here/ref_harness.cpp" ]; then
    g++ "${common[@]}" -DHYDRA_DEVICE_SYSTEM=CPP "$here/ref_harness.cpp" -o "$out/ref_harness_cpp" & pids+=($!)
fi
if ! [ "$out/ref_harness_omp" -nt "$here/ref_harness.cpp" ]; then
    g++ "${common[@]}" -fopenmp -DHYDRA_DEVICE_SYSTEM=OMP "$here/ref_harness.cpp" -o "$out/ref_harness_omp" & pids+=($!)
fi
if ! [ "$out/ref_gpu.cubin" -nt "$here/ref_gpu.cu" ]; then
    "$nvcc" -std=c++20 -O3 --extended-lambda --expt-relaxed-constexpr -w -gencode arch=compute_103a,code=sm_103a \
        -I"$src" -DHYDRA_HOST_SYSTEM=CPP -DHYDRA_DEVICE_SYSTEM=CUDA -cubin "$here/ref_gpu.cu" \
        -o "$out/ref_gpu.cubin" & pids+=($!)
fi
for p in "${pids[@]}"; do wait "$p"; done
echo "build_ref.sh: $out up to date (ref_harness_cpp, ref_harness_omp, ref_gpu.cubin)"
