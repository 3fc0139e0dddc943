#!/usr/bin/env bash
# Builds oracle/ref_harness.cpp against the unmodified Hydra headers into
# oracle/_ref/ (git-ignored).  Test infrastructure only: the binaries are the
# reference implementation, used to pin the C restatement, to make the golden
# fixtures, and as the timed CPU baseline of bench.py --impl reference.
#
# Hydra source tree: $HYDRA_SRC, else a `reference` checkout beside this
# repository.  Where it is present, the headers ref_harness.cpp can reach (every
# #include followed, oracle/stage_ref_headers.py) are also staged into
# oracle/_ref/src/ -- a build input kept out of git like the binaries -- so that the harness can be rebuilt on a machine
# that has the staged copy but not the source tree (the GPU host: binaries built
# here are x86 and do not run there).  With neither, it exits 0 without building.
#
#   ref_harness_cpp : HYDRA_DEVICE_SYSTEM=CPP, sequential, -ffp-contract=off (parity build)
#   ref_harness_omp : HYDRA_DEVICE_SYSTEM=OMP, all host threads, -ffp-contract=off
#   ref_gpu.cubin   : the reference's DecayMother / AverageMother device code for sm_103a
#                     (oracle/ref_gpu.cu, the reference build's nvcc flags); loaded by
#                     oracle/ref_gpu.py on a GPU host (only built where the full tree is)
set -euo pipefail
here="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
out="$here/_ref"
staged="$out/src"
src="${HYDRA_SRC:-$here/../../reference}"
common_defs=(-DHYDRA_HOST_SYSTEM=CPP)
if [ -f "$src/hydra/PhaseSpace.h" ]; then
    src="$(cd "$src" && pwd)"
    full=1
elif [ -f "$staged/hydra/PhaseSpace.h" ]; then
    src="$staged"
    full=0
else
    echo "build_ref.sh: no Hydra source tree (HYDRA_SRC) and no staged copy; skipping reference build"
    exit 0
fi
mkdir -p "$out"
# the machine's own g++ builds the host binaries: a binary built on another architecture is removed
# first (the stamp records where the binaries were built)
stamp="$out/.arch"
arch="$(uname -m)"
if [ -f "$stamp" ] && [ "$(cat "$stamp")" != "$arch" ]; then
    rm -f "$out/ref_harness_cpp" "$out/ref_harness_omp"
fi
echo "$arch" > "$stamp"

if [ "$full" = 1 ]; then
    # stage the headers the harness includes, for machines without the tree
    if ! [ "$staged/.complete" -nt "$here/ref_harness.cpp" ]; then
        rm -rf "$staged"
        mkdir -p "$staged"
        for sys in CPP OMP; do
            g++ -std=c++17 -M -w -I"$src" "${common_defs[@]}" -DHYDRA_DEVICE_SYSTEM=$sys -fopenmp \
                "$here/ref_harness.cpp" -MF "$staged/.deps_$sys"
        done
        python3 "$here/stage_ref_headers.py" "$src" "$staged" "$here/ref_harness.cpp" "$staged"/.deps_*
        rm -f "$staged"/.deps_*
        touch "$staged/.complete"
    fi
fi

nvcc="${NVCC:-$(command -v nvcc || echo /usr/local/cuda/bin/nvcc)}"
pids=()
common=(-std=c++17 -O2 -ffp-contract=off -fno-fast-math -w -I"$src" "${common_defs[@]}")
if ! [ "$out/ref_harness_cpp" -nt "$here/ref_harness.cpp" ]; then
    g++ "${common[@]}" -DHYDRA_DEVICE_SYSTEM=CPP "$here/ref_harness.cpp" -o "$out/ref_harness_cpp" & pids+=($!)
fi
if ! [ "$out/ref_harness_omp" -nt "$here/ref_harness.cpp" ]; then
    g++ "${common[@]}" -fopenmp -DHYDRA_DEVICE_SYSTEM=OMP "$here/ref_harness.cpp" -o "$out/ref_harness_omp" & pids+=($!)
fi
if [ "$full" = 1 ] && ! [ "$out/ref_gpu.cubin" -nt "$here/ref_gpu.cu" ]; then
    "$nvcc" -std=c++20 -O3 --extended-lambda --expt-relaxed-constexpr -w -gencode arch=compute_103a,code=sm_103a \
        -I"$src" -DHYDRA_HOST_SYSTEM=CPP -DHYDRA_DEVICE_SYSTEM=CUDA -cubin "$here/ref_gpu.cu" \
        -o "$out/ref_gpu.cubin" & pids+=($!)
fi
for p in "${pids[@]}"; do wait "$p"; done
echo "build_ref.sh: $out up to date (ref_harness_cpp, ref_harness_omp$([ "$full" = 1 ] && echo ", ref_gpu.cubin"); headers from $([ "$full" = 1 ] && echo "the source tree" || echo "the staged copy"))"
