"""Host-side layout of the kernel parameters oracle/ref_gpu.py passes to the reference's CUDA
functors (oracle/ref_gpu.cu checks the device side against the functors with static_asserts):
MotherArgs<N> = {size_t seed; double ecm, maxw, beta[3], masses[N]} and AvgArgs<N> =
{MotherArgs<N>; {int i, j; double a, b}}, as DecayMother.h:64-73 / AverageMother.h:60-70."""
from __future__ import annotations

import ctypes

import pytest

from oracle import ref_gpu


@pytest.mark.parametrize("n", range(2, 11))
def test_mother_args_layout(n):
    M = ref_gpu._mother_args(n)
    assert ctypes.sizeof(M) == 8 * (6 + n)
    assert M.ecm.offset == 8 and M.maxw.offset == 16 and M.beta.offset == 24 and M.masses.offset == 48

    A = ref_gpu._avg_args(n)
    a = A()
    a.m = M()                     # the cached classes are the same type on every call
    assert A.f.offset == 8 * (6 + n)
    assert ctypes.sizeof(A) == 8 * (6 + n) + 24
    assert ref_gpu._BW.a.offset == 8


def test_add_stats_matches_definition():
    # AddStatsPHSP: W = Wx + Wy, mean = (mx Wx + my Wy) / W, M2 = M2x + M2y + d^2 Wx Wy / W
    x, y = (2.0, 0.5, 3.0), (4.0, 0.25, 1.0)
    mean, m2, w = ref_gpu.add_stats(x, y)
    assert w == 4.0 and mean == (2.0 * 3.0 + 4.0 * 1.0) / 4.0
    assert m2 == 0.5 + 0.25 + 4.0 * 3.0 * 1.0 / 4.0


@pytest.mark.parametrize("n", range(2, 11))
def test_mothers_args_layout(n):
    # MothersArgs<N> = {size_t seed; double ecm, maxw, masses[N]} (DecayMothers.h:59-63)
    M = ref_gpu._mothers_args(n)
    assert ctypes.sizeof(M) == 8 * (3 + n)
    assert M.masses.offset == 24
