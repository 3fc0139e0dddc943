"""The FP64 oracle (the reference's arithmetic) against the same events in 50-digit arithmetic.

The reference draws its uniforms as double(word) / 2^64 and then works in IEEE double.  On a
stage near threshold, a - b - c cancels: the FP64 weight of such an event is off by far more than
1e-15.  These tests measure that on ordinary events and on events 21689203-21689204 of the
ten-pion channel (M = 5.0, Philox seed 0x3039), whose stage gap is 5e-11 GeV, so that the FP32_FIX
comparisons against the FP64 oracle can be read correctly.  CPU only; needs mpmath.
"""
from __future__ import annotations

import numpy as np
import pytest

mp = pytest.importorskip("mpmath")

PI_D = 3.1415926535897932384626422832795028841971   # the reference's PI, a double literal


def exact_event(words, masses, ch):
    """DecayMother's event (DecayMother.h:163-277) in 50-digit arithmetic from the reference's
    own double uniforms and double constants."""
    mp.mp.dps = 50
    N = len(masses)
    m = [mp.mpf(float(x)) for x in masses]
    u = [mp.mpf(float(int(w))) / mp.mpf(2) ** 64 for w in words]
    rno = [mp.mpf(0)] + sorted(u[:N - 2]) + [mp.mpf(1)]
    ecm = mp.mpf(ch.ecm)
    inv, s = [], mp.mpf(0)
    for n in range(N):
        s += m[n]
        inv.append(rno[n] * ecm + s)

    def pdk(a, b, c):
        return mp.sqrt((a - b - c) * (a + b + c) * (a - b + c) * (a + b - c)) / (2 * a)
    pd = [pdk(inv[n + 1], inv[n], m[n + 1]) for n in range(N - 1)]
    wt = mp.mpf(ch.max_weight)
    for x in pd:
        wt *= x
    p = [[mp.sqrt(pd[0] ** 2 + m[0] ** 2), mp.mpf(0), pd[0], mp.mpf(0)]]
    for i in range(1, N):
        p.append([mp.sqrt(pd[i - 1] ** 2 + m[i] ** 2), mp.mpf(0), -pd[i - 1], mp.mpf(0)])
        cz = 2 * u[N - 2 + 2 * (i - 1)] - 1
        sz = mp.sqrt(1 - cz * cz)
        ang = mp.mpf(2.0 * PI_D * float(u[N - 2 + 2 * (i - 1) + 1]))
        cy, sy = mp.cos(ang), mp.sin(ang)
        for j in range(i + 1):
            x, y, z = p[j][1], p[j][2], p[j][3]
            x1 = cz * x - sz * y
            p[j][2] = sz * x + cz * y
            p[j][1] = cy * x1 - sy * z
            p[j][3] = sy * x1 + cy * z
        if i == N - 1:
            break
        beta = pd[i] / mp.sqrt(pd[i] ** 2 + inv[i] ** 2)
        g = 1 / mp.sqrt(1 - beta * beta)
        for j in range(i + 1):
            e, py = p[j][0], p[j][2]
            p[j][0] = g * (e + beta * py)
            p[j][2] = g * (py + beta * e)
    gap = min(inv[n + 1] - inv[n] - m[n + 1] for n in range(N - 1))
    return wt, np.array([[float(c) for c in v] for v in p]), float(gap)


def fp64_errors(oracle, masses, M, seed, evt):
    ch = oracle.make_channel(masses, M, seed, oracle.ENGINE_PHILOX)
    four, w = oracle.generate(ch, evt, 1)
    words = oracle.rng_words(len(masses), oracle.ENGINE_PHILOX, seed, evt, 1)[0]
    wt, ex, gap = exact_event(words, masses, ch)
    ew = float(abs((mp.mpf(float(w[0])) - wt) / wt))
    e4 = float((np.abs(four[:, 0] - ex).max(axis=1) / ex[:, 0]).max())
    return ew, e4, gap


def test_fp64_oracle_is_exact_to_1e13_on_ordinary_events(oracle):
    for evt in (0, 1, 12345, 999_999):
        ew, e4, gap = fp64_errors(oracle, [0.13957] * 10, 5.0, 0x3039, evt)
        assert gap > 1e-3
        assert ew < 1e-13 and e4 < 1e-13, (evt, ew, e4)


def test_fp64_oracle_cancels_near_threshold(oracle):
    """Events 21689203 and 21689204 share two uniforms 1.4e-11 apart: the stage between them is
    5e-11 GeV above threshold and the FP64 weight is off by about 2.5e-7."""
    for evt in (21689203, 21689204):
        ew, e4, gap = fp64_errors(oracle, [0.13957] * 10, 5.0, 0x3039, evt)
        assert gap < 1e-10
        assert 1e-7 < ew < 1e-6, ew
        assert e4 < 1e-10
