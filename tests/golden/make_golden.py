"""Regenerates the golden fixtures in this directory from the REFERENCE itself.

Runs oracle/_ref/ref_harness_cpp (Hydra's own PhaseSpace / Decays / engines,
built by oracle/build_ref.sh with the sequential cpp backend and
-ffp-contract=off) on small seeded cases and stores its outputs as .npz.
Needs the Hydra source tree, so it runs only where that tree exists; the
fixtures it writes are committed and read by tests/test_oracle_golden.py and
tests/test_gpu_parity.py.

    python tests/golden/make_golden.py [NAME_PREFIX]
"""
from __future__ import annotations

import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
REF = REPO / "oracle" / "_ref" / "ref_harness_cpp"
UNWEIGHT_SEED = 0x180EC6D33CFD0ABA   # hydra/Decays.h:253 default

PI = 0.13957
K = 0.493677
# (name, N, engine, seed, n, M, masses, functor(sel,i,j,a,b), mother momentum)
GEN_CASES = [
    ("b0_jpsikpi_n3_philox", 3, 0, 0x3039, 256, 5.27934, [3.0969, K, PI], (1, 0, 1, 0.0, 0.0), (0, 0, 0)),
    ("d0_kpipipipi_n5_philox", 5, 0, 0x3039, 256, 1.86484, [K, PI, PI, PI, PI], (2, 0, 1, 0.8955, 0.0473),
     (0, 0, 0)),
    ("pions_n10_philox", 10, 0, 0x3039, 128, 5.0, [PI] * 10, (2, 0, 1, 0.8955, 0.0473), (0, 0, 0)),
    ("n2_philox", 2, 0, 7, 64, 1.0, [0.2, 0.3], (1, 0, 1, 0.0, 0.0), (0, 0, 0)),
    ("n4_squares3", 4, 1, 12345, 128, 3.0, [0.1, 0.2, 0.3, 0.4], (1, 1, 3, 0.0, 0.0), (0, 0, 0)),
    ("n7_squares3", 7, 1, 99, 96, 4.0, [PI] * 4 + [K, 0.938272, PI], (2, 2, 5, 1.0, 0.1), (0, 0, 0)),
    ("n6_philox_moving", 6, 0, 2024, 64, 3.5, [PI, K, PI, K, PI, 0.2], (1, 0, 5, 0.0, 0.0),
     (0.3, -1.2, 0.7)),
    ("n3_philox_defaultseed", 3, 0, -1, 64, 5.27934, [3.0969, K, PI], (0, 0, 1, 0.0, 0.0), (0, 0, 0)),
    ("n8_philox_threshold", 8, 0, 31337, 128, 8 * PI + 0.01, [PI] * 8, (1, 0, 7, 0.0, 0.0), (0, 0, 0)),
]
# (name, N, engine, seed, n)
RNG_CASES = [
    ("rng_n3_philox", 3, 0, 0x3039, 64),
    ("rng_n5_philox", 5, 0, 0x3039, 64),
    ("rng_n10_philox", 10, 0, 0xDEADBEEFCAFEF00D, 48),
    ("rng_n5_squares3", 5, 1, 0x3039, 64),
    ("rng_n2_squares3", 2, 1, 1, 16),
]
# (name, N, engine, seed, n, M, masses, functor)
AVG_CASES = [
    ("avg_b0_jpsikpi_m2", 3, 0, 0x3039, 20000, 5.27934, [3.0969, K, PI], (1, 0, 1, 0.0, 0.0)),
    ("avg_d0_kpipipipi_bw", 5, 0, 0x3039, 20000, 1.86484, [K, PI, PI, PI, PI], (2, 0, 1, 0.8955, 0.0473)),
    ("avg_n10_bw", 10, 0, 0x3039, 5000, 5.0, [PI] * 10, (2, 0, 1, 0.8955, 0.0473)),
    ("avg_n4_sq_one", 4, 1, 12345, 5000, 3.0, [0.1, 0.2, 0.3, 0.4], (0, 0, 1, 0.0, 0.0)),
]


# Consumers of a stored sample and the lazy generator (ref_harness "extras"):
# (name, N, engine, seed, n, M, masses, functor, fixed max weight for Unweight(functor, w), grid,
#  phase_space_range seed, range mother momentum)
FUNCTOR_UNWEIGHT_SEED = 0x39ABDC4529B1661C   # hydra/Decays.h:261 default
EXTRA_CASES = [
    ("extras_b0_jpsikpi_n3_philox", 3, 0, 0x3039, 1024, 5.27934, [3.0969, K, PI], (2, 1, 2, 0.8955, 0.0473), 50.0,
     (20, 25), 321, (0.1, -0.2, 0.3)),
    ("extras_n5_squares3", 5, 1, 777, 512, 1.86484, [K, PI, PI, PI, PI], (1, 0, 1, 0.0, 0.0), 0.2,
     (16, 12), 0xFFFFFFFF00000005, (0.0, 0.0, 0.0)),
    ("extras_n2_philox", 2, 0, 5, 128, 3.0969, [0.10566, 0.10566], (0, 0, 1, 0.0, 0.0), 0.9,
     (4, 4), 0, (0.5, 0.2, -1.0)),
    ("extras_n10_philox", 10, 0, 0x3039, 128, 5.0, [PI] * 10, (2, 0, 1, 0.8955, 0.0473), 1e-6,
     (10, 10), 2147483647, (0.0, 0.0, 0.0)),
]


# Functors written as the reference's phase-space examples write them (ref_harness "functors"):
# cos(theta_K) by hydra::CosHelicityAngle inside a wrap_lambda over declarg arguments, m13^2, m23^2;
# (name, engine, seed, n, M, masses)
FUNCTOR_CASES = [
    ("functors_b0_jpsikpi", 0, 0x3039, 1024, 5.27955, [3.0969, K, 0.13957061]),
    ("functors_b0_jpsikpi_sq", 1, 777, 512, 5.27955, [3.0969, K, 0.13957061]),
]


def dalitz_limits(M, m):
    """Kinematic limits of (m2(p0+p1), m2(p1+p2)), the example's histogram range."""
    rest01 = sum(m[2:])
    rest12 = m[0] + sum(m[3:])
    lo = ((m[0] + m[1]) ** 2, (m[1] + m[2]) ** 2)
    hi = ((M - rest01) ** 2, (M - rest12) ** 2)
    return lo, hi


# (name, N, engine, seed, n, M, masses, functor over (mother, daughters...))
MOTHER_CASES = [
    ("mothers_n3_philox", 3, 0, 12345, 96, 5.27934, [3.0969, K, PI], (1, 0, 2, 0.0, 0.0)),
    ("mothers_n5_squares3", 5, 1, 777, 64, 1.86484, [K, PI, PI, PI, PI], (2, 1, 2, 0.8955, 0.0473)),
    ("mothers_n2_philox", 2, 0, 3, 64, 3.0969, [0.10566, 0.10566], (1, 1, 2, 0.0, 0.0)),
]


def run(args, out):
    subprocess.run([str(REF)] + [str(a) for a in args] + [str(out)], check=True)
    return out


def fnum(x):
    return repr(float(x))


def main():
    if not REF.exists():
        sys.exit(f"{REF} missing: run oracle/build_ref.sh first")
    only = sys.argv[1] if len(sys.argv) > 1 else ""      # name prefix: regenerate only those
    tmp = HERE / "_tmp.bin"
    fixtures = {}
    for name, eng, seed, n, M, m in FUNCTOR_CASES:
        if not name.startswith(only):
            continue
        args = ["functors", 3, eng, seed, n, fnum(M)] + [fnum(x) for x in m] + \
               [0, 0, 1, fnum(0.0), fnum(0.0), hex(FUNCTOR_UNWEIGHT_SEED)]
        d = np.fromfile(run(args, tmp), dtype=np.float64)
        rows = d[2:2 + 4 * n].reshape(n, 4)
        o = 2 + 4 * n
        fixtures[name] = dict(N=3, engine=eng, seed=seed, n=n, M=M, masses=np.array(m),
                              fseed=np.uint64(FUNCTOR_UNWEIGHT_SEED), avg_mean=d[0], avg_err=d[1],
                              eval_w=rows[:, 0].copy(), eval_m13=rows[:, 1].copy(), eval_m23=rows[:, 2].copy(),
                              eval_cos=rows[:, 3].copy(),
                              unw_four=d[o:o + n * 12].reshape(n, 3, 4).transpose(1, 0, 2).copy(),
                              unw_kept=int(d[o + n * 12]))
        assert o + n * 12 + 1 == len(d), (name, len(d))
    for name, N, eng, seed, n, M, m, f, mom in GEN_CASES:
        if not name.startswith(only):
            continue
        args = ["gen", N, eng, seed, n, fnum(M)] + [fnum(x) for x in m] + \
               [f[0], f[1], f[2], fnum(f[3]), fnum(f[4]), hex(UNWEIGHT_SEED)] + [fnum(x) for x in mom]
        d = np.fromfile(run(args, tmp), dtype=np.float64)
        o = n * N * 4
        E = float(np.sqrt(M * M + sum(x * x for x in mom)))
        fixtures[name] = dict(
            N=N, engine=eng, seed=seed, n=n, M=M, masses=np.array(m), functor=np.array(f),
            mother=np.array([E, *mom]), useed=np.uint64(UNWEIGHT_SEED),
            four=d[:o].reshape(n, N, 4).transpose(1, 0, 2).copy(),
            w_gen=d[o:o + n], f_val=d[o + n:o + 2 * n], w_rec=d[o + 2 * n:o + 3 * n],
            flags=d[o + 3 * n:o + 4 * n].astype(np.uint8),
            max_weight=d[o + 4 * n], decays_max_weight=d[o + 4 * n + 1], ecm=d[o + 4 * n + 2],
            get_seed=d[o + 4 * n + 3], n_unweighted=d[o + 4 * n + 4],
            default_seed=d[o + 4 * n + 5:o + 4 * n + 6].view(np.uint64)[0])
    for name, N, eng, seed, n in RNG_CASES:
        if not name.startswith(only):
            continue
        d = np.fromfile(run(["rng", N, eng, seed, n], tmp), dtype=np.uint64)
        fixtures[name] = dict(N=N, engine=eng, seed=np.uint64(seed), n=n, words=d.reshape(n, 3 * N - 4))
    for name, N, eng, seed, n, M, m, f in AVG_CASES:
        if not name.startswith(only):
            continue
        args = ["avg", N, eng, seed, n, fnum(M)] + [fnum(x) for x in m] + \
               [f[0], f[1], f[2], fnum(f[3]), fnum(f[4])]
        d = np.fromfile(run(args, tmp), dtype=np.float64)
        fixtures[name] = dict(N=N, engine=eng, seed=seed, n=n, M=M, masses=np.array(m),
                              functor=np.array(f), mean=d[0], err=d[1])
    for name, N, eng, seed, n, M, m, f in MOTHER_CASES:
        if not name.startswith(only):
            continue
        args = ["mothers", N, eng, seed, n, fnum(M)] + [fnum(x) for x in m] + \
               [f[0], f[1], f[2], fnum(f[3]), fnum(f[4])]
        d = np.fromfile(run(args, tmp), dtype=np.float64)
        o = n * 4
        fx = dict(N=N, engine=eng, seed=seed, n=n, M=M, masses=np.array(m), functor=np.array(f),
                  mothers=d[:o].reshape(n, 4))
        fx["four"] = d[o:o + n * N * 4].reshape(n, N, 4).transpose(1, 0, 2).copy()
        o += n * N * 4
        fx["eval_w"], fx["eval_f"] = d[o:o + n], d[o + n:o + 2 * n]
        fx["avg_mean"], fx["avg_err"] = d[o + 2 * n], d[o + 2 * n + 1]
        fixtures[name] = fx
    for name, N, eng, seed, n, M, m, f, fmax, grid, rseed, mom in EXTRA_CASES:
        if not name.startswith(only):
            continue
        if N >= 3:
            lo, hi = dalitz_limits(M, m)
        else:
            lo, hi = (0.0, 0.0), (1.0, 1.0)
        args = ["extras", N, eng, seed, n, fnum(M)] + [fnum(x) for x in m] + \
               [f[0], f[1], f[2], fnum(f[3]), fnum(f[4]), hex(FUNCTOR_UNWEIGHT_SEED), fnum(fmax),
                grid[0], grid[1], fnum(lo[0]), fnum(lo[1]), fnum(hi[0]), fnum(hi[1]), rseed] + [fnum(x) for x in mom]
        d = np.fromfile(run(args, tmp), dtype=np.float64)
        E = float(np.sqrt(M * M + sum(x * x for x in mom)))
        fx = dict(N=N, engine=eng, seed=seed, n=n, M=M, masses=np.array(m), functor=np.array(f),
                  fseed=np.uint64(FUNCTOR_UNWEIGHT_SEED), fmax=fmax, grid=np.array(grid, dtype=np.uint64),
                  lower=np.array(lo), upper=np.array(hi), rseed=np.uint64(rseed), range_mother=np.array([E, *mom]))
        nf = n * N * 4
        o = 0

        def four_at(o):
            return d[o:o + nf].reshape(n, N, 4).transpose(1, 0, 2).copy()
        fx["four"] = four_at(o); o += nf
        fx["reweight"] = d[o:o + n]; o += n
        fx["unw_max_four"] = four_at(o); o += nf
        fx["unw_max_kept"] = int(d[o]); o += 1
        fx["unw_fixed_four"] = four_at(o); o += nf
        fx["unw_fixed_kept"] = int(d[o]); o += 1
        if N >= 3:
            nb = grid[0] * grid[1] + 2
            fx["hist"] = d[o:o + nb]; o += nb
        r = d[o:o + n * (1 + 4 * N)].reshape(n, 1 + 4 * N); o += n * (1 + 4 * N)
        fx["range_w"] = r[:, 0].copy()
        fx["range_four"] = r[:, 1:].reshape(n, N, 4).transpose(1, 0, 2).copy()
        fx["integ_mean"], fx["integ_err"] = d[o], d[o + 1]
        fx["integ_seed"] = d[o + 2:o + 3].view(np.uint64)[0]
        assert o + 3 == len(d), (name, o, len(d))
        fixtures[name] = fx
    tmp.unlink()
    for name, fx in fixtures.items():
        np.savez_compressed(HERE / f"{name}.npz", **fx)
    print(f"wrote {len(fixtures)} fixtures to {HERE}")


if __name__ == "__main__":
    main()
