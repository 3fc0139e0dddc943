// genbod.cuh -- per-event Raubold-Lynch (GENBOD) body, FP64 form.
//
// Restates hydra::detail::DecayMother<N,GRND>::process (hydra/detail/functors/DecayMother.h:163-277;
// AverageMother.h:156-270 and EvalMother.h:169-283 are the same body) for one event held in
// registers.  The FP64 form issues every double operation that can round as a separately
// rounded IEEE operation in the reference's order (__dadd_rn / __dmul_rn / __dsqrt_rn /
// __ddiv_rn, no FMA contraction), so invariant masses, pdk momenta, the event weight,
// energies, rotations and boosts round exactly as the reference built without FMA
// contraction.  The only operations whose last bit may differ are cos/sin of the azimuth
// (CUDA's sincos versus the host libm).
#pragma once
#include <cstdint>
#include "../../include/hps.h"
#include "rng.cuh"

namespace hps {

// Channel constants as the kernels see them (passed by value as a kernel parameter).
struct DevChannel {
    double masses[10];
    double ecm;
    double max_weight;
    double beta[3];       // final-boost vector (DecayMother.h:88-98)
    uint64_t key;         // splitmix64(seed): Philox key / squares3 key
    int boost_active;     // 0 < |beta|^2 < 1: only then does applyBoostTo change anything
};

// Host side: the kernel-side form of a validated channel (the reference's functor members:
// masses, ECM, max weight, final-boost vector; the engine key splitmix64(seed)).
inline void make_channel(const hps_channel& c, DevChannel& out)
{
    out = DevChannel{};
    for (int i = 0; i < c.n_daughters && i < 10; ++i) out.masses[i] = c.masses[i];
    out.ecm = c.ecm;
    out.max_weight = c.max_weight;
    for (int k = 0; k < 3; ++k) out.beta[k] = c.beta[k];
    out.key = splitmix64(c.seed);
    const double b2 = c.beta[0] * c.beta[0] + c.beta[1] * c.beta[1] + c.beta[2] * c.beta[2];
    out.boost_active = (b2 > 0.0 && b2 < 1.0) ? 1 : 0;
}

namespace f64 {

__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dvd(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ double sqr(double a) { return __dsqrt_rn(a); }

// DecayMother::pdk (DecayMother.h:119-126): sqrt((a-b-c)(a+b+c)(a-b+c)(a+b-c)) / (2a).
__device__ __forceinline__ double pdk(double a, double b, double c)
{
    const double amb = sub(a, b), apb = add(a, b);
    const double x = mul(mul(mul(sub(amb, c), add(apb, c)), add(amb, c)), sub(apb, c));
    return dvd(sqr(x), mul(2.0, a));
}

// Vector4R::applyBoostTo(Vector3R(bx,by,bz)) (hydra/detail/Vector4R.inl:249-310), general form.
__device__ __forceinline__ void boost_general(double (&v)[4], double bx, double by, double bz)
{
    const double bxx = mul(bx, bx), byy = mul(by, by), bzz = mul(bz, bz);
    const double b2 = add(add(bxx, byy), bzz);
    if (b2 > 0.0 && b2 < 1.0) {
        const double gamma = dvd(1.0, sqr(sub(1.0, b2)));
        const double gb2 = dvd(sub(gamma, 1.0), b2);
        const double gb2xy = mul(mul(gb2, bx), by);
        const double gb2xz = mul(mul(gb2, bx), bz);
        const double gb2yz = mul(mul(gb2, by), bz);
        const double gbx = mul(gamma, bx), gby = mul(gamma, by), gbz = mul(gamma, bz);
        const double e2 = v[0], px2 = v[1], py2 = v[2], pz2 = v[3];
        v[0] = add(add(add(mul(gamma, e2), mul(gbx, px2)), mul(gby, py2)), mul(gbz, pz2));
        v[1] = add(add(add(add(mul(gbx, e2), mul(mul(gb2, bxx), px2)), px2), mul(gb2xy, py2)),
                   mul(gb2xz, pz2));
        v[2] = add(add(add(add(mul(gby, e2), mul(mul(gb2, byy), py2)), py2), mul(gb2xy, px2)),
                   mul(gb2yz, pz2));
        v[3] = add(add(add(add(mul(gbz, e2), mul(mul(gb2, bzz), pz2)), pz2), mul(gb2yz, py2)),
                   mul(gb2xz, px2));
    }
}

// Vector4R::mass (Vector4R.inl:195-209).
__device__ __forceinline__ double mass(const double (&v)[4])
{
    const double m2 = sub(sub(sub(mul(v[0], v[0]), mul(v[1], v[1])), mul(v[2], v[2])), mul(v[3], v[3]));
    return (m2 > 0.0) ? sqr(m2) : 0.0;
}

__device__ __forceinline__ double mass2(const double (&v)[4])
{
    return sub(sub(sub(mul(v[0], v[0]), mul(v[1], v[1])), mul(v[2], v[2])), mul(v[3], v[3]));
}

// The event body up to (not including) the final boost, from the stream (key, base), the
// kinetic energy `ecm` and the initial weight factor `wt0`.  p[k] = {E, px, py, pz} of daughter
// k.  Returns the generation-time weight wt0 * prod pdk.
template <int N, int ENGINE>
__device__ __forceinline__ double event_core(const DevChannel& ch, uint64_t key, uint64_t base, double ecm,
                                             double wt0, double (&p)[N][4])
{
    constexpr int NW = 3 * N - 4;
    uint64_t w[NW];
    stream_words<N, ENGINE>(key, base, w);
    if constexpr (N > 3) sort_words<N - 2>(w);

    // invariant masses of the intermediate systems (DecayMother.h:170-197)
    double invMas[N];
    {
        double sum = 0.0;
#pragma unroll
        for (int n = 0; n < N; ++n) {
            const double rno = (n == 0) ? 0.0 : (n == N - 1) ? 1.0 : word_to_uniform<ENGINE>(w[n - 1]);
            sum = add(sum, ch.masses[n]);
            invMas[n] = add(mul(rno, ecm), sum);
        }
    }
    // weight (DecayMother.h:203-212)
    double pd[N - 1];
    double wt = wt0;
#pragma unroll
    for (int n = 0; n < N - 1; ++n) {
        pd[n] = pdk(invMas[n + 1], invMas[n], ch.masses[n + 1]);
        wt = mul(wt, pd[n]);
    }
    // Raubold-Lynch construction (DecayMother.h:218-257)
    p[0][0] = sqr(add(mul(pd[0], pd[0]), mul(ch.masses[0], ch.masses[0])));
    p[0][1] = 0.0; p[0][2] = pd[0]; p[0][3] = 0.0;
#pragma unroll
    for (int i = 1; i < N; ++i) {
        p[i][0] = sqr(add(mul(pd[i - 1], pd[i - 1]), mul(ch.masses[i], ch.masses[i])));
        p[i][1] = 0.0; p[i][2] = -pd[i - 1]; p[i][3] = 0.0;

        const double cZ = sub(mul(2.0, word_to_uniform<ENGINE>(w[N - 2 + 2 * (i - 1)])), 1.0);
        const double sZ = sqr(sub(1.0, mul(cZ, cZ)));
        const double angY = mul(2.0 * 3.1415926535897932384626422832795028841971,
                                word_to_uniform<ENGINE>(w[N - 2 + 2 * (i - 1) + 1]));
        double sY, cY;
        sincos(angY, &sY, &cY);
#pragma unroll
        for (int j = 0; j <= i; ++j) {
            const double x = p[j][1], y = p[j][2];
            const double x1 = sub(mul(cZ, x), mul(sZ, y));
            p[j][2] = add(mul(sZ, x), mul(cZ, y));
            const double z = p[j][3];
            p[j][1] = sub(mul(cY, x1), mul(sY, z));
            p[j][3] = add(mul(sY, x1), mul(cY, z));
        }
        if (i == N - 1) break;
        // boost along y by beta = pd/E of the (0..i) system: applyBoostTo(Vector3R(0, beta, 0))
        // with the zero components folded (adding a signed zero to a non-zero sum is exact).
        const double beta = dvd(pd[i], sqr(add(mul(pd[i], pd[i]), mul(invMas[i], invMas[i]))));
        const double b2 = mul(beta, beta);
        if (b2 > 0.0 && b2 < 1.0) {
            const double gamma = dvd(1.0, sqr(sub(1.0, b2)));
            const double gby = mul(gamma, beta);
            const double gb2byy = mul(dvd(sub(gamma, 1.0), b2), b2);
#pragma unroll
            for (int j = 0; j <= i; ++j) {
                const double e2 = p[j][0], py2 = p[j][2];
                p[j][0] = add(mul(gamma, e2), mul(gby, py2));
                p[j][2] = add(add(mul(gby, e2), mul(gb2byy, py2)), py2);
            }
        }
    }
    return wt;
}

// One event of DecayMother / AverageMother / EvalMother (DecayMother.h:163-277): the engine after
// discard(evt + 3N), the constructor's ECM and max weight, final boost by the channel's beta
// vector (DecayMother.h:264-269).
template <int N, int ENGINE>
__device__ __forceinline__ double event(const DevChannel& ch, uint64_t evt, double (&p)[N][4])
{
    const double wt = event_core<N, ENGINE>(ch, ch.key, evt + 3u * N, ch.ecm, ch.max_weight, p);
    if (ch.boost_active) {
#pragma unroll
        for (int n = 0; n < N; ++n) boost_general(p[n], ch.beta[0], ch.beta[1], ch.beta[2]);
    }
    return wt;
}

// Vector4R::applyBoostTo(Vector4R) (Vector4R.inl:236-248): boost by (px, py, pz) / E of mo.
template <int N>
__device__ __forceinline__ void boost_by_mother(double (&p)[N][4], const double (&mo)[4])
{
    const double bx = dvd(mo[1], mo[0]), by = dvd(mo[2], mo[0]), bz = dvd(mo[3], mo[0]);
#pragma unroll
    for (int n = 0; n < N; ++n) boost_general(p[n], bx, by, bz);
}

// DecayMothers / AverageMothers (DecayMothers.h:131-242): the same stream, ECM and weight as
// `event`, final boost by the event's own mother.
template <int N, int ENGINE>
__device__ __forceinline__ double event_mother(const DevChannel& ch, uint64_t evt, const double (&mo)[4],
                                               double (&p)[N][4])
{
    const double wt = event_core<N, ENGINE>(ch, ch.key, evt + 3u * N, ch.ecm, ch.max_weight, p);
    boost_by_mother<N>(p, mo);
    return wt;
}

// EvalMothers::hash, Szudzik pairing in size_t arithmetic (EvalMothers.h:131-140).
__device__ __forceinline__ uint64_t szudzik(uint64_t a, uint64_t b)
{
    const uint64_t A = 2 * a, B = 2 * b;
    return ((A >= B) ? A * A + A + B : A + B * B) / 2;
}

// EvalMothers (EvalMothers.h:143-283): engine seeded with hash(evt, seed) where evt passes
// through GInt_t, no discard; ECM and maximum weight from the mother's own mass; final boost
// by the mother.
template <int N, int ENGINE>
__device__ __forceinline__ double event_evalmothers(const DevChannel& ch, uint64_t evt, uint64_t seed,
                                                    const double (&mo)[4], double (&p)[N][4])
{
    const int32_t ievt = static_cast<int32_t>(static_cast<uint32_t>(evt));
    const uint64_t key = splitmix64(szudzik(static_cast<uint64_t>(static_cast<int64_t>(ievt)), seed));
    double ecm = mass(mo);
#pragma unroll
    for (int n = 0; n < N; ++n) ecm = sub(ecm, ch.masses[n]);
    double emmax = add(ecm, ch.masses[0]), emmin = 0.0, wtmax = 1.0;
#pragma unroll
    for (int n = 1; n < N; ++n) {
        emmin = add(emmin, ch.masses[n - 1]);
        emmax = add(emmax, ch.masses[n]);
        wtmax = mul(wtmax, pdk(emmax, emmin, ch.masses[n]));
    }
    const double wt = event_core<N, ENGINE>(ch, key, 0, ecm, dvd(1.0, wtmax), p);
    boost_by_mother<N>(p, mo);
    return wt;
}

// PhaseSpaceWeight::Evaluate (hydra/detail/Decays.inl:215-231): weight recomputed from
// stored four-vectors, R the running sum of daughters.
template <int N>
__device__ __forceinline__ double recomputed_weight(const double* masses, double max_weight,
                                                    const double (&p)[N][4])
{
    double R[4] = {p[0][0], p[0][1], p[0][2], p[0][3]};
    double w = max_weight;
#pragma unroll
    for (int i = 1; i < N; ++i) {
        double S[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) S[c] = add(R[c], p[i][c]);
        w = mul(w, pdk(mass(S), masses[i], mass(R)));
#pragma unroll
        for (int c = 0; c < 4; ++c) R[c] = S[c];
    }
    return w;
}

}  // namespace f64

// Functor menu (include/hps.h, hps_functor): 1, mass2(p_i+p_j), |BW(mass2(p_i+p_j))|^2.
struct DevFunctor {
    int kind, i, j;
    double a, b;
    float fa, fb;     // a and b rounded to float once on the host, for the FP32_FIX functor
};

template <int N>
__device__ __forceinline__ double functor_f64(const DevFunctor& f, const double (&p)[N][4])
{
    if (f.kind == 0) return 1.0;
    double s[4];
#pragma unroll
    for (int k = 0; k < N; ++k) {
        if (k == f.i) {
#pragma unroll
            for (int c = 0; c < 4; ++c) s[c] = p[k][c];
        }
    }
#pragma unroll
    for (int k = 0; k < N; ++k) {
        if (k == f.j) {
#pragma unroll
            for (int c = 0; c < 4; ++c) s[c] = f64::add(s[c], p[k][c]);
        }
    }
    const double m2 = f64::mass2(s);
    if (f.kind == 1) return m2;
    const double d = f64::sub(f64::mul(f.a, f.a), m2);
    const double g = f64::mul(f.a, f.b);
    return f64::dvd(1.0, f64::add(f64::mul(d, d), f64::mul(g, g)));
}

}  // namespace hps
