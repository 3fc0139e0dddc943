/*
 * genbod_oracle.c -- CPU oracle for the phase-space hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is a plain-C restatement of Hydra's
 * Raubold-Lynch (GENBOD) event generator and of the arithmetic it depends on.
 * It is used by tests/ (as the checker), by __graft_entry__.smoke() and by the
 * CPU-baseline legs of bench.py.  Nothing in the product library links it.
 *
 * Build: -O3 -ffp-contract=off (no -ffast-math, no FMA contraction) so that
 * every double operation rounds exactly as the reference does when it is built
 * the same way; oracle/build_ref.sh builds the reference with the same flags
 * and tests/test_oracle_golden.py checks the two agree bit for bit.
 *
 * Each function names the reference code it restates (paths inside Hydra):
 *   splitmix64 ............ hydra/detail/random/splitmix.h:56-61
 *   philox2x64, 7 rounds .. hydra/detail/external/hydra_R123/philox.h:281-358 (rounds :266-268)
 *   EngineR123 stream ..... hydra/detail/random/EngineR123.h:97-172, array.h:151-183 (incr)
 *   squares3 .............. hydra/detail/random/squares3.h:81-125
 *   uniform [0,1) ......... hydra/detail/external/hydra_thrust/random/detail/uniform_real_distribution.inl:62-80
 *   event body ............ hydra/detail/functors/DecayMother.h:119-126 (pdk), 128-151 (sort), 163-277 (process)
 *   Lorentz boost ......... hydra/detail/Vector4R.inl:249-310 (applyBoostTo(Vector3R))
 *   final-boost vector .... hydra/detail/functors/DecayMother.h:88-98
 *   ECM / max weight ...... hydra/detail/PhaseSpace.inl:67-89, hydra/PhaseSpace.h:321-326 (PDK)
 *   recomputed weight ..... hydra/detail/Decays.inl:215-231 (PhaseSpaceWeight::Evaluate)
 *   hit-or-miss flag ...... hydra/detail/Decays.inl:75-89 (FlagDaugthers)
 *   AverageOn statistics .. hydra/detail/functors/StatsPHSP.h:67-84 (AddStatsPHSP),
 *                           hydra/detail/PhaseSpace.inl:255-273, sequential fold order of
 *                           hydra_thrust/system/detail/sequential/reduce.h
 *   Evaluate .............. hydra/detail/functors/EvalMother.h:285-307
 */
#include <math.h>
#include <stdint.h>
#include <stddef.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define HPSO_MAXN 10
#define HPSO_PI 3.1415926535897932384626422832795028841971

/* Same field meaning as hps_channel in the product C ABI. */
typedef struct {
    int32_t n_daughters;
    int32_t engine;        /* 0 = Philox2x64-7, 1 = squares3 */
    uint64_t seed;         /* engine seed (size_t fSeed of the reference functor) */
    double ecm;            /* M - sum(m_i) */
    double max_weight;     /* 1 / prod PDK(...) */
    double beta[3];        /* final-boost vector exactly as DecayMother builds it */
    double masses[HPSO_MAXN];
} hpso_channel;

/* Functor menu: sel 0 -> 1, 1 -> mass2(p_i + p_j),
 * 2 -> 1 / ((a^2 - mass2(p_i+p_j))^2 + (a*b)^2)   (|relativistic BW|^2, a = mass, b = width). */
typedef struct {
    int32_t sel;
    int32_t i;
    int32_t j;
    int32_t pad;
    double a;
    double b;
} hpso_functor;

/* ---------------------------------------------------------------- RNG --- */

static inline uint64_t splitmix64(uint64_t x)
{
    uint64_t z = x + 0x9e3779b97f4a7c15ULL;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

static inline void philox2x64_7(uint64_t c0, uint64_t c1, uint64_t key, uint64_t out[2])
{
    const uint64_t M = 0xD2B74407B1CE6E93ULL;
    const uint64_t W = 0x9E3779B97F4A7C15ULL;
    for (int r = 0; r < 7; ++r) {
        if (r > 0) key += W;
        __uint128_t prod = (__uint128_t)M * (__uint128_t)c0;
        uint64_t hi = (uint64_t)(prod >> 64);
        uint64_t lo = (uint64_t)prod;
        uint64_t n0 = hi ^ key ^ c1;
        c0 = n0;
        c1 = lo;
    }
    out[0] = c0;
    out[1] = c1;
}

static inline uint32_t squares3_word(uint64_t key, uint64_t ctr)
{
    uint64_t x, y, z;
    y = x = key * ctr;
    z = y + key;
    x = x * x + y; x = (x >> 32) | (x << 32);
    x = x * x + z; x = (x >> 32) | (x << 32);
    return (uint32_t)((x * x + y) >> 32);
}

/* A per-event stream: the reference constructs the engine from the seed and
 * calls discard(evt + 3N) before the first draw. */
typedef struct {
    int engine;
    uint64_t key;
    uint64_t c0, c1;     /* Philox 128-bit counter (v[0], v[1]) */
    uint64_t cache[2];
    int trigger;
    uint64_t sq_state;   /* squares3 counter */
    uint32_t lcg;        /* minstd_rand state */
} hpso_stream;

/* thrust's default_random_engine, minstd_rand: x <- 48271 x mod (2^31 - 1)
 * (hydra_thrust/random/linear_congruential_engine.h:279).  Seeding reduces the 32-bit seed mod
 * 2^31 - 1 and maps 0 to 1 (linear_congruential_engine.inl:41-50); discard(z) multiplies the state by
 * 48271^z mod 2^31 - 1 (linear_congruential_engine_discard.h:47-74).  All products below fit 64 bits. */
#define HPSO_LCG_A 48271u
#define HPSO_LCG_M 2147483647u

static inline uint32_t lcg_seed(uint64_t seed)
{
    uint32_t s = (uint32_t)seed % HPSO_LCG_M;
    return s == 0 ? 1u : s;
}

static inline uint32_t lcg_discard(uint32_t state, uint64_t z)
{
    uint64_t mult = HPSO_LCG_A, acc = 1;
    while (z > 0) {
        if (z & 1) acc = (acc * mult) % HPSO_LCG_M;
        z >>= 1;
        mult = (mult * mult) % HPSO_LCG_M;
    }
    return (uint32_t)((acc * state) % HPSO_LCG_M);
}

static inline void stream_init(hpso_stream* s, int engine, uint64_t seed, uint64_t skip)
{
    memset(s, 0, sizeof(*s));
    s->engine = engine;
    s->key = splitmix64(seed);
    if (engine == 2) {
        s->lcg = lcg_discard(lcg_seed(seed), skip);
    } else if (engine == 0) {
        s->c0 = skip;                  /* incr(n) from {0,0}: carry only on wrap */
        s->c1 = 0;
        s->trigger = 2;
    } else {
        s->sq_state = skip;
    }
}

static inline uint64_t stream_word(hpso_stream* s)
{
    if (s->engine == 0) {
        if (s->trigger == 2) {
            s->c0 += 1;
            if (s->c0 == 0) s->c1 += 1;
            philox2x64_7(s->c0, s->c1, s->key, s->cache);
            s->trigger = 0;
        }
        return s->cache[s->trigger++];
    }
    if (s->engine == 2) {
        s->lcg = (uint32_t)(((uint64_t)s->lcg * HPSO_LCG_A) % HPSO_LCG_M);
        return s->lcg;
    }
    uint32_t w = squares3_word(s->key, s->sq_state);
    s->sq_state += 1;
    return (uint64_t)w;
}

static inline double stream_uniform(hpso_stream* s)
{
    uint64_t w = stream_word(s);
    double r;
    if (s->engine == 2) {
        r = (double)(uint32_t)(w - 1u);                 /* urng() - min, min = 1 */
        r /= 2147483646.0;                              /* 1 + double(max - min) */
    } else {
        r = (double)w;
        if (s->engine == 0) r /= 18446744073709551616.0;   /* 1 + double(2^64 - 1) == 2^64 */
        else r /= 4294967296.0;                             /* 1 + double(2^32 - 1) == 2^32 */
    }
    return r * (1.0 - 0.0) + 0.0;
}

/* ------------------------------------------------------------ kinematics --- */

static inline double pdk(double a, double b, double c)
{
    return sqrt((a - b - c) * (a + b + c) * (a - b + c) * (a + b - c)) / (2 * a);
}

static inline void boost(double v[4], double bx, double by, double bz)
{
    double bxx = bx * bx;
    double byy = by * by;
    double bzz = bz * bz;
    double b2 = bxx + byy + bzz;
    if (b2 > 0.0 && b2 < 1.0) {
        double gamma = 1.0 / sqrt(1.0 - b2);
        double gb2 = (gamma - 1.0) / b2;
        double gb2xy = gb2 * bx * by;
        double gb2xz = gb2 * bx * bz;
        double gb2yz = gb2 * by * bz;
        double gbx = gamma * bx;
        double gby = gamma * by;
        double gbz = gamma * bz;
        double e2 = v[0], px2 = v[1], py2 = v[2], pz2 = v[3];
        v[0] = gamma * e2 + gbx * px2 + gby * py2 + gbz * pz2;
        v[1] = gbx * e2 + gb2 * bxx * px2 + px2 + gb2xy * py2 + gb2xz * pz2;
        v[2] = gby * e2 + gb2 * byy * py2 + py2 + gb2xy * px2 + gb2yz * pz2;
        v[3] = gbz * e2 + gb2 * bzz * pz2 + pz2 + gb2yz * py2 + gb2xz * px2;
    }
}

static inline double mass_of(const double v[4])
{
    double m2 = v[0] * v[0] - v[1] * v[1] - v[2] * v[2] - v[3] * v[3];
    return (m2 > 0.0) ? sqrt(m2) : 0.0;
}

static inline double mass2_of(const double v[4])
{
    return v[0] * v[0] - v[1] * v[1] - v[2] * v[2] - v[3] * v[3];
}

/* Szudzik pairing of EvalMothers::hash (hydra/detail/functors/EvalMothers.h:131-140), size_t arithmetic. */
static inline uint64_t szudzik(uint64_t a, uint64_t b)
{
    uint64_t A = 2 * a, B = 2 * b;
    return ((A >= B) ? A * A + A + B : A + B * B) / 2;
}

/* One GENBOD event; p is [N][4] (E, px, py, pz).  Returns the generation-time weight.
 * mode 0: DecayMother / AverageMother / EvalMother (DecayMother.h:163-277): engine seeded with
 *         the channel seed after discard(evt+3N); final boost by the channel's beta vector.
 * mode 1: DecayMothers / AverageMothers (DecayMothers.h:131-242): same stream and ECM, final boost
 *         by the event's mother four-vector (applyBoostTo(Vector4R), Vector4R.inl:236-248).
 * mode 2: EvalMothers (EvalMothers.h:143-283): engine seeded with hash((int)evt, seed) and no
 *         discard; ECM and the maximum weight from the event mother's own mass; weight
 *         (1/wtmax) * prod pdk; final boost by the mother. */
static double event_body_ex(const hpso_channel* ch, uint64_t evt, double p[][4], int mode, const double* mother)
{
    const int N = ch->n_daughters;
    const double* m = ch->masses;
    hpso_stream s;
    double ecm = ch->ecm;
    double wt;
    if (mode == 2) {
        const int32_t ievt = (int32_t)(uint32_t)evt;               /* process(const GInt_t evt, ...) */
        stream_init(&s, ch->engine, szudzik((uint64_t)(int64_t)ievt, ch->seed), 0);
        ecm = mass_of(mother);
        for (int n = 0; n < N; ++n) ecm -= m[n];
        double emmax = ecm + m[0], emmin = 0.0, wtmax = 1.0;
        for (int n = 1; n < N; ++n) {
            emmin += m[n - 1];
            emmax += m[n];
            wtmax *= pdk(emmax, emmin, m[n]);
        }
        wt = 1.0 / wtmax;
    } else {
        stream_init(&s, ch->engine, ch->seed, evt + 3u * (uint64_t)N);
        wt = ch->max_weight;
    }

    double rno[HPSO_MAXN];
    rno[0] = 0.0;
    rno[N - 1] = 1.0;
    if (N > 2) {
        for (int n = 1; n < N - 1; ++n) rno[n] = stream_uniform(&s);
        /* the reference bubble-sorts rno[1..N-2] ascending; any correct
         * ascending sort of finite doubles gives the same sequence */
        for (int a = 2; a < N - 1; ++a) {
            double key = rno[a];
            int b = a - 1;
            while (b >= 1 && rno[b] > key) { rno[b + 1] = rno[b]; --b; }
            rno[b + 1] = key;
        }
    }

    double invMas[HPSO_MAXN], sum = 0.0;
    for (int n = 0; n < N; ++n) {
        sum += m[n];
        invMas[n] = rno[n] * ecm + sum;
    }

    double pd[HPSO_MAXN] = {0};
    for (int n = 0; n < N - 1; ++n) {
        pd[n] = pdk(invMas[n + 1], invMas[n], m[n + 1]);
        wt *= pd[n];
    }

    p[0][0] = sqrt(pd[0] * pd[0] + m[0] * m[0]);
    p[0][1] = 0.0; p[0][2] = pd[0]; p[0][3] = 0.0;

    for (int i = 1; i < N; ++i) {
        p[i][0] = sqrt(pd[i - 1] * pd[i - 1] + m[i] * m[i]);
        p[i][1] = 0.0; p[i][2] = -pd[i - 1]; p[i][3] = 0.0;

        double cZ = 2 * stream_uniform(&s) - 1;
        double sZ = sqrt(1 - cZ * cZ);
        double angY = 2 * HPSO_PI * stream_uniform(&s);
        double cY = cos(angY);
        double sY = sin(angY);
        for (int j = 0; j <= i; ++j) {
            double x = p[j][1];
            double y = p[j][2];
            p[j][1] = cZ * x - sZ * y;
            p[j][2] = sZ * x + cZ * y;
            x = p[j][1];
            double z = p[j][3];
            p[j][1] = cY * x - sY * z;
            p[j][3] = sY * x + cY * z;
        }
        if (i == N - 1) break;
        double beta = pd[i] / sqrt(pd[i] * pd[i] + invMas[i] * invMas[i]);
        for (int j = 0; j <= i; ++j) boost(p[j], 0, beta, 0);
    }
    if (mode == 0) {
        for (int n = 0; n < N; ++n) boost(p[n], ch->beta[0], ch->beta[1], ch->beta[2]);
    } else {
        const double e = mother[0];
        const double bx = mother[1] / e, by = mother[2] / e, bz = mother[3] / e;
        for (int n = 0; n < N; ++n) boost(p[n], bx, by, bz);
    }
    return wt;
}

static double event_body(const hpso_channel* ch, uint64_t evt, double p[][4])
{
    return event_body_ex(ch, evt, p, 0, NULL);
}

static inline double functor_eval(const hpso_functor* f, double p[][4])
{
    if (f->sel == 0) return 1.0;
    double s[4];
    for (int c = 0; c < 4; ++c) s[c] = p[f->i][c] + p[f->j][c];
    double m2 = mass2_of(s);
    if (f->sel == 1) return m2;
    double d = f->a * f->a - m2;
    double g = f->a * f->b;
    return 1.0 / (d * d + g * g);
}

/* ------------------------------------------------------------ public API --- */

/* Host set-up of a channel as the reference constructor does it.
 * mother = (E, px, py, pz) of the mother passed to Generate; only the
 * final-boost vector depends on it (the ECM uses motherMass).
 * Returns 0, or -1 (mass <= 0: std::invalid_argument), -2 (ECM <= 0: std::runtime_error). */
int hpso_channel_init(hpso_channel* ch, int n, int engine, uint64_t seed,
                      double mother_mass, const double* masses, const double* mother)
{
    if (n < 2 || n > HPSO_MAXN) return -3;
    memset(ch, 0, sizeof(*ch));
    ch->n_daughters = n;
    ch->engine = engine;
    ch->seed = seed;
    if (mother_mass <= 0.0) return -1;
    for (int i = 0; i < n; ++i) {
        ch->masses[i] = masses[i];
        if (masses[i] <= 0.0) return -1;
    }
    double ecm = mother_mass;
    for (int i = 0; i < n; ++i) ecm -= masses[i];
    if (ecm <= 0.0) return -2;
    ch->ecm = ecm;
    double emmax = ecm + masses[0], emmin = 0.0, wtmax = 1.0;
    for (int i = 1; i < n; ++i) {
        emmin += masses[i - 1];
        emmax += masses[i];
        double x = (emmax - emmin - masses[i]) * (emmax + emmin + masses[i]) *
                   (emmax - emmin + masses[i]) * (emmax + emmin - masses[i]);
        x = sqrt(x) / (2 * emmax);
        wtmax *= x;
    }
    ch->max_weight = 1.0 / wtmax;
    double d3 = sqrt(mother[1] * mother[1] + mother[2] * mother[2] + mother[3] * mother[3]);
    double beta = d3 / mother[0];
    if (beta) {
        double w = beta / d3;
        ch->beta[0] = mother[0] * w;
        ch->beta[1] = mother[1] * w;
        ch->beta[2] = mother[2] * w;
    }
    return 0;
}

/* Raw stream words: out[(e - first) * (3N-4) + k] for event e, draw k. */
void hpso_rng_words(int n_daughters, int engine, uint64_t seed, uint64_t first, uint64_t n,
                    uint64_t* out)
{
    const int nw = 3 * n_daughters - 4;
    for (uint64_t e = 0; e < n; ++e) {
        hpso_stream s;
        stream_init(&s, engine, seed, first + e + 3u * (uint64_t)n_daughters);
        for (int k = 0; k < nw; ++k) out[e * nw + k] = stream_word(&s);
    }
}

/* Generate: four-vectors as one [N][n][4] block (Decays column layout),
 * optional gen-time weights [n].  nthreads <= 0 uses all OpenMP threads. */
void hpso_generate(const hpso_channel* ch, uint64_t first, uint64_t n, double* out4,
                   double* weights, int nthreads)
{
    const int N = ch->n_daughters;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(static) num_threads(nthreads)
#endif
    for (int64_t e = 0; e < (int64_t)n; ++e) {
        double p[HPSO_MAXN][4];
        double w = event_body(ch, first + (uint64_t)e, p);
        for (int k = 0; k < N; ++k)
            memcpy(out4 + (((size_t)k * n + (size_t)e) * 4), p[k], 4 * sizeof(double));
        if (weights) weights[e] = w;
    }
    (void)nthreads;
}

/* Recomputed weight from stored four-vectors ([N][n][4]), with the
 * PhaseSpaceWeight max weight `max_weight`. */
void hpso_recompute_weights(int n_daughters, const double* masses, double max_weight,
                            uint64_t n, const double* four, double* out, int nthreads)
{
    const int N = n_daughters;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(static) num_threads(nthreads)
#endif
    for (int64_t e = 0; e < (int64_t)n; ++e) {
        double R[4], S[4];
        memcpy(R, four + ((size_t)e) * 4, sizeof(R));
        double w = max_weight;
        for (int i = 1; i < N; ++i) {
            const double* pi = four + (((size_t)i * n + (size_t)e) * 4);
            for (int c = 0; c < 4; ++c) S[c] = R[c] + pi[c];
            w *= pdk(mass_of(S), masses[i], mass_of(R));
            for (int c = 0; c < 4; ++c) R[c] += pi[c];
        }
        out[e] = w;
    }
    (void)nthreads;
}

/* PhaseSpaceReweight::Evaluate (hydra/detail/Decays.inl:372-386): the PhaseSpaceWeight of each
 * stored event times the functor of its daughters, w * f(p). */
void hpso_reweight(int n_daughters, const double* masses, double max_weight, const hpso_functor* f,
                   uint64_t n, const double* four, double* out, int nthreads)
{
    const int N = n_daughters;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(static) num_threads(nthreads)
#endif
    for (int64_t e = 0; e < (int64_t)n; ++e) {
        double p[HPSO_MAXN][4], R[4], S[4];
        for (int i = 0; i < N; ++i) memcpy(p[i], four + (((size_t)i * n + (size_t)e) * 4), sizeof(p[i]));
        memcpy(R, p[0], sizeof(R));
        double w = max_weight;
        for (int i = 1; i < N; ++i) {
            for (int c = 0; c < 4; ++c) S[c] = R[c] + p[i][c];
            w *= pdk(mass_of(S), masses[i], mass_of(R));
            for (int c = 0; c < 4; ++c) R[c] += p[i][c];
        }
        out[e] = w * functor_eval(f, p);
    }
    (void)nthreads;
}

/* GetGlobalBin (hydra/detail/functors/GetGlobalBin.h:120-138) for two dimensions: x_d is mapped to
 * (x_d - lo_d) * grid_d / (hi_d - lo_d); all coordinates below 0 -> bin g0*g1 (underflow), all above
 * grid_d -> g0*g1 + 1 (overflow), otherwise size_t(x0) * g1 + size_t(x1).  The reference converts a
 * negative coordinate to size_t there (undefined) and lets an index of g_d land in another row; this
 * restatement sends every point with any coordinate outside [0, g_d) (and not all below / all above)
 * to the overflow bin, as the CUDA kernel does. */
static inline uint64_t global_bin2(const double x[2], const uint64_t g[2], const double lo[2], const double hi[2])
{
    double X[2];
    int under = 1, over = 1, inside = 1;
    for (int d = 0; d < 2; ++d) {
        X[d] = (x[d] - lo[d]) * (double)g[d] / (hi[d] - lo[d]);
        under = under && (X[d] < 0.0);
        over = over && (X[d] > (double)g[d]);
        inside = inside && (X[d] >= 0.0) && (X[d] < (double)g[d]);
    }
    const uint64_t nb = g[0] * g[1];
    if (under) return nb;
    if (over || !inside) return nb + 1;
    return (uint64_t)X[0] * g[1] + (uint64_t)X[1];
}

/* DenseHistogram<double,2>::Fill(data, weights) (hydra/detail/DenseHistogram.inl:45-103) of the
 * Dalitz variables (m2(p_a0 + p_a1), m2(p_b0 + p_b1)) of stored events, weighted by w[e] (NULL: 1).
 * bins has g0*g1 + 2 entries and is overwritten; sums run in event order per bin, as the
 * reference's sort_by_key + reduce_by_key does on a sequential backend. */
void hpso_dalitz_histogram(int n_daughters, uint64_t n, const double* four, const double* w,
                           const int32_t pairs[4], const uint64_t grid[2], const double lo[2],
                           const double hi[2], double* bins)
{
    const uint64_t nb = grid[0] * grid[1] + 2;
    for (uint64_t b = 0; b < nb; ++b) bins[b] = 0.0;
    for (uint64_t e = 0; e < n; ++e) {
        double x[2];
        for (int d = 0; d < 2; ++d) {
            const double* a = four + (((size_t)pairs[2 * d] * n + e) * 4);
            const double* b = four + (((size_t)pairs[2 * d + 1] * n + e) * 4);
            double s[4];
            for (int c = 0; c < 4; ++c) s[c] = a[c] + b[c];
            x[d] = mass2_of(s);
        }
        bins[global_bin2(x, grid, lo, hi)] += w ? w[e] : 1.0;
    }
    (void)n_daughters;
}

/* Hit-or-miss flags as Decays::Unweight: squares3(useed), discard(index),
 * accept when weight / max_weight > u.  index = first + e. */
void hpso_flags(const double* weights, double max_weight, uint64_t useed, uint64_t first,
                uint64_t n, uint8_t* flags)
{
    const uint64_t key = splitmix64(useed);
    for (uint64_t e = 0; e < n; ++e) {
        double u = (double)squares3_word(key, first + e) / 4294967296.0;
        u = u * (1.0 - 0.0) + 0.0;
        flags[e] = (weights[e] / max_weight > u) ? 1 : 0;
    }
}

/* The uniforms FlagDaugthers draws: squares3(useed) after discard(first + e). */
void hpso_unweight_uniforms(uint64_t useed, uint64_t first, uint64_t n, double* out)
{
    const uint64_t key = splitmix64(useed);
    for (uint64_t e = 0; e < n; ++e) out[e] = (double)squares3_word(key, first + e) / 4294967296.0;
}

/* Evaluate: out_w[n] = gen-time weight, out_f[n] = functor value. */
void hpso_evaluate(const hpso_channel* ch, const hpso_functor* f, uint64_t first, uint64_t n,
                   double* out_w, double* out_f, int nthreads)
{
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(static) num_threads(nthreads)
#endif
    for (int64_t e = 0; e < (int64_t)n; ++e) {
        double p[HPSO_MAXN][4];
        double w = event_body(ch, first + (uint64_t)e, p);
        out_w[e] = w;
        out_f[e] = functor_eval(f, p);
    }
    (void)nthreads;
}

typedef struct { double mean, m2, w; } hpso_stats;

static inline hpso_stats stats_add(hpso_stats x, hpso_stats y)
{
    hpso_stats r;
    double w = x.w + y.w;
    double delta = y.mean - x.mean;
    double delta2 = delta * delta;
    r.w = w;
    r.mean = (x.mean * x.w + y.mean * y.w) / w;
    r.m2 = x.m2 + y.m2;
    r.m2 += delta2 * x.w * y.w / w;
    return r;
}

/* AverageOn.  nthreads == 1: the sequential left fold of the cpp backend,
 * bit-identical to the reference built with HYDRA_DEVICE_SYSTEM=CPP.
 * nthreads != 1: contiguous per-thread folds merged in thread order.
 * out = {mean, M2, W}; the reference returns (mean, sqrt(M2)/W). */
void hpso_average_on(const hpso_channel* ch, const hpso_functor* f, uint64_t first, uint64_t n,
                     double* out, int nthreads)
{
    hpso_stats total = {0.0, 0.0, 0.0};
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#else
    nthreads = 1;
#endif
    if (nthreads == 1) {
        for (uint64_t e = 0; e < n; ++e) {
            double p[HPSO_MAXN][4];
            hpso_stats y;
            y.w = event_body(ch, first + e, p);
            y.mean = functor_eval(f, p);
            y.m2 = 0.0;
            total = stats_add(total, y);
        }
    } else {
        hpso_stats part[512];
        if (nthreads > 512) nthreads = 512;
#ifdef _OPENMP
#pragma omp parallel num_threads(nthreads)
#endif
        {
            int t = 0, nt = 1;
#ifdef _OPENMP
            t = omp_get_thread_num();
            nt = omp_get_num_threads();
#endif
            uint64_t lo = n * (uint64_t)t / (uint64_t)nt, hi = n * (uint64_t)(t + 1) / (uint64_t)nt;
            hpso_stats acc = {0.0, 0.0, 0.0};
            for (uint64_t e = lo; e < hi; ++e) {
                double p[HPSO_MAXN][4];
                hpso_stats y;
                y.w = event_body(ch, first + e, p);
                y.mean = functor_eval(f, p);
                y.m2 = 0.0;
                acc = stats_add(acc, y);
            }
            part[t] = acc;
#ifdef _OPENMP
#pragma omp barrier
#pragma omp single
#endif
            {
                int have = 0;
                for (int k = 0; k < nt; ++k) {
                    uint64_t klo = n * (uint64_t)k / (uint64_t)nt, khi = n * (uint64_t)(k + 1) / (uint64_t)nt;
                    if (khi == klo) continue;
                    total = have ? stats_add(total, part[k]) : part[k];
                    have = 1;
                }
            }
        }
    }
    out[0] = total.mean;
    out[1] = total.m2;
    out[2] = total.w;
}

/* Timed CPU baseline of the whole store step (Generate + gen-time weight +
 * recomputed-weight flags) over events [first, first+n), into caller buffers. */
void hpso_store_step(const hpso_channel* ch, uint64_t first, uint64_t n, double* out4,
                     double* weights, uint64_t useed, uint8_t* flags, int nthreads)
{
    const int N = ch->n_daughters;
    const uint64_t key = splitmix64(useed);
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(static) num_threads(nthreads)
#endif
    for (int64_t e = 0; e < (int64_t)n; ++e) {
        double p[HPSO_MAXN][4];
        double w = event_body(ch, first + (uint64_t)e, p);
        for (int k = 0; k < N; ++k)
            memcpy(out4 + (((size_t)k * n + (size_t)e) * 4), p[k], 4 * sizeof(double));
        weights[e] = w;
        if (flags) {
            double R[4], S[4];
            memcpy(R, p[0], sizeof(R));
            double wr = ch->max_weight;
            for (int i = 1; i < N; ++i) {
                for (int c = 0; c < 4; ++c) S[c] = R[c] + p[i][c];
                wr *= pdk(mass_of(S), ch->masses[i], mass_of(R));
                for (int c = 0; c < 4; ++c) R[c] += p[i][c];
            }
            double u = (double)squares3_word(key, first + (uint64_t)e) / 4294967296.0;
            flags[e] = (wr / ch->max_weight > u) ? 1 : 0;
        }
    }
    (void)nthreads;
}

/* Generate / AverageOn / Evaluate over a range of mothers ([n][4] doubles, one per event).
 * mode 1 (Generate, AverageOn) follows DecayMothers / AverageMothers, mode 2 (Evaluate) EvalMothers.
 * The functor sees (mother, daughter 0, ..., daughter N-1) (AverageMothers.h:258-269,
 * EvalMothers.h:295-302): its indices count the mother as particle 0. */
void hpso_generate_mothers(const hpso_channel* ch, uint64_t first, uint64_t n, const double* mothers,
                           double* out4, double* weights, int nthreads)
{
    const int N = ch->n_daughters;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(static) num_threads(nthreads)
#endif
    for (int64_t e = 0; e < (int64_t)n; ++e) {
        double p[HPSO_MAXN][4];
        double w = event_body_ex(ch, first + (uint64_t)e, p, 1, mothers + 4 * e);
        for (int k = 0; k < N; ++k)
            memcpy(out4 + (((size_t)k * n + (size_t)e) * 4), p[k], 4 * sizeof(double));
        if (weights) weights[e] = w;
    }
    (void)nthreads;
}

void hpso_average_mothers(const hpso_channel* ch, const hpso_functor* f, uint64_t first, uint64_t n,
                          const double* mothers, double* out)
{
    hpso_stats total = {0.0, 0.0, 0.0};
    for (uint64_t e = 0; e < n; ++e) {
        double p[HPSO_MAXN][4];
        hpso_stats y;
        y.w = event_body_ex(ch, first + e, p, 1, mothers + 4 * e);
        double pm[HPSO_MAXN + 1][4];                   /* (mother, daughters...) as the functor sees them */
        memcpy(pm[0], mothers + 4 * e, sizeof(pm[0]));
        memcpy(pm[1], p, sizeof(double) * 4 * (size_t)ch->n_daughters);
        y.mean = functor_eval(f, pm);
        y.m2 = 0.0;
        total = stats_add(total, y);
    }
    out[0] = total.mean;
    out[1] = total.m2;
    out[2] = total.w;
}

void hpso_evaluate_mothers(const hpso_channel* ch, const hpso_functor* f, uint64_t first, uint64_t n,
                           const double* mothers, double* out_w, double* out_f, double* out4, int nthreads)
{
    const int N = ch->n_daughters;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(static) num_threads(nthreads)
#endif
    for (int64_t e = 0; e < (int64_t)n; ++e) {
        double p[HPSO_MAXN][4];
        out_w[e] = event_body_ex(ch, first + (uint64_t)e, p, 2, mothers + 4 * e);
        double pm[HPSO_MAXN + 1][4];
        memcpy(pm[0], mothers + 4 * e, sizeof(pm[0]));
        memcpy(pm[1], p, sizeof(double) * 4 * (size_t)N);
        out_f[e] = functor_eval(f, pm);
        if (out4)
            for (int k = 0; k < N; ++k)
                memcpy(out4 + (((size_t)k * n + (size_t)e) * 4), p[k], 4 * sizeof(double));
    }
    (void)nthreads;
}

int hpso_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
