/*
 * ref_harness.cpp -- test infrastructure, NOT product code.
 *
 * A command-line driver over the UNMODIFIED Hydra headers (hydra::PhaseSpace,
 * hydra::Decays, hydra::PhaseSpaceWeight, hydra::random engines).  It is built
 * by oracle/build_ref.sh straight from the Hydra source tree, with the cpp
 * (sequential) or omp backend, and its outputs pin the C restatement in
 * oracle/genbod_oracle.c and the golden fixtures under tests/golden/.
 *
 * Reference calls exercised (paths inside the Hydra project):
 *   hydra/detail/PhaseSpace.inl:42-90      ctor: ECM, max weight, default seed
 *   hydra/detail/PhaseSpace.inl:377-394    Generate(mother, Decays&)
 *   hydra/detail/PhaseSpace.inl:255-273    AverageOn(policy, mother, functor, n)
 *   hydra/detail/PhaseSpace.inl:314-329    Evaluate(mother, result, functor)
 *   hydra/detail/Decays.inl:215-231        PhaseSpaceWeight::Evaluate (recomputed weight)
 *   hydra/detail/Decays.inl:75-89          FlagDaugthers (hit-or-miss flag)
 *   hydra/detail/Decays.inl:415-455        Decays::Unweight()
 *   hydra/detail/random/EngineR123.h:97-172, squares3.h:105-125  raw RNG words
 *   hydra/detail/Decays.inl:258-411, 458-511  PhaseSpaceReweight, Decays::Unweight(functor, w, seed)
 *   hydra/detail/DenseHistogram.inl:45-103  2-D DenseHistogram::Fill(data, weights)
 *   hydra/detail/PhaseSpaceRange.inl:46-73  phase_space_range (GenerateDecay, thrust minstd_rand)
 *   hydra/detail/PhaseSpaceIntegrator.inl:37-42  PhaseSpaceIntegrator::Integrate
 *   examples/phase_space/phsp_averaging_functor.inl, phsp_evaluating_functor.inl: wrap_lambda functors
 *       over declarg arguments with hydra::CosHelicityAngle, through AverageOn, Evaluate, Unweight
 *
 * Usage:
 *   ref_harness rng  N engine seed n                      out.bin
 *   ref_harness gen  N engine seed n M m0..m{N-1} fsel fi fj fa fb useed mx my mz out.bin
 *   ref_harness avg  N engine seed n M m0..m{N-1} fsel fi fj fa fb out.bin
 *   ref_harness time N engine seed n M m0..m{N-1} fsel fi fj fa fb reps
 *   ref_harness mothers N engine seed n M m0..m{N-1} fsel fi fj fa fb out.bin
 *   ref_harness functors 3 engine seed n M m0 m1 m2 fsel fi fj fa fb fseed out.bin
 *   ref_harness extras N engine seed n M m0..m{N-1} fsel fi fj fa fb fseed fmax g0 g1 lo0 lo1 hi0 hi1
 *                      rseed mx my mz out.bin
 * engine: 0 = hydra::philox (Philox2x64, 7 rounds), 1 = hydra::default_random_engine (squares3)
 * fsel:   0 = constant 1, 1 = mass2(p_i+p_j), 2 = 1/((a^2 - mass2(p_i+p_j))^2 + (a*b)^2)
 * seed:   gen/avg/time: passed to PhaseSpace::SetSeed(GInt_t), -1 keeps the default (hash) seed;
 *         rng: the raw 64-bit engine seed.
 */
#include <hydra/Types.h>
#include <hydra/Vector4R.h>
#include <hydra/PhaseSpace.h>
#include <hydra/Decays.h>
#include <hydra/Lambda.h>
#include <hydra/Tuple.h>
#include <hydra/multivector.h>
#include <hydra/Range.h>
#include <hydra/DenseHistogram.h>
#include <hydra/PhaseSpaceIntegrator.h>
#include <hydra/Placeholders.h>
#include <hydra/host/System.h>
#include <hydra/device/System.h>
#include <hydra/detail/random/EngineR123.h>
#include <hydra/detail/random/squares3.h>
#include <hydra/functions/CosHelicityAngle.h>

#include <array>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

declarg(FJpsi, hydra::Vector4R)
declarg(FKaon, hydra::Vector4R)
declarg(FPion, hydra::Vector4R)
declarg(D0, hydra::Vector4R)
declarg(D1, hydra::Vector4R)
declarg(D2, hydra::Vector4R)
declarg(D3, hydra::Vector4R)
declarg(D4, hydra::Vector4R)
declarg(D5, hydra::Vector4R)
declarg(D6, hydra::Vector4R)
declarg(D7, hydra::Vector4R)
declarg(D8, hydra::Vector4R)
declarg(D9, hydra::Vector4R)

declarg(WCol, double)
declarg(FCol, double)

using namespace hydra::arguments;

namespace {

template <size_t N> struct ptypes;
template <> struct ptypes<2>  { typedef hydra::tuple<D0, D1> type; };
template <> struct ptypes<3>  { typedef hydra::tuple<D0, D1, D2> type; };
template <> struct ptypes<4>  { typedef hydra::tuple<D0, D1, D2, D3> type; };
template <> struct ptypes<5>  { typedef hydra::tuple<D0, D1, D2, D3, D4> type; };
template <> struct ptypes<6>  { typedef hydra::tuple<D0, D1, D2, D3, D4, D5> type; };
template <> struct ptypes<7>  { typedef hydra::tuple<D0, D1, D2, D3, D4, D5, D6> type; };
template <> struct ptypes<8>  { typedef hydra::tuple<D0, D1, D2, D3, D4, D5, D6, D7> type; };
template <> struct ptypes<9>  { typedef hydra::tuple<D0, D1, D2, D3, D4, D5, D6, D7, D8> type; };
template <> struct ptypes<10> { typedef hydra::tuple<D0, D1, D2, D3, D4, D5, D6, D7, D8, D9> type; };

struct FSpec { int sel; int i; int j; double a; double b; };

// Scalar form of the functor menu; every implementation in this project
// (C oracle, CUDA kernels) evaluates the same expression.
inline double fmenu(FSpec const& f, hydra::Vector4R const* p)
{
    if (f.sel == 0) return 1.0;
    hydra::Vector4R s = p[f.i] + p[f.j];
    double m2 = s.mass2();
    if (f.sel == 1) return m2;
    double d = f.a * f.a - m2;
    double g = f.a * f.b;
    return 1.0 / (d * d + g * g);
}

#define HV hydra::Vector4R
#define LAM_ARGS_2  HV p0, HV p1
#define LAM_ARGS_3  LAM_ARGS_2, HV p2
#define LAM_ARGS_4  LAM_ARGS_3, HV p3
#define LAM_ARGS_5  LAM_ARGS_4, HV p4
#define LAM_ARGS_6  LAM_ARGS_5, HV p5
#define LAM_ARGS_7  LAM_ARGS_6, HV p6
#define LAM_ARGS_8  LAM_ARGS_7, HV p7
#define LAM_ARGS_9  LAM_ARGS_8, HV p8
#define LAM_ARGS_10 LAM_ARGS_9, HV p9
#define LAM_ARGS_11 LAM_ARGS_10, HV p10
#define LAM_NAMES_2  p0, p1
#define LAM_NAMES_3  LAM_NAMES_2, p2
#define LAM_NAMES_4  LAM_NAMES_3, p3
#define LAM_NAMES_5  LAM_NAMES_4, p4
#define LAM_NAMES_6  LAM_NAMES_5, p5
#define LAM_NAMES_7  LAM_NAMES_6, p6
#define LAM_NAMES_8  LAM_NAMES_7, p7
#define LAM_NAMES_9  LAM_NAMES_8, p8
#define LAM_NAMES_10 LAM_NAMES_9, p9
#define LAM_NAMES_11 LAM_NAMES_10, p10

#define TLAM_ARGS_2  D0 p0, D1 p1
#define TLAM_ARGS_3  TLAM_ARGS_2, D2 p2
#define TLAM_ARGS_4  TLAM_ARGS_3, D3 p3
#define TLAM_ARGS_5  TLAM_ARGS_4, D4 p4
#define TLAM_ARGS_6  TLAM_ARGS_5, D5 p5
#define TLAM_ARGS_7  TLAM_ARGS_6, D6 p6
#define TLAM_ARGS_8  TLAM_ARGS_7, D7 p7
#define TLAM_ARGS_9  TLAM_ARGS_8, D8 p8
#define TLAM_ARGS_10 TLAM_ARGS_9, D9 p9

template <size_t N> struct menu_lambda;
#define MENU_LAMBDA(NN)                                                        \
    template <> struct menu_lambda<NN> {                                       \
        static auto make(FSpec f) {                                            \
            return hydra::wrap_lambda([f](LAM_ARGS_##NN) {                     \
                HV arr[NN] = {LAM_NAMES_##NN};                                 \
                return fmenu(f, arr);                                          \
            });                                                                \
        }                                                                      \
    };
MENU_LAMBDA(2) MENU_LAMBDA(3) MENU_LAMBDA(4) MENU_LAMBDA(5) MENU_LAMBDA(6)
MENU_LAMBDA(7) MENU_LAMBDA(8) MENU_LAMBDA(9) MENU_LAMBDA(10) MENU_LAMBDA(11)

// The menu over the typed daughter columns: PhaseSpaceReweight hands its functor a tuple of the
// Decays' own argument types (Decays.inl:383), which a lambda picks by type.
template <size_t N> struct typed_menu_lambda;
#define TYPED_MENU_LAMBDA(NN)                                                  \
    template <> struct typed_menu_lambda<NN> {                                 \
        static auto make(FSpec f) {                                            \
            return hydra::wrap_lambda([f](TLAM_ARGS_##NN) {                    \
                HV arr[NN] = {LAM_NAMES_##NN};                                 \
                return fmenu(f, arr);                                          \
            });                                                                \
        }                                                                      \
    };
TYPED_MENU_LAMBDA(2) TYPED_MENU_LAMBDA(3) TYPED_MENU_LAMBDA(4) TYPED_MENU_LAMBDA(5) TYPED_MENU_LAMBDA(6)
TYPED_MENU_LAMBDA(7) TYPED_MENU_LAMBDA(8) TYPED_MENU_LAMBDA(9) TYPED_MENU_LAMBDA(10)

// (m^2(p0 + p1), m^2(p1 + p2)): the Dalitz variables of the reference's phsp_basic example.
template <size_t N> struct dalitz_lambda;
#define DALITZ_LAMBDA(NN)                                                      \
    template <> struct dalitz_lambda<NN> {                                     \
        static auto make() {                                                   \
            return hydra::wrap_lambda([](TLAM_ARGS_##NN) {                     \
                HV arr[NN] = {LAM_NAMES_##NN};                                 \
                return hydra::make_tuple((arr[0] + arr[1]).mass2(),            \
                                         (arr[1] + arr[2]).mass2());           \
            });                                                                \
        }                                                                      \
    };
DALITZ_LAMBDA(3) DALITZ_LAMBDA(4) DALITZ_LAMBDA(5) DALITZ_LAMBDA(6)
DALITZ_LAMBDA(7) DALITZ_LAMBDA(8) DALITZ_LAMBDA(9) DALITZ_LAMBDA(10)

template <typename T>
void write_bin(const char* path, std::vector<T> const& v)
{
    FILE* fp = std::fopen(path, "wb");
    if (!fp) { std::perror(path); std::exit(3); }
    if (!v.empty() && std::fwrite(v.data(), sizeof(T), v.size(), fp) != v.size()) {
        std::perror("fwrite"); std::exit(3);
    }
    std::fclose(fp);
}

struct Args {
    std::string mode;
    int N = 0, engine = 0;
    long long seed = 0;
    size_t n = 0;
    double M = 0;
    double m[10] = {0};
    FSpec f{0, 0, 1, 0.0, 0.0};
    unsigned long long useed = 0x180ec6d33cfd0abaULL;
    double mom[3] = {0, 0, 0};
    unsigned long long fseed = 0x39abdc4529b1661cULL;
    double fmax = -1.0;
    size_t grid[2] = {0, 0};
    double lo[2] = {0, 0}, hi[2] = {0, 0};
    unsigned long long rseed = 0;
    const char* out = nullptr;
    int reps = 1;
};

template <size_t N, typename GRND>
void run_rng(Args const& a)
{
    const size_t nw = 3 * N - 4;
    std::vector<unsigned long long> words(a.n * nw);
    for (size_t evt = 0; evt < a.n; ++evt) {
        GRND eng(static_cast<size_t>(a.seed));
        eng.discard(evt + 3 * N);
        for (size_t k = 0; k < nw; ++k) words[evt * nw + k] = eng();
    }
    write_bin(a.out, words);
}

template <size_t N, typename GRND>
hydra::PhaseSpace<N, GRND> make_phsp(Args const& a)
{
    double masses[N];
    for (size_t i = 0; i < N; ++i) masses[i] = a.m[i];
    hydra::PhaseSpace<N, GRND> phsp(a.M, masses);
    if (a.seed != -1) phsp.SetSeed(static_cast<hydra::GInt_t>(a.seed));
    return phsp;
}

template <size_t N, typename GRND>
void run_gen(Args const& a)
{
    typedef typename ptypes<N>::type PT;
    auto phsp = make_phsp<N, GRND>(a);
    double masses[N];
    for (size_t i = 0; i < N; ++i) masses[i] = a.m[i];
    double E = std::sqrt(a.M * a.M + a.mom[0] * a.mom[0] + a.mom[1] * a.mom[1] + a.mom[2] * a.mom[2]);
    hydra::Vector4R mother(E, a.mom[0], a.mom[1], a.mom[2]);

    hydra::Decays<PT, hydra::host::sys_t> events(a.M, masses, a.n);
    phsp.Generate(mother, events);

    auto functor = menu_lambda<N>::make(a.f);
    hydra::multivector<hydra::tuple<WCol, FCol>, hydra::host::sys_t> evals(a.n);
    phsp.Evaluate(mother, evals, functor);

    auto wfun = events.GetEventWeightFunctor();
    typedef hydra::detail::FlagDaugthers<decltype(wfun)> tagger_t;
    tagger_t tagger(wfun, events.GetMaxWeight(), static_cast<size_t>(a.useed));

    // layout: [n*N*4 four-vectors][n gen weights][n functor values]
    //         [n recomputed weights][n flags][maxW_phsp, maxW_decays, ECM, seed, n_unweighted,
    //          default-seed bits]
    std::vector<double> out;
    out.reserve(a.n * (4 * N + 4) + 5);
    for (size_t i = 0; i < a.n; ++i) {
        auto ev = events[i];
        hydra::Vector4R p[N];
        hydra::detail::assignTupleToArray(ev, p);
        for (size_t k = 0; k < N; ++k)
            for (int c = 0; c < 4; ++c) out.push_back(p[k].get(c));
    }
    for (size_t i = 0; i < a.n; ++i) out.push_back(hydra::get<0>(evals[i]));
    for (size_t i = 0; i < a.n; ++i) out.push_back(hydra::get<1>(evals[i]));
    for (size_t i = 0; i < a.n; ++i) out.push_back(wfun(events[i]));
    for (size_t i = 0; i < a.n; ++i)
        out.push_back(tagger(hydra::make_tuple(i, events[i])) ? 1.0 : 0.0);
    out.push_back(phsp.GetMaxWeight());
    out.push_back(events.GetMaxWeight());
    out.push_back(phsp.GetECM());
    out.push_back(static_cast<double>(phsp.GetSeed()));
    auto kept = events.Unweight(static_cast<size_t>(a.useed));
    out.push_back(static_cast<double>(kept.size()));
    // default seed of the constructor (PhaseSpace.inl:44,64), bit pattern stored in a double slot
    size_t dseed = 1;
    dseed *= (1 + hydra::detail::hash_range(&masses[0], &masses[0] + N));
    double dbits;
    std::memcpy(&dbits, &dseed, sizeof(dbits));
    out.push_back(dbits);
    write_bin(a.out, out);
}

template <size_t N, typename GRND>
void run_avg(Args const& a)
{
    auto phsp = make_phsp<N, GRND>(a);
    hydra::Vector4R mother(a.M, 0.0, 0.0, 0.0);
    auto functor = menu_lambda<N>::make(a.f);
    auto r = phsp.AverageOn(hydra::device::sys, mother, functor, a.n);
    std::vector<double> out{r.first, r.second};
    write_bin(a.out, out);
}

// Threads the OMP backend uses (1 for the sequential build).
int ref_threads()
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

template <size_t N, typename GRND>
void run_time(Args const& a)
{
    typedef typename ptypes<N>::type PT;
    auto phsp = make_phsp<N, GRND>(a);
    double masses[N];
    for (size_t i = 0; i < N; ++i) masses[i] = a.m[i];
    hydra::Vector4R mother(a.M, 0.0, 0.0, 0.0);
    auto functor = menu_lambda<N>::make(a.f);
    hydra::Decays<PT, hydra::device::sys_t> events(a.M, masses, a.n);
    double best_gen = 1e30, best_avg = 1e30;
    std::vector<double> gen_s, avg_s;
    for (int r = 0; r < a.reps; ++r) {
        auto t0 = std::chrono::steady_clock::now();
        phsp.Generate(mother, events);
        auto t1 = std::chrono::steady_clock::now();
        auto s = phsp.AverageOn(hydra::device::sys, mother, functor, a.n);
        auto t2 = std::chrono::steady_clock::now();
        (void)s;
        gen_s.push_back(std::chrono::duration<double>(t1 - t0).count());
        avg_s.push_back(std::chrono::duration<double>(t2 - t1).count());
        best_gen = std::min(best_gen, gen_s.back());
        best_avg = std::min(best_avg, avg_s.back());
    }
    // best times, then every repetition in order (generate_all / average_all)
    std::printf("{\"n\": %zu, \"N\": %zu, \"generate_s\": %.6f, \"average_s\": %.6f, \"threads\": %d",
                a.n, N, best_gen, best_avg, ref_threads());
    for (int k = 0; k < 2; ++k) {
        const std::vector<double>& v = k ? avg_s : gen_s;
        std::printf(", \"%s\": [", k ? "average_all" : "generate_all");
        for (size_t r = 0; r < v.size(); ++r) std::printf("%s%.6f", r ? ", " : "", v[r]);
        std::printf("]");
    }
    std::printf("}\n");
}

// Per-event mothers for the *Mothers variants: mass M(1 + 0.05 sin(0.7 i)), momentum
// (0.3 sin(0.1 i), -0.7 cos(0.37 i), 1.1 sin(0.23 i + 1)) GeV, on shell.
std::vector<hydra::Vector4R> make_mothers(double M, size_t n)
{
    std::vector<hydra::Vector4R> v(n);
    for (size_t i = 0; i < n; ++i) {
        const double mi = M * (1.0 + 0.05 * std::sin(0.7 * i));
        const double px = 0.3 * std::sin(0.1 * i), py = -0.7 * std::cos(0.37 * i), pz = 1.1 * std::sin(0.23 * i + 1.0);
        v[i] = hydra::Vector4R(std::sqrt(mi * mi + px * px + py * py + pz * pz), px, py, pz);
    }
    return v;
}

// Generate(mothers, daughters) (DecayMothers), AverageOn(begin, end, functor) (AverageMothers) and
// Evaluate(mothers, result, functor) (EvalMothers).
// layout: [n*4 mothers][n*N*4 Generate four-vectors][n Evaluate weights][n Evaluate functor values]
//         [mean, err of AverageOn]
template <size_t N, typename GRND>
void run_mothers(Args const& a)
{
    typedef typename ptypes<N>::type PT;
    auto phsp = make_phsp<N, GRND>(a);
    double masses[N];
    for (size_t i = 0; i < N; ++i) masses[i] = a.m[i];
    auto mothers_v = make_mothers(a.M, a.n);
    hydra::multivector<hydra::tuple<D0>, hydra::host::sys_t> mothers(a.n);
    for (size_t i = 0; i < a.n; ++i) hydra::get<0>(mothers[i]) = mothers_v[i];
    hydra::Decays<PT, hydra::host::sys_t> events(a.M, masses, a.n);
    auto mbegin = mothers.begin(hydra::placeholders::_0);
    auto mend = mothers.end(hydra::placeholders::_0);
    phsp.Generate(mbegin, mend, events.begin());
    // AverageMothers / EvalMothers hand the functor (mother, daughter 0, ..., daughter N-1)
    auto functor = menu_lambda<N + 1>::make(a.f);
    hydra::multivector<hydra::tuple<WCol, FCol>, hydra::host::sys_t> evals(a.n);
    // the range overload (PhaseSpace.inl:331-348); the iterator overload (:302-309) passes
    // fMotherMass to EvalMothers' constructor and does not compile
    phsp.Evaluate(hydra::make_range(mbegin, mend), evals, functor);
    auto avg = phsp.AverageOn(mbegin, mend, functor);
    std::vector<double> out;
    for (size_t i = 0; i < a.n; ++i)
        for (int c = 0; c < 4; ++c) out.push_back(mothers_v[i].get(c));
    for (size_t i = 0; i < a.n; ++i) {
        auto ev = events[i];
        hydra::Vector4R p[N];
        hydra::detail::assignTupleToArray(ev, p);
        for (size_t k = 0; k < N; ++k)
            for (int c = 0; c < 4; ++c) out.push_back(p[k].get(c));
    }
    for (size_t i = 0; i < a.n; ++i) out.push_back(hydra::get<0>(evals[i]));
    for (size_t i = 0; i < a.n; ++i) out.push_back(hydra::get<1>(evals[i]));
    out.push_back(avg.first);
    out.push_back(avg.second);
    write_bin(a.out, out);
}

template <size_t N>
void push_events(std::vector<double>& out, hydra::Decays<typename ptypes<N>::type, hydra::host::sys_t>& ev, size_t n)
{
    for (size_t i = 0; i < n; ++i) {
        auto t = ev[i];
        hydra::Vector4R p[N];
        hydra::detail::assignTupleToArray(t, p);
        for (size_t k = 0; k < N; ++k)
            for (int c = 0; c < 4; ++c) out.push_back(p[k].get(c));
    }
}

template <typename Tup, size_t... K>
void push_range_event(std::vector<double>& out, Tup const& t, std::index_sequence<K...>)
{
    out.push_back(hydra::get<0>(t));
    hydra::Vector4R p[sizeof...(K)] = {hydra::get<K + 1>(t)...};
    for (size_t k = 0; k < sizeof...(K); ++k)
        for (int c = 0; c < 4; ++c) out.push_back(p[k].get(c));
}

// Consumers of a stored sample and the lazy generator.
// layout: [n*N*4 Generate four-vectors (mother at rest)]
//         [n PhaseSpaceReweight(functor) values]
//         [n*N*4 after Unweight(functor, -1, fseed)] [kept]
//         [n*N*4 after Unweight(functor, fmax, fseed)] [kept]
//         [g0*g1+2 DenseHistogram<double,2> of (m2(p0+p1), m2(p1+p2)) weighted by PhaseSpaceWeight]
//              (N >= 3 only)
//         [n*(1+4N) phase_space_range(mother (E, mx, my, mz) of mass M, masses, rseed, n): weight, p...]
//         [mean, err of PhaseSpaceIntegrator<N>(M, masses, n).Integrate(functor), its seed bits]
template <size_t N, typename GRND>
void run_extras(Args const& a)
{
    typedef typename ptypes<N>::type PT;
    auto phsp = make_phsp<N, GRND>(a);
    double masses[N];
    std::array<double, N> amasses;
    for (size_t i = 0; i < N; ++i) amasses[i] = masses[i] = a.m[i];
    hydra::Vector4R rest(a.M, 0.0, 0.0, 0.0);
    auto functor = menu_lambda<N>::make(a.f);
    auto tfunctor = typed_menu_lambda<N>::make(a.f);
    std::vector<double> out;

    hydra::Decays<PT, hydra::host::sys_t> events(a.M, masses, a.n);
    phsp.Generate(rest, events);
    push_events<N>(out, events, a.n);
    auto rw = events.GetEventWeightFunctor(tfunctor);
    for (size_t i = 0; i < a.n; ++i) out.push_back(rw(events[i]));

    for (int pass = 0; pass < 2; ++pass) {
        hydra::Decays<PT, hydra::host::sys_t> ev2(a.M, masses, a.n);
        phsp.Generate(rest, ev2);
        auto kept = ev2.Unweight(tfunctor, pass == 0 ? -1.0 : a.fmax, static_cast<size_t>(a.fseed));
        push_events<N>(out, ev2, a.n);
        out.push_back(static_cast<double>(kept.size()));
    }

    if constexpr (N >= 3) {
        auto dalitz_variables = events | dalitz_lambda<N>::make();
        auto dalitz_weights = events | events.GetEventWeightFunctor();
        auto hist = hydra::make_dense_histogram<double, 2>(hydra::host::sys, {a.grid[0], a.grid[1]},
                                                            {a.lo[0], a.lo[1]}, {a.hi[0], a.hi[1]},
                                                            dalitz_variables, dalitz_weights);
        for (auto it = hist.begin(); it != hist.end(); ++it) out.push_back(*it);
    }

    {
        const double E = std::sqrt(a.M * a.M + a.mom[0] * a.mom[0] + a.mom[1] * a.mom[1] + a.mom[2] * a.mom[2]);
        hydra::Vector4R mother(E, a.mom[0], a.mom[1], a.mom[2]);
        auto range = hydra::phase_space_range(mother, amasses, static_cast<size_t>(a.rseed), a.n);
        auto first = range.begin();
        for (size_t i = 0; i < a.n; ++i) push_range_event(out, first[i], std::make_index_sequence<N>{});
    }

    {
        hydra::PhaseSpaceIntegrator<N, hydra::host::sys_t, GRND> integ(a.M, masses, a.n);
        auto r = integ.Integrate(functor);
        out.push_back(r.first);
        out.push_back(r.second);
        // the integrator's generator keeps the default seed; its bit pattern in a double slot
        size_t dseed = 1;
        dseed *= (1 + hydra::detail::hash_range(&masses[0], &masses[0] + N));
        double dbits;
        std::memcpy(&dbits, &dseed, sizeof(dbits));
        out.push_back(dbits);
    }
    write_bin(a.out, out);
}

// Functors written as the reference's phase-space examples write them: a wrap_lambda over
// declarg arguments (positional conversion from the event's Vector4R tuple) calling
// hydra::CosHelicityAngle, and two invariant masses.
// layout: [mean, err of AverageOn(device::sys, rest, cos_theta, n)]
//         [n rows of Evaluate(rest, (w, m13^2, m23^2, cos_theta))]
//         [n*3*4 four-vectors after Unweight(1 + cos_theta^2 over the Decays' typed columns, -1, fseed)] [kept]
template <size_t N, typename GRND>
void run_functors(Args const& a)
{
    if constexpr (N != 3) {
        std::fprintf(stderr, "functors mode needs N = 3\n");
        std::exit(2);
    } else {
        typedef typename ptypes<N>::type PT;
        auto phsp = make_phsp<N, GRND>(a);
        double masses[N];
        for (size_t i = 0; i < N; ++i) masses[i] = a.m[i];
        hydra::Vector4R rest(a.M, 0.0, 0.0, 0.0);
        auto cos_theta = hydra::wrap_lambda([](FJpsi j, FKaon k, FPion p) {
            hydra::CosHelicityAngle h;
            return h(j + k + p, k + p, k);
        });
        auto m13 = hydra::wrap_lambda([](FJpsi j, FKaon k, FPion p) { return (j + p).mass2(); });
        auto m23 = hydra::wrap_lambda([](FJpsi j, FKaon k, FPion p) { return (k + p).mass2(); });
        std::vector<double> out;
        auto r = phsp.AverageOn(hydra::device::sys, rest, cos_theta, a.n);
        out.push_back(r.first);
        out.push_back(r.second);
        hydra::multivector<hydra::tuple<double, double, double, double>, hydra::host::sys_t> data(a.n);
        phsp.Evaluate(rest, data, m13, m23, cos_theta);
        for (size_t i = 0; i < a.n; ++i) {
            auto row = data[i];
            out.push_back(hydra::get<0>(row));
            out.push_back(hydra::get<1>(row));
            out.push_back(hydra::get<2>(row));
            out.push_back(hydra::get<3>(row));
        }
        auto u = hydra::wrap_lambda([](D0 j, D1 k, D2 p) {
            hydra::CosHelicityAngle h;
            const double c = h(j + k + p, k + p, k);
            return 1.0 + c * c;
        });
        hydra::Decays<PT, hydra::host::sys_t> ev(a.M, masses, a.n);
        phsp.Generate(rest, ev);
        auto kept = ev.Unweight(u, -1.0, static_cast<size_t>(a.fseed));
        push_events<N>(out, ev, a.n);
        out.push_back(static_cast<double>(kept.size()));
        write_bin(a.out, out);
    }
}

template <size_t N, typename GRND>
void dispatch_mode(Args const& a)
{
    if (a.mode == "rng") run_rng<N, GRND>(a);
    else if (a.mode == "gen") run_gen<N, GRND>(a);
    else if (a.mode == "avg") run_avg<N, GRND>(a);
    else if (a.mode == "time") run_time<N, GRND>(a);
    else if (a.mode == "mothers") run_mothers<N, GRND>(a);
    else if (a.mode == "extras") run_extras<N, GRND>(a);
    else if (a.mode == "functors") run_functors<N, GRND>(a);
    else { std::fprintf(stderr, "unknown mode %s\n", a.mode.c_str()); std::exit(2); }
}

template <size_t N>
void dispatch_engine(Args const& a)
{
    if (a.engine == 0) dispatch_mode<N, hydra::philox>(a);
    else dispatch_mode<N, hydra::default_random_engine>(a);
}

} // namespace

int main(int argc, char** argv)
{
    if (argc < 6) { std::fprintf(stderr, "see header for usage\n"); return 2; }
    Args a;
    int k = 1;
    a.mode = argv[k++];
    a.N = std::atoi(argv[k++]);
    a.engine = std::atoi(argv[k++]);
    {
        const char* sarg = argv[k++];
        a.seed = (sarg[0] == '-') ? std::strtoll(sarg, nullptr, 0)
                                  : static_cast<long long>(std::strtoull(sarg, nullptr, 0));
    }
    a.n = std::strtoull(argv[k++], nullptr, 0);
    if (a.N < 2 || a.N > 10) { std::fprintf(stderr, "N out of range\n"); return 2; }
    if (a.mode != "rng") {
        if (argc < k + 1 + a.N + 5) { std::fprintf(stderr, "missing args\n"); return 2; }
        a.M = std::strtod(argv[k++], nullptr);
        for (int i = 0; i < a.N; ++i) a.m[i] = std::strtod(argv[k++], nullptr);
        a.f.sel = std::atoi(argv[k++]);
        a.f.i = std::atoi(argv[k++]);
        a.f.j = std::atoi(argv[k++]);
        a.f.a = std::strtod(argv[k++], nullptr);
        a.f.b = std::strtod(argv[k++], nullptr);
        if (a.mode == "gen") {
            a.useed = std::strtoull(argv[k++], nullptr, 0);
            for (int c = 0; c < 3; ++c) a.mom[c] = std::strtod(argv[k++], nullptr);
        }
        if (a.mode == "functors") a.fseed = std::strtoull(argv[k++], nullptr, 0);
        if (a.mode == "extras") {
            if (argc < k + 12) { std::fprintf(stderr, "missing args\n"); return 2; }
            a.fseed = std::strtoull(argv[k++], nullptr, 0);
            a.fmax = std::strtod(argv[k++], nullptr);
            for (int c = 0; c < 2; ++c) a.grid[c] = std::strtoull(argv[k++], nullptr, 0);
            for (int c = 0; c < 2; ++c) a.lo[c] = std::strtod(argv[k++], nullptr);
            for (int c = 0; c < 2; ++c) a.hi[c] = std::strtod(argv[k++], nullptr);
            a.rseed = std::strtoull(argv[k++], nullptr, 0);
            for (int c = 0; c < 3; ++c) a.mom[c] = std::strtod(argv[k++], nullptr);
        }
    }
    if (a.mode == "time") a.reps = (k < argc) ? std::atoi(argv[k++]) : 3;
    else a.out = (k < argc) ? argv[k++] : "out.bin";
    switch (a.N) {
    case 2: dispatch_engine<2>(a); break;
    case 3: dispatch_engine<3>(a); break;
    case 4: dispatch_engine<4>(a); break;
    case 5: dispatch_engine<5>(a); break;
    case 6: dispatch_engine<6>(a); break;
    case 7: dispatch_engine<7>(a); break;
    case 8: dispatch_engine<8>(a); break;
    case 9: dispatch_engine<9>(a); break;
    case 10: dispatch_engine<10>(a); break;
    }
    return 0;
}
