// The FP32_FIX event body (hydra_gb300/csrc/genbod_f32.cuh) run on the CPU against the FP64 body of
// the same events (genbod.cuh, the reference's arithmetic operation for operation), over every event
// of a range, on all host threads.  Prints the largest four-vector error max_k |dp_k| / E and the
// largest weight error |dw| / w, with the events where they occur.  Test infrastructure: it sizes
// the precision contract of the float body on channels and event counts beyond the GPU tests
// (tests/test_f32_emulation.py; build with tests/f32_emulation/build.sh).
//
//   emulate_f32 N M m0,m1,... n_events [first] [engine 0 philox | 1 squares3] [seed] [form]
// form -1 (default): the library's choice for the channel; 0: the plain form; 1: the float-float
// boosts (N = 4..6; from N = 7 the full form is taken whatever is asked).
#include "cuda_shim.h"
#include "hydra_gb300/csrc/genbod_f32.cuh"

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <vector>

using namespace hps;

namespace {

struct Worst {
    double e4 = 0.0, ew = 0.0;
    uint64_t ev4 = 0, evw = 0;
    void take(const Worst& o)
    {
        if (o.e4 > e4) { e4 = o.e4; ev4 = o.ev4; }
        if (o.ew > ew) { ew = o.ew; evw = o.evw; }
    }
};

template <int N, int ENGINE>
Worst run(const DevChannel& ch, const DevChannelF& chf, uint64_t first, uint64_t n)
{
    Worst total;
#pragma omp parallel
    {
        Worst mine;
#pragma omp for schedule(static, 4096)
        for (long long i = 0; i < static_cast<long long>(n); ++i) {
            const uint64_t evt = first + static_cast<uint64_t>(i);
            double p64[N][4];
            const double w64 = f64::event<N, engine_of(ENGINE)>(ch, evt, p64);
            uint64_t w[3 * N - 4];
            event_words<N, engine_of(ENGINE)>(ch.key, evt, w);
            float p[N][4];
            const f32::EventWeight ew = f32::event_from_words<N, ENGINE>(ch, chf, w, p);
            Worst one;
            for (int k = 0; k < N; ++k)
                for (int c = 0; c < 4; ++c)
                    one.e4 = std::max(one.e4, std::fabs(static_cast<double>(p[k][c]) - p64[k][c]) / p64[k][0]);
            one.ew = w64 > 0.0 ? std::fabs(ew.weight - w64) / w64 : 0.0;
            one.ev4 = one.evw = evt;
            mine.take(one);
        }
#pragma omp critical
        total.take(mine);
    }
    return total;
}

template <int N>
Worst dispatch(const DevChannel& ch, const DevChannelF& chf, uint64_t first, uint64_t n, int engine)
{
    const bool ff = chf.precise != 0;
    if (engine == HPS_ENGINE_PHILOX)
        return ff ? run<N, kPhilox | kPreciseForm>(ch, chf, first, n) : run<N, kPhilox>(ch, chf, first, n);
    return ff ? run<N, kSquares3 | kPreciseForm>(ch, chf, first, n) : run<N, kSquares3>(ch, chf, first, n);
}

}  // namespace

int main(int argc, char** argv)
{
    if (argc < 5) {
        std::fprintf(stderr, "usage: %s N M m0,m1,... n_events [first] [engine] [seed]\n", argv[0]);
        return 2;
    }
    const int N = std::atoi(argv[1]);
    const double M = std::atof(argv[2]);
    std::vector<double> m;
    for (char* s = argv[3]; *s;) {
        m.push_back(std::strtod(s, &s));
        if (*s == ',') ++s;
    }
    if (N < 2 || N > HPS_MAX_DAUGHTERS || static_cast<int>(m.size()) != N) {
        std::fprintf(stderr, "N must be 2..10 with N masses\n");
        return 2;
    }
    const uint64_t n = std::strtoull(argv[4], nullptr, 0);
    const uint64_t first = argc > 5 ? std::strtoull(argv[5], nullptr, 0) : 0;
    const int engine = argc > 6 ? std::atoi(argv[6]) : HPS_ENGINE_PHILOX;
    hps_channel c{};
    c.n_daughters = N;
    c.engine = engine;
    c.seed = argc > 7 ? std::strtoull(argv[7], nullptr, 0) : 0x3039;
    double S = 0.0;
    for (int i = 0; i < N; ++i) {
        c.masses[i] = m[i];
        S += m[i];
    }
    // the constructor's ECM and maximum weight (PhaseSpace.inl:42-90), in its order
    c.ecm = M - S;
    double emmax = c.ecm + m[0], emmin = 0.0, wtmax = 1.0;
    for (int k = 1; k < N; ++k) {
        emmin += m[k - 1];
        emmax += m[k];
        wtmax *= f64::pdk(emmax, emmin, m[k]);
    }
    c.max_weight = 1.0 / wtmax;
    DevChannel ch;
    make_channel(c, ch);
    DevChannelF chf;
    f32::make_channel_f(c, chf);
    if (argc > 8 && std::atoi(argv[8]) >= 0) chf.precise = std::atoi(argv[8]) ? 1 : 0;
    Worst r;
    switch (N) {
    case 2: r = dispatch<2>(ch, chf, first, n, engine); break;
    case 3: r = dispatch<3>(ch, chf, first, n, engine); break;
    case 4: r = dispatch<4>(ch, chf, first, n, engine); break;
    case 5: r = dispatch<5>(ch, chf, first, n, engine); break;
    case 6: r = dispatch<6>(ch, chf, first, n, engine); break;
    case 7: r = dispatch<7>(ch, chf, first, n, engine); break;
    case 8: r = dispatch<8>(ch, chf, first, n, engine); break;
    case 9: r = dispatch<9>(ch, chf, first, n, engine); break;
    default: r = dispatch<10>(ch, chf, first, n, engine); break;
    }
    std::printf("{\"n_daughters\": %d, \"events\": %llu, \"first\": %llu, \"float_float_form\": %d, "
                "\"four_vectors\": %.4e, \"four_vectors_event\": %llu, \"weights\": %.4e, \"weights_event\": %llu}\n",
                N, static_cast<unsigned long long>(n), static_cast<unsigned long long>(first), chf.precise, r.e4,
                static_cast<unsigned long long>(r.ev4), r.ew, static_cast<unsigned long long>(r.evw));
    return 0;
}
