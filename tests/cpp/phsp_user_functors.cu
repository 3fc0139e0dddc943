// Drop-in test with functors outside the C ABI's menu, written as the reference's phase-space
// examples write them (examples/phase_space/phsp_averaging_functor.inl and
// phsp_evaluating_functor.inl): hydra::wrap_lambda over declarg arguments, hydra::CosHelicityAngle,
// AverageOn, Evaluate into a hydra::multivector, and Decays::Unweight(functor).  Compiled by nvcc
// against include/ (the functors are compiled into the library's kernel templates), linked with
// libhps.so.  Writes the same binary layout as oracle/ref_harness.cpp mode "functors":
//   [mean, err of AverageOn] [n rows (w, m13^2, m23^2, cos)] [n*3*4 four-vectors after Unweight] [kept]
//
//   phsp_user_functors ENGINE SEED N_EVENTS M m0 m1 m2 FSEED PRECISION OUT
#include <hydra/Types.h>
#include <hydra/Vector4R.h>
#include <hydra/PhaseSpace.h>
#include <hydra/Function.h>
#include <hydra/Lambda.h>
#include <hydra/Tuple.h>
#include <hydra/host/System.h>
#include <hydra/device/System.h>
#include <hydra/Decays.h>
#include <hydra/multivector.h>
#include <hydra/functions/CosHelicityAngle.h>

#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <vector>

declarg(Jpsi, hydra::Vector4R)
declarg(Kaon, hydra::Vector4R)
declarg(Pion, hydra::Vector4R)
declarg(Weight, double)
declarg(M13Sq, double)
declarg(M23Sq, double)
declarg(CosTheta, double)

using namespace hydra::arguments;

template <typename GRND>
int run(char** argv)
{
    const long seed = std::strtol(argv[2], nullptr, 0);
    const size_t n = std::strtoull(argv[3], nullptr, 0);
    const double M = std::strtod(argv[4], nullptr);
    const double masses[3] = {std::strtod(argv[5], nullptr), std::strtod(argv[6], nullptr),
                              std::strtod(argv[7], nullptr)};
    const size_t fseed = std::strtoull(argv[8], nullptr, 0);
    const int precision = std::atoi(argv[9]);

    auto cos_theta = hydra::wrap_lambda([] __hydra_dual__(Jpsi jpsi, Kaon kaon, Pion pion) {
        hydra::CosHelicityAngle h;
        return h(jpsi + kaon + pion, kaon + pion, kaon);
    });
    auto m13 = hydra::wrap_lambda([] __hydra_dual__(Jpsi jpsi, Kaon kaon, Pion pion) { return (jpsi + pion).mass2(); });
    auto m23 = hydra::wrap_lambda([] __hydra_dual__(Jpsi jpsi, Kaon kaon, Pion pion) { return (kaon + pion).mass2(); });

    hydra::Vector4R parent(M, 0.0, 0.0, 0.0);
    hydra::PhaseSpace<3, GRND> phsp{M, masses};
    phsp.SetSeed(static_cast<hydra::GInt_t>(seed));
    phsp.SetPrecision(precision);
    std::vector<double> out;

    auto r = phsp.AverageOn(hydra::device::sys, parent, cos_theta, n);
    out.push_back(r.first);
    out.push_back(r.second);

    hydra::multivector<hydra::tuple<Weight, M13Sq, M23Sq, CosTheta>, hydra::device::sys_t> dataset(n);
    phsp.Evaluate(parent, dataset, m13, m23, cos_theta);
    std::vector<double> col[4];
    for (int k = 0; k < 4; ++k) col[k] = dataset.GetColumn(k);
    for (size_t i = 0; i < n; ++i)
        for (int k = 0; k < 4; ++k) out.push_back(col[k][i]);

    // Unweight by a functor of the Decays' typed columns: 1 + cos^2
    auto u = hydra::wrap_lambda([] __hydra_dual__(Jpsi jpsi, Kaon kaon, Pion pion) {
        hydra::CosHelicityAngle h;
        const double c = h(jpsi + kaon + pion, kaon + pion, kaon);
        return 1.0 + c * c;
    });
    hydra::Decays<hydra::tuple<Jpsi, Kaon, Pion>, hydra::device::sys_t> events(M, masses, n);
    phsp.Generate(parent, events);
    const size_t kept = events.Unweight(u, -1.0, fseed);
    for (size_t i = 0; i < n; ++i) {
        auto ev = events[i];
        const hydra::Vector4R p[3] = {std::get<0>(ev), std::get<1>(ev), std::get<2>(ev)};
        for (int k = 0; k < 3; ++k)
            for (int c = 0; c < 4; ++c) out.push_back(p[k].get(c));
    }
    out.push_back(static_cast<double>(kept));

    FILE* fp = std::fopen(argv[10], "wb");
    if (!fp || std::fwrite(out.data(), sizeof(double), out.size(), fp) != out.size()) return 3;
    std::fclose(fp);
    // the reference example prints rows of the dataset like this
    std::cout << "<0>: " << dataset[0] << std::endl;
    return 0;
}

int main(int argc, char** argv)
{
    if (argc != 11) {
        std::fprintf(stderr, "usage: %s ENGINE SEED N M m0 m1 m2 FSEED PRECISION OUT\n", argv[0]);
        return 2;
    }
    return std::atoi(argv[1]) == 0 ? run<hydra::philox>(argv) : run<hydra::default_random_engine>(argv);
}
