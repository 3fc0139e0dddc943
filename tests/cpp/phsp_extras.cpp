// phsp_extras.cpp -- reference-style user code for what follows Generate in Hydra's phase-space
// examples, compiled against include/hydra/*.h (libhps): Unweight(functor, weight, seed) with
// its reweight values, the Dalitz histogram of phsp_basic, PhaseSpaceIntegrator and
// phase_space_range.  Prints one JSON object for tests/test_cpp_dropin.py to check.
#include <hydra/Types.h>
#include <hydra/Vector4R.h>
#include <hydra/PhaseSpace.h>
#include <hydra/PhaseSpaceIntegrator.h>
#include <hydra/Range.h>
#include <hydra/Decays.h>
#include <hydra/device/System.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

declarg(A, hydra::Vector4R)
declarg(B, hydra::Vector4R)
declarg(C, hydra::Vector4R)

static void print_array(const char* name, const std::vector<double>& v, bool comma = true)
{
    std::printf("\"%s\": [", name);
    for (size_t i = 0; i < v.size(); ++i) std::printf("%s%.17g", i ? ", " : "", v[i]);
    std::printf("]%s\n", comma ? "," : "");
}

template <typename D>
static std::vector<double> flatten(const D& ev)
{
    std::vector<double> out;
    for (size_t i = 0; i < ev.size(); ++i) {
        auto t = ev[i];
        const hydra::Vector4R p[3] = {std::get<0>(t), std::get<1>(t), std::get<2>(t)};
        for (int k = 0; k < 3; ++k)
            for (int c = 0; c < 4; ++c) out.push_back(p[k].get(c));
    }
    return out;
}

int main(int argc, char** argv)
{
    const size_t n = argc > 1 ? std::strtoull(argv[1], nullptr, 10) : 1024;
    const double fmax = argc > 2 ? std::strtod(argv[2], nullptr) : 50.0;
    const double P_mass = 5.27934;
    const double masses[3]{3.0969, 0.493677, 0.13957};
    const hydra::Vector4R Parent(P_mass, 0.0, 0.0, 0.0);
    hydra::PhaseSpace<3, hydra::philox> phsp{P_mass, masses};
    phsp.SetSeed(0x3039);
    const hydra::hps_fn::BW2 kstar(1, 2, 0.8955, 0.0473);

    std::printf("{\n");
    hydra::Decays<hydra::tuple<A, B, C>, hydra::device::sys_t> Events(P_mass, masses, n);
    phsp.Generate(Parent, Events);
    print_array("reweight", Events.GetEventWeights(kstar));

    const double lo[2] = {std::pow(masses[0] + masses[1], 2), std::pow(masses[1] + masses[2], 2)};
    const double hi[2] = {std::pow(P_mass - masses[2], 2), std::pow(P_mass - masses[0], 2)};
    print_array("hist", Events.DalitzHistogram({20, 25}, {lo[0], lo[1]}, {hi[0], hi[1]}));

    size_t kept = Events.Unweight(kstar);
    print_array("unw_max_four", flatten(Events));
    std::printf("\"unw_max_kept\": %zu,\n", kept);

    hydra::Decays<hydra::tuple<A, B, C>, hydra::host::sys_t> HostEvents(P_mass, masses, n);
    phsp.Generate(Parent, HostEvents);
    kept = HostEvents.Unweight(kstar, fmax);
    print_array("unw_fixed_four", flatten(HostEvents));
    std::printf("\"unw_fixed_kept\": %zu,\n", kept);

    hydra::PhaseSpaceIntegrator<3, hydra::device::sys_t, hydra::philox> integ(P_mass, masses, n);
    auto r = integ.Integrate(kstar);
    std::printf("\"integ_mean\": %.17g, \"integ_err\": %.17g,\n", r.first, r.second);

    const double mom[3] = {0.1, -0.2, 0.3};
    const hydra::Vector4R mover(std::sqrt(P_mass * P_mass + mom[0] * mom[0] + mom[1] * mom[1] + mom[2] * mom[2]),
                                mom[0], mom[1], mom[2]);
    auto range = hydra::phase_space_range(mover, std::array<double, 3>{masses[0], masses[1], masses[2]}, 321, n);
    std::vector<double> rw, rf;
    for (auto it = range.begin(); it != range.end(); ++it) {
        auto t = *it;
        rw.push_back(std::get<0>(t));
        const hydra::Vector4R p[3] = {std::get<1>(t), std::get<2>(t), std::get<3>(t)};
        for (int k = 0; k < 3; ++k)
            for (int c = 0; c < 4; ++c) rf.push_back(p[k].get(c));
    }
    print_array("range_w", rw);
    print_array("range_four", rf, false);
    std::printf("}\n");
    return 0;
}
