// phsp_dropin.cpp -- reference-style user code compiled against include/hydra/*.h (libhps).
// Written the way Hydra's examples/phase_space programs use the API: PhaseSpace<3> for
// B0 -> J/psi K pi at rest, Decays on the device and on the host, event weights, Unweight,
// AverageOn and Evaluate; prints one JSON object for tests/test_cpp_dropin.py to check.
#include <hydra/Types.h>
#include <hydra/Vector4R.h>
#include <hydra/PhaseSpace.h>
#include <hydra/Decays.h>
#include <hydra/multivector.h>
#include <hydra/host/System.h>
#include <hydra/device/System.h>

#include <cstdio>
#include <cstdlib>
#include <stdexcept>
#include <vector>

declarg(A, hydra::Vector4R)
declarg(B, hydra::Vector4R)
declarg(C, hydra::Vector4R)
declarg(Weight, double)
declarg(M12Sq, double)

static void print_array(const char* name, const std::vector<double>& v, bool comma = true)
{
    std::printf("\"%s\": [", name);
    for (size_t i = 0; i < v.size(); ++i) std::printf("%s%.17g", i ? ", " : "", v[i]);
    std::printf("]%s\n", comma ? "," : "");
}

int main(int argc, char** argv)
{
    const size_t n = argc > 1 ? std::strtoull(argv[1], nullptr, 10) : 256;
    const size_t n_avg = argc > 2 ? std::strtoull(argv[2], nullptr, 10) : 20000;
    double P_mass = 5.27934;
    double masses[3]{3.0969, 0.493677, 0.13957};
    hydra::Vector4R Parent(P_mass, 0.0, 0.0, 0.0);

    hydra::PhaseSpace<3, hydra::philox> phsp{P_mass, masses};
    phsp.SetSeed(0x3039);

    hydra::Decays<hydra::tuple<A, B, C>, hydra::device::sys_t> Events(P_mass, masses, n);
    phsp.Generate(Parent, Events);

    hydra::Decays<hydra::tuple<A, B, C>, hydra::host::sys_t> HostEvents(P_mass, masses, n);
    phsp.Generate(Parent, HostEvents);

    std::vector<double> four;
    bool host_equal = true;
    for (size_t i = 0; i < n; ++i) {
        auto ev = Events[i];
        auto hv = HostEvents[i];
        const hydra::Vector4R p[3] = {std::get<0>(ev), std::get<1>(ev), std::get<2>(ev)};
        const hydra::Vector4R h[3] = {std::get<0>(hv), std::get<1>(hv), std::get<2>(hv)};
        for (int k = 0; k < 3; ++k)
            for (int c = 0; c < 4; ++c) {
                four.push_back(p[k].get(c));
                host_equal = host_equal && (p[k].get(c) == h[k].get(c));
            }
    }
    const std::vector<double> wgen = Events.GetWeights();
    const std::vector<double> wrec = Events.GetEventWeights();
    auto res = phsp.AverageOn(hydra::device::sys, Parent, hydra::hps_fn::Mass2(0, 1), n_avg);

    hydra::multivector<hydra::tuple<Weight, M12Sq>, hydra::device::sys_t> dataset(n);
    phsp.Evaluate(Parent, dataset, hydra::hps_fn::Mass2(0, 1));

    const size_t kept = Events.Unweight();

    int errors_ok = 0;
    try { hydra::PhaseSpace<3> bad(P_mass, {3.0969, -0.493677, 0.13957}); } catch (std::invalid_argument const&) { errors_ok++; }
    try { hydra::PhaseSpace<3> bad(1.0, {3.0969, 0.493677, 0.13957}); } catch (std::runtime_error const&) { errors_ok++; }

    std::printf("{\n\"n\": %zu, \"max_weight\": %.17g, \"ecm\": %.17g, \"seed\": %d,\n", n, phsp.GetMaxWeight(),
                phsp.GetECM(), phsp.GetSeed());
    print_array("four", four);
    print_array("w_gen", wgen);
    print_array("w_rec", wrec);
    print_array("eval_w", dataset.GetColumn(0));
    print_array("eval_f", dataset.GetColumn(1));
    std::printf("\"avg_mean\": %.17g, \"avg_err\": %.17g, \"n_avg\": %zu,\n", res.first, res.second, n_avg);
    std::printf("\"unweighted\": %zu, \"host_equal\": %s, \"errors_ok\": %d\n}\n", kept, host_equal ? "true" : "false",
                errors_ok);
    return 0;
}
