// Per-event-mother forms with a functor outside the C ABI's menu: a decay chain in the manner of
// the reference's phsp_chain example (B0 -> J/psi K pi, then J/psi -> mu+ mu- pi0 with the J/psi
// column as the mothers; three bodies, so that the pair masses vary from event to event),
// AverageOn(mothers, functor) and Evaluate(mothers, result, functor) once with the menu functor
// Mass2(1, 3) and once with the same quantity, m^2(mu+ pi0), as a hydra::wrap_lambda over
// (mother, mu+, mu-, pi0), compiled into the kernels by nvcc.  Prints one JSON object for
// tests/test_cpp_user_functors.py.
//
//   phsp_user_mothers N_EVENTS PRECISION
#include <hydra/Types.h>
#include <hydra/Vector4R.h>
#include <hydra/PhaseSpace.h>
#include <hydra/Decays.h>
#include <hydra/Function.h>
#include <hydra/Lambda.h>
#include <hydra/Placeholders.h>
#include <hydra/multivector.h>
#include <hydra/device/System.h>

#include <cstdio>
#include <cstdlib>
#include <vector>

declarg(Jpsi, hydra::Vector4R)
declarg(Kaon, hydra::Vector4R)
declarg(Pion, hydra::Vector4R)
declarg(MuonP, hydra::Vector4R)
declarg(MuonM, hydra::Vector4R)
declarg(Pi0, hydra::Vector4R)
declarg(W, double)
declarg(F, double)

using namespace hydra::placeholders;

static void print_array(const char* name, const std::vector<double>& v)
{
    std::printf("\"%s\": [", name);
    for (size_t i = 0; i < v.size(); ++i) std::printf("%s%.17g", i ? ", " : "", v[i]);
    std::printf("],\n");
}

int main(int argc, char** argv)
{
    if (argc != 3) {
        std::fprintf(stderr, "usage: %s N_EVENTS PRECISION\n", argv[0]);
        return 2;
    }
    const size_t n = std::strtoull(argv[1], nullptr, 10);
    const int precision = std::atoi(argv[2]);
    const double B0_mass = 5.27955, Jpsi_mass = 3.0969, K_mass = 0.493677, pi_mass = 0.13957,
                 mu_mass = 0.1056583745, pi0_mass = 0.1349768;
    hydra::Vector4R B0(B0_mass, 0.0, 0.0, 0.0);
    hydra::PhaseSpace<3, hydra::philox> ThreeBodyPHSP(B0_mass, {Jpsi_mass, K_mass, pi_mass});
    hydra::PhaseSpace<3, hydra::philox> DimuonPi0PHSP(Jpsi_mass, {mu_mass, mu_mass, pi0_mass});
    ThreeBodyPHSP.SetSeed(0x3039);
    DimuonPi0PHSP.SetSeed(0x3040);
    DimuonPi0PHSP.SetPrecision(precision);

    hydra::Decays<hydra::tuple<Jpsi, Kaon, Pion>, hydra::device::sys_t> ThreeBodyDecay(
        B0_mass, {Jpsi_mass, K_mass, pi_mass}, n);
    ThreeBodyPHSP.Generate(B0, ThreeBodyDecay);
    auto mothers = ThreeBodyDecay.GetDaugtherRange(_0);

    // m^2(mu+ pi0): indices of the menu count the mother as particle 0
    auto mup_pi0 = hydra::wrap_lambda([] __hydra_dual__(Jpsi jpsi, MuonP mup, MuonM mum, Pi0 pi0) {
        return (mup + pi0).mass2();
    });
    const auto avg_menu = DimuonPi0PHSP.AverageOn(mothers, hydra::hps_fn::Mass2(1, 3));
    const auto avg_user = DimuonPi0PHSP.AverageOn(mothers, mup_pi0);

    hydra::multivector<hydra::tuple<W, F>, hydra::device::sys_t> menu(n), user(n);
    DimuonPi0PHSP.Evaluate(mothers, menu, hydra::hps_fn::Mass2(1, 3));
    DimuonPi0PHSP.Evaluate(mothers, user, mup_pi0);

    std::printf("{\n");
    print_array("menu_w", menu.GetColumn(0));
    print_array("menu_f", menu.GetColumn(1));
    print_array("user_w", user.GetColumn(0));
    print_array("user_f", user.GetColumn(1));
    std::printf("\"avg_menu\": [%.17g, %.17g], \"avg_user\": [%.17g, %.17g]\n}\n", avg_menu.first, avg_menu.second,
                avg_user.first, avg_user.second);
    return 0;
}
