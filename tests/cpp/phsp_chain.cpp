// phsp_chain.cpp -- a decay chain written the way the reference's phsp_chain example writes it,
// compiled against include/hydra/*.h (libhps): B0 -> J/psi K pi, then J/psi -> mu+ mu- with the
// J/psi column as the mothers (Generate(GetDaugtherRange(_0), events)); AverageOn and Evaluate
// over the same mothers.  Prints one JSON object for tests/test_cpp_dropin.py to check.
#include <hydra/Types.h>
#include <hydra/Vector4R.h>
#include <hydra/PhaseSpace.h>
#include <hydra/Decays.h>
#include <hydra/Placeholders.h>
#include <hydra/multivector.h>
#include <hydra/device/System.h>
#include <hydra/host/System.h>

#include <cstdio>
#include <cstdlib>
#include <vector>

declarg(Jpsi, hydra::Vector4R)
declarg(Kaon, hydra::Vector4R)
declarg(Pion, hydra::Vector4R)
declarg(MuonP, hydra::Vector4R)
declarg(MuonM, hydra::Vector4R)
declarg(W, double)
declarg(F, double)

using namespace hydra::placeholders;

static void print_array(const char* name, const std::vector<double>& v, bool comma = true)
{
    std::printf("\"%s\": [", name);
    for (size_t i = 0; i < v.size(); ++i) std::printf("%s%.17g", i ? ", " : "", v[i]);
    std::printf("]%s\n", comma ? "," : "");
}

template <typename D>
static std::vector<double> column_values(const D& ev, size_t k)
{
    std::vector<double> out(ev.size() * 4);
    cudaMemcpy(out.data(), ev.column(k), out.size() * 8, cudaMemcpyDeviceToHost);
    return out;
}

int main(int argc, char** argv)
{
    const size_t n = argc > 1 ? std::strtoull(argv[1], nullptr, 10) : 2048;
    const int precision = argc > 2 ? std::atoi(argv[2]) : HPS_PREC_FP64;
    const double B0_mass = 5.27955, Jpsi_mass = 3.0969, K_mass = 0.493677, pi_mass = 0.13957,
                 mu_mass = 0.1056583745;
    hydra::Vector4R B0(B0_mass, 0.0, 0.0, 0.0);
    hydra::PhaseSpace<3, hydra::philox> ThreeBodyPHSP(B0_mass, {Jpsi_mass, K_mass, pi_mass});
    hydra::PhaseSpace<2, hydra::philox> TwoBodyPHSP(Jpsi_mass, {mu_mass, mu_mass});
    ThreeBodyPHSP.SetSeed(0x3039);
    TwoBodyPHSP.SetSeed(0x3040);
    TwoBodyPHSP.SetPrecision(precision);

    hydra::Decays<hydra::tuple<Jpsi, Kaon, Pion>, hydra::device::sys_t> ThreeBodyDecay(
        B0_mass, {Jpsi_mass, K_mass, pi_mass}, n);
    hydra::Decays<hydra::tuple<MuonP, MuonM>, hydra::device::sys_t> TwoBodyDecay(Jpsi_mass, {mu_mass, mu_mass}, n);
    ThreeBodyPHSP.Generate(B0, ThreeBodyDecay);
    TwoBodyPHSP.Generate(ThreeBodyDecay.GetDaugtherRange(_0), TwoBodyDecay);

    // AverageOn over the same mothers: m^2(mu+ mu-) (indices count the mother as 0)
    auto avg = TwoBodyPHSP.AverageOn(ThreeBodyDecay.GetDaugtherRange(_0), hydra::hps_fn::Mass2(1, 2));
    hydra::multivector<hydra::tuple<W, F>, hydra::device::sys_t> evals(n);
    TwoBodyPHSP.Evaluate(ThreeBodyDecay.GetDaugtherRange(_0), evals, hydra::hps_fn::Mass2(0, 1));
    std::vector<double> ew(n), ef(n);
    cudaMemcpy(ew.data(), evals.column(0), n * 8, cudaMemcpyDeviceToHost);
    cudaMemcpy(ef.data(), evals.column(1), n * 8, cudaMemcpyDeviceToHost);

    std::printf("{\n");
    print_array("jpsi", column_values(ThreeBodyDecay, 0));
    print_array("mup", column_values(TwoBodyDecay, 0));
    print_array("mum", column_values(TwoBodyDecay, 1));
    print_array("eval_w", ew);
    print_array("eval_f", ef);
    std::printf("\"avg_mean\": %.17g, \"avg_err\": %.17g\n}\n", avg.first, avg.second);
    return 0;
}
