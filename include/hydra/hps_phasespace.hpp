/*
 * hps_phasespace.hpp -- C++ drop-in for Hydra's phase-space classes over the libhps C ABI.
 *
 * Mirrors the public interface of the reference for this path, so code written against
 *   hydra::PhaseSpace<N,GRND>   (hydra/PhaseSpace.h:86-346, hydra/detail/PhaseSpace.inl)
 *   hydra::Decays<tuple<P...>,Backend>  (hydra/Decays.h:67-651, hydra/detail/Decays.inl)
 *   hydra::Vector4R             (hydra/Vector4R.h:59-138)
 * compiles against these headers (put <repo>/include first on the include path, link with
 * libhps.so and the CUDA runtime).  Calls block like the reference's Thrust algorithms.
 * Constructors throw std::invalid_argument / std::runtime_error with the reference's messages;
 * CUDA failures throw std::system_error.
 *
 * Functors: what crosses the C ABI is the functor menu of hps.h (hydra::hps_fn::One,
 * Mass2(i, j), BW2(i, j, mass, width)); those calls need only a C++ compiler.  Any other functor
 * -- a hydra::wrap_lambda of a __hydra_dual__ lambda over declarg arguments, a CosHelicityAngle,
 * a struct with a __host__ __device__ call operator -- is compiled into the kernel templates of
 * detail/hps_user_kernels.cuh in the caller's translation unit, as the reference compiles it into
 * its Thrust functors; such a translation unit is built with nvcc for sm_103a
 * (--extended-lambda --expt-relaxed-constexpr, as the reference's own CUDA build).
 * hydra::Decays stores the generation-time weight beside the four-vectors (the reference
 * drops it, DecayMother.h:285); Unweight() reorders accepted events to the front.
 */
#ifndef HYDRA_HPS_PHASESPACE_HPP_
#define HYDRA_HPS_PHASESPACE_HPP_

#include <cuda_runtime_api.h>

#include <array>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <functional>
#include <initializer_list>
#include <ostream>
#include <stdexcept>
#include <string>
#include <system_error>
#include <tuple>
#include <type_traits>
#include <utility>
#include <vector>

#include "../hps.h"

// Host/device qualifiers of the reference (hydra/detail/Config.h), empty for a host compiler.
#if defined(__CUDACC__)
#define HPS_HD __host__ __device__
#ifndef __hydra_dual__
#define __hydra_dual__ __host__ __device__
#endif
#ifndef __hydra_host__
#define __hydra_host__ __host__
#endif
#ifndef __hydra_device__
#define __hydra_device__ __device__
#endif
#else
#define HPS_HD
#ifndef __hydra_dual__
#define __hydra_dual__
#endif
#ifndef __hydra_host__
#define __hydra_host__
#endif
#ifndef __hydra_device__
#define __hydra_device__
#endif
#endif

namespace hydra {

typedef double GReal_t;
typedef int GInt_t;
typedef unsigned int GUInt_t;
typedef long GLong_t;

template <typename... T> using tuple = std::tuple<T...>;
using std::get;
using std::make_tuple;

namespace detail {
template <typename T> struct is_std_tuple : std::false_type {};
template <typename... T> struct is_std_tuple<std::tuple<T...>> : std::true_type {};
template <typename T> struct always_false : std::false_type {};
}  // namespace detail

// ---------------------------------------------------------------------------------- Vector4R

class Vector4R {
public:
    Vector4R() = default;
    HPS_HD Vector4R(GReal_t e, GReal_t px, GReal_t py, GReal_t pz) : v_{e, px, py, pz} {}
    HPS_HD GReal_t get(GInt_t i) const { return v_[i]; }
    HPS_HD void set(GInt_t i, GReal_t d) { v_[i] = d; }
    HPS_HD void set(GReal_t e, GReal_t px, GReal_t py, GReal_t pz) { v_[0] = e; v_[1] = px; v_[2] = py; v_[3] = pz; }
    HPS_HD GReal_t mass2() const { return v_[0] * v_[0] - v_[1] * v_[1] - v_[2] * v_[2] - v_[3] * v_[3]; }
    HPS_HD GReal_t mass() const { const GReal_t m2 = mass2(); return m2 > 0.0 ? ::sqrt(m2) : 0.0; }
    HPS_HD GReal_t d3mag() const { return ::sqrt(v_[1] * v_[1] + v_[2] * v_[2] + v_[3] * v_[3]); }
    HPS_HD Vector4R& operator+=(const Vector4R& o) { for (int i = 0; i < 4; ++i) v_[i] += o.v_[i]; return *this; }
    HPS_HD Vector4R& operator-=(const Vector4R& o) { for (int i = 0; i < 4; ++i) v_[i] -= o.v_[i]; return *this; }
    HPS_HD Vector4R& operator*=(GReal_t c) { for (int i = 0; i < 4; ++i) v_[i] *= c; return *this; }
    HPS_HD friend Vector4R operator+(Vector4R a, const Vector4R& b) { return a += b; }
    HPS_HD friend Vector4R operator-(Vector4R a, const Vector4R& b) { return a -= b; }
    HPS_HD friend Vector4R operator*(GReal_t c, Vector4R a) { return a *= c; }
    HPS_HD friend Vector4R operator*(Vector4R a, GReal_t c) { return a *= c; }
    // Minkowski product E1 E2 - p1.p2
    HPS_HD friend GReal_t operator*(const Vector4R& a, const Vector4R& b)
    {
        return a.v_[0] * b.v_[0] - a.v_[1] * b.v_[1] - a.v_[2] * b.v_[2] - a.v_[3] * b.v_[3];
    }
    friend std::ostream& operator<<(std::ostream& s, const Vector4R& v)
    {
        return s << "(" << v.v_[0] << "," << v.v_[1] << "," << v.v_[2] << "," << v.v_[3] << ")";
    }
    HPS_HD const GReal_t* data() const { return v_; }

private:
    alignas(16) GReal_t v_[4] = {0.0, 0.0, 0.0, 0.0};
};

// A named argument type, as the reference's declarg (a Vector4R or a double with a name): it
// converts from and to its value type and hands the value out through operator().
namespace detail {
template <typename T, bool = std::is_class<T>::value>
struct arg_base : public T {
    arg_base() = default;
    HPS_HD arg_base(T const& x) : T(x) {}
    HPS_HD T& operator()() { return *this; }
    HPS_HD T const& operator()() const { return *this; }
};
template <typename T>
struct arg_base<T, false> {
    T value{};
    arg_base() = default;
    HPS_HD arg_base(T x) : value(x) {}
    HPS_HD operator T() const { return value; }
    HPS_HD T& operator()() { return value; }
    HPS_HD T const& operator()() const { return value; }
};
}  // namespace detail

// The namespace the reference's declarg puts its argument types in (code says
// `using namespace hydra::arguments;`); the types below are declared where declarg is used.
namespace arguments {}

#define declarg(NAME, TYPE)                                              \
    struct NAME : public ::hydra::detail::arg_base<TYPE> {               \
        using ::hydra::detail::arg_base<TYPE>::arg_base;                 \
        NAME() = default;                                                \
    };

// hydra::wrap_lambda (hydra/Lambda.h:528-531): a callable that takes either the lambda's own
// arguments or one tuple whose elements convert, in order, to them -- the form in which the
// phase-space algorithms hand an event to a functor.
template <typename L>
class Lambda {
public:
    explicit Lambda(L const& l) : fLambda(l) {}
    template <typename... T>
    HPS_HD auto operator()(std::tuple<T...> const& t) const
    {
        return call(t, std::index_sequence_for<T...>{});
    }
    template <typename A0, typename... T,
              typename std::enable_if<!detail::is_std_tuple<typename std::decay<A0>::type>::value, int>::type = 0>
    HPS_HD auto operator()(A0 const& a0, T const&... x) const
    {
        return fLambda(a0, x...);
    }
    HPS_HD L const& GetLambda() const { return fLambda; }

private:
    template <typename Tup, size_t... I>
    HPS_HD auto call(Tup const& t, std::index_sequence<I...>) const
    {
        return fLambda(std::get<I>(t)...);
    }
    L fLambda;
};

template <typename L>
Lambda<L> wrap_lambda(L const& l)
{
    return Lambda<L>(l);
}

// ----------------------------------------------------------------------------- back-ends

namespace detail {
// tuple<double, Vector4R x N>: an element of phase_space_range
template <size_t N, typename... T> struct tuple_cat_helper : tuple_cat_helper<N - 1, Vector4R, T...> {};
template <typename... T> struct tuple_cat_helper<0, T...> { typedef std::tuple<double, T...> type; };

struct HostBackend {};
struct DeviceBackend {};

inline void throw_status(hps_status st)
{
    if (st == HPS_OK) return;
    const std::string msg = hps_last_error();
    if (st == HPS_ERR_BAD_ARG) throw std::invalid_argument(msg);
    if (st == HPS_ERR_NO_ENERGY) throw std::runtime_error(msg);
    throw std::system_error(std::error_code(static_cast<int>(st), std::generic_category()), msg);
}

inline void throw_cuda(cudaError_t e, const char* what)
{
    if (e != cudaSuccess)
        throw std::system_error(std::error_code(static_cast<int>(e), std::generic_category()),
                                std::string(what) + ": " + cudaGetErrorString(e));
}

template <typename T> struct DeviceBuffer {
    T* p = nullptr;
    size_t n = 0;
    DeviceBuffer() = default;
    explicit DeviceBuffer(size_t count) { resize(count); }
    DeviceBuffer(const DeviceBuffer&) = delete;
    DeviceBuffer& operator=(const DeviceBuffer&) = delete;
    DeviceBuffer(DeviceBuffer&& o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
    DeviceBuffer& operator=(DeviceBuffer&& o) noexcept { std::swap(p, o.p); std::swap(n, o.n); return *this; }
    ~DeviceBuffer() { if (p) cudaFree(p); }
    void resize(size_t count)
    {
        if (p) { cudaFree(p); p = nullptr; }
        n = count;
        void* q = nullptr;
        if (count) throw_cuda(cudaMalloc(&q, count * sizeof(T)), "cudaMalloc");
        p = static_cast<T*>(q);
    }
};
}  // namespace detail

namespace host { typedef detail::HostBackend sys_t; static const sys_t sys{}; }
namespace device { typedef detail::DeviceBackend sys_t; static const sys_t sys{}; }

// ------------------------------------------------------------------------------- engines

// Engine tags: hydra::philox (EngineR123<Philox2x64>, 7 rounds) and
// hydra::default_random_engine (squares3), as the reference's typedefs name them.
namespace random { struct philox {}; struct squares3 {}; }
typedef random::philox philox;
typedef random::squares3 default_random_engine;

namespace detail {
template <typename GRND> struct engine_id;
template <> struct engine_id<random::philox> { static constexpr int32_t value = HPS_ENGINE_PHILOX; };
template <> struct engine_id<random::squares3> { static constexpr int32_t value = HPS_ENGINE_SQUARES3; };
}  // namespace detail

// ------------------------------------------------------------------------------ functors

namespace hps_fn {
struct One { hps_functor f{HPS_FN_ONE, 0, 1, 0, 0.0, 0.0}; };
struct Mass2 { hps_functor f; Mass2(int i, int j) : f{HPS_FN_MASS2, i, j, 0, 0.0, 0.0} {} };
struct BW2 { hps_functor f; BW2(int i, int j, double m, double w) : f{HPS_FN_BW2, i, j, 0, m, w} {} };
template <typename F> struct is_menu : std::false_type {};
template <> struct is_menu<One> : std::true_type {};
template <> struct is_menu<Mass2> : std::true_type {};
template <> struct is_menu<BW2> : std::true_type {};
}  // namespace hps_fn

namespace detail {
template <typename... F> struct all_menu : std::true_type {};
template <typename F, typename... R>
struct all_menu<F, R...> : std::integral_constant<bool, hps_fn::is_menu<F>::value && all_menu<R...>::value> {};
}  // namespace detail

}  // namespace hydra

#if defined(__CUDACC__)
#include "detail/hps_user_kernels.cuh"
#endif

namespace hydra {

// --------------------------------------------------------------------------------- Decays

// Column selectors of the reference (hydra/Placeholders.h): hydra::placeholders::_0 ... _9.
namespace placeholders {
template <unsigned I> struct placeholder { static constexpr unsigned index = I; };
static const placeholder<0> _0{}; static const placeholder<1> _1{}; static const placeholder<2> _2{};
static const placeholder<3> _3{}; static const placeholder<4> _4{}; static const placeholder<5> _5{};
static const placeholder<6> _6{}; static const placeholder<7> _7{}; static const placeholder<8> _8{};
static const placeholder<9> _9{};
}  // namespace placeholders

// One daughter column of a Decays, as Decays::GetDaugtherRange(_k) hands it out (a range of
// Vector4R): here its raw pointer ({E,px,py,pz} per event), its length and where it lives.
struct DaughterRange {
    const double* data;
    size_t n;
    bool on_device;
    size_t size() const { return n; }
};

template <typename Tuple, typename Backend> class Decays;

template <typename... Particles, typename Backend>
class Decays<hydra::tuple<Particles...>, Backend> {
public:
    enum { nparticles = sizeof...(Particles) };
    static_assert(nparticles >= 2 && nparticles <= HPS_MAX_DAUGHTERS, "2..10 daughters");
    typedef hydra::tuple<Particles...> value_type;
    static constexpr bool on_device = std::is_same<Backend, detail::DeviceBackend>::value;

    Decays(double motherMass, std::array<double, nparticles> const& masses, size_t nentries = 0)
        : fMotherMass(motherMass)
    {
        for (size_t i = 0; i < nparticles; ++i) fMasses[i] = masses[i];
        init(nentries);
    }
    Decays(double motherMass, const double (&masses)[nparticles], size_t nentries = 0) : fMotherMass(motherMass)
    {
        for (size_t i = 0; i < nparticles; ++i) fMasses[i] = masses[i];
        init(nentries);
    }

    size_t size() const { return fN; }
    bool empty() const { return fN == 0; }
    double GetMaxWeight() const { return fMaxWeight; }
    double GetMotherMass() const { return fMotherMass; }
    const std::array<double, nparticles> GetMasses() const
    {
        std::array<double, nparticles> a;
        for (size_t i = 0; i < nparticles; ++i) a[i] = fMasses[i];
        return a;
    }

    void resize(size_t n) { init(n); }

    // Event i as a tuple of daughters (copied from the device for a device Decays).
    value_type operator[](size_t i) const
    {
        Vector4R p[nparticles];
        for (size_t k = 0; k < nparticles; ++k) {
            double v[4];
            if (on_device)
                detail::throw_cuda(cudaMemcpy(v, column(k) + 4 * i, sizeof(v), cudaMemcpyDeviceToHost), "cudaMemcpy");
            else
                for (int c = 0; c < 4; ++c) v[c] = column(k)[4 * i + c];
            p[k].set(v[0], v[1], v[2], v[3]);
        }
        return make(p, std::index_sequence_for<Particles...>{});
    }

    // Decays::GetDaugtherRange(placeholder) (hydra/Decays.h:279-284): daughter I's column, e.g.
    // the mothers of the next step of a decay chain (examples/phase_space/phsp_chain.inl:236).
    template <unsigned I>
    DaughterRange GetDaugtherRange(placeholders::placeholder<I>) const
    {
        static_assert(I < nparticles, "no such daughter");
        return DaughterRange{column(I), fN, on_device};
    }

    // Raw column k ({E,px,py,pz} per event) and the weight column.
    double* column(size_t k) { return on_device ? fDevCols[k].p : fHostCols[k].data(); }
    const double* column(size_t k) const { return on_device ? fDevCols[k].p : fHostCols[k].data(); }
    double* weights() { return on_device ? fDevW.p : fHostW.data(); }

    // Generation-time weights (what the reference's Generate computes and drops).
    std::vector<double> GetWeights() const
    {
        std::vector<double> w(fN);
        if (on_device && fN)
            detail::throw_cuda(cudaMemcpy(w.data(), fDevW.p, fN * 8, cudaMemcpyDeviceToHost), "cudaMemcpy");
        else if (fN)
            w = fHostW;
        return w;
    }

    // Events | Events.GetEventWeightFunctor(): PhaseSpaceWeight recomputed from the stored
    // four-vectors (Decays.inl:215-231), evaluated eagerly.
    std::vector<double> GetEventWeights() const
    {
        std::vector<double> w(fN);
        if (!fN) return w;
        with_device_columns([&](const double* const* cols) {
            detail::DeviceBuffer<double> out(fN);
            detail::throw_status(hps_event_weights(nparticles, fMasses, fMaxWeight, fN, cols, out.p, nullptr));
            detail::throw_cuda(cudaMemcpy(w.data(), out.p, fN * 8, cudaMemcpyDeviceToHost), "cudaMemcpy");
        });
        return w;
    }

    // Decays::Unweight(seed) (Decays.inl:415-455): hit-or-miss on PhaseSpaceWeight/max weight;
    // accepted events move to the front in their original order; returns how many.
    size_t Unweight(size_t seed = 0x180ec6d33cfd0abaULL)
    {
        if (!fN) return 0;
        std::vector<uint8_t> flags(fN);
        with_device_columns([&](const double* const* cols) {
            detail::DeviceBuffer<uint8_t> f(fN);
            detail::throw_status(hps_unweight_flags(nparticles, fMasses, fMaxWeight, fN, cols, seed, 0, f.p, nullptr));
            if (on_device) {
                compact_device(f.p);       // flags and the stable partition stay on the device
                return;
            }
            detail::throw_cuda(cudaMemcpy(flags.data(), f.p, fN, cudaMemcpyDeviceToHost), "cudaMemcpy");
        });
        if (on_device) return fKept;
        return partition_host(flags);
    }

    // Events | Events.GetEventWeightFunctor(functor) (Decays.h:243-250): PhaseSpaceWeight times
    // the functor, evaluated eagerly (PhaseSpaceReweight, Decays.inl:372-386).
    template <typename Functor, typename std::enable_if<!hps_fn::is_menu<Functor>::value, int>::type = 0>
    std::vector<double> GetEventWeights(Functor const& functor) const
    {
        std::vector<double> w(fN);
        if (!fN) return w;
        with_device_columns([&](const double* const* cols) {
            detail::DeviceBuffer<double> out(fN), mx(1);
            user_reweight(cols, functor, out.p, mx.p);
            detail::throw_cuda(cudaMemcpy(w.data(), out.p, fN * 8, cudaMemcpyDeviceToHost), "cudaMemcpy");
        });
        return w;
    }

    template <typename Functor, typename std::enable_if<hps_fn::is_menu<Functor>::value, int>::type = 0>
    std::vector<double> GetEventWeights(Functor const& functor) const
    {
        std::vector<double> w(fN);
        if (!fN) return w;
        with_device_columns([&](const double* const* cols) {
            detail::DeviceBuffer<double> out(fN);
            detail::throw_status(hps_reweight(nparticles, fMasses, fMaxWeight, &functor.f, fN, cols, out.p, nullptr,
                                              nullptr));
            detail::throw_cuda(cudaMemcpy(w.data(), out.p, fN * 8, cudaMemcpyDeviceToHost), "cudaMemcpy");
        });
        return w;
    }

    // Decays::Unweight(functor, weight, seed) (Decays.inl:458-511): hit-or-miss on
    // PhaseSpaceWeight * functor against weight, or against the largest such value when
    // weight <= 0; accepted events move to the front in their original order; returns how many.
    template <typename Functor, typename std::enable_if<!hps_fn::is_menu<Functor>::value, int>::type = 0>
    size_t Unweight(Functor const& functor, double weight = -1.0, size_t seed = 0x39abdc4529b1661cULL)
    {
        if (!fN) return 0;
        std::vector<uint8_t> flags(fN);
        detail::DeviceBuffer<uint8_t> f(fN);
        with_device_columns([&](const double* const* cols) {
            detail::DeviceBuffer<double> rw(fN), mx(1);
            user_reweight(cols, functor, rw.p, mx.p);
            detail::throw_status(hps_weight_flags(fN, rw.p, weight, weight > 0.0 ? nullptr : mx.p, seed, 0, f.p,
                                                  nullptr));
            if (on_device) {
                compact_device(f.p);
                return;
            }
            detail::throw_cuda(cudaMemcpy(flags.data(), f.p, fN, cudaMemcpyDeviceToHost), "cudaMemcpy");
        });
        if (on_device) return fKept;
        return partition_host(flags);
    }

    template <typename Functor, typename std::enable_if<hps_fn::is_menu<Functor>::value, int>::type = 0>
    size_t Unweight(Functor const& functor, double weight = -1.0, size_t seed = 0x39abdc4529b1661cULL)
    {
        if (!fN) return 0;
        std::vector<uint8_t> flags(fN);
        detail::DeviceBuffer<uint8_t> f(fN);
        with_device_columns([&](const double* const* cols) {
            detail::DeviceBuffer<double> rw(fN);
            detail::DeviceBuffer<double> mx(1);
            detail::throw_status(hps_reweight(nparticles, fMasses, fMaxWeight, &functor.f, fN, cols, rw.p, mx.p,
                                              nullptr));
            detail::throw_status(hps_weight_flags(fN, rw.p, weight, weight > 0.0 ? nullptr : mx.p, seed, 0, f.p,
                                                  nullptr));
            if (on_device) {
                compact_device(f.p);
                return;
            }
            detail::throw_cuda(cudaMemcpy(flags.data(), f.p, fN, cudaMemcpyDeviceToHost), "cudaMemcpy");
        });
        if (on_device) return fKept;
        return partition_host(flags);
    }

    // Not in the reference as one call: the Dalitz plot of its phsp_basic example,
    // make_dense_histogram<double,2>(sys, grid, lower, upper, Events | dalitz, Events | weights)
    // with dalitz = (m2(p[a0] + p[a1]), m2(p[b0] + p[b1])) and the recomputed PhaseSpaceWeight.
    // Returns grid[0]*grid[1] bin contents followed by the underflow and overflow bins.
    std::vector<double> DalitzHistogram(std::array<size_t, 2> const& grid, std::array<double, 2> const& lower,
                                        std::array<double, 2> const& upper, std::array<int, 2> const& pair_a = {0, 1},
                                        std::array<int, 2> const& pair_b = {1, 2},
                                        int32_t weight_mode = HPS_HIST_PHSP_WEIGHT) const
    {
        hps_hist2d h{{pair_a[0], pair_a[1]}, {pair_b[0], pair_b[1]}, {grid[0], grid[1]}, {lower[0], lower[1]},
                     {upper[0], upper[1]}};
        std::vector<double> bins(grid[0] * grid[1] + 2);
        with_device_columns([&](const double* const* cols) {
            detail::DeviceBuffer<double> b(bins.size());
            detail::throw_status(hps_dalitz_histogram(nparticles, fMasses, fMaxWeight, fN, cols, nullptr, weight_mode,
                                                      &h, b.p, nullptr));
            detail::throw_cuda(cudaMemcpy(bins.data(), b.p, bins.size() * 8, cudaMemcpyDeviceToHost), "cudaMemcpy");
        });
        return bins;
    }

private:
    // PhaseSpaceWeight x functor on the stored events with the functor compiled in
    // (detail/hps_user_kernels.cuh, nvcc only); out[i] per event, *max_dev the largest.
    template <typename Functor>
    void user_reweight(const double* const* cols, Functor const& functor, double* out, double* max_dev) const
    {
#if defined(__CUDACC__)
        detail::user::InColumns<nparticles> in;
        for (size_t k = 0; k < nparticles; ++k) in.p[k] = cols[k];
        hps_channel ch{};
        ch.n_daughters = nparticles;
        for (size_t k = 0; k < nparticles; ++k) ch.masses[k] = fMasses[k];
        ch.max_weight = fMaxWeight;
        hps::DevChannel dc;
        hps::make_channel(ch, dc);
        const unsigned grid = detail::user::grid_for(fN, detail::user::kThreads);
        detail::DeviceBuffer<double> bmax(grid);
        detail::user::k_reweight<nparticles, Vector4R, value_type>
            <<<grid, detail::user::kThreads>>>(in, dc, functor, fN, out, bmax.p);
        detail::user::k_max_final<><<<1, detail::user::kFinal>>>(bmax.p, grid, max_dev);
        detail::throw_cuda(cudaGetLastError(), "reweight launch");
        detail::throw_cuda(cudaStreamSynchronize(nullptr), "cudaStreamSynchronize");
#else
        (void)cols; (void)functor; (void)out; (void)max_dev;
        static_assert(detail::always_false<Functor>::value,
                      "a functor outside the C ABI's menu (hydra::hps_fn::One, Mass2, BW2) is compiled into the "
                      "kernels: build this translation unit with nvcc");
#endif
    }

    // stable partition of the device columns by flags (hps_unweight_compact); sets fKept
    void compact_device(const uint8_t* flags)
    {
        const double* cols[nparticles];
        double* outc[nparticles];
        detail::DeviceBuffer<double> out[nparticles];
        for (size_t k = 0; k < nparticles; ++k) {
            cols[k] = fDevCols[k].p;
            out[k].resize(4 * fN);
            outc[k] = out[k].p;
        }
        detail::DeviceBuffer<double> wout(fN);
        detail::DeviceBuffer<uint64_t> nacc(1);
        detail::throw_status(hps_unweight_compact(nparticles, fN, cols, fDevW.p, flags, outc, wout.p, nacc.p, nullptr,
                                                  0, nullptr));
        uint64_t kept = 0;
        detail::throw_cuda(cudaMemcpy(&kept, nacc.p, sizeof(kept), cudaMemcpyDeviceToHost), "cudaMemcpy");
        for (size_t k = 0; k < nparticles; ++k) std::swap(fDevCols[k], out[k]);
        std::swap(fDevW, wout);
        fKept = static_cast<size_t>(kept);
    }

    size_t partition_host(const std::vector<uint8_t>& flags)
    {
        std::vector<size_t> order;
        order.reserve(fN);
        for (size_t i = 0; i < fN; ++i) if (flags[i]) order.push_back(i);
        const size_t kept = order.size();
        for (size_t i = 0; i < fN; ++i) if (!flags[i]) order.push_back(i);
        permute(order);
        return kept;
    }

    template <size_t... I>
    static value_type make(const Vector4R (&p)[nparticles], std::index_sequence<I...>)
    {
        return value_type(Particles(p[I])...);
    }

    void init(size_t n)
    {
        double ecm = fMotherMass;
        for (size_t i = 0; i < nparticles; ++i) ecm -= fMasses[i];
        double emmax = ecm + fMasses[0], emmin = 0.0, wtmax = 1.0;
        for (size_t i = 1; i < nparticles; ++i) {                 // Decays.h:100-118
            emmin += fMasses[i - 1];
            emmax += fMasses[i];
            const double a = emmax, b = emmin, c = fMasses[i];
            wtmax *= std::sqrt((a - b - c) * (a + b + c) * (a - b + c) * (a + b - c)) / (2 * a);
        }
        fMaxWeight = 1.0 / wtmax;
        fN = n;
        for (size_t k = 0; k < nparticles; ++k) {
            if (on_device) fDevCols[k].resize(4 * n);
            else fHostCols[k].assign(4 * n, 0.0);
        }
        if (on_device) fDevW.resize(n); else fHostW.assign(n, 0.0);
    }

    template <typename F> void with_device_columns(F&& f) const
    {
        const double* cols[nparticles];
        if (on_device) {
            for (size_t k = 0; k < nparticles; ++k) cols[k] = fDevCols[k].p;
            f(cols);
            return;
        }
        detail::DeviceBuffer<double> tmp[nparticles];
        for (size_t k = 0; k < nparticles; ++k) {
            tmp[k].resize(4 * fN);
            detail::throw_cuda(cudaMemcpy(tmp[k].p, fHostCols[k].data(), fN * 32, cudaMemcpyHostToDevice), "cudaMemcpy");
            cols[k] = tmp[k].p;
        }
        f(cols);
    }

    void permute(const std::vector<size_t>& order)
    {
        for (size_t k = 0; k <= nparticles; ++k) {
            const size_t width = (k < nparticles) ? 4 : 1;
            std::vector<double> src(fN * width), dst(fN * width);
            double* col = (k < nparticles) ? column(k) : weights();
            if (on_device)
                detail::throw_cuda(cudaMemcpy(src.data(), col, fN * width * 8, cudaMemcpyDeviceToHost), "cudaMemcpy");
            else
                std::copy(col, col + fN * width, src.begin());
            for (size_t i = 0; i < fN; ++i)
                for (size_t c = 0; c < width; ++c) dst[i * width + c] = src[order[i] * width + c];
            if (on_device)
                detail::throw_cuda(cudaMemcpy(col, dst.data(), fN * width * 8, cudaMemcpyHostToDevice), "cudaMemcpy");
            else
                std::copy(dst.begin(), dst.end(), col);
        }
    }

    double fMotherMass = 0.0;
    double fMaxWeight = 0.0;
    double fMasses[HPS_MAX_DAUGHTERS] = {};
    size_t fN = 0;
    size_t fKept = 0;
    detail::DeviceBuffer<double> fDevCols[nparticles];
    detail::DeviceBuffer<double> fDevW;
    std::vector<double> fHostCols[nparticles];
    std::vector<double> fHostW;
};

// ------------------------------------------------------------------------------ multivector

// Result columns of Evaluate: hydra::multivector<hydra::tuple<T...>, Backend> with one double
// column per element (the first holds the weight).
template <typename Tuple, typename Backend> class multivector;

template <typename... T, typename Backend>
class multivector<hydra::tuple<T...>, Backend> {
public:
    enum { ncols = sizeof...(T) };
    static constexpr bool on_device = std::is_same<Backend, detail::DeviceBackend>::value;
    explicit multivector(size_t n) : fN(n)
    {
        for (size_t k = 0; k < ncols; ++k) {
            if (on_device) fDev[k].resize(n); else fHost[k].assign(n, 0.0);
        }
    }
    size_t size() const { return fN; }
    double* column(size_t k) { return on_device ? fDev[k].p : fHost[k].data(); }

    // Row i as a tuple of the element types (copied from the device for a device multivector);
    // prints as (c0, c1, ...), as the reference's tuples do.
    struct row : public hydra::tuple<T...> {
        using hydra::tuple<T...>::tuple;
        friend std::ostream& operator<<(std::ostream& o, row const& r)
        {
            o << "(";
            print(o, r, std::index_sequence_for<T...>{});
            return o << ")";
        }
        template <size_t... I>
        static void print(std::ostream& o, row const& r, std::index_sequence<I...>)
        {
            const double v[] = {static_cast<double>(std::get<I>(r))...};
            for (size_t k = 0; k < sizeof...(I); ++k) o << (k ? ", " : "") << v[k];
        }
    };
    row operator[](size_t i) const
    {
        double v[ncols];
        for (size_t k = 0; k < ncols; ++k) {
            if (on_device)
                detail::throw_cuda(cudaMemcpy(&v[k], fDev[k].p + i, 8, cudaMemcpyDeviceToHost), "cudaMemcpy");
            else
                v[k] = fHost[k][i];
        }
        return make_row(v, std::index_sequence_for<T...>{});
    }

    std::vector<double> GetColumn(size_t k) const
    {
        std::vector<double> out(fN);
        if (on_device && fN)
            detail::throw_cuda(cudaMemcpy(out.data(), fDev[k].p, fN * 8, cudaMemcpyDeviceToHost), "cudaMemcpy");
        else
            out = fHost[k];
        return out;
    }

private:
    template <size_t... I>
    static row make_row(const double (&v)[ncols], std::index_sequence<I...>)
    {
        return row(T(v[I])...);
    }
    size_t fN;
    detail::DeviceBuffer<double> fDev[ncols];
    std::vector<double> fHost[ncols];
};

// ------------------------------------------------------------------------------ PhaseSpace

template <size_t N, typename GRND = default_random_engine>
class PhaseSpace {
    static_assert(N >= 2 && N <= HPS_MAX_DAUGHTERS, "2..10 daughters");

public:
    PhaseSpace(double motherMass, const double (&daughtersMasses)[N]) { init(motherMass, daughtersMasses); }
    PhaseSpace(double motherMass, std::array<GReal_t, N> const& daughtersMasses)
    {
        init(motherMass, daughtersMasses.data());
    }
    PhaseSpace(double motherMass, std::initializer_list<GReal_t> const& daughtersMasses)
    {
        if (daughtersMasses.size() < N) throw std::invalid_argument("[hydra::PhaseSpace]: too few masses");
        init(motherMass, daughtersMasses.begin());
    }

    // Generate(mother, Decays) (PhaseSpace.inl:377-394): device Decays through hps_generate,
    // host Decays through hps_generate_host.
    template <typename... P, typename Backend>
    void Generate(Vector4R const& mother, Decays<hydra::tuple<P...>, Backend>& events)
    {
        static_assert(sizeof...(P) == N, "Decays must hold N daughters");
        hps_channel ch = channel(mother);
        double* cols[N];
        for (size_t k = 0; k < N; ++k) cols[k] = events.column(k);
        if (Decays<hydra::tuple<P...>, Backend>::on_device) {
            detail::throw_status(hps_generate(&ch, 0, events.size(), cols, events.weights(), nullptr, 0, fPrecision,
                                              nullptr));
            detail::throw_cuda(cudaStreamSynchronize(nullptr), "cudaStreamSynchronize");
        } else {
            detail::throw_status(hps_generate_host(&ch, 0, events.size(), cols, events.weights(), nullptr, 0,
                                                   fPrecision, 0, nullptr));
        }
    }

    // AverageOn(policy, mother, functor, n) (PhaseSpace.inl:255-273): (mean, sqrt(M2)/W).  A menu
    // functor goes through hps_average_on; any other is compiled into the tile kernels of
    // detail/hps_user_kernels.cuh (nvcc only).
    template <typename Functor, typename Policy,
              typename std::enable_if<!hps_fn::is_menu<Functor>::value, int>::type = 0>
    std::pair<GReal_t, GReal_t> AverageOn(Policy const&, Vector4R const& mother, Functor const& functor, size_t n)
    {
#if defined(__CUDACC__)
        hps_channel ch = channel(mother);
        const detail::user::LaunchChannel lc = detail::user::launch_channel(ch);
        const uint64_t ntiles = (n + HPS_AVG_TILE - 1) / HPS_AVG_TILE;
        detail::DeviceBuffer<hps_stats> part(ntiles ? ntiles : 1), out(1);
        const unsigned grid = static_cast<unsigned>(ntiles < 152u * 16u ? (ntiles ? ntiles : 1) : 152u * 16u);
        const int32_t prec = fPrecision;
        if (prec == HPS_PREC_FP32_FIX) {
            // the shifted float-float tile sums of the library's FP32_FIX AverageOn
            detail::DeviceBuffer<float> k0(1);
            if (ntiles) {
                detail::user::with_engine<N>(lc, prec, [&](auto E) {
                    constexpr int EE = decltype(E)::value;
                    detail::user::k_user_shift_f32<N, EE, false, Vector4R><<<1, 32>>>(lc.ch, lc.chf, functor, 0, k0.p);
                    detail::user::k_average_tiles_f32<N, EE, false, Vector4R>
                        <<<grid, detail::user::kThreads>>>(lc.ch, lc.chf, functor, 0, n, ntiles, k0.p, part.p);
                });
            } else {
                detail::throw_cuda(cudaMemset(k0.p, 0, sizeof(float)), "cudaMemset");
            }
            detail::user::k_average_final_sums<><<<1, detail::user::kFinal>>>(part.p, ntiles, k0.p, out.p);
        } else {
            if (ntiles) {
                detail::user::with_engine<N>(lc, prec, [&](auto E) {
                    constexpr int EE = decltype(E)::value;
                    detail::user::k_average_tiles<N, EE, HPS_PREC_FP64, Vector4R>
                        <<<grid, detail::user::kThreads>>>(lc.ch, lc.chf, functor, 0, n, ntiles, part.p);
                });
            }
            detail::user::k_average_final<><<<1, detail::user::kFinal>>>(part.p, ntiles, out.p);
        }
        detail::throw_cuda(cudaGetLastError(), "AverageOn launch");
        hps_stats s;
        detail::throw_cuda(cudaMemcpy(&s, out.p, sizeof(s), cudaMemcpyDeviceToHost), "cudaMemcpy");
        return std::make_pair(s.mean, std::sqrt(s.m2) / s.w);
#else
        (void)mother; (void)functor; (void)n;
        static_assert(detail::always_false<Functor>::value,
                      "a functor outside the C ABI's menu (hydra::hps_fn::One, Mass2, BW2) is compiled into the "
                      "kernels: build this translation unit with nvcc");
        return {};
#endif
    }

    template <typename Functor, typename Policy,
              typename std::enable_if<hps_fn::is_menu<Functor>::value, int>::type = 0>
    std::pair<GReal_t, GReal_t> AverageOn(Policy const&, Vector4R const& mother, Functor const& functor, size_t n)
    {
        hps_channel ch = channel(mother);
        detail::DeviceBuffer<hps_stats> out(1);
        detail::throw_status(hps_average_on(&ch, 0, n, &functor.f, out.p, nullptr, 0, fPrecision, nullptr));
        hps_stats s;
        detail::throw_cuda(cudaMemcpy(&s, out.p, sizeof(s), cudaMemcpyDeviceToHost), "cudaMemcpy");
        return std::make_pair(s.mean, std::sqrt(s.m2) / s.w);
    }

    // Evaluate(mother, result, functors...) (PhaseSpace.inl:314-329): column 0 the weight,
    // column k the k-th functor.  All-menu functors go through hps_evaluate; otherwise the
    // functors are compiled into the evaluate kernel of detail/hps_user_kernels.cuh (nvcc only).
    template <typename... T, typename Backend, typename... Functors>
    void Evaluate(Vector4R const& mother, multivector<hydra::tuple<T...>, Backend>& result, Functors const&... fs)
    {
        static_assert(sizeof...(T) == sizeof...(Functors) + 1, "one result column per functor plus the weight");
        evaluate_impl(std::integral_constant<bool, detail::all_menu<Functors...>::value>{}, mother, result, fs...);
    }

private:
    template <typename... T, typename Backend, typename... Functors>
    void evaluate_impl(std::false_type, Vector4R const& mother, multivector<hydra::tuple<T...>, Backend>& result,
                       Functors const&... fs)
    {
#if defined(__CUDACC__)
        constexpr int K = sizeof...(Functors);
        hps_channel ch = channel(mother);
        const detail::user::LaunchChannel lc = detail::user::launch_channel(ch);
        const size_t n = result.size();
        const bool dev = multivector<hydra::tuple<T...>, Backend>::on_device;
        std::vector<detail::DeviceBuffer<double>> tmp;
        tmp.reserve(K + 1);
        detail::user::OutColumns<K> out;
        for (int k = 0; k <= K; ++k) {
            if (dev) {
                out.p[k] = result.column(k);
            } else {
                tmp.emplace_back(n);
                out.p[k] = tmp.back().p;
            }
        }
        const auto fns = std::make_tuple(fs...);
        const unsigned grid = detail::user::grid_for(n, detail::user::kThreads);
        const int32_t prec = fPrecision;
        if (n) {
            detail::user::with_engine<N>(lc, prec, [&](auto E) {
                constexpr int EE = decltype(E)::value;
                if (prec == HPS_PREC_FP32_FIX)
                    detail::user::k_evaluate<N, EE, HPS_PREC_FP32_FIX, Vector4R>
                        <<<grid, detail::user::kThreads>>>(lc.ch, lc.chf, fns, out, 0, n);
                else
                    detail::user::k_evaluate<N, EE, HPS_PREC_FP64, Vector4R>
                        <<<grid, detail::user::kThreads>>>(lc.ch, lc.chf, fns, out, 0, n);
            });
            detail::throw_cuda(cudaGetLastError(), "Evaluate launch");
        }
        detail::throw_cuda(cudaStreamSynchronize(nullptr), "cudaStreamSynchronize");
        if (!dev)
            for (int k = 0; k <= K; ++k)
                detail::throw_cuda(cudaMemcpy(result.column(k), out.p[k], n * 8, cudaMemcpyDeviceToHost), "cudaMemcpy");
#else
        (void)mother; (void)result;
        static_assert(detail::always_false<hydra::tuple<Functors...>>::value,
                      "a functor outside the C ABI's menu (hydra::hps_fn::One, Mass2, BW2) is compiled into the "
                      "kernels: build this translation unit with nvcc");
#endif
    }

    template <typename... T, typename Backend, typename... Functors>
    void evaluate_impl(std::true_type, Vector4R const& mother, multivector<hydra::tuple<T...>, Backend>& result,
                       Functors const&... fs)
    {
        const hps_functor menu[] = {fs.f...};
        hps_channel ch = channel(mother);
        const size_t n = result.size();
        const bool dev = multivector<hydra::tuple<T...>, Backend>::on_device;
        std::vector<detail::DeviceBuffer<double>> tmp;
        double* out[sizeof...(Functors) + 1];
        for (size_t k = 0; k <= sizeof...(Functors); ++k) {
            if (dev) {
                out[k] = result.column(k);
            } else {
                tmp.emplace_back(n);
                out[k] = tmp.back().p;
            }
        }
        detail::throw_status(hps_evaluate(&ch, 0, n, menu, sizeof...(Functors), out[0], out + 1, fPrecision, nullptr));
        detail::throw_cuda(cudaStreamSynchronize(nullptr), "cudaStreamSynchronize");
        if (!dev)
            for (size_t k = 0; k <= sizeof...(Functors); ++k)
                detail::throw_cuda(cudaMemcpy(result.column(k), out[k], n * 8, cudaMemcpyDeviceToHost), "cudaMemcpy");
    }

public:
    // Generate(mothers, daughters) (PhaseSpace.inl:399-417, DecayMothers): event i is boosted by
    // mothers[i]; the stream, ECM and weights are those of Generate(mother, daughters).
    template <typename... P, typename Backend>
    void Generate(DaughterRange const& mothers, Decays<hydra::tuple<P...>, Backend>& events)
    {
        static_assert(sizeof...(P) == N, "Decays must hold N daughters");
        if (mothers.n != events.size()) throw std::invalid_argument("[hydra::PhaseSpace]: mothers and daughters differ in size");
        hps_channel ch = channel(Vector4R(fMotherMass, 0, 0, 0));
        detail::DeviceBuffer<double> tmo;
        const double* mo = device_mothers(mothers, tmo);
        const bool dev = Decays<hydra::tuple<P...>, Backend>::on_device;
        std::vector<detail::DeviceBuffer<double>> tmp;
        double* cols[N];
        for (size_t k = 0; k < N; ++k) {
            if (dev) {
                cols[k] = events.column(k);
            } else {
                tmp.emplace_back(4 * events.size());
                cols[k] = tmp.back().p;
            }
        }
        detail::DeviceBuffer<double> tw(dev ? 0 : events.size());
        detail::throw_status(hps_generate_mothers(&ch, 0, events.size(), mo, cols, dev ? events.weights() : tw.p,
                                                  fPrecision, nullptr));
        detail::throw_cuda(cudaStreamSynchronize(nullptr), "cudaStreamSynchronize");
        if (!dev) {
            for (size_t k = 0; k < N; ++k)
                detail::throw_cuda(cudaMemcpy(events.column(k), cols[k], events.size() * 32, cudaMemcpyDeviceToHost),
                                   "cudaMemcpy");
            detail::throw_cuda(cudaMemcpy(events.weights(), tw.p, events.size() * 8, cudaMemcpyDeviceToHost),
                               "cudaMemcpy");
        }
    }

    // AverageOn(mothers, functor) (PhaseSpace.inl:276-287, AverageMothers): the functor sees
    // (mother, daughter 0, ..., daughter N-1).
    template <typename Functor, typename std::enable_if<!hps_fn::is_menu<Functor>::value, int>::type = 0>
    std::pair<GReal_t, GReal_t> AverageOn(DaughterRange const& mothers, Functor const& functor)
    {
#if defined(__CUDACC__)
        hps_channel ch = channel(Vector4R(fMotherMass, 0, 0, 0));
        const detail::user::LaunchChannel lc = detail::user::launch_channel(ch);
        detail::DeviceBuffer<double> tmo;
        const double* mo = device_mothers(mothers, tmo);
        const uint64_t n = mothers.n, ntiles = (n + HPS_AVG_TILE - 1) / HPS_AVG_TILE;
        detail::DeviceBuffer<hps_stats> part(ntiles ? ntiles : 1), out(1);
        const unsigned grid = static_cast<unsigned>(ntiles < 152u * 16u ? (ntiles ? ntiles : 1) : 152u * 16u);
        const int32_t prec = fPrecision;
        if (prec == HPS_PREC_FP32_FIX) {
            // the shifted float-float tile sums of the library's FP32_FIX AverageMothers
            detail::DeviceBuffer<float> k0(1);
            if (ntiles) {
                detail::user::with_engine<N>(lc, prec, [&](auto E) {
                    constexpr int EE = decltype(E)::value;
                    detail::user::k_user_shift_f32<N, EE, true, Vector4R>
                        <<<1, 32>>>(lc.ch, lc.chf, functor, 0, k0.p, mo);
                    detail::user::k_average_tiles_f32<N, EE, true, Vector4R>
                        <<<grid, detail::user::kThreads>>>(lc.ch, lc.chf, functor, 0, n, ntiles, k0.p, part.p, mo);
                });
            } else {
                detail::throw_cuda(cudaMemset(k0.p, 0, sizeof(float)), "cudaMemset");
            }
            detail::user::k_average_final_sums<><<<1, detail::user::kFinal>>>(part.p, ntiles, k0.p, out.p);
        } else {
            if (ntiles) {
                detail::user::with_engine<N>(lc, prec, [&](auto E) {
                    constexpr int EE = decltype(E)::value;
                    detail::user::k_average_mothers_tiles<N, EE, HPS_PREC_FP64, Vector4R>
                        <<<grid, detail::user::kThreads>>>(lc.ch, lc.chf, functor, mo, 0, n, ntiles, part.p);
                });
            }
            detail::user::k_average_final<><<<1, detail::user::kFinal>>>(part.p, ntiles, out.p);
        }
        detail::throw_cuda(cudaGetLastError(), "AverageOn launch");
        hps_stats st;
        detail::throw_cuda(cudaMemcpy(&st, out.p, sizeof(st), cudaMemcpyDeviceToHost), "cudaMemcpy");
        return std::make_pair(st.mean, std::sqrt(st.m2) / st.w);
#else
        (void)mothers; (void)functor;
        static_assert(detail::always_false<Functor>::value,
                      "a functor outside the C ABI's menu (hydra::hps_fn::One, Mass2, BW2) is compiled into the "
                      "kernels: build this translation unit with nvcc");
        return {};
#endif
    }

    template <typename Functor, typename std::enable_if<hps_fn::is_menu<Functor>::value, int>::type = 0>
    std::pair<GReal_t, GReal_t> AverageOn(DaughterRange const& mothers, Functor const& functor)
    {
        hps_channel ch = channel(Vector4R(fMotherMass, 0, 0, 0));
        detail::DeviceBuffer<double> tmo;
        const double* mo = device_mothers(mothers, tmo);
        detail::DeviceBuffer<hps_stats> out(1);
        detail::throw_status(hps_average_on_mothers(&ch, 0, mothers.n, mo, &functor.f, out.p, nullptr, 0, fPrecision,
                                                    nullptr));
        hps_stats st;
        detail::throw_cuda(cudaMemcpy(&st, out.p, sizeof(st), cudaMemcpyDeviceToHost), "cudaMemcpy");
        return std::make_pair(st.mean, std::sqrt(st.m2) / st.w);
    }

    // Evaluate(mothers, result, functors...) (PhaseSpace.inl:334-348, EvalMothers): its own stream
    // per event (hash(event, seed)), ECM and maximum weight from each mother's mass; the functors
    // see (mother, daughters...).  All-menu functors go through hps_evaluate_mothers; otherwise they
    // are compiled into the kernel of detail/hps_user_kernels.cuh (nvcc only).
    template <typename... T, typename Backend, typename... Functors>
    void Evaluate(DaughterRange const& mothers, multivector<hydra::tuple<T...>, Backend>& result, Functors const&... fs)
    {
        static_assert(sizeof...(T) == sizeof...(Functors) + 1, "one result column per functor plus the weight");
        evaluate_mothers_impl(std::integral_constant<bool, detail::all_menu<Functors...>::value>{}, mothers, result,
                              fs...);
    }

private:
    template <typename... T, typename Backend, typename... Functors>
    void evaluate_mothers_impl(std::false_type, DaughterRange const& mothers,
                               multivector<hydra::tuple<T...>, Backend>& result, Functors const&... fs)
    {
#if defined(__CUDACC__)
        constexpr int K = sizeof...(Functors);
        hps_channel ch = channel(Vector4R(fMotherMass, 0, 0, 0));
        const detail::user::LaunchChannel lc = detail::user::launch_channel(ch);
        detail::DeviceBuffer<double> tmo;
        const double* mo = device_mothers(mothers, tmo);
        const size_t n = mothers.n;
        const bool dev = multivector<hydra::tuple<T...>, Backend>::on_device;
        std::vector<detail::DeviceBuffer<double>> tmp;
        tmp.reserve(K + 1);
        detail::user::OutColumns<K> out;
        for (int k = 0; k <= K; ++k) {
            if (dev) {
                out.p[k] = result.column(k);
            } else {
                tmp.emplace_back(n);
                out.p[k] = tmp.back().p;
            }
        }
        const auto fns = std::make_tuple(fs...);
        const unsigned grid = detail::user::grid_for(n, detail::user::kThreads);
        const int32_t prec = fPrecision;
        if (n) {
            detail::user::with_engine<N>(lc, prec, [&](auto E) {
                constexpr int EE = decltype(E)::value;
                if (prec == HPS_PREC_FP32_FIX)
                    detail::user::k_evaluate_mothers<N, EE, HPS_PREC_FP32_FIX, Vector4R>
                        <<<grid, detail::user::kThreads>>>(lc.ch, lc.chf, ch.seed, mo, fns, out, 0, n);
                else
                    detail::user::k_evaluate_mothers<N, EE, HPS_PREC_FP64, Vector4R>
                        <<<grid, detail::user::kThreads>>>(lc.ch, lc.chf, ch.seed, mo, fns, out, 0, n);
            });
            detail::throw_cuda(cudaGetLastError(), "Evaluate launch");
        }
        detail::throw_cuda(cudaStreamSynchronize(nullptr), "cudaStreamSynchronize");
        if (!dev)
            for (int k = 0; k <= K; ++k)
                detail::throw_cuda(cudaMemcpy(result.column(k), out.p[k], n * 8, cudaMemcpyDeviceToHost), "cudaMemcpy");
#else
        (void)mothers; (void)result;
        static_assert(detail::always_false<hydra::tuple<Functors...>>::value,
                      "a functor outside the C ABI's menu (hydra::hps_fn::One, Mass2, BW2) is compiled into the "
                      "kernels: build this translation unit with nvcc");
#endif
    }

    template <typename... T, typename Backend, typename... Functors>
    void evaluate_mothers_impl(std::true_type, DaughterRange const& mothers,
                               multivector<hydra::tuple<T...>, Backend>& result, Functors const&... fs)
    {
        const hps_functor menu[] = {fs.f...};
        hps_channel ch = channel(Vector4R(fMotherMass, 0, 0, 0));
        detail::DeviceBuffer<double> tmo;
        const double* mo = device_mothers(mothers, tmo);
        const size_t n = mothers.n;
        const bool dev = multivector<hydra::tuple<T...>, Backend>::on_device;
        std::vector<detail::DeviceBuffer<double>> tmp;
        double* out[sizeof...(Functors) + 1];
        for (size_t k = 0; k <= sizeof...(Functors); ++k) {
            if (dev) {
                out[k] = result.column(k);
            } else {
                tmp.emplace_back(n);
                out[k] = tmp.back().p;
            }
        }
        detail::throw_status(hps_evaluate_mothers(&ch, 0, n, mo, menu, sizeof...(Functors), out[0], out + 1,
                                                  fPrecision, nullptr));
        detail::throw_cuda(cudaStreamSynchronize(nullptr), "cudaStreamSynchronize");
        if (!dev)
            for (size_t k = 0; k <= sizeof...(Functors); ++k)
                detail::throw_cuda(cudaMemcpy(result.column(k), out[k], n * 8, cudaMemcpyDeviceToHost), "cudaMemcpy");
    }

public:
    GInt_t GetSeed() const { return static_cast<GInt_t>(fSeed); }
    void SetSeed(GInt_t seed) { fSeed = static_cast<size_t>(static_cast<long long>(seed)); }
    const GReal_t* GetMasses() const { return fMasses; }
    double GetMaxWeight() const { return fMaxWeight; }
    void SetMaxWeight(double w) { fMaxWeight = w; }
    double GetMotherMass() const { return fMotherMass; }
    void SetMotherMass(double m) { fMotherMass = m; }
    double GetECM() const { return fECM; }
    void SetECM(double e) { fECM = e; }
    static double PDK(double a, double b, double c)
    {
        double x = (a - b - c) * (a + b + c) * (a - b + c) * (a + b - c);
        x = std::sqrt(x) / (2 * a);
        return x;
    }

    // Not in the reference: arithmetic of the kernels (HPS_PREC_FP64 default, HPS_PREC_FP32_FIX).
    void SetPrecision(int32_t precision) { fPrecision = precision; }

private:
    void init(double motherMass, const double* masses)
    {
        hps_channel ch;
        const double mother[4] = {motherMass, 0.0, 0.0, 0.0};
        detail::throw_status(hps_channel_init(&ch, N, detail::engine_id<GRND>::value, 0, motherMass, masses, mother));
        fMotherMass = motherMass;
        for (size_t i = 0; i < N; ++i) fMasses[i] = masses[i];
        fECM = ch.ecm;
        fMaxWeight = ch.max_weight;
        // default seed: 1 * (1 + hash_range(masses)) (PhaseSpace.inl:44,64)
        fSeed = hps_default_seed(N, masses);
    }

    // The mothers column on the device (copied there for a host Decays).
    static const double* device_mothers(DaughterRange const& m, detail::DeviceBuffer<double>& tmp)
    {
        if (m.on_device) return m.data;
        tmp.resize(4 * m.n);
        if (m.n)
            detail::throw_cuda(cudaMemcpy(tmp.p, m.data, m.n * 32, cudaMemcpyHostToDevice), "cudaMemcpy");
        return tmp.p;
    }

    hps_channel channel(Vector4R const& mother) const
    {
        hps_channel ch;
        detail::throw_status(hps_channel_init(&ch, N, detail::engine_id<GRND>::value, fSeed, fMotherMass, fMasses,
                                              mother.data()));
        ch.ecm = fECM;                // the values this object holds (SetECM / SetMaxWeight apply)
        ch.max_weight = fMaxWeight;
        return ch;
    }

    size_t fSeed = 1;
    double fMotherMass = 0.0;
    double fMaxWeight = 0.0;
    double fECM = 0.0;
    GReal_t fMasses[N] = {};
    int32_t fPrecision = HPS_PREC_FP64;
};

// -------------------------------------------------------------------- PhaseSpaceIntegrator

// hydra::PhaseSpaceIntegrator<N, Backend, GRND> (hydra/PhaseSpaceIntegrator.h:52-160):
// Integrate(functor) = AverageOn(mother at rest, functor, n) of a PhaseSpace that keeps the
// default seed (PhaseSpaceIntegrator.inl:37-42).
template <size_t N, typename Backend = device::sys_t, typename GRND = default_random_engine>
class PhaseSpaceIntegrator {
public:
    PhaseSpaceIntegrator(double motherMass, const double (&daughtersMasses)[N], size_t n)
        : fGenerator(motherMass, daughtersMasses), fMother(motherMass, 0, 0, 0), fNSamples(n) {}
    PhaseSpaceIntegrator(double motherMass, std::array<GReal_t, N> const& daughtersMasses, size_t n)
        : fGenerator(motherMass, daughtersMasses), fMother(motherMass, 0, 0, 0), fNSamples(n) {}
    PhaseSpaceIntegrator(double motherMass, std::initializer_list<GReal_t> const& daughtersMasses, size_t n)
        : fGenerator(motherMass, daughtersMasses), fMother(motherMass, 0, 0, 0), fNSamples(n) {}

    template <typename Functor>
    std::pair<GReal_t, GReal_t> Integrate(Functor const& functor)
    {
        return fGenerator.AverageOn(Backend{}, fMother, functor, fNSamples);
    }

    const PhaseSpace<N, GRND>& GetGenerator() const { return fGenerator; }
    PhaseSpace<N, GRND>& GetGenerator() { return fGenerator; }
    const Vector4R& GetMother() const { return fMother; }
    void SetMother(Vector4R const& m) { fMother = m; }
    size_t GetNSamples() const { return fNSamples; }
    void SetNSamples(size_t n) { fNSamples = n; }

private:
    PhaseSpace<N, GRND> fGenerator;
    Vector4R fMother;
    size_t fNSamples;
};

// --------------------------------------------------------------------- phase_space_range

// phase_space_range(mother, masses, seed, length) (hydra/detail/PhaseSpaceRange.inl:46-73): the
// reference returns a lazy range of tuple(weight, Vector4R...) over GenerateDecay with thrust's
// minstd_rand.  Here the range is materialised on the device when it is created (length must be
// given: the reference's length 0 means "unbounded"), then read like the lazy one:
// range[i] / begin()[i] is the same tuple.
template <size_t N>
class PhaseSpaceRange {
public:
    typedef typename detail::tuple_cat_helper<N>::type value_type;

    PhaseSpaceRange(Vector4R const& mother, std::array<double, N> const& masses, size_t seed, size_t length)
        : fN(length)
    {
        if (length == 0) throw std::invalid_argument("phase_space_range: a materialised range needs its length");
        hps_channel ch;
        detail::throw_status(hps_range_channel(&ch, N, masses.data(), mother.data(), seed));
        double* cols[N];
        for (size_t k = 0; k < N; ++k) {
            fCols[k].resize(4 * length);
            cols[k] = fCols[k].p;
        }
        fW.resize(length);
        detail::throw_status(hps_generate_range(&ch, 0, length, cols, fW.p, nullptr));
        detail::throw_cuda(cudaStreamSynchronize(nullptr), "cudaStreamSynchronize");
    }

    size_t size() const { return fN; }

    value_type operator[](size_t i) const
    {
        double w;
        Vector4R p[N];
        detail::throw_cuda(cudaMemcpy(&w, fW.p + i, 8, cudaMemcpyDeviceToHost), "cudaMemcpy");
        for (size_t k = 0; k < N; ++k) {
            double v[4];
            detail::throw_cuda(cudaMemcpy(v, fCols[k].p + 4 * i, sizeof(v), cudaMemcpyDeviceToHost), "cudaMemcpy");
            p[k].set(v[0], v[1], v[2], v[3]);
        }
        return make(w, p, std::make_index_sequence<N>{});
    }

    struct iterator {
        const PhaseSpaceRange* r;
        size_t i;
        value_type operator*() const { return (*r)[i]; }
        value_type operator[](size_t k) const { return (*r)[i + k]; }
        iterator& operator++() { ++i; return *this; }
        iterator operator+(size_t k) const { return iterator{r, i + k}; }
        bool operator!=(iterator const& o) const { return i != o.i; }
        bool operator==(iterator const& o) const { return i == o.i; }
    };
    iterator begin() const { return iterator{this, 0}; }
    iterator end() const { return iterator{this, fN}; }

    // device columns: weights and daughter k ({E,px,py,pz} per event)
    const double* weights() const { return fW.p; }
    const double* column(size_t k) const { return fCols[k].p; }

private:
    template <size_t... I>
    static value_type make(double w, const Vector4R (&p)[N], std::index_sequence<I...>)
    {
        return value_type(w, p[I]...);
    }

    size_t fN;
    detail::DeviceBuffer<double> fCols[N];
    detail::DeviceBuffer<double> fW;
};

template <size_t N>
PhaseSpaceRange<N> phase_space_range(Vector4R const& mother, std::array<double, N> masses, size_t seed,
                                     size_t length = 0)
{
    return PhaseSpaceRange<N>(mother, masses, seed, length);
}

}  // namespace hydra

#endif  // HYDRA_HPS_PHASESPACE_HPP_
