/*
 * ref_gpu.cu -- test infrastructure, NOT product code.
 *
 * The reference's own device code for the GENBOD path, compiled by nvcc for
 * sm_103a from the UNMODIFIED Hydra headers into a cubin (oracle/_ref/ref_gpu.cubin)
 * by oracle/build_ref.sh, so that the reference's CUDA functors can run on a GB300
 * where the Hydra sources are absent.  oracle/ref_gpu.py loads the cubin with the
 * CUDA driver API.  Used only to check the product against the reference's own
 * CUDA arithmetic and to time that arithmetic; nothing in the product calls it.
 *
 * Reference code exercised (paths inside the Hydra project):
 *   hydra/detail/functors/DecayMother.h:163-290    DecayMother::process / operator()(evt)
 *   hydra/detail/functors/AverageMother.h:156-296  AverageMother::process / operator()(evt)
 *   hydra/detail/functors/EvalMother.h:169-305     EvalMother::operator()(evt) (Evaluate)
 *   hydra/detail/functors/DecayMothers.h:131-260   DecayMothers::operator()(evt, mother)
 *   hydra/detail/functors/AverageMothers.h:134-285 AverageMothers::operator()((evt, mother))
 *   hydra/detail/functors/StatsPHSP.h:38-86        StatsPHSP, AddStatsPHSP
 *   hydra/detail/random/EngineR123.h:244           hydra::philox (Philox2x64, 7 rounds)
 *   hydra/detail/random/squares3.h                 hydra::squares3 (default_random_engine)
 *
 * Thrust's host-side launchers (tabulate for Generate, launch_decayers.inl:133-138;
 * transform_reduce for AverageOn, launch_decayers.inl:94-106) need the Hydra tree at
 * build time on the machine that runs them, so the kernels below stand in for them:
 * a grid-stride loop calls the reference functor once per event and stores what it
 * returns (Generate: N Vector4R columns, 32 B per particle, the Decays layout), or
 * folds the StatsPHSP it returns with AddStatsPHSP in a per-block tree (AverageOn;
 * the per-block partials are folded on the host).  All arithmetic per event is the
 * reference's; the reduction order is not thrust's.
 *
 * Flags follow the reference build (CMakeLists.txt: -std=c++20, -extended-lambda,
 * --expt-relaxed-constexpr, nvcc's default FMA contraction).
 */
#include <hydra/detail/Config.h>
#include <hydra/Types.h>
#include <hydra/Vector4R.h>
#include <hydra/detail/functors/DecayMother.h>
#include <hydra/detail/functors/AverageMother.h>
#include <hydra/detail/functors/StatsPHSP.h>
#include <hydra/detail/random/EngineR123.h>
#include <hydra/detail/random/squares3.h>
#include <hydra/detail/PRNGTypedefs.h>

#include <hydra/detail/functors/EvalMother.h>
#include <hydra/detail/functors/DecayMothers.h>
#include <hydra/detail/functors/AverageMothers.h>

#include <cstddef>
#include <cstdint>
#include <new>

namespace hpsref {

constexpr int kThreads = 256;

// Kernel-parameter mirror of the functors' data members, in their declaration order
// (DecayMother.h:64-73, AverageMother.h:60-70).  The functors' value constructors are
// host-only, so the device code copies from a mirror of identical layout (checked below).
template <size_t N> struct MotherArgs {
    size_t seed;
    double ecm, maxw, beta0, beta1, beta2;
    double masses[N];
};

// The functor menu's Breit-Wigner |BW(m_ij)|^2 = 1/((a^2 - m_ij^2)^2 + (a b)^2), called
// by AverageMother / EvalMother with the tuple of N Vector4R (AverageMother.h:285,
// EvalMother.h:302; the *Mothers forms pass N+1 with the mother first).
struct BWij {
    typedef double return_type;
    int i, j;
    double a, b;
    template <typename Tuple>
    __hydra_host__ __hydra_device__ double operator()(Tuple const& t) const
    {
        hydra::Vector4R p[hydra::thrust::tuple_size<Tuple>::value];
        hydra::detail::assignTupleToArray(t, p);
        hydra::Vector4R s = p[i] + p[j];
        double m2 = s.mass2();
        double d = a * a - m2;
        double g = a * b;
        return 1.0 / (d * d + g * g);
    }
};

// The menu's m^2(p_i + p_j).
struct M2ij {
    typedef double return_type;
    int i, j;
    double a, b;    // unused; same layout as BWij
    template <typename Tuple>
    __hydra_host__ __hydra_device__ double operator()(Tuple const& t) const
    {
        hydra::Vector4R p[hydra::thrust::tuple_size<Tuple>::value];
        hydra::detail::assignTupleToArray(t, p);
        hydra::Vector4R s = p[i] + p[j];
        return s.mass2();
    }
};

// Kernel parameters of the per-event-mother functors (DecayMothers.h:59-63,
// AverageMothers.h:59-63): no beta, the mother comes per event.
template <size_t N> struct MothersArgs {
    size_t seed;
    double ecm, maxw;
    double masses[N];
};

// Builds functor F on the device without its host-only value constructor: the data members
// are assigned by name in raw storage and the object is then copy-constructed from it (the
// copy constructors are __host__ __device__).
template <typename F, typename A>
__device__ __forceinline__ void fill_common(F* f, A const& a)
{
    f->fSeed = a.seed;
    f->fECM = a.ecm;
    f->fMaxWeight = a.maxw;
    for (size_t k = 0; k < sizeof(a.masses) / sizeof(a.masses[0]); ++k) f->fMasses[k] = a.masses[k];
}

template <size_t N> struct AvgArgs {
    MotherArgs<N> m;
    BWij f;
};

#define CHECK_LAYOUT(T, M)                                                                        \
    static_assert(offsetof(T, fSeed) == offsetof(M, seed) && offsetof(T, fECM) == offsetof(M, ecm) && \
                      offsetof(T, fMaxWeight) == offsetof(M, maxw) &&                               \
                      offsetof(T, fBeta0) == offsetof(M, beta0) &&                                  \
                      offsetof(T, fBeta2) == offsetof(M, beta2) &&                                  \
                      offsetof(T, fMasses) == offsetof(M, masses),                                  \
                  "reference functor layout differs from its mirror")

template <size_t N, typename GRND>
__device__ void generate(MotherArgs<N> const& args, uint64_t first, uint64_t n, hydra::Vector4R* const* cols)
{
    typedef hydra::detail::DecayMother<N, GRND> F;
    CHECK_LAYOUT(F, MotherArgs<N>);
    static_assert(sizeof(F) == sizeof(MotherArgs<N>), "reference functor size differs from its mirror");
    F decayer(*reinterpret_cast<F const*>(&args));
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < n; e += (uint64_t)gridDim.x * blockDim.x) {
        typename F::particles_tuple_type t = decayer(first + e);
        hydra::Vector4R p[N];
        hydra::detail::assignTupleToArray(t, p);
#pragma unroll
        for (size_t i = 0; i < N; i++) cols[i][e] = p[i];
    }
}

template <size_t N, typename GRND>
__device__ void average(AvgArgs<N> const& args, uint64_t first, uint64_t n, hydra::detail::StatsPHSP* partial)
{
    typedef hydra::detail::AverageMother<N, GRND, BWij> F;
    CHECK_LAYOUT(F, MotherArgs<N>);
    static_assert(offsetof(F, fFunctor) == offsetof(AvgArgs<N>, f) && sizeof(F) == sizeof(AvgArgs<N>),
                  "reference functor layout differs from its mirror");
    F avg(*reinterpret_cast<F const*>(&args));
    hydra::detail::AddStatsPHSP add;
    hydra::detail::StatsPHSP acc;
    bool any = false;
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < n; e += (uint64_t)gridDim.x * blockDim.x) {
        hydra::detail::StatsPHSP s = avg(first + e);
        acc = any ? add(acc, s) : s;
        any = true;
    }
    __shared__ hydra::detail::StatsPHSP sh[kThreads];
    __shared__ bool shany[kThreads];
    sh[threadIdx.x] = acc;
    shany[threadIdx.x] = any;
    __syncthreads();
    for (int w = kThreads / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w && shany[threadIdx.x + w]) {
            sh[threadIdx.x] = shany[threadIdx.x] ? add(sh[threadIdx.x], sh[threadIdx.x + w]) : sh[threadIdx.x + w];
            shany[threadIdx.x] = true;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        hydra::detail::StatsPHSP r = sh[0];
        if (!shany[0]) r.fW = 0.0;
        partial[blockIdx.x] = r;
    }
}

template <size_t N, typename GRND>
__device__ void evaluate(MotherArgs<N> const& args, BWij bw, M2ij m2, uint64_t first, uint64_t n, double* w,
                         double* f_bw, double* f_m2)
{
    typedef hydra::detail::EvalMother<N, GRND, BWij, M2ij> F;
    alignas(F) unsigned char raw[sizeof(F)];
    F* f = reinterpret_cast<F*>(raw);
    fill_common(f, args);
    f->fBeta0 = args.beta0;
    f->fBeta1 = args.beta1;
    f->fBeta2 = args.beta2;
    ::new (static_cast<void*>(&f->fFunctors)) typename F::functors_tuple_type(bw, m2);
    F ev(*f);
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < n; e += (uint64_t)gridDim.x * blockDim.x) {
        typename F::result_tuple_type r = ev(first + e);
        w[e] = hydra::thrust::get<0>(r);
        f_bw[e] = hydra::thrust::get<1>(r);
        f_m2[e] = hydra::thrust::get<2>(r);
    }
}

template <size_t N, typename GRND>
__device__ void generate_mothers(MothersArgs<N> const& args, uint64_t first, uint64_t n,
                                 const hydra::Vector4R* mothers, hydra::Vector4R* const* cols)
{
    typedef hydra::detail::DecayMothers<N, GRND> F;
    alignas(F) unsigned char raw[sizeof(F)];
    F* f = reinterpret_cast<F*>(raw);
    fill_common(f, args);
    F decayer(*f);
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < n; e += (uint64_t)gridDim.x * blockDim.x) {
        typename F::particles_tuple_type t = decayer(first + e, mothers[e]);
        hydra::Vector4R p[N];
        hydra::detail::assignTupleToArray(t, p);
#pragma unroll
        for (size_t i = 0; i < N; i++) cols[i][e] = p[i];
    }
}

template <size_t N, typename GRND>
__device__ void average_mothers(MothersArgs<N> const& args, BWij bw, uint64_t first, uint64_t n,
                                const hydra::Vector4R* mothers, hydra::detail::StatsPHSP* partial)
{
    typedef hydra::detail::AverageMothers<N, GRND, BWij> F;
    alignas(F) unsigned char raw[sizeof(F)];
    F* f = reinterpret_cast<F*>(raw);
    fill_common(f, args);
    f->fFunctor = bw;                       // BWij is trivially copyable
    F avg(*f);
    hydra::detail::AddStatsPHSP add;
    hydra::detail::StatsPHSP acc;
    bool any = false;
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < n; e += (uint64_t)gridDim.x * blockDim.x) {
        hydra::detail::StatsPHSP s = avg(hydra::thrust::make_tuple(size_t(first + e), mothers[e]));
        acc = any ? add(acc, s) : s;
        any = true;
    }
    __shared__ hydra::detail::StatsPHSP sh[kThreads];
    __shared__ bool shany[kThreads];
    sh[threadIdx.x] = acc;
    shany[threadIdx.x] = any;
    __syncthreads();
    for (int w = kThreads / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w && shany[threadIdx.x + w]) {
            sh[threadIdx.x] = shany[threadIdx.x] ? add(sh[threadIdx.x], sh[threadIdx.x + w]) : sh[threadIdx.x + w];
            shany[threadIdx.x] = true;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        hydra::detail::StatsPHSP r = sh[0];
        if (!shany[0]) r.fW = 0.0;
        partial[blockIdx.x] = r;
    }
}

}  // namespace hpsref

using namespace hpsref;

// Generate: cols is a device array of N pointers, each to n Vector4R (32 B, 16-B aligned).
#define REF_GEN(NN, ENG, GRND)                                                                            \
    extern "C" __global__ void __launch_bounds__(kThreads)                                               \
        ref_generate_##NN##_##ENG(MotherArgs<NN> args, uint64_t first, uint64_t n, hydra::Vector4R* const* cols) \
    {                                                                                                     \
        generate<NN, GRND>(args, first, n, cols);                                                         \
    }
// AverageOn of |BW(m_ij)|^2: one StatsPHSP {mean, M2, W} per block into partial[blockIdx.x].
#define REF_AVG(NN, ENG, GRND)                                                                            \
    extern "C" __global__ void __launch_bounds__(kThreads)                                               \
        ref_average_bw_##NN##_##ENG(AvgArgs<NN> args, uint64_t first, uint64_t n,                   \
                                    hydra::detail::StatsPHSP* partial)                                    \
    {                                                                                                     \
        average<NN, GRND>(args, first, n, partial);                                                       \
    }

// Evaluate with two functors (|BW(m_ij)|^2 and m^2(p_k + p_l)): weight and both values per event.
#define REF_EVAL(NN, ENG, GRND)                                                                           \
    extern "C" __global__ void __launch_bounds__(kThreads)                                               \
        ref_evaluate_##NN##_##ENG(MotherArgs<NN> args, BWij bw, M2ij m2, uint64_t first, uint64_t n,      \
                                  double* w, double* f_bw, double* f_m2)                                  \
    {                                                                                                     \
        evaluate<NN, GRND>(args, bw, m2, first, n, w, f_bw, f_m2);                                        \
    }
// Generate and AverageOn with one mother per event (mothers: n Vector4R).
#define REF_MOTHERS(NN, ENG, GRND)                                                                        \
    extern "C" __global__ void __launch_bounds__(kThreads)                                               \
        ref_generate_mothers_##NN##_##ENG(MothersArgs<NN> args, uint64_t first, uint64_t n,              \
                                          const hydra::Vector4R* mothers, hydra::Vector4R* const* cols)   \
    {                                                                                                     \
        generate_mothers<NN, GRND>(args, first, n, mothers, cols);                                        \
    }                                                                                                     \
    extern "C" __global__ void __launch_bounds__(kThreads)                                               \
        ref_average_mothers_bw_##NN##_##ENG(MothersArgs<NN> args, BWij bw, uint64_t first, uint64_t n,   \
                                            const hydra::Vector4R* mothers,                               \
                                            hydra::detail::StatsPHSP* partial)                            \
    {                                                                                                     \
        average_mothers<NN, GRND>(args, bw, first, n, mothers, partial);                                  \
    }

#define REF_ENGINE(NN, ENG, GRND) REF_GEN(NN, ENG, GRND) REF_AVG(NN, ENG, GRND) REF_EVAL(NN, ENG, GRND) \
    REF_MOTHERS(NN, ENG, GRND)
#define REF_ALL(NN)                                         \
    REF_ENGINE(NN, philox, hydra::philox)                   \
    REF_ENGINE(NN, squares3, hydra::default_random_engine)

REF_ALL(2)
REF_ALL(3)
REF_ALL(4)
REF_ALL(5)
REF_ALL(6)
REF_ALL(7)
REF_ALL(8)
REF_ALL(9)
REF_ALL(10)
