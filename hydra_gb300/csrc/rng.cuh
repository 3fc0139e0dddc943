// rng.cuh -- counter-based random streams of the phase-space generator.
//
// Bit-exact with Hydra's engines as DecayMother uses them
// (hydra/detail/functors/DecayMother.h:166-168: construct from the seed, discard(evt+3N)):
//   * splitmix64 key derivation   hydra/detail/random/splitmix.h:56-61
//   * Philox2x64, 7 rounds        hydra/detail/external/hydra_R123/philox.h:266-268,281-358
//     EngineR123 pre-increments its 128-bit counter before each 2-word block
//     (EngineR123.h:149-166, array.h:151-183), so event evt reads blocks at
//     counters evt+3N+1, evt+3N+2, ... two 64-bit words each.
//   * squares3                    hydra/detail/random/squares3.h:104-125: one 32-bit word
//     per counter, counters evt+3N, evt+3N+1, ...
//   * uniform on [0,1)            hydra_thrust/random/detail/uniform_real_distribution.inl:70-79:
//     double(x) / 2^64 (Philox: double(2^64-1) rounds to 2^64) or x / 2^32 (squares3).
//   * thrust's default_random_engine (minstd_rand), used only by phase_space_range
//     (hydra/detail/PhaseSpaceRange.inl:46-73): x <- 48271 x mod 2^31-1, seeded with seed mod
//     2^31-1 (0 -> 1), discard(z) = multiply by 48271^z; uniform = double(x - 1) / 2147483646.
#pragma once
#include <cstdint>

namespace hps {

enum : int { kPhilox = 0, kSquares3 = 1, kMinstd = 2 };

// The FP32_FIX kernels carry one more compile-time choice in their ENGINE parameter: bit
// kPreciseForm selects the float-float boosts of the event body (genbod_f32.cuh, event_body).
// The random streams depend only on engine_of(ENGINE).
constexpr int kPreciseForm = 4;
__host__ __device__ constexpr int engine_of(int e) { return e & 3; }

// minstd_rand arithmetic modulo the Mersenne prime 2^31 - 1: x < 2^62 folds as
// (x mod 2^31) + (x >> 31), twice, then one conditional subtraction; exact.
constexpr uint32_t kLcgA = 48271u;
constexpr uint32_t kLcgM = 2147483647u;

__host__ __device__ __forceinline__ uint32_t lcg_mulmod(uint32_t a, uint32_t b)
{
    uint64_t x = static_cast<uint64_t>(a) * b;
    x = (x & kLcgM) + (x >> 31);
    x = (x & kLcgM) + (x >> 31);
    return static_cast<uint32_t>(x >= kLcgM ? x - kLcgM : x);
}

// 48271^z mod 2^31 - 1 by square-and-multiply.
__host__ __device__ __forceinline__ uint32_t lcg_pow(uint64_t z)
{
    uint32_t acc = 1u, mult = kLcgA;
    while (z) {
        if (z & 1u) acc = lcg_mulmod(acc, mult);
        mult = lcg_mulmod(mult, mult);
        z >>= 1;
    }
    return acc;
}

// The engine state after seeding: the 32-bit seed reduced mod 2^31 - 1, 0 mapped to 1.
__host__ __device__ __forceinline__ uint32_t lcg_seed_state(uint64_t seed)
{
    const uint32_t s = static_cast<uint32_t>(seed) % kLcgM;
    return s == 0u ? 1u : s;
}

__host__ __device__ __forceinline__ uint64_t splitmix64(uint64_t x)
{
    uint64_t z = x + 0x9e3779b97f4a7c15ULL;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

// Philox2x64 bijection with 7 rounds: round = (hi(M*c0) ^ key ^ c1, lo(M*c0)),
// key bumped by the golden-ratio Weyl constant between rounds.
__device__ __forceinline__ void philox2x64_7(uint64_t c0, uint64_t c1, uint64_t key,
                                             uint64_t& o0, uint64_t& o1)
{
    constexpr uint64_t M = 0xD2B74407B1CE6E93ULL;
    constexpr uint64_t W = 0x9E3779B97F4A7C15ULL;
#pragma unroll
    for (int r = 0; r < 7; ++r) {
        if (r > 0) key += W;
        const uint64_t hi = __umul64hi(M, c0);
        const uint64_t lo = M * c0;
        c0 = hi ^ key ^ c1;
        c1 = lo;
    }
    o0 = c0;
    o1 = c1;
}

__host__ __device__ __forceinline__ uint32_t squares3_word(uint64_t key, uint64_t ctr)
{
    uint64_t x = key * ctr;
    const uint64_t y = x;
    const uint64_t z = y + key;
    x = x * x + y; x = (x >> 32) | (x << 32);
    x = x * x + z; x = (x >> 32) | (x << 32);
    return static_cast<uint32_t>((x * x + y) >> 32);
}

// Number of uniforms one event draws: N-2 invariant masses + 2(N-1) angles.
template <int N> struct Draws { static constexpr int value = 3 * N - 4; };

// All raw words a stream yields from counter state `base` (zero-extended for squares3).
template <int N, int ENGINE>
__device__ __forceinline__ void stream_words(uint64_t key, uint64_t base, uint64_t (&w)[3 * N - 4])
{
    constexpr int NW = 3 * N - 4;
    if constexpr (engine_of(ENGINE) == kPhilox) {
        constexpr int NB = (NW + 1) / 2;
#pragma unroll
        for (int b = 0; b < NB; ++b) {
            const uint64_t c0 = base + 1u + b;
            const uint64_t c1 = (c0 < base) ? 1u : 0u;     // carry of the 128-bit counter
            uint64_t o0, o1;
            philox2x64_7(c0, c1, key, o0, o1);
            w[2 * b] = o0;
            if (2 * b + 1 < NW) w[2 * b + 1] = o1;
        }
    } else if constexpr (engine_of(ENGINE) == kMinstd) {
        // key = seeded state; the first draw after discard(base) is state * 48271^(base+1)
        uint32_t x = lcg_mulmod(static_cast<uint32_t>(key), lcg_pow(base + 1u));
        w[0] = x;
#pragma unroll
        for (int k = 1; k < NW; ++k) {
            x = lcg_mulmod(x, kLcgA);
            w[k] = x;
        }
    } else {
#pragma unroll
        for (int k = 0; k < NW; ++k) w[k] = squares3_word(key, base + k);
    }
}

// All raw words of event `evt`: the engine after discard(evt + 3N), size_t arithmetic.
template <int N, int ENGINE>
__device__ __forceinline__ void event_words(uint64_t key, uint64_t evt, uint64_t (&w)[3 * N - 4])
{
    stream_words<N, ENGINE>(key, evt + 3u * N, w);
}

template <int ENGINE>
__device__ __forceinline__ double word_to_uniform(uint64_t x)
{
    if constexpr (engine_of(ENGINE) == kPhilox) return __ull2double_rn(x) * 0x1p-64;
    else if constexpr (engine_of(ENGINE) == kMinstd)
        return __ddiv_rn(static_cast<double>(static_cast<uint32_t>(x) - 1u), 2147483646.0);
    else return static_cast<double>(static_cast<uint32_t>(x)) * 0x1p-32;
}

// Compare-exchange on raw words: the uniform map is monotone, so sorting the
// words sorts the uniforms exactly as the reference's bubble sort of doubles
// (DecayMother.h:128-151, 184) -- equal doubles are interchangeable.
__device__ __forceinline__ void cswap(uint64_t& a, uint64_t& b)
{
    const uint64_t lo = a < b ? a : b;
    const uint64_t hi = a < b ? b : a;
    a = lo;
    b = hi;
}

// Odd-even transposition network on w[0..K-1]; K <= 8 here.
template <int K>
__device__ __forceinline__ void sort_words(uint64_t* w)
{
#pragma unroll
    for (int pass = 0; pass < K; ++pass) {
#pragma unroll
        for (int i = pass & 1; i + 1 < K; i += 2) cswap(w[i], w[i + 1]);
    }
}

}  // namespace hps

namespace hps {

// ---------------------------------------------------------------------------------------------
// CTA-shared random words.  Event e draws the stream at counters e+3N+1+b (Philox blocks) or
// e+3N+k (squares3 words), so the NT consecutive events of a CTA need only NT + B - 1 distinct
// Philox blocks (B = blocks per event) instead of NT*B: each thread computes one block (B - 1
// threads a second), parks it in shared memory, and reads back the B blocks of its own event.
// The words are the same words, bit for bit; only who computes them changes.
// ---------------------------------------------------------------------------------------------

template <int N, int ENGINE, int NT> struct WordShare {
    static constexpr int NW = 3 * N - 4;
    static constexpr int B = (engine_of(ENGINE) == kPhilox) ? (NW + 1) / 2 : NW;   // items per event
    static constexpr int SLOTS = NT + B - 1;
    static constexpr int BYTES = SLOTS * ((engine_of(ENGINE) == kPhilox) ? 16 : 8);
    static constexpr int BYTES2 = 2 * BYTES;                            // two buffers, see below
};

// All NT threads of the CTA must call together; e0 = event of thread 0.  smem holds two buffers
// (WordShare::BYTES2) and `parity` picks one: a call writes its buffer, waits at one barrier, and
// reads it back.  Consecutive calls alternate the parity, so the next call's writes go to the
// other buffer, and the barrier of that call keeps the writes of the call after it away from this
// one's reads; a call that repeats the previous call's parity must follow a __syncthreads.  Near
// the end of the 2^64 counter range the Philox carry into the high counter word differs between
// neighbouring events, so there each thread computes its own blocks (a CTA-uniform branch).
template <int N, int ENGINE, int NT>
__device__ __forceinline__ void cta_event_words(uint64_t key, uint64_t e0, void* smem, uint64_t (&w)[3 * N - 4],
                                                int parity)
{
    using S = WordShare<N, ENGINE, NT>;
    const int t = threadIdx.x;
    smem = static_cast<unsigned char*>(smem) + (parity & 1) * S::BYTES;
    if constexpr (engine_of(ENGINE) == kPhilox) {
        ulonglong2* slots = static_cast<ulonglong2*>(smem);
        const uint64_t c_first = e0 + 3u * N + 1u;                 // counter of slot 0
        if (e0 <= ~uint64_t(0) - (3u * N + S::SLOTS)) {            // no counter of the CTA wraps
            {
                uint64_t o0, o1;
                philox2x64_7(c_first + t, 0, key, o0, o1);
                slots[t] = make_ulonglong2(o0, o1);
            }
            if (t < S::B - 1) {
                uint64_t o0, o1;
                philox2x64_7(c_first + NT + t, 0, key, o0, o1);
                slots[NT + t] = make_ulonglong2(o0, o1);
            }
            __syncthreads();
#pragma unroll
            for (int b = 0; b < S::B; ++b) {
                const ulonglong2 v = slots[t + b];
                w[2 * b] = v.x;
                if (2 * b + 1 < S::NW) w[2 * b + 1] = v.y;
            }
        } else {
            event_words<N, kPhilox>(key, e0 + t, w);
        }
    } else {
        uint64_t* slots = static_cast<uint64_t*>(smem);
        const uint64_t c_first = e0 + 3u * N;                      // squares3 counters wrap with no carry
        slots[t] = squares3_word(key, c_first + t);
        if (t < S::B - 1) slots[NT + t] = squares3_word(key, c_first + NT + t);
        __syncthreads();
#pragma unroll
        for (int k = 0; k < S::NW; ++k) w[k] = slots[t + k];
    }
}


// Two chunks of NT events per call (thread t owns events e0 + t and e0 + NT + t): the 2NT
// consecutive events' words with one barrier, laid out as cta_event_words lays out 2NT events.
// smem holds two buffers of WordShare<N, ENGINE, 2 NT>::BYTES; parity as in cta_event_words.
template <int N, int ENGINE, int NT>
__device__ __forceinline__ void cta_event_words_pair(uint64_t key, uint64_t e0, void* smem,
                                                     uint64_t (&wa)[3 * N - 4], uint64_t (&wb)[3 * N - 4],
                                                     int parity)
{
    using S = WordShare<N, ENGINE, 2 * NT>;
    const int t = threadIdx.x;
    smem = static_cast<unsigned char*>(smem) + (parity & 1) * S::BYTES;
    if constexpr (engine_of(ENGINE) == kPhilox) {
        ulonglong2* slots = static_cast<ulonglong2*>(smem);
        const uint64_t c_first = e0 + 3u * N + 1u;
        if (e0 <= ~uint64_t(0) - (3u * N + S::SLOTS)) {
            uint64_t o0, o1;
            philox2x64_7(c_first + t, 0, key, o0, o1);
            slots[t] = make_ulonglong2(o0, o1);
            philox2x64_7(c_first + NT + t, 0, key, o0, o1);
            slots[NT + t] = make_ulonglong2(o0, o1);
            if (t < S::B - 1) {
                philox2x64_7(c_first + 2 * NT + t, 0, key, o0, o1);
                slots[2 * NT + t] = make_ulonglong2(o0, o1);
            }
            __syncthreads();
#pragma unroll
            for (int b = 0; b < S::B; ++b) {
                const ulonglong2 va = slots[t + b], vb = slots[NT + t + b];
                wa[2 * b] = va.x;
                wb[2 * b] = vb.x;
                if (2 * b + 1 < S::NW) {
                    wa[2 * b + 1] = va.y;
                    wb[2 * b + 1] = vb.y;
                }
            }
        } else {
            event_words<N, kPhilox>(key, e0 + t, wa);
            event_words<N, kPhilox>(key, e0 + NT + t, wb);
        }
    } else {
        uint64_t* slots = static_cast<uint64_t*>(smem);
        const uint64_t c_first = e0 + 3u * N;
        slots[t] = squares3_word(key, c_first + t);
        slots[NT + t] = squares3_word(key, c_first + NT + t);
        if (t < S::B - 1) slots[2 * NT + t] = squares3_word(key, c_first + 2 * NT + t);
        __syncthreads();
#pragma unroll
        for (int k = 0; k < S::NW; ++k) {
            wa[k] = slots[t + k];
            wb[k] = slots[NT + t + k];
        }
    }
}


// The fill half of cta_event_words_pair: the 2NT events' words into the parity buffer and one
// barrier.  Returns false (and writes nothing) near the end of the counter range, where each
// thread computes its own words.
template <int N, int ENGINE, int NT>
__device__ __forceinline__ bool cta_words_pair_fill(uint64_t key, uint64_t e0, void* smem, int parity)
{
    using S = WordShare<N, ENGINE, 2 * NT>;
    const int t = threadIdx.x;
    smem = static_cast<unsigned char*>(smem) + (parity & 1) * S::BYTES;
    if constexpr (engine_of(ENGINE) == kPhilox) {
        if (!(e0 <= ~uint64_t(0) - (3u * N + S::SLOTS))) return false;
        ulonglong2* slots = static_cast<ulonglong2*>(smem);
        const uint64_t c_first = e0 + 3u * N + 1u;
        uint64_t o0, o1;
        philox2x64_7(c_first + t, 0, key, o0, o1);
        slots[t] = make_ulonglong2(o0, o1);
        philox2x64_7(c_first + NT + t, 0, key, o0, o1);
        slots[NT + t] = make_ulonglong2(o0, o1);
        if (t < S::B - 1) {
            philox2x64_7(c_first + 2 * NT + t, 0, key, o0, o1);
            slots[2 * NT + t] = make_ulonglong2(o0, o1);
        }
    } else {
        uint64_t* slots = static_cast<uint64_t*>(smem);
        const uint64_t c_first = e0 + 3u * N;
        slots[t] = squares3_word(key, c_first + t);
        slots[NT + t] = squares3_word(key, c_first + NT + t);
        if (t < S::B - 1) slots[2 * NT + t] = squares3_word(key, c_first + 2 * NT + t);
    }
    __syncthreads();
    return true;
}

// The read half: the words of event e0 + h NT + t (h = 0 or 1) from the filled buffer.
template <int N, int ENGINE, int NT>
__device__ __forceinline__ void cta_words_pair_read(const void* smem, int parity, int h, uint64_t (&w)[3 * N - 4])
{
    using S = WordShare<N, ENGINE, 2 * NT>;
    const int t = threadIdx.x + h * NT;
    smem = static_cast<const unsigned char*>(smem) + (parity & 1) * S::BYTES;
    if constexpr (engine_of(ENGINE) == kPhilox) {
        const ulonglong2* slots = static_cast<const ulonglong2*>(smem);
#pragma unroll
        for (int b = 0; b < S::B; ++b) {
            const ulonglong2 v = slots[t + b];
            w[2 * b] = v.x;
            if (2 * b + 1 < S::NW) w[2 * b + 1] = v.y;
        }
    } else {
        const uint64_t* slots = static_cast<const uint64_t*>(smem);
#pragma unroll
        for (int k = 0; k < S::NW; ++k) w[k] = slots[t + k];
    }
}

// Two threads per event: NE consecutive events (e0 + t, t = threadIdx.x % NE) on 2 NE threads.
// Thread k < NE + B - 1 computes slot k; every thread reads back the B items of its event.  smem
// and parity as in cta_event_words, with WordShare<N, ENGINE, NE>.
template <int N, int ENGINE, int NE>
__device__ __forceinline__ void cta_event_words_split(uint64_t key, uint64_t e0, void* smem, uint64_t (&w)[3 * N - 4],
                                                      int parity)
{
    using S = WordShare<N, ENGINE, NE>;
    const int k = threadIdx.x, t = threadIdx.x % NE;
    smem = static_cast<unsigned char*>(smem) + (parity & 1) * S::BYTES;
    if constexpr (engine_of(ENGINE) == kPhilox) {
        ulonglong2* slots = static_cast<ulonglong2*>(smem);
        const uint64_t c_first = e0 + 3u * N + 1u;
        if (e0 <= ~uint64_t(0) - (3u * N + S::SLOTS)) {
            if (k < S::SLOTS) {
                uint64_t o0, o1;
                philox2x64_7(c_first + k, 0, key, o0, o1);
                slots[k] = make_ulonglong2(o0, o1);
            }
            __syncthreads();
#pragma unroll
            for (int b = 0; b < S::B; ++b) {
                const ulonglong2 v = slots[t + b];
                w[2 * b] = v.x;
                if (2 * b + 1 < S::NW) w[2 * b + 1] = v.y;
            }
        } else {
            event_words<N, kPhilox>(key, e0 + t, w);
        }
    } else {
        uint64_t* slots = static_cast<uint64_t*>(smem);
        const uint64_t c_first = e0 + 3u * N;
        if (k < S::SLOTS) slots[k] = squares3_word(key, c_first + k);
        __syncthreads();
#pragma unroll
        for (int i = 0; i < S::NW; ++i) w[i] = slots[t + i];
    }
}

}  // namespace hps
