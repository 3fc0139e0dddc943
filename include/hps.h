/*
 * hps.h -- C ABI of the GB300-native phase-space generator (libhps.so).
 *
 * This is the drop-in seam for Hydra's phase-space hot path.  In Hydra the
 * user calls hydra::PhaseSpace<N,GRND>::{Generate, AverageOn, Evaluate}; each
 * builds a by-value functor {seed, ECM, max weight, beta, masses[N]} and hands
 * it to exactly one Thrust algorithm through the launch helpers in
 * hydra/detail/launch_decayers.inl:66-182.  Every entry point below replaces
 * one of those launches (or a Decays member that walks the same storage); the
 * reference line it replaces is cited beside it.  hps_channel carries the same
 * scalars as the reference functor, computed on the host exactly as the
 * reference constructor does (hps_channel_init).
 *
 * Conventions
 *  - All calls are asynchronous on the given CUDA stream (cudaStream_t passed
 *    as void*, NULL = legacy default stream) unless stated otherwise; inputs
 *    and outputs are DEVICE pointers owned by the caller.  The library never
 *    allocates an output.
 *  - Event e of a call [first_evt, first_evt + n) is the reference's event
 *    index first_evt + e: its random stream is the reference engine seeded
 *    with channel.seed after discard(first_evt + e + 3N).
 *  - Four-vectors are stored as Hydra's Decays does (hydra/Decays.h:72 and
 *    hydra/multivector.h:70-108): one column per daughter, each column an
 *    array of n Vector4R = {E, px, py, pz} doubles (32 bytes per event,
 *    hydra/Vector4R.h:59,130).  Columns must be 32-byte aligned.
 *  - Errors: every call returns hps_status; hps_last_error() gives a message
 *    for the calling thread.  Where the reference throws, the status maps to
 *    its exception (HPS_ERR_BAD_ARG -> std::invalid_argument,
 *    HPS_ERR_NO_ENERGY -> std::runtime_error, HPS_ERR_CUDA -> thrust::system_error).
 */
#ifndef HPS_H_
#define HPS_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HPS_MAX_DAUGHTERS 10
#define HPS_ABI_VERSION 4

typedef enum hps_status {
    HPS_OK = 0,
    HPS_ERR_BAD_ARG = 1,      /* invalid masses, N, pointers or sizes        */
    HPS_ERR_NO_ENERGY = 2,    /* M - sum(m_i) <= 0                           */
    HPS_ERR_OOM = 3,          /* a scratch allocation failed                 */
    HPS_ERR_BUDGET = 4,       /* request above the admission budget          */
    HPS_ERR_TIMEOUT = 5,      /* a bounded wait gave up                      */
    HPS_ERR_CUDA = 6,         /* CUDA runtime error (message in last_error)  */
    HPS_ERR_UNSUPPORTED = 7   /* combination not built into this library     */
} hps_status;

/* Random engines (template parameter GRND of hydra::PhaseSpace). */
typedef enum hps_engine {
    HPS_ENGINE_PHILOX = 0,    /* hydra::philox  = EngineR123<Philox2x64>, 7 rounds
                                 (hydra/detail/random/EngineR123.h:244, hydra_R123/philox.h:266) */
    HPS_ENGINE_SQUARES3 = 1,  /* hydra::default_random_engine = squares3
                                 (hydra/detail/PRNGTypedefs.h:59, random/squares3.h:67) */
    HPS_ENGINE_MINSTD = 2     /* thrust::random::default_random_engine = minstd_rand
                                 (hydra_thrust/random/linear_congruential_engine.h:279), the engine
                                 of phase_space_range only: accepted by hps_generate_range alone */
} hps_engine;

/* Arithmetic of the kinematics.  FP64 follows the reference in IEEE double;
 * FP32_FIX does rotations and boosts in float, keeping the threshold-sensitive
 * pdk terms, the weight product and all reductions in double. */
typedef enum hps_precision {
    HPS_PREC_FP64 = 0,
    HPS_PREC_FP32_FIX = 1
} hps_precision;

/* One decay channel: the scalars of hydra::detail::DecayMother
 * (hydra/detail/functors/DecayMother.h:63-73). */
typedef struct hps_channel {
    int32_t n_daughters;                 /* N, 2..10                                   */
    int32_t engine;                      /* hps_engine                                 */
    uint64_t seed;                       /* size_t fSeed                               */
    double ecm;                          /* fECM = M - sum(m_i)                        */
    double max_weight;                   /* fMaxWeight = 1/prod PDK                    */
    double beta[3];                      /* fBeta0..2, built as DecayMother.h:88-98    */
    double masses[HPS_MAX_DAUGHTERS];    /* fMasses[N]                                 */
} hps_channel;

/* Per-event functor menu for AverageOn / Evaluate (arbitrary C++ functors
 * cannot cross a C ABI; the C++ headers in include/hydra/ compile any functor
 * into the kernel instead).
 *   HPS_FN_ONE     f = 1
 *   HPS_FN_MASS2   f = mass2(p_i + p_j)
 *   HPS_FN_BW2     f = 1 / ((a^2 - mass2(p_i + p_j))^2 + (a b)^2),
 *                  |relativistic Breit-Wigner|^2 with mass a and width b. */
typedef enum hps_functor_kind { HPS_FN_ONE = 0, HPS_FN_MASS2 = 1, HPS_FN_BW2 = 2 } hps_functor_kind;

typedef struct hps_functor {
    int32_t kind;   /* hps_functor_kind */
    int32_t i;
    int32_t j;
    int32_t reserved;
    double a;
    double b;
} hps_functor;

/* Weighted statistics of AverageOn: hydra::detail::StatsPHSP
 * (hydra/detail/functors/StatsPHSP.h:38-59).  The reference returns
 * (mean, sqrt(m2)/w) (hydra/detail/PhaseSpace.inl:271). */
typedef struct hps_stats {
    double mean;
    double m2;
    double w;
} hps_stats;

/* ---------------------------------------------------------------- set-up -- */

/* Fills *ch as hydra::PhaseSpace<N,GRND>'s constructor (hydra/detail/PhaseSpace.inl:42-90)
 * plus DecayMother's constructor (DecayMother.h:76-101) do.  mother = {E,px,py,pz}
 * of the mother four-vector given to Generate (only the final-boost vector
 * depends on it; ECM uses mother_mass, as in the reference).
 * Returns HPS_ERR_BAD_ARG for a mass <= 0 or N outside 2..10, HPS_ERR_NO_ENERGY when
 * M - sum(m_i) <= 0.  Host-only, synchronous. */
hps_status hps_channel_init(hps_channel* ch, int32_t n_daughters, int32_t engine, uint64_t seed,
                            double mother_mass, const double* masses, const double* mother);

/* The reference's default seed when SetSeed is never called:
 * 1 * (1 + hash_range(masses)) with std::hash<double> of the C++ standard library
 * (hydra/detail/PhaseSpace.inl:44,64; hydra/detail/Hash.h:45-58). */
uint64_t hps_default_seed(int32_t n_daughters, const double* masses);

/* --------------------------------------------------------------- compute -- */

/* Generate: replaces hydra::detail::launch_decayer -> thrust::tabulate(Decays, DecayMother)
 * (hydra/detail/launch_decayers.inl:133-149, called from PhaseSpace.inl:351-394).
 * cols[k] (host array of N device pointers) receives daughter k's Vector4R column.
 * Optional outputs (NULL to skip):
 *   weights[n]  generation-time event weight (the value DecayMother::process returns and
 *               Generate discards, DecayMother.h:285; Evaluate's first column, EvalMother.h:305)
 *   flags[n]    hit-or-miss flag of Decays::Unweight (hydra/detail/Decays.inl:75-89,415-455):
 *               1 when PhaseSpaceWeight(p)/max_weight > u, u from squares3(unweight_seed)
 *               after discard(first_evt + e). */
hps_status hps_generate(const hps_channel* ch, uint64_t first_evt, uint64_t n,
                        double* const* cols, double* weights, uint8_t* flags,
                        uint64_t unweight_seed, int32_t precision, void* stream);

/* Generate into HOST memory: the GPU form of Generate(mother, Decays<..., hydra::host::sys_t>)
 * (PhaseSpace.inl:377-394 with a host-backend Decays).  Same outputs as hps_generate, but
 * host_cols / host_weights / host_flags are host pointers.
 *   chunk_events == 0 and every buffer pinned, device-mapped memory (cudaHostAlloc, or
 *     cudaHostRegister with the mapped flag): the kernel writes straight into host memory
 *     across the CPU-GPU link, no staging.
 *   otherwise: events are produced in chunks of chunk_events (0 = 2^20) into two device staging
 *     buffers from the stream-ordered allocator; each chunk's device->host copies run on a second
 *     stream while the next chunk is generated.
 * Returns when the host memory holds the results (synchronous, like the reference call). */
hps_status hps_generate_host(const hps_channel* ch, uint64_t first_evt, uint64_t n,
                             double* const* host_cols, double* host_weights, uint8_t* host_flags,
                             uint64_t unweight_seed, int32_t precision, uint64_t chunk_events,
                             void* stream);

/* Evaluate: replaces launch_evaluator -> thrust::tabulate(multivector, EvalMother)
 * (hydra/detail/launch_decayers.inl:66-72, PhaseSpace.inl:314-329): per event the
 * tuple (w, f_1(p), ..., f_k(p)) as k+1 columns; weights[n] = w, out[f][n] = f_f(p). */
hps_status hps_evaluate(const hps_channel* ch, uint64_t first_evt, uint64_t n,
                        const hps_functor* functors, int32_t n_functors,
                        double* weights, double* const* out, int32_t precision, void* stream);

/* AverageOn: replaces launch_reducer -> thrust::transform_reduce(AverageMother, AddStatsPHSP)
 * (hydra/detail/launch_decayers.inl:94-106, PhaseSpace.inl:255-273).  Storage-free:
 * events are generated, weighted and reduced in registers.  The reduction tree is fixed
 * by n alone (tiles of HPS_AVG_TILE events, merged pairwise), so the result is
 * bit-identical for every launch shape.  *out (device pointer) receives {mean, M2, W}.
 * Scratch: ceil(n / HPS_AVG_TILE) * 24 bytes; pass workspace/workspace_bytes (device
 * memory, >= hps_average_on_workspace_size(n)) or workspace = NULL to let the library
 * take it from the stream-ordered allocator (cudaMallocAsync) for the call. */
#define HPS_AVG_TILE 4096
size_t hps_average_on_workspace_size(uint64_t n);
hps_status hps_average_on(const hps_channel* ch, uint64_t first_evt, uint64_t n,
                          const hps_functor* functor, hps_stats* out, void* workspace,
                          size_t workspace_bytes, int32_t precision, void* stream);

/* Generate and AverageOn of the same events in one pass: the reference needs two calls,
 * PhaseSpace::Generate(mother, events) and AverageOn(policy, mother, functor, n)
 * (PhaseSpace.inl:255-273, 377-394), which each generate events [first_evt, first_evt + n).
 * The stored events, weights and flags equal those of hps_generate, and *out equals the
 * hps_average_on result, bit for bit (same tiles, same order); the event body runs once instead
 * of twice.  Arguments as in hps_generate and hps_average_on. */
hps_status hps_generate_average(const hps_channel* ch, uint64_t first_evt, uint64_t n, double* const* cols,
                                double* weights, uint8_t* flags, uint64_t unweight_seed,
                                const hps_functor* functor, hps_stats* out, void* workspace,
                                size_t workspace_bytes, int32_t precision, void* stream);

/* hps_generate_average with the Decays, weights and flags in HOST memory (like hps_generate_host):
 * with pinned, device-mapped host buffers one kernel writes the events across the CPU-GPU link and
 * reduces AverageOn meanwhile; otherwise hps_generate_host then hps_average_on.  out is a device
 * pointer; the call returns when both results are complete. */
hps_status hps_generate_average_host(const hps_channel* ch, uint64_t first_evt, uint64_t n,
                                     double* const* host_cols, double* host_weights, uint8_t* host_flags,
                                     uint64_t unweight_seed, const hps_functor* functor, hps_stats* out,
                                     int32_t precision, void* stream);

/* AverageOn that makes no device allocation at all (no counterpart in the reference; Hydra's
 * own reduction always takes temporary storage from its allocator).  It is meant for host
 * programs that may not allocate device memory once they are running -- for example a
 * framework that hands every byte of the GPU to its own pool at start-up, or a process held
 * to a fixed memory quota on a shared GPU -- and so can give neither a workspace nor let the
 * library call cudaMallocAsync.  Same arguments and result as hps_average_on without the
 * workspace; the tile partials live in one fixed device array of HPS_NOALLOC_MAX_EVENTS /
 * HPS_AVG_TILE entries (384 KiB) that every GPU loading the library keeps until the process
 * exits.  Limits and rules:
 *  - n above HPS_NOALLOC_MAX_EVENTS (2^26 events) is rejected with HPS_ERR_BAD_ARG;
 *  - the first call on each device looks up the array's device address (with that device
 *    current) and caches it; make that first call before any stream capture on the device; the
 *    cache assumes the device's primary context lives until the process exits (no
 *    cudaDeviceReset of that device between calls);
 *  - all calls share the one array, so calls that overlap on the GPU (different streams, or
 *    different host threads, on the same device) race and must be serialised by the caller;
 *  - nothing in the array needs clearing between calls: each call writes every entry it reads. */
#define HPS_NOALLOC_MAX_EVENTS (16384ull * HPS_AVG_TILE)
hps_status hps_average_on_noalloc(const hps_channel* ch, uint64_t first_evt, uint64_t n,
                                  const hps_functor* functor, hps_stats* out, int32_t precision,
                                  void* stream);

/* Per-event mothers: mothers[n][4] is a device column of Vector4R, e.g. a daughter column
 * of an earlier hps_generate for a decay chain (examples/phase_space/phsp_chain.inl:216-238).
 *  hps_generate_mothers    Generate(mothers, daughters): DecayMothers (hydra/detail/functors/
 *                          DecayMothers.h:131-260), the stream and ECM of hps_generate, each event
 *                          boosted by its own mother.
 *  hps_average_on_mothers  AverageOn(begin, end, functor): AverageMothers (AverageMothers.h:134-285).
 *  hps_evaluate_mothers    Evaluate(mothers, result, functors): EvalMothers (EvalMothers.h:143-305):
 *                          engine seeded with hash(evt, seed) without discard, ECM and maximum
 *                          weight from each mother's mass.
 * The functor sees (mother, daughter 0, ..., daughter N-1): its indices count the mother as 0.
 * Precision: HPS_PREC_FP64 for all three; HPS_PREC_FP32_FIX for hps_generate_mothers and
 * hps_average_on_mothers (the boost into each mother's frame in light-cone form, the mother's mass
 * formed in float-float; the float errors of the rest-frame kinematics, about 5e-7 of the
 * daughters' energies there, grow to about gamma * 5e-7 of a daughter thrown backwards by a mother
 * of Lorentz factor gamma); hps_evaluate_mothers returns HPS_ERR_UNSUPPORTED for it. */
hps_status hps_generate_mothers(const hps_channel* ch, uint64_t first_evt, uint64_t n, const double* mothers,
                                double* const* cols, double* weights, int32_t precision, void* stream);
hps_status hps_average_on_mothers(const hps_channel* ch, uint64_t first_evt, uint64_t n, const double* mothers,
                                  const hps_functor* functor, hps_stats* out, void* workspace,
                                  size_t workspace_bytes, int32_t precision, void* stream);
hps_status hps_evaluate_mothers(const hps_channel* ch, uint64_t first_evt, uint64_t n, const double* mothers,
                                const hps_functor* functors, int32_t n_functors, double* weights,
                                double* const* out, int32_t precision, void* stream);

/* PhaseSpaceWeight over stored events: replaces Events | Events.GetEventWeightFunctor()
 * (hydra/Decays.h:235-239, hydra/detail/Decays.inl:215-231).  out[n] = max_weight *
 * prod_i pdk(|R + p_i|, m_i, |R|). */
hps_status hps_event_weights(int32_t n_daughters, const double* masses, double max_weight,
                             uint64_t n, const double* const* cols, double* out, void* stream);

/* Unweight flags over stored events: the tagger of Decays::Unweight()
 * (hydra/detail/Decays.inl:75-89, 444-445): flags[e] = weight/max_weight > u(first_evt + e). */
hps_status hps_unweight_flags(int32_t n_daughters, const double* masses, double max_weight,
                              uint64_t n, const double* const* cols, uint64_t unweight_seed,
                              uint64_t first_evt, uint8_t* flags, void* stream);

/* Unweight compaction: the stable_partition of Decays::Unweight() (hydra/detail/Decays.inl:444-453),
 * out of place.  Events with flags[e] != 0 go to cols_out[.][0, A), the others to [A, n), each
 * group in index order; *n_accepted (device pointer, may be NULL) receives A.  weights_in /
 * weights_out (both or neither) carry the weight column along.  Scratch: workspace of at least
 * hps_compact_workspace_size(n) bytes, or NULL for the stream-ordered allocator. */
size_t hps_compact_workspace_size(uint64_t n);
hps_status hps_unweight_compact(int32_t n_daughters, uint64_t n, const double* const* cols_in,
                                const double* weights_in, const uint8_t* flags, double* const* cols_out,
                                double* weights_out, uint64_t* n_accepted, void* workspace,
                                size_t workspace_bytes, void* stream);

/* PhaseSpaceReweight (hydra/detail/Decays.inl:258-411) over a stored sample: out[e] =
 * PhaseSpaceWeight(event e) * functor(event e), the value Decays::Unweight(functor, ...) tests
 * (Decays.inl:472-476).  out may be NULL.  max_out (device, may be NULL) receives the largest
 * value, as thrust::max_element over the same values gives it (Decays.inl:472-474); it is also
 * used as 8 bytes of scratch while the call runs. */
hps_status hps_reweight(int32_t n_daughters, const double* masses, double max_weight, const hps_functor* functor,
                        uint64_t n, const double* const* cols, double* out, double* max_out, void* stream);

/* Hit-or-miss flags from a weight column: flags[e] = weights[e] / W > u(first_evt + e), u the
 * squares3(unweight_seed) uniform after discard(first_evt + e) (FlagDaugthers,
 * Decays.inl:75-89).  W = *max_weight_dev when that device pointer is given (the max_out of
 * hps_reweight), else max_weight.  With hps_reweight and hps_unweight_compact this is
 * Decays::Unweight(functor, weight, seed) (Decays.inl:458-511). */
hps_status hps_weight_flags(uint64_t n, const double* weights, double max_weight, const double* max_weight_dev,
                            uint64_t unweight_seed, uint64_t first_evt, uint8_t* flags, void* stream);

/* Two-dimensional dense histogram of two invariant masses squared, as
 * DenseHistogram<double,2>::Fill(data, weights) (hydra/detail/DenseHistogram.inl:45-103) fills it
 * with data = (m2(p[pair_a0] + p[pair_a1]), m2(p[pair_b0] + p[pair_b1])) -- the Dalitz plot of the
 * reference's phsp_basic example.  Binning is GetGlobalBin's (functors/GetGlobalBin.h:120-138):
 * x_d -> (x_d - lower_d) * grid_d / (upper_d - lower_d); both below 0 -> bin grid0*grid1
 * (underflow), both above grid_d -> grid0*grid1 + 1 (overflow), else x0_bin * grid1 + x1_bin.  A
 * point with one coordinate outside [0, grid_d) and the other not, which the reference maps through
 * an undefined conversion, goes to the overflow bin.  bins has grid0*grid1 + 2 doubles and is
 * overwritten, as Fill overwrites.  Bin sums are formed with atomic additions, so they agree with
 * the reference's in-order sums to rounding (about 1e-15 relative), not bit for bit. */
typedef struct hps_hist2d {
    int32_t pair_a[2];
    int32_t pair_b[2];
    uint64_t grid[2];
    double lower[2];
    double upper[2];
} hps_hist2d;

typedef enum hps_hist_weight {
    HPS_HIST_UNIT = 0,          /* weight 1 */
    HPS_HIST_COLUMN = 1,        /* weights[e] */
    HPS_HIST_PHSP_WEIGHT = 2    /* PhaseSpaceWeight recomputed from the event (Decays.inl:215-231),
                                   the example's dalitz_weights; hps_generate_dalitz: the
                                   generation-time weight instead */
} hps_hist_weight;

hps_status hps_dalitz_histogram(int32_t n_daughters, const double* masses, double max_weight, uint64_t n,
                                const double* const* cols, const double* weights, int32_t weight_mode,
                                const hps_hist2d* hist, double* bins, void* stream);

/* Generate + histogram fused: the events of hps_generate(channel, first_evt, n, ..., precision)
 * binned as hps_dalitz_histogram bins them, never stored.  weight_mode HPS_HIST_UNIT or
 * HPS_HIST_PHSP_WEIGHT (the generation-time weight, which differs from the recomputed
 * PhaseSpaceWeight by rounding only).  HPS_PREC_FP64: the reference's arithmetic throughout.
 * HPS_PREC_FP32_FIX: the FP32_FIX events, their pair masses squared and bins formed in float
 * (X = (x - lower) * (grid / (upper - lower))); every event is counted, and one whose Dalitz
 * variable lies within the float form's error of a bin edge may land in the neighbouring bin. */
hps_status hps_generate_dalitz(const hps_channel* channel, uint64_t first_evt, uint64_t n, int32_t weight_mode,
                               const hps_hist2d* hist, double* bins, int32_t precision, void* stream);

/* phase_space_range (hydra/detail/PhaseSpaceRange.inl:46-73): the lazy range of GenerateDecay
 * (functors/GenerateDecay.h:222-334) with thrust's minstd_rand.  hps_range_channel sets up the
 * channel as GenerateDecay's constructor does: ECM = mother.mass() - sum(m_i), the maximum weight
 * from mother.mass(), the final-boost vector of the moving-mother quirk, seed truncated to the
 * 32-bit GInt_t and engine HPS_ENGINE_MINSTD.  Where GenerateDecay has no checks this returns
 * HPS_ERR_BAD_ARG (a mass <= 0) or HPS_ERR_NO_ENERGY.  hps_generate_range materialises events
 * [first_evt, first_evt + n) of the range: element e is (weights[e], cols[0][e], ...). */
hps_status hps_range_channel(hps_channel* ch, int32_t n_daughters, const double* masses, const double* mother,
                             uint64_t seed);
hps_status hps_generate_range(const hps_channel* ch, uint64_t first_evt, uint64_t n, double* const* cols,
                              double* weights, void* stream);

/* Raw random words of each event's stream (parity instrument): out[e*(3N-4)+k] is the k-th
 * word the reference engine returns for event first_evt+e (EngineR123.h:149-166 returns 64-bit
 * Philox words; squares3.h:105-119 returns 32-bit words, stored zero-extended). */
hps_status hps_rng_words(int32_t n_daughters, int32_t engine, uint64_t seed, uint64_t first_evt,
                         uint64_t n, uint64_t* out, void* stream);

/* ------------------------------------------------------ batched channels, one graph launch -- */

/* Many decay channels of different N and event counts in one graph launch of persistent kernels
 * (FP32_FIX arithmetic): one per N and mode, so that each runs at the occupancy of its own
 * register count, or one over every N (hps_batch_tuning.kernel_form; the autotuner tries both).  There is no
 * single reference call for this: it batches what would be one PhaseSpace::Generate or AverageOn
 * call per channel (PhaseSpace.inl:255-444).  Each item's
 * results are bit-identical to the same request made alone with hps_generate / hps_average_on
 * at HPS_PREC_FP32_FIX: the work units are the same functions of (channel, event index). */
typedef enum hps_batch_mode { HPS_MODE_STORE = 0, HPS_MODE_AVERAGE = 1 } hps_batch_mode;

typedef struct hps_batch_item {
    hps_channel channel;
    uint64_t first_evt;
    uint64_t n_events;
    int32_t mode;                        /* hps_batch_mode                                   */
    int32_t reserved;
    hps_functor functor;                 /* AVERAGE                                          */
    double* cols[HPS_MAX_DAUGHTERS];     /* STORE: device columns, 16-byte aligned           */
    double* weights;                     /* STORE: optional generation-time weights          */
    uint8_t* flags;                      /* STORE: optional unweight flags                   */
    uint64_t unweight_seed;              /* STORE: seed of the unweight uniforms             */
    hps_stats* stats;                    /* AVERAGE: device output {mean, M2, W}             */
} hps_batch_item;

/* Launch shape of the persistent kernels: each gets min(ctas_per_sm, the CTAs of it that fit
 * on an SM) x SM count CTAs of 256 threads; store items are cut into work units of
 * store_tile_events events (a multiple of 256), AverageOn items into tiles of HPS_AVG_TILE events.
 * kernel_form: HPS_BATCH_PER_N runs one persistent kernel per N and mode as parallel branches of
 * the graph, each at the occupancy of its own register count and with no more CTAs than its work
 * units; HPS_BATCH_ONE_KERNEL runs one
 * persistent kernel over every N (the register count of N = 10 for all).  threads_per_event: 1,
 * each thread owns one event (its kinematics stay in that thread's registers; the random words
 * of a CTA's events are computed cooperatively); 2 (per-N form only), each store event with
 * N >= 7 is computed by two threads of different warps, each holding half of the daughter pairs
 * and computing the stage arithmetic and weight in full.  Results do not depend on the shape. */
typedef enum hps_batch_form { HPS_BATCH_PER_N = 0, HPS_BATCH_ONE_KERNEL = 1 } hps_batch_form;

typedef struct hps_batch_tuning {
    int32_t ctas_per_sm;
    int32_t store_tile_events;
    int32_t kernel_form;                 /* hps_batch_form */
    int32_t threads_per_event;           /* 1 (0 reads as 1), or 2 for the store items with N >= 7: each event's
                                            daughter pairs split between two threads (fewer
                                            registers per thread, the stage arithmetic twice) */
} hps_batch_tuning;

typedef struct hps_batch_plan hps_batch_plan;

/* A plan owns the device item table (max_items entries), the AverageOn tile partials
 * (max_average_tiles x 24 bytes), a pinned staging copy of the table and the instantiated
 * CUDA graph (counter reset, the persistent kernel(s), per-item merge).  tuning = NULL picks the default shape; hps_batch_autotune chooses one by timing. */
hps_status hps_batch_create(hps_batch_plan** plan, int32_t max_items, uint64_t max_average_tiles,
                            int32_t precision, const hps_batch_tuning* tuning);
/* Validates the items and uploads the table asynchronously on `stream`; sets each class kernel's
 * grid in the plan's graph to at most its number of work units (from the next launch; no new graph). */
hps_status hps_batch_set_items(hps_batch_plan* plan, const hps_batch_item* items, int32_t n_items,
                               void* stream);
/* One graph launch over the current items, asynchronous on `stream`. */
hps_status hps_batch_launch(hps_batch_plan* plan, void* stream);
hps_status hps_batch_get_tuning(const hps_batch_plan* plan, hps_batch_tuning* out);
hps_status hps_batch_set_tuning(hps_batch_plan* plan, const hps_batch_tuning* tuning);
/* Times candidate launch shapes on the current items (each run writes the items' outputs) and
 * keeps the fastest; with cache_path, results are read from / appended to that text file,
 * keyed by device, precision and the item mix.  Synchronous. */
hps_status hps_batch_autotune(hps_batch_plan* plan, void* stream, const char* cache_path,
                              hps_batch_tuning* chosen);
hps_status hps_batch_destroy(hps_batch_plan* plan);

/* ------------------------------------------------------------ serving loop -- */

/* A request server with continuous batching: requests (Generate-into-Decays or AverageOn of
 * one channel) are submitted from any host thread, admitted in arrival order while their
 * output memory fits the device budget, and run by a scheduler thread as batched persistent
 * launches (hps_batch_*).  A launch takes every admitted request that still has work, store
 * requests in slices of at most slice_events events, so requests that arrive while others are
 * on the GPU join the next launch and run alongside them.  Results are bit-identical to the
 * same request run alone with hps_generate / hps_average_on at HPS_PREC_FP32_FIX.
 * The channel table and each request's event counters live in the device item table of the
 * launch.  No reference counterpart: Hydra runs one blocking call per request. */
typedef struct hps_server hps_server;
typedef uint64_t hps_ticket;

typedef struct hps_server_config {
    uint64_t budget_bytes;       /* device bytes for request outputs (store columns etc.)    */
    uint64_t slice_events;       /* max events of one store request per launch (0: 2^22)    */
    int32_t max_batch_items;     /* items per launch (0: 1024)                              */
    int32_t max_inflight;        /* admitted requests not yet released (0: 4096)            */
    uint64_t max_average_events; /* AverageOn events per launch (0: 2^30)                   */
    int32_t fail_alloc_after;    /* test hook: the n-th output allocation fails (0: never)  */
    int32_t reserved;
} hps_server_config;

typedef struct hps_request {
    hps_channel channel;
    uint64_t first_evt;
    uint64_t n_events;
    int32_t mode;                /* HPS_MODE_STORE or HPS_MODE_AVERAGE                      */
    int32_t want_flags;          /* store: also produce unweight flags                      */
    hps_functor functor;         /* AverageOn                                               */
    uint64_t unweight_seed;
} hps_request;

typedef struct hps_result {
    int32_t status;              /* HPS_OK, or the error that ended the request             */
    int32_t mode;
    uint64_t n_events;
    double* cols[HPS_MAX_DAUGHTERS];   /* store: device columns, valid until hps_server_release */
    double* weights;             /* store: generation-time weights                          */
    uint8_t* flags;              /* store: unweight flags, if requested                     */
    hps_stats stats;             /* AverageOn: {mean, M2, W}                                */
    double t_submit, t_admit, t_done;  /* seconds on the server's steady clock              */
} hps_result;

typedef struct hps_server_stats {
    uint64_t submitted, admitted, completed, cancelled, failed, released;
    uint64_t launches, events_done;
    uint64_t bytes_in_use, bytes_peak;
} hps_server_stats;

/* Starts the scheduler thread on the current device. */
hps_status hps_server_create(hps_server** server, const hps_server_config* config);
/* Queues a request (thread-safe, non-blocking).  HPS_ERR_BUDGET if it can never fit. */
hps_status hps_server_submit(hps_server* server, const hps_request* request, hps_ticket* ticket);
/* *done = 1 and *result filled once the request has finished (or failed / been cancelled). */
hps_status hps_server_poll(hps_server* server, hps_ticket ticket, hps_result* result, int32_t* done);
/* Waits at most timeout_s seconds; HPS_ERR_TIMEOUT if the request is still running. */
hps_status hps_server_wait(hps_server* server, hps_ticket ticket, hps_result* result, double timeout_s);
/* Completion queue: hands out finished requests in the order they finished, each once;
 * waits at most timeout_s seconds (HPS_ERR_TIMEOUT when none finished). */
hps_status hps_server_next_done(hps_server* server, hps_ticket* ticket, hps_result* result, double timeout_s);
/* Cancels a request that has not been admitted yet (HPS_ERR_BAD_ARG once it runs). */
hps_status hps_server_cancel(hps_server* server, hps_ticket ticket);
/* Returns a finished request's output memory to the budget; the ticket becomes invalid. */
hps_status hps_server_release(hps_server* server, hps_ticket ticket);
hps_status hps_server_get_stats(hps_server* server, hps_server_stats* stats);
/* Stops the scheduler after the running launches finish; queued requests are cancelled. */
hps_status hps_server_destroy(hps_server* server);

/* ------------------------------------------------------------------ misc -- */

const char* hps_last_error(void);
int32_t hps_abi_version(void);

#ifdef __cplusplus
}
#endif

#endif /* HPS_H_ */
