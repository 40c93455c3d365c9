/*
 * polyq_gb300.h -- C-ABI of the GB300 amplitude-evaluation path for polyq.
 *
 * Drop-in boundary for the reference crate's Simulator API (src/sim.rs).  A Rust,
 * Python (ctypes) or C++ host binds these plain-C entry points; the library owns all
 * device memory, streams and kernels.  Every entry point returns a pq_status and never
 * aborts; pq_last_error() returns the message of the calling thread's last failure.
 *
 * Conventions
 *   gate codes   0 H, 1 X, 2 Y, 3 Z, 4 S, 5 SDG, 6 T, 7 TDG, 8 P(phase), 9 CZ(q0,q1),
 *                10 CX(control q0, target q1), 11 SWAP(q0,q1), 12 GPHASE(phase)
 *                (src/circuit.rs:25-42)
 *   phase        uint32 k meaning the angle 2*pi*k/2^32 (src/phase.rs:22-24)
 *   bitstrings   ceil(num_qubits/64) little-endian uint64 words per bitstring,
 *                qubit q = bit q (src/sim.rs:74-76)
 *   complex      interleaved (re, im) doubles
 *   strategy     0 Auto, 1 Cached, 2 Pairs(pairs) (src/sim.rs:41-48)
 *
 * An amplitude that is exactly zero (contradictory boundary, inconsistent radical
 * system) is a value, not an error (src/sim.rs:172-174, src/engine.rs:595-597).
 */
#ifndef POLYQ_GB300_H
#define POLYQ_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define PQ_API __attribute__((visibility("default")))
#else
#define PQ_API
#endif

typedef enum pq_status {
    PQ_OK = 0,
    PQ_ERR_INVALID_ARG = 1,        /* malformed circuit, boundary or handle (the reference panics) */
    PQ_ERR_OUT_OF_MEMORY = 2,      /* device or host allocation failed */
    PQ_ERR_ADMISSION_REFUSED = 3,  /* branch dimension above the cap, or memory budget exceeded */
    PQ_ERR_TIMEOUT = 4,            /* a bounded wait expired */
    PQ_ERR_DEVICE = 5,             /* CUDA error (message in pq_last_error) */
    PQ_ERR_UNSUPPORTED = 6,        /* structure outside the kernels' limits (d > 62 or > 64 pivots) */
    PQ_ERR_NO_DEVICE = 7,          /* no CUDA device visible */
    PQ_ERR_INTERNAL = 8
} pq_status;

typedef struct pq_sim pq_sim;
typedef struct pq_batch pq_batch;
typedef struct pq_server pq_server;

/* Circuit description; the arrays stay owned by the caller (read during the call only). */
typedef struct pq_circuit_desc {
    int32_t num_qubits;
    int32_t num_gates;
    const uint8_t *op;
    const int32_t *q0;
    const int32_t *q1;
    const uint32_t *phase;
} pq_circuit_desc;

/* Engine statistics: EngineStats of branch 0 (src/engine.rs:64-79) + pairs (src/sim.rs:161-168). */
typedef struct pq_stats {
    int64_t free_vars, planes, lines, radical, terms, branch_dim;
    int64_t pairs;          /* decomposed T-pairs p */
    int64_t num_branches;   /* 2^p branch engines */
    double branches_per_amplitude;  /* sum over branch engines of 2^d */
    int64_t device_bytes;   /* HBM held by the simulator's resident structures (main and
                               cached marginal engines) */
    double build_seconds;   /* host compile + elimination + upload time */
} pq_stats;

/* Enumeration tuning (0 fields take the library defaults / autotuned values). */
typedef struct pq_tuning {
    int32_t inner_dims;      /* Gray steps per lane chunk = 2^inner_dims (4..14) */
    int32_t chunks_per_lane; /* chunks a lane walks per work item (1..64) */
    int32_t block_warps;     /* warps per CTA of the enumeration kernel (1..8) */
    int32_t max_branch_dim;  /* admission cap on d per branch engine (<= 62) */
    int32_t blocks_per_sm;   /* enumeration kernel register budget: 2, 3 or 4 blocks of 256 per SM */
    int32_t unit_chunks;     /* at most this many chunks (1, 2, 4, 8) share each weight-table load */
    int32_t chunk_tables;    /* 1: sum each chunk by one lookup in its engine's chunk-sum table (a
                                Walsh transform of the weight table over the walked coordinates,
                                FP64) instead of enumerating its branches; 2 or 0: enumerate */
} pq_tuning;

/* ---- library ------------------------------------------------------------------------ */
PQ_API const char *pq_version(void);
PQ_API const char *pq_last_error(void);
/* Select the CUDA device used by subsequently created objects (default 0). */
PQ_API pq_status pq_init(int32_t device);
PQ_API pq_status pq_set_default_tuning(const pq_tuning *t);
PQ_API pq_status pq_get_default_tuning(pq_tuning *t);

/* ---- Simulator (src/sim.rs:139-198) --------------------------------------------------- */
/* Simulator::with_options(circuit, SimOptions{strategy, ..}) -- sim.rs:144-148.
 * Compiles, eliminates and uploads every branch engine; structures stay resident in HBM. */
PQ_API pq_status pq_sim_create(const pq_circuit_desc *circuit, int32_t strategy, int32_t pairs, pq_sim **out);
/* Host-only analysis: compile, eliminate and build every branch engine without a device
 * (stats, canonical dumps; evaluation calls on it return PQ_ERR_NO_DEVICE). */
PQ_API pq_status pq_analyze(const pq_circuit_desc *circuit, int32_t strategy, int32_t pairs, pq_sim **out);
PQ_API void pq_sim_destroy(pq_sim *sim);
/* Simulator::stats / pairs -- sim.rs:161-168 */
PQ_API pq_status pq_sim_stats(const pq_sim *sim, pq_stats *out);

/* Simulator::amplitude / amplitude_index for n boundaries -- sim.rs:171-182.
 * x, y: n bitstrings each (host memory).  out: 2n doubles.  errbound (optional, n doubles):
 * bound on |out - exact| from the FP32 weight arithmetic (exact-grid hi sums, FP32 lo sums,
 * FP64 reduction). */
PQ_API pq_status pq_amplitudes(pq_sim *sim, int64_t n, const uint64_t *x, const uint64_t *y, double *out,
                               double *errbound);
/* Low-latency single amplitudes (no counterpart in the reference crate).  idle_seconds > 0:
 * one-boundary pq_amplitudes calls are served by a kernel that stays resident on one SM (one
 * block) and takes requests through mapped host memory, so a call costs no launch and finds the
 * kernel's code and the engine's data in that SM's caches; the kernel returns after
 * idle_seconds without a request and is launched again by the next one.  0 turns it off.  Only
 * for simulators whose single amplitude is small (at most 2^14 branches over at most 64 branch
 * engines; else PQ_ERR_UNSUPPORTED).  Results are those of the regular path.  While the kernel
 * is resident, device-wide synchronisation in the process (cudaDeviceSynchronize, cudaFree)
 * waits for it to return. */
PQ_API pq_status pq_sim_set_resident(pq_sim *sim, double idle_seconds);
/* Simulator::probability -- sim.rs:196-198: |amplitude|^2, n doubles. */
PQ_API pq_status pq_probabilities(pq_sim *sim, int64_t n, const uint64_t *x, const uint64_t *y, double *out);
/* Simulator::marginal_probability -- sim.rs:225-231, for one input x and nmeas (qubit, outcome)
 * pairs.  The sandwich engine of each distinct measured-qubit set is built once and cached. */
PQ_API pq_status pq_marginal(pq_sim *sim, const uint64_t *x, int32_t nmeas, const int32_t *qubits,
                             const uint8_t *outcomes, double *out);
/* Simulator::amplitude_estimate -- sim.rs:184-193 / rank.rs:149-171: unbiased Monte-Carlo
 * estimate of <y|C|x> from `samples` draws with the reference's seeding.  One branch engine:
 * points of its branch subspace (engine.rs:616-659; the exact sum when 2^d <= samples; d <= 64);
 * 2^p engines: branch engines drawn uniformly and evaluated exactly.  out: (re, im);
 * stderr (optional): the standard error. */
PQ_API pq_status pq_amplitude_estimate(pq_sim *sim, const uint64_t *x, const uint64_t *y, int64_t samples,
                                       uint64_t seed, double *out, double *stderr_out);
/* approx::estimate_amplitude -- approx.rs:96-135: lazy pair sampling.  Sample i seeds
 * Rng::new(seed ^ i * golden), draws one bit per pair for the first min(pairs, candidates, 62)
 * pair candidates of the circuit's path sum, builds that branch engine (equal patterns share
 * one) and evaluates it exactly when its dimension is <= exact_dim_limit, else with
 * Engine::estimate (2^14 points, the sample's next draw as seed).  out: 2^p * mean (re, im);
 * stderr (optional): 2^p * sqrt(var / samples).  samples <= 2^24, at most 2^14 distinct
 * sampled patterns per call (their engines are held for the call). */
PQ_API pq_status pq_amplitude_estimate_pairs(pq_sim *sim, const uint64_t *x, const uint64_t *y, int32_t pairs,
                                             int64_t samples, uint64_t seed, int32_t exact_dim_limit, double *out,
                                             double *stderr_out);
/* Simulator::sample_many -- sim.rs:253-284: `shots` computational-basis samples of C|x>, drawn
 * by the chain rule over qubit prefixes with the reference's SplitMix64 streams (one seed per
 * shot from seed), so the same seed gives the reference's samples.  out: shots bitstrings.
 * All shots advance together: one launch per qubit over the cached prefix engines. */
PQ_API pq_status pq_sample_many(pq_sim *sim, const uint64_t *x, int64_t shots, uint64_t seed, uint64_t *out);
/* Device-resident variant of pq_amplitudes: x, y, out, errbound are device pointers; the work
 * is ordered after, and waited for by, `stream` (cudaStream_t; NULL = the legacy default
 * stream) without a host synchronisation. */
PQ_API pq_status pq_amplitudes_device(pq_sim *sim, int64_t n, const uint64_t *x, const uint64_t *y, double *out,
                                      double *errbound, void *stream);
/* Device self-check of the last launch of the simulator's size-n plan (pq_amplitudes_device,
 * and every host-buffer call of that size): waits for it, then *failed = 1 if its prepare kernel
 * saw an odd Z8 increment -- impossible for a correct closed form; its results are then NaN --
 * else 0.  The host-buffer calls check this themselves and return PQ_ERR_INTERNAL. */
PQ_API pq_status pq_sim_device_check(pq_sim *sim, int64_t n, int32_t *failed);
/* Same evaluation split into one launch sequence per boundary (the plain one-circuit,
 * one-boundary-per-launch path, kept as the comparison baseline for batching). */
PQ_API pq_status pq_amplitudes_plain(pq_sim *sim, int64_t n, const uint64_t *x, const uint64_t *y, double *out);

/* Allocation-free amplitudes (no counterpart in the reference crate).  For callers that may
 * not allocate device memory when they need results: hosts whose device memory belongs to an
 * outer allocator with a fixed budget (a framework's caching allocator, a server that reserved
 * its memory up front), and plugin or callback code running where an allocation would block,
 * fragment the caller's pool or fail.  x, y (n bitstrings each), out (2n doubles) and errbound
 * (optional, n doubles, NULL = not wanted) are DEVICE pointers owned by the caller; the work is
 * enqueued on `stream` (NULL = legacy default stream) and not waited for.  It runs on the
 * structures uploaded by pq_sim_create and, for all per-call state, one fixed 1.6 MiB static
 * device array: n x (branch engines) <= 4096 and at most 65536 work items, else
 * PQ_ERR_INVALID_ARG.  The results are those of pq_amplitudes_device at the simulator's launch
 * shape (same per-job work decomposition and summation order); a failed device self-check
 * shows as NaN in out and errbound.  The first call on a device looks up that array's address,
 * so make one call before any stream capture.  Calls share the array, which keeps the last
 * call's contents: calls that overlap on the GPU race, serialise them. */
PQ_API pq_status pq_amplitudes_noalloc(pq_sim *sim, int64_t n, const uint64_t *x, const uint64_t *y, double *out,
                                       double *errbound, void *stream);

/* ---- batched multi-circuit launch (one persistent, graph-captured launch) ------------ */
/* Amplitudes of counts[i] boundaries on sims[i], all i, in one CUDA-graph launch of a
 * persistent kernel whose warps pull (circuit, boundary, chunk-range) work items. */
PQ_API pq_status pq_batch_create(int32_t nsims, pq_sim *const *sims, const int64_t *counts, pq_batch **out);
PQ_API void pq_batch_destroy(pq_batch *b);
/* x, y: boundaries of sims[0] then sims[1] ... with words_per_bitstring words each
 * (= ceil(max num_qubits / 64)); out: 2*sum(counts) doubles. */
PQ_API pq_status pq_batch_run(pq_batch *b, const uint64_t *x, const uint64_t *y, double *out, double *errbound);
PQ_API pq_status pq_batch_run_device(pq_batch *b, const uint64_t *x, const uint64_t *y, double *out,
                                     double *errbound, void *stream);
PQ_API int32_t pq_batch_words(const pq_batch *b);
PQ_API int64_t pq_batch_branches(const pq_batch *b);

/* ---- serving loop (continuous batching) --------------------------------------------- */
/* Requests against resident simulators are admitted while device slots and the memory
 * budget allow; admitted requests are launched in waves on a pool of streams, so work of
 * requests that arrive while others run overlaps on the device. */
typedef enum pq_req_kind { PQ_REQ_AMPLITUDE = 0, PQ_REQ_PROBABILITY = 1, PQ_REQ_MARGINAL = 2 } pq_req_kind;
typedef struct pq_request {
    int32_t sim;          /* index into the server's simulator table */
    int32_t kind;         /* pq_req_kind */
    uint64_t x[2];        /* input bitstring (num_qubits <= 128) */
    uint64_t y[2];        /* output bitstring (AMPLITUDE/PROBABILITY) */
    int32_t qubit;        /* measured qubit (MARGINAL) */
    int32_t outcome;      /* measured outcome (MARGINAL) */
    int64_t tag;          /* caller's identifier, returned with the result */
} pq_request;
typedef struct pq_result {
    int64_t tag;
    int32_t status;       /* pq_status of this request */
    int32_t kind;
    double re, im;        /* amplitude, or probability in re */
    double errbound;
    double submit_s, done_s;  /* seconds on the server's monotonic clock */
    int32_t level;        /* evaluation that produced it: 0 the FP32 walk, 1 chunk-sum tables,
                             2 the FP64 walk (probabilities and marginals whose bound could not
                             show 1e-12 absolute are re-evaluated at the next level) */
    int32_t pieces;       /* background pieces the request was evaluated in (0: one wave) */
} pq_result;
/* max_slots: requests per launched wave; mem_budget_bytes: device memory the in-flight waves
 * may hold; max_branch_dim: a request whose work -- branches summed over its branch engines --
 * exceeds 2^max_branch_dim is refused (PQ_ERR_ADMISSION_REFUSED) rather than run. */
PQ_API pq_status pq_server_create(int32_t nsims, pq_sim *const *sims, int32_t max_slots, int64_t mem_budget_bytes,
                                  int32_t max_branch_dim, pq_server **out);
/* Requests whose work is above 2^split_log2 branches (default 28) are not refused but evaluated
 * in the background, in pieces of at most 2^piece_log2 branches (default 32) -- ranges of their
 * branch engines or of one engine's work items -- one piece at a time on half of the SMs, beside
 * the waves of smaller requests; a request's pieces are summed in FP64 and its bounds added.
 * Only requests above 2^max_branch_dim branches are refused. */
PQ_API pq_status pq_server_set_pieces(pq_server *s, int32_t split_log2, int32_t piece_log2);
PQ_API void pq_server_destroy(pq_server *s);
/* Non-blocking: queues n requests; refused requests complete immediately with a status. */
PQ_API pq_status pq_server_submit(pq_server *s, int64_t n, const pq_request *reqs);
/* Collects up to cap finished results; waits up to timeout_s for at least one. */
PQ_API int64_t pq_server_poll(pq_server *s, pq_result *out, int64_t cap, double timeout_s);
PQ_API double pq_server_now(const pq_server *s);
PQ_API pq_status pq_server_drain(pq_server *s, double timeout_s);

/* ---- autotuner (no counterpart in the reference crate, whose enumeration is a CPU loop) -- */
/* Times the evaluation of n representative boundaries (host bitstrings) under candidate launch
 * shapes -- lane chunk length 2^inner_dims (8..10), chunks_per_lane, block_warps, blocks_per_sm --
 * by coordinate descent from the simulator's current tuning (best of `reps` device timings
 * per candidate after a warm-up; reps 0 = 3), and leaves the simulator on the fastest.
 * Amplitudes do not depend on the choice beyond FP64 summation order.  best (optional)
 * receives the tuning, best_ms (optional) its device time. */
PQ_API pq_status pq_sim_autotune(pq_sim *sim, int64_t n, const uint64_t *x, const uint64_t *y, int32_t reps,
                                 pq_tuning *best, double *best_ms);
/* The same search for a batch (pq_batch_run inputs x, y).  A candidate lane chunk length
 * rebuilds the member simulators' weight tables (their own cached launch plans are rebuilt on
 * next use), so do not run the members concurrently with this call.  The batch's later
 * launches use the fastest shape. */
PQ_API pq_status pq_batch_autotune(pq_batch *b, const uint64_t *x, const uint64_t *y, int32_t reps, pq_tuning *best,
                                   double *best_ms);
/* The launch shape the simulator's plans use. */
PQ_API pq_status pq_sim_get_tuning(const pq_sim *sim, pq_tuning *out);

/* ---- measurement -------------------------------------------------------------------- */
/* Device times (ms) of the last completed launch of the simulator's size-n plan (and of a
 * batch): [0] prepare, [1] enumeration, [2] reductions.  Blocks until that launch is done. */
PQ_API pq_status pq_sim_kernel_ms(pq_sim *sim, int64_t n, float *ms);
PQ_API pq_status pq_batch_kernel_ms(pq_batch *b, float *ms);
/* Work of the last launch of the simulator's size-n plan (and of a batch), over the
 * (boundary, branch engine) pairs whose sum did not vanish: out[0] branches enumerated (2^d
 * each), out[1] the reference engine's integer ops for them (5 W_o + 6 W_g 64-bit ops per
 * branch, W_o / W_g = words of odd lines / planes), out[2] the popcounts among them, out[3] the
 * logic ops.  per_boundary (optional, n doubles) splits out[0] by boundary.  Blocks until that
 * launch is done. */
PQ_API pq_status pq_sim_enumerated(pq_sim *sim, int64_t n, double *out, double *per_boundary);
PQ_API pq_status pq_batch_enumerated(pq_batch *b, double *out);
/* Work items of the simulator's size-n plan (-1 if it has no such plan yet). */
PQ_API int64_t pq_sim_launch_items(pq_sim *sim, int64_t n);
/* Issue rates measured on the current device: [0] lop3.b32 ops/s, [1] popc.b32 ops/s,
 * [2] fma.f32 ops/s, [3] SM count. */
PQ_API pq_status pq_measure_peaks(double out[4]);
/* FP32 FMA operations per second issued as paired fma.rn.f32x2 (two per instruction), the form
 * the enumeration's even steps use. */
PQ_API pq_status pq_measure_fma2_rate(double *out);

/* ---- checks (bit-exact comparisons against a CPU restatement) ------------------------ */
/* Canonical dump of branch engine `branch`: normal form, diagonal masks, kernel and
 * boundary columns, RREF; returns the word count (out = NULL to size), < 0 on error. */
PQ_API int64_t pq_debug_engine_dump(const pq_sim *sim, int32_t branch, uint64_t *out, int64_t cap);
/* Shape of branch engine `branch`: out[0] d, [1] pivots, [2] low coordinates of the weight
 * table, [3] joint table (1/0), [4] pair coordinate (-1 none), [5] coordinates touching no
 * pivot, [6] of which high (>= out[2]), [7] terms. */
PQ_API pq_status pq_debug_engine_shape(const pq_sim *sim, int32_t branch, int64_t out[8]);
/* Z8 index of every branch s < 2^d of branch engine `branch` for boundary (x, y), as the
 * enumeration kernel computes it on the device.  Returns d, or -1 (vanishing boundary),
 * or -2 (error). */
PQ_API int32_t pq_debug_branch_phases(pq_sim *sim, int32_t branch, const uint64_t *x, const uint64_t *y,
                                      uint8_t *out);
/* Engine::prepare (src/engine.rs:569-610, Elim::solve_into :188-201) as the device's prepare
 * kernel computes it, for n boundaries x every branch engine (boundary-major), 12 uint64 words
 * per job: [0] 1 if the job vanishes (contradictory boundary, zero engine or inconsistent
 * radical system; the other words are then 0), [1] the constant phase (uint32 ring units),
 * [2] k0 = the Z8 index at the start shift (src/normal_form.rs:479-493), [3] the particular
 * solution's pivot bits y0 (pivots in elimination order), [4..11] the Z4 increments Lp_j of the
 * kernel coordinates j < min(d, 64) as bytes, in the reference's coordinate order. */
PQ_API pq_status pq_debug_prepare(pq_sim *sim, int64_t n, const uint64_t *x, const uint64_t *y, uint64_t *out);
/* Same amplitudes as pq_amplitudes with FP64 branch weights and FP64 accumulation on the
 * device (verification mode). */
PQ_API pq_status pq_amplitudes_fp64(pq_sim *sim, int64_t n, const uint64_t *x, const uint64_t *y, double *out);

#ifdef __cplusplus
}
#endif
#endif
