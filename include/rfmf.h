/*
 * rfmf.h -- C ABI of the GB300-native RFMF annealer (librfmf.so).
 *
 * Drop-in boundary for the reference's annealer path (gt-tinker/rfmf).  The
 * reference's boundary is the C++ function gpu3::annealGpu
 * (src/anneal_gpu.cuh:76-88, defined at src/anneal_kernels.cu:835-884) plus
 * the host helpers of src/host_common.h; every entry point below names the
 * reference interface it replaces.  include/rfmf_annealgpu.hpp re-exposes
 * gpu3::annealGpu with the reference's exact C++ signature on top of this ABI.
 *
 * Conventions: plain pointers and sizes, caller-owned buffers, no CUDA or
 * torch types.  Every function returns an rfmf_status (never exits or
 * throws); rfmf_last_error() gives the message of the calling thread's last
 * failure.  A context owns one device and one CUDA stream; calls on one
 * context are not thread-safe, separate contexts are independent.
 *
 * Spins are int8 +1/-1, one per vertex, chain-major (chain c's vertex v at
 * c*n + v).  Vertex ids are the dense ids of the reference's AnnealCsr.
 */
#ifndef RFMF_H
#define RFMF_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum rfmf_status {
    RFMF_OK = 0,
    RFMF_ERR_INVALID = 1,    /* bad argument or malformed graph */
    RFMF_ERR_CUDA = 2,       /* a CUDA runtime call failed */
    RFMF_ERR_NOMEM = 3,      /* device or host allocation failed */
    RFMF_ERR_CAPACITY = 4,   /* request exceeds a documented limit */
    RFMF_ERR_DEVICE = 5,     /* the kernel reported an inconsistency */
    RFMF_ERR_BETA_RUNS = 6   /* beta run tables would exceed the run cap */
} rfmf_status;

typedef struct rfmf_context rfmf_context;
typedef struct rfmf_graph rfmf_graph;
typedef struct rfmf_batch rfmf_batch;

/* Library version string. */
const char* rfmf_version(void);

/* Message of the calling thread's last failing call ("" if none). */
const char* rfmf_last_error(void);

/* Open a context on CUDA device `device`: replaces the cudaSetDevice and the
 * default-stream use of src/anneal_kernels.cu:874. */
int rfmf_context_create(int device, rfmf_context** out);
/* Release the caller's handle.  Graphs, batches and servers made on the
 * context hold it too: its streams and tables go when the last of them is
 * destroyed, so the order of the destroy calls does not matter.  The handle
 * itself must not be used after this call. */
int rfmf_context_destroy(rfmf_context* ctx);

/* Device properties the autotuner uses (SM count, opt-in shared memory per
 * block).  Either pointer may be NULL. */
int rfmf_context_info(const rfmf_context* ctx, int* sm_count, int* smem_optin);

/* The context's CUDA stream (a cudaStream_t) in *stream: every launch and
 * copy of the context's batches goes to it, so a caller can order its own
 * work against them or time them with its own events.  No reference
 * counterpart (the reference uses the default stream). */
int rfmf_context_stream(const rfmf_context* ctx, void** stream);

/* The context's device-resident beta run tables (one per (t0, sweeps) in
 * use, shared by every batch, rfmf_anneal call and served request of the
 * context; the reference builds and uploads a set per launch,
 * src/host_common.cpp:277-294): *tables live now, *device_bytes they hold,
 * *uploads performed since the context was created.  Any pointer may be
 * NULL. */
int rfmf_context_beta_cache(rfmf_context* ctx, int64_t* tables, int64_t* device_bytes,
                            uint64_t* uploads);

/*
 * Upload a CSR graph: n vertices, offsets[n+1], col/weight[offsets[n]].
 * Replaces the CSR flatten + upload of src/anneal_kernels.cu:666-741 (the
 * DevCsr of src/anneal_gpu.cuh:23-28) for the AnnealCsr layout of
 * src/immutable_graph.hpp:36-38.  The CSR must be symmetric (each undirected
 * edge twice, equal weights), without self loops, rows strictly ascending.
 * Limits: n < 2^31, offsets[n] < 2^32.
 */
int rfmf_graph_create(rfmf_context* ctx, int64_t n, const uint32_t* offsets,
                      const int32_t* col, const int32_t* weight, rfmf_graph** out);

/* Host-only check of the invariants rfmf_graph_create requires (no device
 * work); on success *max_weighted_degree (may be NULL) receives B. */
int rfmf_csr_validate(int64_t n, const uint32_t* offsets, const int32_t* col,
                      const int32_t* weight, int64_t* max_weighted_degree);
/* Release the caller's handle.  Batches and server requests on the graph
 * hold it until they are destroyed or released; the handle itself must not
 * be used after this call. */
int rfmf_graph_destroy(rfmf_graph* g);

/* n, m (undirected edges) and B = max weighted degree; any pointer may be NULL.
 * B replaces maxWeightedDegree (src/host_common.cpp:314-325). */
int rfmf_graph_info(const rfmf_graph* g, int64_t* n, int64_t* m,
                    int64_t* max_weighted_degree);

/* ---- host helpers of src/host_common.{h,cpp}, src/max_cut.cpp, src/rng.hpp */

/* annealTotalSteps (src/host_common.cpp:196-210): sum of iters, capped at
 * 10^12; returns -1 past the cap. */
int64_t rfmf_total_steps(int64_t nphases, const uint64_t* iters);

/* betaFixedForStep (src/host_common.h:73-76). */
int32_t rfmf_beta_fixed(uint64_t step, double t0);

/* annealScoreSafeInt32 (src/host_common.cpp:296-312): 1 if int32 scores are
 * exact for every sweep of a run of total_steps at temperature t0. */
int rfmf_score_safe_int32(int64_t total_steps, double t0, int64_t delta_bound);

/* maxWeightedDegree (src/host_common.cpp:314-325) on a host CSR. */
int64_t rfmf_max_weighted_degree(int64_t n, const uint32_t* offsets,
                                 const int32_t* weight);

/* cutValueCsr (src/max_cut.cpp:5-15) on a host CSR. */
int64_t rfmf_cut_value(int64_t n, const uint32_t* offsets, const int32_t* col,
                       const int32_t* weight, const int8_t* spin);

/* Initial spins of a chain from its RAW seed: xoshiro256++ seeded by
 * splitmix64, one bit per vertex (src/rng.hpp, src/host_common.cpp:40-45). */
void rfmf_initial_spins(uint64_t seed, int64_t n, int8_t* out);

/*
 * buildBetaRunTables (src/host_common.cpp:212-294): run-length beta tables,
 * one per distinct t0 (exact double equality), runs as (0-based exclusive end
 * step, beta_fixed).  Writes at most `cap` runs, the run count to *runs and
 * each chain's first-run index to chain_off[C].  RFMF_ERR_BETA_RUNS past
 * 33,000,000 runs (kMaxBetaRuns, src/host_common.h:96-99).
 */
int rfmf_beta_tables(const double* t0s, int64_t C, int64_t total_steps,
                     int64_t* run_end, int32_t* run_val, int64_t* chain_off,
                     int64_t cap, int64_t* runs);

/* ---- graph ingest -------------------------------------------------------- */

/* Header "N M" of Gset/MQLib text (first line that is neither blank nor a
 * '#' comment; src/read_gset.cpp:61-75). */
int rfmf_gset_header(const char* text, size_t len, int64_t* n, int64_t* m);

/*
 * parseAndScale (src/read_gset.cpp:61-170) on Gset/MQLib text: the M edge
 * lines "u v w" in file order into u/v/w (cap >= M entries each); when a
 * weight is fractional the whole instance is scaled by the largest power of
 * ten (10^-12 .. 10^12) that keeps B and every weight inside the reference's
 * budgets (forced_scale > 0 overrides), weights are rounded and zeros
 * dropped.  *nedges = surviving edges, *scale_out the scale, *zero_dropped
 * the dropped count (both may be NULL).  Not deduplicated.
 */
int rfmf_gset_parse(const char* text, size_t len, double forced_scale, int64_t cap,
                    int64_t* u, int64_t* v, int64_t* w, int64_t* nedges, double* scale_out,
                    int64_t* zero_dropped);

/*
 * Graph::addEdge + ImmutableGraph(Graph) (src/graph.cpp, src/immutable_graph.hpp
 * :44-120) built on the device from an edge list: zero weights are dropped,
 * an undirected edge seen twice keeps its first weight, the vertices are the
 * endpoints renumbered densely in ascending original id, each row sorted
 * ascending.  Ids must lie in [0, 2^28); self loops are refused (the
 * reference would store them; Gset has none).  *n_out = vertex count (may be
 * NULL).  The graph is then used exactly like one from rfmf_graph_create.
 */
int rfmf_graph_from_edges(rfmf_context* ctx, int64_t nedges, const int64_t* u, const int64_t* v,
                          const int64_t* w, rfmf_graph** out, int64_t* n_out);

/* Original vertex id of every dense id (graphs from rfmf_graph_from_edges). */
int rfmf_graph_orig_ids(const rfmf_graph* g, int64_t* out);

/* The graph's CSR copied to the host: offsets[n+1], col/weight[2m] (any may
 * be NULL). */
int rfmf_graph_csr(const rfmf_graph* g, uint32_t* offsets, int32_t* col, int32_t* weight);

/* ---- the annealer ------------------------------------------------------ */

/* Mirrors gpu3::LaunchConfig (src/anneal_gpu.cuh:52-58) plus the knobs the
 * reference fixed in src/tuning.hpp; every knob is output-invariant.
 * Zero-initialise for defaults (autotuned). */
typedef struct rfmf_launch_config {
    int corr;              /* CorrMode; accepted, no effect (FLIP needs no corr walk) */
    int device;            /* informational; the context's device is used */
    int s_width;           /* 32 or 64; accepted (the per-vertex gain width is gain_width) */
    int threads_per_chain; /* 0 = auto, else 32, 64, 128 or 256 (one chain's warp group) */
    int score_path;        /* 0 = gate (src/host_common.cpp:296-312), 1 = int32, 2 = int64 */
    int chains_per_cta;    /* 0 = auto, else chains sharing one CTA's copy of the graph */
    int csr_format;        /* 0 = auto, 1 = unit16 (shared), 2 = packed32 (shared),
                              3 = HBM (the graph's most compact entries: 2, 4 or 8 bytes),
                              4 = HBM with 8-byte {col, weight} entries */
    int gain_width;        /* 0 = auto, 1 = int8 (needs B <= 127), 4 = int32 */
} rfmf_launch_config;

/*
 * gpu3::annealGpu (src/anneal_gpu.cuh:76-88): run C independent chains over
 * one graph, chain c with (initial_spins[c], t0s[c], solver_seeds[c]) and the
 * shared schedule (phases, iters).  Synchronous; host buffers in and out:
 * end_spins/best_spins C*n int8, kernel_best_vals/kernel_final_vals C int64
 * (may be NULL), *kernel_ms the device time of the annealing launch(es).
 * n == 0 or nphases == 0 returns the inputs with cutValueCsr-seeded values
 * (src/anneal_kernels.cu:856-868).  solver_seeds[c] is the raw seed plus
 * 0xC2B2AE3D27D4EB4F, as main.cu:27-29 computes it.
 */
int rfmf_anneal(rfmf_context* ctx, const rfmf_graph* g, int64_t max_weighted_deg,
                int64_t C, const int8_t* initial_spins, const double* t0s,
                int64_t nphases, const uint64_t* phases, const uint64_t* iters,
                const uint64_t* solver_seeds, const rfmf_launch_config* cfg,
                int8_t* end_spins, int8_t* best_spins, float* kernel_ms,
                int64_t* kernel_best_vals, int64_t* kernel_final_vals);

/*
 * Batched, device-resident form (no reference counterpart: the reference
 * runs one graph per launch and keeps nothing between calls).  A batch holds
 * chains over any number of graphs, each with its own t0 and seed, all on one
 * schedule.  Chain state (spins, best spins, cut values, progress) stays in
 * device memory between rfmf_batch_run calls; each run advances every
 * unfinished chain by up to `sweeps` sweeps in ONE persistent launch, and a
 * sequence of runs equals one uninterrupted anneal bit for bit.
 *
 * graphs[c], t0s[c], solver_seeds[c]: per chain.  initial_spins: the chains'
 * spins concatenated in chain order (n of chain c's graph each).
 */
int rfmf_batch_create(rfmf_context* ctx, int64_t nchains, const rfmf_graph* const* graphs,
                      const double* t0s, const uint64_t* solver_seeds,
                      const int8_t* initial_spins, int64_t nphases,
                      const uint64_t* phases, const uint64_t* iters,
                      const rfmf_launch_config* cfg, rfmf_batch** out);

/* Enqueue one launch advancing every unfinished chain by up to `sweeps`
 * sweeps, on the context stream; returns without waiting.  Work items are
 * re-sized between launches from the per-graph costs the library learns
 * from earlier launches' timings (output-invariant). */
int rfmf_batch_run(rfmf_batch* b, uint64_t sweeps);

/* Capture `launches` rfmf_batch_run(b, sweeps) steps in a CUDA graph and
 * replay it `replays` times (fixed-size sweep batches without per-launch
 * host work).  Asynchronous like rfmf_batch_run. */
int rfmf_batch_run_graph(rfmf_batch* b, uint64_t sweeps, int launches, int replays);

/* rfmf_batch_run, then wait; *ms receives the device time of the launch
 * (CUDA events on the context stream). */
int rfmf_batch_run_timed(rfmf_batch* b, uint64_t sweeps, float* ms);

/* Per chain: number of sweeps so far that raised its best cut (the sweeps on
 * which the best-spin snapshot was taken).  Synchronous. */
int rfmf_batch_stats(rfmf_batch* b, uint64_t* improved_sweeps);

/* Wait for the batch's work; reports a device-side error if one occurred. */
int rfmf_batch_synchronize(rfmf_batch* b);

/* Copy chain state to the host (synchronous).  Any pointer may be NULL.
 * end_spins/best_spins: concatenated like initial_spins. */
int rfmf_batch_read(rfmf_batch* b, int8_t* end_spins, int8_t* best_spins,
                    int64_t* cur_vals, int64_t* best_vals, uint64_t* sweeps_done);

/*
 * Resume from saved state (no reference counterpart: a chain is a pure
 * function of its graph, seed, t0, schedule and sweep index,
 * src/anneal_gpu.cuh:4-8, so what rfmf_batch_read returns is a checkpoint).
 * Creates a batch like rfmf_batch_create whose chain c starts from
 * end_spins / best_spins (concatenated like initial_spins), cur_vals[c] /
 * best_vals[c] (their cut values) and sweeps_done[c] <= the schedule's total;
 * running it to the end of the schedule gives exactly the results of one
 * uninterrupted run.  The cut values are recomputed from the spins on the
 * device and a checkpoint whose values disagree is refused
 * (RFMF_ERR_INVALID).  The improved-sweeps statistic restarts at 0.
 */
int rfmf_batch_restore(rfmf_context* ctx, int64_t nchains, const rfmf_graph* const* graphs,
                       const double* t0s, const uint64_t* solver_seeds, int64_t nphases,
                       const uint64_t* phases, const uint64_t* iters,
                       const rfmf_launch_config* cfg, const int8_t* end_spins,
                       const int8_t* best_spins, const int64_t* cur_vals,
                       const int64_t* best_vals, const uint64_t* sweeps_done, rfmf_batch** out);

/*
 * Measured launch planning (in place of the reference's fixed V100 table,
 * src/tuning.hpp:10-17, applied at src/anneal_kernels.cu:641-662).  Times
 * candidate plans on short trial batches of these very chains (their graphs,
 * seeds, t0s and initial spins; the schedule compressed to trial_sweeps
 * sweeps with every phase keeping its share, 0 = 2048) and writes the fastest
 * to *best, starting from *base (NULL: all automatic).  Candidates: warps per
 * chain from the planner's rule or fixed at 1, 2 or 4, each with the rule's
 * CSR residency or with HBM walks.  Each candidate runs twice and keeps its
 * faster time.  Results never depend on the plan.  The choice is cached in
 * the context under the batch's shape (graph sizes, chains per graph,
 * schedule), so later calls for the same shape return at once.  If cand_us
 * is not NULL it receives each candidate's microseconds per chain-sweep (at
 * most *ncand entries; *ncand is set to the candidate count, and a candidate
 * that cannot be planned gets a negative time), and cand (may be NULL) the
 * candidates' configs.
 */
int rfmf_autotune(rfmf_context* ctx, int64_t nchains, const rfmf_graph* const* graphs,
                  const double* t0s, const uint64_t* solver_seeds, const int8_t* initial_spins,
                  int64_t nphases, const uint64_t* phases, const uint64_t* iters,
                  uint64_t trial_sweeps, const rfmf_launch_config* base,
                  rfmf_launch_config* best, int* ncand, rfmf_launch_config* cand,
                  float* cand_us);

/* The launch plan the autotuner chose for a batch. */
typedef struct rfmf_batch_plan {
    int64_t nchains;
    uint64_t total_sweeps;     /* sum of iters over phases with P != 0 */
    int threads_per_chain;
    int chains_per_cta;
    int grid;                  /* persistent CTAs per launch */
    int items;                 /* work items (chain groups) per launch */
    int score64;               /* 1 if the int64 score path is used */
    int csr_format;            /* 1 unit16, 2 packed32 (shared memory); HBM walks of
                                  3 8-byte, 4 16-bit, 5 32-bit entries */
    int gain_width;            /* bytes per vertex gain: 1 or 4 */
    int smem_bytes;            /* dynamic shared memory per CTA */
    int balanced;              /* 1 once every multi-graph launch class sizes its work items per graph (from learned costs, else a shape model) */
    int launch_classes;        /* launches per window (graphs grouped by kernel variant and size) */
    int64_t launches;          /* kernel launches enqueued so far (a window of a multi-graph class
                                  is cut at phase boundaries; graph replays count theirs) */
} rfmf_batch_plan;

int rfmf_batch_info(const rfmf_batch* b, rfmf_batch_plan* out);

int rfmf_batch_destroy(rfmf_batch* b);

/* Output path on the device.  cutValueCsr (src/max_cut.cpp:5-15) of every
 * chain's end spins (which = 0) or best spins (which = 1), recomputed from
 * the spins in int64. */
int rfmf_batch_cuts(rfmf_batch* b, int which, int64_t* out_cuts);

/* Partition strings, the payload of the Solution-*-partition: lines
 * (src/host_common.cpp:412-422): chain c's n characters '0' (spin -1) /
 * '1' (spin +1) at out + c * stride (stride >= the largest n; the bytes
 * past a chain's n are 0). */
int rfmf_batch_partitions(rfmf_batch* b, int which, char* out, int64_t stride);

/* ---- request server ------------------------------------------------------
 * Serving form of annealGpu (the reference serves one annealGpu call per
 * process; proposed in its place: rfmf_submit / rfmf_poll).  A server owns a
 * worker thread and a stream on the context's device.  Each submitted
 * request is one annealGpu call's worth of chains (one graph, one schedule,
 * per-chain t0 and seed).  The worker advances every admitted request's
 * chains together, `window_sweeps` sweeps per persistent launch (continuous
 * batching); requests join at the next window boundary and leave when their
 * chains finish.  Results are bit-identical to rfmf_anneal on the same
 * inputs.  All calls are thread-safe.  A graph must outlive the requests
 * that use it. */
typedef struct rfmf_server rfmf_server;

typedef struct rfmf_server_config {
    uint64_t window_sweeps;      /* sweeps per launch window (0 = 4096) */
    int64_t max_chains;          /* chains admitted at once (0 = 1 << 20); later requests queue */
    rfmf_launch_config launch;   /* threads_per_chain / gain_width / csr_format / score_path */
    int64_t max_device_bytes;    /* device bytes of the admitted requests' own state at once
                                    (0 = no limit); later requests queue, and a request that
                                    alone exceeds it is refused (RFMF_ERR_CAPACITY) */
} rfmf_server_config;

enum rfmf_request_state {
    RFMF_REQ_QUEUED = 0,
    RFMF_REQ_RUNNING = 1,
    RFMF_REQ_DONE = 2,
    RFMF_REQ_FAILED = 3,
    RFMF_REQ_CANCELLED = 4
};

typedef struct rfmf_request_status {
    int state;                   /* rfmf_request_state */
    int error;                   /* rfmf_status of a failed request */
    uint64_t sweeps_done;        /* sweeps every chain of the request has completed */
    uint64_t sweeps_total;
    double submit_s;             /* server clock (seconds since create) */
    double start_s;              /* admitted to the GPU (0 while queued) */
    double finish_s;             /* results on the host (0 until done) */
} rfmf_request_status;

typedef struct rfmf_server_stats {
    uint64_t windows;            /* launch windows run */
    uint64_t launches;           /* kernel launches (one per launch class per window) */
    uint64_t chain_sweeps;       /* chain-sweeps completed */
    double busy_s;               /* wall time inside windows (admission + launches + harvest) */
    double kernel_s;             /* device time of the launches (CUDA events) */
    int64_t queued, running, done;   /* requests by state */
} rfmf_server_stats;

int rfmf_server_create(rfmf_context* ctx, const rfmf_server_config* cfg, rfmf_server** out);

/* Stops the worker after the window in flight; unread results are dropped. */
int rfmf_server_destroy(rfmf_server* s);

/* Copies the inputs (laid out as for rfmf_anneal) and queues the request. */
int rfmf_submit(rfmf_server* s, const rfmf_graph* g, int64_t nchains, const int8_t* initial_spins,
                const double* t0s, int64_t nphases, const uint64_t* phases, const uint64_t* iters,
                const uint64_t* solver_seeds, uint64_t* request_id);

int rfmf_poll(rfmf_server* s, uint64_t request_id, rfmf_request_status* status);

/* Blocks until the request is done or failed, or timeout_s passes
 * (timeout_s < 0: no limit); RFMF_ERR_CAPACITY on timeout. */
int rfmf_wait(rfmf_server* s, uint64_t request_id, double timeout_s, rfmf_request_status* status);

/* Results of a done request (layouts as rfmf_anneal; any pointer may be
 * NULL); releases the request.  A failed request returns its error. */
int rfmf_result(rfmf_server* s, uint64_t request_id, int8_t* end_spins, int8_t* best_spins,
                int64_t* best_vals, int64_t* final_vals);

int rfmf_server_stats_get(rfmf_server* s, rfmf_server_stats* out);

/* Cancel a request (no reference counterpart: the reference runs one solve
 * per process and stops only by exiting).  A queued request is cancelled at
 * once; a running one leaves at the next window boundary, its device state
 * and chain slots freed for the requests behind it (the others' results are
 * unaffected).  Its state becomes RFMF_REQ_CANCELLED; rfmf_wait returns for
 * it and rfmf_result releases it with RFMF_ERR_INVALID.  Cancelling a request
 * that has already finished changes nothing. */
int rfmf_cancel(rfmf_server* s, uint64_t request_id);

/*
 * The annealer for callers that cannot allocate device memory.  No reference
 * counterpart: an addition for hosts whose allocator owns all device memory,
 * code that must not allocate in the middle of its work, and embedders that
 * hand the library pre-sized buffers.  It allocates nothing: inputs and
 * outputs are the caller's device buffers, and the kernel's scratch (graph,
 * schedule and chain records, work items, queue head, error word) lives in a
 * fixed 476,672-byte (about 466 KiB) file-scope device array that every GPU
 * loading this library holds until the process exits.
 *
 * Limits: C <= 4096 chains, nphases <= 64 (RFMF_ERR_CAPACITY beyond).
 * Inputs (device): d_offsets[n+1] (uint32, 4-byte aligned), d_edges[2 *
 * offsets[n]] as {int32 col, int32 weight} pairs (8-byte aligned; the
 * symmetric, row-sorted CSR that rfmf_csr_validate accepts), d_beta_end /
 * d_beta_val (8- / 4-byte aligned: the beta_runs runs of rfmf_beta_tables
 * for these t0s over the executed sweeps), d_spin_bits (4-byte aligned,
 * C * ceil(n/32) words, bit v of chain c = spin +1; overwritten with the final
 * spins).  Host: t0s, solver_seeds, phases, iters, chain_beta_off (first run
 * of each chain's table), chain_beta_runs (its run count; off + runs <=
 * beta_runs), and max_weighted_deg = a bound on every row's sum of |w|.
 * Outputs (device): d_best_bits (same layout), d_cur / d_best (C int64 each,
 * 8-byte aligned).  The CSR is checked on the device before the anneal; one
 * that breaks the invariants or the bound gives RFMF_ERR_INVALID without
 * annealing (outputs then unspecified).  Misaligned pointers give
 * RFMF_ERR_INVALID before any device work.  Synchronous on `stream` (a
 * cudaStream_t, NULL for the legacy default stream): it returns once the
 * anneal has finished.  The first call on a device looks up the array's
 * address; the array is shared by all calls, which clear what they need,
 * and calls that overlap on the GPU race on it.
 */
int rfmf_anneal_noalloc(int device, void* stream, int64_t n, const uint32_t* d_offsets,
                        const int32_t* d_edges, int64_t max_weighted_deg, int64_t C,
                        const double* t0s, const uint64_t* solver_seeds, int64_t nphases,
                        const uint64_t* phases, const uint64_t* iters, const int64_t* d_beta_end,
                        const int32_t* d_beta_val, int64_t beta_runs,
                        const int64_t* chain_beta_off, const int64_t* chain_beta_runs,
                        uint32_t* d_spin_bits, uint32_t* d_best_bits, int64_t* d_cur,
                        int64_t* d_best);

#ifdef __cplusplus
}
#endif

#endif /* RFMF_H */
