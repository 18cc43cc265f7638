/* pdpd_gpu.h -- C ABI of the GB300 DPD engine.
 *
 * This is the boundary between the reference's engine plug-in API and the GPU runtime.
 * The reference's plug-in interface is the C++ class DPDEngine
 * (include/dpd/core/dpd_engine.hpp:10-216 in the reference); the adapter
 * poets-dpd_gb300/host/gb300_dpd_engine.hpp subclasses it and forwards every call here.
 * Each entry point below names the DPDEngine member it serves.
 *
 * Conventions: every call returns PDPD_OK (0) or a positive PDPD_E_* status; no exception
 * or C++ type crosses this boundary.  After a failure, pdpd_last_error() returns a
 * human-readable message.  All pointers are host pointers; arrays are indexed by bead id
 * (the bead's index in WorldState::beads).  Functions are not thread-safe per engine: one
 * caller thread per engine, as in the reference (the interval callback runs on that thread).
 */
#ifndef PDPD_GPU_H
#define PDPD_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PDPD_ABI_VERSION 1

enum pdpd_status {
    PDPD_OK = 0,
    PDPD_E_INVALID = 1,      /* bad argument, or a world that fails validation */
    PDPD_E_UNSUPPORTED = 2,  /* the world uses a feature this engine does not support */
    PDPD_E_CUDA = 3,         /* CUDA runtime error (message has the CUDA error string) */
    PDPD_E_STATE = 4,        /* call out of order, e.g. Run before Attach */
    PDPD_E_BOND_SNAPPED = 5, /* a Hookean bond grew beyond the maximum bond length */
    PDPD_E_BEAD_LOST = 6,    /* a bead position or velocity became non-finite */
    PDPD_E_NOMEM = 7         /* device memory exhausted, or a fixed budget exceeded */
};

enum pdpd_precision {
    PDPD_FP32 = 0, /* FP32 forces; positions as integer cell + FP32 offset */
    PDPD_FP64 = 1  /* FP64 everywhere, same operation order as the reference's FP64 engines */
};

/* A world in flat form: the fields of the reference's WorldState
 * (include/dpd/core/dpd_state.hpp:245-264) that the integrator reads, with the polymer
 * templates expanded into per-bond lists.  x/v/f point at the first bead's vector; bead i's
 * vector starts bead_stride_bytes * i bytes later (0 means packed, 24 bytes), so the adapter
 * can pass &state.beads[0].x[0] with stride sizeof(Bead) and no copy. */
typedef struct pdpd_world {
    int32_t box[3];                /* integer box sides (WorldState::box) */
    double dt;                     /* WorldState::dt */
    double lambda;                 /* WorldState::lambda (the half-step integrator uses 0.5) */
    uint64_t seed;                 /* WorldState::seed */
    int64_t t;                     /* WorldState::t */
    uint32_t n_bead_types;
    const double *conservative;    /* n_bead_types^2 row-major, a_ij */
    const double *dissipative;     /* n_bead_types^2 row-major, gamma_ij */
    const uint8_t *stationary;     /* n_bead_types flags, may be NULL */
    uint32_t n_beads;
    const uint32_t *hash;          /* BeadHash::hash of each bead (dpd_state.hpp:52-60) */
    const double *x, *v, *f;       /* bead vectors, see bead_stride_bytes */
    size_t bead_stride_bytes;
    uint32_t n_bonds;              /* Hookean bonds, polymer-major, polymer-type order */
    const uint32_t *bond_beads;    /* 2*n_bonds: head, tail bead ids */
    const double *bond_kappa, *bond_r0;
    uint32_t n_angles;             /* angle bonds (BondPair), polymer-major */
    const uint32_t *angle_beads;   /* 3*n_angles: head, middle, tail bead ids */
    const double *angle_kappa, *angle_theta0;
    /* Spatially varying DPD parameters (InteractionStrength Parameters that are expressions of
     * x, y, z, ux, uy, uz; dpd_engine.hpp:59-82): per cell, x-major with z fastest, the
     * n_bead_types^2 values of a_ij and of gamma_ij as the reference evaluates them per cell
     * (naive_dpd_engine_half_merge.hpp:221-236).  A pair then uses the mean of the two beads'
     * cell values of a_ij and of sqrt(gamma_ij) (:570-583).  NULL (both): the matrices above
     * apply everywhere.  The FP32 engine runs such worlds with force_kernel 1. */
    const double *cell_conservative, *cell_dissipative;
} pdpd_world;

/* Phase timings, same meaning as DPDEngine::timings_t (dpd_engine.hpp:38-46); -1 = unset. */
typedef struct pdpd_timings {
    double compile, aquire, configure, execute_to_first_bead, execute_to_last_bead,
        perf_counters;
} pdpd_timings;

typedef struct pdpd_engine pdpd_engine;

/* Interval callback for pdpd_run_intervals: called on the caller's thread after the
 * interval's state has been written to the host arrays.  Return nonzero to continue.  The
 * state is a snapshot for reading: the next interval is already running on the device from
 * the state as reported, so edits to the host arrays do not reach the engine (and are
 * overwritten by the next interval's write).  A caller that changes beads between intervals
 * stops (returns 0), edits, re-attaches and runs again. */
typedef int (*pdpd_interval_fn)(void *user, int64_t t);

/* Create/destroy an engine (DPDEngineFactory::create, dpd_engine.hpp:244-252).
 * device < 0 uses the current CUDA device. */
int pdpd_create(int precision, int device, pdpd_engine **out);
void pdpd_destroy(pdpd_engine *e);

/* Message for the last failed call on e (or on a NULL engine: the last failed create or
 * can_support on this thread).  Never NULL. */
const char *pdpd_last_error(const pdpd_engine *e);

/* DPDEngine::CanSupport (dpd_engine.hpp:57-128): PDPD_OK, or PDPD_E_UNSUPPORTED /
 * PDPD_E_INVALID with the reason in reason[0..reason_len).  Host-only, touches no GPU. */
int pdpd_can_support(const pdpd_world *w, char *reason, size_t reason_len);

/* DPDEngine::GetMaxBondLength (dpd_engine.hpp:130): the length beyond which a Hookean bond
 * counts as snapped (2.0, as naive_dpd_engine_half_step.hpp:96). */
double pdpd_max_bond_length(void);

/* DPDEngine::Attach (dpd_engine.hpp:177): copy the world to the device and build its cell
 * list.  w == NULL detaches.  The host arrays are not retained.  With config host_direct (the
 * default) on a device that reaches pageable host memory through the host's page tables, a
 * GPU kernel reads x, v, f and hash from the caller's arrays directly (vectors 8-byte aligned
 * at a stride that is a multiple of 8, hashes 4-byte aligned; else, or on other devices,
 * through pinned staging): they must be ordinary host memory, readable until the call
 * returns. */
int pdpd_attach(pdpd_engine *e, const pdpd_world *w);

/* Batched attach: n independent worlds share one device arena and are stepped together;
 * each keeps its own box, parameters, seed and t.  Bead ids are per world. */
int pdpd_attach_batch(pdpd_engine *e, const pdpd_world *worlds, uint32_t n_worlds);

/* DPDEngine::Run(nSteps) (dpd_engine.hpp:185): advance every attached world by n_steps.
 * Blocks until the device has finished and reports device-side errors. */
int pdpd_run(pdpd_engine *e, uint32_t n_steps);

/* Enqueue n_steps on the engine's stream and return at once (no error check). */
int pdpd_run_async(pdpd_engine *e, uint32_t n_steps);

/* Wait for queued work and report device-side errors. */
int pdpd_sync(pdpd_engine *e);

/* The engine's CUDA stream (a cudaStream_t), for timing with events. */
void *pdpd_stream(pdpd_engine *e);

/* Copy world `world`'s state x(t), v(t), f(t) and t to host arrays (bead-id order, vector
 * layout as in pdpd_world; any pointer may be NULL).  With host_direct (see pdpd_attach) a GPU
 * kernel writes the arrays directly; nothing outside the vectors is written either way, and
 * nothing at all when a world has failed. */
int pdpd_read_state(pdpd_engine *e, uint32_t world, double *x, double *v, double *f,
                    size_t bead_stride_bytes, int64_t *t);

/* Every world of an attached batch at once (after Run(nSteps) of a batch, DPDEngine::Run's
 * write-back of dpd_engine.hpp:179-184 for each state): one gather kernel writing every
 * world's arrays (host_direct), or one device unsort, one copy and a parallel host scatter,
 * instead of one round trip per world.  out[i] receives world i's state as pdpd_read_state
 * would (any of its pointers may be NULL). */
typedef struct pdpd_state_view {
    double *x, *v, *f;
    int64_t *t;
} pdpd_state_view;
int pdpd_read_states(pdpd_engine *e, uint32_t n_worlds, const pdpd_state_view *out,
                     size_t bead_stride_bytes);

/* DPDEngine::Run(interval_count, interval_size, callback) (dpd_engine.hpp:195-215) for a
 * single attached world: after each interval the state is written to x/v/f (layout as in
 * pdpd_world) and cb is called; the next interval already runs on the device meanwhile.
 * interval_count < 0 runs until cb returns 0.  *steps_done receives the steps completed;
 * on an early stop the device state is rolled back to the last reported interval. */
int pdpd_run_intervals(pdpd_engine *e, int32_t interval_count, uint32_t interval_size,
                       double *x, double *v, double *f, size_t bead_stride_bytes,
                       pdpd_interval_fn cb, void *user, uint32_t *steps_done);

/* DPDEngine::GetTimings (dpd_engine.hpp:145-148). */
int pdpd_get_timings(pdpd_engine *e, pdpd_timings *out);

/* DPDEngine::GetConfigEntries / SetConfigEntry (dpd_engine.hpp:150-169).  Entry i's name,
 * description and value are copied into the buffers; returns PDPD_E_INVALID past the end. */
int pdpd_get_config(pdpd_engine *e, uint32_t index, char *name, size_t name_len, char *desc,
                    size_t desc_len, char *value, size_t value_len);
int pdpd_set_config(pdpd_engine *e, const char *key, const char *value);

/* Per-phase device time of a run, in milliseconds, measured with CUDA events on the
 * engine's stream around each kernel group.  `force` covers the force kernels (pair + bond
 * forces, velocity update, next position update and cell count), `sort` the counting sort
 * (scan, place, canon), `other` the first position update and the final copy. */
typedef struct pdpd_phase_times {
    double force_ms;
    double sort_ms;
    double other_ms;
    uint32_t force_launches;
    uint32_t sort_launches;
} pdpd_phase_times;

/* Run n_steps like pdpd_run, but launch kernels one by one (no graph) with CUDA events
 * between phases, and report the per-phase device times.  The trajectory is identical to
 * pdpd_run's. */
int pdpd_profile_run(pdpd_engine *e, uint32_t n_steps, pdpd_phase_times *out);

/* Observables of attached world `world` at its current time, reduced on the GPU in FP64
 * (no counterpart in the reference, which has no observables of its own; used to compare
 * long runs with an FP64 oracle statistically):
 *   ke2       sum of |v|^2 over beads (kinetic temperature kT = ke2 / (3 N), unit mass)
 *   momentum  total momentum
 *   virial    sum over bead pairs with r < 1 of r a_ij (1 - r) (conservative pair virial)
 *             + sum over Hookean bonds of r kappa (r0 - r); pressure = (ke2 + virial) / (3 V)
 * and, when the arrays are given, rdf[(ti * n_types + tj) * n_bins + b] (ti <= tj) = number
 * of pairs of bead types ti, tj with r in [b, b+1) / n_bins, and bond_hist[b] = number of
 * Hookean bonds with length in [2b, 2(b+1)) / n_bond_bins.  Deterministic. */
typedef struct pdpd_observables {
    double ke2;
    double momentum[3];
    double virial;
} pdpd_observables;
int pdpd_observe(pdpd_engine *e, uint32_t world, pdpd_observables *out, uint32_t n_bins,
                 uint64_t *rdf, uint32_t n_bond_bins, uint64_t *bond_hist);

/* Evaluate the engine's device RNG on n host-supplied records: for each i,
 * h_out[i] = hash_rng_sym(get_t_hash(t[i], seed[i]), a[i], b[i]) and
 * u_out[i] = default_hash(...) (reference include/dpd/core/hash.hpp:61-65,81-88 and
 * include/dpd/maths/dpd_maths_core.hpp:55-79), computed by the same device functions the
 * force kernels use.  For known-answer tests of the RNG; either output may be NULL. */
int pdpd_rng_eval(size_t n, const uint32_t *t, const uint64_t *seed, const uint32_t *a,
                  const uint32_t *b, uint32_t *h_out, float *u_out);

/* Per-pair force log, the counterpart of the reference's ForceLogging (logging.hpp:9-100) as
 * its half-step engine feeds it from calc_force (dpd_maths_core_half_step.hpp:131-153,
 * naive_dpd_engine_half_step.hpp:239-263): one record per in-range pair (home, other) whose
 * home bead was asked for, with the names the reference logs the values under.  The FP64
 * engine records the very values its force pass uses (bit-identical to the reference's);
 * the FP32 engine records its own FP32 values, f being the pair's contribution exactly as
 * its force kernels add it. */
typedef struct pdpd_pair_terms {
    int64_t t;                       /* the step's time: the state's t before the step */
    uint32_t home_id, other_id;      /* bead ids within the world */
    uint32_t home_hash, other_hash;  /* BeadHash codes (the reference's FileLogger prints
                                        reduced hashes: hash & 0x0fffffff) */
    double dx[3];       /* "dx": home - other, periodic image applied, not normalised */
    double dr;          /* "dr" */
    double inv_root_dt; /* "dpd-invrootdt": sqrt(24 kT / dt) */
    double gammap;      /* "dpd-gammap": (sqrt(gamma_ij) (1 - dr))^2 */
    double rng;         /* "dpd-rng": default_hash of the pair, in [-0.5, 0.5) */
    double con;         /* "dpd-con" */
    double diss;        /* "dpd-diss" */
    double rng_scale;   /* "dpd-rng-scale" */
    double rand;        /* "dpd-rand" */
    double f[3];        /* "f_next_dpd": the pair's force on the home bead */
} pdpd_pair_terms;

/* Advance the attached world(s) by one step, as pdpd_run(e, 1) does, recording the pair
 * terms of that step for the n_ids beads bead_ids[] (ids within world `world`; duplicates
 * are ignored).  Records are grouped by bead in ascending id order, each bead's pairs in the
 * reference's walk order (27 directions, (-1..1)^3 with z fastest, then the cell's beads in
 * id order; in the FP32 engine a cell holds its beads with z offset < 0.5 first, each half in
 * id order).  The first min(total, capacity) records go to out; *n_pairs receives the total.
 * A debugging aid: it synchronises the device twice and allocates small device buffers. */
int pdpd_log_pair_terms(pdpd_engine *e, uint32_t world, const uint32_t *bead_ids, uint32_t n_ids,
                        pdpd_pair_terms *out, uint32_t capacity, uint32_t *n_pairs);

/* Allocation-free stepping -- this entry point has no counterpart in the reference.
 *
 * For callers that must not allocate device memory while they run: a framework that owns
 * all device memory through its own pool and forbids side allocations, or a host loop that
 * reserves its memory at start-up and cannot afford the device-wide synchronisation that
 * cudaMalloc and cudaFree may cause.  It advances one bond-free world by n_steps with the
 * FP64 integrator (bit-identical to pdpd_run's FP64 engine) on caller-owned device arrays
 * and allocates nothing: no cudaMalloc, cudaFree or allocating library call.
 *   w       box, dt, seed, t, bead types, interaction matrices (host pointers) and n_beads;
 *           its bead-array pointers are ignored.  Step k draws the random numbers of time
 *           w->t + k; the caller advances its own t by n_steps afterwards.
 *   d_x, d_v, d_f  device arrays, 3 doubles per bead in bead-id order, read and updated
 *           in place (x(t), v(t), f(t) in; x(t+n), v(t+n), f(t+n) out).
 *   d_hash  device array of the beads' BeadHash values.
 *   stream  a cudaStream_t (NULL: the legacy default stream).  The call synchronises this
 *           stream at its end and reads back a device error word, so it returns after the
 *           steps have finished; a bead that leaves the box or becomes non-finite in any
 *           of the n_steps steps makes it return PDPD_E_BEAD_LOST.
 * Limits: at most PDPD_NOALLOC_MAX_BEADS beads and PDPD_NOALLOC_MAX_CELLS cells; worlds with
 * Hookean or angle bonds are rejected (PDPD_E_UNSUPPORTED); larger worlds get PDPD_E_NOMEM.
 * Scratch memory is one fixed array inside the library (about 1.3 MB), held on every GPU that
 * loads the library until the process exits.  The first call on a device looks up that
 * array's device address (cudaGetSymbolAddress); make that first call before any stream
 * capture begins.  Every call reuses the same array: calls that overlap on the GPU (on
 * different streams or from different threads) race on it. */
#define PDPD_NOALLOC_MAX_BEADS 65536
#define PDPD_NOALLOC_MAX_CELLS 32768
int pdpd_step_noalloc(const pdpd_world *w, double *d_x, double *d_v, double *d_f,
                      const uint32_t *d_hash, uint32_t n_steps, void *stream);

/* Number of kernel launches the engine has issued since creation (graph replays count
 * each kernel node).  For accounting in benchmarks. */
uint64_t pdpd_kernel_launches(pdpd_engine *e);

/* ---- v2binary snapshots encoded on the GPU. ------------------------------------------------
 *
 * The reference writes a world state as text plus, in its "WorldState v2binary" form, a
 * BinaryData section of about 22 bytes per bead (write_world_state, dpd_state_io.hpp:408-466;
 * write_polymer_binary :182-247; CVec3Half, cvec3.hpp:132-252): per polymer a 16-bit header
 * and id deltas, per bead its position as 3 x uint32 with 16 fractional bits and v, f as
 * CVec3Half.  These calls produce and consume that section (the bytes after "BinaryData\n"
 * and its zero byte) straight from and to the device state, byte for byte what the
 * reference's writer produces for the same state (the text header stays the caller's, e.g.
 * the reference's own writer).
 *
 * prepare: the world's polymers in the order they are written (WorldState::polymers):
 *   polymer_types[p], bead ids polymer_beads[polymer_start[p] .. polymer_start[p+1]) in
 *   offset order, polymer_ids[p] (NULL: p).  Every bead must appear exactly once.
 *   *section_bytes receives the section size.  Valid until the next attach.
 * encode: write the section of the world's current state (x(t), v(t), f(t) after the last
 *   Run) into out[0..capacity); out == NULL only reports the size.  PDPD_E_INVALID if a
 *   velocity or force is not representable (non-finite, magnitude >= 2^15 after rounding).
 * decode: set the world's x, v, f from a section with the prepared structure (headers and
 *   deltas must match; PDPD_E_INVALID otherwise) -- the reference's reader
 *   (read_polymer_binary, dpd_state_io.hpp:249-330) -- and rebuild its cell list; t and the
 *   parameters are unchanged. */
int pdpd_v2binary_prepare(pdpd_engine *e, uint32_t world, uint32_t n_polymers,
                          const uint32_t *polymer_ids, const uint32_t *polymer_types,
                          const uint32_t *polymer_start, const uint32_t *polymer_beads,
                          size_t *section_bytes);
int pdpd_v2binary_encode(pdpd_engine *e, uint32_t world, uint8_t *out, size_t capacity,
                         size_t *bytes);
int pdpd_v2binary_decode(pdpd_engine *e, uint32_t world, const uint8_t *in, size_t bytes);

/* ---- Job server (continuous batching) -- no counterpart in the reference. ----------------
 *
 * The reference serves one world per engine: a caller with many independent simulations runs
 * them one after another (DPDEngine::Attach + Run(interval_count, interval_size, callback),
 * dpd_engine.hpp:176-212).  A server runs many such jobs at once on one GPU: a worker thread
 * admits submitted jobs in arrival order while their estimated device footprint fits the
 * memory budget, attaches all admitted worlds as one batch and steps them together; jobs that
 * finish leave and waiting jobs join at interval boundaries, continuing worlds keeping their
 * state on the device.  Each job's results are bit-identical to running its world alone on an
 * engine of the same precision and configuration.
 *
 * Job callback, called on the server's worker thread:
 *   status 0   interval snapshot after every interval_steps steps of the job,
 *   status 1   final state after n_steps (one call, then the job is done),
 *   status < 0 the job failed: -PDPD_E_* code (x, v, f are NULL; the message is returned by
 *              pdpd_server_drain's pdpd_last_error(NULL)).
 * x, v, f point at n_beads rows stride_bytes apart, in bead-id order, valid during the call.
 * t is the job's time after the snapshot.  Return nonzero to continue; 0 on a snapshot ends
 * the job there (like the reference's interval callback returning false) -- the job counts as
 * done and gets no further calls.  A callback may submit jobs; it must not drain or destroy
 * the server. */
typedef struct pdpd_server pdpd_server;
typedef int (*pdpd_job_fn)(void *user, uint64_t job, int64_t t, const double *x, const double *v,
                           const double *f, size_t stride_bytes, uint32_t n_beads, int status);

typedef struct pdpd_server_stats {
    uint64_t jobs_submitted, jobs_done, jobs_failed;
    uint64_t bead_steps;   /* bead-steps computed (beads x steps, summed over epochs) */
    uint64_t repacks;      /* batch re-attaches (membership changes) */
    uint32_t max_active;   /* largest number of jobs in one batch */
    uint32_t pad;
    double busy_s;         /* wall time with at least one job admitted */
    double wall_s;         /* first submit to last completion */
    double latency_p50_s, latency_p99_s, latency_max_s;  /* submit -> final callback done */
    double repack_s;       /* host wall time spent in re-packs */
    uint64_t wasted_bead_steps;  /* steps of ended jobs' worlds kept in the batch until the
                                    next re-pack (not counted in bead_steps) */
    double step_s;         /* device time of the epochs' steps (CUDA events on the engine's
                              stream); wall_s minus it is time the GPU spent on re-packs,
                              snapshots or waiting for the host */
    double host_gap_s;     /* wall time from the host seeing an epoch finish to its launch of
                              the next (re-packs included): the GPU waits for the host */
    double callback_s;     /* wall time in job callbacks (they overlap the running epoch) */
    uint64_t epochs;       /* batch runs between interval boundaries / job ends */
    double between_s;      /* device time from one epoch's end to the next one's start
                              (snapshot unsorts, re-packs, waits for the host), while busy */
    double copy_wait_s;    /* host wall time waiting for a snapshot buffer's last copy */
    double sync_wait_s;    /* host wall time waiting for epochs to finish (the GPU is busy) */
    double snap_alloc_s;   /* host wall time growing the pinned snapshot buffers */
    double post_launch_s;  /* host wall time from an epoch's launch to its snapshot enqueued */
} pdpd_server_stats;

/* Create a server with its own engine (precision, device as pdpd_create) and worker thread.
 * memory_budget_bytes bounds the summed footprint estimate of the admitted jobs (a job larger
 * than the budget still runs, alone); interval_steps >= 1 is the snapshot interval.  The
 * server reserves two pinned host buffers for the snapshots of a batch that fills the budget
 * (72 bytes per bead, at most 16 GiB each): creation takes a moment, later batches do not
 * wait for host memory to be pinned. */
int pdpd_server_create(int precision, int device, size_t memory_budget_bytes,
                       uint32_t interval_steps, pdpd_server **out);
/* Queue a job: the world (copied; the caller's arrays may be reused at once) advanced by
 * n_steps.  n_steps == 0 completes at once with one final callback on the calling thread. */
int pdpd_server_submit(pdpd_server *s, const pdpd_world *w, uint32_t n_steps, pdpd_job_fn cb,
                       void *user, uint64_t *job_id);
/* Wait until every submitted job is done or failed.  Returns PDPD_OK, or the status of the
 * last failure since the previous drain. */
int pdpd_server_drain(pdpd_server *s);
/* Set an engine configuration entry (as pdpd_set_config) while the server is idle;
 * PDPD_E_STATE while jobs are queued or running. */
int pdpd_server_config(pdpd_server *s, const char *key, const char *value);
int pdpd_server_stats_get(pdpd_server *s, pdpd_server_stats *out);
/* The server's engine, for read-only queries (pdpd_kernel_launches, pdpd_get_timings). */
pdpd_engine *pdpd_server_engine(pdpd_server *s);
/* Finish the queued jobs, stop the worker and free everything. */
void pdpd_server_destroy(pdpd_server *s);

#ifdef __cplusplus
}
#endif

#endif
