/*
 * sbc_gb300.h -- C-ABI of the GB300 StreamingBC hot path (libsbc_gb300.so).
 *
 * Plain pointers and sizes only.  Every function returns SBC_OK (0) or a
 * negative SBC_ERR_* code; sbc_last_error() gives the calling thread's last
 * message.  Vertex ids are int64 on the host side (as in the reference) and
 * must be < 2^31 - 1.
 *
 * Objects:
 *   sbc_graph   device-resident slack-CSR adjacency that accepts insertions in
 *               place; replaces the STINGER instance (struct stinger,
 *               src/stinger/stinger.h) of the reference.
 *   sbc_forest  per-root state of K roots on one graph -- dist int32, sigma
 *               int64, delta fp64 in [K][V] structure-of-arrays -- plus BC[V];
 *               replaces bcForest/bcTree (src/streamingbc_aux.h:21-40).
 * All device work of a graph and its forests runs in order on one CUDA stream
 * owned by the graph.  Calls on different graphs may run concurrently from
 * different host threads.
 */
#ifndef SBC_GB300_H_
#define SBC_GB300_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SBC_OK 0
#define SBC_ERR_ARG (-1)         /* bad argument */
#define SBC_ERR_CUDA (-2)        /* CUDA runtime error (message in sbc_last_error) */
#define SBC_ERR_NOMEM (-3)       /* device or host allocation failed */
#define SBC_ERR_STATE (-4)       /* call out of order (e.g. insert before static init) */
#define SBC_ERR_UNSUPPORTED (-5) /* operation not provided (reserved; no entry point returns it) */
#define SBC_ERR_NOGPU (-6)       /* no CUDA device */

typedef struct sbc_graph sbc_graph;
typedef struct sbc_forest sbc_forest;
typedef struct sbc_group sbc_group;

/* Per-call statistics of an insertion batch (counters match the reference's
 * COUNT_TRAVERSALS counters, src/streamingbc_internal.c:107-110,203-206,
 * 365-368,537-540, summed over roots).  A call that asks for statistics
 * restarts the counters read by sbc_read_counters. */
typedef struct {
    int64_t inserted;     /* insertions applied */
    int64_t duplicates;   /* rejected: edge already present */
    int64_t invalid;      /* rejected: self loop or vertex id out of range */
    int64_t roots_active; /* roots not culled at batch start */
    int64_t case1;        /* (insertion, root) pairs with |d| == 1 */
    int64_t case2;        /* (insertion, root) pairs with |d| > 1 */
    int64_t vertices;     /* traversed vertices */
    int64_t edges;        /* traversed edges (sum of degrees of traversed vertices) */
    int64_t scanned;      /* adjacency slots the kernels actually scanned (fewer than
                             `edges` where parents were found from the parent side) */
} sbc_batch_stats;

/* Device time per kernel kind, accumulated while profiling is on. */
typedef struct {
    double static_ms;   int64_t static_launches;
    double append_ms;   int64_t append_launches;
    double classify_ms; int64_t classify_launches;
    double update_ms;   int64_t update_launches;
    double batch_ms;    int64_t batches;
} sbc_profile;

const char *sbc_last_error(void);

/* Select the CUDA device used by objects created afterwards on this thread. */
int sbc_set_device(int device);

/* ---- graph -------------------------------------------------------------- */

/* Bulk build from a symmetric CSR (both directions stored), the shape of the
 * reference's csrGraph (src/streamingbc.h:30-35) fed to CreateStingerFromCSR
 * (src/sbcMain_utils.c:306-338) / stinger_set_initial_edges
 * (src/stinger/stinger.c:1142-1282).  off[nv+1], adj[off[nv]]. */
int sbc_graph_create(sbc_graph **out, int64_t nv, const int64_t *off, const int64_t *adj);
int sbc_graph_destroy(sbc_graph *g);
int sbc_graph_num_vertices(const sbc_graph *g, int64_t *nv);
/* Live degree of v (synchronises the graph's stream).
 * Replaces stinger_outdegree (src/stinger/stinger.h). */
int sbc_graph_degree(sbc_graph *g, int64_t v, int64_t *deg);
/* Directed insertion with stinger_insert_edge's result convention
 * (src/stinger/stinger.c:778-876): *result = 1 new, 0 already present,
 * -1 self loop.  Synchronous. */
int sbc_graph_insert_directed(sbc_graph *g, int64_t from, int64_t to, int *result);
/* Make room in the adjacency for n future undirected insertions (u[i], v[i])
 * (host arrays), re-packing the slack CSR if needed.  Needed before
 * sbc_insert_batch_device, whose endpoints the host cannot see; the host-array
 * entry points plan capacity themselves.  Synchronous. */
int sbc_graph_reserve(sbc_graph *g, int64_t n, const int64_t *u, const int64_t *v);
/* Number of adjacency re-packs so far. */
int sbc_graph_repacks(const sbc_graph *g, int64_t *count);
/* Copy the live adjacency back as CSR: off[nv+1]; adj may be NULL to query
 * off[nv] first.  Neighbour order is storage order. */
int sbc_graph_to_csr(sbc_graph *g, int64_t *off, int64_t *adj);
/* DIMACS graph files (ParseDimacsGraph, src/sbcMain_utils.c:382-422): header
 * "NV NE", then line u (u = 1, 2, ...) lists vertex u's neighbours, 1-based
 * ids used as they stand, reading stopping at a line's first non-integer
 * token.  The CSR has nv = NV + 1 vertices (vertex 0 isolated) and ne entries.
 * Parsed by all host threads; more lines than NV or an id outside 0..NV is an
 * error.  *off (nv+1) and *adj (ne) are malloc'd: release them with sbc_free.
 * No device needed. */
int sbc_dimacs_read(const char *path, int64_t *nv, int64_t *ne, int64_t **off, int64_t **adj);
void sbc_free(void *p);
/* sbc_dimacs_read + sbc_graph_create (nv, ne may be NULL). */
int sbc_graph_create_dimacs(sbc_graph **out, const char *path, int64_t *nv, int64_t *ne);

/* ---- forest ------------------------------------------------------------- */

/* K roots (roots[K], distinct vertex ids; identity of length NV for exact BC).
 * Replaces CreateForestApproximate / CreateForestExact
 * (src/streamingbc_aux.c:103-118, :51-66) plus the per-thread scratch of
 * createExtraArraysForThreads (src/streamingbc_aux.c:234-296).  `workers`
 * persistent CTAs are sized from occupancy and free memory (0 = automatic). */
int sbc_forest_create(sbc_forest **out, sbc_graph *g, int64_t nk, const int64_t *roots, int64_t workers);
/* As sbc_forest_create with an explicit launch shape of the update kernel
 * (variant -1: the SBC_UPDATE_VARIANT environment variable, else the default). */
int sbc_forest_create_ex(sbc_forest **out, sbc_graph *g, int64_t nk, const int64_t *roots, int64_t workers,
                         int variant);
/* Launch shapes of the update kernel in this build: threads per CTA and the
 * CTAs one SM keeps resident (results never depend on the shape). */
int sbc_update_variant_count(int *count);
int sbc_update_variant_info(int v, int *threads_per_cta, int *min_ctas_per_sm, int *ctas_per_sm);
int sbc_forest_destroy(sbc_forest *f);
/* nv, nk, workers, device bytes held by the forest. */
int sbc_forest_info(const sbc_forest *f, int64_t *nv, int64_t *nk, int64_t *workers, int64_t *bytes);

/* Static Brandes init over the forest's roots.  Replaces
 * BrandesApproxCaseParallel / BrandesExactParallel (src/streamingbc_init.c:60-84,
 * :24-44).  Asynchronous on the graph's stream. */
int sbc_static_init(sbc_forest *f);

/* Insert n undirected edges (u[i], v[i]) from HOST arrays, in order: each is
 * appended to the adjacency (both directions) and applied to every root, with
 * the same result as n calls of stinger_insert_edge x2 + insertEdgeStreamingBC
 * (src/sbcMain_utils.c:458-471, src/streamingbc.c:88-226).  Duplicates and self
 * loops are rejected and counted, not applied.  Synchronous; stats may be NULL. */
int sbc_insert_batch(sbc_forest *f, int64_t n, const int64_t *u, const int64_t *v, sbc_batch_stats *stats);

/* As sbc_insert_batch, but returns once the batch is queued on the graph's
 * stream (no statistics): the endpoints are copied into the graph's pinned
 * staging before return, so u and v may be reused at once; a later batch on
 * the same graph waits only until this one's staging copies have run.
 * sbc_sync waits for completion and reports slack errors. */
int sbc_insert_batch_async(sbc_forest *f, int64_t n, const int64_t *u, const int64_t *v);

/* As sbc_insert_batch, with int32 vertex ids already in DEVICE memory; returns
 * without synchronising (results are ordered on the graph's stream).  Slack for
 * these insertions must have been reserved with sbc_graph_reserve; an insertion
 * that finds no slack is not applied and the next sbc_sync reports it. */
int sbc_insert_batch_device(sbc_forest *f, int64_t n, const int32_t *d_u, const int32_t *d_v);

/* Replay device-input batches from CUDA graphs (on by default): each batch
 * size is captured once (input copies, append, classify, update, seal) and
 * replayed with only the input copies re-pointed; re-captured after an
 * adjacency re-pack.  Not used while profiling is on.  Results are the same
 * either way. */
int sbc_set_graph_capture(sbc_forest *f, int on);

/* Launch-shape selection.  The reference picks its work split with the
 * BALANCE/COARSE flags of insertEdgeStreamingBC (src/streamingbc.c:88-226,
 * enums src/streamingbc.h:9-22); here the split is the update kernel's shape
 * (threads per root, roots in flight per SM).  No shape changes any result.
 * sbc_forest_set_variant re-sizes the worker scratch for shape `variant`
 * (synchronous).  sbc_forest_autotune inserts the batch (u[i], v[i]) exactly
 * like sbc_insert_batch, but first times the update of this same batch under
 * every shape whose worker scratch fits in half the free memory, each on a
 * fresh copy of the forest's state (reps runs, fastest kept; reps 0 = 2), and
 * keeps the fastest shape for this and later batches.  ms[v] gets shape v's
 * time in ms, -1 where skipped (ms may be NULL when ms_len is 0); *chosen the
 * shape index (may be NULL).  The copy needs 21 B per root per vertex; when
 * that does not fit in half the free memory a prefix of the roots is timed. */
int sbc_forest_set_variant(sbc_forest *f, int variant);
/* The forest's roots in creation order: roots[nk]. */
int sbc_forest_roots(const sbc_forest *f, int64_t *roots);
int sbc_forest_variant(const sbc_forest *f, int *variant);
int sbc_forest_autotune(sbc_forest *f, int64_t n, const int64_t *u, const int64_t *v, int reps, int *chosen,
                        double *ms, int ms_len);

/* Apply n insertions whose edges are ALREADY in the adjacency (inserted by
 * sbc_graph_insert_directed in both directions), exactly like
 * insertEdgeStreamingBC after the caller's stinger_insert_edge calls.
 * Synchronous; stats may be NULL. */
int sbc_update_inserted(sbc_forest *f, int64_t n, const int64_t *u, const int64_t *v, sbc_batch_stats *stats);

/* ---- learned cost model and batch schedule --------------------------------
 * The reference orders roots statically under BALANCE (qsort by
 * 2*edgesBelow + edgesAbove, src/streamingbc.c:171-188).  Here an FP32 MLP
 * (8 features -> 64 -> 64 -> 1, ReLU; sbc_cost_model_size gives the parameter
 * count) predicts log(1 + touched vertices) of each (insertion, root) job
 * from features taken at batch start: d(r,a), d(r,b) for the shallower and
 * deeper endpoint (64 = unreachable), their level difference, log1p of
 * deg(a), deg(b), |sigma(r,a)|, |sigma(r,b)| (sigma wraps like the reference's
 * int64), and log1p of the number of vertices
 * at level d(r,a)+1 of r's tree.  Under SBC_SCHED_MODEL each batch's active
 * roots are queued longest predicted batch cost first; SBC_SCHED_STATIC
 * (the default and the fallback) keeps the classify order.  Results never
 * depend on the schedule.  Training data are logged by the update kernel:
 * sbc_cost_log_start makes every later batch append (features, log1p of the
 * job's touched vertices) of each job it runs, up to `capacity` samples. */
#define SBC_SCHED_STATIC 0
#define SBC_SCHED_MODEL 1
typedef struct {
    int64_t samples, train_samples, val_samples, steps;
    int epochs;
    double train_ms;      /* device time of the training kernels */
    double val_mae;       /* held-out mean |error| in log(1 + touched) */
    double val_rmse;
    double val_mae_mean;  /* held-out mean |error| of predicting the training mean */
} sbc_model_stats;
int sbc_cost_model_size(int *n_params, int *n_features);
int sbc_cost_log_start(sbc_forest *f, int64_t capacity);
int sbc_cost_log_stop(sbc_forest *f, int64_t *samples);
/* Logged samples [first, first+count): x[count][n_features], y[count]. */
int sbc_cost_log_read(sbc_forest *f, int64_t first, int64_t count, float *x, float *y);
/* Adam on the mean squared error over the first (1 - val_frac) of the logged
 * samples, `epochs` passes in minibatches of `batch` (a multiple of 128);
 * the rest is held out for the reported error.  Synchronous. */
int sbc_cost_model_train(sbc_forest *f, int epochs, int batch, double lr, double val_frac, uint64_t seed,
                         sbc_model_stats *stats);
int sbc_set_schedule(sbc_forest *f, int schedule);
/* Insert the batch (u[i], v[i]) like sbc_insert_batch, after timing its
 * update (classify or features + ordering, and the update kernel) under each
 * schedule on fresh copies of the state (reps runs each, fastest kept).
 * Needs a trained model; the forest's own schedule is unchanged. */
int sbc_forest_compare_schedules(sbc_forest *f, int64_t n, const int64_t *u, const int64_t *v, int reps,
                                 double *ms_static, double *ms_model);
/* Read (get) and/or replace (set) the n_params parameters (set marks the
 * model trained).  Layout: W1[8][64], b1[64], W2[64][64], b2[64], w3[64], b3,
 * feature means[8], inverse feature standard deviations[8]. */
int sbc_cost_model_params(sbc_forest *f, float *get, const float *set);
/* Model outputs for n feature rows (host arrays). */
int sbc_cost_model_predict(sbc_forest *f, int64_t n, const float *x, float *out);
/* Gradient of the mean squared error over n <= 65536 samples at the current
 * parameters (n_params - 16 trained entries), and the predictions. */
int sbc_cost_model_grad(sbc_forest *f, int64_t n, const float *x, const float *y, float *grad, float *pred);
/* Per-root level histograms rows [r0, r0+nr): 64 counts each (the last
 * counts level 63 and deeper). */
int sbc_get_level_hist(sbc_forest *f, int64_t r0, int64_t nr, int32_t *out);
/* Roster of level `level` (2..15) of root row r: the members of a level with at
 * most 256 vertices, kept for finding parents by lookup instead of adjacency
 * scans (after each batch it holds exactly the level's members).  *n = -1 if
 * the level is not tracked (too large, or rosters disabled); out holds up to
 * 256 entries and may be NULL. */
int sbc_get_roster(sbc_forest *f, int64_t r, int level, int32_t *out, int *n);

/* ---- groups: many forests updated by one launch per batch --------------
 * The reference updates one forest per insertEdgeStreamingBC call
 * (src/streamingbc.c:88-226); a group applies one batch to each of up to 64
 * forests, each over its own graph, with one append, one classify and one
 * persistent update launch whose work items are (forest, root) pairs from a
 * single queue.  Results equal those of per-forest sbc_insert_batch calls.
 * The group has its own stream and worker scratch; work queued on the members'
 * graph streams is ordered before and after each group batch.  A member
 * forest cannot be destroyed while a group holding it is alive. */
int sbc_group_create(sbc_group **out, int n, sbc_forest *const *forests, int variant /* -1: by size */);
int sbc_group_destroy(sbc_group *G);
int sbc_group_info(const sbc_group *G, int *n, int64_t *workers, int64_t *bytes, int *variant);
int sbc_group_set_variant(sbc_group *G, int variant);
/* counts[i] insertions for forests[i] (creation order); u/v hold them
 * concatenated in that order.  Synchronous; device_ms (may be NULL) receives
 * the device time of the batch's append..seal launches. */
int sbc_group_insert_batch(sbc_group *G, const int64_t *counts, const int64_t *u, const int64_t *v,
                           double *device_ms);
/* As sbc_group_insert_batch, after timing the update of this batch under every
 * launch shape that fits, on copies of all members' state (see
 * sbc_forest_autotune); the fastest shape is kept. */
int sbc_group_autotune(sbc_group *G, const int64_t *counts, const int64_t *u, const int64_t *v, int reps,
                       int *chosen, double *ms, int ms_len);
int sbc_group_read_counters(sbc_group *G, int64_t *vertices, int64_t *edges, int64_t *case1, int64_t *case2,
                            int64_t *scanned);
/* Every member's BC vector, concatenated in the order the members were given
 * to sbc_group_create (bc[Σ nv]), after all work queued on the group and its
 * members: one wait for all of them. */
int sbc_group_get_bc(sbc_group *G, double *bc);

/* ---- serving loop ---------------------------------------------------------
 * A server keeps many graphs (each with its forest of K roots) resident on
 * one device and batches insertion requests per graph as they arrive; the
 * reference's callers apply one insertion at a time (src/sbcMain_utils.c:
 * 458-471, src/streamingbc.c:56-77).  Graphs are admitted in registration
 * order while the sum of their estimated device footprints (adjacency,
 * per-root state, worker scratch) fits hbm_budget_bytes; requests for a graph
 * not yet admitted wait in its queue.  A scheduler thread launches, for every
 * graph with queued requests and no batch on the device, all of them (up to
 * max_batch) as its next batch on the graph's own stream, so graphs overlap on
 * the device and requests arriving meanwhile join the next batch.  Latency is
 * measured from each request's arrival to its batch's completion.  Per-graph
 * order is kept, so every graph ends where applying its own stream alone ends. */
typedef struct sbc_server sbc_server;
typedef struct {
    int64_t submitted, completed, batches, graphs_admitted, graphs_waiting;
    double p50_us, p99_us, mean_us, max_us;  /* arrival -> batch completion */
    double throughput;      /* completed / (last completion - first arrival), insertions/s */
    double mean_batch;      /* requests per launched batch */
    int64_t bytes_admitted, bytes_budget;
} sbc_server_stats;
int sbc_server_create(sbc_server **out, int device, int64_t hbm_budget_bytes, int max_batch);
int sbc_server_destroy(sbc_server *s);
/* At most max_inflight batches on the device at once over all graphs (0, the
 * default, means no limit); graphs are served round-robin.  max_batch 1 with
 * max_inflight 1 is the plain path: one insertion at a time. */
int sbc_server_set_max_inflight(sbc_server *s, int max_inflight);
/* Tuning of the served graphs (off by default; set before requests arrive).
 * autotune != 0: a graph registered with variant -1 has its first batch of
 * at least 64 requests (any size when max_batch < 64) applied through
 * sbc_forest_autotune, which keeps the fastest launch shape for its later
 * batches.  train_insertions > 0: every graph logs its jobs'
 * costs over its first train_insertions applied insertions (after the tuned
 * batch), then trains its cost model (sbc_cost_model_train: 4 epochs,
 * minibatch 4096, lr 2e-3, 10 % held out) and is scheduled by it
 * (SBC_SCHED_MODEL); with fewer than 128 logged jobs to train on it keeps the
 * static schedule.  Neither changes any result. */
int sbc_server_set_tuning(sbc_server *s, int autotune, int64_t train_insertions);
/* Register a graph (symmetric CSR, copied) with nk roots; variant -1 picks the
 * update launch shape by size.  *id is its index (0, 1, ...). */
int sbc_server_add_graph(sbc_server *s, int64_t nv, const int64_t *off, const int64_t *adj, int64_t nk,
                         const int64_t *roots, int variant, int *id);
/* state: 0 waiting for admission, 1 admitted, 2 released, 3 evicted (its
 * forest checkpointed in host memory, waiting to be admitted again). */
int sbc_server_graph_info(sbc_server *s, int id, int *state, int64_t *footprint_bytes, int64_t *completed,
                          int64_t *batches);
/* One insertion request (arrival time = now).  Thread-safe. */
int sbc_server_submit(sbc_server *s, int id, int64_t u, int64_t v);
/* Trace player: request i (graph[i], u[i], v[i]) arrives t_offset_s[i]
 * seconds after the call (non-decreasing); returns once all are submitted. */
int sbc_server_play(sbc_server *s, int64_t n, const int32_t *graph, const int64_t *u, const int64_t *v,
                    const double *t_offset_s);
/* Wait until every admitted graph's static init and submitted requests have
 * completed and no release or admission is left to carry out (requests of
 * graphs that do not fit the budget yet stay queued). */
int sbc_server_drain(sbc_server *s);
const char *sbc_server_error(sbc_server *s);
/* Free graph id's device memory once its queue is empty (waiting graphs may
 * then be admitted); later requests for it are refused. */
int sbc_server_release(sbc_server *s, int id);
/* Evict graph id once no batch of it is on the device: its forest is
 * checkpointed into host memory (sbc_checkpoint_take), its device memory
 * freed, and it joins the end of the admission queue; requests for it keep
 * queueing.  When it fits again it is restored from the checkpoint (no static
 * init) and its queued requests run.  Results equal never evicting it. */
int sbc_server_evict(sbc_server *s, int id);
/* Results of an idle admitted graph, or of an evicted one with no queued
 * requests (from its checkpoint); any pointer may be NULL:
 * dist[nk][nv], sigma[nk][nv], bc[nv]. */
int sbc_server_read(sbc_server *s, int id, int32_t *dist, int64_t *sigma, double *bc);
int sbc_server_get_stats(sbc_server *s, sbc_server_stats *stats, int reset);

/* ---- edge deletion --------------------------------------------------------
 * Replaces deleteEdgeStreamingBC (src/streamingbc.c:258-416): per root, the
 * endpoints on one level (or both unreachable) change nothing; otherwise the
 * deeper endpoint b either keeps a parent -- sigma-only decrease and
 * dependency ascent, the reference's removeEdgeWithoutMovementBrandes
 * (src/streamingbc_internal.c:607-868) -- or loses its last one, the
 * reference's moveDownTreeBrandes (:880-1401), whose results disagree with a
 * recomputation of the modified graph.  Here that case either moves the
 * affected vertices down in place (exact: new levels, sigma and dependencies
 * of the changed part only) or recomputes the root from scratch once, after
 * the call's last deletion (BC moved by its new minus old dependencies; the
 * root skips the call's later deletions).  SBC_DELETE_AUTO moves down on
 * graphs of >= 32768 vertices and recomputes on smaller ones, where a whole
 * recompute is cheap; a move-down whose affected set exceeds max(1024, V/16)
 * vertices falls back to the recompute.  Results equal a static recompute of
 * the modified graph in every mode (tested).  stats->inserted counts edges
 * removed, duplicates edges absent, invalid bad ids; case1/case2 the
 * (root, deletion) pairs whose deeper endpoint keeps / loses its parents. */
#define SBC_DELETE_AUTO 0
#define SBC_DELETE_MOVE_DOWN 1
#define SBC_DELETE_RECOMPUTE 2
/* A setting of the forest object (a new or restored forest starts in
 * SBC_DELETE_AUTO); it applies to the deletions issued after the call. */
int sbc_forest_set_delete_mode(sbc_forest *f, int mode);
/* Remove n undirected edges in order, with the update of every root after
 * each, as n single deletions would.  One update launch serves the whole
 * call: the removed slots stay marked in place until it ends, so each
 * deletion's jobs see the graph without the edges of that deletion and the
 * earlier ones.  Synchronous; stats may be NULL. */
int sbc_delete_batch(sbc_forest *f, int64_t n, const int64_t *u, const int64_t *v, sbc_batch_stats *stats);
/* The update for one deletion whose edge the caller has already removed in
 * both directions (sbc_graph_remove_directed x2, or stinger_remove_edge x2),
 * exactly like deleteEdgeStreamingBC after the caller's removals. */
int sbc_update_deleted(sbc_forest *f, int64_t u, int64_t v, sbc_batch_stats *stats);
/* Directed removal with stinger_remove_edge's result: 1 removed, 0 absent,
 * -1 self loop / bad id.  Synchronous. */
int sbc_graph_remove_directed(sbc_graph *g, int64_t from, int64_t to, int *result);
/* Live neighbours of v: *n = its degree; the first min(cap, *n) are copied to
 * out (cap 0 / out NULL to query the degree).  Synchronous. */
int sbc_graph_neighbors(sbc_graph *g, int64_t v, int64_t *out, int64_t cap, int64_t *n);

/* Wait for all work queued on the forest's graph stream. */
int sbc_sync(sbc_forest *f);
/* Read and reset the traversal/case counters accumulated since the last read
 * (any pointer may be NULL); `scanned` is the adjacency slots actually read. */
int sbc_read_counters(sbc_forest *f, int64_t *vertices, int64_t *edges, int64_t *case1, int64_t *case2,
                      int64_t *scanned);

/* ---- forest checkpoints ---------------------------------------------------
 * No counterpart in the reference (its forest lives in host records for the
 * life of the process; STINGER's save/open, src/stinger/stinger.c:1808,1936,
 * stores the graph alone).  A checkpoint holds the graph's live adjacency as a
 * CSR, the roots, every root's dist / sigma / delta row and BC, in host
 * memory.  Restoring builds a new graph and forest in exactly that state with
 * no static init (one-byte distances, level histograms and rosters are derived
 * from dist on the device); the restored forest continues where the saved one
 * stood.  All synchronous. */
typedef struct sbc_checkpoint sbc_checkpoint;
int sbc_checkpoint_take(sbc_forest *f, sbc_checkpoint **out);
/* variant -1: the default update launch shape. */
int sbc_checkpoint_restore(const sbc_checkpoint *c, int variant, sbc_graph **g, sbc_forest **f);
/* File form: a 40-byte header ("SBCCKPT1", version 1, nv, nk, ne), then off,
 * adj (int32), roots, bc, dist, sigma, delta, little-endian. */
int sbc_checkpoint_save(const sbc_checkpoint *c, const char *path);
int sbc_checkpoint_load(const char *path, sbc_checkpoint **out);
/* nv, nk, directed adjacency entries, host bytes held (any may be NULL). */
int sbc_checkpoint_info(const sbc_checkpoint *c, int64_t *nv, int64_t *nk, int64_t *ne, int64_t *bytes);
/* The saved state: dist[nk][nv], sigma[nk][nv], bc[nv] (any may be NULL). */
int sbc_checkpoint_read(const sbc_checkpoint *c, int32_t *dist, int64_t *sigma, double *bc);
int sbc_checkpoint_free(sbc_checkpoint *c);

/* ---- state read-back (synchronous) ------------------------------------- */

int sbc_get_bc(sbc_forest *f, double *out /* [nv] */);
/* Rows [r0, r0+nr) of the root-major state; dist uses INT32_MAX for
 * unreachable, sigma is 0 where unreachable. */
int sbc_get_dist(sbc_forest *f, int64_t r0, int64_t nr, int32_t *out);
int sbc_get_sigma(sbc_forest *f, int64_t r0, int64_t nr, int64_t *out);
int sbc_get_delta(sbc_forest *f, int64_t r0, int64_t nr, double *out);

/* ---- timing -------------------------------------------------------------- */

/* Record CUDA events around every kernel launch of this forest (off by default). */
int sbc_set_profiling(sbc_forest *f, int on);
int sbc_get_profile(sbc_forest *f, sbc_profile *out);
int sbc_reset_profile(sbc_forest *f);
/* Device-time stopwatch on the forest's stream: sbc_timer_start records an
 * event; sbc_timer_stop records another, synchronises and returns the ms between. */
int sbc_timer_start(sbc_forest *f);
int sbc_timer_stop(sbc_forest *f, double *ms);

/* ---- static init that allocates nothing ---------------------------------- */

/* This entry point has no counterpart in the reference.
 *
 * For callers that cannot call cudaMalloc themselves or let a library do it
 * -- code running inside another runtime that owns the device memory pool,
 * or a process whose device memory is reserved up front -- this runs the
 * static Brandes init (the same kernel as sbc_static_init) with all of its
 * scratch taken from one fixed array compiled into libsbc_gb300.so: every GPU
 * that loads the library holds SBC_NOALLOC_SCRATCH_BYTES (about 37 MiB) of
 * device memory for it until the process exits.  The call allocates nothing:
 * no cudaMalloc, no cudaFree, no allocating library routine.
 *
 * All pointers are DEVICE memory owned by the caller:
 *   d_off[nv+1] int64, d_col[d_off[nv]] int32  symmetric CSR of the graph:
 *                                              d_off[0] == 0, non-decreasing,
 *                                              every neighbour id in [0, nv)
 *   d_roots[nk] int64                          distinct root vertices, each in [0, nv)
 *   d_dist[nk][nv] int32 (INT32_MAX = unreachable), d_sigma[nk][nv] int64,
 *   d_delta[nk][nv] fp64, d_bc[nv] fp64         outputs, as sbc_get_dist/...
 * Limits: nv <= SBC_NOALLOC_MAX_VERTICES and nk * nv <= SBC_NOALLOC_MAX_CELLS;
 * larger sizes are rejected with SBC_ERR_ARG before any GPU work.
 * The work is queued on `stream` (a cudaStream_t; NULL = the legacy default
 * stream) and the call waits for it before returning.  The ids are checked on
 * the device first: a root or neighbour id outside [0, nv), or an offset
 * array that does not start at 0 or decreases, makes the call return
 * SBC_ERR_ARG without running the init (the outputs are then not written; a
 * root outside the graph is never used as an index).
 *
 * The first call on a device looks up the device address of the array on the
 * current device (cudaGetSymbolAddress) and keeps it for later calls on that
 * device; make that first call before any CUDA stream capture.  The kept
 * address belongs to the device's context at the time: after
 * cudaDeviceReset on that device the library must be unloaded and loaded
 * again before this entry point is used there.  Every call on a device uses
 * the same array and leaves its contents behind for the next; what must
 * start at zero is cleared on the stream at the start of each call.  Calls
 * whose GPU work overlaps -- on different streams, or from different host
 * threads -- race on the array and give undefined results: serialise them.
 * A CUDA error left pending by earlier work of the caller is reported as
 * such (SBC_ERR_CUDA) before anything is queued.
 * Errors: SBC_ERR_ARG, SBC_ERR_NOGPU, SBC_ERR_CUDA; message from
 * sbc_noalloc_last_error(). */
#define SBC_NOALLOC_MAX_VERTICES 262144
#define SBC_NOALLOC_MAX_CELLS 4194304
#define SBC_NOALLOC_WORKERS 8
#define SBC_NOALLOC_SCRATCH_BYTES 38797824
int sbc_static_init_noalloc(int64_t nv, const int64_t *d_off, const int32_t *d_col, int64_t nk,
                            const int64_t *d_roots, int32_t *d_dist, int64_t *d_sigma, double *d_delta,
                            double *d_bc, void *stream);
const char *sbc_noalloc_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* SBC_GB300_H_ */
