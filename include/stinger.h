/*
 * stinger.h -- minimal STINGER-compatible graph handle over the GB300 device
 * adjacency (libsbc_gb300.so).
 *
 * Reference-style callers of streamingbc.h build and grow their graph through
 * these STINGER entry points (src/stinger/stinger.h of the reference); here
 * each one forwards to an sbc_graph (include/sbc_gb300.h).  Only the calls the
 * betweenness-centrality path uses are provided.  Differences:
 *   - no edge types, weights or timestamps (accepted and ignored);
 *   - vertex ids up to 2^31-2 instead of STINGER_MAX_LVERTICES = 2^22;
 *   - each graph owns its storage (the reference's edge-block pool is process
 *     global and stinger_free releases it for every instance,
 *     src/stinger/stinger.c:557-568);
 *   - edge removal (src/stinger/stinger.c:1055-1090) compacts the slot out of
 *     the vertex's sorted segment instead of marking it deleted.
 */
#ifndef SBC_STINGER_SHIM_H_
#define SBC_STINGER_SHIM_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

struct stinger; /* opaque; wraps an sbc_graph */

/* src/stinger/stinger.c:520 -- an empty graph; vertices appear with
 * stinger_set_initial_edges. */
struct stinger *stinger_new(void);

/* src/stinger/stinger.c:1142-1282 -- bulk load of a directed CSR with nv
 * vertices (off[nv+1], phys_to[off[nv]]).  Type, weights and times ignored. */
void stinger_set_initial_edges(struct stinger *G, const size_t nv, const int64_t etype, const int64_t *off,
                               const int64_t *phys_to, const int64_t *weights, const int64_t *times,
                               const int64_t *first_times, const int64_t single_ts);

/* src/stinger/stinger.c:778-876 -- directed insertion: 1 new, 0 present,
 * -1 self loop / invalid. */
int stinger_insert_edge(struct stinger *G, int64_t type, int64_t from, int64_t to, int64_t weight,
                        int64_t timestamp);

/* src/stinger/stinger.c:990-1010 -- both directions; -1 if either failed. */
int stinger_insert_edge_pair(struct stinger *G, int64_t type, int64_t from, int64_t to, int64_t weight,
                             int64_t timestamp);

/* src/stinger/stinger.c:1055-1090 -- directed removal: 1 removed, -1 absent,
 * self loop or invalid id (the reference's code returns -1 for an absent edge,
 * although its comment says 0).  Synchronous (reads the result back). */
int stinger_remove_edge(struct stinger *G, int64_t type, int64_t from, int64_t to);

int64_t stinger_outdegree(const struct stinger *G, int64_t v);
int64_t stinger_typed_outdegree(const struct stinger *G, int64_t v, int64_t type);

/* Frees this graph only; returns NULL. */
struct stinger *stinger_free(struct stinger *G);

/* The sbc_graph behind a handle (NULL before stinger_set_initial_edges). */
struct sbc_graph *stinger_sbc_graph(struct stinger *G);

#ifdef __cplusplus
}
#endif

#endif /* SBC_STINGER_SHIM_H_ */
