/*
 * pado_gpu.h -- C ABI of the GB300 PADO library: pruned landmark (2-hop)
 * labeling and exact distance queries on one GPU.
 *
 * The reference (johnpzh/parallel_distance_oracle, "PADO") exposes this path
 * as C++ class templates whose constructor labels a rank-relabeled Graph and
 * whose query_distance() answers a pair.  Every entry point below names the
 * reference interface it replaces; include/pado_gpu.hpp wraps them back into
 * those class names so pado.cpp / query_distance.cpp compile unchanged.
 *
 * Conventions (includes/globals.h:27-40 of the reference):
 *   vertex ids uint32; unweighted distances uint8 with 255 = unreachable;
 *   weighted edge weights uint8 (graph.h:300), distances int16 with
 *   32767 = unreachable.
 *   "rank" arrays follow Graph::id_transfer (graph.h:176-206): rank[v] is the
 *   position of original vertex v in the vertex order, 0 = most important.
 *   Query endpoints are ORIGINAL ids (as after order_labels() /
 *   load_index_from_file() in the reference); a hub id in an exported label is
 *   a RANK, exactly like the reference's Index.
 *
 * All functions return a pado_status; pado_last_error() gives the message of
 * the most recent failure on the calling thread.  No function exits the
 * process.  One GPU: the device current on the calling thread when the index
 * is created is used for its whole life.  An index may be queried from
 * several host threads at once; building, loading and freeing are
 * single-owner.
 */
#ifndef PADO_GPU_H_
#define PADO_GPU_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum pado_status {
    PADO_OK = 0,
    PADO_E_ARG = 1,       /* invalid argument (sizes, ids, batch size, ...) */
    PADO_E_NOMEM = 2,     /* device or host allocation failed */
    PADO_E_CUDA = 3,      /* a CUDA call failed */
    PADO_E_OVERFLOW = 4,  /* a distance does not fit the reference's type
                             (unweighted BFS level >= 255) */
    PADO_E_IO = 5,        /* index file could not be read or written */
    PADO_E_TIMEOUT = 6,   /* a bounded device wait gave up */
    PADO_E_STATE = 7      /* call not valid for this index (e.g. weighted vs
                             unweighted) */
} pado_status;

typedef struct pado_index pado_index;

/* Label set kind. */
#define PADO_UNWEIGHTED 0
#define PADO_WEIGHTED 1

/* Maximum bit-parallel roots and root batch size the kernels accept. */
#define PADO_MAX_BP_ROOTS 64u
#define PADO_MAX_BATCH 2048u

const char *pado_last_error(void);
const char *pado_status_string(int status);
/* Library version string, e.g. "pado-gpu 0.1 sm_103a". */
const char *pado_version(void);

/* ---------------------------------------------------------------------------
 * Building.
 *
 * pado_unw_build replaces the labeling constructor
 *   VertexCentricPLL<BATCH_SIZE>::VertexCentricPLL(const Graph &G)
 *     (includes/pado_unw_unv_unp.h:260-264, construct :990-1118)
 *   ParaVertexCentricPLL<BATCH_SIZE>::ParaVertexCentricPLL(const Graph &G)
 *     (includes/pado_unw_unv_para.201912311607.parallel_bp_labeling.h:307-311)
 * extended, as the rebuild's interface asks, with the vertex order, the
 * bit-parallel root count (a class constant, 50, in the reference:
 * pado_unw_unv_unp.h:46) and the root batch size (the BATCH_SIZE template
 * argument).
 *
 * The graph is an undirected CSR over ORIGINAL ids with both directions
 * stored: off[n+1] (off[n] = number of directed entries), adj[off[n]].
 * Duplicate entries are kept and self-loops are honoured exactly as the
 * reference's Graph does (graph.h:125-153).  rank[n] is the vertex order.
 * bp_roots <= 64, 1 <= batch <= 2048.
 * ------------------------------------------------------------------------- */
int pado_unw_build(uint32_t n, const uint64_t *off, const uint32_t *adj, const uint32_t *rank,
                   uint32_t bp_roots, uint32_t batch, pado_index **out);

/* Same, for a graph that is ALREADY rank-relabeled (ids are ranks), which is
 * what the reference's constructors receive after Graph::id_transfer().  The
 * neighbour lists need not be sorted.  Query endpoints are ranks until
 * pado_set_order() installs the original-id mapping (order_labels,
 * pado_unw_unv_unp.h:1227-1310). */
int pado_unw_build_ranked(uint32_t n, const uint64_t *off, const uint32_t *adj, uint32_t bp_roots,
                          uint32_t batch, pado_index **out);

/* Labels G independent unweighted graphs together and returns one index per
 * graph in out[0..G): every graph gets exactly the labels pado_unw_build
 * would give it alone (same bp_roots and batch), but one persistent launch
 * advances all graphs by one BFS level per step, so small graphs no longer
 * cost a launch sequence each.  Graph i has n[i] vertices, CSR off[i]
 * (n[i] + 1 entries) and adj[i], and vertex order rank[i] (rank itself or
 * rank[i] NULL: the ids are already ranks, as in pado_unw_build_ranked).
 * Replaces calling the labeling constructor (pado_unw_unv_unp.h:176-189) once
 * per graph.  Sum of n[i] < 2^32 - 1, 1 <= G <= 65535.  On error no handle is
 * returned. */
int pado_unw_build_many(uint32_t G, const uint32_t *n, const uint64_t *const *off,
                        const uint32_t *const *adj, const uint32_t *const *rank,
                        uint32_t bp_roots, uint32_t batch, pado_index **out);

/* Batch-size tuner for pado_unw_build_many: labels `sample` of the graphs
 * (evenly spaced in size order, smallest and largest included; 0 = all) once
 * per candidate batch size in candidates[0..ncand), times each on the device
 * and writes the fastest to *best (ms[c], if not NULL, receives candidate c's
 * time).  The labels depend on the batch size (as the reference's do), so
 * the tuned size is an input the caller then passes to pado_unw_build_many. */
int pado_unw_tune_batch(uint32_t G, const uint32_t *n, const uint64_t *const *off,
                        const uint32_t *const *adj, const uint32_t *const *rank,
                        uint32_t bp_roots, const uint32_t *candidates, uint32_t ncand,
                        uint32_t sample, uint32_t *best, float *ms);

/* Weighted labeling; replaces
 *   WeightedVertexCentricPLL<BATCH_SIZE>::WeightedVertexCentricPLL(const WeightedGraph &)
 *     (includes/pado_weighted_unv_unp.h:275-279, construct :1408-1526)
 *   WeightedParaVertexCentricPLL<BATCH_SIZE>::WeightedParaVertexCentricPLL(...)
 *     (includes/pado_weighted_unv_para.h:296-300).
 * w[off[n]] are the per-entry edge weights (uint8, as WeightedGraph stores
 * them). */
int pado_w_build(uint32_t n, const uint64_t *off, const uint32_t *adj, const uint8_t *w,
                 const uint32_t *rank, uint32_t batch, pado_index **out);
int pado_w_build_ranked(uint32_t n, const uint64_t *off, const uint32_t *adj, const uint8_t *w,
                        uint32_t batch, pado_index **out);

/* ---------------------------------------------------------------------------
 * Graph ingest on the device.
 *
 * These replace the reference's host-side graph preparation, run before any
 * labeler:
 *   Graph::Graph(const char *) / WeightedGraph::WeightedGraph(const char *)
 *     (includes/graph.h:95-117, :262-290): "head tail [weight]" text lines,
 *     lines starting with '#' or '%' skipped;
 *   Graph::construct (graph.h:125-153; weighted :292-309): both directions
 *     of every edge stored, duplicates and self-loops kept, n = max id + 1;
 *   Graph::make_rank (graph.h:156-174): degree descending -- ties broken by
 *     ascending id here (the reference adds rand()/RAND_MAX, which no two
 *     hosts reproduce);
 *   Graph::id_transfer (graph.h:176-206; weighted :367-400): ids relabeled
 *     to ranks, every list in descending (id, weight) order.
 * With PADO_INGEST_DEDUPE, self-loops are dropped and repeated undirected
 * pairs merged first (the first weight in input order wins), the cleaning a
 * benchmark generator applies to an edge sample.  Edge counts m < 2^31,
 * fewer than 2^28 vertices.
 * ------------------------------------------------------------------------- */
#define PADO_INGEST_DEDUPE 1u

/* Edge list (u[i], v[i]) with optional uint8 weights w[i] (NULL:
 * unweighted) over ids < n, to the ranked CSR: off[n+1], adj[*entries] (room
 * for 2m), w_out[*entries] (weighted), and the order rank[n] (rank[v] = new
 * id of original vertex v).  The output is what pado_unw_build_ranked /
 * pado_w_build_ranked take, with rank for pado_set_order. */
int pado_graph_ingest(uint64_t m, const uint32_t *u, const uint32_t *v, const uint8_t *w, uint32_t n,
                      uint32_t flags, uint64_t *off, uint32_t *adj, uint8_t *w_out, uint32_t *rank,
                      uint64_t *entries);

/* Same with every array in device memory (the current device): d_adj /
 * d_w_out need room for 2m entries.  Runs on `stream` (a cudaStream_t; NULL:
 * the legacy default stream) and returns when the outputs are written. */
int pado_graph_ingest_device(uint64_t m, const uint32_t *d_u, const uint32_t *d_v, const uint8_t *d_w, uint32_t n,
                             uint32_t flags, uint64_t *d_off, uint32_t *d_adj, uint8_t *d_w_out, uint32_t *d_rank,
                             uint64_t *entries, void *stream);

/* ---------------------------------------------------------------------------
 * Graph reductions: the reference's two graph-conversion tools on the device.
 * Both take an edge list (u[i], v[i]) in input order over ids < n (the tools
 * use n = max id + 1), build the tools' adjacency (both directions of every
 * input edge; repeats and self-loops stay and count), and return per-vertex
 * flags plus the indices of the input edges that survive, in input order --
 * the edges the tools write.  m < 2^31 edges, n < 2^31 vertices.
 * ------------------------------------------------------------------------- */

/* Replaces tools/pseudocode-delete_1-degree_vertices.cpp
 * (Graph::delete_1_degree_vertices, :127-199): every vertex with one
 * adjacency entry is deleted together with the chain of two-entry vertices
 * behind it, up to but not including the first vertex whose entry count is
 * not 2 (a path component goes entirely).  deleted[n]: 1 = deleted;
 * kept[*m_kept] (room for m): indices of the edges with no deleted end. */
int pado_reduce_degree1(uint64_t m, const uint32_t *u, const uint32_t *v, uint32_t n, uint8_t *deleted,
                        uint64_t *kept, uint64_t *m_kept);

/* Replaces distributed_version/tools/graph-convert/remove_equivalent_vertices.cpp
 * (eliminate_vertices, :96-338): vertices whose sets {x} + adjacency entries
 * are equal multisets form a class; the smallest id of a class stays and the
 * others get redundant[x] = 1.  new_id[n] numbers the vertices that stay in
 * ascending id (2^32 - 1 for redundant ones); kept as above; *n_out = 1 + the
 * largest new id on a kept edge (0 if none), the vertex count the tool
 * writes before its (new_id[u], new_id[v]) pairs. */
int pado_reduce_equivalent(uint64_t m, const uint32_t *u, const uint32_t *v, uint32_t n, uint8_t *redundant,
                           uint32_t *new_id, uint64_t *kept, uint64_t *m_kept, uint32_t *n_out);

/* Same with every array in device memory (the current device), on `stream`
 * (a cudaStream_t; NULL: the legacy default stream); they return when the
 * outputs are written.  d_kept needs room for m entries. */
int pado_reduce_degree1_device(uint64_t m, const uint32_t *d_u, const uint32_t *d_v, uint32_t n, uint8_t *d_deleted,
                               uint64_t *d_kept, uint64_t *m_kept, void *stream);
int pado_reduce_equivalent_device(uint64_t m, const uint32_t *d_u, const uint32_t *d_v, uint32_t n,
                                  uint8_t *d_redundant, uint32_t *d_new_id, uint64_t *d_kept, uint64_t *m_kept,
                                  uint32_t *n_out, void *stream);

/* The ingest calls take their scratch (sort keys and buffers, about 24
 * bytes per edge) from a memory pool of the library's own, in stream order.
 * Up to `bytes` of it stay reserved on the current device between calls
 * (default 0: every call returns its scratch); a service that ingests
 * graphs repeatedly keeps them to skip the device allocations.  Setting 0
 * releases what is kept. */
int pado_set_scratch_cache(uint64_t bytes);

/* Ingest + labeling in one call, the graph staying on the device between
 * them: the index answers queries by ORIGINAL id (the reference's sequence
 * Graph -> make_rank -> id_transfer -> labeler -> order_labels, pado.cpp
 * main).  n = 0 takes max id + 1. */
int pado_unw_build_edges(uint64_t m, const uint32_t *u, const uint32_t *v, uint32_t n, uint32_t flags,
                         uint32_t bp_roots, uint32_t batch, pado_index **out);
int pado_w_build_edges(uint64_t m, const uint32_t *u, const uint32_t *v, const uint8_t *w, uint32_t n,
                       uint32_t flags, uint32_t batch, pado_index **out);

/* Same from an edge-list file (kind PADO_UNWEIGHTED or PADO_WEIGHTED): the
 * text is read in pieces and parsed on the device.  Lines that are empty,
 * start with '#' or '%', or do not begin with two decimal ids below 2^32 are
 * skipped; a missing weight is 0 and weights are cast to uint8 (graph.h:300).
 * Errors: PADO_E_IO when the file cannot be read. */
int pado_build_edge_file(const char *path, uint32_t kind, uint32_t flags, uint32_t bp_roots, uint32_t batch,
                         pado_index **out);

/* The device text parser alone: text[0..bytes) to at most `capacity` edges in
 * line order; *m receives the edge count (also when it exceeds capacity,
 * which fails with PADO_E_ARG). */
int pado_edge_text_parse(const char *text, uint64_t bytes, uint32_t weighted, uint64_t capacity, uint32_t *u,
                         uint32_t *v, uint8_t *w, uint64_t *m);

/* Install the original-id mapping (rank[v] = rank of original vertex v).
 * Replaces order_labels(rank2id, rank) (pado_unw_unv_unp.h:1227-1310,
 * pado_weighted_unv_unp.h:1715-1779) for indexes built from ranked graphs. */
int pado_set_order(pado_index *h, const uint32_t *rank);

void pado_free(pado_index *h);

/* ---------------------------------------------------------------------------
 * Introspection and export (canonical form = the reference's Index after
 * order_labels: per ORIGINAL vertex, its (rank hub, distance) labels sorted by
 * hub, plus for unweighted indexes the bp_roots bit-parallel rows).
 * ------------------------------------------------------------------------- */
typedef struct pado_info {
    uint32_t n;
    uint32_t kind;        /* PADO_UNWEIGHTED or PADO_WEIGHTED */
    uint32_t bp_roots;
    uint32_t batch;
    uint64_t num_labels;  /* total normal labels (canonical) */
    double build_seconds; /* device time of the labeling (BP + batches) */
    double bp_seconds;    /* device time of the bit-parallel labeling */
    uint64_t device_bytes;/* device memory held by the index */
    uint32_t levels;      /* BFS levels / relaxation rounds run */
    uint32_t batches;
} pado_info;

int pado_get_info(const pado_index *h, pado_info *info);

/* Host buffers: off[n+1], hub[num_labels], dist[num_labels] (uint8 for
 * unweighted, int16 for weighted), bp_dist[n*bp_roots] and
 * bp_sets[n*bp_roots*2] (S^-1, S^0 per root; unweighted only, may be NULL).
 * Page-locked buffers (cudaHostAlloc / cudaHostRegister) are written by the
 * device directly; pageable ones are staged through device memory. */
int pado_export(const pado_index *h, uint64_t *off, uint32_t *hub, void *dist, uint8_t *bp_dist,
                uint64_t *bp_sets);

/* Create a query-only index from canonical arrays (e.g. labels produced by
 * the reference); the inverse of pado_export. */
int pado_import(uint32_t kind, uint32_t n, uint32_t bp_roots, const uint64_t *off, const uint32_t *hub,
                const void *dist, const uint8_t *bp_dist, const uint64_t *bp_sets, pado_index **out);

/* ---------------------------------------------------------------------------
 * Queries; replace query_distance(a, b)
 *   (pado_unw_unv_unp.h:1312-1445 -> uint8, pado_weighted_unv_unp.h:1782-1900
 *   -> int16).  Out-of-range ids give 0 when a == b, else unreachable.
 * ------------------------------------------------------------------------- */
/* Host arrays: a[k], b[k], out[k] (uint8_t for unweighted, int16_t for
 * weighted).  Synchronous. */
int pado_query(pado_index *h, uint64_t k, const uint32_t *a, const uint32_t *b, void *out);

/* Device arrays, enqueued on `stream` (a cudaStream_t, 0 = legacy default);
 * returns once enqueued. */
int pado_query_device(pado_index *h, uint64_t k, const uint32_t *d_a, const uint32_t *d_b,
                      void *d_out, void *stream);

/* ---------------------------------------------------------------------------
 * Index files, in the reference's on-disk format:
 *   store_index_to_file (pado_unw_unv_unp.h:1120-1180,
 *                        pado_weighted_unv_unp.h:1639-1676)
 *   load_index_from_file (pado_unw_unv_unp.h:1182-1224,
 *                         pado_weighted_unv_unp.h:1678-1711)
 * Unweighted: [n u32][K u32] then per original vertex K x (u8 d, u64 S^-1,
 * u64 S^0), u32 count, count x (u32 hub, u8 d).  Weighted: [n u32] then per
 * vertex u32 count, count x (u32 hub, i16 d).
 * ------------------------------------------------------------------------- */
int pado_store(const pado_index *h, const char *path);
int pado_load(const char *path, uint32_t kind, pado_index **out);

/* ---------------------------------------------------------------------------
 * Queries without device allocation.  No counterpart in the reference (whose
 * queries run on the CPU).  For callers that must not have a library allocate
 * device memory -- latency-bound serving threads, where cudaMalloc/cudaFree can
 * block on device-wide synchronisation, and processes whose GPU memory is owned
 * by another allocator: the pairs and results are staged through a fixed
 * 2.5 MiB area compiled into the library, so at most PADO_NOALLOC_MAX_PAIRS
 * pairs per call (more -> PADO_E_ARG).  Same arguments and results as
 * pado_query; synchronous; the caller's current device is left as it was.
 * The first call on a device is the slow one: it looks the area's address up,
 * and with lazy module loading (the CUDA default) it is what loads the
 * library's device code and so creates the area.  Make one warm-up call per
 * device (k >= 1) before any latency-sensitive section and before any stream
 * capture.  After a device reset (cudaDeviceReset) the area is gone and the
 * address this library remembered is stale: do not use this entry point on a
 * device that was reset.  All calls on a device share the area: calls that
 * overlap on the GPU (e.g. from two host threads at once) race on it and must
 * be serialised by the caller.
 * ------------------------------------------------------------------------- */
#define PADO_NOALLOC_MAX_PAIRS 262144u
int pado_query_noalloc(pado_index *h, uint64_t k, const uint32_t *a, const uint32_t *b, void *out);

/* ---------------------------------------------------------------------------
 * Accounting (no counterpart in the reference, which prints wall-clock
 * timers such as Total_labeling_time, pado_unw_unv_unp.h:1000-1116).
 * ------------------------------------------------------------------------- */
/* Kernel launches this library has made in the process so far. */
uint64_t pado_kernel_launches(void);

/* ---------------------------------------------------------------------------
 * Failure detection, for tests (no counterpart in the reference, which exits
 * on I/O errors and has no device code).  None of them faults or hangs a GPU.
 * ------------------------------------------------------------------------- */
/* Make the nth device allocation of this library from now on (1 = the next)
 * fail as if the device were out of memory: the call that makes it returns
 * PADO_E_NOMEM and releases what it had allocated.  0 disarms. */
int pado_debug_fail_alloc(uint64_t nth);
/* Device buffers of this library currently allocated (indexes, servers and
 * scratch in use); a failed call leaves it where it was. */
int64_t pado_debug_live_allocations(void);
/* Runs the labeling loops' bounded grid barrier in a cooperative launch of
 * `blocks` blocks (1..152) in which block `absent_block` never arrives
 * (absent_block >= blocks: all arrive), each waiting block giving up after
 * timeout_ns (at most 1 s).  Returns PADO_E_TIMEOUT when the wait ran out,
 * PADO_OK when the barrier completed; *blocks_returned counts the blocks that
 * returned (all of them, either way). */
int pado_selftest_barrier(uint32_t blocks, uint32_t absent_block, uint64_t timeout_ns, uint32_t *blocks_returned);

/* ---------------------------------------------------------------------------
 * Serving loop (continuous batching).  The reference answers pairs one call
 * at a time on the host (query_distance, pado_unw_unv_unp.h:1312-1445, driven
 * by query_distance.cpp:25-78); a server keeps label sets in HBM and
 * coalesces concurrently arriving requests of any size into mixed batches:
 * up to `slots` batches of at most max_batch_pairs pairs are in flight, each
 * answered by one kernel launch, and requests that arrive meanwhile fill the
 * next free slot.  Label sets are admitted and evicted (offloaded to
 * page-locked host memory, least recently used first) to keep the resident
 * bytes within hbm_budget_bytes and free HBM.  A request's results are the
 * same as pado_query's on its own, whatever else is in the batch.
 * ------------------------------------------------------------------------- */
typedef struct pado_server pado_server;

typedef struct pado_server_stats {
    uint64_t requests, batches, pairs, max_batch_pairs;
    uint64_t admissions, evictions;   /* label sets copied in / offloaded */
    uint64_t resident_bytes;
    uint32_t resident_indexes, pad;
} pado_server_stats;

int pado_server_create(uint64_t hbm_budget_bytes, uint32_t max_batch_pairs, uint32_t slots,
                       pado_server **out);
/* Registers an index (built or loaded, on the server's device).  The server
 * borrows the handle: it may offload and reload its device arrays, and the
 * caller must not use or free the handle until pado_server_destroy, which
 * leaves every registered handle resident again. */
int pado_server_add(pado_server *s, pado_index *h, uint32_t *index_id);
/* Queues k pairs for index index_id; a, b and out (uint8 unweighted, int16
 * weighted) must stay valid until the request completes.  Every ticket must
 * be waited for once. */
int pado_server_submit(pado_server *s, uint32_t index_id, uint64_t k, const uint32_t *a,
                       const uint32_t *b, void *out, uint64_t *ticket);
/* Waits (timeout_s < 0: forever) and reports the request's latency from
 * submission to completion. */
int pado_server_wait(pado_server *s, uint64_t ticket, double timeout_s, double *latency_s);
int pado_server_get_stats(pado_server *s, pado_server_stats *out);
/* Open-loop load replay: request i arrives arrival_s[i] seconds after the
 * start (non-decreasing), asks index_id[i] for the k[i] pairs at
 * a/b[pair_off[i] ...], and writes its results to out8 (unweighted) or out16
 * (weighted) at pair_off[i].  mode 0 submits through the serving loop; mode 1
 * answers each request on its own (copy in, one launch, copy back, in arrival
 * order) as the unbatched comparison.  latency_s[i] = completion time minus
 * scheduled arrival, so queueing behind a slow generator counts. */
int pado_server_replay(pado_server *s, uint64_t nreq, const double *arrival_s,
                       const uint32_t *index_id, const uint64_t *k, const uint64_t *pair_off,
                       const uint32_t *a, const uint32_t *b, uint8_t *out8, int16_t *out16,
                       uint32_t mode, double *latency_s);
void pado_server_destroy(pado_server *s);

/* Enable (1) or disable (0) per-kernel timing: while enabled every launch is
 * bracketed by CUDA events on its stream and hot kernels count their
 * algorithmic bytes.  Adds overhead; for profiling runs only.  2 times the
 * launches without the byte counters (whose atomics slow the hot kernels). */
int pado_profile(int enable);

/* Write the profile table as text lines "kernel launches total_ms bytes" into
 * buf (NUL-terminated, truncated to len); returns the size needed.  reset != 0
 * clears the table afterwards.  Synchronizes the device. */
size_t pado_profile_read(char *buf, size_t len, int reset);

#ifdef __cplusplus
}
#endif

#endif /* PADO_GPU_H_ */
