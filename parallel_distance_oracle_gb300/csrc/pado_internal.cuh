// pado_internal.cuh -- device views and host launchers shared by the .cu files.
#pragma once

#include "pado_common.cuh"

namespace pado {

// Read-only view of a finished label set, indexed by RANK.  Queries map their
// original-id endpoints through `rank` (identity when null).
struct IndexView {
    uint32_t n = 0;
    uint32_t K = 0;             // bit-parallel roots (unweighted only)
    const uint32_t *rank = nullptr;
    const uint64_t *off = nullptr;   // n + 1
    const uint32_t *hub = nullptr;   // rank-id hubs, ascending per vertex
    const uint8_t *dist8 = nullptr;  // unweighted distances
    const int16_t *dist16 = nullptr; // weighted distances
    const uint8_t *bpd = nullptr;    // n * K
    const uint64_t *bps = nullptr;   // n * K * 2  (S^-1, S^0)
    unsigned long long *work = nullptr;  // profiling counters
};

// query.cu
void launch_query_unw(const IndexView &v, uint64_t k, const uint32_t *a, const uint32_t *b, uint8_t *out,
                      cudaStream_t s);
void launch_query_w(const IndexView &v, uint64_t k, const uint32_t *a, const uint32_t *b, int16_t *out,
                    cudaStream_t s);

// A graph already relabeled by rank, neighbour lists in descending id order
// (Graph::id_transfer, graph.h:176-206), on the device.
struct DevGraph {
    uint32_t n = 0;
    uint64_t m = 0;              // directed entries
    DBuf<uint32_t> off;          // n + 1 (m must fit 32 bits)
    DBuf<uint32_t> adj;          // m
    DBuf<uint8_t> w;             // m (weighted only)
};

// Host-side relabel + sort (graph.h:176-206 semantics).
struct HostGraph {
    uint32_t n = 0;
    std::vector<uint32_t> off;
    std::vector<uint32_t> adj;
    std::vector<uint8_t> w;
    // When the caller's arrays are already in this form (ids are ranks, lists
    // descending) they are used in place: the views point at them and adj / w
    // stay empty.  Such a graph lives no longer than the call that made it.
    const uint32_t *adj_view = nullptr;
    const uint8_t *w_view = nullptr;
    const uint32_t *adjp() const { return adj_view ? adj_view : adj.data(); }
    const uint8_t *wp() const { return w_view ? w_view : w.data(); }
    uint64_t m() const { return off.empty() ? 0 : off.back(); }
};
HostGraph relabel_host(uint32_t n, const uint64_t *off, const uint32_t *adj, const uint8_t *w,
                       const uint32_t *rank);

// bp.cu: bit-parallel labeling (pado_unw_unv_unp.h:268-384).  `used` (host,
// n) is updated with the roots and their selected neighbours.  Writes
// bpd[n*K], bps[n*K*2] on the device.
struct BpResult {
    float ms = 0.f;
    uint32_t levels = 0;
};
BpResult bp_label(const HostGraph &hg, const DevGraph &g, uint32_t K, std::vector<uint8_t> &used,
                  uint8_t *d_bpd, uint64_t *d_bps, cudaStream_t s);

// The two halves of bp_label.  bp_select appends, for BP slot i, the root and
// selected neighbours of the graph occupying ids [lo, hi) to seeds[i] and
// marks them used; called once per graph of a union it gives every graph its
// own slot roots.  bp_run labels all slots over the (union) graph: graphs are
// disjoint, so one BFS per slot serves every graph's root at once.
struct BpSeed {
    uint32_t v, lvl;
    uint64_t bits;
};
void bp_select(const HostGraph &hg, uint32_t lo, uint32_t hi, uint32_t K, std::vector<uint8_t> &used,
               std::vector<std::vector<BpSeed>> &seeds);
BpResult bp_run(const HostGraph &hg, const DevGraph &g, uint32_t K, const std::vector<std::vector<BpSeed>> &seeds,
                uint8_t *d_bpd, uint64_t *d_bps, cudaStream_t s);

// Final label store produced by a labeler (rank-indexed, sorted by hub).
struct LabelStore {
    DBuf<uint64_t> off;
    DBuf<uint32_t> hub;
    DBuf<uint8_t> dist8;
    DBuf<int16_t> dist16;
    uint64_t total = 0;
};

struct LabelRun {
    float ms = 0.f;          // device time of the batch labeling
    uint32_t levels = 0;
    uint32_t batches = 0;
};

// unw.cu: batched pruned BFS labeling (pado_unw_unv_unp.h:425-1118).
LabelRun unw_label(const DevGraph &g, uint32_t K, uint32_t B, const std::vector<uint8_t> &used,
                   const uint8_t *d_bpd, const uint64_t *d_bps, LabelStore &out, cudaStream_t s);

// unw_many.cu: the same labeling for many independent graphs at once.  `g` is
// the disjoint union, graph i owning ids [gbase[i], gbase[i+1]); every graph
// runs its own batch sequence, all advancing one level per step of one
// persistent launch.  `out` is indexed by union id with graph-local hubs.
LabelRun unw_label_many(const DevGraph &g, const std::vector<uint32_t> &gbase, uint32_t K, uint32_t B,
                        const std::vector<uint8_t> &used, const uint8_t *d_bpd, const uint64_t *d_bps,
                        LabelStore &out, cudaStream_t s);

// weighted.cu: batched pruned relaxation (pado_weighted_unv_unp.h:281-1526).
LabelRun w_label(const DevGraph &g, uint32_t B, LabelStore &out, cudaStream_t s);

// ingest.cu: an undirected edge list (device arrays, original ids) to the
// ranked CSR: Graph::construct + make_rank + id_transfer (graph.h:125-206)
// with degree ties broken by ascending id.  n = 0 takes max id + 1; dedupe
// drops self-loops and merges repeated pairs (first weight wins) first.  The
// adjacency (and weights) go to adj_out / w_out (device, room for 2m) when
// given, else into the result's own buffers.
struct IngestResult {  // all on the device
    uint32_t n = 0;
    uint64_t m = 0;                  // directed entries
    DBuf<uint32_t> rank;             // n: original id -> rank
    DBuf<uint32_t> off;              // n + 1, rank-indexed
    DBuf<uint32_t> adj;              // m: rank ids, every list descending (id, weight)
    DBuf<uint8_t> w;                 // m (weighted only)
};
IngestResult ingest_edges(uint64_t m, const uint32_t *d_u, const uint32_t *d_v, const uint8_t *d_w, uint32_t n,
                          bool dedupe, cudaStream_t s, uint32_t *adj_out = nullptr, uint8_t *w_out = nullptr);
// CSR input (host arrays: off[n+1] with off[n] < 2^32, adj, optional
// weights, optional rank over original ids) to the device graph the labelers
// take, on the device: the offsets, ids and rank are checked there; a ranked
// CSR whose lists are already descending is used as uploaded, anything else
// is relabeled and sorted by the entry sort (Graph::id_transfer,
// graph.h:176-206).  With rank, *rank_out receives it on the device.
DevGraph prepare_csr(uint32_t n, const uint64_t *off, const uint32_t *adj, const uint8_t *w, const uint32_t *rank,
                     cudaStream_t s, DBuf<uint32_t> *rank_out);
// Graph reductions of the reference's conversion tools (ingest.cu), over an
// edge list in device memory with ids < n: per-vertex flags (n bytes), the
// indices of the surviving edges in input order (room for m), and for the
// equivalence reduction the new ids (n entries).  Stream-ordered; return when
// the outputs are written.
struct ReduceResult {
    uint32_t n = 0;     // vertices
    uint64_t kept = 0;  // surviving edges
    uint32_t n_out = 0; // equivalence: 1 + the largest new id on a kept edge
};
ReduceResult reduce_degree1(uint64_t m, const uint32_t *du, const uint32_t *dv, uint32_t n, cudaStream_t s,
                            uint8_t *deleted, uint64_t *kept);
ReduceResult reduce_equivalent(uint64_t m, const uint32_t *du, const uint32_t *dv, uint32_t n, cudaStream_t s,
                               uint8_t *redundant, uint32_t *new_id, uint64_t *kept);

// Trims the ingest scratch pool of the current device to keep_bytes.
void release_scratch(uint64_t keep_bytes);
// b[i] = a[i] for i < n (device arrays, stream-ordered).
void widen_u32(const uint32_t *a, uint64_t n, uint64_t *b, cudaStream_t s);

// Edge-list text ("head tail [weight]" lines, graph.h:95-117, :262-290)
// parsed on the device into u / v / w (device, m edges so far, in line
// order).  feed() takes whole lines; every call completes before returning.
class EdgeTextParser {
public:
    EdgeTextParser(bool weighted, uint64_t max_edges, cudaStream_t s);
    void feed(const char *text, uint64_t bytes);
    uint64_t m = 0;
    DBuf<uint32_t> u, v;
    DBuf<uint8_t> w;

private:
    bool weighted_;
    cudaStream_t s_;
    uint64_t cap_ = 0;
    DBuf<uint8_t> text_;
    DBuf<uint32_t> cnt_, nl_, ok_, lu_, lv_;
    DBuf<uint8_t> lw_;
};
uint64_t edge_bound_for_text(uint64_t bytes);
uint64_t text_piece_bytes(uint64_t dflt);
EdgeTextParser read_edge_file(const char *path, bool weighted, cudaStream_t s);

// hostcopy.cu: the device alias of page-locked host memory (null for any other
// pointer), and copies between host and device memory that the SMs carry out
// when the host side is page-locked (the copy engines otherwise), enqueued on s.
void *mapped_host(const void *p);
void download_bytes(void *h, const void *d, uint64_t bytes, cudaStream_t s);
void upload_bytes(void *d, const void *h, uint64_t bytes, cudaStream_t s);

// capi.cu: the calling thread's last-error message, and read-only access to
// an index handle, for entry points defined in other files.
int set_error(int code, const std::string &msg);
IndexView index_view(const pado_index *h);
uint32_t index_kind(const pado_index *h);
int index_device(const pado_index *h);

// Residency of an index's device arrays, for the serving loop's admission
// control: offload copies them to page-locked host memory and frees the
// device copies; reload brings them back (both complete before returning).
// Queries on an offloaded index fail with PADO_E_STATE.
bool index_resident(const pado_index *h);
uint64_t index_device_bytes(const pado_index *h);
void index_offload(pado_index *h, cudaStream_t s);
void index_reload(pado_index *h, cudaStream_t s);

}  // namespace pado
