// ingest.cu -- from an edge-list text or an undirected edge list to the
// ranked CSR the labelers take, on the device.
//
// The reference prepares its graph on the host before labeling:
//   Graph(const char *) / WeightedGraph(const char *) (graph.h:95-117,
//     :262-290) read "head tail [weight]" lines, skipping lines that start
//     with '#' or '%';
//   Graph::construct (graph.h:125-153; weighted :292-309) stores both
//     directions of every edge, keeping duplicates and self-loops (a
//     self-loop appears twice in its vertex's list), n = max id + 1;
//   make_rank (graph.h:156-174) orders vertices by degree, descending;
//   id_transfer (graph.h:176-206; weighted :367-400) relabels every id to its
//     rank and sorts each list in descending (id, weight) order.
// make_rank breaks degree ties with rand(), which no two hosts reproduce, so
// ties are broken by ascending id here (as everywhere in this library).  An
// optional dedupe step drops self-loops and merges repeated undirected pairs
// (the first weight in input order wins), which is how benchmark generators
// clean an edge sample before handing it to the reference.
//
// Device mapping.  Text: newlines are located per 16-byte chunk (count, scan,
// write), every line is parsed by one thread, and the parsed edges are
// compacted in line order.  Graph: degrees are counted with atomics; the rank
// order is a counting sort of the n degrees on the host (O(n + max degree));
// each directed entry becomes one 64-bit key
//     rank(src) << (b + 8) | (2^b - 1 - rank(dst)) << 8 | (255 - weight)
// (b = bits of n), so ascending key order is "by source rank, then
// destination rank descending, then weight descending"; the keys are sorted
// by a stable LSD radix sort (8-bit digits, a warp per tile: per-tile digit
// counts, one exclusive scan over (digit, tile), then a scatter in which
// lanes holding the same digit are ranked with __match_any_sync), and the
// adjacency and weights are read back out of the sorted keys.  Offsets follow
// from the degrees in rank order.

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <memory>

#include "pado_internal.cuh"

namespace pado {
namespace {

constexpr unsigned FULLW = 0xffffffffu;
constexpr uint32_t RS_TILE = 2048;   // keys per warp tile in the radix sort
constexpr int RS_WARPS = 8;          // warps per block
constexpr uint32_t TEXT_CHUNK = 16;  // bytes per thread when locating newlines

// ---- scan -------------------------------------------------------------------

// Exclusive scan of a[0, L) in blocks of 1024: per-block scan, block totals in sums.
__global__ void __launch_bounds__(1024) scan_block_kernel(uint32_t *a, uint64_t L, uint32_t *sums)
{
    __shared__ uint32_t s[1024];
    const uint64_t i = (uint64_t)blockIdx.x * 1024 + threadIdx.x;
    const uint32_t x = i < L ? a[i] : 0u;
    s[threadIdx.x] = x;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        const uint32_t y = threadIdx.x >= (unsigned)o ? s[threadIdx.x - o] : 0u;
        __syncthreads();
        s[threadIdx.x] += y;
        __syncthreads();
    }
    if (i < L) a[i] = s[threadIdx.x] - x;
    if (threadIdx.x == 1023) sums[blockIdx.x] = s[1023];
}

// One block: exclusive scan of the nb block totals, 1024 at a time.
__global__ void __launch_bounds__(1024) scan_sums_kernel(uint32_t *sums, uint32_t nb)
{
    __shared__ uint32_t s[1024];
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (uint32_t c0 = 0; c0 < nb; c0 += 1024) {
        const uint32_t i = c0 + threadIdx.x;
        const uint32_t x = i < nb ? sums[i] : 0u;
        s[threadIdx.x] = x;
        __syncthreads();
        for (int o = 1; o < 1024; o <<= 1) {
            const uint32_t y = threadIdx.x >= (unsigned)o ? s[threadIdx.x - o] : 0u;
            __syncthreads();
            s[threadIdx.x] += y;
            __syncthreads();
        }
        if (i < nb) sums[i] = carry + s[threadIdx.x] - x;
        __syncthreads();
        if (threadIdx.x == 0) carry += s[1023];
        __syncthreads();
    }
}

__global__ void __launch_bounds__(1024) scan_add_kernel(uint32_t *a, uint64_t L, const uint32_t *sums)
{
    const uint64_t i = (uint64_t)blockIdx.x * 1024 + threadIdx.x;
    if (i < L) a[i] += sums[blockIdx.x];
}

// In place; the caller keeps the sums below 2^32.
void exclusive_scan(uint32_t *a, uint64_t L, cudaStream_t s)
{
    if (L == 0) return;
    const uint32_t nb = (uint32_t)((L + 1023) / 1024);
    DBuf<uint32_t> sums(nb);
    PADO_LAUNCH("scan_block_kernel", s, scan_block_kernel<<<nb, 1024, 0, s>>>(a, L, sums.p));
    PADO_LAUNCH("scan_sums_kernel", s, scan_sums_kernel<<<1, 1024, 0, s>>>(sums.p, nb));
    PADO_LAUNCH("scan_add_kernel", s, scan_add_kernel<<<nb, 1024, 0, s>>>(a, L, sums.p));
    PADO_CUDA(cudaStreamSynchronize(s));  // `sums` is freed on return
}

template <typename T>
T read_back(const T *d, cudaStream_t s)
{
    T x{};
    PADO_CUDA(cudaMemcpyAsync(&x, d, sizeof(T), cudaMemcpyDeviceToHost, s));
    PADO_CUDA(cudaStreamSynchronize(s));
    return x;
}

// ---- radix sort -------------------------------------------------------------

// counts[d * ntiles + tile] = keys of `tile` whose digit at `shift` is d.
__global__ void __launch_bounds__(RS_WARPS * 32) rs_hist_kernel(const uint64_t *keys, uint64_t L, uint32_t shift,
                                                                uint32_t ntiles, uint32_t *counts)
{
    __shared__ uint32_t h[RS_WARPS][256];
    const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t tile = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; tile < ntiles; tile += nw) {
        for (int d = lane; d < 256; d += 32) h[wl][d] = 0;
        __syncwarp();
        const uint64_t t0 = (uint64_t)tile * RS_TILE, t1 = min(L, t0 + RS_TILE);
        for (uint64_t i = t0 + lane; i < t1; i += 32) atomicAdd(&h[wl][(keys[i] >> shift) & 255u], 1u);
        __syncwarp();
        for (int d = lane; d < 256; d += 32) counts[(uint64_t)d * ntiles + tile] = h[wl][d];
        __syncwarp();
    }
}

// Stable scatter: a tile's keys in order, 32 at a time; lanes holding the
// same digit are ranked by lane order.
__global__ void __launch_bounds__(RS_WARPS * 32) rs_scatter_kernel(const uint64_t *in, uint64_t *out, uint64_t L,
                                                                   uint32_t shift, uint32_t ntiles,
                                                                   const uint32_t *offsets)
{
    __shared__ uint32_t base[RS_WARPS][256];
    const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    const uint32_t below = (1u << lane) - 1u;
    for (uint32_t tile = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; tile < ntiles; tile += nw) {
        for (int d = lane; d < 256; d += 32) base[wl][d] = offsets[(uint64_t)d * ntiles + tile];
        __syncwarp();
        const uint64_t t0 = (uint64_t)tile * RS_TILE, t1 = min(L, t0 + RS_TILE);
        for (uint64_t c0 = t0; c0 < t1; c0 += 32) {
            const uint64_t i = c0 + lane;
            const bool live = i < t1;
            const uint64_t key = live ? in[i] : 0ull;
            const uint32_t dig = live ? (uint32_t)((key >> shift) & 255u) : 256u + lane;  // idle lanes stand alone
            const uint32_t peers = __match_any_sync(FULLW, dig);
            if (live) out[base[wl][dig] + __popc(peers & below)] = key;
            __syncwarp();
            if (live && (peers & below) == 0) base[wl][dig] += __popc(peers);
            __syncwarp();
        }
    }
}

// Sorts keys[0, L) ascending on bits [lo, hi), stably; the result is in `keys`.
void radix_sort(DBuf<uint64_t> &keys, uint64_t L, uint32_t lo, uint32_t hi, cudaStream_t s)
{
    if (L < 2 || lo >= hi) return;
    const uint32_t ntiles = (uint32_t)((L + RS_TILE - 1) / RS_TILE);
    DBuf<uint64_t> tmp(L);
    DBuf<uint32_t> counts((uint64_t)256 * ntiles);
    const unsigned grid = grid_for((uint64_t)ntiles * 32, RS_WARPS * 32, 152u * 16u);
    uint64_t *src = keys.p, *dst = tmp.p;
    for (uint32_t shift = lo; shift < hi; shift += 8) {
        PADO_LAUNCH("rs_hist_kernel", s,
                    rs_hist_kernel<<<grid, RS_WARPS * 32, 0, s>>>(src, L, shift, ntiles, counts.p));
        exclusive_scan(counts.p, (uint64_t)256 * ntiles, s);
        PADO_LAUNCH("rs_scatter_kernel", s,
                    rs_scatter_kernel<<<grid, RS_WARPS * 32, 0, s>>>(src, dst, L, shift, ntiles, counts.p));
        std::swap(src, dst);
    }
    if (src != keys.p) PADO_CUDA(cudaMemcpyAsync(keys.p, src, L * 8, cudaMemcpyDeviceToDevice, s));
    PADO_CUDA(cudaStreamSynchronize(s));  // `tmp` and `counts` are freed on return
}

// ---- edge list -> ranked CSR ------------------------------------------------

__global__ void __launch_bounds__(256) max_id_kernel(const uint32_t *u, const uint32_t *v, uint64_t m, uint32_t *mx)
{
    uint32_t x = 0;
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < m; e += (uint64_t)gridDim.x * blockDim.x)
        x = max(x, max(u[e], v[e]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x = max(x, __shfl_xor_sync(FULLW, x, o));
    if ((threadIdx.x & 31) == 0) atomicMax(mx, x);
}

// One key per undirected edge for the dedupe sort: (min, max) over original
// ids with the weight riding in the low byte (not sorted on, so a stable sort
// keeps repeated pairs in input order); self-loops become ~0 and sort last.
__global__ void __launch_bounds__(256) canon_key_kernel(const uint32_t *u, const uint32_t *v, const uint8_t *w,
                                                        uint64_t m, uint32_t n, uint32_t bits, uint64_t *keys,
                                                        uint32_t *bad)
{
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < m; e += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t a = u[e], b = v[e];
        if (a >= n || b >= n) {
            atomicOr(bad, 1u);
            keys[e] = ~0ull;
            continue;
        }
        keys[e] = a == b ? ~0ull
                         : (uint64_t)min(a, b) << (bits + 8) | (uint64_t)max(a, b) << 8 | (w ? w[e] : 0u);
    }
}

__device__ __forceinline__ uint32_t first_of_run(const uint64_t *keys, uint64_t i)
{
    const uint64_t k = keys[i];
    return k != ~0ull && (i == 0 || (keys[i - 1] >> 8) != (k >> 8)) ? 1u : 0u;
}

__global__ void __launch_bounds__(256) unique_flag_kernel(const uint64_t *keys, uint64_t m, uint32_t *pos)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i <= m; i += (uint64_t)gridDim.x * blockDim.x)
        pos[i] = i < m ? first_of_run(keys, i) : 0u;
}

__global__ void __launch_bounds__(256) unique_scatter_kernel(const uint64_t *keys, uint64_t m, uint32_t bits,
                                                             const uint32_t *pos, uint32_t *u, uint32_t *v,
                                                             uint8_t *w)
{
    const uint64_t dmask = (1ull << bits) - 1;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m; i += (uint64_t)gridDim.x * blockDim.x) {
        if (!first_of_run(keys, i)) continue;
        const uint64_t k = keys[i];
        const uint32_t o = pos[i];
        u[o] = (uint32_t)(k >> (bits + 8));
        v[o] = (uint32_t)((k >> 8) & dmask);
        if (w) w[o] = (uint8_t)(k & 255u);
    }
}

__global__ void __launch_bounds__(256) degree_kernel(const uint32_t *u, const uint32_t *v, uint64_t m, uint32_t n,
                                                     uint32_t *deg, uint32_t *bad)
{
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < m; e += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t a = u[e], b = v[e];
        if (a >= n || b >= n) {
            atomicOr(bad, 1u);
            continue;
        }
        atomicAdd(&deg[a], 1u);
        atomicAdd(&deg[b], 1u);
    }
}

// Both directions of edge e as sort keys (see the file comment).
__global__ void __launch_bounds__(256) entry_key_kernel(const uint32_t *u, const uint32_t *v, const uint8_t *w,
                                                        uint64_t m, const uint32_t *rank, uint32_t bits,
                                                        uint64_t *keys)
{
    const uint64_t dmask = (1ull << bits) - 1;
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < m; e += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t ra = rank[u[e]], rb = rank[v[e]];
        const uint64_t lw = 255u - (w ? w[e] : 0u);
        keys[2 * e] = ra << (bits + 8) | (dmask - rb) << 8 | lw;
        keys[2 * e + 1] = rb << (bits + 8) | (dmask - ra) << 8 | lw;
    }
}

__global__ void __launch_bounds__(256) extract_kernel(const uint64_t *keys, uint64_t L, uint32_t bits, uint32_t *adj,
                                                      uint8_t *w)
{
    const uint64_t dmask = (1ull << bits) - 1;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < L; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t k = keys[i];
        adj[i] = (uint32_t)(dmask - ((k >> 8) & dmask));
        if (w) w[i] = (uint8_t)(255u - (uint32_t)(k & 255u));
    }
}

uint32_t id_bits(uint32_t n)
{
    uint32_t b = 1;
    while (b < 32 && (1ull << b) < n) ++b;
    return b;
}

// ---- text -------------------------------------------------------------------

__device__ __forceinline__ bool is_blank(uint8_t c)
{
    return c == ' ' || c == '\t' || c == '\r' || c == '\v' || c == '\f';
}

// Unsigned decimal after optional blanks and an optional '+', as an
// istream >> into uint32_t reads it; false when no digit follows.  A value
// above 2^32 - 1 sets `over` (the stream would fail, storing the maximum).
__device__ bool parse_u32(const uint8_t *t, uint32_t &i, uint32_t end, uint32_t &val, bool &over)
{
    while (i < end && is_blank(t[i])) ++i;
    if (i < end && t[i] == '+') ++i;
    if (i >= end || t[i] < '0' || t[i] > '9') return false;
    uint64_t x = 0;
    over = false;
    while (i < end && t[i] >= '0' && t[i] <= '9') {
        x = x * 10 + (t[i] - '0');
        if (x > 0xffffffffull) {
            over = true;
            x = 0xffffffffull;
        }
        ++i;
    }
    val = (uint32_t)x;
    return true;
}

__global__ void __launch_bounds__(256) nl_count_kernel(const uint8_t *t, uint32_t bytes, uint32_t nchunks,
                                                       uint32_t *cnt)
{
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < nchunks; c += gridDim.x * blockDim.x) {
        const uint32_t b0 = c * TEXT_CHUNK, b1 = min(bytes, b0 + TEXT_CHUNK);
        uint32_t k = 0;
        for (uint32_t i = b0; i < b1; ++i) k += t[i] == '\n';
        cnt[c] = k;
    }
}

__global__ void __launch_bounds__(256) nl_write_kernel(const uint8_t *t, uint32_t bytes, uint32_t nchunks,
                                                       const uint32_t *pos, uint32_t *nl)
{
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < nchunks; c += gridDim.x * blockDim.x) {
        const uint32_t b0 = c * TEXT_CHUNK, b1 = min(bytes, b0 + TEXT_CHUNK);
        uint32_t o = pos[c];
        for (uint32_t i = b0; i < b1; ++i)
            if (t[i] == '\n') nl[o++] = i;
    }
}

// Line k spans [nl[k-1] + 1, nl[k]) (line 0 starts at 0).  ok[k] = 1 when it
// holds an edge: not empty, not a '#' / '%' comment, two ids that parse.  A
// missing or unparsable weight is 0; weights are cast to uint8.  ok[lines] = 0
// closes the array for the scan.
__global__ void __launch_bounds__(256) parse_line_kernel(const uint8_t *t, const uint32_t *nl, uint32_t lines,
                                                         int weighted, uint32_t *lu, uint32_t *lv, uint8_t *lw,
                                                         uint32_t *ok)
{
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k <= lines; k += gridDim.x * blockDim.x) {
        if (k == lines) {
            ok[k] = 0;
            continue;
        }
        uint32_t i = k ? nl[k - 1] + 1 : 0;
        const uint32_t end = nl[k];
        uint32_t a = 0, b = 0, w = 0;
        bool oa = false, ob = false, ow = false;
        bool good = i < end && t[i] != '#' && t[i] != '%';
        good = good && parse_u32(t, i, end, a, oa) && !oa;
        good = good && parse_u32(t, i, end, b, ob) && !ob;
        if (good && weighted && !parse_u32(t, i, end, w, ow)) w = 0;
        ok[k] = good;
        lu[k] = a;
        lv[k] = b;
        if (weighted) lw[k] = (uint8_t)w;
    }
}

__global__ void __launch_bounds__(256) edge_compact_kernel(const uint32_t *lu, const uint32_t *lv, const uint8_t *lw,
                                                           const uint32_t *pos, uint32_t lines, uint32_t *u,
                                                           uint32_t *v, uint8_t *w)
{
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < lines; k += gridDim.x * blockDim.x) {
        const uint32_t o = pos[k];
        if (pos[k + 1] == o) continue;
        u[o] = lu[k];
        v[o] = lv[k];
        if (w) w[o] = lw[k];
    }
}

}  // namespace

IngestResult ingest_edges(uint64_t m, const uint32_t *du, const uint32_t *dv, const uint8_t *dw, uint32_t n,
                          bool dedupe, cudaStream_t s, uint32_t *adj_out, uint8_t *w_out)
{
    IngestResult r;
    PADO_CHECK(m < (1ull << 31), PADO_E_ARG, "at most 2^31 - 1 edges (2^32 - 2 adjacency entries)");
    DBuf<uint32_t> scal(1);
    if (n == 0 && m) {  // n = max id + 1, as Graph::construct sets it
        scal.fill_bytes(0, s);
        PADO_LAUNCH("max_id_kernel", s, max_id_kernel<<<grid_for(m, 256), 256, 0, s>>>(du, dv, m, scal.p));
        const uint32_t mx = read_back(scal.p, s);
        PADO_CHECK(mx < 0xffffffffu, PADO_E_ARG, "vertex id 2^32 - 1 is reserved");
        n = mx + 1;
    }
    const uint32_t bits = id_bits(n);
    PADO_CHECK(bits <= 28, PADO_E_ARG, "graph ingest supports fewer than 2^28 vertices");
    r.n = n;

    // optional dedupe over original ids
    DBuf<uint32_t> u2, v2;
    DBuf<uint8_t> w2;
    if (dedupe && m) {
        DBuf<uint64_t> ck(m);
        scal.fill_bytes(0, s);
        PADO_LAUNCH("canon_key_kernel", s,
                    canon_key_kernel<<<grid_for(m, 256), 256, 0, s>>>(du, dv, dw, m, n, bits, ck.p, scal.p));
        PADO_CHECK(read_back(scal.p, s) == 0, PADO_E_ARG, "edge endpoint out of range");
        radix_sort(ck, m, 8, 2 * bits + 8, s);
        DBuf<uint32_t> pos(m + 1);
        PADO_LAUNCH("unique_flag_kernel", s, unique_flag_kernel<<<grid_for(m + 1, 256), 256, 0, s>>>(ck.p, m, pos.p));
        exclusive_scan(pos.p, m + 1, s);
        const uint32_t mu = read_back(pos.p + m, s);
        u2.alloc(std::max<uint32_t>(mu, 1));
        v2.alloc(std::max<uint32_t>(mu, 1));
        if (dw) w2.alloc(std::max<uint32_t>(mu, 1));
        PADO_LAUNCH("unique_scatter_kernel", s,
                    unique_scatter_kernel<<<grid_for(m, 256), 256, 0, s>>>(ck.p, m, bits, pos.p, u2.p, v2.p,
                                                                         dw ? w2.p : nullptr));
        PADO_CUDA(cudaStreamSynchronize(s));
        du = u2.p;
        dv = v2.p;
        dw = dw ? w2.p : nullptr;
        m = mu;
    }

    // degrees -> rank (degree descending, ties by ascending id) -> offsets
    DBuf<uint32_t> deg(std::max<uint32_t>(n, 1));
    deg.fill_bytes(0, s);
    scal.fill_bytes(0, s);
    if (m)
        PADO_LAUNCH("degree_kernel", s, degree_kernel<<<grid_for(m, 256), 256, 0, s>>>(du, dv, m, n, deg.p, scal.p));
    std::vector<uint32_t> hdeg(n);
    deg.download(hdeg.data(), n, s);
    PADO_CHECK(read_back(scal.p, s) == 0, PADO_E_ARG, "edge endpoint out of range");
    uint32_t maxdeg = 0;
    for (uint32_t x = 0; x < n; ++x) maxdeg = std::max(maxdeg, hdeg[x]);
    std::vector<uint32_t> start((uint64_t)maxdeg + 2, 0);
    for (uint32_t x = 0; x < n; ++x) ++start[maxdeg - hdeg[x] + 1];
    for (uint64_t k = 1; k < start.size(); ++k) start[k] += start[k - 1];
    r.rank.resize(n);
    for (uint32_t x = 0; x < n; ++x) r.rank[x] = start[maxdeg - hdeg[x]]++;
    r.off.assign((uint64_t)n + 1, 0);
    for (uint32_t x = 0; x < n; ++x) r.off[r.rank[x] + 1] = hdeg[x];
    for (uint32_t k = 0; k < n; ++k) r.off[k + 1] += r.off[k];

    // keys -> sort -> adjacency (and weights)
    const uint64_t L = 2 * m;
    r.m = L;
    if (!adj_out) {
        r.adj.alloc(std::max<uint64_t>(L, 1));
        adj_out = r.adj.p;
    }
    if (dw && !w_out) {
        r.w.alloc(std::max<uint64_t>(L, 1));
        w_out = r.w.p;
    }
    if (L) {
        DBuf<uint32_t> drank(n);
        drank.upload(r.rank.data(), n, s);
        DBuf<uint64_t> keys(L);
        PADO_LAUNCH("entry_key_kernel", s,
                    entry_key_kernel<<<grid_for(m, 256), 256, 0, s>>>(du, dv, dw, m, drank.p, bits, keys.p));
        // after dedupe no (src, dst) pair repeats, so the weight byte needs no pass
        radix_sort(keys, L, dw && !dedupe ? 0u : 8u, 2 * bits + 8, s);
        PADO_LAUNCH("extract_kernel", s,
                    extract_kernel<<<grid_for(L, 256), 256, 0, s>>>(keys.p, L, bits, adj_out, dw ? w_out : nullptr));
        PADO_CUDA(cudaStreamSynchronize(s));
    }
    return r;
}

// ---- text parsing -----------------------------------------------------------

EdgeTextParser::EdgeTextParser(bool weighted, uint64_t max_edges, cudaStream_t s) : weighted_(weighted), s_(s)
{
    PADO_CHECK(max_edges < (1ull << 32), PADO_E_ARG, "edge capacity above 2^32 - 1");
    u.alloc(std::max<uint64_t>(max_edges, 1));
    v.alloc(std::max<uint64_t>(max_edges, 1));
    if (weighted) w.alloc(std::max<uint64_t>(max_edges, 1));
    cap_ = max_edges;
}

void EdgeTextParser::feed(const char *text, uint64_t bytes)
{
    if (bytes == 0) return;
    const bool terminated = text[bytes - 1] == '\n';
    const uint64_t tb = bytes + (terminated ? 0 : 1);  // a last line without '\n' gets one
    PADO_CHECK(tb < (1ull << 32) - TEXT_CHUNK, PADO_E_ARG, "text pieces must stay below 4 GiB");
    if (text_.n < tb) text_.alloc(tb);
    PADO_CUDA(cudaMemcpyAsync(text_.p, text, bytes, cudaMemcpyHostToDevice, s_));
    if (!terminated) PADO_CUDA(cudaMemsetAsync(text_.p + bytes, '\n', 1, s_));
    const uint32_t tbytes = (uint32_t)tb;
    const uint32_t nchunks = (tbytes + TEXT_CHUNK - 1) / TEXT_CHUNK;
    if (cnt_.n < (uint64_t)nchunks + 1) cnt_.alloc((uint64_t)nchunks + 1);
    PADO_LAUNCH("nl_count_kernel", s_,
                nl_count_kernel<<<grid_for(nchunks, 256), 256, 0, s_>>>(text_.p, tbytes, nchunks, cnt_.p));
    PADO_CUDA(cudaMemsetAsync(cnt_.p + nchunks, 0, 4, s_));
    exclusive_scan(cnt_.p, (uint64_t)nchunks + 1, s_);
    const uint32_t lines = read_back(cnt_.p + nchunks, s_);  // >= 1: the text ends with '\n'
    if (nl_.n < lines) nl_.alloc(lines);
    if (ok_.n < (uint64_t)lines + 1) {
        ok_.alloc((uint64_t)lines + 1);
        lu_.alloc(lines);
        lv_.alloc(lines);
        if (weighted_) lw_.alloc(lines);
    }
    PADO_LAUNCH("nl_write_kernel", s_,
                nl_write_kernel<<<grid_for(nchunks, 256), 256, 0, s_>>>(text_.p, tbytes, nchunks, cnt_.p, nl_.p));
    PADO_LAUNCH("parse_line_kernel", s_,
                parse_line_kernel<<<grid_for((uint64_t)lines + 1, 256), 256, 0, s_>>>(
                    text_.p, nl_.p, lines, weighted_, lu_.p, lv_.p, weighted_ ? lw_.p : nullptr, ok_.p));
    exclusive_scan(ok_.p, (uint64_t)lines + 1, s_);
    const uint32_t got = read_back(ok_.p + lines, s_);
    PADO_CHECK(m + got <= cap_, PADO_E_ARG, "more edges than the parser's capacity");
    if (got)
        PADO_LAUNCH("edge_compact_kernel", s_,
                    edge_compact_kernel<<<grid_for(lines, 256), 256, 0, s_>>>(
                        lu_.p, lv_.p, weighted_ ? lw_.p : nullptr, ok_.p, lines, u.p + m, v.p + m,
                        weighted_ ? w.p + m : nullptr));
    PADO_CUDA(cudaStreamSynchronize(s_));
    m += got;
}

uint64_t text_piece_bytes(uint64_t dflt)
{
    // PADO_DEBUG_TEXT_PIECE (tests only) makes pieces tiny, so that lines
    // cut at piece ends are exercised on small files
    const char *e = std::getenv("PADO_DEBUG_TEXT_PIECE");
    const uint64_t d = e ? std::strtoull(e, nullptr, 10) : 0;
    return d ? d : dflt;
}

uint64_t edge_bound_for_text(uint64_t bytes)
{
    // a line holding an edge has at least "a b" and its line end: 4 bytes
    // (the last one may lack its '\n')
    return bytes / 4 + 1;
}

EdgeTextParser read_edge_file(const char *path, bool weighted, cudaStream_t s)
{
    PADO_CHECK(path != nullptr, PADO_E_ARG, "null path");
    std::unique_ptr<FILE, int (*)(FILE *)> f(std::fopen(path, "rb"), &std::fclose);
    PADO_CHECK(f != nullptr, PADO_E_IO, std::string("cannot open file ") + path);
    PADO_CHECK(std::fseek(f.get(), 0, SEEK_END) == 0, PADO_E_IO, "cannot seek");
    const long size = std::ftell(f.get());
    PADO_CHECK(size >= 0, PADO_E_IO, "cannot size file");
    std::rewind(f.get());
    EdgeTextParser p(weighted, std::min<uint64_t>(edge_bound_for_text((uint64_t)size), (1ull << 32) - 1), s);
    // read in pieces that end at a line end; the unfinished tail of one
    // piece opens the next
    const uint64_t piece = std::min<uint64_t>(std::max<uint64_t>((uint64_t)size, 1), text_piece_bytes(256ull << 20));
    HBuf<char> buf(piece);
    uint64_t have = 0;
    for (;;) {
        const size_t got = std::fread(buf.p + have, 1, piece - have, f.get());
        PADO_CHECK(!std::ferror(f.get()), PADO_E_IO, "read error");
        have += got;
        const bool eof = std::feof(f.get()) || got == 0;
        if (have == 0) break;
        uint64_t cut = have;
        if (!eof) {
            while (cut > 0 && buf.p[cut - 1] != '\n') --cut;
            PADO_CHECK(cut > 0, PADO_E_ARG, "a line longer than the read piece (256 MiB)");
        }
        p.feed(buf.p, cut);
        std::memmove(buf.p, buf.p + cut, have - cut);
        have -= cut;
        if (eof) break;
    }
    return p;
}

}  // namespace pado
