// ingest.cu -- from an edge-list text or an undirected edge list to the
// ranked CSR the labelers take, on the device; and the reference's two
// graph-reduction tools over the same edge lists (the last section).
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
// compacted in line order.  Graph: degrees are counted in per-block shared
// tables with a global fallback; the vertex order is a stable radix sort of (max degree - degree,
// id) keys, so ties keep ascending ids; offsets are the scan of the degrees in
// rank order.  Each directed entry becomes one 64-bit key
//     rank(src) << (b + 8) | (2^b - 1 - rank(dst)) << 8 | (255 - weight)
// (b = bits of n), so ascending key order is "by source rank, then
// destination rank descending, then weight descending"; the keys are sorted
// by the same stable LSD radix sort and the adjacency and weights are read
// back out of them.
//
// The radix sort: 8-bit digits, tiles of 4096 keys, three kernels per digit
// -- per-tile digit counts, one exclusive scan over the (digit, tile) matrix,
// and a scatter in which each block ranks its tile's keys by digit (lanes
// holding the same digit ranked with __match_any_sync, warps by a prefix over
// the block), reorders the tile in shared memory and writes every digit's
// run to its global position in coalesced stores.

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <optional>

#include "pado_internal.cuh"

namespace pado {
namespace {

constexpr unsigned FULLW = 0xffffffffu;
constexpr int RS_THREADS = 256;                  // radix sort block
constexpr int RS_PER = 16;                       // keys per thread
constexpr uint32_t RS_TILE = RS_THREADS * RS_PER;  // 4096 keys per tile
constexpr uint32_t TEXT_CHUNK = 16;              // bytes per thread when locating newlines

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

uint64_t scan_sums_needed(uint64_t L) { return std::max<uint64_t>((L + 1023) / 1024, 1); }

// In place, stream-ordered; `sums` holds scan_sums_needed(L) entries; the
// caller keeps the total below 2^32.
void exclusive_scan(uint32_t *a, uint64_t L, uint32_t *sums, cudaStream_t s)
{
    if (L == 0) return;
    const uint32_t nb = (uint32_t)((L + 1023) / 1024);
    PADO_LAUNCH("scan_block_kernel", s, scan_block_kernel<<<nb, 1024, 0, s>>>(a, L, sums));
    PADO_LAUNCH("scan_sums_kernel", s, scan_sums_kernel<<<1, 1024, 0, s>>>(sums, nb));
    PADO_LAUNCH("scan_add_kernel", s, scan_add_kernel<<<nb, 1024, 0, s>>>(a, L, sums));
}

// Same with its own block-sum buffer; completes before returning.
void exclusive_scan(uint32_t *a, uint64_t L, cudaStream_t s)
{
    DBuf<uint32_t> sums(scan_sums_needed(L));
    exclusive_scan(a, L, sums.p, s);
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

// Scratch comes from a memory pool of this library's own (one per device),
// allocated and freed in stream order: a call's buffers are reused by its
// later steps without device-wide synchronisation, and up to
// the caller's chosen amount stays reserved for the next call
// (release_scratch trims it).
cudaMemPool_t scratch_pool()
{
    static std::mutex mu;
    static std::map<int, cudaMemPool_t> pools;
    int dev = 0;
    PADO_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(mu);
    auto it = pools.find(dev);
    if (it != pools.end()) return it->second;
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t pool;
    PADO_CUDA(cudaMemPoolCreate(&pool, &props));
    uint64_t keep = ~0ull;  // nothing is returned implicitly at synchronisation points
    PADO_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
    pools[dev] = pool;
    return pool;
}

template <typename T>
struct PBuf {
    T *p = nullptr;
    size_t n = 0;
    cudaStream_t s = nullptr;
    PBuf(size_t count, cudaStream_t st) : n(count), s(st)
    {
        if (count) {
            alloc_point();
            PADO_CUDA(cudaMallocFromPoolAsync((void **)&p, count * sizeof(T), scratch_pool(), s));
            alloc_live(1);
        }
    }
    PBuf(const PBuf &) = delete;
    PBuf &operator=(const PBuf &) = delete;
    ~PBuf()
    {
        if (p) {
            cudaFreeAsync(p, s);
            alloc_live(-1);
        }
    }
    void zero()
    {
        if (n) PADO_CUDA(cudaMemsetAsync(p, 0, n * sizeof(T), s));
    }
};

// ---- radix sort -------------------------------------------------------------

// counts[d * ntiles + tile] = keys of `tile` whose digit at `shift` is d.
__global__ void __launch_bounds__(RS_THREADS) rs_hist_kernel(const uint64_t *keys, uint64_t L, uint32_t shift,
                                                             uint32_t ntiles, uint32_t *counts)
{
    __shared__ uint32_t h[256];
    for (uint32_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        h[threadIdx.x] = 0;
        __syncthreads();
        const uint64_t t0 = (uint64_t)tile * RS_TILE, t1 = min(L, t0 + RS_TILE);
        for (uint64_t i = t0 + threadIdx.x; i < t1; i += RS_THREADS)
            atomicAdd(&h[(keys[i] >> shift) & 255u], 1u);
        __syncthreads();
        counts[(uint64_t)threadIdx.x * ntiles + tile] = h[threadIdx.x];
        __syncthreads();
    }
}

// Stable scatter of one digit.  Warp w owns keys [512 w, 512 w + 512) of the
// tile, 32 per round; a key's place among the tile's keys with its digit is
// (keys of lower warps) + (keys of earlier rounds of its warp) + (lower lanes
// of its round), which is its input order.  A thread's 16 keys are loaded
// before any ranking so that their loads are in flight together.
__global__ void __launch_bounds__(RS_THREADS, 4) rs_scatter_kernel(const uint64_t *in, uint64_t *out, uint64_t L,
                                                                uint32_t shift, uint32_t ntiles,
                                                                const uint32_t *offsets)
{
    constexpr int NW = RS_THREADS / 32;
    __shared__ uint64_t sk[RS_TILE];      // the tile, reordered by digit
    __shared__ uint16_t slr[RS_TILE];     // rank of key i among its warp's keys with its digit
    __shared__ uint16_t wcnt[NW][256];    // per warp and digit: count, then prefix over warps
    __shared__ uint32_t dstart[256];      // first slot of each digit in the reordered tile
    __shared__ uint32_t gbase[256];       // global position of each digit's run
    __shared__ uint32_t wsum[NW];
    const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
    const uint32_t below = (1u << lane) - 1u;
    for (uint32_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const uint64_t t0 = (uint64_t)tile * RS_TILE;
        const uint32_t cnt = (uint32_t)min(L - t0, (uint64_t)RS_TILE);
        const uint32_t i0 = wl * (RS_PER * 32) + lane;
        uint64_t key[RS_PER];
#pragma unroll
        for (int r = 0; r < RS_PER; ++r) key[r] = i0 + r * 32 < cnt ? in[t0 + i0 + r * 32] : 0ull;
#pragma unroll
        for (int w = 0; w < NW; ++w) wcnt[w][threadIdx.x] = 0;
        gbase[threadIdx.x] = offsets[(uint64_t)threadIdx.x * ntiles + tile];
        __syncthreads();
#pragma unroll
        for (int r = 0; r < RS_PER; ++r) {
            const uint32_t i = i0 + r * 32;
            const bool live = i < cnt;
            const uint32_t dig = live ? (uint32_t)((key[r] >> shift) & 255u) : 256u + lane;  // idle lanes alone
            const uint32_t peers = __match_any_sync(FULLW, dig);
            if (live) slr[i] = (uint16_t)(wcnt[wl][dig] + __popc(peers & below));
            __syncwarp();
            if (live && (peers & below) == 0) wcnt[wl][dig] += (uint16_t)__popc(peers);
            __syncwarp();
        }
        __syncthreads();
        // thread d: prefix of digit d over the warps, and the digit's total
        uint32_t tot = 0;
#pragma unroll
        for (int w = 0; w < NW; ++w) {
            const uint32_t c = wcnt[w][threadIdx.x];
            wcnt[w][threadIdx.x] = (uint16_t)tot;
            tot += c;
        }
        // exclusive scan of the 256 totals -> dstart
        uint32_t inc = tot;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(FULLW, inc, o);
            if (lane >= o) inc += y;
        }
        if (lane == 31) wsum[wl] = inc;
        __syncthreads();
        uint32_t wpre = 0;
#pragma unroll
        for (int w = 0; w < NW; ++w) wpre += w < wl ? wsum[w] : 0u;
        dstart[threadIdx.x] = wpre + inc - tot;
        __syncthreads();
#pragma unroll
        for (int r = 0; r < RS_PER; ++r) {
            const uint32_t i = i0 + r * 32;
            if (i < cnt) {
                const uint32_t dig = (uint32_t)((key[r] >> shift) & 255u);
                sk[dstart[dig] + wcnt[wl][dig] + slr[i]] = key[r];
            }
        }
        __syncthreads();
        for (uint32_t p = threadIdx.x; p < cnt; p += RS_THREADS) {
            const uint64_t k = sk[p];
            const uint32_t dig = (uint32_t)((k >> shift) & 255u);
            out[gbase[dig] + (p - dstart[dig])] = k;
        }
        __syncthreads();
    }
}

uint64_t sort_tiles(uint64_t L) { return std::max<uint64_t>((L + RS_TILE - 1) / RS_TILE, 1); }

// Scratch of a radix sort of up to L keys.
struct SortSpace {
    PBuf<uint64_t> tmp;
    PBuf<uint32_t> counts, sums;
    SortSpace(uint64_t L, cudaStream_t s)
        : tmp(std::max<uint64_t>(L, 1), s), counts(256 * sort_tiles(L), s),
          sums(scan_sums_needed(256 * sort_tiles(L)), s)
    {
    }
};

// Sorts keys[0, L) ascending on bits [lo, hi), stably, stream-ordered;
// returns the buffer holding the result (`keys` or ws.tmp).  The dedupe and
// vertex-order sorts (`aux`) are profiled under their own names, so that the
// entry sort's launches all process the same 2m keys.
uint64_t *radix_sort(uint64_t *keys, uint64_t L, uint32_t lo, uint32_t hi, SortSpace &ws, cudaStream_t s,
                     bool aux = false)
{
    if (L < 2 || lo >= hi) return keys;
    PADO_CHECK(ws.tmp.n >= L, PADO_E_ARG, "sort scratch too small");
    const uint32_t ntiles = (uint32_t)((L + RS_TILE - 1) / RS_TILE);
    const unsigned grid = std::min<uint32_t>(ntiles, 152u * 8u);
    const char *hname = aux ? "rs_hist_kernel.aux" : "rs_hist_kernel";
    const char *sname = aux ? "rs_scatter_kernel.aux" : "rs_scatter_kernel";
    uint64_t *src = keys, *dst = ws.tmp.p;
    for (uint32_t shift = lo; shift < hi; shift += 8) {
        PADO_LAUNCH(hname, s, rs_hist_kernel<<<grid, RS_THREADS, 0, s>>>(src, L, shift, ntiles, ws.counts.p));
        exclusive_scan(ws.counts.p, (uint64_t)256 * ntiles, ws.sums.p, s);
        PADO_LAUNCH(sname, s, rs_scatter_kernel<<<grid, RS_THREADS, 0, s>>>(src, dst, L, shift, ntiles, ws.counts.p));
        std::swap(src, dst);
    }
    return src;
}

uint32_t id_bits(uint64_t n)
{
    uint32_t b = 1;
    while (b < 40 && (1ull << b) < n) ++b;
    return b;
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

// deg[x] += 1 for both ends of every edge.  Each block counts its share of
// the edges in a shared-memory table of DEG_SLOTS (vertex, count) slots,
// claimed by the first vertex that hashes there; vertices that find their
// slot taken add to global memory directly.  The heavy vertices of a skewed
// graph claim their slots early (they are most of the endpoints) and then
// cost one global atomic per block instead of one per endpoint.
constexpr uint32_t DEG_SLOTS = 2048;

__device__ __forceinline__ void count_endpoint(uint32_t a, uint32_t *cid, uint32_t *ccnt, uint32_t *deg)
{
    const uint32_t slot = (a * 2654435761u) >> 21;  // top 11 bits: DEG_SLOTS slots
    const uint32_t old = atomicCAS(&cid[slot], 0xffffffffu, a);
    if (old == 0xffffffffu || old == a)
        atomicAdd(&ccnt[slot], 1u);
    else
        atomicAdd(&deg[a], 1u);
}

__global__ void __launch_bounds__(256) degree_kernel(const uint32_t *u, const uint32_t *v, uint64_t m, uint32_t n,
                                                     uint32_t *deg, uint32_t *bad)
{
    __shared__ uint32_t cid[DEG_SLOTS], ccnt[DEG_SLOTS];
    for (uint32_t k = threadIdx.x; k < DEG_SLOTS; k += blockDim.x) {
        cid[k] = 0xffffffffu;
        ccnt[k] = 0;
    }
    __syncthreads();
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < m; e += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t a = u[e], b = v[e];
        if (a >= n || b >= n) {
            atomicOr(bad, 1u);
            continue;
        }
        count_endpoint(a, cid, ccnt, deg);
        count_endpoint(b, cid, ccnt, deg);
    }
    __syncthreads();
    for (uint32_t k = threadIdx.x; k < DEG_SLOTS; k += blockDim.x)
        if (ccnt[k]) atomicAdd(&deg[cid[k]], ccnt[k]);
}

__global__ void __launch_bounds__(256) max_deg_kernel(const uint32_t *deg, uint32_t n, uint32_t *mx)
{
    uint32_t x = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) x = max(x, deg[i]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x = max(x, __shfl_xor_sync(FULLW, x, o));
    if ((threadIdx.x & 31) == 0) atomicMax(mx, x);
}

// (max degree - degree, id): ascending order = degree descending, ties by id.
__global__ void __launch_bounds__(256) order_key_kernel(const uint32_t *deg, uint32_t n, uint32_t maxdeg,
                                                        uint64_t *keys)
{
    for (uint32_t x = blockIdx.x * blockDim.x + threadIdx.x; x < n; x += gridDim.x * blockDim.x)
        keys[x] = (uint64_t)(maxdeg - deg[x]) << 32 | x;
}

// rank[id] = position; degr[position] = degree (degr[n] = 0 closes the scan).
__global__ void __launch_bounds__(256) rank_kernel(const uint64_t *keys, uint32_t n, uint32_t maxdeg, uint32_t *rank,
                                                   uint32_t *degr)
{
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p <= n; p += gridDim.x * blockDim.x) {
        if (p == n) {
            degr[n] = 0;
            continue;
        }
        const uint64_t k = keys[p];
        rank[(uint32_t)k] = p;
        degr[p] = maxdeg - (uint32_t)(k >> 32);
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

__global__ void __launch_bounds__(256) widen_kernel(const uint32_t *a, uint64_t n, uint64_t *b)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        b[i] = a[i];
}

// ---- CSR input -> ranked CSR -------------------------------------------------

// One warp per vertex: offsets non-decreasing (bit 0), ids < n (bit 1),
// neighbour lists in descending (id, weight) order (bit 2 clear when not),
// and the offsets narrowed to 32 bits.
__global__ void __launch_bounds__(256) csr_check_kernel(const uint64_t *off, const uint32_t *adj, const uint8_t *w,
                                                        uint32_t n, uint64_t m, uint32_t *off32, uint32_t *flags)
{
    const int lane = threadIdx.x & 31;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    uint32_t f = 0;
    for (uint32_t v = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; v <= n; v += nw) {
        if (lane == 0) off32[v] = (uint32_t)off[v];
        if (v == n) continue;
        const uint64_t b = off[v], e = off[v + 1];
        if (e < b || e > m) {  // decreasing somewhere; no entry outside [0, m) is read
            f |= 1u;
            continue;
        }
        for (uint64_t k = b + lane; k < e; k += 32) {
            const uint32_t x = adj[k];
            if (x >= n) f |= 2u;
            if (k > b) {
                const uint32_t y = adj[k - 1];
                if (y < x || (y == x && w && w[k - 1] < w[k])) f |= 4u;
            }
        }
    }
    if (f) atomicOr(flags, f);
}

// rank must be a permutation of 0..n-1: seen[] counts each value once.
__global__ void __launch_bounds__(256) rank_check_kernel(const uint32_t *rank, uint32_t n, uint32_t *seen,
                                                         uint32_t *flags)
{
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        const uint32_t r = rank[v];
        if (r >= n || atomicExch(&seen[r], 1u) != 0u) atomicOr(flags, 8u);
    }
}

// Keys of every CSR entry (warp per vertex), the entry_key layout:
// rank(src) << (b + 8) | (2^b - 1 - rank(dst)) << 8 | (255 - weight).
__global__ void __launch_bounds__(256) csr_key_kernel(const uint64_t *off, const uint32_t *adj, const uint8_t *w,
                                                      const uint32_t *rank, uint32_t n, uint32_t bits, uint64_t *keys,
                                                      uint32_t *degr)
{
    const int lane = threadIdx.x & 31;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    const uint64_t dmask = (1ull << bits) - 1;
    for (uint32_t v = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; v <= n; v += nw) {
        if (v == n) {
            if (lane == 0) degr[n] = 0;
            continue;
        }
        const uint64_t b = off[v], e = off[v + 1];
        const uint64_t rv = rank ? rank[v] : v;
        if (lane == 0) degr[rv] = (uint32_t)(e - b);
        for (uint64_t k = b + lane; k < e; k += 32) {
            const uint64_t rd = rank ? rank[adj[k]] : adj[k];
            keys[k] = rv << (bits + 8) | (dmask - rd) << 8 | (255u - (w ? w[k] : 0u));
        }
    }
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

// ---- graph reductions (the reference's conversion tools) -------------------

// For vertices with at most two adjacency entries, the entries themselves
// (any order): nb[2x], nb[2x + 1].  Ids were range-checked by degree_kernel.
__global__ void __launch_bounds__(256) red_small_adj_kernel(const uint32_t *u, const uint32_t *v, uint64_t m,
                                                            const uint32_t *deg, uint32_t *fill, uint32_t *nb)
{
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < m; e += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t a = u[e], b = v[e];
        if (deg[a] <= 2) nb[2ull * a + atomicAdd(&fill[a], 1u)] = b;
        if (deg[b] <= 2) nb[2ull * b + atomicAdd(&fill[b], 1u)] = a;
    }
}

// Every vertex with one entry deletes itself and the chain of two-entry
// vertices behind it, stopping before the first vertex whose entry count is
// not 2.  Two walks meet only on a path component (both ends have one
// entry); their marks are the same idempotent stores, so the flags do not
// depend on the order the walks run in.  A chain cannot close on itself (its
// vertices have two entries each); the step bound only guards that.
__global__ void __launch_bounds__(256) red_walk_kernel(uint32_t n, const uint32_t *deg, const uint32_t *nb,
                                                       uint8_t *del, uint32_t *status)
{
    for (uint32_t x = blockIdx.x * blockDim.x + threadIdx.x; x < n; x += gridDim.x * blockDim.x) {
        if (deg[x] != 1) continue;
        del[x] = 1;
        uint32_t prev = x, cur = nb[2ull * x];
        for (uint32_t steps = 0; deg[cur] == 2; ++steps) {
            if (steps >= n) {
                atomicOr(status, 1u);
                break;
            }
            del[cur] = 1;
            const uint32_t a = nb[2ull * cur], b = nb[2ull * cur + 1];
            const uint32_t nx = a != prev ? a : b;
            if (nx == prev) break;  // both entries lead back: nothing further on
            prev = cur;
            cur = nx;
        }
    }
}

// flag[e] = 1 when edge e has no dropped end (flag[m] stays 0 for the scan).
__global__ void __launch_bounds__(256) red_keep_flag_kernel(const uint32_t *u, const uint32_t *v, uint64_t m,
                                                            const uint8_t *drop, uint32_t *flag)
{
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < m; e += (uint64_t)gridDim.x * blockDim.x)
        flag[e] = (!drop[u[e]] && !drop[v[e]]) ? 1u : 0u;
}

__global__ void __launch_bounds__(256) red_keep_scatter_kernel(const uint32_t *pos, uint64_t m, uint64_t *kept)
{
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < m; e += (uint64_t)gridDim.x * blockDim.x)
        if (pos[e + 1] != pos[e]) kept[pos[e]] = e;
}

// Both adjacency entries of every edge as (src << bits | dst) keys; ids must
// be below n (a flag otherwise).
__global__ void __launch_bounds__(256) red_entry_key_kernel(const uint32_t *u, const uint32_t *v, uint64_t m,
                                                            uint32_t n, uint32_t bits, uint64_t *keys,
                                                            uint32_t *bad)
{
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < m; e += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t a = u[e], b = v[e];
        if (a >= n || b >= n) atomicOr(bad, 1u);
        keys[2 * e] = a << bits | b;
        keys[2 * e + 1] = b << bits | a;
    }
}

// SplitMix64's output function (Steele, Lea and Flood, "Fast splittable
// pseudorandom number generators", OOPSLA 2014): a bijective 64-bit mixer.
__device__ __forceinline__ uint64_t mix64(uint64_t x)
{
    x += 0x9e3779b97f4a7c15ull;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
    return x ^ (x >> 31);
}

// The sorted entries: adjacency out, and per source vertex the sum of its
// entries' mixed values (a sum does not depend on order).  A warp takes 32
// consecutive entries; equal sources are contiguous, so a segmented scan over
// the lanes sums each run and its last lane adds the run with one atomic.
__global__ void __launch_bounds__(256) red_extract_hash_kernel(const uint64_t *keys, uint64_t L, uint32_t bits,
                                                               uint32_t *adj, unsigned long long *h)
{
    const int lane = threadIdx.x & 31;
    const uint64_t mask = (1ull << bits) - 1;
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t base = (((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32; base < L; base += nw * 32) {
        const uint64_t k = base + lane;
        const bool live = k < L;
        const uint64_t key = live ? keys[k] : 0ull;
        const uint32_t src = live ? (uint32_t)(key >> bits) : 0xffffffffu;
        if (live) adj[k] = (uint32_t)(key & mask);
        uint64_t c = live ? mix64(key & mask) : 0ull;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint64_t t = __shfl_up_sync(FULLW, c, o);
            const uint32_t s2 = __shfl_up_sync(FULLW, src, o);
            if (lane >= o && s2 == src) c += t;
        }
        const uint32_t nsrc = __shfl_down_sync(FULLW, src, 1);
        if (live && (lane == 31 || nsrc != src)) atomicAdd(&h[src], (unsigned long long)c);
    }
}

// Offsets of the sorted entries' sources: thread k (0 <= k <= L) writes
// off[x] = k for every x in (src(k-1), src(k)], with src(-1) = -1 and
// src(L) = n, so vertices without entries get the next start and off[n] = L.
__global__ void __launch_bounds__(256) red_offsets_kernel(const uint64_t *keys, uint64_t L, uint32_t bits,
                                                          uint32_t n, uint32_t *off)
{
    for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k <= L; k += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t cur = k < L ? (uint32_t)(keys[k] >> bits) : n;
        const int64_t prev = k > 0 ? (int64_t)(keys[k - 1] >> bits) : -1;
        for (int64_t x = prev + 1; x <= (int64_t)cur; ++x) off[x] = (uint32_t)k;
    }
}

// The set hash of every vertex x: its entries' sum plus x itself, folded
// with the set size into 32 bits, as the key (hash << 32 | x).  Equal sets
// have equal upper halves; the converse is checked exactly afterwards.
__global__ void __launch_bounds__(256) red_hash_finish_kernel(uint32_t n, const uint32_t *off,
                                                              const unsigned long long *h, uint64_t *keys)
{
    for (uint32_t x = blockIdx.x * blockDim.x + threadIdx.x; x < n; x += gridDim.x * blockDim.x) {
        const uint64_t sum = (uint64_t)h[x] + mix64(x);
        const uint64_t f = mix64(sum ^ ((uint64_t)(off[x + 1] - off[x] + 1) << 40));
        keys[x] = (f >> 32) << 32 | x;
    }
}

// Element k of x's sorted set: its sorted entries A[0, d) with x inserted at
// position px (the count of entries below x).
__device__ __forceinline__ uint32_t set_elem(const uint32_t *A, uint32_t px, uint32_t x, uint32_t k)
{
    return k < px ? A[k] : (k == px ? x : A[k - 1]);
}

// Whether x and y have equal sets (every lane returns it).
__device__ bool same_set(uint32_t x, uint32_t y, const uint32_t *off, const uint32_t *adj, int lane)
{
    const uint32_t d = off[x + 1] - off[x];
    if (off[y + 1] - off[y] != d) return false;
    const uint32_t *A = adj + off[x], *B = adj + off[y];
    uint32_t px = 0, py = 0;
    for (uint32_t k = lane; k < d; k += 32) {
        px += A[k] < x ? 1u : 0u;
        py += B[k] < y ? 1u : 0u;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        px += __shfl_xor_sync(FULLW, px, o);
        py += __shfl_xor_sync(FULLW, py, o);
    }
    for (uint32_t k0 = 0; k0 <= d; k0 += 32) {
        const uint32_t k = k0 + lane;
        const bool diff = k <= d && set_elem(A, px, x, k) != set_elem(B, py, y, k);
        if (__any_sync(FULLW, diff)) return false;
    }
    return true;
}

// A warp per position p of the (hash, id)-sorted keys: a vertex that is not
// the first of its hash run compares its set with the run's earlier vertices
// in ascending id and is redundant at the first equal one -- so exactly the
// smallest id of every class of equal sets stays.
__global__ void __launch_bounds__(256) red_twin_kernel(uint32_t n, const uint64_t *keys, const uint32_t *off,
                                                       const uint32_t *adj, uint8_t *red)
{
    const int lane = threadIdx.x & 31;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t p = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; p < n; p += nw) {
        const uint64_t hi = keys[p] >> 32;
        if (p == 0 || (keys[p - 1] >> 32) != hi) continue;
        // first position of the run: lower bound of hi among keys[0, p)
        uint32_t lo = 0, up = p;
        while (lo < up) {
            const uint32_t mid = lo + (up - lo) / 2;
            if ((keys[mid] >> 32) < hi) lo = mid + 1;
            else up = mid;
        }
        const uint32_t y = (uint32_t)keys[p];
        for (uint32_t q = lo; q < p; ++q)
            if (same_set((uint32_t)keys[q], y, off, adj, lane)) {
                if (lane == 0) red[y] = 1;
                break;
            }
    }
}

// flag[x] = 1 for vertices that stay (flag[n] stays 0 for the scan).
__global__ void __launch_bounds__(256) red_stay_flag_kernel(uint32_t n, const uint8_t *red, uint32_t *flag)
{
    for (uint32_t x = blockIdx.x * blockDim.x + threadIdx.x; x < n; x += gridDim.x * blockDim.x)
        flag[x] = red[x] ? 0u : 1u;
}

__global__ void __launch_bounds__(256) red_new_id_kernel(uint32_t n, const uint8_t *red, const uint32_t *pos,
                                                         uint32_t *new_id)
{
    for (uint32_t x = blockIdx.x * blockDim.x + threadIdx.x; x < n; x += gridDim.x * blockDim.x)
        new_id[x] = red[x] ? 0xffffffffu : pos[x];
}

// 1 + the largest new id on a kept edge.
__global__ void __launch_bounds__(256) red_top_kernel(const uint32_t *u, const uint32_t *v, const uint64_t *kept,
                                                      uint64_t k, const uint32_t *new_id, uint32_t *top)
{
    uint32_t t = 0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < k; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t e = kept[i];
        t = max(t, max(new_id[u[e]], new_id[v[e]]) + 1u);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t = max(t, __shfl_xor_sync(FULLW, t, o));
    if ((threadIdx.x & 31) == 0 && t) atomicMax(top, t);
}

}  // namespace

IngestResult ingest_edges(uint64_t m, const uint32_t *du, const uint32_t *dv, const uint8_t *dw, uint32_t n,
                          bool dedupe, cudaStream_t s, uint32_t *adj_out, uint8_t *w_out)
{
    IngestResult r;
    PADO_CHECK(m < (1ull << 31), PADO_E_ARG, "at most 2^31 - 1 edges (2^32 - 2 adjacency entries)");
    PBuf<uint32_t> scal(1, s);
    if (n == 0 && m) {  // n = max id + 1, as Graph::construct sets it
        scal.zero();
        PADO_LAUNCH("max_id_kernel", s, max_id_kernel<<<grid_for(m, 256), 256, 0, s>>>(du, dv, m, scal.p));
        const uint32_t mx = read_back(scal.p, s);
        PADO_CHECK(mx < 0xffffffffu, PADO_E_ARG, "vertex id 2^32 - 1 is reserved");
        n = mx + 1;
    }
    const uint32_t bits = id_bits(n);
    PADO_CHECK(bits <= 28, PADO_E_ARG, "graph ingest supports fewer than 2^28 vertices");
    r.n = n;
    // one sort scratch for every sort of the call: the dedupe sort (m keys),
    // the order sort (n keys) and the entry sort (2m keys after dedupe)
    SortSpace ws(std::max<uint64_t>(2 * m, n), s);

    // optional dedupe over original ids
    std::optional<PBuf<uint32_t>> u2, v2;
    std::optional<PBuf<uint8_t>> w2;
    if (dedupe && m) {
        PBuf<uint64_t> ck(m, s);
        scal.zero();
        PADO_LAUNCH("canon_key_kernel", s,
                    canon_key_kernel<<<grid_for(m, 256), 256, 0, s>>>(du, dv, dw, m, n, bits, ck.p, scal.p));
        PADO_CHECK(read_back(scal.p, s) == 0, PADO_E_ARG, "edge endpoint out of range");
        const uint64_t *sorted = radix_sort(ck.p, m, 8, 2 * bits + 8, ws, s, true);
        PBuf<uint32_t> pos(m + 1, s), psums(scan_sums_needed(m + 1), s);
        PADO_LAUNCH("unique_flag_kernel", s,
                    unique_flag_kernel<<<grid_for(m + 1, 256), 256, 0, s>>>(sorted, m, pos.p));
        exclusive_scan(pos.p, m + 1, psums.p, s);
        const uint32_t mu = read_back(pos.p + m, s);
        u2.emplace(std::max<uint32_t>(mu, 1), s);
        v2.emplace(std::max<uint32_t>(mu, 1), s);
        if (dw) w2.emplace(std::max<uint32_t>(mu, 1), s);
        PADO_LAUNCH("unique_scatter_kernel", s,
                    unique_scatter_kernel<<<grid_for(m, 256), 256, 0, s>>>(sorted, m, bits, pos.p, u2->p, v2->p,
                                                                         dw ? w2->p : nullptr));
        du = u2->p;
        dv = v2->p;
        dw = dw ? w2->p : nullptr;
        m = mu;
    }

    // degrees -> order (degree descending, ties by ascending id) -> offsets
    r.rank.alloc(std::max<uint32_t>(n, 1));
    r.off.alloc((uint64_t)n + 1);
    {
        PBuf<uint32_t> deg(std::max<uint32_t>(n, 1), s);
        deg.zero();
        scal.zero();
        if (m)
            PADO_LAUNCH("degree_kernel", s,
                        degree_kernel<<<grid_for(m, 256, 152u * 8u), 256, 0, s>>>(du, dv, m, n, deg.p, scal.p));
        PADO_CHECK(read_back(scal.p, s) == 0, PADO_E_ARG, "edge endpoint out of range");
        scal.zero();
        if (n) PADO_LAUNCH("max_deg_kernel", s, max_deg_kernel<<<grid_for(n, 256), 256, 0, s>>>(deg.p, n, scal.p));
        const uint32_t maxdeg = read_back(scal.p, s);
        PBuf<uint64_t> ok(std::max<uint32_t>(n, 1), s);
        if (n)
            PADO_LAUNCH("order_key_kernel", s,
                        order_key_kernel<<<grid_for(n, 256), 256, 0, s>>>(deg.p, n, maxdeg, ok.p));
        const uint64_t *order =
            radix_sort(ok.p, n, 32, 32 + (maxdeg ? id_bits((uint64_t)maxdeg + 1) : 0), ws, s, true);
        PADO_LAUNCH("rank_kernel", s,
                    rank_kernel<<<grid_for((uint64_t)n + 1, 256), 256, 0, s>>>(order, n, maxdeg, r.rank.p, r.off.p));
        PBuf<uint32_t> osums(scan_sums_needed((uint64_t)n + 1), s);
        exclusive_scan(r.off.p, (uint64_t)n + 1, osums.p, s);
    }

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
        PBuf<uint64_t> keys(L, s);
        PADO_LAUNCH("entry_key_kernel", s,
                    entry_key_kernel<<<grid_for(m, 256), 256, 0, s>>>(du, dv, dw, m, r.rank.p, bits, keys.p));
        // after dedupe no (src, dst) pair repeats, so the weight byte needs no pass
        const uint64_t *sorted = radix_sort(keys.p, L, dw && !dedupe ? 0u : 8u, 2 * bits + 8, ws, s);
        PADO_LAUNCH("extract_kernel", s,
                    extract_kernel<<<grid_for(L, 256), 256, 0, s>>>(sorted, L, bits, adj_out, dw ? w_out : nullptr));
    }
    PADO_CUDA(cudaStreamSynchronize(s));
    return r;
}

void release_scratch(uint64_t keep_bytes)
{
    PADO_CUDA(cudaMemPoolTrimTo(scratch_pool(), keep_bytes));
}

void widen_u32(const uint32_t *a, uint64_t n, uint64_t *b, cudaStream_t s)
{
    if (n) PADO_LAUNCH("widen_kernel", s, widen_kernel<<<grid_for(n, 256), 256, 0, s>>>(a, n, b));
}

DevGraph prepare_csr(uint32_t n, const uint64_t *off, const uint32_t *adj, const uint8_t *w, const uint32_t *rank,
                     cudaStream_t s, DBuf<uint32_t> *rank_out)
{
    const uint64_t m = off[n];
    DevGraph g;
    g.n = n;
    g.m = m;
    {
        HostPhase ph("csr alloc");
        g.off.alloc((uint64_t)n + 1);
        g.adj.alloc(std::max<uint64_t>(m, 1));
        if (w) g.w.alloc(std::max<uint64_t>(m, 1));
    }
    HostPhase ph("csr upload+check");
    // page-locked inputs are read by the SMs, others go through the copy engines
    upload_bytes(g.adj.p, adj, m * 4, s);
    if (w) upload_bytes(g.w.p, w, m, s);
    PBuf<uint64_t> off64((uint64_t)n + 1, s);
    upload_bytes(off64.p, off, ((uint64_t)n + 1) * 8, s);
    PBuf<uint32_t> flags(1, s);
    flags.zero();
    PADO_LAUNCH("csr_check_kernel", s,
                csr_check_kernel<<<grid_for(((uint64_t)n + 1) * 32, 256), 256, 0, s>>>(off64.p, g.adj.p,
                                                                                     w ? g.w.p : nullptr, n, m,
                                                                                     g.off.p, flags.p));
    if (rank) {
        rank_out->alloc(std::max<uint32_t>(n, 1));
        upload_bytes(rank_out->p, rank, (uint64_t)n * 4, s);
        PBuf<uint32_t> seen(std::max<uint32_t>(n, 1), s);
        seen.zero();
        if (n)
            PADO_LAUNCH("rank_check_kernel", s,
                        rank_check_kernel<<<grid_for(n, 256), 256, 0, s>>>(rank_out->p, n, seen.p, flags.p));
    }
    const uint32_t f = read_back(flags.p, s);
    PADO_CHECK(!(f & 1u), PADO_E_ARG, "offsets must be non-decreasing");
    PADO_CHECK(!(f & 2u), PADO_E_ARG, "adjacency id out of range");
    PADO_CHECK(!(f & 8u), PADO_E_ARG, "rank is not a permutation of 0..n-1");
    if (!rank && !(f & 4u)) return g;  // ranked and sorted: used as uploaded
    // relabel by rank and sort every list: the entry sort of the edge-list path
    const uint32_t bits = id_bits(n);
    PADO_CHECK(bits <= 28, PADO_E_ARG, "relabeling on the device supports fewer than 2^28 vertices");
    if (m) {
        PBuf<uint64_t> keys(m, s);
        SortSpace ws(m, s);
        PADO_LAUNCH("csr_key_kernel", s,
                    csr_key_kernel<<<grid_for(((uint64_t)n + 1) * 32, 256), 256, 0, s>>>(
                        off64.p, g.adj.p, w ? g.w.p : nullptr, rank ? rank_out->p : nullptr, n, bits, keys.p,
                        g.off.p));
        PBuf<uint32_t> osums(scan_sums_needed((uint64_t)n + 1), s);
        exclusive_scan(g.off.p, (uint64_t)n + 1, osums.p, s);
        const uint64_t *sorted = radix_sort(keys.p, m, w ? 0u : 8u, 2 * bits + 8, ws, s);
        PADO_LAUNCH("extract_kernel", s,
                    extract_kernel<<<grid_for(m, 256), 256, 0, s>>>(sorted, m, bits, g.adj.p, w ? g.w.p : nullptr));
    } else {
        g.off.fill_bytes(0, s);
    }
    PADO_CUDA(cudaStreamSynchronize(s));
    return g;
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

// ---- graph reductions --------------------------------------------------------

namespace {

// Adjacency entries per vertex (a self-loop counts twice), with the range
// check both reductions share.
void entry_degrees(uint64_t m, const uint32_t *du, const uint32_t *dv, uint32_t n, uint32_t *deg, uint32_t *scal,
                   cudaStream_t s)
{
    PADO_CUDA(cudaMemsetAsync(deg, 0, (size_t)n * 4, s));
    PADO_CUDA(cudaMemsetAsync(scal, 0, 4, s));
    if (m)
        PADO_LAUNCH("degree_kernel", s,
                    degree_kernel<<<grid_for(m, 256, 152u * 8u), 256, 0, s>>>(du, dv, m, n, deg, scal));
    PADO_CHECK(read_back(scal, s) == 0, PADO_E_ARG, "edge endpoint out of range");
}

// Indices of the edges with no dropped end, in input order; returns the count.
uint64_t keep_edges(uint64_t m, const uint32_t *du, const uint32_t *dv, const uint8_t *drop, uint64_t *kept,
                    cudaStream_t s)
{
    if (!m) return 0;
    PBuf<uint32_t> flag(m + 1, s), sums(scan_sums_needed(m + 1), s);
    PADO_CUDA(cudaMemsetAsync(flag.p + m, 0, 4, s));
    PADO_LAUNCH("red_keep_flag_kernel", s,
                red_keep_flag_kernel<<<grid_for(m, 256), 256, 0, s>>>(du, dv, m, drop, flag.p));
    exclusive_scan(flag.p, m + 1, sums.p, s);
    PADO_LAUNCH("red_keep_scatter_kernel", s,
                red_keep_scatter_kernel<<<grid_for(m, 256), 256, 0, s>>>(flag.p, m, kept));
    return read_back(flag.p + m, s);
}

void reduce_limits(uint64_t m, uint32_t n)
{
    PADO_CHECK(m < (1ull << 31), PADO_E_ARG, "at most 2^31 - 1 edges");
    PADO_CHECK(n < (1u << 31), PADO_E_ARG, "fewer than 2^31 vertices");
    PADO_CHECK(n > 0 || m == 0, PADO_E_ARG, "edge endpoint out of range");
}

}  // namespace

ReduceResult reduce_degree1(uint64_t m, const uint32_t *du, const uint32_t *dv, uint32_t n, cudaStream_t s,
                            uint8_t *deleted, uint64_t *kept)
{
    reduce_limits(m, n);
    ReduceResult r;
    r.n = n;
    if (!n) return r;
    PADO_CUDA(cudaMemsetAsync(deleted, 0, n, s));
    PBuf<uint32_t> scal(1, s), deg(n, s), fill(n, s), nb(2ull * n, s);
    entry_degrees(m, du, dv, n, deg.p, scal.p, s);
    fill.zero();
    if (m)
        PADO_LAUNCH("red_small_adj_kernel", s,
                    red_small_adj_kernel<<<grid_for(m, 256), 256, 0, s>>>(du, dv, m, deg.p, fill.p, nb.p));
    scal.zero();
    PADO_LAUNCH("red_walk_kernel", s,
                red_walk_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, deg.p, nb.p, deleted, scal.p));
    PADO_CHECK(read_back(scal.p, s) == 0, PADO_E_CUDA, "degree-1 chain walk exceeded n steps");
    r.kept = keep_edges(m, du, dv, deleted, kept, s);
    PADO_CUDA(cudaStreamSynchronize(s));
    return r;
}

ReduceResult reduce_equivalent(uint64_t m, const uint32_t *du, const uint32_t *dv, uint32_t n, cudaStream_t s,
                               uint8_t *redundant, uint32_t *new_id, uint64_t *kept)
{
    reduce_limits(m, n);
    ReduceResult r;
    r.n = n;
    if (!n) return r;
    PADO_CUDA(cudaMemsetAsync(redundant, 0, n, s));
    const uint32_t bits = id_bits(n);
    const uint64_t L = 2 * m;
    PBuf<uint32_t> scal(1, s), off((uint64_t)n + 1, s), adj(std::max<uint64_t>(L, 1), s);
    PBuf<unsigned long long> h(n, s);
    h.zero();
    SortSpace ws(std::max<uint64_t>(L, n), s);
    {
        // every vertex's entries, ascending: keys (src, dst) sorted; then the
        // adjacency, the entry sums of the set hashes and the offsets
        PBuf<uint64_t> keys(std::max<uint64_t>(L, 1), s);
        const uint64_t *sorted = keys.p;
        if (L) {
            scal.zero();
            PADO_LAUNCH("red_entry_key_kernel", s,
                        red_entry_key_kernel<<<grid_for(m, 256), 256, 0, s>>>(du, dv, m, n, bits, keys.p, scal.p));
            PADO_CHECK(read_back(scal.p, s) == 0, PADO_E_ARG, "edge endpoint out of range");
            sorted = radix_sort(keys.p, L, 0, 2 * bits, ws, s, true);
            PADO_LAUNCH("red_extract_hash_kernel", s,
                        red_extract_hash_kernel<<<grid_for(L, 256), 256, 0, s>>>(sorted, L, bits, adj.p, h.p));
        }
        PADO_LAUNCH("red_offsets_kernel", s,
                    red_offsets_kernel<<<grid_for(L + 1, 256), 256, 0, s>>>(sorted, L, bits, n, off.p));
    }
    {
        // (hash, id) keys sorted on the hash alone: the sort is stable and
        // the keys start in id order, so every run of one hash is in id order
        PBuf<uint64_t> hk(n, s);
        PADO_LAUNCH("red_hash_finish_kernel", s,
                    red_hash_finish_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, off.p, h.p, hk.p));
        const uint64_t *sorted = radix_sort(hk.p, n, 32, 64, ws, s, true);
        PADO_LAUNCH("red_twin_kernel", s,
                    red_twin_kernel<<<grid_for((uint64_t)n * 32, 256), 256, 0, s>>>(n, sorted, off.p, adj.p,
                                                                                    redundant));
    }
    {
        PBuf<uint32_t> pos((uint64_t)n + 1, s), psums(scan_sums_needed((uint64_t)n + 1), s);
        PADO_CUDA(cudaMemsetAsync(pos.p + n, 0, 4, s));
        PADO_LAUNCH("red_stay_flag_kernel", s,
                    red_stay_flag_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, redundant, pos.p));
        exclusive_scan(pos.p, (uint64_t)n + 1, psums.p, s);
        PADO_LAUNCH("red_new_id_kernel", s,
                    red_new_id_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, redundant, pos.p, new_id));
    }
    r.kept = keep_edges(m, du, dv, redundant, kept, s);
    scal.zero();
    if (r.kept)
        PADO_LAUNCH("red_top_kernel", s,
                    red_top_kernel<<<grid_for(r.kept, 256), 256, 0, s>>>(du, dv, kept, r.kept, new_id, scal.p));
    r.n_out = read_back(scal.p, s);
    PADO_CUDA(cudaStreamSynchronize(s));
    return r;
}

}  // namespace pado
