// unw_device.cuh -- device side of the batched pruned-BFS labeling, shared by
// the one-graph driver (unw.cu) and the many-graph driver (unw_many.cu).
//
// Restates the batched vertex-centric labeling of the reference
// (includes/pado_unw_unv_unp.h:425-1118; OpenMP variant
// pado_unw_unv_para.201912311607.parallel_bp_labeling.h:848-1737); the
// algorithm and its device mapping are described at the top of unw.cu.  Every
// phase below is a grid-stride __device__ function so that it can run inside a
// plain kernel or inside a persistent cooperative loop.
#pragma once

#include "grid_barrier.cuh"
#include "pado_internal.cuh"

namespace pado {
namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int SMALL_CAP = 384;                 // labels with d < iter staged in smem per chunk
// distance test of a light tail: staged lists at least this long, tested
// against at most this many candidates, are walked per candidate with the
// entries across the lanes instead of a lane per candidate (R-MAT s20:
// 64 / 16 gave 155.5 ms per build, 16 / 32 153.7 ms; 32 graphs of up to 60k
// vertices: 0.422 and 0.354 s, against 0.497 s with lanes per candidate only;
// walking every staged list, 1 / 32, was 152.7 ms against 151.8 ms for 16 / 32)
constexpr uint32_t WALK_MIN_STAGED = 16, WALK_MAX_CANDIDATES = 32;
constexpr uint32_t HEAVY_DEG = 2048;           // tails this large are processed by a block

// A vertex's label group of one level: list position, size and the level id
// (stamp) at which it was added -- one 16-byte record, so a reader learns
// whether a neighbour is active and where its new labels are in one load.
struct __align__(16) LastGroup {
    unsigned long long pos;
    uint32_t cnt;
    uint32_t stamp;
};

// Device bounds checks of a PADO_DEBUG_BOUNDS build.  UD_AT(arr, i, lim, site)
// is arr[i]; in such a build an index i >= lim sets bit `site` of the device
// word d.dbg and the access goes to a scratch slot instead (never a trap), so
// a run reports where it would have left its buffer and keeps going.  Sites:
// 0 CSR, 1 per-vertex state, 2 label pool, 3 BP rows, 4 dist_matrix,
// 5 indicator rows, 6 tail / frontier / retry lists.  Release builds compile
// the checks away.
#ifdef PADO_DEBUG_BOUNDS
#define UD_AT(arr, i, lim, site) (::pado::dbg_ref((arr), (uint64_t)(i), (uint64_t)(lim), (site), d.dbg))
#else
#define UD_AT(arr, i, lim, site) ((arr)[i])
#endif

struct UnwDev {
    uint32_t n, K, B, words;
    uint64_t m;             // adjacency entries
    uint32_t *dbg;          // bounds-check error word (PADO_DEBUG_BOUNDS builds)
    const uint32_t *off;
    const uint32_t *adj;
    const uint8_t *used;    // per vertex: bit 0 BP vertex (never a tail), bit 1 heavy (degree >= HEAVY_DEG)
    const uint8_t *bpd;
    const uint64_t *bps;
    const uint8_t *bpmin;   // per vertex: least BP distance over the roots (255: none)
    uint32_t *pool_hub;
    uint8_t *pool_dist;
    unsigned long long pool_cap;
    unsigned long long *pool_top;
    uint64_t *lab_off;
    uint32_t *lab_len;
    uint32_t *lab_cap;
    LastGroup *last[2];      // by level parity: the vertex's newest label group and its level id
    uint32_t *last_min[2];
    uint32_t *tail_stamp;
    uint32_t *ind;        // n * words
    uint32_t *ind_stamp;  // batch + 1 when the row is valid
    uint8_t *dm;          // B * n
    uint32_t *status;
    unsigned long long *work;  // algorithmic-byte counters (profiling only)
};

// Per-graph state when many graphs are labeled together in one union id space:
// graph g owns ids [base, base + n); its batch b holds the roots of
// [base + b*B, base + (b+1)*B) and its dist_matrix is a [B][n] block at
// dm + dm_off, entry (root idx, hub h) at idx * n + (h - base).
struct GDesc {
    uint32_t base, n;        // id range
    uint32_t nb;             // number of batches
    uint32_t b;              // current batch
    uint32_t s, e;           // current batch's id range [s, e)
    uint32_t iter;           // level computed in the current step
    uint32_t state;          // GS_* below
    uint32_t tc[3];          // tails marked for stamp x, in tc[x % 3]
    uint32_t roff, nr;       // current batch's roots: broots[roff, roff + nr)
    uint32_t bfirst;         // this graph's entries in the per-batch root counts
    uint32_t dmp;            // dist_matrix buffer of the current batch (0/1)
    uint32_t zqp;            // buffer of the batch whose rows are queued for reset
    uint64_t dm_off;         // offset of the graph's two dist_matrix blocks ([2][B][n])
};
enum : uint32_t { GS_START = 0, GS_LEVEL = 1, GS_DONE = 2 };

// Graph descriptors change between the steps of a persistent launch (written
// by one warp, read by every SM), so they are read at L2 (ld.global.cg), never
// from a possibly stale L1 line.
__device__ __forceinline__ uint32_t gd_u32(const uint32_t &f) { return __ldcg(&f); }
__device__ __forceinline__ uint64_t gd_u64(const uint64_t &f)
{
    return (uint64_t)__ldcg(reinterpret_cast<const unsigned long long *>(&f));
}

// Adds the heavy bit (bit 1) to the per-vertex flags that hold the BP bit.
__global__ void heavy_flag_kernel(const uint32_t *off, uint32_t n, uint8_t *flags)
{
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
        if (off[v + 1] - off[v] >= HEAVY_DEG) flags[v] |= 2u;
}

// bpmin[v] = least BP distance of v over the K roots (255 if none reaches it).
__global__ void bpmin_kernel(const uint8_t *bpd, uint32_t n, uint32_t K, uint8_t *bpmin)
{
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        uint32_t m = U8_INF;
        for (uint32_t i = 0; i < K; ++i) m = min(m, (uint32_t)bpd[(uint64_t)v * K + i]);
        bpmin[v] = (uint8_t)m;
    }
}

__device__ __forceinline__ uint32_t warp_min_u32(uint32_t v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(FULL, v, o));
    return v;
}

// Reserve room for `need` entries in v's list; relocates (warp-cooperative
// copy) when the slot is too small.  Returns false, with nothing changed
// except pool_top, when the pool is exhausted.
__device__ __forceinline__ bool warp_reserve(const UnwDev &d, uint32_t v, uint32_t need, uint64_t &base, int lane)
{
    const uint32_t len = UD_AT(d.lab_len, v, d.n, 1), cap = UD_AT(d.lab_cap, v, d.n, 1);
    base = UD_AT(d.lab_off, v, d.n, 1);
    if (need <= cap) return true;
    uint32_t ncap = max(max(2u * cap, need), 8u);
    ncap = (ncap + 7u) & ~7u;
    unsigned long long pos = 0;
    if (lane == 0) pos = atomicAdd(d.pool_top, (unsigned long long)ncap);
    pos = __shfl_sync(FULL, pos, 0);
    if (pos + ncap > d.pool_cap) return false;
    for (uint32_t j = lane; j < len; j += 32) {
        UD_AT(d.pool_hub, pos + j, d.pool_cap, 2) = UD_AT(d.pool_hub, base + j, d.pool_cap, 2);
        UD_AT(d.pool_dist, pos + j, d.pool_cap, 2) = UD_AT(d.pool_dist, base + j, d.pool_cap, 2);
    }
    __syncwarp();
    if (lane == 0) {
        UD_AT(d.lab_off, v, d.n, 1) = pos;
        UD_AT(d.lab_cap, v, d.n, 1) = ncap;
    }
    base = pos;
    return true;
}

// Batch start: self label (r, 0) for every non-BP root, indicator row with
// the root's own bit, active at level stamp lid0 (pado_unw_unv_unp.h:425-491).
// With gmap set, each root's batch (start s, id b) is its graph's current one.
__device__ void root_init_phase(const UnwDev &d, const uint32_t *roots, uint32_t nroots, uint32_t s, uint32_t b,
                                uint32_t lid0, uint32_t *front, uint32_t *front_cnt, uint32_t *retry,
                                uint32_t *retry_cnt, const GDesc *gd = nullptr, const uint16_t *gmap = nullptr)
{
    const int lane = threadIdx.x & 31;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    const int p = lid0 & 1;
    for (uint32_t q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < nroots; q += nw) {
        const uint32_t r = roots[q];
        uint64_t base;
        if (!warp_reserve(d, r, UD_AT(d.lab_len, r, d.n, 1) + 1, base, lane)) {
            if (lane == 0) {
                atomicOr(d.status, ST_POOL_RETRY);
                UD_AT(retry, atomicAdd(retry_cnt, 1u), d.n, 6) = r;
            }
            continue;
        }
        const uint32_t len = UD_AT(d.lab_len, r, d.n, 1);
        uint32_t rs = s, rb = b;
        if (gmap) {
            const GDesc &x = gd[gmap[r]];
            rs = gd_u32(x.s);
            rb = gd_u32(x.b);
        }
        const uint32_t idx = r - rs;
        for (uint32_t w = lane; w < d.words; w += 32)
            UD_AT(d.ind, (uint64_t)r * d.words + w, (uint64_t)d.n * d.words, 5) = (w == (idx >> 5)) ? (1u << (idx & 31)) : 0u;
        if (lane == 0) {
            if (d.work) atomicAdd(&d.work[W_EV_LABELS], 1ull);
            UD_AT(d.pool_hub, base + len, d.pool_cap, 2) = r;
            UD_AT(d.pool_dist, base + len, d.pool_cap, 2) = 0;
            UD_AT(d.lab_len, r, d.n, 1) = len + 1;
            UD_AT(d.last[p], r, d.n, 1) = LastGroup{base + len, 1u, lid0};
            UD_AT(d.last_min[p], r, d.n, 1) = r;
            UD_AT(d.ind_stamp, r, d.n, 1) = rb + 1;
            UD_AT(front, atomicAdd(front_cnt, 1u), d.n, 6) = r;
        }
    }
}

// dist_matrix rows of the batch roots: fill from their labels (value = d) or
// reset to 255 (pado_unw_unv_unp.h:492-526 and :780-816).
// With gmap set, root r's row is (r - base) % B of its graph's block (batches
// are B-aligned within a graph, so this is r - s of the batch r belongs to).
__device__ void dm_rows_phase(const UnwDev &d, const uint32_t *roots, uint32_t nroots, uint32_t s, int fill,
                              const GDesc *gd = nullptr, const uint16_t *gmap = nullptr, uint8_t *dm = nullptr)
{
    const int lane = threadIdx.x & 31;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < nroots; q += nw) {
        const uint32_t r = roots[q];
        uint8_t *row;
        uint32_t hb = 0, rn = d.n;
        if (gmap) {  // reset of a finished batch: its buffer is zqp
            const GDesc &x = gd[gmap[r]];
            hb = x.base;
            rn = x.n;
            row = d.dm + x.dm_off + ((uint64_t)gd_u32(x.zqp) * d.B + (r - hb) % d.B) * x.n;
        } else {
            row = (dm ? dm : d.dm) + (uint64_t)(r - s) * d.n;
        }
        const uint64_t base = UD_AT(d.lab_off, r, d.n, 1);
        const uint32_t len = UD_AT(d.lab_len, r, d.n, 1);
        for (uint32_t j = lane; j < len; j += 32)
            UD_AT(row, UD_AT(d.pool_hub, base + j, d.pool_cap, 2) - hb, rn, 4) =
                fill ? UD_AT(d.pool_dist, base + j, d.pool_cap, 2) : U8_INF;
    }
}

// Tail marking: for each active head, neighbours t (descending) with
// t > min(root of its last group) that are not BP vertices.
__device__ void mark_phase(const UnwDev &d, const uint32_t *front, uint32_t cnt, uint32_t lid_cur, uint32_t *tails,
                           uint32_t *tails_cnt, uint32_t *htails, uint32_t *htails_cnt)
{
    const int lane = threadIdx.x & 31;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    const int pp = (lid_cur - 1) & 1;
    unsigned long long bytes = 0;
    for (uint32_t q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < cnt; q += nw) {
        const uint32_t h = front[q];
        const uint32_t mn = UD_AT(d.last_min[pp], h, d.n, 1);
        const uint32_t e_end = UD_AT(d.off, h + 1, (uint64_t)d.n + 1, 0);
        bytes += 16;  // front entry, last_min, offsets
        for (uint32_t e0 = UD_AT(d.off, h, (uint64_t)d.n + 1, 0); e0 < e_end; e0 += 32) {
            const uint32_t e = e0 + lane;
            const bool in = e < e_end;
            const uint32_t t = in ? UD_AT(d.adj, e, d.m, 0) : 0u;
            const bool ok = in && t > mn;
            if (d.work) bytes += __popc(__ballot_sync(FULL, in)) * 4ull + __popc(__ballot_sync(FULL, ok)) * 5ull;
            bool appended = false;
            const uint32_t f = ok ? UD_AT(d.used, t, d.n, 1) : 1u;
            const uint32_t ts = ok ? UD_AT(d.tail_stamp, t, d.n, 1) : lid_cur;
            if (!(f & 1u) && ts != lid_cur) {
                if (atomicExch(&UD_AT(d.tail_stamp, t, d.n, 1), lid_cur) != lid_cur) {
                    const bool heavy = f & 2u;
                    if (heavy)
                        UD_AT(htails, agg_append_by(htails_cnt, 1u), d.n, 6) = t;
                    else
                        UD_AT(tails, agg_append_by(tails_cnt, 0u), d.n, 6) = t;
                    appended = true;
                }
            }
            if (d.work) bytes += __popc(__ballot_sync(FULL, appended)) * 8ull;
            if (__ballot_sync(FULL, in && !ok)) break;  // descending: the rest are smaller
        }
    }
    if (d.work && lane == 0 && bytes) atomicAdd(&d.work[W_MARK], bytes);
}

// Shared-memory layout of the pull kernel, carved from dynamic shared memory
// by batch size: 8 per-warp regions for light tails, aliased by one
// block-wide region for heavy tails (the two phases do not overlap).
constexpr int PULL_THREADS = 256;
constexpr int PULL_NW = PULL_THREADS / 32;
constexpr int HSMALL_CAP = 1024;          // heavy tail: labels with d < iter staged
constexpr uint32_t SMALL_LEVEL_PER_BLOCK = 1;  // levels with at most this many tails per block use the block path

__host__ __device__ __forceinline__ uint32_t align16(uint32_t x) { return (x + 15u) & ~15u; }

struct WarpRegion {
    uint32_t *ind;        // words
    uint16_t *offered;    // B
    uint32_t *sh;         // SMALL_CAP
    uint8_t *sd;          // SMALL_CAP
    uint32_t *ctr;        // spare
};

__host__ __device__ __forceinline__ uint32_t warp_region_bytes(uint32_t words, uint32_t B)
{
    return align16(words * 4) + align16(B * 2) + SMALL_CAP * 4 + SMALL_CAP + 16;
}

__host__ __device__ __forceinline__ uint32_t heavy_region_bytes(uint32_t words, uint32_t B)
{
    return align16(words * 4) + 2 * align16(B * 2) + HSMALL_CAP * 4 + HSMALL_CAP + 64;
}

__host__ __device__ __forceinline__ uint32_t pull_smem_bytes(uint32_t words, uint32_t B)
{
    const uint32_t l = PULL_NW * warp_region_bytes(words, B), h = heavy_region_bytes(words, B);
    return l > h ? l : h;
}

__device__ __forceinline__ WarpRegion warp_region(unsigned char *base, uint32_t words, uint32_t B, int w)
{
    unsigned char *p = base + (size_t)w * warp_region_bytes(words, B);
    WarpRegion r;
    r.ind = reinterpret_cast<uint32_t *>(p);
    p += align16(words * 4);
    r.sh = reinterpret_cast<uint32_t *>(p);
    p += SMALL_CAP * 4;
    r.ctr = reinterpret_cast<uint32_t *>(p);
    p += 16;
    r.offered = reinterpret_cast<uint16_t *>(p);
    p += align16(B * 2);
    r.sd = p;
    return r;
}

struct HeavyRegion {
    uint32_t *ind;
    uint32_t *sh;
    uint16_t *offered;
    uint16_t *surv;
    uint8_t *sd;
    uint32_t *ctr;                   // noff, nsurv, nsmall, nadd, mn, ok, reloc, ncap, nsurv2
    unsigned long long *base;
};

__device__ __forceinline__ HeavyRegion heavy_region(unsigned char *p, uint32_t words, uint32_t B)
{
    HeavyRegion r;
    r.base = reinterpret_cast<unsigned long long *>(p);
    p += 16;
    r.ctr = reinterpret_cast<uint32_t *>(p);
    p += 48;
    r.ind = reinterpret_cast<uint32_t *>(p);
    p += align16(words * 4);
    r.sh = reinterpret_cast<uint32_t *>(p);
    p += HSMALL_CAP * 4;
    r.offered = reinterpret_cast<uint16_t *>(p);
    p += align16(B * 2);
    r.surv = reinterpret_cast<uint16_t *>(p);
    p += align16(B * 2);
    r.sd = p;
    return r;
}

// BP test of one (root, tail) pair on BP root i only.
__device__ __forceinline__ bool bp_one(uint8_t rd, ulonglong2 rs, uint8_t td, ulonglong2 ts, uint32_t iter)
{
    uint32_t x = (uint32_t)rd + (uint32_t)td;
    if (x - 2u > iter) return false;
    if (rs.x & ts.x)
        x -= 2u;
    else if ((rs.x & ts.y) | (rs.y & ts.x))
        x -= 1u;
    return x <= iter;
}

// Warp-cooperative BP test of candidate root r against the tail's row held in
// registers (lane i holds BP roots i and i + 32); roots < skip were already
// tested.  Pruned iff any root covers the pair -- order-independent.  The
// candidate's distances and sets are loaded in one round.
__device__ __forceinline__ bool bp_covered_warp(const UnwDev &d, uint32_t r, int lane, uint32_t skip, uint8_t td0,
                                                ulonglong2 ts0, uint8_t td1, ulonglong2 ts1, uint32_t iter)
{
    const uint8_t *rd = d.bpd + (uint64_t)r * d.K;
    const ulonglong2 *rs = reinterpret_cast<const ulonglong2 *>(d.bps + (uint64_t)r * d.K * 2);
    const uint32_t i0 = lane, i1 = lane + 32;
    const bool v0 = i0 >= skip && i0 < d.K, v1 = i1 >= skip && i1 < d.K;
    const ulonglong2 z = make_ulonglong2(0, 0);
    const uint8_t a0 = v0 ? rd[i0] : (uint8_t)U8_INF, a1 = v1 ? rd[i1] : (uint8_t)U8_INF;
    const ulonglong2 s0 = v0 ? rs[i0] : z, s1 = v1 ? rs[i1] : z;
    const bool cov = (v0 && bp_one(a0, s0, td0, ts0, iter)) || (v1 && bp_one(a1, s1, td1, ts1, iter));
    return __ballot_sync(FULL, cov) != 0;
}

// Warp-cooperative BP test of up to BP_GROUP candidates at once (the first
// `nc` of r[]): each candidate's distances and the 16-byte sets of lane i's
// two roots are loaded in one round (1 KB per candidate at K = 64), then
// tested.  On social graphs nearly every pair that reaches this stage needs
// most roots' sets, so loading them with the distances saves a round trip per
// candidate; one candidate per step keeps the loop kernel free of register
// spills.  Bit c of the result: r[c] covered.
constexpr int BP_GROUP = 1;
__device__ __forceinline__ uint32_t bp_covered_group(const UnwDev &d, const uint32_t (&r)[BP_GROUP], uint32_t nc,
                                                     int lane, uint32_t skip, uint8_t td0, ulonglong2 ts0, uint8_t td1,
                                                     ulonglong2 ts1, uint32_t iter)
{
    const uint32_t K = d.K, i0 = lane, i1 = lane + 32;
    const bool v0 = i0 >= skip && i0 < K, v1 = i1 >= skip && i1 < K;
    const ulonglong2 z = make_ulonglong2(0, 0);
    uint32_t x0[BP_GROUP], x1[BP_GROUP];
    ulonglong2 s0[BP_GROUP], s1[BP_GROUP];
#pragma unroll
    for (int c = 0; c < BP_GROUP; ++c) {
        const bool in = (uint32_t)c < nc;
        const uint8_t *rd = d.bpd + (uint64_t)r[c] * K;
        const ulonglong2 *rs = reinterpret_cast<const ulonglong2 *>(d.bps) + (uint64_t)r[c] * K;
        x0[c] = in && v0 ? (uint32_t)rd[i0] + td0 : 0u;  // 0: fails the test like x < 2 does
        x1[c] = in && v1 ? (uint32_t)rd[i1] + td1 : 0u;
        s0[c] = in && v0 ? rs[i0] : z;
        s1[c] = in && v1 ? rs[i1] : z;
    }
    auto cut = [&](uint32_t x, ulonglong2 rs, ulonglong2 ts) {
        if (x - 2u > iter) return false;
        if (rs.x & ts.x)
            x -= 2u;
        else if ((rs.x & ts.y) | (rs.y & ts.x))
            x -= 1u;
        return x <= iter;
    };
    uint32_t res = 0;
#pragma unroll
    for (int c = 0; c < BP_GROUP; ++c)
        if (__ballot_sync(FULL, cut(x0[c], s0[c], ts0) || cut(x1[c], s1[c], ts1))) res |= 1u << c;
    return res;
}

struct PullArgs {
    const uint32_t *tails;        // light tails
    const uint32_t *tails_cnt;
    const uint32_t *htails;       // heavy tails
    const uint32_t *htails_cnt;
    uint32_t s, e_roots, b, iter, lid_cur;
    uint32_t *front_next;
    uint32_t *front_next_cnt;
    uint32_t *retry;
    uint32_t *retry_cnt;
    const GDesc *gd = nullptr;       // many-graph labeling: per-graph state ...
    const uint16_t *gmap = nullptr;  // ... and the graph of each vertex
    GDesc *gd_mut = nullptr;         // the same array, for the per-graph counters
    // Fused marking (persistent one-graph loop): a tail that gains labels marks
    // its own tails for the next level right away (stamp next_stamp) instead of
    // joining front_next for a separate mark phase.
    uint32_t *next_tails = nullptr, *next_tails_cnt = nullptr;
    uint32_t *next_htails = nullptr, *next_htails_cnt = nullptr;
    uint32_t next_stamp = 0;
    uint8_t *dm = nullptr;           // dist_matrix of the current batch (default d.dm)
    // Work counters for dynamic assignment (zero at the start of the level):
    // warps / blocks claim the next light / heavy tail from them, so that the
    // level ends when the work runs out rather than when the unluckiest
    // static share is done.  Null: static grid-stride assignment.
    uint32_t *tail_q = nullptr, *htail_q = nullptr;
};

// The batch a tail belongs to: roots [s, e), batch id b, level iter, and its
// graph's dist_matrix rows (entry for root idx, hub h: dm[idx * dn + h - base]).
struct BatchCtx {
    uint32_t s, e, b, iter, base, dn;
    uint8_t *dm;
    uint32_t g;
};

__device__ __forceinline__ BatchCtx tail_ctx(const UnwDev &d, const PullArgs &a, uint32_t t)
{
    if (!a.gmap) return BatchCtx{a.s, a.e_roots, a.b, a.iter, 0u, d.n, a.dm ? a.dm : d.dm, 0u};
    const uint32_t g = a.gmap[t];
    const GDesc &x = a.gd[g];
    return BatchCtx{gd_u32(x.s),    gd_u32(x.e), gd_u32(x.b),
                    gd_u32(x.iter), x.base,      x.n,
                    d.dm + x.dm_off + (uint64_t)gd_u32(x.dmp) * d.B * x.n, g};
}

// Marks the tails of head h for the level stamped `stamp`: neighbours t > mn
// (descending list, so the scan stops at the first t <= mn) that are not BP
// vertices, each once per level (tail stamp), into the light or heavy list.
// A warp scans 32 entries per step; warp w of `nw` starts at chunk w.
__device__ __forceinline__ void mark_tails(const UnwDev &d, uint32_t h, uint32_t mn, uint32_t stamp, uint32_t *tails,
                                           uint32_t *tails_cnt, uint32_t *htails, uint32_t *htails_cnt, int lane,
                                           uint32_t w, uint32_t nw, unsigned long long &bytes,
                                           uint32_t *gcnt = nullptr)
{
    const uint32_t e_end = UD_AT(d.off, h + 1, (uint64_t)d.n + 1, 0);
    for (uint32_t e0 = UD_AT(d.off, h, (uint64_t)d.n + 1, 0) + 32 * w; e0 < e_end; e0 += 32 * nw) {
        const uint32_t e = e0 + lane;
        const bool in = e < e_end;
        const uint32_t t = in ? UD_AT(d.adj, e, d.m, 0) : 0u;
        const bool ok = in && t > mn;
        if (d.work) bytes += __popc(__ballot_sync(FULL, in)) * 4ull + __popc(__ballot_sync(FULL, ok)) * 5ull;
        bool appended = false;
        // flags and stamp are independent loads: one round trip
        const uint32_t f = ok ? UD_AT(d.used, t, d.n, 1) : 1u;
        const uint32_t ts = ok ? UD_AT(d.tail_stamp, t, d.n, 1) : stamp;
        if (!(f & 1u) && ts != stamp) {
            if (atomicExch(&UD_AT(d.tail_stamp, t, d.n, 1), stamp) != stamp) {
                if (f & 2u)
                    UD_AT(htails, agg_append_by(htails_cnt, 1u), d.n, 6) = t;
                else
                    UD_AT(tails, agg_append_by(tails_cnt, 0u), d.n, 6) = t;
                appended = true;
            }
        }
        if (gcnt || d.work) {
            const uint32_t na = __popc(__ballot_sync(FULL, appended));
            bytes += na * 8ull;
            if (gcnt && na && lane == 0) atomicAdd(gcnt, na);  // the head's graph's tails for this stamp
        }
        if (__ballot_sync(FULL, in && !ok)) break;
    }
}

// One heavy tail, processed by the whole block.
__device__ void pull_heavy_tail(const UnwDev &d, const PullArgs &a, uint32_t t, HeavyRegion &hs,
                                unsigned long long &bytes)
{
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const BatchCtx bc = tail_ctx(d, a, t);
    const uint32_t s = bc.s, iter = bc.iter;
    const int pp = (a.lid_cur - 1) & 1, cp = a.lid_cur & 1;
    const uint32_t lid_prev = a.lid_cur - 1;
    const bool valid = UD_AT(d.ind_stamp, t, d.n, 1) == bc.b + 1;
    for (uint32_t x = tid; x < d.words; x += blockDim.x) hs.ind[x] = valid ? UD_AT(d.ind, (uint64_t)t * d.words + x, (uint64_t)d.n * d.words, 5) : 0u;
    if (tid < 9) hs.ctr[tid] = (tid == 4) ? 0xffffffffu : 0u;
    if (tid == 0) bytes += 8 + 8ull * d.words;
    __syncthreads();
    // (a) first offers from active neighbours, warps striding over the list
    const uint32_t e_end = UD_AT(d.off, t + 1, (uint64_t)d.n + 1, 0);
    for (uint32_t e0 = UD_AT(d.off, t, (uint64_t)d.n + 1, 0) + 32 * warp; e0 < e_end; e0 += 32 * (blockDim.x >> 5)) {
        const uint32_t e = e0 + lane;
        const bool in = e < e_end;
        const uint32_t h = in ? UD_AT(d.adj, e, d.m, 0) : 0u;
        const bool ge = in && h >= s;
        const LastGroup lg = ge ? UD_AT(d.last[pp], h, d.n, 1) : LastGroup{0ull, 0u, 0u};
        const bool act = ge && lg.stamp == lid_prev;
        uint32_t mask = __ballot_sync(FULL, act);
        if (lane == 0) bytes += __popc(__ballot_sync(FULL, in)) * 4ull + __popc(__ballot_sync(FULL, ge)) * 4ull;
        else { __ballot_sync(FULL, in); __ballot_sync(FULL, ge); }
        const uint64_t mpos = act ? lg.pos : 0ull;
        const uint32_t mcnt = act ? lg.cnt : 0u;
        while (mask) {
            const int src = __ffs(mask) - 1;
            mask &= mask - 1;
            const uint64_t pos = __shfl_sync(FULL, mpos, src);
            const uint32_t c = __shfl_sync(FULL, mcnt, src);
            if (lane == 0) bytes += 12 + 4ull * c;
            for (uint32_t j = lane; j < c; j += 32) {
                const uint32_t r = UD_AT(d.pool_hub, pos + j, d.pool_cap, 2);
                if (r < t) {
                    const uint32_t idx = r - s;
                    const uint32_t bit = 1u << (idx & 31);
                    const uint32_t old = atomicOr(&hs.ind[idx >> 5], bit);
                    if (!(old & bit)) hs.offered[atomicAdd(&hs.ctr[0], 1u)] = (uint16_t)idx;
                }
            }
        }
        if (__ballot_sync(FULL, in && !ge)) break;  // descending list: the rest are < s
    }
    __syncthreads();
    const uint32_t noff = hs.ctr[0];
    if (noff == 0) return;  // uniform: nothing changed
    if (d.work && tid == 0) atomicAdd(&d.work[W_EV_OFFERS], (unsigned long long)noff);
    // (b) BP test: thread per candidate on BP root 0, then warps take the
    // survivors one at a time over the remaining roots.
    if (tid == 0) bytes += 17ull * d.K;
    const ulonglong2 zero2 = make_ulonglong2(0, 0);
    const uint8_t td0 = lane < (int)d.K ? UD_AT(d.bpd, (uint64_t)t * d.K + lane, (uint64_t)d.n * d.K, 3) : (uint8_t)U8_INF;
    const uint8_t td1 = lane + 32 < (int)d.K ? UD_AT(d.bpd, (uint64_t)t * d.K + lane + 32, (uint64_t)d.n * d.K, 3) : (uint8_t)U8_INF;
    const ulonglong2 ts0 = lane < (int)d.K ? UD_AT(reinterpret_cast<const ulonglong2 *>(d.bps), (uint64_t)t * d.K + lane, (uint64_t)d.n * d.K, 3) : zero2;
    const ulonglong2 ts1 =
        lane + 32 < (int)d.K ? UD_AT(reinterpret_cast<const ulonglong2 *>(d.bps), (uint64_t)t * d.K + lane + 32, (uint64_t)d.n * d.K, 3) : zero2;
    const uint8_t tr0d = __shfl_sync(FULL, td0, 0);
    const ulonglong2 tr0s = make_ulonglong2(__shfl_sync(FULL, ts0.x, 0), __shfl_sync(FULL, ts0.y, 0));
    const uint32_t tmin = d.K ? UD_AT(d.bpmin, t, d.n, 1) : (uint32_t)U8_INF;
    for (uint32_t c = tid; c < noff; c += blockDim.x) {
        const uint16_t idx = hs.offered[c];
        const uint64_t rr = s + idx;
        if (d.K == 0 || (uint32_t)UD_AT(d.bpmin, rr, d.n, 1) + tmin > iter + 2u)  // cannot be covered: no second stage
            hs.surv[atomicAdd(&hs.ctr[1], 1u)] = idx | 0x8000u;
        else if (!bp_one(UD_AT(d.bpd, rr * d.K, (uint64_t)d.n * d.K, 3), UD_AT(reinterpret_cast<const ulonglong2 *>(d.bps), rr * d.K, (uint64_t)d.n * d.K, 3), tr0d, tr0s, iter))
            hs.surv[atomicAdd(&hs.ctr[1], 1u)] = idx;
    }
    __syncthreads();
    // every thread reads the count before anything changes it; the second
    // stage counts its survivors in a slot of its own (ctr[8])
    const uint32_t nsurv1 = hs.ctr[1];
    uint32_t nsurv = nsurv1;
    if (d.K > 1 && nsurv1) {
        for (uint32_t c = warp; c < nsurv1; c += blockDim.x >> 5) {
            const uint16_t ent = hs.surv[c];
            const uint16_t idx = ent & 0x7fffu;
            const bool cov = !(ent & 0x8000u) && bp_covered_warp(d, s + idx, lane, 1, td0, ts0, td1, ts1, iter);
            if (!cov && lane == 0) hs.offered[atomicAdd(&hs.ctr[8], 1u)] = idx;
        }
        __syncthreads();
        // survivors now sit in `offered`; move them back for the distance test
        const uint32_t ns2 = hs.ctr[8];
        for (uint32_t c = tid; c < ns2; c += blockDim.x) hs.surv[c] = hs.offered[c];
        __syncthreads();
        nsurv = ns2;
    } else {
        for (uint32_t c = tid; c < nsurv1; c += blockDim.x) hs.surv[c] &= 0x7fffu;
        __syncthreads();
    }
    const uint32_t len = UD_AT(d.lab_len, t, d.n, 1);
    const uint64_t base = UD_AT(d.lab_off, t, d.n, 1);
    // (c) distance test
    if (nsurv) {
        for (uint32_t j = tid; j < len; j += blockDim.x) {
            const uint8_t dd = UD_AT(d.pool_dist, base + j, d.pool_cap, 2);
            if (dd < iter) {
                const uint32_t slot = atomicAdd(&hs.ctr[2], 1u);
                if (slot < HSMALL_CAP) {
                    hs.sh[slot] = UD_AT(d.pool_hub, base + j, d.pool_cap, 2);
                    hs.sd[slot] = dd;
                }
            }
        }
        __syncthreads();
        const uint32_t nsmall = hs.ctr[2];
        if (tid == 0) bytes += 12 + (uint64_t)len + 4ull * min(nsmall, (uint32_t)HSMALL_CAP) + (uint64_t)nsurv * nsmall;
        for (uint32_t c = tid; c < nsurv; c += blockDim.x) {
            const uint16_t idx = hs.surv[c];
            const uint32_t rr = s + idx;
            const uint8_t *row = bc.dm + (uint64_t)idx * bc.dn;
            bool keep = true;
            if (nsmall <= HSMALL_CAP) {
                for (uint32_t k = 0; k < nsmall; ++k) {
                    const uint32_t hh = hs.sh[k];
                    if (hh < rr && (uint32_t)hs.sd[k] + (uint32_t)UD_AT(row, hh - bc.base, bc.dn, 4) <= iter) { keep = false; break; }
                }
            } else {
                for (uint32_t j = 0; j < len; ++j) {
                    const uint32_t dd = UD_AT(d.pool_dist, base + j, d.pool_cap, 2);
                    if (dd >= iter) continue;
                    const uint32_t hh = UD_AT(d.pool_hub, base + j, d.pool_cap, 2);
                    if (hh < rr && dd + (uint32_t)UD_AT(row, hh - bc.base, bc.dn, 4) <= iter) { keep = false; break; }
                }
            }
            if (keep) hs.offered[atomicAdd(&hs.ctr[3], 1u)] = idx;
        }
        __syncthreads();
    }
    const uint32_t nadd = hs.ctr[3];
    if (nadd) {
        // (d) reserve, relocating if the slot is too small
        if (tid == 0) {
            const uint32_t cap = UD_AT(d.lab_cap, t, d.n, 1), need = len + nadd;
            hs.ctr[5] = 1;
            hs.ctr[6] = 0;
            *hs.base = base;
            if (need > cap) {
                uint32_t ncap = max(max(2u * cap, need), 8u);
                ncap = (ncap + 7u) & ~7u;
                const unsigned long long pos = atomicAdd(d.pool_top, (unsigned long long)ncap);
                if (pos + ncap > d.pool_cap) {
                    hs.ctr[5] = 0;
                } else {
                    hs.ctr[6] = 1;
                    hs.ctr[7] = ncap;
                    *hs.base = pos;
                }
            }
        }
        __syncthreads();
        if (!hs.ctr[5]) {
            if (tid == 0) {
                atomicOr(d.status, ST_POOL_RETRY);
                UD_AT(a.retry, atomicAdd(a.retry_cnt, 1u), d.n, 6) = t;
            }
            return;  // uniform; nothing committed
        }
        const uint64_t nbase = *hs.base;
        if (hs.ctr[6]) {
            for (uint32_t j = tid; j < len; j += blockDim.x) {
                UD_AT(d.pool_hub, nbase + j, d.pool_cap, 2) = UD_AT(d.pool_hub, base + j, d.pool_cap, 2);
                UD_AT(d.pool_dist, nbase + j, d.pool_cap, 2) = UD_AT(d.pool_dist, base + j, d.pool_cap, 2);
            }
        }
        const bool is_root = t >= s && t < bc.e;
        for (uint32_t j = tid; j < nadd; j += blockDim.x) {
            const uint32_t idx = hs.offered[j];
            UD_AT(d.pool_hub, nbase + len + j, d.pool_cap, 2) = s + idx;
            UD_AT(d.pool_dist, nbase + len + j, d.pool_cap, 2) = (uint8_t)iter;
            if (is_root) UD_AT(bc.dm, (uint64_t)(t - s) * bc.dn + (s + idx - bc.base), (uint64_t)d.B * bc.dn, 4) = (uint8_t)iter;
            atomicMin(&hs.ctr[4], s + idx);
        }
        __syncthreads();
        if (tid == 0) {
            if (d.work) atomicAdd(&d.work[W_EV_LABELS], (unsigned long long)nadd);
            if (hs.ctr[6]) {
                UD_AT(d.lab_off, t, d.n, 1) = nbase;
                UD_AT(d.lab_cap, t, d.n, 1) = hs.ctr[7];
            }
            UD_AT(d.lab_len, t, d.n, 1) = len + nadd;
            UD_AT(d.last[cp], t, d.n, 1) = LastGroup{nbase + len, nadd, a.lid_cur};
            UD_AT(d.last_min[cp], t, d.n, 1) = hs.ctr[4];
            if (!a.next_tails) UD_AT(a.front_next, atomicAdd(a.front_next_cnt, 1u), d.n, 6) = t;
            bytes += 5ull * nadd + 28 + (is_root ? (uint64_t)nadd : 0) + (hs.ctr[6] ? 10ull * len : 0);
        }
        if (a.next_tails)
            mark_tails(d, t, hs.ctr[4], a.next_stamp, a.next_tails, a.next_tails_cnt, a.next_htails,
                       a.next_htails_cnt, lane, warp, blockDim.x >> 5, bytes,
                       a.gd_mut ? &a.gd_mut[bc.g].tc[a.next_stamp % 3] : nullptr);
    }
    for (uint32_t x = tid; x < d.words; x += blockDim.x) UD_AT(d.ind, (uint64_t)t * d.words + x, (uint64_t)d.n * d.words, 5) = hs.ind[x];
    if (tid == 0) UD_AT(d.ind_stamp, t, d.n, 1) = bc.b + 1;
}

// One light tail, processed by one warp.
__device__ void pull_light_tail(const UnwDev &d, const PullArgs &a, uint32_t t, WarpRegion &wr,
                                unsigned long long &bytes)
{
    const int lane = threadIdx.x & 31;
    long long c0 = d.work ? clock64() : 0, c1 = 0;
    // phase clock: adds the cycles since the last mark to slot `w` (profiling only)
    auto tick = [&](int w) {
        if (d.work) {
            c1 = clock64();
            if (lane == 0) atomicAdd(&d.work[w], (unsigned long long)(c1 - c0));
            c0 = c1;
        }
    };
    const BatchCtx bc = tail_ctx(d, a, t);
    const uint32_t s = bc.s, iter = bc.iter;
    const int pp = (a.lid_cur - 1) & 1, cp = a.lid_cur & 1;
    const uint32_t lid_prev = a.lid_cur - 1;
    bytes += 8 + 4ull * d.words;  // tail entry, indicator stamp and row
    // (a) indicator row of t for this batch
    const bool valid = UD_AT(d.ind_stamp, t, d.n, 1) == bc.b + 1;
    for (uint32_t x = lane; x < d.words; x += 32) wr.ind[x] = valid ? UD_AT(d.ind, (uint64_t)t * d.words + x, (uint64_t)d.n * d.words, 5) : 0u;
    uint32_t noff = 0;  // first offers so far, in wr.offered
    __syncwarp();
    // (b) gather first offers from active neighbours (heads >= s), 64
    // neighbours per step.  The hubs of all active heads' last groups are
    // flattened into one item list (inclusive counts sa / sb over the two
    // halves) and spread over the lanes, so one round of loads covers 32 hubs
    // whichever heads they belong to.
    const uint32_t e_end = UD_AT(d.off, t + 1, (uint64_t)d.n + 1, 0);
    for (uint32_t e0 = UD_AT(d.off, t, (uint64_t)d.n + 1, 0); e0 < e_end; e0 += 64) {
        const uint32_t ea = e0 + lane, eb = ea + 32;
        const bool ina = ea < e_end, inb = eb < e_end;
        const uint32_t ha = ina ? UD_AT(d.adj, ea, d.m, 0) : 0u, hb = inb ? UD_AT(d.adj, eb, d.m, 0) : 0u;
        const bool gea = ina && ha >= s, geb = inb && hb >= s;
        // every head's newest group (stamp, position, size): one load each, in parallel
        const LastGroup la = gea ? UD_AT(d.last[pp], ha, d.n, 1) : LastGroup{0ull, 0u, 0u};
        const LastGroup lb = geb ? UD_AT(d.last[pp], hb, d.n, 1) : LastGroup{0ull, 0u, 0u};
        const bool acta = gea && la.stamp == lid_prev, actb = geb && lb.stamp == lid_prev;
        const uint64_t pa = acta ? la.pos : 0ull, pb = actb ? lb.pos : 0ull;
        const uint32_t ca = acta ? la.cnt : 0u, cb = actb ? lb.cnt : 0u;
        uint32_t sa = ca, sb = cb;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t ya = __shfl_up_sync(FULL, sa, o), yb = __shfl_up_sync(FULL, sb, o);
            if (lane >= o) {
                sa += ya;
                sb += yb;
            }
        }
        const uint32_t ta = __shfl_sync(FULL, sa, 31), tot = ta + __shfl_sync(FULL, sb, 31);
        if (d.work)
            bytes += __popc(__ballot_sync(FULL, ina)) * 4ull + __popc(__ballot_sync(FULL, gea)) * 4ull +
                 __popc(__ballot_sync(FULL, inb)) * 4ull + __popc(__ballot_sync(FULL, geb)) * 4ull +
                 12ull * (__popc(__ballot_sync(FULL, acta)) + __popc(__ballot_sync(FULL, actb))) + 4ull * tot;
        for (uint32_t i0 = 0; i0 < tot; i0 += 32) {
            const uint32_t i = i0 + lane;
            const bool second = i >= ta;
            const uint32_t key = second ? i - ta : i;
            // head lane: the number of lanes of the half whose inclusive count is <= key
            uint32_t L = 0;
#pragma unroll
            for (uint32_t step = 16; step > 0; step >>= 1) {
                const uint32_t va = __shfl_sync(FULL, sa, L + step - 1), vb = __shfl_sync(FULL, sb, L + step - 1);
                if ((second ? vb : va) <= key) L += step;
            }
            const uint64_t qa = __shfl_sync(FULL, pa, L), qb = __shfl_sync(FULL, pb, L);
            const uint32_t xa = __shfl_sync(FULL, sa - ca, L), xb = __shfl_sync(FULL, sb - cb, L);
            bool fresh = false;
            uint32_t idx = 0;
            if (i < tot) {
                const uint32_t r = UD_AT(d.pool_hub, (second ? qb : qa) + (key - (second ? xb : xa)), d.pool_cap, 2);
                if (r < t) {
                    idx = r - s;
                    const uint32_t bit = 1u << (idx & 31);
                    fresh = !(atomicOr(&wr.ind[idx >> 5], bit) & bit);
                }
            }
            // first offers of this round appended in lane order (no shared counter)
            const uint32_t fm = __ballot_sync(FULL, fresh);
            if (fresh) wr.offered[noff + __popc(fm & ((1u << lane) - 1u))] = (uint16_t)idx;
            noff += __popc(fm);
        }
        // descending list: once a neighbour is < s, the rest are too
        if (__ballot_sync(FULL, (ina && !gea) || (inb && !geb))) break;
    }
    __syncwarp();
    tick(W_CYC_SCAN);
    if (noff == 0) return;
    if (d.work && lane == 0) atomicAdd(&d.work[W_EV_OFFERS], (unsigned long long)noff);
    bytes += 17ull + 4ull * d.words + 4;  // tail root-0 BP entry; indicator write-back
    // (c) BP test in two stages: lane per candidate on BP root 0 (which settles
    // most pairs), then warp-cooperative over the remaining roots for the rest.
    const ulonglong2 zero2 = make_ulonglong2(0, 0);
    // Any root i gives td_i >= bpmin[r] + bpmin[t], so a pair with
    // bpmin[r] + bpmin[t] - 2 > iter cannot be covered: it survives BP without
    // a row load (flag 0x8000: no second stage).
    const uint32_t tmin = d.K ? UD_AT(d.bpmin, t, d.n, 1) : (uint32_t)U8_INF;
    uint32_t nsurv = 0;
    bool need2 = false;  // some survivor needs the second stage
    for (uint32_t c0 = 0; c0 < noff; c0 += 32) {
        const uint32_t c = c0 + lane;
        bool keep = false;
        uint16_t ent = 0;
        if (c < noff) {
            const uint16_t idx = wr.offered[c];
            const uint64_t rr = s + idx;
            // the candidate's and the tail's root-0 entries (the latter the same
            // address in every lane) are independent loads: one round trip
            const uint32_t bm = d.K ? UD_AT(d.bpmin, rr, d.n, 1) : (uint32_t)U8_INF;
            const uint8_t r0d = d.K ? UD_AT(d.bpd, rr * d.K, (uint64_t)d.n * d.K, 3) : (uint8_t)U8_INF;
            const ulonglong2 r0s = d.K ? UD_AT(reinterpret_cast<const ulonglong2 *>(d.bps), rr * d.K, (uint64_t)d.n * d.K, 3) : zero2;
            const uint8_t t0d = d.K ? UD_AT(d.bpd, (uint64_t)t * d.K, (uint64_t)d.n * d.K, 3) : (uint8_t)U8_INF;
            const ulonglong2 t0s = d.K ? UD_AT(reinterpret_cast<const ulonglong2 *>(d.bps), (uint64_t)t * d.K, (uint64_t)d.n * d.K, 3) : zero2;
            if (d.K == 0 || bm + tmin > iter + 2u) {
                keep = true;
                ent = idx | 0x8000u;
            } else {
                keep = !bp_one(r0d, r0s, t0d, t0s, iter);
                ent = idx;
            }
        }
        const uint32_t km = __ballot_sync(FULL, keep);
        need2 = need2 || __any_sync(FULL, keep && !(ent & 0x8000u));
        __syncwarp();
        if (keep) wr.offered[nsurv + __popc(km & ((1u << lane) - 1u))] = ent;
        nsurv += __popc(km);
        __syncwarp();
    }
    if (d.K > 1 && need2) {
        // second stage for the unflagged survivors, two candidates per step,
        // against t's whole row (lane i: roots i and i + 32), loaded only now
        const uint8_t td0 = lane < (int)d.K ? UD_AT(d.bpd, (uint64_t)t * d.K + lane, (uint64_t)d.n * d.K, 3) : (uint8_t)U8_INF;
        const uint8_t td1 = lane + 32 < (int)d.K ? UD_AT(d.bpd, (uint64_t)t * d.K + lane + 32, (uint64_t)d.n * d.K, 3) : (uint8_t)U8_INF;
        const ulonglong2 ts0 =
            lane < (int)d.K ? UD_AT(reinterpret_cast<const ulonglong2 *>(d.bps), (uint64_t)t * d.K + lane, (uint64_t)d.n * d.K, 3) : zero2;
        const ulonglong2 ts1 =
            lane + 32 < (int)d.K ? UD_AT(reinterpret_cast<const ulonglong2 *>(d.bps), (uint64_t)t * d.K + lane + 32, (uint64_t)d.n * d.K, 3) : zero2;
        bytes += 17ull * (d.K - 1);
        uint32_t n2 = 0;
        for (uint32_t c0 = 0; c0 < nsurv; c0 += 32) {
            const uint32_t c = c0 + lane;
            const bool in = c < nsurv;
            const uint16_t ent = in ? wr.offered[c] : (uint16_t)0;
            uint32_t need = __ballot_sync(FULL, in && !(ent & 0x8000u));
            bool covered = false;
            while (need) {
                int kk[BP_GROUP];
                uint32_t rg[BP_GROUP], nc = 0;
#pragma unroll
                for (int g = 0; g < BP_GROUP; ++g) {
                    kk[g] = need ? __ffs(need) - 1 : 0;
                    if (need) {
                        need &= need - 1;
                        ++nc;
                    }
                    rg[g] = s + (__shfl_sync(FULL, (uint32_t)ent, kk[g]) & 0x7fffu);
                }
                const uint32_t cov = bp_covered_group(d, rg, nc, lane, 1, td0, ts0, td1, ts1, iter);
#pragma unroll
                for (int g = 0; g < BP_GROUP; ++g)
                    if ((uint32_t)g < nc && lane == kk[g] && (cov >> g & 1u)) covered = true;
            }
            const bool keep = in && !covered;
            const uint32_t km = __ballot_sync(FULL, keep);
            __syncwarp();
            if (keep) wr.offered[n2 + __popc(km & ((1u << lane) - 1u))] = ent & 0x7fffu;
            n2 += __popc(km);
            __syncwarp();
        }
        nsurv = n2;
    } else {
        for (uint32_t c = lane; c < nsurv; c += 32) wr.offered[c] &= 0x7fffu;
        __syncwarp();
    }
    tick(W_CYC_BP);
    // (d) distance test against t's labels with d < iter.  Those labels are
    // staged in shared memory as (hub, slack = iter - d) SMALL_CAP at a time
    // (ballot compaction, in list order); when they all fit, one staging
    // serves every candidate group.
    uint32_t nadd = 0;
    const uint32_t len = UD_AT(d.lab_len, t, d.n, 1);
    uint64_t base = UD_AT(d.lab_off, t, d.n, 1);
    if (nsurv) {
        uint32_t nst = 0;
        // stage labels with d < iter from list position `from`; returns where it stopped
        auto stage = [&](uint32_t from) -> uint32_t {
            uint32_t cnt = 0, j = from;
            for (; j < len && cnt + 32 <= (uint32_t)SMALL_CAP; j += 32) {
                const uint32_t jj = j + lane;
                const bool in = jj < len;
                // hub and distance are independent loads: one round trip
                const uint8_t dd = in ? UD_AT(d.pool_dist, base + jj, d.pool_cap, 2) : (uint8_t)U8_INF;
                const uint32_t hb = in ? UD_AT(d.pool_hub, base + jj, d.pool_cap, 2) : 0u;
                const bool sm = in && dd < iter;
                const uint32_t m = __ballot_sync(FULL, sm);
                if (sm) {
                    const uint32_t p = cnt + __popc(m & ((1u << lane) - 1u));
                    wr.sh[p] = hb;
                    wr.sd[p] = (uint8_t)(iter - dd);  // slack: covered iff d(r, h) <= slack
                }
                cnt += __popc(m);
            }
            __syncwarp();
            nst = cnt;
            bytes += (uint64_t)min(j, len) - from + 4ull * cnt;
            return min(j, len);
        };
        uint32_t next = stage(0);
        const bool whole = next >= len;
        bytes += 12;
        for (uint32_t c0 = 0; c0 < nsurv; c0 += 32) {
            const uint32_t c = c0 + lane;
            bool keep = c < nsurv;
            const uint16_t idx = keep ? wr.offered[c] : (uint16_t)0;
            const uint32_t rr = s + idx;
            const uint8_t *row = bc.dm + (uint64_t)idx * bc.dn - bc.base;  // row[h] for a hub h of this graph
            if (!whole && c0 > 0) next = stage(0);
            for (;;) {
                const uint32_t nk = __popc(__ballot_sync(FULL, keep));
                if (nst >= WALK_MIN_STAGED && nk <= WALK_MAX_CANDIDATES) {
                    // a staged list of WALK_MIN_STAGED or more entries: each
                    // pending candidate walks it with 32 entries across the
                    // lanes (a ballot per candidate and chunk), four
                    // candidates' gathers in flight per step; a candidate
                    // leaves at the chunk that covers it
                    uint32_t pend = __ballot_sync(FULL, keep);
                    const uint64_t rl = (uint64_t)bc.base + bc.dn;
                    for (uint32_t k0 = 0; k0 < nst && pend; k0 += 32) {
                        const bool in = k0 + lane < nst;
                        const uint32_t hl = in ? wr.sh[k0 + lane] : 0xffffffffu;
                        const uint32_t sl = in ? (uint32_t)wr.sd[k0 + lane] : 0u;
                        uint32_t todo = pend;
                        while (todo) {
                            int jj[4];
                            uint32_t vv[4];
                            bool ok[4];
#pragma unroll
                            for (int u = 0; u < 4; ++u) {
                                jj[u] = todo ? __ffs(todo) - 1 : -1;
                                todo &= todo - 1;  // (0 stays 0)
                            }
#pragma unroll
                            for (int u = 0; u < 4; ++u) {
                                const uint32_t ix = __shfl_sync(FULL, (uint32_t)idx, jj[u] & 31);
                                const uint8_t *rw = bc.dm + (uint64_t)ix * bc.dn - bc.base;
                                ok[u] = jj[u] >= 0 && in && hl < s + ix;
                                vv[u] = ok[u] ? (uint32_t)UD_AT(rw, hl, rl, 4) : 255u;
                            }
#pragma unroll
                            for (int u = 0; u < 4; ++u)
                                if (__ballot_sync(FULL, ok[u] && vv[u] <= sl)) pend &= ~(1u << jj[u]);
                        }
                    }
                    keep = keep && ((pend >> lane) & 1u);
                } else if (keep) {
                    uint32_t k = 0;
                    // four dist_matrix gathers in flight per lane
                    for (; k + 4 <= nst; k += 4) {
                        const uint32_t h0 = wr.sh[k], h1 = wr.sh[k + 1], h2 = wr.sh[k + 2], h3 = wr.sh[k + 3];
                        const uint64_t rl = (uint64_t)bc.base + bc.dn;
                        const uint32_t v0 = UD_AT(row, h0, rl, 4), v1 = UD_AT(row, h1, rl, 4), v2 = UD_AT(row, h2, rl, 4),
                                       v3 = UD_AT(row, h3, rl, 4);
                        if ((h0 < rr && v0 <= wr.sd[k]) || (h1 < rr && v1 <= wr.sd[k + 1]) ||
                            (h2 < rr && v2 <= wr.sd[k + 2]) || (h3 < rr && v3 <= wr.sd[k + 3])) {
                            keep = false;
                            break;
                        }
                    }
                    for (; keep && k < nst; ++k) {
                        const uint32_t hh = wr.sh[k];
                        if (hh < rr && (uint32_t)UD_AT(row, hh, (uint64_t)bc.base + bc.dn, 4) <= wr.sd[k]) keep = false;
                    }
                }
                if (d.work) bytes += (uint64_t)__popc(__ballot_sync(FULL, c < nsurv)) * nst;
                if (whole || next >= len || !__any_sync(FULL, keep)) break;
                next = stage(next);
            }
            const uint32_t km = __ballot_sync(FULL, keep);
            __syncwarp();
            if (keep) wr.offered[nadd + __popc(km & ((1u << lane) - 1u))] = idx;
            nadd += __popc(km);
            __syncwarp();
        }
    }
    tick(W_CYC_DIST);
    // (e) reserve room and commit
    if (nadd) {
        if (!warp_reserve(d, t, len + nadd, base, lane)) {
            if (lane == 0) {
                atomicOr(d.status, ST_POOL_RETRY);
                UD_AT(a.retry, atomicAdd(a.retry_cnt, 1u), d.n, 6) = t;
            }
            return;  // nothing committed; re-run after the pool grows
        }
        const bool is_root = t >= s && t < bc.e;
        uint32_t mn = 0xffffffffu;
        for (uint32_t j = lane; j < nadd; j += 32) {
            const uint32_t idx = wr.offered[j];
            UD_AT(d.pool_hub, base + len + j, d.pool_cap, 2) = s + idx;
            UD_AT(d.pool_dist, base + len + j, d.pool_cap, 2) = (uint8_t)iter;
            if (is_root) UD_AT(bc.dm, (uint64_t)(t - s) * bc.dn + (s + idx - bc.base), (uint64_t)d.B * bc.dn, 4) = (uint8_t)iter;
            mn = min(mn, s + idx);
        }
        mn = warp_min_u32(mn);
        bytes += 5ull * nadd + 28 + (is_root ? (uint64_t)nadd : 0);
        if (d.work && lane == 0) atomicAdd(&d.work[W_EV_LABELS], (unsigned long long)nadd);
        if (lane == 0) {
            UD_AT(d.lab_len, t, d.n, 1) = len + nadd;
            UD_AT(d.last[cp], t, d.n, 1) = LastGroup{base + len, nadd, a.lid_cur};
            UD_AT(d.last_min[cp], t, d.n, 1) = mn;
            if (!a.next_tails) UD_AT(a.front_next, atomicAdd(a.front_next_cnt, 1u), d.n, 6) = t;
        }
        if (a.next_tails)
            mark_tails(d, t, mn, a.next_stamp, a.next_tails, a.next_tails_cnt, a.next_htails, a.next_htails_cnt, lane,
                       0, 1, bytes, a.gd_mut ? &a.gd_mut[bc.g].tc[a.next_stamp % 3] : nullptr);
    }
    for (uint32_t x = lane; x < d.words; x += 32) UD_AT(d.ind, (uint64_t)t * d.words + x, (uint64_t)d.n * d.words, 5) = wr.ind[x];
    if (lane == 0) UD_AT(d.ind_stamp, t, d.n, 1) = bc.b + 1;
    __syncwarp();
    tick(W_CYC_COMMIT);
}

// Pull phase of a level: heavy tails block-by-block, then light tails
// warp-by-warp.  Ends with the block converged.
__device__ void pull_phase(const UnwDev &d, const PullArgs &a, unsigned char *pull_smem)
{
    const int lane = threadIdx.x & 31;
    unsigned long long bytes = 0;
    const uint32_t hcnt = a.htails_cnt ? *a.htails_cnt : 0u;
    const uint32_t cnt = *a.tails_cnt;
    if (a.tail_q && hcnt + cnt <= SMALL_LEVEL_PER_BLOCK * gridDim.x) {
        // a small level: every tail gets a whole block (the heavy path), so
        // that its scan and tests spread over 8 warps instead of one
        HeavyRegion hs = heavy_region(pull_smem, d.words, d.B);
        for (uint32_t q = blockIdx.x; q < hcnt + cnt; q += gridDim.x) {
            pull_heavy_tail(d, a, q < hcnt ? a.htails[q] : a.tails[q - hcnt], hs, bytes);
            __syncthreads();
        }
        if (d.work && lane == 0 && bytes) atomicAdd(&d.work[W_PULL], bytes);
        __syncthreads();
        return;
    }
    if (hcnt) {
        const long long h0 = d.work ? clock64() : 0;
        HeavyRegion hs = heavy_region(pull_smem, d.words, d.B);
        if (a.htail_q) {
            __shared__ uint32_t hq;
            for (;;) {
                if (threadIdx.x == 0) hq = atomicAdd(a.htail_q, 1u);
                __syncthreads();
                const uint32_t q = hq;
                __syncthreads();
                if (q >= hcnt) break;
                pull_heavy_tail(d, a, a.htails[q], hs, bytes);
                __syncthreads();
            }
        } else {
            for (uint32_t q = blockIdx.x; q < hcnt; q += gridDim.x) {
                pull_heavy_tail(d, a, a.htails[q], hs, bytes);
                __syncthreads();
            }
        }
        if (d.work && threadIdx.x == 0) atomicAdd(&d.work[W_CYC_HEAVY], (unsigned long long)(clock64() - h0));
    }
    WarpRegion wr = warp_region(pull_smem, d.words, d.B, threadIdx.x >> 5);
    if (a.tail_q) {
        // the next claim is issued before the current tail is processed, so
        // its latency is hidden; each warp over-claims once at the end
        uint32_t q = 0;
        if (lane == 0) q = atomicAdd(a.tail_q, 1u);
        q = __shfl_sync(FULL, q, 0);
        while (q < cnt) {
            uint32_t nq = 0;
            if (lane == 0) nq = atomicAdd(a.tail_q, 1u);
            pull_light_tail(d, a, a.tails[q], wr, bytes);
            q = __shfl_sync(FULL, nq, 0);
        }
    } else {
        const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
        for (uint32_t q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < cnt; q += nw)
            pull_light_tail(d, a, a.tails[q], wr, bytes);
    }
    if (d.work && lane == 0 && bytes) atomicAdd(&d.work[W_PULL], bytes);
    __syncthreads();
}

constexpr int FIN_WARPS = 8;  // finalize kernels run blocks of 256 threads

// Final store: copy every list out of the pool, sorting each batch run by hub.
// Runs are contiguous because batches append in order; the batch of hub h is
// (h - base) / B, base = first id of the vertex's graph (0 for one graph, else
// gbase[gmap[v]]), and hubs are stored graph-local (h - base).  Entries are
// unique per vertex, so ranking by count (short runs) or by a bitmap of the
// batch's B ids (long runs) is exact.
__device__ void finalize_phase(const UnwDev &d, const uint64_t *fin_off, uint32_t *fin_hub, uint8_t *fin_dist,
                               const uint16_t *gmap, const uint32_t *gbase)
{
    const int lane = threadIdx.x & 31;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    // per warp: a bitmap of one batch's ids and its words' prefix counts
    __shared__ uint32_t fin_bm[FIN_WARPS][MAX_BATCH / 32], fin_pre[FIN_WARPS][MAX_BATCH / 32];
    uint32_t *bm = fin_bm[threadIdx.x >> 5], *pre = fin_pre[threadIdx.x >> 5];
    for (uint32_t v = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; v < d.n; v += nw) {
        const uint64_t base = UD_AT(d.lab_off, v, d.n, 1), fo = fin_off[v];
        const uint32_t len = UD_AT(d.lab_len, v, d.n, 1);
        const uint32_t gb = gmap ? gbase[gmap[v]] : 0u;
        if (len <= 128) {
            // a short list: batch ranges are disjoint and ascending, so sorting
            // the whole list by hub sorts every run; all of it is loaded in one
            // round (lane i: entries i, i + 32, i + 64, i + 96) and each entry
            // is ranked by counting the smaller hubs
            uint32_t key[4];
            uint8_t dist[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const uint32_t j = lane + 32u * q;
                key[q] = j < len ? UD_AT(d.pool_hub, base + j, d.pool_cap, 2) : 0xffffffffu;
                dist[q] = j < len ? UD_AT(d.pool_dist, base + j, d.pool_cap, 2) : (uint8_t)0;
            }
            uint32_t rank[4] = {0, 0, 0, 0};
            const uint32_t nq = (len + 31) / 32;
#pragma unroll
            for (int q2 = 0; q2 < 4; ++q2) {
                if ((uint32_t)q2 >= nq) break;
                for (int k = 0; k < 32; ++k) {
                    const uint32_t other = __shfl_sync(FULL, key[q2], k);
#pragma unroll
                    for (int q = 0; q < 4; ++q) rank[q] += other < key[q] ? 1u : 0u;
                }
            }
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const uint32_t j = lane + 32u * q;
                if (j < len) {
                    fin_hub[fo + rank[q]] = key[q] - gb;
                    fin_dist[fo + rank[q]] = dist[q];
                }
            }
            continue;
        }
        uint32_t rs = 0;
        while (rs < len) {
            const uint32_t batch = (UD_AT(d.pool_hub, base + rs, d.pool_cap, 2) - gb) / d.B;
            // run end: first entry of a later batch (monotone by batch)
            uint32_t re = rs;
            for (;;) {
                const uint32_t j = re + lane;
                const bool same = j < len && (UD_AT(d.pool_hub, base + j, d.pool_cap, 2) - gb) / d.B == batch;
                const uint32_t m = __ballot_sync(FULL, same);
                if (m == FULL) { re += 32; continue; }
                re += __ffs(~m) - 1;
                break;
            }
            if (re - rs <= 32) {
                // a short run: rank by counting within one chunk
                const uint32_t j = rs + lane;
                const bool mine = j < re;
                const uint32_t key = mine ? UD_AT(d.pool_hub, base + j, d.pool_cap, 2) : 0xffffffffu;
                const uint8_t dist = mine ? UD_AT(d.pool_dist, base + j, d.pool_cap, 2) : 0;
                uint32_t rank = 0;
                for (int k = 0; k < 32; ++k) rank += (__shfl_sync(FULL, key, k) < key) ? 1u : 0u;
                if (mine) {
                    fin_hub[fo + rs + rank] = key - gb;
                    fin_dist[fo + rs + rank] = dist;
                }
            } else {
                // a long run: its hubs lie in one batch's id range [lo, lo + B),
                // so a B-bit bitmap of the run (shared memory) and the prefix
                // popcounts of its words give each entry its rank
                const uint32_t lo = gb + batch * d.B, words = (d.B + 31) / 32;
                for (uint32_t x = lane; x < words; x += 32) bm[x] = 0;
                __syncwarp();
                for (uint32_t c0 = rs; c0 < re; c0 += 32) {
                    const uint32_t j = c0 + lane;
                    if (j < re) {
                        const uint32_t idx = UD_AT(d.pool_hub, base + j, d.pool_cap, 2) - lo;
                        atomicOr(&bm[idx >> 5], 1u << (idx & 31));
                    }
                }
                __syncwarp();
                // exclusive prefix of the words' popcounts (lane i: words i, i + 32)
                const uint32_t p0 = lane < (int)words ? __popc(bm[lane]) : 0u;
                const uint32_t p1 = lane + 32 < (int)words ? __popc(bm[lane + 32]) : 0u;
                uint32_t s0 = p0, s1 = p1;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const uint32_t y0 = __shfl_up_sync(FULL, s0, o), y1 = __shfl_up_sync(FULL, s1, o);
                    if (lane >= o) {
                        s0 += y0;
                        s1 += y1;
                    }
                }
                const uint32_t t0 = __shfl_sync(FULL, s0, 31);
                if (lane < (int)words) pre[lane] = s0 - p0;
                if (lane + 32 < (int)words) pre[lane + 32] = t0 + s1 - p1;
                __syncwarp();
                for (uint32_t c0 = rs; c0 < re; c0 += 32) {
                    const uint32_t j = c0 + lane;
                    if (j < re) {
                        const uint32_t key = UD_AT(d.pool_hub, base + j, d.pool_cap, 2);
                        const uint8_t dist = UD_AT(d.pool_dist, base + j, d.pool_cap, 2);
                        const uint32_t idx = key - lo;
                        const uint32_t rank = pre[idx >> 5] + __popc(bm[idx >> 5] & ((1u << (idx & 31)) - 1u));
                        fin_hub[fo + rs + rank] = key - gb;
                        fin_dist[fo + rs + rank] = dist;
                    }
                }
                __syncwarp();
            }
            rs = re;
        }
    }
}

}  // namespace
}  // namespace pado
