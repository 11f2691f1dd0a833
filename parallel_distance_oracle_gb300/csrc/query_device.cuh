// query_device.cuh -- one exact 2-hop distance query per warp, shared by the
// plain query kernels (query.cu) and the serving loop's mixed-batch kernel
// (serve.cu).
//
// Restates query_distance (reference includes/pado_unw_unv_unp.h:1312-1445;
// weighted includes/pado_weighted_unv_unp.h:1782-1900):
//   d = INF; for each BP root i: td = bpd_a[i] + bpd_b[i]; if td-2 <= d then
//   td -= 2 / 1 / 0 by the S^-1 / S^0 intersections and d = min(d, td);
//   then d = min over common hubs h of dist_a(h) + dist_b(h); saturate.
// Lane i evaluates BP roots i and i+32 (K <= 64), and the two hub-sorted label
// lists are intersected 32 x 32 entries at a time: each lane binary-searches
// its a-hub among the b-block with warp shuffles, and the block whose last
// hub is smaller advances.  The result is a warp
// min-reduction.  Everything is integer arithmetic with the reference's
// unsigned comparisons, so results are bit-exact.
#pragma once

#include "pado_internal.cuh"

namespace pado {
namespace {

constexpr unsigned FULL = 0xffffffffu;

__device__ __forceinline__ uint32_t warp_min(uint32_t v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(FULL, v, o));
    return v;
}

// Minimum of dist_a(h) + dist_b(h) over hubs h common to the two sorted lists.
template <typename D>
__device__ __forceinline__ uint32_t intersect_min(const uint32_t *__restrict__ ha, const D *__restrict__ da,
                                                  uint32_t la, const uint32_t *__restrict__ hb,
                                                  const D *__restrict__ db, uint32_t lb, uint32_t d,
                                                  int lane)
{
    uint32_t ia = 0, ib = 0;
    while (ia < la && ib < lb) {
        const uint32_t ra = la - ia, rb = lb - ib;
        const bool va = (uint32_t)lane < ra, vb = (uint32_t)lane < rb;
        const uint32_t av = va ? __ldg(ha + ia + lane) : 0xffffffffu;
        const uint32_t bv = vb ? __ldg(hb + ib + lane) : 0xfffffffeu;
        const uint32_t ad = va ? (uint32_t)(int32_t)da[ia + lane] : 0u;
        const uint32_t bd = vb ? (uint32_t)(int32_t)db[ib + lane] : 0u;
        // each a-hub finds its place in the (sorted) b-chunk by a binary
        // search over the lanes: 5 shuffles instead of comparing all 32
        uint32_t lo = 0;
#pragma unroll
        for (uint32_t step = 16; step > 0; step >>= 1)
            if (__shfl_sync(FULL, bv, lo + step - 1) < av) lo += step;
        const uint32_t x = __shfl_sync(FULL, bv, lo);
        const uint32_t y = __shfl_sync(FULL, bd, lo);
        if (va && x == av) {
            const uint32_t td = ad + y;
            d = td < d ? td : d;
        }
        const uint32_t amax = __shfl_sync(FULL, av, (int)(ra < 32 ? ra - 1 : 31));
        const uint32_t bmax = __shfl_sync(FULL, bv, (int)(rb < 32 ? rb - 1 : 31));
        if (amax <= bmax) ia += 32;
        if (bmax <= amax) ib += 32;
    }
    return d;
}

// Distance between original ids x and y on an unweighted index (every lane
// returns it).  `bytes` accumulates the algorithmic bytes read (lane 0 only).
__device__ __forceinline__ uint8_t query_unw_pair(const IndexView &v, uint32_t x, uint32_t y, int lane,
                                                  unsigned long long &bytes)
{
    if (x >= v.n || y >= v.n) return (x == y) ? 0 : U8_INF;
    const uint32_t rx = v.rank ? v.rank[x] : x;
    const uint32_t ry = v.rank ? v.rank[y] : y;
    // BP part: lane i takes roots i and i + 32, sets loaded with the distances
    // (one round trip); a root takes part when td - 2 <= 255 (unsigned).
    uint32_t d = U8_INF;
    for (uint32_t i = lane; i < v.K; i += 32) {
        const uint32_t td = (uint32_t)v.bpd[(uint64_t)rx * v.K + i] + (uint32_t)v.bpd[(uint64_t)ry * v.K + i];
        const ulonglong2 sx = *reinterpret_cast<const ulonglong2 *>(v.bps + ((uint64_t)rx * v.K + i) * 2);
        const ulonglong2 sy = *reinterpret_cast<const ulonglong2 *>(v.bps + ((uint64_t)ry * v.K + i) * 2);
        if (td - 2u <= (uint32_t)U8_INF) {
            const uint32_t adj = (sx.x & sy.x) ? 2u : (((sx.x & sy.y) | (sx.y & sy.x)) ? 1u : 0u);
            const uint32_t t = td - adj;
            d = t < d ? t : d;
        }
    }
    const uint64_t oa = v.off[rx], ob = v.off[ry];
    const uint32_t la = (uint32_t)(v.off[rx + 1] - oa), lb = (uint32_t)(v.off[ry + 1] - ob);
    d = intersect_min<uint8_t>(v.hub + oa, v.dist8 + oa, la, v.hub + ob, v.dist8 + ob, lb, d, lane);
    d = warp_min(d);
    // rank map, offsets, two BP rows, two label lists (u32 hub + u8 dist)
    bytes += (v.rank ? 8 : 0) + 32 + 34ull * v.K + 5ull * (la + lb);
    return (uint8_t)(d >= (uint32_t)(U8_INF - 2) ? U8_INF : d);
}

// Same on a weighted index (int16 distances, I16_INF = unreachable).
__device__ __forceinline__ int16_t query_w_pair(const IndexView &v, uint32_t x, uint32_t y, int lane,
                                                unsigned long long &bytes)
{
    if (x >= v.n || y >= v.n) return (x == y) ? 0 : I16_INF;
    const uint32_t rx = v.rank ? v.rank[x] : x;
    const uint32_t ry = v.rank ? v.rank[y] : y;
    const uint64_t oa = v.off[rx], ob = v.off[ry];
    const uint32_t la = (uint32_t)(v.off[rx + 1] - oa), lb = (uint32_t)(v.off[ry + 1] - ob);
    uint32_t d = (uint32_t)I16_INF;
    d = intersect_min<int16_t>(v.hub + oa, v.dist16 + oa, la, v.hub + ob, v.dist16 + ob, lb, d, lane);
    d = warp_min(d);
    bytes += (v.rank ? 8 : 0) + 32 + 6ull * (la + lb);
    return (int16_t)(d >= (uint32_t)(I16_INF - 2) ? I16_INF : d);
}

}  // namespace
}  // namespace pado
