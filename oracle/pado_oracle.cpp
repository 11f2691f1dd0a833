// pado_oracle.cpp -- TEST INFRASTRUCTURE ONLY.
//
// CPU restatement of PADO's pruned landmark (2-hop) labeling and its exact
// distance query, written from the reference's published algorithm so that the
// GPU library can be checked against it.  Nothing in the product library links
// or calls this file: only the tests, the smoke check and the bench's CPU
// baseline leg load it (as liboracle.so, through ctypes).
//
// Every routine names the reference file:line it restates.  The restatement
// keeps the reference's sequential processing order (queues, label insertion
// order) so that even order-sensitive steps (the weighted filter) come out the
// same; it is pinned against the compiled reference by the golden fixtures
// under tests/golden/.
//
// Conventions shared with the reference (includes/globals.h:27-40):
//   vertex ids   uint32;   unweighted distance uint8, INF = 255;
//   weighted edge weight uint8 (graph.h:300), distance int16, INF = 32767.
// Vertex ids inside the labeler are RANKS (id_transfer, graph.h:176-206):
// rank 0 is the most important vertex.  Exported labels are keyed by the
// ORIGINAL id and carry rank-id hubs, exactly like order_labels()
// (pado_unw_unv_unp.h:1227-1310).

#include <algorithm>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <queue>
#include <utility>
#include <vector>

namespace {

constexpr uint8_t U8_INF = 255;
constexpr int16_t I16_INF = 32767;

// ---------------------------------------------------------------------------
// Graph relabelling: graph.h:176-206 (Graph::id_transfer) and graph.h:367-400
// (WeightedGraph::id_transfer).  New id = rank[old id]; every adjacency list is
// sorted in DESCENDING (id, weight) order, so the lowest-rank (largest id)
// neighbour comes first.
// ---------------------------------------------------------------------------
struct RankedGraph {
    uint32_t n = 0;
    std::vector<uint64_t> off;   // n + 1
    std::vector<uint32_t> adj;   // off[n]
    std::vector<uint8_t> w;      // off[n] (weighted graphs only)
};

RankedGraph relabel(uint32_t n, const uint64_t *off, const uint32_t *adj,
                    const uint8_t *w, const uint32_t *rank)
{
    RankedGraph g;
    g.n = n;
    std::vector<std::vector<std::pair<uint32_t, uint8_t>>> lists(n);
    for (uint32_t v = 0; v < n; ++v) {
        uint32_t nv = rank[v];
        for (uint64_t e = off[v]; e < off[v + 1]; ++e)
            lists[nv].emplace_back(rank[adj[e]], w ? w[e] : 0);
    }
    g.off.assign(n + 1, 0);
    for (uint32_t v = 0; v < n; ++v) g.off[v + 1] = g.off[v] + lists[v].size();
    g.adj.resize(g.off[n]);
    if (w) g.w.resize(g.off[n]);
    for (uint32_t v = 0; v < n; ++v) {
        auto &L = lists[v];
        std::sort(L.rbegin(), L.rend());
        for (size_t i = 0; i < L.size(); ++i) {
            g.adj[g.off[v] + i] = L[i].first;
            if (w) g.w[g.off[v] + i] = L[i].second;
        }
    }
    return g;
}

// ---------------------------------------------------------------------------
// Bit-parallel labels: pado_unw_unv_unp.h:268-384 (bit_parallel_labeling).
// Root i is the smallest unused rank; up to 64 unused neighbours, scanned from
// the END of its descending list (ascending id), get bits 0..63 in that order.
// Then a BFS where, per level d, sibling edges (both ends at d, v < tv) OR the
// other end's S^-1 into S^0 first, and child edges (d -> d+1) OR the parent's
// S^-1 / S^0 into the child's.  Stored S^0 excludes S^-1 (:377-381).
// ---------------------------------------------------------------------------
void bp_labeling(const RankedGraph &g, uint32_t K, std::vector<uint8_t> &used,
                 std::vector<uint8_t> &bpd, std::vector<uint64_t> &bps)
{
    const uint32_t n = g.n;
    bpd.assign((size_t)n * K, 0);
    bps.assign((size_t)n * K * 2, 0);
    std::vector<uint8_t> td(n);
    std::vector<uint64_t> sm1(n), s0(n);
    std::vector<uint32_t> que(n);
    std::vector<std::pair<uint32_t, uint32_t>> sib, child;
    uint32_t r = 0;
    for (uint32_t i = 0; i < K; ++i) {
        while (r < n && used[r]) ++r;
        if (r == n) {  // :288-292 -- no root left: distance INF, empty sets
            for (uint32_t v = 0; v < n; ++v) bpd[(size_t)v * K + i] = U8_INF;
            continue;
        }
        used[r] = 1;
        std::fill(td.begin(), td.end(), U8_INF);
        std::fill(sm1.begin(), sm1.end(), 0);
        std::fill(s0.begin(), s0.end(), 0);
        uint32_t t0 = 0, t1, h = 0;
        que[h++] = r;
        td[r] = 0;
        t1 = h;
        int ns = 0;
        for (uint64_t k = 0, deg = g.off[r + 1] - g.off[r]; k < deg; ++k) {
            uint32_t v = g.adj[g.off[r + 1] - 1 - k];
            if (!used[v]) {
                used[v] = 1;
                que[h++] = v;
                td[v] = 1;
                sm1[v] = 1ULL << ns;
                if (++ns == 64) break;
            }
        }
        for (uint8_t d = 0; t0 < h; ++d) {
            sib.clear();
            child.clear();
            for (uint32_t q = t0; q < t1; ++q) {
                uint32_t v = que[q];
                for (uint64_t e = g.off[v]; e < g.off[v + 1]; ++e) {
                    uint32_t tv = g.adj[e];
                    if (d > td[tv]) {
                    } else if (d == td[tv]) {
                        if (v < tv) sib.emplace_back(v, tv);
                    } else {
                        if (td[tv] == U8_INF) {
                            que[h++] = tv;
                            td[tv] = (uint8_t)(d + 1);
                        }
                        child.emplace_back(v, tv);
                    }
                }
            }
            for (auto &p : sib) {
                s0[p.first] |= sm1[p.second];
                s0[p.second] |= sm1[p.first];
            }
            for (auto &p : child) {
                sm1[p.second] |= sm1[p.first];
                s0[p.second] |= s0[p.first];
            }
            t0 = t1;
            t1 = h;
        }
        for (uint32_t v = 0; v < n; ++v) {
            bpd[(size_t)v * K + i] = td[v];
            bps[((size_t)v * K + i) * 2 + 0] = sm1[v];
            bps[((size_t)v * K + i) * 2 + 1] = s0[v] & ~sm1[v];
        }
    }
}

// BP pruning test used while labeling: pado_unw_unv_unp.h:599-623.  The
// arithmetic is unsigned 32-bit like the reference's `inti td`, so td < 2
// wraps and never prunes.
inline bool bp_covers(const uint8_t *da, const uint64_t *sa, const uint8_t *db,
                      const uint64_t *sb, uint32_t K, uint32_t iter)
{
    for (uint32_t i = 0; i < K; ++i) {
        uint32_t td = (uint32_t)da[i] + (uint32_t)db[i];
        if (td - 2u <= iter) {
            if (sa[2 * i] & sb[2 * i])
                td -= 2u;
            else if ((sa[2 * i] & sb[2 * i + 1]) | (sa[2 * i + 1] & sb[2 * i]))
                td -= 1u;
            if (td <= iter) return true;
        }
    }
    return false;
}

// ---------------------------------------------------------------------------
// Unweighted batched vertex-centric labeling: pado_unw_unv_unp.h:425-1118.
// ---------------------------------------------------------------------------
struct UnwStats {
    uint64_t batches = 0, levels = 0;
    uint64_t head_visits = 0;      // active vertices processed by push
    uint64_t edges_scanned = 0;    // adjacency entries read by push
    uint64_t pairs_offered = 0;    // (tail, root) pairs reaching the indicator
    uint64_t bp_checks = 0;        // first offers: BP test run
    uint64_t bp_pruned = 0;
    uint64_t dist_checks = 0;      // distance_query calls
    uint64_t dist_entries = 0;     // label entries inspected by distance_query
    uint64_t labels_added = 0;     // labels inserted (root self labels included)
    uint64_t root_rows = 0;        // dist_matrix cells written at batch start
    uint64_t cand_vertices = 0;    // candidate-queue entries (vertices given candidates in a level)
};

struct UnwLabeler {
    const RankedGraph &g;
    uint32_t K, B, n;
    std::vector<uint8_t> used, bpd;
    std::vector<uint64_t> bps;
    // Labels per rank vertex in insertion order.  lgrp_* is the last
    // distance group (the labels the vertex got at its latest level), which
    // push_labels walks (:543-545).
    std::vector<std::vector<uint32_t>> hub;   // real (rank) hub ids
    std::vector<std::vector<uint8_t>> dist;
    std::vector<uint32_t> lgrp_start, lgrp_cnt;
    std::vector<uint8_t> got_batch;           // indicator[BATCH_SIZE]
    std::vector<uint64_t> ind;                // indicator bits, n * words
    uint32_t words;
    std::vector<uint8_t> dm;                  // dist_matrix [B][n]
    UnwStats st;

    UnwLabeler(const RankedGraph &g_, uint32_t K_, uint32_t B_)
        : g(g_), K(K_), B(B_), n(g_.n) {}

    bool ind_test_set(uint32_t v, uint32_t r)
    {
        uint64_t &w = ind[(size_t)v * words + (r >> 6)];
        uint64_t bit = 1ULL << (r & 63);
        bool was = (w & bit) != 0;
        w |= bit;
        return was;
    }

    uint32_t max_batches = 0xffffffffu;  // bounded prefix for CPU timing samples
    double bp_seconds = 0;

    void run()
    {
        used.assign(n, 0);
        auto t0 = std::chrono::steady_clock::now();
        bp_labeling(g, K, used, bpd, bps);
        bp_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        hub.assign(n, {});
        dist.assign(n, {});
        lgrp_start.assign(n, 0);
        lgrp_cnt.assign(n, 0);
        got_batch.assign(n, 0);
        words = (B + 63) / 64;
        ind.assign((size_t)n * words, 0);
        dm.assign((size_t)B * n, U8_INF);
        std::vector<uint32_t> active, cand_q, once_q;
        std::vector<uint8_t> is_active(n, 0), got_cand(n, 0), once(n, 0);
        std::vector<std::vector<uint32_t>> cand_roots(n);
        for (uint32_t s = 0, nb = 0; s < n && nb < max_batches; s += B, ++nb) {
            uint32_t size = std::min(B, n - s);
            batch(s / B, s, size, active, cand_q, once_q, is_active, got_cand, once, cand_roots);
        }
    }

    void batch(uint32_t /*b_id*/, uint32_t s, uint32_t size, std::vector<uint32_t> &active,
               std::vector<uint32_t> &cand_q, std::vector<uint32_t> &once_q,
               std::vector<uint8_t> &is_active, std::vector<uint8_t> &got_cand,
               std::vector<uint8_t> &once, std::vector<std::vector<uint32_t>> &cand_roots)
    {
        ++st.batches;
        const uint32_t e = s + size;
        // initialize (:425-528)
        active.clear();
        for (uint32_t r = s; r < e; ++r)
            if (!used[r]) active.push_back(r);
        for (uint32_t v : once_q) {
            std::fill(&ind[(size_t)v * words], &ind[(size_t)v * words] + words, 0);
            got_batch[v] = 0;
            once[v] = 0;
        }
        once_q.clear();
        for (uint32_t r = s; r < e; ++r) {
            if (used[r]) continue;
            ind_test_set(r, r - s);
            got_batch[r] = 1;
            // The roots' own indicator rows must be reset at the next batch
            // too; the reference resets them through once_candidated_queue
            // only when they were offered something, and otherwise relies on
            // indicator[BATCH_SIZE]/the self bit being overwritten.  Track
            // them explicitly (same effect: every row is clean at batch start).
            if (!once[r]) { once[r] = 1; once_q.push_back(r); }
        }
        for (uint32_t r = s; r < e; ++r) {
            if (used[r]) continue;
            lgrp_start[r] = (uint32_t)hub[r].size();
            lgrp_cnt[r] = 1;
            hub[r].push_back(r);
            dist[r].push_back(0);
            ++st.labels_added;
        }
        for (uint32_t r = s; r < e; ++r) {
            if (used[r]) continue;
            uint8_t *row = &dm[(size_t)(r - s) * n];
            for (size_t i = 0; i < hub[r].size(); ++i) { row[hub[r][i]] = dist[r][i]; ++st.root_rows; }
        }
        uint32_t iter = 0;
        while (!active.empty()) {
            ++iter;
            ++st.levels;
            if (iter >= U8_INF) {
                fprintf(stderr, "oracle: BFS level reached 255 (uint8 distance overflow)\n");
                abort();
            }
            // push (:531-641)
            for (uint32_t h : active) {
                is_active[h] = 0;
                push(h, s, iter, cand_q, once_q, got_cand, once, cand_roots);
            }
            active.clear();
            // add (:900-968)
            for (uint32_t v : cand_q) {
                got_cand[v] = 0;
                uint32_t inserted = 0;
                uint32_t start = (uint32_t)hub[v].size();
                for (uint32_t c : cand_roots[v]) {
                    if (dist_query(c, v, s, iter)) {
                        if (!is_active[v]) { is_active[v] = 1; active.push_back(v); }
                        ++inserted;
                        hub[v].push_back(c + s);
                        dist[v].push_back((uint8_t)iter);
                        ++st.labels_added;
                        if (v >= s && v - s < size) dm[(size_t)(v - s) * n + c + s] = (uint8_t)iter;
                    }
                }
                cand_roots[v].clear();
                if (inserted) {
                    got_batch[v] = 1;
                    lgrp_start[v] = start;
                    lgrp_cnt[v] = inserted;
                }
            }
            cand_q.clear();
        }
        // reset_at_end (:780-816)
        for (uint32_t r = s; r < e; ++r) {
            uint8_t *row = &dm[(size_t)(r - s) * n];
            for (uint32_t h2 : hub[r]) row[h2] = U8_INF;
        }
    }

    void push(uint32_t h, uint32_t s, uint32_t iter, std::vector<uint32_t> &cand_q,
              std::vector<uint32_t> &once_q, std::vector<uint8_t> &got_cand,
              std::vector<uint8_t> &once, std::vector<std::vector<uint32_t>> &cand_roots)
    {
        ++st.head_visits;
        const uint32_t ls = lgrp_start[h], lc = lgrp_cnt[h];
        for (uint64_t e = g.off[h]; e < g.off[h + 1]; ++e) {
            uint32_t t = g.adj[e];
            ++st.edges_scanned;
            if (used[t]) continue;
            if (t < s) return;
            const uint8_t *dt = &bpd[(size_t)t * K];
            const uint64_t *stt = &bps[(size_t)t * K * 2];
            for (uint32_t l = ls; l < ls + lc; ++l) {
                uint32_t rr = hub[h][l];
                if (t <= rr) continue;
                ++st.pairs_offered;
                if (ind_test_set(t, rr - s)) continue;
                if (!once[t]) { once[t] = 1; once_q.push_back(t); }
                ++st.bp_checks;
                if (bp_covers(&bpd[(size_t)rr * K], &bps[(size_t)rr * K * 2], dt, stt, K, iter)) {
                    ++st.bp_pruned;
                    continue;
                }
                cand_roots[t].push_back(rr - s);
                if (!got_cand[t]) { got_cand[t] = 1; cand_q.push_back(t); ++st.cand_vertices; }
            }
        }
    }

    // distance_query (:647-724): prune when a hub h < cand with dist(v,h) <
    // iter gives dist(v,h) + dist_matrix[cand][h] <= iter.
    bool dist_query(uint32_t c, uint32_t v, uint32_t s, uint32_t iter)
    {
        ++st.dist_checks;
        const uint32_t creal = c + s;
        const uint8_t *row = &dm[(size_t)c * n];
        const auto &H = hub[v];
        const auto &D = dist[v];
        for (size_t i = 0; i < H.size(); ++i) {
            if (D[i] >= iter) continue;
            ++st.dist_entries;
            uint32_t hh = H[i];
            if (hh >= creal) continue;
            if ((uint32_t)D[i] + row[hh] <= iter) return false;
        }
        return true;
    }
};

// ---------------------------------------------------------------------------
// Weighted batched labeling: pado_weighted_unv_unp.h:281-1404.  Restated with
// the same queue orders as the sequential reference.
// ---------------------------------------------------------------------------
struct WStats {
    uint64_t batches = 0, rounds = 0;
    uint64_t edges_scanned = 0, relax_tries = 0, relax_accepted = 0;
    uint64_t checks = 0, check_entries = 0, temp_labels = 0, filtered = 0;
    uint64_t labels_added = 0;
};

struct WLabeler {
    const RankedGraph &g;
    uint32_t B, n;
    std::vector<std::vector<uint32_t>> hub;   // real ids
    std::vector<std::vector<int16_t>> dist;
    // short_index, flattened [n][B] where needed
    std::vector<std::vector<uint32_t>> cand_que, vq, reached, last_new;
    std::vector<int16_t> cand_d, vd, dt;      // [n][B]
    std::vector<int16_t> buf;                 // roots_labels_buffer [B][n]
    std::vector<uint8_t> is_active, has_c, has_new, once;
    WStats st;

    // mode bit 0: part (2) of the check reads the temporary labels as they
    //             were when the check phase started (level-synchronous);
    // mode bits 1-2: filter order -- 0 reference queue order, 1 roots first
    //             then others, each row in ascending root index, in place;
    //             2 every test reads the pre-filter values.
    uint32_t mode = 0;
    std::vector<int16_t> snap;                // [B][B] rows of vertices < B
    std::vector<uint32_t> snap_len;           // vq length of v at phase start
    std::vector<int16_t> own_snap;            // v's own row at phase start
    WLabeler(const RankedGraph &g_, uint32_t B_, uint32_t mode_ = 0) : g(g_), B(B_), n(g_.n), mode(mode_) {}

    void run()
    {
        hub.assign(n, {});
        dist.assign(n, {});
        cand_que.assign(n, {});
        vq.assign(n, {});
        reached.assign(n, {});
        last_new.assign(n, {});
        cand_d.assign((size_t)n * B, I16_INF);
        vd.assign((size_t)n * B, I16_INF);
        dt.assign((size_t)n * B, I16_INF);
        buf.assign((size_t)B * n, I16_INF);
        is_active.assign(n, 0);
        has_c.assign(n, 0);
        has_new.assign(n, 0);
        once.assign(n, 0);
        for (uint32_t s = 0; s < n; s += B) batch(s, std::min(B, n - s));
    }

    void batch(uint32_t s, uint32_t size)
    {
        ++st.batches;
        const uint32_t e = s + size;
        std::vector<uint32_t> active, has_cand, new_q, once_q;
        // initialize_tables (:281-330)
        for (uint32_t c = 0; c < size; ++c) {
            uint32_t r = c + s;
            for (size_t i = 0; i < hub[r].size(); ++i) buf[(size_t)c * n + hub[r][i]] = dist[r][i];
            buf[(size_t)c * n + r] = 0;
        }
        for (uint32_t r = s; r < e; ++r) {
            uint32_t c = r - s;
            vq[r].push_back(c);
            vd[(size_t)r * B + c] = 0;
            last_new[r].push_back(c);
        }
        for (uint32_t r = s; r < e; ++r) active.push_back(r);
        for (uint32_t r = s; r < e; ++r) { new_q.push_back(r); has_new[r] = 1; }

        while (!active.empty()) {
            ++st.rounds;
            for (uint32_t h : active) {
                is_active[h] = 0;
                send(h, s, has_cand, once_q);
            }
            active.clear();
            if (mode & 1) {
                uint32_t lim = std::min(n, B);
                snap.assign(vd.begin(), vd.begin() + (size_t)lim * B);
                snap.resize((size_t)B * B, I16_INF);
                snap_len.resize(n);
                for (uint32_t v : has_cand) snap_len[v] = (uint32_t)vq[v].size();
            }
            for (uint32_t v : has_cand) {
                bool act = false;
                if (mode & 1) own_snap.assign(&vd[(size_t)v * B], &vd[(size_t)v * B] + B);
                for (uint32_t c : cand_que[v]) {
                    int16_t t = cand_d[(size_t)v * B + c];
                    int16_t q = query(v, c, s, t);
                    if (q == I16_INF) {
                        if (vd[(size_t)v * B + c] == I16_INF) vq[v].push_back(c);
                        vd[(size_t)v * B + c] = t;
                        last_new[v].push_back(c);
                        act = true;
                        ++st.temp_labels;
                    } else if (q < t) {
                        dt[(size_t)v * B + c] = q;
                    }
                }
                if (act) {
                    if (!is_active[v]) { is_active[v] = 1; active.push_back(v); }
                    if (!has_new[v]) { has_new[v] = 1; new_q.push_back(v); }
                }
            }
            for (uint32_t v : has_cand) {
                has_c[v] = 0;
                for (uint32_t c : cand_que[v]) cand_d[(size_t)v * B + c] = I16_INF;
                cand_que[v].clear();
            }
            has_cand.clear();
        }
        filter(new_q, s);
        // reset_tables (:872-911)
        for (uint32_t c = 0; c < size; ++c) {
            uint32_t r = c + s;
            for (uint32_t h2 : hub[r]) buf[(size_t)c * n + h2] = I16_INF;
            buf[(size_t)c * n + r] = I16_INF;
        }
        for (uint32_t v : once_q) {
            once[v] = 0;
            for (uint32_t c : reached[v]) dt[(size_t)v * B + c] = I16_INF;
            reached[v].clear();
        }
        // update_index (:913-950)
        for (uint32_t v : new_q) {
            has_new[v] = 0;
            for (uint32_t c : vq[v]) {
                int16_t d = vd[(size_t)v * B + c];
                if (d == I16_INF) continue;
                vd[(size_t)v * B + c] = I16_INF;
                hub[v].push_back(c + s);
                dist[v].push_back(d);
                ++st.labels_added;
            }
            vq[v].clear();
        }
    }

    // send_messages (:409-474)
    void send(uint32_t h, uint32_t s, std::vector<uint32_t> &has_cand, std::vector<uint32_t> &once_q)
    {
        for (uint64_t e = g.off[h]; e < g.off[h + 1]; ++e) {
            uint32_t t = g.adj[e];
            ++st.edges_scanned;
            if (t <= s) break;
            int16_t w = g.w[e];
            bool got = false;
            for (uint32_t c : last_new[h]) {
                if (t <= c + s) continue;
                ++st.relax_tries;
                int16_t td = (int16_t)(vd[(size_t)h * B + c] + w);
                int16_t &dtc = dt[(size_t)t * B + c];
                int16_t &cdc = cand_d[(size_t)t * B + c];
                if (td < dtc && td < cdc) {
                    if (cdc == I16_INF) cand_que[t].push_back(c);
                    cdc = td;
                    if (dtc == I16_INF) reached[t].push_back(c);
                    dtc = td;
                    got = true;
                    ++st.relax_accepted;
                }
            }
            if (got && !has_c[t]) {
                has_c[t] = 1;
                has_cand.push_back(t);
                if (!once[t]) { once[t] = 1; once_q.push_back(t); }
            }
        }
        last_new[h].clear();
    }

    // distance_query (:476-870).  Returns the FIRST covering distance found,
    // or INF.  Part (2) reads the temporary labels of the vertex whose id is
    // the candidate's batch-local index (:585), as the reference does.
    int16_t query(uint32_t v, uint32_t c, uint32_t s, int16_t t)
    {
        ++st.checks;
        const uint32_t creal = c + s;
        for (size_t i = 0; i < hub[v].size(); ++i) {
            ++st.check_entries;
            uint32_t r = hub[v][i];
            int16_t b = buf[(size_t)c * n + r];
            if (creal <= r || b == I16_INF) continue;
            int16_t d = (int16_t)(dist[v][i] + b);
            if (d <= t) return d;
        }
        const int16_t *vdc = &vd[(size_t)c * B];  // short_index[cand_root_id]
        if (mode & 1) {
            if (c >= std::min(n, B)) return I16_INF;
            const int16_t *sc = &snap[(size_t)c * B];
            const int16_t *sv = own_snap.data();
            for (uint32_t i = 0; i < snap_len[v]; ++i) {
                uint32_t r = vq[v][i];
                ++st.check_entries;
                if (creal <= r + s) continue;
                if (sc[r] != I16_INF) {
                    int16_t d = (int16_t)(sv[r] + sc[r]);
                    if (d <= t) return d;
                }
            }
            return I16_INF;
        }
        for (uint32_t r : vq[v]) {
            ++st.check_entries;
            if (creal <= r + s) continue;
            if (vdc[r] != I16_INF) {
                int16_t d = (int16_t)(vd[(size_t)v * B + r] + vdc[r]);
                if (d <= t) return d;
            }
        }
        return I16_INF;
    }

    // filter_out_labels (:1052-1184), in place, in has_new_labels_queue order.
    void filter(const std::vector<uint32_t> &new_q, uint32_t s)
    {
        uint32_t fm = (mode >> 1) & 3;
        if (fm == 1) {
            for (uint32_t v : new_q) std::sort(vq[v].begin(), vq[v].end());
        } else if (fm == 2) {
            std::vector<int16_t> pre(vd);
            for (uint32_t v : new_q) {
                const auto &Q = vq[v];
                const int16_t *prow = &pre[(size_t)v * B];
                for (uint32_t c : Q) {
                    int16_t dvc = prow[c];
                    const int16_t *crow = &pre[(size_t)(c + s) * B];
                    for (uint32_t r : Q) {
                        if (c <= r) continue;
                        int16_t dvr = prow[r], dcr = crow[r];
                        if (dvr > dvc || dcr > dvc) continue;
                        if (dvr + dcr <= dvc) { vd[(size_t)v * B + c] = I16_INF; }
                    }
                }
            }
            return;
        }
        for (uint32_t v : new_q) {
            const auto &Q = vq[v];
            int16_t *row = &vd[(size_t)v * B];
            for (uint32_t c : Q) {
                int16_t dvc = row[c];
                const int16_t *crow = &vd[(size_t)(c + s) * B];
                for (uint32_t r : Q) {
                    if (c <= r) continue;
                    int16_t dvr = row[r];
                    if (dvr > dvc) continue;
                    int16_t dcr = crow[r];
                    if (dcr > dvc) continue;
                    if (dvr + dcr <= dvc) {
                        if (row[c] != I16_INF) ++st.filtered;
                        row[c] = I16_INF;
                    }
                }
            }
        }
    }
};

// ---------------------------------------------------------------------------
// Canonical (order_labels) form, keyed by original id.
// ---------------------------------------------------------------------------
template <typename D>
struct Canon {
    uint32_t n = 0, K = 0;
    std::vector<uint64_t> off;    // n + 1
    std::vector<uint32_t> hub;
    std::vector<D> dist;
    std::vector<uint8_t> bpd;     // n * K (original-id order)
    std::vector<uint64_t> bps;    // n * K * 2
};

template <typename D>
Canon<D> canonicalize(uint32_t n, const std::vector<std::vector<uint32_t>> &hub,
                      const std::vector<std::vector<D>> &dist, const uint32_t *rank)
{
    Canon<D> c;
    c.n = n;
    c.off.assign(n + 1, 0);
    for (uint32_t v = 0; v < n; ++v) c.off[v + 1] = c.off[v] + hub[rank[v]].size();
    c.hub.resize(c.off[n]);
    c.dist.resize(c.off[n]);
    std::vector<std::pair<uint32_t, D>> tmp;
    for (uint32_t v = 0; v < n; ++v) {
        uint32_t r = rank[v];
        tmp.clear();
        for (size_t i = 0; i < hub[r].size(); ++i) tmp.emplace_back(hub[r][i], dist[r][i]);
        std::sort(tmp.begin(), tmp.end());
        for (size_t i = 0; i < tmp.size(); ++i) {
            c.hub[c.off[v] + i] = tmp[i].first;
            c.dist[c.off[v] + i] = tmp[i].second;
        }
    }
    return c;
}

// query_distance: pado_unw_unv_unp.h:1312-1445 (BP part :1343-1355, merge
// :1423-1439, saturation :1441-1443).
uint8_t unw_query_one(const Canon<uint8_t> &c, uint32_t a, uint32_t b)
{
    const uint32_t n = c.n, K = c.K;
    if (a >= n || b >= n) return a == b ? 0 : U8_INF;
    uint32_t d = U8_INF;
    const uint8_t *da = &c.bpd[(size_t)a * K], *db = &c.bpd[(size_t)b * K];
    const uint64_t *sa = &c.bps[(size_t)a * K * 2], *sb = &c.bps[(size_t)b * K * 2];
    for (uint32_t i = 0; i < K; ++i) {
        int td = (int)da[i] + (int)db[i];
        if ((uint32_t)(td - 2) <= d) {
            td += (sa[2 * i] & sb[2 * i]) ? -2
                  : ((sa[2 * i] & sb[2 * i + 1]) | (sa[2 * i + 1] & sb[2 * i])) ? -1 : 0;
            if ((uint32_t)td < d) d = (uint32_t)td;
        }
    }
    uint64_t i1 = c.off[a], e1 = c.off[a + 1], i2 = c.off[b], e2 = c.off[b + 1];
    while (i1 < e1 && i2 < e2) {
        uint32_t v1 = c.hub[i1], v2 = c.hub[i2];
        if (v1 == v2) {
            uint32_t td = (uint32_t)c.dist[i1] + (uint32_t)c.dist[i2];
            if (td < d) d = td;
            ++i1;
            ++i2;
        } else if (v1 < v2) {
            ++i1;
        } else {
            ++i2;
        }
    }
    if (d >= U8_INF - 2) d = U8_INF;
    return (uint8_t)d;
}

// Weighted query_distance: pado_weighted_unv_unp.h:1782-1900.
int16_t w_query_one(const Canon<int16_t> &c, uint32_t a, uint32_t b)
{
    const uint32_t n = c.n;
    if (a >= n || b >= n) return a == b ? 0 : I16_INF;
    uint32_t d = (uint32_t)I16_INF;
    uint64_t i1 = c.off[a], e1 = c.off[a + 1], i2 = c.off[b], e2 = c.off[b + 1];
    while (i1 < e1 && i2 < e2) {
        uint32_t v1 = c.hub[i1], v2 = c.hub[i2];
        if (v1 == v2) {
            uint32_t td = (uint32_t)((int)c.dist[i1] + (int)c.dist[i2]);
            if (td < d) d = td;
            ++i1;
            ++i2;
        } else if (v1 < v2) {
            ++i1;
        } else {
            ++i2;
        }
    }
    if (d >= (uint32_t)(I16_INF - 2)) d = I16_INF;
    return (int16_t)d;
}

}  // namespace

// ===========================================================================
// C ABI for ctypes
// ===========================================================================
struct orc_unw {
    Canon<uint8_t> c;
    UnwStats st;
};
struct orc_w {
    Canon<int16_t> c;
    WStats st;
};

extern "C" {

orc_unw *orc_unw_build(uint32_t n, const uint64_t *off, const uint32_t *adj, const uint32_t *rank,
                       uint32_t K, uint32_t B)
{
    RankedGraph g = relabel(n, off, adj, nullptr, rank);
    UnwLabeler L(g, K, B);
    L.run();
    orc_unw *h = new orc_unw;
    h->c = canonicalize<uint8_t>(n, L.hub, L.dist, rank);
    h->c.K = K;
    h->c.bpd.resize((size_t)n * K);
    h->c.bps.resize((size_t)n * K * 2);
    for (uint32_t v = 0; v < n; ++v) {
        memcpy(&h->c.bpd[(size_t)v * K], &L.bpd[(size_t)rank[v] * K], K);
        memcpy(&h->c.bps[(size_t)v * K * 2], &L.bps[(size_t)rank[v] * K * 2], K * 16);
    }
    h->st = L.st;
    return h;
}

uint64_t orc_unw_num_labels(const orc_unw *h) { return h->c.off[h->c.n]; }

// Timing sample for the CPU baseline: BP labeling plus the first `nbatches`
// root batches of the sequential restatement.  Returns wall seconds; the
// labels produced go to *labels_out, the BP share to *bp_seconds.
double orc_unw_prefix(uint32_t n, const uint64_t *off, const uint32_t *adj, const uint32_t *rank, uint32_t K,
                      uint32_t B, uint32_t nbatches, uint64_t *labels_out, double *bp_seconds)
{
    RankedGraph g = relabel(n, off, adj, nullptr, rank);
    UnwLabeler L(g, K, B);
    L.max_batches = nbatches;
    auto t0 = std::chrono::steady_clock::now();
    L.run();
    double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    uint64_t cnt = 0;
    for (uint32_t v = 0; v < n; ++v) cnt += L.hub[v].size();
    *labels_out = cnt;
    *bp_seconds = L.bp_seconds;
    return secs;
}

void orc_unw_export(const orc_unw *h, uint64_t *off, uint32_t *hub, uint8_t *dist, uint8_t *bpd,
                    uint64_t *bps)
{
    const auto &c = h->c;
    memcpy(off, c.off.data(), (c.n + 1) * sizeof(uint64_t));
    memcpy(hub, c.hub.data(), c.hub.size() * sizeof(uint32_t));
    memcpy(dist, c.dist.data(), c.dist.size());
    memcpy(bpd, c.bpd.data(), c.bpd.size());
    memcpy(bps, c.bps.data(), c.bps.size() * sizeof(uint64_t));
}

// stats: batches, levels, head_visits, edges_scanned, pairs_offered,
// bp_checks, bp_pruned, dist_checks, dist_entries, labels_added, root_rows,
// cand_vertices
void orc_unw_stats(const orc_unw *h, uint64_t *out)
{
    const UnwStats &s = h->st;
    uint64_t v[] = {s.batches, s.levels, s.head_visits, s.edges_scanned, s.pairs_offered,
                    s.bp_checks, s.bp_pruned, s.dist_checks, s.dist_entries, s.labels_added,
                    s.root_rows, s.cand_vertices};
    memcpy(out, v, sizeof(v));
}

void orc_unw_query(const orc_unw *h, uint64_t k, const uint32_t *a, const uint32_t *b, uint8_t *out)
{
    for (uint64_t i = 0; i < k; ++i) out[i] = unw_query_one(h->c, a[i], b[i]);
}

// Query over caller-supplied canonical arrays (used to check a GPU-built
// label set without rebuilding it on the CPU).
void orc_unw_query_arrays(uint32_t n, uint32_t K, const uint64_t *off, const uint32_t *hub,
                          const uint8_t *dist, const uint8_t *bpd, const uint64_t *bps, uint64_t k,
                          const uint32_t *a, const uint32_t *b, uint8_t *out)
{
    Canon<uint8_t> c;
    c.n = n;
    c.K = K;
    c.off.assign(off, off + n + 1);
    c.hub.assign(hub, hub + off[n]);
    c.dist.assign(dist, dist + off[n]);
    c.bpd.assign(bpd, bpd + (size_t)n * K);
    c.bps.assign(bps, bps + (size_t)n * K * 2);
    for (uint64_t i = 0; i < k; ++i) out[i] = unw_query_one(c, a[i], b[i]);
}

void orc_unw_free(orc_unw *h) { delete h; }

// store_index_to_file format (pado_unw_unv_unp.h:1120-1180):
// [n u32][K u32] then per original vertex: K x (u8 d, u64 S-1, u64 S0),
// u32 count, count x (u32 hub, u8 d).
int orc_unw_store(const orc_unw *h, const char *path)
{
    const auto &c = h->c;
    FILE *f = fopen(path, "wb");
    if (!f) return -1;
    fwrite(&c.n, 4, 1, f);
    fwrite(&c.K, 4, 1, f);
    for (uint32_t v = 0; v < c.n; ++v) {
        for (uint32_t i = 0; i < c.K; ++i) {
            fwrite(&c.bpd[(size_t)v * c.K + i], 1, 1, f);
            fwrite(&c.bps[((size_t)v * c.K + i) * 2], 8, 2, f);
        }
        uint32_t cnt = (uint32_t)(c.off[v + 1] - c.off[v]);
        fwrite(&cnt, 4, 1, f);
        for (uint64_t j = c.off[v]; j < c.off[v + 1]; ++j) {
            fwrite(&c.hub[j], 4, 1, f);
            fwrite(&c.dist[j], 1, 1, f);
        }
    }
    return fclose(f) == 0 ? 0 : -1;
}

orc_w *orc_w_build(uint32_t n, const uint64_t *off, const uint32_t *adj, const uint8_t *w,
                   const uint32_t *rank, uint32_t B, uint32_t mode)
{
    RankedGraph g = relabel(n, off, adj, w, rank);
    WLabeler L(g, B, mode);
    L.run();
    orc_w *h = new orc_w;
    h->c = canonicalize<int16_t>(n, L.hub, L.dist, rank);
    h->st = L.st;
    return h;
}

uint64_t orc_w_num_labels(const orc_w *h) { return h->c.off[h->c.n]; }

void orc_w_export(const orc_w *h, uint64_t *off, uint32_t *hub, int16_t *dist)
{
    const auto &c = h->c;
    memcpy(off, c.off.data(), (c.n + 1) * sizeof(uint64_t));
    memcpy(hub, c.hub.data(), c.hub.size() * sizeof(uint32_t));
    memcpy(dist, c.dist.data(), c.dist.size() * sizeof(int16_t));
}

// stats: batches, rounds, edges_scanned, relax_tries, relax_accepted, checks,
// check_entries, temp_labels, filtered, labels_added
void orc_w_stats(const orc_w *h, uint64_t *out)
{
    const WStats &s = h->st;
    uint64_t v[] = {s.batches, s.rounds, s.edges_scanned, s.relax_tries, s.relax_accepted,
                    s.checks, s.check_entries, s.temp_labels, s.filtered, s.labels_added};
    memcpy(out, v, sizeof(v));
}

void orc_w_query(const orc_w *h, uint64_t k, const uint32_t *a, const uint32_t *b, int16_t *out)
{
    for (uint64_t i = 0; i < k; ++i) out[i] = w_query_one(h->c, a[i], b[i]);
}

void orc_w_query_arrays(uint32_t n, const uint64_t *off, const uint32_t *hub, const int16_t *dist,
                        uint64_t k, const uint32_t *a, const uint32_t *b, int16_t *out)
{
    Canon<int16_t> c;
    c.n = n;
    c.off.assign(off, off + n + 1);
    c.hub.assign(hub, hub + off[n]);
    c.dist.assign(dist, dist + off[n]);
    for (uint64_t i = 0; i < k; ++i) out[i] = w_query_one(c, a[i], b[i]);
}

void orc_w_free(orc_w *h) { delete h; }

// weighted store_index_to_file (pado_weighted_unv_unp.h:1639-1676):
// [n u32] then per original vertex: u32 count, count x (u32 hub, i16 d).
int orc_w_store(const orc_w *h, const char *path)
{
    const auto &c = h->c;
    FILE *f = fopen(path, "wb");
    if (!f) return -1;
    fwrite(&c.n, 4, 1, f);
    for (uint32_t v = 0; v < c.n; ++v) {
        uint32_t cnt = (uint32_t)(c.off[v + 1] - c.off[v]);
        fwrite(&cnt, 4, 1, f);
        for (uint64_t j = c.off[v]; j < c.off[v + 1]; ++j) {
            fwrite(&c.hub[j], 4, 1, f);
            fwrite(&c.dist[j], 2, 1, f);
        }
    }
    return fclose(f) == 0 ? 0 : -1;
}

// ---------------------------------------------------------------------------
// Independent truth: BFS (unreachable = 255, distances >= 253 saturate to 255
// like the query) and Dijkstra (unreachable = 32767).  These ignore the
// labeling entirely.
// ---------------------------------------------------------------------------
void orc_bfs(uint32_t n, const uint64_t *off, const uint32_t *adj, uint32_t src, uint8_t *out)
{
    std::vector<uint32_t> d(n, UINT32_MAX);
    std::vector<uint32_t> q;
    q.reserve(n);
    d[src] = 0;
    q.push_back(src);
    for (size_t i = 0; i < q.size(); ++i) {
        uint32_t v = q[i];
        for (uint64_t e = off[v]; e < off[v + 1]; ++e)
            if (d[adj[e]] == UINT32_MAX) { d[adj[e]] = d[v] + 1; q.push_back(adj[e]); }
    }
    for (uint32_t v = 0; v < n; ++v) out[v] = d[v] >= 253 ? U8_INF : (uint8_t)d[v];
}

void orc_dijkstra(uint32_t n, const uint64_t *off, const uint32_t *adj, const uint8_t *w,
                  uint32_t src, int32_t *out)
{
    std::vector<int64_t> d(n, INT64_MAX);
    using P = std::pair<int64_t, uint32_t>;
    std::priority_queue<P, std::vector<P>, std::greater<P>> pq;
    d[src] = 0;
    pq.emplace(0, src);
    while (!pq.empty()) {
        auto [dv, v] = pq.top();
        pq.pop();
        if (dv != d[v]) continue;
        for (uint64_t e = off[v]; e < off[v + 1]; ++e) {
            int64_t nd = dv + w[e];
            if (nd < d[adj[e]]) { d[adj[e]] = nd; pq.emplace(nd, adj[e]); }
        }
    }
    for (uint32_t v = 0; v < n; ++v) out[v] = d[v] >= I16_INF - 2 ? I16_INF : (int32_t)d[v];
}

// ---------------------------------------------------------------------------
// Graph preparation, the steps the reference runs before any labeler:
//   Graph::construct (graph.h:125-153; weighted :292-309): both directions of
//     every edge, duplicates and self-loops kept, n = max id + 1;
//   make_rank (graph.h:156-174): degree descending, ties by ascending id
//     (the reference's rand() jitter is not reproducible);
//   id_transfer (graph.h:176-206; weighted :367-400): relabel to ranks, every
//     list sorted descending by (id, weight).
// dedupe != 0 first drops self-loops and keeps the first occurrence (input
// order, hence its weight) of every undirected pair.  n = 0 takes max id + 1.
// Returns 0, or -1 when an id is >= n.  adj / w_out need room for 2m.
// ---------------------------------------------------------------------------
int orc_graph_ingest(uint64_t m, const uint32_t *u, const uint32_t *v, const uint8_t *w, uint32_t n, int dedupe,
                     uint64_t *off, uint32_t *adj, uint8_t *w_out, uint32_t *rank, uint64_t *entries,
                     uint32_t *n_out)
{
    if (n == 0)
        for (uint64_t e = 0; e < m; ++e) n = std::max(n, std::max(u[e], v[e]) + 1);
    for (uint64_t e = 0; e < m; ++e)
        if (u[e] >= n || v[e] >= n) return -1;
    std::vector<uint64_t> keep;  // edge indexes, input order
    keep.reserve(m);
    if (dedupe) {
        std::vector<std::pair<uint64_t, uint64_t>> key;  // ((lo, hi), index)
        for (uint64_t e = 0; e < m; ++e)
            if (u[e] != v[e])
                key.push_back({(uint64_t)std::min(u[e], v[e]) << 32 | std::max(u[e], v[e]), e});
        std::stable_sort(key.begin(), key.end(),
                         [](const auto &a, const auto &b) { return a.first < b.first; });
        for (size_t i = 0; i < key.size(); ++i)
            if (i == 0 || key[i].first != key[i - 1].first) keep.push_back(key[i].second);
        std::sort(keep.begin(), keep.end());
    } else {
        for (uint64_t e = 0; e < m; ++e) keep.push_back(e);
    }
    std::vector<uint32_t> deg(n, 0);
    for (uint64_t e : keep) {
        ++deg[u[e]];
        ++deg[v[e]];
    }
    std::vector<uint32_t> order(n);
    for (uint32_t x = 0; x < n; ++x) order[x] = x;
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return deg[a] > deg[b]; });
    for (uint32_t r = 0; r < n; ++r) rank[order[r]] = r;
    std::vector<std::vector<std::pair<uint32_t, uint8_t>>> lists(n);
    for (uint64_t e : keep) {
        const uint8_t we = w ? w[e] : 0;
        lists[rank[u[e]]].push_back({rank[v[e]], we});
        lists[rank[v[e]]].push_back({rank[u[e]], we});
    }
    off[0] = 0;
    for (uint32_t x = 0; x < n; ++x) {
        std::sort(lists[x].rbegin(), lists[x].rend());
        for (size_t i = 0; i < lists[x].size(); ++i) {
            adj[off[x] + i] = lists[x][i].first;
            if (w_out) w_out[off[x] + i] = lists[x][i].second;
        }
        off[x + 1] = off[x] + lists[x].size();
    }
    *entries = off[n];
    *n_out = n;
    return 0;
}

// Edge-list text, line by line as Graph(const char *) reads it
// (graph.h:95-117; weighted :262-290): a line is the bytes before '\n'; it is
// skipped when empty or when it starts with '#' or '%'.  Otherwise it must
// begin with two unsigned decimal ids (each after optional blanks -- space,
// \t, \r, \v, \f -- and an optional '+', at most 2^32 - 1), like
// `lin >> head >> tail`; a line where that fails is skipped (the reference
// would repeat the previous line's values).  A weight follows the same rule,
// is 0 when absent or unparsable and 2^32 - 1 on overflow, and is cast to
// uint8 (graph.h:300).  Extra columns are ignored.  Returns the number of
// edges; only the first `cap` are stored.
uint64_t orc_edge_text_parse(const char *text, uint64_t bytes, int weighted, uint64_t cap, uint32_t *u,
                             uint32_t *v, uint8_t *w)
{
    auto blank = [](char c) { return c == ' ' || c == '\t' || c == '\r' || c == '\v' || c == '\f'; };
    // returns 0 = no number, 1 = number, 2 = number above 2^32 - 1
    auto number = [&](uint64_t &i, uint64_t end, uint32_t &val) {
        while (i < end && blank(text[i])) ++i;
        if (i < end && text[i] == '+') ++i;
        if (i >= end || text[i] < '0' || text[i] > '9') return 0;
        uint64_t x = 0;
        bool over = false;
        for (; i < end && text[i] >= '0' && text[i] <= '9'; ++i) {
            x = x * 10 + (uint64_t)(text[i] - '0');
            if (x > 0xffffffffull) {
                over = true;
                x = 0xffffffffull;
            }
        }
        val = (uint32_t)x;
        return over ? 2 : 1;
    };
    uint64_t count = 0, start = 0;
    while (start < bytes) {
        uint64_t end = start;
        while (end < bytes && text[end] != '\n') ++end;
        uint64_t i = start;
        uint32_t a = 0, b = 0, c = 0;
        if (end > start && text[start] != '#' && text[start] != '%' && number(i, end, a) == 1 &&
            number(i, end, b) == 1) {
            if (weighted && number(i, end, c) == 0) c = 0;
            if (count < cap) {
                u[count] = a;
                v[count] = b;
                if (weighted) w[count] = (uint8_t)c;
            }
            ++count;
        }
        start = end + 1;
    }
    return count;
}

// ---- graph reductions (the reference's conversion tools) --------------------
//
// Both take the edge list in input order over ids < n and keep every input
// edge's two adjacency entries (repeats and self-loops included), as the tools
// build their adjacency; both return per-vertex flags and the indices of the
// input edges that survive, in input order -- the lines the tools write.

// tools/pseudocode-delete_1-degree_vertices.cpp: adjacency in input order
// (construct :101-124; a self-loop is two entries of its vertex), degrees of
// the input graph throughout (:130, :153); for every vertex in ascending id
// that is not deleted and has one entry, a walk (:131-166) deletes the current
// vertex, takes its first entry that is not deleted (the last entry if all
// are), and continues there if that vertex has two entries.  Kept edges have
// no deleted end (:185-191).  The reference's walk can bounce for ever between
// deleted vertices of two entries (e.g. the path 0-2-3-1 given as the lines
// "0 2", "3 1", "2 3", whose end 1 walks 1 -> 3 -> 2 -> 3 -> ...); after
// n + 1 steps without a new deletion the restatement ends such a walk and sets
// *nonterminating (no deletion can happen in it any more).
int orc_reduce_degree1(uint64_t m, const uint32_t *u, const uint32_t *v, uint32_t n, uint8_t *deleted,
                       uint64_t *kept, uint64_t *m_kept, int *nonterminating)
{
    for (uint64_t e = 0; e < m; ++e)
        if (u[e] >= n || v[e] >= n) return 1;
    std::vector<std::vector<uint32_t>> adj(n);
    for (uint64_t e = 0; e < m; ++e) {
        adj[u[e]].push_back(v[e]);
        adj[v[e]].push_back(u[e]);
    }
    const uint32_t NONE = 0xffffffffu;
    std::fill(deleted, deleted + n, (uint8_t)0);
    *nonterminating = 0;
    for (uint32_t s = 0; s < n; ++s) {
        uint32_t next = (!deleted[s] && adj[s].size() == 1) ? s : NONE;
        uint64_t idle = 0;  // steps since the last new deletion
        while (next != NONE) {
            const uint32_t x = next;
            if (deleted[x]) {
                if (++idle > (uint64_t)n + 1) {
                    *nonterminating = 1;
                    break;
                }
            } else {
                idle = 0;
            }
            deleted[x] = 1;
            uint32_t w = NONE;
            for (uint32_t y : adj[x]) {
                w = y;
                if (!deleted[y]) break;
            }
            next = (w != NONE && adj[w].size() == 2) ? w : NONE;
        }
    }
    uint64_t k = 0;
    for (uint64_t e = 0; e < m; ++e)
        if (!deleted[u[e]] && !deleted[v[e]]) kept[k++] = e;
    *m_kept = k;
    return 0;
}

// distributed_version/tools/graph-convert/remove_equivalent_vertices.cpp:
// vertex x's set is {x} plus its adjacency entries, sorted (:151-167, a
// multiset); vertices are taken by (set size, id) (:168-181) and within one
// size every vertex that is not yet redundant marks each later vertex with an
// equal set redundant (:230-287).  Set equality is an equivalence, so that
// leaves exactly the smallest id of every class of equal sets; the
// restatement finds the classes with an ordered map instead of comparing
// pairs within a size.  The rest are numbered by ascending id (:295-303) and
// the kept edges (no redundant end, :318-327) written with those ids; the
// tool's vertex count is 1 + the largest new id on a kept edge (:322), 0 when
// no edge is kept.  new_id of a redundant vertex is 2^32 - 1.
int orc_reduce_equivalent(uint64_t m, const uint32_t *u, const uint32_t *v, uint32_t n, uint8_t *redundant,
                          uint32_t *new_id, uint64_t *kept, uint64_t *m_kept, uint32_t *n_out)
{
    for (uint64_t e = 0; e < m; ++e)
        if (u[e] >= n || v[e] >= n) return 1;
    std::vector<std::vector<uint32_t>> set(n);
    for (uint32_t x = 0; x < n; ++x) set[x].push_back(x);
    for (uint64_t e = 0; e < m; ++e) {
        set[u[e]].push_back(v[e]);
        set[v[e]].push_back(u[e]);
    }
    for (auto &l : set) std::sort(l.begin(), l.end());
    std::map<std::vector<uint32_t>, uint32_t> first;
    for (uint32_t x = 0; x < n; ++x) redundant[x] = first.emplace(set[x], x).second ? 0 : 1;
    uint32_t next = 0;
    for (uint32_t x = 0; x < n; ++x) new_id[x] = redundant[x] ? 0xffffffffu : next++;
    uint64_t k = 0;
    uint32_t top = 0;
    for (uint64_t e = 0; e < m; ++e)
        if (!redundant[u[e]] && !redundant[v[e]]) {
            kept[k++] = e;
            top = std::max(top, std::max(new_id[u[e]], new_id[v[e]]) + 1);
        }
    *m_kept = k;
    *n_out = top;
    return 0;
}

}  // extern "C"
