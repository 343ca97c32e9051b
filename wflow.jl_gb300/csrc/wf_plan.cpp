// wf_plan.cpp -- long-path chain decomposition and slot layout of a drainage forest.
#include "wf_plan.h"

#include <algorithm>
#include <numeric>

#include "wflow_gb300.h"

int wf_build_plan(int64_t n, const int32_t* ds, int32_t members, WfRoutingPlan& P, std::string& err,
                  const int64_t* heavy_hint) {
    P = WfRoutingPlan();
    P.n = n;
    P.M = members < 1 ? 1 : members;
    if (P.M <= 32) {
        if ((P.M & (P.M - 1)) != 0) {
            err = "members must be a power of two up to 32 or a multiple of 32";
            return -1;
        }
        P.G = 32 / P.M;
    } else {
        if (P.M % 32 != 0) {
            err = "members must be a power of two up to 32 or a multiple of 32";
            return -1;
        }
        P.G = 1;
    }
    if (n == 0) {
        P.chunk_base.assign(1, 0);
        P.up_ptr.assign(1, 0);
        return 0;
    }
    for (int64_t i = 0; i < n; ++i) {
        if (ds[i] < -1 || ds[i] >= n || ds[i] == i) {
            err = "downstream index out of range at node " + std::to_string(i);
            return ds[i] == i ? WF_ERR_CYCLE : -1;
        }
    }
    // children CSR (ascending node index)
    std::vector<int32_t> indeg(n, 0);
    for (int64_t i = 0; i < n; ++i)
        if (ds[i] >= 0) indeg[ds[i]]++;
    std::vector<int64_t> cptr(n + 1, 0);
    for (int64_t i = 0; i < n; ++i) cptr[i + 1] = cptr[i] + indeg[i];
    std::vector<int64_t> child(cptr[n]);
    {
        std::vector<int64_t> fill(cptr.begin(), cptr.end() - 1);
        for (int64_t i = 0; i < n; ++i)
            if (ds[i] >= 0) child[fill[ds[i]]++] = i;
    }
    // heights by Kahn order from the leaves
    std::vector<int32_t> height(n, 0), left(indeg);
    std::vector<int64_t> order;
    order.reserve(n);
    for (int64_t i = 0; i < n; ++i)
        if (left[i] == 0) order.push_back(i);
    for (size_t q = 0; q < order.size(); ++q) {
        int64_t v = order[q];
        int64_t d = ds[v];
        if (d >= 0) {
            if (height[v] + 1 > height[d]) height[d] = height[v] + 1;
            if (--left[d] == 0) order.push_back(d);
        }
    }
    if ((int64_t)order.size() != n) {
        err = "cycle in drainage graph";
        return WF_ERR_CYCLE;
    }
    // heavy child: the hinted child, else the highest child (ties to the lowest node index)
    std::vector<int64_t> heavy(n, -1);
    for (int64_t v = 0; v < n; ++v) {
        int64_t best = -1;
        for (int64_t k = cptr[v]; k < cptr[v + 1]; ++k) {
            int64_t u = child[k];
            if (best < 0 || height[u] > height[best]) best = u;
        }
        if (heavy_hint && heavy_hint[v] >= 0) {
            const int64_t u = heavy_hint[v];
            if (u >= n || ds[u] != v) {
                err = "heavy-child hint is not a child of its node";
                return -1;
            }
            best = u;
        }
        heavy[v] = best;
    }
    // chains from every leaf; key = height of the chain's end + 1, which equals the length when
    // every heavy child is the highest one, and which grows strictly from a chain to the chain
    // it flows into whatever the heavy children are (heights grow strictly downstream), so that
    // ordering by key is a dependency order with heavy-child hints too
    struct Chain {
        int64_t start;
        int32_t len;
        int64_t end;
        int32_t key;
    };
    std::vector<Chain> chains;
    for (int64_t v = 0; v < n; ++v) {
        if (indeg[v] != 0) continue;
        int64_t u = v;
        int32_t len = 1;
        while (ds[u] >= 0 && heavy[ds[u]] == u) {
            u = ds[u];
            ++len;
        }
        chains.push_back({v, len, u, height[u] + 1});
    }
    std::stable_sort(chains.begin(), chains.end(), [](const Chain& a, const Chain& b) {
        return a.key != b.key ? a.key < b.key : a.end < b.end;
    });
    P.hinted = heavy_hint != nullptr;
    const int G = P.G;
    const int64_t nc_real = (int64_t)chains.size();
    // Dispatch order. The sweeps first dispatch, all at once, the chains at the end of the order
    // (one chain per chunk; wave_grid caps them at half the resident warps), then the others in
    // key order (the length, without heavy-child hints), which is a dependency order (a light
    // child is strictly shorter than its consumer, and its end strictly lower), short chains
    // batched. The first group holds up to kFirst chains: the longest
    // ones (at least max(64, longest / 8) nodes), which carry the critical path, and then the
    // most urgent of the rest: with one time unit per position, a chain ending at position k of
    // its consumer must start by LS(c) = LS(consumer) + k - len(c) (a chain ending at a pit by
    // longest - len(c)), and the chains of smallest LS are the short tributaries the critical
    // chains would otherwise wait for while the bulk of the short chains is walked. A consumer
    // never has a later LS than its light children and is longer, so the group holds the
    // consumer of every chain in it. Within the group the order is by latest finish LS + len,
    // again a dependency order (a light child finishes strictly before its consumer), the
    // longest-finishing chain (the main stem) last, so dispatched first.
    constexpr int64_t kFirst = 256;
    int64_t n_solo = 0;
    if (nc_real > 0) {
        int32_t longest = 0;
        for (const Chain& c : chains) longest = std::max(longest, c.len);
        std::vector<int64_t> chain_of(n, -1), pos_of(n, -1);
        for (int64_t c = 0; c < nc_real; ++c) {
            int64_t u = chains[c].start;
            for (int32_t k = 0; k < chains[c].len; ++k) {
                chain_of[u] = c;
                pos_of[u] = k;
                u = ds[u];
            }
        }
        std::vector<int64_t> ls(nc_real, 0);
        for (int64_t c = nc_real - 1; c >= 0; --c) {  // consumers (longer) before their light children
            const int64_t d = ds[chains[c].end];
            ls[c] = d < 0 ? (int64_t)longest - chains[c].len : ls[chain_of[d]] + pos_of[d] - chains[c].len;
        }
        std::vector<char> first(nc_real, 0);
        const int32_t thr = std::max<int32_t>(64, longest / 8);
        for (int64_t c = nc_real - 1; c >= 0 && n_solo < kFirst && chains[c].key >= thr; --c) {
            first[c] = 1;
            ++n_solo;
        }
        std::vector<int64_t> by_ls(nc_real);
        for (int64_t c = 0; c < nc_real; ++c) by_ls[c] = c;
        std::stable_sort(by_ls.begin(), by_ls.end(), [&](int64_t x, int64_t y) {
            return ls[x] != ls[y] ? ls[x] < ls[y] : chains[x].len > chains[y].len;
        });
        for (int64_t i = 0; i < nc_real && n_solo < kFirst; ++i)
            if (!first[by_ls[i]]) {
                first[by_ls[i]] = 1;
                ++n_solo;
            }
        // the first group's consumers: the urgent prefix is closed under consumers, the long
        // chains too (a consumer is longer); add any consumer missed at the budget's edge
        for (bool grew = true; grew;) {
            grew = false;
            for (int64_t c = 0; c < nc_real; ++c) {
                const int64_t d = ds[chains[c].end];
                if (first[c] && d >= 0 && !first[chain_of[d]]) {
                    first[chain_of[d]] = 1;
                    ++n_solo;
                    grew = true;
                }
            }
        }
        std::vector<int64_t> grp;
        std::vector<Chain> re;
        re.reserve(nc_real);
        for (int64_t c = 0; c < nc_real; ++c) {
            if (first[c]) grp.push_back(c);
            else re.push_back(chains[c]);  // length order kept
        }
        std::stable_sort(grp.begin(), grp.end(), [&](int64_t x, int64_t y) {
            const int64_t fx = ls[x] + chains[x].len, fy = ls[y] + chains[y].len;
            return fx != fy ? fx < fy : chains[x].len < chains[y].len;
        });
        for (int64_t c : grp) re.push_back(chains[c]);
        chains.swap(re);
    }
    const int64_t n_packed = nc_real - n_solo;
    const int64_t packed_chains = (n_packed + G - 1) / G * G;
    const int64_t packed_chunks = packed_chains / G;
    P.n_chains = packed_chains + n_solo;
    P.n_chunks = packed_chunks + n_solo;
    P.chain_len.assign(P.n_chains, 0);
    P.chunk_len.assign(P.n_chunks, 0);
    P.chunk_g.assign(P.n_chunks, G);
    P.chunk_chain0.assign(P.n_chunks, 0);
    P.chunk_base.assign(P.n_chunks + 1, 0);
    std::vector<int64_t> chain_id(nc_real);  // sorted chain -> chain index (padding skipped)
    for (int64_t c = 0; c < nc_real; ++c) {
        chain_id[c] = c < n_packed ? c : packed_chains + (c - n_packed);
        P.chain_len[chain_id[c]] = chains[c].len;
    }
    for (int64_t k = 0; k < P.n_chunks; ++k) {
        const int gk = k < packed_chunks ? G : 1;
        const int64_t c0 = k < packed_chunks ? k * G : packed_chains + (k - packed_chunks);
        P.chunk_g[k] = gk;
        P.chunk_chain0[k] = c0;
        int32_t mx = 0;
        for (int g = 0; g < gk; ++g) mx = std::max(mx, P.chain_len[c0 + g]);
        P.chunk_len[k] = mx;
        P.chunk_base[k + 1] = P.chunk_base[k] + (int64_t)mx * gk;
        P.max_len = std::max(P.max_len, mx);
    }
    P.n_slots = P.chunk_base[P.n_chunks];
    P.n_long_chunks = n_solo;  // the first group, dispatched first
    P.slot_of_node.assign(n, -1);
    P.node_of_slot.assign(P.n_slots, -1);
    P.chain_of_node.assign(n, -1);
    P.is_chain_end.assign(P.n_slots, 0);
    for (int64_t c = 0; c < nc_real; ++c) {
        const int64_t id = chain_id[c];
        const int64_t chunk = id < packed_chains ? id / G : packed_chunks + (id - packed_chains);
        const int64_t g = id < packed_chains ? id % G : 0;
        const int gk = P.chunk_g[chunk];
        int64_t u = chains[c].start;
        for (int32_t k = 0; k < chains[c].len; ++k) {
            int64_t s = P.chunk_base[chunk] + (int64_t)k * gk + g;
            P.slot_of_node[u] = s;
            P.node_of_slot[s] = u;
            P.chain_of_node[u] = (int32_t)id;
            if (k == chains[c].len - 1) P.is_chain_end[s] = 1;
            u = ds[u];
        }
    }
    P.ds_slot.assign(P.n_slots, -1);
    P.up_ptr.assign(P.n_slots + 1, 0);
    for (int64_t s = 0; s < P.n_slots; ++s) {
        int64_t v = P.node_of_slot[s];
        P.up_ptr[s + 1] = P.up_ptr[s] + (v >= 0 ? (int32_t)(cptr[v + 1] - cptr[v]) : 0);
        if (v >= 0 && ds[v] >= 0) P.ds_slot[s] = P.slot_of_node[ds[v]];
    }
    P.up_slot.resize(P.up_ptr[P.n_slots]);
    P.up_chain.resize(P.up_ptr[P.n_slots]);
    for (int64_t s = 0; s < P.n_slots; ++s) {
        int64_t v = P.node_of_slot[s];
        if (v < 0) continue;
        int32_t o = P.up_ptr[s];
        for (int64_t k = cptr[v]; k < cptr[v + 1]; ++k, ++o) {
            int64_t u = child[k];
            P.up_slot[o] = P.slot_of_node[u];
            P.up_chain[o] = (u == heavy[v]) ? -1 : P.chain_of_node[u];
        }
    }
    return 0;
}

bool wf_check_plan(const WfRoutingPlan& P, const int32_t* ds, std::string& err) {
    // chain lengths sorted before the first-dispatched group (padding chains have length 0;
    // with heavy-child hints the order is by end height, checked through the per-node condition
    // below); every chain waits only for chains of smaller index (checked per node below)
    int32_t prev = 0;
    for (int64_t c = 0; c < P.n_chains - P.n_long_chunks && !P.hinted; ++c) {
        if (P.chain_len[c] == 0) continue;
        if (P.chain_len[c] < prev) {
            err = "chains not sorted by length";
            return false;
        }
        prev = P.chain_len[c];
    }
    for (int64_t s = 0; s < P.n_slots; ++s) {
        int64_t v = P.node_of_slot[s];
        if (v < 0) continue;
        int64_t chunk = 0;
        while (P.chunk_base[chunk + 1] <= s) ++chunk;
        const int G = P.chunk_g[chunk];
        int64_t k = (s - P.chunk_base[chunk]) / G;
        int64_t my_chain = P.chain_of_node[v];
        for (int32_t o = P.up_ptr[s]; o < P.up_ptr[s + 1]; ++o) {
            int64_t us = P.up_slot[o];
            int64_t u = P.node_of_slot[us];
            if (u < 0 || ds[u] != v) {
                err = "upstream list mismatch";
                return false;
            }
            if (P.up_chain[o] < 0) {
                if (us != s - G) {
                    err = "heavy child is not the previous chain position";
                    return false;
                }
            } else {
                int64_t uc = P.up_chain[o];
                if (!P.is_chain_end[us] || uc >= my_chain || (!P.hinted && P.chain_len[uc] > k)) {
                    err = "light child chain does not precede its consumer";
                    return false;
                }
            }
        }
    }
    return true;
}

extern "C" {

// Host-only entry used by the tests: plan a graph and return its schedule summary.
//   out_counts[0..3] = n_chains, n_chunks, n_slots, max_len
//   slot_of_node[n] (may be null), ok = 1 when wf_check_plan passes.
int32_t wf_plan_routing(int64_t n, const int32_t* downstream, int32_t members, int64_t* out_counts,
                        int64_t* slot_of_node, int32_t* ok, int32_t* g_out) {
    WfRoutingPlan P;
    std::string err;
    int rc = wf_build_plan(n, downstream, members, P, err);
    if (rc != 0) return rc;
    out_counts[0] = P.n_chains;
    out_counts[1] = P.n_chunks;
    out_counts[2] = P.n_slots;
    out_counts[3] = P.max_len;
    if (slot_of_node)
        for (int64_t i = 0; i < n; ++i) slot_of_node[i] = P.slot_of_node[i];
    *ok = wf_check_plan(P, downstream, err) ? 1 : 0;
    *g_out = P.G;
    return 0;
}

// The same with heavy-child hints (heavy_hint [n], -1: none): chain_of_node [n] (optional)
// receives each node's chain.
int32_t wf_plan_routing_hinted(int64_t n, const int32_t* downstream, int32_t members, const int64_t* heavy_hint,
                               int64_t* out_counts, int64_t* chain_of_node, int32_t* ok, int32_t* g_out) {
    WfRoutingPlan P;
    std::string err;
    int rc = wf_build_plan(n, downstream, members, P, err, heavy_hint);
    if (rc != 0) return rc;
    out_counts[0] = P.n_chains;
    out_counts[1] = P.n_chunks;
    out_counts[2] = P.n_slots;
    out_counts[3] = P.max_len;
    if (chain_of_node)
        for (int64_t i = 0; i < n; ++i) chain_of_node[i] = P.chain_of_node[i];
    *ok = wf_check_plan(P, downstream, err) ? 1 : 0;
    *g_out = P.G;
    return 0;
}

}  // extern "C"
