/*
 * oracle_clust.cpp -- CPU restatement of CRiSPy's aveclust
 * (src/aveclust/aveclust.cpp), step for step.
 *
 * TEST INFRASTRUCTURE ONLY (what tests compare crispy_aveclust with, and the
 * timed CPU baseline of bench.py; the product never links it).  Tree nodes live
 * on the heap and point at each other, link maps are std::unordered_map
 * keyed by node ID, every merge scans the active nodes between the two IDs
 * and takes min_element over all exact / inexact distances -- the
 * reference's own data flow, so it also has the reference's cost.  It
 * writes only the _Merge file (the decisions); pinned against the
 * reference's aveclust compiled from source (oracle/_ref/aveclust) by
 * tests/test_clust_host.py.
 */
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <map>
#include <string>
#include <unordered_map>
#include <vector>

#include "oracle.h"

namespace {

struct Edge {
    unsigned int num = 0;
    float sum = 0.0f;
};

struct TNode {
    unsigned int id;
    TNode* top;
    TNode* parent = nullptr;
    TNode* left = nullptr;
    TNode* right = nullptr;
    float dist = 0.0f;
    unsigned int members = 1;
    std::unordered_map<unsigned int, Edge> links;
    explicit TNode(unsigned int i) : id(i), top(this) {}
};

struct State {
    std::vector<TNode*> leaves, activeN, exactN;
    std::vector<float> exactD, inexactD;
    unsigned int next_id = 0;
    unsigned long long edges = 0;
    bool loaded = false;
    float lam = 0.0f;
};

void set_top(TNode* n, TNode* p) {   // updateTopParent (aveclust.cpp:372-378)
    if (!n) return;
    n->top = p;
    set_top(n->left, p);
    set_top(n->right, p);
}

// computeDist (aveclust.cpp:381-412)
void cdist(State& S, TNode* x, TNode* y, float level) {
    auto it = x->links.find(y->id);
    if (it == x->links.end()) return;
    const unsigned int tot = x->members * y->members;
    const float s = it->second.sum;
    const unsigned int miss = tot - it->second.num;
    if (miss == 0 || S.loaded) {
        const float d = (s + level * miss) / tot;
        if (d < S.exactD[x->id]) { S.exactD[x->id] = d; S.exactN[x->id] = y; }
    } else {
        const float d = (s + S.lam * miss) / tot;
        if (d < S.inexactD[x->id]) S.inexactD[x->id] = d;
    }
}

void umin(State& S, TNode* x, float level) {   // updateMin (aveclust.cpp:414-435)
    S.exactD[x->id] = 1.0f;
    for (auto& kv : x->links) {
        TNode* t = S.activeN[kv.first];
        if (x->id > kv.first) cdist(S, x, t, level);
        else cdist(S, t, x, level);
    }
}

// addNode (aveclust.cpp:439-538), x->id > y->id
void join(State& S, TNode* x, TNode* y, TNode* p, float d, float level) {
    const unsigned int ix = x->id, iy = y->id;
    p->left = x;
    p->right = y;
    x->parent = p;
    y->parent = p;
    set_top(x, p);
    set_top(y, p);
    p->dist = d;
    p->members = x->members + y->members;
    x->links.erase(iy);
    --S.edges;
    p->links = x->links;
    for (auto& kv : y->links) {
        p->links[kv.first].num += kv.second.num;
        p->links[kv.first].sum += kv.second.sum;
    }
    x->links.clear();
    y->links.clear();
    for (unsigned int i = iy + 1; i < ix; ++i) {
        TNode* t = S.activeN[i];
        if (t && t->links.find(iy) != t->links.end()) {
            p->links[i].sum += t->links[iy].sum;
            p->links[i].num += t->links[iy].num;
            t->links.erase(iy);
            --S.edges;
        }
    }
    for (unsigned int i = ix + 1; i < S.next_id; ++i) {
        TNode* t = S.activeN[i];
        if (!t) continue;
        if (t->links.find(ix) != t->links.end()) {
            p->links[i].sum += t->links[ix].sum;
            p->links[i].num += t->links[ix].num;
            t->links.erase(ix);
            --S.edges;
        }
        if (t->links.find(iy) != t->links.end()) {
            p->links[i].sum += t->links[iy].sum;
            p->links[i].num += t->links[iy].num;
            t->links.erase(iy);
            --S.edges;
        }
    }
    S.edges += p->links.size();
    S.activeN[ix] = S.activeN[iy] = nullptr;
    S.exactN[ix] = S.exactN[iy] = nullptr;
    S.exactD[ix] = S.exactD[iy] = 1.0f;
    S.inexactD[ix] = S.inexactD[iy] = 1.0f;
    for (auto& kv : p->links) {
        TNode* t = S.activeN[kv.first];
        cdist(S, p, t, level);
        if (S.exactN[kv.first] == x || S.exactN[kv.first] == y) umin(S, t, level);
    }
}

}  // namespace

extern "C" int oracle_aveclust(const uint32_t* const* pairs, const float* const* dists,
                               const int64_t* counts, int nchunks, int num_reads, float end_level,
                               const char* merge_path, int64_t* merges_out) {
    if (num_reads < 1 || nchunks < 1) return -1;
    if (end_level < 0.0f || end_level > 1.0f)
        end_level = (float)(num_reads > 500 ? std::min(1 / std::log2((double)num_reads), 1.0)
                                            : std::min(1 / std::log10((double)num_reads), 1.0));
    State S;
    const size_t cap = 2 * (size_t)num_reads + 1;
    S.activeN.assign(cap, nullptr);
    S.exactN.assign(cap, nullptr);
    S.exactD.assign(cap, 1.0f);
    S.inexactD.assign(cap, 1.0f);
    for (int i = 0; i < num_reads; ++i) {
        S.leaves.push_back(new TNode((unsigned)i));
        S.activeN[i] = S.leaves.back();
    }
    S.next_id = (unsigned)num_reads;
    FILE* mf = std::fopen(merge_path, "w");
    if (!mf) return -3;
    struct Key { unsigned int x, y; int c; };
    std::multimap<float, Key> heads;
    std::vector<int64_t> pos((size_t)nchunks, 0);
    unsigned int ix = 0, iy = 0;
    float dist = 0.0f;
    auto next = [&](int c) {
        if (pos[c] >= counts[c]) return false;
        ix = pairs[c][2 * pos[c]];
        iy = pairs[c][2 * pos[c] + 1];
        dist = dists[c][pos[c]];
        ++pos[c];
        return true;
    };
    for (int c = 0; c < nchunks; ++c)
        if (next(c)) heads.insert(std::make_pair(dist, Key{ix, iy, c}));
    unsigned long long cap_edges = (unsigned long long)num_reads;
    int64_t merges = 0;
    while (!S.loaded) {
        if (S.edges < cap_edges) {
            while (S.edges <= cap_edges && !heads.empty()) {
                auto it = heads.begin();
                const int c = it->second.c;
                ix = it->second.x;
                iy = it->second.y;
                dist = it->first;
                if (dist < end_level || std::fabs(dist - end_level) < 1e-6) {   // absorb (aveclust.cpp:562-590)
                    TNode* a = S.leaves[ix]->top;   // leaves are the first num_reads entries
                    TNode* b = S.leaves[iy]->top;
                    if (a->id < b->id) std::swap(a, b);
                    if (a->id > b->id) {
                        if (a->links.find(b->id) == a->links.end()) ++S.edges;
                        a->links[b->id].sum += dist;
                        ++a->links[b->id].num;
                    }
                }
                heads.erase(it);
                if (next(c)) heads.insert(std::make_pair(dist, Key{ix, iy, c}));
            }
            if (dist > S.lam) S.lam = dist;
        } else {
            cap_edges *= 2;
            if (cap_edges > 2e8) end_level = S.lam;
        }
        if (heads.empty()) S.loaded = true;
        // updateAllMin (aveclust.cpp:621-647)
        std::fill(S.exactD.begin(), S.exactD.end(), 1.0f);
        std::fill(S.inexactD.begin(), S.inexactD.end(), 1.0f);
        for (TNode* x : S.activeN) {
            if (!x || x->links.empty()) continue;
            for (auto& kv : x->links) {
                TNode* y = S.activeN[kv.first];
                if (x->id > y->id) cdist(S, x, y, end_level);
                else cdist(S, y, x, end_level);
            }
        }
        float min_in = *std::min_element(S.inexactD.begin(), S.inexactD.end());
        auto mi = std::min_element(S.exactD.begin(), S.exactD.end());
        float min_ex = *mi;
        while (min_ex < 1.0f && (min_ex < min_in || std::fabs(min_ex - min_in) < 1e-6)) {
            const size_t k = (size_t)(mi - S.exactD.begin());
            TNode* a = S.activeN[k]->top;
            TNode* b = S.exactN[k]->top;
            TNode* p = new TNode(S.next_id);   // merge (aveclust.cpp:541-559)
            S.leaves.push_back(p);             // kept for the clean-up below
            S.activeN[S.next_id] = p;
            if (a->id > b->id) join(S, a, b, p, min_ex, end_level);
            else join(S, b, a, p, min_ex, end_level);
            ++S.next_id;
            std::fprintf(mf, "%d %d %.6f\n", (int)a->id + 1, (int)b->id + 1, min_ex);
            ++merges;
            min_in = *std::min_element(S.inexactD.begin(), S.inexactD.end());
            mi = std::min_element(S.exactD.begin(), S.exactD.end());
            min_ex = *mi;
        }
    }
    std::fclose(mf);
    if (merges_out) *merges_out = merges;
    for (TNode* n : S.leaves) delete n;
    return 0;
}
