// clust.cpp -- aveclust: sparse average-linkage clustering of the genDist
// chunks (src/aveclust/aveclust.cpp), the step crispy.sh:24 runs after
// genDist.
//
// The reference streams the .npair_N / .ndist_N chunks through a multimap
// (the smallest distance of all chunk heads first, equal distances in
// insertion order), absorbs each edge into the link map of the larger of the
// two current cluster roots, and between batches merges the pair of clusters
// with the smallest exact average distance while it does not exceed the
// smallest lower bound of the incomplete ones (lambda bound).  Every
// decision depends on the exact float values and on the iteration order of
// the link maps (std::unordered_map: a strict `<` keeps the first minimum
// met), so this restatement performs the same container operations in the
// same order.  What changes is only how the work is found:
//   * addNode scans every active node between two IDs for links to the two
//     merged clusters (aveclust.cpp:466-520); here a reverse index lists the
//     holders of each key, visited in the same ascending order;
//   * min_element over the 2n+1 exact / inexact distances after every merge
//     (aveclust.cpp:978-986) becomes a tournament tree with the same
//     leftmost-minimum answer;
//   * updateTopParent re-labels a whole subtree at every merge
//     (aveclust.cpp:372-378); here the root of a leaf is found on demand
//     through the parent links (with path compression), which yields the
//     same node;
//   * the parent takes over the larger node's link map by a move, not a
//     copy (the map is cleared right after), and a computeDist for a link
//     found by iterating the map uses that entry instead of a second lookup.
// The _Merge file and the -o edge files are byte-identical to the
// reference's.  The .Cluster / .Cluster_List lines hold the same clusters;
// the reference orders them by iterating a hash set of node pointers
// (aveclust.cpp:244-305), an order this code cannot and does not copy: it
// visits roots by ascending node ID.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "internal.h"

namespace {

constexpr double kEps = 1e-6;              // EPSILON (aveclust.cpp:18)
constexpr double kUpperEdges = 2e8;        // UPPER_BOUND_NUM_EDGES (aveclust.cpp:19)

struct Link {
    unsigned int num = 0;
    float sum = 0.0f;
};
using LinkMap = std::unordered_map<unsigned int, Link>;

struct Node {
    unsigned int id = 0;
    int parent = -1, left = -1, right = -1;   // node indices (= IDs)
    float dist = 0.0f;
    unsigned int members = 1;
    LinkMap links;
};

// Leftmost minimum over a float array with point updates (a min_element
// that stays current).  Writes land in the array at once; the tree above
// them is brought up to date when the minimum is next asked for, so the
// many updates of one entry between two queries cost one path.
struct MinTree {
    int n = 1;
    std::vector<float> v;
    std::vector<int> t;          // index of the leftmost minimum of each subtree
    std::vector<int> pending;    // entries written since the last query
    std::vector<char> marked;
    void init(int size, float fill) {
        n = 1;
        while (n < size) n <<= 1;
        v.assign(n, 0.0f);
        t.assign(2 * n, 0);
        marked.assign(n, 0);
        pending.clear();
        for (int i = 0; i < n; ++i) v[i] = i < size ? fill : INFINITY;
        for (int i = 0; i < n; ++i) t[n + i] = i;
        rebuild();
    }
    int pick(int a, int b) const { return v[b] < v[a] ? b : a; }   // ties: the left one
    void rebuild() {
        for (int i = n - 1; i > 0; --i) t[i] = pick(t[2 * i], t[2 * i + 1]);
        for (int i : pending) marked[i] = 0;
        pending.clear();
    }
    void set(int i, float x) {
        v[i] = x;
        if (!marked[i]) { marked[i] = 1; pending.push_back(i); }
    }
    void fill(float x, int size) {
        for (int i = 0; i < size; ++i) v[i] = x;
        rebuild();
    }
    void flush() {
        for (int i : pending) {
            marked[i] = 0;
            for (int p = (n + i) >> 1; p; p >>= 1) t[p] = pick(t[2 * p], t[2 * p + 1]);
        }
        pending.clear();
    }
    int argmin() { flush(); return t[1]; }
    float min() { flush(); return v[t[1]]; }
    float operator[](int i) const { return v[i]; }
};

struct Clusterer {
    int num_reads;
    float end_level;
    float lambda = 0.0f;
    bool all_loaded = false;
    unsigned long long total_edges = 0;
    unsigned int new_id;
    std::vector<Node> nodes;            // every node ever made, index = ID
    std::vector<char> active;           // vActiveNodes[i] != 0
    std::vector<int> exact_node;        // vExactNodes (node ID, -1 = none)
    MinTree exact, inexact;             // vExactDist, vInexactDist
    // key -> IDs that may hold it: one singly linked list per key in a
    // shared pool (head[key], then next[] through pool entries)
    std::vector<int> hold_head;
    std::vector<unsigned int> hold_id;
    std::vector<int> hold_next;
    std::vector<int> owner;             // a merged node's link map moved to this node
    std::vector<int> up;                // root search shortcut (path-compressed parents)

    explicit Clusterer(int n, float level) : num_reads(n), end_level(level), new_id((unsigned)n) {
        const size_t cap = 2 * (size_t)n + 1;
        nodes.resize(cap);
        active.assign(cap, 0);
        exact_node.assign(cap, -1);
        hold_head.assign(cap, -1);
        owner.assign(cap, -1);
        up.assign(cap, -1);
        for (int i = 0; i < n; ++i) {
            nodes[i].id = (unsigned)i;
            active[i] = 1;
        }
        exact.init((int)cap, 1.0f);
        inexact.init((int)cap, 1.0f);
    }

    // topParent: the root of the tree that holds node i
    int root(int i) {
        int r = i;
        while (up[r] >= 0) r = up[r];
        while (up[i] >= 0) {
            const int nx = up[i];
            up[i] = r;
            i = nx;
        }
        return r;
    }

    void add_holder(unsigned int key, unsigned int id) {
        hold_id.push_back(id);
        hold_next.push_back(hold_head[key]);
        hold_head[key] = (int)hold_id.size() - 1;
    }

    // linkMap[key] (inserting a zero link when absent, at the same place
    // operator[] would), recording a new holder; *fresh tells whether it
    // was inserted
    Link& link_at(Node& holder, unsigned int key, bool* fresh = nullptr) {
        auto r = holder.links.try_emplace(key);
        if (r.second) add_holder(key, holder.id);
        if (fresh) *fresh = r.second;
        return r.first->second;
    }

    // absorb (aveclust.cpp:562-590)
    void absorb(unsigned int a, unsigned int b, float d) {
        Node& x = nodes[root((int)a)];
        Node& y = nodes[root((int)b)];
        bool fresh = false;
        if (x.id > y.id) {
            Link& l = link_at(x, y.id, &fresh);
            if (fresh) ++total_edges;
            l.sum += d;
            ++l.num;
        } else if (y.id > x.id) {
            Link& l = link_at(y, x.id, &fresh);
            if (fresh) ++total_edges;
            l.sum += d;
            ++l.num;
        }
    }

    // computeDist (aveclust.cpp:381-412), x.id > y.id
    void compute(Node& x, Node& y) {
        auto it = x.links.find(y.id);
        if (it != x.links.end()) compute_link(x, y, it->second);
    }
    // the same for a link entry of x already in hand (no second lookup)
    void compute_link(Node& x, Node& y, const Link& lk) {
        const unsigned int total = x.members * y.members;
        const float sum = lk.sum;
        const unsigned int unlinked = total - lk.num;
        if (unlinked == 0 || all_loaded) {
            const float d = (sum + end_level * (float)unlinked) / (float)total;
            if (d < exact[x.id]) {
                exact.set((int)x.id, d);
                exact_node[x.id] = (int)y.id;
            }
        } else {
            const float d = (sum + lambda * (float)unlinked) / (float)total;
            if (d < inexact[x.id]) inexact.set((int)x.id, d);
        }
    }

    // updateMin (aveclust.cpp:414-435)
    void update_min(Node& x) {
        exact.set((int)x.id, 1.0f);
        for (auto& kv : x.links) {
            Node& t = nodes[kv.first];
            if (x.id > kv.first) compute_link(x, t, kv.second);
            else compute(t, x);
        }
    }

    // the node whose link map now holds what node i held
    unsigned int owner_of(unsigned int i) {
        unsigned int r = i;
        while (owner[r] >= 0) r = (unsigned)owner[r];
        while (owner[i] >= 0) {
            const unsigned int nx = (unsigned)owner[i];
            owner[i] = (int)r;
            i = nx;
        }
        return r;
    }

    // IDs in (lo, hi) that hold `key`, ascending
    std::vector<unsigned int> holders_in(unsigned int key, unsigned int lo, unsigned int hi) {
        std::vector<unsigned int> out;
        for (int e = hold_head[key]; e >= 0; e = hold_next[e]) {
            const unsigned int i = owner_of(hold_id[e]);
            if (i > lo && i < hi && active[i] && nodes[i].links.count(key)) out.push_back(i);
        }
        std::sort(out.begin(), out.end());
        out.erase(std::unique(out.begin(), out.end()), out.end());
        return out;
    }

    // addNode (aveclust.cpp:439-538), x.id > y.id
    void add_node(Node& x, Node& y, Node& p, float d) {
        const unsigned int ix = x.id, iy = y.id;
        p.left = (int)ix;
        p.right = (int)iy;
        x.parent = (int)p.id;
        y.parent = (int)p.id;
        up[ix] = (int)p.id;
        up[iy] = (int)p.id;
        p.dist = d;
        p.members = x.members + y.members;
        x.links.erase(iy);
        --total_edges;
        // parentNode->linkMap = nodeX->linkMap: x's map is cleared right
        // after, so it moves (same table, same iteration order), and the
        // holders of its keys reach p through owner[]
        p.links = std::move(x.links);
        x.links = LinkMap();
        owner[ix] = (int)p.id;
        for (auto& kv : y.links) {
            Link& l = link_at(p, kv.first);
            l.num += kv.second.num;
            l.sum += kv.second.sum;
        }
        x.links.clear();
        y.links.clear();
        // holders of y's key between the two IDs, ascending
        for (unsigned int i : holders_in(iy, iy, ix)) {
            Node& t = nodes[i];
            Link& src = t.links[iy];
            Link& l = link_at(p, i);
            l.sum += src.sum;
            l.num += src.num;
            t.links.erase(iy);
            --total_edges;
        }
        // holders of x's or y's key above x's ID, ascending; x's first
        std::vector<unsigned int> hx = holders_in(ix, ix, new_id), hy = holders_in(iy, ix, new_id);
        std::vector<unsigned int> all;
        std::merge(hx.begin(), hx.end(), hy.begin(), hy.end(), std::back_inserter(all));
        all.erase(std::unique(all.begin(), all.end()), all.end());
        for (unsigned int i : all) {
            Node& t = nodes[i];
            auto ax = t.links.find(ix);
            if (ax != t.links.end()) {
                const Link src = ax->second;
                Link& l = link_at(p, i);
                l.sum += src.sum;
                l.num += src.num;
                t.links.erase(ix);
                --total_edges;
            }
            auto ay = t.links.find(iy);
            if (ay != t.links.end()) {
                const Link src = ay->second;
                Link& l = link_at(p, i);
                l.sum += src.sum;
                l.num += src.num;
                t.links.erase(iy);
                --total_edges;
            }
        }
        total_edges += p.links.size();
        active[ix] = active[iy] = 0;
        exact_node[ix] = exact_node[iy] = -1;
        exact.set((int)ix, 1.0f);
        exact.set((int)iy, 1.0f);
        inexact.set((int)ix, 1.0f);
        inexact.set((int)iy, 1.0f);
        hold_head[ix] = hold_head[iy] = -1;   // the keys die with the two nodes
        for (auto& kv : p.links) {
            Node& t = nodes[kv.first];
            compute_link(p, t, kv.second);
            if (exact_node[kv.first] == (int)ix || exact_node[kv.first] == (int)iy) update_min(t);
        }
    }

    // merge (aveclust.cpp:541-559)
    void merge(int a, int b, float d) {
        Node& p = nodes[new_id];
        p.id = new_id;
        active[new_id] = 1;
        if (nodes[a].id > nodes[b].id) add_node(nodes[a], nodes[b], p, d);
        else add_node(nodes[b], nodes[a], p, d);
        ++new_id;
    }

    // updateAllMin (aveclust.cpp:621-647).  A node's links are keyed by
    // smaller IDs, so computeDist only ever writes the node's own exact /
    // inexact entries: the nodes are independent and run on up to 16
    // threads, each node in its own link-map order, and the minimum trees
    // are rebuilt once at the end.
    void update_all_min() {
        const int64_t total = (int64_t)nodes.size();
        for (int64_t i = 0; i < total; ++i) { exact.v[i] = 1.0f; inexact.v[i] = 1.0f; }
        auto range = [&](int64_t lo, int64_t hi) {
            for (int64_t i = lo; i < hi; ++i) {
                if (!active[i] || nodes[i].links.empty()) continue;
                Node& x = nodes[i];
                float ex = 1.0f, in = 1.0f;
                int exn = exact_node[i];
                for (auto& kv : x.links) {
                    if (kv.first >= x.id) continue;   // links are keyed by smaller IDs
                    const Node& y = nodes[kv.first];
                    const unsigned int tot = x.members * y.members;
                    const unsigned int unlinked = tot - kv.second.num;
                    if (unlinked == 0 || all_loaded) {
                        const float d = (kv.second.sum + end_level * (float)unlinked) / (float)tot;
                        if (d < ex) { ex = d; exn = (int)y.id; }
                    } else {
                        const float d = (kv.second.sum + lambda * (float)unlinked) / (float)tot;
                        if (d < in) in = d;
                    }
                }
                exact.v[i] = ex;
                inexact.v[i] = in;
                exact_node[i] = exn;
            }
        };
        const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
        const int nt = (int)std::max<int64_t>(1, std::min<int64_t>(std::min(16u, hw), total / 16384));
        if (nt == 1) {
            range(0, total);
        } else {
            std::vector<std::thread> th;
            for (int t = 0; t < nt; ++t) th.emplace_back(range, total * t / nt, total * (t + 1) / nt);
            for (auto& x : th) x.join();
        }
        exact.rebuild();
        inexact.rebuild();
    }
};

// The chunk heads in the multimap's order: smallest distance first, equal
// distances in insertion order (a std::multimap<float, ...> inserts a key
// after those equal to it).  A binary heap on (distance, insertion number)
// gives the same order without a node allocation per edge.
struct Head {
    float d;
    unsigned long long seq;
    unsigned int x, y, chunk;
};
struct HeadAfter {   // heap order: the head that comes later is "less"
    bool operator()(const Head& a, const Head& b) const {
        return a.d > b.d || (a.d == b.d && a.seq > b.seq);
    }
};

// Decimal digits of v into the end of buf; returns the first digit.
char* put_uint(char* end, unsigned long long v) {
    do { *--end = (char)('0' + v % 10); v /= 10; } while (v);
    return end;
}

void put_level_line(std::string& cl, std::string& cf, float level) {
    char b[64];
    std::snprintf(b, sizeof b, " %.6f ", level);
    cl += b;
    cf += b;
}

// printClusters (aveclust.cpp:244-340; sparsecut.cpp:146-272 is the same
// function with EPSILON 1e-5): per distance level, the clusters a cut at
// that level leaves (a node is kept whole when its dist is below the level
// or within eps of it), each with its leaves in the reference's depth-first
// order, then the singletons.  Roots are visited by ascending node ID (the
// reference iterates a hash set of node pointers).  One thread per level;
// each reads the finished tree only.  NodeT: id, left, right (-1: none),
// dist, members.
template <typename NodeT>
void cluster_levels(const std::vector<NodeT>& nodes, const std::vector<int>& roots,
                    const std::vector<int>& orphans, const std::vector<float>& levels, double eps,
                    std::string& cl_out, std::string& cf_out, std::string& report) {
    const size_t nl = levels.size();
    std::vector<std::string> cls(nl), cfs(nl), reps(nl);
    auto one_level = [&](size_t li) {
        const float level = levels[li];
        std::string& cl = cls[li];
        std::string& cf = cfs[li];
        char buf[96];
        auto within = [&](int i) { return nodes[i].dist < level || std::fabs(nodes[i].dist - level) < eps; };
        std::vector<int> cut;   // the reference's nodeList, built with push_front
        for (int r : roots) {
            if (within(r)) { cut.push_back(r); continue; }
            std::vector<int> todo{r};
            while (!todo.empty()) {
                const int t = todo.back();
                todo.pop_back();
                const int lf = nodes[t].left, rt = nodes[t].right;
                if (within(lf)) cut.push_back(lf); else todo.push_back(lf);
                if (within(rt)) cut.push_back(rt); else todo.push_back(rt);
            }
        }
        std::reverse(cut.begin(), cut.end());
        put_level_line(cl, cf, level);
        std::vector<int> todo;
        for (int top : cut) {
            cf += '|';
            todo.assign(1, top);
            bool first = true;
            unsigned int size = 0;
            while (!todo.empty()) {
                const int t = todo.back();
                todo.pop_back();
                const NodeT& nd = nodes[t];
                if (nd.left < 0 && nd.right < 0) {
                    char* e = buf + sizeof buf;
                    char* b = put_uint(e, nd.id);
                    if (!first) *--b = ' ';
                    cf.append(b, (size_t)(e - b));
                    first = false;
                    size += nd.members;
                }
                if (nd.right >= 0) todo.push_back(nd.right);
                if (nd.left >= 0) todo.push_back(nd.left);
            }
            char* e = buf + sizeof buf;
            *--e = ' ';
            char* b = put_uint(e, size);   // "%d " of an unsigned count below 2^31
            cl.append(b, (size_t)(buf + sizeof buf - b));
        }
        for (int o : orphans) {
            char* e = buf + sizeof buf;
            char* b = put_uint(e, (unsigned)o);
            *--b = '|';
            cf.append(b, (size_t)(e - b));
            cl += "1 ";
        }
        cf += "|\n";
        cl += "\n";
        std::snprintf(buf, sizeof buf, "Dist: %.6f. numOTUs: %u. numSingletons: %lu\n", level,
                      (unsigned)(cut.size() + orphans.size()), (unsigned long)orphans.size());
        reps[li] = buf;
    };
    {
        std::vector<std::thread> th;
        for (size_t li = 0; li < nl; ++li) th.emplace_back(one_level, li);
        for (auto& t : th) t.join();
    }
    for (size_t li = 0; li < nl; ++li) {
        cl_out += cls[li];
        cf_out += cfs[li];
        report += reps[li];
    }
}

int write_files(const char* who, const std::string* names, const std::string* const* bodies, int n) {
    for (int i = 0; i < n; ++i) {
        FILE* f = std::fopen(names[i].c_str(), "wb");
        if (!f) return crispy::fail(nullptr, CRISPY_E_IO, "%s: cannot write %s", who, names[i].c_str());
        const bool ok = std::fwrite(bodies[i]->data(), 1, bodies[i]->size(), f) == bodies[i]->size();
        if (std::fclose(f) != 0 || !ok)
            return crispy::fail(nullptr, CRISPY_E_IO, "%s: short write to %s", who, names[i].c_str());
    }
    return CRISPY_OK;
}

}  // namespace

extern "C" int crispy_aveclust(const uint32_t* const* pairs, const float* const* dists, const int64_t* counts,
                               int nchunks, int num_reads, float end_level, const char* out_base,
                               const char* edge_out, crispy_clust_stats* stats) {
    using crispy::fail;
    if (num_reads < 1 || nchunks < 1 || !pairs || !dists || !counts || !out_base)
        return fail(nullptr, CRISPY_E_INPUT, "aveclust: need reads, at least one chunk and an output name");
    for (int c = 0; c < nchunks; ++c) {
        if (counts[c] < 0 || (counts[c] && (!pairs[c] || !dists[c])))
            return fail(nullptr, CRISPY_E_INPUT, "aveclust: chunk %d is NULL", c);
        for (int64_t k = 0; k < 2 * counts[c]; ++k)
            if (pairs[c][k] >= (uint32_t)num_reads)
                return fail(nullptr, CRISPY_E_INPUT, "aveclust: chunk %d names read %u of %d", c, pairs[c][k], num_reads);
    }
    if (end_level < 0.0f || end_level > 1.0f)   // aveclust.cpp:695-700
        end_level = (float)(num_reads > 500 ? std::min(1 / std::log2((double)num_reads), 1.0)
                                            : std::min(1 / std::log10((double)num_reads), 1.0));
    FILE* fo = nullptr;
    FILE* fo1 = nullptr;
    if (edge_out) {
        fo = std::fopen(edge_out, "w");
        fo1 = std::fopen((std::string(edge_out) + "_Index1").c_str(), "w");
        if (!fo || !fo1) {
            if (fo) std::fclose(fo);
            if (fo1) std::fclose(fo1);
            return fail(nullptr, CRISPY_E_IO, "aveclust: cannot open %s", edge_out);
        }
    }
    Clusterer C(num_reads, end_level);
    std::string merges;
    std::vector<int64_t> pos((size_t)nchunks, 0);
    unsigned int ix = 0, iy = 0;
    float dist = 0.0f;
    // loadAPair: the chunk's next entry into (ix, iy, dist), false at its end
    auto load = [&](int c) -> bool {
        if (pos[c] >= counts[c]) return false;
        ix = pairs[c][2 * pos[c]];
        iy = pairs[c][2 * pos[c] + 1];
        dist = dists[c][pos[c]];
        ++pos[c];
        return true;
    };
    std::vector<Head> heads;   // heap under HeadAfter
    unsigned long long seq = 0;
    auto push_head = [&](int c) {
        heads.push_back(Head{dist, seq++, ix, iy, (unsigned)c});
        std::push_heap(heads.begin(), heads.end(), HeadAfter());
    };
    for (int c = 0; c < nchunks; ++c)
        if (load(c)) push_head(c);
    unsigned long long max_edges = (unsigned long long)num_reads;
    int64_t read_pairs = 0;
    char line[96];
    using tclock = std::chrono::steady_clock;
    auto ms_since = [](tclock::time_point t) {
        return std::chrono::duration<double, std::milli>(tclock::now() - t).count();
    };
    double ms_edges = 0, ms_update = 0, ms_merges = 0;
    while (!C.all_loaded) {
        const auto t_edges = tclock::now();
        if (C.total_edges < max_edges) {
            while (C.total_edges <= max_edges && !heads.empty()) {
                std::pop_heap(heads.begin(), heads.end(), HeadAfter());
                const Head h = heads.back();
                heads.pop_back();
                const int c = (int)h.chunk;
                ix = h.x;
                iy = h.y;
                dist = h.d;
                ++read_pairs;
                if (fo) {
                    std::fprintf(fo, "%d %d %f\n", (int)ix, (int)iy, dist);
                    std::fprintf(fo1, "%d %d %f\n", (int)ix + 1, (int)iy + 1, dist);
                }
                if (dist < C.end_level || std::fabs(dist - C.end_level) < kEps) C.absorb(ix, iy, dist);
                if (load(c)) push_head(c);
            }
            if (dist > C.lambda) C.lambda = dist;
        } else {
            max_edges *= 2;
            if ((double)max_edges > kUpperEdges) C.end_level = C.lambda;
        }
        if (heads.empty()) C.all_loaded = true;
        ms_edges += ms_since(t_edges);
        const auto t_update = tclock::now();
        C.update_all_min();
        ms_update += ms_since(t_update);
        const auto t_merges = tclock::now();
        float min_in = C.inexact.min();
        int mi = C.exact.argmin();
        float min_ex = C.exact[mi];
        while (min_ex < 1.0f && (min_ex < min_in || std::fabs(min_ex - min_in) < kEps)) {
            const int a = C.root(mi);
            const int b = C.root(C.exact_node[mi]);
            C.merge(a, b, min_ex);
            std::snprintf(line, sizeof line, "%d %d %.6f\n", (int)C.nodes[a].id + 1, (int)C.nodes[b].id + 1, min_ex);
            merges += line;
            min_in = C.inexact.min();
            mi = C.exact.argmin();
            min_ex = C.exact[mi];
        }
        ms_merges += ms_since(t_merges);
    }
    if (fo) { std::fclose(fo); std::fclose(fo1); }
    const auto t_output = tclock::now();

    // roots and singletons (aveclust.cpp:944-955), then printClusters at
    // the levels the reference's float loop visits
    std::vector<int> roots, orphans;
    std::vector<char> seen(C.nodes.size(), 0);
    for (int i = 0; i < num_reads; ++i) {
        if (C.nodes[i].parent < 0) {
            orphans.push_back(i);
            continue;
        }
        const int r = C.root(i);
        if (!seen[r]) { seen[r] = 1; roots.push_back(r); }
    }
    std::sort(roots.begin(), roots.end());
    const float step = C.end_level / 10;
    std::vector<float> levels;
    for (float level = step; level < C.end_level || std::fabs(level - C.end_level) < kEps; level += step)
        levels.push_back(level);
    std::string cl, cf, report;
    cluster_levels(C.nodes, roots, orphans, levels, kEps, cl, cf, report);
    const std::string base(out_base);
    const std::string names[] = {base + "_Merge", base + ".Cluster_List", base + ".Cluster"};
    const std::string* bodies[] = {&merges, &cl, &cf};
    CRISPY_TRY(write_files("aveclust", names, bodies, 3));
    if (stats) {
        stats->pairs_read = read_pairs;
        stats->merges = (int64_t)(C.new_id - (unsigned)num_reads);
        stats->roots = (int32_t)roots.size();
        stats->singletons = (int32_t)orphans.size();
        stats->end_level = C.end_level;
        std::snprintf(stats->report, sizeof stats->report, "%s", report.c_str());
        stats->ms_edges = ms_edges;
        stats->ms_update = ms_update;
        stats->ms_merges = ms_merges;
        stats->ms_output = ms_since(t_output);
    }
    return CRISPY_OK;
}

namespace {

constexpr double kCutEps = 1e-5;   // EPSILON (sparsecut.cpp:18)

struct CutNode {
    unsigned int id = 0;
    int parent = -1, left = -1, right = -1;
    float dist = 0.0f;
    unsigned int members = 1;
};

}  // namespace

// sparsecut (src/sparsecut/sparsecut.cpp, the step crispy.sh:29 runs after
// the changepoint cutoffs): rebuild the dendrogram from <in_base>_Merge
// (sparsecut.cpp:361-367: "%d %d %f" lines of 1-based node IDs; merge k
// creates node num_reads + k with the larger-ID child on the left,
// sparsecut.cpp:283-315) and print the clusters at each cutoff.  Merge
// lines that do not join two current clusters are refused (the reference
// does not check them).
extern "C" int crispy_sparsecut(const char* in_base, int num_reads, const float* cutoffs, int ncutoffs,
                                crispy_clust_stats* stats) {
    using crispy::fail;
    if (!in_base || num_reads < 1 || ncutoffs < 0 || (ncutoffs > 0 && !cutoffs))
        return fail(nullptr, CRISPY_E_INPUT, "sparsecut: need an input name, reads and the cutoffs");
    const std::string base(in_base);
    const std::string merge_name = base + "_Merge";
    FILE* f = std::fopen(merge_name.c_str(), "r");
    if (!f) return fail(nullptr, CRISPY_E_IO, "sparsecut: cannot open %s", merge_name.c_str());
    std::vector<CutNode> nodes((size_t)2 * num_reads);
    for (int i = 0; i < num_reads; ++i) nodes[i].id = (unsigned)i;
    int new_id = num_reads;
    int idx = 0, idy = 0;
    float dist = 0.0f;
    while (std::fscanf(f, "%d %d %f", &idx, &idy, &dist) == 3) {
        const int a = idx - 1, b = idy - 1;
        if (new_id >= 2 * num_reads || a < 0 || b < 0 || a >= new_id || b >= new_id || a == b ||
            nodes[a].parent >= 0 || nodes[b].parent >= 0) {
            std::fclose(f);
            return fail(nullptr, CRISPY_E_INPUT, "sparsecut: %s merges %d and %d, not two current clusters",
                        merge_name.c_str(), idx, idy);
        }
        CutNode& p = nodes[new_id];
        p.id = (unsigned)new_id;
        const int x = std::max(a, b), y = std::min(a, b);   // addNode(nodeX, nodeY): larger ID left
        p.left = x;
        p.right = y;
        p.dist = dist;
        p.members = nodes[x].members + nodes[y].members;
        nodes[x].parent = nodes[y].parent = new_id;
        ++new_id;
    }
    std::fclose(f);
    // each leaf's top node: parents come after their children
    std::vector<int> top(new_id);
    for (int i = new_id - 1; i >= 0; --i) top[i] = nodes[i].parent < 0 ? i : top[nodes[i].parent];
    std::vector<int> roots, orphans;
    std::vector<char> seen(new_id, 0);
    for (int i = 0; i < num_reads; ++i) {
        if (nodes[i].parent < 0) {
            orphans.push_back(i);
            continue;
        }
        if (!seen[top[i]]) { seen[top[i]] = 1; roots.push_back(top[i]); }
    }
    std::sort(roots.begin(), roots.end());
    std::string cl, cf, report;
    cluster_levels(nodes, roots, orphans, std::vector<float>(cutoffs, cutoffs + ncutoffs), kCutEps, cl, cf,
                   report);
    const std::string names[] = {base + ".Cluster_List", base + ".Cluster"};
    const std::string* bodies[] = {&cl, &cf};
    CRISPY_TRY(write_files("sparsecut", names, bodies, 2));
    if (stats) {
        stats->pairs_read = 0;
        stats->merges = (int64_t)(new_id - num_reads);
        stats->roots = (int32_t)roots.size();
        stats->singletons = (int32_t)orphans.size();
        stats->end_level = ncutoffs > 0 ? cutoffs[ncutoffs - 1] : 0.0f;
        std::snprintf(stats->report, sizeof stats->report, "%s", report.c_str());
    }
    return CRISPY_OK;
}
