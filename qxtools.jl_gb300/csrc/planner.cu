// qxg_plan_contraction: contraction trees for a tensor network given as a hypergraph, with
// slicing.  It stands in for the planners that QXTools calls but does not ship: FlowCutter's
// tree decompositions (flow_cutter_contraction_plan, src/contraction_planning.jl:90-113) and the
// greedy treewidth deletion that chooses the bonds to slice (contraction_scheme, :219-299).
// Host code only.
//
// Trees come from two published methods, run for several seeded trials each:
//  * recursive bisection of the hypergraph (tensors = vertices, labels = hyperedges weighted by
//    log2 of their dimension).  Each split minimises the weight of the cut labels under a balance
//    bound, by multilevel Fiduccia-Mattheyses refinement (heavy-edge coarsening, greedy-growth
//    initial parts, FM passes with rollback at every level).  Parts of at most `cutoff` tensors are
//    finished greedily.  This is the divisive scheme of Gray & Kourtis, "Hyper-optimized tensor
//    network contraction", Quantum 5, 410 (2021), with a partitioner of this file's own;
//  * randomised greedy pairing: contract the pair sharing a label whose result grows least,
//    |C| - |A| - |B|, perturbed by Gumbel noise (the same paper's greedy baseline).
// Every tree is scored by the executor's step model: a step costs
// max(8 |A u B| / flops_per_s, 8 (|A| + |B| + |C|) / bytes_per_s) (complex multiply-adds; Complex64
// bytes).  Slicing then fixes labels one at a time, each time the label among the largest
// intermediates that gives the lowest (largest intermediate, modelled time x slices), until
// every intermediate has at most 2^max_log2 elements or max_sliced labels are fixed; the best
// trees are sliced and the cheapest result wins.
//
// A label is kept by a contraction while a tensor outside it still holds the label, or when the
// label is open or held by a single tensor; this is the rule of QXTns contraction_indices
// (called at src/compute_graph/compute_graph.jl:65), so the plan's intermediates are the ones
// the executor builds.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <exception>
#include <numeric>
#include <queue>
#include <string>
#include <utility>
#include <vector>

#include "../../include/qxgpu.h"

namespace qxg {
int ncon_fail(int code, const char* msg);
}

namespace {

// splitmix64: a small, seedable generator with the same stream on every platform.
struct Rng {
    uint64_t s;
    explicit Rng(uint64_t seed) : s(seed * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull) {}
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }  // [0, 1)
    int below(int n) { return (int)(next() % (uint64_t)n); }
    double gumbel() {
        double u = uniform();
        if (u <= 0.0) u = 1e-300;
        return -std::log(-std::log(u) + 1e-300);
    }
};

struct Net {
    int V = 0, E = 0;
    std::vector<std::vector<int>> vlab;  // distinct labels of each tensor
    std::vector<std::vector<int>> pins;  // tensors holding each label
    std::vector<int> w;                  // log2 dimension of each label
    std::vector<char> keep;              // open, or held by one tensor: never summed
    std::vector<char> batched;           // tensors that carry the bitstring batch
};

using Labels = std::vector<std::pair<int, int>>;  // (label, holders inside), sorted by label

// Labels of the union of two nodes, counts summed, fully enclosed labels dropped.  `all` gets
// every label of either operand (the summed ones included), when given.
void merge_labels(const Net& n, const Labels& a, const Labels& b, Labels* out, std::vector<int>* all) {
    out->clear();
    if (all) all->clear();
    size_t i = 0, j = 0;
    while (i < a.size() || j < b.size()) {
        int lab, cnt;
        if (j == b.size() || (i < a.size() && a[i].first < b[j].first)) {
            lab = a[i].first;
            cnt = a[i++].second;
        } else if (i == a.size() || b[j].first < a[i].first) {
            lab = b[j].first;
            cnt = b[j++].second;
        } else {
            lab = a[i].first;
            cnt = a[i++].second + b[j++].second;
        }
        if (all) all->push_back(lab);
        if (n.keep[lab] || cnt < (int)n.pins[lab].size()) out->push_back({lab, cnt});
    }
}

int weight(const Net& n, const Labels& l, const std::vector<int>& w) {
    int s = 0;
    for (const auto& x : l) s += w[x.first];
    (void)n;
    return s;
}

int weight_of(const Labels& l, const std::vector<int>& w) {
    int s = 0;
    for (const auto& x : l) s += w[x.first];
    return s;
}

Labels leaf_labels(const Net& n, int v) {
    Labels l;
    for (int lab : n.vlab[v]) l.push_back({lab, 1});
    std::sort(l.begin(), l.end());
    return l;
}

struct Model {
    double flops_rate = 1e14, bytes_rate = 5e12;
    double batch = 1.0;  // bitstrings run together: the factor on every tensor that depends on a batched one
};

// The steps of a tree with their label sets, for costing under any label weights.
struct Steps {
    std::vector<std::vector<int>> all;  // labels of A u B
    std::vector<std::vector<int>> res;  // labels of C
    std::vector<int> a, b;              // operand node ids
    int V = 0;
};

Steps tree_steps(const Net& n, const std::vector<std::pair<int, int>>& pairs) {
    Steps s;
    s.V = n.V;
    std::vector<Labels> lab(n.V + pairs.size());
    for (int v = 0; v < n.V; v++) lab[v] = leaf_labels(n, v);
    std::vector<int> all;
    for (size_t k = 0; k < pairs.size(); k++) {
        Labels c;
        merge_labels(n, lab[pairs[k].first], lab[pairs[k].second], &c, &all);
        s.all.push_back(all);
        std::vector<int> r;
        for (const auto& x : c) r.push_back(x.first);
        s.res.push_back(r);
        s.a.push_back(pairs[k].first);
        s.b.push_back(pairs[k].second);
        lab[n.V + k] = std::move(c);
        Labels().swap(lab[pairs[k].first]);
        Labels().swap(lab[pairs[k].second]);
    }
    return s;
}

struct Cost {
    double flops = 0, time = 0;
    int max_log2 = 0;
};

// FLOPs are counted for one bitstring; the modelled time carries the batch on every step that
// depends on a batched tensor.
Cost cost_of(const Net& n, const Steps& s, const std::vector<int>& w, const Model& m) {
    Cost c;
    std::vector<int> sz(s.V + s.all.size(), 0);
    std::vector<char> dep(s.V + s.all.size(), 0);
    for (int v = 0; v < s.V; v++) {
        int t = 0;
        for (int lab : n.vlab[v]) t += w[lab];
        sz[v] = t;
        dep[v] = n.batched[v];
    }
    for (size_t k = 0; k < s.all.size(); k++) {
        int ga = 0, gc = 0;
        for (int lab : s.all[k]) ga += w[lab];
        for (int lab : s.res[k]) gc += w[lab];
        sz[s.V + k] = gc;
        const bool da = dep[s.a[k]], db = dep[s.b[k]], dc = da || db;
        dep[s.V + k] = dc;
        const double f = 8.0 * std::ldexp(1.0, ga);
        const double by = 8.0 * (std::ldexp(1.0, sz[s.a[k]]) * (da ? m.batch : 1.0) +
                                 std::ldexp(1.0, sz[s.b[k]]) * (db ? m.batch : 1.0) +
                                 std::ldexp(1.0, gc) * (dc ? m.batch : 1.0));
        c.flops += f;
        c.time += std::max(f * (dc ? m.batch : 1.0) / m.flops_rate, by / m.bytes_rate);
        c.max_log2 = std::max(c.max_log2, gc);
    }
    return c;
}

// ---------------------------------------------------------------------------------------------
// greedy pairing (whole network, or the nodes of one part)
// ---------------------------------------------------------------------------------------------
struct Greedy {
    const Net& n;
    Rng& rng;
    double temperature;
    std::vector<Labels>* lab;                 // labels of every node id (grows)
    std::vector<std::pair<int, int>>* pairs;  // steps appended here
    int next_id;

    double score(const Labels& c, const Labels& a, const Labels& b) {
        const double d = std::ldexp(1.0, weight(n, c, n.w)) - std::ldexp(1.0, weight(n, a, n.w)) -
                         std::ldexp(1.0, weight(n, b, n.w));
        double s = std::copysign(std::log2(std::fabs(d) + 1.0), d);
        if (temperature > 0) s -= temperature * rng.gumbel();
        return s;
    }

    // Contract `nodes` (node ids) to one; returns its id.
    int run(std::vector<int> nodes) {
        if (nodes.empty()) return -1;
        std::vector<int> alive_set;  // node ids still open, in creation order
        std::vector<std::vector<int>> holders(n.E);  // label -> open node ids holding it
        std::vector<char> alive;
        auto ensure = [&](int id) {
            if ((int)alive.size() <= id) alive.resize(id + 1, 0);
        };
        for (int id : nodes) {
            ensure(id);
            alive[id] = 1;
            for (const auto& x : (*lab)[id]) holders[x.first].push_back(id);
        }
        using Entry = std::pair<double, std::pair<int, int>>;
        std::priority_queue<Entry, std::vector<Entry>, std::greater<Entry>> heap;
        Labels tmp;
        auto push_pairs = [&](int id) {
            std::vector<int> seen;
            for (const auto& x : (*lab)[id])
                for (int o : holders[x.first])
                    if (o != id && alive[o]) seen.push_back(o);
            std::sort(seen.begin(), seen.end());
            seen.erase(std::unique(seen.begin(), seen.end()), seen.end());
            for (int o : seen) {
                merge_labels(n, (*lab)[id], (*lab)[o], &tmp, nullptr);
                heap.push({score(tmp, (*lab)[id], (*lab)[o]), {std::min(id, o), std::max(id, o)}});
            }
        };
        for (int id : nodes) push_pairs(id);
        int remaining = (int)nodes.size();
        std::vector<int> open_ids = nodes;
        while (remaining > 1) {
            int a = -1, b = -1;
            while (!heap.empty()) {
                auto e = heap.top();
                heap.pop();
                if (alive[e.second.first] && alive[e.second.second]) {
                    a = e.second.first;
                    b = e.second.second;
                    break;
                }
            }
            if (a < 0) {  // no shared labels left: join the two smallest parts (an outer product)
                std::vector<std::pair<int, int>> by_size;
                for (int id : open_ids)
                    if (alive[id]) by_size.push_back({weight(n, (*lab)[id], n.w), id});
                std::sort(by_size.begin(), by_size.end());
                a = std::min(by_size[0].second, by_size[1].second);
                b = std::max(by_size[0].second, by_size[1].second);
            }
            Labels c;
            merge_labels(n, (*lab)[a], (*lab)[b], &c, nullptr);
            const int id = next_id++;
            if ((int)lab->size() <= id) lab->resize(id + 1);
            (*lab)[id] = std::move(c);
            pairs->push_back({a, b});
            alive[a] = alive[b] = 0;
            ensure(id);
            alive[id] = 1;
            open_ids.push_back(id);
            for (const auto& x : (*lab)[id]) holders[x.first].push_back(id);
            // drop dead holders lazily: compact the lists of this node's labels
            for (const auto& x : (*lab)[id]) {
                auto& h = holders[x.first];
                h.erase(std::remove_if(h.begin(), h.end(), [&](int o) { return !alive[o]; }), h.end());
            }
            push_pairs(id);
            remaining--;
        }
        for (int id : open_ids)
            if (alive[id]) return id;
        return -1;
    }
};

// ---------------------------------------------------------------------------------------------
// hypergraph bisection
// ---------------------------------------------------------------------------------------------
struct HG {
    int n = 0;
    std::vector<int> vw;                 // vertex weights
    std::vector<int> eoff, epin, ew;     // edges (CSR over pins), edge weights
    std::vector<int> voff, vedge;        // incidence (CSR over edges)
    int total = 0, maxvw = 0;
    int nedges() const { return (int)ew.size(); }
    void finish() {
        std::vector<int> deg(n, 0);
        for (int e = 0; e < nedges(); e++)
            for (int p = eoff[e]; p < eoff[e + 1]; p++) deg[epin[p]]++;
        voff.assign(n + 1, 0);
        for (int v = 0; v < n; v++) voff[v + 1] = voff[v] + deg[v];
        vedge.assign(voff[n], 0);
        std::vector<int> fill(voff.begin(), voff.end() - 1);
        for (int e = 0; e < nedges(); e++)
            for (int p = eoff[e]; p < eoff[e + 1]; p++) vedge[fill[epin[p]]++] = e;
        total = std::accumulate(vw.begin(), vw.end(), 0);
        maxvw = n ? *std::max_element(vw.begin(), vw.end()) : 0;
    }
};

// Coarsen by heavy-edge matching; cluster[v] = coarse vertex.  Returns the coarse graph.
HG coarsen(const HG& g, Rng& rng, int maxw, std::vector<int>* cluster) {
    std::vector<int> order(g.n);
    std::iota(order.begin(), order.end(), 0);
    for (int i = g.n - 1; i > 0; i--) std::swap(order[i], order[rng.below(i + 1)]);
    cluster->assign(g.n, -1);
    std::vector<double> rating(g.n, 0.0);
    std::vector<int> touched;
    int nc = 0;
    for (int v : order) {
        if ((*cluster)[v] >= 0) continue;
        touched.clear();
        for (int q = g.voff[v]; q < g.voff[v + 1]; q++) {
            const int e = g.vedge[q];
            const int sz = g.eoff[e + 1] - g.eoff[e];
            if (sz < 2 || sz > 64) continue;
            const double r = (double)g.ew[e] / (sz - 1);
            for (int p = g.eoff[e]; p < g.eoff[e + 1]; p++) {
                const int u = g.epin[p];
                if (u == v || (*cluster)[u] >= 0) continue;
                if (rating[u] == 0.0) touched.push_back(u);
                rating[u] += r;
            }
        }
        int best = -1;
        double br = 0.0;
        for (int u : touched) {
            const double r = rating[u] + 1e-9 * rng.uniform();
            if (g.vw[u] + g.vw[v] <= maxw && r > br) {
                br = r;
                best = u;
            }
            rating[u] = 0.0;
        }
        (*cluster)[v] = nc;
        if (best >= 0) (*cluster)[best] = nc;
        nc++;
    }
    HG c;
    c.n = nc;
    c.vw.assign(nc, 0);
    for (int v = 0; v < g.n; v++) c.vw[(*cluster)[v]] += g.vw[v];
    c.eoff.push_back(0);
    std::vector<int> pin;
    for (int e = 0; e < g.nedges(); e++) {
        pin.clear();
        for (int p = g.eoff[e]; p < g.eoff[e + 1]; p++) pin.push_back((*cluster)[g.epin[p]]);
        std::sort(pin.begin(), pin.end());
        pin.erase(std::unique(pin.begin(), pin.end()), pin.end());
        if (pin.size() < 2) continue;
        c.epin.insert(c.epin.end(), pin.begin(), pin.end());
        c.eoff.push_back((int)c.epin.size());
        c.ew.push_back(g.ew[e]);
    }
    c.finish();
    return c;
}

struct Bounds {
    int hi;  // largest weight either side may take
};

Bounds bounds(const HG& g, double eps) {
    const double half = g.total / 2.0;
    int hi = (int)std::floor((1.0 + eps) * half);
    hi = std::max(hi, (int)std::ceil(half) + g.maxvw / 2);
    hi = std::min(hi, g.total - 1);
    return {std::max(hi, 1)};
}

int cut_of(const HG& g, const std::vector<char>& part) {
    int cut = 0;
    for (int e = 0; e < g.nedges(); e++) {
        bool s0 = false, s1 = false;
        for (int p = g.eoff[e]; p < g.eoff[e + 1]; p++) (part[g.epin[p]] ? s1 : s0) = true;
        if (s0 && s1) cut += g.ew[e];
    }
    return cut;
}

// Fiduccia-Mattheyses passes with rollback to the best prefix; returns the cut.
int fm_refine(const HG& g, std::vector<char>& part, const Bounds& bd, Rng& rng, int max_passes) {
    std::vector<int> cnt0(g.nedges()), cnt1(g.nedges());
    int W[2] = {0, 0};
    for (int v = 0; v < g.n; v++) W[(int)part[v]] += g.vw[v];
    for (int e = 0; e < g.nedges(); e++) {
        cnt0[e] = cnt1[e] = 0;
        for (int p = g.eoff[e]; p < g.eoff[e + 1]; p++) (part[g.epin[p]] ? cnt1[e] : cnt0[e])++;
    }
    auto gain_of = [&](int v) {
        int gsum = 0;
        const int s = part[v];
        for (int q = g.voff[v]; q < g.voff[v + 1]; q++) {
            const int e = g.vedge[q];
            const int from = s ? cnt1[e] : cnt0[e], to = s ? cnt0[e] : cnt1[e];
            if (from == 1 && to > 0) gsum += g.ew[e];
            if (to == 0 && from > 1) gsum -= g.ew[e];
        }
        return gsum;
    };
    std::vector<int> gain(g.n), stamp(g.n, 0);
    std::vector<char> locked(g.n);
    std::vector<uint32_t> tieb(g.n);
    using Entry = std::pair<std::pair<int, uint32_t>, std::pair<int, int>>;  // (gain, tie), (v, stamp)
    for (int pass = 0; pass < max_passes; pass++) {
        std::priority_queue<Entry> heap[2];
        std::fill(locked.begin(), locked.end(), 0);
        for (int v = 0; v < g.n; v++) {
            gain[v] = gain_of(v);
            tieb[v] = (uint32_t)rng.next();
            heap[(int)part[v]].push({{gain[v], tieb[v]}, {v, ++stamp[v]}});
        }
        std::vector<int> moves;
        int cum = 0, best = 0, best_len = 0;
        const int bal0 = std::abs(W[0] - W[1]);
        int best_bal = bal0;
        while (true) {
            int pick[2] = {-1, -1};
            for (int s = 0; s < 2; s++) {
                while (!heap[s].empty()) {
                    const Entry& e = heap[s].top();
                    const int v = e.second.first;
                    if (locked[v] || part[v] != s || e.second.second != stamp[v]) {
                        heap[s].pop();
                        continue;
                    }
                    if (W[1 - s] + g.vw[v] > bd.hi) {  // the move would overfill the other side
                        locked[v] = 1;
                        heap[s].pop();
                        continue;
                    }
                    pick[s] = v;
                    break;
                }
            }
            int v = -1;
            if (pick[0] >= 0 && pick[1] >= 0) {
                // prefer the higher gain; on a tie, the move from the heavier side
                if (gain[pick[0]] != gain[pick[1]]) v = gain[pick[0]] > gain[pick[1]] ? pick[0] : pick[1];
                else v = W[0] >= W[1] ? pick[0] : pick[1];
            } else {
                v = pick[0] >= 0 ? pick[0] : pick[1];
            }
            if (v < 0) break;
            const int s = part[v];
            heap[s].pop();
            cum += gain[v];
            locked[v] = 1;
            part[v] = (char)(1 - s);
            W[s] -= g.vw[v];
            W[1 - s] += g.vw[v];
            for (int q = g.voff[v]; q < g.voff[v + 1]; q++) {
                const int e = g.vedge[q];
                if (s) {
                    cnt1[e]--;
                    cnt0[e]++;
                } else {
                    cnt0[e]--;
                    cnt1[e]++;
                }
            }
            for (int q = g.voff[v]; q < g.voff[v + 1]; q++) {
                const int e = g.vedge[q];
                for (int p = g.eoff[e]; p < g.eoff[e + 1]; p++) {
                    const int u = g.epin[p];
                    if (locked[u]) continue;
                    const int ng = gain_of(u);
                    if (ng != gain[u]) {
                        gain[u] = ng;
                        heap[(int)part[u]].push({{ng, tieb[u]}, {u, ++stamp[u]}});
                    }
                }
            }
            moves.push_back(v);
            const int bal = std::abs(W[0] - W[1]);
            if (cum > best || (cum == best && bal < best_bal)) {
                best = cum;
                best_bal = bal;
                best_len = (int)moves.size();
            }
            if ((int)moves.size() - best_len > 150) break;
        }
        for (int k = (int)moves.size() - 1; k >= best_len; k--) {  // roll back past the best prefix
            const int u = moves[k];
            const int s = part[u];
            part[u] = (char)(1 - s);
            W[s] -= g.vw[u];
            W[1 - s] += g.vw[u];
            for (int q = g.voff[u]; q < g.voff[u + 1]; q++) {
                const int e = g.vedge[q];
                if (s) {
                    cnt1[e]--;
                    cnt0[e]++;
                } else {
                    cnt0[e]--;
                    cnt1[e]++;
                }
            }
        }
        if (best <= 0 && best_bal >= bal0) break;
    }
    return cut_of(g, part);
}

// Initial part 1: grown from a random vertex, taking the frontier vertex with the best gain until
// half the weight has moved.
std::vector<char> grow(const HG& g, Rng& rng) {
    std::vector<char> part(g.n, 0);
    if (g.n < 2) return part;
    std::vector<int> in_edge(g.nedges(), 0);  // pins already in part 1
    std::vector<char> frontier(g.n, 0);
    std::vector<int> fr;
    int w1 = 0;
    const int target = g.total / 2;
    int v = rng.below(g.n);
    while (true) {
        part[v] = 1;
        w1 += g.vw[v];
        if (w1 >= target) break;
        for (int q = g.voff[v]; q < g.voff[v + 1]; q++) {
            const int e = g.vedge[q];
            in_edge[e]++;
            for (int p = g.eoff[e]; p < g.eoff[e + 1]; p++) {
                const int u = g.epin[p];
                if (!part[u] && !frontier[u]) {
                    frontier[u] = 1;
                    fr.push_back(u);
                }
            }
        }
        // the frontier vertex whose move cuts least: labels it would close minus labels it opens
        int best = -1, bestg = 0;
        for (size_t i = 0; i < fr.size(); i++) {
            const int u = fr[i];
            if (part[u]) continue;
            int gsum = 0;
            for (int q = g.voff[u]; q < g.voff[u + 1]; q++) {
                const int e = g.vedge[q];
                const int sz = g.eoff[e + 1] - g.eoff[e];
                if (in_edge[e] == sz - 1) gsum += g.ew[e];
                else if (in_edge[e] == 0) gsum -= g.ew[e];
            }
            if (best < 0 || gsum > bestg || (gsum == bestg && (rng.next() & 1))) {
                best = u;
                bestg = gsum;
            }
        }
        fr.erase(std::remove_if(fr.begin(), fr.end(), [&](int u) { return part[u] != 0; }), fr.end());
        if (best < 0) {  // disconnected: restart from any vertex of part 0
            std::vector<int> rest;
            for (int u = 0; u < g.n; u++)
                if (!part[u]) rest.push_back(u);
            if (rest.empty()) break;
            best = rest[rng.below((int)rest.size())];
        }
        v = best;
    }
    return part;
}

std::vector<char> bisect(const HG& g0, double eps, Rng& rng) {
    std::vector<HG> levels;
    std::vector<std::vector<int>> maps;
    levels.push_back(g0);
    while (levels.back().n > 48) {
        const HG& g = levels.back();
        std::vector<int> cl;
        const int maxw = std::max(1, g.total / 24);
        HG c = coarsen(g, rng, maxw, &cl);
        if (c.n > 0.92 * g.n) break;
        maps.push_back(std::move(cl));
        levels.push_back(std::move(c));
    }
    const HG& top = levels.back();
    std::vector<char> best;
    int bestcut = -1;
    for (int t = 0; t < 6; t++) {
        std::vector<char> p = grow(top, rng);
        const int cut = fm_refine(top, p, bounds(top, eps), rng, 6);
        if (bestcut < 0 || cut < bestcut) {
            bestcut = cut;
            best = p;
        }
    }
    for (int l = (int)levels.size() - 2; l >= 0; l--) {
        const HG& g = levels[l];
        std::vector<char> p(g.n);
        for (int v = 0; v < g.n; v++) p[v] = best[maps[l][v]];
        fm_refine(g, p, bounds(g, eps), rng, 4);
        best.swap(p);
    }
    return best;
}

// ---------------------------------------------------------------------------------------------
// recursive bisection trees
// ---------------------------------------------------------------------------------------------
struct Divider {
    const Net& n;
    Rng& rng;
    double eps;
    int cutoff;
    double leaf_temperature;
    std::vector<Labels> lab;
    std::vector<std::pair<int, int>> pairs;
    int next_id;

    Divider(const Net& net, Rng& r, double e, int c, double t) : n(net), rng(r), eps(e), cutoff(c), leaf_temperature(t) {
        lab.resize(n.V);
        for (int v = 0; v < n.V; v++) lab[v] = leaf_labels(n, v);
        next_id = n.V;
    }

    int greedy(const std::vector<int>& vs) {
        Greedy gr{n, rng, leaf_temperature, &lab, &pairs, next_id};
        const int id = gr.run(vs);
        next_id = gr.next_id;
        return id;
    }

    int build(const std::vector<int>& vs) {
        if ((int)vs.size() <= cutoff) return greedy(vs);
        HG g;
        g.n = (int)vs.size();
        g.vw.assign(g.n, 1);
        std::vector<int> local(n.V, -1);  // tensor -> index in vs
        for (int i = 0; i < g.n; i++) local[vs[i]] = i;
        std::vector<int> labs;
        for (int v : vs)
            for (int l : n.vlab[v]) labs.push_back(l);
        std::sort(labs.begin(), labs.end());
        labs.erase(std::unique(labs.begin(), labs.end()), labs.end());
        g.eoff.push_back(0);
        for (int l : labs) {
            if (n.w[l] == 0) continue;
            int k = 0;
            for (int t : n.pins[l])
                if (local[t] >= 0) k++;
            if (k < 2) continue;
            for (int t : n.pins[l])
                if (local[t] >= 0) g.epin.push_back(local[t]);
            g.eoff.push_back((int)g.epin.size());
            g.ew.push_back(n.w[l]);
        }
        g.finish();
        std::vector<char> part = bisect(g, eps, rng);
        std::vector<int> s0, s1;
        for (int i = 0; i < g.n; i++) (part[i] ? s1 : s0).push_back(vs[i]);
        if (s0.empty() || s1.empty()) {  // nothing to cut: split in half
            s0.assign(vs.begin(), vs.begin() + vs.size() / 2);
            s1.assign(vs.begin() + vs.size() / 2, vs.end());
        }
        const int a = build(s0);
        const int b = build(s1);
        Labels c;
        merge_labels(n, lab[a], lab[b], &c, nullptr);
        const int id = next_id++;
        lab.resize(id + 1);
        lab[id] = std::move(c);
        pairs.push_back({std::min(a, b), std::max(a, b)});
        return id;
    }
};

// ---------------------------------------------------------------------------------------------
// subtree reconfiguration: every subtree cut off at up to `k` frontier nodes is replaced by the
// cheapest contraction of those nodes, found by dynamic programming over their subsets (the
// local optimisation of Gray & Kourtis, section on tree refinement)
// ---------------------------------------------------------------------------------------------
struct Tree {
    int V = 0, root = 0;
    std::vector<int> L, R;    // children of node id >= V (leaves: -1)
    std::vector<Labels> lab;  // labels of every node
    std::vector<char> dep;    // node depends on a batched tensor
};

Tree tree_of(const Net& n, const std::vector<std::pair<int, int>>& pairs) {
    Tree t;
    t.V = n.V;
    const int N = n.V + (int)pairs.size();
    t.L.assign(N, -1);
    t.R.assign(N, -1);
    t.lab.resize(N);
    t.dep.assign(N, 0);
    for (int v = 0; v < n.V; v++) {
        t.lab[v] = leaf_labels(n, v);
        t.dep[v] = n.batched[v];
    }
    for (size_t k = 0; k < pairs.size(); k++) {
        const int id = n.V + (int)k;
        t.L[id] = pairs[k].first;
        t.R[id] = pairs[k].second;
        merge_labels(n, t.lab[t.L[id]], t.lab[t.R[id]], &t.lab[id], nullptr);
        t.dep[id] = t.dep[t.L[id]] || t.dep[t.R[id]];
    }
    t.root = N - 1;
    return t;
}

// Post-order steps of a tree, internal nodes renumbered in order of creation.
std::vector<std::pair<int, int>> pairs_of(const Tree& t) {
    std::vector<std::pair<int, int>> out;
    if (t.root < t.V) return out;
    std::vector<int> id(t.L.size(), -1);
    for (int v = 0; v < t.V; v++) id[v] = v;
    std::vector<std::pair<int, bool>> stack{{t.root, false}};
    int next = t.V;
    while (!stack.empty()) {
        auto [x, done] = stack.back();
        stack.pop_back();
        if (x < t.V) continue;
        if (done) {
            const int a = id[t.L[x]], b = id[t.R[x]];
            out.push_back({std::min(a, b), std::max(a, b)});
            id[x] = next++;
        } else {
            stack.push_back({x, true});
            stack.push_back({t.R[x], false});
            stack.push_back({t.L[x], false});
        }
    }
    return out;
}

int union_weight(const Labels& a, const Labels& b, const std::vector<int>& w) {
    int s = 0;
    size_t i = 0, j = 0;
    while (i < a.size() || j < b.size()) {
        if (j == b.size() || (i < a.size() && a[i].first < b[j].first)) s += w[a[i++].first];
        else if (i == a.size() || b[j].first < a[i].first) s += w[b[j++].first];
        else {
            s += w[a[i].first];
            i++;
            j++;
        }
    }
    return s;
}

double step_time(const Labels& a, bool da, const Labels& b, bool db, const Labels& c, const std::vector<int>& w,
                 const Model& m) {
    const double bc = (da || db) ? m.batch : 1.0;
    const double f = 8.0 * std::ldexp(1.0, union_weight(a, b, w)) * bc;
    const double by = 8.0 * (std::ldexp(1.0, weight_of(a, w)) * (da ? m.batch : 1.0) +
                             std::ldexp(1.0, weight_of(b, w)) * (db ? m.batch : 1.0) + std::ldexp(1.0, weight_of(c, w)) * bc);
    return std::max(f / m.flops_rate, by / m.bytes_rate);
}

double node_time(const Tree& t, int x, const std::vector<int>& w, const Model& m) {
    return step_time(t.lab[t.L[x]], t.dep[t.L[x]], t.lab[t.R[x]], t.dep[t.R[x]], t.lab[x], w, m);
}

// One sweep over the internal nodes, largest steps first; returns the time saved.  New
// intermediates wider than 2^cap elements are not formed.
double reconfigure_pass(const Net& n, Tree& t, const std::vector<int>& w, const Model& m, int k, int cap) {
    const int N = (int)t.L.size();
    std::vector<std::pair<double, int>> order;
    for (int x = t.V; x < N; x++) order.push_back({-node_time(t, x, w, m), x});
    std::sort(order.begin(), order.end());
    double saved = 0;
    std::vector<Labels> sl;
    std::vector<char> sdep;
    std::vector<double> best;
    std::vector<int> split;
    for (const auto& ox : order) {
        const int x = ox.second;
        // frontier: expand the heaviest internal node until k nodes
        std::vector<int> front{x}, inner;
        while ((int)front.size() < k) {
            int bi = -1, bw = -1;
            for (int i = 0; i < (int)front.size(); i++)
                if (front[i] >= t.V) {
                    const int ww = weight_of(t.lab[front[i]], w);
                    if (ww > bw) {
                        bw = ww;
                        bi = i;
                    }
                }
            if (bi < 0) break;
            const int y = front[bi];
            inner.push_back(y);
            front[bi] = t.L[y];
            front.push_back(t.R[y]);
        }
        const int f = (int)front.size();
        if (f < 3) continue;
        double cur = 0;
        for (int y : inner) cur += node_time(t, y, w, m);
        const int full = (1 << f) - 1;
        sl.assign(full + 1, Labels());
        sdep.assign(full + 1, 0);
        best.assign(full + 1, 0.0);
        split.assign(full + 1, 0);
        for (int i = 0; i < f; i++) {
            sl[1 << i] = t.lab[front[i]];
            sdep[1 << i] = t.dep[front[i]];
        }
        for (int mask = 1; mask <= full; mask++) {
            if ((mask & (mask - 1)) == 0) continue;
            const int low = mask & -mask;
            merge_labels(n, sl[low], sl[mask ^ low], &sl[mask], nullptr);
            sdep[mask] = sdep[low] || sdep[mask ^ low];
            if (mask != full && weight_of(sl[mask], w) > cap) {
                best[mask] = -1;  // not formed
                continue;
            }
            double bt = -1;
            int bs = 0;
            // splits with the lowest member in `sub`, so each unordered pair is seen once
            for (int sub = (mask - 1) & mask; sub; sub = (sub - 1) & mask) {
                if (!(sub & low)) continue;
                const int rest = mask ^ sub;
                if (best[sub] < 0 || best[rest] < 0) continue;
                const double c = best[sub] + best[rest] + step_time(sl[sub], sdep[sub], sl[rest], sdep[rest], sl[mask], w, m);
                if (bt < 0 || c < bt) {
                    bt = c;
                    bs = sub;
                }
            }
            best[mask] = bt;
            split[mask] = bs;
        }
        if (best[full] < 0 || best[full] >= cur * (1.0 - 1e-9)) continue;
        saved += cur - best[full];
        // rebuild: x stays the subtree's root; the other inner ids are reused
        std::vector<int> free_ids(inner.begin() + 1, inner.end());
        std::vector<std::pair<int, int>> todo{{full, x}};
        while (!todo.empty()) {
            auto [mask, id] = todo.back();
            todo.pop_back();
            const int a = split[mask], b = mask ^ a;
            int ids[2];
            const int parts[2] = {a, b};
            for (int s = 0; s < 2; s++) {
                if ((parts[s] & (parts[s] - 1)) == 0) {
                    ids[s] = front[__builtin_ctz(parts[s])];
                } else {
                    ids[s] = free_ids.back();
                    free_ids.pop_back();
                    todo.push_back({parts[s], ids[s]});
                }
            }
            t.L[id] = ids[0];
            t.R[id] = ids[1];
            t.lab[id] = sl[mask];
            t.dep[id] = sdep[mask];
        }
    }
    return saved;
}

Cost cost_tree(const Net& n, const Tree& t, const std::vector<int>& w, const Model& m) {
    return cost_of(n, tree_steps(n, pairs_of(t)), w, m);
}

// ---------------------------------------------------------------------------------------------
// slicing
// ---------------------------------------------------------------------------------------------
struct Scored {
    std::vector<std::pair<int, int>> pairs;
    std::vector<int> sliced;
    Cost cost;
    double slices_log2 = 0;
    double key() const { return cost.time * std::ldexp(1.0, (int)slices_log2); }
};

// Adds at most `limit` labels to s->sliced; returns how many it added.
int slice_greedy(const Net& n, const Steps& st, const Model& m, double max_log2, int max_sliced, int num, Scored* s,
                 int limit) {
    std::vector<int> w = n.w;
    for (int l : s->sliced) w[l] = 0;
    s->cost = cost_of(n, st, w, m);
    int added = 0;
    while (added < limit) {
        const bool need_width = max_log2 > 0 && s->cost.max_log2 > max_log2;
        const bool need_num = num > 0 && (int)s->sliced.size() < num;
        if (!need_width && !need_num) break;
        if (max_sliced > 0 && (int)s->sliced.size() >= max_sliced) break;
        // candidates: labels of the intermediates within 1 of the largest, not open
        std::vector<int> cand;
        for (size_t k = 0; k < st.res.size(); k++) {
            int gc = 0;
            for (int l : st.res[k]) gc += w[l];
            if (gc + 1 >= s->cost.max_log2)
                for (int l : st.res[k])
                    if (w[l] > 0 && !n.keep[l]) cand.push_back(l);
        }
        std::sort(cand.begin(), cand.end());
        cand.erase(std::unique(cand.begin(), cand.end()), cand.end());
        if (cand.empty()) break;
        int best = -1;
        Cost bc;
        double bkey = 0;
        for (int l : cand) {
            const int keepw = w[l];
            w[l] = 0;
            const Cost c = cost_of(n, st, w, m);
            w[l] = keepw;
            const double key = c.time * std::ldexp(1.0, keepw);
            if (best < 0 || c.max_log2 < bc.max_log2 || (c.max_log2 == bc.max_log2 && key < bkey)) {
                best = l;
                bc = c;
                bkey = key;
            }
        }
        s->slices_log2 += w[best];
        w[best] = 0;
        s->sliced.push_back(best);
        s->cost = bc;
        added++;
    }
    return added;
}

}  // namespace

extern "C" int qxg_plan_contraction(int32_t ntensors, const int64_t* label_off, const int32_t* labels, int32_t nlabels,
                                    const int32_t* label_log2dim, const uint8_t* label_open,
                                    const qxg_plan_options* opts, int32_t* pairs_out, uint8_t* label_sliced,
                                    qxg_plan_stats* stats) {
    if (ntensors < 1 || nlabels < 0 || !label_off || (label_off[ntensors] > 0 && !labels) ||
        (nlabels > 0 && !label_log2dim) || (ntensors > 1 && !pairs_out))
        return qxg::ncon_fail(QXG_ERR_INVALID, "qxg_plan_contraction: bad arguments");
    try {
        Net n;
        n.V = ntensors;
        n.E = nlabels;
        n.vlab.resize(n.V);
        n.pins.resize(n.E);
        n.w.assign(label_log2dim, label_log2dim + nlabels);
        for (int l = 0; l < n.E; l++)
            if (n.w[l] < 0 || n.w[l] > 16) return qxg::ncon_fail(QXG_ERR_INVALID, "qxg_plan_contraction: label log2 dimension outside 0..16");
        if (label_off[0] < 0) return qxg::ncon_fail(QXG_ERR_INVALID, "qxg_plan_contraction: negative label offset");
        // every offset first: labels are then read only within [label_off[0], label_off[V]),
        // the extent the caller declares for its array
        for (int v = 0; v < n.V; v++)
            if (label_off[v + 1] < label_off[v]) return qxg::ncon_fail(QXG_ERR_INVALID, "qxg_plan_contraction: label offsets decrease");
        for (int v = 0; v < n.V; v++) {
            for (int64_t p = label_off[v]; p < label_off[v + 1]; p++) {
                const int l = labels[p];
                if (l < 0 || l >= n.E) return qxg::ncon_fail(QXG_ERR_INVALID, "qxg_plan_contraction: label id out of range");
                n.vlab[v].push_back(l);
            }
            std::sort(n.vlab[v].begin(), n.vlab[v].end());
            n.vlab[v].erase(std::unique(n.vlab[v].begin(), n.vlab[v].end()), n.vlab[v].end());
            for (int l : n.vlab[v]) n.pins[l].push_back(v);
        }
        n.keep.assign(n.E, 0);
        for (int l = 0; l < n.E; l++) n.keep[l] = (char)((label_open && label_open[l]) || n.pins[l].size() <= 1);
        n.batched.assign(n.V, 0);

        qxg_plan_options o;
        std::memset(&o, 0, sizeof(o));
        if (opts) o = *opts;
        const int trials = o.trials > 0 ? o.trials : 64;
        const int gtrials = o.greedy_trials < 0 ? 0 : (o.greedy_trials > 0 ? o.greedy_trials : 16);
        Model m;
        if (o.flops_per_s > 0) m.flops_rate = o.flops_per_s;
        if (o.bytes_per_s > 0) m.bytes_rate = o.bytes_per_s;
        if (o.tensor_batched && o.batch_log2 > 0) {
            if (o.batch_log2 > 40) return qxg::ncon_fail(QXG_ERR_INVALID, "qxg_plan_contraction: batch_log2 above 40");
            m.batch = std::exp2(o.batch_log2);
            for (int v = 0; v < n.V; v++) n.batched[v] = o.tensor_batched[v] ? 1 : 0;
        }

        std::vector<Scored> trees;
        std::vector<int> all(n.V);
        std::iota(all.begin(), all.end(), 0);
        for (int t = 0; t < gtrials + trials; t++) {
            Rng rng((uint64_t)o.seed * 1000003ull + (uint64_t)t);
            Scored s;
            if (t < gtrials) {
                std::vector<Labels> lab(n.V);
                for (int v = 0; v < n.V; v++) lab[v] = leaf_labels(n, v);
                Greedy gr{n, rng, t == 0 ? 0.0 : 0.05 + 0.5 * rng.uniform(), &lab, &s.pairs, n.V};
                gr.run(all);
            } else {
                const double eps = 0.02 + 0.5 * rng.uniform() * rng.uniform();
                const int cutoff = 2 + rng.below(12);
                Divider d(n, rng, eps, cutoff, 0.0);
                d.build(all);
                s.pairs = std::move(d.pairs);
            }
            const Steps st = tree_steps(n, s.pairs);
            s.cost = cost_of(n, st, n.w, m);
            trees.push_back(std::move(s));
        }
        // refine the best trees (by modelled time, and the narrowest ones, which slice cheaply),
        // slice them, refine again under the sliced dimensions, and keep the cheapest
        std::vector<int> idx(trees.size());
        std::iota(idx.begin(), idx.end(), 0);
        std::sort(idx.begin(), idx.end(), [&](int a, int b) {
            if (trees[a].cost.time != trees[b].cost.time) return trees[a].cost.time < trees[b].cost.time;
            return a < b;
        });
        const bool slicing = o.max_log2 > 0 || o.num_sliced > 0;
        constexpr int kNoCap = 1 << 30;
        const int width_cap = o.max_log2 > 0 ? (int)std::floor(o.max_log2) : kNoCap;
        std::vector<int> pick(idx.begin(), idx.begin() + std::min<int>((int)idx.size(), 6));
        if (slicing) {
            std::vector<int> by_width = idx;
            std::stable_sort(by_width.begin(), by_width.end(),
                             [&](int a, int b) { return trees[a].cost.max_log2 < trees[b].cost.max_log2; });
            for (int k = 0; k < std::min<int>((int)by_width.size(), 4); k++) pick.push_back(by_width[k]);
        }
        std::sort(pick.begin(), pick.end());
        pick.erase(std::unique(pick.begin(), pick.end()), pick.end());
        auto refine = [&](Scored& s, const std::vector<int>& w, int k, int cap) {
            Tree t = tree_of(n, s.pairs);
            double cur = cost_tree(n, t, w, m).time;
            for (int pass = 0; pass < 8; pass++) {
                const double saved = reconfigure_pass(n, t, w, m, k, cap);
                cur -= saved;
                if (saved <= 1e-3 * cur) break;
            }
            s.pairs = pairs_of(t);
        };
        int best = -1;
        for (int i : pick) {
            Scored& s = trees[i];
            refine(s, n.w, 8, kNoCap);
            if (slicing) {  // one label at a time, the tree reconfigured under each new slicing
                while (slice_greedy(n, tree_steps(n, s.pairs), m, o.max_log2, o.max_sliced, o.num_sliced, &s, 1)) {
                    std::vector<int> w = n.w;
                    for (int l : s.sliced) w[l] = 0;
                    refine(s, w, 8, width_cap);
                }
            }
            std::vector<int> w = n.w;
            for (int l : s.sliced) w[l] = 0;
            s.cost = cost_of(n, tree_steps(n, s.pairs), w, m);
            const bool ok = !(o.max_log2 > 0) || s.cost.max_log2 <= o.max_log2;
            const bool bok = best < 0 ? false : (!(o.max_log2 > 0) || trees[best].cost.max_log2 <= o.max_log2);
            if (best < 0 || (ok && !bok) || (ok == bok && (ok ? s.key() < trees[best].key()
                                                              : s.cost.max_log2 < trees[best].cost.max_log2)))
                best = i;
        }
        {  // a last refinement of the winner over larger subtrees
            Scored& s = trees[best];
            std::vector<int> w = n.w;
            for (int l : s.sliced) w[l] = 0;
            refine(s, w, 10, width_cap);
            s.cost = cost_of(n, tree_steps(n, s.pairs), w, m);
        }
        const Scored& b = trees[best];
        for (size_t k = 0; k < b.pairs.size(); k++) {
            pairs_out[2 * k] = b.pairs[k].first;
            pairs_out[2 * k + 1] = b.pairs[k].second;
        }
        if (label_sliced) {
            std::memset(label_sliced, 0, (size_t)nlabels);
            for (int l : b.sliced) label_sliced[l] = 1;
        }
        if (stats) {
            std::memset(stats, 0, sizeof(*stats));
            stats->log2_flops = std::log2(std::max(b.cost.flops, 1.0));
            stats->log2_flops_total = stats->log2_flops + b.slices_log2;
            stats->max_log2 = b.cost.max_log2;
            stats->time = b.cost.time;
            stats->log2_slices = b.slices_log2;
            stats->num_sliced = (int32_t)b.sliced.size();
            stats->trees_tried = (int32_t)trees.size();
        }
    } catch (const std::exception& e) {
        return qxg::ncon_fail(QXG_ERR_INVALID, (std::string("qxg_plan_contraction: ") + e.what()).c_str());
    }
    return QXG_OK;
}
