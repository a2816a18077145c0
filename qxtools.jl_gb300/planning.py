"""Contraction planning (mirror of src/contraction_planning.jl).

The plan format is the reference's: an ordered list of `(A, B, C)` tensor-symbol triples
(`order_to_contraction_plan`, contraction_planning.jl:386-448; `tree_to_contraction_plan`
:476-485).  The executor consumes plans unchanged; this module only produces them.

The reference's planners live in un-vendored packages: FlowCutter (a native program inside
QXGraphDecompositions, called by `flow_cutter_contraction_plan` :90-113 and
`contraction_scheme` :219-299), `min_fill` and `greedy_treewidth_deletion`
(QXGraphDecompositions) and netcon (`TensorOperations.optimaltree`, :318-331).  This module
restates the published algorithms in its own code:
  - `min_fill`: the min-fill elimination heuristic on the line graph (ties -> lowest
    degree, then lowest vertex id; seeded random ties when `seed` is given);
  - `order_to_contraction_plan`: restated from :386-448 (two-tensor edges -> one pairwise
    contraction named `I<i>`; larger hyperedges -> netcon when < 37 tensors, else min fill);
  - `netcon`: exact minimum-FLOP contraction tree by dynamic programming over subsets for
    up to 12 tensors, greedy beyond that;
  - `flow_cutter_contraction_plan`: FlowCutter is unavailable, so this stand-in keeps the
    signature and returns the cheapest of min-fill and seeded random-greedy plans (`time`
    scales the number of trials; `time=0` gives the min-fill plan, the reference's
    fall-back at :102-106);
  - `contraction_scheme`: greedy slicing: repeatedly slice the hyperedge whose removal
    most reduces the largest intermediate (then total FLOPs), re-planning without it, like
    greedy treewidth deletion with modified orders (:254-270).
Plans are deterministic for a given seed.
"""
from __future__ import annotations

import heapq
import itertools
import math
from collections import OrderedDict

import numpy as np

__all__ = [
    "HyperNet", "hyper_network", "contraction_indices", "plan_cost",
    "convert_to_graph", "convert_to_line_graph", "min_fill",
    "order_to_contraction_plan", "netcon", "greedy_contraction_plan",
    "flow_cutter_contraction_plan", "min_fill_contraction_plan", "contraction_scheme",
    "native_plan", "native_contraction_scheme",
]


class HyperNet:
    """Planning view of a tensor network: tensor -> hyperedge labels, label -> dimension,
    and the set of open labels (unterminated wires, which survive every contraction)."""

    def __init__(self, tensors: "OrderedDict[str, list]", dims: dict, open_labels=()):
        self.tensors = OrderedDict((k, list(v)) for k, v in tensors.items())
        self.dims = dict(dims)
        self.open = set(open_labels)
        self._counter = 0
        self._names = set(self.tensors)

    def copy(self) -> "HyperNet":
        h = HyperNet(self.tensors, self.dims, self.open)
        h._counter = self._counter
        h._names = set(self._names)
        return h

    def holders(self, label) -> list:
        return [t for t, ls in self.tensors.items() if label in ls]

    def next_tensor_id(self) -> str:
        while True:
            self._counter += 1
            name = f"t{len(self._names) + self._counter}"
            if name not in self._names:
                self._names.add(name)
                return name


def hyper_network(tnc_or_tn) -> HyperNet:
    """HyperNet of a TensorNetworkCircuit (labels = hyperedge roots of each tensor's groups)."""
    tn = getattr(tnc_or_tn, "tn", tnc_or_tn)
    opens = tnc_or_tn.open_labels() if hasattr(tnc_or_tn, "open_labels") else set()
    tensors = OrderedDict((name, tn.labels(name)) for name in tn.tensors)
    dims = {tn.root(ix): d for ix, d in tn.dims.items()}
    return HyperNet(tensors, dims, opens)


def contraction_indices(net: HyperNet, a: str, b: str):
    """Result labels of contracting tensors a and b (QXTns `contraction_indices`, called at
    src/compute_graph/compute_graph.jl:65): a label shared by a and b is summed unless another
    tensor holds it or it is open; kept labels are a's in order, then b's new ones."""
    la, lb = net.tensors[a], net.tensors[b]
    others = set()
    for t, ls in net.tensors.items():
        if t != a and t != b:
            others.update(ls)
    keep = []
    for lab in la + lb:
        if lab in keep:
            continue
        shared = lab in la and lab in lb
        if not shared or lab in others or lab in net.open:
            keep.append(lab)
    return keep, list(la), list(lb)


def mock_contract(net: HyperNet, a: str, b: str, c: str | None = None) -> str:
    """`contract_pair!(tn, a, b, c; mock=true)`: replace a and b by c with the result labels."""
    lc, _, _ = contraction_indices(net, a, b)
    if c is None:
        c = net.next_tensor_id()
    del net.tensors[a]
    del net.tensors[b]
    net.tensors[c] = lc
    net._names.add(c)
    return c


# ---------------------------------------------------------------------------------------
# cost model
# ---------------------------------------------------------------------------------------
def _lg(net: HyperNet, labels, sliced=()) -> float:
    return sum(0.0 if l in sliced else math.log2(net.dims[l]) for l in labels)


# roofline of one step on the GPU executor, for ranking plans: FLOPs at 1e14 /s (split-precision
# tensor cores) against Complex64 bytes (|A| + |B| + |C|) at 5e12 /s, whichever is longer
_RANK_FLOPS = 1e14
_RANK_BYTES = 5e12


def plan_cost(net: HyperNet, plan, sliced=(), batched=(), beta: int = 1) -> dict:
    """FLOPs (8 |C| K per step, complex), largest intermediate (log2 elements) and the
    per-step shapes of `plan` on `net` with `sliced` labels at dimension 1 (one slice).

    For ranking plans on the GPU executor, which runs `beta` bitstrings at once: the tensors
    that depend on the `batched` tensors (the outputs) carry a batch of `beta`; "time" is the
    sum over steps of max(FLOPs / 1e14, 8 (|A| + |B| + |C|) / 5e12) seconds with those batches,
    and "max_log2_batched" the largest batched intermediate."""
    st = net.copy()
    dep = set(batched)
    lbeta = math.log2(beta) if beta > 1 else 0.0
    flops = 0.0
    est = 0.0
    max_lg = 0.0
    max_lgb = 0.0
    steps = []
    for (a, b, c) in plan:
        lc, la, lb = contraction_indices(st, a, b)
        every = set(la) | set(lb)
        lg_all = _lg(st, every, sliced)
        lg_c = _lg(st, lc, sliced)
        lg_a, lg_b = _lg(st, la, sliced), _lg(st, lb, sliced)
        f = 8.0 * 2.0 ** lg_all
        flops += f
        da, db = a in dep, b in dep
        dc = da or db
        if dc:
            dep.add(c)
        ba, bb, bc = (lbeta if da else 0.0), (lbeta if db else 0.0), (lbeta if dc else 0.0)
        est += max(f * 2.0 ** bc / _RANK_FLOPS,
                   8.0 * (2.0 ** (lg_a + ba) + 2.0 ** (lg_b + bb) + 2.0 ** (lg_c + bc)) / _RANK_BYTES)
        max_lg = max(max_lg, lg_c)
        max_lgb = max(max_lgb, lg_c + bc)
        steps.append((lg_c, lg_a, lg_b, lg_all - lg_c))
        mock_contract(st, a, b, c)
    return {"flops": flops, "max_log2": max_lg, "time": est, "max_log2_batched": max_lgb, "steps": steps}


# ---------------------------------------------------------------------------------------
# graphs (convert_to_graph :18-29, convert_to_line_graph :47-63)
# ---------------------------------------------------------------------------------------
def convert_to_graph(tnc):
    """Simple graph: a vertex per tensor, an edge per plain bond shared by two tensors."""
    import networkx as nx
    tn = getattr(tnc, "tn", tnc)
    g = nx.Graph()
    names = list(tn.tensors)
    pos = {n: i for i, n in enumerate(names)}
    g.add_nodes_from(range(len(names)))
    for ix in tn.bonds():
        ts = tn.tensors_with_index(ix)
        if len(ts) == 2:
            g.add_edge(pos[ts[0]], pos[ts[1]])
    return g


def _edges(tnc, use_hyperedges: bool) -> list:
    tn = getattr(tnc, "tn", tnc)
    if use_hyperedges:
        return [ts for _, ts in tn.hyperedges().items()]
    return [tn.tensors_with_index(ix) for ix in tn.bonds()]


def convert_to_line_graph(tnc, use_hyperedges: bool = False):
    """Line graph: a vertex per (hyper)edge, joined when the edges share a tensor.  Returns
    (networkx graph on vertex ids 0.., symbol_map: vertex id -> tensor names)."""
    import networkx as nx
    edges = _edges(tnc, use_hyperedges)
    g = nx.Graph()
    g.add_nodes_from(range(len(edges)))
    holder: dict = {}
    for i, ts in enumerate(edges):
        for t in ts:
            holder.setdefault(t, []).append(i)
    for vs in holder.values():
        for i, j in itertools.combinations(sorted(set(vs)), 2):
            g.add_edge(i, j)
    return g, {i: list(ts) for i, ts in enumerate(edges)}


def min_fill(graph, seed=None):
    """Min-fill elimination order of an undirected graph -> (width, order).

    Each step eliminates the vertex whose neighbourhood needs the fewest fill edges (ties:
    smaller degree, then smaller id, or a seeded random choice), connects its neighbours
    and records its degree; width = the largest such degree."""
    adj = {v: set(graph.neighbors(v)) for v in graph.nodes}
    rng = np.random.default_rng(seed) if seed is not None else None

    def fill(v):
        nb = list(adj[v])
        f = 0
        for i in range(len(nb)):
            ai = adj[nb[i]]
            for j in range(i + 1, len(nb)):
                if nb[j] not in ai:
                    f += 1
        return f

    score = {v: fill(v) for v in adj}
    order, width = [], 0
    while adj:
        best = min(score[v] for v in adj)
        cands = [v for v in adj if score[v] == best]
        if rng is not None and len(cands) > 1:
            v = cands[int(rng.integers(len(cands)))]
        else:
            v = min(cands, key=lambda x: (len(adj[x]), x))
        nb = list(adj[v])
        width = max(width, len(nb))
        for i in range(len(nb)):
            for j in range(i + 1, len(nb)):
                adj[nb[i]].add(nb[j]); adj[nb[j]].add(nb[i])
        for u in nb:
            adj[u].discard(v)
        del adj[v]
        del score[v]
        touched = set(nb)
        for u in nb:
            touched.update(adj[u])
        for u in touched:
            if u in adj:
                score[u] = fill(u)
        order.append(v)
    return width, order


# ---------------------------------------------------------------------------------------
# order -> plan (:386-448) and netcon (:318-367, tree_to_contraction_plan :476-485)
# ---------------------------------------------------------------------------------------
def _intermediate(imap: dict, t: str) -> str:
    """`_get_intermediate_tensor` (:460-467)."""
    while True:
        i = imap[t]
        if i == t:
            return i
        t = i


def order_to_contraction_plan(order, net: HyperNet) -> list:
    """Edge elimination order -> plan (restated from contraction_planning.jl:386-448)."""
    plan = []
    imap = {t: t for t in net.tensors}
    for i, edge in enumerate(order, start=1):
        if len(edge) == 2:
            a = _intermediate(imap, edge[0])
            b = _intermediate(imap, edge[1])
            if a != b:
                c = f"I{i}"
                plan.append((a, b, c))
                imap[a] = c; imap[b] = c; imap[c] = c
        elif len(edge) > 2:
            group: "OrderedDict[str, list]" = OrderedDict()
            for t in edge:
                it = _intermediate(imap, t)
                prev = group.get(it, [])
                inds = net.tensors[t]
                group[it] = [x for x in prev if x not in inds] + [x for x in inds if x not in prev]
            if len(group) > 1:
                if len(group) < 37:
                    local = _netcon_plan(net, group)
                else:
                    local = _min_fill_group_plan(net, group)
                plan.extend(local)
                for (a, b, c) in local:
                    imap[a] = c; imap[b] = c; imap[c] = c
    return plan


def _netcon_plan(net: HyperNet, group: "OrderedDict[str, list]") -> list:
    """Contraction plan for a small set of tensors, named with `next_tensor_id`."""
    names = list(group)
    lsets = [frozenset(group[n]) for n in names]
    tree = _optimal_tree(lsets, net.dims) if len(names) <= 12 else _greedy_tree(lsets, net.dims)
    plan = []

    def walk(node):
        if isinstance(node, int):
            return names[node]
        a = walk(node[0]); b = walk(node[1])
        c = net.next_tensor_id()
        plan.append((a, b, c))
        return c
    walk(tree)
    return plan


def _min_fill_group_plan(net: HyperNet, group) -> list:
    """Fallback for large hyperedge groups: contract along min-fill order of the tensor graph."""
    names = list(group)
    plan = []
    cur = names[0]
    for n in names[1:]:
        c = net.next_tensor_id()
        plan.append((cur, n, c))
        cur = c
    return plan


def _result_labels(la: frozenset, lb: frozenset, outside: frozenset) -> frozenset:
    return (la ^ lb) | ((la & lb) & outside)


def _optimal_tree(lsets, dims):
    """Exact minimum-FLOP binary contraction tree over <= 12 tensors (subset DP)."""
    n = len(lsets)
    full = (1 << n) - 1
    every = frozenset().union(*lsets)
    # labels a subset's result keeps: those also held outside the subset
    lab_of = {}
    for m in range(1, full + 1):
        inside = frozenset().union(*[lsets[i] for i in range(n) if m >> i & 1])
        outside = frozenset().union(*[lsets[i] for i in range(n) if not m >> i & 1]) if m != full else frozenset()
        keep = frozenset(l for l in inside if l in outside)
        lab_of[m] = keep
    best = {1 << i: (0.0, i) for i in range(n)}
    for m in range(1, full + 1):
        if m & (m - 1) == 0:
            continue
        bc, bt = math.inf, None
        sub = (m - 1) & m
        while sub:
            other = m ^ sub
            if sub < other and sub in best and other in best:
                labels = lab_of[sub] | lab_of[other]
                cost = best[sub][0] + best[other][0] + math.prod(dims[l] for l in labels)
                if cost < bc:
                    bc, bt = cost, (best[sub][1], best[other][1])
            sub = (sub - 1) & m
        best[m] = (bc, bt)
    del every
    return best[full][1]


def _greedy_tree(lsets, dims):
    nodes = {i: (lsets[i], i) for i in range(len(lsets))}
    nxt = len(lsets)
    while len(nodes) > 1:
        keys = list(nodes)
        bestc, bp = math.inf, None
        for i, j in itertools.combinations(keys, 2):
            la, lb = nodes[i][0], nodes[j][0]
            outside = frozenset().union(*[nodes[k][0] for k in keys if k != i and k != j]) if len(keys) > 2 else frozenset()
            lc = _result_labels(la, lb, outside)
            c = math.prod(dims[l] for l in lc) - math.prod(dims[l] for l in la) - math.prod(dims[l] for l in lb)
            if (la & lb) and c < bestc or bp is None:
                bestc, bp = c, (i, j)
        i, j = bp
        la, lb = nodes[i][0], nodes[j][0]
        outside = frozenset().union(*[nodes[k][0] for k in nodes if k != i and k != j]) if len(nodes) > 2 else frozenset()
        nodes[nxt] = (_result_labels(la, lb, outside), (nodes[i][1], nodes[j][1]))
        del nodes[i], nodes[j]
        nxt += 1
    return next(iter(nodes.values()))[1]


def netcon(tnc) -> list:
    """Contraction plan of the whole network by netcon (:318-331): exact for <= 12 tensors,
    greedy beyond."""
    net = tnc if isinstance(tnc, HyperNet) else hyper_network(tnc)
    return _netcon_plan(net, OrderedDict((k, v) for k, v in net.tensors.items()))


# ---------------------------------------------------------------------------------------
# greedy planner (seeded, randomised)
# ---------------------------------------------------------------------------------------
def greedy_contraction_plan(net: HyperNet, seed=0, temperature: float = 0.0, exclude=(),
                            score: str = "size") -> list:
    """Seeded greedy contraction: repeatedly contract the pair of tensors sharing a
    (non-excluded) label with the lowest score, plus Gumbel noise of the given temperature.
    Scores (log2 units): "size" = signed log of size(C) - size(A) - size(B) (the classic
    greedy), "growth" = log size(C) - max(log size(A), log size(B)).  Intermediates are named
    `I<k>`.  Disconnected components are left for the caller (build_compute_graph joins
    them)."""
    rng = np.random.default_rng(seed)
    excl = set(exclude)
    lg = {l: (0.0 if l in excl else math.log2(d)) for l, d in net.dims.items()}
    tens = {n: set(ls) for n, ls in net.tensors.items()}
    holders: dict = {}
    for n, ls in tens.items():
        for l in ls:
            holders.setdefault(l, set()).add(n)
    opens = set(net.open)

    def size_lg(ls):
        return sum(lg[l] for l in ls)

    def result(a, b):
        la, lb = tens[a], tens[b]
        out = set()
        for l in la | lb:
            if l in la and l in lb:
                if len(holders[l]) > 2 or l in opens:
                    out.add(l)
            else:
                out.add(l)
        return out

    def cost(a, b):
        c = size_lg(result(a, b))
        x, y = size_lg(tens[a]), size_lg(tens[b])
        if score == "growth":
            s = c - max(x, y)
        else:
            d = 2.0 ** c - 2.0 ** x - 2.0 ** y
            s = math.copysign(math.log2(abs(d) + 1.0), d)
        if temperature > 0:
            s -= temperature * float(rng.gumbel())
        return s

    heap = []
    counter = itertools.count()
    order_idx = {n: i for i, n in enumerate(tens)}

    def push_pairs(n):
        # sets are walked in a fixed order (labels by name, tensors by creation): the pushes and
        # the random draws must not depend on string hashing
        seen = set()
        for l in sorted(tens[n], key=str):
            if l in excl:
                continue
            for m in sorted(holders[l], key=order_idx.__getitem__):
                if m != n and m not in seen:
                    seen.add(m)
                    a, b = (n, m) if order_idx[n] < order_idx[m] else (m, n)
                    heapq.heappush(heap, (cost(a, b), next(counter), a, b))

    for n in list(tens):
        push_pairs(n)
    plan = []
    k = 0
    while heap:
        _, _, a, b = heapq.heappop(heap)
        if a not in tens or b not in tens:
            continue
        k += 1
        c = f"I{k}"
        while c in tens or c in order_idx:
            k += 1
            c = f"I{k}"
        lc = result(a, b)
        for l in tens[a] | tens[b]:
            holders[l].discard(a)
            holders[l].discard(b)
        del tens[a], tens[b]
        tens[c] = lc
        order_idx[c] = len(order_idx)
        for l in lc:
            holders[l].add(c)
        plan.append((a, b, c))
        push_pairs(c)
    return plan


def _sort_key_cost(net, plan, sliced=(), width_cap=None, batched=(), beta=1):
    """(largest intermediate, FLOPs); with `width_cap`, every plan whose largest batched
    intermediate is at most 2^width_cap ranks by its estimated time alone (plan_cost)."""
    pc = plan_cost(net, plan, sliced, batched, beta)
    if width_cap is not None:
        return (max(pc["max_log2_batched"], width_cap), pc["time"])
    return (pc["max_log2"], pc["flops"])


_TRIAL_SETTINGS = [("size", 0.0), ("growth", 0.0), ("growth", 0.5), ("size", 0.2), ("growth", 0.3),
                   ("size", 0.5)]


def random_greedy_plans(net: HyperNet, trials: int, seed: int = 0, exclude=()):
    """`trials` seeded greedy plans cycling through score functions and temperatures."""
    for t in range(trials):
        score, temp = _TRIAL_SETTINGS[t % len(_TRIAL_SETTINGS)]
        yield greedy_contraction_plan(net, seed=seed * 7919 + t, temperature=temp, exclude=exclude,
                                      score=score)


def flow_cutter_contraction_plan(tnc, time: int = 60, seed: int = -1, hypergraph: bool = True,
                                 width_cap: float | None = None, batched=(), beta: int = 1) -> list:
    """Stand-in for FlowCutter planning (:90-113): best of the min-fill plan and
    `8 * time` seeded random-greedy plans by (largest intermediate, FLOPs) -- the reference
    minimises the tree width first; `width_cap` (log2 elements) ranks every plan whose largest
    intermediate, batched by `beta` bitstrings where it depends on the `batched` (output)
    tensors, is within the cap by its estimated time alone (plan_cost).  `time=0` returns the min-fill plan (the reference's fall-back,
    :102-106)."""
    net = hyper_network(tnc) if not isinstance(tnc, HyperNet) else tnc
    base = min_fill_contraction_plan(tnc, hypergraph=hypergraph)
    if time <= 0:
        return base
    seed0 = 0 if seed is None or seed < 0 else int(seed)
    best, bestk = base, _sort_key_cost(net, base, (), width_cap, batched, beta)
    for p in random_greedy_plans(net, max(1, 8 * int(time)), seed0):
        if len(p) < len(base):
            continue
        k = _sort_key_cost(net, p, (), width_cap, batched, beta)
        if k < bestk:
            best, bestk = p, k
    return best


def min_fill_contraction_plan(tnc, hypergraph: bool = False) -> list:
    """Min-fill plan (:127-140): line graph -> min-fill order -> order_to_contraction_plan."""
    net = hyper_network(tnc) if not isinstance(tnc, HyperNet) else tnc
    lg, symbol_map = convert_to_line_graph(tnc, use_hyperedges=hypergraph)
    _, order = min_fill(lg)
    return order_to_contraction_plan([symbol_map[v] for v in order], net)


def _slice_candidates(net, plan, sliced):
    """Labels of the largest intermediates of `plan` (not yet sliced, not open)."""
    pc = plan_cost(net, plan, sliced)
    st = net.copy()
    scored = {}
    for (a, b, c), (lgc, _, _, _) in zip(plan, pc["steps"]):
        lc, _, _ = contraction_indices(st, a, b)
        if lgc >= pc["max_log2"] - 2:
            for l in lc:
                if l not in sliced and l not in net.open:
                    scored[l] = scored.get(l, 0) + 1
        mock_contract(st, a, b, c)
    return sorted(scored, key=lambda l: (-scored[l], l))[:24]


def _scheme_key(net, plan, sliced, width_cap=None, batched=(), beta=1):
    q = plan_cost(net, plan, sliced, batched, beta)
    nsl = math.prod(net.dims[x] for x in sliced) if sliced else 1
    if width_cap is not None:
        return (max(q["max_log2_batched"], width_cap), q["time"] * nsl)
    return (q["max_log2"], q["flops"] * nsl)


def _done(net, plan, sliced, num, max_log2):
    if max_log2 is not None:
        return plan_cost(net, plan, sliced)["max_log2"] <= max_log2
    return len(sliced) >= num


def _scheme_by_order(tnc, net, num, hypergraph, max_log2):
    """Reference-style slicing: remove sliced line-graph vertices from the elimination order
    and convert the modified order to a plan (contraction_planning.jl:254-270)."""
    tn = getattr(tnc, "tn", tnc)
    lg, smap = convert_to_line_graph(tnc, use_hyperedges=hypergraph)
    _, order = min_fill(lg)
    if hypergraph:
        vlabel = {v: l for v, l in zip(sorted(smap), net_labels_in_order(tn))}
    else:
        bonds = tn.bonds()
        vlabel = {v: tn.root(bonds[v]) for v in smap}
    removed: list = []
    sliced: list = []
    plan = order_to_contraction_plan([smap[v] for v in order], net)
    widths = []
    while len(removed) < len(order) and (len(removed) < num if max_log2 is None else
                                         not _done(net, plan, sliced, num, max_log2)):
        best = None
        cand_labels = set(_slice_candidates(net, plan, sliced)) or {vlabel[v] for v in order if v not in removed}
        for v in order:
            if v in removed or vlabel[v] not in cand_labels and vlabel[v] not in sliced:
                continue
            rem = removed + [v]
            sl = sliced if vlabel[v] in sliced else sliced + [vlabel[v]]
            p = order_to_contraction_plan([smap[u] for u in order if u not in rem], net)
            k = _scheme_key(net, p, sl)
            if best is None or k < best[0]:
                best = (k, v, p, sl)
        if best is None:
            break
        _, v, plan, sliced = best
        removed.append(v)
        widths.append(plan_cost(net, plan, sliced)["max_log2"])
    return plan, sliced, widths


def net_labels_in_order(tn):
    return list(tn.hyperedges().keys())


def _scheme_by_greedy(net, num, seed0, max_log2, base_plan, replan_trials=6):
    plan = base_plan
    sliced: list = []
    widths = []
    while not _done(net, plan, sliced, num, max_log2):
        cands = _slice_candidates(net, plan, sliced)
        if not cands:
            break
        best = min(cands, key=lambda l: _scheme_key(net, plan, sliced + [l]))
        sliced.append(best)
        for p in random_greedy_plans(net, replan_trials, seed0 * 31 + len(sliced), exclude=sliced):
            if _scheme_key(net, p, sliced) < _scheme_key(net, plan, sliced):
                plan = p
        widths.append(plan_cost(net, plan, sliced)["max_log2"])
    return plan, sliced, widths


def contraction_scheme(tnc, num: int, time: int = 120, seed: int = -1,
                       score_function: str = "tree_trimming", hypergraph: bool = True,
                       max_log2: float | None = None, width_cap: float | None = None,
                       batched=(), beta: int = 1):
    """Plan plus bonds to slice (:219-299) -> (index_groups_to_slice, plan, metadata).

    Two greedy slicers, the cheaper result (largest intermediate, then FLOPs x slices) wins:
      - order based (the reference's structure): min-fill elimination order of the line graph;
        repeatedly remove the line-graph vertex whose removal gives the cheapest plan
        (`order_to_contraction_plan` of the modified order, like greedy treewidth deletion's
        modified orders at :254-270);
      - plan based (hypergraph mode, `time > 0`): slice the hyperedge of the largest
        intermediates that gives the cheapest plan, then re-plan with seeded greedy searches
        that ignore the sliced hyperedges.
    Stops after `num` bonds, or, when `max_log2` is given, once the largest intermediate is at
    most 2^max_log2 elements.  With `width_cap` (log2 elements), candidate plans whose largest
    intermediate -- batched by `beta` bitstrings where it depends on the `batched` (output)
    tensors -- is within the cap rank by estimated time alone (plan_cost; default: largest
    intermediate first, like the reference's tree-width minimisation).  Index groups are the plain index ids of each sliced hyperedge
    (`expand_slice_bonds_to_hyperindices`, :190-203).  Tensors left disconnected by slicing are
    joined by build_compute_graph (compute_graph.jl:77-90)."""
    tn = getattr(tnc, "tn", tnc)
    net = hyper_network(tnc)
    seed0 = 0 if seed is None or seed < 0 else int(seed)
    plan, sliced, widths = _scheme_by_order(tnc, net, num, hypergraph, max_log2)
    method = "min fill heuristic"
    if hypergraph and time > 0:
        base = flow_cutter_contraction_plan(tnc, time=time, seed=seed, hypergraph=hypergraph, width_cap=width_cap,
                                            batched=batched, beta=beta)
        p2, s2, w2 = _scheme_by_greedy(net, num, seed0, max_log2, base, replan_trials=max(6, 2 * int(time)))
        if (_scheme_key(net, p2, s2, width_cap, batched, beta) <
                _scheme_key(net, plan, sliced, width_cap, batched, beta)):
            plan, sliced, widths = p2, s2, w2
            method = "greedy stand-in for flow cutter"
    groups = []
    for l in sliced:
        groups.append(sorted(ix for ix in tn.dims if tn.root(ix) == l and tn.tensors_with_index(ix)))
    metadata = OrderedDict()
    metadata["Determination of contraction plan"] = OrderedDict([
        ("Method used", method),
        ("Treewidth", int(round(plan_cost(net, plan)["max_log2"]))),
        ("Time allocated", time), ("Seed used", seed), ("Hypergraph used", hypergraph),
        ("Hyperedge contraction method", "Netcon where possible, min fill heuristic otherwise."),
    ])
    metadata["Slicing"] = OrderedDict([
        ("Method used", "greedy deletion of the largest intermediate's bonds"),
        ("Edges sliced", len(sliced)), ("Score function used", score_function),
        ("Log2 largest intermediate after slicing consecutive edges", widths),
    ])
    return groups, plan, metadata


# ---------------------------------------------------------------------------------------
# the library's planner (qxg_plan_contraction)
# ---------------------------------------------------------------------------------------
def native_plan(net: HyperNet, trials: int = 64, greedy_trials: int = 16, seed: int = 0,
                max_log2: float | None = None, num_sliced: int = 0, max_sliced: int = 0, batched=(),
                beta: int = 1, lib=None):
    """Plan (and labels to slice) from the library's planner: recursive hypergraph bisection and
    random-greedy trees scored by the executor's step model, then greedy slicing until every
    intermediate has at most 2^max_log2 elements (or `num_sliced` labels are sliced).  Steps that
    depend on a `batched` tensor (the outputs) run `beta` times in the step model.
    -> (plan, sliced labels, stats dict).  Intermediates are named `I<k>`."""
    import ctypes as ct
    from .executor import _check, load_library, qxg_plan_options, qxg_plan_stats
    lib = lib or load_library()
    names = list(net.tensors)
    labs = sorted({l for ls in net.tensors.values() for l in ls}, key=lambda x: (str(type(x)), str(x)))
    lid = {l: i for i, l in enumerate(labs)}
    off, flat = [0], []
    for n in names:
        flat += [lid[l] for l in dict.fromkeys(net.tensors[n])]
        off.append(len(flat))
    log2dim = [max(0, int(math.ceil(math.log2(net.dims[l])))) for l in labs]
    opens = [1 if l in net.open else 0 for l in labs]
    V = len(names)
    a_off = (ct.c_int64 * (V + 1))(*off)
    a_lab = (ct.c_int32 * max(1, len(flat)))(*flat)
    a_w = (ct.c_int32 * max(1, len(labs)))(*log2dim)
    a_open = (ct.c_uint8 * max(1, len(labs)))(*opens)
    o = qxg_plan_options(trials=trials, greedy_trials=greedy_trials if greedy_trials else -1, seed=seed,
                         max_log2=float(max_log2 or 0.0), num_sliced=num_sliced, max_sliced=max_sliced)
    bset = set(batched)
    a_batched = (ct.c_uint8 * V)(*[1 if nm in bset else 0 for nm in names])
    if bset and beta > 1:
        o.tensor_batched = a_batched
        o.batch_log2 = math.log2(beta)
    pairs = (ct.c_int32 * max(1, 2 * (V - 1)))()
    sl = (ct.c_uint8 * max(1, len(labs)))()
    st = qxg_plan_stats()
    _check(lib, lib.qxg_plan_contraction(V, a_off, a_lab, len(labs), a_w, a_open, ct.byref(o), pairs, sl,
                                         ct.byref(st)))
    node = list(names)
    taken = set(names)
    plan, k = [], 0
    for s in range(V - 1):
        k += 1
        while f"I{k}" in taken:
            k += 1
        c = f"I{k}"
        taken.add(c)
        plan.append((node[pairs[2 * s]], node[pairs[2 * s + 1]], c))
        node.append(c)
    sliced = [labs[i] for i in range(len(labs)) if sl[i]]
    stats = {f: getattr(st, f) for f, _ in qxg_plan_stats._fields_ if f != "reserved"}
    return plan, sliced, stats


def native_contraction_scheme(tnc, num: int = 0, seed: int = 0, max_log2: float | None = None,
                              trials: int = 64, greedy_trials: int = 16, batched=(), beta: int = 1, lib=None):
    """`contraction_scheme` (:219-299) through the library's planner -> (index_groups_to_slice,
    plan, metadata): `num` bonds sliced (number_bonds_to_slice), or as many as bring every
    intermediate to at most 2^max_log2 elements; steps that depend on the `batched` tensors run
    `beta` times in the step model."""
    tn = getattr(tnc, "tn", tnc)
    net = hyper_network(tnc)
    plan, sliced, st = native_plan(net, trials=trials, greedy_trials=greedy_trials, seed=seed, max_log2=max_log2,
                                   num_sliced=num, batched=batched, beta=beta, lib=lib)
    groups = [sorted(ix for ix in tn.dims if tn.root(ix) == l and tn.tensors_with_index(ix)) for l in sliced]
    metadata = OrderedDict()
    metadata["Determination of contraction plan"] = OrderedDict([
        ("Method used", "recursive hypergraph bisection and random greedy (qxg_plan_contraction)"),
        ("Treewidth", int(round(plan_cost(net, plan)["max_log2"]))),
        ("Trees tried", int(st["trees_tried"])), ("Seed used", seed), ("Hypergraph used", True),
    ])
    metadata["Slicing"] = OrderedDict([
        ("Method used", "greedy: the label of the largest intermediates that minimises modelled time x slices"),
        ("Edges sliced", len(sliced)), ("Log2 largest intermediate after slicing", st["max_log2"]),
        ("Log2 FLOPs over all slices", st["log2_flops_total"]),
    ])
    return groups, plan, metadata
