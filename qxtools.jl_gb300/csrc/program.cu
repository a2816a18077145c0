// Host side of the executor: compiles a `.qx` command list (include/qxgpu.h, qxg_instr) into
// per-step bit maps, plans the device workspace, and runs the programme over batches of
// slices and bitstrings.  This replaces QXContexts.execute's walk (bin/qxrun.jl:83-87) and
// `single_amplitude`'s contract_tn! (src/simulation.jl:86-91).
//
// Execution model.  Tensors that depend on neither the output bitstring nor a slice variable
// ("invariant") are computed once per call; tensors that depend on slice variables only are
// computed once per slice batch; tensors that depend on output tensors are computed once per
// (slice batch, bitstring batch).  Slice and bitstring batches are extra bit fields ("sigma",
// "beta") of the tensors that depend on them, so a batch of slices or bitstrings is one
// larger contraction instead of many small ones.  The saved tensor is summed over the slice
// batch in FP64 and accumulated across slice batches (users_guide.md:11-17).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "../../include/qxgpu.h"
#include "qxgpu_internal.h"
#include "tc_gemm.h"

using namespace qxg;

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}

#define QXG_CUDA(call)                                                                       \
    do {                                                                                     \
        cudaError_t _e = (call);                                                             \
        if (_e != cudaSuccess)                                                               \
            return fail(QXG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e));   \
    } while (0)

int ilog2(int64_t x) {
    int b = 0;
    while ((int64_t(1) << b) < x) b++;
    return b;
}
int64_t pow2ceil(int64_t x) { return int64_t(1) << ilog2(x < 1 ? 1 : x); }

// A physical bit of a tensor: logical axis `axis` bit `j`, or a batch bit.
constexpr int16_t kBeta = -1, kSigma = -2;
struct PBit {
    int16_t axis;
    int16_t j;
    bool operator==(const PBit& o) const { return axis == o.axis && j == o.j; }
};

struct Tensor {
    int kind = 0;                       // QXG_OP_*
    int instr = -1;
    std::vector<int64_t> dims;          // logical dims (views: sliced axis 1)
    std::vector<int64_t> pdims;         // padded to powers of two
    bool beta = false, sigma = false;
    int group = 0;                      // 0 invariant, 1 slice, 2 bitstring
    int data_id = -1;                   // LOAD
    int qubit = -1;                     // OUTPUT
    int view_root = -1;                 // VIEW: LOAD/OUTPUT tensor at the start of the chain
    std::vector<std::pair<int, int>> fixes;   // VIEW: (axis, slice variable)
    bool needed = false;                // read by an ncon or the save
    // per batch plan
    std::vector<PBit> layout;
    int64_t arena_off = -1;
    int slot = -1;                      // exponent slot
};

// Tensors of at most this many bytes get arena space of their own (no reuse within a pass), up
// to kSmallTensorBudget bytes in all; later small tensors share space like the large ones.
constexpr int64_t kSmallTensorBytes = int64_t(256) << 10;
constexpr int64_t kSmallTensorBudget = int64_t(1) << 30;

// Backward (adjoint) step kinds of gradient plans.
constexpr int kBwdNcon = 1, kBwdView = 2, kBwdLeaf = 3;

struct Step {                           // an executable item of a pass
    int kind;                           // QXG_OP_NCON / VIEW / OUTPUT (forward)
    int tensor;                         // tensor produced (table index; adjoints offset by ntensors)
    int bkind = 0;                      // 0 forward, else kBwd*
    int instr = -1;                     // instruction whose command this step serves
    int reads[2] = {-1, -1};            // table indices read (arena lifetimes)
    int64_t goff = 0;                   // leaf-gradient steps: offset in the gradient vector
    StepArgs sargs;
    ViewArgs vargs;
    OutputArgs oargs;
    ViewAdjArgs vaargs;
    LeafGradArgs largs;
    bool use_tc = false;                // tensor-core path (split modes)
    bool use_join = false;              // tensor-core final join (split TF32; tc_join.cu)
    TcJoinArgs join{};                  // its plan (operand pointers bound at launch)
    int batch = -1;                     // batch of small steps it runs in (index in its list's batches)
    bool tc_tuned = false;              // the tile variant has been chosen
    std::string tune_note;              // autotuner: milliseconds per candidate variant
    TcStep tc;                          // tensor-core step description
    double flops = 0, bytes = 0;
};

struct Plan {
    int bc = 0, sc = 0;                 // bitstring / slice batch sizes (powers of two)
    std::vector<Tensor> T;              // tensors with layouts for this plan
    std::vector<Step> steps[3];         // per group, in execution order
    int slot_begin[3], slot_end[3];
    size_t arena_bytes = 0;
    size_t tc_scratch_bytes = 0;
    ReduceArgs red;
    double flops_pass[3] = {0, 0, 0}, bytes_pass[3] = {0, 0, 0};
    // gradient plans: adjoint tensors live at table index ntensors + t
    bool grad = false;
    int ntensors = 0;
    std::vector<Step> bsteps;           // backward steps in execution order
    SeedArgs seed;
    int slot_all_end = 0;               // slots [slot_begin[0], slot_all_end) reset every pass
    double flops_bwd = 0;
    // small CUDA-core steps run in batches (lists 0-2: the groups' steps, 3: the backward steps):
    // each list runs as `order` -- (0, step index) or (1, batch index) -- a topological order by
    // dependency level in which the small steps of one level form one batch
    struct Batch { std::vector<int> members; int first = 0, nblocks = 0; double flops = 0, bytes = 0; };
    std::vector<Batch> batches[4];
    std::vector<std::pair<int, int>> order[4];
    BatchStep* d_batch = nullptr;       // device copies of the batched steps' arguments
    LeafGradArgs* d_leaf = nullptr;     // device copies of the leaf-gradient steps' arguments
    int nleaf = 0;                      // (one launch adds every leaf's gradient)
    ~Plan() {
        if (d_batch) cudaFree(d_batch);
        if (d_leaf) cudaFree(d_leaf);
    }
};

}  // namespace

struct qxg_program {
    qxg_options opts;
    bool fp64 = true;
    int esize = 16;
    int device = 0;
    int sm_count = 148;
    cudaStream_t stream = nullptr;
    int nqubits = 0;
    std::vector<qxg_instr> ins;
    std::vector<int32_t> labels;
    std::vector<std::vector<int64_t>> ddims, dpdims;
    std::vector<void*> d_data;
    std::vector<int> data_m;
    std::vector<bool> data_set;
    std::vector<Tensor> base;           // tensors without batch layouts
    int root = -1;
    std::vector<int64_t> var_dim;
    int64_t nslices = 1;
    double flops_per_amp = 0;
    // batch plans (forward; gradient) and device buffers
    std::unique_ptr<Plan> plan;
    std::unique_ptr<Plan> gplan;
    double* d_grad = nullptr;           // FP64 leaf gradients
    size_t d_grad_cap = 0;
    double* d_ampbar = nullptr;         // adjoint seed per bitstring
    size_t d_ampbar_cap = 0;
    void* d_arena = nullptr;
    size_t arena_cap = 0;
    void* d_scratch = nullptr;
    size_t scratch_cap = 0;
    int* d_exps = nullptr;
    int nslots = 0;
    int* d_tc_err = nullptr;            // code of a tensor-core wait that gave up (0: none)
    PassParams* d_params = nullptr;
    PassParams* h_params = nullptr;     // pinned, one per pass
    size_t h_params_cap = 0;
    char* d_bits = nullptr;
    size_t d_bits_cap = 0;
    double* d_out = nullptr;
    size_t d_out_cap = 0;
    std::vector<int> h_exps_init;
    // tensor-core autotuner: chosen variant per step shape + bit maps, events for timing
    std::map<std::string, TcVariant> tune_cache;
    std::map<std::string, std::string> tune_notes;
    cudaEvent_t tune_ev[2] = {nullptr, nullptr};
    int tuned_steps = 0;                // steps whose variant was picked by timing
    // profiling: CUDA events around launches, aggregated per command on read
    bool profiling = false;
    std::vector<cudaEvent_t> ev_pool;
    size_t ev_used = 0;
    struct Rec { int instr, kind; size_t ev; double flops, bytes; };
    std::vector<Rec> recs;
    int64_t launches = 0;
    // CUDA graphs: one executable graph per pass group, captured on the group's second run
    cudaGraphExec_t gexec[3] = {nullptr, nullptr, nullptr};
    int group_runs[3] = {0, 0, 0};
    int64_t launches_per_group[3] = {0, 0, 0};
    // gradient pass graph: captured on the second pass with the same output, seed and gradient
    // buffers (its kernels' arguments), replayed afterwards
    cudaGraphExec_t grad_exec = nullptr;
    int grad_runs = 0;
    int64_t launches_per_gradpass = 0;
    const void* grad_key[3] = {nullptr, nullptr, nullptr};
    // streams and events of captures with concurrent branches (created on first capture)
    std::vector<cudaStream_t> cap_streams;
    std::vector<cudaEvent_t> cap_ev;
};

namespace {

// ------------------------------------------------------------------------------------------
// structural compile
// ------------------------------------------------------------------------------------------
int compile_structure(qxg_program* P) {
    const int n = (int)P->ins.size();
    int ntensors = 0;
    for (const auto& I : P->ins)
        if (I.op != QXG_OP_SAVE) ntensors = std::max(ntensors, I.dst + 1);
    if (ntensors <= 0) return fail(QXG_ERR_INVALID, "programme defines no tensors");
    P->base.assign(ntensors, Tensor());
    std::vector<bool> defined(ntensors, false);
    std::map<int, int64_t> vdim;
    int nsave = 0;
    auto need_def = [&](int t, int line) -> int {
        if (t < 0 || t >= ntensors || !defined[t])
            return fail(QXG_ERR_INVALID, "instruction " + std::to_string(line) + ": tensor " +
                                             std::to_string(t) + " used before definition");
        return 0;
    };
    for (int i = 0; i < n; i++) {
        const qxg_instr& I = P->ins[i];
        if (I.op != QXG_OP_SAVE) {
            if (I.dst < 0 || I.dst >= ntensors) return fail(QXG_ERR_INVALID, "bad tensor id");
            if (defined[I.dst])
                return fail(QXG_ERR_INVALID, "tensor " + std::to_string(I.dst) + " defined twice");
        }
        Tensor& t = P->base[I.op == QXG_OP_SAVE ? 0 : I.dst];
        switch (I.op) {
        case QXG_OP_LOAD: {
            if (I.a < 0 || I.a >= (int)P->ddims.size()) return fail(QXG_ERR_INVALID, "load: bad data id");
            t.kind = I.op; t.instr = i; t.data_id = I.a;
            t.dims = P->ddims[I.a];
            break;
        }
        case QXG_OP_OUTPUT: {
            if (I.a < 0 || I.a >= P->nqubits) return fail(QXG_ERR_INVALID, "output: qubit out of range");
            if (I.b != 2) return fail(QXG_ERR_UNSUPPORTED, "output: only dimension 2 is supported");
            t.kind = I.op; t.instr = i; t.qubit = I.a; t.dims = {2};
            t.beta = true;
            break;
        }
        case QXG_OP_VIEW: {
            if (int r = need_def(I.a, i)) return r;
            const Tensor& s = P->base[I.a];
            if (s.kind != QXG_OP_LOAD && s.kind != QXG_OP_OUTPUT && s.kind != QXG_OP_VIEW)
                return fail(QXG_ERR_UNSUPPORTED, "view: only leaf, output and view tensors can be viewed");
            if (I.pos < 0 || I.pos >= (int)s.dims.size()) return fail(QXG_ERR_INVALID, "view: rank position out of range");
            if (I.b < 0 || I.b >= kMaxViewFix * 64) return fail(QXG_ERR_INVALID, "view: bad slice variable");
            if (I.dim <= 0 || s.dims[I.pos] != I.dim)
                return fail(QXG_ERR_INVALID, "view: dimension does not match the viewed index");
            auto it = vdim.find(I.b);
            if (it != vdim.end() && it->second != I.dim)
                return fail(QXG_ERR_INVALID, "view: slice variable used with two dimensions");
            vdim[I.b] = I.dim;
            t.kind = I.op; t.instr = i;
            t.dims = s.dims; t.dims[I.pos] = 1;
            t.view_root = s.kind == QXG_OP_VIEW ? s.view_root : I.a;
            t.fixes = s.fixes;
            t.fixes.push_back({I.pos, I.b});
            if ((int)t.fixes.size() > kMaxViewFix) return fail(QXG_ERR_UNSUPPORTED, "view: too many chained views");
            t.beta = s.beta; t.sigma = true;
            break;
        }
        case QXG_OP_NCON: {
            if (int r = need_def(I.a, i)) return r;
            if (int r = need_def(I.b, i)) return r;
            if (I.nc < 0 || I.na < 0 || I.nb < 0 || I.label_off < 0 ||
                (int64_t)I.label_off + I.nc + I.na + I.nb > (int64_t)P->labels.size())
                return fail(QXG_ERR_INVALID, "ncon: label range out of bounds");
            const Tensor& A = P->base[I.a];
            const Tensor& B = P->base[I.b];
            if ((int)A.dims.size() != I.na || (int)B.dims.size() != I.nb)
                return fail(QXG_ERR_INVALID, "ncon " + std::to_string(i) + ": label count does not match operand rank");
            const int32_t* lc = &P->labels[I.label_off];
            const int32_t* la = lc + I.nc;
            const int32_t* lb = la + I.na;
            std::map<int32_t, int64_t> ld;
            for (int q = 0; q < I.na; q++) {
                if (la[q] <= 0) return fail(QXG_ERR_INVALID, "ncon: labels must be positive");
                if (ld.count(la[q])) return fail(QXG_ERR_UNSUPPORTED, "ncon: repeated label within an operand");
                ld[la[q]] = A.dims[q];
            }
            std::map<int32_t, int64_t> lbm;
            for (int q = 0; q < I.nb; q++) {
                if (lb[q] <= 0) return fail(QXG_ERR_INVALID, "ncon: labels must be positive");
                if (lbm.count(lb[q])) return fail(QXG_ERR_UNSUPPORTED, "ncon: repeated label within an operand");
                lbm[lb[q]] = B.dims[q];
                auto it = ld.find(lb[q]);
                if (it != ld.end() && it->second != B.dims[q])
                    return fail(QXG_ERR_INVALID, "ncon " + std::to_string(i) + ": label " + std::to_string(lb[q]) +
                                                     " has different dimensions in the operands");
                ld[lb[q]] = B.dims[q];
            }
            t.kind = I.op; t.instr = i;
            t.dims.clear();
            std::map<int32_t, int> seen;
            for (int q = 0; q < I.nc; q++) {
                auto it = ld.find(lc[q]);
                if (it == ld.end()) return fail(QXG_ERR_INVALID, "ncon: result label not in operands");
                if (seen.count(lc[q])) return fail(QXG_ERR_INVALID, "ncon: repeated result label");
                seen[lc[q]] = q;
                t.dims.push_back(it->second);
            }
            t.beta = A.beta || B.beta;
            t.sigma = A.sigma || B.sigma;
            P->base[I.a].needed = true;
            P->base[I.b].needed = true;
            // algorithmic flops: 8 |C| K over the unsliced dims is accumulated below
            break;
        }
        case QXG_OP_SAVE: {
            if (int r = need_def(I.a, i)) return r;
            P->root = I.a;
            P->base[I.a].needed = true;
            nsave++;
            break;
        }
        default:
            return fail(QXG_ERR_INVALID, "unknown opcode " + std::to_string(I.op));
        }
        if (I.op != QXG_OP_SAVE) defined[I.dst] = true;
    }
    if (nsave != 1) return fail(QXG_ERR_INVALID, "programme must have exactly one save");
    for (auto& t : P->base) {
        t.pdims.clear();
        for (int64_t d : t.dims) t.pdims.push_back(pow2ceil(d));
        t.group = t.beta ? 2 : (t.sigma ? 1 : 0);
        if (t.kind == QXG_OP_VIEW && t.needed) P->base[t.view_root].needed = true;
    }
    // slice variables: dense ids 0..V-1 required
    P->var_dim.clear();
    for (auto& kv : vdim) {
        if (kv.first != (int)P->var_dim.size()) return fail(QXG_ERR_INVALID, "slice variables must be numbered 0..V-1");
        P->var_dim.push_back(kv.second);
    }
    P->nslices = 1;
    for (int64_t d : P->var_dim) {
        if (P->nslices > (int64_t(1) << 40) / d) return fail(QXG_ERR_UNSUPPORTED, "too many slices");
        P->nslices *= d;
    }
    // algorithmic flops per amplitude: each ncon's 8 |C| K with sliced dims at 1, times slices
    double f = 0;
    for (int i = 0; i < n; i++) {
        const qxg_instr& I = P->ins[i];
        if (I.op != QXG_OP_NCON) continue;
        const int32_t* lc = &P->labels[I.label_off];
        const int32_t* la = lc + I.nc;
        const int32_t* lb = la + I.na;
        std::map<int32_t, int64_t> ld;
        for (int q = 0; q < I.na; q++) ld[la[q]] = P->base[I.a].dims[q];
        for (int q = 0; q < I.nb; q++) ld[lb[q]] = P->base[I.b].dims[q];
        double all = 1;
        for (auto& kv : ld) all *= (double)kv.second;
        f += 8.0 * all;
    }
    P->flops_per_amp = f * (double)P->nslices;
    return 0;
}

// ------------------------------------------------------------------------------------------
// batch plan
// ------------------------------------------------------------------------------------------
int bits_of(const Tensor& t, int axis) { return ilog2(t.pdims[axis]); }

BitMap make_map(const std::vector<std::pair<int, int>>& pairs /* (src bit, dst bit) */, int* err) {
    std::vector<std::pair<int, int>> p = pairs;
    std::sort(p.begin(), p.end());
    BitMap m;
    m.n = 0;
    for (size_t i = 0; i < p.size();) {
        size_t j = i + 1;
        while (j < p.size() && p[j].first == p[j - 1].first + 1 && p[j].second == p[j - 1].second + 1) j++;
        if (m.n >= kMaxRuns) { *err = 1; return m; }
        m.r[m.n].src = (uint8_t)p[i].first;
        m.r[m.n].len = (uint8_t)(j - i);
        m.r[m.n].dst = (uint8_t)p[i].second;
        m.r[m.n].pad = 0;
        m.n++;
        i = j;
    }
    return m;
}

int position_of(const Tensor& t, PBit b) {
    for (size_t p = 0; p < t.layout.size(); p++)
        if (t.layout[p] == b) return (int)p;
    return -1;
}

// Bit maps of R = sum X (x) Y (one `ncon`): lr / lx / ly give the label of each logical axis of
// R, X and Y.  A bit of R comes from X and/or Y by label (axis bits) or by identity (slice and
// bitstring batch bits); every operand bit that R lacks is summed.  Summed bits are ordered by
// the larger operand's physical order, then the smaller operand's own.  X and Y become the
// StepArgs' A and B.
int build_maps(const Tensor& R, const int32_t* lr, int nr, const Tensor& X, const int32_t* lx, int nx,
               const Tensor& Y, const int32_t* ly, int ny, StepArgs* s, int* err) {
    auto axis_in = [](const int32_t* ls, int n, int32_t L) {
        for (int q = 0; q < n; q++) if (ls[q] == L) return q;
        return -1;
    };
    auto trans = [&](PBit b, const int32_t* ls, const int32_t* lt, int nt) -> PBit {
        if (b.axis < 0) return b;
        const int ax = axis_in(lt, nt, ls[b.axis]);
        if (ax < 0) return PBit{-3, 0};
        return PBit{(int16_t)ax, b.j};
    };
    std::vector<std::pair<int, int>> cX, cY, kX, kY;
    for (int p = 0; p < (int)R.layout.size(); p++) {
        const PBit b = R.layout[p];
        const int px = position_of(X, trans(b, lr, lx, nx));
        const int py = position_of(Y, trans(b, lr, ly, ny));
        if (px < 0 && py < 0) return fail(QXG_ERR_INVALID, "internal: result bit without source");
        if (px >= 0) cX.push_back({p, px});
        if (py >= 0) cY.push_back({p, py});
    }
    const bool x_big = X.layout.size() >= Y.layout.size();
    const Tensor& Z = x_big ? X : Y;
    const Tensor& W = x_big ? Y : X;
    const int32_t* lz = x_big ? lx : ly;
    const int32_t* lw = x_big ? ly : lx;
    const int nz = x_big ? nx : ny, nw = x_big ? ny : nx;
    std::vector<std::pair<int, int>>& kZ = x_big ? kX : kY;
    std::vector<std::pair<int, int>>& kW = x_big ? kY : kX;
    int kbit = 0;
    for (int p = 0; p < (int)Z.layout.size(); p++) {
        const PBit b = Z.layout[p];
        if (position_of(R, trans(b, lz, lr, nr)) >= 0) continue;
        kZ.push_back({kbit, p});
        const int q = position_of(W, trans(b, lz, lw, nw));
        if (q >= 0) kW.push_back({kbit, q});
        kbit++;
    }
    for (int p = 0; p < (int)W.layout.size(); p++) {
        const PBit b = W.layout[p];
        if (position_of(R, trans(b, lw, lr, nr)) >= 0) continue;
        if (position_of(Z, trans(b, lw, lz, nz)) >= 0) continue;
        kW.push_back({kbit, p});
        kbit++;
    }
    s->nC = int64_t(1) << R.layout.size();
    s->nk = kbit;
    s->cA = make_map(cX, err);
    s->cB = make_map(cY, err);
    s->kA = make_map(kX, err);
    s->kB = make_map(kY, err);
    return 0;
}

// Complex offsets of each `load` command's gradient in the caller's gradient vector (every load,
// in instruction order, -1 for other commands) and the vector's length.
std::vector<int64_t> leaf_offsets(const qxg_program* P, int64_t* total) {
    std::vector<int64_t> off(P->ins.size(), -1);
    int64_t o = 0;
    for (size_t i = 0; i < P->ins.size(); i++) {
        if (P->ins[i].op != QXG_OP_LOAD) continue;
        off[i] = o;
        int64_t n = 1;
        for (int64_t d : P->ddims[P->ins[i].a]) n *= d;
        o += n;
    }
    *total = o;
    return off;
}

// Backward steps of a gradient plan (reverse-mode, Wirtinger derivatives of a real loss L with
// X_bar = dL/d conj X).  For a forward step C = ncon(A, B): A_bar = ncon(C_bar, conj B) and
// B_bar = ncon(conj A, C_bar) -- the same einsum machinery with one operand conjugated; a view's
// adjoint gathers the slice batch back into its leaf; every leaf's adjoint is added to its FP64
// gradient.  Adjoint tensors are table entries ntensors + t with the forward tensor's layout.
// tc_tuning = k >= 1: candidate k-1 of every tensor-core step (the last one where a step has
// fewer), chosen at plan time; 0 leaves the choice to the autotuner.
// The final joins of a split-TF32 programme go to the tensor-core join when they fit it (and the
// options do not keep them on the CUDA cores).
bool join_eligible(const qxg_program* P, Step& st) {
    if (P->fp64 || P->opts.precision != QXG_PREC_SPLIT_TF32 || P->opts.cuda_core_joins) return false;
    return tc_join_plan(st.sargs, P->sm_count, &st.join);
}

// Launch a tensor-core join with the step's current operand pointers and the programme's
// error word and wait controls.
cudaError_t launch_join(const qxg_program* P, const Step& st, int* exps, cudaStream_t s, int* launches) {
    TcJoinArgs g = st.join;
    g.P = static_cast<const float2*>(g.p_is_a ? st.sargs.A : st.sargs.B);
    g.Q = static_cast<const float2*>(g.p_is_a ? st.sargs.B : st.sargs.A);
    g.C = static_cast<float2*>(st.sargs.C);
    g.err = P->d_tc_err;
    g.wait_limit = P->opts.tc_wait_limit > 0 ? (uint32_t)P->opts.tc_wait_limit : 0;
    g.stall = P->opts.tc_stall_test != 0 ? 1 : 0;
    if (g.nsplit > 1 && P->scratch_cap < tc_join_partial_bytes(g)) return cudaErrorInvalidValue;
    return tc_join_launch(g, exps, P->d_scratch, s, launches);
}

void tc_fix_variant(const qxg_program* P, Step& st) {
    // the programme's own timeout word, and the options' test hooks for the bounded waits
    st.tc.err_word = P->d_tc_err;
    st.tc.wait_limit = P->opts.tc_wait_limit > 0 ? (uint32_t)P->opts.tc_wait_limit : 0;
    st.tc.stall_first_cta = P->opts.tc_stall_test != 0;
    if (P->opts.tc_tuning <= 0) return;
    TcVariant cand[kTcMaxVariants];
    const int nc = tc_variants(st.tc, cand);
    tc_set_variant(st.tc, cand[std::min(P->opts.tc_tuning, nc) - 1]);
    st.tc_tuned = true;
}

int build_backward(qxg_program* P, Plan& pl, int* err) {
    auto& T = pl.T;
    const int n = (int)T.size();
    std::vector<int> nreads(n, 0);
    for (int g = 0; g < 3; g++)
        for (auto& st : pl.steps[g])
            for (int r : st.reads) if (r >= 0) nreads[r]++;
    for (int t = 0; t < n; t++)
        if (nreads[t] > 1) return fail(QXG_ERR_UNSUPPORTED, "gradient: tensor " + std::to_string(t) + " is read twice");
    std::vector<char> needs(n, 0);
    for (const qxg_instr& I : P->ins) {
        if (I.op == QXG_OP_SAVE) continue;
        const int t = I.dst;
        if (I.op == QXG_OP_LOAD) needs[t] = 1;
        else if (I.op == QXG_OP_VIEW) needs[t] = T[T[t].view_root].kind == QXG_OP_LOAD;
        else if (I.op == QXG_OP_NCON) needs[t] = needs[I.a] || needs[I.b];
    }
    if (!needs[P->root]) return fail(QXG_ERR_INVALID, "gradient: the saved tensor depends on no leaf");
    T.resize(2 * n);
    int slot = pl.slot_all_end;
    for (int t = 0; t < n; t++) {
        if (!needs[t] || !(T[t].needed || t == P->root)) continue;
        T[n + t] = T[t];
        T[n + t].kind = 0;              // an adjoint: always an arena buffer, never leaf data
        T[n + t].arena_off = -1;
        T[n + t].slot = slot++;
    }
    pl.slot_all_end = slot;
    const double es = P->fp64 ? 16.0 : 8.0;
    auto sz = [&](int t) { return (double)(int64_t(1) << T[t].layout.size()); };
    auto add_ncon = [&](int res, const int32_t* lr, int nr, int x, const int32_t* lx, int nx, int cx, int y,
                        const int32_t* ly, int ny, int cy, int instr) -> int {
        Step st;
        memset(&st.sargs, 0, sizeof(st.sargs));
        st.kind = QXG_OP_NCON;
        st.bkind = kBwdNcon;
        st.tensor = res;
        st.instr = instr;
        st.reads[0] = x;
        st.reads[1] = y;
        if (int r = build_maps(T[res], lr, nr, T[x], lx, nx, T[y], ly, ny, &st.sargs, err)) return r;
        st.sargs.conjA = cx;
        st.sargs.conjB = cy;
        st.sargs.expA = T[x].slot;
        st.sargs.expB = T[y].slot;
        st.sargs.expC = T[res].slot;
        st.flops = 8.0 * (double)st.sargs.nC * (double)(int64_t(1) << st.sargs.nk);
        st.bytes = es * (sz(x) + sz(y) + sz(res));
        st.use_join = join_eligible(P, st);
        if (!st.use_join && !P->fp64 && P->opts.precision != QXG_PREC_FP32 &&
            !contract_prefers_cuda_cores(st.sargs, P->fp64, P->sm_count))
            st.use_tc = tc_plan_step(st.sargs, T[x].layout.size(), T[y].layout.size(), T[res].layout.size(),
                                     P->opts.precision == QXG_PREC_SPLIT_TF32, &st.tc,
                                     (double)P->opts.tc_plane_budget_mb * (1 << 20));
        if (st.use_tc) tc_fix_variant(P, st);
        pl.flops_bwd += st.flops;
        pl.bsteps.push_back(st);
        return 0;
    };
    for (int g = 2; g >= 0; g--) {
        for (auto it = pl.steps[g].rbegin(); it != pl.steps[g].rend(); ++it) {
            const Step& f = *it;
            const int t = f.tensor;
            if (!needs[t]) continue;
            const qxg_instr& I = P->ins[f.instr];
            if (f.kind == QXG_OP_NCON) {
                const int32_t* lc = &P->labels[I.label_off];
                const int32_t* la = lc + I.nc;
                const int32_t* lb = la + I.na;
                if (needs[I.a])
                    if (int r = add_ncon(n + I.a, la, I.na, n + t, lc, I.nc, 0, I.b, lb, I.nb, 1, f.instr)) return r;
                if (needs[I.b])
                    if (int r = add_ncon(n + I.b, lb, I.nb, I.a, la, I.na, 1, n + t, lc, I.nc, 0, f.instr)) return r;
            } else if (f.kind == QXG_OP_VIEW) {
                const int r = T[t].view_root;
                const Tensor& S = T[r];
                const Tensor& V = T[t];
                Step st;
                memset(&st.vaargs, 0, sizeof(st.vaargs));
                st.kind = QXG_OP_VIEW;
                st.bkind = kBwdView;
                st.tensor = n + r;
                st.instr = f.instr;
                st.reads[0] = n + t;
                ViewAdjArgs& va = st.vaargs;
                std::vector<std::pair<int, int>> pairs;
                for (int p = 0; p < (int)S.layout.size(); p++) {
                    const PBit b = S.layout[p];
                    bool fixed = false;
                    for (auto& fx : V.fixes) if (fx.first == b.axis) fixed = true;
                    if (fixed) continue;
                    const int q = position_of(V, b);
                    if (q < 0) return fail(QXG_ERR_INVALID, "internal: view adjoint layout");
                    pairs.push_back({p, q});
                }
                va.s2v = make_map(pairs, err);
                va.sigma_shift = f.vargs.sigma_shift;
                va.nsigma = pl.sc;
                va.ns = int64_t(1) << S.layout.size();
                va.nfix = f.vargs.nfix;
                for (int k = 0; k < va.nfix; k++) {
                    va.fix_shift[k] = f.vargs.fix_shift[k];
                    va.fix_bits[k] = bits_of(S, V.fixes[k].first);
                    va.var_stride[k] = f.vargs.var_stride[k];
                    va.var_dim[k] = f.vargs.var_dim[k];
                }
                va.exp_v = T[n + t].slot;
                va.exp_s = T[n + r].slot;
                pl.bsteps.push_back(st);
            }
        }
    }
    // leaf gradients in instruction order (the gradient pointer is bound with the buffers)
    int64_t total = 0;
    const std::vector<int64_t> goff = leaf_offsets(P, &total);
    for (size_t ii = 0; ii < P->ins.size(); ii++) {
        const qxg_instr& I = P->ins[ii];
        if (I.op != QXG_OP_LOAD || T[n + I.dst].slot < 0 || !needs[I.dst] || !T[I.dst].needed) continue;
        const Tensor& L = T[I.dst];
        if ((int)L.dims.size() > 16) return fail(QXG_ERR_UNSUPPORTED, "gradient: leaf of rank above 16");
        Step st;
        memset(&st.largs, 0, sizeof(st.largs));
        st.kind = QXG_OP_LOAD;
        st.bkind = kBwdLeaf;
        st.tensor = -1;
        st.instr = (int)ii;
        st.reads[0] = n + I.dst;
        LeafGradArgs& la = st.largs;
        la.rank = (int)L.dims.size();
        la.n = 1;
        for (int d = 0; d < la.rank; d++) {
            la.dims[d] = (int32_t)L.dims[d];
            la.pdims[d] = (int32_t)L.pdims[d];
            la.n *= L.dims[d];
        }
        st.goff = goff[ii];             // complex offset in the gradient vector, bound at launch
        la.exp_s = T[n + I.dst].slot;
        pl.bsteps.push_back(st);
    }
    return 0;
}

// Scratch a tensor-core step may use: any candidate variant when the autotuner is on.
size_t tc_scratch_need(const qxg_program* P, const Step& st) {
    return P->opts.tc_tuning == 0 && !st.tc_tuned ? st.tc.scratch_max : st.tc.scratch_bytes;
}

int build_plan(qxg_program* P, int bc, int sc, std::unique_ptr<Plan>& out, bool grad = false) {
    auto plan = std::make_unique<Plan>();
    plan->bc = bc;
    plan->sc = sc;
    plan->T = P->base;
    auto& T = plan->T;
    const int nbb = ilog2(bc), nsb = ilog2(sc);
    const int ntensors = (int)T.size();
    int err = 0;
    // layouts in instruction order
    for (const auto& I : P->ins) {
        if (I.op == QXG_OP_SAVE) continue;
        Tensor& t = T[I.dst];
        t.layout.clear();
        if (I.op == QXG_OP_LOAD) {
            for (int a = 0; a < (int)t.pdims.size(); a++)
                for (int j = 0; j < bits_of(t, a); j++) t.layout.push_back({(int16_t)a, (int16_t)j});
        } else if (I.op == QXG_OP_OUTPUT) {
            t.layout.push_back({0, 0});
            for (int j = 0; j < nbb; j++) t.layout.push_back({kBeta, (int16_t)j});
        } else if (I.op == QXG_OP_VIEW) {
            const Tensor& r = T[t.view_root];
            for (const PBit& b : r.layout) {
                bool fixed = false;
                if (b.axis >= 0)
                    for (auto& f : t.fixes) if (f.first == b.axis) fixed = true;
                if (!fixed) t.layout.push_back(b);
            }
            for (int j = 0; j < nsb; j++) t.layout.push_back({kSigma, (int16_t)j});
        } else if (I.op == QXG_OP_NCON) {
            const Tensor& A = T[I.a];
            const Tensor& B = T[I.b];
            const int32_t* lc = &P->labels[I.label_off];
            const int32_t* la = lc + I.nc;
            const int32_t* lb = la + I.na;
            auto axis_in = [](const int32_t* ls, int n, int32_t L) {
                for (int q = 0; q < n; q++) if (ls[q] == L) return q;
                return -1;
            };
            // translate an operand bit into the result's bit (or mark K with axis -3)
            auto to_c = [&](const int32_t* ls, PBit b) -> PBit {
                if (b.axis < 0) return b;
                const int ca = axis_in(lc, I.nc, ls[b.axis]);
                if (ca < 0) return {-3, 0};
                return {(int16_t)ca, b.j};
            };
            const bool a_big = A.layout.size() >= B.layout.size();
            const Tensor& X = a_big ? A : B;
            const Tensor& Y = a_big ? B : A;
            const int32_t* lx = a_big ? la : lb;
            const int32_t* ly = a_big ? lb : la;
            std::vector<PBit> from_x;
            for (const PBit& b : X.layout) { PBit c = to_c(lx, b); if (c.axis != -3) from_x.push_back(c); }
            // C follows X's bit order, and the free bits new from Y take the places of the summed
            // bits.  In the Complex64 modes the batch bits (slice and bitstring) go on top, X's
            // first: every batch value of every intermediate is then one contiguous block, which
            // keeps the final joins -- the steps where both operands carry the batch -- reading
            // whole sectors and pages instead of pieces strided by the batch.  The FP64 kernels
            // (compute-bound on the FP64 pipe) run faster with the batch bits where the summed bits
            // were, so FP64 programmes keep them there.
            const bool fp64 = P->fp64;
            auto is_batch = [fp64](const PBit& b) { return !fp64 && (b.axis == kBeta || b.axis == kSigma); };
            std::vector<PBit> fresh, fresh_batch, top;
            for (const PBit& b : Y.layout) {
                PBit c = to_c(ly, b);
                if (c.axis == -3) continue;
                if (std::find(from_x.begin(), from_x.end(), c) == from_x.end())
                    (is_batch(c) ? fresh_batch : fresh).push_back(c);
            }
            size_t fi = 0;
            for (const PBit& b : X.layout) {
                PBit c = to_c(lx, b);
                if (c.axis == -3) {
                    if (fi < fresh.size()) t.layout.push_back(fresh[fi++]);
                } else if (is_batch(c)) {
                    top.push_back(c);
                } else {
                    t.layout.push_back(c);
                }
            }
            while (fi < fresh.size()) t.layout.push_back(fresh[fi++]);
            for (const PBit& b : top) t.layout.push_back(b);
            for (const PBit& b : fresh_batch) t.layout.push_back(b);
        }
        if (t.layout.size() > 46) return fail(QXG_ERR_UNSUPPORTED, "tensor with more than 2^46 elements");
    }
    // steps, groups and exponent slots
    // leaves first (their slots are set once per call), then one contiguous range per group
    // (reset before every pass of that group)
    int slot = 0;
    for (int i = 0; i < ntensors; i++)
        if (T[i].kind == QXG_OP_LOAD) T[i].slot = slot++;
    for (int g = 0; g < 3; g++) {
        plan->slot_begin[g] = slot;
        for (int i = 0; i < ntensors; i++)
            if (T[i].group == g && T[i].kind != QXG_OP_LOAD) T[i].slot = slot++;
        plan->slot_end[g] = slot;
    }
    for (int ii = 0; ii < (int)P->ins.size(); ii++) {
        const qxg_instr& I = P->ins[ii];
        if (I.op == QXG_OP_SAVE || I.op == QXG_OP_LOAD) continue;
        Tensor& t = T[I.dst];
        if (!t.needed) continue;
        Step st;
        memset(&st.sargs, 0, sizeof(st.sargs));
        memset(&st.vargs, 0, sizeof(st.vargs));
        memset(&st.oargs, 0, sizeof(st.oargs));
        st.kind = I.op;
        st.tensor = I.dst;
        st.instr = ii;
        if (I.op == QXG_OP_NCON) { st.reads[0] = I.a; st.reads[1] = I.b; }
        if (I.op == QXG_OP_VIEW) st.reads[0] = t.view_root;
        if (I.op == QXG_OP_OUTPUT) {
            st.oargs.qubit = t.qubit;
            st.oargs.nqubits = P->nqubits;
            st.oargs.nbeta = bc;
            st.oargs.exp_dst = t.slot;
        } else if (I.op == QXG_OP_VIEW) {
            const Tensor& r = T[t.view_root];
            std::vector<std::pair<int, int>> pairs;
            int sig = 0;
            for (int p = 0; p < (int)t.layout.size(); p++) {
                if (t.layout[p].axis == kSigma) { sig++; continue; }
                const int q = position_of(r, t.layout[p]);
                if (q < 0) return fail(QXG_ERR_INVALID, "internal: view layout");
                pairs.push_back({p, q});
            }
            st.vargs.sigma_shift = (int)t.layout.size() - sig;
            st.vargs.map = make_map(pairs, &err);
            st.vargs.n = int64_t(1) << t.layout.size();
            st.vargs.nfix = (int)t.fixes.size();
            for (int f = 0; f < st.vargs.nfix; f++) {
                const int ax = t.fixes[f].first, var = t.fixes[f].second;
                st.vargs.fix_shift[f] = position_of(r, PBit{(int16_t)ax, 0});
                if (st.vargs.fix_shift[f] < 0) return fail(QXG_ERR_INVALID, "internal: view fix");
                int64_t stride = 1;
                for (int v = 0; v < var; v++) stride *= P->var_dim[v];
                st.vargs.var_stride[f] = stride;
                st.vargs.var_dim[f] = P->var_dim[var];
                for (int j = 1; j < bits_of(r, ax); j++)
                    if (position_of(r, PBit{(int16_t)ax, (int16_t)j}) != st.vargs.fix_shift[f] + j)
                        return fail(QXG_ERR_INVALID, "internal: viewed axis bits not contiguous");
            }
            st.vargs.exp_src = T[t.view_root].slot;
            st.vargs.exp_dst = t.slot;
        } else {  // NCON
            const Tensor& A = T[I.a];
            const Tensor& B = T[I.b];
            const int32_t* lc = &P->labels[I.label_off];
            const int32_t* la = lc + I.nc;
            const int32_t* lb = la + I.na;
            if (int r = build_maps(t, lc, I.nc, A, la, I.na, B, lb, I.nb, &st.sargs, &err)) return r;
            const int kbit = st.sargs.nk;
            st.sargs.expA = A.slot;
            st.sargs.expB = B.slot;
            st.sargs.expC = t.slot;
            const double s = P->fp64 ? 16.0 : 8.0;
            st.flops = 8.0 * (double)st.sargs.nC * (double)(int64_t(1) << kbit);
            st.bytes = s * ((double)(int64_t(1) << A.layout.size()) + (double)(int64_t(1) << B.layout.size()) +
                            (double)st.sargs.nC);
            st.use_join = join_eligible(P, st);
            if (!st.use_join && !P->fp64 && P->opts.precision != QXG_PREC_FP32 &&
                !contract_prefers_cuda_cores(st.sargs, P->fp64, P->sm_count))
                st.use_tc = tc_plan_step(st.sargs, A.layout.size(), B.layout.size(), t.layout.size(),
                                         P->opts.precision == QXG_PREC_SPLIT_TF32, &st.tc,
                                         (double)P->opts.tc_plane_budget_mb * (1 << 20));
            if (st.use_tc) tc_fix_variant(P, st);
        }
        if (err) return fail(QXG_ERR_UNSUPPORTED, "bit map needs more than the supported number of runs");
        plan->flops_pass[t.group] += st.flops;
        plan->bytes_pass[t.group] += st.bytes;
        plan->steps[t.group].push_back(st);
    }
    plan->ntensors = ntensors;
    plan->slot_all_end = slot;
    if (grad) {
        if (int r = build_backward(P, *plan, &err)) return r;
        if (err) return fail(QXG_ERR_UNSUPPORTED, "adjoint bit map needs more than the supported number of runs");
    }
    // arena: lifetimes over the execution sequence group0, group1, group2 (then, in gradient
    // plans, the backward steps; every group runs in every gradient pass)
    const int ntab = (int)T.size();
    struct Item { int tensor; int def; int last; int64_t bytes; };
    std::vector<int> pos_of(ntab, -1);
    int pos = 0;
    for (int g = 0; g < 3; g++)
        for (auto& st : plan->steps[g]) pos_of[st.tensor] = pos++;
    const int fwd_end = pos;
    for (auto& st : plan->bsteps)
        if (st.bkind != kBwdLeaf) { if (pos_of[st.tensor] < 0) pos_of[st.tensor] = pos; pos++; }
        else pos++;
    if (grad) pos_of[ntensors + P->root] = fwd_end;          // the seed, written before the backward
    const int end_pos = pos + 1;
    std::vector<int> last(ntab, -1);
    auto use = [&](int t, int at) {
        if (t < 0 || pos_of[t] < 0) return;
        last[t] = std::max(last[t], at);
        if (grad) return;
        // used by a later group -> alive until the end (the later group repeats)
        const int gt = T[t].group;
        int gat = 0;
        int acc = 0;
        for (int g = 0; g < 3; g++) { acc += (int)plan->steps[g].size(); if (at < acc) { gat = g; break; } }
        if (gat > gt) last[t] = end_pos;
    };
    pos = 0;
    for (int g = 0; g < 3; g++)
        for (auto& st : plan->steps[g]) { use(st.reads[0], pos); use(st.reads[1], pos); pos++; }
    if (grad) use(P->root, fwd_end);
    for (auto& st : plan->bsteps) { use(st.reads[0], pos); use(st.reads[1], pos); pos++; }
    if (!grad && pos_of[P->root] >= 0) last[P->root] = end_pos;
    std::vector<Item> items;
    int64_t small_total = 0;
    for (int t = 0; t < ntab; t++) {
        if (pos_of[t] < 0) continue;
        const int64_t bytes = ((int64_t(1) << T[t].layout.size()) * (int64_t)P->esize + 255) & ~int64_t(255);
        // small tensors keep their own bytes for the whole pass: reusing them would order
        // independent sub-trees one after another (a write after another branch's read) and keep
        // their small steps out of each other's batches and graph branches
        if (bytes <= kSmallTensorBytes && small_total + bytes <= kSmallTensorBudget) {
            small_total += bytes;
            items.push_back({t, 0, end_pos, bytes});
        } else {
            items.push_back({t, pos_of[t], std::max(last[t], pos_of[t]), bytes});
        }
    }
    std::vector<int> order(items.size());
    for (size_t i = 0; i < items.size(); i++) order[i] = (int)i;
    std::sort(order.begin(), order.end(), [&](int x, int y) {
        if (items[x].bytes != items[y].bytes) return items[x].bytes > items[y].bytes;
        return items[x].def < items[y].def;
    });
    struct Placed { int64_t off, bytes; int def, last; };
    std::vector<Placed> placed;
    int64_t total = 0;
    for (int oi : order) {
        const Item& it = items[oi];
        std::vector<std::pair<int64_t, int64_t>> busy;
        for (auto& p : placed)
            if (!(p.last < it.def || it.last < p.def)) busy.push_back({p.off, p.off + p.bytes});
        std::sort(busy.begin(), busy.end());
        int64_t off = 0;
        for (auto& b : busy) {
            if (off + it.bytes <= b.first) break;
            off = std::max(off, b.second);
        }
        placed.push_back({off, it.bytes, it.def, it.last});
        T[it.tensor].arena_off = off;
        total = std::max(total, off + it.bytes);
    }
    plan->arena_bytes = (size_t)total;
    size_t scratch = 0;
    for (int g = 0; g < 3; g++)
        for (auto& st : plan->steps[g]) if (st.use_tc) scratch = std::max(scratch, tc_scratch_need(P, st));
    for (auto& st : plan->bsteps) if (st.use_tc) scratch = std::max(scratch, tc_scratch_need(P, st));
    // FP64 partials of tensor-core joins with several K ranges per batch value
    for (int g = 0; g < 3; g++)
        for (auto& st : plan->steps[g]) if (st.use_join) scratch = std::max(scratch, tc_join_partial_bytes(st.join));
    for (auto& st : plan->bsteps) if (st.use_join) scratch = std::max(scratch, tc_join_partial_bytes(st.join));
    // split-K partials of CUDA-core steps with few results and a long sum share the scratch
    for (int g = 0; g < 3; g++)
        for (auto& st : plan->steps[g])
            if (st.kind == QXG_OP_NCON && !st.use_tc && !st.use_join)
                scratch = std::max(scratch, contract_scratch_bytes(st.sargs, P->fp64, P->sm_count));
    for (auto& st : plan->bsteps)
        if (st.bkind == kBwdNcon && !st.use_tc && !st.use_join)
            scratch = std::max(scratch, contract_scratch_bytes(st.sargs, P->fp64, P->sm_count));
    plan->tc_scratch_bytes = scratch;
    // reduction of the root
    {
        const Tensor& r = T[P->root];
        ReduceArgs& ra = plan->red;
        memset(&ra, 0, sizeof(ra));
        ra.naxes = (int)r.dims.size();
        if (ra.naxes > kMaxOutAxes) return fail(QXG_ERR_UNSUPPORTED, "saved tensor has too many axes");
        int64_t osz = 1;
        for (int a = 0; a < ra.naxes; a++) {
            ra.axis_dim[a] = (int32_t)r.dims[a];
            ra.axis_nbits[a] = bits_of(r, a);
            if (ra.axis_nbits[a] > 3) return fail(QXG_ERR_UNSUPPORTED, "saved tensor axis wider than 8");
            for (int j = 0; j < ra.axis_nbits[a]; j++) {
                ra.axis_bitpos[a][j] = position_of(r, PBit{(int16_t)a, (int16_t)j});
                if (ra.axis_bitpos[a][j] < 0) return fail(QXG_ERR_INVALID, "internal: root layout");
            }
            osz *= r.dims[a];
        }
        ra.out_size = osz;
        std::vector<std::pair<int, int>> bm, sm;
        for (int p = 0; p < (int)r.layout.size(); p++) {
            if (r.layout[p].axis == kBeta) bm.push_back({r.layout[p].j, p});
            if (r.layout[p].axis == kSigma) sm.push_back({r.layout[p].j, p});
        }
        ra.beta_map = make_map(bm, &err);
        ra.sigma_map = make_map(sm, &err);
        ra.nbeta = r.beta ? bc : 1;
        ra.nsigma = r.sigma ? sc : 1;
        ra.broadcast = r.beta ? 0 : 1;
        ra.exp_root = r.slot;
        if (err) return fail(QXG_ERR_UNSUPPORTED, "root bit map too fragmented");
        if (grad) {
            SeedArgs& sd = plan->seed;
            memset(&sd, 0, sizeof(sd));
            sd.out_size = ra.out_size;
            sd.nbeta = ra.nbeta;
            sd.nsigma = ra.nsigma;
            sd.beta_map = ra.beta_map;
            sd.sigma_map = ra.sigma_map;
            sd.naxes = ra.naxes;
            for (int a = 0; a < ra.naxes; a++) {
                sd.axis_dim[a] = ra.axis_dim[a];
                sd.axis_nbits[a] = ra.axis_nbits[a];
                for (int j = 0; j < 3; j++) sd.axis_bitpos[a][j] = ra.axis_bitpos[a][j];
            }
            sd.exp_root = ra.exp_root;
            sd.exp_dst = T[ntensors + P->root].slot;
        }
    }
    plan->grad = grad;
    out = std::move(plan);
    return 0;
}

void drop_graphs(qxg_program* P);
void drop_grad_graph(qxg_program* P);
int plan_batches(qxg_program* P, Plan& pl);

// Choose batch sizes whose workspace fits the limit, (re)build the forward plan (grad = false)
// or the gradient plan (grad = true), grow the shared device buffers and bind pointers.  Both
// plans use the same arena and scratch: growing either drops the other plan (its bound pointers
// are stale) and the captured graphs.
int ensure_plan(qxg_program* P, int nbits_call, bool grad = false) {
    std::unique_ptr<Plan>& slot = grad ? P->gplan : P->plan;
    const int64_t want_b = std::max<int64_t>(1, pow2ceil(nbits_call));
    const int64_t max_b = P->opts.max_bitstring_batch > 0 ? pow2ceil(P->opts.max_bitstring_batch) : 256;
    const int64_t max_s = P->opts.max_slice_batch > 0 ? pow2ceil(P->opts.max_slice_batch) : 1024;
    int64_t bc = std::min(want_b, max_b);
    int64_t sc = std::min(pow2ceil(P->nslices), max_s);
    bool has_out = false;
    for (auto& t : P->base) if (t.kind == QXG_OP_OUTPUT && t.needed) has_out = true;
    if (!has_out) bc = 1;
    if (slot && slot->bc == bc && slot->sc == sc) return 0;
    size_t limit = (size_t)P->opts.workspace_limit;
    if (limit == 0) {
        size_t fr = 0, tot = 0;
        QXG_CUDA(cudaMemGetInfo(&fr, &tot));
        limit = fr / 4 * 3 + P->arena_cap + P->scratch_cap;
    }
    while (true) {
        std::unique_ptr<Plan> pl;
        if (int r = build_plan(P, (int)bc, (int)sc, pl, grad)) return r;
        if (pl->arena_bytes + pl->tc_scratch_bytes <= limit) {
            if (P->stream) cudaStreamSynchronize(P->stream);
            if (!grad) drop_graphs(P);
            else drop_grad_graph(P);
            slot = std::move(pl);
            break;
        }
        if (sc == 1 && bc == 1)
            return fail(QXG_ERR_OOM, "workspace of " + std::to_string(pl->arena_bytes) +
                                         " bytes for one slice and one bitstring exceeds the limit");
        if (sc >= bc && sc > 1) sc /= 2; else bc /= 2;
    }
    Plan& pl = *slot;
    std::unique_ptr<Plan>& other = grad ? P->plan : P->gplan;
    if (pl.arena_bytes > P->arena_cap) {
        if (P->d_arena) cudaFree(P->d_arena);
        P->d_arena = nullptr; P->arena_cap = 0;
        QXG_CUDA(cudaMalloc(&P->d_arena, std::max<size_t>(pl.arena_bytes, 256)));
        P->arena_cap = pl.arena_bytes;
        other.reset();
        drop_graphs(P);
    }
    if (pl.tc_scratch_bytes > P->scratch_cap) {
        if (P->d_scratch) cudaFree(P->d_scratch);
        P->d_scratch = nullptr; P->scratch_cap = 0;
        QXG_CUDA(cudaMalloc(&P->d_scratch, pl.tc_scratch_bytes));
        P->scratch_cap = pl.tc_scratch_bytes;
        other.reset();
        drop_graphs(P);
    }
    const int ns = std::max(pl.slot_end[2], pl.slot_all_end);
    if (ns > P->nslots) {
        if (P->d_exps) cudaFree(P->d_exps);
        P->d_exps = nullptr;
        QXG_CUDA(cudaMalloc(&P->d_exps, sizeof(int) * 2 * std::max(ns, 1)));
        P->nslots = ns;
    }
    // bind pointers
    char* arena = static_cast<char*>(P->d_arena);
    auto ptr = [&](int t) -> void* {
        const Tensor& x = pl.T[t];
        if (x.kind == QXG_OP_LOAD) return P->d_data[x.data_id];
        return arena + x.arena_off;
    };
    for (int g = 0; g < 3; g++)
        for (auto& st : pl.steps[g]) {
            const Tensor& t = pl.T[st.tensor];
            const qxg_instr& I = P->ins[t.instr];
            if (st.kind == QXG_OP_NCON) {
                st.sargs.A = ptr(I.a); st.sargs.B = ptr(I.b); st.sargs.C = ptr(st.tensor);
            } else if (st.kind == QXG_OP_VIEW) {
                st.vargs.src = ptr(t.view_root); st.vargs.dst = ptr(st.tensor); st.vargs.params = P->d_params;
            } else {
                st.oargs.dst = ptr(st.tensor); st.oargs.params = P->d_params;
            }
        }
    pl.red.root = ptr(P->root);
    pl.red.params = P->d_params;
    if (grad) {
        const int n = pl.ntensors;
        for (auto& st : pl.bsteps) {
            if (st.bkind == kBwdNcon) {
                st.sargs.A = ptr(st.reads[0]); st.sargs.B = ptr(st.reads[1]); st.sargs.C = ptr(st.tensor);
            } else if (st.bkind == kBwdView) {
                st.vaargs.vbar = ptr(st.reads[0]); st.vaargs.sbar = ptr(st.tensor); st.vaargs.params = P->d_params;
            } else {
                st.largs.sbar = ptr(st.reads[0]);
            }
        }
        pl.seed.dst = ptr(n + P->root);
        pl.seed.root = ptr(P->root);
        pl.seed.params = P->d_params;
    }
    // initial exponent slots: LOAD tensors carry their data's maximum exponent
    P->h_exps_init.assign(2 * std::max(ns, 1), 0);
    for (auto& t : pl.T) {
        if (t.slot < 0) continue;
        P->h_exps_init[2 * t.slot] = 0;
        P->h_exps_init[2 * t.slot + 1] = t.kind == QXG_OP_LOAD ? P->data_m[t.data_id] : kExpUnset;
    }
    return plan_batches(P, pl);
}

// Event pair around one launch when profiling; returns the index of the first event.
int prof_begin(qxg_program* P, size_t* ev) {
    if (!P->profiling) return 0;
    while (P->ev_pool.size() < P->ev_used + 2) {
        cudaEvent_t e;
        QXG_CUDA(cudaEventCreate(&e));
        P->ev_pool.push_back(e);
    }
    *ev = P->ev_used;
    P->ev_used += 2;
    QXG_CUDA(cudaEventRecord(P->ev_pool[*ev], P->stream));
    return 0;
}

int prof_end(qxg_program* P, size_t ev, int instr, int kind, double flops, double bytes) {
    P->launches++;
    if (!P->profiling) return 0;
    QXG_CUDA(cudaEventRecord(P->ev_pool[ev + 1], P->stream));
    P->recs.push_back({instr, kind, ev, flops, bytes});
    return 0;
}

int run_group_eager(qxg_program* P, int g, Plan* plp = nullptr);

// Autotuner: the first time a tensor-core step runs (its operands are in place), time each
// candidate variant (fused X gather or X planes; N tiles of 16/32/64) on the step itself, twice
// each, and keep the fastest of the second runs.  Re-running a step is harmless: it overwrites
// its result and re-raises the same exponent slot, which is cleared before every candidate.
// Identical steps (shape and bit maps) share the choice.  Not done under stream capture, and
// the tuning launches are not counted as pass launches.
int tune_tc_step(qxg_program* P, Step& st, int* exps) {
    if (st.tc_tuned) return 0;
    st.tc_tuned = true;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    QXG_CUDA(cudaStreamIsCapturing(P->stream, &cs));
    if (cs != cudaStreamCaptureStatusNone) return 0;
    const std::string key = tc_key(st.tc);
    auto it = P->tune_cache.find(key);
    if (it != P->tune_cache.end()) {
        tc_set_variant(st.tc, it->second);
        st.tune_note = P->tune_notes[key];
        return 0;
    }
    TcVariant cand[kTcMaxVariants];
    const int nc = tc_variants(st.tc, cand);
    TcVariant best = cand[0];
    if (nc > 1) {
        for (auto& e : P->tune_ev)
            if (!e) QXG_CUDA(cudaEventCreate(&e));
        float best_ms = 0.f;
        bool have = false;
        int* cslot = exps + 2 * st.sargs.expC + 1;
        for (int i = 0; i < nc; i++) {
            tc_set_variant(st.tc, cand[i]);
            if (st.tc.scratch_bytes > P->scratch_cap) continue;
            float ms = 0.f;
            for (int rep = 0; rep < 2; rep++) {
                QXG_CUDA(cudaMemsetAsync(cslot, 0x80, sizeof(int), P->stream));   // kExpUnset
                QXG_CUDA(cudaEventRecord(P->tune_ev[0], P->stream));
                QXG_CUDA(tc_run_step(st.tc, st.sargs, exps, P->d_scratch, P->stream, P->sm_count, nullptr));
                QXG_CUDA(cudaEventRecord(P->tune_ev[1], P->stream));
            }
            QXG_CUDA(cudaEventSynchronize(P->tune_ev[1]));
            QXG_CUDA(cudaEventElapsedTime(&ms, P->tune_ev[0], P->tune_ev[1]));
            if (!have || ms < best_ms) { best_ms = ms; best = cand[i]; have = true; }
            char note[64];
            snprintf(note, sizeof(note), "%s%s%d:%.3fms", st.tune_note.empty() ? "" : ",",
                     cand[i].fused ? (cand[i].tma ? "tma" : (cand[i].tmem ? "tmem" : (cand[i].bulk ? "bulk" : "rows")))
                                   : "planes",
                     cand[i].ntile, ms);
            st.tune_note += note;
        }
        QXG_CUDA(cudaMemsetAsync(cslot, 0x80, sizeof(int), P->stream));
        P->tuned_steps++;
    }
    tc_set_variant(st.tc, best);
    P->tune_cache[key] = best;
    P->tune_notes[key] = st.tune_note;
    return 0;
}

void drop_grad_graph(qxg_program* P) {
    if (P->grad_exec) cudaGraphExecDestroy(P->grad_exec);
    P->grad_exec = nullptr;
    P->grad_runs = 0;
}

void drop_graphs(qxg_program* P) {
    for (int g = 0; g < 3; g++) {
        if (P->gexec[g]) cudaGraphExecDestroy(P->gexec[g]);
        P->gexec[g] = nullptr;
        P->group_runs[g] = 0;
    }
    drop_grad_graph(P);
}

// One pass group: eager launches, or (with use_graphs, outside profiling) a CUDA graph captured
// from the group's second run and replayed afterwards.  Kernel arguments are fixed per plan (the
// arena, leaves, bitstring buffer and pass-parameter block do not move), so the graph stays valid
// until the plan changes.
int run_group(qxg_program* P, int g) {
    Plan& pl = *P->plan;
    if (pl.steps[g].empty()) return 0;
    const bool graphs = P->opts.use_graphs && !P->profiling;
    if (!graphs || P->group_runs[g] < 1) {
        const int64_t before = P->launches;
        if (int r = run_group_eager(P, g)) return r;
        P->launches_per_group[g] = P->launches - before;
        P->group_runs[g]++;
        return 0;
    }
    if (!P->gexec[g]) {
        cudaGraph_t graph = nullptr;
        QXG_CUDA(cudaStreamBeginCapture(P->stream, cudaStreamCaptureModeThreadLocal));
        const int64_t before = P->launches;
        const int r = run_group_eager(P, g);
        const cudaError_t e = cudaStreamEndCapture(P->stream, &graph);
        P->launches = before;
        if (r) { if (graph) cudaGraphDestroy(graph); return r; }
        if (e != cudaSuccess) return fail(QXG_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
        const cudaError_t ei = cudaGraphInstantiate(&P->gexec[g], graph, 0);
        cudaGraphDestroy(graph);
        if (ei != cudaSuccess) {
            P->gexec[g] = nullptr;
            return fail(QXG_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ei));
        }
    }
    QXG_CUDA(cudaGraphLaunch(P->gexec[g], P->stream));
    P->launches += P->launches_per_group[g];
    P->group_runs[g]++;
    return 0;
}

// ---- launches with their dependencies ------------------------------------------------------
// Under stream capture a pass becomes a graph whose edges are the launches' true dependencies
// instead of one chain.  Each unit of work names the device ranges it reads and writes (arena
// bytes of its tensors, the shared scratch, its span of the gradient vector, the amplitude
// output); work j follows work i < j when one of them writes what the other touches.  The
// independent sub-trees of the contraction tree (the many small gate-absorption steps, whose
// kernels fill a fraction of the GPU) then run side by side.  Eager runs, and profiling, keep
// one stream and the plan's order.
struct Span { int space; int64_t lo, hi; };
constexpr int kSpanArena = 0, kSpanScratch = 1, kSpanGrad = 2, kSpanOut = 3;
constexpr int kCaptureStreams = 8;

struct Work {
    std::function<int(cudaStream_t)> launch;
    std::vector<Span> rd, wr;
};

bool spans_meet(const std::vector<Span>& a, const std::vector<Span>& b) {
    for (const Span& x : a)
        for (const Span& y : b)
            if (x.space == y.space && x.lo < y.hi && y.lo < x.hi) return true;
    return false;
}

void add_tensor_span(const qxg_program* P, const Plan& pl, int t, std::vector<Span>& out) {
    if (t < 0 || pl.T[t].arena_off < 0) return;          // leaves live outside the arena, read-only
    const int64_t bytes = ((int64_t(1) << pl.T[t].layout.size()) * (int64_t)P->esize + 255) & ~int64_t(255);
    out.push_back({kSpanArena, pl.T[t].arena_off, pl.T[t].arena_off + bytes});
}

bool step_uses_scratch(const qxg_program* P, const Step& st) {
    if (st.kind != QXG_OP_NCON) return false;
    if (st.use_join) return tc_join_partial_bytes(st.join) > 0;
    return st.use_tc || contract_scratch_bytes(st.sargs, P->fp64, P->sm_count) > 0;
}

void add_step_spans(const qxg_program* P, const Plan& pl, const Step& st, Work& w) {
    add_tensor_span(P, pl, st.reads[0], w.rd);
    add_tensor_span(P, pl, st.reads[1], w.rd);
    add_tensor_span(P, pl, st.tensor, w.wr);
    if (step_uses_scratch(P, st)) w.wr.push_back({kSpanScratch, 0, 1});
    if (st.bkind == kBwdLeaf) w.wr.push_back({kSpanGrad, st.goff, st.goff + st.largs.n});
}

int launch_works(qxg_program* P, std::vector<Work>& w) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    QXG_CUDA(cudaStreamIsCapturing(P->stream, &cs));
    const int n = (int)w.size();
    if (cs != cudaStreamCaptureStatusActive || n < 2) {
        for (auto& x : w)
            if (int r = x.launch(P->stream)) return r;
        return 0;
    }
    // direct dependencies, less those implied through another dependency (ancestor bit sets)
    const int words = (n + 63) / 64;
    std::vector<uint64_t> anc((size_t)n * words, 0), cover(words);
    std::vector<std::vector<int>> deps(n);
    std::vector<int> cand;
    for (int j = 0; j < n; j++) {
        cand.clear();
        for (int i = 0; i < j; i++)
            if (spans_meet(w[j].wr, w[i].rd) || spans_meet(w[j].wr, w[i].wr) || spans_meet(w[j].rd, w[i].wr))
                cand.push_back(i);
        std::fill(cover.begin(), cover.end(), 0);
        for (int i : cand)
            for (int q = 0; q < words; q++) cover[q] |= anc[(size_t)i * words + q];
        uint64_t* aj = &anc[(size_t)j * words];
        for (int q = 0; q < words; q++) aj[q] = cover[q];
        for (int i : cand) {
            if (!((cover[i / 64] >> (i % 64)) & 1)) deps[j].push_back(i);
            aj[i / 64] |= uint64_t(1) << (i % 64);
        }
    }
    while ((int)P->cap_streams.size() < kCaptureStreams) {
        cudaStream_t s;
        QXG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        P->cap_streams.push_back(s);
    }
    while ((int)P->cap_ev.size() < n + 1 + kCaptureStreams) {
        cudaEvent_t e;
        QXG_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        P->cap_ev.push_back(e);
    }
    // stream 0 is the capturing stream; the others fork from it and join it at the end
    cudaStream_t streams[kCaptureStreams];
    streams[0] = P->stream;
    for (int s = 1; s < kCaptureStreams; s++) streams[s] = P->cap_streams[s];
    cudaEvent_t fork = P->cap_ev[n];
    QXG_CUDA(cudaEventRecord(fork, P->stream));
    int last[kCaptureStreams];
    bool joined[kCaptureStreams];
    for (int s = 0; s < kCaptureStreams; s++) { last[s] = -1; joined[s] = s == 0; }
    std::vector<int> on(n, 0);
    for (int j = 0; j < n; j++) {
        int s = -1;
        for (int i : deps[j])                           // continue the chain of a dependency
            if (last[on[i]] == i && (s < 0 || i > last[s])) s = on[i];
        if (s < 0) {                                    // else the stream idle the longest
            s = 0;
            for (int q = 1; q < kCaptureStreams; q++) if (last[q] < last[s]) s = q;
        }
        if (!joined[s]) {
            QXG_CUDA(cudaStreamWaitEvent(streams[s], fork, 0));
            joined[s] = true;
        }
        for (int i : deps[j])
            if (on[i] != s) QXG_CUDA(cudaStreamWaitEvent(streams[s], P->cap_ev[i], 0));
        if (int r = w[j].launch(streams[s])) return r;
        QXG_CUDA(cudaEventRecord(P->cap_ev[j], streams[s]));
        on[j] = s;
        last[s] = j;
    }
    for (int s = 1; s < kCaptureStreams; s++) {
        if (!joined[s]) continue;
        cudaEvent_t e = P->cap_ev[n + s];
        QXG_CUDA(cudaEventRecord(e, streams[s]));
        QXG_CUDA(cudaStreamWaitEvent(P->stream, e, 0));
    }
    return 0;
}

// The launches of one forward step on stream `s` (profiled in eager runs, where s is the
// programme's stream).
int launch_fwd_step(qxg_program* P, Plan& pl, Step& st, int* exps, cudaStream_t s) {
    const int instr = pl.T[st.tensor].instr;
    if (st.use_tc)
        if (int r = tune_tc_step(P, st, exps)) return r;
    size_t ev = 0;
    if (int r = prof_begin(P, &ev)) return r;
    int kind;
    if (st.kind == QXG_OP_NCON) {
        if (st.use_tc && st.tc.nouter > 0) {
            // outer N blocks: pack and GEMM per block under one record
            kind = QXG_KERNEL_CONTRACT_TC;
            int nl = 0;
            QXG_CUDA(tc_run_step(st.tc, st.sargs, exps, P->d_scratch, s, P->sm_count, &nl));
            P->launches += nl - 1;
        } else if (st.use_tc) {
            // pack both operands (its own record), then the tensor-core GEMM
            QXG_CUDA(tc_run_pack(st.tc, st.sargs, exps, P->d_scratch, s, P->sm_count));
            const double pack_bytes = (double)P->esize *
                    (double)((int64_t(1) << pl.T[P->ins[instr].a].layout.size()) +
                             (int64_t(1) << pl.T[P->ins[instr].b].layout.size())) +
                (double)st.tc.scratch_bytes;
            if (int r = prof_end(P, ev, instr, QXG_KERNEL_TC_PACK, 0.0, pack_bytes)) return r;
            if (!st.tc.fused) P->launches++;             // X and Y both packed
            if (int r = prof_begin(P, &ev)) return r;
            kind = QXG_KERNEL_CONTRACT_TC;
            QXG_CUDA(tc_run_gemm(st.tc, st.sargs, exps, P->d_scratch, s, P->sm_count));
            if (st.tc.ks > 0) P->launches++;            // the split-K sum
        } else if (st.use_join) {
            kind = QXG_KERNEL_CONTRACT_TC;
            int nl = 1;
            QXG_CUDA(launch_join(P, st, exps, s, &nl));
            P->launches += nl - 1;
        } else {
            kind = P->fp64 ? QXG_KERNEL_CONTRACT_FP64 : QXG_KERNEL_CONTRACT_FP32;
            int nl = 1;
            QXG_CUDA(launch_contract(st.sargs, P->fp64, exps, s, P->sm_count, P->d_scratch, P->scratch_cap, &nl));
            P->launches += nl - 1;
        }
    } else if (st.kind == QXG_OP_VIEW) {
        kind = QXG_KERNEL_VIEW;
        QXG_CUDA(launch_view(st.vargs, P->fp64, exps, s));
    } else {
        kind = QXG_KERNEL_OUTPUT;
        st.oargs.bitstrings = P->d_bits;
        QXG_CUDA(launch_output(st.oargs, P->fp64, exps, s));
    }
    return prof_end(P, ev, instr, kind, st.flops, st.bytes);
}

// A step small enough to share a launch: a CUDA-core contraction (forward or adjoint) with at
// most kBatchMaxResults results, K <= kBatchMaxK and no scratch.
bool step_small(const qxg_program* P, const Step& st) {
    if (st.kind != QXG_OP_NCON || st.use_tc || st.use_join) return false;
    if (st.bkind != 0 && st.bkind != kBwdNcon) return false;
    if (st.sargs.nC > kBatchMaxResults || (int64_t(1) << st.sargs.nk) > kBatchMaxK) return false;
    return contract_scratch_bytes(st.sargs, P->fp64, P->sm_count) == 0;
}

// Order each step list by dependency level (a step's level is one above the highest level of the
// earlier steps it conflicts with: it reads what they write, or writes what they touch) and
// gather the small steps of each level into one batch; upload the batched steps' arguments.
// Called after the plan's pointers are bound.
int plan_batches(qxg_program* P, Plan& pl) {
    std::vector<BatchStep> host;
    for (int L = 0; L < 4; L++) {
        std::vector<Step>& steps = L < 3 ? pl.steps[L] : pl.bsteps;
        pl.batches[L].clear();
        pl.order[L].clear();
        const int n = (int)steps.size();
        std::vector<Work> sp(n);
        for (int j = 0; j < n; j++) {
            steps[j].batch = -1;
            add_step_spans(P, pl, steps[j], sp[j]);
        }
        std::vector<int> level(n, 0);
        int top = 0;
        for (int j = 0; j < n; j++) {
            for (int i = 0; i < j; i++)
                if (level[i] + 1 > level[j] &&
                    (spans_meet(sp[j].wr, sp[i].rd) || spans_meet(sp[j].wr, sp[i].wr) || spans_meet(sp[j].rd, sp[i].wr)))
                    level[j] = level[i] + 1;
            top = std::max(top, level[j]);
        }
        std::vector<std::vector<int>> at(top + 1);
        // the leaf gradients are the list's last steps (their adjoints live to its end): one
        // launch after every other step, not one per leaf
        for (int j = 0; j < n; j++)
            if (steps[j].bkind != kBwdLeaf) at[level[j]].push_back(j);
        for (auto& lv : at) {
            std::vector<int> small;
            for (int j : lv)
                if (step_small(P, steps[j])) small.push_back(j);
            for (int j : lv)
                if (small.size() < 2 || !step_small(P, steps[j])) pl.order[L].push_back({0, j});
            if (small.size() < 2) continue;
            Plan::Batch b;
            b.first = (int)host.size();
            for (int j : small) {
                BatchStep d;
                d.a = steps[j].sargs;
                if (contract_x_is_b(d.a, P->fp64)) {       // same factor order as the step's own kernel
                    std::swap(d.a.A, d.a.B);
                    std::swap(d.a.cA, d.a.cB);
                    std::swap(d.a.kA, d.a.kB);
                    std::swap(d.a.conjA, d.a.conjB);
                    std::swap(d.a.expA, d.a.expB);
                }
                d.first_block = b.nblocks;
                d.nblocks = (int)((steps[j].sargs.nC + kBatchResults - 1) / kBatchResults);
                b.nblocks += d.nblocks;
                b.flops += steps[j].flops;
                b.bytes += steps[j].bytes;
                steps[j].batch = (int)pl.batches[L].size();
                b.members.push_back(j);
                host.push_back(d);
            }
            pl.order[L].push_back({1, (int)pl.batches[L].size()});
            pl.batches[L].push_back(std::move(b));
        }
    }
    if (pl.d_batch) cudaFree(pl.d_batch);
    pl.d_batch = nullptr;
    if (!host.empty()) {
        QXG_CUDA(cudaMalloc(&pl.d_batch, sizeof(BatchStep) * host.size()));
        QXG_CUDA(cudaMemcpy(pl.d_batch, host.data(), sizeof(BatchStep) * host.size(), cudaMemcpyHostToDevice));
    }
    std::vector<LeafGradArgs> leaves;
    for (const Step& st : pl.bsteps)
        if (st.bkind == kBwdLeaf) {
            LeafGradArgs la = st.largs;
            la.goff = st.goff;
            leaves.push_back(la);
        }
    if (pl.d_leaf) cudaFree(pl.d_leaf);
    pl.d_leaf = nullptr;
    pl.nleaf = (int)leaves.size();
    if (!leaves.empty()) {
        QXG_CUDA(cudaMalloc(&pl.d_leaf, sizeof(LeafGradArgs) * leaves.size()));
        QXG_CUDA(cudaMemcpy(pl.d_leaf, leaves.data(), sizeof(LeafGradArgs) * leaves.size(), cudaMemcpyHostToDevice));
    }
    return 0;
}

int launch_batch_work(qxg_program* P, Plan& pl, int L, int b, int* exps, cudaStream_t s) {
    const Plan::Batch& bt = pl.batches[L][b];
    size_t ev = 0;
    if (int r = prof_begin(P, &ev)) return r;
    QXG_CUDA(launch_batch(pl.d_batch + bt.first, (int)bt.members.size(), bt.nblocks, P->fp64, exps, s));
    return prof_end(P, ev, -2, QXG_KERNEL_CONTRACT_BATCH, bt.flops, bt.bytes);
}

// The works of step list L in its batched order; `one` launches a single step of the list.
void append_list_works(qxg_program* P, Plan& pl, int L, int* exps, std::vector<Work>& w,
                       const std::function<int(Step&, cudaStream_t)>& one) {
    std::vector<Step>& steps = L < 3 ? pl.steps[L] : pl.bsteps;
    for (const auto& it : pl.order[L]) {
        Work x;
        if (it.first == 0) {
            Step* sp = &steps[it.second];
            x.launch = [one, sp](cudaStream_t s) { return one(*sp, s); };
            add_step_spans(P, pl, *sp, x);
        } else {
            Plan* pp = &pl;
            const int b = it.second;
            x.launch = [P, pp, L, b, exps](cudaStream_t s) { return launch_batch_work(P, *pp, L, b, exps, s); };
            for (int j : pl.batches[L][b].members) add_step_spans(P, pl, steps[j], x);
        }
        w.push_back(std::move(x));
    }
}

void append_group_works(qxg_program* P, Plan& pl, int g, int* exps, std::vector<Work>& w) {
    Plan* pp = &pl;
    append_list_works(P, pl, g, exps, w,
                      [P, pp, exps](Step& st, cudaStream_t s) { return launch_fwd_step(P, *pp, st, exps, s); });
}

int run_group_eager(qxg_program* P, int g, Plan* plp) {
    Plan& pl = plp ? *plp : *P->plan;
    int* exps = P->fp64 ? nullptr : P->d_exps;
    if (exps) {
        QXG_CUDA(launch_reset_exps(exps, pl.slot_begin[g], pl.slot_end[g], P->stream));
        P->launches++;
    }
    std::vector<Work> w;
    append_group_works(P, pl, g, exps, w);
    return launch_works(P, w);
}

int run_reduce(qxg_program* P, Plan* plp = nullptr) {
    Plan& pl = plp ? *plp : *P->plan;
    size_t ev = 0;
    if (int r = prof_begin(P, &ev)) return r;
    QXG_CUDA(launch_reduce(pl.red, P->fp64, P->fp64 ? nullptr : P->d_exps, P->stream));
    return prof_end(P, ev, -1, QXG_KERNEL_REDUCE, 0.0, 0.0);
}

int set_params(qxg_program* P, size_t k, const PassParams& pp) {
    P->h_params[k] = pp;
    QXG_CUDA(cudaMemcpyAsync(P->d_params, &P->h_params[k], sizeof(PassParams), cudaMemcpyHostToDevice, P->stream));
    return 0;
}

int run_passes(qxg_program* P, int nbits, int64_t s0, int64_t s1, double* d_out) {
    Plan& pl = *P->plan;
    const Tensor& root = pl.T[P->root];
    const int64_t nsl = s1 - s0;
    const int64_t nsc = (nsl + pl.sc - 1) / pl.sc;
    const int64_t nbc = root.beta ? (nbits + pl.bc - 1) / pl.bc : 1;
    const size_t npass = (size_t)(1 + nsc * (1 + nbc));
    // the pinned pass parameters of a previous asynchronous call may still be in flight
    QXG_CUDA(cudaStreamSynchronize(P->stream));
    if (npass > P->h_params_cap) {
        if (P->h_params) { cudaStreamSynchronize(P->stream); cudaFreeHost(P->h_params); }
        P->h_params = nullptr;
        QXG_CUDA(cudaMallocHost(&P->h_params, sizeof(PassParams) * npass));
        P->h_params_cap = npass;
    }
    QXG_CUDA(cudaMemcpyAsync(P->d_exps, P->h_exps_init.data(), sizeof(int) * P->h_exps_init.size(),
                             cudaMemcpyHostToDevice, P->stream));
    size_t k = 0;
    PassParams pp;
    memset(&pp, 0, sizeof(pp));
    pp.num_slices = P->nslices;
    pp.slice_base = s0;
    pp.slices_valid = (int32_t)std::min<int64_t>(pl.sc, nsl);
    pp.bits_valid = root.beta ? std::min(pl.bc, nbits) : nbits;
    if (int r = set_params(P, k++, pp)) return r;
    if (int r = run_group(P, 0)) return r;
    pl.red.out = d_out;
    for (int64_t c = 0; c < nsc; c++) {
        pp.slice_base = s0 + c * pl.sc;
        pp.slices_valid = (int32_t)std::min<int64_t>(pl.sc, s1 - pp.slice_base);
        pp.bit_base = 0;
        pp.bits_valid = root.beta ? std::min(pl.bc, nbits) : nbits;
        if (int r = set_params(P, k++, pp)) return r;
        if (int r = run_group(P, 1)) return r;
        if (!root.beta && root.group <= 1) {
            if (int r = run_reduce(P)) return r;
            continue;
        }
        for (int64_t b = 0; b < nbc; b++) {
            pp.bit_base = (int32_t)(b * pl.bc);
            pp.bits_valid = root.beta ? (int32_t)std::min<int64_t>(pl.bc, nbits - pp.bit_base) : nbits;
            if (int r = set_params(P, k++, pp)) return r;
            if (int r = run_group(P, 2)) return r;
            if (int r = run_reduce(P)) return r;
        }
    }
    return 0;
}

// Gradient passes.  Every (slice batch, bitstring batch) runs all forward groups (the shared
// sub-trees are recomputed per pass instead of stored across passes), optionally adds its slice
// sum to the amplitudes, seeds the root's adjoint and runs the backward steps; leaf adjoints are
// added into the FP64 gradient, so the gradient is the sum over passes (the loss's seed is linear).
int run_grad_passes(qxg_program* P, int nbits, int64_t s0, int64_t s1, double* d_out, const double* d_ampbar,
                    double* d_grad) {
    Plan& pl = *P->gplan;
    const Tensor& root = pl.T[P->root];
    const int64_t nsl = s1 - s0;
    const int64_t nsc = (nsl + pl.sc - 1) / pl.sc;
    const int64_t nbc = root.beta ? (nbits + pl.bc - 1) / pl.bc : 1;
    if (!d_ampbar && nsc > 1)
        return fail(QXG_ERR_UNSUPPORTED, "gradient of sum |amplitude|^2 needs the slice range in one pass "
                                         "(raise max_slice_batch or pass amp_bar)");
    if (!root.beta && nbits != 1)
        return fail(QXG_ERR_UNSUPPORTED, "gradient: the saved tensor does not depend on the bitstring; pass one");
    const size_t npass = (size_t)(nsc * nbc);
    QXG_CUDA(cudaStreamSynchronize(P->stream));
    if (npass > P->h_params_cap) {
        if (P->h_params) cudaFreeHost(P->h_params);
        P->h_params = nullptr;
        QXG_CUDA(cudaMallocHost(&P->h_params, sizeof(PassParams) * npass));
        P->h_params_cap = npass;
    }
    QXG_CUDA(cudaMemcpyAsync(P->d_exps, P->h_exps_init.data(), sizeof(int) * P->h_exps_init.size(),
                             cudaMemcpyHostToDevice, P->stream));
    int* exps = P->fp64 ? nullptr : P->d_exps;
    pl.red.out = d_out;
    pl.seed.amp_bar = d_ampbar;
    const int n = pl.ntensors;
    const size_t seed_bytes = (size_t)P->esize << pl.T[n + P->root].layout.size();
    // one pass: forward recomputation, seed, adjoint steps (kernel arguments: the plan's buffers
    // and d_out / d_ampbar / d_grad)
    auto bwd_step = [&](Step& st, cudaStream_t s) -> int {
        if (st.use_tc)
            if (int r = tune_tc_step(P, st, exps)) return r;
        size_t ev = 0;
        if (int r = prof_begin(P, &ev)) return r;
        int kind = QXG_KERNEL_REDUCE;
        if (st.bkind == kBwdNcon) {
            if (st.use_tc) {
                int nl = 0;
                QXG_CUDA(tc_run_step(st.tc, st.sargs, exps, P->d_scratch, s, P->sm_count, &nl));
                P->launches += nl - 1;
                kind = QXG_KERNEL_CONTRACT_TC;
            } else if (st.use_join) {
                int nl = 1;
                QXG_CUDA(launch_join(P, st, exps, s, &nl));
                P->launches += nl - 1;
                kind = QXG_KERNEL_CONTRACT_TC;
            } else {
                int nl = 1;
                QXG_CUDA(launch_contract(st.sargs, P->fp64, exps, s, P->sm_count, P->d_scratch, P->scratch_cap, &nl));
                P->launches += nl - 1;
                kind = P->fp64 ? QXG_KERNEL_CONTRACT_FP64 : QXG_KERNEL_CONTRACT_FP32;
            }
        } else if (st.bkind == kBwdView) {
            QXG_CUDA(launch_view_adjoint(st.vaargs, P->fp64, exps, s));
            kind = QXG_KERNEL_VIEW;
        } else {
            LeafGradArgs la = st.largs;
            la.grad = d_grad + 2 * st.goff;
            QXG_CUDA(launch_leaf_grad(la, P->fp64, exps, s));
        }
        return prof_end(P, ev, st.instr, kind, st.flops, st.bytes);
    };
    auto body = [&]() -> int {
        if (exps) {
            QXG_CUDA(launch_reset_exps(exps, pl.slot_begin[0], pl.slot_all_end, P->stream));
            P->launches++;
        }
        std::vector<Work> w;
        for (int g = 0; g < 3; g++) append_group_works(P, pl, g, exps, w);
        if (d_out) {
            Work x;
            x.launch = [&](cudaStream_t s) -> int {
                size_t ev = 0;
                if (int r = prof_begin(P, &ev)) return r;
                QXG_CUDA(launch_reduce(pl.red, P->fp64, exps, s));
                return prof_end(P, ev, -1, QXG_KERNEL_REDUCE, 0.0, 0.0);
            };
            add_tensor_span(P, pl, P->root, x.rd);
            x.wr.push_back({kSpanOut, 0, 1});
            w.push_back(std::move(x));
        }
        {
            Work x;
            x.launch = [&](cudaStream_t s) -> int {
                QXG_CUDA(cudaMemsetAsync(pl.seed.dst, 0, seed_bytes, s));
                QXG_CUDA(launch_seed(pl.seed, P->fp64, exps, s));
                P->launches++;
                return 0;
            };
            add_tensor_span(P, pl, P->root, x.rd);
            add_tensor_span(P, pl, n + P->root, x.wr);
            w.push_back(std::move(x));
        }
        append_list_works(P, pl, 3, exps, w, [&bwd_step](Step& st, cudaStream_t s) { return bwd_step(st, s); });
        if (pl.nleaf > 0) {
            Work x;
            x.launch = [&](cudaStream_t s) -> int {
                size_t ev = 0;
                if (int r = prof_begin(P, &ev)) return r;
                QXG_CUDA(launch_leaf_grads(pl.d_leaf, pl.nleaf, d_grad, P->fp64, exps, s));
                return prof_end(P, ev, -1, QXG_KERNEL_REDUCE, 0.0, 0.0);
            };
            for (const Step& st : pl.bsteps)
                if (st.bkind == kBwdLeaf) add_step_spans(P, pl, st, x);
            w.push_back(std::move(x));
        }
        return launch_works(P, w);
    };
    // with use_graphs (outside profiling) the pass is captured on its second run with the same
    // buffers and replayed for every later pass
    const bool graphs = P->opts.use_graphs && !P->profiling;
    const void* key[3] = {d_out, d_ampbar, d_grad};
    if (graphs && (key[0] != P->grad_key[0] || key[1] != P->grad_key[1] || key[2] != P->grad_key[2])) {
        drop_grad_graph(P);
        for (int i = 0; i < 3; i++) P->grad_key[i] = key[i];
    }
    size_t k = 0;
    PassParams pp;
    memset(&pp, 0, sizeof(pp));
    pp.num_slices = P->nslices;
    for (int64_t c = 0; c < nsc; c++) {
        for (int64_t b = 0; b < nbc; b++) {
            pp.slice_base = s0 + c * pl.sc;
            pp.slices_valid = (int32_t)std::min<int64_t>(pl.sc, s1 - pp.slice_base);
            pp.bit_base = (int32_t)(b * pl.bc);
            pp.bits_valid = root.beta ? (int32_t)std::min<int64_t>(pl.bc, nbits - pp.bit_base) : nbits;
            if (int r = set_params(P, k++, pp)) return r;
            if (!graphs || P->grad_runs < 1) {
                const int64_t before = P->launches;
                if (int r = body()) return r;
                P->launches_per_gradpass = P->launches - before;
                P->grad_runs++;
                continue;
            }
            if (!P->grad_exec) {
                cudaGraph_t graph = nullptr;
                QXG_CUDA(cudaStreamBeginCapture(P->stream, cudaStreamCaptureModeThreadLocal));
                const int64_t before = P->launches;
                const int r = body();
                const cudaError_t e = cudaStreamEndCapture(P->stream, &graph);
                P->launches = before;
                if (r) { if (graph) cudaGraphDestroy(graph); return r; }
                if (e != cudaSuccess) return fail(QXG_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
                const cudaError_t ei = cudaGraphInstantiate(&P->grad_exec, graph, 0);
                cudaGraphDestroy(graph);
                if (ei != cudaSuccess) {
                    P->grad_exec = nullptr;
                    return fail(QXG_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ei));
                }
            }
            QXG_CUDA(cudaGraphLaunch(P->grad_exec, P->stream));
            P->launches += P->launches_per_gradpass;
            P->grad_runs++;
        }
    }
    return 0;
}

// Grow the programme's bitstring buffer; captured graphs hold its address, so a new buffer
// drops them.
int ensure_bits(qxg_program* P, size_t nb) {
    if (nb <= P->d_bits_cap) return 0;
    QXG_CUDA(cudaStreamSynchronize(P->stream));
    drop_graphs(P);
    if (P->d_bits) cudaFree(P->d_bits);
    P->d_bits = nullptr;
    P->d_bits_cap = 0;
    QXG_CUDA(cudaMalloc(&P->d_bits, nb));
    P->d_bits_cap = nb;
    return 0;
}

// A tensor-core kernel whose bounded wait gave up leaves a code in a device word; read and clear.
int check_tc_plan(qxg_program* P, const Plan* pl) {
    if (!pl) return 0;
    bool any = false;
    for (int g = 0; g < 3; g++) for (auto& st : pl->steps[g]) any = any || st.use_tc || st.use_join;
    for (auto& st : pl->bsteps) any = any || st.use_tc || st.use_join;
    if (!any) return 0;
    int code = 0;
    QXG_CUDA(tc_read_error(&code, P->d_tc_err, P->stream));
    if (code) return fail(QXG_ERR_TIMEOUT, "a tensor-core kernel gave up waiting (code " + std::to_string(code) + ")");
    return 0;
}

int check_tc(qxg_program* P) { return check_tc_plan(P, P->plan.get()); }

int check_ready(qxg_program* P) {
    for (size_t i = 0; i < P->data_set.size(); i++) {
        bool used = false;
        for (auto& t : P->base) if (t.kind == QXG_OP_LOAD && t.data_id == (int)i && t.needed) used = true;
        if (used && !P->data_set[i]) return fail(QXG_ERR_STATE, "leaf data " + std::to_string(i) + " not set");
    }
    return 0;
}

int validate_bits(const char* bits, int64_t n) {
    for (int64_t i = 0; i < n; i++) {
        const char c = bits[i];
        if (c != '0' && c != '1' && c != '+' && c != '-')
            return fail(QXG_ERR_INVALID, "bitstring character outside '01+-' at position " + std::to_string(i));
    }
    return 0;
}

}  // namespace

namespace qxg {
int ncon_fail(int code, const char* msg) { return fail(code, msg); }
}  // namespace qxg

extern "C" {

const char* qxg_last_error(void) { return g_last_error.c_str(); }

const char* qxg_version(void) { return "qxgpu 0.1.0 sm_103a"; }

int qxg_program_create(const qxg_instr* instrs, int32_t ninstr, const int32_t* labels, int64_t nlabels,
                       const int32_t* data_rank, const int64_t* data_dims, int32_t ndata, int32_t nqubits,
                       const qxg_options* opts, qxg_program** out) {
    g_last_error.clear();
    if (!out) return fail(QXG_ERR_INVALID, "out is NULL");
    *out = nullptr;
    if (!instrs || ninstr <= 0 || (nlabels > 0 && !labels) || ndata < 0 || (ndata > 0 && (!data_rank || !data_dims)) ||
        nqubits < 0)
        return fail(QXG_ERR_INVALID, "bad arguments");
    auto P = std::make_unique<qxg_program>();
    memset(&P->opts, 0, sizeof(P->opts));
    if (opts) P->opts = *opts;
    if (P->opts.precision < QXG_PREC_FP64 || P->opts.precision > QXG_PREC_FP32)
        return fail(QXG_ERR_INVALID, "unknown precision");
    P->fp64 = P->opts.precision == QXG_PREC_FP64;
    P->esize = P->fp64 ? 16 : 8;
    P->device = P->opts.device;
    P->nqubits = nqubits;
    P->ins.assign(instrs, instrs + ninstr);
    if (nlabels > 0) P->labels.assign(labels, labels + nlabels);
    int64_t off = 0;
    for (int d = 0; d < ndata; d++) {
        if (data_rank[d] < 0 || data_rank[d] > 64) return fail(QXG_ERR_INVALID, "bad data rank");
        std::vector<int64_t> dims(data_dims + off, data_dims + off + data_rank[d]);
        std::vector<int64_t> pd;
        for (int64_t x : dims) {
            if (x <= 0 || x > (1 << 20)) return fail(QXG_ERR_INVALID, "bad data dimension");
            pd.push_back(pow2ceil(x));
        }
        P->ddims.push_back(dims);
        P->dpdims.push_back(pd);
        off += data_rank[d];
    }
    if (int r = compile_structure(P.get())) return r;
    int ndev = 0;
    QXG_CUDA(cudaGetDeviceCount(&ndev));
    if (P->device < 0 || P->device >= ndev) return fail(QXG_ERR_INVALID, "device ordinal out of range");
    QXG_CUDA(cudaSetDevice(P->device));
    QXG_CUDA(cudaDeviceGetAttribute(&P->sm_count, cudaDevAttrMultiProcessorCount, P->device));
    QXG_CUDA(cudaStreamCreateWithFlags(&P->stream, cudaStreamNonBlocking));
    QXG_CUDA(cudaMalloc(&P->d_params, sizeof(PassParams)));
    QXG_CUDA(cudaMalloc(&P->d_tc_err, sizeof(int)));
    QXG_CUDA(cudaMemset(P->d_tc_err, 0, sizeof(int)));
    P->d_data.assign(ndata, nullptr);
    P->data_m.assign(ndata, 0);
    P->data_set.assign(ndata, false);
    for (int d = 0; d < ndata; d++) {
        int64_t n = 1;
        for (int64_t x : P->dpdims[d]) n *= x;
        QXG_CUDA(cudaMalloc(&P->d_data[d], (size_t)std::max<int64_t>(n, 1) * P->esize));
    }
    *out = P.release();
    return QXG_OK;
}

int qxg_program_set_data(qxg_program* P, int32_t id, const double* re_im, int64_t nelem) {
    g_last_error.clear();
    if (!P || !re_im || id < 0 || id >= (int)P->ddims.size()) return fail(QXG_ERR_INVALID, "bad arguments");
    const auto& dims = P->ddims[id];
    const auto& pd = P->dpdims[id];
    int64_t n = 1, pn = 1;
    for (int64_t x : dims) n *= x;
    for (int64_t x : pd) pn *= x;
    if (nelem != n) return fail(QXG_ERR_INVALID, "leaf data size does not match its dimensions");
    QXG_CUDA(cudaSetDevice(P->device));
    std::vector<double> padded((size_t)std::max<int64_t>(pn, 1) * 2, 0.0);
    const int r = (int)dims.size();
    std::vector<int64_t> idx(r, 0);
    for (int64_t e = 0; e < n; e++) {
        int64_t po = 0, st = 1;
        for (int a = 0; a < r; a++) { po += idx[a] * st; st *= pd[a]; }
        padded[2 * po] = re_im[2 * e];
        padded[2 * po + 1] = re_im[2 * e + 1];
        for (int a = 0; a < r; a++) { if (++idx[a] < dims[a]) break; idx[a] = 0; }
    }
    if (P->fp64) {
        QXG_CUDA(cudaMemcpy(P->d_data[id], padded.data(), sizeof(double) * padded.size(), cudaMemcpyHostToDevice));
        P->data_m[id] = 0;
    } else {
        std::vector<float> f(padded.size());
        int m = kExpUnset;
        for (size_t i = 0; i < padded.size(); i++) {
            f[i] = (float)padded[i];
            if (f[i] != 0.f) { int e; std::frexp(std::fabs(f[i]), &e); m = std::max(m, e); }
        }
        P->data_m[id] = m;
        QXG_CUDA(cudaMemcpy(P->d_data[id], f.data(), sizeof(float) * f.size(), cudaMemcpyHostToDevice));
    }
    P->data_set[id] = true;
    return QXG_OK;
}

int qxg_amplitudes_device(qxg_program* P, const char* d_bitstrings, int32_t nbits, int64_t s0, int64_t s1,
                          double* d_out) {
    g_last_error.clear();
    if (!P || nbits <= 0 || (P->nqubits > 0 && !d_bitstrings) || !d_out) return fail(QXG_ERR_INVALID, "bad arguments");
    if (s0 < 0 || s1 > P->nslices || s0 >= s1) return fail(QXG_ERR_INVALID, "slice range out of bounds");
    if (int r = check_ready(P)) return r;
    QXG_CUDA(cudaSetDevice(P->device));
    if (int r = ensure_plan(P, nbits)) return r;
    const int64_t osz = P->plan->red.out_size;
    // bitstrings are copied into the programme's own buffer, whose address captured passes keep
    if (int r = ensure_bits(P, (size_t)nbits * (size_t)std::max(P->nqubits, 1))) return r;
    if (P->nqubits > 0)
        QXG_CUDA(cudaMemcpyAsync(P->d_bits, d_bitstrings, (size_t)nbits * P->nqubits, cudaMemcpyDeviceToDevice,
                                 P->stream));
    QXG_CUDA(cudaMemsetAsync(d_out, 0, sizeof(double) * 2 * (size_t)osz * nbits, P->stream));
    return run_passes(P, nbits, s0, s1, d_out);
}

int qxg_amplitudes(qxg_program* P, const char* bits, int32_t nbits, int64_t s0, int64_t s1, double* out) {
    g_last_error.clear();
    if (!P || nbits <= 0 || (P->nqubits > 0 && !bits) || !out) return fail(QXG_ERR_INVALID, "bad arguments");
    if (s0 < 0 || s1 > P->nslices || s0 >= s1) return fail(QXG_ERR_INVALID, "slice range out of bounds");
    if (int r = validate_bits(bits, (int64_t)nbits * P->nqubits)) return r;
    if (int r = check_ready(P)) return r;
    QXG_CUDA(cudaSetDevice(P->device));
    if (int r = ensure_plan(P, nbits)) return r;
    if (int r = ensure_bits(P, (size_t)nbits * (size_t)std::max(P->nqubits, 1))) return r;
    const int64_t osz = P->plan->red.out_size;
    const size_t ob = sizeof(double) * 2 * (size_t)osz * nbits;
    if (ob > P->d_out_cap) {
        if (P->d_out) cudaFree(P->d_out);
        P->d_out = nullptr; P->d_out_cap = 0;
        QXG_CUDA(cudaMalloc(&P->d_out, ob));
        P->d_out_cap = ob;
    }
    if (P->nqubits > 0)
        QXG_CUDA(cudaMemcpyAsync(P->d_bits, bits, (size_t)nbits * P->nqubits, cudaMemcpyHostToDevice, P->stream));
    QXG_CUDA(cudaMemsetAsync(P->d_out, 0, ob, P->stream));
    if (int r = run_passes(P, nbits, s0, s1, P->d_out)) return r;
    QXG_CUDA(cudaMemcpyAsync(out, P->d_out, ob, cudaMemcpyDeviceToHost, P->stream));
    QXG_CUDA(cudaStreamSynchronize(P->stream));
    if (int r = check_tc(P)) return r;
    return QXG_OK;
}

int qxg_gradient(qxg_program* P, const char* bits, int32_t nbits, int64_t s0, int64_t s1, const double* amp_bar,
                 double* out, double* leaf_grads) {
    g_last_error.clear();
    if (!P || nbits <= 0 || (P->nqubits > 0 && !bits) || !leaf_grads) return fail(QXG_ERR_INVALID, "bad arguments");
    if (s0 < 0 || s1 > P->nslices || s0 >= s1) return fail(QXG_ERR_INVALID, "slice range out of bounds");
    if (int r = validate_bits(bits, (int64_t)nbits * P->nqubits)) return r;
    if (int r = check_ready(P)) return r;
    QXG_CUDA(cudaSetDevice(P->device));
    if (int r = ensure_plan(P, nbits, true)) return r;
    if (int r = ensure_bits(P, (size_t)nbits * (size_t)std::max(P->nqubits, 1))) return r;
    if (P->nqubits > 0)
        QXG_CUDA(cudaMemcpyAsync(P->d_bits, bits, (size_t)nbits * P->nqubits, cudaMemcpyHostToDevice, P->stream));
    const int64_t osz = P->gplan->red.out_size;
    const size_t ob = sizeof(double) * 2 * (size_t)osz * nbits;
    auto grow = [&](double** buf, size_t* cap, size_t bytes) -> int {
        if (bytes <= *cap) return 0;
        QXG_CUDA(cudaStreamSynchronize(P->stream));
        if (*buf) cudaFree(*buf);
        *buf = nullptr;
        *cap = 0;
        QXG_CUDA(cudaMalloc((void**)buf, bytes));
        *cap = bytes;
        return 0;
    };
    if (out) {
        if (int r = grow(&P->d_out, &P->d_out_cap, ob)) return r;
        QXG_CUDA(cudaMemsetAsync(P->d_out, 0, ob, P->stream));
    }
    int64_t gtotal = 0;
    leaf_offsets(P, &gtotal);
    const size_t gb = sizeof(double) * 2 * (size_t)std::max<int64_t>(gtotal, 1);
    if (int r = grow(&P->d_grad, &P->d_grad_cap, gb)) return r;
    QXG_CUDA(cudaMemsetAsync(P->d_grad, 0, gb, P->stream));
    if (amp_bar) {
        if (int r = grow(&P->d_ampbar, &P->d_ampbar_cap, ob)) return r;
        QXG_CUDA(cudaMemcpyAsync(P->d_ampbar, amp_bar, ob, cudaMemcpyHostToDevice, P->stream));
    }
    if (int r = run_grad_passes(P, nbits, s0, s1, out ? P->d_out : nullptr, amp_bar ? P->d_ampbar : nullptr,
                                P->d_grad))
        return r;
    if (out) QXG_CUDA(cudaMemcpyAsync(out, P->d_out, ob, cudaMemcpyDeviceToHost, P->stream));
    QXG_CUDA(cudaMemcpyAsync(leaf_grads, P->d_grad, sizeof(double) * 2 * (size_t)gtotal, cudaMemcpyDeviceToHost,
                             P->stream));
    QXG_CUDA(cudaStreamSynchronize(P->stream));
    if (int r = check_tc_plan(P, P->gplan.get())) return r;
    return QXG_OK;
}

int qxg_program_synchronize(qxg_program* P) {
    if (!P) return fail(QXG_ERR_INVALID, "bad arguments");
    QXG_CUDA(cudaStreamSynchronize(P->stream));
    if (int r = check_tc(P)) return r;
    return QXG_OK;
}

void* qxg_program_stream(qxg_program* P) { return P ? (void*)P->stream : nullptr; }

int qxg_program_info_get(const qxg_program* P, qxg_program_info* info) {
    if (!P || !info) return fail(QXG_ERR_INVALID, "bad arguments");
    memset(info, 0, sizeof(*info));
    info->num_slices = P->nslices;
    int64_t osz = 1;
    for (int64_t d : P->base[P->root].dims) osz *= d;
    info->output_size = osz;
    info->num_qubits = P->nqubits;
    int ns = 0;
    for (auto& I : P->ins) if (I.op == QXG_OP_NCON) ns++;
    info->num_steps = ns;
    info->flops_per_amplitude = P->flops_per_amp;
    if (P->plan) {
        const Plan& pl = *P->plan;
        info->bitstring_batch = pl.bc;
        info->slice_batch = pl.sc;
        info->workspace_bytes = (int64_t)(pl.arena_bytes + pl.tc_scratch_bytes);
        info->flops_executed_per_pass = pl.flops_pass[0] + pl.flops_pass[1] + pl.flops_pass[2];
        info->bytes_executed_per_pass = pl.bytes_pass[0] + pl.bytes_pass[1] + pl.bytes_pass[2];
        int c[3] = {0, 0, 0}, ntc = 0;
        for (int g = 0; g < 3; g++)
            for (auto& st : pl.steps[g]) {
                if (st.kind == QXG_OP_NCON) c[g]++;
                if (st.use_tc || st.use_join) ntc++;
            }
        info->num_steps_tensor_core = ntc;
        int nf = 0;
        for (int g = 0; g < 3; g++)
            for (auto& st : pl.steps[g]) if (st.use_tc && st.tc.fused) nf++;
        info->num_steps_fused = nf;
        info->num_steps_tuned = P->tuned_steps;
        info->num_steps_invariant = c[0];
        info->num_steps_slice = c[1];
        info->num_steps_bitstring = c[2];
    }
    return QXG_OK;
}

int qxg_program_profile(qxg_program* P, int32_t enable) {
    if (!P) return fail(QXG_ERR_INVALID, "bad arguments");
    QXG_CUDA(cudaSetDevice(P->device));
    QXG_CUDA(cudaStreamSynchronize(P->stream));
    P->profiling = enable != 0;
    P->recs.clear();
    P->ev_used = 0;
    return QXG_OK;
}

int qxg_program_profile_read(qxg_program* P, qxg_step_profile* out, int32_t max_entries, int32_t* n_entries,
                             int64_t* kernel_launches) {
    if (!P || (max_entries > 0 && !out)) return fail(QXG_ERR_INVALID, "bad arguments");
    QXG_CUDA(cudaSetDevice(P->device));
    QXG_CUDA(cudaStreamSynchronize(P->stream));
    std::map<std::pair<int, int>, qxg_step_profile> agg;
    for (const auto& r : P->recs) {
        float ms = 0.f;
        QXG_CUDA(cudaEventElapsedTime(&ms, P->ev_pool[r.ev], P->ev_pool[r.ev + 1]));
        auto& a = agg[{r.instr, r.kind}];
        a.instr = r.instr;
        a.kernel = r.kind;
        a.launches += 1;
        a.ms += ms;
        a.flops += r.flops;
        a.bytes += r.bytes;
    }
    int32_t n = 0;
    for (auto& kv : agg) {
        if (n < max_entries) out[n] = kv.second;
        n++;
    }
    if (n_entries) *n_entries = n;
    if (kernel_launches) *kernel_launches = P->launches;
    return QXG_OK;
}

namespace {
std::string describe_step(const qxg_program* P, const Step& st, int group, int instr);
}

// Tuning text: one line per decision, "<hex of the shape key> <fused> <ntile> <bulk> <tmem> <tma>".
int qxg_program_tuning_get(const qxg_program* P, char* buf, int64_t len) {
    if (!P) return fail(QXG_ERR_INVALID, "tuning: null programme");
    std::string out;
    static const char* hex = "0123456789abcdef";
    for (const auto& kv : P->tune_cache) {
        for (unsigned char ch : kv.first) { out += hex[ch >> 4]; out += hex[ch & 15]; }
        const TcVariant& v = kv.second;
        out += " " + std::to_string((int)v.fused) + " " + std::to_string(v.ntile) + " " + std::to_string((int)v.bulk) +
               " " + std::to_string((int)v.tmem) + " " + std::to_string((int)v.tma) + "\n";
    }
    if (buf && len > 0) snprintf(buf, (size_t)len, "%s", out.c_str());
    return (int)out.size();
}

int qxg_program_tuning_set(qxg_program* P, const char* text) {
    if (!P || !text) return fail(QXG_ERR_INVALID, "tuning: null programme or text");
    const char* p = text;
    while (*p) {
        const char* e = p;
        while (*e && *e != ' ' && *e != '\n') e++;
        std::string key;
        for (const char* h = p; h + 1 < e; h += 2) {
            auto nib = [](char c) { return c >= 'a' ? c - 'a' + 10 : c - '0'; };
            key += (char)((nib(h[0]) << 4) | nib(h[1]));
        }
        int f = 0, nt = 0, b = 0, tm = 0, ta = 0, used = 0;
        if (*e == ' ' && sscanf(e, " %d %d %d %d %d%n", &f, &nt, &b, &tm, &ta, &used) == 5 &&
            (nt == 16 || nt == 32 || nt == 64) && !key.empty()) {
            P->tune_cache[key] = TcVariant{f != 0, nt, b != 0, tm != 0, ta != 0};
            e += used;
        } else {
            return fail(QXG_ERR_INVALID, "tuning: malformed line");
        }
        while (*e && *e != '\n') e++;
        p = *e ? e + 1 : e;
    }
    return 0;
}

int qxg_program_explain(const qxg_program* P, int32_t instr, char* buf, int32_t len) {
    if (!P || !buf || len <= 0) return fail(QXG_ERR_INVALID, "explain: null programme or buffer");
    // the forward plan, else the gradient plan (which holds the forward steps too)
    const Plan* fpl = P->plan ? P->plan.get() : P->gplan.get();
    if (!fpl) return fail(QXG_ERR_INVALID, "explain: no plan yet (run amplitudes or a gradient first)");
    const Plan& pl = *fpl;
    const Step* found = nullptr;
    int group = -1;
    for (int g = 0; g < 3 && !found; g++)
        for (auto& st : pl.steps[g])
            if (st.kind == QXG_OP_NCON && pl.T[st.tensor].instr == instr) { found = &st; group = g; break; }
    if (!found) return fail(QXG_ERR_INVALID, "explain: instruction " + std::to_string(instr) + " is not an executed ncon");
    std::string d = describe_step(P, *found, group, instr);
    // the gradient plan's adjoint contractions of the same command
    if (P->gplan)
        for (const auto& bs : P->gplan->bsteps)
            if (bs.bkind == kBwdNcon && bs.instr == instr) d += " | adjoint: " + describe_step(P, bs, -1, instr);
    snprintf(buf, (size_t)len, "%s", d.c_str());
    return 0;
}

namespace {
std::string describe_step(const qxg_program* P, const Step& st, int group, int instr) {
    static const char* gname[3] = {"invariant", "slice", "bitstring"};
    std::string d = group >= 0 ? "instr " + std::to_string(instr) + " group " + gname[group] + " " : std::string();
    auto bits_of_map = [](const BitMap& m, char cls, std::vector<std::string>& at) {
        for (int i = 0; i < m.n; i++)
            for (int j = 0; j < m.r[i].len; j++) {
                const int dst = m.r[i].dst + j;
                if ((int)at.size() <= dst) at.resize(dst + 1, "-");
                at[dst] = std::string(1, cls) + std::to_string(m.r[i].src + j);
            }
    };
    if (st.use_tc && !st.use_join) {
        const TcStep& t = st.tc;
        if (t.ks > 0) d += "split-K=" + std::to_string(1 << t.ks) + " ";
        if (t.nouter > 0) d += "n-blocks=" + std::to_string(1 << t.nouter) + " ";
        d += std::string("tensor-core ") + (t.tf32 ? "3xTF32 " : "3xBF16 ") + (t.fused ? (t.tma ? "tma-gather" : (t.tmem ? "tmem-gather" : (t.bulk ? "bulk-gather" : "row-gather"))) : "planes") +
             " ntile=" + std::to_string(t.ntile_n) + " nb=" + std::to_string(t.nb) + " nm=" + std::to_string(t.nm) +
             " nn=" + std::to_string(t.nn) + " nk=" + std::to_string(t.nk) + " X=" + (t.x_is_a ? "A" : "B") +
             " x_bits=";
        std::vector<std::string> at;
        bits_of_map(t.xb, 'b', at); bits_of_map(t.xm, 'm', at); bits_of_map(t.xk, 'k', at);
        for (size_t i = 0; i < at.size(); i++) d += (i ? "," : "") + at[i];
        d += " c_bits=";
        at.clear();
        bits_of_map(t.cb, 'b', at); bits_of_map(t.cm, 'm', at); bits_of_map(t.cn, 'n', at);
        for (size_t i = 0; i < at.size(); i++) d += (i ? "," : "") + at[i];
        if (!st.tune_note.empty()) d += " tuned=" + st.tune_note;
    } else {
        const std::string form = st.use_join ? tc_join_describe(st.join)
                                 : st.batch >= 0 ? "cuda-core batched small step"
                                                 : contract_form(st.sargs, P->fp64, P->sm_count);
        d += form;
        int ncb = 0;
        while ((int64_t(1) << ncb) < st.sargs.nC) ncb++;
        d += " c_bits=" + std::to_string(ncb) + " nk=" + std::to_string(st.sargs.nk);
        if (st.use_join || form.find("batched-gemm") != std::string::npos ||
            form.find("long-sum") != std::string::npos) {
            // which index bit lies at each address bit of A and of B (b: in A, B and C; m: A and C;
            // n: B and C; k: summed), from the lowest
            const StepArgs& s = st.sargs;
            auto one = [](const BitMap& m, int bit) {
                const int64_t o = pdep(int64_t(1) << bit, m);
                return o ? __builtin_ctzll((unsigned long long)o) : -1;
            };
            std::vector<std::string> aat, bat;
            auto put = [](std::vector<std::string>& at, int pos, const std::string& v) {
                if (pos < 0) return;
                if ((int)at.size() <= pos) at.resize(pos + 1, "-");
                at[pos] = v;
            };
            int nbat = 0, nm = 0, nn = 0;
            for (int p = 0; p < ncb; p++) {
                const int ia = one(s.cA, p), ib = one(s.cB, p);
                if (ia >= 0 && ib >= 0) {
                    const std::string v = "b" + std::to_string(nbat++);
                    put(aat, ia, v);
                    put(bat, ib, v);
                } else if (ia >= 0) {
                    put(aat, ia, "m" + std::to_string(nm++));
                } else {
                    put(bat, ib, "n" + std::to_string(nn++));
                }
            }
            for (int j = 0; j < s.nk; j++) {
                put(aat, one(s.kA, j), "k" + std::to_string(j));
                put(bat, one(s.kB, j), "k" + std::to_string(j));
            }
            d += " a_bits=";
            for (size_t i = 0; i < aat.size(); i++) d += (i ? "," : "") + aat[i];
            d += " b_bits=";
            for (size_t i = 0; i < bat.size(); i++) d += (i ? "," : "") + bat[i];
        }
    }
    return d;
}
}  // namespace

void qxg_program_destroy(qxg_program* P) {
    if (!P) return;
    cudaSetDevice(P->device);
    if (P->stream) cudaStreamSynchronize(P->stream);
    for (cudaEvent_t e : P->ev_pool) cudaEventDestroy(e);
    drop_graphs(P);
    for (cudaEvent_t e : P->cap_ev) cudaEventDestroy(e);
    for (cudaStream_t s : P->cap_streams) cudaStreamDestroy(s);
    for (void* p : P->d_data) if (p) cudaFree(p);
    if (P->d_arena) cudaFree(P->d_arena);
    for (auto& e : P->tune_ev)
        if (e) cudaEventDestroy(e);
    if (P->d_scratch) cudaFree(P->d_scratch);
    if (P->d_exps) cudaFree(P->d_exps);
    if (P->d_tc_err) cudaFree(P->d_tc_err);
    if (P->d_params) cudaFree(P->d_params);
    if (P->h_params) cudaFreeHost(P->h_params);
    if (P->d_bits) cudaFree(P->d_bits);
    if (P->d_out) cudaFree(P->d_out);
    if (P->d_grad) cudaFree(P->d_grad);
    if (P->d_ampbar) cudaFree(P->d_ampbar);
    if (P->stream) cudaStreamDestroy(P->stream);
    delete P;
}

}  // extern "C"
