// qxg_parse_qx: the `.qx` DSL text that generate_simulation_files writes (grammar of
// docs/src/users_guide.md:93-165; writer QXContexts.generate_dsl_files, called at
// src/simulation.jl:73) parsed into qxg_program_create's arguments, so that a caller can hand the
// file to the library as it is.  Host code only.
//
//   load <t> <data key> <d1,d2,..>       leaf tensor t = data[key] with the given dims
//   view <new> <t> v<i> <pos> <dim>      new = t with rank position pos fixed to slice variable i
//   output <t> <qubit> <dim>             t = basis vector of output qubit `qubit`
//   ncon <C> <c labels> <A> <a labels> <B> <b labels>   (labels comma separated, `0` = none)
//   save <label> <t>
//
// `#` lines are comments (the first may carry `# version: ...`); blank lines are skipped.  Tensor
// names become dense ids in order of definition; data keys are numbered in order of first `load`.
#include <cctype>
#include <cerrno>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../../include/qxgpu.h"
#include "qxgpu_internal.h"

namespace qxg {
int ncon_fail(int code, const char* msg);
}

namespace {

struct Parsed {
    std::vector<qxg_instr> ins;
    std::vector<int32_t> labels;
    std::vector<std::string> keys;
    std::vector<std::vector<int64_t>> dims;
    int32_t nqubits = 0;
};

std::vector<std::string> split_ws(const std::string& s) {
    std::vector<std::string> t;
    size_t i = 0;
    while (i < s.size()) {
        while (i < s.size() && std::isspace((unsigned char)s[i])) i++;
        size_t j = i;
        while (j < s.size() && !std::isspace((unsigned char)s[j])) j++;
        if (j > i) t.push_back(s.substr(i, j - i));
        i = j;
    }
    return t;
}

// A decimal integer filling the whole token.
bool to_int(const std::string& s, int64_t* v) {
    if (s.empty()) return false;
    size_t i = s[0] == '-' || s[0] == '+' ? 1 : 0;
    if (i == s.size()) return false;
    for (size_t j = i; j < s.size(); j++)
        if (!std::isdigit((unsigned char)s[j])) return false;
    errno = 0;
    char* end = nullptr;
    const long long x = std::strtoll(s.c_str(), &end, 10);
    if (errno || *end) return false;
    *v = x;
    return true;
}

// Comma-separated integers; "0" alone is the empty list (a scalar operand or result).
bool to_list(const std::string& s, std::vector<int64_t>* out) {
    out->clear();
    if (s == "0") return true;
    size_t i = 0;
    while (i <= s.size()) {
        const size_t j = s.find(',', i);
        const std::string tok = s.substr(i, j == std::string::npos ? std::string::npos : j - i);
        int64_t v;
        if (!to_int(tok, &v)) return false;
        out->push_back(v);
        if (j == std::string::npos) break;
        i = j + 1;
    }
    return !out->empty();
}

int parse(const char* text, Parsed* p) {
    std::map<std::string, int32_t> ids, key_ids;
    std::string src(text);
    size_t pos = 0;
    int line_no = 0;
    auto bad = [&](const std::string& why) {
        return qxg::ncon_fail(QXG_ERR_INVALID, ("qxg_parse_qx: line " + std::to_string(line_no) + ": " + why).c_str());
    };
    while (pos <= src.size()) {
        size_t end = src.find('\n', pos);
        if (end == std::string::npos) end = src.size();
        std::string line = src.substr(pos, end - pos);
        pos = end + 1;
        line_no++;
        const std::vector<std::string> t = split_ws(line);
        if (t.empty() || t[0][0] == '#') {
            if (end >= src.size()) break;
            continue;
        }
        qxg_instr I;
        std::memset(&I, 0, sizeof(I));
        auto use = [&](const std::string& name, int32_t* id) -> bool {
            auto it = ids.find(name);
            if (it == ids.end()) return false;
            *id = it->second;
            return true;
        };
        auto define = [&](const std::string& name, int32_t* id) -> bool {
            if (ids.count(name)) return false;
            *id = (int32_t)ids.size();
            ids[name] = *id;
            return true;
        };
        const std::string& op = t[0];
        if (op == "load") {
            if (t.size() != 3 && t.size() != 4) return bad("load takes a name, a data key and dims");
            std::vector<int64_t> d;
            if (t.size() == 4 && !to_list(t[3], &d)) return bad("bad dims '" + t[3] + "'");
            for (int64_t x : d)
                if (x <= 0) return bad("dims must be positive");
            I.op = QXG_OP_LOAD;
            auto k = key_ids.find(t[2]);
            if (k == key_ids.end()) {
                I.a = (int32_t)p->keys.size();
                key_ids[t[2]] = I.a;
                p->keys.push_back(t[2]);
                p->dims.push_back(d);
            } else {
                I.a = k->second;
                if (p->dims[I.a] != d) return bad("data key " + t[2] + " loaded with two shapes");
            }
            if (!define(t[1], &I.dst)) return bad("tensor " + t[1] + " defined twice");
        } else if (op == "view") {
            int64_t rp, dim, var;
            if (t.size() != 6) return bad("view takes a name, a tensor, v<i>, a position and a dimension");
            if (t[3].size() < 2 || t[3][0] != 'v' || !to_int(t[3].substr(1), &var) || var < 1)
                return bad("bad slice variable '" + t[3] + "'");
            if (!to_int(t[4], &rp) || rp < 1 || !to_int(t[5], &dim) || dim < 1)
                return bad("bad view position or dimension");
            I.op = QXG_OP_VIEW;
            if (!use(t[2], &I.a)) return bad("tensor " + t[2] + " used before definition");
            I.b = (int32_t)(var - 1);
            I.pos = (int32_t)(rp - 1);
            I.dim = (int32_t)dim;
            if (!define(t[1], &I.dst)) return bad("tensor " + t[1] + " defined twice");
        } else if (op == "output") {
            int64_t qubit, dim;
            if (t.size() != 4 || !to_int(t[2], &qubit) || qubit < 1 || !to_int(t[3], &dim) || dim < 1)
                return bad("output takes a name, a qubit (from 1) and a dimension");
            I.op = QXG_OP_OUTPUT;
            I.a = (int32_t)(qubit - 1);
            I.b = (int32_t)dim;
            if ((int32_t)qubit > p->nqubits) p->nqubits = (int32_t)qubit;
            if (!define(t[1], &I.dst)) return bad("tensor " + t[1] + " defined twice");
        } else if (op == "ncon") {
            std::vector<int64_t> lc, la, lb;
            if (t.size() != 7) return bad("ncon takes C, its labels, A, its labels, B, its labels");
            if (!to_list(t[2], &lc) || !to_list(t[4], &la) || !to_list(t[6], &lb)) return bad("bad label list");
            I.op = QXG_OP_NCON;
            if (!use(t[3], &I.a)) return bad("tensor " + t[3] + " used before definition");
            if (!use(t[5], &I.b)) return bad("tensor " + t[5] + " used before definition");
            I.nc = (int32_t)lc.size();
            I.na = (int32_t)la.size();
            I.nb = (int32_t)lb.size();
            I.label_off = (int32_t)p->labels.size();
            for (const auto* l : {&lc, &la, &lb})
                for (int64_t x : *l) {
                    if (x < 0 || x > INT32_MAX) return bad("label out of range");
                    p->labels.push_back((int32_t)x);
                }
            if (!define(t[1], &I.dst)) return bad("tensor " + t[1] + " defined twice");
        } else if (op == "save") {
            if (t.size() != 3) return bad("save takes a label and a tensor");
            I.op = QXG_OP_SAVE;
            if (!use(t[2], &I.a)) return bad("tensor " + t[2] + " used before definition");
        } else {
            return bad("unknown command '" + op + "'");
        }
        p->ins.push_back(I);
        if (end >= src.size()) break;
    }
    if (p->ins.empty()) return qxg::ncon_fail(QXG_ERR_INVALID, "qxg_parse_qx: no commands");
    return QXG_OK;
}

}  // namespace

extern "C" int qxg_parse_qx(const char* text, qxg_qx_sizes* sizes, qxg_instr* instrs, int32_t* labels,
                            int32_t* data_rank, int64_t* data_dims, char* data_keys) {
    if (!text || !sizes) return qxg::ncon_fail(QXG_ERR_INVALID, "qxg_parse_qx: text and sizes are required");
    Parsed p;
    if (int r = parse(text, &p)) return r;
    qxg_qx_sizes need;
    std::memset(&need, 0, sizeof(need));
    need.ninstr = (int32_t)p.ins.size();
    need.nlabels = (int64_t)p.labels.size();
    need.ndata = (int32_t)p.keys.size();
    for (const auto& d : p.dims) need.ndims += (int64_t)d.size();
    for (const auto& k : p.keys) need.key_bytes += (int64_t)k.size() + 1;
    need.nqubits = p.nqubits;
    const bool fill = instrs || labels || data_rank || data_dims || data_keys;
    if (fill) {
        if (!instrs || !data_rank || (need.nlabels && !labels) || (need.ndims && !data_dims) || !data_keys)
            return qxg::ncon_fail(QXG_ERR_INVALID, "qxg_parse_qx: an output array is NULL");
        if (sizes->ninstr < need.ninstr || sizes->nlabels < need.nlabels || sizes->ndata < need.ndata ||
            sizes->ndims < need.ndims || sizes->key_bytes < need.key_bytes)
            return qxg::ncon_fail(QXG_ERR_INVALID, "qxg_parse_qx: output arrays smaller than the sizes needed");
        std::memcpy(instrs, p.ins.data(), sizeof(qxg_instr) * p.ins.size());
        if (need.nlabels) std::memcpy(labels, p.labels.data(), sizeof(int32_t) * p.labels.size());
        int64_t off = 0, koff = 0;
        for (size_t i = 0; i < p.keys.size(); i++) {
            data_rank[i] = (int32_t)p.dims[i].size();
            for (int64_t x : p.dims[i]) data_dims[off++] = x;
            std::memcpy(data_keys + koff, p.keys[i].c_str(), p.keys[i].size() + 1);
            koff += (int64_t)p.keys[i].size() + 1;
        }
    }
    *sizes = need;
    return QXG_OK;
}
