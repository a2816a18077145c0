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
#include <exception>
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

// qxg_parse_yml_output: the `output:` block of the `.yml` parameter file that
// generate_parameter_file writes (src/simulation.jl:149-155) from output_params_dict
// (src/outputs.jl:47-78); layout of docs/src/users_guide.md:22-35.  The YAML read is the subset
// those writers produce: block mappings, block (`- x`) or flow (`[x, y]`) sequences of scalars,
// plain or quoted scalars, `~`/null, `#` comment lines.  Indentation is spaces only.
namespace {

struct YNode {
    enum Kind { NONE, SCALAR, MAP, SEQ } kind = NONE;
    std::string text;  // SCALAR: the value as written, quotes removed
    bool quoted = false;
    int line = 0;
    std::vector<std::pair<std::string, YNode>> map;
    std::vector<YNode> seq;
    const YNode* get(const char* k) const {
        for (const auto& kv : map)
            if (kv.first == k) return &kv.second;
        return nullptr;
    }
};

struct YRow {
    int indent;
    std::string body;
    int line;
};

struct YError {
    int line;
    std::string why;
};

std::string trim(const std::string& s) {
    size_t a = 0, b = s.size();
    while (a < b && std::isspace((unsigned char)s[a])) a++;
    while (b > a && std::isspace((unsigned char)s[b - 1])) b--;
    return s.substr(a, b - a);
}

bool is_item(const std::string& body) { return body == "-" || body.compare(0, 2, "- ") == 0; }

// One scalar: "..." (with \x escapes taken as x), '...' (with '' for '), or plain text.
void y_scalar(const std::string& raw, int line, YNode* n) {
    const std::string s = trim(raw);
    n->kind = YNode::SCALAR;
    n->line = line;
    if (!s.empty() && (s[0] == '"' || s[0] == '\'')) {
        const char q = s[0];
        std::string out;
        size_t i = 1;
        bool closed = false;
        for (; i < s.size(); i++) {
            const char c = s[i];
            if (q == '"' && c == '\\' && i + 1 < s.size()) {
                out += s[++i];
                continue;
            }
            if (c == q) {
                if (q == '\'' && i + 1 < s.size() && s[i + 1] == '\'') {
                    out += q;
                    i++;
                    continue;
                }
                closed = true;
                i++;
                break;
            }
            out += c;
        }
        if (!closed || !trim(s.substr(i)).empty()) throw YError{line, "bad quoted scalar " + s};
        n->text = out;
        n->quoted = true;
        return;
    }
    n->text = s;
}

// `[a, b, "c"]`: commas outside quotes separate the items.
void y_flow_seq(const std::string& s, int line, YNode* n) {
    n->kind = YNode::SEQ;
    n->line = line;
    if (s.size() < 2 || s.back() != ']') throw YError{line, "unterminated flow sequence"};
    const std::string body = s.substr(1, s.size() - 2);
    if (trim(body).empty()) return;
    char q = 0;
    size_t start = 0;
    for (size_t i = 0; i <= body.size(); i++) {
        const char c = i < body.size() ? body[i] : ',';
        if (q) {
            if (c == '\\' && q == '"') i++;
            else if (c == q) q = 0;
        } else if (c == '"' || c == '\'') {
            q = c;
        } else if (c == '[' || c == '{') {
            throw YError{line, "nested flow collections are not read"};
        } else if (c == ',') {
            YNode item;
            y_scalar(body.substr(start, i - start), line, &item);
            if (item.text.empty() && !item.quoted) throw YError{line, "empty flow sequence item"};
            n->seq.push_back(item);
            start = i + 1;
        }
    }
    if (q) throw YError{line, "unterminated quote in flow sequence"};
}

void y_value(const std::string& rest, int line, YNode* v) {
    if (!rest.empty() && rest[0] == '[') y_flow_seq(rest, line, v);
    else if (!rest.empty() && rest[0] == '{') throw YError{line, "flow mappings are not read"};
    else y_scalar(rest, line, v);
}

// The colon ending a mapping key: the first ':' outside quotes followed by a space or the end.
size_t key_colon(const std::string& body) {
    char q = 0;
    for (size_t i = 0; i < body.size(); i++) {
        const char c = body[i];
        if (q) {
            if (c == q) q = 0;
        } else if (c == '"' || c == '\'') {
            q = c;
        } else if (c == ':' && (i + 1 == body.size() || body[i + 1] == ' ')) {
            return i;
        }
    }
    return std::string::npos;
}

void y_block(const std::vector<YRow>& rows, size_t* i, int ind, YNode* out) {
    out->line = rows[*i].line;
    if (is_item(rows[*i].body)) {
        out->kind = YNode::SEQ;
        while (*i < rows.size() && rows[*i].indent == ind && is_item(rows[*i].body)) {
            const std::string rest = trim(rows[*i].body.substr(1));
            YNode item;
            if (key_colon(rest) != std::string::npos) throw YError{rows[*i].line, "mappings inside sequences are not read"};
            y_value(rest, rows[*i].line, &item);
            out->seq.push_back(item);
            (*i)++;
        }
        return;
    }
    out->kind = YNode::MAP;
    while (*i < rows.size() && rows[*i].indent == ind) {
        const YRow& r = rows[*i];
        if (is_item(r.body)) throw YError{r.line, "sequence item where a key was expected"};
        const size_t c = key_colon(r.body);
        if (c == std::string::npos) throw YError{r.line, "expected 'key: value'"};
        YNode k;
        y_scalar(r.body.substr(0, c), r.line, &k);
        if (k.text.empty()) throw YError{r.line, "empty key"};
        for (const auto& kv : out->map)
            if (kv.first == k.text) throw YError{r.line, "key " + k.text + " given twice"};
        const std::string rest = trim(r.body.substr(c + 1));
        (*i)++;
        YNode v;
        v.line = r.line;
        if (rest.empty()) {
            if (*i < rows.size() && (rows[*i].indent > ind || (rows[*i].indent == ind && is_item(rows[*i].body))))
                y_block(rows, i, rows[*i].indent, &v);
        } else {
            y_value(rest, r.line, &v);
        }
        out->map.emplace_back(k.text, std::move(v));
    }
}

YNode y_parse(const char* text) {
    std::vector<YRow> rows;
    const std::string src(text);
    size_t pos = 0;
    int line_no = 0;
    while (pos < src.size()) {
        size_t end = src.find('\n', pos);
        if (end == std::string::npos) end = src.size();
        std::string line = src.substr(pos, end - pos);
        pos = end + 1;
        line_no++;
        if (!line.empty() && line.back() == '\r') line.pop_back();
        const std::string body = trim(line);
        if (body.empty() || body[0] == '#' || body == "---") continue;
        size_t ind = 0;
        while (ind < line.size() && line[ind] == ' ') ind++;
        if (line[ind] == '\t') throw YError{line_no, "tab in indentation"};
        rows.push_back({(int)ind, body, line_no});
    }
    YNode root;
    root.kind = YNode::MAP;
    if (rows.empty()) return root;
    size_t i = 0;
    y_block(rows, &i, rows[0].indent, &root);
    if (i < rows.size()) throw YError{rows[i].line, "bad indentation"};
    if (root.kind != YNode::MAP) throw YError{rows[0].line, "the document is not a mapping"};
    return root;
}

bool y_null(const YNode* n) {
    return !n || n->kind == YNode::NONE ||
           (n->kind == YNode::SCALAR && !n->quoted && (n->text == "~" || n->text == "null" || n->text == "Null" ||
                                                         n->text == "NULL" || n->text.empty()));
}

int64_t y_int(const YNode* n, const char* what) {
    int64_t v;
    if (n->kind != YNode::SCALAR || !to_int(n->text, &v)) throw YError{n->line, std::string(what) + " is not an integer"};
    return v;
}

double y_double(const YNode* n, const char* what) {
    if (n->kind == YNode::SCALAR && !n->text.empty()) {
        errno = 0;
        char* end = nullptr;
        const double v = std::strtod(n->text.c_str(), &end);
        if (!errno && end && !*end) return v;
    }
    throw YError{n->line, std::string(what) + " is not a number"};
}

bool y_bool(const YNode* n, const char* what) {
    if (n->kind == YNode::SCALAR && !n->quoted) {
        if (n->text == "true" || n->text == "True" || n->text == "TRUE") return true;
        if (n->text == "false" || n->text == "False" || n->text == "FALSE") return false;
    }
    throw YError{n->line, std::string(what) + " is not a boolean"};
}

void read_output(const YNode& root, qxg_yml_output* o, std::vector<std::string>* bits) {
    const YNode* ob = root.get("output");
    if (!ob || ob->kind != YNode::MAP) throw YError{ob ? ob->line : 0, "no output: block"};
    const YNode* m = ob->get("method");
    if (!m || m->kind != YNode::SCALAR) throw YError{ob->line, "output: has no method"};
    std::string method = m->text;
    if (!method.empty() && method[0] == ':') method = method.substr(1);  // a Julia Symbol written as-is
    if (method == "List") o->method = QXG_OUTPUT_LIST;
    else if (method == "Uniform") o->method = QXG_OUTPUT_UNIFORM;
    else if (method == "Rejection") o->method = QXG_OUTPUT_REJECTION;
    else throw YError{m->line, "output method " + m->text + " not supported"};
    const YNode* p = ob->get("params");
    if (!p || p->kind != YNode::MAP) throw YError{ob->line, "output: has no params"};
    o->M = 1e-4;
    if (const YNode* s = p->get("seed"); !y_null(s)) {
        o->seed = y_int(s, "params.seed");
        o->has_seed = 1;
    }
    const YNode* ns = p->get("num_samples");
    if (!y_null(ns)) {
        o->num_samples = y_int(ns, "params.num_samples");
        if (o->num_samples < 0) throw YError{ns->line, "params.num_samples is negative"};
    }
    const YNode* nq = p->get("num_qubits");
    if (o->method == QXG_OUTPUT_LIST) {
        const YNode* b = p->get("bitstrings");
        if (!b) throw YError{p->line, "List output without params.bitstrings"};
        if (b->kind != YNode::SEQ && !y_null(b)) throw YError{b->line, "params.bitstrings is not a sequence"};
        int64_t len = -1;
        for (const YNode& x : b->seq) {
            if (x.kind != YNode::SCALAR) throw YError{x.line, "a bitstring is not a scalar"};
            for (char ch : x.text)
                if (ch != '0' && ch != '1' && ch != '+' && ch != '-')
                    throw YError{x.line, "bitstring '" + x.text + "' has a character other than 0 1 + -"};
            if (len >= 0 && (int64_t)x.text.size() != len)
                throw YError{x.line, "bitstring '" + x.text + "' differs in length from the first"};
            len = (int64_t)x.text.size();
            bits->push_back(x.text);
        }
        o->nbitstrings = (int64_t)bits->size();
        if (len > INT32_MAX) throw YError{b->line, "bitstrings too long"};
        o->num_qubits = len < 0 ? 0 : (int32_t)len;
        if (!y_null(nq) && len >= 0 && y_int(nq, "params.num_qubits") != len)
            throw YError{nq->line, "params.num_qubits differs from the bitstrings' length"};
        if (y_null(ns)) o->num_samples = o->nbitstrings;
        return;
    }
    if (y_null(nq)) throw YError{p->line, "params.num_qubits missing"};
    const int64_t q = y_int(nq, "params.num_qubits");
    if (q < 0 || q > INT32_MAX) throw YError{nq->line, "params.num_qubits out of range"};
    o->num_qubits = (int32_t)q;
    if (y_null(ns)) throw YError{p->line, "params.num_samples missing"};
    if (o->method == QXG_OUTPUT_REJECTION) {
        if (const YNode* x = p->get("M"); !y_null(x)) o->M = y_double(x, "params.M");
        if (const YNode* x = p->get("fix_M"); !y_null(x)) o->fix_M = y_bool(x, "params.fix_M") ? 1 : 0;
    }
}

}  // namespace

extern "C" int qxg_parse_yml_output(const char* text, qxg_yml_output* out, char* bitstrings, int64_t capacity) {
    if (!text || !out) return qxg::ncon_fail(QXG_ERR_INVALID, "qxg_parse_yml_output: text and out are required");
    qxg_yml_output o;
    std::memset(&o, 0, sizeof(o));
    std::vector<std::string> bits;
    try {
        read_output(y_parse(text), &o, &bits);
    } catch (const YError& e) {
        const std::string where = e.line > 0 ? "line " + std::to_string(e.line) + ": " : "";
        return qxg::ncon_fail(QXG_ERR_INVALID, ("qxg_parse_yml_output: " + where + e.why).c_str());
    } catch (const std::exception& e) {
        return qxg::ncon_fail(QXG_ERR_INVALID, (std::string("qxg_parse_yml_output: ") + e.what()).c_str());
    }
    if (bitstrings && o.method == QXG_OUTPUT_LIST) {
        const int64_t need = o.nbitstrings * (int64_t)o.num_qubits;
        if (capacity < need)
            return qxg::ncon_fail(QXG_ERR_INVALID, "qxg_parse_yml_output: bitstring buffer smaller than needed");
        int64_t off = 0;
        for (const std::string& b : bits) {
            std::memcpy(bitstrings + off, b.data(), b.size());
            off += (int64_t)b.size();
        }
    }
    *out = o;
    return QXG_OK;
}
