// Runs qxg_parse_qx and qxg_parse_yml_output over many texts, for a sanitizer build of the
// readers (host code).  Arguments: kind ("qx" or "yml") and a file of texts, each preceded by a
// line "<byte count>\n".  Each text is parsed with the two-call protocol into heap buffers of
// exactly the reported sizes, so AddressSanitizer sees any access past them or past the text.
// Prints "accepted N rejected M"; exits 1 when a status is positive or the second call of an
// accepted text fails.
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "qxgpu.h"

static thread_local std::string g_err;
namespace qxg {
int ncon_fail(int code, const char* msg) {
    g_err = msg;
    return code;
}
}  // namespace qxg

static int parse_qx(const std::string& text) {
    qxg_qx_sizes sz{};
    int rc = qxg_parse_qx(text.c_str(), &sz, nullptr, nullptr, nullptr, nullptr, nullptr);
    if (rc != 0) return rc < 0 ? -1 : 2;
    std::vector<qxg_instr> ins((size_t)sz.ninstr);
    std::vector<int32_t> labels((size_t)sz.nlabels), rank((size_t)sz.ndata);
    std::vector<int64_t> dims((size_t)sz.ndims);
    std::vector<char> keys((size_t)sz.key_bytes);
    rc = qxg_parse_qx(text.c_str(), &sz, ins.data(), labels.data(), rank.data(), dims.data(), keys.data());
    return rc == 0 ? 0 : 2;
}

static int parse_yml(const std::string& text) {
    qxg_yml_output o{};
    int rc = qxg_parse_yml_output(text.c_str(), &o, nullptr, 0);
    if (rc != 0) return rc < 0 ? -1 : 2;
    const int64_t n = o.nbitstrings * (int64_t)o.num_qubits;
    if (n < 0) return 2;
    std::vector<char> bits((size_t)n);
    rc = qxg_parse_yml_output(text.c_str(), &o, bits.data(), n);
    return rc == 0 ? 0 : 2;
}

int main(int argc, char** argv) {
    if (argc < 3) return 2;
    const std::string kind = argv[1];
    std::ifstream f(argv[2], std::ios::binary);
    std::stringstream ss;
    ss << f.rdbuf();
    const std::string all = ss.str();
    size_t at = 0;
    long accepted = 0, rejected = 0;
    while (at < all.size()) {
        const size_t nl = all.find('\n', at);
        if (nl == std::string::npos) return 2;
        const size_t len = std::strtoull(all.c_str() + at, nullptr, 10);
        at = nl + 1;
        if (at + len > all.size()) return 2;
        const std::string text = all.substr(at, len);   // its own allocation, NUL-terminated
        at += len;
        const int r = kind == "qx" ? parse_qx(text) : parse_yml(text);
        if (r == 2) {
            std::fprintf(stderr, "bad status for text at byte %zu: %s\n", at - len, g_err.c_str());
            return 1;
        }
        (r == 0 ? accepted : rejected)++;
    }
    std::printf("accepted %ld rejected %ld\n", accepted, rejected);
    return 0;
}
