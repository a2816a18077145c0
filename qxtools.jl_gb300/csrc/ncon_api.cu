// qxg_ncon: one pairwise contraction on caller-owned device buffers (one `ncon` command of
// docs/src/users_guide.md:124-146, a ContractCommand of src/compute_graph/compute_graph.jl:61-74).
// Operands and result are column-major in their label order; dimensions must be powers of two.
#include <cstring>
#include <string>
#include <vector>

#include "../../include/qxgpu.h"
#include "qxgpu_internal.h"

using namespace qxg;

namespace qxg {
int ncon_fail(int code, const char* msg);
}

namespace {

int ilog2_exact(int64_t x) {
    int b = 0;
    while ((int64_t(1) << b) < x) b++;
    return (int64_t(1) << b) == x ? b : -1;
}

BitMap runs_of(std::vector<std::pair<int, int>> p, bool* ok) {
    BitMap m;
    m.n = 0;
    for (size_t i = 0; i < p.size();) {
        size_t j = i + 1;
        while (j < p.size() && p[j].first == p[j - 1].first + 1 && p[j].second == p[j - 1].second + 1) j++;
        if (m.n >= kMaxRuns) { *ok = false; return m; }
        m.r[m.n] = Run{(uint8_t)p[i].first, (uint8_t)(j - i), (uint8_t)p[i].second, 0};
        m.n++;
        i = j;
    }
    return m;
}

}  // namespace

// Build the bit maps of C = ncon(A, B) for column-major operands.  Returns 0 or a status.
namespace qxg {
int ncon_build_args(StepArgs* s, int32_t nc, const int32_t* lc, int32_t na, const int32_t* la,
                    const int64_t* ad, int32_t nb, const int32_t* lb, const int64_t* bd) {
    memset(s, 0, sizeof(*s));
    // bit offsets of each axis
    std::vector<int> aoff(na + 1, 0), boff(nb + 1, 0), abits(na), bbits(nb);
    for (int i = 0; i < na; i++) {
        abits[i] = ilog2_exact(ad[i]);
        if (abits[i] < 0) return ncon_fail(QXG_ERR_UNSUPPORTED, "qxg_ncon: dimensions must be powers of two");
        aoff[i + 1] = aoff[i] + abits[i];
    }
    for (int i = 0; i < nb; i++) {
        bbits[i] = ilog2_exact(bd[i]);
        if (bbits[i] < 0) return ncon_fail(QXG_ERR_UNSUPPORTED, "qxg_ncon: dimensions must be powers of two");
        boff[i + 1] = boff[i] + bbits[i];
    }
    if (aoff[na] > 46 || boff[nb] > 46) return ncon_fail(QXG_ERR_UNSUPPORTED, "qxg_ncon: operand too large");
    auto find = [](const int32_t* ls, int n, int32_t L) {
        for (int i = 0; i < n; i++) if (ls[i] == L) return i;
        return -1;
    };
    for (int i = 0; i < na; i++) if (find(la, i, la[i]) >= 0) return ncon_fail(QXG_ERR_UNSUPPORTED, "qxg_ncon: repeated label");
    for (int i = 0; i < nb; i++) if (find(lb, i, lb[i]) >= 0) return ncon_fail(QXG_ERR_UNSUPPORTED, "qxg_ncon: repeated label");
    std::vector<std::pair<int, int>> cA, cB, kA, kB;
    int cbit = 0;
    for (int i = 0; i < nc; i++) {
        const int ia = find(la, na, lc[i]), ib = find(lb, nb, lc[i]);
        if (ia < 0 && ib < 0) return ncon_fail(QXG_ERR_INVALID, "qxg_ncon: result label not in operands");
        if (find(lc, i, lc[i]) >= 0) return ncon_fail(QXG_ERR_INVALID, "qxg_ncon: repeated result label");
        const int nbit = ia >= 0 ? abits[ia] : bbits[ib];
        if (ia >= 0 && ib >= 0 && abits[ia] != bbits[ib]) return ncon_fail(QXG_ERR_INVALID, "qxg_ncon: dimension mismatch");
        for (int j = 0; j < nbit; j++) {
            if (ia >= 0) cA.push_back({cbit + j, aoff[ia] + j});
            if (ib >= 0) cB.push_back({cbit + j, boff[ib] + j});
        }
        cbit += nbit;
    }
    if (cbit > 46) return ncon_fail(QXG_ERR_UNSUPPORTED, "qxg_ncon: result too large");
    int kbit = 0;
    for (int i = 0; i < na; i++) {
        if (find(lc, nc, la[i]) >= 0) continue;
        const int ib = find(lb, nb, la[i]);
        if (ib >= 0 && bbits[ib] != abits[i]) return ncon_fail(QXG_ERR_INVALID, "qxg_ncon: dimension mismatch");
        for (int j = 0; j < abits[i]; j++) {
            kA.push_back({kbit + j, aoff[i] + j});
            if (ib >= 0) kB.push_back({kbit + j, boff[ib] + j});
        }
        kbit += abits[i];
    }
    for (int i = 0; i < nb; i++) {
        if (find(lc, nc, lb[i]) >= 0 || find(la, na, lb[i]) >= 0) continue;
        for (int j = 0; j < bbits[i]; j++) kB.push_back({kbit + j, boff[i] + j});
        kbit += bbits[i];
    }
    bool ok = true;
    s->nC = int64_t(1) << cbit;
    s->nk = kbit;
    s->cA = runs_of(cA, &ok);
    s->cB = runs_of(cB, &ok);
    s->kA = runs_of(kA, &ok);
    s->kB = runs_of(kB, &ok);
    s->expA = s->expB = s->expC = -1;
    if (!ok) return ncon_fail(QXG_ERR_UNSUPPORTED, "qxg_ncon: permutation too fragmented");
    return 0;
}
}  // namespace qxg

extern "C" int qxg_ncon(int32_t precision, void* C, int32_t nc, const int32_t* c_labels, const void* A, int32_t na,
                        const int32_t* a_labels, const int64_t* a_dims, const void* B, int32_t nb,
                        const int32_t* b_labels, const int64_t* b_dims, void* stream) {
    if (!C || !A || !B || nc < 0 || na < 0 || nb < 0 || (nc && !c_labels) || (na && (!a_labels || !a_dims)) ||
        (nb && (!b_labels || !b_dims)))
        return ncon_fail(QXG_ERR_INVALID, "qxg_ncon: bad arguments");
    if (precision < QXG_PREC_FP64 || precision > QXG_PREC_FP32)
        return ncon_fail(QXG_ERR_INVALID, "qxg_ncon: unknown precision");
    StepArgs s;
    if (int r = ncon_build_args(&s, nc, c_labels, na, a_labels, a_dims, nb, b_labels, b_dims)) return r;
    s.A = A; s.B = B; s.C = C;
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    // steps with few results and a long sum keep per-block partials in stream-ordered scratch
    const bool fp64 = precision == QXG_PREC_FP64;
    const size_t need = contract_scratch_bytes(s, fp64, sms);
    void* scratch = nullptr;
    if (need) {
        const cudaError_t ea = cudaMallocAsync(&scratch, need, (cudaStream_t)stream);
        if (ea != cudaSuccess) return ncon_fail(QXG_ERR_CUDA, cudaGetErrorString(ea));
    }
    const cudaError_t e = launch_contract(s, fp64, nullptr, (cudaStream_t)stream, sms, scratch, need);
    if (scratch) cudaFreeAsync(scratch, (cudaStream_t)stream);
    if (e != cudaSuccess) return ncon_fail(QXG_ERR_CUDA, cudaGetErrorString(e));
    return QXG_OK;
}
