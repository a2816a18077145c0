// qxg_ncon_tc_static: the tensor-core pairwise contraction without any device allocation.
//
// Some callers cannot call cudaMalloc: code that runs while a CUDA graph is being captured,
// hosts whose device allocator belongs to another runtime, allocation-free real-time loops.  For
// them this entry point keeps its scratch -- the packed hi/lo operand planes and three exponent
// slots and a timeout word -- in one file-scope device array of QXG_TC_STATIC_SCRATCH_BYTES.
// Host code may not use the array's name as a device address; the address is looked up once per
// device with cudaGetSymbolAddress (on the first call made with that device current).  Shapes
// whose planes do not fit are rejected.  All calls on a device share the array; it keeps the last
// call's contents, and calls that overlap on one GPU race.  The GEMM's bounded waits report to the
// timeout word in the array's header (not to the word programme walks read), so a call outside
// stream capture waits for its stream and returns QXG_ERR_TIMEOUT when a wait gave up.
#include <mutex>
#include <string>

#include "../../include/qxgpu.h"
#include "qxgpu_internal.h"
#include "tc_gemm.h"

namespace qxg {
int ncon_fail(int code, const char* msg);
int ncon_build_args(StepArgs* s, int32_t nc, const int32_t* lc, int32_t na, const int32_t* la,
                    const int64_t* ad, int32_t nb, const int32_t* lb, const int64_t* bd);
}  // namespace qxg

namespace {

constexpr size_t kStaticBytes = (size_t)QXG_TC_STATIC_SCRATCH_BYTES;
constexpr size_t kExpBytes = 256;   // header: exponent slots (A, B, C) and the timeout word
constexpr size_t kErrWord = 32;     // int index of the timeout word in the header (byte 128)
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_static_scratch[kStaticBytes];

std::mutex g_mu;
void* g_addr[kMaxDevices] = {};

// Device address of g_static_scratch on the current device (looked up once per device).
int static_scratch(int dev, void** out) {
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_addr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
        if (e != cudaSuccess || !p) {
            std::string m = std::string("qxg_ncon_tc_static: cudaGetSymbolAddress failed: ") + cudaGetErrorString(e);
            return qxg::ncon_fail(QXG_ERR_CUDA, m.c_str());
        }
        g_addr[dev] = p;
    }
    *out = g_addr[dev];
    return 0;
}

int bits_of(const int64_t* dims, int32_t n) {
    int b = 0;
    for (int i = 0; i < n; i++) {
        int x = 0;
        while ((int64_t(1) << x) < dims[i]) x++;
        b += x;
    }
    return b;
}

}  // namespace

extern "C" int qxg_ncon_tc_static(int32_t precision, void* C, int32_t nc, const int32_t* c_labels, const void* A,
                                  int32_t na, const int32_t* a_labels, const int64_t* a_dims, const void* B,
                                  int32_t nb, const int32_t* b_labels, const int64_t* b_dims, void* stream) {
    using namespace qxg;
    if (precision != QXG_PREC_SPLIT_BF16 && precision != QXG_PREC_SPLIT_TF32)
        return ncon_fail(QXG_ERR_INVALID, "qxg_ncon_tc_static: precision must be QXG_PREC_SPLIT_BF16 or _TF32");
    if (!C || !A || !B || nc < 0 || na < 0 || nb < 0 || (nc && !c_labels) || (na && (!a_labels || !a_dims)) ||
        (nb && (!b_labels || !b_dims)))
        return ncon_fail(QXG_ERR_INVALID, "qxg_ncon_tc_static: bad arguments");
    StepArgs s;
    if (int r = ncon_build_args(&s, nc, c_labels, na, a_labels, a_dims, nb, b_labels, b_dims)) return r;
    s.A = A; s.B = B; s.C = C;
    s.expA = 0; s.expB = 1; s.expC = 2;
    int cbits = 0;
    while ((int64_t(1) << cbits) < s.nC) cbits++;
    TcStep t;
    // the Y planes are cut into outer column blocks before they outgrow the array (partial sums
    // of a split K come on top; the size check below has the final word)
    if (!tc_plan_step(s, (size_t)bits_of(a_dims, na), (size_t)bits_of(b_dims, nb), (size_t)cbits,
                      precision == QXG_PREC_SPLIT_TF32, &t, (double)((kStaticBytes - kExpBytes) / 4)))
        return ncon_fail(QXG_ERR_UNSUPPORTED,
                         "qxg_ncon_tc_static: shape not served by the tensor cores (needs >= 128 free rows on the "
                         "larger operand, or >= 16 with a summed extent above 1024, a summed extent >= 8 and "
                         ">= 4 free columns on the smaller)");
    if (t.scratch_bytes > kStaticBytes - kExpBytes) {
        std::string m = "qxg_ncon_tc_static: the packed operands need " + std::to_string(t.scratch_bytes) +
                        " bytes, more than the static scratch of " + std::to_string(kStaticBytes - kExpBytes) + " bytes";
        return ncon_fail(QXG_ERR_UNSUPPORTED, m.c_str());
    }
    int dev = 0, sms = 148;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return ncon_fail(QXG_ERR_CUDA, cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return ncon_fail(QXG_ERR_UNSUPPORTED, "qxg_ncon_tc_static: device ordinal too large");
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    void* base = nullptr;
    if (int r = static_scratch(dev, &base)) return r;
    int* exps = static_cast<int*>(base);
    void* planes = static_cast<unsigned char*>(base) + kExpBytes;
    t.err_word = exps + kErrWord;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // the header starts at zero: exponent slots at 0 (operands enter unscaled, the result is
    // stored as is) and no timeout
    e = cudaMemsetAsync(exps, 0, kExpBytes, st);
    if (e == cudaSuccess) e = tc_run_step(t, s, exps, planes, st, sms, nullptr);
    if (e != cudaSuccess) return ncon_fail(QXG_ERR_CUDA, cudaGetErrorString(e));
    // outside stream capture, wait for the call and report a wait that gave up; under capture
    // nothing can be read back, and a replay that timed out leaves its code in the header
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cap) != cudaSuccess) {
        cudaGetLastError();             // a query refused during another stream's capture
        return QXG_OK;
    }
    if (cap != cudaStreamCaptureStatusNone) return QXG_OK;
    int code = 0;
    e = cudaMemcpyAsync(&code, t.err_word, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return ncon_fail(QXG_ERR_CUDA, cudaGetErrorString(e));
    if (code) {
        std::string m = "qxg_ncon_tc_static: a tensor-core wait gave up (code " + std::to_string(code) + ")";
        return ncon_fail(QXG_ERR_TIMEOUT, m.c_str());
    }
    return QXG_OK;
}
