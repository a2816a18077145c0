// Tensor-core (tcgen05) path of the split-precision executors.
//
// A contraction step C[b,m,n] = sum_k X[b,m,k] Y[b,k,n] (X the larger operand, Y the smaller)
// runs as a real GEMM on the 5th-generation tensor cores:
//   A_op[m, (q,k)]         = (Re X, Im X)[m, k]                  (M x 2K, K-major)
//   B_op[(p,n), (q,k)]     = [[Re Y, -Im Y], [Im Y, Re Y]]       (2N x 2K, K-major)
//   D[m, (p,n)]            = (Re C, Im C)[m, n]                  (FP32 in tensor memory)
// Each operand is split into hi + lo planes (3xBF16: bf16 round-to-nearest of x and of x-hi;
// 3xTF32 the same with tf32), scaled by 2^-(max exponent) so nothing underflows, and the three
// products hi*hi + hi*lo + lo*hi accumulate in FP32 (the lo*lo term is dropped): hi*hi in one
// tensor-memory accumulator and the two small correction products in a second one, added in the
// epilogue, so the corrections are not lost against the large running sum.
#pragma once

#include <cstddef>
#include <string>
#include <cuda_runtime.h>

#include "qxgpu_internal.h"

namespace qxg {

constexpr int kTcTileM = 128;       // MMA M (rows of X per CTA)
constexpr int kTcChunkBytes = 64;   // bytes of one operand row per K chunk (4 core-matrix columns)

struct TcStep {
    bool x_is_a = true;             // the larger operand (M side) is the step's A
    bool tf32 = false;
    bool fused = true;              // the GEMM gathers and splits X itself (no X planes in scratch)
    bool bulk = false;              // fused, with X's contiguous segments fetched by cp.async.bulk
    bool tmem = false;              // fused row gather, A tiles in tensor memory
    bool tma = false;               // fused TMA tensor gather, A tiles in tensor memory
    bool tma_ok = false;            // X's blocks fit one 5-D TMA box (see tc_gemm.cu)
    int tma_npiece = 0;             // TMA box: runs of the block's address bits (<= 4 pieces of <= 8 bits)
    int tma_pos[4] = {0, 0, 0, 0}, tma_len[4] = {0, 0, 0, 0};
    int tma_lead = 0;               // the block holds X's address bits 0 .. tma_lead-1
    bool bulk_ok = false;           // X's (128 rows x chunk) blocks are segments of >= 16 elements
    bool bfast = false;             // X's lowest address bit is a batch bit (tile order: batch first)
    BitMap segmap{}, rowmap_c{}, kmap_c{};   // bulk gather plan (see tc_gemm.cu)
    int seg_bits = 0, nseg = 0;
    bool planes_ok = false;         // the planes variant's scratch fits the cap
    int nb = 0, nm = 0, nn = 0, nk = 0;        // bits of batch, M, N, K
    int64_t M = 0, N = 0, K = 0, batch = 0;
    int ntile_n = 0;                // complex columns per N tile (N'' = 2 ntile_n)
    int kc = 0;                     // complex K per chunk (16 bf16, 8 tf32)
    int64_t mtiles = 0, ntiles = 0, kchunks = 0;
    // bit maps: index space -> operand / result offsets
    BitMap xb{}, xm{}, xk{};        // X offset of batch / m / k index
    BitMap yb{}, yn{}, yk{};        // Y offset of batch / n / k index
    BitMap cb{}, cm{}, cn{};        // C offset of batch / m / n index
    int ks = 0;                     // split K: K blocks = 2^ks (their index bits count in nb)
    int nouter = 0;                 // outer N blocks = 2^nouter, looped on the host
    BitMap yo{}, co{};              // outer block index -> Y / C offset (n = 0: no blocks)
    int64_t c_elems = 0;            // elements of the result
    size_t a_plane_bytes = 0, b_plane_bytes = 0, partial_bytes = 0;
    size_t scratch_bytes = 0;       // 2 planes of A_op (planes variant) + 2 planes of B_op + partials
    size_t scratch_max = 0;         // the largest scratch of any candidate variant
    // launch controls, not part of the step's shape
    uint32_t wait_limit = 0;        // mbarrier polls before a wait gives up (0: 2^20)
    bool stall_first_cta = false;   // test hook: CTA 0's operand producer issues no copies, so its
                                    // MMA issuer's wait runs out (exercises the timeout path)
    int* err_word = nullptr;        // device word a wait that gives up writes its code to
                                    // (nullptr: the library-wide word tc_read_error reads)
};

// A tile variant of a tensor-core step: X gathered in the GEMM (fused: by rows or by contiguous
// segments) or packed into planes first, and the complex columns per N tile.
struct TcVariant {
    bool fused;
    int ntile;
    bool bulk;                      // fused only: bulk segment gather instead of row gather
    bool tmem;                      // fused only: row gather with the A tiles in tensor memory
    bool tma;                       // fused only: TMA tensor gather, A tiles in tensor memory
};

// Decide whether a step goes to the tensor cores; fills `tc` (default variant: fused, the
// widest N tile) when it does.
// plane_budget: bytes of Y planes above which the N range is cut into outer blocks (0: 4 GiB).
bool tc_plan_step(const StepArgs& s, size_t a_bits, size_t b_bits, size_t c_bits, bool tf32, TcStep* tc,
                  double plane_budget = 0);

// Candidate variants of a planned step (at most kTcMaxVariants), for the autotuner.
constexpr int kTcMaxVariants = 12;
int tc_variants(const TcStep& t, TcVariant* out);

// Switch a planned step to a variant (recomputes tile counts and scratch sizes).
void tc_set_variant(TcStep& t, TcVariant v);

// Autotuner cache key: the step's shape and bit maps (identical steps share a choice).
std::string tc_key(const TcStep& t);

// Run a planned tensor-core step (scratch: at least tc.scratch_bytes of device memory):
// tc_run_pack (both operands) then tc_run_gemm.
cudaError_t tc_run_pack(const TcStep& tc, const StepArgs& s, int* exps, void* scratch, cudaStream_t st,
                        int sm_count);
cudaError_t tc_run_gemm(const TcStep& tc, const StepArgs& s, int* exps, void* scratch, cudaStream_t st,
                        int sm_count);

// The whole step, outer N blocks included (pack and GEMM per block, then the split-K sum);
// *launches receives the kernels launched.  Steps with nouter == 0 may use the two calls above.
cudaError_t tc_run_step(const TcStep& tc, const StepArgs& s, int* exps, void* scratch, cudaStream_t st,
                        int sm_count, int* launches);

// Read and clear the error word a tensor-core kernel whose bounded wait gave up has set (0 =
// none): d_word (a TcStep's err_word), or the library-wide word when d_word is null.  Waits for st.
cudaError_t tc_read_error(int* host_code, int* d_word, cudaStream_t st);

}  // namespace qxg

namespace qxg {

// ---- Final joins on the tensor cores (tc_join.cu) ----------------------------------------------
// C[b, i, j] = sum_k P[b, k, i] Q[b, k, j] with 32 free values i of one operand (P), 8-32 of the
// other (Q), 2^10+ summed terms per batch value b and both operands large.  The MMA's A operand
// (128 rows, in tensor memory) stacks P four times -- (Re P | -Im P) and (Im P | Re P), each as
// tf32 hi and lo parts -- and its B operand (2 NQ rows, in shared memory) stacks Q's hi and lo
// parts as (Re Q | Im Q), so one M = 128 MMA per 8 summed terms yields all four hi/lo products of
// the complex product (see tc_join.cu).
constexpr int kJoinKR = 64;         // summed terms per raw chunk (its 6 summed bits are planned)
constexpr int kJoinMaxSeg = 256;    // contiguous segments per operand in a raw chunk

// One operand's raw tile as a TMA tensor box: dimension 0 is contiguous with extent 2^H (H the
// operand's lowest batch bit), so its coordinate carries the chunk's offset; the tile's other
// runs of address bits follow (coordinate 0, box = extent); the batch bits, contiguous from bit H
// in any order, are dimension tb (box 1, coordinate = the operand's batch offset >> H).  The box
// lands in shared memory in the tile's address order.
struct JoinBox {
    int32_t td, tb, th;             // dimensions used (<= 5); the batch dimension (-1: none); H
    int64_t dim[5], stride[5];      // extents and strides, in elements (stride[0] = 1)
    int32_t box[5];
};

struct TcJoinArgs {
    const float2* P;
    const float2* Q;
    float2* C;
    int32_t nq;                     // free values of Q (8, 16 or 32)
    int32_t p_is_a;                 // P is the step's A operand
    int32_t conjP, conjQ, expP, expQ, expC;
    int64_t nbatch;
    int32_t nsplit;                 // K ranges per batch value (FP64 partials when > 1)
    int64_t nchunks;                // raw chunks of one K range
    int32_t flush;                  // MMA stages (16 terms) between accumulator drains (power of two)
    int32_t ring;                   // raw chunks in the ring
    BitMap bP, bQ, bC;              // batch index -> P / Q / C offset
    BitMap iC, jC;                  // free index of P / Q -> C offset
    BitMap hP, hQ;                  // chunk index within the whole K -> P / Q offset
    // a raw chunk of P: its tile (32 free values x 64 summed terms) in P's address order, as
    // nsegP segments of 2^sbP contiguous elements; segment s starts at P offset pdep(s << sbP, eP)
    // from the chunk's base and lands at byte s * segP_stride of the ring slot
    BitMap eP, tPi, tPk;            // tile element -> P offset; i / summed index -> tile element
    int32_t sbP, nsegP, segP_stride;
    BitMap eQ, tQj, tQk;            // the same for Q (after P in the slot)
    int32_t sbQ, nsegQ, segQ_stride;
    int32_t slotP_bytes, slot_bytes;
    uint32_t idesc;
    uint32_t wait_limit;            // mbarrier polls before a wait gives up (0: 2^20)
    int32_t stall;                  // test hook: CTA 0's loader issues no copies
    int* err;                       // word a wait that gives up writes its code to
    int32_t chunk_k[6];             // the chunk's summed bits (step k indices), for describe
    int32_t run_p, run_q;           // contiguous elements per segment (2^sbP, 2^sbQ)
    int32_t tma;                    // 1: one TMA tensor copy per operand and chunk (boxP, boxQ);
                                    // 0: the segments by cp.async.bulk
    JoinBox boxP, boxQ;
};

// Plan a step as a tensor-core join (false: it does not fit); operands of at least 2^min_log2
// elements.
bool tc_join_plan(const StepArgs& s, int sm_count, TcJoinArgs* g, int min_log2 = 20);
// Scratch for the FP64 partials of the K ranges (0 with one range per batch value).
size_t tc_join_partial_bytes(const TcJoinArgs& g);
// Launch it (and the ordered sum of the K-range partials); *launches receives 1 or 2.
// err_word / wait_limit / stall as in TcStep.
cudaError_t tc_join_launch(const TcJoinArgs& g, int* exps, void* scratch, cudaStream_t st, int* launches);
// One line for the programme's explain output.
std::string tc_join_describe(const TcJoinArgs& g);

}  // namespace qxg
