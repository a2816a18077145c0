// Final joins of a sliced, bitstring-batched contraction tree on the tensor cores (3xTF32).
//
//     C[b, i, j] = sum_k P[b, k, i] Q[b, k, j]
// with 32 free values i of one operand (P), NQ = 8..32 free values j of the other (Q), 2^10 to
// 2^25 summed terms per batch value b, and both operands of 2^28 to 2^33 elements.  Every operand
// element is used by 32 or NQ results only, so the step streams both operands once; the CUDA
// cores run out of FP32 issue before HBM does, and the tensor-core GEMM would first pack the
// smaller operand into planes four times its size.  Here the operands are split on the fly:
//
//   A (MMA M = 128 rows, tensor memory): row (role, i) of P's stack
//       role 0: hi(Re P | -Im P)   role 1: hi(Im P | Re P)   role 2 / 3: the lo parts of 0 / 1
//   B (MMA N = 2 NQ rows, shared memory): row j = hi(Re Q | Im Q), row NQ + j = lo(Re Q | Im Q)
//   D[(role, i), (h, j)] = sum over the chunk's terms of A . B          (FP32, tensor memory)
// so Re C[i, j] = sum over h of D[(0, i), (h, j)] + D[(2, i), (h, j)] and Im C from roles 1 and
// 3: the four hi/lo products of each complex product (lo*lo included) come from one M = 128,
// N = 2 NQ, K = 8 MMA per 8 summed terms, each in its own accumulator entry.  (hi, lo): tf32
// round-to-nearest (ties away) of x and of x - hi.  The row of role r for free value i sits at
// tensor-memory lane 32 q + 8 r + (i mod 8) with q = i / 8, so the warp that owns lanes
// 32 q .. 32 q + 31 holds all four roles of eight free values.
//
// One CTA (15 warps) per (batch value, K range):
//   warp 1         loader: per raw chunk of 64 summed terms, the chunk's P tile (32 x 64) and Q
//                  tile (NQ x 64) land in a ring slot in each operand's address order: one TMA
//                  tensor copy per operand (the tile's runs of address bits as box dimensions),
//                  or, where the layout does not fit a box, its contiguous segments by
//                  cp.async.bulk.  The chunk's six summed bits are planned so both tiles are runs
//                  of >= 8 elements;
//   warps 4-11     P splitters, two groups on alternate MMA stages (16 summed terms each): warp
//                  4 + 4 g + q reads the stage's terms for its eight free values from the slot,
//                  splits them into the four roles and stores 32 columns of its lanes with
//                  tcgen05.st.  Group 0 also drains: every `flush` stages (128 terms) each MMA
//                  issuer commits one of its accumulators and switches to the other; group 0
//                  adds the committed accumulators (h = hi and lo summed in FP32) into FP32 pairs
//                  in shared memory (Knuth's TwoSum) before the stage that reuses them, so the
//                  FP32 sums never run over more than 128 terms, and at the end combines the four
//                  roles with shuffles and writes C (or its FP64 partial, added in K-range order
//                  by tc_join_reduce_kernel);
//   warps 2-3, 12-13  Q splitters: a whole raw chunk at a time, each thread reading elements in the
//                  slot's order (consecutive threads, consecutive elements) and storing their
//                  four split words into the chunk's eight B tiles (K-major core matrices, 64-byte
//                  rows: real parts in core columns 0-1, imaginary in 2-3; the tiles 16 bytes
//                  apart in bank position), two chunks of B stages in flight;
//   warps 0, 14    MMA issuers, lane 0 of each on alternate stages into its own two accumulators
//                  (a thread issues about one small MMA per 200 cycles): four tcgen05.mma
//                  (kind::tf32, A from tensor memory) per stage and one commit, whose barrier frees
//                  the stage's B buffer and, four stages on, its A stage.
// Waiting warps sleep in their barrier polls (a suspend-time hint), so they leave the issue slots
// to the splitters.
// Every wait is bounded; a wait that gives up writes its code to the programme's error word, the
// CTA skips its remaining work, frees its tensor memory and returns.
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "tc_gemm.h"
#include "tc_ptx.h"

namespace qxg {
namespace {

constexpr int kJoinSub = 16;                        // summed terms per MMA stage
constexpr int kJoinSubs = kJoinKR / kJoinSub;       // MMA stages per raw chunk (4)
constexpr int kJoinStages = 4;                      // A stages in tensor memory
constexpr int kJoinQBufs = 2 * kJoinSubs;           // B stages in shared memory (two raw chunks)
static_assert(kJoinSubs == 4 && kJoinStages == 4 && kJoinQBufs == 8,
              "the kernel's loops index stages with shifts by 2 (4 per chunk, 4 A stages) and 3 (8 B stages)");
constexpr int kJoinMaxRing = 4;                     // raw chunks in the ring
constexpr int kJoinPGroups = 2;                     // P splitter groups (alternate stages)
constexpr int kJoinQWarps = 4;                      // Q splitter warps (2, 3 and the two after the P groups)
constexpr int kJoinQThreads = 32 * kJoinQWarps;
constexpr int kJoinIssuers = 2;                     // MMA issuing threads (alternate stages)
constexpr int kJoinThreads = 32 * (2 + kJoinQWarps + 4 * kJoinPGroups + (kJoinIssuers - 1));
static_assert(kJoinIssuers == 2 && kJoinPGroups == 2, "stage parity decides both the issuer and the P group");
constexpr uint32_t kJoinSleepNs = 2000;             // suspend hint of a barrier poll
constexpr int kJoinStageCols = 2 * kJoinSub;        // tensor-memory columns of one A stage (32)
constexpr int kJoinFlushTerms = 128;                // summed terms per FP32 accumulator
constexpr int kJoinChunkBits = 48;                  // delta-table entries (chunk index bits)
constexpr size_t kJoinSmemCap = 200 * 1024;         // ring + B stages + drained sums (one CTA per SM)
constexpr int kJoinPadBytes = 16;                   // padding after each bulk segment and each B tile
constexpr int kJoinMaxBulkSegs = 96;                // bulk segments per chunk above which the join declines
                                                    // (each cp.async.bulk costs ~70 cycles of the loader)

// Byte of tile element e inside a slot: segment e >> sb, element e mod 2^sb.
__host__ __device__ __forceinline__ int join_slot_byte(int64_t e, int sb, int stride) {
    return (int)((e >> sb) * stride + (e & ((int64_t(1) << sb) - 1)) * 8);
}
// ---- index work of the kernel, shared with its host emulation -----------------------------------
// Chunk bases walk in order: base(c + 1) = base(c) + delta(ctz(c + 1)).
__host__ __device__ __forceinline__ int64_t join_delta(const BitMap& h, int t) {
    return pdep(int64_t(1) << t, h) - pdep((int64_t(1) << t) - 1, h);
}
// Offsets of chunk c of K range si for batch value bi (the walk's first base and its check).
__host__ __device__ __forceinline__ int64_t join_base_p(const TcJoinArgs& g, int64_t bi, int64_t si, int64_t c) {
    return pdep(bi, g.bP) + pdep(si * g.nchunks + c, g.hP);
}
__host__ __device__ __forceinline__ int64_t join_base_q(const TcJoinArgs& g, int64_t bi, int64_t si, int64_t c) {
    return pdep(bi, g.bQ) + pdep(si * g.nchunks + c, g.hQ);
}
// Operand offset (from the chunk's base) of a raw chunk's segment sg.
__host__ __device__ __forceinline__ int64_t join_seg_p(const TcJoinArgs& g, int sg) {
    return pdep((int64_t)sg << g.sbP, g.eP);
}
__host__ __device__ __forceinline__ int64_t join_seg_q(const TcJoinArgs& g, int sg) {
    return pdep((int64_t)sg << g.sbQ, g.eQ);
}
// Slot bytes of P's free value i and summed index kl (they add), and of Q's j and kl.
__host__ __device__ __forceinline__ int join_prow(const TcJoinArgs& g, int i) {
    return join_slot_byte(pdep(i, g.tPi), g.sbP, g.segP_stride);
}
__host__ __device__ __forceinline__ int join_pcol(const TcJoinArgs& g, int kl) {
    return join_slot_byte(pdep(kl, g.tPk), g.sbP, g.segP_stride);
}
// Inverse of pdep: the index bits that the map deposits at x's bits.
__host__ __device__ __forceinline__ int64_t join_pext(int64_t x, const BitMap& m) {
    int64_t o = 0;
    for (int i = 0; i < m.n; i++) {
        const Run r = m.r[i];
        o |= ((x >> r.dst) & ((int64_t(1) << r.len) - 1)) << r.src;
    }
    return o;
}
// B tiles: 2 NQ rows of 64 bytes (one 8-term group), 16 bytes of padding after each.
__host__ __device__ __forceinline__ int join_qtile_bytes(int nq) { return 2 * nq * kTcChunkBytes + kJoinPadBytes; }
// Q's tile element e (in Q's address order): its slot byte (from the start of Q's part), and the
// byte of its hi real word in the chunk's eight B tiles -- tile 2 (kl / 16) + (kl / 8 mod 2),
// row j, core column (kl mod 8) / 4, word kl mod 4 (the imaginary word is 256 bytes further, the
// lo row NQ + j is NQ / 8 row groups further).  Both add over disjoint bits of e.
__host__ __device__ __forceinline__ int join_qsrc(const TcJoinArgs& g, int64_t e) {
    return join_slot_byte(e, g.sbQ, g.segQ_stride);
}
__host__ __device__ __forceinline__ int join_qdst(const TcJoinArgs& g, int64_t e) {
    const int j = (int)join_pext(e, g.tQj), kl = (int)join_pext(e, g.tQk);
    const int t = kl & 7;
    return (kl >> 3) * join_qtile_bytes(g.nq) + (j >> 3) * 512 + (t >> 2) * 128 + (j & 7) * 16 + (t & 3) * 4;
}
__host__ __device__ __forceinline__ int64_t join_c_offset(const TcJoinArgs& g, int64_t bi, int i, int j) {
    return pdep(bi, g.bC) + pdep(i, g.iC) + pdep(j, g.jC);
}

template <int NQ>
struct JoinShape {
    static constexpr int kQTile = 2 * NQ * kTcChunkBytes + kJoinPadBytes;   // B tile of 8 summed terms
    static constexpr int kQStage = 2 * kQTile;                 // B operand of one MMA stage
    static constexpr int kQLo = (NQ / 8) * 512;                // lo rows NQ + j: NQ / 8 row groups on
    static constexpr uint32_t kAccCols = 2 * NQ;               // columns of one accumulator
    static constexpr uint32_t kACol0 = 2 * kJoinIssuers * kAccCols;   // first A stage column
    static constexpr uint32_t kNeed = kACol0 + kJoinStages * kJoinStageCols;
    static constexpr uint32_t kCols = kNeed <= 128 ? 128 : (kNeed <= 256 ? 256 : 512);
};

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
// tf32 round to nearest, ties away from zero, on the binary32 bit pattern (finite x): add half a
// unit in the last place of the 10-bit mantissa (bit 12) and clear the 13 bits below it -- two
// integer operations.
__device__ __forceinline__ uint32_t tf32_bits(float x) { return (__float_as_uint(x) + 0x1000u) & 0xffffe000u; }

template <int NQ, bool SCALED>
__global__ void __launch_bounds__(kJoinThreads, 1)
    tc_join_kernel(const TcJoinArgs g, double2* partial, int* exps, const __grid_constant__ CUtensorMap mapP,
                   const __grid_constant__ CUtensorMap mapQ) {
    using S = JoinShape<NQ>;
    extern __shared__ uint8_t join_smem_raw[];
    // rfull / rempty per ring slot, fullA per A stage, qfull per B stage, sdone per B stage (the
    // MMAs of stage u done: u's B stage and, four stages on, its A stage are free), accf / acce per
    // accumulator, drain
    __shared__ uint64_t bars[2 * kJoinMaxRing + kJoinStages + 2 * kJoinQBufs + 4 * kJoinIssuers + 1];
    constexpr int kQPer = NQ * kJoinKR / kJoinQThreads;        // Q elements per splitter thread
    __shared__ int32_t prow[32], pcol[kJoinKR], qsrc_hi[kQPer], qdst_hi[kQPer];
    __shared__ int64_t psegoff[kJoinMaxSeg], qsegoff[kJoinMaxSeg];
    __shared__ int64_t dP[kJoinChunkBits], dQ[kJoinChunkBits];
    __shared__ uint32_t tmem_holder;
    __shared__ int abort_flag;
    // aligned by pointer arithmetic on the shared array (not through an integer), so the compiler
    // keeps the shared address space: shared loads and stores, not generic ones
    uint8_t* smem = join_smem_raw + ((128u - (smem_u32(join_smem_raw) & 127u)) & 127u);
    uint64_t* rfull = bars;
    uint64_t* rempty = bars + kJoinMaxRing;
    uint64_t* fullA = bars + 2 * kJoinMaxRing;
    uint64_t* qfull = fullA + kJoinStages;
    uint64_t* sdone = qfull + kJoinQBufs;
    uint64_t* accf = sdone + kJoinQBufs;    // [issuer][buffer]
    uint64_t* acce = accf + 2 * kJoinIssuers;
    uint64_t* drain = acce + 2 * kJoinIssuers;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int* const errw = g.err;
    const uint32_t wl = g.wait_limit ? g.wait_limit : kWaitLimit;
    const int64_t bi = (int64_t)blockIdx.x % g.nbatch;
    const int64_t si = (int64_t)blockIdx.x / g.nbatch;
    // the host guarantees these; never index past the ring or the segment tables
    const bool bad = g.ring < 2 || g.ring > kJoinMaxRing || g.nsegP > kJoinMaxSeg || g.nsegQ > kJoinMaxSeg ||
                     g.flush < 1 || (g.flush & (g.flush - 1)) != 0 || g.flush % kJoinPGroups != 0 || g.nq != NQ;
    const int R = g.ring;
    uint8_t* ring = smem;
    uint8_t* qst = smem + (size_t)R * g.slot_bytes;
    const int64_t nchunks = bad ? 0 : g.nchunks;
    const int64_t U = nchunks * kJoinSubs;                      // MMA stages of this CTA
    // flush is a power of two: shifts and masks, no 64-bit divisions in the loops
    const int fsh = bad ? 0 : __ffs(g.flush) - 1;
    const int64_t fmask = (int64_t(1) << fsh) - 1;
    const int64_t V = bad ? 0 : (U + fmask) >> fsh;             // accumulator drains

    if (threadIdx.x == 0) {
        for (int r = 0; r < kJoinMaxRing; r++) {
            mbar_init(&rfull[r], 1u);
            mbar_init(&rempty[r], (uint32_t)(kJoinQWarps + 4 * kJoinPGroups));
        }
        for (int s = 0; s < kJoinStages; s++) mbar_init(&fullA[s], 4u);
        for (int s = 0; s < kJoinQBufs; s++) { mbar_init(&qfull[s], (uint32_t)kJoinQWarps); mbar_init(&sdone[s], 1u); }
        for (int j = 0; j < 2 * kJoinIssuers; j++) { mbar_init(&accf[j], 1u); mbar_init(&acce[j], 4u); }
        mbar_init(drain, (uint32_t)kJoinIssuers);
        abort_flag = 0;
        if (bad) atomicExch(errw, 10);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_holder)),
                     "r"(S::kCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (!bad) {
        for (int t = threadIdx.x; t < kJoinKR; t += kJoinThreads) pcol[t] = join_pcol(g, t);
        for (int t = threadIdx.x; t < 32; t += kJoinThreads) prow[t] = join_prow(g, t);
        for (int t = threadIdx.x; t < kQPer; t += kJoinThreads) {
            qsrc_hi[t] = join_qsrc(g, (int64_t)t * kJoinQThreads);
            qdst_hi[t] = join_qdst(g, (int64_t)t * kJoinQThreads);
        }
        for (int t = threadIdx.x; t < g.nsegP; t += kJoinThreads) psegoff[t] = join_seg_p(g, t);
        for (int t = threadIdx.x; t < g.nsegQ; t += kJoinThreads) qsegoff[t] = join_seg_q(g, t);
        for (int t = threadIdx.x; t < kJoinChunkBits; t += kJoinThreads) {
            dP[t] = join_delta(g.hP, t);
            dQ[t] = join_delta(g.hQ, t);
        }
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = tmem_holder;

    auto wait = [&](uint64_t* bar, uint32_t parity) { return mbar_wait_sleep(bar, parity, wl, kJoinSleepNs); };
    auto give_up = [&](int code) { atomicExch(&abort_flag, 1); atomicExch(errw, code); };
    auto aborted = [&]() { return __any_sync(0xffffffffu, *(volatile int*)&abort_flag != 0); };
    if (warp == 1) {
        // loader: chunk c into slot c mod R once the splitters have released it
        const bool stall = g.stall != 0 && blockIdx.x == 0;   // test hook: its waits run out
        const int64_t c0 = si * nchunks;
        // the chunk's offset below the batch bits (a TMA box's dimension-0 coordinate) and the
        // batch value's offset
        const int64_t bP0 = pdep(bi, g.bP), bQ0 = pdep(bi, g.bQ);
        int64_t chP = join_base_p(g, bi, si, 0) - bP0, chQ = join_base_q(g, bi, si, 0) - bQ0;
        const uint32_t segP = 8u << g.sbP, segQ = 8u << g.sbQ;
        const uint32_t tx = (uint32_t)g.nsegP * segP + (uint32_t)g.nsegQ * segQ;
        int slot = 0;
        uint32_t ph = 0;
        int64_t issued = 0;
        for (int64_t c = 0; c < (stall ? 0 : nchunks); c++) {
            const bool ok = wait(&rempty[slot], ph ^ 1u);
            if (!__all_sync(0xffffffffu, ok)) {
                if (lane == 0) give_up(11);
                break;
            }
            if (aborted()) break;
            uint8_t* dst = ring + (size_t)slot * g.slot_bytes;
            if (lane == 0) mbar_expect_tx(&rfull[slot], tx);
            __syncwarp();
            if (g.tma) {
                if (lane == 0) {
                    int co[5] = {(int)chP, 0, 0, 0, 0};
                    if (g.boxP.tb >= 0) co[g.boxP.tb] = (int)(bP0 >> g.boxP.th);
                    tma_load_5d(dst, &mapP, co, &rfull[slot]);
                    int cq[5] = {(int)chQ, 0, 0, 0, 0};
                    if (g.boxQ.tb >= 0) cq[g.boxQ.tb] = (int)(bQ0 >> g.boxQ.th);
                    tma_load_5d(dst + g.slotP_bytes, &mapQ, cq, &rfull[slot]);
                }
            } else {
                for (int sg = lane; sg < g.nsegP; sg += 32)
                    bulk_copy(dst + sg * g.segP_stride, g.P + bP0 + chP + psegoff[sg], segP, &rfull[slot]);
                for (int sg = lane; sg < g.nsegQ; sg += 32)
                    bulk_copy(dst + g.slotP_bytes + sg * g.segQ_stride, g.Q + bQ0 + chQ + qsegoff[sg], segQ,
                              &rfull[slot]);
            }
            issued++;
            const int t = __ffsll((unsigned long long)(c0 + c + 1)) - 1;
            if (c + 1 < nchunks) {
                chP += dP[t];
                chQ += dQ[t];
            }
            if (++slot == R) { slot = 0; ph ^= 1u; }
        }
        // copies still in flight (only after an abort) must land before the CTA leaves
        if (lane == 0)
            for (int64_t q = issued - 1; q >= 0 && q >= issued - R; q--)
                mbar_wait(&rfull[q % R], (uint32_t)((q / R) & 1));     // full limit: copies must land
    } else if (warp == 2 || warp == 3 || (warp >= 4 + 4 * kJoinPGroups && warp < 4 + 4 * kJoinPGroups + kJoinQWarps - 2)) {
        // Q splitters: a raw chunk at a time; thread tq takes the chunk's elements tq + 128 m (in
        // the slot's order) and stores their split words into the chunk's B stages 4 (c mod 2) ..
        const int tq = (warp < 4 ? warp - 2 : warp - 2 - 4 * kJoinPGroups) * 32 + lane;
        float s = 1.f;
        if (SCALED) s = pow2f(-read_m(exps, g.expQ));
        const float si_ = g.conjQ ? -s : s;
        const int src0 = g.slotP_bytes + join_qsrc(g, tq), dst0 = join_qdst(g, tq);
        int slot = 0;                       // ring slot of chunk c and its phase
        uint32_t rph = 0;
        for (int64_t c = 0; c < nchunks; c++) {
            bool ok = wait(&rfull[slot], rph);
            // the chunk's B stages are free once the MMAs of the stages two chunks back are done
            for (int sb = 0; sb < kJoinSubs && ok; sb++) {
                const int64_t u = c * kJoinSubs + sb;
                if (u >= kJoinQBufs) ok = wait(&sdone[u & (kJoinQBufs - 1)], (uint32_t)(((u - kJoinQBufs) >> 3) & 1));
            }
            if (!__all_sync(0xffffffffu, ok)) {
                if (lane == 0) give_up(12);
                break;
            }
            if (aborted()) break;
            const uint8_t* raw = ring + (size_t)slot * g.slot_bytes + src0;
            uint8_t* qb = qst + (size_t)(c & 1) * (2 * kJoinSubs) * S::kQTile + dst0;
            // eight elements' loads before their stores (the stores could alias later loads)
            constexpr int kQB = kQPer < 8 ? kQPer : 8;
#pragma unroll 1
            for (int m0 = 0; m0 < kQPer; m0 += kQB) {
                float2 v[kQB];
                int dd[kQB];
#pragma unroll
                for (int r = 0; r < kQB; r++) {
                    v[r] = *reinterpret_cast<const float2*>(raw + qsrc_hi[m0 + r]);
                    dd[r] = qdst_hi[m0 + r];
                }
#pragma unroll
                for (int r = 0; r < kQB; r++) {
                    const float re = v[r].x * s, im = v[r].y * si_;
                    const uint32_t hr = tf32_bits(re), hm = tf32_bits(im);
                    const uint32_t lr = tf32_bits(re - __uint_as_float(hr)), lm = tf32_bits(im - __uint_as_float(hm));
                    uint8_t* d = qb + dd[r];
                    *reinterpret_cast<uint32_t*>(d) = hr;
                    *reinterpret_cast<uint32_t*>(d + 256) = hm;
                    *reinterpret_cast<uint32_t*>(d + S::kQLo) = lr;
                    *reinterpret_cast<uint32_t*>(d + S::kQLo + 256) = lm;
                }
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncwarp();
            if (lane == 0) {
                for (int sb = 0; sb < kJoinSubs; sb++) mbar_arrive(&qfull[(c * kJoinSubs + sb) & (kJoinQBufs - 1)]);
                mbar_arrive(&rempty[slot]);
            }
            if (++slot == R) { slot = 0; rph ^= 1u; }
        }
    } else if (warp >= 4 && warp < 4 + 4 * kJoinPGroups) {
        // P splitters: group pg takes the stages u = pg mod kJoinPGroups; warp 4 pg + q stores the
        // tensor-memory lanes 32 q .. 32 q + 31 (roles 0-3 of free values 8 q .. 8 q + 7).  Group 0
        // also drains: accumulator v is added into FP32 register pairs just before the stage that
        // starts interval v + 2 (which reuses it) is written -- its MMAs finished several stages
        // earlier -- and the last two at the end.
        const int pg = (warp - 4) >> 2, q4 = warp & 3, role = lane >> 3;
        const uint32_t lane_base = tmem + ((uint32_t)(32 * q4) << 16);
        float s = 1.f;
        if (SCALED) s = pow2f(-read_m(exps, g.expP));
        const float si_ = g.conjP ? -s : s;
        // (x0, x1) = (re, -im) for roles 0 and 2, (im, re) for roles 1 and 3; lo parts for 2 and 3
        const float a0 = (role & 1) ? 0.f : s, b0 = (role & 1) ? si_ : 0.f;
        const float a1 = (role & 1) ? s : 0.f, b1 = (role & 1) ? 0.f : -si_;
        const bool lo = role >= 2;
        const int rb = prow[q4 * 8 + (lane & 7)];
        int pc[kJoinSub];                   // slot bytes of the terms within a stage
#pragma unroll
        for (int t = 0; t < kJoinSub; t++) pc[t] = pcol[t];
        // the drained sums as unevaluated FP32 pairs (hi + lo), added with Knuth's TwoSum: about 48
        // bits of precision without the FP64 pipe, which GB300 runs at a small fraction of FP32.
        // They live in shared memory ([quadrant][j][lane]: a warp's lanes on consecutive words), so
        // the splitters keep their registers for loads in flight.
        float2* accs = reinterpret_cast<float2*>(qst + (size_t)kJoinQBufs * S::kQStage) + q4 * NQ * 32 + lane;
        if (pg == 0)
            for (int j = 0; j < NQ; j++) accs[j * 32] = make_float2(0.f, 0.f);
        auto two_sum = [](float2& a, float x) {
            const float t = a.x + x, bp = t - a.x;
            a.y += (a.x - (t - bp)) + (x - bp);
            a.x = t;
        };
        int64_t drained = 0;
        auto drain_acc = [&](int64_t v) -> bool {
            const uint32_t buf = (uint32_t)(v & 1);
            bool ok = true;
            for (int k = 0; k < kJoinIssuers && ok; k++) ok = wait(&accf[2 * k + buf], (uint32_t)((v >> 1) & 1));
            fence_after();
            if (!__all_sync(0xffffffffu, ok)) {
                if (lane == 0) give_up(16);
                return false;
            }
            // the issuers' accumulators of this interval (hi and lo rows of Q) summed in FP32
            auto col = [&](int k, uint32_t c) { return lane_base + (uint32_t)(2 * k + buf) * S::kAccCols + c; };
            if constexpr (NQ >= 16) {
#pragma unroll
                for (int j0 = 0; j0 < NQ; j0 += 16) {
                    float x[16];
#pragma unroll
                    for (int j = 0; j < 16; j++) x[j] = 0.f;
#pragma unroll
                    for (int k = 0; k < kJoinIssuers; k++) {
                        uint32_t hi[16], lo16[16];
                        tmem_ld16(col(k, j0), hi);
                        tmem_ld16(col(k, NQ + j0), lo16);
                        tmem_wait_ld();
#pragma unroll
                        for (int j = 0; j < 16; j++) x[j] += __uint_as_float(hi[j]) + __uint_as_float(lo16[j]);
                    }
#pragma unroll
                    for (int j = 0; j < 16; j++)
                        if (j0 + j < NQ) {
                            float2 a = accs[(j0 + j) * 32];
                            two_sum(a, x[j]);
                            accs[(j0 + j) * 32] = a;
                        }
                }
            } else {
                float x[NQ];
#pragma unroll
                for (int j = 0; j < NQ; j++) x[j] = 0.f;
#pragma unroll
                for (int k = 0; k < kJoinIssuers; k++) {
                    uint32_t w[16];         // hi columns 0 .. NQ-1, lo columns NQ .. 2NQ-1
                    tmem_ld16(col(k, 0), w);
                    tmem_wait_ld();
#pragma unroll
                    for (int j = 0; j < NQ; j++) x[j] += __uint_as_float(w[j]) + __uint_as_float(w[NQ + j]);
                }
#pragma unroll
                for (int j = 0; j < NQ; j++) {
                    float2 a = accs[j * 32];
                    two_sum(a, x[j]);
                    accs[j * 32] = a;
                }
            }
            // the accumulators may be overwritten once all four warps' loads have completed
            fence_before();
            __syncwarp();
            if (lane == 0)
                for (int k = 0; k < kJoinIssuers; k++) mbar_arrive(&acce[2 * k + buf]);
            return true;
        };
        bool ok_all = true;
        int slot = 0;                       // ring slot of the current chunk and its phase
        uint32_t rph = 0;
        for (int64_t u = pg; u < U; u += kJoinPGroups) {
            const int sub = (int)(u & (kJoinSubs - 1)), st = (int)(u & (kJoinStages - 1));
            if (pg == 0 && (u & fmask) == 0 && (u >> fsh) >= 2) {
                if (!drain_acc(drained)) { ok_all = false; break; }
                drained++;
            }
            bool ok = sub != pg || wait(&rfull[slot], rph);
            // the A stage is free once the MMAs of stage u - 4 are done
            if (u >= kJoinStages) ok = ok && wait(&sdone[(u - kJoinStages) & (kJoinQBufs - 1)], (uint32_t)(((u - kJoinStages) >> 3) & 1));
            if (!__all_sync(0xffffffffu, ok)) {
                if (lane == 0) give_up(13);
                ok_all = false;
                break;
            }
            if (aborted()) { ok_all = false; break; }
            fence_after();                  // the MMAs that read this A stage have completed
            const uint8_t* raw = ring + (size_t)slot * g.slot_bytes + rb + pcol[sub * kJoinSub];
            // all sixteen loads first, then each 8-term group's 16 words and its tensor-memory store
            float2 v[kJoinSub];
#pragma unroll
            for (int t = 0; t < kJoinSub; t++) v[t] = *reinterpret_cast<const float2*>(raw + pc[t]);
            const uint32_t ta = lane_base + S::kACol0 + (uint32_t)st * kJoinStageCols;
#pragma unroll
            for (int h8 = 0; h8 < 2; h8++) {
                uint32_t w[16];
#pragma unroll
                for (int t = 0; t < 8; t++) {
                    const float2 x = v[8 * h8 + t];
                    const float x0 = fmaf(x.x, a0, x.y * b0), x1 = fmaf(x.x, a1, x.y * b1);
                    const uint32_t h0 = tf32_bits(x0), h1 = tf32_bits(x1);
                    const uint32_t l0 = tf32_bits(x0 - __uint_as_float(h0)), l1 = tf32_bits(x1 - __uint_as_float(h1));
                    w[t] = lo ? l0 : h0;
                    w[8 + t] = lo ? l1 : h1;
                }
                tmem_st16(ta + 16 * h8, w);
            }
            tmem_wait_st();
            fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&fullA[st]);
            if (sub + kJoinPGroups >= kJoinSubs) {      // this group's last stage of the chunk
                __syncwarp();
                if (lane == 0) mbar_arrive(&rempty[slot]);
                if (++slot == R) { slot = 0; rph ^= 1u; }
            }
        }
        if (pg == 0) {
            for (; ok_all && drained < V; drained++) {
                if (aborted() || !drain_acc(drained)) break;
            }
            // roles 0 + 2 give Re C, 1 + 3 Im C; lanes 0-7 write free values 8 q .. 8 q + 7
            const int i = q4 * 8 + (lane & 7);
            int emax = kExpUnset;
#pragma unroll
            for (int j = 0; j < NQ; j++) {
                const float2 a = accs[j * 32];
                double x = (double)a.x + (double)a.y;
                x += __shfl_xor_sync(0xffffffffu, x, 16);
                const double im = __shfl_down_sync(0xffffffffu, x, 8);
                if (lane < 8) {
                    if (g.nsplit == 1) {
                        const float2 r = make_float2((float)x, (float)im);
                        g.C[join_c_offset(g, bi, i, j)] = r;
                        const float mx = fmaxf(fabsf(r.x), fabsf(r.y));
                        if (SCALED && mx > 0.f) emax = max(emax, exp_of(mx));
                    } else {
                        partial[((si * g.nbatch + bi) * 32 + i) * NQ + j] = make_double2(x, im);
                    }
                }
            }
            if (SCALED && g.nsplit == 1) {
                if (blockIdx.x == 0 && warp == 4 && lane == 0)
                    exps[2 * g.expC] = exps[2 * g.expP] + exps[2 * g.expQ] + read_m(exps, g.expP) + read_m(exps, g.expQ);
                for (int o = 16; o > 0; o >>= 1) emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, o));
                if (lane == 0 && emax != kExpUnset) atomicMax(&exps[2 * g.expC + 1], emax);
            }
        }
    } else if (lane == 0 && (warp == 0 || warp >= kJoinThreads / 32 - (kJoinIssuers - 1))) {
        // MMA issuer k takes the stages u = k mod kJoinIssuers into its own two accumulators
        const int k = warp == 0 ? 0 : warp - (kJoinThreads / 32 - kJoinIssuers);
        const int64_t fm = fmask;
        for (int64_t u = k; u < U; u += kJoinIssuers) {
            const int64_t v = u >> fsh;
            const uint32_t buf = (uint32_t)(v & 1);
            const int st = (int)(u & (kJoinStages - 1));
            const bool first = (u & fm) == k;
            if (first) {
                if (!wait(&acce[2 * k + buf], (uint32_t)((v >> 1) & 1) ^ 1u)) { give_up(14); break; }
                fence_after();
            }
            if (!wait(&fullA[st], (uint32_t)((u >> 2) & 1)) ||
                !wait(&qfull[u & (kJoinQBufs - 1)], (uint32_t)((u >> 3) & 1))) {
                give_up(15);
                break;
            }
            fence_after();
            const uint32_t d = tmem + (uint32_t)(2 * k + buf) * S::kAccCols;
            const uint32_t ta = tmem + S::kACol0 + (uint32_t)st * kJoinStageCols;
            const uint32_t qb = smem_u32(qst + (size_t)(u & (kJoinQBufs - 1)) * S::kQStage);
#pragma unroll
            for (int ks = 0; ks < kJoinSub / 4; ks++) {
                const uint64_t db = smem_desc(qb + (ks >> 1) * S::kQTile + (ks & 1) * 256);
                mma_ts<true>(d, ta + ks * 8, db, g.idesc, (first && ks == 0) ? 0u : 1u);
            }
            mma_commit(&sdone[u & (kJoinQBufs - 1)]);
            if ((u & fm) == fm - (kJoinIssuers - 1) + k || u + kJoinIssuers >= U) mma_commit(&accf[2 * k + buf]);
        }
        // the MMAs must have finished before the tensor memory is freed
        mma_commit(drain);
        mbar_wait(drain, 0);                // full limit: the MMAs must finish
    }
    fence_before();
    __syncthreads();
    if (warp == 0) {
        fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(S::kCols) : "memory");
    }
}

// C from the K-range partials, summed in range order (deterministic).
template <int NQ, bool SCALED>
__global__ void tc_join_reduce_kernel(const TcJoinArgs g, const double2* partial, int* exps) {
    const int64_t per = 32 * NQ, total = g.nbatch * per;
    int emax = kExpUnset;
    if (SCALED && blockIdx.x == 0 && threadIdx.x == 0)
        exps[2 * g.expC] = exps[2 * g.expP] + exps[2 * g.expQ] + read_m(exps, g.expP) + read_m(exps, g.expQ);
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        double re = 0.0, im = 0.0;
        for (int s = 0; s < g.nsplit; s++) {
            const double2 v = partial[s * total + idx];
            re += v.x;
            im += v.y;
        }
        const int64_t b = idx / per, r = idx % per;
        const float2 c = make_float2((float)re, (float)im);
        g.C[join_c_offset(g, b, (int)(r / NQ), (int)(r % NQ))] = c;
        const float mx = fmaxf(fabsf(c.x), fabsf(c.y));
        if (SCALED && mx > 0.f) emax = max(emax, exp_of(mx));
    }
    if (SCALED) {
        for (int o = 16; o > 0; o >>= 1) emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, o));
        if ((threadIdx.x & 31) == 0 && emax != kExpUnset) atomicMax(&exps[2 * g.expC + 1], emax);
    }
}

int join_ilog2(int64_t x) {
    int b = 0;
    while ((int64_t(1) << b) < x) b++;
    return b;
}

// Ring, B stages, and the drained sums (128 lanes x NQ FP32 pairs).
size_t join_smem_bytes(const TcJoinArgs& g) {
    return (size_t)g.ring * g.slot_bytes + (size_t)kJoinQBufs * 2 * join_qtile_bytes(g.nq) + (size_t)128 * g.nq * 8 + 128;
}

// Slot layout for the copy mode: TMA boxes land densely, bulk segments with 16 bytes of padding
// each (they spread the splitters' reads over the banks); the ring takes as many raw chunks
// (2..4) as fit beside the B stages.
bool join_layout(TcJoinArgs& a, bool tma) {
    a.tma = tma ? 1 : 0;
    const int pad = tma ? 0 : kJoinPadBytes;
    a.segP_stride = (8 << a.sbP) + pad;
    a.segQ_stride = (8 << a.sbQ) + pad;
    a.slotP_bytes = (a.nsegP * a.segP_stride + 127) / 128 * 128;
    a.slot_bytes = a.slotP_bytes + (a.nsegQ * a.segQ_stride + 127) / 128 * 128;
    const size_t stages = (size_t)kJoinQBufs * 2 * join_qtile_bytes(a.nq) + (size_t)128 * a.nq * 8;
    a.ring = 0;
    for (int r = kJoinMaxRing; r >= 2 && !a.ring; r--)
        if ((size_t)r * a.slot_bytes + stages <= kJoinSmemCap) a.ring = r;
    return a.ring != 0;
}

// One operand's tile (address positions `tile`, ascending, the lowest run starting at bit 0) as a
// TMA box, when its batch bits (positions `batch`) are contiguous above every other bit of the
// operand (maxnb: the highest non-batch position) and five dimensions suffice.
bool join_box(const std::vector<int>& tile, std::vector<int> batch, int maxnb, JoinBox* b) {
    memset(b, 0, sizeof(*b));
    std::sort(batch.begin(), batch.end());
    const int H = batch.empty() ? maxnb + 1 : batch[0];
    for (size_t i = 0; i < batch.size(); i++)
        if (batch[i] != H + (int)i) return false;
    if (maxnb >= H || H > 31) return false;
    b->th = H;
    std::vector<std::pair<int, int>> runs;  // (position, length)
    for (int p : tile) {
        if (!runs.empty() && runs.back().first + runs.back().second == p) runs.back().second++;
        else runs.push_back({p, 1});
    }
    if (runs.empty() || runs[0].first != 0) return false;
    int nd = 0;
    auto add = [&](int64_t dim, int64_t stride, int box) {
        if (nd >= 5) return false;
        b->dim[nd] = dim;
        b->stride[nd] = stride;
        b->box[nd] = box;
        nd++;
        return true;
    };
    // dimension 0: the leading run (up to 8 bits of it), extent 2^H for the chunk's offset
    const int l0 = std::min(runs[0].second, 8);
    if (!add(int64_t(1) << H, 1, 1 << l0)) return false;
    std::vector<std::pair<int, int>> rest;
    if (runs[0].second > l0) rest.push_back({l0, runs[0].second - l0});
    for (size_t r = 1; r < runs.size(); r++) rest.push_back(runs[r]);
    for (const auto& pr : rest)
        for (int pos = pr.first, len = pr.second; len > 0;) {
            const int l = std::min(len, 8);
            if (!add(int64_t(1) << l, int64_t(1) << pos, 1 << l)) return false;
            pos += l;
            len -= l;
        }
    b->tb = -1;
    if (!batch.empty()) {
        b->tb = nd;
        if (!add(int64_t(1) << batch.size(), int64_t(1) << H, 1)) return false;
    }
    b->td = nd;
    return true;
}

// The box's tensor map over the operand at `base` (8-byte elements; unused dimensions of extent 1).
bool join_map(const JoinBox& b, const void* base, CUtensorMap* map) {
    const EncodeTiledFn encode = encode_tiled();
    if (!encode) return false;
    cuuint64_t dims[5], strides[4];
    cuuint32_t box[5], estr[5] = {1, 1, 1, 1, 1};
    for (int d = 0; d < 5; d++) {
        dims[d] = d < b.td ? (cuuint64_t)b.dim[d] : 1;
        box[d] = d < b.td ? (cuuint32_t)b.box[d] : 1;
        if (d > 0) strides[d - 1] = d < b.td ? (cuuint64_t)(8 * b.stride[d]) : (cuuint64_t)(8ll << 36);
    }
    return encode(map, CU_TENSOR_MAP_DATA_TYPE_UINT64, 5, const_cast<void*>(base), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int NQ, bool SCALED>
cudaError_t launch_join_shape(const TcJoinArgs& g, double2* partial, int* exps, cudaStream_t st,
                              const CUtensorMap& mp, const CUtensorMap& mq) {
    static bool attr = false;               // the kernel's dynamic shared memory limit, once
    if (!attr) {
        const cudaError_t e = cudaFuncSetAttribute(tc_join_kernel<NQ, SCALED>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   (int)(kJoinSmemCap + 128));
        if (e != cudaSuccess) return e;
        attr = true;
    }
    tc_join_kernel<NQ, SCALED>
        <<<(unsigned)(g.nbatch * g.nsplit), kJoinThreads, join_smem_bytes(g), st>>>(g, partial, exps, mp, mq);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || g.nsplit == 1) return e;
    const int64_t total = g.nbatch * 32 * NQ;
    const int grid = (int)std::min<int64_t>((total + 255) / 256, 4096);
    tc_join_reduce_kernel<NQ, SCALED><<<grid, 256, 0, st>>>(g, partial, exps);
    return cudaGetLastError();
}

}  // namespace

// Plan: every result bit in P or Q or both (batch), every summed bit in both; 32 free values on
// the P side (the step's B when both sides have 32) and 8-32 on the Q side; at least 2^10 summed
// terms.  The chunk's six summed bits are chosen one at a time for whichever operand's run of
// contiguous tile bits (free bits and chosen summed bits from address bit 0 up) is shorter, so
// both tiles are copied as segments of 2^sb >= 8 elements.
bool tc_join_plan(const StepArgs& s, int sm_count, TcJoinArgs* out, int min_log2) {
    if (s.nk < 10 || s.nk - 6 >= kJoinChunkBits) return false;
    auto one = [](const BitMap& m, int bit) {
        const int64_t o = pdep(int64_t(1) << bit, m);
        return o ? __builtin_ctzll((unsigned long long)o) : -1;
    };
    const int ncb = join_ilog2(s.nC);
    std::vector<int> gb, ab, bb;             // result bits: batch, A only, B only
    for (int p = 0; p < ncb; p++) {
        const bool ia = one(s.cA, p) >= 0, ib = one(s.cB, p) >= 0;
        if (ia && ib) gb.push_back(p);
        else if (ia) ab.push_back(p);
        else if (ib) bb.push_back(p);
        else return false;
    }
    for (int j = 0; j < s.nk; j++)
        if (one(s.kA, j) < 0 || one(s.kB, j) < 0) return false;
    const int na = (int)ab.size(), nb = (int)bb.size(), ng = (int)gb.size();
    bool p_is_a;
    if (nb == 5 && na >= 3 && na <= 5) p_is_a = false;
    else if (na == 5 && nb >= 3 && nb <= 4) p_is_a = true;
    else return false;
    if (ng > 30) return false;
    const int nqb = p_is_a ? nb : na;
    if (ng + 5 + s.nk < min_log2 || ng + nqb + s.nk < min_log2) return false;
    const BitMap& cP = p_is_a ? s.cA : s.cB;
    const BitMap& cQ = p_is_a ? s.cB : s.cA;
    const BitMap& kP = p_is_a ? s.kA : s.kB;
    const BitMap& kQ = p_is_a ? s.kB : s.kA;
    const std::vector<int>& fP = p_is_a ? ab : bb;
    const std::vector<int>& fQ = p_is_a ? bb : ab;
    std::vector<char> freeP(64, 0), freeQ(64, 0);
    std::vector<int> kAtP(64, -1), kAtQ(64, -1), posP(s.nk), posQ(s.nk);
    for (int b : fP) freeP[one(cP, b)] = 1;
    for (int b : fQ) freeQ[one(cQ, b)] = 1;
    for (int k = 0; k < s.nk; k++) {
        posP[k] = one(kP, k);
        posQ[k] = one(kQ, k);
        kAtP[posP[k]] = k;
        kAtQ[posQ[k]] = k;
    }
    std::vector<char> chosen(s.nk, 0);
    auto run = [&](const std::vector<char>& fr, const std::vector<int>& kat) {
        int r = 0;
        while (r < 64 && (fr[r] || (kat[r] >= 0 && chosen[kat[r]]))) r++;
        return r;
    };
    std::vector<int> ks;
    for (int step = 0; step < 6; step++) {
        const int rp = run(freeP, kAtP), rq = run(freeQ, kAtQ);
        const int kp = rp < 64 ? kAtP[rp] : -1, kq = rq < 64 ? kAtQ[rq] : -1;
        int pick = -1;
        if (rp <= rq && kp >= 0) pick = kp;
        else if (kq >= 0) pick = kq;
        else if (kp >= 0) pick = kp;
        else
            for (int k = 0; k < s.nk; k++)
                if (!chosen[k] && (pick < 0 || std::min(posP[k], posQ[k]) < std::min(posP[pick], posQ[pick]))) pick = k;
        chosen[pick] = 1;
        ks.push_back(pick);
    }
    std::sort(ks.begin(), ks.end(), [&](int x, int y) { return posP[x] < posP[y]; });
    const int sbP = run(freeP, kAtP), sbQ = run(freeQ, kAtQ);
    const int tbP = 5 + 6, tbQ = nqb + 6;     // tile bits
    if (sbP < 3 || sbQ < 3 || tbP - sbP > 8 || tbQ - sbQ > 8) return false;
    TcJoinArgs a;
    memset(&a, 0, sizeof(a));
    a.nq = 1 << nqb;
    a.p_is_a = p_is_a ? 1 : 0;
    a.sbP = sbP;
    a.sbQ = sbQ;
    a.nsegP = 1 << (tbP - sbP);
    a.nsegQ = 1 << (tbQ - sbQ);
    // one TMA box per operand and chunk where the layouts allow it
    {
        auto box_of = [&](const BitMap& cm, const std::vector<int>& fr, const std::vector<int>& pos, JoinBox* b) {
            std::vector<int> tile, batch;
            int maxnb = 0;
            for (int f : fr) {
                tile.push_back(one(cm, f));
                maxnb = std::max(maxnb, one(cm, f));
            }
            for (int k = 0; k < s.nk; k++) maxnb = std::max(maxnb, pos[k]);
            for (int k : ks) tile.push_back(pos[k]);
            std::sort(tile.begin(), tile.end());
            for (int b2 : gb) batch.push_back(one(cm, b2));
            return join_box(tile, batch, maxnb, b);
        };
        const bool tma = box_of(cP, fP, posP, &a.boxP) && box_of(cQ, fQ, posQ, &a.boxQ);
        // without boxes the loader issues one bulk copy per segment: many small ones are slower
        // than the batched small GEMM
        if (!tma && a.nsegP + a.nsegQ > kJoinMaxBulkSegs) return false;
        if (!join_layout(a, tma)) return false;
    }
    a.run_p = 1 << sbP;
    a.run_q = 1 << sbQ;
    for (int t = 0; t < 6; t++) a.chunk_k[t] = ks[t];
    // tile element maps: the tile's bits in the operand's address order
    auto tile_maps = [&](const BitMap& cm, const std::vector<int>& fr, const std::vector<int>& pos, BitMap* e,
                         BitMap* ti, BitMap* tk) {
        struct Bit { int pos, kind, idx; };
        std::vector<Bit> bits;
        for (int i = 0; i < (int)fr.size(); i++) bits.push_back({one(cm, fr[i]), 0, i});
        for (int t = 0; t < 6; t++) bits.push_back({pos[ks[t]], 1, t});
        std::sort(bits.begin(), bits.end(), [](const Bit& x, const Bit& y) { return x.pos < y.pos; });
        std::vector<std::pair<int, int>> pe, pi, pk;
        for (int t = 0; t < (int)bits.size(); t++) {
            pe.push_back({t, bits[t].pos});
            (bits[t].kind == 0 ? pi : pk).push_back({bits[t].idx, t});
        }
        std::sort(pi.begin(), pi.end());
        std::sort(pk.begin(), pk.end());
        return make_runs(pe, e) && make_runs(pi, ti) && make_runs(pk, tk);
    };
    if (!tile_maps(cP, fP, posP, &a.eP, &a.tPi, &a.tPk)) return false;
    if (!tile_maps(cQ, fQ, posQ, &a.eQ, &a.tQj, &a.tQk)) return false;
    std::vector<std::pair<int, int>> bP, bQ, bC, iC, jC, hP, hQ;
    for (int i = 0; i < ng; i++) {
        bP.push_back({i, one(cP, gb[i])});
        bQ.push_back({i, one(cQ, gb[i])});
        bC.push_back({i, gb[i]});
    }
    for (int i = 0; i < 5; i++) iC.push_back({i, fP[i]});
    for (int j = 0; j < nqb; j++) jC.push_back({j, fQ[j]});
    // the chunk index walks the other summed bits, lowest operand address first
    std::vector<int> rest;
    for (int k = 0; k < s.nk; k++)
        if (!chosen[k]) rest.push_back(k);
    std::sort(rest.begin(), rest.end(), [&](int x, int y) {
        const int px = std::min(posP[x], posQ[x]), py = std::min(posP[y], posQ[y]);
        return px != py ? px < py : x < y;
    });
    for (int t = 0; t < (int)rest.size(); t++) {
        hP.push_back({t, posP[rest[t]]});
        hQ.push_back({t, posQ[rest[t]]});
    }
    if (!make_runs(bP, &a.bP) || !make_runs(bQ, &a.bQ) || !make_runs(bC, &a.bC) || !make_runs(iC, &a.iC) ||
        !make_runs(jC, &a.jC) || !make_runs(hP, &a.hP) || !make_runs(hQ, &a.hQ))
        return false;
    a.nbatch = int64_t(1) << ng;
    const int64_t chunks = int64_t(1) << (s.nk - 6);
    // K ranges: two CTAs' worth per SM at least, each range at least 16 chunks (1,024 terms)
    int64_t nsplit = 1;
    while (a.nbatch * nsplit < (int64_t)sm_count * 2 && chunks / (nsplit * 2) >= 16) nsplit *= 2;
    if (a.nbatch * nsplit > (int64_t(1) << 31) - 1) return false;
    a.nsplit = (int)nsplit;
    a.nchunks = chunks / nsplit;
    a.flush = kJoinFlushTerms / kJoinSub;
    const uint32_t nmma = (uint32_t)(2 * a.nq);
    a.idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((nmma >> 3) << 17) | ((uint32_t)(kTcTileM >> 4) << 24);
    a.P = static_cast<const float2*>(p_is_a ? s.A : s.B);
    a.Q = static_cast<const float2*>(p_is_a ? s.B : s.A);
    a.C = static_cast<float2*>(s.C);
    a.conjP = p_is_a ? s.conjA : s.conjB;
    a.conjQ = p_is_a ? s.conjB : s.conjA;
    a.expP = p_is_a ? s.expA : s.expB;
    a.expQ = p_is_a ? s.expB : s.expA;
    a.expC = s.expC;
    *out = a;
    return true;
}

size_t tc_join_partial_bytes(const TcJoinArgs& g) {
    return g.nsplit > 1 ? (size_t)g.nsplit * (size_t)g.nbatch * 32 * g.nq * sizeof(double2) : 0;
}

cudaError_t tc_join_launch(const TcJoinArgs& g0, int* exps, void* scratch, cudaStream_t st, int* launches) {
    TcJoinArgs g = g0;
    if (!g.err) return cudaErrorInvalidValue;
    if (g.nsplit > 1 && !scratch) return cudaErrorInvalidValue;
    // cp.async.bulk and TMA need 16-byte aligned sources
    if ((reinterpret_cast<uintptr_t>(g.P) & 15) != 0 || (reinterpret_cast<uintptr_t>(g.Q) & 15) != 0)
        return cudaErrorInvalidValue;
    alignas(64) CUtensorMap mp, mq;
    memset(&mp, 0, sizeof(mp));
    memset(&mq, 0, sizeof(mq));
    // the segments by cp.async.bulk where the driver rejects a box
    if (g.tma && !(join_map(g.boxP, g.P, &mp) && join_map(g.boxQ, g.Q, &mq)) && !join_layout(g, false))
        return cudaErrorInvalidValue;
    double2* partial = static_cast<double2*>(scratch);
    cudaError_t e = cudaErrorInvalidValue;
    switch (g.nq) {
        case 8:
            e = exps ? launch_join_shape<8, true>(g, partial, exps, st, mp, mq)
                     : launch_join_shape<8, false>(g, partial, exps, st, mp, mq);
            break;
        case 16:
            e = exps ? launch_join_shape<16, true>(g, partial, exps, st, mp, mq)
                     : launch_join_shape<16, false>(g, partial, exps, st, mp, mq);
            break;
        case 32:
            e = exps ? launch_join_shape<32, true>(g, partial, exps, st, mp, mq)
                     : launch_join_shape<32, false>(g, partial, exps, st, mp, mq);
            break;
        default: break;
    }
    if (launches) *launches = g.nsplit > 1 ? 2 : 1;
    return e;
}

std::string tc_join_describe(const TcJoinArgs& g) {
    std::string d = "tensor-core join 3xTF32 P=" + std::string(g.p_is_a ? "A" : "B") + " nq=" + std::to_string(g.nq) +
                    " batch=" + std::to_string(g.nbatch) + " ranges=" + std::to_string(g.nsplit) +
                    " chunks=" + std::to_string(g.nchunks) + " ring=" + std::to_string(g.ring) + " chunk_k=";
    for (int t = 0; t < 6; t++) d += (t ? "," : "") + std::string("k") + std::to_string(g.chunk_k[t]);
    d += " runs=" + std::to_string(g.run_p) + "/" + std::to_string(g.run_q) + " segments=" + std::to_string(g.nsegP) +
         "/" + std::to_string(g.nsegQ) + (g.tma ? " copies=tma" : " copies=bulk");
    return d;
}

}  // namespace qxg
