// Tensor-core path of the split-precision executors (see tc_gemm.h).
//
// Per contraction step:
//   pack (x2): gather an operand through its bit maps, scale by 2^-max exponent, split into hi/lo
//           planes and write them as tcgen05 K-major core-matrix tiles (no swizzle: 8 rows x 16
//           bytes per core matrix, 64-byte K chunks so 8-row groups are 512 bytes apart).  The
//           larger operand X becomes the MMA's A (M side); the smaller Y is written in the
//           complex-doubled form [[Re,-Im],[Im,Re]] as the MMA's B (N side);
//   gemm:   one CTA per (batch, 128-row M tile, N tile), two CTAs per SM.  A producer thread
//           streams the K chunks of the four planes into shared memory with cp.async.bulk (three
//           stages, mbarrier transaction counts); one thread issues tcgen05.mma (kind::f16 with
//           BF16 planes or kind::tf32) -- hi*hi, hi*lo, lo*hi per 32-byte K step -- into an FP32
//           accumulator in tensor memory; four epilogue warps read it with tcgen05.ld and scatter
//           the complex result through the result's bit map (offsets of the tile's columns are
//           tabulated in shared memory), raising the result's exponent slot.
// Every wait is bounded; a wait that gives up sets g_tc_error, the CTA skips its remaining work,
// frees its tensor memory and returns.
#include <cuda_bf16.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "tc_gemm.h"
#include "tc_ptx.h"

#include <cuda.h>

namespace qxg {

__device__ int g_tc_error = 0;

namespace {

// Operand paths of the GEMM kernel for the larger operand X.
constexpr int kModePlanes = 0;    // X packed into hi/lo planes beforehand, staged by cp.async.bulk
constexpr int kModeRows = 1;      // X rows gathered by 8-byte cp.async in the kernel, then split
constexpr int kModeBulk = 2;      // X's contiguous segments fetched by cp.async.bulk, then split
constexpr int kModeTmem = 3;      // as kModeRows, but the split A tiles go to tensor memory
constexpr int kModeTma = 4;       // X's blocks fetched by one TMA tensor copy each, split into tensor memory
// kModeTma runs two groups of four split warps (7-10 and 11-14) on alternate chunks
constexpr int threads_of(int mode) {
    return mode == kModePlanes ? 192 : (mode == kModeBulk ? 352 : (mode == kModeTma ? 480 : 320));
}
constexpr int kATmemCols = 32;    // tensor-memory columns of one A stage (hi and lo, 16 each)
constexpr int kMaxRing = 8;                              // raw X chunks in a gather ring
constexpr int kMaxStages = 6;                            // operand stages in shared memory
constexpr int kATileBytes = kTcTileM * kTcChunkBytes;    // 8 KB
constexpr int kKSteps = kTcChunkBytes / 32;              // MMA K steps (32 bytes each) per chunk
constexpr int kKTable = 4096;                            // k offsets tabulated by the pack kernel

struct PackArgs {
    const void* src;        // float2 operand
    void* hi;               // plane of hi parts
    void* lo;               // plane of lo parts
    BitMap mb, mr, mk;      // operand offset of batch / row (m or n) / k index
    int64_t rows, rows_pad, K, batch;
    int64_t kchunks, row_tiles;
    int tile_rows;          // 128 for X, 2*ntile_n for Y
    int ntile;              // Y only: complex columns per tile
    int slot_src;           // exponent slot of the operand
    int doubled;            // 1: complex-doubled Y form
    int exp_c, slot_other;  // Y pack writes exps[C] = e_x + e_y + m_x + m_y
    int conj;               // 1: pack the complex conjugate (adjoint steps)
};

struct GemmArgs {
    const void *a_hi, *a_lo, *b_hi, *b_lo;
    const float2* X;        // fused: the larger operand itself, gathered and split in the kernel
    BitMap xb, xm, xk;      // fused: X offset of batch / m / k index
    int64_t K;              // fused: complex extent of K
    int x_slot, x_conj;     // fused: X's exponent slot, conjugation
    float2* C;
    BitMap cb, cm, cn;
    int64_t M, N, mtiles, ntiles, kchunks, batch;
    int ntile;              // complex columns per N tile (16..64)
    int stages;             // operand stages (<= kMaxStages)
    int nbuf;               // accumulator buffers in tensor memory (1 or 2)
    int tmem_cols;          // tensor-memory columns allocated (a power of two >= 32)
    int ring_chunks;        // fused: raw X chunks in the gather ring (2 .. kMaxRing)
    int bfast;              // tile order: batch fastest (X's lowest address bit is a batch bit)
    // bulk gather: the (128 rows x KC k) block of X is nseg contiguous segments of 2^seg_bits
    // elements; segment s starts at X offset pdep(s, segmap) from the block's base and lands at
    // byte s * seg_stride of the ring slot (16 bytes of padding per segment spread the banks);
    // element (r, j) sits at byte rtab(r) + ktab(j) of the slot
    BitMap segmap, rowmap_c, kmap_c;
    int seg_bits, nseg, seg_stride, slot_bytes;
    // TMA gather: the block is one box of the tensor map; the tensor map's dimension tma_outer
    // walks X in steps of 2^tma_lead elements and is positioned at the block's base >> tma_lead
    int tma_lead, tma_outer, box_bytes;
    uint32_t b_tile_bytes;
    uint32_t idesc;
    int exp_c;
    int* exps;
    uint32_t wait_limit;    // mbarrier polls before a wait gives up
    int stall;              // test hook: CTA 0's operand producer issues nothing (its waits run out)
    int* err;               // word a wait that gives up writes its code to (nullptr: g_tc_error)
};

// One thread: one row, one 16-byte group g (0..1) of one K chunk: NE complex values of k, whose
// real parts go to column g and imaginary parts to column 2 + g.
template <bool TF32>
__global__ void pack_kernel(const PackArgs p, int* exps) {
    using S = Split<TF32>;
    using E = typename S::E;
    constexpr int NE = 16 / sizeof(E);          // elements per 16 bytes: 8 bf16 / 4 tf32
    constexpr int KC = 2 * NE;                  // complex k per chunk
    __shared__ int64_t ktab[kKTable];
    const float2* __restrict__ X = static_cast<const float2*>(p.src);
    uint8_t* __restrict__ hi = static_cast<uint8_t*>(p.hi);
    uint8_t* __restrict__ lo = static_cast<uint8_t*>(p.lo);
    const int64_t kt = p.K < kKTable ? p.K : kKTable;
    for (int64_t k = threadIdx.x; k < kt; k += blockDim.x) ktab[k] = pdep(k, p.mk);
    __syncthreads();
    const float s = pow2f(-read_m(exps, p.slot_src));
    const float si = p.conj ? -s : s;
    if (p.doubled && blockIdx.x == 0 && threadIdx.x == 0) {
        const int mo = read_m(exps, p.slot_other), my = read_m(exps, p.slot_src);
        exps[2 * p.exp_c] = exps[2 * p.slot_other] + exps[2 * p.slot_src] + mo + my;
    }
    const int64_t total = p.batch * p.kchunks * p.rows_pad * 2;
    const int64_t tile_bytes = (int64_t)p.tile_rows * kTcChunkBytes;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = t % p.rows_pad;
        int64_t rest = t / p.rows_pad;
        const int g = (int)(rest & 1);
        rest >>= 1;
        const int64_t c = rest % p.kchunks;
        const int64_t b = rest / p.kchunks;
        float re[NE], im[NE];
        const bool row_ok = r < p.rows;
        const int64_t base = row_ok ? pdep(b, p.mb) + pdep(r, p.mr) : 0;
#pragma unroll
        for (int j = 0; j < NE; j++) {
            const int64_t k = c * KC + g * NE + j;
            re[j] = 0.f; im[j] = 0.f;
            if (row_ok && k < p.K) {
                const float2 v = X[base + (k < kKTable ? ktab[k] : pdep(k, p.mk))];
                re[j] = v.x * s;
                im[j] = v.y * si;
            }
        }
        E hr[NE], lr[NE], hm[NE], lm[NE];
#pragma unroll
        for (int j = 0; j < NE; j++) { S::go(re[j], hr[j], lr[j]); S::go(im[j], hm[j], lm[j]); }
        if (!p.doubled) {
            const int64_t tile = (b * p.row_tiles + r / kTcTileM) * p.kchunks + c;
            const int row = (int)(r % kTcTileM);
            uint8_t* th = hi + tile * tile_bytes;
            uint8_t* tl = lo + tile * tile_bytes;
            st16(th + core_off(row, g), hr);
            st16(tl + core_off(row, g), lr);
            st16(th + core_off(row, 2 + g), hm);
            st16(tl + core_off(row, 2 + g), lm);
        } else {
            // B_op rows (0,n): [Re Y | -Im Y], (1,n): [Im Y | Re Y]
            E nhm[NE], nlm[NE];
#pragma unroll
            for (int j = 0; j < NE; j++) { S::go(-im[j], nhm[j], nlm[j]); }
            const int64_t tile = (b * p.row_tiles + r / p.ntile) * p.kchunks + c;
            const int n = (int)(r % p.ntile);
            uint8_t* th = hi + tile * tile_bytes;
            uint8_t* tl = lo + tile * tile_bytes;
            const int r0 = n, r1 = p.ntile + n;
            st16(th + core_off(r0, g), hr);
            st16(tl + core_off(r0, g), lr);
            st16(th + core_off(r0, 2 + g), nhm);
            st16(tl + core_off(r0, 2 + g), nlm);
            st16(th + core_off(r1, g), hm);
            st16(tl + core_off(r1, g), lm);
            st16(th + core_off(r1, 2 + g), hr);
            st16(tl + core_off(r1, 2 + g), lr);
        }
    }
}

// ---- PTX wrappers ------------------------------------------------------------------------------
// 8-byte asynchronous global -> shared copies (the fused X gather keeps several K chunks in flight
// without holding registers for them).
__device__ __forceinline__ void cp_async8(void* dst, const void* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// Fused operand staging: one thread takes row `row` of X's K chunk (2*NE complex values, already
// gathered into a raw ring slot), scales, splits and stores it into the stage's hi/lo A tiles
// (real parts in 16-byte columns 0-1, imaginary parts in 2-3).
// `get(i)` returns element i < 2*NE of the row's chunk from the raw shared-memory copy.
template <bool TF32, typename Get>
__device__ __forceinline__ void split_a_row(uint8_t* th, uint8_t* tl, int row, Get get, bool row_ok, int64_t k0,
                                            int64_t K, float s, float si) {
    using S = Split<TF32>;
    using E = typename S::E;
    constexpr int NE = 16 / sizeof(E);
#pragma unroll
    for (int g = 0; g < 2; g++) {
        float re[NE], im[NE];
#pragma unroll
        for (int j = 0; j < NE; j++) {
            const int64_t k = k0 + g * NE + j;
            re[j] = 0.f; im[j] = 0.f;
            if (row_ok && k < K) {
                const float2 v = get(g * NE + j);
                re[j] = v.x * s;
                im[j] = v.y * si;
            }
        }
        E hr[NE], lr[NE], hm[NE], lm[NE];
#pragma unroll
        for (int j = 0; j < NE; j++) { S::go(re[j], hr[j], lr[j]); S::go(im[j], hm[j], lm[j]); }
        st16(th + core_off(row, g), hr);
        st16(tl + core_off(row, g), lr);
        st16(th + core_off(row, 2 + g), hm);
        st16(tl + core_off(row, 2 + g), lm);
    }
}

// Split of one row's K chunk into the 32-bit words of its tensor-memory A columns: hi[0..7] /
// lo[0..7] hold the real parts, hi[8..15] / lo[8..15] the imaginary parts (TF32: one k per
// column; BF16: k pairs, the even k in the low half).
template <bool TF32, typename Get>
__device__ __forceinline__ void split_row_words(Get get, bool row_ok, int64_t k0, int64_t K, float s, float si,
                                                uint32_t (&hi)[16], uint32_t (&lo)[16]) {
    constexpr int KC = TF32 ? 8 : 16;
    float re[KC], im[KC];
#pragma unroll
    for (int j = 0; j < KC; j++) {
        re[j] = 0.f; im[j] = 0.f;
        if (row_ok && k0 + j < K) {
            const float2 v = get(j);
            re[j] = v.x * s;
            im[j] = v.y * si;
        }
    }
    if (TF32) {
#pragma unroll
        for (int j = 0; j < 8; j++) {
            Split<true>::go(re[j], hi[j], lo[j]);
            Split<true>::go(im[j], hi[8 + j], lo[8 + j]);
        }
    } else {
#pragma unroll
        for (int j = 0; j < 8; j++) {
            unsigned short h0, l0, h1, l1;
            Split<false>::go(re[2 * j], h0, l0);
            Split<false>::go(re[2 * j + 1], h1, l1);
            hi[j] = (uint32_t)h0 | ((uint32_t)h1 << 16);
            lo[j] = (uint32_t)l0 | ((uint32_t)l1 << 16);
            Split<false>::go(im[2 * j], h0, l0);
            Split<false>::go(im[2 * j + 1], h1, l1);
            hi[8 + j] = (uint32_t)h0 | ((uint32_t)h1 << 16);
            lo[8 + j] = (uint32_t)l0 | ((uint32_t)l1 << 16);
        }
    }
}

// Persistent warp-specialised GEMM: a CTA walks the tiles blockIdx.x, +gridDim.x, ... (N tile
// fastest, then M tile, then batch).  The operand stages form one ring across all of the CTA's
// tiles; the accumulator is double-buffered in tensor memory, so the epilogue of one tile runs
// while the MMAs of the next accumulate into the other buffer.
//   warp 0 lane 0   stages Y's planes (and X's planes, kModePlanes) with cp.async.bulk
//   warp 1 lane 0   issues tcgen05.mma into accumulator buffer (tile index & 1)
//   warps 2-5       epilogue: tcgen05.ld, add the correction accumulator, scatter into C
//   warps 6-9       (kModeRows) gather X's rows through a cp.async ring, split, store the A tiles
//                   (kModeTmem) the same, storing the split words into tensor memory
//   warp 6          (kModeBulk) fetch X's contiguous segments into a ring with cp.async.bulk
//   warps 7-10      (kModeBulk) split the ring's chunks and store the A tiles
template <bool TF32, int MODE>
__global__ void __launch_bounds__(threads_of(MODE), MODE == kModeTma ? 1 : 2)
    tc_gemm_kernel(const GemmArgs g, const __grid_constant__ CUtensorMap tmap) {
    constexpr bool FUSED = MODE != kModePlanes;
    constexpr bool ROWS = MODE == kModeRows || MODE == kModeTmem;
    constexpr bool A_TMEM = MODE == kModeTmem || MODE == kModeTma;
    constexpr bool SEGS = MODE == kModeBulk || MODE == kModeTma;     // loader warp 6 + split warps 7-10
    constexpr int KC = TF32 ? 8 : 16;            // complex k per 64-byte chunk
    constexpr int SPLIT0 = SEGS ? 224 : 192;   // first thread of the split warps
    int* const errw = g.err ? g.err : &g_tc_error;
    const uint32_t wl = g.wait_limit ? g.wait_limit : kWaitLimit;
    extern __shared__ uint8_t smem_raw[];
    // fullB[NS] (bulk bytes of a stage), fullA[NS] (fused: the four split warps), empty[NS],
    // accf[2], acce[2], drain (the MMA thread's last commit)
    __shared__ uint64_t bars[3 * kMaxStages + 5];
    __shared__ uint64_t rbars[2 * kMaxRing];     // bulk: ring slot full / empty
    __shared__ int64_t jtab[64];                 // C offsets of the columns inside an N tile
    __shared__ int64_t xkoff[KC];                // rows: X offsets of the k values inside a chunk
    __shared__ int64_t segoff[MODE == kModeBulk ? 128 : 1];   // bulk: X offsets of the segments
    __shared__ int32_t rtab[SEGS ? 128 : 1];     // bulk / TMA: slot bytes of row r
    __shared__ int32_t ktab[SEGS ? KC : 1];      // bulk / TMA: slot bytes of k index j
    __shared__ uint32_t tmem_holder;
    __shared__ int abort_flag;
    // aligned by pointer arithmetic on the shared array (not through an integer), so the compiler
    // keeps the shared address space: shared loads and stores, not generic ones
    uint8_t* smem = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);
    const int NS = g.stages;
    const uint32_t a_stage = A_TMEM ? 0u : 2u * kATileBytes;    // A tiles' bytes in a stage
    const uint32_t stage_bytes = a_stage + 2u * g.b_tile_bytes;
    uint64_t* fullB = bars;
    uint64_t* fullA = bars + kMaxStages;
    uint64_t* empty = bars + 2 * kMaxStages;
    uint64_t* accf = bars + 3 * kMaxStages;
    uint64_t* acce = accf + 2;
    uint64_t* drain = acce + 2;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t total = g.batch * g.mtiles * g.ntiles;
    const int64_t ntl = total > (int64_t)blockIdx.x ? (total - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    const uint32_t acc_cols = 4u * (uint32_t)g.ntile;      // main (Re|Im) + corrections (Re|Im)
    const uint32_t ncols = (uint32_t)g.tmem_cols;
    const uint32_t nbuf = (uint32_t)g.nbuf;
    const uint32_t a_col0 = nbuf * acc_cols;               // kModeTmem: first A stage column
    // tile counts stay below 2^31 (checked on the host), so 32-bit division suffices
    auto tile_of = [&](int64_t i, int64_t& b, int64_t& mt, int64_t& nt) {
        uint32_t t = (uint32_t)(blockIdx.x + i * (int64_t)gridDim.x);
        const uint32_t nts = (uint32_t)g.ntiles, mts = (uint32_t)g.mtiles, bs = (uint32_t)g.batch;
        if (g.bfast) {                      // neighbouring batches share X's sectors
            b = t % bs;
            t /= bs;
            nt = t % nts;
            mt = t / nts;
        } else {
            nt = t % nts;
            t /= nts;
            mt = t % mts;
            b = t / mts;
        }
    };

    if (threadIdx.x == 0) {
        for (int i = 0; i < NS; i++) { mbar_init(&fullB[i], 1u); mbar_init(&fullA[i], 4u); mbar_init(&empty[i], 1u); }
        for (int j = 0; j < 2; j++) { mbar_init(&accf[j], 1u); mbar_init(&acce[j], 4u); }
        mbar_init(drain, 1u);
        if (SEGS)
            for (int j = 0; j < g.ring_chunks; j++) { mbar_init(&rbars[j], 1u); mbar_init(&rbars[kMaxRing + j], 4u); }
        abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_holder)),
                     "r"(ncols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    // column j < ntile of N tile nt sits at pdep(nt * ntile, cn) + pdep(j, cn): ntile is a power
    // of two, so the two bit sets are disjoint
    if (warp >= 2 && warp < 6)
        for (int j = threadIdx.x - 64; j < g.ntile; j += 128) jtab[j] = pdep(j, g.cn);
    if (ROWS && threadIdx.x >= 192 && threadIdx.x < 192 + KC)
        xkoff[threadIdx.x - 192] = pdep(threadIdx.x - 192, g.xk);
    if (SEGS && threadIdx.x >= 224 && threadIdx.x < 224 + 128) {
        // byte of compact index c in a slot: segment c >> seg_bits, element c & (2^seg_bits - 1)
        const int r = threadIdx.x - 224;
        auto slot_byte = [&](int64_t c) {
            return (int32_t)((c >> g.seg_bits) * g.seg_stride + (c & ((int64_t(1) << g.seg_bits) - 1)) * 8);
        };
        rtab[r] = slot_byte(pdep(r, g.rowmap_c));
        if (r < KC) ktab[r] = slot_byte(pdep(r, g.kmap_c));
        if (MODE == kModeBulk)
            for (int sg = r; sg < g.nseg; sg += 128) segoff[sg] = pdep(sg, g.segmap);
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = tmem_holder;

    if (warp == 0 && lane == 0) {
        // operand producer: Y's (and unfused X's) planes for every (tile, chunk) in order
        int s = 0;                          // stage and its phase parity, advanced per chunk
        uint32_t ph = 0;
        int64_t issued = 0;
        // test hook: CTA 0 issues no copies, so the MMA issuer's first wait runs out
        const bool stall = g.stall != 0 && blockIdx.x == 0;
        for (int64_t i = 0; i < (stall ? 0 : ntl); i++) {
            int64_t b, mt, nt;
            tile_of(i, b, mt, nt);
            const int64_t a_tile0 = (b * g.mtiles + mt) * g.kchunks;
            const int64_t b_tile0 = (b * g.ntiles + nt) * g.kchunks;
            bool stop = false;
            for (int64_t c = 0; c < g.kchunks; c++) {
                if (!mbar_wait(&empty[s], ph ^ 1u, wl)) { atomicExch(&abort_flag, 1); atomicExch(errw, 1); stop = true; break; }
                if (*(volatile int*)&abort_flag) { stop = true; break; }
                uint8_t* st = smem + s * stage_bytes;
                mbar_expect_tx(&fullB[s], FUSED ? 2u * g.b_tile_bytes : stage_bytes);
                const int64_t ao = (a_tile0 + c) * kATileBytes, bo = (b_tile0 + c) * (int64_t)g.b_tile_bytes;
                if (!FUSED) {
                    bulk_copy(st, static_cast<const uint8_t*>(g.a_hi) + ao, kATileBytes, &fullB[s]);
                    bulk_copy(st + kATileBytes, static_cast<const uint8_t*>(g.a_lo) + ao, kATileBytes, &fullB[s]);
                }
                bulk_copy(st + a_stage, static_cast<const uint8_t*>(g.b_hi) + bo, g.b_tile_bytes, &fullB[s]);
                bulk_copy(st + a_stage + g.b_tile_bytes, static_cast<const uint8_t*>(g.b_lo) + bo,
                          g.b_tile_bytes, &fullB[s]);
                issued++;
                if (++s == NS) { s = 0; ph ^= 1u; }
            }
            if (stop) break;
        }
        // copies still in flight (only after an abort) must land before the CTA leaves
        for (int64_t q = issued - 1; q >= 0 && q >= issued - NS; q--)
            mbar_wait(&fullB[q % NS], (uint32_t)((q / NS) & 1));   // full limit: copies must land
    } else if (warp == 1 && lane == 0) {
        // MMA issuer: per tile, into accumulator buffer i & 1 once the epilogue has drained it
        int s = 0;
        uint32_t ph = 0;
        for (int64_t i = 0; i < ntl; i++) {
            const uint32_t buf = (uint32_t)(i % nbuf);
            const uint32_t use = (uint32_t)(i / nbuf);
            if (!mbar_wait(&acce[buf], (use & 1u) ^ 1u, wl)) { atomicExch(&abort_flag, 1); atomicExch(errw, 5); break; }
            fence_after();
            const uint32_t d = tmem + buf * acc_cols;
            bool stop = false;
            for (int64_t c = 0; c < g.kchunks; c++) {
                if (!mbar_wait(&fullB[s], ph, wl) || (FUSED && !mbar_wait(&fullA[s], ph, wl))) {
                    atomicExch(&abort_flag, 1); atomicExch(errw, 2); stop = true; break;
                }
                fence_after();
                const uint32_t st = smem_u32(smem + s * stage_bytes);
                const uint32_t ahi = st, alo = st + kATileBytes, bhi = st + a_stage, blo = st + a_stage + g.b_tile_bytes;
                const uint32_t ta = tmem + a_col0 + (uint32_t)s * kATmemCols;
#pragma unroll
                for (int ks = 0; ks < kKSteps; ks++) {
                    const uint32_t off = ks * 256;     // two 16-byte core-matrix columns per K step
                    const uint64_t dbh = smem_desc(bhi + off), dbl = smem_desc(blo + off);
                    const uint32_t first = (c | ks) != 0 ? 1u : 0u;
                    // hi*hi into the main accumulator; the small hi*lo + lo*hi corrections into their
                    // own accumulator, so they are not rounded away against the large running sum
                    if (A_TMEM) {
                        const uint32_t tah = ta + ks * 8, tal = ta + 16 + ks * 8;   // 8 columns per K step
                        mma_ts<TF32>(d, tah, dbh, g.idesc, first);
                        mma_ts<TF32>(d + 2 * g.ntile, tah, dbl, g.idesc, first);
                        mma_ts<TF32>(d + 2 * g.ntile, tal, dbh, g.idesc, 1u);
                    } else {
                        const uint64_t dah = smem_desc(ahi + off), dal = smem_desc(alo + off);
                        mma<TF32>(d, dah, dbh, g.idesc, first);
                        mma<TF32>(d + 2 * g.ntile, dah, dbl, g.idesc, first);
                        mma<TF32>(d + 2 * g.ntile, dal, dbh, g.idesc, 1u);
                    }
                }
                mma_commit(&empty[s]);
                if (++s == NS) { s = 0; ph ^= 1u; }
            }
            if (stop) break;
            mma_commit(&accf[buf]);
        }
        // the MMAs must have finished before the tensor memory is freed
        mma_commit(drain);
        mbar_wait(drain, 0);                // full limit: the MMAs must finish
    } else if (ROWS && warp >= 6) {
        // X producers: thread r gathers row r of every (tile, chunk) with 8-byte cp.async into a
        // ring of R raw chunks ([R][KC][128 rows], R - 1 chunks in flight ahead of the one being
        // split, across tile boundaries), then scales, splits and stores each chunk into the
        // stage's A tiles, makes the stores visible to the tensor core's async proxy, and one lane
        // per warp arrives.  Each thread reads back only its own copies, so waiting on its own
        // copy groups is enough.
        const int R = g.ring_chunks;
        bool ntl_guard = false;
        if (R != 2 && R != 4 && R != 8) {   // the host guarantees it; never index past the ring
            if (lane == 0) { atomicExch(&abort_flag, 1); atomicExch(errw, 8); }
            ntl_guard = true;
        }
        float2* ring = reinterpret_cast<float2*>(smem + NS * stage_bytes);
        // warp w may reach tensor-memory lanes 32 (w % 4) .. +31 only: rows follow that quarter
        const int row = 32 * (warp & 3) + lane;
        const uint32_t a_lane = tmem + ((uint32_t)(32 * (warp & 3)) << 16) + a_col0;
        const float s = pow2f(-read_m(g.exps, g.x_slot));
        const float si = g.x_conj ? -s : s;
        const int64_t Q = ntl_guard ? 0 : ntl * g.kchunks;
        // issue side: (tile, chunk, ring slot) of the next chunk to fetch, advanced per issue
        int64_t iss_q = 0, iss_i = 0, iss_c = 0, iss_base = 0;
        int iss_slot = 0;
        bool iss_ok = false;
        auto set_tile = [&](int64_t i, int64_t& base, bool& ok) {
            int64_t b, mt, nt;
            tile_of(i, b, mt, nt);
            const int64_t m = mt * kTcTileM + row;
            ok = m < g.M;
            base = ok ? pdep(b, g.xb) + pdep(m, g.xm) : 0;
        };
        if (ntl > 0) set_tile(0, iss_base, iss_ok);
        auto issue = [&]() {                // one copy group per chunk (empty past the end)
            if (iss_q < Q) {
                if (iss_ok) {
                    float2* slot = ring + iss_slot * (KC * kTcTileM) + row;
                    const int64_t k0 = iss_c * KC;
                    const float2* src = g.X + iss_base + pdep(k0, g.xk);
#pragma unroll
                    for (int j = 0; j < KC; j++)
                        if (k0 + j < g.K) cp_async8(slot + j * kTcTileM, src + xkoff[j]);
                }
                iss_q++;
                if (++iss_slot == R) iss_slot = 0;
                if (++iss_c == g.kchunks) {
                    iss_c = 0;
                    if (++iss_i < ntl) set_tile(iss_i, iss_base, iss_ok);
                }
            }
            cp_async_commit();
        };
        for (int j = 0; j < R - 1; j++) issue();
        // consumer side: (tile, chunk, ring slot, stage, stage phase) of the chunk being split
        int64_t c = 0, cur_i = 0, cur_base = 0;
        bool row_ok = false;
        if (ntl > 0) set_tile(0, cur_base, row_ok);
        int slot = 0, st_i = 0;
        uint32_t ph = 0;
        for (int64_t qq = 0; qq < Q; qq++) {
            issue();
            if (R == 8) cp_async_wait<7>(); else if (R == 4) cp_async_wait<3>(); else cp_async_wait<1>();
            const bool ok = mbar_wait(&empty[st_i], ph ^ 1u, wl);
            // leave the loop as a whole warp (the __syncwarp below needs every lane)
            if (!__all_sync(0xffffffffu, ok)) { atomicExch(&abort_flag, 1); atomicExch(errw, 4); break; }
            if (__any_sync(0xffffffffu, *(volatile int*)&abort_flag != 0)) break;
            uint8_t* st = smem + st_i * stage_bytes;
            const float2* raw = ring + slot * (KC * kTcTileM) + row;
            if (A_TMEM) {
                fence_after();                  // the MMAs that read this A stage have completed
                uint32_t hw[16], lw[16];
                split_row_words<TF32>([&](int j) { return raw[j * kTcTileM]; }, row_ok, c * KC, g.K, s, si, hw, lw);
                const uint32_t ta = a_lane + (uint32_t)st_i * kATmemCols;
                tmem_st16(ta, hw);
                tmem_st16(ta + 16, lw);
                tmem_wait_st();
                fence_before();
            } else {
                split_a_row<TF32>(st, st + kATileBytes, row, [&](int j) { return raw[j * kTcTileM]; }, row_ok, c * KC,
                                  g.K, s, si);
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            }
            __syncwarp();
            if (lane == 0)
                asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&fullA[st_i])) : "memory");
            if (++slot == R) slot = 0;
            if (++st_i == NS) { st_i = 0; ph ^= 1u; }
            if (++c == g.kchunks) {
                c = 0;
                if (++cur_i < ntl) set_tile(cur_i, cur_base, row_ok);
            }
        }
        cp_async_wait_all();                // no copy may land after the CTA has left
    } else if (MODE == kModeTma && warp == 6) {
        // X loader: per (tile, chunk), once the splitters have released the ring slot, one TMA
        // tensor copy brings the (128 rows x chunk) block
        const int R = g.ring_chunks;
        uint8_t* ring = smem + NS * stage_bytes;
        uint64_t* rfull = rbars;
        uint64_t* rempty = rbars + kMaxRing;
        int64_t c = 0, i = 0, tbase = 0;
        auto set_tile = [&](int64_t ti) {
            int64_t b, mt, nt;
            tile_of(ti, b, mt, nt);
            tbase = pdep(b, g.xb) + pdep(mt * kTcTileM, g.xm);
        };
        if (ntl > 0) set_tile(0);
        int slot = 0;
        uint32_t ph = 0;
        int64_t issued = 0;
        const int64_t Q = ntl * g.kchunks;
        if (lane == 0) {
            for (int64_t qq = 0; qq < Q; qq++) {
                if (!mbar_wait(&rempty[slot], ph ^ 1u, wl)) { atomicExch(&abort_flag, 1); atomicExch(errw, 6); break; }
                if (*(volatile int*)&abort_flag) break;
                int co[5] = {0, 0, 0, 0, 0};
                co[g.tma_outer] = (int)((tbase + pdep(c * KC, g.xk)) >> g.tma_lead);
                mbar_expect_tx(&rfull[slot], (uint32_t)g.box_bytes);
                tma_load_5d(ring + slot * g.slot_bytes, &tmap, co, &rfull[slot]);
                issued++;
                if (++slot == R) { slot = 0; ph ^= 1u; }
                if (++c == g.kchunks) {
                    c = 0;
                    if (++i < ntl) set_tile(i);
                }
            }
            // boxes still in flight (only after an abort) must land before the CTA leaves
            for (int64_t q = issued - 1; q >= 0 && q >= issued - R; q--)
                mbar_wait(&rfull[q % R], (uint32_t)((q / R) & 1));     // full limit: copies must land
        }
    } else if (MODE == kModeBulk && warp == 6) {
        // X loader: per (tile, chunk), once the splitters have released the ring slot, fetch the
        // block's nseg contiguous segments with cp.async.bulk (one transaction count per slot)
        const int R = g.ring_chunks;
        uint8_t* ring = smem + NS * stage_bytes;
        const uint32_t seg_bytes = 8u << g.seg_bits;
        uint64_t* rfull = rbars;
        uint64_t* rempty = rbars + kMaxRing;
        int64_t c = 0, i = 0, tbase = 0;
        auto set_tile = [&](int64_t ti) {
            int64_t b, mt, nt;
            tile_of(ti, b, mt, nt);
            tbase = pdep(b, g.xb) + pdep(mt * kTcTileM, g.xm);
        };
        if (ntl > 0) set_tile(0);
        int slot = 0;
        uint32_t ph = 0;
        int64_t issued = 0;
        const int64_t Q = ntl * g.kchunks;
        for (int64_t qq = 0; qq < Q; qq++) {
            const bool ok = mbar_wait(&rempty[slot], ph ^ 1u, wl);
            if (!__all_sync(0xffffffffu, ok)) { atomicExch(&abort_flag, 1); atomicExch(errw, 6); break; }
            if (__any_sync(0xffffffffu, *(volatile int*)&abort_flag != 0)) break;
            const float2* src = g.X + tbase + pdep(c * KC, g.xk);
            uint8_t* dst = ring + slot * g.slot_bytes;
            if (lane == 0) mbar_expect_tx(&rfull[slot], (uint32_t)g.nseg * seg_bytes);
            __syncwarp();
            for (int sg = lane; sg < g.nseg; sg += 32)
                bulk_copy(dst + sg * g.seg_stride, src + segoff[sg], seg_bytes, &rfull[slot]);
            issued++;
            if (++slot == R) { slot = 0; ph ^= 1u; }
            if (++c == g.kchunks) {
                c = 0;
                if (++i < ntl) set_tile(i);
            }
        }
        // segments still in flight (only after an abort) must land before the CTA leaves
        for (int64_t q = issued - 1; q >= 0 && q >= issued - R; q--)
            mbar_wait(&rfull[q % R], (uint32_t)((q / R) & 1));     // full limit: copies must land
    } else if (SEGS && warp >= 7) {
        // splitters: thread r splits row r of each ring slot into the stage's A tiles (bulk) or
        // its tensor-memory A columns (TMA), then releases the slot to the loader and arrives on
        // the stage's full barrier
        const int R = g.ring_chunks;
        const uint8_t* ring = smem + NS * stage_bytes;
        uint64_t* rfull = rbars;
        uint64_t* rempty = rbars + kMaxRing;
        // warp w may reach tensor-memory lanes 32 (w % 4) .. +31 only: rows follow that quarter
        const int row = A_TMEM ? 32 * (warp & 3) + lane : threadIdx.x - SPLIT0;
        const uint32_t a_lane = tmem + ((uint32_t)(32 * (warp & 3)) << 16) + a_col0;
        const float s = pow2f(-read_m(g.exps, g.x_slot));
        const float si = g.x_conj ? -s : s;
        const int rb = rtab[row];
        // group grp of NG takes chunks grp, grp + NG, ...; slot, stage and chunk advance by NG
        constexpr int NG = MODE == kModeTma ? 2 : 1;
        const int grp = (warp - 7) / 4;
        int slot = grp, st_i = grp;
        uint32_t rph = 0, ph = 0;
        int64_t c = grp;
        while (c >= g.kchunks) c -= g.kchunks;
        const int64_t Q = ntl * g.kchunks;
        for (int64_t qq = grp; qq < Q; qq += NG) {
            const bool ok = mbar_wait(&rfull[slot], rph, wl) && mbar_wait(&empty[st_i], ph ^ 1u, wl);
            if (!__all_sync(0xffffffffu, ok)) { atomicExch(&abort_flag, 1); atomicExch(errw, 7); break; }
            if (__any_sync(0xffffffffu, *(volatile int*)&abort_flag != 0)) break;
            uint8_t* st = smem + st_i * stage_bytes;
            const uint8_t* raw = ring + slot * g.slot_bytes + rb;
            auto get = [&](int j) { return *reinterpret_cast<const float2*>(raw + ktab[j]); };
            if (A_TMEM) {
                fence_after();                  // the MMAs that read this A stage have completed
                uint32_t hw[16], lw[16];
                split_row_words<TF32>(get, true, c * KC, g.K, s, si, hw, lw);
                const uint32_t ta = a_lane + (uint32_t)st_i * kATmemCols;
                tmem_st16(ta, hw);
                tmem_st16(ta + 16, lw);
                tmem_wait_st();
                fence_before();
            } else {
                split_a_row<TF32>(st, st + kATileBytes, row, get, true, c * KC, g.K, s, si);
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            }
            __syncwarp();
            if (lane == 0) {
                asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&fullA[st_i])) : "memory");
                asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&rempty[slot])) : "memory");
            }
            slot += NG;
            if (slot >= R) { slot -= R; rph ^= 1u; }
            st_i += NG;
            if (st_i >= NS) { st_i -= NS; ph ^= 1u; }
            c += NG;
            while (c >= g.kchunks) c -= g.kchunks;
        }
    } else if (warp >= 2 && warp < 6) {
        // epilogue: warp w reads tensor-memory lanes 32*(w%4) .. +31 of buffer (tile & 1)
        const int q4 = warp & 3;
        const int row = q4 * 32 + lane;
        const uint32_t lane_base = tmem + ((uint32_t)(q4 * 32) << 16);
        int emax = -2139062144;
        for (int64_t i = 0; i < ntl; i++) {
            const uint32_t buf = (uint32_t)(i % nbuf);
            const uint32_t use = (uint32_t)(i / nbuf);
            const bool ok = mbar_wait(&accf[buf], use & 1u, wl);
            fence_after();
            if (!__all_sync(0xffffffffu, ok)) { atomicExch(&abort_flag, 1); atomicExch(errw, 3); break; }
            if (__any_sync(0xffffffffu, *(volatile int*)&abort_flag != 0)) break;
            int64_t b, mt, nt;
            tile_of(i, b, mt, nt);
            const int64_t m = mt * kTcTileM + row;
            const bool live = m < g.M;
            float2* __restrict__ Crow =
                g.C + (live ? pdep(b, g.cb) + pdep(m, g.cm) + pdep(nt * g.ntile, g.cn) : 0);
            const int64_t nleft = g.N - nt * g.ntile;
            const int nvalid = nleft < g.ntile ? (int)nleft : g.ntile;
            const uint32_t a0 = lane_base + buf * acc_cols;
            for (int n0 = 0; n0 < g.ntile; n0 += 16) {
                uint32_t vr[16], vi[16], cr[16], ci[16];
                tmem_ld16(a0 + n0, vr);
                tmem_ld16(a0 + g.ntile + n0, vi);
                tmem_ld16(a0 + 2 * g.ntile + n0, cr);
                tmem_ld16(a0 + 3 * g.ntile + n0, ci);
                tmem_wait_ld();
                if (live) {
#pragma unroll
                    for (int j = 0; j < 16; j++) {
                        if (n0 + j < nvalid) {
                            float2 v;
                            v.x = __uint_as_float(vr[j]) + __uint_as_float(cr[j]);
                            v.y = __uint_as_float(vi[j]) + __uint_as_float(ci[j]);
                            Crow[jtab[n0 + j]] = v;
                            const float mx = fmaxf(fabsf(v.x), fabsf(v.y));
                            if (mx > 0.f) emax = max(emax, exp_of(mx));
                        }
                    }
                }
            }
            // the buffer may be overwritten once all four warps' loads have completed
            fence_before();
            __syncwarp();
            if (lane == 0)
                asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&acce[buf])) : "memory");
        }
        for (int o = 16; o > 0; o >>= 1) emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, o));
        if (lane == 0 && emax != -2139062144 && g.exp_c >= 0) atomicMax(&g.exps[2 * g.exp_c + 1], emax);
    }
    fence_before();
    __syncthreads();
    if (warp == 0) {
        fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols) : "memory");
    }
}

// Split-K sum: C[c] = sum over the K blocks s (in order, in FP64) of partial[s * nC + c], raising
// the result's exponent slot (the partials share the result's scale).
__global__ void tc_ksum_kernel(const float2* __restrict__ partial, float2* __restrict__ C, int64_t nC, int nsplit,
                               int* exps, int exp_c) {
    int emax = -2139062144;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nC; c += (int64_t)gridDim.x * blockDim.x) {
        // FP64 sum of the FP32 block partials: thousands of blocks add no error of their own
        double re = 0.0, im = 0.0;
        for (int j = 0; j < nsplit; j++) {
            const float2 v = partial[(int64_t)j * nC + c];
            re += (double)v.x;
            im += (double)v.y;
        }
        const float2 r = make_float2((float)re, (float)im);
        C[c] = r;
        const float mx = fmaxf(fabsf(r.x), fabsf(r.y));
        if (mx > 0.f) emax = max(emax, exp_of(mx));
    }
    for (int o = 16; o > 0; o >>= 1) emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, o));
    if ((threadIdx.x & 31) == 0 && emax != -2139062144 && exp_c >= 0) atomicMax(&exps[2 * exp_c + 1], emax);
}

// ---- host helpers --------------------------------------------------------------------------------
void expand(const BitMap& m, std::vector<int>& dst_of_src) {
    for (int i = 0; i < m.n; i++)
        for (int j = 0; j < m.r[i].len; j++) {
            const int s = m.r[i].src + j;
            if ((int)dst_of_src.size() <= s) dst_of_src.resize(s + 1, -1);
            dst_of_src[s] = m.r[i].dst + j;
        }
}

BitMap runs(const std::vector<std::pair<int, int>>& pairs, bool* ok) {
    BitMap m;
    m.n = 0;
    for (size_t i = 0; i < pairs.size();) {
        size_t j = i + 1;
        while (j < pairs.size() && pairs[j].first == pairs[j - 1].first + 1 && pairs[j].second == pairs[j - 1].second + 1)
            j++;
        if (m.n >= kMaxRuns) { *ok = false; return m; }
        m.r[m.n] = Run{(uint8_t)pairs[i].first, (uint8_t)(j - i), (uint8_t)pairs[i].second, 0};
        m.n++;
        i = j;
    }
    return m;
}

int64_t cdiv(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Launch shapes.  An N tile of 64 complex columns needs 2 x 256 tensor-memory columns for its two
// accumulator buffers, the whole SM's 512: one CTA per SM with deep rings (about 192 KB of shared
// memory).  Narrower tiles leave room for two CTAs per SM with about 100 KB each.
struct GemmShape {
    int ctas_per_sm, stages, ring_bytes;
};
// kModeTmem: the accumulators (single-buffered for 64-column tiles) and the A stages share the
// tensor memory; shared memory holds only Y's stages and the gather ring.
GemmShape gemm_shape(int ntile, int mode, size_t stage_bytes) {
    const bool wide = ntile >= 64;
    if (mode == kModePlanes) return wide ? GemmShape{1, 6, 0} : GemmShape{2, 4, 0};
    if (mode == kModeRows) return wide ? GemmShape{1, 4, 64 * 1024} : GemmShape{2, 3, 32 * 1024};
    if (mode == kModeTmem || mode == kModeTma)
        return ntile >= 32 ? GemmShape{1, 6, 64 * 1024} : GemmShape{2, 4, 32 * 1024};
    // bulk: what the operand stages leave of about 220 KB (one CTA) or 108 KB (two CTAs)
    const int stages = wide ? 4 : 3;
    const size_t budget = wide ? 220 * 1024 : 108 * 1024;
    return GemmShape{wide ? 1 : 2, stages, (int)(budget - stages * stage_bytes)};
}
constexpr size_t kMaxDynSmem = 220 * 1024 + 128;

template <bool TF32, int MODE>
cudaError_t set_smem_attr() {
    static bool done = false;
    if (done) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(tc_gemm_kernel<TF32, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)kMaxDynSmem);
    if (e == cudaSuccess) done = true;
    return e;
}

}  // namespace

void plan_bulk(TcStep& t);

bool tc_plan_step(const StepArgs& s, size_t a_bits, size_t b_bits, size_t c_bits, bool tf32, TcStep* tc,
                  double plane_budget) {
    if (plane_budget <= 0) plane_budget = 4.0 * (1 << 30);
    std::vector<int> ca, cb, ka, kb;
    expand(s.cA, ca);
    expand(s.cB, cb);
    expand(s.kA, ka);
    expand(s.kB, kb);
    ca.resize(c_bits, -1);
    cb.resize(c_bits, -1);
    ka.resize(s.nk, -1);
    kb.resize(s.nk, -1);
    TcStep t;
    t.tf32 = tf32;
    t.x_is_a = a_bits >= b_bits;
    const std::vector<int>& cx = t.x_is_a ? ca : cb;
    const std::vector<int>& cy = t.x_is_a ? cb : ca;
    const std::vector<int>& kx = t.x_is_a ? ka : kb;
    const std::vector<int>& ky = t.x_is_a ? kb : ka;
    std::vector<std::pair<int, int>> xb, yb, cbm, xm, cm, yn, cn, xk, yk;
    for (int p = 0; p < (int)c_bits; p++) {
        if (cx[p] >= 0 && cy[p] >= 0) {
            const int j = (int)cbm.size();
            xb.push_back({j, cx[p]}); yb.push_back({j, cy[p]}); cbm.push_back({j, p});
        } else if (cx[p] >= 0) {
            const int j = (int)cm.size();
            xm.push_back({j, cx[p]}); cm.push_back({j, p});
        } else if (cy[p] >= 0) {
            const int j = (int)cn.size();
            yn.push_back({j, cy[p]}); cn.push_back({j, p});
        } else {
            return false;
        }
    }
    for (int j = 0; j < s.nk; j++) {
        if (kx[j] >= 0) xk.push_back({j, kx[j]});
        if (ky[j] >= 0) yk.push_back({j, ky[j]});
    }
    t.nb = (int)cbm.size();
    t.nm = (int)cm.size();
    t.nn = (int)cn.size();
    t.nk = s.nk;
    // eligibility: a real GEMM (M >= 128 rows, enough K x N reuse to leave the HBM roofline); a
    // long sum (K > 1024) also with 16 to 64 rows when the result has >= 4096 elements -- the
    // tile's other rows stay zero, which costs tensor time only, while the CUDA-core general
    // form would re-read both operands per result.  Smaller results of long sums go to the
    // CUDA-core split-K reduction (a 64-element result of a 2^27-term sum would otherwise be
    // 2^17 one-tile K blocks).
    const bool short_m = t.nm >= 4 && t.nk > 10 && t.nb + t.nm + t.nn >= 12;
    if ((t.nm < 7 && !short_m) || t.nk < 3 || t.nn < 2 || t.nn + t.nk < 8) return false;
    // split K: the tensor cores accumulate in FP32 with an error that grows about linearly with
    // the number of K steps (2^-24 per step of 8 products: 1e-5 of the result near K = 1024), so
    // K is cut into blocks of at most 2^10 -- and of down to 2^8 while the tiles are fewer than
    // 512.  The high K bits become batch bits, each block writes its own partial result (the
    // partials' index bits sit above the result's), and tc_run_gemm sums the partials in order.
    {
        const int64_t tiles = (int64_t(1) << t.nb) * std::max<int64_t>(1, (int64_t(1) << t.nm) / kTcTileM) *
                              std::max<int64_t>(1, (int64_t(1) << t.nn) / 64);
        int ks = std::max(0, t.nk - 10);
        while (ks < t.nk - 8 && (tiles << ks) < 512) ks++;
        t.ks = ks;
        t.c_elems = int64_t(1) << c_bits;
        if (ks > 0) {
            const int k0 = t.nk - ks;
            std::vector<std::pair<int, int>> xk2, yk2;
            for (auto& pr : xk) {
                if (pr.first >= k0) xb.push_back({t.nb + pr.first - k0, pr.second});
                else xk2.push_back(pr);
            }
            for (auto& pr : yk) {
                if (pr.first >= k0) yb.push_back({t.nb + pr.first - k0, pr.second});
                else yk2.push_back(pr);
            }
            for (int i = 0; i < ks; i++) cbm.push_back({t.nb + i, (int)c_bits + i});
            xk.swap(xk2);
            yk.swap(yk2);
            t.nb += ks;
            t.nk -= ks;
        }
    }
    // outer N blocks: when Y's packed planes (complex-doubled hi/lo: 4 words per element of Y)
    // would pass the budget, the high n bits become a loop on the host; each block packs only its part
    // of Y and runs the GEMM on pointers offset by the block's Y and C offsets (bit maps are
    // additive over disjoint bits)
    {
        const int es = tf32 ? 4 : 2;
        int no = 0;
        auto ybytes = [&](int nn) {
            return 4.0 * es * std::ldexp(1.0, t.nb + nn + t.nk);
        };
        while (ybytes(t.nn - no) > plane_budget && t.nn - no > 6) no++;
        if (no > 0) {
            std::vector<std::pair<int, int>> yo, co;
            const int n0 = t.nn - no;
            std::vector<std::pair<int, int>> yn2, cn2;
            for (auto& pr : yn) (pr.first >= n0 ? yo.push_back({pr.first - n0, pr.second}) : yn2.push_back(pr));
            for (auto& pr : cn) (pr.first >= n0 ? co.push_back({pr.first - n0, pr.second}) : cn2.push_back(pr));
            bool ok2 = true;
            t.yo = runs(yo, &ok2);
            t.co = runs(co, &ok2);
            if (!ok2) return false;
            yn.swap(yn2);
            cn.swap(cn2);
            t.nn = n0;
            t.nouter = no;
        }
    }
    bool ok = true;
    t.xb = runs(xb, &ok); t.yb = runs(yb, &ok); t.cb = runs(cbm, &ok);
    t.xm = runs(xm, &ok); t.cm = runs(cm, &ok);
    t.yn = runs(yn, &ok); t.cn = runs(cn, &ok);
    t.xk = runs(xk, &ok); t.yk = runs(yk, &ok);
    if (!ok) return false;
    t.M = int64_t(1) << t.nm;
    t.N = int64_t(1) << t.nn;
    t.K = int64_t(1) << t.nk;
    t.batch = int64_t(1) << t.nb;
    t.kc = (kTcChunkBytes / 2) / (tf32 ? 4 : 2);     // complex k per chunk: half the row is Re
    t.mtiles = cdiv(t.M, kTcTileM);
    t.kchunks = cdiv(t.K, t.kc);
    plan_bulk(t);
    {
        std::vector<int> xbv;
        expand(t.xb, xbv);
        t.bfast = false;
        for (int p2 : xbv) if (p2 == 0) t.bfast = true;
    }
    TcVariant v[kTcMaxVariants];
    const int nv = tc_variants(t, v);
    if (nv == 0) return false;
    // the autotuner tries a candidate only when the workspace holds its scratch: reserve up to
    // kTuneScratch for candidates beyond the default, so tuning never shrinks the batches much
    constexpr size_t kTuneScratch = size_t(4) << 30;
    t.planes_ok = false;
    tc_set_variant(t, v[0]);
    t.scratch_max = t.scratch_bytes;
    for (int i = 1; i < nv; i++) {
        tc_set_variant(t, v[i]);
        if (t.scratch_bytes <= kTuneScratch) t.scratch_max = std::max(t.scratch_max, t.scratch_bytes);
        if (!v[i].fused) t.planes_ok = true;
    }
    tc_set_variant(t, v[0]);
    *tc = t;
    return true;
}

void tc_set_variant(TcStep& t, TcVariant v) {
    t.fused = v.fused;
    t.bulk = v.fused && v.bulk;
    t.tmem = v.fused && v.tmem;
    t.tma = v.fused && v.tma;
    t.ntile_n = v.ntile;
    t.ntiles = cdiv(t.N, t.ntile_n);
    t.a_plane_bytes = t.fused ? 0 : (size_t)(t.batch * t.mtiles * t.kchunks) * kATileBytes;
    t.b_plane_bytes = (size_t)(t.batch * t.ntiles * t.kchunks) * (size_t)(2 * t.ntile_n * kTcChunkBytes);
    t.partial_bytes = t.ks > 0 ? ((size_t)t.c_elems << t.ks) * sizeof(float2) : 0;
    t.scratch_bytes = 2 * (t.a_plane_bytes + t.b_plane_bytes) + t.partial_bytes;
}

// N tiles of 16, 32 or 64 complex columns (two accumulators of 2*ntile FP32 columns: at 64 two
// CTAs fill an SM's 512 tensor-memory columns), no wider than N needs; fused first, then the
// planes variants whose scratch stays under 96 GB.  The first entry is the default.
int tc_variants(const TcStep& t, TcVariant* out) {
    const int widest = (int)std::min<int64_t>(64, std::max<int64_t>(16, t.N));
    int n = 0;
    // 4: TMA tensor gather into tensor-memory A tiles (when a block is one TMA box), 3: row
    // gather into tensor-memory A tiles, 2: bulk gather (when X's blocks are long segments),
    // 1: row gather, 0: planes; the fused forms with N tiles of 64 and 32 only
    for (int f = 4; f >= 0; f--) {
        if (f == 2 && !t.bulk_ok) continue;
        if (f == 4 && !t.tma_ok) continue;
        if (f == 0 && t.nouter > 0) continue;      // X would be packed again for every block
        for (int nt = widest; nt >= 16; nt /= 2) {
            if (f >= 1 && nt == 16 && widest > 16) continue;
            const TcVariant v{f >= 1, nt, f == 2, f == 3, f == 4};
            TcStep u = t;
            tc_set_variant(u, v);
            if (u.batch * u.mtiles * u.ntiles > (int64_t(1) << 31) - 1) continue;
            if (u.scratch_bytes > (size_t(96) << 30)) continue;
            if (n < kTcMaxVariants) out[n++] = v;
        }
    }
    return n;
}

// Bulk gather plan.  The block of X read by one (M tile, K chunk) is indexed by the tile's 7 row
// bits and the chunk's k bits; sorted by their position in X, those bits give a compact index c
// (c's low seg_bits bits are X's address bits 0 .. seg_bits-1, i.e. contiguous elements).  The
// block is then nseg = 2^(bits - seg_bits) segments of 2^seg_bits elements, segment s at X offset
// pdep(s, segmap) from the block's base; rowmap_c / kmap_c give c of row r / k index j.
// Eligible when the segments are at least 16 elements (128 bytes) long.
void plan_bulk(TcStep& t) {
    t.bulk_ok = false;
    std::vector<int> xm, xk;
    expand(t.xm, xm);
    expand(t.xk, xk);
    const int kbits = std::min(t.nk, t.tf32 ? 3 : 4);
    if ((int)xm.size() < 7 || (int)xk.size() < kbits) return;
    std::vector<std::pair<int, int>> bits;        // (X position, 0..6 row bit / 100+j k bit)
    for (int i = 0; i < 7; i++) bits.push_back({xm[i], i});
    for (int j = 0; j < kbits; j++) bits.push_back({xk[j], 100 + j});
    std::sort(bits.begin(), bits.end());
    int lead = 0;
    while (lead < (int)bits.size() && bits[lead].first == lead) lead++;
    if (lead < 1) return;                      // X's address bit 0 must lie in the block
    std::vector<std::pair<int, int>> seg, rowc, kc;
    for (int c = 0; c < (int)bits.size(); c++) {
        if (c >= lead) seg.push_back({c - lead, bits[c].first});
        if (bits[c].second < 100) rowc.push_back({bits[c].second, c});
        else kc.push_back({bits[c].second - 100, c});
    }
    std::sort(rowc.begin(), rowc.end());
    std::sort(kc.begin(), kc.end());
    bool ok = true;
    t.segmap = runs(seg, &ok);
    t.rowmap_c = runs(rowc, &ok);
    t.kmap_c = runs(kc, &ok);
    if (!ok) return;
    t.seg_bits = lead;
    t.nseg = 1 << ((int)bits.size() - lead);
    t.bulk_ok = lead >= 4;
    // TMA box: the block's address bits as runs of consecutive positions, cut into pieces of at
    // most 8 bits (a box dimension holds <= 256 elements); the first piece starts at bit 0
    t.tma_ok = false;
    t.tma_npiece = 0;
    for (size_t c = 0; c < bits.size();) {
        size_t e = c + 1;
        while (e < bits.size() && bits[e].first == bits[e - 1].first + 1 && (int)(e - c) < 8) e++;
        if (t.tma_npiece == 4) return;
        t.tma_pos[t.tma_npiece] = bits[c].first;
        t.tma_len[t.tma_npiece] = (int)(e - c);
        t.tma_npiece++;
        c = e;
    }
    t.tma_lead = lead;
    // the innermost box dimension holds the leading run: at least 16 elements (128 bytes), and
    // every box coordinate below 2^31
    const int xbits = t.nb + t.nm + t.nk;
    t.tma_ok = lead >= 4 && xbits - lead <= 31;
}

std::string tc_key(const TcStep& t) {
    std::string k;
    auto put = [&](int64_t x) { k.append(reinterpret_cast<const char*>(&x), sizeof(x)); };
    auto map = [&](const BitMap& m) {
        put(m.n);
        for (int i = 0; i < m.n; i++) put(m.r[i].src | (m.r[i].len << 8) | (m.r[i].dst << 16));
    };
    put(t.tf32); put(t.nb); put(t.nm); put(t.nn); put(t.nk);
    map(t.xb); map(t.xm); map(t.xk); map(t.yb); map(t.yn); map(t.yk); map(t.cb); map(t.cm); map(t.cn);
    return k;
}

cudaError_t tc_run_pack(const TcStep& t, const StepArgs& s, int* exps, void* scratch, cudaStream_t st, int sm_count) {
    uint8_t* base = static_cast<uint8_t*>(scratch);
    const int slot_x = t.x_is_a ? s.expA : s.expB;
    const int slot_y = t.x_is_a ? s.expB : s.expA;
    PackArgs px;
    memset(&px, 0, sizeof(px));
    px.src = t.x_is_a ? s.A : s.B;
    px.hi = base; px.lo = base + t.a_plane_bytes;
    px.mb = t.xb; px.mr = t.xm; px.mk = t.xk;
    px.rows = t.M; px.rows_pad = t.mtiles * kTcTileM; px.K = t.K; px.batch = t.batch;
    px.kchunks = t.kchunks; px.row_tiles = t.mtiles; px.tile_rows = kTcTileM; px.ntile = 0;
    px.slot_src = slot_x; px.doubled = 0; px.exp_c = s.expC; px.slot_other = slot_y;
    px.conj = t.x_is_a ? s.conjA : s.conjB;
    PackArgs py = px;
    py.conj = t.x_is_a ? s.conjB : s.conjA;
    py.src = t.x_is_a ? s.B : s.A;
    py.hi = base + 2 * t.a_plane_bytes; py.lo = base + 2 * t.a_plane_bytes + t.b_plane_bytes;
    py.mb = t.yb; py.mr = t.yn; py.mk = t.yk;
    py.rows = t.N; py.rows_pad = t.ntiles * t.ntile_n; py.row_tiles = t.ntiles;
    py.tile_rows = 2 * t.ntile_n; py.ntile = t.ntile_n;
    py.slot_src = slot_y; py.doubled = 1; py.slot_other = slot_x;
    auto grid_of = [&](const PackArgs& p) {
        const int64_t n = p.batch * p.kchunks * p.rows_pad * 2;
        return (int)std::max<int64_t>(1, std::min<int64_t>(cdiv(n, 256), (int64_t)sm_count * 16));
    };
    // fused steps pack only Y: the GEMM gathers and splits X itself
    if (t.tf32) {
        if (!t.fused) pack_kernel<true><<<grid_of(px), 256, 0, st>>>(px, exps);
        pack_kernel<true><<<grid_of(py), 256, 0, st>>>(py, exps);
    } else {
        if (!t.fused) pack_kernel<false><<<grid_of(px), 256, 0, st>>>(px, exps);
        pack_kernel<false><<<grid_of(py), 256, 0, st>>>(py, exps);
    }
    return cudaGetLastError();
}

// Tensor map of X for the TMA gather: the box pieces (positions tma_pos, 2^tma_len elements),
// ordered by stride, with one more dimension (box 1) that walks X in steps of 2^tma_lead elements
// -- placed right after the pieces below tma_lead so that the strides grow -- and dimensions of
// extent 1 up to rank 5.  Every block's base offset is a multiple of 2^tma_lead (its lower
// address bits all belong to the block), so the copy of a block is the box at coordinate
// base >> tma_lead of that dimension.  False when the driver rejects the map.
bool make_x_map(const TcStep& t, const void* X, CUtensorMap* map, GemmArgs* g) {
    const EncodeTiledFn encode = encode_tiled();
    if (!encode) return false;
    cuuint64_t dims[5];
    cuuint64_t strides[4];
    cuuint32_t box[5], estr[5] = {1, 1, 1, 1, 1};
    int nd = 0, outer = -1;
    const int64_t xbits = (int64_t)t.nb + t.nm + t.nk;   // X's address bits
    int64_t box_elems = 1;
    for (int i = 0; i < t.tma_npiece; i++) {
        if (outer < 0 && t.tma_pos[i] >= t.tma_lead) {
            outer = nd;
            dims[nd] = (cuuint64_t)(int64_t(1) << (xbits - t.tma_lead));
            box[nd] = 1;
            if (nd > 0) strides[nd - 1] = (cuuint64_t)(8ll << t.tma_lead);
            nd++;
        }
        dims[nd] = (cuuint64_t)1 << t.tma_len[i];
        box[nd] = 1u << t.tma_len[i];
        if (nd > 0) strides[nd - 1] = (cuuint64_t)(8ll << t.tma_pos[i]);
        box_elems <<= t.tma_len[i];
        nd++;
    }
    if (outer < 0) {
        outer = nd;
        dims[nd] = (cuuint64_t)(int64_t(1) << (xbits - t.tma_lead));
        box[nd] = 1;
        strides[nd - 1] = (cuuint64_t)(8ll << t.tma_lead);
        nd++;
    }
    // box coordinates are signed 32-bit: the outer coordinate (offset >> tma_lead) must stay below 2^31
    if (nd > 5 || xbits - t.tma_lead > 31) return false;
    while (nd < 5) {
        dims[nd] = 1;
        box[nd] = 1;
        strides[nd - 1] = (cuuint64_t)(8ll << xbits);
        nd++;
    }
    const CUresult r = encode(map, CU_TENSOR_MAP_DATA_TYPE_UINT64, 5, const_cast<void*>(X), dims,
                                              strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                              CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return false;
    g->tma_lead = t.tma_lead;
    g->tma_outer = outer;
    g->box_bytes = (int)(box_elems * 8);
    return true;
}

cudaError_t tc_launch_gemm(const TcStep& t, const StepArgs& s, int* exps, void* scratch, cudaStream_t st,
                           int sm_count, int64_t c_off, bool ksum);

cudaError_t tc_run_gemm(const TcStep& t, const StepArgs& s, int* exps, void* scratch, cudaStream_t st,
                        int sm_count) {
    return tc_launch_gemm(t, s, exps, scratch, st, sm_count, 0, true);
}

cudaError_t tc_run_step(const TcStep& t, const StepArgs& s, int* exps, void* scratch, cudaStream_t st, int sm_count,
                        int* launches) {
    const int64_t nblk = int64_t(1) << t.nouter;
    int nl = 0;
    for (int64_t o = 0; o < nblk; o++) {
        StepArgs so = s;
        const int64_t yoff = pdep(o, t.yo), coff = pdep(o, t.co);
        if (t.x_is_a) so.B = static_cast<const float2*>(s.B) + yoff;
        else so.A = static_cast<const float2*>(s.A) + yoff;
        so.C = static_cast<float2*>(s.C) + coff;
        cudaError_t e = tc_run_pack(t, so, exps, scratch, st, sm_count);
        if (e != cudaSuccess) return e;
        e = tc_launch_gemm(t, so, exps, scratch, st, sm_count, coff, o == nblk - 1);
        if (e != cudaSuccess) return e;
        nl += (t.fused ? 1 : 2) + 1;
    }
    if (t.ks > 0) nl++;
    if (launches) *launches = nl;
    return cudaSuccess;
}

cudaError_t tc_launch_gemm(const TcStep& t, const StepArgs& s, int* exps, void* scratch, cudaStream_t st,
                           int sm_count, int64_t c_off, bool ksum) {
    uint8_t* base = static_cast<uint8_t*>(scratch);
    GemmArgs g;
    memset(&g, 0, sizeof(g));
    g.a_hi = base; g.a_lo = base + t.a_plane_bytes;
    g.b_hi = base + 2 * t.a_plane_bytes; g.b_lo = base + 2 * t.a_plane_bytes + t.b_plane_bytes;
    // split K: the GEMM writes the partials after the planes; the sum below writes C
    float2* partial = reinterpret_cast<float2*>(base + 2 * (t.a_plane_bytes + t.b_plane_bytes));
    g.C = t.ks > 0 ? partial + c_off : static_cast<float2*>(s.C);
    g.cb = t.cb; g.cm = t.cm; g.cn = t.cn;
    g.M = t.M; g.N = t.N; g.mtiles = t.mtiles; g.ntiles = t.ntiles; g.kchunks = t.kchunks; g.batch = t.batch;
    g.ntile = t.ntile_n;
    g.b_tile_bytes = (uint32_t)(2 * t.ntile_n * kTcChunkBytes);
    const uint32_t nmma = (uint32_t)(2 * t.ntile_n);
    const uint32_t fmt = t.tf32 ? 2u : 1u;           // TF32 : BF16 operand format
    g.idesc = (1u << 4) | (fmt << 7) | (fmt << 10) | ((nmma >> 3) << 17) | ((uint32_t)(kTcTileM >> 4) << 24);
    g.exp_c = t.ks > 0 ? -1 : s.expC;
    g.exps = exps;
    g.wait_limit = t.wait_limit;
    g.stall = t.stall_first_cta ? 1 : 0;
    g.err = t.err_word;
    g.X = static_cast<const float2*>(t.x_is_a ? s.A : s.B);
    g.xb = t.xb; g.xm = t.xm; g.xk = t.xk;
    g.K = t.K;
    g.x_slot = t.x_is_a ? s.expA : s.expB;
    g.x_conj = t.x_is_a ? s.conjA : s.conjB;
    g.bfast = t.bfast ? 1 : 0;
    int mode = !t.fused ? kModePlanes
                        : (t.tma ? kModeTma : (t.tmem ? kModeTmem : (t.bulk ? kModeBulk : kModeRows)));
    alignas(64) CUtensorMap tmap;
    memset(&tmap, 0, sizeof(tmap));
    if (mode == kModeTma && !make_x_map(t, g.X, &tmap, &g)) mode = kModeTmem;
    // cp.async.bulk needs 16-byte aligned sources: fall back to the row gather otherwise
    if (mode == kModeBulk && (reinterpret_cast<uintptr_t>(g.X) & 15) != 0) mode = kModeRows;
    const size_t stage = ((mode == kModeTmem || mode == kModeTma) ? 0 : 2 * kATileBytes) + 2 * (size_t)g.b_tile_bytes;
    GemmShape sh = gemm_shape(t.ntile_n, mode, stage);
    g.stages = sh.stages;
    const int acc_cols = 4 * t.ntile_n;
    const bool a_tmem = mode == kModeTmem || mode == kModeTma;
    g.nbuf = (a_tmem && t.ntile_n >= 64) ? 1 : 2;
    {
        const int need = g.nbuf * acc_cols + (a_tmem ? sh.stages * kATmemCols : 0);
        int cols = 32;
        while (cols < need) cols *= 2;
        g.tmem_cols = cols;                 // <= 512: 2 x 256 or 256 + 6 x 32
    }
    if (mode == kModeBulk) {
        g.segmap = t.segmap; g.rowmap_c = t.rowmap_c; g.kmap_c = t.kmap_c;
        g.seg_bits = t.seg_bits;
        g.nseg = t.nseg;
        g.seg_stride = (8 << t.seg_bits) + 16;
        g.slot_bytes = (int)(((size_t)t.nseg * g.seg_stride + 127) / 128 * 128);
        g.ring_chunks = std::min(kMaxRing, sh.ring_bytes / g.slot_bytes);
        if (g.ring_chunks < 2) {                // blocks too large for the ring: row gather
            mode = kModeRows;
            sh = gemm_shape(t.ntile_n, mode, stage);
            g.stages = sh.stages;
        } else {
            sh.ring_bytes = g.ring_chunks * g.slot_bytes;
        }
    }
    if (mode == kModeTma) {
        g.seg_bits = 0;
        g.seg_stride = 8;                   // dense box: compact index c at byte 8 c
        g.rowmap_c = t.rowmap_c;
        g.kmap_c = t.kmap_c;
        g.slot_bytes = (g.box_bytes + 127) / 128 * 128;
        g.ring_chunks = std::min(kMaxRing, sh.ring_bytes / g.slot_bytes) & ~1;   // even: two split groups
        if (g.ring_chunks < 2 || (g.stages & 1)) return cudaErrorInvalidValue;
        sh.ring_bytes = g.ring_chunks * g.slot_bytes;
    }
    if (mode == kModeRows || mode == kModeTmem) g.ring_chunks = sh.ring_bytes / (kTcTileM * t.kc * 8);
    // the row gather waits with cp.async.wait_group R-1 for R in {2, 4, 8}
    if ((mode == kModeRows || mode == kModeTmem) && g.ring_chunks != 2 && g.ring_chunks != 4 && g.ring_chunks != 8)
        return cudaErrorInvalidValue;
    if (mode == kModeBulk && (g.ring_chunks < 2 || g.ring_chunks > kMaxRing)) return cudaErrorInvalidValue;
    const size_t smem = (size_t)sh.stages * stage + (size_t)sh.ring_bytes + 128;
    const int64_t tiles = t.batch * t.mtiles * t.ntiles;
    const int64_t ctas = std::max<int64_t>(1, std::min<int64_t>(tiles, (int64_t)sm_count * sh.ctas_per_sm));
    cudaError_t e = cudaSuccess;
#define QXG_LAUNCH_GEMM(TF, MD)                                                               \
    do {                                                                                      \
        if ((e = set_smem_attr<TF, MD>()) != cudaSuccess) return e;                           \
        tc_gemm_kernel<TF, MD><<<(unsigned)ctas, threads_of(MD), smem, st>>>(g, tmap);        \
    } while (0)
    if (t.tf32) {
        if (mode == kModePlanes) QXG_LAUNCH_GEMM(true, kModePlanes);
        else if (mode == kModeRows) QXG_LAUNCH_GEMM(true, kModeRows);
        else if (mode == kModeBulk) QXG_LAUNCH_GEMM(true, kModeBulk);
        else if (mode == kModeTmem) QXG_LAUNCH_GEMM(true, kModeTmem);
        else QXG_LAUNCH_GEMM(true, kModeTma);
    } else {
        if (mode == kModePlanes) QXG_LAUNCH_GEMM(false, kModePlanes);
        else if (mode == kModeRows) QXG_LAUNCH_GEMM(false, kModeRows);
        else if (mode == kModeBulk) QXG_LAUNCH_GEMM(false, kModeBulk);
        else if (mode == kModeTmem) QXG_LAUNCH_GEMM(false, kModeTmem);
        else QXG_LAUNCH_GEMM(false, kModeTma);
    }
#undef QXG_LAUNCH_GEMM
    if (t.ks > 0 && ksum) {
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        const int64_t blocks = std::min<int64_t>(cdiv(t.c_elems, 256), (int64_t)sm_count * 8);
        tc_ksum_kernel<<<(unsigned)std::max<int64_t>(1, blocks), 256, 0, st>>>(
            partial, static_cast<float2*>(s.C) - c_off, t.c_elems, 1 << t.ks, exps, s.expC);
    }
    return cudaGetLastError();
}

cudaError_t tc_read_error(int* host_code, int* d_word, cudaStream_t st) {
    cudaError_t e = d_word ? cudaMemcpyAsync(host_code, d_word, sizeof(int), cudaMemcpyDeviceToHost, st)
                           : cudaMemcpyFromSymbolAsync(host_code, g_tc_error, sizeof(int), 0, cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess) return e;
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess || *host_code == 0) return e;
    const int zero = 0;
    e = d_word ? cudaMemcpyAsync(d_word, &zero, sizeof(int), cudaMemcpyHostToDevice, st)
               : cudaMemcpyToSymbolAsync(g_tc_error, &zero, sizeof(int), 0, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(st);
}

}  // namespace qxg
