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

namespace qxg {

__device__ int g_tc_error = 0;

namespace {

constexpr int kThreadsGemm = 192;                        // warp 0 producer, 1 MMA, 2-5 epilogue
constexpr int kThreadsFused = 320;                       // + warps 6-9 gather and split X rows
constexpr int kStages = 3;                               // operand stages, planes kernel
constexpr int kStagesFused = 2;                          // operand stages, fused kernel
constexpr int kRingBytes = 32 * 1024;                    // fused: raw X rows in flight per CTA
constexpr int kCols16 = kTcChunkBytes / 16;              // 16-byte core-matrix columns per chunk (4)
constexpr int kSbo = kCols16 * 128;                      // bytes between 8-row groups (512)
constexpr int kATileBytes = kTcTileM * kTcChunkBytes;    // 8 KB
constexpr int kKSteps = kTcChunkBytes / 32;              // MMA K steps (32 bytes each) per chunk
constexpr uint32_t kWaitLimit = 1u << 20;                // try_wait polls before giving up
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
    uint32_t b_tile_bytes;
    uint32_t idesc;
    int exp_c;
    int* exps;
};

__device__ __forceinline__ int read_m(const int* exps, int slot) {
    const int m = exps[2 * slot + 1];
    return m < -400 ? 0 : m;
}
__device__ __forceinline__ float pow2f(int n) {
    n = n < -126 ? -126 : (n > 127 ? 127 : n);
    return __int_as_float((n + 127) << 23);
}
__device__ __forceinline__ int exp_of(float x) { return (int)((__float_as_uint(x) >> 23) & 0xffu) - 126; }

__device__ __forceinline__ uint32_t to_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}

// hi/lo split of one value into the element type's bit pattern
template <bool TF32> struct Split;
template <> struct Split<false> {
    using E = unsigned short;
    __device__ static void go(float v, E& hi, E& lo) {
        const __nv_bfloat16 h = __float2bfloat16_rn(v);
        const __nv_bfloat16 l = __float2bfloat16_rn(v - __bfloat162float(h));
        hi = __bfloat16_as_ushort(h);
        lo = __bfloat16_as_ushort(l);
    }
};
template <> struct Split<true> {
    using E = uint32_t;
    __device__ static void go(float v, E& hi, E& lo) {
        hi = to_tf32(v);
        lo = to_tf32(v - __uint_as_float(hi));
    }
};

// Byte offset of (row, 16-byte column) inside a K-major no-swizzle tile of 64-byte rows.
__device__ __forceinline__ int64_t core_off(int row, int col16) {
    return (int64_t)(row >> 3) * kSbo + col16 * 128 + (row & 7) * 16;
}

template <typename E, int NE>
__device__ __forceinline__ void st16(uint8_t* dst, const E (&v)[NE]) {
    uint4 w;
    memcpy(&w, v, 16);
    *reinterpret_cast<uint4*>(dst) = w;
}

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
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait for the phase with the given parity; false when it gave up.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    for (uint32_t i = 0; i < kWaitLimit; i++)
        if (mbar_try(bar, parity)) return true;
    return false;
}
__device__ __forceinline__ void bulk_copy(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}
// Shared-memory matrix descriptor: K-major, no swizzle; LBO = 128 B between core matrices along
// K, SBO = 512 B between 8-row groups; descriptor version 1.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr) {
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)(128 >> 4) << 16) | ((uint64_t)(kSbo >> 4) << 32) |
           (1ull << 46);
}
template <bool TF32>
__device__ __forceinline__ void mma(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    if (TF32) {
        asm volatile(
            "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
            "l"(a), "l"(b), "r"(idesc), "r"(acc)
            : "memory");
    } else {
        asm volatile(
            "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
            "l"(a), "l"(b), "r"(idesc), "r"(acc)
            : "memory");
    }
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

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
// gathered into the raw ring: element j at raw[j * kTcTileM]), scales, splits and stores it into
// the stage's hi/lo A tiles (real parts in 16-byte columns 0-1, imaginary parts in 2-3).
template <bool TF32>
__device__ __forceinline__ void split_a_row(uint8_t* th, uint8_t* tl, int row, const float2* raw, bool row_ok,
                                            int64_t k0, int64_t K, float s, float si) {
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
                const float2 v = raw[(g * NE + j) * kTcTileM];
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

template <bool TF32, bool FUSED>
__global__ void __launch_bounds__(FUSED ? kThreadsFused : kThreadsGemm, 2) tc_gemm_kernel(const GemmArgs g) {
    constexpr int NS = FUSED ? kStagesFused : kStages;
    constexpr int KC = TF32 ? 8 : 16;            // complex k per 64-byte chunk
    extern __shared__ uint8_t smem_raw[];
    __shared__ uint64_t bars[2 * NS + 1];        // full[NS], empty[NS], accum
    __shared__ int64_t noff[128];                // result offsets of this tile's columns
    __shared__ int64_t xkoff[KC];                // fused: X offsets of the k values inside a chunk
    __shared__ uint32_t tmem_holder;
    __shared__ int abort_flag;
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
    const uint32_t stage_bytes = 2u * kATileBytes + 2u * g.b_tile_bytes;
    uint64_t* full = bars;
    uint64_t* empty = bars + NS;
    uint64_t* accum = bars + 2 * NS;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int64_t tile = blockIdx.x;
    const int64_t nt = tile % g.ntiles;
    tile /= g.ntiles;
    const int64_t mt = tile % g.mtiles;
    const int64_t b = tile / g.mtiles;
    // two accumulators (main, corrections) of 2*ntile FP32 columns each
    const uint32_t ncols = (uint32_t)(4 * g.ntile) < 32u ? 32u : (uint32_t)(4 * g.ntile);

    if (threadIdx.x == 0) {
        // a full barrier completes on the bulk copies' bytes and, when fused, the four X warps
        for (int i = 0; i < NS; i++) mbar_init(&full[i], FUSED ? 5u : 1u);
        for (int i = NS; i < 2 * NS + 1; i++) mbar_init(&bars[i], 1);
        abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_holder)),
                     "r"(ncols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (warp >= 2 && warp < 6) {
        for (int j = threadIdx.x - 64; j < g.ntile; j += 128) {
            const int64_t n = nt * g.ntile + j;
            noff[j] = n < g.N ? pdep(n, g.cn) : 0;
        }
    }
    // chunk k0 has its low log2(KC) bits clear, so X's offset of k0 + j is pdep(k0) + pdep(j)
    if (FUSED && threadIdx.x >= 192 && threadIdx.x < 192 + KC) xkoff[threadIdx.x - 192] = pdep(threadIdx.x - 192, g.xk);
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = tmem_holder;

    if (warp == 0 && lane == 0) {
        // producer: stream K chunks of the four planes into the stages
        const int64_t a_tile0 = (b * g.mtiles + mt) * g.kchunks;
        const int64_t b_tile0 = (b * g.ntiles + nt) * g.kchunks;
        for (int64_t c = 0; c < g.kchunks; c++) {
            const int s = (int)(c % NS);
            const uint32_t u = (uint32_t)(c / NS);
            if (!mbar_wait(&empty[s], (u & 1u) ^ 1u)) { atomicExch(&abort_flag, 1); atomicExch(&g_tc_error, 1); break; }
            if (*(volatile int*)&abort_flag) break;
            uint8_t* st = smem + s * stage_bytes;
            mbar_expect_tx(&full[s], FUSED ? 2u * g.b_tile_bytes : stage_bytes);
            const int64_t ao = (a_tile0 + c) * kATileBytes, bo = (b_tile0 + c) * (int64_t)g.b_tile_bytes;
            if (!FUSED) {
                bulk_copy(st, static_cast<const uint8_t*>(g.a_hi) + ao, kATileBytes, &full[s]);
                bulk_copy(st + kATileBytes, static_cast<const uint8_t*>(g.a_lo) + ao, kATileBytes, &full[s]);
            }
            bulk_copy(st + 2 * kATileBytes, static_cast<const uint8_t*>(g.b_hi) + bo, g.b_tile_bytes, &full[s]);
            bulk_copy(st + 2 * kATileBytes + g.b_tile_bytes, static_cast<const uint8_t*>(g.b_lo) + bo, g.b_tile_bytes,
                      &full[s]);
        }
    } else if (warp == 1 && lane == 0) {
        // MMA issuer: kKSteps K steps of 32 bytes per chunk, three products each
        for (int64_t c = 0; c < g.kchunks; c++) {
            const int s = (int)(c % NS);
            const uint32_t u = (uint32_t)(c / NS);
            if (!mbar_wait(&full[s], u & 1u)) { atomicExch(&abort_flag, 1); atomicExch(&g_tc_error, 2); break; }
            fence_after();
            const uint32_t st = smem_u32(smem + s * stage_bytes);
            const uint32_t ahi = st, alo = st + kATileBytes, bhi = st + 2 * kATileBytes,
                           blo = st + 2 * kATileBytes + g.b_tile_bytes;
#pragma unroll
            for (int ks = 0; ks < kKSteps; ks++) {
                const uint32_t off = ks * 256;     // two 16-byte core-matrix columns per K step
                const uint64_t dah = smem_desc(ahi + off), dal = smem_desc(alo + off);
                const uint64_t dbh = smem_desc(bhi + off), dbl = smem_desc(blo + off);
                const uint32_t first = (c | ks) != 0 ? 1u : 0u;
                // hi*hi into the main accumulator; the small hi*lo + lo*hi corrections into their
                // own accumulator, so they are not rounded away against the large running sum
                mma<TF32>(tmem, dah, dbh, g.idesc, first);
                mma<TF32>(tmem + 2 * g.ntile, dah, dbl, g.idesc, first);
                mma<TF32>(tmem + 2 * g.ntile, dal, dbh, g.idesc, 1u);
            }
            mma_commit(&empty[s]);
        }
        mma_commit(accum);
    } else if (FUSED && warp >= 6) {
        // X producers: thread r gathers row r of X's K chunks with 8-byte cp.async into a ring of
        // R raw chunks ([R][KC][128 rows], R - 1 chunks in flight ahead of the one being split),
        // then scales, splits and stores each chunk into the stage's A tiles, makes the stores
        // visible to the tensor core's async proxy, and one lane per warp arrives.  Each thread
        // reads back only its own copies, so waiting on its own copy groups is enough.
        constexpr int R = kRingBytes / (kTcTileM * KC * 8);
        float2* ring = reinterpret_cast<float2*>(smem + NS * stage_bytes);
        const int row = threadIdx.x - 192;
        const int64_t m = mt * kTcTileM + row;
        const bool row_ok = m < g.M;
        const int64_t base = row_ok ? pdep(b, g.xb) + pdep(m, g.xm) : 0;
        const float s = pow2f(-read_m(g.exps, g.x_slot));
        const float si = g.x_conj ? -s : s;
        auto issue = [&](int64_t c) {       // one copy group per chunk (empty past the end)
            if (row_ok && c < g.kchunks) {
                float2* slot = ring + (c % R) * (KC * kTcTileM) + row;
                const int64_t k0 = c * KC;
                const float2* src = g.X + base + pdep(k0, g.xk);
#pragma unroll
                for (int j = 0; j < KC; j++)
                    if (k0 + j < g.K) cp_async8(slot + j * kTcTileM, src + xkoff[j]);
            }
            cp_async_commit();
        };
        for (int c = 0; c < R - 1; c++) issue(c);
        for (int64_t c = 0; c < g.kchunks; c++) {
            issue(c + R - 1);
            cp_async_wait<R - 1>();
            const int st_i = (int)(c % NS);
            const uint32_t u = (uint32_t)(c / NS);
            const bool ok = mbar_wait(&empty[st_i], (u & 1u) ^ 1u);
            // leave the loop as a whole warp (the __syncwarp below needs every lane)
            if (!__all_sync(0xffffffffu, ok)) { atomicExch(&abort_flag, 1); atomicExch(&g_tc_error, 4); break; }
            if (__any_sync(0xffffffffu, *(volatile int*)&abort_flag != 0)) break;
            uint8_t* st = smem + st_i * stage_bytes;
            split_a_row<TF32>(st, st + kATileBytes, row, ring + (c % R) * (KC * kTcTileM) + row, row_ok, c * KC,
                              g.K, s, si);
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncwarp();
            if (lane == 0)
                asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&full[st_i])) : "memory");
        }
        cp_async_wait_all();                // no copy may land after the CTA has left
    } else if (warp >= 2 && warp < 6) {
        // epilogue: warp w reads tensor-memory lanes 32*(w%4) .. +31
        const bool ok = mbar_wait(accum, 0);
        fence_after();
        if (!ok) atomicExch(&g_tc_error, 3);
        const int q = warp & 3;
        const int row = q * 32 + lane;
        const int64_t m = mt * kTcTileM + row;
        const bool live = ok && !*(volatile int*)&abort_flag && m < g.M;
        int emax = -2139062144;
        float2* __restrict__ Crow = g.C + ((m < g.M) ? pdep(b, g.cb) + pdep(m, g.cm) : 0);
        const int64_t nleft = g.N - nt * g.ntile;
        const int nvalid = nleft < g.ntile ? (int)nleft : g.ntile;
        const uint32_t lane_addr = tmem + ((uint32_t)(q * 32) << 16);
        for (int n0 = 0; n0 < g.ntile; n0 += 16) {
            uint32_t vr[16], vi[16], cr[16], ci[16];
            tmem_ld16(lane_addr + n0, vr);
            tmem_ld16(lane_addr + g.ntile + n0, vi);
            tmem_ld16(lane_addr + 2 * g.ntile + n0, cr);
            tmem_ld16(lane_addr + 3 * g.ntile + n0, ci);
            tmem_wait_ld();
            if (live) {
#pragma unroll
                for (int j = 0; j < 16; j++) {
                    if (n0 + j < nvalid) {
                        float2 v;
                        v.x = __uint_as_float(vr[j]) + __uint_as_float(cr[j]);
                        v.y = __uint_as_float(vi[j]) + __uint_as_float(ci[j]);
                        Crow[noff[n0 + j]] = v;
                        const float mx = fmaxf(fabsf(v.x), fabsf(v.y));
                        if (mx > 0.f) emax = max(emax, exp_of(mx));
                    }
                }
            }
        }
        for (int o = 16; o > 0; o >>= 1) emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, o));
        if (lane == 0 && emax != -2139062144) atomicMax(&g.exps[2 * g.exp_c + 1], emax);
    }
    fence_before();
    __syncthreads();
    if (warp == 0) {
        fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols) : "memory");
    }
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

constexpr size_t kMaxStageBytes = 2 * kATileBytes + 2 * (2 * 64 * kTcChunkBytes);
constexpr size_t kMaxDynSmem = std::max(kStages * kMaxStageBytes, kStagesFused * kMaxStageBytes + kRingBytes) + 128;

template <bool TF32, bool FUSED>
cudaError_t set_smem_attr() {
    static bool done = false;
    if (done) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(tc_gemm_kernel<TF32, FUSED>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)kMaxDynSmem);
    if (e == cudaSuccess) done = true;
    return e;
}

}  // namespace

bool tc_plan_step(const StepArgs& s, size_t a_bits, size_t b_bits, size_t c_bits, bool tf32, TcStep* tc) {
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
    // eligibility: a real GEMM (M >= 128 rows, enough K x N reuse to leave the HBM roofline)
    if (t.nm < 7 || t.nk < 3 || t.nn < 2 || t.nn + t.nk < 8) return false;
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
    TcVariant v[kTcMaxVariants];
    const int nv = tc_variants(t, v);
    if (nv == 0) return false;
    t.planes_ok = false;
    t.scratch_max = 0;
    for (int i = 0; i < nv; i++) {
        tc_set_variant(t, v[i]);
        t.scratch_max = std::max(t.scratch_max, t.scratch_bytes);
        if (!v[i].fused) t.planes_ok = true;
    }
    tc_set_variant(t, v[0]);
    *tc = t;
    return true;
}

void tc_set_variant(TcStep& t, TcVariant v) {
    t.fused = v.fused;
    t.ntile_n = v.ntile;
    t.ntiles = cdiv(t.N, t.ntile_n);
    t.a_plane_bytes = t.fused ? 0 : (size_t)(t.batch * t.mtiles * t.kchunks) * kATileBytes;
    t.b_plane_bytes = (size_t)(t.batch * t.ntiles * t.kchunks) * (size_t)(2 * t.ntile_n * kTcChunkBytes);
    t.scratch_bytes = 2 * (t.a_plane_bytes + t.b_plane_bytes);
}

// N tiles of 16, 32 or 64 complex columns (two accumulators of 2*ntile FP32 columns: at 64 two
// CTAs fill an SM's 512 tensor-memory columns), no wider than N needs; fused first, then the
// planes variants whose scratch stays under 96 GB.  The first entry is the default.
int tc_variants(const TcStep& t, TcVariant* out) {
    const int widest = (int)std::min<int64_t>(64, std::max<int64_t>(16, t.N));
    int n = 0;
    for (int f = 1; f >= 0; f--)
        for (int nt = widest; nt >= 16; nt /= 2) {
            TcStep u = t;
            tc_set_variant(u, TcVariant{f == 1, nt});
            if (u.batch * u.mtiles * u.ntiles > (int64_t(1) << 31) - 1) continue;
            if (u.scratch_bytes > (size_t(96) << 30)) continue;
            if (n < kTcMaxVariants) out[n++] = TcVariant{f == 1, nt};
        }
    return n;
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

cudaError_t tc_run_gemm(const TcStep& t, const StepArgs& s, int* exps, void* scratch, cudaStream_t st) {
    uint8_t* base = static_cast<uint8_t*>(scratch);
    GemmArgs g;
    memset(&g, 0, sizeof(g));
    g.a_hi = base; g.a_lo = base + t.a_plane_bytes;
    g.b_hi = base + 2 * t.a_plane_bytes; g.b_lo = base + 2 * t.a_plane_bytes + t.b_plane_bytes;
    g.C = static_cast<float2*>(s.C);
    g.cb = t.cb; g.cm = t.cm; g.cn = t.cn;
    g.M = t.M; g.N = t.N; g.mtiles = t.mtiles; g.ntiles = t.ntiles; g.kchunks = t.kchunks; g.batch = t.batch;
    g.ntile = t.ntile_n;
    g.b_tile_bytes = (uint32_t)(2 * t.ntile_n * kTcChunkBytes);
    const uint32_t nmma = (uint32_t)(2 * t.ntile_n);
    const uint32_t fmt = t.tf32 ? 2u : 1u;           // TF32 : BF16 operand format
    g.idesc = (1u << 4) | (fmt << 7) | (fmt << 10) | ((nmma >> 3) << 17) | ((uint32_t)(kTcTileM >> 4) << 24);
    g.exp_c = s.expC;
    g.exps = exps;
    g.X = static_cast<const float2*>(t.x_is_a ? s.A : s.B);
    g.xb = t.xb; g.xm = t.xm; g.xk = t.xk;
    g.K = t.K;
    g.x_slot = t.x_is_a ? s.expA : s.expB;
    g.x_conj = t.x_is_a ? s.conjA : s.conjB;
    const size_t stage = 2 * kATileBytes + 2 * (size_t)g.b_tile_bytes;
    const size_t smem = (t.fused ? kStagesFused * stage + kRingBytes : kStages * stage) + 128;
    const int64_t ctas = t.batch * t.mtiles * t.ntiles;
    cudaError_t e;
    if (t.tf32 && t.fused) {
        if ((e = set_smem_attr<true, true>()) != cudaSuccess) return e;
        tc_gemm_kernel<true, true><<<(unsigned)ctas, kThreadsFused, smem, st>>>(g);
    } else if (t.tf32) {
        if ((e = set_smem_attr<true, false>()) != cudaSuccess) return e;
        tc_gemm_kernel<true, false><<<(unsigned)ctas, kThreadsGemm, smem, st>>>(g);
    } else if (t.fused) {
        if ((e = set_smem_attr<false, true>()) != cudaSuccess) return e;
        tc_gemm_kernel<false, true><<<(unsigned)ctas, kThreadsFused, smem, st>>>(g);
    } else {
        if ((e = set_smem_attr<false, false>()) != cudaSuccess) return e;
        tc_gemm_kernel<false, false><<<(unsigned)ctas, kThreadsGemm, smem, st>>>(g);
    }
    return cudaGetLastError();
}

cudaError_t tc_read_error(int* host_code, cudaStream_t st) {
    int zero = 0;
    cudaError_t e = cudaMemcpyFromSymbolAsync(host_code, g_tc_error, sizeof(int), 0, cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess) return e;
    e = cudaMemcpyToSymbolAsync(g_tc_error, &zero, sizeof(int), 0, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(st);
}

}  // namespace qxg
