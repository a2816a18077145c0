// Batched small GEMM with a long sum on the CUDA cores (Complex64 storage, FP32 products).
//
// The last joins of a sliced, bitstring-batched contraction tree contract two large halves of the
// network into a small result per (slice, bitstring):
//     C[b, m, n] = sum_k A[b, m, k] B[b, k, n]
// with M, N <= 64 free values per batch value b, 2^10 to 2^25 summed terms and 2^5 to 2^12 batch
// values, both operands holding 2^28 to 2^33 elements.  Each operand element is used by M or N
// results only (16 FLOPs per byte at M = N = 32), so the step is bound by HBM and by the FP32
// pipe together; the tensor-core path would first have to pack the smaller operand into hi/lo
// planes four times its size, and the long-sum kernel (built for a few dozen results) re-reads the
// operands once per block of 16 results.
//
// Here one block owns one batch value and one range of K:
//   * the block's threads tile the M x N result (TM x TN complex results per thread, in
//     registers);
//   * the K range is walked in chunks of 8 terms.  A chunk's A values (M x 8) and B values
//     (8 x N) are copied with 8-byte cp.async into a ring of raw chunks in shared memory, several
//     chunks ahead of the one being multiplied, in the order of the operands' own address bits (so
//     a warp's copies coalesce when the lowest address bits are result or summed bits).  Each
//     thread then turns its own elements of the current chunk, scaled by the operands'
//     power-of-two exponents, into (ar, ar, -ai, ai) and (br, bi, bi, br) quadruples, and a
//     complex multiply-add is two paired FMAs (fma.rn.f32x2) on one 16-byte read of each
//     (two quadruple buffers, one barrier per chunk).  The ring keeps tens of KB per SM in flight
//     without holding registers, which the step needs to reach HBM speed;
//   * every thread sums at most kFlushK terms in FP32 before adding them into FP32 TwoSum pairs
//     (about 48 bits, no FP64 pipe), so the error does not grow with K (the long-sum kernel's rule);
//   * with one K range per batch value the block writes C directly; otherwise it writes FP64
//     partials and bgemm_reduce_kernel adds them in range order (deterministic).
// Blocks are numbered batch value first, so blocks running side by side read neighbouring batch
// values: where a batch bit is among an operand's lowest address bits, the sectors one block
// fetches are read by its neighbour from L2.
#include <algorithm>

#include "simt_common.h"

namespace qxg {

constexpr int kFlushK = 512;            // FP32 terms per thread before the FP64 accumulation
constexpr size_t kBGemmMaxSmem = 96 * 1024;
constexpr size_t kBGemmRingTarget = 36 * 1024;   // quadruple buffers plus ring, per block
constexpr int kBGemmMaxChunkBits = 48;  // delta table entries (bits of the chunk index)
constexpr int kBGemmKC = 8;             // summed values per chunk

// ---- tile geometry, fixed at compile time per result shape (M x N per batch value) ----------------
//   threads    64 up to 1024 results per batch value, else M N / 16;
//   TM x TN    results per thread (4 or 2 each): thread (tm, tn) owns rows tm TM .. + TM-1 and
//              columns tn TN .. + TN-1;
//   kc         summed values per chunk (8): every thread copies 1..kBGemmMaxL elements of each
//              operand per chunk;
//   layout     a chunk's A quadruples as [k][row group][TM + 1] (one padding quadruple per group
//              keeps the groups of a warp in different banks) plus one per k, B likewise;
//   ring       raw chunks in flight, 3..8, as many as fit kBGemmRingTarget with the two
//              quadruple buffers (each raw chunk [j][thread] float2 for A, then for B).
struct BGemmShape {
    int M, N, nthr, tm, tn, thr_m, thr_n, kc, la, lb, ra, rb, ring;
    size_t quad_bytes, raw_bytes, smem;
};
constexpr BGemmShape bgemm_shape(int M, int N) {
    BGemmShape g{M, N, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    g.nthr = M * N / 16 > 64 ? M * N / 16 : 64;
    const int cand[4][2] = {{4, 4}, {2, 4}, {4, 2}, {2, 2}};     // (tm, tn)
    for (int c = 0; c < 4 && !g.tm; c++)
        if (M % cand[c][0] == 0 && N % cand[c][1] == 0 && (M / cand[c][0]) * (N / cand[c][1]) == g.nthr) {
            g.tm = cand[c][0];
            g.tn = cand[c][1];
        }
    if (!g.tm) return g;
    g.thr_m = M / g.tm;
    g.thr_n = N / g.tn;
    // one more padding quadruple per summed value: lanes that hold consecutive k of a chunk (the
    // summed bits are often an operand's lowest address bits) store into different banks
    g.ra = g.thr_m * (g.tm + 1) + 1;
    g.rb = g.thr_n * (g.tn + 1) + 1;
    const int kc = kBGemmKC;
    if (M * kc < g.nthr || N * kc < g.nthr || M * kc > g.nthr * kBGemmMaxL || N * kc > g.nthr * kBGemmMaxL) {
        g.tm = 0;
        return g;
    }
    g.kc = kc;
    g.la = M * kc / g.nthr;
    g.lb = N * kc / g.nthr;
    g.quad_bytes = (size_t)2 * kc * (g.ra + g.rb) * 16;
    g.raw_bytes = (size_t)(M + N) * kc * 8;
    g.ring = 3;
    while (g.ring < 8 && g.quad_bytes + (size_t)(g.ring + 1) * g.raw_bytes <= kBGemmRingTarget) g.ring++;
    g.smem = g.quad_bytes + (size_t)g.ring * g.raw_bytes;
    if (g.smem > kBGemmMaxSmem) g.tm = 0;
    return g;
}

__device__ __forceinline__ void bg_cp_async8(void* dst, const void* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)), "l"(src)
                 : "memory");
}
__device__ __forceinline__ void bg_cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void bg_cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// ---- phases of the kernel, shared with the host emulation of its index work --------------------

// Element j of thread tid in a chunk of A (j < la): its offset from the chunk's base and its
// shared-memory slot (in quadruples); the same for B (j < lb).
__host__ __device__ __forceinline__ void bgemm_elem_a(const BGemmArgs& g, int tid, int j, int64_t* off, int* slot) {
    const int64_t e = tid + (int64_t)j * (g.thr_m * g.thr_n);
    *off = pdep(e, g.eA);
    const int m = (int)pdep(e, g.eAm), tm = g.M / g.thr_m;
    *slot = (int)pdep(e, g.eAk) * g.ra + (m / tm) * (tm + 1) + m % tm;
}
__host__ __device__ __forceinline__ void bgemm_elem_b(const BGemmArgs& g, int tid, int j, int64_t* off, int* slot) {
    const int64_t e = tid + (int64_t)j * (g.thr_m * g.thr_n);
    *off = pdep(e, g.eB);
    const int n = (int)pdep(e, g.eBn), tn = g.N / g.thr_n;
    *slot = (int)pdep(e, g.eBk) * g.rb + (n / tn) * (tn + 1) + n % tn;
}
// Base offsets of chunk c of K range si for batch value bi.
__host__ __device__ __forceinline__ int64_t bgemm_base_a(const BGemmArgs& g, int64_t bi, int64_t si, int64_t c) {
    return pdep(bi, g.bA) + pdep(si * g.nchunks + c, g.hA);
}
__host__ __device__ __forceinline__ int64_t bgemm_base_b(const BGemmArgs& g, int64_t bi, int64_t si, int64_t c) {
    return pdep(bi, g.bB) + pdep(si * g.nchunks + c, g.hB);
}
// Walking chunk indices in order: base(c + 1) = base(c) + delta(t) with t = ctz(c + 1), where
// delta(t) = pdep(2^t) - pdep(2^t - 1) (bit t set, bits 0..t-1 cleared), so a chunk's base costs
// one table read and one add instead of a deposit over every run of the map.
__host__ __device__ __forceinline__ int64_t bgemm_delta(const BitMap& h, int t) {
    return pdep(int64_t(1) << t, h) - pdep((int64_t(1) << t) - 1, h);
}

// Shared-memory quadruples: A as (ar, ar, -ai, ai), B as (br, bi, bi, br), scaled (s) with the
// imaginary part's sign folded in for conjugation (si = -s).
__host__ __device__ __forceinline__ float4 bgemm_quad_a(float2 v, float s, float si) {
    const float ar = v.x * s, ai = v.y * si;
    return make_float4(ar, ar, -ai, ai);
}
__host__ __device__ __forceinline__ float4 bgemm_quad_b(float2 v, float s, float si) {
    const float br = v.x * s, bi = v.y * si;
    return make_float4(br, bi, bi, br);
}
// One chunk's products for thread (tm, tn).  A quadruple is read as two 64-bit halves -- (ar, ar)
// and (-ai, ai); (br, bi) and (bi, br) -- which are the paired FMAs' operands as they lie, and
// every read is at a compile-time offset from one of two base addresses.
template <int M, int N>
__host__ __device__ __forceinline__ void bgemm_chunk(const float4* as, const float4* bs, int tm, int tn,
                                                     unsigned long long (&acc)[bgemm_shape(M, N).tm]
                                                                              [bgemm_shape(M, N).tn]) {
    constexpr BGemmShape S = bgemm_shape(M, N);
    const ulonglong2* pa = reinterpret_cast<const ulonglong2*>(as) + tm * (S.tm + 1);
    const ulonglong2* pb = reinterpret_cast<const ulonglong2*>(bs) + tn * (S.tn + 1);
#pragma unroll
    for (int k = 0; k < S.kc; k++) {
        ulonglong2 qa[S.tm], qb[S.tn];
#pragma unroll
        for (int i = 0; i < S.tm; i++) qa[i] = pa[k * S.ra + i];
#pragma unroll
        for (int j = 0; j < S.tn; j++) qb[j] = pb[k * S.rb + j];
#pragma unroll
        for (int i = 0; i < S.tm; i++)
#pragma unroll
            for (int j = 0; j < S.tn; j++) fma2(acc[i][j], qa[i].x, qb[j].x);
#pragma unroll
        for (int i = 0; i < S.tm; i++)
#pragma unroll
            for (int j = 0; j < S.tn; j++) fma2(acc[i][j], qa[i].y, qb[j].y);
    }
}
// Knuth's TwoSum: (h, l) accumulates the flushed FP32 sums as an unevaluated pair (about 48 bits)
// without the FP64 pipe, which GB300 runs at a small fraction of FP32.
__host__ __device__ __forceinline__ void bgemm_two_sum(float& h, float& l, float x) {
    const float t = h + x, bp = t - h;
    l += (h - (t - bp)) + (x - bp);
    h = t;
}
// dacc = (re hi, re lo, im hi, im lo)
template <int TM, int TN>
__host__ __device__ __forceinline__ void bgemm_flush(unsigned long long (&acc)[TM][TN], float4 (&dacc)[TM][TN]) {
#pragma unroll
    for (int i = 0; i < TM; i++)
#pragma unroll
        for (int j = 0; j < TN; j++) {
            bgemm_two_sum(dacc[i][j].x, dacc[i][j].y, u2f((unsigned)acc[i][j]));
            bgemm_two_sum(dacc[i][j].z, dacc[i][j].w, u2f((unsigned)(acc[i][j] >> 32)));
            acc[i][j] = 0ull;
        }
}
__host__ __device__ __forceinline__ int64_t bgemm_c_offset(const BGemmArgs& g, int64_t bi, int m, int n) {
    return pdep(bi, g.bC) + pdep(m, g.mC) + pdep(n, g.nC);
}
// Result idx (batch-major, then m, then n) from the K-range partials, summed in range order.
__host__ __device__ __forceinline__ float2 bgemm_reduce_one(const BGemmArgs& g, const double2* partial, int64_t idx,
                                                            int64_t* c_off) {
    const int64_t per = (int64_t)g.M * g.N, total = g.nbatch * per;
    double re = 0.0, im = 0.0;
    for (int s = 0; s < g.nsplit; s++) {
        const double2 v = partial[s * total + idx];
        re += v.x;
        im += v.y;
    }
    const int64_t r = idx % per;
    *c_off = bgemm_c_offset(g, idx / per, (int)(r / g.N), (int)(r % g.N));
    return make_float2((float)re, (float)im);
}

// The result shapes served (M, N per batch value); F(M, N) is expanded once per shape.
#define QXG_BGEMM_SHAPES(F)                                                                           \
    F(8, 32) F(8, 64) F(16, 16) F(16, 32) F(16, 64) F(32, 8) F(32, 16) F(32, 32) F(32, 64) F(64, 8) \
    F(64, 16) F(64, 32) F(64, 64)

namespace {

// at least six blocks of 64 threads (12 warps) per SM: the registers are capped to fit them
template <int M, int N, bool SCALED>
__global__ void __launch_bounds__(bgemm_shape(M, N).nthr, bgemm_shape(M, N).nthr <= 64 ? 6 : 384 / bgemm_shape(M, N).nthr)
    contract_bgemm_kernel(const BGemmArgs g, double2* partial, int* exps) {
    constexpr BGemmShape S = bgemm_shape(M, N);
    constexpr int NT = S.nthr, R = S.ring;
    extern __shared__ float4 bg_smem[];
    const int tid = threadIdx.x;
    const int tn = tid % S.thr_n, tm = tid / S.thr_n;
    const int64_t bi = (int64_t)blockIdx.x % g.nbatch;
    const int64_t si = (int64_t)blockIdx.x / g.nbatch;
    float4* As = bg_smem;                                  // [2][kc][ra]
    float4* Bs = bg_smem + 2 * S.kc * S.ra;                // [2][kc][rb]
    float2* raw = reinterpret_cast<float2*>(Bs + 2 * S.kc * S.rb);   // [R][la + lb][NT]
    __shared__ int64_t dA[kBGemmMaxChunkBits], dB[kBGemmMaxChunkBits];
    for (int t = tid; t < kBGemmMaxChunkBits; t += NT) {
        dA[t] = bgemm_delta(g.hA, t);
        dB[t] = bgemm_delta(g.hB, t);
    }
    float sa = 1.f, sb = 1.f;
    if (SCALED) {
        sa = pow2f(-read_m(exps, g.expA));
        sb = pow2f(-read_m(exps, g.expB));
    }
    const float sai = g.conjA ? -sa : sa, sbi = g.conjB ? -sb : sb;
    int64_t offA[S.la], offB[S.lb];
    int slotA[S.la], slotB[S.lb];
#pragma unroll
    for (int j = 0; j < S.la; j++) bgemm_elem_a(g, tid, j, &offA[j], &slotA[j]);
#pragma unroll
    for (int j = 0; j < S.lb; j++) bgemm_elem_b(g, tid, j, &offB[j], &slotB[j]);
    // chunk c's raw elements go to ring slot c % R: [j][tid], A's la rows then B's lb rows; each
    // thread copies and later reads back only its own elements.  Chunks are issued in order, so
    // their bases advance by the delta table (the first from a full deposit).
    const int64_t c0 = si * g.nchunks;
    int64_t baseA = bgemm_base_a(g, bi, si, 0), baseB = bgemm_base_b(g, bi, si, 0);
    __syncthreads();                        // delta tables written
    auto issue = [&](int64_t c) {
        if (c < g.nchunks) {
            const float2* a = g.A + baseA;
            const float2* b = g.B + baseB;
            const int t = __ffsll((unsigned long long)(c0 + c + 1)) - 1;
            baseA += dA[t];
            baseB += dB[t];
            float2* r = raw + (size_t)(c % R) * (S.la + S.lb) * NT + tid;
#pragma unroll
            for (int j = 0; j < S.la; j++) bg_cp_async8(r + j * NT, a + offA[j]);
#pragma unroll
            for (int j = 0; j < S.lb; j++) bg_cp_async8(r + (S.la + j) * NT, b + offB[j]);
        }
        bg_cp_async_commit();               // one group per chunk (empty past the end)
    };
    auto stage = [&](int64_t c) {
        const float2* r = raw + (size_t)(c % R) * (S.la + S.lb) * NT + tid;
        float4* as = As + (int)(c & 1) * S.kc * S.ra;
        float4* bs = Bs + (int)(c & 1) * S.kc * S.rb;
#pragma unroll
        for (int j = 0; j < S.la; j++) as[slotA[j]] = bgemm_quad_a(r[j * NT], sa, sai);
#pragma unroll
        for (int j = 0; j < S.lb; j++) bs[slotB[j]] = bgemm_quad_b(r[(S.la + j) * NT], sb, sbi);
    };
    unsigned long long acc[S.tm][S.tn];
    float4 dacc[S.tm][S.tn];
#pragma unroll
    for (int i = 0; i < S.tm; i++)
#pragma unroll
        for (int j = 0; j < S.tn; j++) {
            acc[i][j] = 0ull;
            dacc[i][j] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
#pragma unroll
    for (int c = 0; c < R - 1; c++) issue(c);
    for (int64_t c = 0; c < g.nchunks; c++) {
        issue(c + R - 1);
        bg_cp_async_wait<R - 1>();          // chunk c's own copies have landed
        stage(c);
        __syncthreads();                    // chunk c's quadruples are complete
        bgemm_chunk<M, N>(As + (int)(c & 1) * S.kc * S.ra, Bs + (int)(c & 1) * S.kc * S.rb, tm, tn, acc);
        if (((c + 1) & (g.flush - 1)) == 0 || c + 1 == g.nchunks) bgemm_flush<S.tm, S.tn>(acc, dacc);
    }
    bg_cp_async_wait<0>();                  // nothing lands after the block has left
    if (g.nsplit == 1) {
        int emax = kExpUnset;
#pragma unroll
        for (int i = 0; i < S.tm; i++)
#pragma unroll
            for (int j = 0; j < S.tn; j++) {
                const float2 v = make_float2(dacc[i][j].x + dacc[i][j].y, dacc[i][j].z + dacc[i][j].w);
                g.C[bgemm_c_offset(g, bi, tm * S.tm + i, tn * S.tn + j)] = v;
                const float mx = fmaxf(fabsf(v.x), fabsf(v.y));
                if (SCALED && mx > 0.f) emax = max(emax, exp_of(mx));
            }
        if (SCALED) {
            if (blockIdx.x == 0 && tid == 0)
                exps[2 * g.expC] = exps[2 * g.expA] + exps[2 * g.expB] + read_m(exps, g.expA) + read_m(exps, g.expB);
            for (int o = 16; o > 0; o >>= 1) emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, o));
            if ((tid & 31) == 0 && emax != kExpUnset) atomicMax(&exps[2 * g.expC + 1], emax);
        }
    } else {
        // partial[si][bi][m][n] in FP64, added in K-range order by bgemm_reduce_kernel
        double2* p = partial + ((si * g.nbatch + bi) * M) * N;
#pragma unroll
        for (int i = 0; i < S.tm; i++)
#pragma unroll
            for (int j = 0; j < S.tn; j++)
                p[(tm * S.tm + i) * N + tn * S.tn + j] =
                    make_double2((double)dacc[i][j].x + (double)dacc[i][j].y, (double)dacc[i][j].z + (double)dacc[i][j].w);
    }
}

template <bool SCALED>
__global__ void bgemm_reduce_kernel(const BGemmArgs g, const double2* partial, int* exps) {
    const int64_t total = g.nbatch * g.M * g.N;
    int emax = kExpUnset;
    if (SCALED && blockIdx.x == 0 && threadIdx.x == 0)
        exps[2 * g.expC] = exps[2 * g.expA] + exps[2 * g.expB] + read_m(exps, g.expA) + read_m(exps, g.expB);
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        int64_t off;
        const float2 v = bgemm_reduce_one(g, partial, idx, &off);
        g.C[off] = v;
        const float mx = fmaxf(fabsf(v.x), fabsf(v.y));
        if (SCALED && mx > 0.f) emax = max(emax, exp_of(mx));
    }
    if (SCALED) {
        for (int o = 16; o > 0; o >>= 1) emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, o));
        if ((threadIdx.x & 31) == 0 && emax != kExpUnset) atomicMax(&exps[2 * g.expC + 1], emax);
    }
}

int ilog2(int64_t x) {
    int b = 0;
    while ((int64_t(1) << b) < x) b++;
    return b;
}

// A run of length one per element bit: the element index's bits go to scattered places.
bool bit_runs(const std::vector<std::pair<int, int>>& p, BitMap* m) {
    memset(m, 0, sizeof(*m));
    for (auto& x : p) {
        if (m->n >= kMaxRuns) return false;
        m->r[m->n++] = Run{(uint8_t)x.first, 1, (uint8_t)x.second, 0};
    }
    return true;
}

}  // namespace

// Plan the batched small GEMM form of a step (Complex64 storage only).  Eligible: every result
// bit in A or B, every summed bit in both; a result shape of QXG_BGEMM_SHAPES (8 to 64 free values
// on each side, at least 256 results per batch value); at least 2^10 summed terms; both operands
// of at least 2^min_log2 elements (smaller steps are served by the row forms and the tensor
// cores; the host emulation of the kernel lowers the floor).
bool plan_bgemm(const StepArgs& s, int sm_count, BGemmArgs* g, int min_log2) {
    if (s.nk < 10) return false;
    auto one = [](const BitMap& m, int bit) {
        const int64_t o = pdep(int64_t(1) << bit, m);
        return o ? __builtin_ctzll((unsigned long long)o) : -1;
    };
    const int ncb = ilog2(s.nC);
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
    if (na < 3 || nb < 3 || na > 6 || nb > 6 || na + nb < 8 || ng > 30) return false;
    if (ng + std::min(na, nb) + s.nk < min_log2) return false;
    const BGemmShape S = bgemm_shape(1 << na, 1 << nb);
    if (!S.tm) return false;
    bool served = false;
#define QXG_BGEMM_IS(M_, N_) served = served || (S.M == M_ && S.N == N_);
    QXG_BGEMM_SHAPES(QXG_BGEMM_IS)
#undef QXG_BGEMM_IS
    if (!served) return false;
    BGemmArgs a;
    memset(&a, 0, sizeof(a));
    a.M = S.M;
    a.N = S.N;
    a.thr_m = S.thr_m;
    a.thr_n = S.thr_n;
    a.kc = S.kc;
    a.la = S.la;
    a.lb = S.lb;
    a.ra = S.ra;
    a.rb = S.rb;
    const int lkc = ilog2(S.kc);
    if (lkc > s.nk) return false;
    // the chunk's summed bits: those at the lowest address positions of either operand
    std::vector<int> ks(s.nk), posA(s.nk), posB(s.nk);
    for (int j = 0; j < s.nk; j++) { ks[j] = j; posA[j] = one(s.kA, j); posB[j] = one(s.kB, j); }
    std::sort(ks.begin(), ks.end(), [&](int x, int y) {
        const int px = std::min(posA[x], posB[x]), py = std::min(posA[y], posB[y]);
        return px != py ? px < py : x < y;
    });
    // chunk element e: its bits are the chunk's (m, k) bits of A in A's address order (and (n, k)
    // of B in B's), so consecutive elements are at ascending addresses
    auto element_maps = [&](const BitMap& cmap, const std::vector<int>& freebits, const BitMap& kmap,
                            BitMap* e_off, BitMap* e_free, BitMap* e_k) {
        struct Bit { int pos, kind, idx; };
        std::vector<Bit> bits;
        for (int i = 0; i < (int)freebits.size(); i++) bits.push_back({one(cmap, freebits[i]), 0, i});
        for (int i = 0; i < lkc; i++) bits.push_back({one(kmap, ks[i]), 1, i});
        std::sort(bits.begin(), bits.end(), [](const Bit& x, const Bit& y) { return x.pos < y.pos; });
        std::vector<std::pair<int, int>> off, fr, kk;
        for (int e = 0; e < (int)bits.size(); e++) {
            off.push_back({e, bits[e].pos});
            (bits[e].kind == 0 ? fr : kk).push_back({e, bits[e].idx});
        }
        return bit_runs(off, e_off) && bit_runs(fr, e_free) && bit_runs(kk, e_k);
    };
    if (!element_maps(s.cA, ab, s.kA, &a.eA, &a.eAm, &a.eAk)) return false;
    if (!element_maps(s.cB, bb, s.kB, &a.eB, &a.eBn, &a.eBk)) return false;
    std::vector<std::pair<int, int>> bA, bB, bC, mC, nC, hA, hB;
    for (int i = 0; i < ng; i++) {
        bA.push_back({i, one(s.cA, gb[i])});
        bB.push_back({i, one(s.cB, gb[i])});
        bC.push_back({i, gb[i]});
    }
    for (int i = 0; i < na; i++) mC.push_back({i, ab[i]});
    for (int i = 0; i < nb; i++) nC.push_back({i, bb[i]});
    for (int i = lkc; i < s.nk; i++) {
        hA.push_back({i - lkc, posA[ks[i]]});
        hB.push_back({i - lkc, posB[ks[i]]});
    }
    if (!make_runs(bA, &a.bA) || !make_runs(bB, &a.bB) || !make_runs(bC, &a.bC) || !make_runs(mC, &a.mC) ||
        !make_runs(nC, &a.nC) || !make_runs(hA, &a.hA) || !make_runs(hB, &a.hB))
        return false;
    a.nbatch = int64_t(1) << ng;
    const int64_t chunks = int64_t(1) << (s.nk - lkc);
    // K ranges: enough blocks for about four per SM, each range at least 2^9 terms
    int64_t nsplit = 1;
    while (a.nbatch * nsplit < (int64_t)sm_count * 4 && chunks / (nsplit * 2) * S.kc >= 512) nsplit *= 2;
    if (a.nbatch * nsplit > (int64_t(1) << 31) - 1) return false;
    a.nsplit = (int)nsplit;
    a.nchunks = chunks / nsplit;
    a.flush = std::max(1, kFlushK / S.kc);  // a power of two
    if (s.nk - lkc >= kBGemmMaxChunkBits) return false;
    a.A = static_cast<const float2*>(s.A);
    a.B = static_cast<const float2*>(s.B);
    a.C = static_cast<float2*>(s.C);
    a.conjA = s.conjA;
    a.conjB = s.conjB;
    a.expA = s.expA;
    a.expB = s.expB;
    a.expC = s.expC;
    *g = a;
    return true;
}

size_t bgemm_partial_bytes(const BGemmArgs& g) {
    return g.nsplit > 1 ? (size_t)g.nsplit * (size_t)g.nbatch * g.M * g.N * sizeof(double2) : 0;
}

namespace {
template <int M, int N, bool SCALED>
cudaError_t launch_bgemm_shape(const BGemmArgs& g, double2* partial, int* exps, cudaStream_t s) {
    constexpr BGemmShape S = bgemm_shape(M, N);
    static bool attr = false;                   // the kernel's dynamic shared memory limit, once
    if (!attr) {
        const cudaError_t e = cudaFuncSetAttribute(contract_bgemm_kernel<M, N, SCALED>,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S.smem);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    contract_bgemm_kernel<M, N, SCALED><<<(unsigned)(g.nbatch * g.nsplit), S.nthr, S.smem, s>>>(g, partial, exps);
    return cudaGetLastError();
}
}  // namespace

cudaError_t launch_bgemm(const BGemmArgs& g, void* scratch, int* exps, cudaStream_t s, int* launches) {
    if (g.nsplit > 1 && !scratch) return cudaErrorInvalidValue;
    double2* partial = static_cast<double2*>(scratch);
    cudaError_t e = cudaErrorInvalidValue;
#define QXG_BGEMM_LAUNCH(M_, N_)                                                              \
    if (g.M == M_ && g.N == N_)                                                               \
        e = exps ? launch_bgemm_shape<M_, N_, true>(g, partial, exps, s)                      \
                 : launch_bgemm_shape<M_, N_, false>(g, partial, exps, s);
    QXG_BGEMM_SHAPES(QXG_BGEMM_LAUNCH)
#undef QXG_BGEMM_LAUNCH
    if (e != cudaSuccess) return e;
    if (launches) *launches = 1;
    if (g.nsplit > 1) {
        const int64_t total = g.nbatch * g.M * g.N;
        const int grid = (int)std::min<int64_t>((total + 255) / 256, 4096);
        if (exps) bgemm_reduce_kernel<true><<<grid, 256, 0, s>>>(g, partial, exps);
        else bgemm_reduce_kernel<false><<<grid, 256, 0, s>>>(g, partial, exps);
        if (launches) *launches = 2;
        e = cudaGetLastError();
    }
    return e;
}

}  // namespace qxg
