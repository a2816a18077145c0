// Helpers shared by the CUDA-core kernels (kernels_simt.cu) and the compact row form
// (kernels_rows.cu): value types, exponent arithmetic, paired FP32 FMAs, the row-form arguments.
#pragma once

#include <cstring>
#include <vector>

#include "qxgpu_internal.h"

namespace qxg {

template <typename T> struct Real;
template <> struct Real<double2> { using type = double; };
template <> struct Real<float2> { using type = float; };

constexpr int kThreads = 256;

// 2^n as a float for |n| <= 126 by building the IEEE bits directly (exact power of two).
__device__ __forceinline__ float pow2f(int n) {
    n = n < -126 ? -126 : (n > 127 ? 127 : n);
    return __int_as_float((n + 127) << 23);
}
__device__ __forceinline__ double pow2d(int n) {
    n = n < -1022 ? -1022 : (n > 1023 ? 1023 : n);
    return __longlong_as_double((long long)(n + 1023) << 52);
}
// Binary exponent e of |x| with |x| in [2^(e-1), 2^e) for normal floats (frexp convention).
__host__ __device__ __forceinline__ int exp_of(float x) {
#ifdef __CUDA_ARCH__
    const unsigned u = __float_as_uint(x);
#else
    unsigned u;
    std::memcpy(&u, &x, sizeof(u));
#endif
    return (int)((u >> 23) & 0xffu) - 126;
}

__device__ __forceinline__ int read_m(const int* exps, int slot) {
    int m = exps[2 * slot + 1];
    return m < -400 ? 0 : m;            // all-zero tensor: no scaling
}

__host__ __device__ __forceinline__ unsigned f2u(float x) {
#ifdef __CUDA_ARCH__
    return __float_as_uint(x);
#else
    unsigned u;
    std::memcpy(&u, &x, sizeof(u));
    return u;
#endif
}
__host__ __device__ __forceinline__ float u2f(unsigned u) {
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float x;
    std::memcpy(&x, &u, sizeof(x));
    return x;
#endif
}
__host__ __device__ __forceinline__ unsigned long long f2pack(float lo, float hi) {
    return (unsigned long long)f2u(lo) | ((unsigned long long)f2u(hi) << 32);
}
// d += a * b on both FP32 halves, each rounded once (fused).
__host__ __device__ __forceinline__ void fma2(unsigned long long& d, unsigned long long a, unsigned long long b) {
#ifdef __CUDA_ARCH__
    asm("fma.rn.f32x2 %0, %1, %2, %0;" : "+l"(d) : "l"(a), "l"(b));
#else
    const float lo = std::fmaf(u2f((unsigned)a), u2f((unsigned)b), u2f((unsigned)d));
    const float hi = std::fmaf(u2f((unsigned)(a >> 32)), u2f((unsigned)(b >> 32)), u2f((unsigned)(d >> 32)));
    d = f2pack(lo, hi);
#endif
}

// Row form of a contraction whose smaller operand Y is small (gate-like steps:
// C[b,m,n] = sum_k X[b,m,k] Y[b,k,n] with K and N small); rows enumerate the result's bits other
// than the n bits (rowmap).
struct RowArgs {
    const void* X;
    const void* Y;
    void* C;
    int64_t nrows;
    int32_t N, K, ny;          // result columns, summed extent, elements of Y
    int32_t conjX, conjY;
    int32_t expX, expY, expC;
    BitMap rowmap, nmap;       // row index / n index -> result index
    BitMap cX, cY;             // result index -> X / Y offset
    BitMap kX, kY;             // k -> X / Y offset
};

// Row form, compact: the row form with the loop work cut to the arithmetic, for FP32 steps with
// compile-time K and N.  The row kernel above spends most of its issue slots on index work (bit
// deposits per row, table reads and address arithmetic per (k, n)); here
//   * a warp walks a contiguous range of 32-row groups (lanes = the 5 lowest row bits) and moves
//     from one group to the next by adding per-bit offset deltas (the bits of g+1 that differ
//     from g are 0..ctz(g+1)), so a row costs a few integer adds instead of three deposits;
//   * Y is restaged densely as [batch][k][n] of (re, im, im, re) quadruples, so every (k, n)
//     reads one 16-byte word at a compile-time offset from the row's batch base (batches padded
//     by one word so lanes of different batches fall in different banks);
//   * the complex product uses paired FP32 FMAs (fma.rn.f32x2): acc += (xr, xr) * (yr, yi) and
//     acc += (-xi, xi) * (yi, yr), the same roundings in the same order as four scalar FMAs;
//   * X pairs (k, k+1) and C pairs (n, n+1) move as 16-byte words when k bit 0 / n bit 0 is the
//     operand's / result's lowest address bit;
//   * more than N result columns run as nchunk chunks of N from the same X registers, and steps
//     with fewer than 32 rows leave the lanes above 2^(row bits) idle.
struct Rows2Args {
    const void* X;
    const void* Y;
    void* C;
    int64_t ngroups;           // groups of `lanes` rows
    int32_t lanes;             // active lanes (rows per group): 32, or 2^(row bits) below that
    int32_t nchunk;            // chunks of N result columns
    int32_t ncol;              // N: result columns per chunk (the kernel's template parameter)
    int32_t nbatch;            // Y batches (values of the row bits Y has)
    int32_t conjX, conjY;
    int32_t expX, expY, expC;
    int32_t xpair, cpair;
    BitMap laneX, laneC, laneB;    // lane -> X offset / C offset / batch index
    BitMap grpX, grpC, grpB;       // group index -> X / C offset / batch index
    BitMap kX, kY, nC, nY;         // k -> X / Y offset, n -> C / Y offset
    BitMap bY;                     // batch index -> Y offset
};
constexpr int kRows2MaxY = 8192;        // elements of Y (a 16-byte quadruple each in shared memory)
constexpr int kRows2MaxYBits = 13;

// Batched small GEMM with a long sum (kernels_bgemm.cu): C[b, m, n] = sum_k A[b, m, k] B[b, k, n]
// with 4..64 free values per side and at least 2^10 summed terms, both operands large -- the
// final joins of sliced, bitstring-batched trees.
constexpr int kBGemmMaxL = 8;           // operand elements one thread loads per chunk (per operand)
struct BGemmArgs {
    const float2* A;
    const float2* B;
    float2* C;
    int32_t M, N;              // free values of A (rows) and of B (columns) per batch value
    int32_t thr_m, thr_n;      // thread grid: thread (tm, tn) owns rows tm TM + i, columns tn TN + j
    int32_t kc;                // summed values per chunk
    int32_t la, lb;            // A / B elements one thread loads per chunk
    int32_t ra, rb;            // quadruples per summed value of a chunk in shared memory (A / B)
    int64_t nchunks;           // chunks of one K range
    int32_t nsplit;            // K ranges per batch value (a power of two)
    int32_t flush;             // chunks between FP64 accumulations
    int64_t nbatch;
    int32_t conjA, conjB, expA, expB, expC;
    BitMap bA, bB, bC;         // batch index -> A / B / C offset
    BitMap mC, nC;             // m / n -> C offset
    BitMap eA, eB;             // chunk element (in address order) -> A / B offset within the chunk
    BitMap eAm, eAk, eBn, eBk; // chunk element -> m / k-in-chunk (A); n / k-in-chunk (B)
    BitMap hA, hB;             // chunk index within the whole K -> A / B offset
};
// Fill the batched small GEMM form of a step (false: the step does not fit it); both operands
// need at least 2^min_log2 elements.
bool plan_bgemm(const StepArgs& s, int sm_count, BGemmArgs* g, int min_log2 = 20);
// Scratch for the FP64 partials of its K ranges (0 with one range per batch value).
size_t bgemm_partial_bytes(const BGemmArgs& g);
// Launch it (and the ordered sum of the K-range partials); *launches receives 1 or 2.
cudaError_t launch_bgemm(const BGemmArgs& g, void* scratch, int* exps, cudaStream_t s, int* launches);

// Fill the compact row form from a row form (false: the step does not fit it).
bool plan_rows2(const RowArgs& ra, Rows2Args* r2);
// Launch the compact row form with K summed values and N result columns per chunk.
cudaError_t launch_rows2(const Rows2Args& r2, int K, int N, int* exps, cudaStream_t s, int sm_count);

}  // namespace qxg
