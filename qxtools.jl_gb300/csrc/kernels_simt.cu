// CUDA-core kernels of the executor: the pairwise contraction (one `ncon` command,
// docs/src/users_guide.md:124-146) in its general, row (FP64), long-sum, split-K and batched
// forms, view materialisation for a batch of slices (users_guide.md:104-122), output vectors for
// a batch of bitstrings (users_guide.md:149-158), the FP64 sum over slices (users_guide.md:11-17)
// and the gradient's seed, view-adjoint and leaf-gradient kernels.  The compact row form of the
// Complex64 gate steps is in kernels_rows.cu; launch_contract picks the form of a step.
//
// The general kernel is the plain executor's hot loop (ComplexF64 on the FP64 pipe) and the
// fallback of the Complex64 executors (FP32 FMA).  A block owns tiles of 2^TB
// consecutive result elements; because a bit permutation is additive over disjoint bits,
// offset(tile | lo) = offset(tile) + offset(lo), so the low-bit offsets of the result and all
// K offsets (up to 2^kKTableBits) are tabulated once per block in shared memory and each
// element costs two table reads instead of a full bit deposit.
#include <algorithm>
#include <cstring>
#include <vector>

#include "qxgpu_internal.h"
#include "simt_common.h"

namespace qxg {

// Resident blocks per SM of the long-sum kernel instance (NA, NB) with `smem` bytes (2 when the
// query fails, e.g. without a device).
int lsum_blocks_per_sm(int NA, int NB, size_t smem);

namespace {

constexpr int kTileBits = 10;          // 1024 result elements per tile, 4 per thread

// CONJ bit 0 / bit 1: use the complex conjugate of A / B (adjoint steps).  A compile-time sign
// folds into the FMA operands, so the forward path pays nothing for it.
template <typename T, bool SCALED, int CONJ>
__global__ void __launch_bounds__(kThreads)
contract_kernel(const StepArgs a, int* exps) {
    using R = typename Real<T>::type;
    __shared__ int64_t tA[1 << kKTableBits], tB[1 << kKTableBits];
    __shared__ int64_t lA[1 << kTileBits], lB[1 << kTileBits];
    const int nkt = a.nk < kKTableBits ? a.nk : kKTableBits;
    const int KT = 1 << nkt;
    int ncb = 0;
    while ((int64_t(1) << ncb) < a.nC) ncb++;
    const int tb = ncb < kTileBits ? ncb : kTileBits;
    const int TS = 1 << tb;
    for (int k = threadIdx.x; k < KT; k += kThreads) { tA[k] = pdep(k, a.kA); tB[k] = pdep(k, a.kB); }
    for (int i = threadIdx.x; i < TS; i += kThreads) { lA[i] = pdep(i, a.cA); lB[i] = pdep(i, a.cB); }
    __syncthreads();

    const T* __restrict__ A = static_cast<const T*>(a.A);
    const T* __restrict__ B = static_cast<const T*>(a.B);
    T* __restrict__ C = static_cast<T*>(a.C);
    const int64_t KO = int64_t(1) << (a.nk - nkt);
    R scale = R(1);
    if (SCALED) {
        const int mA = read_m(exps, a.expA), mB = read_m(exps, a.expB);
        scale = (R)pow2f(-(mA + mB));
        if (blockIdx.x == 0 && threadIdx.x == 0)
            exps[2 * a.expC] = exps[2 * a.expA] + exps[2 * a.expB] + mA + mB;
    }
    int emax = kExpUnset;
    const int64_t ntiles = a.nC >> tb;
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int64_t tbase = t << tb;
        const int64_t ta = pdep(tbase, a.cA), tbb = pdep(tbase, a.cB);
        for (int i = threadIdx.x; i < TS; i += kThreads) {
            const int64_t a0 = ta + lA[i], b0 = tbb + lB[i];
            R re = R(0), im = R(0);
            for (int64_t ko = 0; ko < KO; ko++) {
                const int64_t ah = a0 + (ko ? pdep(ko << nkt, a.kA) : 0);
                const int64_t bh = b0 + (ko ? pdep(ko << nkt, a.kB) : 0);
#pragma unroll 4
                for (int k = 0; k < KT; k++) {
                    const T x = A[ah + tA[k]];
                    const T y = B[bh + tB[k]];
                    const R xi = (CONJ & 1) ? -x.y : x.y, yi = (CONJ & 2) ? -y.y : y.y;
                    re = fma(x.x, y.x, re);
                    re = fma(-xi, yi, re);
                    im = fma(x.x, yi, im);
                    im = fma(xi, y.x, im);
                }
            }
            if (SCALED) {
                re *= scale; im *= scale;
                const float mx = fmaxf(fabsf((float)re), fabsf((float)im));
                if (mx > 0.f) emax = max(emax, exp_of(mx));
            }
            T out; out.x = re; out.y = im;
            C[tbase + i] = out;
        }
    }
    if (SCALED) {
        for (int o = 16; o > 0; o >>= 1) emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, o));
        if ((threadIdx.x & 31) == 0 && emax != kExpUnset) atomicMax(&exps[2 * a.expC + 1], emax);
    }
}

// Row form of a contraction whose smaller operand Y fits in shared memory (gate-like steps:
// C[b,m,n] = sum_k X[b,m,k] Y[b,k,n] with K and N small).  A thread owns one row (b,m): it loads
// the row's K values of X once into registers and writes all N results, so X is read once and C
// written once, and Y is read from its shared-memory copy.  Rows enumerate the result's bits
// other than the n bits (rowmap), consecutive rows are consecutive result bits, so the X loads
// and C stores of a warp fall on consecutive addresses whenever the layouts allow it.
constexpr int kRowMaxN = 1024;          // result columns per row (tabulated offsets)

template <typename T, bool SCALED, int KMAX>
__global__ void __launch_bounds__(kThreads) contract_rows_kernel(const RowArgs a, int* exps) {
    using R = typename Real<T>::type;
    extern __shared__ __align__(16) unsigned char rows_smem[];
    T* Ys = reinterpret_cast<T*>(rows_smem);
    int64_t* kx = reinterpret_cast<int64_t*>(Ys + a.ny);
    int64_t* cn = kx + KMAX;
    int32_t* ky = reinterpret_cast<int32_t*>(cn + a.N);
    int32_t* cyn = ky + KMAX;
    const T* __restrict__ X = static_cast<const T*>(a.X);
    const T* __restrict__ Y = static_cast<const T*>(a.Y);
    T* __restrict__ C = static_cast<T*>(a.C);
    for (int j = threadIdx.x; j < a.ny; j += kThreads) {
        T y = Y[j];
        if (a.conjY) y.y = -y.y;                 // the shared copy holds conj(Y) when asked
        Ys[j] = y;
    }
    for (int k = threadIdx.x; k < KMAX; k += kThreads) {
        kx[k] = k < a.K ? pdep(k, a.kX) : 0;
        ky[k] = k < a.K ? (int32_t)pdep(k, a.kY) : 0;
    }
    for (int n = threadIdx.x; n < a.N; n += kThreads) {
        cn[n] = pdep(n, a.nmap);
        cyn[n] = (int32_t)pdep(cn[n], a.cY);
    }
    __syncthreads();
    R scale = R(1);
    if (SCALED) {
        const int mX = read_m(exps, a.expX), mY = read_m(exps, a.expY);
        scale = (R)pow2f(-(mX + mY));
        if (blockIdx.x == 0 && threadIdx.x == 0)
            exps[2 * a.expC] = exps[2 * a.expX] + exps[2 * a.expY] + mX + mY;
    }
    int emax = kExpUnset;
    const R sx = a.conjX ? R(-1) : R(1);
    for (int64_t r = blockIdx.x * (int64_t)kThreads + threadIdx.x; r < a.nrows; r += (int64_t)gridDim.x * kThreads) {
        const int64_t ir = pdep(r, a.rowmap);
        const int64_t xo = pdep(ir, a.cX);
        const int yo = (int)pdep(ir, a.cY);
        R xr[KMAX], xi[KMAX];
#pragma unroll
        for (int k = 0; k < KMAX; k++) {
            xr[k] = R(0); xi[k] = R(0);
            if (k < a.K) {
                const T v = X[xo + kx[k]];
                xr[k] = v.x; xi[k] = sx * v.y;
            }
        }
        for (int n = 0; n < a.N; n++) {
            const T* yrow = Ys + yo + cyn[n];
            R re = R(0), im = R(0);
#pragma unroll
            for (int k = 0; k < KMAX; k++) {
                if (k < a.K) {
                    const T y = yrow[ky[k]];
                    re = fma(xr[k], y.x, re);
                    re = fma(-xi[k], y.y, re);
                    im = fma(xr[k], y.y, im);
                    im = fma(xi[k], y.x, im);
                }
            }
            if (SCALED) {
                re *= scale; im *= scale;
                const float mx = fmaxf(fabsf((float)re), fabsf((float)im));
                if (mx > 0.f) emax = max(emax, exp_of(mx));
            }
            T out; out.x = re; out.y = im;
            C[ir + cn[n]] = out;
        }
    }
    if (SCALED) {
        for (int o = 16; o > 0; o >>= 1) emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, o));
        if ((threadIdx.x & 31) == 0 && emax != kExpUnset) atomicMax(&exps[2 * a.expC + 1], emax);
    }
}

// Long sum with a small result (FP32): C[a, b, g] = sum_r A[a, g, r] B[b, g, r], the summed index
// r long (the adjoint steps that end in a gate's gradient sum over every other index of the
// network); "a" are the result bits only A has, "b" those only B has, "g" those both have.  It
// walks r the way the compact row form walks rows: a warp takes a contiguous range of groups of
// 2^LR values of r (the LR summed bits lowest in the larger operand), two groups per step, and
// moves between groups by per-bit offset deltas.  The results are cut into lane blocks of NA a
// values x NB b values: the 32 lanes of a warp are 2^LR values of r times S = 32 / 2^LR
// sub-lanes (consecutive a blocks), and the CW = CA x CB warps of a block that share a row range
// take different a and b blocks (8 / CW such warp sets divide the block's rows).  A lane loads
// its r's NA values of A and NB of B (16-byte pairs where a / b bit 0 is the lowest address
// bit) and adds their outer product into NA x NB registers with paired FP32 FMAs; elements that
// several lanes need come from memory once per warp instruction or from L1.  Block (g, part)
// sums its lanes in FP64 (fixed butterfly, then its warps in order) into one partial per result;
// a second kernel adds the parts in order, scales and stores: deterministic.  At most
// kLSumRowsPerLane values of r per lane go through FP32 sums.
struct LSumArgs {
    const void* A;
    const void* B;
    void* C;
    int64_t ngroups;           // groups of 2^LR values of r
    int32_t LR;                // r bits per lane group (2..5)
    int32_t CA, CB;            // a / b blocks across the warps of one row range
    int32_t nrc;               // chunks of the a values over the grid's second dimension
    int32_t G;                 // blocks per g value
    int32_t ng;                // g values
    int32_t apair, bpair;
    int32_t conjA, conjB;
    int32_t expA, expB, expC;
    BitMap laneA, laneB, grpA, grpB;   // lane / group index of r -> A / B offset
    BitMap gA, gB, gC;                 // g -> A / B / C offset
    BitMap aA, aC, bB, bC;             // a -> A / C offset; b -> B / C offset
};
constexpr int kLSumOut = 16;            // results per lane (NA x NB)
constexpr int kLSumRowsPerLane = 512;
constexpr int kLSumWarps = kThreads / 32;
constexpr int kLSumAhead = 8;           // groups between a lane's L2 prefetch and its loads

// a values of one chunk (lsum_na) and of the whole result (lsum_na_all)
__host__ __device__ __forceinline__ int lsum_na(const LSumArgs& a, int NA) { return a.CA * (32 >> a.LR) * NA; }
__host__ __device__ __forceinline__ int lsum_na_all(const LSumArgs& a, int NA) { return a.nrc * lsum_na(a, NA); }

struct LSumSmem {
    int64_t *dA, *dB, *ao, *bo;
    double* red;                       // [warp][lane-block result][re, im]
};
__host__ __device__ __forceinline__ LSumSmem lsum_carve(unsigned char* base, int Na, int Nb) {
    LSumSmem t;
    t.dA = reinterpret_cast<int64_t*>(base);
    t.dB = t.dA + 48;
    t.bo = t.dB + 48;
    t.ao = t.bo + Nb;
    t.red = reinterpret_cast<double*>(t.ao + Na);
    return t;
}
// per warp: S NA NB results
inline size_t lsum_smem_bytes(int Na, int Nb, int per_warp) {
    return sizeof(int64_t) * (96 + Na + Nb) + sizeof(double) * 2 * per_warp * kLSumWarps;
}

__host__ __device__ __forceinline__ void lsum_fill(const LSumArgs& a, const LSumSmem& t, int Na, int Nb, int tid,
                                                   int nthr) {
    for (int j = tid; j < 46; j += nthr) {
        const int64_t bit = int64_t(1) << j, low = bit - 1;
        t.dA[j] = pdep(bit, a.grpA) - pdep(low, a.grpA);
        t.dB[j] = pdep(bit, a.grpB) - pdep(low, a.grpB);
    }
    for (int i = tid; i < Na; i += nthr) t.ao[i] = pdep(i, a.aA);
    for (int i = tid; i < Nb; i += nthr) t.bo[i] = pdep(i, a.bB);
}

template <int NA, int NB>
__host__ __device__ __forceinline__ void lsum_load(const LSumArgs& a, const float2* arow, const float2* brow,
                                                   const int64_t* ao, const int64_t* bo, float* ar, float* ai,
                                                   float* br, float* bi) {
    bool done = false;
    if constexpr (NA > 1) {
        if (a.apair) {
            done = true;
#pragma unroll
            for (int i = 0; i < NA; i += 2) {
                const float4 v = *reinterpret_cast<const float4*>(arow + ao[i]);
                ar[i] = v.x; ai[i] = v.y; ar[i + 1] = v.z; ai[i + 1] = v.w;
            }
        }
    }
    if (!done) {
#pragma unroll
        for (int i = 0; i < NA; i++) { const float2 v = arow[ao[i]]; ar[i] = v.x; ai[i] = v.y; }
    }
    done = false;
    if constexpr (NB > 1) {
        if (a.bpair) {
            done = true;
#pragma unroll
            for (int i = 0; i < NB; i += 2) {
                const float4 v = *reinterpret_cast<const float4*>(brow + bo[i]);
                br[i] = v.x; bi[i] = v.y; br[i + 1] = v.z; bi[i + 1] = v.w;
            }
        }
    }
    if (!done) {
#pragma unroll
        for (int i = 0; i < NB; i++) { const float2 v = brow[bo[i]]; br[i] = v.x; bi[i] = v.y; }
    }
}

template <int NA, int NB>
__host__ __device__ __forceinline__ void lsum_madd(const float* ar, const float* ai, const float* br, const float* bi,
                                                   float sa, float sb, unsigned long long (&acc)[NA][NB]) {
    unsigned long long y1[NB], y2[NB];
#pragma unroll
    for (int j = 0; j < NB; j++) {
        const float bij = sb * bi[j];
        y1[j] = f2pack(br[j], bij);
        y2[j] = f2pack(bij, br[j]);
    }
#pragma unroll
    for (int i = 0; i < NA; i++) {
        const float aii = sa * ai[i];
        const unsigned long long xx = f2pack(ar[i], ar[i]), xj = f2pack(-aii, aii);
#pragma unroll
        for (int j = 0; j < NB; j++) {
            fma2(acc[i][j], xx, y1[j]);
            fma2(acc[i][j], xj, y2[j]);
        }
    }
}

// L2 prefetch of one row's A and B values (no data returned, no fault on a valid address).
template <int NA, int NB>
__host__ __device__ __forceinline__ void lsum_prefetch(const LSumArgs& a, const float2* arow, const float2* brow,
                                                       const int64_t* ao, const int64_t* bo) {
#ifdef __CUDA_ARCH__
    const int sa = a.apair ? 2 : 1, sb = a.bpair ? 2 : 1;
#pragma unroll
    for (int i = 0; i < NA; i++)
        if (i % sa == 0) asm volatile("prefetch.global.L2 [%0];" ::"l"(arow + ao[i]));
#pragma unroll
    for (int i = 0; i < NB; i++)
        if (i % sb == 0) asm volatile("prefetch.global.L2 [%0];" ::"l"(brow + bo[i]));
#else
    (void)a; (void)arow; (void)brow; (void)ao; (void)bo;
#endif
}

__host__ __device__ __forceinline__ int lsum_ctz(unsigned long long v) {
#ifdef __CUDA_ARCH__
    return __ffsll((long long)v) - 1;
#else
    return __builtin_ctzll(v);
#endif
}

// Lane `lane` of warp slot w (of nwarps sharing the g value's rows), lane block (a0, b0): FP32
// sums into acc (re, im pairs), two groups of r per step.
template <int NA, int NB>
__host__ __device__ __forceinline__ void lsum_walk(const LSumArgs& a, const LSumSmem& t, int64_t abase, int64_t bbase,
                                                   int64_t w, int64_t nwarps, int lane, int a0, int b0,
                                                   unsigned long long (&acc)[NA][NB]) {
    const int rl = lane & ((1 << a.LR) - 1);
    const int64_t lA = pdep(rl, a.laneA), lB = pdep(rl, a.laneB);
    const int64_t g0 = a.ngroups * w / nwarps, g1 = a.ngroups * (w + 1) / nwarps;
    int64_t oA = pdep(g0, a.grpA), oB = pdep(g0, a.grpB);
    const float2* __restrict__ Ag = static_cast<const float2*>(a.A) + abase + lA;
    const float2* __restrict__ Bg = static_cast<const float2*>(a.B) + bbase + lB;
    const int64_t* ao = t.ao + a0;
    const int64_t* bo = t.bo + b0;
    const float sa = a.conjA ? -1.f : 1.f, sb = a.conjB ? -1.f : 1.f;
    // a second walker kLSumAhead groups ahead issues L2 prefetches of the rows to come
    int64_t gp = g0 + kLSumAhead;
    int64_t pA = gp < g1 ? pdep(gp, a.grpA) : 0, pB = gp < g1 ? pdep(gp, a.grpB) : 0;
    for (int64_t g = g0; g < g1; g += 2) {
        const bool two = g + 1 < g1;
        for (int u = 0; u < 2 && gp < g1; u++, gp++) {
            lsum_prefetch<NA, NB>(a, Ag + pA, Bg + pB, ao, bo);
            const int jp = lsum_ctz((unsigned long long)(gp + 1));
            pA += t.dA[jp];
            pB += t.dB[jp];
        }
        const int j1 = lsum_ctz((unsigned long long)(g + 1));
        const int64_t oA1 = oA + t.dA[j1], oB1 = oB + t.dB[j1];
        float ar[NA], ai[NA], br[NB], bi[NB], ar1[NA], ai1[NA], br1[NB], bi1[NB];
        lsum_load<NA, NB>(a, Ag + oA, Bg + oB, ao, bo, ar, ai, br, bi);
        if (two) lsum_load<NA, NB>(a, Ag + oA1, Bg + oB1, ao, bo, ar1, ai1, br1, bi1);
        lsum_madd<NA, NB>(ar, ai, br, bi, sa, sb, acc);
        if (two) {
            lsum_madd<NA, NB>(ar1, ai1, br1, bi1, sa, sb, acc);
            const int j2 = lsum_ctz((unsigned long long)(g + 2));
            oA = oA1 + t.dA[j2];
            oB = oB1 + t.dB[j2];
        }
    }
}

// Lane block of warp `warp`, lane `lane`: first a and b values (a0, b0).
__host__ __device__ __forceinline__ void lsum_lane_block(const LSumArgs& a, int NA, int NB, int warp, int lane, int* a0,
                                                         int* b0) {
    const int CW = a.CA * a.CB, c = warp % CW, S = 32 >> a.LR;
    *a0 = ((c / a.CB) * S + (lane >> a.LR)) * NA;
    *b0 = (c % a.CB) * NB;
}

// Launched with kThreads threads, grid (ng x G, nrc); dynamic shared memory lsum_smem_bytes.
template <int NA, int NB>
__global__ void __launch_bounds__(kThreads) contract_lsum_kernel(const LSumArgs a, double2* partial) {
    extern __shared__ __align__(16) unsigned char lsum_smem[];
    const int Na = lsum_na(a, NA), NaAll = lsum_na_all(a, NA), Nb = a.CB * NB;
    const LSumSmem t = lsum_carve(lsum_smem, NaAll, Nb);
    lsum_fill(a, t, NaAll, Nb, threadIdx.x, kThreads);
    __syncthreads();
    const int g = blockIdx.x / a.G, part = blockIdx.x % a.G, chunk = blockIdx.y;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int CW = a.CA * a.CB, sets = kLSumWarps / CW;      // warp sets dividing the rows
    int a0, b0;
    lsum_lane_block(a, NA, NB, warp, lane, &a0, &b0);
    a0 += chunk * Na;
    unsigned long long acc[NA][NB];
#pragma unroll
    for (int i = 0; i < NA; i++)
#pragma unroll
        for (int j = 0; j < NB; j++) acc[i][j] = 0ull;
    lsum_walk<NA, NB>(a, t, pdep(g, a.gA), pdep(g, a.gB), (int64_t)part * sets + warp / CW, (int64_t)a.G * sets, lane,
                      a0, b0, acc);
    // FP64: butterfly over the lanes of one sub-lane (the low LR lane bits) ...
    const int S = 32 >> a.LR, R = 1 << a.LR, sub = lane >> a.LR;
    const int pw = S * NA * NB;                                 // results of one warp
#pragma unroll
    for (int i = 0; i < NA; i++)
#pragma unroll
        for (int j = 0; j < NB; j++) {
            double re = (double)u2f((unsigned)(acc[i][j] & 0xffffffffull));
            double im = (double)u2f((unsigned)(acc[i][j] >> 32));
            for (int o = 1; o < R; o <<= 1) {
                re += __shfl_xor_sync(0xffffffffu, re, o);
                im += __shfl_xor_sync(0xffffffffu, im, o);
            }
            if ((lane & (R - 1)) == 0) {
                const int res = (sub * NA + i) * NB + j;
                t.red[2 * (warp * pw + res)] = re;
                t.red[2 * (warp * pw + res) + 1] = im;
            }
        }
    __syncthreads();
    // ... then the warp sets in order, one partial per result (a, b) of the chunk
    for (int o = threadIdx.x; o < Na * Nb; o += kThreads) {
        const int av = o / Nb, bv = o % Nb;
        const int ca = av / (S * NA), sub2 = (av % (S * NA)) / NA, i = av % NA;
        const int cb = bv / NB, j = bv % NB;
        const int c = ca * a.CB + cb, res = (sub2 * NA + i) * NB + j;
        double re = 0.0, im = 0.0;
        for (int st = 0; st < sets; st++) {
            const int w = st * CW + c;
            re += t.red[2 * (w * pw + res)];
            im += t.red[2 * (w * pw + res) + 1];
        }
        partial[((int64_t)g * a.G + part) * (NaAll * Nb) + (int64_t)chunk * Na * Nb + o] = make_double2(re, im);
    }
}

// One result (idx over g and the per = Na Nb results (a, b) of a g value): the parts in order,
// scaled, stored at its C offset; returns its magnitude.
__host__ __device__ __forceinline__ float lsum_reduce_one(const LSumArgs& a, int per, int Nb, const double2* partial,
                                                          int64_t idx, double scale) {
    const int g = (int)(idx / per), o = (int)(idx % per);
    double r = 0.0, i = 0.0;
    for (int p = 0; p < a.G; p++) {
        const double2 v = partial[((int64_t)g * a.G + p) * per + o];
        r += v.x;
        i += v.y;
    }
    r *= scale; i *= scale;
    float2* C = static_cast<float2*>(a.C);
    C[pdep(g, a.gC) + pdep(o / Nb, a.aC) + pdep(o % Nb, a.bC)] = make_float2((float)r, (float)i);
    return fmaxf(fabsf((float)r), fabsf((float)i));
}

template <bool SCALED>
__global__ void lsum_reduce_kernel(const LSumArgs a, int per, int Nb, const double2* partial, int* exps) {
    double scale = 1.0;
    if (SCALED) {
        const int mA = read_m(exps, a.expA), mB = read_m(exps, a.expB);
        scale = pow2d(-(mA + mB));
        if (blockIdx.x == 0 && threadIdx.x == 0)
            exps[2 * a.expC] = exps[2 * a.expA] + exps[2 * a.expB] + mA + mB;
    }
    const int64_t total = (int64_t)a.ng * per;
    int emax = kExpUnset;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const float mx = lsum_reduce_one(a, per, Nb, partial, idx, scale);
        if (SCALED && mx > 0.f) emax = max(emax, exp_of(mx));
    }
    if (SCALED) {
        for (int o = 16; o > 0; o >>= 1) emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, o));
        if ((threadIdx.x & 31) == 0 && emax != kExpUnset) atomicMax(&exps[2 * a.expC + 1], emax);
    }
}

// Batch of small independent contractions in one launch (the gate absorptions of a pass, whose
// own launches would cost more than their work).  Block b finds its step by binary search over
// the steps' first blocks, copies the step's arguments and its K offsets into shared memory and
// computes up to kBatchResults results, each summing its K <= kBatchMaxK products in order; the
// step's first block sets the result's base exponent and every block raises its maximum, as the
// single-step kernels do.  Launched with kThreads threads.
template <typename T, bool SCALED>
__global__ void __launch_bounds__(kThreads) contract_batch_kernel(const BatchStep* steps, int n, int* exps) {
    using R = typename Real<T>::type;
    __shared__ int sel;
    __shared__ __align__(16) StepArgs a;
    __shared__ int64_t tA[kBatchMaxK], tB[kBatchMaxK];
    if (threadIdx.x == 0) {
        int lo = 0, hi = n - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) / 2;
            if (steps[mid].first_block <= (int)blockIdx.x) lo = mid; else hi = mid - 1;
        }
        sel = lo;
    }
    __syncthreads();
    {
        const int* src = reinterpret_cast<const int*>(&steps[sel].a);
        int* dst = reinterpret_cast<int*>(&a);
        for (int i = threadIdx.x; i < (int)(sizeof(StepArgs) / sizeof(int)); i += kThreads) dst[i] = src[i];
    }
    __syncthreads();
    const int K = 1 << a.nk;
    for (int k = threadIdx.x; k < K; k += kThreads) { tA[k] = pdep(k, a.kA); tB[k] = pdep(k, a.kB); }
    __syncthreads();
    const int part = (int)blockIdx.x - steps[sel].first_block;
    R scale = R(1);
    if (SCALED) {
        const int mA = read_m(exps, a.expA), mB = read_m(exps, a.expB);
        scale = (R)pow2f(-(mA + mB));
        if (part == 0 && threadIdx.x == 0) exps[2 * a.expC] = exps[2 * a.expA] + exps[2 * a.expB] + mA + mB;
    }
    const T* __restrict__ A = static_cast<const T*>(a.A);
    const T* __restrict__ B = static_cast<const T*>(a.B);
    T* __restrict__ C = static_cast<T*>(a.C);
    const R ca = a.conjA ? R(-1) : R(1), cb = a.conjB ? R(-1) : R(1);
    const int64_t c0 = (int64_t)part * kBatchResults;
    const int64_t c1 = c0 + kBatchResults < a.nC ? c0 + kBatchResults : a.nC;
    int emax = kExpUnset;
    for (int64_t c = c0 + threadIdx.x; c < c1; c += kThreads) {
        const int64_t ao = pdep(c, a.cA), bo = pdep(c, a.cB);
        R re = R(0), im = R(0);
        for (int k = 0; k < K; k++) {
            const T x = A[ao + tA[k]];
            const T y = B[bo + tB[k]];
            const R xi = ca * x.y, yi = cb * y.y;
            re = fma(x.x, y.x, re);
            re = fma(-xi, yi, re);
            im = fma(x.x, yi, im);
            im = fma(xi, y.x, im);
        }
        if (SCALED) {
            re *= scale; im *= scale;
            const float mx = fmaxf(fabsf((float)re), fabsf((float)im));
            if (mx > 0.f) emax = max(emax, exp_of(mx));
        }
        T out; out.x = re; out.y = im;
        C[c] = out;
    }
    if (SCALED) {
        for (int o = 16; o > 0; o >>= 1) emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, o));
        if ((threadIdx.x & 31) == 0 && emax != kExpUnset) atomicMax(&exps[2 * a.expC + 1], emax);
    }
}

// Split-K form of a contraction with few results and a long sum (the adjoint steps that end in
// gate-sized leaf gradients sum over every other index of the network).  Pass 1: block
// (result tile, split) sums the split's range of the high K index (all 2^nkt low K values) for
// up to kSplitTile results, its threads grouped by result, and writes one partial per result;
// pass 2 adds the partials of each result in split order (deterministic), scales, stores and
// raises the exponent slot like the general kernel.
constexpr int kSplitTile = 256;         // results per block of pass 1

template <typename T, int CONJ>
__global__ void __launch_bounds__(kThreads) contract_splitk_kernel(const StepArgs a, int nsplit, T* partial) {
    using R = typename Real<T>::type;
    __shared__ int64_t tA[1 << kKTableBits], tB[1 << kKTableBits];
    __shared__ R red[2][kThreads];
    const int nkt = a.nk < kKTableBits ? a.nk : kKTableBits;
    const int KT = 1 << nkt;
    const int64_t KO = int64_t(1) << (a.nk - nkt);
    for (int k = threadIdx.x; k < KT; k += kThreads) { tA[k] = pdep(k, a.kA); tB[k] = pdep(k, a.kB); }
    __syncthreads();
    const int64_t ntile = (a.nC + kSplitTile - 1) / kSplitTile;
    const int64_t tile = blockIdx.x % ntile;
    const int split = (int)(blockIdx.x / ntile);
    const int64_t c0 = tile * kSplitTile;
    const int nres = (int)(a.nC - c0 < kSplitTile ? a.nC - c0 : kSplitTile);
    const int per = kThreads / nres;        // threads per result (>= 1)
    const int r = threadIdx.x % nres, sub = threadIdx.x / nres;
    const bool active = sub < per;
    const int64_t ko0 = KO * split / nsplit, ko1 = KO * (split + 1) / nsplit;
    R re = R(0), im = R(0);
    if (active) {
        const int64_t c = c0 + r;
        const int64_t a0 = pdep(c, a.cA), b0 = pdep(c, a.cB);
        for (int64_t ko = ko0; ko < ko1; ko++) {
            const int64_t ah = a0 + (ko ? pdep(ko << nkt, a.kA) : 0);
            const int64_t bh = b0 + (ko ? pdep(ko << nkt, a.kB) : 0);
            for (int k = sub; k < KT; k += per) {
                const T x = static_cast<const T*>(a.A)[ah + tA[k]];
                const T y = static_cast<const T*>(a.B)[bh + tB[k]];
                const R xi = (CONJ & 1) ? -x.y : x.y, yi = (CONJ & 2) ? -y.y : y.y;
                re = fma(x.x, y.x, re);
                re = fma(-xi, yi, re);
                im = fma(x.x, yi, im);
                im = fma(xi, y.x, im);
            }
        }
    }
    red[0][threadIdx.x] = re;
    red[1][threadIdx.x] = im;
    __syncthreads();
    if (threadIdx.x < nres) {               // fixed order over the result's threads
        R sr = R(0), si = R(0);
        for (int j = 0; j < per; j++) { sr += red[0][threadIdx.x + j * nres]; si += red[1][threadIdx.x + j * nres]; }
        T out; out.x = sr; out.y = si;
        partial[(int64_t)split * a.nC + c0 + threadIdx.x] = out;
    }
}

template <typename T, bool SCALED>
__global__ void splitk_reduce_kernel(const StepArgs a, int nsplit, const T* partial, int* exps) {
    using R = typename Real<T>::type;
    R scale = R(1);
    if (SCALED) {
        const int mA = read_m(exps, a.expA), mB = read_m(exps, a.expB);
        scale = (R)pow2f(-(mA + mB));
        if (blockIdx.x == 0 && threadIdx.x == 0)
            exps[2 * a.expC] = exps[2 * a.expA] + exps[2 * a.expB] + mA + mB;
    }
    int emax = kExpUnset;
    T* C = static_cast<T*>(a.C);
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < a.nC; c += (int64_t)gridDim.x * blockDim.x) {
        R re = R(0), im = R(0);
        for (int j = 0; j < nsplit; j++) {
            const T v = partial[(int64_t)j * a.nC + c];
            re += v.x;
            im += v.y;
        }
        if (SCALED) {
            re *= scale; im *= scale;
            const float mx = fmaxf(fabsf((float)re), fabsf((float)im));
            if (mx > 0.f) emax = max(emax, exp_of(mx));
        }
        T out; out.x = re; out.y = im;
        C[c] = out;
    }
    if (SCALED) {
        for (int o = 16; o > 0; o >>= 1) emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, o));
        if ((threadIdx.x & 31) == 0 && emax != kExpUnset) atomicMax(&exps[2 * a.expC + 1], emax);
    }
}

template <typename T>
__global__ void view_kernel(const ViewArgs a, int* exps) {
    const T* __restrict__ S = static_cast<const T*>(a.src);
    T* __restrict__ D = static_cast<T*>(a.dst);
    if (exps && blockIdx.x == 0 && threadIdx.x == 0) {
        exps[2 * a.exp_dst] = exps[2 * a.exp_src];
        exps[2 * a.exp_dst + 1] = exps[2 * a.exp_src + 1];
    }
    const PassParams p = *a.params;
    const int64_t lomask = (int64_t(1) << a.sigma_shift) - 1;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < a.n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t sigma = i >> a.sigma_shift;
        const int64_t s = p.slice_base + sigma;
        T v; v.x = 0; v.y = 0;
        if (sigma < p.slices_valid && s < p.num_slices) {
            int64_t off = pdep(i & lomask, a.map);
            for (int f = 0; f < a.nfix; f++) {
                const int64_t val = (s / a.var_stride[f]) % a.var_dim[f];
                off += val << a.fix_shift[f];
            }
            v = S[off];
        }
        D[i] = v;
    }
}

template <typename T>
__global__ void output_kernel(const OutputArgs a, int* exps) {
    T* __restrict__ D = static_cast<T*>(a.dst);
    if (exps && blockIdx.x == 0 && threadIdx.x == 0) { exps[2 * a.exp_dst] = 0; exps[2 * a.exp_dst + 1] = 1; }
    const PassParams p = *a.params;
    const double r = 0.70710678118654752440;
    for (int beta = blockIdx.x * blockDim.x + threadIdx.x; beta < a.nbeta; beta += gridDim.x * blockDim.x) {
        double v0 = 0.0, v1 = 0.0;
        if (beta < p.bits_valid) {
            const char ch = a.bitstrings[(int64_t)(p.bit_base + beta) * a.nqubits + a.qubit];
            if (ch == '0') { v0 = 1.0; }
            else if (ch == '1') { v1 = 1.0; }
            else if (ch == '+') { v0 = r; v1 = r; }
            else if (ch == '-') { v0 = r; v1 = -r; }
        }
        T x0, x1;
        x0.x = v0; x0.y = 0; x1.x = v1; x1.y = 0;
        D[2 * beta] = x0;
        D[2 * beta + 1] = x1;
    }
}

template <typename T>
__global__ void reduce_kernel(const ReduceArgs a, const int* exps) {
    const T* __restrict__ Rt = static_cast<const T*>(a.root);
    const PassParams p = *a.params;
    const int64_t total = a.out_size * a.nbeta;
    const double scale = exps ? pow2d(exps[2 * a.exp_root]) : 1.0;
    const int ns = a.nsigma > 1 ? min(a.nsigma, p.slices_valid) : 1;
    const double mult = a.nsigma > 1 ? 1.0 : (double)p.slices_valid;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total; idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = idx % a.out_size;
        const int beta = (int)(idx / a.out_size);
        if (beta >= p.bits_valid && !a.broadcast) continue;
        int64_t off = pdep(beta, a.beta_map);
        int64_t rem = e;
        for (int ax = 0; ax < a.naxes; ax++) {
            const int64_t d = rem % a.axis_dim[ax];
            rem /= a.axis_dim[ax];
            for (int j = 0; j < a.axis_nbits[ax]; j++)
                if ((d >> j) & 1) off += int64_t(1) << a.axis_bitpos[ax][j];
        }
        double re = 0.0, im = 0.0;
        for (int s = 0; s < ns; s++) {
            const T v = Rt[off + pdep(s, a.sigma_map)];
            re += (double)v.x;
            im += (double)v.y;
        }
        re *= scale * mult; im *= scale * mult;
        if (a.broadcast) {
            for (int b = 0; b < p.bits_valid; b++) {
                double* o = a.out + 2 * ((int64_t)(p.bit_base + b) * a.out_size + e);
                o[0] += re; o[1] += im;
            }
        } else {
            double* o = a.out + 2 * ((int64_t)(p.bit_base + beta) * a.out_size + e);
            o[0] += re; o[1] += im;
        }
    }
}

template <typename T>
__global__ void seed_kernel(const SeedArgs a, int* exps) {
    using R = typename Real<T>::type;
    T* __restrict__ D = static_cast<T*>(a.dst);
    const T* __restrict__ Rt = static_cast<const T*>(a.root);
    const PassParams p = *a.params;
    if (exps && blockIdx.x == 0 && threadIdx.x == 0) exps[2 * a.exp_dst] = 0;
    const double scale = (exps && !a.amp_bar) ? pow2d(exps[2 * a.exp_root]) : 1.0;
    const int64_t total = a.out_size * a.nbeta;
    int emax = kExpUnset;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total; idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = idx % a.out_size;
        const int beta = (int)(idx / a.out_size);
        if (beta >= p.bits_valid) continue;
        int64_t off = pdep(beta, a.beta_map);
        int64_t rem = e;
        for (int ax = 0; ax < a.naxes; ax++) {
            const int64_t d = rem % a.axis_dim[ax];
            rem /= a.axis_dim[ax];
            for (int j = 0; j < a.axis_nbits[ax]; j++)
                if ((d >> j) & 1) off += int64_t(1) << a.axis_bitpos[ax][j];
        }
        const int ns = a.nsigma > 1 ? min(a.nsigma, p.slices_valid) : 1;
        double vr, vi;
        if (a.amp_bar) {
            const double* s = a.amp_bar + 2 * ((int64_t)(p.bit_base + beta) * a.out_size + e);
            vr = s[0]; vi = s[1];
        } else {          // L = sum |a|^2: dL/d conj(a) = a, the root summed over the slice batch
            vr = 0.0; vi = 0.0;
            for (int s = 0; s < ns; s++) {
                const T v = Rt[off + pdep(s, a.sigma_map)];
                vr += (double)v.x;
                vi += (double)v.y;
            }
            vr *= scale; vi *= scale;
        }
        T v;
        v.x = (R)vr; v.y = (R)vi;
        for (int s = 0; s < ns; s++) D[off + pdep(s, a.sigma_map)] = v;
        if (exps) {
            const float mx = fmaxf(fabsf((float)vr), fabsf((float)vi));
            if (mx > 0.f) emax = max(emax, exp_of(mx));
        }
    }
    if (exps) {
        for (int o = 16; o > 0; o >>= 1) emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, o));
        if ((threadIdx.x & 31) == 0 && emax != kExpUnset) atomicMax(&exps[2 * a.exp_dst + 1], emax);
    }
}

template <typename T>
__global__ void view_adjoint_kernel(const ViewAdjArgs a, int* exps) {
    using R = typename Real<T>::type;
    const T* __restrict__ V = static_cast<const T*>(a.vbar);
    T* __restrict__ S = static_cast<T*>(a.sbar);
    const PassParams p = *a.params;
    if (exps && blockIdx.x == 0 && threadIdx.x == 0) exps[2 * a.exp_s] = exps[2 * a.exp_v];
    const int ns = min(a.nsigma, p.slices_valid);
    int emax = kExpUnset;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < a.ns; j += (int64_t)gridDim.x * blockDim.x) {
        const int64_t base = pdep(j, a.s2v);
        R re = R(0), im = R(0);
        for (int s = 0; s < ns; s++) {
            const int64_t sid = p.slice_base + s;
            if (sid >= p.num_slices) break;
            bool hit = true;
            for (int f = 0; f < a.nfix; f++) {
                const int64_t want = (j >> a.fix_shift[f]) & ((int64_t(1) << a.fix_bits[f]) - 1);
                if ((sid / a.var_stride[f]) % a.var_dim[f] != want) { hit = false; break; }
            }
            if (hit) {
                const T v = V[base + ((int64_t)s << a.sigma_shift)];
                re += v.x;
                im += v.y;
            }
        }
        T o;
        o.x = re; o.y = im;
        S[j] = o;
        if (exps) {
            const float mx = fmaxf(fabsf((float)re), fabsf((float)im));
            if (mx > 0.f) emax = max(emax, exp_of(mx));
        }
    }
    if (exps) {
        for (int o = 16; o > 0; o >>= 1) emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, o));
        if ((threadIdx.x & 31) == 0 && emax != kExpUnset) atomicMax(&exps[2 * a.exp_s + 1], emax);
    }
}

template <typename T>
__global__ void leaf_grad_kernel(const LeafGradArgs a, const int* exps) {
    const T* __restrict__ S = static_cast<const T*>(a.sbar);
    const double scale = exps ? pow2d(exps[2 * a.exp_s]) : 1.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < a.n; i += (int64_t)gridDim.x * blockDim.x) {
        int64_t rem = i, off = 0, st = 1;
        for (int d = 0; d < a.rank; d++) {
            off += (rem % a.dims[d]) * st;
            rem /= a.dims[d];
            st *= a.pdims[d];
        }
        const T v = S[off];
        a.grad[2 * i] += (double)v.x * scale;
        a.grad[2 * i + 1] += (double)v.y * scale;
    }
}

// Every leaf's gradient in one launch: block b adds leaf tab[b]'s adjoint into grad + 2 goff.
template <typename T>
__global__ void leaf_grad_batch_kernel(const LeafGradArgs* __restrict__ tab, double* grad, const int* exps) {
    const LeafGradArgs& a = tab[blockIdx.x];
    const T* __restrict__ S = static_cast<const T*>(a.sbar);
    const double scale = exps ? pow2d(exps[2 * a.exp_s]) : 1.0;
    double* gp = grad + 2 * a.goff;
    for (int64_t i = threadIdx.x; i < a.n; i += blockDim.x) {
        int64_t rem = i, off = 0, st = 1;
        for (int d = 0; d < a.rank; d++) {
            off += (rem % a.dims[d]) * st;
            rem /= a.dims[d];
            st *= a.pdims[d];
        }
        const T v = S[off];
        gp[2 * i] += (double)v.x * scale;
        gp[2 * i + 1] += (double)v.y * scale;
    }
}

__global__ void reset_exps_kernel(int* exps, int begin, int end) {
    for (int i = begin + blockIdx.x * blockDim.x + threadIdx.x; i < end; i += gridDim.x * blockDim.x) {
        exps[2 * i] = 0;
        exps[2 * i + 1] = kExpUnset;
    }
}

int grid_for(int64_t n, int threads, int cap) {
    int64_t g = (n + threads - 1) / threads;
    if (g < 1) g = 1;
    if (g > cap) g = cap;
    return (int)g;
}

// ---- host: choosing the row form ----------------------------------------------------------
void expand_map(const BitMap& m, std::vector<std::pair<int, int>>& out) {
    for (int i = 0; i < m.n; i++)
        for (int j = 0; j < m.r[i].len; j++) out.push_back({m.r[i].src + j, m.r[i].dst + j});
}

int dst_bits(const BitMap& c, const BitMap& k) {
    std::vector<std::pair<int, int>> v;
    expand_map(c, v);
    expand_map(k, v);
    uint64_t used = 0;
    for (auto& p : v) used |= uint64_t(1) << p.second;
    return __builtin_popcountll(used);
}

// Fill the row form of a step when its smaller operand has at most 2^max_ybits elements (the row
// kernel stages up to 2^11 in shared memory) and K <= kmax.
bool plan_rows(const StepArgs& a, int kmax, RowArgs* ra, int max_ybits = 11, bool wide_ok = false) {
    if (a.nk > 31 || (int64_t(1) << a.nk) > kmax) return false;
    const int abits = dst_bits(a.cA, a.kA), bbits = dst_bits(a.cB, a.kB);
    const bool x_is_a = abits >= bbits;
    const int ybits = x_is_a ? bbits : abits;
    if (ybits > max_ybits) return false;
    const BitMap& cX = x_is_a ? a.cA : a.cB;
    const BitMap& cY = x_is_a ? a.cB : a.cA;
    int ncb = 0;
    while ((int64_t(1) << ncb) < a.nC) ncb++;
    std::vector<int> inx(ncb, 0), iny(ncb, 0);
    std::vector<std::pair<int, int>> v;
    expand_map(cX, v);
    for (auto& p : v) if (p.first < ncb) inx[p.first] = 1;
    v.clear();
    expand_map(cY, v);
    for (auto& p : v) if (p.first < ncb) iny[p.first] = 1;
    std::vector<std::pair<int, int>> rows, cols;
    for (int p = 0; p < ncb; p++) {
        if (iny[p] && !inx[p]) cols.push_back({(int)cols.size(), p});
        else rows.push_back({(int)rows.size(), p});
    }
    if ((int64_t(1) << cols.size()) > kRowMaxN) return false;
    // the row kernel's thread writes its N results one after another: wide rows need many rows
    if (!wide_ok && cols.size() > 5 && rows.size() < 16) return false;
    memset(ra, 0, sizeof(*ra));
    if (!make_runs(rows, &ra->rowmap) || !make_runs(cols, &ra->nmap)) return false;
    ra->X = x_is_a ? a.A : a.B;
    ra->Y = x_is_a ? a.B : a.A;
    ra->C = a.C;
    ra->nrows = int64_t(1) << rows.size();
    ra->N = 1 << (int)cols.size();
    ra->K = 1 << a.nk;
    ra->ny = 1 << ybits;
    ra->conjX = x_is_a ? a.conjA : a.conjB;
    ra->conjY = x_is_a ? a.conjB : a.conjA;
    ra->expX = x_is_a ? a.expA : a.expB;
    ra->expY = x_is_a ? a.expB : a.expA;
    ra->expC = a.expC;
    ra->cX = cX;
    ra->cY = cY;
    ra->kX = x_is_a ? a.kA : a.kB;
    ra->kY = x_is_a ? a.kB : a.kA;
    return true;
}

// Fill the long sum (FP32): at least 2^12 summed terms, every summed bit in both operands; "a" is
// the side with more result bits.  Lane blocks of NA x NB results (NB <= 4, NA NB <= kLSumOut),
// up to 8 sub-lanes, up to 8 warps per row range; at most 2^20 values of the shared result bits.
// sm_count, blocks_per_sm: the grid fills the GPU once (blocks_per_sm 0: occupancy query).
bool plan_lsum(const StepArgs& s0, int sm_count, LSumArgs* la, int* NA, int* NB, int blocks_per_sm = 0) {
    if (s0.nk < 12 || s0.nk > 46) return false;
    auto one = [](const BitMap& m, int bit) {              // destination bit of one index bit, or -1
        const int64_t o = pdep(int64_t(1) << bit, m);
        return o ? __builtin_ctzll((unsigned long long)o) : -1;
    };
    int ncb = 0;
    while ((int64_t(1) << ncb) < s0.nC) ncb++;
    std::vector<int> ab, bb, gb;
    for (int p = 0; p < ncb; p++) {
        const bool ia = one(s0.cA, p) >= 0, ib = one(s0.cB, p) >= 0;
        if (ia && ib) gb.push_back(p);
        else if (ia) ab.push_back(p);
        else if (ib) bb.push_back(p);
        else return false;
    }
    for (int j = 0; j < s0.nk; j++)
        if (one(s0.kA, j) < 0 || one(s0.kB, j) < 0) return false;
    // the chunked side is the one with more result bits
    const bool swap = bb.size() > ab.size();
    const BitMap& cA = swap ? s0.cB : s0.cA;
    const BitMap& cB = swap ? s0.cA : s0.cB;
    const BitMap& kA = swap ? s0.kB : s0.kA;
    const BitMap& kB = swap ? s0.kA : s0.kB;
    if (swap) std::swap(ab, bb);
    const int na = (int)ab.size(), nb = (int)bb.size(), nk = s0.nk;
    if (gb.size() > 20) return false;
    const int nbv = 1 << nb, nav = 1 << na;
    const int NBv = std::min(nbv, 4), NAv = std::min(nav, kLSumOut / NBv);
    const int S = std::min(8, nav / NAv), CB = nbv / NBv;
    if (CB > kLSumWarps) return false;
    int CA = nav / (S * NAv), nrc = 1;                      // more lane blocks than warps: chunks
    while (CA * CB > kLSumWarps) { CA /= 2; nrc *= 2; }
    if (nrc > 16) return false;
    int LR = 5;
    while ((32 >> LR) < S) LR--;
    // summed bits by position in the larger operand
    int amax = 0, bmax = 0;
    for (int j = 0; j < nk; j++) { amax = std::max(amax, one(kA, j)); bmax = std::max(bmax, one(kB, j)); }
    for (int p : ab) amax = std::max(amax, one(cA, p));
    for (int p : bb) bmax = std::max(bmax, one(cB, p));
    for (int p : gb) { amax = std::max(amax, one(cA, p)); bmax = std::max(bmax, one(cB, p)); }
    const bool by_a = amax >= bmax;
    std::vector<int> ks(nk);
    for (int j = 0; j < nk; j++) ks[j] = j;
    std::sort(ks.begin(), ks.end(), [&](int x, int y) {
        return by_a ? one(kA, x) < one(kA, y) : one(kB, x) < one(kB, y);
    });
    std::vector<std::pair<int, int>> lA, lB, gA_, gB_, pgA, pgB, pgC, paA, paC, pbB, pbC;
    for (int i = 0; i < nk; i++) {
        auto& mA = i < LR ? lA : gA_;
        auto& mB = i < LR ? lB : gB_;
        const int src = i < LR ? i : i - LR;
        mA.push_back({src, one(kA, ks[i])});
        mB.push_back({src, one(kB, ks[i])});
    }
    for (int i = 0; i < (int)gb.size(); i++) {
        pgA.push_back({i, one(cA, gb[i])});
        pgB.push_back({i, one(cB, gb[i])});
        pgC.push_back({i, gb[i]});
    }
    for (int j = 0; j < na; j++) { paA.push_back({j, one(cA, ab[j])}); paC.push_back({j, ab[j]}); }
    for (int j = 0; j < nb; j++) { pbB.push_back({j, one(cB, bb[j])}); pbC.push_back({j, bb[j]}); }
    memset(la, 0, sizeof(*la));
    if (!make_runs(lA, &la->laneA) || !make_runs(lB, &la->laneB) || !make_runs(gA_, &la->grpA) ||
        !make_runs(gB_, &la->grpB) || !make_runs(pgA, &la->gA) || !make_runs(pgB, &la->gB) ||
        !make_runs(pgC, &la->gC) || !make_runs(paA, &la->aA) || !make_runs(paC, &la->aC) ||
        !make_runs(pbB, &la->bB) || !make_runs(pbC, &la->bC))
        return false;
    la->A = swap ? s0.B : s0.A;
    la->B = swap ? s0.A : s0.B;
    la->C = s0.C;
    la->conjA = swap ? s0.conjB : s0.conjA;
    la->conjB = swap ? s0.conjA : s0.conjB;
    la->expA = swap ? s0.expB : s0.expA;
    la->expB = swap ? s0.expA : s0.expB;
    la->expC = s0.expC;
    *NB = NBv;
    *NA = NAv;
    la->LR = LR;
    la->CA = CA;
    la->CB = CB;
    la->nrc = nrc;
    la->ng = 1 << (int)gb.size();
    la->ngroups = int64_t(1) << (nk - LR);
    const int sets = kLSumWarps / (CA * CB);
    if (blocks_per_sm <= 0) blocks_per_sm = lsum_blocks_per_sm(NAv, NBv, lsum_smem_bytes(nav, nbv, S * NAv * NBv));
    const int64_t slots = (int64_t)la->ng * nrc;
    int64_t G = ((int64_t)sm_count * std::max(blocks_per_sm, 1) + slots - 1) / slots;
    // at most kLSumRowsPerLane groups per warp set; at least one
    G = std::max<int64_t>(G, (la->ngroups + (int64_t)sets * kLSumRowsPerLane - 1) / ((int64_t)sets * kLSumRowsPerLane));
    G = std::max<int64_t>(1, std::min<int64_t>(G, la->ngroups / sets));
    if ((int64_t)la->ng * G > (int64_t(1) << 30)) return false;
    la->G = (int)G;
    la->apair = *NA > 1 && pdep(1, la->aA) == 1 && (reinterpret_cast<uintptr_t>(la->A) & 15) == 0;
    la->bpair = *NB > 1 && pdep(1, la->bB) == 1 && (reinterpret_cast<uintptr_t>(la->B) & 15) == 0;
    return true;
}

// The compact row form of a step, when it has one (FP32; Y up to kRows2MaxY elements).
bool use_rows2(const StepArgs& a, bool fp64, RowArgs* ra, Rows2Args* r2) {
    return !fp64 && plan_rows(a, 32, ra, kRows2MaxYBits, true) && plan_rows2(*ra, r2);
}

size_t lsum_partial_bytes(const LSumArgs& la, int NA, int NB) {
    return (size_t)la.ng * la.G * lsum_na_all(la, NA) * (la.CB * NB) * sizeof(double2);
}

// Splits of the split-K form: used when the results are few (<= 2^14) and each sums at least
// 2^8 terms (with fewer results than SMs the general form would leave most of the GPU idle);
// enough splits of the high K index to give about 8 blocks per SM, at least 2^12 terms per split
// (2^6 below 2^14 summed terms), and at most 2^22 partials in all.
int splitk_count(const StepArgs& a, int sm_count) {
    if (a.nC > (int64_t(1) << 14) || a.nk < 8) return 0;
    const int nkt = a.nk < kKTableBits ? a.nk : kKTableBits;
    const int64_t KO = int64_t(1) << (a.nk - nkt);
    const int64_t ntile = (a.nC + kSplitTile - 1) / kSplitTile;
    int64_t want = std::max<int64_t>(1, (int64_t)sm_count * 8 / ntile);
    want = std::min<int64_t>(want, std::max<int64_t>(1, (int64_t(1) << a.nk) >> (a.nk < 14 ? 6 : 12)));
    want = std::min<int64_t>(want, KO);
    want = std::min<int64_t>(want, std::max<int64_t>(1, (int64_t(1) << 22) / a.nC));
    return (int)want;
}

template <int CONJ>
void launch_general(const StepArgs& a, bool fp64, int* exps, cudaStream_t s, int grid) {
    if (fp64) contract_kernel<double2, false, CONJ><<<grid, kThreads, 0, s>>>(a, exps);
    else if (exps) contract_kernel<float2, true, CONJ><<<grid, kThreads, 0, s>>>(a, exps);
    else contract_kernel<float2, false, CONJ><<<grid, kThreads, 0, s>>>(a, exps);
}

template <typename T, int KMAX>
cudaError_t launch_rows(const RowArgs& ra, int* exps, cudaStream_t s, int sm_count) {
    const size_t smem = (size_t)ra.ny * sizeof(T) + (size_t)KMAX * 12 + (size_t)ra.N * 12;
    const int64_t want = (ra.nrows + kThreads - 1) / kThreads;
    const int64_t cap = (int64_t)sm_count * 8;
    const int grid = (int)std::max<int64_t>(1, std::min(want, cap));
    if (sizeof(T) == 16) contract_rows_kernel<T, false, KMAX><<<grid, kThreads, smem, s>>>(ra, exps);
    else if (exps) contract_rows_kernel<T, true, KMAX><<<grid, kThreads, smem, s>>>(ra, exps);
    else contract_rows_kernel<T, false, KMAX><<<grid, kThreads, smem, s>>>(ra, exps);
    return cudaGetLastError();
}

}  // namespace

size_t contract_scratch_bytes(const StepArgs& a, bool fp64, int sm_count) {
    RowArgs ra;
    Rows2Args r2;
    if (use_rows2(a, fp64, &ra, &r2) || plan_rows(a, fp64 ? 16 : 32, &ra)) return 0;
    BGemmArgs bg;
    if (!fp64 && plan_bgemm(a, sm_count, &bg)) return bgemm_partial_bytes(bg);
    LSumArgs la;
    int NA = 0, NB = 0;
    if (!fp64 && plan_lsum(a, sm_count, &la, &NA, &NB)) return lsum_partial_bytes(la, NA, NB);
    const int ns = splitk_count(a, sm_count);
    return ns > 0 ? (size_t)ns * (size_t)a.nC * (fp64 ? 16 : 8) : 0;
}

// The CUDA cores serve two kinds of long sums better than a tensor-core GEMM: the batched small
// GEMM of a final join (both operands large, so the tensor cores' packed planes would be several
// times the operand), and the long sum of a step with few results (a gate's gradient: tens of
// results, each a sum over the whole network).  Other steps with many results and a long sum are
// independent GEMMs that the tensor cores serve at a far higher rate than the long sum, so they
// are left to the tensor-core planner (it falls back to the CUDA cores when it cannot serve them).
constexpr int64_t kLSumPreferMaxResults = int64_t(1) << 12;

bool contract_prefers_cuda_cores(const StepArgs& a, bool fp64, int sm_count) {
    if (fp64) return false;
    BGemmArgs bg;
    if (plan_bgemm(a, sm_count, &bg)) return true;
    LSumArgs la;
    int NA = 0, NB = 0;
    return a.nC <= kLSumPreferMaxResults && plan_lsum(a, sm_count, &la, &NA, &NB) && la.nrc <= 2;
}

template <int NA, int NB>
cudaError_t launch_lsum_ab(const LSumArgs& la, void* scratch, int* exps, cudaStream_t s) {
    double2* partial = static_cast<double2*>(scratch);
    const int Na = lsum_na_all(la, NA), Nb = la.CB * NB, S = 32 >> la.LR;
    const size_t smem = lsum_smem_bytes(Na, Nb, S * NA * NB);
    const dim3 grid((unsigned)((int64_t)la.ng * la.G), (unsigned)la.nrc);
    contract_lsum_kernel<NA, NB><<<grid, kThreads, smem, s>>>(la, partial);
    const int per = Na * Nb;
    const int g = grid_for((int64_t)la.ng * per, 256, 1024);
    if (exps) lsum_reduce_kernel<true><<<g, 256, 0, s>>>(la, per, Nb, partial, exps);
    else lsum_reduce_kernel<false><<<g, 256, 0, s>>>(la, per, Nb, partial, exps);
    return cudaGetLastError();
}

template <int NA, int NB>
int lsum_occupancy(size_t smem) {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, contract_lsum_kernel<NA, NB>, kThreads, smem) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

int lsum_blocks_per_sm(int NA, int NB, size_t smem) {
    static int cache[5][6][2] = {};                 // [log2 NB][log2 NA][large smem]
    int lb = 0, la = 0;
    while ((1 << lb) < NB) lb++;
    while ((1 << la) < NA) la++;
    if (lb > 4 || la > 5) return 2;
    int& c = cache[lb][la][smem > 16384];
    if (c) return c;
    int n = 0;
#define QXG_LSUM_OCC(A_, B_) if (NA == A_ && NB == B_) n = lsum_occupancy<A_, B_>(smem);
    QXG_LSUM_OCC(1, 1) QXG_LSUM_OCC(2, 1) QXG_LSUM_OCC(4, 1) QXG_LSUM_OCC(8, 1) QXG_LSUM_OCC(16, 1)
    QXG_LSUM_OCC(1, 2) QXG_LSUM_OCC(2, 2) QXG_LSUM_OCC(4, 2) QXG_LSUM_OCC(8, 2)
    QXG_LSUM_OCC(1, 4) QXG_LSUM_OCC(2, 4) QXG_LSUM_OCC(4, 4)
#undef QXG_LSUM_OCC
    c = n > 0 ? n : 2;
    return c;
}

template <int NB>
cudaError_t launch_lsum_b(const LSumArgs& la, int NA, void* scratch, int* exps, cudaStream_t s) {
    switch (NA) {
        case 1: return launch_lsum_ab<1, NB>(la, scratch, exps, s);
        case 2: if constexpr (2 * NB <= kLSumOut) return launch_lsum_ab<2, NB>(la, scratch, exps, s); break;
        case 4: if constexpr (4 * NB <= kLSumOut) return launch_lsum_ab<4, NB>(la, scratch, exps, s); break;
        case 8: if constexpr (8 * NB <= kLSumOut) return launch_lsum_ab<8, NB>(la, scratch, exps, s); break;
        case 16: if constexpr (16 * NB <= kLSumOut) return launch_lsum_ab<16, NB>(la, scratch, exps, s); break;
        default: break;
    }
    return cudaErrorInvalidValue;
}

cudaError_t launch_lsum(const LSumArgs& la, int NA, int NB, void* scratch, int* exps, cudaStream_t s) {
    switch (NB) {
        case 1: return launch_lsum_b<1>(la, NA, scratch, exps, s);
        case 2: return launch_lsum_b<2>(la, NA, scratch, exps, s);
        case 4: return launch_lsum_b<4>(la, NA, scratch, exps, s);
        default: return cudaErrorInvalidValue;
    }
}

template <typename T, int CONJ>
void launch_splitk_t(const StepArgs& a, int ns, T* partial, int* exps, cudaStream_t s) {
    const int64_t ntile = (a.nC + kSplitTile - 1) / kSplitTile;
    contract_splitk_kernel<T, CONJ><<<(unsigned)(ntile * ns), kThreads, 0, s>>>(a, ns, partial);
}

template <typename T>
cudaError_t launch_splitk(const StepArgs& a, int ns, void* scratch, int* exps, cudaStream_t s) {
    T* partial = static_cast<T*>(scratch);
    switch ((a.conjA ? 1 : 0) | (a.conjB ? 2 : 0)) {
        case 0: launch_splitk_t<T, 0>(a, ns, partial, exps, s); break;
        case 1: launch_splitk_t<T, 1>(a, ns, partial, exps, s); break;
        case 2: launch_splitk_t<T, 2>(a, ns, partial, exps, s); break;
        default: launch_splitk_t<T, 3>(a, ns, partial, exps, s); break;
    }
    const int g = grid_for(a.nC, 256, 1024);
    if (exps && sizeof(T) == 8) splitk_reduce_kernel<T, true><<<g, 256, 0, s>>>(a, ns, partial, exps);
    else splitk_reduce_kernel<T, false><<<g, 256, 0, s>>>(a, ns, partial, exps);
    return cudaGetLastError();
}

bool contract_x_is_b(const StepArgs& a, bool fp64) {
    RowArgs ra;
    Rows2Args r2;
    if (!use_rows2(a, fp64, &ra, &r2) && !plan_rows(a, fp64 ? 16 : 32, &ra)) return false;
    return dst_bits(a.cA, a.kA) < dst_bits(a.cB, a.kB);      // plan_rows' choice of X
}

const char* contract_form(const StepArgs& a, bool fp64, int sm_count) {
    RowArgs ra;
    Rows2Args r2;
    if (use_rows2(a, fp64, &ra, &r2)) return "cuda-core compact row-form";
    if (plan_rows(a, fp64 ? 16 : 32, &ra)) return "cuda-core row-form";
    BGemmArgs bg;
    if (!fp64 && plan_bgemm(a, sm_count, &bg)) return "cuda-core batched-gemm";
    LSumArgs la;
    int NA = 0, NB = 0;
    if (!fp64 && plan_lsum(a, sm_count, &la, &NA, &NB)) return "cuda-core long-sum";
    return splitk_count(a, sm_count) > 0 ? "cuda-core split-K" : "cuda-core general";
}

cudaError_t launch_contract(const StepArgs& a, bool fp64, int* exps, cudaStream_t s, int sm_count, void* scratch,
                            size_t scratch_bytes, int* launches) {
    if (launches) *launches = 1;
    RowArgs ra;
    Rows2Args r2;
    if (use_rows2(a, fp64, &ra, &r2)) return launch_rows2(r2, ra.K, r2.ncol, exps, s, sm_count);
    if (!plan_rows(a, fp64 ? 16 : 32, &ra)) {
        BGemmArgs bg;
        if (!fp64 && plan_bgemm(a, sm_count, &bg) &&
            (bg.nsplit == 1 || (scratch && scratch_bytes >= bgemm_partial_bytes(bg))))
            return launch_bgemm(bg, scratch, exps, s, launches);
        LSumArgs la;
        int NA = 0, NB = 0;
        if (!fp64 && plan_lsum(a, sm_count, &la, &NA, &NB) && scratch && scratch_bytes >= lsum_partial_bytes(la, NA, NB)) {
            if (launches) *launches = 2;
            return launch_lsum(la, NA, NB, scratch, exps, s);
        }
        const int ns = splitk_count(a, sm_count);
        if (ns > 0 && scratch && scratch_bytes >= (size_t)ns * (size_t)a.nC * (fp64 ? 16 : 8)) {
            if (launches) *launches = 2;
            return fp64 ? launch_splitk<double2>(a, ns, scratch, exps, s) : launch_splitk<float2>(a, ns, scratch, exps, s);
        }
    }
    if (plan_rows(a, fp64 ? 16 : 32, &ra)) {
        if (fp64) return ra.K <= 4 ? launch_rows<double2, 4>(ra, exps, s, sm_count)
                                   : launch_rows<double2, 16>(ra, exps, s, sm_count);
        if (ra.K <= 4) return launch_rows<float2, 4>(ra, exps, s, sm_count);
        if (ra.K <= 16) return launch_rows<float2, 16>(ra, exps, s, sm_count);
        return launch_rows<float2, 32>(ra, exps, s, sm_count);
    }
    int ncb = 0;
    while ((int64_t(1) << ncb) < a.nC) ncb++;
    const int tb = ncb < kTileBits ? ncb : kTileBits;
    const int64_t ntiles = a.nC >> tb;
    const int64_t cap = (int64_t)sm_count * 8;
    const int grid = (int)(ntiles < cap ? ntiles : cap);
    const int conj = (a.conjA ? 1 : 0) | (a.conjB ? 2 : 0);
    switch (conj) {
        case 0: launch_general<0>(a, fp64, exps, s, grid); break;
        case 1: launch_general<1>(a, fp64, exps, s, grid); break;
        case 2: launch_general<2>(a, fp64, exps, s, grid); break;
        default: launch_general<3>(a, fp64, exps, s, grid); break;
    }
    return cudaGetLastError();
}

cudaError_t launch_batch(const BatchStep* d_steps, int n, int nblocks, bool fp64, int* exps, cudaStream_t s) {
    if (n <= 0 || nblocks <= 0) return cudaSuccess;
    if (fp64) contract_batch_kernel<double2, false><<<nblocks, kThreads, 0, s>>>(d_steps, n, exps);
    else if (exps) contract_batch_kernel<float2, true><<<nblocks, kThreads, 0, s>>>(d_steps, n, exps);
    else contract_batch_kernel<float2, false><<<nblocks, kThreads, 0, s>>>(d_steps, n, exps);
    return cudaGetLastError();
}

cudaError_t launch_view(const ViewArgs& a, bool fp64, int* exps, cudaStream_t s) {
    const int g = grid_for(a.n, 256, 4096);
    if (fp64) view_kernel<double2><<<g, 256, 0, s>>>(a, exps);
    else view_kernel<float2><<<g, 256, 0, s>>>(a, exps);
    return cudaGetLastError();
}

cudaError_t launch_output(const OutputArgs& a, bool fp64, int* exps, cudaStream_t s) {
    const int g = grid_for(a.nbeta, 256, 1024);
    if (fp64) output_kernel<double2><<<g, 256, 0, s>>>(a, exps);
    else output_kernel<float2><<<g, 256, 0, s>>>(a, exps);
    return cudaGetLastError();
}

cudaError_t launch_reduce(const ReduceArgs& a, bool fp64, const int* exps, cudaStream_t s) {
    const int g = grid_for(a.out_size * a.nbeta, 256, 4096);
    if (fp64) reduce_kernel<double2><<<g, 256, 0, s>>>(a, exps);
    else reduce_kernel<float2><<<g, 256, 0, s>>>(a, exps);
    return cudaGetLastError();
}

cudaError_t launch_seed(const SeedArgs& a, bool fp64, int* exps, cudaStream_t s) {
    const int g = grid_for(a.out_size * a.nbeta, 256, 4096);
    if (fp64) seed_kernel<double2><<<g, 256, 0, s>>>(a, exps);
    else seed_kernel<float2><<<g, 256, 0, s>>>(a, exps);
    return cudaGetLastError();
}

cudaError_t launch_view_adjoint(const ViewAdjArgs& a, bool fp64, int* exps, cudaStream_t s) {
    const int g = grid_for(a.ns, 256, 1024);
    if (fp64) view_adjoint_kernel<double2><<<g, 256, 0, s>>>(a, exps);
    else view_adjoint_kernel<float2><<<g, 256, 0, s>>>(a, exps);
    return cudaGetLastError();
}

cudaError_t launch_leaf_grad(const LeafGradArgs& a, bool fp64, const int* exps, cudaStream_t s) {
    const int g = grid_for(a.n, 256, 1024);
    if (fp64) leaf_grad_kernel<double2><<<g, 256, 0, s>>>(a, exps);
    else leaf_grad_kernel<float2><<<g, 256, 0, s>>>(a, exps);
    return cudaGetLastError();
}

cudaError_t launch_leaf_grads(const LeafGradArgs* d_tab, int n, double* grad, bool fp64, const int* exps,
                              cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    if (fp64) leaf_grad_batch_kernel<double2><<<n, 64, 0, s>>>(d_tab, grad, exps);
    else leaf_grad_batch_kernel<float2><<<n, 64, 0, s>>>(d_tab, grad, exps);
    return cudaGetLastError();
}

cudaError_t launch_reset_exps(int* exps, int begin, int end, cudaStream_t s) {
    if (end <= begin) return cudaSuccess;
    reset_exps_kernel<<<grid_for(end - begin, 256, 64), 256, 0, s>>>(exps, begin, end);
    return cudaGetLastError();
}

}  // namespace qxg
