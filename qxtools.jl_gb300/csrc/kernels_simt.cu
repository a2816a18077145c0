// CUDA-core kernels of the executor: the general pairwise contraction (one `ncon` command,
// docs/src/users_guide.md:124-146), view materialisation for a batch of slices
// (users_guide.md:104-122), output vectors for a batch of bitstrings (users_guide.md:149-158)
// and the FP64 sum over slices (users_guide.md:11-17).
//
// The contraction kernel is the plain executor's hot loop (ComplexF64 on the FP64 pipe) and
// the small-K path of the Complex64 executors (FP32 FMA).  A block owns tiles of 2^TB
// consecutive result elements; because a bit permutation is additive over disjoint bits,
// offset(tile | lo) = offset(tile) + offset(lo), so the low-bit offsets of the result and all
// K offsets (up to 2^kKTableBits) are tabulated once per block in shared memory and each
// element costs two table reads instead of a full bit deposit.
#include <algorithm>
#include <cstring>
#include <vector>

#include "qxgpu_internal.h"

namespace qxg {

namespace {

template <typename T> struct Real;
template <> struct Real<double2> { using type = double; };
template <> struct Real<float2> { using type = float; };

constexpr int kThreads = 256;
constexpr int kTileBits = 10;          // 1024 result elements per tile, 4 per thread

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
__device__ __forceinline__ int exp_of(float x) {
    return (int)((__float_as_uint(x) >> 23) & 0xffu) - 126;
}

__device__ __forceinline__ int read_m(const int* exps, int slot) {
    int m = exps[2 * slot + 1];
    return m < -400 ? 0 : m;            // all-zero tensor: no scaling
}

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
constexpr int kRowMaxY = 2048;          // elements of Y staged in shared memory
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

// Consecutive (src, dst) pairs with both sides increasing by one collapse into one run.
bool make_runs(const std::vector<std::pair<int, int>>& pairs, BitMap* m) {
    m->n = 0;
    for (size_t i = 0; i < pairs.size();) {
        size_t j = i + 1;
        while (j < pairs.size() && pairs[j].first == pairs[j - 1].first + 1 && pairs[j].second == pairs[j - 1].second + 1)
            j++;
        if (m->n >= kMaxRuns) return false;
        m->r[m->n] = Run{(uint8_t)pairs[i].first, (uint8_t)(j - i), (uint8_t)pairs[i].second, 0};
        m->n++;
        i = j;
    }
    return true;
}

// Fill the row form of a step when its smaller operand fits in shared memory and K <= kmax.
bool plan_rows(const StepArgs& a, int kmax, RowArgs* ra) {
    if (a.nk > 31 || (int64_t(1) << a.nk) > kmax) return false;
    const int abits = dst_bits(a.cA, a.kA), bbits = dst_bits(a.cB, a.kB);
    const bool x_is_a = abits >= bbits;
    const int ybits = x_is_a ? bbits : abits;
    if (ybits > 11 || (int64_t(1) << ybits) > kRowMaxY) return false;
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
    // a thread writes its N results one after another: wide rows need many of them
    if (cols.size() > 5 && rows.size() < 16) return false;
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

// Splits of the split-K form: used when the results are few (<= 2^14) and each sums at least
// 2^14 terms; enough splits of the high K index to give about 8 blocks per SM, at least 2^12
// terms per split, and at most 2^22 partials in all.
int splitk_count(const StepArgs& a, int sm_count) {
    if (a.nC > (int64_t(1) << 14) || a.nk < 14) return 0;
    const int nkt = a.nk < kKTableBits ? a.nk : kKTableBits;
    const int64_t KO = int64_t(1) << (a.nk - nkt);
    const int64_t ntile = (a.nC + kSplitTile - 1) / kSplitTile;
    int64_t want = std::max<int64_t>(1, (int64_t)sm_count * 8 / ntile);
    want = std::min<int64_t>(want, std::max<int64_t>(1, (int64_t(1) << a.nk) >> 12));
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
    if (plan_rows(a, fp64 ? 16 : 32, &ra)) return 0;
    const int ns = splitk_count(a, sm_count);
    return ns > 0 ? (size_t)ns * (size_t)a.nC * (fp64 ? 16 : 8) : 0;
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

bool contract_uses_rows(const StepArgs& a, bool fp64) {
    RowArgs ra;
    return plan_rows(a, fp64 ? 16 : 32, &ra);
}

cudaError_t launch_contract(const StepArgs& a, bool fp64, int* exps, cudaStream_t s, int sm_count, void* scratch,
                            size_t scratch_bytes, int* launches) {
    if (launches) *launches = 1;
    RowArgs ra;
    if (!plan_rows(a, fp64 ? 16 : 32, &ra)) {
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

cudaError_t launch_reset_exps(int* exps, int begin, int end, cudaStream_t s) {
    if (end <= begin) return cudaSuccess;
    reset_exps_kernel<<<grid_for(end - begin, 256, 64), 256, 0, s>>>(exps, begin, end);
    return cudaGetLastError();
}

}  // namespace qxg
