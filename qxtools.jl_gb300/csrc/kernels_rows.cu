// Compact row form of the CUDA-core contraction (FP32 gate-like steps; see simt_common.h for the
// design): kernel, planner and launcher.  Kept in its own translation unit so that its template
// instances compile in parallel with the other kernels.
#include <algorithm>
#include <cstring>
#include <vector>

#include "qxgpu_internal.h"
#include "simt_common.h"

namespace qxg {

namespace {

// Shared tables of the compact row form: Y quadruples [batch][chunk][k][n] (batches padded by one),
// per group-bit deltas of the X / C offsets and batch index, X offsets of k, C offsets of n.
struct Rows2Smem {
    float4* Ys;
    int64_t *dX, *dC, *dB, *kx, *cn;
};
template <int K, int N>
__host__ __device__ __forceinline__ Rows2Smem rows2_carve(const Rows2Args& a, unsigned char* base) {
    Rows2Smem t;
    t.Ys = reinterpret_cast<float4*>(base);
    t.dX = reinterpret_cast<int64_t*>(t.Ys + (size_t)a.nbatch * (K * N * a.nchunk + 1));
    t.dC = t.dX + 48;
    t.dB = t.dC + 48;
    t.kx = t.dB + 48;
    t.cn = t.kx + K;
    return t;
}

// Table entries written by thread tid of nthr.
template <int K, int N>
__host__ __device__ __forceinline__ void rows2_fill(const Rows2Args& a, const Rows2Smem& t, int tid, int nthr) {
    const int KNF = K * N * a.nchunk, BS = KNF + 1;
    const float* __restrict__ Yg = static_cast<const float*>(a.Y);
    for (int i = tid; i < a.nbatch * KNF; i += nthr) {
        const int b = i / KNF, r = i % KNF;                 // r = (chunk K + k) N + n
        const int c = r / (K * N), k = (r % (K * N)) / N, n = r % N;
        const int64_t yo = pdep(b, a.bY) + pdep(k, a.kY) + pdep(c * N + n, a.nY);
        const float yr = Yg[2 * yo], yi = a.conjY ? -Yg[2 * yo + 1] : Yg[2 * yo + 1];
        t.Ys[b * BS + r] = make_float4(yr, yi, yi, yr);
    }
    for (int j = tid; j < 46; j += nthr) {
        const int64_t bit = int64_t(1) << j, low = bit - 1;
        t.dX[j] = pdep(bit, a.grpX) - pdep(low, a.grpX);
        t.dC[j] = pdep(bit, a.grpC) - pdep(low, a.grpC);
        t.dB[j] = pdep(bit, a.grpB) - pdep(low, a.grpB);
    }
    for (int k = tid; k < K; k += nthr) t.kx[k] = pdep(k, a.kX);
    for (int n = tid; n < N * a.nchunk; n += nthr) t.cn[n] = pdep(n, a.nC);
}

// The rows of lane `lane` of warp w (of nwarps): its row groups one after another.  MULTI: more
// than one chunk of N columns (a runtime loop; a single chunk compiles without it).
template <int K, int N, bool SCALED, bool MULTI>
__host__ __device__ __forceinline__ void rows2_walk(const Rows2Args& a, const Rows2Smem& t, int64_t w, int64_t nwarps,
                                                    int lane, float scale, int& emax) {
    if (lane >= a.lanes) return;
    const int BS = K * N * a.nchunk + 1;
    const int64_t lx = pdep(lane, a.laneX), lc = pdep(lane, a.laneC), lb = pdep(lane, a.laneB);
    const int64_t g0 = a.ngroups * w / nwarps, g1 = a.ngroups * (w + 1) / nwarps;
    int64_t ox = pdep(g0, a.grpX), oc = pdep(g0, a.grpC), ob = pdep(g0, a.grpB);
    const float2* __restrict__ X = static_cast<const float2*>(a.X);
    float2* __restrict__ C = static_cast<float2*>(a.C);
    const float sx = a.conjX ? -1.f : 1.f;
    for (int64_t g = g0; g < g1; g++) {
        const float2* xrow = X + (lx + ox);
        const float4* yb = t.Ys + (lb + ob) * BS;
        float xr[K], xi[K];
        bool paired = false;
        if constexpr (K > 1) {
            if (a.xpair) {                                  // k, k+1 adjacent in X
                paired = true;
#pragma unroll
                for (int k = 0; k < K; k += 2) {
                    const float4 v = *reinterpret_cast<const float4*>(xrow + t.kx[k]);
                    xr[k] = v.x; xi[k] = v.y; xr[k + 1] = v.z; xi[k + 1] = v.w;
                }
            }
        }
        if (!paired) {
#pragma unroll
            for (int k = 0; k < K; k++) {
                const float2 v = xrow[t.kx[k]];
                xr[k] = v.x; xi[k] = v.y;
            }
        }
        float2* crow = C + (lc + oc);
        const int nch = MULTI ? a.nchunk : 1;
        for (int ch = 0; ch < nch; ch++) {
        const float4* ybc = yb + ch * (K * N);
        const int64_t* cnc = t.cn + ch * N;
        unsigned long long acc[N];
#pragma unroll
        for (int n = 0; n < N; n++) acc[n] = 0ull;
#pragma unroll
        for (int k = 0; k < K; k++) {
            const float xik = sx * xi[k];
            const unsigned long long xx = f2pack(xr[k], xr[k]), xj = f2pack(-xik, xik);
#pragma unroll
            for (int n = 0; n < N; n++) {
                const float4 y = ybc[k * N + n];
                fma2(acc[n], xx, f2pack(y.x, y.y));
                fma2(acc[n], xj, f2pack(y.z, y.w));
            }
        }
        float re[N], im[N];
#pragma unroll
        for (int n = 0; n < N; n++) {
            re[n] = u2f((unsigned)(acc[n] & 0xffffffffull));
            im[n] = u2f((unsigned)(acc[n] >> 32));
            if (SCALED) {
                re[n] *= scale; im[n] *= scale;
                const float mx = fmaxf(fabsf(re[n]), fabsf(im[n]));
                if (mx > 0.f) emax = emax > exp_of(mx) ? emax : exp_of(mx);
            }
        }
        bool cpaired = false;
        if constexpr (N > 1) {
            if (a.cpair) {                                  // n, n+1 adjacent in C
                cpaired = true;
#pragma unroll
                for (int n = 0; n < N; n += 2)
                    *reinterpret_cast<float4*>(crow + cnc[n]) = make_float4(re[n], im[n], re[n + 1], im[n + 1]);
            }
        }
        if (!cpaired) {
#pragma unroll
            for (int n = 0; n < N; n++) crow[cnc[n]] = make_float2(re[n], im[n]);
        }
        }
        const unsigned long long next = (unsigned long long)(g + 1);
#ifdef __CUDA_ARCH__
        const int j = __ffsll((long long)next) - 1;        // bits 0..j of g flip
#else
        const int j = __builtin_ctzll(next);
#endif
        ox += t.dX[j];
        oc += t.dC[j];
        ob += t.dB[j];
    }
}

// Launched with kThreads threads; dynamic shared memory: rows2_smem_bytes.
template <int K, int N, bool SCALED, bool MULTI>
__global__ void __launch_bounds__(kThreads) contract_rows2_kernel(const Rows2Args a, int* exps) {
    extern __shared__ __align__(16) unsigned char rows2_smem[];
    const Rows2Smem t = rows2_carve<K, N>(a, rows2_smem);
    rows2_fill<K, N>(a, t, threadIdx.x, kThreads);
    __syncthreads();
    float scale = 1.f;
    if (SCALED) {
        const int mX = read_m(exps, a.expX), mY = read_m(exps, a.expY);
        scale = pow2f(-(mX + mY));
        if (blockIdx.x == 0 && threadIdx.x == 0)
            exps[2 * a.expC] = exps[2 * a.expX] + exps[2 * a.expY] + mX + mY;
    }
    int emax = kExpUnset;
    rows2_walk<K, N, SCALED, MULTI>(a, t, (int64_t)blockIdx.x * (kThreads / 32) + (threadIdx.x >> 5),
                             (int64_t)gridDim.x * (kThreads / 32), threadIdx.x & 31, scale, emax);
    if (SCALED) {
        for (int o = 16; o > 0; o >>= 1) emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, o));
        if ((threadIdx.x & 31) == 0 && emax != kExpUnset) atomicMax(&exps[2 * a.expC + 1], emax);
    }
}

size_t rows2_smem_bytes(const Rows2Args& a, int K, int N) {
    return sizeof(float4) * (size_t)a.nbatch * (size_t)(K * N * a.nchunk + 1) +
           sizeof(int64_t) * (3 * 48 + K + N * a.nchunk);
}

}  // namespace

// Fill the compact row form (FP32) from a row form: K <= 32, Y (batches x K x N) at most
// kRows2MaxY elements; N in chunks of min(16, 256 / K) columns.
bool plan_rows2(const RowArgs& ra, Rows2Args* r2) {
    auto lg = [](int64_t v) { int b = 0; while ((int64_t(1) << b) < v) b++; return b; };
    auto pos_of = [](const BitMap& m, int64_t bit) {
        const int64_t o = pdep(bit, m);
        return o ? __builtin_ctzll((unsigned long long)o) : -1;
    };
    const int R = lg(ra.nrows);
    if (ra.K > 32) return false;
    const int nlb = std::min(R, 5);                         // row bits on the lanes
    std::vector<std::pair<int, int>> lX, lC, lB, gX, gC, gB, nY, bY;
    int nb = 0;
    for (int i = 0; i < R; i++) {
        const int c = pos_of(ra.rowmap, int64_t(1) << i);
        const int x = pos_of(ra.cX, int64_t(1) << c), y = pos_of(ra.cY, int64_t(1) << c);
        if (c < 0 || x < 0) return false;
        auto& mx = i < nlb ? lX : gX;
        auto& mc = i < nlb ? lC : gC;
        auto& mb = i < nlb ? lB : gB;
        const int src = i < nlb ? i : i - nlb;
        mx.push_back({src, x});
        mc.push_back({src, c});
        if (y >= 0) {
            mb.push_back({src, nb});
            bY.push_back({nb, y});
            nb++;
        }
    }
    for (int j = 0; (1 << j) < ra.N; j++) {
        const int c = pos_of(ra.nmap, int64_t(1) << j);
        const int y = c < 0 ? -1 : pos_of(ra.cY, int64_t(1) << c);
        if (y < 0) return false;
        nY.push_back({j, y});
    }
    memset(r2, 0, sizeof(*r2));
    if (!make_runs(lX, &r2->laneX) || !make_runs(lC, &r2->laneC) || !make_runs(lB, &r2->laneB) ||
        !make_runs(gX, &r2->grpX) || !make_runs(gC, &r2->grpC) || !make_runs(gB, &r2->grpB) ||
        !make_runs(nY, &r2->nY) || !make_runs(bY, &r2->bY))
        return false;
    r2->kX = ra.kX;
    r2->kY = ra.kY;
    r2->nC = ra.nmap;
    r2->X = ra.X;
    r2->Y = ra.Y;
    r2->C = ra.C;
    r2->ngroups = int64_t(1) << (R - nlb);
    r2->lanes = 1 << nlb;
    r2->ncol = std::min({ra.N, 16, 256 / ra.K});
    r2->nchunk = ra.N / r2->ncol;
    r2->nbatch = 1 << nb;
    if ((int64_t)r2->nbatch * ra.K * ra.N > kRows2MaxY) return false;
    r2->conjX = ra.conjX;
    r2->conjY = ra.conjY;
    r2->expX = ra.expX;
    r2->expY = ra.expY;
    r2->expC = ra.expC;
    r2->xpair = ra.K > 1 && pdep(1, ra.kX) == 1 && (reinterpret_cast<uintptr_t>(ra.X) & 15) == 0;
    r2->cpair = ra.N > 1 && pdep(1, ra.nmap) == 1 && (reinterpret_cast<uintptr_t>(ra.C) & 15) == 0;
    return true;
}

namespace {

template <int K, int N>
cudaError_t launch_rows2_kn(const Rows2Args& r2, int* exps, cudaStream_t s, int sm_count) {
    const size_t smem = rows2_smem_bytes(r2, K, N);
    auto launch = [&](auto kern) -> cudaError_t {
        if (smem > 48 * 1024) {
            const cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return e;
        }
        int per_sm = 0;
        const cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, smem);
        if (e != cudaSuccess) return e;
        const int64_t cap = (int64_t)sm_count * std::max(per_sm, 1);
        const int64_t want = (r2.ngroups + kThreads / 32 - 1) / (kThreads / 32);
        const int grid = (int)std::max<int64_t>(1, std::min(want, cap));
        kern<<<grid, kThreads, smem, s>>>(r2, exps);
        return cudaGetLastError();
    };
    if (r2.nchunk > 1) {
        // several column chunks: only the widest chunk of a K has them
        if constexpr (N == (K == 32 ? 8 : 16))
            return exps ? launch(contract_rows2_kernel<K, N, true, true>) : launch(contract_rows2_kernel<K, N, false, true>);
        return cudaErrorInvalidValue;
    }
    return exps ? launch(contract_rows2_kernel<K, N, true, false>) : launch(contract_rows2_kernel<K, N, false, false>);
}

template <int K>
cudaError_t launch_rows2_k(const Rows2Args& r2, int N, int* exps, cudaStream_t s, int sm_count) {
    switch (N) {
        case 1: return launch_rows2_kn<K, 1>(r2, exps, s, sm_count);
        case 2: return launch_rows2_kn<K, 2>(r2, exps, s, sm_count);
        case 4: return launch_rows2_kn<K, 4>(r2, exps, s, sm_count);
        case 8: if constexpr (K <= 32) return launch_rows2_kn<K, 8>(r2, exps, s, sm_count); break;
        case 16: if constexpr (K <= 16) return launch_rows2_kn<K, 16>(r2, exps, s, sm_count); break;
        default: break;
    }
    return cudaErrorInvalidValue;
}

}  // namespace

cudaError_t launch_rows2(const Rows2Args& r2, int K, int N, int* exps, cudaStream_t s, int sm_count) {
    switch (K) {
        case 1: return launch_rows2_k<1>(r2, N, exps, s, sm_count);
        case 2: return launch_rows2_k<2>(r2, N, exps, s, sm_count);
        case 4: return launch_rows2_k<4>(r2, N, exps, s, sm_count);
        case 8: return launch_rows2_k<8>(r2, N, exps, s, sm_count);
        case 16: return launch_rows2_k<16>(r2, N, exps, s, sm_count);
        case 32: return launch_rows2_k<32>(r2, N, exps, s, sm_count);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace qxg
