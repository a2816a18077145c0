// Host emulation of the index work of two CUDA-core kernels, checked against a direct evaluation
// of the contraction on random bit layouts (CPU only; a CPU test builds and runs this file).
//
//   * compact row form (kernels_rows.cu): the host planner plan_rows2 and the kernel's phases
//     rows2_fill / rows2_walk, run for every lane of every warp;
//   * long sum (kernels_simt.cu): plan_lsum and the phases lsum_fill / lsum_walk /
//     lsum_lane_block, the FP64 butterfly over lanes and the warp-order sums emulated as the
//     kernel performs them, and lsum_reduce_one;
//   * batched small GEMM (kernels_bgemm.cu): plan_bgemm (with a lower operand-size floor, so
//     the cases stay small) and the phases bgemm_elem_a/_b, bgemm_base_a/_b, bgemm_quad_a/_b,
//     bgemm_chunk, bgemm_flush, bgemm_c_offset and bgemm_reduce_one, run for every thread of every
//     block over exactly sized shared-memory buffers and partials.
//
// Paired FP32 FMAs run as two fused multiply-adds on the host.  Inputs are seeded; every layout
// is a random permutation of operand bits (rows, summed, result columns, batch bits), with and
// without conjugation.  Exit status 0 when every case agrees within 1e-5 of its largest result.
#include "../../qxtools.jl_gb300/csrc/kernels_simt.cu"
#include "../../qxtools.jl_gb300/csrc/kernels_rows.cu"
#include "../../qxtools.jl_gb300/csrc/kernels_bgemm.cu"

#include <complex>
#include <cstdio>
#include <cstdlib>
#include <array>
#include <random>

using namespace qxg;

static int g_lsum_chunked = 0;

static BitMap mk(std::vector<std::pair<int, int>> v) {
    std::sort(v.begin(), v.end());
    BitMap m;
    memset(&m, 0, sizeof(m));
    if (!make_runs(v, &m)) { printf("too many runs\n"); exit(1); }
    return m;
}

template <int K, int N>
void emulate_rows(const Rows2Args& r2, int64_t nwarps) {
    std::vector<unsigned char> smem(rows2_smem_bytes(r2, K, N) + 64);
    if (r2.ncol != N) { printf("ncol mismatch\n"); exit(1); }
    unsigned char* base = smem.data() + (16 - ((uintptr_t)smem.data() & 15)) % 16;
    Rows2Smem t = rows2_carve<K, N>(r2, base);
    for (int tid = 0; tid < 256; tid++) rows2_fill<K, N>(r2, t, tid, 256);
    int emax = kExpUnset;
    for (int64_t w = 0; w < nwarps; w++)
        for (int lane = 0; lane < 32; lane++) {
            if (r2.nchunk > 1) rows2_walk<K, N, false, true>(r2, t, w, nwarps, lane, 1.f, emax);
            else rows2_walk<K, N, false, false>(r2, t, w, nwarps, lane, 1.f, emax);
        }
}

template <int K>
bool emulate_rows_k(const Rows2Args& r2, int N, int64_t nw) {
    switch (N) {
        case 1: emulate_rows<K, 1>(r2, nw); return true;
        case 2: emulate_rows<K, 2>(r2, nw); return true;
        case 4: emulate_rows<K, 4>(r2, nw); return true;
        case 8: emulate_rows<K, 8>(r2, nw); return true;
        case 16: if constexpr (K <= 16) { emulate_rows<K, 16>(r2, nw); return true; } return false;
    }
    return false;
}
bool emulate_rows_any(const Rows2Args& r2, int K, int N, int64_t nw) {
    switch (K) {
        case 1: return emulate_rows_k<1>(r2, N, nw);
        case 2: return emulate_rows_k<2>(r2, N, nw);
        case 4: return emulate_rows_k<4>(r2, N, nw);
        case 8: return emulate_rows_k<8>(r2, N, nw);
        case 16: return emulate_rows_k<16>(r2, N, nw);
        case 32: return emulate_rows_k<32>(r2, N, nw);
    }
    return false;
}

int rows_case(std::mt19937& rng, int R, int nk, int nn, int nbatch, bool conjX, bool conjY, bool ordered, int* used) {
    const int xb = R + nk, cb = R + nn, yb = nk + nn + nbatch;
    std::vector<int> xp(xb), cp(cb), yp(yb);
    for (int i = 0; i < xb; i++) xp[i] = i;
    for (int i = 0; i < cb; i++) cp[i] = i;
    for (int i = 0; i < yb; i++) yp[i] = i;
    std::shuffle(xp.begin(), xp.end(), rng);
    std::shuffle(yp.begin(), yp.end(), rng);
    if (ordered) {
        std::vector<int> kind(xb);
        for (int i = 0; i < R; i++) kind[xp[i]] = i;
        for (int j = 0; j < nk; j++) kind[xp[R + j]] = -1 - j;
        int p = 0, ni = 0;
        for (int q = 0; q < xb; q++) {
            if (kind[q] >= 0) cp[kind[q]] = p++;
            else if (ni < nn) cp[R + ni++] = p++;
        }
        while (ni < nn) cp[R + ni++] = p++;
    } else std::shuffle(cp.begin(), cp.end(), rng);
    std::vector<std::pair<int,int>> cA, kA, cB, kB;
    for (int i = 0; i < R; i++) cA.push_back({cp[i], xp[i]});
    for (int i = 0; i < nbatch; i++) cB.push_back({cp[i], yp[nk + nn + i]});
    for (int j = 0; j < nn; j++) cB.push_back({cp[R + j], yp[nk + j]});
    for (int j = 0; j < nk; j++) { kA.push_back({j, xp[R + j]}); kB.push_back({j, yp[j]}); }
    const int64_t NX = int64_t(1) << xb, NY = int64_t(1) << yb, NC = int64_t(1) << cb;
    // 16-byte aligned storage
    std::vector<float4> Xs((NX + 1) / 2 + 1), Ys((NY + 1) / 2 + 1), Cs((NC + 1) / 2 + 1);
    float2* X = reinterpret_cast<float2*>(Xs.data());
    float2* Y = reinterpret_cast<float2*>(Ys.data());
    float2* C = reinterpret_cast<float2*>(Cs.data());
    std::uniform_real_distribution<double> U(-1, 1);
    for (int64_t i = 0; i < NX; i++) X[i] = make_float2(U(rng), U(rng));
    for (int64_t i = 0; i < NY; i++) Y[i] = make_float2(U(rng), U(rng));
    for (int64_t i = 0; i < NC; i++) C[i] = make_float2(NAN, NAN);
    StepArgs a; memset(&a, 0, sizeof(a));
    a.A = X; a.B = Y; a.C = C; a.nC = NC; a.nk = nk; a.conjA = conjX; a.conjB = conjY;
    a.cA = mk(cA); a.kA = mk(kA); a.cB = mk(cB); a.kB = mk(kB);
    RowArgs ra;
    Rows2Args r2;
    if (!use_rows2(a, false, &ra, &r2)) return 0;
    (*used)++;
    const int64_t nw = 1 + rng() % 40;
    if (!emulate_rows_any(r2, ra.K, r2.ncol, nw)) { printf("no instance K=%d N=%d\n", ra.K, r2.ncol); return -1; }
    double maxerr = 0, maxv = 0;
    for (int64_t c = 0; c < NC; c++) {
        std::complex<double> acc = 0;
        for (int64_t k = 0; k < (int64_t(1) << nk); k++) {
            float2 x = X[pdep(c, a.cA) + pdep(k, a.kA)], y = Y[pdep(c, a.cB) + pdep(k, a.kB)];
            acc += std::complex<double>(x.x, conjX ? -x.y : x.y) * std::complex<double>(y.x, conjY ? -y.y : y.y);
        }
        const double e = std::abs(acc - std::complex<double>(C[c].x, C[c].y));
        if (!(e <= 1e30)) { maxerr = INFINITY; break; }
        maxerr = std::max(maxerr, e);
        maxv = std::max(maxv, std::abs(acc));
    }
    if (!(maxerr <= 1e-5 * std::max(1.0, maxv))) {
        printf("FAIL R=%d nk=%d nn=%d nb=%d xpair=%d cpair=%d nw=%lld err=%g\n", R, nk, nn, nbatch, r2.xpair, r2.cpair,
               (long long)nw, maxerr);
        return -1;
    }
    return 1;
}

template <int NA, int NB>
void emulate_lsum(const LSumArgs& la, std::vector<double2>& partial) {
    const int Na = lsum_na(la, NA), NaAll = lsum_na_all(la, NA), Nb = la.CB * NB, S = 32 >> la.LR, R = 1 << la.LR,
              pw = S * NA * NB;
    const int CW = la.CA * la.CB, sets = kLSumWarps / CW;
    std::vector<unsigned char> smem(lsum_smem_bytes(NaAll, Nb, pw) + 64);
    unsigned char* base = smem.data() + (16 - ((uintptr_t)smem.data() & 15)) % 16;
    LSumSmem t = lsum_carve(base, NaAll, Nb);
    for (int tid = 0; tid < kThreads; tid++) lsum_fill(la, t, NaAll, Nb, tid, kThreads);
    for (int blk = 0; blk < la.ng * la.G * la.nrc; blk++) {
        const int chunk = blk / (la.ng * la.G);
        const int g = (blk % (la.ng * la.G)) / la.G, part = blk % la.G;
        for (int warp = 0; warp < kLSumWarps; warp++) {
            static double vr[32][16][4], vi[32][16][4];
            for (int lane = 0; lane < 32; lane++) {
                int a0, b0;
                lsum_lane_block(la, NA, NB, warp, lane, &a0, &b0);
                a0 += chunk * Na;
                unsigned long long acc[NA][NB];
                for (int i = 0; i < NA; i++) for (int j = 0; j < NB; j++) acc[i][j] = 0ull;
                lsum_walk<NA, NB>(la, t, pdep(g, la.gA), pdep(g, la.gB), (int64_t)part * sets + warp / CW,
                                  (int64_t)la.G * sets, lane, a0, b0, acc);
                for (int i = 0; i < NA; i++) for (int j = 0; j < NB; j++) {
                    vr[lane][i][j] = u2f((unsigned)(acc[i][j] & 0xffffffffull));
                    vi[lane][i][j] = u2f((unsigned)(acc[i][j] >> 32));
                }
            }
            for (int o = 1; o < R; o <<= 1) {
                static double nr[32][16][4], ni[32][16][4];
                for (int l = 0; l < 32; l++) for (int i = 0; i < NA; i++) for (int j = 0; j < NB; j++) {
                    nr[l][i][j] = vr[l][i][j] + vr[l ^ o][i][j];
                    ni[l][i][j] = vi[l][i][j] + vi[l ^ o][i][j];
                }
                for (int l = 0; l < 32; l++) for (int i = 0; i < NA; i++) for (int j = 0; j < NB; j++) {
                    vr[l][i][j] = nr[l][i][j]; vi[l][i][j] = ni[l][i][j];
                }
            }
            for (int l = 0; l < 32; l++) {
                if (l & (R - 1)) continue;
                const int sub = l >> la.LR;
                for (int i = 0; i < NA; i++) for (int j = 0; j < NB; j++) {
                    const int res = (sub * NA + i) * NB + j;
                    t.red[2 * (warp * pw + res)] = vr[l][i][j];
                    t.red[2 * (warp * pw + res) + 1] = vi[l][i][j];
                }
            }
        }
        for (int o = 0; o < Na * Nb; o++) {
            const int av = o / Nb, bv = o % Nb;
            const int ca = av / (S * NA), sub2 = (av % (S * NA)) / NA, i = av % NA;
            const int cb = bv / NB, j = bv % NB;
            const int c = ca * la.CB + cb, res = (sub2 * NA + i) * NB + j;
            double re = 0, im = 0;
            for (int st = 0; st < sets; st++) { const int w = st * CW + c; re += t.red[2 * (w * pw + res)]; im += t.red[2 * (w * pw + res) + 1]; }
            partial[((size_t)g * la.G + part) * (NaAll * Nb) + (size_t)chunk * Na * Nb + o] = make_double2(re, im);
        }
    }
    for (int64_t idx = 0; idx < (int64_t)la.ng * NaAll * Nb; idx++) lsum_reduce_one(la, NaAll * Nb, Nb, partial.data(), idx, 1.0);
}

template <int NB>
bool emulate_lsum_b(const LSumArgs& la, int NA, std::vector<double2>& p) {
    switch (NA) {
        case 1: emulate_lsum<1, NB>(la, p); return true;
        case 2: if constexpr (2 * NB <= kLSumOut) { emulate_lsum<2, NB>(la, p); return true; } return false;
        case 4: if constexpr (4 * NB <= kLSumOut) { emulate_lsum<4, NB>(la, p); return true; } return false;
        case 8: if constexpr (8 * NB <= kLSumOut) { emulate_lsum<8, NB>(la, p); return true; } return false;
        case 16: if constexpr (16 * NB <= kLSumOut) { emulate_lsum<16, NB>(la, p); return true; } return false;
    }
    return false;
}
bool emulate_lsum_any(const LSumArgs& la, int NA, int NB, std::vector<double2>& p) {
    switch (NB) {
        case 1: return emulate_lsum_b<1>(la, NA, p);
        case 2: return emulate_lsum_b<2>(la, NA, p);
        case 4: return emulate_lsum_b<4>(la, NA, p);

    }
    return false;
}

int lsum_case(std::mt19937& rng, int nk, int na, int nb, int ng, bool cA_, bool cB_, int* used) {
    const int abits = na + ng + nk, bbits = nb + ng + nk, cbits = na + nb + ng;
    std::vector<int> ap(abits), bp(bbits), cp(cbits);
    for (int i = 0; i < abits; i++) ap[i] = i;
    for (int i = 0; i < bbits; i++) bp[i] = i;
    for (int i = 0; i < cbits; i++) cp[i] = i;
    std::shuffle(ap.begin(), ap.end(), rng);
    std::shuffle(bp.begin(), bp.end(), rng);
    std::shuffle(cp.begin(), cp.end(), rng);
    std::vector<std::pair<int,int>> cA, cB, kA, kB;
    for (int j = 0; j < na; j++) cA.push_back({cp[j], ap[j]});
    for (int j = 0; j < nb; j++) cB.push_back({cp[na + j], bp[j]});
    for (int j = 0; j < ng; j++) { cA.push_back({cp[na + nb + j], ap[na + j]}); cB.push_back({cp[na + nb + j], bp[nb + j]}); }
    for (int j = 0; j < nk; j++) { kA.push_back({j, ap[na + ng + j]}); kB.push_back({j, bp[nb + ng + j]}); }
    const int64_t NA_ = int64_t(1) << abits, NB_ = int64_t(1) << bbits, NC = int64_t(1) << cbits;
    std::vector<float4> As(NA_ / 2 + 1), Bs(NB_ / 2 + 1), Cs(NC / 2 + 1);
    float2* A = reinterpret_cast<float2*>(As.data());
    float2* B = reinterpret_cast<float2*>(Bs.data());
    float2* C = reinterpret_cast<float2*>(Cs.data());
    std::uniform_real_distribution<double> U(-1, 1);
    for (int64_t i = 0; i < NA_; i++) A[i] = make_float2(U(rng), U(rng));
    for (int64_t i = 0; i < NB_; i++) B[i] = make_float2(U(rng), U(rng));
    for (int64_t i = 0; i < NC; i++) C[i] = make_float2(NAN, NAN);
    StepArgs s; memset(&s, 0, sizeof(s));
    s.A = A; s.B = B; s.C = C; s.nC = NC; s.nk = nk; s.conjA = cA_; s.conjB = cB_;
    s.cA = mk(cA); s.cB = mk(cB); s.kA = mk(kA); s.kB = mk(kB);
    LSumArgs la; int NA = 0, NB = 0;
    if (!plan_lsum(s, 4 + rng() % 30, &la, &NA, &NB, 1 + rng() % 3)) return 0;
    (*used)++;
    if (la.nrc > 1) g_lsum_chunked++;
    std::vector<double2> partial(lsum_partial_bytes(la, NA, NB) / sizeof(double2), make_double2(NAN, NAN));
    if (!emulate_lsum_any(la, NA, NB, partial)) { printf("no instance NA=%d NB=%d\n", NA, NB); return -1; }
    double maxerr = 0, maxv = 0;
    for (int64_t c = 0; c < NC; c++) {
        std::complex<double> acc = 0;
        for (int64_t k = 0; k < (int64_t(1) << nk); k++) {
            float2 x = A[pdep(c, s.cA) + pdep(k, s.kA)], y = B[pdep(c, s.cB) + pdep(k, s.kB)];
            acc += std::complex<double>(x.x, cA_ ? -x.y : x.y) * std::complex<double>(y.x, cB_ ? -y.y : y.y);
        }
        const double e = std::abs(acc - std::complex<double>(C[c].x, C[c].y));
        if (!(e <= 1e30)) { maxerr = INFINITY; break; }
        maxerr = std::max(maxerr, e);
        maxv = std::max(maxv, std::abs(acc));
    }
    if (!(maxerr <= 1e-5 * std::max(1.0, maxv))) {
        printf("FAIL nk=%d na=%d nb=%d ng=%d NA=%d NB=%d LR=%d CA=%d CB=%d nrc=%d G=%d ap=%d bp=%d err=%g max=%g\n", nk,
               na, nb, ng, NA, NB, la.LR, la.CA, la.CB, la.nrc, la.G, la.apair, la.bpair, maxerr, maxv);
        return -1;
    }
    return 1;
}

static int g_bgemm_split = 0;

template <int M, int N>
void emulate_bgemm(const BGemmArgs& g, std::vector<double2>& partial) {
    constexpr BGemmShape S = bgemm_shape(M, N);
    constexpr int TM = S.tm, TN = S.tn;
    const int nthr = S.nthr;
    if (g.M != M || g.N != N || g.thr_m != S.thr_m || g.thr_n != S.thr_n || g.kc != S.kc || g.ra != S.ra ||
        g.rb != S.rb) { printf("shape mismatch\n"); exit(1); }
    for (int64_t blk = 0; blk < g.nbatch * g.nsplit; blk++) {
        const int64_t bi = blk % g.nbatch, si = blk / g.nbatch;
        std::vector<float4> As((size_t)2 * S.kc * S.ra), Bs((size_t)2 * S.kc * S.rb);
        std::vector<std::array<unsigned long long, TM * TN>> acc(nthr);
        std::vector<std::array<float4, TM * TN>> dacc(nthr);
        for (int t = 0; t < nthr; t++)
            for (int q = 0; q < TM * TN; q++) { acc[t][q] = 0ull; dacc[t][q] = make_float4(0, 0, 0, 0); }
        int64_t wa = bgemm_base_a(g, bi, si, 0), wb = bgemm_base_b(g, bi, si, 0);
        for (int64_t c = 0; c < g.nchunks; c++) {
            const int buf = (int)(c & 1);
            // the kernel walks chunk bases with the delta table: it must agree with the deposit
            if (wa != bgemm_base_a(g, bi, si, c) || wb != bgemm_base_b(g, bi, si, c)) {
                printf("delta walk differs from the deposit at chunk %lld\n", (long long)c);
                exit(1);
            }
            const int tz = __builtin_ctzll((unsigned long long)(si * g.nchunks + c + 1));
            wa += bgemm_delta(g.hA, tz);
            wb += bgemm_delta(g.hB, tz);
            for (int t = 0; t < nthr; t++) {
                for (int j = 0; j < S.la; j++) {
                    int64_t off;
                    int slot;
                    bgemm_elem_a(g, t, j, &off, &slot);
                    As.at((size_t)buf * S.kc * S.ra + (size_t)slot) =
                        bgemm_quad_a(g.A[bgemm_base_a(g, bi, si, c) + off], 1.f, g.conjA ? -1.f : 1.f);
                }
                for (int j = 0; j < S.lb; j++) {
                    int64_t off;
                    int slot;
                    bgemm_elem_b(g, t, j, &off, &slot);
                    Bs.at((size_t)buf * S.kc * S.rb + (size_t)slot) =
                        bgemm_quad_b(g.B[bgemm_base_b(g, bi, si, c) + off], 1.f, g.conjB ? -1.f : 1.f);
                }
            }
            for (int t = 0; t < nthr; t++) {
                const int tm = t / S.thr_n, tn = t % S.thr_n;
                // the reads of bgemm_chunk stay inside the buffer (its largest offset)
                const size_t last_a = (size_t)buf * S.kc * S.ra + tm * (TM + 1) + (S.kc - 1) * S.ra + TM - 1;
                const size_t last_b = (size_t)buf * S.kc * S.rb + tn * (TN + 1) + (S.kc - 1) * S.rb + TN - 1;
                if (last_a >= As.size() || last_b >= Bs.size()) { printf("chunk read out of range\n"); exit(1); }
                unsigned long long a2[TM][TN];
                float4 d2[TM][TN];
                for (int i = 0; i < TM; i++)
                    for (int j = 0; j < TN; j++) { a2[i][j] = acc[t][i * TN + j]; d2[i][j] = dacc[t][i * TN + j]; }
                bgemm_chunk<M, N>(As.data() + (size_t)buf * S.kc * S.ra, Bs.data() + (size_t)buf * S.kc * S.rb, tm, tn, a2);
                if (((c + 1) & (g.flush - 1)) == 0 || c + 1 == g.nchunks) bgemm_flush<TM, TN>(a2, d2);
                for (int i = 0; i < TM; i++)
                    for (int j = 0; j < TN; j++) { acc[t][i * TN + j] = a2[i][j]; dacc[t][i * TN + j] = d2[i][j]; }
            }
        }
        for (int t = 0; t < nthr; t++) {
            const int tm = t / S.thr_n, tn = t % S.thr_n;
            for (int i = 0; i < TM; i++)
                for (int j = 0; j < TN; j++) {
                    const int m = tm * TM + i, n = tn * TN + j;
                    const float4 f = dacc[t][i * TN + j];
                    const double2 v = make_double2((double)f.x + (double)f.y, (double)f.z + (double)f.w);
                    if (g.nsplit == 1) g.C[bgemm_c_offset(g, bi, m, n)] = make_float2((float)v.x, (float)v.y);
                    else partial.at((size_t)((si * g.nbatch + bi) * M + m) * N + n) = v;
                }
        }
    }
    if (g.nsplit > 1)
        for (int64_t idx = 0; idx < g.nbatch * g.M * g.N; idx++) {
            int64_t off;
            const float2 v = bgemm_reduce_one(g, partial.data(), idx, &off);
            g.C[off] = v;
        }
}

int bgemm_case(std::mt19937& rng, int nk, int na, int nb, int ng, bool cA_, bool cB_, int* used) {
    const int abits = na + ng + nk, bbits = nb + ng + nk, cbits = na + nb + ng;
    std::vector<int> ap(abits), bp(bbits), cp(cbits);
    for (int i = 0; i < abits; i++) ap[i] = i;
    for (int i = 0; i < bbits; i++) bp[i] = i;
    for (int i = 0; i < cbits; i++) cp[i] = i;
    std::shuffle(ap.begin(), ap.end(), rng);
    std::shuffle(bp.begin(), bp.end(), rng);
    std::shuffle(cp.begin(), cp.end(), rng);
    std::vector<std::pair<int,int>> cA, cB, kA, kB;
    for (int j = 0; j < na; j++) cA.push_back({cp[j], ap[j]});
    for (int j = 0; j < nb; j++) cB.push_back({cp[na + j], bp[j]});
    for (int j = 0; j < ng; j++) { cA.push_back({cp[na + nb + j], ap[na + j]}); cB.push_back({cp[na + nb + j], bp[nb + j]}); }
    for (int j = 0; j < nk; j++) { kA.push_back({j, ap[na + ng + j]}); kB.push_back({j, bp[nb + ng + j]}); }
    const int64_t NA_ = int64_t(1) << abits, NB_ = int64_t(1) << bbits, NC = int64_t(1) << cbits;
    std::vector<float2> A(NA_), B(NB_), C(NC, make_float2(NAN, NAN));
    std::uniform_real_distribution<double> U(-1, 1);
    for (int64_t i = 0; i < NA_; i++) A[i] = make_float2(U(rng), U(rng));
    for (int64_t i = 0; i < NB_; i++) B[i] = make_float2(U(rng), U(rng));
    StepArgs s; memset(&s, 0, sizeof(s));
    s.A = A.data(); s.B = B.data(); s.C = C.data(); s.nC = NC; s.nk = nk; s.conjA = cA_; s.conjB = cB_;
    s.cA = mk(cA); s.cB = mk(cB); s.kA = mk(kA); s.kB = mk(kB);
    BGemmArgs g;
    if (!plan_bgemm(s, 1 + rng() % 8, &g, 12)) return 0;
    (*used)++;
    if (g.nsplit > 1) g_bgemm_split++;
    std::vector<double2> partial(bgemm_partial_bytes(g) / sizeof(double2), make_double2(NAN, NAN));
    bool ran = false;
#define QXG_EMU_BGEMM(M_, N_) if (!ran && g.M == M_ && g.N == N_) { emulate_bgemm<M_, N_>(g, partial); ran = true; }
    QXG_BGEMM_SHAPES(QXG_EMU_BGEMM)
#undef QXG_EMU_BGEMM
    if (!ran) { printf("no instance M=%d N=%d\n", g.M, g.N); return -1; }
    double maxerr = 0, maxv = 0;
    for (int64_t c = 0; c < NC; c++) {
        std::complex<double> acc = 0;
        for (int64_t k = 0; k < (int64_t(1) << nk); k++) {
            float2 x = A[pdep(c, s.cA) + pdep(k, s.kA)], y = B[pdep(c, s.cB) + pdep(k, s.kB)];
            acc += std::complex<double>(x.x, cA_ ? -x.y : x.y) * std::complex<double>(y.x, cB_ ? -y.y : y.y);
        }
        const double e = std::abs(acc - std::complex<double>(C[c].x, C[c].y));
        if (!(e <= 1e30)) { maxerr = INFINITY; break; }
        maxerr = std::max(maxerr, e);
        maxv = std::max(maxv, std::abs(acc));
    }
    if (!(maxerr <= 1e-5 * std::max(1.0, maxv))) {
        printf("FAIL bgemm nk=%d na=%d nb=%d ng=%d kc=%d thr=%dx%d nsplit=%d err=%g max=%g\n", nk, na, nb, ng, g.kc,
               g.thr_m, g.thr_n, g.nsplit, maxerr, maxv);
        return -1;
    }
    return 1;
}

int main(int argc, char** argv) {
    const unsigned seed = argc > 1 ? (unsigned)atoi(argv[1]) : 1u;
    const int nrows = argc > 2 ? atoi(argv[2]) : 300, nsums = argc > 3 ? atoi(argv[3]) : 60;
    std::mt19937 rng(seed);
    int rows_used = 0, rows_fail = 0, lsum_used = 0, lsum_fail = 0;
    for (int it = 0; it < nrows; it++) {
        const int nk = rng() % 6, nn = rng() % 7, nbatch = rng() % 7;
        const int R = rng() % 14;
        if (nk + nn + nbatch > 13 || nbatch > R) continue;
        if (rows_case(rng, R, nk, nn, nbatch, rng() % 2, rng() % 2, rng() % 3 != 0, &rows_used) < 0) rows_fail++;
    }
    for (int it = 0; it < nsums; it++) {
        const int nk = 12 + rng() % 2, na = rng() % 7, nb = rng() % 6, ng = rng() % 3;
        if (lsum_case(rng, nk, na, nb, ng, rng() % 2, rng() % 2, &lsum_used) < 0) lsum_fail++;
    }
    for (int it = 0; it < nsums / 5; it++) {      // wide results: chunks over the grid
        const int na = 5 + rng() % 2, nb = 4 + rng() % 2, ng = rng() % 2;
        if (lsum_case(rng, 12, na, nb, ng, rng() % 2, rng() % 2, &lsum_used) < 0) lsum_fail++;
    }
    int bg_used = 0, bg_fail = 0;
    for (int it = 0; it < nsums / 2; it++) {        // both operands of 2^12 and more elements
        const int na = 3 + rng() % 4, nb = 3 + rng() % 4, ng = rng() % 4;
        if (na + nb < 8 || na + nb > 10) continue;
        const int nk = std::max(10, 13 - ng) + (int)(rng() % 2);
        if (bgemm_case(rng, nk, na, nb, ng, rng() % 2, rng() % 2, &bg_used) < 0) bg_fail++;
    }
    for (int it = 0; it < 4; it++)                  // one batch value, K cut into ranges
        if (bgemm_case(rng, 14, 4 + it % 2, 4, 0, rng() % 2, rng() % 2, &bg_used) < 0) bg_fail++;
    printf("compact row form: %d cases, %d failed; long sum: %d cases (%d in chunks), %d failed; batched gemm: %d "
           "cases (%d with K ranges), %d failed\n", rows_used, rows_fail, lsum_used, g_lsum_chunked, lsum_fail, bg_used,
           g_bgemm_split, bg_fail);
    return rows_fail || lsum_fail || bg_fail || rows_used == 0 || lsum_used == 0 || bg_used == 0 ? 1 : 0;
}
