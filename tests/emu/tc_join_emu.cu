// Host emulation of the tensor-core join's index work (tc_join.cu), built with AddressSanitizer.
//
// For seeded random operand layouts that the join's planner accepts, every block (batch value,
// K range) is walked as the kernel walks it: chunk bases by the delta table (checked against the
// direct deposit), each raw chunk's segments copied into a ring slot of the planned size (every
// byte written at most once, inside the slot), and the splitters' reads of P[i, kl] and Q[j, kl]
// through the slot-byte tables.  The products are summed in FP64 per block, written through the
// result offsets (or the K-range partials and their ordered sum), and compared with a direct
// evaluation of the contraction.  The tf32 split and the MMA are the GPU tests' part.
#include "../../qxtools.jl_gb300/csrc/tc_join.cu"

#include <complex>
#include <cstdio>
#include <cstdlib>
#include <random>

using namespace qxg;

static BitMap mk(std::vector<std::pair<int, int>> v) {
    std::sort(v.begin(), v.end());
    BitMap m;
    memset(&m, 0, sizeof(m));
    if (!make_runs(v, &m)) { printf("too many runs\n"); exit(1); }
    return m;
}

static int g_split = 0, g_tma = 0;

// One block's sums: acc[i * nq + j] over the block's K range.
static bool emulate_block(const TcJoinArgs& g, int64_t bi, int64_t si, std::vector<std::complex<double>>& acc) {
    std::vector<uint8_t> slot((size_t)g.slot_bytes);
    std::vector<uint8_t> written((size_t)g.slot_bytes);
    const int tileB = join_qtile_bytes(g.nq);
    std::vector<uint8_t> btiles((size_t)2 * kJoinSubs * tileB);
    std::vector<uint8_t> bwritten(btiles.size());
    const int64_t bP0 = pdep(bi, g.bP), bQ0 = pdep(bi, g.bQ);
    int64_t wp = join_base_p(g, bi, si, 0), wq = join_base_q(g, bi, si, 0);
    auto mark = [&](std::vector<uint8_t>& w, size_t at, size_t n) {
        for (size_t b = 0; b < n; b++) {
            if (w.at(at + b)) { printf("byte %zu written twice\n", at + b); return false; }
            w.at(at + b) = 1;
        }
        return true;
    };
    for (int64_t c = 0; c < g.nchunks; c++) {
        if (wp != join_base_p(g, bi, si, c) || wq != join_base_q(g, bi, si, c)) {
            printf("delta walk differs from the deposit at chunk %lld\n", (long long)c);
            return false;
        }
        std::fill(written.begin(), written.end(), 0);
        // the loader: segments by cp.async.bulk, or one TMA box per operand
        auto copy_segments = [&](const float2* src, int64_t base, bool p) {
            const int nseg = p ? g.nsegP : g.nsegQ, sb = p ? g.sbP : g.sbQ;
            const int stride = p ? g.segP_stride : g.segQ_stride, base_byte = p ? 0 : g.slotP_bytes;
            for (int sg = 0; sg < nseg; sg++) {
                const int64_t off = base + (p ? join_seg_p(g, sg) : join_seg_q(g, sg));
                const int bytes = 8 << sb;
                const int dst = base_byte + sg * stride;
                if (dst % 16 != 0 || (off * 8) % 16 != 0) { printf("unaligned segment\n"); return false; }
                if (dst + bytes > g.slot_bytes) { printf("segment outside the slot\n"); return false; }
                if (!mark(written, (size_t)dst, (size_t)bytes)) return false;
                memcpy(&slot.at((size_t)dst), src + off, (size_t)bytes);
            }
            return true;
        };
        auto copy_box = [&](const float2* src, const JoinBox& bx, int64_t chunk_off, bool p) {
            int co[5] = {(int)chunk_off, 0, 0, 0, 0};
            if (bx.tb >= 0) co[bx.tb] = (int)((p ? bP0 : bQ0) >> bx.th);
            if ((co[0] * 8) % 16 != 0) { printf("TMA x coordinate not 16-byte aligned\n"); return false; }
            int64_t n = 1;
            for (int d = 0; d < bx.td; d++) n *= bx.box[d];
            const int base_byte = p ? 0 : g.slotP_bytes;
            if (base_byte % 128 != 0 || base_byte + n * 8 > g.slot_bytes) { printf("box outside the slot\n"); return false; }
            for (int64_t e = 0; e < n; e++) {
                int64_t rem = e, off = 0;
                for (int d = 0; d < bx.td; d++) {
                    const int64_t i = rem % bx.box[d];
                    rem /= bx.box[d];
                    if (co[d] + i >= bx.dim[d]) { printf("box coordinate outside dimension %d\n", d); return false; }
                    off += (co[d] + i) * bx.stride[d];
                }
                if (!mark(written, (size_t)(base_byte + e * 8), 8)) return false;
                memcpy(&slot.at((size_t)(base_byte + e * 8)), src + off, 8);
            }
            return true;
        };
        if (g.tma) {
            if (!copy_box(g.P, g.boxP, wp - bP0, true) || !copy_box(g.Q, g.boxQ, wq - bQ0, false)) return false;
        } else {
            if (!copy_segments(g.P, wp, true) || !copy_segments(g.Q, wq, false)) return false;
        }
        const int t = __builtin_ctzll((unsigned long long)(si * g.nchunks + c + 1));
        wp += join_delta(g.hP, t);
        wq += join_delta(g.hQ, t);
        auto at = [&](int byte) {
            if (byte < 0 || byte + 8 > g.slot_bytes || !written.at((size_t)byte)) {
                printf("read of an unwritten slot byte %d\n", byte);
                exit(1);
            }
            float2 v;
            memcpy(&v, &slot.at((size_t)byte), 8);
            return v;
        };
        // the Q splitters: thread tq takes elements tq + 128 m, stores (re, im) words into the B tiles
        std::fill(bwritten.begin(), bwritten.end(), 0);
        for (int tq = 0; tq < kJoinQThreads; tq++)
            for (int m = 0; m < g.nq * kJoinKR / kJoinQThreads; m++) {
                const int64_t e = tq + (int64_t)kJoinQThreads * m;
                const int src = g.slotP_bytes + join_qsrc(g, tq) + join_qsrc(g, (int64_t)kJoinQThreads * m);
                const int dst = join_qdst(g, tq) + join_qdst(g, (int64_t)kJoinQThreads * m);
                if (src != g.slotP_bytes + join_qsrc(g, e) || dst != join_qdst(g, e)) {
                    printf("Q tables do not add\n");
                    return false;
                }
                const float2 v = at(src);
                const int lo = (g.nq / 8) * 512;
                const int words[4] = {dst, dst + 256, dst + lo, dst + lo + 256};
                const float vals[4] = {v.x, v.y, v.x, v.y};
                for (int w = 0; w < 4; w++) {
                    if (words[w] < 0 || words[w] + 4 > (int)btiles.size() || words[w] % tileB + 4 > tileB - kJoinPadBytes) {
                        printf("B word outside its tile\n");
                        return false;
                    }
                    if (!mark(bwritten, (size_t)words[w], 4)) return false;
                    memcpy(&btiles[(size_t)words[w]], &vals[w], 4);
                }
            }
        // the MMA's view: stage sub, group gg -> tile 2 sub + gg, row j, core column cc, word w
        auto bword = [&](int tile, int row, int cc, int w) {
            float x;
            memcpy(&x, &btiles.at((size_t)tile * tileB + (row >> 3) * 512 + cc * 128 + (row & 7) * 16 + w * 4), 4);
            return x;
        };
        for (int kl = 0; kl < kJoinKR; kl++) {
            const int tile = kl >> 3, tt = kl & 7;
            for (int i = 0; i < 32; i++) {
                const float2 p = at(join_prow(g, i) + join_pcol(g, kl));
                const std::complex<double> pv(p.x, g.conjP ? -p.y : p.y);
                for (int j = 0; j < g.nq; j++) {
                    const float qr = bword(tile, j, tt >> 2, tt & 3), qi = bword(tile, j, 2 + (tt >> 2), tt & 3);
                    const float lr = bword(tile, g.nq + j, tt >> 2, tt & 3), li = bword(tile, g.nq + j, 2 + (tt >> 2), tt & 3);
                    if (qr != lr || qi != li) { printf("hi and lo rows disagree\n"); return false; }
                    acc[(size_t)i * g.nq + j] += pv * std::complex<double>(qr, g.conjQ ? -qi : qi);
                }
            }
        }
    }
    return true;
}

// -1: failed, 0: not planned, 1: passed.
int join_case(std::mt19937& rng, int nk, int nq_bits, int ng, bool p_is_b, bool low_tiles, int min_nsplit_sm,
              int* used) {
    const int na = p_is_b ? nq_bits : 5, nb = p_is_b ? 5 : nq_bits;
    const int abits = na + ng + nk, bbits = nb + ng + nk, cbits = na + nb + ng;
    std::vector<int> ap(abits), bp(bbits), cp(cbits);
    for (int i = 0; i < abits; i++) ap[i] = i;
    for (int i = 0; i < bbits; i++) bp[i] = i;
    for (int i = 0; i < cbits; i++) cp[i] = i;
    std::shuffle(ap.begin(), ap.end(), rng);
    std::shuffle(bp.begin(), bp.end(), rng);
    std::shuffle(cp.begin(), cp.end(), rng);
    // bit roles in each operand: [free][batch][summed]; low_tiles moves the batch bits on top of the
    // address (as the programme's layout rule places them)
    if (low_tiles) {
        auto top = [&](std::vector<int>& pos, int nfree) {
            const int n = (int)pos.size();
            std::vector<int> lo;
            for (int p = 0; p < n - ng; p++) lo.push_back(p);
            std::shuffle(lo.begin(), lo.end(), rng);
            int li = 0, hi = n - ng;
            for (int i = 0; i < n; i++) pos[i] = (i >= nfree && i < nfree + ng) ? hi++ : lo[li++];
        };
        top(ap, na);
        top(bp, nb);
    }
    std::vector<std::pair<int, int>> cA, cB, kA, kB;
    for (int j = 0; j < na; j++) cA.push_back({cp[j], ap[j]});
    for (int j = 0; j < nb; j++) cB.push_back({cp[na + j], bp[j]});
    for (int j = 0; j < ng; j++) { cA.push_back({cp[na + nb + j], ap[na + j]}); cB.push_back({cp[na + nb + j], bp[nb + j]}); }
    for (int j = 0; j < nk; j++) { kA.push_back({j, ap[na + ng + j]}); kB.push_back({j, bp[nb + ng + j]}); }
    const int64_t NA_ = int64_t(1) << abits, NB_ = int64_t(1) << bbits, NC = int64_t(1) << cbits;
    std::vector<float2> A(NA_), B(NB_), C(NC, make_float2(NAN, NAN));
    std::uniform_real_distribution<double> U(-1, 1);
    for (int64_t i = 0; i < NA_; i++) A[i] = make_float2(U(rng), U(rng));
    for (int64_t i = 0; i < NB_; i++) B[i] = make_float2(U(rng), U(rng));
    const bool cA_ = rng() % 2, cB_ = rng() % 2;
    StepArgs s;
    memset(&s, 0, sizeof(s));
    s.A = A.data(); s.B = B.data(); s.C = C.data(); s.nC = NC; s.nk = nk; s.conjA = cA_; s.conjB = cB_;
    s.cA = mk(cA); s.cB = mk(cB); s.kA = mk(kA); s.kB = mk(kB);
    TcJoinArgs g;
    if (!tc_join_plan(s, min_nsplit_sm, &g, 12)) return 0;
    (*used)++;
    if (g.nsplit > 1) g_split++;
    if (g.tma) g_tma++;
    if (g.nq != (1 << nq_bits) || g.ring < 2 || g.ring > kJoinMaxRing || g.nsegP > kJoinMaxSeg ||
        g.nsegQ > kJoinMaxSeg || join_smem_bytes(g) > kJoinSmemCap + 128) {
        printf("plan outside the kernel's limits\n");
        return -1;
    }
    const int64_t per = 32 * (int64_t)g.nq;
    std::vector<std::complex<double>> partial((size_t)(g.nsplit * g.nbatch * per));
    for (int64_t blk = 0; blk < g.nbatch * g.nsplit; blk++) {
        const int64_t bi = blk % g.nbatch, si = blk / g.nbatch;
        std::vector<std::complex<double>> acc((size_t)per);
        if (!emulate_block(g, bi, si, acc)) return -1;
        for (int i = 0; i < 32; i++)
            for (int j = 0; j < g.nq; j++) {
                const std::complex<double> v = acc[(size_t)i * g.nq + j];
                if (g.nsplit == 1) {
                    const int64_t o = join_c_offset(g, bi, i, j);
                    if (o < 0 || o >= NC || !std::isnan(C[o].x)) { printf("result offset %lld reused or out of range\n", (long long)o); return -1; }
                    C[o] = make_float2((float)v.real(), (float)v.imag());
                } else {
                    partial.at((size_t)(((si * g.nbatch + bi) * 32 + i) * g.nq + j)) = v;
                }
            }
    }
    if (g.nsplit > 1)
        for (int64_t idx = 0; idx < g.nbatch * per; idx++) {
            std::complex<double> v = 0;
            for (int s2 = 0; s2 < g.nsplit; s2++) v += partial.at((size_t)(s2 * g.nbatch * per + idx));
            const int64_t o = join_c_offset(g, idx / per, (int)((idx % per) / g.nq), (int)(idx % g.nq));
            if (o < 0 || o >= NC || !std::isnan(C[o].x)) { printf("result offset reused\n"); return -1; }
            C[o] = make_float2((float)v.real(), (float)v.imag());
        }
    double maxerr = 0, maxv = 0;
    for (int64_t c = 0; c < NC; c++) {
        std::complex<double> acc = 0;
        for (int64_t k = 0; k < (int64_t(1) << nk); k++) {
            const float2 x = A[pdep(c, s.cA) + pdep(k, s.kA)], y = B[pdep(c, s.cB) + pdep(k, s.kB)];
            acc += std::complex<double>(x.x, cA_ ? -x.y : x.y) * std::complex<double>(y.x, cB_ ? -y.y : y.y);
        }
        const double e = std::abs(acc - std::complex<double>(C[c].x, C[c].y));
        if (!(e <= 1e30)) { maxerr = INFINITY; break; }
        maxerr = std::max(maxerr, e);
        maxv = std::max(maxv, std::abs(acc));
    }
    if (!(maxerr <= 1e-5 * std::max(1.0, maxv))) {
        printf("FAIL join nk=%d nq=%d ng=%d P=%s nsplit=%d err=%g max=%g\n", nk, g.nq, ng, g.p_is_a ? "A" : "B",
               g.nsplit, maxerr, maxv);
        return -1;
    }
    return 1;
}

int main(int argc, char** argv) {
    const unsigned seed = argc > 1 ? (unsigned)atoi(argv[1]) : 1u;
    const int ncases = argc > 2 ? atoi(argv[2]) : 200;
    std::mt19937 rng(seed);
    int used = 0, fail = 0, tried = 0;
    for (int it = 0; it < ncases; it++) {
        const int nq_bits = 3 + rng() % 3, ng = rng() % 3, nk = 10 + rng() % 2;
        const bool p_is_b = nq_bits == 5 ? true : (rng() % 2 != 0);
        tried++;
        // few SMs: K cut into ranges for one batch value
        const int sms = (rng() % 3 == 0) ? 8 : 1;
        if (join_case(rng, nk, nq_bits, ng, p_is_b, rng() % 4 != 0, sms, &used) < 0) fail++;
    }
    printf("tensor-core join: %d layouts tried, %d planned (%d with K ranges, %d with TMA boxes), %d failed\n", tried,
           used, g_split, g_tma, fail);
    return fail || used < 10 || g_split == 0 || g_tma == 0 ? 1 : 0;
}
