/*
 * qxoracle.c -- CPU FP64 restatement of QXTools' contraction programme.  TEST INFRASTRUCTURE:
 * only the tests, the smoke check and the benchmark's CPU-baseline leg load this code, as the
 * checker; the product (libqxgpu) never calls it.
 *
 * What it restates (the reference's arithmetic lives in un-vendored packages, QXTns "1.0" and
 * QXContexts "1.0", Project.toml:33-38; this follows their call sites and the DSL spec):
 *   - the `.qx` command semantics, docs/src/users_guide.md:93-165:
 *       load   -> leaf tensor from the data table              (users_guide.md:98-102)
 *       view   -> t[.., v, ..] keeping the sliced index with size 1, so the ncon labels of
 *                 the viewed tensor are unchanged               (users_guide.md:104-122;
 *                 the example at :73-90 keeps `t1_s 1,2` rank-2 after `view t1_s t1 v1 1 2`)
 *       ncon   -> Einstein summation; a label in both operands but not the result is summed,
 *                 one in both operands and the result is batched, `0` marks a scalar
 *                                                               (users_guide.md:124-146)
 *       output -> basis vector of output qubit i for the bitstring's character
 *                 ('0','1','+','-', docs/src/basics.md:55-64 and the QXTns add_output! call
 *                 at src/simulation.jl:88)                      (users_guide.md:149-158)
 *       save   -> the programme's result                        (users_guide.md:161-165)
 *   - the amplitude is the sum of the saved tensor over every slice assignment
 *     (docs/src/users_guide.md:11-17: "breaks each contraction into a sum of smaller
 *     contractions by slicing bonds"), one walk per (bitstring, slice) like QXContexts'
 *     executor loop called from bin/qxrun.jl:83-87, and like `single_amplitude`
 *     (src/simulation.jl:86-91) for the unsliced case.
 * Slice id s maps to slice-variable values with the first variable fastest (column-major,
 * Julia CartesianIndices order).  Dimensions are general (no power-of-two assumption).
 * Direct FP64 sums, no compensation.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/qxgpu.h"

#define QXO_MAX_RANK 64

typedef struct { double re, im; } cplx;

typedef struct {
    int rank;
    int64_t dims[QXO_MAX_RANK];
    int64_t size;
    cplx* data;   /* owned unless borrowed */
    int borrowed;
} otensor;

/* 1 while qxo_run executes fewer jobs than threads: contractions are then threaded inside. */
static int qxo_inner_parallel = 0;
/* Time-bounded sampling (qxo_run_timed): stop the walk at the deadline, count FLOPs done. */
static double qxo_deadline = 0.0;
static double qxo_flops_done = 0.0;

#include <time.h>
static double qxo_now(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static int64_t prod_dims(int rank, const int64_t* d) {
    int64_t p = 1;
    for (int i = 0; i < rank; i++) p *= d[i];
    return p;
}

/* C[c] = sum_k A[a] B[b] over labels; general dims, column-major. */
static int ncon_general(otensor* C, const int32_t* lc, int nc,
                        const otensor* A, const int32_t* la, int na,
                        const otensor* B, const int32_t* lb, int nb) {
    /* distinct labels and their dims */
    int32_t lab[3 * QXO_MAX_RANK];
    int64_t ldim[3 * QXO_MAX_RANK];
    int nl = 0;
    #define FINDL(L, out) do { out = -1; for (int _q = 0; _q < nl; _q++) if (lab[_q] == (L)) { out = _q; break; } } while (0)
    for (int i = 0; i < na; i++) {
        int q; FINDL(la[i], q);
        if (q < 0) { lab[nl] = la[i]; ldim[nl] = A->dims[i]; nl++; }
        else if (ldim[q] != A->dims[i]) return -1;
    }
    for (int i = 0; i < nb; i++) {
        int q; FINDL(lb[i], q);
        if (q < 0) { lab[nl] = lb[i]; ldim[nl] = B->dims[i]; nl++; }
        else if (ldim[q] != B->dims[i]) return -1;
    }
    /* C labels must come from A or B */
    int cidx[QXO_MAX_RANK];
    for (int i = 0; i < nc; i++) { int q; FINDL(lc[i], q); if (q < 0) return -1; cidx[i] = q; }
    /* summed labels: those not in C */
    int kidx[3 * QXO_MAX_RANK]; int nk = 0;
    for (int q = 0; q < nl; q++) {
        int inC = 0;
        for (int i = 0; i < nc; i++) if (cidx[i] == q) inC = 1;
        if (!inC) kidx[nk++] = q;
    }
    /* per-label strides in A and B (sum over axes carrying that label) */
    int64_t sA[3 * QXO_MAX_RANK], sB[3 * QXO_MAX_RANK];
    memset(sA, 0, sizeof(sA)); memset(sB, 0, sizeof(sB));
    { int64_t st = 1; for (int i = 0; i < na; i++) { int q; FINDL(la[i], q); sA[q] += st; st *= A->dims[i]; } }
    { int64_t st = 1; for (int i = 0; i < nb; i++) { int q; FINDL(lb[i], q); sB[q] += st; st *= B->dims[i]; } }
    #undef FINDL
    C->rank = nc;
    for (int i = 0; i < nc; i++) C->dims[i] = ldim[cidx[i]];
    C->size = prod_dims(nc, C->dims);
    C->data = (cplx*)malloc(sizeof(cplx) * (size_t)(C->size > 0 ? C->size : 1));
    C->borrowed = 0;
    if (!C->data) return -2;
    int64_t K = 1;
    for (int j = 0; j < nk; j++) K *= ldim[kidx[j]];
    qxo_flops_done += 8.0 * (double)C->size * (double)K;
    /* Result elements are split into contiguous chunks; each chunk starts its odometer from
       the digits of its first element.  Runs threaded when called outside a parallel region
       (one job: all host threads work inside the contraction). */
    const int64_t nchunks = (C->size >= 4096 && qxo_inner_parallel) ? 256 : 1;
    const int64_t csz = (C->size + nchunks - 1) / nchunks;
#ifdef _OPENMP
    #pragma omp parallel for schedule(dynamic, 1) if (nchunks > 1)
#endif
    for (int64_t ch = 0; ch < nchunks; ch++) {
    const int64_t c0 = ch * csz, c1 = (c0 + csz < C->size) ? c0 + csz : C->size;
    int64_t ci[QXO_MAX_RANK]; memset(ci, 0, sizeof(ci));
    int64_t offA = 0, offB = 0;
    { int64_t rem = c0; for (int i = 0; i < nc; i++) { int q = cidx[i]; ci[i] = rem % ldim[q]; rem /= ldim[q]; offA += ci[i] * sA[q]; offB += ci[i] * sB[q]; } }
    for (int64_t c = c0; c < c1; c++) {
        double re = 0.0, im = 0.0;
        int64_t ki[3 * QXO_MAX_RANK]; memset(ki, 0, sizeof(int64_t) * (size_t)(nk ? nk : 1));
        int64_t kA = 0, kB = 0;
        for (int64_t k = 0; k < K; k++) {
            cplx a = A->data[offA + kA], b = B->data[offB + kB];
            re += a.re * b.re - a.im * b.im;
            im += a.re * b.im + a.im * b.re;
            for (int j = 0; j < nk; j++) {   /* odometer over summed labels */
                int q = kidx[j];
                ki[j]++; kA += sA[q]; kB += sB[q];
                if (ki[j] < ldim[q]) break;
                kA -= sA[q] * ldim[q]; kB -= sB[q] * ldim[q]; ki[j] = 0;
            }
        }
        C->data[c].re = re; C->data[c].im = im;
        for (int i = 0; i < nc; i++) {       /* odometer over result labels */
            int q = cidx[i];
            ci[i]++; offA += sA[q]; offB += sB[q];
            if (ci[i] < ldim[q]) break;
            offA -= sA[q] * ldim[q]; offB -= sB[q] * ldim[q]; ci[i] = 0;
        }
    }
    }
    return 0;
}

/* t[.., v, ..] with the sliced index kept at size 1 */
static int view_slice(otensor* dst, const otensor* src, int pos, int64_t v) {
    if (pos < 0 || pos >= src->rank || v < 0 || v >= src->dims[pos]) return -1;
    dst->rank = src->rank;
    memcpy(dst->dims, src->dims, sizeof(int64_t) * (size_t)src->rank);
    dst->dims[pos] = 1;
    dst->size = prod_dims(dst->rank, dst->dims);
    dst->data = (cplx*)malloc(sizeof(cplx) * (size_t)dst->size);
    dst->borrowed = 0;
    if (!dst->data) return -2;
    int64_t inner = 1;
    for (int i = 0; i < pos; i++) inner *= src->dims[i];
    int64_t d = src->dims[pos];
    int64_t outer = dst->size / inner;
    for (int64_t o = 0; o < outer; o++)
        for (int64_t i = 0; i < inner; i++)
            dst->data[o * inner + i] = src->data[(o * d + v) * inner + i];
    return 0;
}

static int output_vector(otensor* dst, char ch, int dim) {
    if (dim != 2) return -1;
    dst->rank = 1; dst->dims[0] = 2; dst->size = 2; dst->borrowed = 0;
    dst->data = (cplx*)malloc(sizeof(cplx) * 2);
    if (!dst->data) return -2;
    const double r = 1.0 / sqrt(2.0);
    switch (ch) {
        case '0': dst->data[0] = (cplx){1, 0}; dst->data[1] = (cplx){0, 0}; break;
        case '1': dst->data[0] = (cplx){0, 0}; dst->data[1] = (cplx){1, 0}; break;
        case '+': dst->data[0] = (cplx){r, 0}; dst->data[1] = (cplx){r, 0}; break;
        case '-': dst->data[0] = (cplx){r, 0}; dst->data[1] = (cplx){-r, 0}; break;
        default: free(dst->data); dst->data = NULL; return -1;
    }
    return 0;
}

typedef struct {
    const qxg_instr* ins; int nins;
    const int32_t* labels;
    const int32_t* data_rank; const int64_t* data_dims; const int64_t* data_off; const double* data;
    int ndata; int nqubits; int ntensors;
    int nvars; int64_t vdim[QXO_MAX_RANK];
    int* last_use;       /* instruction index of the last read of each tensor */
    int save_tensor;
} oprog;

/* One walk for one bitstring and one slice; result copied into out (size out_size). */
static int walk(const oprog* P, const char* bits, int64_t slice, cplx* out, int64_t out_size) {
    otensor* T = (otensor*)calloc((size_t)P->ntensors, sizeof(otensor));
    if (!T) return -2;
    int64_t vval[QXO_MAX_RANK];
    { int64_t s = slice; for (int j = 0; j < P->nvars; j++) { vval[j] = s % P->vdim[j]; s /= P->vdim[j]; } }
    int rc = 0;
    for (int n = 0; n < P->nins && rc == 0; n++) {
        const qxg_instr* I = &P->ins[n];
        if (qxo_deadline > 0.0 && qxo_now() > qxo_deadline) { rc = 1; break; }
        switch (I->op) {
        case QXG_OP_LOAD: {
            otensor* t = &T[I->dst];
            t->rank = P->data_rank[I->a];
            int64_t off = 0; for (int d = 0; d < I->a; d++) off += P->data_rank[d];
            memcpy(t->dims, P->data_dims + off, sizeof(int64_t) * (size_t)t->rank);
            t->size = prod_dims(t->rank, t->dims);
            t->data = (cplx*)(P->data + 2 * P->data_off[I->a]);
            t->borrowed = 1;
            break;
        }
        case QXG_OP_VIEW:
            rc = view_slice(&T[I->dst], &T[I->a], I->pos, vval[I->b]);
            break;
        case QXG_OP_OUTPUT:
            rc = output_vector(&T[I->dst], bits[I->a], I->b);
            break;
        case QXG_OP_NCON: {
            if (I->na != T[I->a].rank || I->nb != T[I->b].rank || I->nc > QXO_MAX_RANK) { rc = -1; break; }
            const int32_t* l = P->labels + I->label_off;
            rc = ncon_general(&T[I->dst], l, I->nc, &T[I->a], l + I->nc, I->na, &T[I->b], l + I->nc + I->na, I->nb);
            break;
        }
        case QXG_OP_SAVE: {
            const otensor* r = &T[I->a];
            if (r->size != out_size) { rc = -1; break; }
            memcpy(out, r->data, sizeof(cplx) * (size_t)out_size);
            break;
        }
        default: rc = -1;
        }
        /* free tensors whose last read was this instruction */
        if (rc == 0) {
            for (int t = 0; t < P->ntensors; t++)
                if (P->last_use[t] == n && T[t].data && !T[t].borrowed) { free(T[t].data); T[t].data = NULL; }
        }
    }
    for (int t = 0; t < P->ntensors; t++) if (T[t].data && !T[t].borrowed) free(T[t].data);
    free(T);
    return rc;
}

/*
 * Run the programme for nbits bitstrings over slices [slice_begin, slice_end).
 * data: all leaves concatenated (interleaved complex, column-major); data_off[i] = complex
 * offset of leaf i.  out: nbits * out_size complex values.  nthreads <= 0: OpenMP default.
 * Returns 0, or -1 (invalid programme), -2 (out of memory).
 */
int qxo_run(const qxg_instr* ins, int nins, const int32_t* labels,
            const int32_t* data_rank, const int64_t* data_dims, const int64_t* data_off,
            const double* data, int ndata, int nqubits,
            const char* bitstrings, int nbits, int64_t slice_begin, int64_t slice_end,
            int nthreads, double* out, int64_t out_size) {
    oprog P;
    memset(&P, 0, sizeof(P));
    P.ins = ins; P.nins = nins; P.labels = labels; P.data_rank = data_rank; P.data_dims = data_dims;
    P.data_off = data_off; P.data = data; P.ndata = ndata; P.nqubits = nqubits;
    P.save_tensor = -1;
    for (int n = 0; n < nins; n++) {
        const qxg_instr* I = &ins[n];
        if (I->op != QXG_OP_SAVE && I->dst + 1 > P.ntensors) P.ntensors = I->dst + 1;
        if (I->op == QXG_OP_VIEW) {
            if (I->b < 0 || I->b >= QXO_MAX_RANK) return -1;
            if (I->b + 1 > P.nvars) P.nvars = I->b + 1;
            P.vdim[I->b] = I->dim;
        }
        if (I->op == QXG_OP_LOAD && (I->a < 0 || I->a >= ndata)) return -1;
        if (I->op == QXG_OP_OUTPUT && (I->a < 0 || I->a >= nqubits)) return -1;
        if (I->op == QXG_OP_SAVE) P.save_tensor = I->a;
    }
    if (P.save_tensor < 0) return -1;
    for (int j = 0; j < P.nvars; j++) if (P.vdim[j] <= 0) return -1;
    int64_t nslices = 1;
    for (int j = 0; j < P.nvars; j++) nslices *= P.vdim[j];
    if (slice_begin < 0 || slice_end > nslices || slice_begin > slice_end) return -1;
    P.last_use = (int*)malloc(sizeof(int) * (size_t)(P.ntensors > 0 ? P.ntensors : 1));
    for (int t = 0; t < P.ntensors; t++) P.last_use[t] = -1;
    for (int n = 0; n < nins; n++) {
        const qxg_instr* I = &ins[n];
        if (I->op == QXG_OP_VIEW) P.last_use[I->a] = n;
        if (I->op == QXG_OP_NCON) { P.last_use[I->a] = n; P.last_use[I->b] = n; }
        if (I->op == QXG_OP_SAVE) P.last_use[I->a] = n;
    }
    int64_t nsl = slice_end - slice_begin;
    int64_t njobs = (int64_t)nbits * nsl;
    cplx* partial = (cplx*)malloc(sizeof(cplx) * (size_t)(njobs > 0 ? njobs : 1) * (size_t)out_size);
    if (!partial) { free(P.last_use); return -2; }
    int err = 0;
    int nthr = 1;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
    nthr = omp_get_max_threads();
#endif
    const int outer = njobs >= nthr;
    qxo_inner_parallel = !outer;
#ifdef _OPENMP
    #pragma omp parallel for schedule(dynamic, 1) if (outer)
#endif
    for (int64_t j = 0; j < njobs; j++) {
        int64_t bi = j / nsl, s = slice_begin + j % nsl;
        int rc = walk(&P, bitstrings + (size_t)bi * (size_t)nqubits, s, partial + j * out_size, out_size);
        if (rc != 0) {
#ifdef _OPENMP
            #pragma omp atomic write
#endif
            err = rc;
        }
    }
    if (err == 0) {
        /* sum over slices in slice order */
        for (int64_t bi = 0; bi < nbits; bi++)
            for (int64_t e = 0; e < out_size; e++) {
                double re = 0.0, im = 0.0;
                for (int64_t s = 0; s < nsl; s++) {
                    re += partial[(bi * nsl + s) * out_size + e].re;
                    im += partial[(bi * nsl + s) * out_size + e].im;
                }
                out[2 * (bi * out_size + e)] = re;
                out[2 * (bi * out_size + e) + 1] = im;
            }
    }
    free(partial);
    free(P.last_use);
    return err;
}

/*
 * CPU-baseline sample: one walk of the programme for bitstring 0 and slice `slice`, all host
 * threads inside the contractions, stopped at the first instruction boundary after
 * `max_seconds`.  Returns 0 (finished) or 1 (stopped at the deadline); *flops receives the
 * FLOPs of the completed contractions (8 |C| K each), *seconds the elapsed time.
 */
int qxo_run_timed(const qxg_instr* ins, int nins, const int32_t* labels,
                  const int32_t* data_rank, const int64_t* data_dims, const int64_t* data_off,
                  const double* data, int ndata, int nqubits, const char* bitstring, int64_t slice,
                  int nthreads, double max_seconds, double* out, int64_t out_size,
                  double* flops, double* seconds) {
    const double t0 = qxo_now();
    qxo_deadline = t0 + max_seconds;
    qxo_flops_done = 0.0;
    const int rc = qxo_run(ins, nins, labels, data_rank, data_dims, data_off, data, ndata, nqubits,
                           bitstring, 1, slice, slice + 1, nthreads, out, out_size);
    *seconds = qxo_now() - t0;
    *flops = qxo_flops_done;
    qxo_deadline = 0.0;
    return rc == 1 ? 1 : (rc == 0 ? 0 : rc);
}

/* Max threads OpenMP would use (for reporting the CPU baseline's core count). */
int qxo_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/*
 * Permute-copy for the BLAS walk (blas_walk.py), the step TensorOperations performs with
 * Strided.jl's threaded permutedims before each GEMM: dst is written contiguously, last axis
 * fastest (numpy's C order), dims[0..rank-1]; element i of dst reads src at sum_k idx_k *
 * strides[k] (complex elements, not bytes).
 * Cache blocking, as blocked tensor transposes do: the last dst axes (up to QXO_TILE elements,
 * contiguous in dst) and the smallest-stride src axes among the others (up to QXO_TILE elements,
 * near-contiguous in src) form a tile that stays in L1 while it is read along src and written
 * along dst.  The remaining axes enumerate the tiles, which are spread over the OpenMP threads.
 * Returns 0, -1 for a rank outside 0..QXO_MAX_RANK, or -2 when the offset tables cannot be allocated.
 */
#define QXO_TILE 32
int qxo_permute_copy(const double* src, double* dst, int rank, const int64_t* dims,
                     const int64_t* strides) {
    if (rank < 0 || rank > QXO_MAX_RANK) return -1;
    const cplx* s = (const cplx*)src;
    cplx* d = (cplx*)dst;
    if (rank == 0) { d[0] = s[0]; return 0; }
    const int64_t total = prod_dims(rank, dims);
    if (total <= 0) return 0;
    int64_t dstr[QXO_MAX_RANK];            /* dst strides of the C-order layout */
    { int64_t st = 1; for (int k = rank - 1; k >= 0; k--) { dstr[k] = st; st *= dims[k]; } }
    /* D: trailing dst axes; S: smallest-stride src axes among the rest; O: the others */
    char role[QXO_MAX_RANK];               /* 'D', 'S' or 'O' */
    int64_t PD = 1, PS = 1;
    for (int k = 0; k < rank; k++) role[k] = 'O';
    for (int k = rank - 1; k >= 0 && PD * dims[k] <= QXO_TILE; k--) { role[k] = 'D'; PD *= dims[k]; }
    if (PD == 1) { role[rank - 1] = 'D'; PD = dims[rank - 1]; }   /* a long last axis is a tile row */
    for (;;) {
        int best = -1;
        for (int k = 0; k < rank; k++)
            if (role[k] == 'O' && PS * dims[k] <= QXO_TILE && (best < 0 || strides[k] < strides[best])) best = k;
        if (best < 0) break;
        role[best] = 'S'; PS *= dims[best];
    }
    int od[QXO_MAX_RANK], no = 0, sd[QXO_MAX_RANK], ns = 0, dd[QXO_MAX_RANK], nd = 0;
    for (int k = 0; k < rank; k++) {
        if (role[k] == 'O') od[no++] = k;
        else if (role[k] == 'S') sd[ns++] = k;
        else dd[nd++] = k;
    }
    /* offsets of the tile's S combinations (src and dst) and D combinations (src; dst is 0..PD-1) */
    int64_t* sofS = (int64_t*)malloc(sizeof(int64_t) * (size_t)(2 * PS + PD));
    if (!sofS) return -2;
    int64_t* dofS = sofS + PS;
    int64_t* sofD = dofS + PS;
    for (int64_t i = 0; i < PS; i++) {
        int64_t rem = i, so = 0, doff = 0;
        for (int j = ns - 1; j >= 0; j--) { const int k = sd[j]; const int64_t x = rem % dims[k]; rem /= dims[k]; so += x * strides[k]; doff += x * dstr[k]; }
        sofS[i] = so; dofS[i] = doff;
    }
    for (int64_t i = 0; i < PD; i++) {
        int64_t rem = i, so = 0;
        for (int j = nd - 1; j >= 0; j--) { const int k = dd[j]; so += (rem % dims[k]) * strides[k]; rem /= dims[k]; }
        sofD[i] = so;
    }
    const int64_t ntiles = total / (PS * PD);
#ifdef _OPENMP
    #pragma omp parallel for schedule(static) if (ntiles >= 64)
#endif
    for (int64_t t = 0; t < ntiles; t++) {
        int64_t rem = t, sb = 0, db = 0;
        for (int j = no - 1; j >= 0; j--) { const int k = od[j]; const int64_t x = rem % dims[k]; rem /= dims[k]; sb += x * strides[k]; db += x * dstr[k]; }
        for (int64_t i = 0; i < PS; i++) {
            const cplx* p = s + sb + sofS[i];
            cplx* o = d + db + dofS[i];
            for (int64_t j = 0; j < PD; j++) o[j] = p[sofD[j]];
        }
    }
    free(sofS);
    return 0;
}
