// Internal declarations shared by the executor's host compiler and its CUDA kernels.
//
// Every tensor dimension on the contraction path is a power of two (qubit bonds are 2,
// decomposed two-qubit bonds 2 or 4; other sizes are zero-padded up at upload), so a tensor's
// linear index is a bit string and every permute/reshape of the reference's `ncon`
// (docs/src/users_guide.md:124-146) is a bit permutation.  A permutation is stored as a few
// "runs": bits [src, src+len) of one index land at bits [dst, dst+len) of another.
#pragma once

#include <cstdint>
#include <utility>
#include <vector>
#include <cuda_runtime.h>

namespace qxg {

constexpr int kMaxRuns = 24;       // runs per bit map (a contraction rarely needs more than 8)
constexpr int kKTableBits = 8;     // K offsets tabulated in shared memory (2^8 entries)

struct Run {
    uint8_t src, len, dst, pad;
};

struct BitMap {                     // index -> offset as a sum of shifted bit fields
    int32_t n;
    Run r[kMaxRuns];
};

__host__ __device__ inline int64_t pdep(int64_t x, const BitMap& m) {
    int64_t o = 0;
    for (int i = 0; i < m.n; i++) {
        const Run q = m.r[i];
        o |= ((x >> q.src) & ((int64_t(1) << q.len) - 1)) << q.dst;
    }
    return o;
}

// Consecutive (src, dst) pairs with both sides increasing by one collapse into one run (host).
inline bool make_runs(const std::vector<std::pair<int, int>>& pairs, BitMap* m) {
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

// Per-pass parameters read by kernels from device memory, so a captured pass can be replayed
// for another (slice batch, bitstring batch) by rewriting this block.
struct PassParams {
    int64_t slice_base;        // first slice id of this pass
    int64_t num_slices;        // total slices of the programme
    int32_t bit_base;          // first bitstring of this pass (row in the bitstring buffer)
    int32_t bits_valid;        // bitstrings of this pass that are real (rest are padding)
    int32_t slices_valid;      // slices of this pass that are real
    int32_t pad;
};

// One pairwise contraction C[c] = sum_k A[a(c,k)] B[b(c,k)] over bit-indexed tensors.
struct StepArgs {
    const void* A;
    const void* B;
    void* C;
    int64_t nC;                // elements of C (a power of two)
    int32_t nk;                // summed bits
    int32_t expA, expB, expC;  // exponent slots (split / fp32 modes), -1 when unused
    int32_t conjA, conjB;      // 1: use the complex conjugate of the operand (adjoint steps)
    BitMap cA, cB;             // C index -> A / B offset
    BitMap kA, kB;             // K index -> A / B offset
};

// Adjoint seed: dL/d conj(root) for a batch, from a caller's per-bitstring seed (amp_bar) or,
// for L = sum |amplitude|^2, from the amplitudes themselves (sum of the root over the slice
// batch).  The destination is zeroed first; only real (beta, sigma) entries are written.
struct SeedArgs {
    void* dst;                 // adjoint of the root (root layout)
    const void* root;          // forward root (norm2 mode)
    const double* amp_bar;     // (nbitstrings x out_size) complex; NULL -> norm2 mode
    int64_t out_size;
    int32_t nbeta, nsigma;
    BitMap beta_map, sigma_map;
    int32_t naxes;
    int32_t axis_dim[48];
    int32_t axis_nbits[48];
    int32_t axis_bitpos[48][3];
    int32_t exp_root, exp_dst;
    const struct PassParams* params;
};

// Adjoint of a (chain of) view(s) of a leaf: S_bar[j] = sum over the slice batch of V_bar at the
// slice's value of every fixed axis (zero where no slice of the batch selects j).
struct ViewAdjArgs {
    const void* vbar;          // adjoint of the view (view layout, sigma bits on top)
    void* sbar;                // adjoint of the leaf (leaf layout)
    int64_t ns;                // leaf elements
    int32_t sigma_shift, nsigma;
    BitMap s2v;                // leaf index (non-fixed bits) -> view offset
    int32_t nfix;
    int32_t fix_shift[8], fix_bits[8];
    int64_t var_stride[8], var_dim[8];
    int32_t exp_v, exp_s;
    const struct PassParams* params;
};

// Accumulate a leaf's adjoint (padded column-major, scaled by 2^e) into its FP64 gradient.
struct LeafGradArgs {
    const void* sbar;
    double* grad;              // logical (unpadded) column-major complex doubles
    int64_t n;                 // logical elements
    int32_t rank;
    int32_t dims[16], pdims[16];
    int32_t exp_s;
    int64_t goff;              // batched launch: complex offset of this leaf in the gradient vector
};

// Materialise a view of a leaf/output tensor for a batch of slices.
constexpr int kMaxViewFix = 8;
struct ViewArgs {
    const void* src;
    void* dst;
    int64_t n;                 // elements of dst
    int32_t sigma_shift;       // dst bits >= sigma_shift are the slice batch index
    int32_t nfix;
    BitMap map;                // dst index (bits below sigma_shift) -> src offset
    int32_t fix_shift[kMaxViewFix];   // src bit position of the fixed axis' lowest bit
    int64_t var_stride[kMaxViewFix];  // slice id / var_stride % var_dim = value of the variable
    int64_t var_dim[kMaxViewFix];
    int32_t exp_src, exp_dst;
    const PassParams* params;
};

// Output (bitstring) vectors for a batch of bitstrings: dst[x + 2*beta].
struct OutputArgs {
    void* dst;
    const char* bitstrings;    // device, nbitstrings x nqubits
    int32_t qubit, nqubits, nbeta;
    int32_t exp_dst;
    const PassParams* params;
};

// Sum of the root tensor over the slice batch, added into the FP64 result.
constexpr int kMaxOutAxes = 48;
struct ReduceArgs {
    const void* root;
    double* out;               // (nbitstrings x out_size) complex doubles
    int64_t out_size;          // logical elements per bitstring
    int32_t nbeta, nsigma;     // batch sizes in the root (1 when absent)
    BitMap beta_map;           // bitstring-batch index -> root offset
    BitMap sigma_map;          // slice-batch index -> root offset
    int32_t naxes;
    int32_t axis_dim[kMaxOutAxes];        // logical (unpadded) dims of the root's axes
    int32_t axis_nbits[kMaxOutAxes];
    int32_t axis_bitpos[kMaxOutAxes][3];  // physical positions of each axis bit (<= 3 bits)
    int32_t exp_root;
    int32_t broadcast;         // 1: root has no beta; write the same value to every bitstring
    const PassParams* params;
};

// A small CUDA-core contraction inside a batch launched at once (contract_batch_kernel): its
// arguments and its blocks [first_block, first_block + nblocks) of the launch.
struct BatchStep {
    StepArgs a;
    int32_t first_block, nblocks;
};
constexpr int kBatchResults = 1024;     // results per block of a batched step
constexpr int kBatchMaxK = 64;          // summed extent of a batched step
constexpr int64_t kBatchMaxResults = int64_t(1) << 15;

// Kernel launchers (kernels_simt.cu).  Storage: double2 when fp64 != 0, else float2.
// scratch (may be null): device memory for the partials of steps with few results and a long
// sum (contract_scratch_bytes); *launches receives the kernels launched (1 or 2).
cudaError_t launch_contract(const StepArgs& a, bool fp64, int* exps, cudaStream_t s, int sm_count,
                            void* scratch = nullptr, size_t scratch_bytes = 0, int* launches = nullptr);
size_t contract_scratch_bytes(const StepArgs& a, bool fp64, int sm_count);
// Whether launch_contract multiplies with B as the first factor of each complex product (the row
// forms put the larger operand first).  The products of a complex multiply-add are summed in a
// fixed order, so swapping the factors changes the rounding: kernels that must reproduce
// launch_contract's results bit for bit follow the same order.
bool contract_x_is_b(const StepArgs& a, bool fp64);
// The CUDA-core form launch_contract picks for a step (for diagnostics).
const char* contract_form(const StepArgs& a, bool fp64, int sm_count);
// Whether a step with a long sum is better served on the CUDA cores than by a tensor-core GEMM:
// the batched small GEMM of a final join (both operands large), or the long sum of a step with few
// results (it reads every element of the operand with more result bits once and the other at most
// twice).
bool contract_prefers_cuda_cores(const StepArgs& a, bool fp64, int sm_count);
// Run n batched steps (device array, blocks numbered consecutively, nblocks in all).
cudaError_t launch_batch(const BatchStep* d_steps, int n, int nblocks, bool fp64, int* exps, cudaStream_t s);
cudaError_t launch_view(const ViewArgs& a, bool fp64, int* exps, cudaStream_t s);
cudaError_t launch_output(const OutputArgs& a, bool fp64, int* exps, cudaStream_t s);
cudaError_t launch_reduce(const ReduceArgs& a, bool fp64, const int* exps, cudaStream_t s);
cudaError_t launch_reset_exps(int* exps, int begin, int end, cudaStream_t s);
cudaError_t launch_seed(const SeedArgs& a, bool fp64, int* exps, cudaStream_t s);
cudaError_t launch_view_adjoint(const ViewAdjArgs& a, bool fp64, int* exps, cudaStream_t s);
cudaError_t launch_leaf_grad(const LeafGradArgs& a, bool fp64, const int* exps, cudaStream_t s);
// All n leaves of a device table in one launch (leaf b into grad + 2 tab[b].goff).
cudaError_t launch_leaf_grads(const LeafGradArgs* d_tab, int n, double* grad, bool fp64, const int* exps,
                              cudaStream_t s);

// Exponent slots: exps[2*i] = e (true value = stored * 2^e), exps[2*i+1] = m (max stored
// exponent, atomically raised by the producer).
constexpr int kExpUnset = -2139062144;  // 0x80808080: memset-able "minus infinity"

}  // namespace qxg
