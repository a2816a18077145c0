// Runs qxg_plan_contraction on a network read from a text file, for a sanitizer build of the
// planner (host code).  File: "V E", E log2 dimensions, E open flags, V batched flags, then per
// tensor "k l1 .. lk".  Arguments: file trials greedy_trials seed max_log2 num_sliced batch_log2.
// Prints the stats and checks the plan: every node consumed exactly once, ids in range.
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <string>
#include <vector>

#include "qxgpu.h"

static thread_local std::string g_err;
namespace qxg {
int ncon_fail(int code, const char* msg) {
    g_err = msg;
    return code;
}
}  // namespace qxg

int main(int argc, char** argv) {
    if (argc < 8) return 2;
    std::ifstream f(argv[1]);
    int V, E;
    f >> V >> E;
    std::vector<int32_t> w(E), labels;
    std::vector<uint8_t> open(E), batched(V);
    for (auto& x : w) f >> x;
    for (auto& x : open) {
        int t;
        f >> t;
        x = (uint8_t)t;
    }
    for (auto& x : batched) {
        int t;
        f >> t;
        x = (uint8_t)t;
    }
    std::vector<int64_t> off{0};
    for (int v = 0; v < V; v++) {
        int k;
        f >> k;
        for (int i = 0; i < k; i++) {
            int l;
            f >> l;
            labels.push_back(l);
        }
        off.push_back((int64_t)labels.size());
    }
    qxg_plan_options o{};
    o.trials = std::atoi(argv[2]);
    o.greedy_trials = std::atoi(argv[3]);
    o.seed = std::atoll(argv[4]);
    o.max_log2 = std::atof(argv[5]);
    o.num_sliced = std::atoi(argv[6]);
    o.batch_log2 = std::atof(argv[7]);
    o.tensor_batched = batched.data();
    std::vector<int32_t> pairs(2 * (V - 1) + 2);
    std::vector<uint8_t> sliced(E + 1);
    qxg_plan_stats st{};
    const int rc = qxg_plan_contraction(V, off.data(), labels.data(), E, w.data(), open.data(), &o, pairs.data(),
                                        sliced.data(), &st);
    if (rc) {
        std::printf("error %d: %s\n", rc, g_err.c_str());
        return 1;
    }
    std::vector<int> used(2 * V - 1, 0);
    for (int k = 0; k < V - 1; k++)
        for (int s = 0; s < 2; s++) {
            const int x = pairs[2 * k + s];
            if (x < 0 || x >= V + k || used[x]++) {
                std::printf("bad plan at step %d\n", k);
                return 1;
            }
        }
    std::printf("log2_flops %.4f max_log2 %.1f log2_slices %.1f sliced %d trees %d ok\n", st.log2_flops, st.max_log2,
                st.log2_slices, st.num_sliced, st.trees_tried);
    return 0;
}
