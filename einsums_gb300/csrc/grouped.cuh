// Grouped (batched) execution plans and the tile autotuner.
#pragma once

#include <string>
#include <vector>

#include "common.cuh"

namespace eg::autotune {
// "<mode>|<ceil log2 M>|<ceil log2 N>|<ceil log2 K>" -- items in one bucket share a tuned choice.
std::string bucket_key(const char *mode, int64_t M, int64_t N, int64_t K);
// Cached choice for this device and library build; false when absent.
bool lookup(const std::string &bucket, int *choice);
void store(const std::string &bucket, int choice);
// Autotuning runs unless EINSUMS_GB300_AUTOTUNE=0.
bool enabled();
// Path of the cache file (EINSUMS_GB300_AUTOTUNE_CACHE, else ~/.cache/einsums_gb300/autotune.txt).
std::string cache_path();
} // namespace eg::autotune

namespace eg::grouped {
// A captured grouped launch: the graph, the device buffers it reads (owned), and
// what it reports.
struct Plan {
    int device = 0;
    int precision = EG_PRECISION_FP64;
    int slices = 0;
    int64_t count = 0;
    int32_t algorithm = 0;
    std::vector<void *> owned; // device buffers owned by the plan
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    uint64_t kernels = 0; // kernels in one replay
    eg_split_report report{};
    // per-role cycle counters of the tensor kernel, summed over replays (EINSUMS_GB300_TC_PROFILE)
    unsigned long long *prof = nullptr;
    ~Plan();
};
eg_status build_f64_plan(Plan &plan, const std::vector<Contraction> &cs, cudaStream_t s);
eg_status build_split_plan(Plan &plan, const std::vector<Contraction> &cs, int slices, cudaStream_t s);
eg_status choose_f64_tiles(const std::vector<Contraction> &cs, cudaStream_t s, std::vector<int> &tiles);
} // namespace eg::grouped
