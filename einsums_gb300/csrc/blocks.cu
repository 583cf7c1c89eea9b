// Block-sparse einsum (C ABI): eg_einsum_blocks.
//
// The reference contracts block-diagonal and tiled tensors by looping over
// block (or tile) combinations and calling einsum once per combination, under
// a lock on the output tile (Backends/BlockAlgebra.hpp:21-50,
// Backends/TileAlgebra.hpp:21-97).  Here the caller lists the combinations as
// items (C block, A block, B block); items may name the same C block, whose
// contributions then add in item order.  Every distinct C block is scaled by
// C_prefactor once (zeroed when it is 0, as the tiled dispatch does), and the
// items run in waves: wave w holds the w-th item of every C block, so no two
// items of a wave write the same block and the wave runs as one grouped
// launch (eg_einsum_batched, cached per wave signature and replayed as a
// CUDA graph); items that cannot share a launch run one by one inside it.
#include <cstring>
#include <map>
#include <tuple>
#include <vector>

#include "common.cuh"

namespace {

eg_status check_block(const eg_tensor &t, const int32_t *labels) {
    if (t.rank < 0 || t.rank > EG_MAX_RANK) return eg::fail(EG_ERROR_RANK, "eg_einsum_blocks: C block rank out of range");
    if (t.rank > 0 && !labels) return eg::fail(EG_ERROR_INVALID_ARGUMENT, "eg_einsum_blocks: C labels are NULL");
    for (int d = 0; d < t.rank; d++)
        if (t.extent[d] < 0 || t.stride[d] < 0)
            return eg::fail(EG_ERROR_DIMENSION, "eg_einsum_blocks: negative extent or stride in a C block");
    return EG_SUCCESS;
}

// Identity of a C block: the view itself (pointer, extents and strides).
struct ViewKey {
    const double *data;
    int32_t rank;
    int64_t ext[EG_MAX_RANK];
    int64_t str[EG_MAX_RANK];
    bool operator<(const ViewKey &o) const {
        if (data != o.data) return data < o.data;
        if (rank != o.rank) return rank < o.rank;
        int c = std::memcmp(ext, o.ext, sizeof ext);
        if (c) return c < 0;
        return std::memcmp(str, o.str, sizeof str) < 0;
    }
};

ViewKey key_of(const eg_tensor &t) {
    ViewKey k{};
    k.data = t.data;
    k.rank = t.rank;
    for (int d = 0; d < t.rank && d < EG_MAX_RANK; d++) {
        k.ext[d] = t.extent[d];
        k.str[d] = t.stride[d];
    }
    return k;
}

} // namespace

extern "C" eg_status eg_einsum_blocks(double C_prefactor, const int32_t *C_labels, const eg_tensor *C_list,
                                      double AB_prefactor, const int32_t *A_labels, const eg_tensor *A_list,
                                      const int32_t *B_labels, const eg_tensor *B_list, int64_t count,
                                      const eg_options *opt, void *stream, int32_t *algorithm_choice) {
    using namespace eg;
    set_error("");
    if (count < 0) return fail(EG_ERROR_INVALID_ARGUMENT, "eg_einsum_blocks: negative count");
    if (count == 0) return EG_SUCCESS;
    if (!C_list || !A_list || !B_list) return fail(EG_ERROR_INVALID_ARGUMENT, "eg_einsum_blocks: NULL list");
    cudaStream_t s = (cudaStream_t)stream;
    eg_status st;
    // waves: the w-th item naming a C block goes to wave w
    std::map<ViewKey, int> seen;
    std::vector<std::vector<int64_t>> waves;
    std::vector<int64_t> firsts;
    for (int64_t i = 0; i < count; i++) {
        if ((st = check_block(C_list[i], C_labels)) != EG_SUCCESS) return st;
        auto it = seen.find(key_of(C_list[i]));
        int w = 0;
        if (it == seen.end()) {
            seen.emplace(key_of(C_list[i]), 1);
            firsts.push_back(i);
        } else {
            w = it->second++;
        }
        if ((int)waves.size() <= w) waves.resize(w + 1);
        waves[w].push_back(i);
    }
    // C = C_prefactor * C once per distinct block
    if (C_prefactor != 1.0) {
        for (int64_t i : firsts) {
            const eg_tensor &c = C_list[i];
            ModeGroup g;
            g.n = c.rank;
            g.total = 1;
            for (int d = 0; d < c.rank; d++) {
                g.ext[d] = c.extent[d];
                g.s[2][d] = c.stride[d];
                g.total *= c.extent[d];
            }
            if (g.total == 0 || !c.data) continue;
            if ((st = launch_scale(g, c.data, C_prefactor, s)) != EG_SUCCESS) return st;
        }
    }
    std::vector<eg_tensor> Cw, Aw, Bw;
    for (size_t w = 0; w < waves.size(); w++) {
        Cw.clear();
        Aw.clear();
        Bw.clear();
        for (int64_t i : waves[w]) {
            Cw.push_back(C_list[i]);
            Aw.push_back(A_list[i]);
            Bw.push_back(B_list[i]);
        }
        int32_t alg = 0;
        st = eg_einsum_batched(1.0, C_labels, Cw.data(), AB_prefactor, A_labels, Aw.data(), B_labels, Bw.data(),
                               (int64_t)Cw.size(), opt, stream, &alg);
        if (st != EG_SUCCESS) return st;
        if (w == 0 && algorithm_choice) *algorithm_choice = alg;
    }
    return EG_SUCCESS;
}
