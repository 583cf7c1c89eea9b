// C ABI of einsums_gb300: argument checking, algorithm reporting, lowering of
// an arbitrary (C, A, B) index pattern to the canonical batched contraction,
// and dispatch to the kernels.  No exception crosses this file's entry points.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "../../include/einsums_gb300/classify.hpp"
#include "common.cuh"

namespace eg {

namespace detail = ::einsums_gb300::detail;

namespace {
thread_local std::string g_last_error;
thread_local eg_split_report g_split_report = {0, 0, 0, 0.0};

// Library-wide registries are allocated once and never destroyed, so objects
// released during static destruction at process exit (cached plans, workspaces)
// never touch an already-destroyed container.
std::mutex &g_mem_mutex = *new std::mutex;
size_t g_budget = 0; // 0 = unlimited
size_t g_in_use = 0;
std::map<void *, size_t> &g_sizes = *new std::map<void *, size_t>;

struct WsKey {
    int dev;
    cudaStream_t stream;
    bool operator<(const WsKey &o) const { return dev != o.dev ? dev < o.dev : stream < o.stream; }
};
struct WsBuf {
    void *ptr = nullptr;
    size_t bytes = 0;
};
std::mutex &g_ws_mutex = *new std::mutex;
std::map<WsKey, WsBuf> &g_ws = *new std::map<WsKey, WsBuf>;
} // namespace

void set_error(const std::string &msg) { g_last_error = msg; }

eg_status fail(eg_status st, const std::string &msg) {
    g_last_error = msg;
    return st;
}

eg_status cuda_fail(cudaError_t err, const char *what) {
    g_last_error = std::string(what) + ": " + cudaGetErrorName(err) + " (" + cudaGetErrorString(err) + ")";
    return err == cudaErrorMemoryAllocation ? EG_ERROR_OUT_OF_MEMORY : EG_ERROR_CUDA;
}

eg_status tracked_malloc(size_t bytes, void **ptr) {
    std::lock_guard<std::mutex> lk(g_mem_mutex);
    if (g_budget && g_in_use + bytes > g_budget)
        return fail(EG_ERROR_OUT_OF_MEMORY, "device allocation of " + std::to_string(bytes) +
                                                " bytes exceeds the memory budget of " + std::to_string(g_budget));
    void *p = nullptr;
    cudaError_t err = cudaMalloc(&p, bytes ? bytes : 1);
    if (err != cudaSuccess) return cuda_fail(err, "cudaMalloc");
    g_sizes[p] = bytes;
    g_in_use += bytes;
    *ptr = p;
    return EG_SUCCESS;
}

eg_status tracked_free(void *ptr) {
    if (!ptr) return EG_SUCCESS;
    {
        std::lock_guard<std::mutex> lk(g_mem_mutex);
        auto it = g_sizes.find(ptr);
        if (it == g_sizes.end()) return fail(EG_ERROR_INVALID_ARGUMENT, "eg_device_free: pointer not from eg_device_alloc");
        g_in_use -= it->second;
        g_sizes.erase(it);
    }
    EG_CUDA(cudaFree(ptr));
    return EG_SUCCESS;
}

eg_status workspace(cudaStream_t stream, size_t bytes, void **ptr) {
    int dev = 0;
    EG_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(g_ws_mutex);
    WsBuf &b = g_ws[WsKey{dev, stream}];
    if (b.bytes < bytes) {
        if (b.ptr) {
            // Earlier work on this stream may still read the old buffer.
            EG_CUDA(cudaStreamSynchronize(stream));
            eg_status st = tracked_free(b.ptr);
            b.ptr = nullptr;
            b.bytes = 0;
            if (st != EG_SUCCESS) return st;
        }
        size_t want = std::max(bytes, b.bytes * 2);
        want = (want + 0xFFFFF) & ~size_t(0xFFFFF);
        eg_status st = tracked_malloc(want, &b.ptr);
        if (st != EG_SUCCESS) {
            b.ptr = nullptr;
            return st;
        }
        b.bytes = want;
    }
    *ptr = b.ptr;
    return EG_SUCCESS;
}

void set_split_report(const eg_split_report &r) { g_split_report = r; }

namespace {
std::mutex &g_status_mutex = *new std::mutex;
std::map<WsKey, int *> &g_status = *new std::map<WsKey, int *>;
} // namespace

// One status word per (device, stream), allocated on first use.  A stream that
// is being captured into a CUDA graph cannot allocate: it gets its own word if
// one exists, else the device's shared word for captured launches (created with
// the first word of the device, outside any capture).
eg_status status_word(cudaStream_t stream, int **ptr) {
    int dev = 0;
    EG_CUDA(cudaGetDevice(&dev));
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    EG_CUDA(cudaStreamIsCapturing(stream, &cap));
    std::lock_guard<std::mutex> lk(g_status_mutex);
    const WsKey shared_key{dev, reinterpret_cast<cudaStream_t>(~uintptr_t(0))};
    auto found = g_status.find(WsKey{dev, stream});
    if (found != g_status.end() && found->second) {
        *ptr = found->second;
        return EG_SUCCESS;
    }
    if (cap != cudaStreamCaptureStatusNone) {
        auto sh = g_status.find(shared_key);
        if (sh == g_status.end() || !sh->second)
            return fail(EG_ERROR_NOT_SUPPORTED, "first call of the library on this device is under stream capture");
        *ptr = sh->second;
        return EG_SUCCESS;
    }
    for (const WsKey &key : {shared_key, WsKey{dev, stream}}) {
        int *&w = g_status[key];
        if (!w) {
            EG_CUDA(cudaMalloc(&w, 256));
            EG_CUDA(cudaMemset(w, 0, 256));
        }
    }
    *ptr = g_status[WsKey{dev, stream}];
    return EG_SUCCESS;
}

namespace {

using detail::Algorithm;
using detail::Labels;
using detail::View;

eg_status check_tensor(const eg_tensor *t, const int32_t *labels, const char *name) {
    if (!t) return fail(EG_ERROR_INVALID_ARGUMENT, std::string(name) + " is NULL");
    if (t->rank < 0 || t->rank > EG_MAX_RANK)
        return fail(EG_ERROR_RANK, std::string(name) + " has rank " + std::to_string(t->rank) + " (max 8)");
    if (t->rank > 0 && !labels) return fail(EG_ERROR_INVALID_ARGUMENT, std::string(name) + " labels are NULL");
    int64_t n = 1;
    for (int i = 0; i < t->rank; i++) {
        if (t->extent[i] < 0) return fail(EG_ERROR_DIMENSION, std::string(name) + " has a negative extent");
        if (t->stride[i] < 0) return fail(EG_ERROR_NOT_SUPPORTED, std::string(name) + " has a negative stride");
        n *= t->extent[i];
    }
    if (n > 0 && !t->data) return fail(EG_ERROR_INVALID_ARGUMENT, std::string(name) + " data is NULL");
    return EG_SUCCESS;
}

View view_of(const eg_tensor *t) {
    View v;
    v.rank = t->rank;
    for (int i = 0; i < t->rank; i++) {
        v.extent[i] = t->extent[i];
        v.stride[i] = t->stride[i];
    }
    return v;
}

Labels labels_of(const int32_t *l, int n) {
    Labels x;
    for (int i = 0; i < n; i++) x.push(l[i]);
    return x;
}

struct Mode {
    int64_t ext;
    int64_t s[3];
};

// Sort by the given operand's stride (descending) and merge neighbours that
// are contiguous in all three operands.
ModeGroup fold(std::vector<Mode> modes, int primary) {
    std::stable_sort(modes.begin(), modes.end(), [&](const Mode &a, const Mode &b) {
        if (a.s[primary] != b.s[primary]) return a.s[primary] > b.s[primary];
        for (int t = 0; t < 3; t++)
            if (a.s[t] != b.s[t]) return a.s[t] > b.s[t];
        return false;
    });
    std::vector<Mode> out;
    for (const Mode &m : modes) {
        if (m.ext == 1) continue; // extent-1 modes contribute nothing
        if (!out.empty()) {
            Mode &p = out.back();
            bool merge = true;
            for (int t = 0; t < 3; t++)
                if (p.s[t] != m.s[t] * m.ext) merge = false;
            if (merge) {
                p.ext *= m.ext;
                for (int t = 0; t < 3; t++) p.s[t] = m.s[t];
                continue;
            }
        }
        out.push_back(m);
    }
    ModeGroup g;
    g.n = (int)out.size();
    g.total = 1;
    for (int d = 0; d < g.n; d++) {
        g.ext[d] = out[d].ext;
        for (int t = 0; t < 3; t++) g.s[t][d] = out[d].s[t];
        g.total *= out[d].ext;
    }
    return g;
}

struct Lowered {
    Contraction c;
    bool empty_c = false;
};

eg_status lower(const int32_t *Cl, const eg_tensor *C, const int32_t *Al, const eg_tensor *A, const int32_t *Bl,
                const eg_tensor *B, int semantics, Lowered &out) {
    struct U {
        int32_t label;
        int64_t ext = -1;
        int64_t s[3] = {0, 0, 0};
        bool in[3] = {false, false, false};
    };
    std::vector<U> us;
    auto add = [&](const int32_t *labels, const eg_tensor *t, int which, const char *name) -> eg_status {
        for (int i = 0; i < t->rank; i++) {
            auto it = std::find_if(us.begin(), us.end(), [&](const U &u) { return u.label == labels[i]; });
            if (it == us.end()) {
                us.push_back(U{labels[i]});
                it = us.end() - 1;
            }
            if (it->ext >= 0 && it->ext != t->extent[i])
                return fail(EG_ERROR_DIMENSION, std::string("index ") + std::to_string(labels[i]) + " of " + name +
                                                    " has extent " + std::to_string(t->extent[i]) + " but " +
                                                    std::to_string(it->ext) + " elsewhere");
            it->ext = t->extent[i];
            it->s[which] += t->stride[i]; // repeated labels walk the diagonal (get_stride_for sums them)
            it->in[which] = true;
        }
        return EG_SUCCESS;
    };
    eg_status st;
    if ((st = add(Cl, C, 2, "C")) != EG_SUCCESS) return st;
    if ((st = add(Al, A, 0, "A")) != EG_SUCCESS) return st;
    if ((st = add(Bl, B, 1, "B")) != EG_SUCCESS) return st;

    std::vector<Mode> batch, m, n, k;
    int64_t c_elems = 1;
    for (const U &u : us) {
        Mode md{u.ext, {u.s[0], u.s[1], u.s[2]}};
        if (u.in[2]) c_elems *= u.ext;
        if (u.in[2] && u.in[0] && u.in[1])
            batch.push_back(md);
        else if (u.in[2] && u.in[1] && !u.in[0])
            n.push_back(md);
        else if (u.in[2])
            m.push_back(md); // in A only, or C-only broadcast (A stride 0)
        else if (u.in[0] && u.in[1])
            k.push_back(md);
        else if (semantics == EG_SEMANTICS_PYTHON)
            k.push_back(md); // operand-only index: summed over the unique-index space
        // else: C++ semantics hold an operand-only index at 0
    }
    // Repeated C labels address the diagonal only; the number of C positions
    // written is the product over unique labels, as in the reference loops.
    out.c = Contraction{};
    out.c.batch = fold(batch, 2);
    out.c.m = fold(m, 0);
    out.c.n = fold(n, 1);
    out.c.k = fold(k, 0);
    out.c.A = A->data;
    out.c.B = B->data;
    out.c.C = C->data;
    out.c.c_elems = c_elems;
    out.empty_c = (c_elems == 0);
    return EG_SUCCESS;
}

eg_status classify_labels(const int32_t *Cl, int cr, const int32_t *Al, int ar, const int32_t *Bl, int br, int semantics,
                          Algorithm &alg) {
    Labels C = labels_of(Cl, cr), A = labels_of(Al, ar), B = labels_of(Bl, br);
    alg = semantics == EG_SEMANTICS_PYTHON ? detail::classify_py(C, A, B) : detail::classify_cpp(C, A, B);
    return EG_SUCCESS;
}

} // namespace

// The algorithm the reference reports for a call (classification and stride
// vetoes), without running it.
eg_status classify_call(const int32_t *Cl, const eg_tensor *C, const int32_t *Al, const eg_tensor *A,
                        const int32_t *Bl, const eg_tensor *B, const eg_options *opt_in, int32_t *alg_out) {
    eg_options opt;
    eg_options_default(&opt);
    if (opt_in) opt = *opt_in;
    eg_status st;
    if ((st = check_tensor(C, Cl, "C")) != EG_SUCCESS) return st;
    if ((st = check_tensor(A, Al, "A")) != EG_SUCCESS) return st;
    if ((st = check_tensor(B, Bl, "B")) != EG_SUCCESS) return st;
    Algorithm alg;
    classify_labels(Cl, C->rank, Al, A->rank, Bl, B->rank, opt.semantics, alg);
    if (opt.only_generic) alg = Algorithm::GENERIC;
    if (opt.semantics == EG_SEMANTICS_CPP)
        alg = detail::apply_vetoes(alg, labels_of(Cl, C->rank), view_of(C), labels_of(Al, A->rank), view_of(A),
                                   labels_of(Bl, B->rank), view_of(B));
    *alg_out = (int32_t)alg;
    return EG_SUCCESS;
}

eg_status einsum_impl(double cp, const int32_t *Cl, const eg_tensor *C, double ab, const int32_t *Al, const eg_tensor *A,
                      const int32_t *Bl, const eg_tensor *B, const eg_options *opt_in, cudaStream_t stream,
                      int32_t *alg_out) {
    eg_options opt;
    eg_options_default(&opt);
    if (opt_in) opt = *opt_in;
    if (opt.semantics != EG_SEMANTICS_CPP && opt.semantics != EG_SEMANTICS_PYTHON)
        return fail(EG_ERROR_INVALID_ARGUMENT, "unknown semantics");
    if (opt.precision != EG_PRECISION_FP64 && opt.precision != EG_PRECISION_SPLIT_BF16)
        return fail(EG_ERROR_INVALID_ARGUMENT, "unknown precision");
    eg_status st;
    if ((st = check_tensor(C, Cl, "C")) != EG_SUCCESS) return st;
    if ((st = check_tensor(A, Al, "A")) != EG_SUCCESS) return st;
    if ((st = check_tensor(B, Bl, "B")) != EG_SUCCESS) return st;

    Algorithm alg;
    classify_labels(Cl, C->rank, Al, A->rank, Bl, B->rank, opt.semantics, alg);
    if (opt.only_generic) alg = Algorithm::GENERIC;
    if (opt.semantics == EG_SEMANTICS_CPP)
        alg = detail::apply_vetoes(alg, labels_of(Cl, C->rank), view_of(C), labels_of(Al, A->rank), view_of(A),
                                   labels_of(Bl, B->rank), view_of(B));
    if (alg_out) *alg_out = (int32_t)alg;

    Lowered low;
    if ((st = lower(Cl, C, Al, A, Bl, B, opt.semantics, low)) != EG_SUCCESS) return st;
    if (low.empty_c) return EG_SUCCESS;
    Contraction &c = low.c;
    c.cp = cp;
    c.ab = ab;
    // The C++ DOT and GER paths multiply C by C_prefactor instead of zeroing it
    // (Dispatch.hpp:907, :343-346), so a NaN in C survives C_prefactor == 0 there.
    c.zero_when_cp_zero = !(opt.semantics == EG_SEMANTICS_CPP && (alg == Algorithm::DOT || alg == Algorithm::GER));

    // A repeated C label addresses only C's diagonal; the prefactor still
    // applies to all of C first (BaseAlgebra.hpp:129-133, PyTensorAlgebra.hpp:541-563).
    bool c_repeats = false;
    for (int i = 0; i < C->rank; i++)
        for (int j = i + 1; j < C->rank; j++) c_repeats |= Cl[i] == Cl[j];
    if (c_repeats && !(c.cp == 1.0)) {
        ModeGroup cg;
        for (int i = 0; i < C->rank; i++) {
            cg.ext[cg.n] = C->extent[i];
            cg.s[2][cg.n] = C->stride[i];
            cg.total *= C->extent[i];
            cg.n++;
        }
        if ((st = launch_scale(cg, C->data, c.cp, stream)) != EG_SUCCESS) return st;
        c.cp = 1.0;
        c.zero_when_cp_zero = false;
    }

    const bool has_k = c.k.n > 0 || c.k.total == 0;
    // The split form pays for splitting both operands (each read twice, S BF16
    // planes written) and pads M and N to 128-row tiles.  When M or N is at most
    // kSplitMinMN (GEMV-shaped products) the FP64 kernels are faster as well as
    // exact to FP64, so they run instead and the split report shows 0 slices.
    constexpr int64_t kSplitMinMN = 4;
    if (opt.precision == EG_PRECISION_SPLIT_BF16 && c.k.total > 0 && c.m.total > kSplitMinMN &&
        c.n.total > kSplitMinMN) {
        eg_split_report rep{};
        st = launch_split_contract(c, opt.slices, stream, &rep);
        if (st == EG_SUCCESS) set_split_report(rep);
        return st;
    }
    set_split_report(eg_split_report{0, 0, 0, 0.0});
    if (!has_k) return launch_elementwise(c, stream);
    if (c.batch.n == 0 && c.m.n == 0 && c.n.n == 0) return launch_dot(c, stream);
    if (c.m.n == 0 || c.n.n == 0) return launch_gemv(c, stream);
    return launch_contract_f64(c, stream);
}

// Validates, classifies and lowers one item of a batch; gemm_shaped tells
// whether it can join a grouped launch (summed modes, an output with more
// than one position, no repeated output index).
eg_status lower_for_group(double cp, const int32_t *Cl, const eg_tensor *C, double ab, const int32_t *Al,
                          const eg_tensor *A, const int32_t *Bl, const eg_tensor *B, const eg_options &opt,
                          Contraction &out, int32_t *alg_out, bool &gemm_shaped) {
    eg_status st;
    if ((st = check_tensor(C, Cl, "C")) != EG_SUCCESS) return st;
    if ((st = check_tensor(A, Al, "A")) != EG_SUCCESS) return st;
    if ((st = check_tensor(B, Bl, "B")) != EG_SUCCESS) return st;
    Algorithm alg;
    classify_labels(Cl, C->rank, Al, A->rank, Bl, B->rank, opt.semantics, alg);
    if (opt.only_generic) alg = Algorithm::GENERIC;
    if (opt.semantics == EG_SEMANTICS_CPP)
        alg = detail::apply_vetoes(alg, labels_of(Cl, C->rank), view_of(C), labels_of(Al, A->rank), view_of(A),
                                   labels_of(Bl, B->rank), view_of(B));
    if (alg_out) *alg_out = (int32_t)alg;
    Lowered low;
    if ((st = lower(Cl, C, Al, A, Bl, B, opt.semantics, low)) != EG_SUCCESS) return st;
    out = low.c;
    out.cp = cp;
    out.ab = ab;
    out.zero_when_cp_zero = !(opt.semantics == EG_SEMANTICS_CPP && (alg == Algorithm::DOT || alg == Algorithm::GER));
    bool c_repeats = false;
    for (int i = 0; i < C->rank; i++)
        for (int j = i + 1; j < C->rank; j++) c_repeats |= Cl[i] == Cl[j];
    gemm_shaped = !low.empty_c && !c_repeats && out.k.n > 0 && out.k.total > 0 &&
                  (out.m.n > 0 || out.n.n > 0 || out.batch.n > 0);
    return EG_SUCCESS;
}

eg_status build_permute_desc(double cp, const int32_t *Cl, const eg_tensor *C, double ap, const int32_t *Al,
                             const eg_tensor *A, PermuteDesc &p) {
    eg_status st;
    if ((st = check_tensor(C, Cl, "C")) != EG_SUCCESS) return st;
    if ((st = check_tensor(A, Al, "A")) != EG_SUCCESS) return st;
    if (C->rank != A->rank) return fail(EG_ERROR_RANK, "permute: C and A ranks differ");
    p = PermuteDesc{};
    p.rank = C->rank;
    p.A = A->data;
    p.C = C->data;
    p.cp = cp;
    p.ap = ap;
    for (int d = 0; d < C->rank; d++) {
        int where = -1, count = 0;
        for (int j = 0; j < A->rank; j++)
            if (Al[j] == Cl[d]) {
                where = j;
                count++;
            }
        if (count != 1) return fail(EG_ERROR_INVALID_ARGUMENT, "permute: every C index must occur exactly once in A");
        if (C->extent[d] < A->extent[where])
            return fail(EG_ERROR_DIMENSION, "permute: dimension " + std::to_string(d) +
                                                " of the output tensor is smaller than the input tensor");
        p.ext[d] = A->extent[where];
        p.sA[d] = A->stride[where];
        p.sC[d] = C->stride[d];
    }
    for (int j = 0; j < A->rank; j++) {
        int count = 0;
        for (int d = 0; d < C->rank; d++) count += (Cl[d] == Al[j]);
        if (count != 1) return fail(EG_ERROR_INVALID_ARGUMENT, "permute: every A index must occur exactly once in C");
    }
    return EG_SUCCESS;
}

eg_status permute_impl(double cp, const int32_t *Cl, const eg_tensor *C, double ap, const int32_t *Al,
                       const eg_tensor *A, cudaStream_t stream) {
    PermuteDesc p;
    const eg_status st = build_permute_desc(cp, Cl, C, ap, Al, A, p);
    if (st != EG_SUCCESS) return st;
    return launch_permute(p, stream);
}

} // namespace eg

extern "C" {

void eg_options_default(eg_options *opt) {
    if (!opt) return;
    opt->precision = EG_PRECISION_FP64;
    opt->slices = 0;
    opt->tolerance = 1e-10;
    opt->semantics = EG_SEMANTICS_CPP;
    opt->only_generic = 0;
}

eg_status eg_einsum(double C_prefactor, const int32_t *C_labels, const eg_tensor *C, double AB_prefactor,
                    const int32_t *A_labels, const eg_tensor *A, const int32_t *B_labels, const eg_tensor *B,
                    const eg_options *opt, void *stream, int32_t *algorithm_choice) {
    eg::set_error("");
    try {
        return eg::einsum_impl(C_prefactor, C_labels, C, AB_prefactor, A_labels, A, B_labels, B, opt,
                               (cudaStream_t)stream, algorithm_choice);
    } catch (const std::exception &e) {
        return eg::fail(EG_ERROR_INVALID_ARGUMENT, e.what());
    } catch (...) {
        return eg::fail(EG_ERROR_INVALID_ARGUMENT, "unknown exception");
    }
}

eg_status eg_classify(int32_t C_rank, const int32_t *C_labels, int32_t A_rank, const int32_t *A_labels, int32_t B_rank,
                      const int32_t *B_labels, int32_t semantics, int32_t *algorithm_choice) {
    eg::set_error("");
    if (!algorithm_choice) return eg::fail(EG_ERROR_INVALID_ARGUMENT, "algorithm_choice is NULL");
    for (int32_t r : {C_rank, A_rank, B_rank})
        if (r < 0 || r > EG_MAX_RANK) return eg::fail(EG_ERROR_RANK, "rank out of range");
    if ((C_rank && !C_labels) || (A_rank && !A_labels) || (B_rank && !B_labels))
        return eg::fail(EG_ERROR_INVALID_ARGUMENT, "labels are NULL");
    eg::detail::Algorithm alg;
    eg::classify_labels(C_labels, C_rank, A_labels, A_rank, B_labels, B_rank, semantics, alg);
    *algorithm_choice = (int32_t)alg;
    return EG_SUCCESS;
}

eg_status eg_permute(double C_prefactor, const int32_t *C_labels, const eg_tensor *C, double A_prefactor,
                     const int32_t *A_labels, const eg_tensor *A, void *stream) {
    eg::set_error("");
    try {
        return eg::permute_impl(C_prefactor, C_labels, C, A_prefactor, A_labels, A, (cudaStream_t)stream);
    } catch (...) {
        return eg::fail(EG_ERROR_INVALID_ARGUMENT, "exception in eg_permute");
    }
}

eg_status eg_einsum_batched(double C_prefactor, const int32_t *C_labels, const eg_tensor *C_list, double AB_prefactor,
                            const int32_t *A_labels, const eg_tensor *A_list, const int32_t *B_labels,
                            const eg_tensor *B_list, int64_t count, const eg_options *opt, void *stream,
                            int32_t *algorithm_choice);

eg_status eg_last_split_report(eg_split_report *out) {
    if (!out) return eg::fail(EG_ERROR_INVALID_ARGUMENT, "out is NULL");
    *out = eg::g_split_report;
    return EG_SUCCESS;
}

eg_status eg_device_alloc(size_t bytes, void **ptr) {
    eg::set_error("");
    if (!ptr) return eg::fail(EG_ERROR_INVALID_ARGUMENT, "ptr is NULL");
    return eg::tracked_malloc(bytes, ptr);
}

eg_status eg_device_free(void *ptr) {
    eg::set_error("");
    return eg::tracked_free(ptr);
}

eg_status eg_set_memory_budget(size_t bytes) {
    std::lock_guard<std::mutex> lk(eg::g_mem_mutex);
    eg::g_budget = bytes;
    return EG_SUCCESS;
}

eg_status eg_memory_in_use(size_t *bytes) {
    if (!bytes) return eg::fail(EG_ERROR_INVALID_ARGUMENT, "bytes is NULL");
    std::lock_guard<std::mutex> lk(eg::g_mem_mutex);
    *bytes = eg::g_in_use;
    return EG_SUCCESS;
}

eg_status eg_copy_to_device(void *dst, const void *src, size_t bytes, void *stream) {
    EG_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, (cudaStream_t)stream));
    return EG_SUCCESS;
}

eg_status eg_copy_to_host(void *dst, const void *src, size_t bytes, void *stream) {
    EG_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, (cudaStream_t)stream));
    return EG_SUCCESS;
}

eg_status eg_stream_synchronize(void *stream) {
    EG_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
    return EG_SUCCESS;
}

eg_status eg_stream_status(void *stream, int32_t *device_code) {
    eg::set_error("");
    int *w = nullptr;
    eg_status st = eg::status_word((cudaStream_t)stream, &w);
    if (st != EG_SUCCESS) return st;
    EG_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
    int code = 0;
    EG_CUDA(cudaMemcpy(&code, w, sizeof(int), cudaMemcpyDeviceToHost));
    if (code) EG_CUDA(cudaMemset(w, 0, sizeof(int)));
    if (device_code) *device_code = code;
    if (code) return eg::fail(EG_ERROR_TIMEOUT, "a bounded device wait gave up (code " + std::to_string(code) + ")");
    return EG_SUCCESS;
}

const char *eg_last_error(void) { return eg::g_last_error.c_str(); }

const char *eg_status_string(eg_status s) {
    switch (s) {
    case EG_SUCCESS: return "success";
    case EG_ERROR_INVALID_ARGUMENT: return "invalid argument";
    case EG_ERROR_RANK: return "rank error";
    case EG_ERROR_DIMENSION: return "dimension error";
    case EG_ERROR_NOT_SUPPORTED: return "not supported";
    case EG_ERROR_CUDA: return "CUDA error";
    case EG_ERROR_OUT_OF_MEMORY: return "out of memory";
    case EG_ERROR_TIMEOUT: return "device wait timed out";
    case EG_ERROR_PRECISION: return "precision target not reachable";
    }
    return "unknown status";
}

const char *eg_version(void) { return "einsums_gb300 0.1.0 (sm_103a)"; }

} // extern "C"
