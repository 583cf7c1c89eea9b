// List einsum and grouped plans (C ABI).  A plan lowers every item once,
// builds the device work lists, and captures the batch as a CUDA graph;
// eg_grouped_plan_execute replays it.  eg_einsum_batched keeps a small cache
// of plans keyed by a hash of the call (pattern, prefactors, options, and
// every item's pointers, extents and strides), so a repeated call replays.
#include <cstdio>
#include <cstring>
#include <list>
#include <map>
#include <memory>
#include <mutex>
#include <vector>

#include "grouped.cuh"

namespace eg {
eg_status einsum_impl(double cp, const int32_t *Cl, const eg_tensor *C, double ab, const int32_t *Al, const eg_tensor *A,
                      const int32_t *Bl, const eg_tensor *B, const eg_options *opt_in, cudaStream_t stream,
                      int32_t *alg_out);
eg_status lower_for_group(double cp, const int32_t *Cl, const eg_tensor *C, double ab, const int32_t *Al,
                          const eg_tensor *A, const int32_t *Bl, const eg_tensor *B, const eg_options &opt,
                          Contraction &out, int32_t *alg_out, bool &gemm_shaped);
void set_split_report(const eg_split_report &r);
void count_launches(uint64_t n);
} // namespace eg

struct eg_grouped_plan {
    std::unique_ptr<eg::grouped::Plan> plan;
};


namespace {

using eg::grouped::Plan;

uint64_t fnv(uint64_t h, const void *p, size_t n) {
    const unsigned char *c = (const unsigned char *)p;
    for (size_t i = 0; i < n; i++) {
        h ^= c[i];
        h *= 0x100000001B3ull;
    }
    return h;
}

// Never destroyed: cached plans outlive static destruction at exit (their
// device memory goes with the process).
std::mutex &g_cache_mu = *new std::mutex;
auto &g_cache = *new std::list<std::pair<uint64_t, std::shared_ptr<Plan>>>; // most recent first
constexpr size_t kCacheSize = 8;

struct StreamForCapture {
    cudaStream_t s = nullptr;
    bool owned = false;
    explicit StreamForCapture(cudaStream_t user) {
        if (user) {
            s = user;
        } else if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) == cudaSuccess) {
            owned = true;
        }
    }
    ~StreamForCapture() {
        if (owned) {
            cudaStreamSynchronize(s);
            cudaStreamDestroy(s);
        }
    }
};

eg_status create_plan(double cp, const int32_t *Cl, const eg_tensor *Cs, double ab, const int32_t *Al,
                      const eg_tensor *As, const int32_t *Bl, const eg_tensor *Bs, int64_t count,
                      const eg_options &opt, cudaStream_t stream, std::unique_ptr<Plan> &out, bool &groupable) {
    std::vector<eg::Contraction> cs;
    cs.reserve((size_t)count);
    groupable = true;
    int32_t alg0 = 0;
    for (int64_t i = 0; i < count; i++) {
        eg::Contraction c;
        int32_t alg = 0;
        bool g = false;
        eg_status st = eg::lower_for_group(cp, Cl, &Cs[i], ab, Al, &As[i], Bl, &Bs[i], opt, c, &alg, g);
        if (st != EG_SUCCESS) return st;
        if (i == 0) alg0 = alg;
        groupable &= g;
        cs.push_back(c);
    }
    if (!groupable) return EG_SUCCESS;
    auto plan = std::make_unique<Plan>();
    cudaGetDevice(&plan->device);
    plan->precision = opt.precision;
    plan->slices = opt.slices;
    plan->count = count;
    plan->algorithm = alg0;
    StreamForCapture cap(stream);
    if (!cap.s) return eg::fail(EG_ERROR_CUDA, "could not create a capture stream");
    eg_status st;
    if (opt.precision == EG_PRECISION_SPLIT_BF16) {
        st = eg::grouped::build_split_plan(*plan, cs, opt.slices, cap.s);
        if (st == EG_ERROR_NOT_SUPPORTED) {
            groupable = false; // items needing several exact passes run one by one
            return EG_SUCCESS;
        }
    } else {
        st = eg::grouped::build_f64_plan(*plan, cs, cap.s);
    }
    if (st != EG_SUCCESS) return st;
    out = std::move(plan);
    return EG_SUCCESS;
}

eg_status run_plan(Plan &plan, cudaStream_t stream) {
    cudaError_t err = cudaGraphLaunch(plan.exec, stream);
    if (err != cudaSuccess) return eg::cuda_fail(err, "cudaGraphLaunch");
    eg::count_launches(plan.kernels);
    if (plan.precision == EG_PRECISION_SPLIT_BF16) eg::set_split_report(plan.report);
    return EG_SUCCESS;
}

} // namespace

namespace eg::grouped {
Plan::~Plan() {
    if (prof) {
        // tracing aid (EINSUMS_GB300_TC_PROFILE): the tensor kernel's per-role cycles over all replays
        std::vector<unsigned long long> h((size_t)num_sms() * 8);
        if (cudaMemcpy(h.data(), prof, h.size() * 8, cudaMemcpyDeviceToHost) == cudaSuccess) {
            double tot[8] = {0};
            int ran = 0;
            for (size_t i = 0; i < h.size(); i++) tot[i % 8] += (double)h[i];
            for (size_t i = 6; i < h.size(); i += 8) ran += h[i] > 0 ? 1 : 0;
            if (tot[6] > 0)
                std::fprintf(stderr,
                             "[tc profile grouped] items=%lld: total %.3g cyc/CTA | producer wait empty %.1f%% | mma wait "
                             "full %.1f%% | mma wait acc %.1f%% | epi wait acc %.1f%% | epi flush %.1f%% | epi final "
                             "%.1f%%\n",
                             (long long)count, tot[6] / (ran > 0 ? ran : 1), 100 * tot[0] / tot[6], 100 * tot[1] / tot[6],
                             100 * tot[2] / tot[6], 100 * tot[3] / tot[6], 100 * tot[4] / tot[6], 100 * tot[5] / tot[6]);
        }
    }
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    for (void *p : owned) tracked_free(p);
}
} // namespace eg::grouped

extern "C" {

eg_status eg_grouped_plan_create(double C_prefactor, const int32_t *C_labels, const eg_tensor *C_list,
                                 double AB_prefactor, const int32_t *A_labels, const eg_tensor *A_list,
                                 const int32_t *B_labels, const eg_tensor *B_list, int64_t count,
                                 const eg_options *opt_in, void *stream, eg_grouped_plan **plan,
                                 int32_t *algorithm_choice) {
    eg::set_error("");
    if (!plan) return eg::fail(EG_ERROR_INVALID_ARGUMENT, "plan is NULL");
    *plan = nullptr;
    if (count <= 0 || !C_list || !A_list || !B_list) return eg::fail(EG_ERROR_INVALID_ARGUMENT, "empty or NULL list");
    eg_options opt;
    eg_options_default(&opt);
    if (opt_in) opt = *opt_in;
    try {
        std::unique_ptr<Plan> p;
        bool groupable = false;
        eg_status st = create_plan(C_prefactor, C_labels, C_list, AB_prefactor, A_labels, A_list, B_labels, B_list,
                                   count, opt, (cudaStream_t)stream, p, groupable);
        if (st != EG_SUCCESS) return st;
        if (!groupable || !p)
            return eg::fail(EG_ERROR_NOT_SUPPORTED,
                            "grouped plan: every item must be a contraction over summed indices with a non-scalar, "
                            "non-diagonal output (and, for the split form, fit one exact pass)");
        if (algorithm_choice) *algorithm_choice = p->algorithm;
        *plan = new eg_grouped_plan{std::move(p)};
        return EG_SUCCESS;
    } catch (const std::exception &e) {
        return eg::fail(EG_ERROR_OUT_OF_MEMORY, e.what());
    }
}

eg_status eg_grouped_plan_execute(eg_grouped_plan *plan, void *stream) {
    eg::set_error("");
    if (!plan || !plan->plan) return eg::fail(EG_ERROR_INVALID_ARGUMENT, "plan is NULL");
    return run_plan(*plan->plan, (cudaStream_t)stream);
}

eg_status eg_grouped_plan_destroy(eg_grouped_plan *plan) {
    if (!plan) return EG_SUCCESS;
    if (plan->plan) {
        cudaSetDevice(plan->plan->device);
        cudaDeviceSynchronize();
    }
    delete plan;
    return EG_SUCCESS;
}

eg_status eg_einsum_batched(double C_prefactor, const int32_t *C_labels, const eg_tensor *C_list, double AB_prefactor,
                            const int32_t *A_labels, const eg_tensor *A_list, const int32_t *B_labels,
                            const eg_tensor *B_list, int64_t count, const eg_options *opt_in, void *stream,
                            int32_t *algorithm_choice) {
    eg::set_error("");
    if (count < 0) return eg::fail(EG_ERROR_INVALID_ARGUMENT, "negative count");
    if (count == 0) return EG_SUCCESS; // the reference returns before dispatching an empty list
    if (!C_list || !A_list || !B_list) return eg::fail(EG_ERROR_INVALID_ARGUMENT, "NULL list");
    eg_options opt;
    eg_options_default(&opt);
    if (opt_in) opt = *opt_in;

    // key: everything that defines the captured graph
    uint64_t h = 0xcbf29ce484222325ull;
    h = fnv(h, &C_prefactor, sizeof C_prefactor);
    h = fnv(h, &AB_prefactor, sizeof AB_prefactor);
    h = fnv(h, &opt, sizeof opt);
    h = fnv(h, &count, sizeof count);
    if (C_list[0].rank > 0) h = fnv(h, C_labels, sizeof(int32_t) * C_list[0].rank);
    if (A_list[0].rank > 0) h = fnv(h, A_labels, sizeof(int32_t) * A_list[0].rank);
    if (B_list[0].rank > 0) h = fnv(h, B_labels, sizeof(int32_t) * B_list[0].rank);
    h = fnv(h, C_list, sizeof(eg_tensor) * count);
    h = fnv(h, A_list, sizeof(eg_tensor) * count);
    h = fnv(h, B_list, sizeof(eg_tensor) * count);
    int dev = 0;
    cudaGetDevice(&dev);
    h = fnv(h, &dev, sizeof dev);

    std::shared_ptr<Plan> plan;
    {
        std::lock_guard<std::mutex> lk(g_cache_mu);
        for (auto it = g_cache.begin(); it != g_cache.end(); ++it)
            if (it->first == h) {
                plan = it->second;
                g_cache.splice(g_cache.begin(), g_cache, it);
                break;
            }
    }
    if (!plan) {
        std::unique_ptr<Plan> p;
        bool groupable = false;
        eg_status st;
        try {
            st = create_plan(C_prefactor, C_labels, C_list, AB_prefactor, A_labels, A_list, B_labels, B_list, count,
                             opt, (cudaStream_t)stream, p, groupable);
        } catch (const std::exception &e) {
            return eg::fail(EG_ERROR_OUT_OF_MEMORY, e.what());
        }
        if (st != EG_SUCCESS) return st;
        if (!groupable || !p) {
            // items that cannot share a launch run one by one
            for (int64_t i = 0; i < count; i++) {
                int32_t alg = 0;
                st = eg::einsum_impl(C_prefactor, C_labels, &C_list[i], AB_prefactor, A_labels, &A_list[i], B_labels,
                                     &B_list[i], &opt, (cudaStream_t)stream, &alg);
                if (st != EG_SUCCESS) return st;
                if (i == 0 && algorithm_choice) *algorithm_choice = alg;
            }
            return EG_SUCCESS;
        }
        plan = std::shared_ptr<Plan>(std::move(p));
        std::lock_guard<std::mutex> lk(g_cache_mu);
        g_cache.emplace_front(h, plan);
        while (g_cache.size() > kCacheSize) g_cache.pop_back();
    }
    if (algorithm_choice) *algorithm_choice = plan->algorithm;
    return run_plan(*plan, (cudaStream_t)stream);
}

} // extern "C"
