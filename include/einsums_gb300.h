/*
 * einsums_gb300 -- C ABI of the GB300 tensor-contraction library.
 *
 * Plain pointers and sizes only; no C++ or torch types cross this boundary.
 * Every entry point returns an eg_status and never throws.  Tensors live in
 * device memory owned by the caller; the library owns only its scratch
 * workspace.  All work is ordered on the CUDA stream passed as `stream`
 * (a cudaStream_t; NULL means the legacy default stream) and no entry point
 * synchronises the host unless it is documented to return a host value.
 *
 * Each entry point names the reference interface it replaces (paths relative
 * to the Einsums project root).
 */
#ifndef EINSUMS_GB300_H
#define EINSUMS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define EG_MAX_RANK 8

typedef enum eg_status {
    EG_SUCCESS = 0,
    EG_ERROR_INVALID_ARGUMENT = 1, /* null pointer, bad option value */
    EG_ERROR_RANK = 2,             /* rank_error: index count differs from tensor rank, or rank > EG_MAX_RANK */
    EG_ERROR_DIMENSION = 3,        /* dimension_error: one index with two extents */
    EG_ERROR_NOT_SUPPORTED = 4,    /* pattern or layout the kernels do not handle */
    EG_ERROR_CUDA = 5,             /* a CUDA runtime call failed (eg_last_error has the text) */
    EG_ERROR_OUT_OF_MEMORY = 6,    /* scratch allocation failed or exceeded the workspace budget */
    EG_ERROR_TIMEOUT = 7,          /* a bounded device-side wait gave up; the context stays usable */
    EG_ERROR_PRECISION = 8         /* split form cannot meet the requested tolerance */
} eg_status;

/* Same enumerators, same order as einsums::tensor_algebra::detail::AlgorithmChoice
 * (libs/Einsums/TensorAlgebra/include/Einsums/TensorAlgebra/Detail/Utilities.hpp:26-34). */
typedef enum eg_algorithm {
    EG_ALGO_GENERIC = 0,
    EG_ALGO_DOT = 1,
    EG_ALGO_DIRECT = 2,
    EG_ALGO_GER = 3,
    EG_ALGO_GEMV = 4,
    EG_ALGO_GEMM = 5,
    EG_ALGO_INDETERMINATE = 6
} eg_algorithm;

typedef enum eg_precision {
    EG_PRECISION_FP64 = 0,      /* plain FP64 kernels */
    EG_PRECISION_SPLIT_BF16 = 1 /* FP64 operands split into exponent-scaled BF16 slices on tcgen05; products
                                 * whose M or N extent is at most 4 (GEMV and DOT shapes) run the FP64
                                 * kernels instead, which are faster for them, and report 0 slices */
} eg_precision;

typedef enum eg_semantics {
    /* C++ einsum: an index found in only one operand and not in C is held at 0
     * (Backends/BaseAlgebra.hpp:85-139); the DOT choice scales C by C_prefactor
     * even when it is 0 (Backends/Dispatch.hpp:903-909). */
    EG_SEMANTICS_CPP = 0,
    /* EinsumsPy plans: every index of the unique-index space is summed and C is
     * zeroed when C_prefactor == 0 (EinsumsPy/TensorAlgebra/PyTensorAlgebra.hpp:520-605). */
    EG_SEMANTICS_PYTHON = 1
} eg_semantics;

/* A strided FP64 view of device memory; strides are in elements. */
typedef struct eg_tensor {
    double *data;
    int32_t rank;
    int64_t extent[EG_MAX_RANK];
    int64_t stride[EG_MAX_RANK];
} eg_tensor;

typedef struct eg_options {
    int32_t precision;    /* eg_precision */
    int32_t slices;       /* split form: BF16 slices per operand, 2..6; 0 = chosen from `tolerance` */
    double tolerance;     /* split form: target relative Frobenius error (default 1e-10) */
    int32_t semantics;    /* eg_semantics */
    int32_t only_generic; /* report and run as the generic algorithm (OnlyUseGenericAlgorithm) */
} eg_options;

/* Fills *opt with FP64 precision, automatic slices, tolerance 1e-10, C++ semantics. */
void eg_options_default(eg_options *opt);

/*
 * C = C_prefactor * C + AB_prefactor * sum_links A * B
 *
 * Replaces einsums::tensor_algebra::einsum(C_prefactor, Indices{...}, &C, AB_prefactor,
 * Indices{...}, A, Indices{...}, B, &algorithm_choice)
 * (libs/Einsums/TensorAlgebra/include/Einsums/TensorAlgebra/TensorAlgebra.hpp:41-50,
 *  implementation Backends/Dispatch.hpp:960-1262) for DeviceTensor operands, and the
 * GPU branch of the EinsumsPy plans' execute
 * (libs/EinsumsPy/TensorAlgebra/src/PyTensorAlgebra.cpp:609-1049).
 * Labels: one int32 per mode; equal labels name the same index.  A rank-0 C is a
 * single device double.  *algorithm_choice (may be NULL) receives the algorithm the
 * reference reports for the same call.
 */
eg_status eg_einsum(double C_prefactor, const int32_t *C_labels, const eg_tensor *C, double AB_prefactor,
                    const int32_t *A_labels, const eg_tensor *A, const int32_t *B_labels, const eg_tensor *B,
                    const eg_options *opt, void *stream, int32_t *algorithm_choice);

/*
 * Complex128 einsum: C = C_prefactor * C + AB_prefactor * sum_links op(A) * op(B), where op
 * conjugates A when conj_A != 0 and B when conj_B != 0.  C, A and B point to interleaved
 * (real, imaginary) doubles; their extents and strides count complex elements.  C_prefactor and
 * AB_prefactor are (real, imaginary) pairs.  Replaces einsum<ConjA, ConjB>(...) on
 * std::complex<double> tensors (Backends/Dispatch.hpp:48,136, conjugation in the generic loops
 * of Backends/BaseAlgebra.hpp:33-38).  Runs as the real contractions of the parts' strided views
 * through eg_einsum (four when AB_prefactor is real, eight otherwise), with opt's precision; a
 * complex C_prefactor is applied to C first.  *algorithm_choice: the choice for the pattern.
 */
eg_status eg_einsum_complex(const double *C_prefactor, const int32_t *C_labels, const eg_tensor *C,
                            const double *AB_prefactor, const int32_t *A_labels, const eg_tensor *A,
                            const int32_t *B_labels, const eg_tensor *B, int32_t conj_A, int32_t conj_B,
                            const eg_options *opt, void *stream, int32_t *algorithm_choice);

/*
 * Algorithm choice of a pattern without running it (no stride vetoes).
 * Replaces the dry-run dispatch detail::einsum<false, true, ...>
 * (Backends/Dispatch.hpp:1276-1279) and compile_plan's plan-type selection
 * (EinsumsPy/TensorAlgebra/src/PyTensorAlgebra.cpp:168-554).
 */
eg_status eg_classify(int32_t C_rank, const int32_t *C_labels, int32_t A_rank, const int32_t *A_labels, int32_t B_rank,
                      const int32_t *B_labels, int32_t semantics, int32_t *algorithm_choice);

/*
 * C = C_prefactor * C + A_prefactor * A[perm]   (C zeroed first when C_prefactor == 0)
 * Replaces einsums::tensor_algebra::permute(UC_prefactor, Indices{...}, &C, UA_prefactor,
 * Indices{...}, A) (libs/Einsums/TensorAlgebra/include/Einsums/TensorAlgebra/Permute.hpp:330-407;
 * device form Backends/DevicePermute.hpp:98-209).  Bit-exact copy when A_prefactor == 1
 * and C_prefactor == 0.  EG_ERROR_DIMENSION when an extent of C is smaller than the
 * matching extent of A.
 */
eg_status eg_permute(double C_prefactor, const int32_t *C_labels, const eg_tensor *C, double A_prefactor,
                     const int32_t *A_labels, const eg_tensor *A, void *stream);

/*
 * Compiled permute: the plan fixes the index permutation, the extents and strides of C and A
 * and the prefactors (the data pointers in C and A are not kept); execute runs it on any C
 * and A of those shapes and strides -- C = C_prefactor * C + A_prefactor * A[perm], as
 * eg_permute.  Replaces compile_permute(beta, Indices{...}, &C, alpha, Indices{...}, A)
 * (libs/Einsums/TensorAlgebra/include/Einsums/TensorAlgebra/Permute.hpp:37-171), which builds
 * a reusable HPTT plan, and permute(&C, A, plan) (Permute.hpp:292-297), which rebinds the
 * plan's input and output pointers and executes it.
 */
typedef struct eg_permute_plan eg_permute_plan;
eg_status eg_permute_plan_create(double C_prefactor, const int32_t *C_labels, const eg_tensor *C, double A_prefactor,
                                 const int32_t *A_labels, const eg_tensor *A, eg_permute_plan **plan);
eg_status eg_permute_plan_execute(const eg_permute_plan *plan, double *C, const double *A, void *stream);
eg_status eg_permute_plan_destroy(eg_permute_plan *plan);

/*
 * List einsum: item i computes C[i] = C_prefactor*C[i] + AB_prefactor * A[i]*B[i] with one
 * shared index pattern.  Items may have different extents.  Lists of contractions run as a
 * grouped plan (see eg_grouped_plan_create), cached by call signature and replayed as a
 * CUDA graph; other lists run item by item.
 * Replaces the batched overload einsum(C_prefactor, Cidx, &C_list, AB_prefactor, Aidx,
 * A_list, Bidx, B_list, &algorithm_choice) (Backends/Dispatch.hpp:1264-1286) and the list
 * form of Plan.execute (EinsumsPy/TensorAlgebra/src/Export.cpp:17-27).
 */
eg_status eg_einsum_batched(double C_prefactor, const int32_t *C_labels, const eg_tensor *C_list, double AB_prefactor,
                            const int32_t *A_labels, const eg_tensor *A_list, const int32_t *B_labels,
                            const eg_tensor *B_list, int64_t count, const eg_options *opt, void *stream,
                            int32_t *algorithm_choice);

/*
 * Block-sparse einsum: item i adds AB_prefactor * A[i]*B[i] into the block C[i], one shared
 * index pattern.  Items may name the same C block (the same view: pointer, extents and
 * strides); its contributions add in item order.  Every distinct C block is first scaled by
 * C_prefactor (zeroed when it is 0).  Items run in waves -- the w-th item of every C block --
 * each wave one grouped launch as in eg_einsum_batched.  Distinct C blocks must not overlap.
 * Replaces the block and tile loops of the reference's einsum on BlockTensor / TiledTensor
 * operands (libs/Einsums/TensorAlgebra/include/Einsums/TensorAlgebra/Backends/BlockAlgebra.hpp:21-50,
 * Backends/TileAlgebra.hpp:21-97), where each combination is one einsum call under a lock on
 * its output tile.
 */
eg_status eg_einsum_blocks(double C_prefactor, const int32_t *C_labels, const eg_tensor *C_list, double AB_prefactor,
                           const int32_t *A_labels, const eg_tensor *A_list, const int32_t *B_labels,
                           const eg_tensor *B_list, int64_t count, const eg_options *opt, void *stream,
                           int32_t *algorithm_choice);

/*
 * C = C_prefactor * C + AB_prefactor * sum_i A[i] * B[i] over n contiguous doubles, without
 * allocating any device memory.  No counterpart in the reference: it is for callers that
 * cannot let a library call cudaMalloc -- applications whose device memory is owned by
 * another allocator (a framework's caching allocator or an arena reserved at start-up) and
 * latency-critical loops that must not pay for an allocation.  The partial sums live in a
 * fixed 32 KB array inside the library (4096 partials of 65536 elements each), so n is at
 * most 2^28; longer inputs return EG_ERROR_NOT_SUPPORTED.  Every call on a device shares that
 * array: calls whose kernels overlap on the GPU race.  Each call looks the array up on the
 * current device (cudaGetSymbolAddress); the first call on a device also loads the library's
 * device code there, so make it before any stream capture.  As in the reference's C++ DOT
 * choice, C is multiplied by C_prefactor even when that is 0, so a NaN in C survives.
 */
eg_status eg_dot_noalloc(double C_prefactor, double *C, double AB_prefactor, const double *A, const double *B,
                         int64_t n, void *stream);

/*
 * Fock two-electron build for integrals with 8-fold permutational symmetry:
 *   F = F_prefactor * F + J_prefactor * J + K_prefactor * K   (F not read when F_prefactor == 0)
 *   J[p,q] = sum_rs g[p,q,r,s] D[r,s],   K[p,q] = sum_rs g[p,r,q,s] D[r,s]
 * g: n^4 contiguous row-major doubles with g[p,q,r,s] = g[q,p,r,s] = g[p,q,s,r] = g[r,s,p,q];
 * D and F: n x n contiguous row-major, D symmetric.  These symmetries are the caller's
 * contract and are not checked: only the canonical eighth of g (p >= q, r >= s,
 * pair(p,q) >= pair(r,s)) is read, and D[r,s] stands for D[s,r].  opt (may be NULL): precision
 * EG_PRECISION_FP64 (default) makes all six contributions of each element in FP64;
 * EG_PRECISION_SPLIT_BF16 cuts g and D into opt->slices (3..6, 0 = 5) 8-bit digits -- the
 * digits of the split-BF16 contraction -- and sums four of the six contributions as exact
 * digit products on the FP32 pipe, the other two in FP64 (error bound as
 * eg_last_split_report states: 1.3e-11 for 5 slices).  The summation order is fixed, so the
 * results are deterministic.  Replaces the pair of einsum calls of the reference's RHF
 * Fock build, F += 2 einsum(pq <- pqrs, rs) and F -= einsum(pq <- prqs, rs)
 * (libs/Einsums/TensorAlgebra/tests/unit/QChemTests.cpp:300-303; dispatch
 * Backends/Dispatch.hpp:444-560 and Backends/BaseAlgebra.hpp:85-139): J_prefactor = 2,
 * K_prefactor = -1, F_prefactor = 1.  EG_ERROR_NOT_SUPPORTED for n above 384 (g is then
 * 174 GB).
 */
eg_status eg_fock_jk_symmetric(double F_prefactor, double *F, double J_prefactor, double K_prefactor, const double *g,
                               const double *D, int64_t n, const eg_options *opt, void *stream);

/*
 * Grouped plan: lowers every item of a list einsum once, builds a device-side work list of
 * output tiles (largest first) and captures the batch as a CUDA graph -- one persistent
 * grouped launch for FP64 (tile size per shape bucket from the autotuner's cache), or the
 * digit-splitting launches plus one persistent tcgen05 launch for the split form.
 * eg_grouped_plan_execute replays the graph on `stream`.  Items must be contractions over
 * summed indices with a non-scalar, non-diagonal output; otherwise EG_ERROR_NOT_SUPPORTED
 * (eg_einsum_batched then runs such lists item by item).  The plan keeps the tensors'
 * addresses: they must stay valid while the plan is used.  Replaces the per-item OpenMP
 * loop of the reference's list einsum (Backends/Dispatch.hpp:1264-1286) and the block loops
 * of BlockAlgebra.hpp:23-50; *algorithm_choice receives item 0's algorithm.
 */
typedef struct eg_grouped_plan eg_grouped_plan;
eg_status eg_grouped_plan_create(double C_prefactor, const int32_t *C_labels, const eg_tensor *C_list,
                                 double AB_prefactor, const int32_t *A_labels, const eg_tensor *A_list,
                                 const int32_t *B_labels, const eg_tensor *B_list, int64_t count,
                                 const eg_options *opt, void *stream, eg_grouped_plan **plan,
                                 int32_t *algorithm_choice);
eg_status eg_grouped_plan_execute(eg_grouped_plan *plan, void *stream);
/* Synchronises the plan's device and frees it. */
eg_status eg_grouped_plan_destroy(eg_grouped_plan *plan);

/* Split-form accounting for the last eg_einsum / eg_einsum_batched call on this host
 * thread: slices used per operand, BF16 slice-pair products issued, and the a-priori
 * relative error bound.  No reference counterpart (the reference has no split form). */
typedef struct eg_split_report {
    int32_t slices;
    int32_t slice_pairs;
    int32_t bits_per_slice;
    double error_bound;
} eg_split_report;
eg_status eg_last_split_report(eg_split_report *out);

/* Device storage for DeviceTensor (Tensor/include/Einsums/Tensor/Backends/DeviceTensor.hpp:246-284,
 * GPUMemory/GPUAllocator.hpp:53-190): allocate / free device memory with an optional byte
 * budget (0 = unlimited).  EG_ERROR_OUT_OF_MEMORY when the budget would be exceeded. */
eg_status eg_device_alloc(size_t bytes, void **ptr);
eg_status eg_device_free(void *ptr);
eg_status eg_set_memory_budget(size_t bytes);
eg_status eg_memory_in_use(size_t *bytes);

/* Error record of kernels with bounded device-side waits (the split form's tensor-core
 * pipeline) for work issued on `stream`: synchronises the stream, returns EG_ERROR_TIMEOUT
 * with the kernel's code in *device_code (may be NULL) when a wait gave up, and clears
 * the record.  Such a kernel returns early instead of hanging, leaving its outputs
 * incomplete; the context stays usable.  No reference counterpart (the reference's
 * kernels have no bounded waits). */
eg_status eg_stream_status(void *stream, int32_t *device_code);

/* Failure-path self-test of the bounded device waits: enqueues on `stream` a kernel that
 * allocates tensor memory, waits on a barrier nothing arrives on until `limit_ns`
 * (0 < limit_ns <= 2e9) passes, records a code for eg_stream_status, frees the tensor memory
 * and returns -- the steps the tensor-core pipeline takes when one of its waits gives up.
 * No reference counterpart. */
eg_status eg_selftest_wait_timeout(uint64_t limit_ns, void *stream);

/* Host<->device copies on `stream` (DeviceTensor::read / operator= in DeviceTensor.hpp). */
eg_status eg_copy_to_device(void *dst, const void *src, size_t bytes, void *stream);
eg_status eg_copy_to_host(void *dst, const void *src, size_t bytes, void *stream);
eg_status eg_stream_synchronize(void *stream);

/* Measures FP64 throughput of this device (TFLOP/s) with a DFMA loop and an
 * mma.sync m8n8k4 f64 (DMMA) loop (best of three runs after a warm-up run);
 * synchronises the device.  The roofline denominator of the plain FP64 form.
 * eg_measure_fp64_peak_clock also gives the SM clock (MHz) the DFMA loop ran at:
 * each block's SM cycles over its own duration (global timer), median over the
 * blocks.  No reference counterpart. */
eg_status eg_measure_fp64_peak(double *dfma_tflops, double *dmma_tflops);
eg_status eg_measure_fp64_peak_clock(double *dfma_tflops, double *dmma_tflops, double *probe_mhz);

/* *clusters receives the number of two-CTA clusters the split-BF16 tensor kernel
 * runs single contractions on (256x128 output tiles, cta_group::2 MMAs), or 0
 * when it runs one CTA per 128x128 tile.  Pairs are used when the process
 * starts with EINSUMS_GB300_TC_PAIRS=1.  No reference counterpart. */
eg_status eg_tc_pair_clusters(int32_t *clusters);

/* Kernel accounting.  eg_kernel_launches: kernels this library has launched in the
 * process.  With profiling on, every launch is bracketed by CUDA events on its own
 * stream; eg_profile_summary synchronises those events and writes one line
 * "name,launches,total_ms" per kernel into buf (NUL-terminated, truncated to cap).
 * Replaces the scoped-zone profiler of the reference
 * (libs/Einsums/Profile/include/Einsums/Profile/Profile.hpp:115-320) for the device path. */
eg_status eg_kernel_launches(uint64_t *count);
eg_status eg_profile_enable(int32_t on);
eg_status eg_profile_reset(void);
eg_status eg_profile_summary(char *buf, size_t cap);

/* Text of the last error on this host thread (empty when none). */
const char *eg_last_error(void);
const char *eg_status_string(eg_status status);
/* Library version string. */
const char *eg_version(void);

#ifdef __cplusplus
}
#endif

#endif /* EINSUMS_GB300_H */
