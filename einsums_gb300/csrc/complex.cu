// Complex128 einsum with conjugation: eg_einsum_complex.
//
// The reference instantiates its einsum for std::complex<double> tensors and
// conjugates A or B through the ConjA / ConjB template flags
// (Backends/Dispatch.hpp:48,136; the generic loops of BaseAlgebra.hpp:33-38
// apply them per element), lowering to zgemm / zgemv / zdot.  Here a complex
// tensor is the pair of FP64 views of its interleaved storage -- the real parts
// at stride 2 s and the imaginary parts one double further on -- and the
// complex contraction is the real contractions of those views that make it up
// (with a = -1 for a conjugated A, b likewise):
//
//   Re(AB) = sum Ar Br - a b Ai Bi        Im(AB) = b sum Ar Bi + a sum Ai Br
//
// each one an eg_einsum through the same dispatch, so every algorithm choice
// and both precisions (FP64 and split-BF16) serve complex operands.  A real
// C_prefactor rides on the first contraction into each part, keeping the real
// path's zeroing rules; a complex one is applied first by k_complex_scale.
#include "common.cuh"

namespace eg {
eg_status einsum_impl(double cp, const int32_t *Cl, const eg_tensor *C, double ab, const int32_t *Al,
                      const eg_tensor *A, const int32_t *Bl, const eg_tensor *B, const eg_options *opt_in,
                      cudaStream_t stream, int32_t *alg_out);
eg_status classify_call(const int32_t *Cl, const eg_tensor *C, const int32_t *Al, const eg_tensor *A,
                        const int32_t *Bl, const eg_tensor *B, const eg_options *opt_in, int32_t *alg_out);

namespace {

__global__ void k_complex_scale(ModeGroup g, double *C, double cr, double ci) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < g.total; i += stride) {
        int64_t oa, ob, oc;
        group_offsets(g, i, oa, ob, oc);
        double *c = C + 2 * oc;
        const double re = c[0], im = c[1];
        c[0] = cr * re - ci * im;
        c[1] = cr * im + ci * re;
    }
}

// The real (part 0) or imaginary (part 1) FP64 view of a complex tensor.
eg_tensor part_view(const eg_tensor &t, int part) {
    eg_tensor v = t;
    v.data = t.data ? t.data + part : nullptr;
    for (int d = 0; d < t.rank && d < EG_MAX_RANK; d++) v.stride[d] = 2 * t.stride[d];
    return v;
}

} // namespace

} // namespace eg

extern "C" eg_status eg_einsum_complex(const double *C_prefactor, const int32_t *C_labels, const eg_tensor *C,
                                       const double *AB_prefactor, const int32_t *A_labels, const eg_tensor *A,
                                       const int32_t *B_labels, const eg_tensor *B, int32_t conj_A, int32_t conj_B,
                                       const eg_options *opt, void *stream, int32_t *algorithm_choice) {
    using namespace eg;
    set_error("");
    if (!C_prefactor || !AB_prefactor) return fail(EG_ERROR_INVALID_ARGUMENT, "eg_einsum_complex: NULL prefactor");
    if (!C || !A || !B) return fail(EG_ERROR_INVALID_ARGUMENT, "eg_einsum_complex: NULL tensor");
    if (C->rank < 0 || C->rank > EG_MAX_RANK) return fail(EG_ERROR_RANK, "eg_einsum_complex: C rank out of range");
    cudaStream_t s = (cudaStream_t)stream;
    // the choice the reference reports for these complex tensors (their own strides)
    int32_t alg_c = 0;
    eg_status st0 = classify_call(C_labels, C, A_labels, A, B_labels, B, opt, &alg_c);
    if (st0 != EG_SUCCESS) return st0;
    if (algorithm_choice) *algorithm_choice = alg_c;
    const double cpr = C_prefactor[0], cpi = C_prefactor[1], abr = AB_prefactor[0], abi = AB_prefactor[1];
    const double sa = conj_A ? -1.0 : 1.0, sb = conj_B ? -1.0 : 1.0;
    double cp0 = cpr; // the prefactor of each part's first contraction
    if (cpi != 0.0) {
        ModeGroup g;
        g.n = C->rank;
        g.total = 1;
        for (int d = 0; d < C->rank; d++) {
            if (C->extent[d] < 0 || C->stride[d] < 0)
                return fail(EG_ERROR_DIMENSION, "eg_einsum_complex: negative extent or stride in C");
            g.ext[d] = C->extent[d];
            g.s[2][d] = C->stride[d];
            g.total *= C->extent[d];
        }
        if (g.total > 0) {
            if (!C->data) return fail(EG_ERROR_INVALID_ARGUMENT, "eg_einsum_complex: C data is NULL");
            const int64_t blocks = (g.total + 255) / 256;
            {
                LaunchScope ls_("k_complex_scale", s);
                k_complex_scale<<<(unsigned)(blocks < num_sms() * 8 ? blocks : num_sms() * 8), 256, 0, s>>>(
                    g, C->data, cpr, cpi);
            }
            EG_CHECK_LAUNCH("k_complex_scale");
        }
        cp0 = 1.0;
    }
    const eg_tensor Cr = part_view(*C, 0), Ci = part_view(*C, 1);
    const eg_tensor Ar = part_view(*A, 0), Ai = part_view(*A, 1);
    const eg_tensor Br = part_view(*B, 0), Bi = part_view(*B, 1);
    // (destination, A part, B part, coefficient): Re gets abr Pr - abi Pi, Im gets abr Pi + abi Pr
    struct Term {
        const eg_tensor *c, *a, *b;
        double coef;
    };
    const Term terms[8] = {
        {&Cr, &Ar, &Br, abr},           {&Cr, &Ai, &Bi, -abr * sa * sb}, {&Cr, &Ar, &Bi, -abi * sb},
        {&Cr, &Ai, &Br, -abi * sa},     {&Ci, &Ar, &Bi, abr * sb},       {&Ci, &Ai, &Br, abr * sa},
        {&Ci, &Ar, &Br, abi},           {&Ci, &Ai, &Bi, -abi * sa * sb},
    };
    bool first[2] = {true, true};
    for (const Term &t : terms) {
        const int part = t.c == &Cr ? 0 : 1;
        if (t.coef == 0.0 && !first[part]) continue;
        int32_t alg = 0;
        const eg_status st = einsum_impl(first[part] ? cp0 : 1.0, C_labels, t.c, t.coef, A_labels, t.a, B_labels, t.b,
                                         opt, s, &alg);
        if (st != EG_SUCCESS) return st;
        first[part] = false;
    }
    return EG_SUCCESS;
}
