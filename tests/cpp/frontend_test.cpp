// C++ front-end test: the reference's einsum call shape over DeviceTensors.
// Compile-time checks (static_assert) pin the pattern analysis on the
// reference's own algorithm-choice assertions; main() runs the known-answer
// tests of libs/Einsums/TensorAlgebra/tests/unit/Einsum1.cpp and Batched.cpp
// on the GPU and checks the reported AlgorithmChoice.
#include <einsums_gb300/TensorAlgebra.hpp>

#include <cmath>
#include <cstdio>
#include <vector>

using namespace einsums;
using namespace einsums::tensor_algebra;
using einsums::tensor_algebra::detail::AlgorithmChoice;
using einsums::tensor_algebra::detail::compile_time_choice;

#define PAT(...) std::tuple<__VA_ARGS__>
using namespace einsums::index;
// Einsum1.cpp:31, Einsum1.cpp:72, Einsum3.cpp:62/79, Einsum4.cpp:46/71, Einsum7.cpp:47/125, Dot.cpp:30
static_assert(compile_time_choice<PAT(struct i, struct j), PAT(struct i, struct k), PAT(struct k, struct j)>() ==
              AlgorithmChoice::GEMM);
static_assert(compile_time_choice<PAT(struct i, struct l), PAT(struct i, struct j, struct k),
                                  PAT(struct j, struct k, struct l)>() == AlgorithmChoice::GEMM);
static_assert(compile_time_choice<PAT(struct i), PAT(struct i, struct j), PAT(struct j)>() == AlgorithmChoice::GEMV);
static_assert(compile_time_choice<PAT(struct i), PAT(struct i, struct j, struct k), PAT(struct j, struct i, struct k)>() ==
              AlgorithmChoice::GENERIC);
static_assert(compile_time_choice<PAT(struct i, struct j, struct k, struct l), PAT(struct i, struct j, struct k, struct p),
                                  PAT(struct p, struct l)>() == AlgorithmChoice::GEMM);
static_assert(compile_time_choice<PAT(struct i, struct j, struct k, struct l), PAT(struct i, struct j, struct p, struct l),
                                  PAT(struct p, struct k)>() == AlgorithmChoice::GENERIC);
static_assert(compile_time_choice<PAT(struct p, struct q), PAT(struct p, struct q), PAT(struct p, struct q)>() ==
              AlgorithmChoice::DIRECT);
static_assert(compile_time_choice<PAT(struct a, struct b), PAT(struct a), PAT(struct b)>() == AlgorithmChoice::GER);
static_assert(compile_time_choice<PAT(), PAT(struct i), PAT(struct i)>() == AlgorithmChoice::DOT);
// the Fock build patterns (QChemTests.cpp:301-304)
static_assert(compile_time_choice<PAT(struct i, struct j), PAT(struct k, struct l),
                                  PAT(struct i, struct j, struct k, struct l)>() == AlgorithmChoice::GEMV);
static_assert(compile_time_choice<PAT(struct i, struct j), PAT(struct k, struct l),
                                  PAT(struct i, struct k, struct j, struct l)>() == AlgorithmChoice::GENERIC);

static int failures = 0;
#define CHECK(cond)                                                                                                    \
    do {                                                                                                               \
        if (!(cond)) {                                                                                                 \
            std::printf("FAILED: %s (line %d)\n", #cond, __LINE__);                                                    \
            failures++;                                                                                                \
        }                                                                                                              \
    } while (0)

int main() {
    AlgorithmChoice alg = AlgorithmChoice::INDETERMINATE;
    {   // Einsum1.cpp "ik=ij,jk"
        DeviceTensor<double, 2> A("A", 3, 3), B("B", 3, 3), C("C", 3, 3);
        std::vector<double> h(9);
        for (int x = 0; x < 9; x++) h[x] = x + 1;
        A.write(h);
        B.write(h);
        einsum(Indices{index::i, index::j}, &C, Indices{index::i, index::k}, A, Indices{index::k, index::j}, B, &alg);
        CHECK(alg == AlgorithmChoice::GEMM);
        const std::vector<double> want = {30, 36, 42, 66, 81, 96, 102, 126, 150};
        CHECK(C.read() == want);
    }
    {   // Einsum1.cpp "il=ijk,jkl" and Batched.cpp (10 tensors)
        std::vector<DeviceTensor<double, 3>> As, Bs;
        std::vector<DeviceTensor<double, 2>> Cs;
        std::vector<double> h(27);
        for (int x = 0; x < 27; x++) h[x] = x + 1;
        for (int t = 0; t < 10; t++) {
            As.emplace_back("A", 3, 3, 3);
            Bs.emplace_back("B", 3, 3, 3);
            Cs.emplace_back("C", 3, 3);
            As.back().write(h);
            Bs.back().write(h);
        }
        einsum(Indices{index::i, index::l}, &Cs, Indices{index::i, index::j, index::k}, As,
               Indices{index::j, index::k, index::l}, Bs, &alg);
        CHECK(alg == AlgorithmChoice::GEMM);
        const std::vector<double> want = {765, 810, 855, 1818, 1944, 2070, 2871, 3078, 3285};
        for (auto &C : Cs) CHECK(C.read() == want);
    }
    {   // dot with the C++ DOT semantics, then GEMV / GENERIC Fock patterns
        DeviceTensor<double, 1> a("a", 1000), b("b", 1000);
        std::vector<double> ha(1000), hb(1000);
        double ref = 0;
        for (int x = 0; x < 1000; x++) {
            ha[x] = std::sin(x);
            hb[x] = std::cos(0.5 * x);
            ref += ha[x] * hb[x];
        }
        a.write(ha);
        b.write(hb);
        DeviceTensor<double, 0> e("e");
        e.write({0.0});
        einsum(0.0, Indices{}, &e, 2.0, Indices{index::i}, a, Indices{index::i}, b, &alg);
        CHECK(alg == AlgorithmChoice::DOT);
        CHECK(std::fabs(e.read()[0] - 2.0 * ref) < 1e-12 * std::fabs(ref) + 1e-12);

        const int n = 6;
        DeviceTensor<double, 4> g("g", n, n, n, n);
        DeviceTensor<double, 2> D("D", n, n), F("F", n, n);
        std::vector<double> hg(n * n * n * n), hD(n * n), hF(n * n, 0.0);
        for (size_t x = 0; x < hg.size(); x++) hg[x] = std::cos(0.37 * x);
        for (size_t x = 0; x < hD.size(); x++) hD[x] = std::sin(0.11 * x);
        g.write(hg);
        D.write(hD);
        F.write(hF);
        einsum(1.0, Indices{index::i, index::j}, &F, 2.0, Indices{index::k, index::l}, D,
               Indices{index::i, index::j, index::k, index::l}, g, &alg);
        CHECK(alg == AlgorithmChoice::GEMV);
        einsum(1.0, Indices{index::i, index::j}, &F, -1.0, Indices{index::k, index::l}, D,
               Indices{index::i, index::k, index::j, index::l}, g, &alg);
        CHECK(alg == AlgorithmChoice::GENERIC);
        std::vector<double> got = F.read();
        double err = 0, nrm = 0;
        for (int i = 0; i < n; i++)
            for (int j = 0; j < n; j++) {
                double v = 0;
                for (int k = 0; k < n; k++)
                    for (int l = 0; l < n; l++)
                        v += 2.0 * hD[k * n + l] * hg[((i * n + j) * n + k) * n + l] -
                             hD[k * n + l] * hg[((i * n + k) * n + j) * n + l];
                err += (got[i * n + j] - v) * (got[i * n + j] - v);
                nrm += v * v;
            }
        CHECK(std::sqrt(err / nrm) < 1e-13);
    }
    {   // permute and the reference's dimension_error
        DeviceTensor<double, 2> A("A", 3, 4), C("C", 4, 3);
        std::vector<double> h(12);
        for (int x = 0; x < 12; x++) h[x] = x;
        A.write(h);
        permute(0.0, Indices{index::j, index::i}, &C, 1.0, Indices{index::i, index::j}, A);
        std::vector<double> got = C.read();
        bool ok = true;
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 4; j++) ok &= got[j * 3 + i] == h[i * 4 + j];
        CHECK(ok);
        DeviceTensor<double, 2> small("small", 3, 3);
        bool threw = false;
        try {
            permute(0.0, Indices{index::j, index::i}, &small, 1.0, Indices{index::i, index::j}, A);
        } catch (const dimension_error &) {
            threw = true;
        }
        CHECK(threw);
        // a compiled plan reused on new data (compile_permute + permute(&C, A, plan))
        auto plan = compile_permute(0.0, Indices{index::j, index::i}, &C, 1.0, Indices{index::i, index::j}, A);
        for (int rep = 1; rep <= 2; rep++) {
            for (int x = 0; x < 12; x++) h[x] = x * 10.0 * rep;
            A.write(h);
            permute(&C, A, plan);
            got = C.read();
            ok = true;
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 4; j++) ok &= got[j * 3 + i] == h[i * 4 + j];
            CHECK(ok);
        }
    }
    if (failures == 0) std::printf("frontend_test: all checks passed\n");
    return failures == 0 ? 0 : 1;
}
