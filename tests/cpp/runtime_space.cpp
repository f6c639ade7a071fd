// Test program of the C++ runtime-space layer (include/anigpu.hpp).
//   runtime_space host               : operator/space metadata and argument errors (no GPU)
//   runtime_space gpu <in> <out>     : fem3Dtet(GRAD P2, GRAD P2) and fem3Dface(IDEN P0, IDEN P2)
//                                      through the layer on the tets of <in> (nt * 12 doubles),
//                                      then fem3Dtet with a user-defined operator (ApplyOpCustom)
//                                      whose functor evaluates GRAD of each P2 basis function with
//                                      fem3DapplyL; results to <out>; an invalid face must throw
#include <cstdio>
#include <cstring>
#include <vector>

#include <cuda_runtime.h>

#include "anigpu.hpp"

using namespace anigpu;

static int fail(const char* what) {
    std::fprintf(stderr, "FAILED: %s\n", what);
    return 1;
}

static int host_checks() {
    const FemSpace p2 = FemSpace::P2(), v2 = FemSpace::Vec3(p2);
    if (p2.getOP(GRAD).Nfa() != 10 || p2.getOP(GRAD).Dim() != 3 || p2.getOP(GRAD).Order() != 1) return fail("P2 GRAD");
    if (v2.getOP(GRAD).Nfa() != 30 || v2.getOP(GRAD).Dim() != 9 || v2.getOP(IDEN).Dim() != 3) return fail("P2^3");
    if (FemSpace::P3().getOP(IDEN).Nfa() != 20 || FemSpace::P0().getOP(IDEN).Nfa() != 1) return fail("P0/P3");
    if (v2.getOP(IDEN).code() != ANIGPU_OP(ANIGPU_VEC3_P2, ANIGPU_IDEN)) return fail("code");
    if (!(p2.getOP(GRAD) == ApplyOp(22)) || p2.getOP(GRAD) == p2.getOP(IDEN)) return fail("equality");
    if (v2.typeName() != "P2^3" || v2.NumDofsOnTet() != 30) return fail("names");
    const FemSpace nd = FemSpace::ND0(), rt = FemSpace::RT0();
    if (nd.getOP(CURL).Dim() != 3 || nd.getOP(GRAD).Dim() != 9 || nd.NumDofsOnTet() != 6) return fail("ND0");
    if (rt.getOP(DIV).Dim() != 1 || rt.getOP(IDEN).Dim() != 3 || rt.getOP(DIV).code() != 103) return fail("RT0");
    bool threw = false;
    try {
        ApplyOp bad(27);
        (void)bad;
    } catch (const std::invalid_argument&) {
        threw = true;
    }
    if (!threw) return fail("invalid code accepted");
    threw = false;
    try {
        FemSpace::Vec3(FemSpace::P3());
    } catch (const std::invalid_argument&) {
        threw = true;
    }
    if (!threw) return fail("P3^3 accepted");
    const ApplyOpCustom c1(3, ApplyOpCustom::Fill(), 6, 12, 1), c2(3, ApplyOpCustom::Fill(), 6, 12), c3(4, ApplyOpCustom::Fill(), 1, 4);
    if (c1.Dim() != 6 || c1.Nfa() != 12 || c1.Order() != 1 || !(c1 == c2) || c1 == c3) return fail("custom operator");
    if (c3.values_size(10, 4) != 10 * 14 * 4) return fail("custom operator values size");
    std::printf("host ok\n");
    return 0;
}

static int gpu_run(const char* in, const char* out) {
    std::FILE* f = std::fopen(in, "rb");
    if (!f) return fail("input");
    std::vector<double> XY;
    double v;
    while (std::fread(&v, sizeof v, 1, f) == 1) XY.push_back(v);
    std::fclose(f);
    const int64_t nt = (int64_t)XY.size() / 12;
    Context ctx(0);
    double *dXY = nullptr, *dA = nullptr, *dF = nullptr;
    if (cudaMalloc(&dXY, sizeof(double) * XY.size()) || cudaMalloc(&dA, sizeof(double) * nt * 100) ||
        cudaMalloc(&dF, sizeof(double) * nt * 10))
        return fail("cudaMalloc");
    cudaMemcpy(dXY, XY.data(), sizeof(double) * XY.size(), cudaMemcpyHostToDevice);
    const FemSpace p2 = FemSpace::P2();
    fem3Dtet(ctx.get(), nt, dXY, p2.getOP(GRAD), p2.getOP(GRAD), ANIGPU_TENSOR_NULL, nullptr, dA, 4);
    fem3Dface(ctx.get(), nt, dXY, 1, FemSpace::P0().getOP(IDEN), p2.getOP(IDEN), ANIGPU_TENSOR_NULL, nullptr, dF, 4);
    bool threw = false;
    try {
        fem3Dface(ctx.get(), nt, dXY, 7, p2.getOP(IDEN), p2.getOP(IDEN), ANIGPU_TENSOR_NULL, nullptr, dA, 4);
    } catch (const std::runtime_error& e) {
        threw = std::strstr(e.what(), "face") != nullptr;
    }
    if (!threw) return fail("invalid face did not throw");
    std::vector<double> A(nt * 210);
    cudaMemcpy(A.data(), dA, sizeof(double) * nt * 100, cudaMemcpyDeviceToHost);
    cudaMemcpy(A.data() + nt * 100, dF, sizeof(double) * nt * 10, cudaMemcpyDeviceToHost);
    // a custom operator: GRAD of the 10 P2 basis functions at the rule's points, from fem3DapplyL
    // on unit DOF vectors, interleaved into U[((t*q + n)*10 + i)*3 + k]
    ApplyOpCustom grad_p2(
        7,
        [](anigpu_handle h, int64_t n, const double* X, int order, double* U) {
            const int q = anigpu_quadrature(order, nullptr, nullptr, 1 << 20);
            std::vector<double> pts(4 * q), w(q), e((size_t)n * 10);
            anigpu_quadrature(order, pts.data(), w.data(), q);
            double *dP = nullptr, *dE = nullptr, *dG = nullptr;
            cudaMalloc(&dP, sizeof(double) * 4 * q);
            cudaMalloc(&dE, sizeof(double) * n * 10);
            cudaMalloc(&dG, sizeof(double) * n * q * 3);
            cudaMemcpy(dP, pts.data(), sizeof(double) * 4 * q, cudaMemcpyHostToDevice);
            for (int i = 0; i < 10; ++i) {
                for (int64_t t = 0; t < n; ++t)
                    for (int j = 0; j < 10; ++j) e[t * 10 + j] = j == i ? 1.0 : 0.0;
                cudaMemcpy(dE, e.data(), sizeof(double) * n * 10, cudaMemcpyHostToDevice);
                fem3DapplyL(h, n, X, q, dP, FemSpace::P2().getOP(GRAD), dE, dG);
                cudaMemcpy2D(U + 3 * i, sizeof(double) * 30, dG, sizeof(double) * 3, sizeof(double) * 3,
                             (size_t)n * q, cudaMemcpyDeviceToDevice);
            }
            cudaFree(dP);
            cudaFree(dE);
            cudaFree(dG);
        },
        3, 10, 1);
    double* dU = nullptr;
    if (cudaMalloc(&dU, sizeof(double) * grad_p2.values_size(nt, 4))) return fail("cudaMalloc U");
    fem3Dtet(ctx.get(), nt, dXY, grad_p2, grad_p2, ANIGPU_TENSOR_NULL, nullptr, dA, dU, nullptr, 4);
    cudaMemcpy(A.data() + nt * 110, dA, sizeof(double) * nt * 100, cudaMemcpyDeviceToHost);
    cudaFree(dU);
    threw = false;
    try {
        ApplyOpCustom bad(8, ApplyOpCustom::Fill(), 12, 10);
        (void)bad;
    } catch (const std::invalid_argument&) {
        threw = true;
    }
    if (!threw) return fail("custom operator with Dim 12 accepted");
    cudaFree(dXY);
    cudaFree(dA);
    cudaFree(dF);
    std::FILE* g = std::fopen(out, "wb");
    std::fwrite(A.data(), sizeof(double), A.size(), g);
    std::fclose(g);
    std::printf("gpu ok %lld tets\n", (long long)nt);
    return 0;
}

int main(int argc, char** argv) {
    if (argc >= 2 && std::strcmp(argv[1], "host") == 0) return host_checks();
    if (argc >= 4 && std::strcmp(argv[1], "gpu") == 0) return gpu_run(argv[2], argv[3]);
    std::fprintf(stderr, "usage: runtime_space host | gpu <in> <out>\n");
    return 2;
}
