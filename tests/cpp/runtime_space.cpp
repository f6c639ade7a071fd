// Test program of the C++ runtime-space layer (include/anigpu.hpp).
//   runtime_space host               : operator/space metadata and argument errors (no GPU)
//   runtime_space gpu <in> <out>     : fem3Dtet(GRAD P2, GRAD P2) and fem3Dface(IDEN P0, IDEN P2)
//                                      through the layer on the tets of <in> (nt * 12 doubles),
//                                      results to <out>; an invalid face must throw
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
    std::vector<double> A(nt * 100 + nt * 10);
    cudaMemcpy(A.data(), dA, sizeof(double) * nt * 100, cudaMemcpyDeviceToHost);
    cudaMemcpy(A.data() + nt * 100, dF, sizeof(double) * nt * 10, cudaMemcpyDeviceToHost);
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
