// Drop-in test of include/anigpu_fem.hpp: code spelled as against AniFem++'s own headers
// (Ani::fem3Dtet<Operator<...>, Operator<...>, DfuncTraits<...>>, tensor functors, DenseMatrix,
// Tetra, applyDir, GenerateElemMatRhs + Assembler) computes on the GPU; the results are written
// for tests/test_gpu_template.py, which compares them with the oracle.
//
//   fem_template <input.bin> <output.bin>
// input: int64 nv, nt, nel; xyz[nv*3]; tets[nt*4] (i32); XY[nel*12] (separate tets for the
// element-level cases).  output: a sequence of named blocks (int32 name length, name, int64
// count, count doubles).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "anigpu_fem.hpp"

using namespace Ani;

namespace {

std::ofstream g_out;

void put(const std::string& name, const std::vector<double>& v) {
    const int32_t len = (int32_t)name.size();
    const int64_t n = (int64_t)v.size();
    g_out.write((const char*)&len, sizeof(len));
    g_out.write(name.data(), len);
    g_out.write((const char*)&n, sizeof(n));
    g_out.write((const char*)v.data(), sizeof(double) * v.size());
}

// an anisotropic symmetric field, the same formulas as the oracle's point tensor fn 2
TensorType aniso(const Coord<>& X, double* D, TensorDims dims, void* user_data, int iTet) {
    (void)dims, (void)user_data, (void)iTet;
    const double x = X[0], y = X[1], z = X[2];
    const double m[9] = {1 + x * x, x * y / 2, 0, x * y / 2, 1 + y * y, z / 3, 0, z / 3, 2 + z * z};
    for (int i = 0; i < 9; ++i) D[i] = m[i];
    return TENSOR_SYMMETRIC;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 3) {
        std::cerr << "usage: fem_template input.bin output.bin\n";
        return 2;
    }
    std::ifstream in(argv[1], std::ios::binary);
    int64_t nv = 0, nt = 0, nel = 0;
    in.read((char*)&nv, 8);
    in.read((char*)&nt, 8);
    in.read((char*)&nel, 8);
    std::vector<double> xyz(3 * nv), XY(12 * nel);
    std::vector<int32_t> tets(4 * nt);
    in.read((char*)xyz.data(), sizeof(double) * xyz.size());
    in.read((char*)tets.data(), sizeof(int32_t) * tets.size());
    in.read((char*)XY.data(), sizeof(double) * XY.size());
    if (!in) {
        std::cerr << "short input\n";
        return 2;
    }
    g_out.open(argv[2], std::ios::binary);
    try {
        // ---------------------------------------------------------------- element level, one tet a call
        std::vector<double> out;
        {
            // GRAD P2 x GRAD P2 with a per-point symmetric tensor (PerPoint traits), order 4
            double Amem[100];
            DenseMatrix<> A(Amem, 10, 10);
            out.clear();
            for (int64_t t = 0; t < nel; ++t) {
                const double* X = XY.data() + 12 * t;
                Tetra<const double> XYZ(X, X + 3, X + 6, X + 9);
                fem3Dtet<Operator<GRAD, FemFix<FEM_P2>>, Operator<GRAD, FemFix<FEM_P2>>, DfuncTraits<TENSOR_SYMMETRIC, false>>(
                    XYZ, aniso, A, 4);
                out.insert(out.end(), Amem, Amem + 100);
            }
            put("p2_aniso_point_o4", out);
        }
        {
            // GRAD P1 x GRAD P1, identity (TensorNull, constant NULL traits), order 2
            double Amem[16];
            DenseMatrix<> A(Amem, 4, 4);
            out.clear();
            for (int64_t t = 0; t < nel; ++t) {
                const double* X = XY.data() + 12 * t;
                fem3Dtet<Operator<GRAD, FemFix<FEM_P1>>, Operator<GRAD, FemFix<FEM_P1>>, DfuncTraits<TENSOR_NULL, true>>(
                    Tetra<const double>(X, X + 3, X + 6, X + 9), TensorNull<>, A, 2);
                out.insert(out.end(), Amem, Amem + 16);
            }
            put("p1_null_o2", out);
        }
        {
            // IDEN P0 x IDEN P2 with a constant scalar (right-hand side), order 3 (the 8-point rule)
            double Amem[10];
            DenseMatrix<> A(Amem, 10, 1);
            out.clear();
            auto c = makeConstantTensorScalar(2.5);
            for (int64_t t = 0; t < nel; ++t) {
                const double* X = XY.data() + 12 * t;
                fem3Dtet<Operator<IDEN, FemFix<FEM_P0>>, Operator<IDEN, FemFix<FEM_P2>>, DfuncTraits<TENSOR_SCALAR, true>>(
                    Tetra<const double>(X, X + 3, X + 6, X + 9), c, A, 3);
                out.insert(out.end(), Amem, Amem + 10);
            }
            put("rhs_p2_const_o3", out);
        }
        {
            // vector P2 elasticity with the isotropic 9x9 tensor C_{(ij)(kl)} = lambda d_ij d_kl +
            // mu (d_ik d_jl + d_il d_jk), lambda = 1, mu = 3, written as a column-major 9x9 DenseMatrix
            auto C_tensor = [](const Coord<>& X, double* D, TensorDims dims, void* user_data, int iTet) -> TensorType {
                (void)X, (void)dims, (void)user_data, (void)iTet;
                DenseMatrix<> C(D, 9, 9);
                double lambda = 1.0, mu = 3.0;
                C.SetZero();
                for (int i = 0; i < 3; ++i)
                    for (int l = 0; l < 3; ++l) {
                        int j = i, k = l;
                        C(i + 3 * j, k + 3 * l) += lambda;
                        k = i, j = l;
                        C(i + 3 * j, k + 3 * l) += mu;
                        C(i + 3 * j, l + 3 * k) += mu;
                    }
                return Ani::TENSOR_SYMMETRIC;
            };
            std::vector<double> Amem(900);
            DenseMatrix<> A(Amem.data(), 30, 30);
            out.clear();
            for (int64_t t = 0; t < nel; ++t) {
                const double* X = XY.data() + 12 * t;
                Tetra<const double> XYZ(X, X + 3, X + 6, X + 9);
                fem3Dtet<Operator<GRAD, FemVec<3, FEM_P2>>, Operator<GRAD, FemVec<3, FEM_P2>>, DfuncTraits<TENSOR_SYMMETRIC>>(
                    XYZ, C_tensor, A, 4);
                out.insert(out.end(), Amem.begin(), Amem.end());
            }
            put("vecp2_lame_o4", out);
        }
        {
            // fused batches of 4 tets (3 x f coordinate matrices), a PerTetra tensor that depends on iTet
            const int F = 4;
            auto per_tet = [](const Coord<>& X, double* D, TensorDims dims, void* user_data, int iTet) {
                (void)X, (void)dims;
                const double base = *static_cast<const double*>(user_data);
                D[0] = base + iTet;
                return TENSOR_SCALAR;
            };
            double base = 1.5;
            std::vector<double> Amem(100 * F);
            out.clear();
            for (int64_t t0 = 0; t0 + F <= nel; t0 += F) {
                double c[4][3 * F];
                for (int r = 0; r < F; ++r)
                    for (int v = 0; v < 4; ++v)
                        for (int k = 0; k < 3; ++k) c[v][3 * r + k] = XY[12 * (t0 + r) + 3 * v + k];
                DenseMatrix<> X0(c[0], 3, F), X1(c[1], 3, F), X2(c[2], 3, F), X3(c[3], 3, F);
                DenseMatrix<> A(Amem.data(), 10, 10 * F);
                fem3Dtet<Operator<GRAD, FemFix<FEM_P2>>, Operator<GRAD, FemFix<FEM_P2>>, DfuncTraits<PerTetra>, F>(
                    X0, X1, X2, X3, per_tet, A, 5, &base);
                out.insert(out.end(), Amem.begin(), Amem.end());
            }
            put("p2_pertet_fused4_o5", out);
        }
        {
            // a fusive (batched) functor: one call fills the tensor at every point of the batch
            auto fusive = [](ArrayView<> X, ArrayView<> D, TensorDims dims, void* user_data, const AniMemory<>& mem) {
                (void)user_data;
                const std::size_t m = dims.first * dims.second;
                for (std::size_t r = 0; r < mem.f; ++r)
                    for (std::size_t n = 0; n < mem.q; ++n) {
                        const double* x = X.data + 3 * (n + mem.q * r);
                        double* d = D.data + m * (n + mem.q * r);
                        const double v[9] = {1 + x[0] * x[0], x[0] * x[1] / 2, 0, x[0] * x[1] / 2, 1 + x[1] * x[1],
                                             x[2] / 3, 0, x[2] / 3, 2 + x[2] * x[2]};
                        for (std::size_t i = 0; i < m; ++i) d[i] = v[i];
                    }
                return TENSOR_GENERAL;
            };
            const int F = 2;
            std::vector<double> Amem(100 * F);
            out.clear();
            for (int64_t t0 = 0; t0 + F <= nel; t0 += F) {
                const double* a = XY.data() + 12 * t0;
                double c[4][3 * F];
                for (int r = 0; r < F; ++r)
                    for (int v = 0; v < 4; ++v)
                        for (int k = 0; k < 3; ++k) c[v][3 * r + k] = a[12 * r + 3 * v + k];
                DenseMatrix<> A(Amem.data(), 10, 10 * F);
                fem3Dtet<Operator<GRAD, FemFix<FEM_P2>>, Operator<GRAD, FemFix<FEM_P2>>, DfuncTraitsFusive<>, F>(
                    make_tetras(c[0], c[1], c[2], c[3], F), fusive, A, 4);
                out.insert(out.end(), Amem.begin(), Amem.end());
            }
            put("p2_fusive_o4", out);
        }
        {
            // the PlainMemory overload at orders above 6 (order 12, 168 points; order 20, 552 points)
            for (int order : {12, 20}) {
                auto req = fem3Dtet_memory_requirements<Operator<GRAD, FemFix<FEM_P2>>, Operator<GRAD, FemFix<FEM_P2>>>(order, 1);
                std::vector<char> raw(req.enoughRawSize());
                req.allocateFromRaw(raw.data(), raw.size());
                double Amem[100];
                DenseMatrix<> A(Amem, 10, 10);
                out.clear();
                for (int64_t t = 0; t < nel; ++t) {
                    const double* X = XY.data() + 12 * t;
                    DenseMatrix<> X0(const_cast<double*>(X), 3, 1), X1(const_cast<double*>(X + 3), 3, 1),
                        X2(const_cast<double*>(X + 6), 3, 1), X3(const_cast<double*>(X + 9), 3, 1);
                    fem3Dtet<Operator<GRAD, FemFix<FEM_P2>>, Operator<GRAD, FemFix<FEM_P2>>, DfuncTraits<TENSOR_SYMMETRIC, false>>(
                        X0, X1, X2, X3, aniso, A, req, order);
                    out.insert(out.end(), Amem, Amem + 100);
                }
                put("p2_aniso_point_o" + std::to_string(order), out);
            }
        }
        {
            // face integrals: a per-point scalar load on face 2 (fem3Dface) and the traction of a
            // general 9 x 3 tensor contracted with the outward normal (fem3DfaceN), order 5
            auto load = [](const Coord<>& X, double* D, TensorDims dims, void* user_data, int iTet) {
                (void)dims, (void)user_data, (void)iTet;
                D[0] = 1 + X[0] * X[1];
                return TENSOR_SCALAR;
            };
            double Amem[30];
            DenseMatrix<> A(Amem, 10, 1);
            out.clear();
            for (int64_t t = 0; t < nel; ++t) {
                const double* X = XY.data() + 12 * t;
                fem3Dface<Operator<IDEN, FemFix<FEM_P0>>, Operator<IDEN, FemFix<FEM_P2>>, DfuncTraits<TENSOR_SCALAR>>(
                    Tetra<const double>(X, X + 3, X + 6, X + 9), 2, load, A, 5);
                out.insert(out.end(), Amem, Amem + 10);
            }
            put("face2_p2_load_o5", out);
            auto trac = [](const Coord<>& X, double* D, TensorDims dims, void* user_data, int iTet) {
                (void)user_data, (void)iTet;
                for (std::size_t j = 0; j < dims.second; ++j)
                    for (std::size_t i = 0; i < dims.first; ++i) D[i + dims.first * j] = (i + 1) * 0.5 + (i + j) * X[2];
                return TENSOR_GENERAL;
            };
            DenseMatrix<> B(Amem, 30, 1);
            out.clear();
            for (int64_t t = 0; t < nel; ++t) {
                const double* X = XY.data() + 12 * t;
                fem3DfaceN<Operator<IDEN, FemFix<FEM_P0>>, Operator<IDEN, FemVec<3, FEM_P2>>, DfuncTraits<TENSOR_GENERAL>>(
                    Tetra<const double>(X, X + 3, X + 6, X + 9), 1, trac, B, 5);
                out.insert(out.end(), Amem, Amem + 30);
            }
            put("facen1_vecp2_trac_o5", out);
        }
        {
            // the reference's errors: order above 6 in the memoryless overload, identity tensor of
            // incompatible operators
            double Amem[100];
            DenseMatrix<> A(Amem, 10, 10);
            const double* X = XY.data();
            int caught = 0;
            try {
                fem3Dtet<Operator<GRAD, FemFix<FEM_P2>>, Operator<GRAD, FemFix<FEM_P2>>, DfuncTraits<TENSOR_NULL, true>>(
                    Tetra<const double>(X, X + 3, X + 6, X + 9), TensorNull<>, A, 7);
            } catch (const std::runtime_error&) {
                caught |= 1;
            }
            try {
                fem3Dtet<Operator<GRAD, FemFix<FEM_P2>>, Operator<IDEN, FemFix<FEM_P2>>, DfuncTraits<TENSOR_NULL, true>>(
                    Tetra<const double>(X, X + 3, X + 6, X + 9), TensorNull<>, A, 2);
            } catch (const std::runtime_error&) {
                caught |= 2;
            }
            put("errors_caught", {(double)caught});
        }

        // ---------------------------------------------------------------- global: the ex1 local assembler
        {
            using UFem = FemFix<FEM_P1>;
            constexpr auto UNF = Operator<IDEN, UFem>::Nfa::value;
            // boundary labels of the unit cube's nodes, as ex1 sets them
            std::vector<int> BndLabel(nv, 0);
            for (int64_t v = 0; v < nv; ++v) {
                int lbl = 0;
                for (int k = 0; k < 3; ++k)
                    if (std::abs(xyz[3 * v + k] - 0) < 10 * std::numeric_limits<double>::epsilon())
                        lbl |= (1 << (2 * k + 0));
                    else if (std::abs(xyz[3 * v + k] - 1) < 10 * std::numeric_limits<double>::epsilon())
                        lbl |= (1 << (2 * k + 1));
                BndLabel[v] = lbl;
            }
            auto D_tensor = [](const Coord<>& X, double* D, TensorDims dims, void* user_data, int iTet) {
                (void)dims;
                (void)user_data;
                (void)iTet;
                D[0] = 1 + X[0] * X[0];
                return Ani::TENSOR_SCALAR;
            };
            auto F_tensor = [](const Coord<>& X, double* F, TensorDims dims, void* user_data, int iTet) {
                (void)X;
                (void)dims;
                (void)user_data;
                (void)iTet;
                F[0] = 1;
                return Ani::TENSOR_SCALAR;
            };
            auto U_0 = [](const Coord<>& X, double* res, unsigned long dim, void* user_data) -> int {
                (void)X;
                (void)dim;
                (void)user_data;
                res[0] = 0.0;
                return 0;
            };
            struct ProbLocData {
                std::array<int, 4> nlbl = {0};
            };
            const int order = 2;
            std::function<void(const double**, double*, double*, void*)> local_assembler =
                [&D_tensor, &F_tensor, &U_0, order](const double** XY, double* Adat, double* Fdat, void* user_data) -> void {
                DenseMatrix<> A(Adat, UNF, UNF), F(Fdat, UNF, 1);
                A.SetZero();
                F.SetZero();
                Tetra<const double> XYZ(XY[0], XY[1], XY[2], XY[3]);
                fem3Dtet<Operator<GRAD, UFem>, Operator<GRAD, UFem>, DfuncTraits<TENSOR_SCALAR, false>>(XYZ, D_tensor, A, order);
                fem3Dtet<Operator<IDEN, FemFix<FEM_P0>>, Operator<IDEN, UFem>, DfuncTraits<TENSOR_SCALAR, true>>(XYZ, F_tensor, F, order);
                auto& dat = *static_cast<ProbLocData*>(user_data);
                for (int i = 0; i < 4; ++i)
                    if (dat.nlbl[i] > 0) {
                        double bc = 0;
                        U_0(std::array<double, 3>{XY[i][0], XY[i][1], XY[i][2]}, &bc, 1, nullptr);
                        applyDir(A, F, i, bc);
                    }
            };
            auto local_data_gatherer = [&BndLabel](ElementalAssembler& p) -> void {
                double* nn_p = p.get_nodes();
                const double* args[] = {nn_p, nn_p + 3, nn_p + 6, nn_p + 9};
                ProbLocData data;
                std::fill(data.nlbl.begin(), data.nlbl.end(), 0);
                for (unsigned i = 0; i < data.nlbl.size(); ++i) data.nlbl[i] = BndLabel[p.node_id(i)];
                p.compute(args, &data);
            };
            Assembler discr(xyz.data(), nv, tets.data(), nt);
            discr.SetMatRHSFunc(GenerateElemMatRhs(local_assembler, UNF, UNF));
            {
                auto Var0Helper = GenerateHelper<UFem>();
                FemExprDescr fed;
                fed.PushTrialFunc(Var0Helper, "u");
                fed.PushTestFunc(Var0Helper, "phi_u");
                discr.SetProbDescr(std::move(fed));
            }
            discr.SetDataGatherer(local_data_gatherer);
            discr.SetChunkSize(1000);  // several record / replay rounds
            discr.PrepareProblem();
            SparseMatrix A;
            Vector b;
            const int status = discr.Assemble(A, b);
            std::vector<int64_t> rp;
            std::vector<int32_t> col;
            std::vector<double> vals, rhs;
            A.download(rp, col, vals);
            b.download(rhs);
            put("ex1_status", {(double)status});
            put("ex1_rowptr", std::vector<double>(rp.begin(), rp.end()));
            put("ex1_col", std::vector<double>(col.begin(), col.end()));
            put("ex1_vals", vals);
            put("ex1_rhs", rhs);
        }
    } catch (const std::exception& e) {
        std::cerr << "fem_template: " << e.what() << "\n";
        return 1;
    }
    g_out.close();
    std::cout << "fem_template ok\n";
    return 0;
}
