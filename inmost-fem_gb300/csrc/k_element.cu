// Element level: the batched fem3Dtet (every operator pair, every tensor kind), the
// physical quadrature points and the element-level Dirichlet elimination.
//
// Ani::fem3Dtet (anifem++/fem/operations/int_tet.inl:93-122 -> core.inl:277-367) computes
//     U = OpA(phi) at every quadrature point, V = OpB(phi),
//     DU = w_n |T| D(x_n) U          (internal_Dfunc::applyDU, diff_tensor.h:275-994)
//     A  = V^T DU                      (fusive_AT_mul_B, core.inl:28-60)
// Three kernels, chosen per call by launch_fem3dtet:
//   fem3dtet_reftensor_lanes_kernel  scalar spaces, IDEN/GRAD, tensors constant on a tet, at most
//                                    100 entries: the same sum regrouped through reference tensors
//                                    (lanes over tets);
//   fem3dtet_reftensor_kernel        the same with lanes over entries, for larger matrices;
//   fem3dtet_kernel                  everything else (FemVec, ND0/RT0, per-point tensors,
//                                    fem3DfaceN, user-defined operators): one warp per tet, the
//                                    per-point quadrature in shared memory.
#include <cstring>

#include "anigpu_internal.h"
#include "basis_eval.h"
#include "fp_convert.cuh"
#include "quad_tables.h"

namespace {

constexpr int kThreads = 128;

struct OpDesc {
    int nf, dim, nfs, bd, ncomp, op;  // op: 1 IDEN, 2 GRAD, 3 DIV, 4 CURL
    int space;                        // base space; ND0 / RT0 are evaluated from the tet geometry
    int tnf;                          // functions in the table: nfs, or 4 (the P1 table: lambda) for ND0 / RT0
    const double* tab;                // device basis table (vals q*tnf, grads q*tnf*3)
    const double* user;               // custom operator: values per (tet, point), dim x nf column-major
};

struct ElemParams {
    OpDesc A, B;
    int q, kind;
    int face;         // -1: the tet integral; 0..3: the integral over face k (fem3Dface)
    int normal;       // fem3DfaceN: the tensor has 3*dimB rows, contracted with the outward normal
    int same;         // OpA == OpB: V is U
    int tab_shared;   // basis tables staged in shared memory (else read through L1 from global memory)
    const double* w;  // device weights
};

// outward unit normal and area of face k (Ani::face_normal, geometry.h:77-93, on the coordinates
// relative to X0; the fourth vertex decides the orientation)
__device__ inline double face_normal(const double* X, int face, double* nrm) {
    double P[4][3];
#pragma unroll
    for (int v = 0; v < 4; ++v) {
        const int node = (face + v) & 3;
#pragma unroll
        for (int i = 0; i < 3; ++i) P[v][i] = node == 0 ? 0.0 : X[3 * node + i] - X[i];
    }
    double a[3] = {P[1][0] - P[0][0], P[1][1] - P[0][1], P[1][2] - P[0][2]};
    const double b[3] = {P[2][0] - P[0][0], P[2][1] - P[0][1], P[2][2] - P[0][2]};
    nrm[0] = a[1] * b[2] - a[2] * b[1];
    nrm[1] = -a[0] * b[2] + a[2] * b[0];
    nrm[2] = a[0] * b[1] - a[1] * b[0];
    const double len = sqrt(nrm[0] * nrm[0] + nrm[1] * nrm[1] + nrm[2] * nrm[2]);
#pragma unroll
    for (int i = 0; i < 3; ++i) a[i] = P[3][i] - P[0][i];
    const double vol = nrm[0] * a[0] + nrm[1] * a[1] + nrm[2] * a[2];
    const double sc = vol > 0 ? -len : len;
#pragma unroll
    for (int i = 0; i < 3; ++i) nrm[i] /= sc;
    return len / 2;
}

// entry (k, j) of the dB x dA tensor at point n of tet t, with applyDU's meaning of the
// identity-type kinds (diff_tensor.h:275-552): NULL/SCALAR are s*I when dA == dB, a column of s
// when dA == 1
__device__ inline double tensor_at(int kind, const double* D, int64_t t, int n, int q, int dA, int dB, int k, int j) {
    switch (kind) {
        case ANIGPU_TENSOR_NULL:
        case ANIGPU_TENSOR_CONST_SCALAR:
        case ANIGPU_TENSOR_TET_SCALAR: {
            const double s = kind == ANIGPU_TENSOR_NULL ? 1.0 : (kind == ANIGPU_TENSOR_CONST_SCALAR ? D[0] : D[t]);
            return (dA == dB) ? (k == j ? s : 0.0) : s;
        }
        case ANIGPU_TENSOR_TET_SYM: {
            const double* s6 = D + 6 * t;
            const int lo = k < j ? k : j, hi = k < j ? j : k;
            return s6[lo == 0 ? hi : (lo == 1 ? 2 + hi : 5)];
        }
        case ANIGPU_TENSOR_TET_GENERAL: return D[(size_t)dA * dB * t + k + dB * j];
        default: return D[(size_t)dA * dB * (n + (size_t)q * t) + k + dB * j];
    }
}

// area of face k = vertices k, k+1, k+2 (mod 4), from the coordinates relative to X0 as the
// reference's XYP (tri_area, geometry.h:67-72; int_face.inl:40-43)
__device__ inline double face_area(const double* X, int face) {
    double P[3][3];
#pragma unroll
    for (int v = 0; v < 3; ++v) {
        const int node = (face + v) & 3;
#pragma unroll
        for (int i = 0; i < 3; ++i) P[v][i] = node == 0 ? 0.0 : X[3 * node + i] - X[i];
    }
    const double a[3] = {P[0][0] - P[2][0], P[0][1] - P[2][1], P[0][2] - P[2][2]};
    const double b[3] = {P[1][0] - P[2][0], P[1][1] - P[2][1], P[1][2] - P[2][2]};
    const double c[3] = {a[1] * b[2] - a[2] * b[1], -a[0] * b[2] + a[2] * b[0], a[0] * b[1] - a[1] * b[0]};
    return sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]) / 2;
}

// cofactors C of the edge matrix [X1-X0, X2-X0, X3-X0] arranged so that PSI = C / det is its
// inverse (inverse3x3, geometry.h:26-44), and det
__device__ inline void tet_cofactors(const double* X, double* C, double* det_out) {
    double m[9];
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int i = 0; i < 3; ++i) m[i + 3 * c] = X[3 * (c + 1) + i] - X[i];
#define M(I, J) m[(I) + 3 * (J)]
    const double da = M(1, 1) * M(2, 2) - M(1, 2) * M(2, 1);
    const double db = M(1, 2) * M(2, 0) - M(1, 0) * M(2, 2);
    const double dc = M(1, 0) * M(2, 1) - M(1, 1) * M(2, 0);
    *det_out = M(0, 0) * da + M(0, 1) * db + M(0, 2) * dc;
    C[0] = da;
    C[1] = db;
    C[2] = dc;
#pragma unroll
    for (int i = 1; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
            C[j + 3 * i] = M((i + 1) % 3, (j + 1) % 3) * M((i + 2) % 3, (j + 2) % 3) -
                           M((i + 1) % 3, (j + 2) % 3) * M((i + 2) % 3, (j + 1) % 3);
#undef M
}

__device__ inline void tet_geometry(const double* X, double* PSI, double* mes, double* det_out = nullptr) {
    // internalFem3DtetGeomInit_Tet (core.inl:217-247) with inverse3x3 (geometry.h:26-44)
    double det;
    tet_cofactors(X, PSI, &det);
#pragma unroll
    for (int i = 0; i < 9; ++i) PSI[i] /= det;
    *mes = fabs(det) / 6.0;
    if (det_out) *det_out = det;
}

// value of operator `o` for column `col`, row `k` at point n (block structure of FemVec,
// operators.h:127-155: component c owns rows [c*bd,(c+1)*bd) and columns [c*nfs,(c+1)*nfs))
// geo: PSI[9], mes, normal[3], vertex coordinates relative to X0 [12] (from 13), signed det (25)
template <typename Real>
__device__ inline Real op_value(const OpDesc& o, const double* tab, int q, int n, int k, int col, const double* geo) {
    const double* PSI = geo;
    if (o.space == ANIGPU_ND0 || o.space == ANIGPU_RT0) {
        const double* l = tab + (size_t)n * 4;  // P1 table values = barycentric coordinates
        return Real(ani_vec_space_value(o.space, o.op, l, PSI, geo + 13, geo[25], col, k));
    }
    const int c = col / o.nfs, i = col - c * o.nfs;
    const int kc = k / o.bd, kk = k - kc * o.bd;
    if (kc != c) return Real(0);
    if (o.op == ANIGPU_IDEN) return Real(tab[n * o.tnf + i]);
    const double* g = tab + (size_t)q * o.tnf + 3 * ((size_t)n * o.tnf + i);
    // U_k = sum_j PSI(j,k) ghat_j (poly_2.h:91-97)
    return Real(PSI[0 + 3 * kk] * g[0] + PSI[1 + 3 * kk] * g[1] + PSI[2 + 3 * kk] * g[2]);
}

// One warp per tet (four tets in flight per 128-thread block): per quadrature point the warp
// fills U, V (= U when both operators are the same), the tensor and DU = w |T| D U in its own
// shared-memory region, then every lane adds V^T DU to the element entries it owns (e = lane + 32m,
// kept in shared memory).  Only warp-level synchronisation; every entry sums its points in
// ascending order and each point's contribution over k in ascending order.
template <typename Real>
__global__ void __launch_bounds__(kThreads) fem3dtet_kernel(ElemParams p, int64_t nt, const double* __restrict__ XY,
                                                             const double* __restrict__ D, Real* __restrict__ A,
                                                             int wstride) {
    extern __shared__ double smem[];
    const int q = p.q;
    const int nfA = p.A.nf, nfB = p.B.nf, dA = p.A.dim, dB = p.B.dim;
    // basis tables: staged in shared memory when they fit (every rule up to order 6); the rules
    // of orders 7-20 (up to 552 points) are read from global memory through L1
    const size_t tabA = p.tab_shared ? (size_t)q * p.A.tnf * 4 : 0, tabB = p.tab_shared ? (size_t)q * p.B.tnf * 4 : 0;
    double* sW = smem + tabA + tabB;
    for (size_t i = threadIdx.x; i < tabA; i += blockDim.x) smem[i] = p.A.tab[i];
    for (size_t i = threadIdx.x; i < tabB; i += blockDim.x) smem[tabA + i] = p.B.tab[i];
    const double* sTabA = p.tab_shared ? smem : p.A.tab;
    const double* sTabB = p.tab_shared ? smem + tabA : p.B.tab;
    for (int i = threadIdx.x; i < q; i += blockDim.x) sW[i] = p.w[i];
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    constexpr int kWarps = kThreads / 32;
    double* sGeo = sW + q + (size_t)warp * wstride;  // PSI[9], mes, normal[3], XYP[12], det
    double* sD = sGeo + 26;                          // dB*dA
    Real* sU = reinterpret_cast<Real*>(sD + ANIGPU_MAX_DIM * ANIGPU_MAX_DIM);
    Real* sV = sU + dA * nfA;
    Real* sDU = sV + (p.same ? 0 : dB * nfB);
    Real* sAcc = sDU + dB * nfA;
    const Real* V = p.same ? sU : sV;
    const int nent = nfA * nfB;
    const int nD = dA * dB;
    for (int64_t t = (int64_t)blockIdx.x * kWarps + warp; t < nt; t += (int64_t)gridDim.x * kWarps) {
        if (lane == 0) {
            const double* X = XY + 12 * t;
            tet_geometry(X, sGeo, sGeo + 9, sGeo + 25);
            for (int v = 0; v < 4; ++v)
                for (int i = 0; i < 3; ++i) sGeo[13 + 3 * v + i] = v == 0 ? 0.0 : X[3 * v + i] - X[i];
            if (p.normal) sGeo[9] = face_normal(X, p.face, sGeo + 10);
            else if (p.face >= 0) sGeo[9] = face_area(X, p.face);
        }
        for (int e = lane; e < nent; e += 32) sAcc[e] = Real(0);
        __syncwarp();
        const double mes = sGeo[9];
        for (int n = 0; n < q; ++n) {
            // U, V and the tensor at point n
            for (int e = lane; e < dA * nfA; e += 32)
                sU[e] = p.A.user ? Real(p.A.user[((size_t)t * q + n) * (dA * nfA) + e])
                                 : op_value<Real>(p.A, sTabA, q, n, e % dA, e / dA, sGeo);
            if (!p.same)
                for (int e = lane; e < dB * nfB; e += 32)
                    sV[e] = p.B.user ? Real(p.B.user[((size_t)t * q + n) * (dB * nfB) + e])
                                     : op_value<Real>(p.B, sTabB, q, n, e % dB, e / dB, sGeo);
            // dense D(k,j), column-major dB x dA; fem3DfaceN: rows l + 3k of the 3dB x dA tensor
            // contracted with the normal (DotWithNormalHelper::ProcessNormal, core.h:175-190)
            for (int e = lane; e < nD; e += 32) {
                const int k = e % dB, j = e / dB;
                if (!p.normal) {
                    sD[e] = tensor_at(p.kind, D, t, n, q, dA, dB, k, j);
                } else {
                    double v = 0.0;
#pragma unroll
                    for (int l = 0; l < 3; ++l) v += tensor_at(p.kind, D, t, n, q, dA, 3 * dB, l + 3 * k, j) * sGeo[10 + l];
                    sD[e] = v;
                }
            }
            __syncwarp();
            const Real wv = Real(sW[n] * mes);
            for (int e = lane; e < dB * nfA; e += 32) {
                const int k = e % dB, ia = e / dB;
                Real s = 0;
                for (int j = 0; j < dA; ++j) s += Real(sD[k + dB * j]) * sU[j + dA * ia];
                sDU[e] = wv * s;
            }
            __syncwarp();
            for (int e = lane; e < nent; e += 32) {
                const int ib = e % nfB, ia = e / nfB;
                Real s = 0;
                for (int k = 0; k < dB; ++k) s += V[k + dB * ib] * sDU[k + dB * ia];
                sAcc[e] += s;
            }
            __syncwarp();
        }
        Real* At = A + (size_t)nent * t;
        for (int e = lane; e < nent; e += 32) At[e] = sAcc[e];
        __syncwarp();
    }
}

// Reference-tensor form for scalar Lagrange-type spaces, IDEN / GRAD operators and tensors constant
// on a tet: U_n = L_A Uhat_n with L = PSI^T (GRAD) or 1 (IDEN), so
//     A(ib, ia) = sum_{m,m'} M(m, m') T(ib, ia, m, m'),   M = mes L_B^T D L_A,
//     T(ib, ia, m, m') = sum_n w_n Vhat_n(m, ib) Uhat_n(m', ia)   (per rule, operator pair and face)
// -- the quadrature sum of fem3Dtet (core.inl:277-367) regrouped exactly.  With the same operator
// on both sides and a symmetric tensor, M is symmetric and A(ib, ia) = A(ia, ib): the kernel then
// forms the upper triangle only, from the six distinct M(m <= m') and T(m, m') + T(m', m) (FP64
// FMA throughput bounds this kernel in double precision).  Phase 1: one thread per tet forms M in
// FP64; phase 2: each warp builds the matrices of 32 tets, lanes over entries (or entry pairs),
// staged in shared memory and written out coalesced.
template <typename Real>
__global__ void __launch_bounds__(128) fem3dtet_reftensor_kernel(int64_t nt, const double* __restrict__ XY, int kind,
                                                                 const double* __restrict__ D, int dA, int dB,
                                                                 int gradA, int gradB, int nfA, int nfB, int face,
                                                                 int sym, const double* __restrict__ T,
                                                                 Real* __restrict__ A) {
    extern __shared__ double rsm[];
    const int rA = gradA ? 3 : 1, rB = gradB ? 3 : 1;
    const int nent = nfA * nfB;
    const int rs = sym ? (rA == 3 ? 6 : 1) : rA * rB;      // M values per tet
    const int nrow = sym ? nfA * (nfA + 1) / 2 : nent;     // entries (pairs) computed per tet
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    Real* sT = reinterpret_cast<Real*>(rsm);
    Real* sM = sT + (size_t)nrow * rs;
    Real* sOut = sM + 128 * 9 + (size_t)warp * nent;
    int* sPair = reinterpret_cast<int*>(sM + 128 * 9 + (size_t)4 * nent);
    for (int i = threadIdx.x; i < nrow * rs; i += blockDim.x) sT[i] = Real(T[i]);
    if (sym)
        for (int i = threadIdx.x; i < nrow; i += blockDim.x) sPair[i] = (int)T[(size_t)nrow * rs + i];
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < nt; base += (int64_t)gridDim.x * blockDim.x) {
        __syncthreads();
        const int64_t t = base + threadIdx.x;
        if (t < nt) {
            const double* X = XY + 12 * t;
            // PSI = C / det with C the cofactors (tet_geometry); the 1/det of each GRAD side goes into
            // the scale factor, one reciprocal per tet
            double PSI[9], det;
            tet_cofactors(X, PSI, &det);
            const double mes = face >= 0 ? face_area(X, face) : fabs(det) / 6.0;
            const double inv = 1.0 / det;
            const double scale = mes * (gradA ? inv : 1.0) * (gradB ? inv : 1.0);
            // L(j, m') = C(m', j) for GRAD, the 1x1 identity for IDEN; W = D L_A, M = scale L_B^T W
            double W[3][3];
#pragma unroll
            for (int k = 0; k < 3; ++k)
#pragma unroll
                for (int mp = 0; mp < 3; ++mp) {
                    double w = 0.0;
#pragma unroll
                    for (int j = 0; j < 3; ++j) {
                        if (k >= dB || j >= dA) continue;
                        const double la = gradA ? PSI[mp + 3 * j] : (j == mp ? 1.0 : 0.0);
                        w += tensor_at(kind, D, t, 0, 1, dA, dB, k, j) * la;
                    }
                    W[k][mp] = w;
                }
            int c = 0;
#pragma unroll
            for (int m = 0; m < 3; ++m)
#pragma unroll
                for (int mp = 0; mp < 3; ++mp) {
                    if (m >= rB || mp >= rA || (sym && mp < m)) continue;
                    double v = 0.0;
#pragma unroll
                    for (int k = 0; k < 3; ++k) {
                        if (k >= dB) continue;
                        const double lb = gradB ? PSI[m + 3 * k] : (k == m ? 1.0 : 0.0);
                        v += lb * W[k][mp];
                    }
                    sM[threadIdx.x * 9 + c++] = Real(scale * v);
                }
        }
        __syncthreads();
        for (int i = 0; i < 32; ++i) {
            const int tl = warp * 32 + i;
            const int64_t tt = base + tl;
            if (tt >= nt) break;
            const Real* M = sM + tl * 9;
            for (int e = lane; e < nrow; e += 32) {
                const Real* Te = sT + (size_t)e * rs;
                Real s = 0;
                for (int k = 0; k < rs; ++k) s += M[k] * Te[k];
                if (sym) {
                    const int ib = sPair[e] & 0xffff, ia = sPair[e] >> 16;
                    sOut[ib + nfB * ia] = s;
                    sOut[ia + nfB * ib] = s;
                } else {
                    sOut[e] = s;  // e = ib + nfB * ia (column-major nfB x nfA)
                }
            }
            __syncwarp();
            Real* At = A + (size_t)nent * tt;
            for (int e = lane; e < nent; e += 32) At[e] = sOut[e];
            __syncwarp();
        }
    }
}

// cofactors C (PSI = C / det) and det of the edge matrix m = [X1-X0, X2-X0, X3-X0] (tet_cofactors)
template <typename R>
__device__ __forceinline__ R cofactors_of(const R* m, R* C) {
#define M_(I, J) m[(I) + 3 * (J)]
    C[0] = M_(1, 1) * M_(2, 2) - M_(1, 2) * M_(2, 1);
    C[1] = M_(1, 2) * M_(2, 0) - M_(1, 0) * M_(2, 2);
    C[2] = M_(1, 0) * M_(2, 1) - M_(1, 1) * M_(2, 0);
#pragma unroll
    for (int i = 1; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
            C[j + 3 * i] = M_((i + 1) % 3, (j + 1) % 3) * M_((i + 2) % 3, (j + 2) % 3) -
                           M_((i + 1) % 3, (j + 2) % 3) * M_((i + 2) % 3, (j + 1) % 3);
    return M_(0, 0) * C[0] + M_(0, 1) * C[1] + M_(0, 2) * C[2];
#undef M_
}

// M = scale L_B^T D L_A with L = C^T (GRAD) or the 1x1 identity (IDEN), in the host's order of
// the M terms (m-major; upper triangle when SYM); Dm(k, j) = D(k, j), zero outside dB x dA
template <typename R, int RS, bool SYM>
__device__ __forceinline__ void reft_m(const R* C, R scale, const R (&Dm)[3][3], int dA, int dB, int gradA, int gradB,
                                       R (&M)[RS]) {
    const int rA = gradA ? 3 : 1, rB = gradB ? 3 : 1;
    R W[3][3];
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int mp = 0; mp < 3; ++mp) {
            R w = R(0);
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                if (k >= dB || j >= dA) continue;
                const R la = gradA ? C[mp + 3 * j] : (j == mp ? R(1) : R(0));
                w += Dm[k][j] * la;
            }
            W[k][mp] = w;
        }
#pragma unroll
    for (int m = 0; m < 3; ++m)
#pragma unroll
        for (int mp = 0; mp < 3; ++mp) {
            if (m >= rB || mp >= rA || (SYM && mp < m)) continue;
            R v = R(0);
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                if (k >= dB) continue;
                const R lb = gradB ? C[m + 3 * k] : (k == m ? R(1) : R(0));
                v += lb * W[k][mp];
            }
            const int c = RS == 9 ? 3 * m + mp : RS == 6 ? 3 * m - m * (m - 1) / 2 + mp - m : RS == 3 ? m + mp : 0;
            M[c] = scale * v;
        }
}

// M of tet t in FP64 (the parity arithmetic)
template <int RS, bool SYM>
__device__ __forceinline__ void reft_m64(const double* X, int64_t t, int kind, const double* D, int dA, int dB,
                                         int gradA, int gradB, int face, double (&M)[RS]) {
    double C[9];
    double scale;
    if (face >= 0 && !gradA && !gradB) {
        scale = face_area(X, face);  // face integral of values: no Jacobian needed
    } else {
        double e[9];
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
            for (int i = 0; i < 3; ++i) e[i + 3 * c] = X[3 * (c + 1) + i] - X[i];
        const double det = cofactors_of(e, C);
        const double mes = face >= 0 ? face_area(X, face) : fabs(det) / 6.0;
        const double inv = 1.0 / det;
        scale = mes * (gradA ? inv : 1.0) * (gradB ? inv : 1.0);
    }
    double Dm[3][3];
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int j = 0; j < 3; ++j) Dm[k][j] = (k < dB && j < dA) ? tensor_at(kind, D, t, 0, 1, dA, dB, k, j) : 0.0;
    reft_m<double, RS, SYM>(C, scale, Dm, dA, dB, gradA, gradB, M);
}

// M of tet t for FP32 output: edges in FP64 (nine subtractions), everything after them in FP32
// (FP64 -> FP32 by the integer conversion); a badly shaped tet (|det| <= 0.05 |e1||e2||e3|) is
// redone in FP64
template <int RS, bool SYM>
__device__ __forceinline__ void reft_m32(const double* X, int64_t t, int kind, const double* D, int dA, int dB,
                                         int gradA, int gradB, int face, float (&M)[RS]) {
    float e[9], C[9];
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int i = 0; i < 3; ++i) e[i + 3 * c] = d2f_rn(X[3 * (c + 1) + i] - X[i]);
    const float det = cofactors_of(e, C);
    const float l0 = e[0] * e[0] + e[1] * e[1] + e[2] * e[2];
    const float l1 = e[3] * e[3] + e[4] * e[4] + e[5] * e[5];
    const float l2 = e[6] * e[6] + e[7] * e[7] + e[8] * e[8];
    if (det * det > 0.0025f * l0 * l1 * l2) {
        const float mes = face >= 0 ? d2f_rn(face_area(X, face)) : fabsf(det) * (1.0f / 6.0f);
        const float inv = 1.0f / det;
        const float scale = mes * (gradA ? inv : 1.0f) * (gradB ? inv : 1.0f);
        float Dm[3][3];
#pragma unroll
        for (int k = 0; k < 3; ++k)
#pragma unroll
            for (int j = 0; j < 3; ++j)
                Dm[k][j] = (k < dB && j < dA) ? d2f_rn(tensor_at(kind, D, t, 0, 1, dA, dB, k, j)) : 0.0f;
        reft_m<float, RS, SYM>(C, scale, Dm, dA, dB, gradA, gradB, M);
    } else {
        double M64[RS];
        reft_m64<RS, SYM>(X, t, kind, D, dA, dB, gradA, gradB, face, M64);
#pragma unroll
        for (int k = 0; k < RS; ++k) M[k] = __double2float_rn(M64[k]);
    }
}

// The same reference-tensor form with lanes over tets: every thread forms the M of one tet in
// registers, and the 16 lanes of a half-warp walk the entries in the same order (uniform loads
// and branches within the half-warp).
// FP32: dense rows of T read as broadcast vectors.  FP64 (bound by the FP64 FMA rate): only the
// non-zero terms of T, a flat list of (value, code) with code = m-index | last-term flag << 4 |
// ib << 8 | ia << 20 -- the exact zeros of the reference tensor (about half of them for P2) cost
// nothing.  A warp owns 32 tets and works on them in two halves of 16: each half-warp takes one
// part of the entry list for all 16 tets (M passed by shuffle); the entries are staged in shared
// memory (row stride nent + 1) and written out as one contiguous, coalesced range of 16 element
// matrices.
template <int RS>
__device__ __forceinline__ double select_m(const double (&M)[RS], int k) {
    double v = M[0];
#pragma unroll
    for (int j = 1; j < RS; ++j) v = k == j ? M[j] : v;
    return v;
}

template <typename Real, int RS, bool SYM>
__global__ void __launch_bounds__(128) fem3dtet_reftensor_lanes_kernel(int64_t nt, const double* __restrict__ XY,
                                                                       int kind, const double* __restrict__ D, int dA,
                                                                       int dB, int gradA, int gradB, int nfA, int nfB,
                                                                       int face, int nlist, const double* __restrict__ T,
                                                                       Real* __restrict__ A) {
    extern __shared__ __align__(16) double lsm[];
    constexpr int RSP = (RS + 3) & ~3;
    constexpr bool LIST = sizeof(Real) == 8;
    const int nent = nfA * nfB, ostride = nent + 1;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // FP32: nlist rows of RSP values, then nlist codes (ib | ia << 16); FP64: four groups of nlist
    // terms, their values, then their codes
    Real* sT = reinterpret_cast<Real*>(lsm);
    const int nval = LIST ? 4 * nlist : nlist * RSP;
    const int ncode = LIST ? 4 * nlist : nlist;
    uint32_t* sCode = reinterpret_cast<uint32_t*>(sT + nval);
    Real* sOut = reinterpret_cast<Real*>(lsm + (((size_t)nval * sizeof(Real) + 4 * (size_t)ncode + 15) / 16) * 2) +
                 (size_t)warp * 16 * ostride;
    for (int i = threadIdx.x; i < nval; i += blockDim.x) sT[i] = Real(T[i]);
    for (int i = threadIdx.x; i < ncode; i += blockDim.x) sCode[i] = (uint32_t)T[nval + i];
    __syncthreads();
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t wbase = (int64_t)blockIdx.x * blockDim.x + warp * 32; wbase < nt; wbase += stride) {
        const int64_t t = wbase + lane;
        const int64_t tc = t < nt ? t : nt - 1;  // lanes past the end compute the last tet again
        // M of this lane's tet; then two halves of 16 tets: lane l works on tet (l & 15) of the
        // half, on the first (l < 16) or second part of the entry list, with that tet's M shuffled
        // from its owner
        Real Mo[RS];
        if constexpr (LIST) {
            double M64[RS];
            reft_m64<RS, SYM>(XY + 12 * tc, tc, kind, D, dA, dB, gradA, gradB, face, M64);
#pragma unroll
            for (int k = 0; k < RS; ++k) Mo[k] = M64[k];
        } else {
            float M32[RS];
            reft_m32<RS, SYM>(XY + 12 * tc, tc, kind, D, dA, dB, gradA, gradB, face, M32);
#pragma unroll
            for (int k = 0; k < RS; ++k) Mo[k] = M32[k];
        }
        const int part = lane >> 4;
        Real* myOut = sOut + (size_t)(lane & 15) * ostride;
        for (int half = 0; half < 2; ++half) {
            Real M[RS];
#pragma unroll
            for (int k = 0; k < RS; ++k) M[k] = __shfl_sync(0xffffffffu, Mo[k], (lane & 15) + 16 * half);
            if constexpr (LIST) {
                // two independent streams per lane over its part's two term groups (rows split
                // into four groups of equal padded length; padding terms are zeros without a row end)
                double s0 = 0.0, s1 = 0.0;
                const uint32_t* c0 = sCode + (2 * part) * nlist;
                const uint32_t* c1 = c0 + nlist;
                const Real* v0 = sT + (2 * part) * nlist;
                const Real* v1 = v0 + nlist;
                for (int j = 0; j < nlist; ++j) {
                    const uint32_t a = c0[j], b = c1[j];
                    s0 = fma(select_m<RS>(M, (int)(a & 15u)), (double)v0[j], s0);
                    s1 = fma(select_m<RS>(M, (int)(b & 15u)), (double)v1[j], s1);
                    if (a & 16u) {
                        const int ib = (a >> 8) & 0xfff, ia = a >> 20;
                        myOut[ib + nfB * ia] = Real(s0);
                        if (SYM) myOut[ia + nfB * ib] = Real(s0);
                        s0 = 0.0;
                    }
                    if (b & 16u) {
                        const int ib = (b >> 8) & 0xfff, ia = b >> 20;
                        myOut[ib + nfB * ia] = Real(s1);
                        if (SYM) myOut[ia + nfB * ib] = Real(s1);
                        s1 = 0.0;
                    }
                }
            } else {
                const int hrows = (nlist + 1) >> 1;
                const int e0 = part * hrows;
#pragma unroll 4
                for (int r = 0; r < hrows; ++r) {
                    const int e = e0 + r;
                    if (e >= nlist) break;
                    const Real* Te = sT + (size_t)e * RSP;
                    Real tv[RSP];
#pragma unroll
                    for (int q = 0; q < RSP / 4; ++q) {
                        const float4 w = reinterpret_cast<const float4*>(Te)[q];
                        tv[4 * q] = w.x;
                        tv[4 * q + 1] = w.y;
                        tv[4 * q + 2] = w.z;
                        tv[4 * q + 3] = w.w;
                    }
                    Real acc = M[0] * tv[0];
#pragma unroll
                    for (int k = 1; k < RS; ++k) acc = fma(M[k], tv[k], acc);
                    const uint32_t code = sCode[e];
                    const int ib = code & 0xffff, ia = code >> 16;
                    myOut[ib + nfB * ia] = acc;
                    if (SYM) myOut[ia + nfB * ib] = acc;
                }
            }
            __syncwarp();
            const int64_t hbase = wbase + 16 * half;
            const int ntw = (int)(nt - hbase < 16 ? (nt - hbase > 0 ? nt - hbase : 0) : 16);
            Real* gout = A + (size_t)nent * hbase;
            int tl = lane / nent, el = lane - tl * nent;
            const int step_t = 32 / nent, step_e = 32 - step_t * nent;
            for (int idx = lane; idx < ntw * nent; idx += 32) {
                gout[idx] = sOut[(size_t)tl * ostride + el];
                tl += step_t;
                el += step_e;
                if (el >= nent) {
                    el -= nent;
                    ++tl;
                }
            }
            __syncwarp();
        }
    }
}

__global__ void quad_points_kernel(int64_t nt, int q, const double* __restrict__ pts, const double* __restrict__ XY,
                                   double* __restrict__ XYG) {
    const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (idx >= nt * q) return;
    const int64_t t = idx / q;
    const int n = (int)(idx - t * q);
    const double* X = XY + 12 * t;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        double s = X[k];
#pragma unroll
        for (int l = 0; l < 3; ++l) s += pts[l + 1 + 4 * n] * (X[3 * (l + 1) + k] - X[k]);
        XYG[3 * idx + k] = s;
    }
}

// Ani::applyDir (dc_on_dof.h:39-45), ascending local k
__global__ void apply_dir_kernel(int64_t nt, int n, double* __restrict__ A, double* __restrict__ F,
                                 const uint32_t* __restrict__ mask, const double* __restrict__ bc) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= nt) return;
    double* At = A + (size_t)n * n * t;
    double* Ft = F + (size_t)n * t;
    const uint32_t m = mask[t];
    for (int k = 0; k < n; ++k) {
        if (!((m >> k) & 1u)) continue;
        const double b = bc ? bc[(size_t)n * t + k] : 0.0;
        for (int i = 0; i < n; ++i) Ft[i] -= At[i + n * k] * b;
        Ft[k] = b;
        for (int i = 0; i < n; ++i) At[i + n * k] = 0.0;
        for (int i = 0; i < n; ++i) At[k + n * i] = 0.0;
        At[k + n * k] = 1.0;
    }
}

// ---------------------------------------------------------------- evaluation of Op(u)
// Ani::fem3DapplyL / fem3DapplyX (anifem++/fem/operations/eval.inl:93-151 -> core.inl:370-404):
// Op(u) at points of each tet, opU[t][n][k].  One thread per tet: its geometry (PSI) once, its
// DOF values once, then per point the barycentric coordinates (given, or from a physical point
// through PSI as getBaryCoord does, core.inl:120-137) and the scalar basis there.  GRAD of a
// Lagrange space combines the reference gradients with the DOF values first and maps the sum
// with PSI^T once (3x3 instead of 3x3 per DOF; the same value up to rounding).
struct ApplyParams {
    int nf, dim, nfs, ncomp, op, base;
    int npts, phys;           // phys: pts are per-tet physical points [nt][npts][3]
    const double* pts;        // barycentric [npts][4] when !phys
    const double* XY;         // [nt][12], or null: the handle's mesh (xyz + oriented tets)
    const double* xyz;
    const int32_t* tets;
    const double* dofs;       // [nt][nf], or null: the global vector x through the DOF table
    const double* x;
    const int32_t* edofs;     // [nt][nloc] scalar element DOFs
    const int8_t* sign;       // [nt][nloc] orientation signs of the global DOFs (oriented spaces) or null
    int nloc;
    int64_t nds;              // scalar DOFs (component c of scalar DOF s is c*nds + s)
    double* out;
};

__global__ void __launch_bounds__(128) fem3d_apply_kernel(ApplyParams p, int64_t nt) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= nt) return;
    double X[12];
    if (p.XY) {
#pragma unroll
        for (int k = 0; k < 12; ++k) X[k] = p.XY[12 * t + k];
    } else {
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            const int64_t node = p.tets[4 * t + v];
#pragma unroll
            for (int i = 0; i < 3; ++i) X[3 * v + i] = p.xyz[3 * node + i];
        }
    }
    double PSI[9], mes, det;
    tet_geometry(X, PSI, &mes, &det);
    double d[ANIGPU_MAX_NF];
    for (int c = 0; c < p.ncomp; ++c)
        for (int i = 0; i < p.nfs; ++i)
            d[c * p.nfs + i] = p.dofs ? p.dofs[(int64_t)p.nf * t + c * p.nfs + i]
                                      : p.x[c * p.nds + p.edofs[(int64_t)p.nloc * t + i]] *
                                            (p.sign ? (double)p.sign[(int64_t)p.nloc * t + i] : 1.0);
    const bool vec = p.base == ANIGPU_ND0 || p.base == ANIGPU_RT0;
    double P[12];
    if (vec) {
#pragma unroll
        for (int v = 0; v < 4; ++v)
#pragma unroll
            for (int i = 0; i < 3; ++i) P[3 * v + i] = v == 0 ? 0.0 : X[3 * v + i] - X[i];
    }
    for (int n = 0; n < p.npts; ++n) {
        double l[4];
        if (p.phys) {
            const double* x = p.pts + 3 * ((int64_t)p.npts * t + n);
            const double dr[3] = {x[0] - X[0], x[1] - X[1], x[2] - X[2]};
            l[1] = l[2] = l[3] = 0.0;
#pragma unroll
            for (int j = 0; j < 3; ++j)
#pragma unroll
                for (int i = 0; i < 3; ++i) l[i + 1] += PSI[i + 3 * j] * dr[j];
            l[0] = 1.0 - l[1] - l[2] - l[3];
        } else {
#pragma unroll
            for (int k = 0; k < 4; ++k) l[k] = p.pts[4 * n + k];
        }
        double* o = p.out + ((int64_t)p.npts * t + n) * p.dim;
        if (vec) {  // vector-valued, from the tet geometry
            for (int k = 0; k < p.dim; ++k) {
                double s = 0.0;
                for (int i = 0; i < p.nf; ++i) s += ani_vec_space_value(p.base, p.op, l, PSI, P, det, i, k) * d[i];
                o[k] = s;
            }
            continue;
        }
        double v[20], g[20][3];
        ani_eval_space(p.base, l, v, g);
        for (int c = 0; c < p.ncomp; ++c) {
            const double* dc = d + c * p.nfs;
            if (p.op == ANIGPU_IDEN) {
                double s = 0.0;
                for (int i = 0; i < p.nfs; ++i) s += v[i] * dc[i];
                o[c] = s;
            } else {
                double r0 = 0.0, r1 = 0.0, r2 = 0.0;  // reference gradient of u
                for (int i = 0; i < p.nfs; ++i) {
                    r0 += g[i][0] * dc[i];
                    r1 += g[i][1] * dc[i];
                    r2 += g[i][2] * dc[i];
                }
#pragma unroll
                for (int k = 0; k < 3; ++k) o[3 * c + k] = PSI[0 + 3 * k] * r0 + PSI[1 + 3 * k] * r1 + PSI[2 + 3 * k] * r2;
            }
        }
    }
}

template <int BASE>
struct LagrangeNf {
    static constexpr int value = BASE == ANIGPU_P0 ? 1 : BASE == ANIGPU_P1 ? 4 : BASE == ANIGPU_P2 ? 10
                               : BASE == ANIGPU_P3 ? 20 : BASE == ANIGPU_CR1 ? 4 : BASE == ANIGPU_B2 ? 6 : 1;
};

// values and reference gradients of the basis at shared barycentric points: table[n][4 * NFS]
// (NFS values, then 3 NFS gradient entries)
template <int BASE>
__global__ void basis_table_kernel(int npts, const double* __restrict__ pts, double* __restrict__ table) {
    constexpr int NFS = LagrangeNf<BASE>::value;
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= npts) return;
    double v[NFS], g[NFS][3];
    ani_eval_space(BASE, pts + 4 * n, v, g);
    double* o = table + (size_t)4 * NFS * n;
#pragma unroll
    for (int i = 0; i < NFS; ++i) {
        o[i] = v[i];
#pragma unroll
        for (int d = 0; d < 3; ++d) o[NFS + 3 * i + d] = g[i][d];
    }
}

// Lagrange-type spaces with the base space known at compile time: basis values, reference
// gradients and DOF values in registers; with a table (shared barycentric points) the basis is
// read from shared memory instead of evaluated per tet
template <int BASE>
__global__ void __launch_bounds__(128) fem3d_apply_lagrange_kernel(ApplyParams p, int64_t nt, const double* table) {
    constexpr int NFS = LagrangeNf<BASE>::value;
    extern __shared__ double sTab[];
    if (table) {
        for (int k = threadIdx.x; k < 4 * NFS * p.npts; k += blockDim.x) sTab[k] = table[k];
        __syncthreads();
    }
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= nt) return;
    double X[12];
    if (p.XY) {
#pragma unroll
        for (int k = 0; k < 12; ++k) X[k] = p.XY[12 * t + k];
    } else {
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            const int64_t node = p.tets[4 * t + v];
#pragma unroll
            for (int i = 0; i < 3; ++i) X[3 * v + i] = p.xyz[3 * node + i];
        }
    }
    double PSI[9], mes, det;
    tet_geometry(X, PSI, &mes, &det);
    for (int c = 0; c < p.ncomp; ++c) {
        double d[NFS];
#pragma unroll
        for (int i = 0; i < NFS; ++i)
            d[i] = p.dofs ? p.dofs[(int64_t)p.nf * t + c * NFS + i]
                          : p.x[c * p.nds + p.edofs[(int64_t)p.nloc * t + i]] *
                                (p.sign ? (double)p.sign[(int64_t)p.nloc * t + i] : 1.0);
        for (int n = 0; n < p.npts; ++n) {
            double l[4];
            if (p.phys) {
                const double* x = p.pts + 3 * ((int64_t)p.npts * t + n);
                const double dr[3] = {x[0] - X[0], x[1] - X[1], x[2] - X[2]};
                l[1] = l[2] = l[3] = 0.0;
#pragma unroll
                for (int j = 0; j < 3; ++j)
#pragma unroll
                    for (int i = 0; i < 3; ++i) l[i + 1] += PSI[i + 3 * j] * dr[j];
                l[0] = 1.0 - l[1] - l[2] - l[3];
            } else {
#pragma unroll
                for (int k = 0; k < 4; ++k) l[k] = p.pts[4 * n + k];
            }
            double v[NFS], g[NFS][3];
            if (table) {
                const double* row = sTab + 4 * NFS * n;
#pragma unroll
                for (int i = 0; i < NFS; ++i) {
                    v[i] = row[i];
#pragma unroll
                    for (int dd = 0; dd < 3; ++dd) g[i][dd] = row[NFS + 3 * i + dd];
                }
            } else {
                ani_eval_space(BASE, l, v, g);
            }
            double* o = p.out + ((int64_t)p.npts * t + n) * p.dim;
            if (p.op == ANIGPU_IDEN) {
                double sv = 0.0;
#pragma unroll
                for (int i = 0; i < NFS; ++i) sv += v[i] * d[i];
                o[c] = sv;
            } else {
                double r0 = 0.0, r1 = 0.0, r2 = 0.0;  // reference gradient of u
#pragma unroll
                for (int i = 0; i < NFS; ++i) {
                    r0 += g[i][0] * d[i];
                    r1 += g[i][1] * d[i];
                    r2 += g[i][2] * d[i];
                }
#pragma unroll
                for (int k = 0; k < 3; ++k) o[3 * c + k] = PSI[0 + 3 * k] * r0 + PSI[1 + 3 * k] * r1 + PSI[2 + 3 * k] * r2;
            }
        }
    }
}

}  // namespace

int get_basis_dev(anigpu_ctx* h, int space, int order, const double** dev, ScalarBasisTable* host, int face) {
    ScalarBasisTable tab;
    const bool ok = face < 0 ? make_scalar_basis(space, order, &tab) : make_scalar_basis_face(space, order, face, &tab);
    if (!ok) return set_err(h, ANIGPU_ERR_UNSUPPORTED, "unsupported space/order");
    if (host) *host = tab;
    const int key = 100 * space + order + 10000 * (face + 1);
    for (auto& kv : h->basis_dev)
        if (kv.first == key) {
            *dev = kv.second;
            return ANIGPU_OK;
        }
    std::vector<double> buf;
    buf.insert(buf.end(), tab.val.begin(), tab.val.end());
    buf.insert(buf.end(), tab.grad.begin(), tab.grad.end());
    buf.insert(buf.end(), tab.wts.begin(), tab.wts.end());
    buf.insert(buf.end(), tab.pts.begin(), tab.pts.end());
    double* d = nullptr;
    ANI_CUDA(h, cudaMalloc((void**)&d, buf.size() * sizeof(double)));
    ANI_CUDA(h, cudaMemcpy(d, buf.data(), buf.size() * sizeof(double), cudaMemcpyHostToDevice));
    h->basis_dev.push_back({key, d});
    *dev = d;
    return ANIGPU_OK;
}

// reference tensors T(ib, ia, m, m') = sum_n w_n Vhat_n(m, ib) Uhat_n(m', ia) of a scalar operator
// pair on the rule of `order` (over face `face` when face >= 0), cached per handle in the layout of
// the kernel that uses them; then the kernel: lanes over tets for element matrices of at most
// kLanesMaxEnt entries, lanes over entries above
constexpr int kLanesMaxEnt = 100;

template <typename Real, int RS, bool SYM>
static int run_lanes(anigpu_ctx* h, unsigned grid, size_t smem, int64_t nt, const double* XY, int kind, const double* D,
                     int dA, int dB, int gradA, int gradB, int nfA, int nfB, int face, int nlist, const double* T,
                     void* A) {
    auto kern = fem3dtet_reftensor_lanes_kernel<Real, RS, SYM>;
    ANI_CUDA(h, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kern<<<grid, 128, smem, h->stream>>>(nt, XY, kind, D, dA, dB, gradA, gradB, nfA, nfB, face, nlist, T, (Real*)A);
    return ANIGPU_OK;
}

static int launch_reftensor(anigpu_ctx* h, int opA, int opB, int order, int face, const ScalarBasisTable& hA,
                            const ScalarBasisTable& hB, int kind, int precision, int64_t nt, const double* XY,
                            const double* D, void* A) {
    const int gradA = opA % 10 == ANIGPU_GRAD, gradB = opB % 10 == ANIGPU_GRAD;
    const int rA = gradA ? 3 : 1, rB = gradB ? 3 : 1, rr = rA * rB;
    const int nfA = hA.nf, nfB = hB.nf, q = hA.q;
    const int dA = gradA ? 3 : 1, dB = gradB ? 3 : 1;
    const bool f32 = precision == ANIGPU_F32;
    // same operator and a symmetric tensor: symmetric element matrix (upper triangle only)
    const int sym = opA == opB && (kind == ANIGPU_TENSOR_NULL || kind == ANIGPU_TENSOR_CONST_SCALAR ||
                                   kind == ANIGPU_TENSOR_TET_SCALAR || kind == ANIGPU_TENSOR_TET_SYM);
    const int rs = sym ? (rA == 3 ? 6 : 1) : rr;
    const int nrow = sym ? nfA * (nfA + 1) / 2 : nfA * nfB;
    const bool lanes = nfA * nfB <= kLanesMaxEnt;
    const int layout = lanes ? (f32 ? 1 : 2) : 0;
    const int key = -(1 + opA + 128 * (opB + 128 * (order + 32 * (face + 1 + 8 * (sym + 2 * layout)))));
    const int rsp = (rs + 3) & ~3;
    const double* T = nullptr;
    int nlist = 0;
    for (auto& kv : h->basis_dev)
        if (kv.first == key) T = kv.second;
    for (auto& kv : h->reft_len)
        if (kv.first == key) nlist = kv.second;
    if (!T) {
        std::vector<double> hT((size_t)nfA * nfB * rr, 0.0);
        for (int ia = 0; ia < nfA; ++ia)
            for (int ib = 0; ib < nfB; ++ib)
                for (int m = 0; m < rB; ++m)
                    for (int mp = 0; mp < rA; ++mp) {
                        double s = 0.0;
                        for (int n = 0; n < q; ++n) {
                            const double vb = gradB ? hB.grad[((size_t)n * nfB + ib) * 3 + m] : hB.val[(size_t)n * nfB + ib];
                            const double ua = gradA ? hA.grad[((size_t)n * nfA + ia) * 3 + mp] : hA.val[(size_t)n * nfA + ia];
                            s += hA.wts[n] * vb * ua;
                        }
                        hT[((size_t)ib + (size_t)nfB * ia) * rr + m * rA + mp] = s;
                    }
        // rows: (ib, ia) and rs coefficients of M; symmetric: pairs ib <= ia, off-diagonal M terms
        // carrying T(m, m') + T(m', m)
        std::vector<double> rows((size_t)nrow * rs);
        std::vector<uint32_t> rcode(nrow);
        if (sym) {
            int pr = 0;
            for (int ia = 0; ia < nfA; ++ia)
                for (int ib = 0; ib <= ia; ++ib, ++pr) {
                    const double* Te = &hT[((size_t)ib + (size_t)nfB * ia) * rr];
                    int c = 0;
                    for (int m = 0; m < rB; ++m)
                        for (int mp = m; mp < rA; ++mp)
                            rows[(size_t)pr * rs + c++] = mp == m ? Te[m * rA + m] : Te[m * rA + mp] + Te[mp * rA + m];
                    rcode[pr] = (uint32_t)(ib | (ia << 16));
                }
        } else {
            for (int e = 0; e < nrow; ++e) {
                std::copy(&hT[(size_t)e * rr], &hT[(size_t)e * rr] + rr, &rows[(size_t)e * rs]);
                rcode[e] = (uint32_t)((e % nfB) | ((e / nfB) << 16));
            }
        }
        std::vector<double> out;
        if (layout == 0) {
            out = rows;
            if (sym)
                for (int e = 0; e < nrow; ++e) out.push_back((double)rcode[e]);
        } else if (layout == 1) {
            out.assign((size_t)nrow * rsp, 0.0);
            for (int e = 0; e < nrow; ++e)
                for (int k = 0; k < rs; ++k) out[(size_t)e * rsp + k] = rows[(size_t)e * rs + k];
            for (int e = 0; e < nrow; ++e) out.push_back((double)rcode[e]);
        } else {
            // non-zero terms only (a row with none keeps one zero term, so that it is written); the
            // rows split into four consecutive groups of about equal term count, each padded with
            // zero terms (no row end) to the longest group's length
            double tmax = 0.0;
            for (double v : rows) tmax = std::max(tmax, std::fabs(v));
            std::vector<double> vals;
            std::vector<uint32_t> codes;
            std::vector<size_t> row_end(nrow);
            for (int e = 0; e < nrow; ++e) {
                const uint32_t ib = rcode[e] & 0xffffu, ia = rcode[e] >> 16;
                const size_t first = vals.size();
                for (int k = 0; k < rs; ++k) {
                    const double v = rows[(size_t)e * rs + k];
                    if (std::fabs(v) <= 1e-14 * tmax) continue;
                    vals.push_back(v);
                    codes.push_back((uint32_t)k | (ib << 8) | (ia << 20));
                }
                if (vals.size() == first) {
                    vals.push_back(0.0);
                    codes.push_back((ib << 8) | (ia << 20));
                }
                codes.back() |= 16u;
                row_end[e] = vals.size();
            }
            size_t gb[5] = {0, 0, 0, 0, vals.size()};
            for (int g = 1; g < 4; ++g) {
                const size_t target = vals.size() * g / 4;
                size_t b = gb[g - 1];
                for (int e = 0; e < nrow; ++e)
                    if (row_end[e] <= target) b = std::max(b, row_end[e]);
                gb[g] = b;
            }
            size_t L = 1;
            for (int g = 0; g < 4; ++g) L = std::max(L, gb[g + 1] - gb[g]);
            out.assign(8 * L, 0.0);
            for (int g = 0; g < 4; ++g)
                for (size_t j = gb[g]; j < gb[g + 1]; ++j) {
                    out[g * L + (j - gb[g])] = vals[j];
                    out[4 * L + g * L + (j - gb[g])] = (double)codes[j];
                }
            nlist = (int)L;
            h->reft_len.push_back({key, nlist});
        }
        double* d = nullptr;
        ANI_CUDA(h, cudaMalloc((void**)&d, out.size() * sizeof(double)));
        ANI_CUDA(h, cudaMemcpy(d, out.data(), out.size() * sizeof(double), cudaMemcpyHostToDevice));
        h->basis_dev.push_back({key, d});
        T = d;
    }
    if (layout == 1) nlist = nrow;
    int dev_sms = 148;
    cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, h->device);
    const size_t rsz = f32 ? sizeof(float) : sizeof(double);
    constexpr int kRT = 128;
    int rc = ANIGPU_OK;
    if (lanes) {
        const size_t nval = f32 ? (size_t)nlist * rsp : 4 * (size_t)nlist;
        const size_t ncode = f32 ? (size_t)nlist : 4 * (size_t)nlist;
        const size_t smem = (nval * rsz + 4 * ncode + 15) / 16 * 16 + rsz * (size_t)(kRT / 2) * (nfA * nfB + 1);
        const unsigned grid = (unsigned)std::min<int64_t>((nt + kRT - 1) / kRT, (int64_t)dev_sms * 16);
#define RUN_LANES(R, RSV, SY) \
    rc = run_lanes<R, RSV, SY>(h, grid, smem, nt, XY, kind, D, dA, dB, gradA, gradB, nfA, nfB, face, nlist, T, A)
        if (f32) {
            if (rs == 1) { if (sym) RUN_LANES(float, 1, true); else RUN_LANES(float, 1, false); }
            else if (rs == 3) RUN_LANES(float, 3, false);
            else if (rs == 6) RUN_LANES(float, 6, true);
            else RUN_LANES(float, 9, false);
        } else {
            if (rs == 1) { if (sym) RUN_LANES(double, 1, true); else RUN_LANES(double, 1, false); }
            else if (rs == 3) RUN_LANES(double, 3, false);
            else if (rs == 6) RUN_LANES(double, 6, true);
            else RUN_LANES(double, 9, false);
        }
#undef RUN_LANES
        if (rc) return rc;
    } else {
        const size_t smem = rsz * ((size_t)nrow * rs + (size_t)kRT * 9 + (size_t)(kRT / 32) * nfA * nfB) +
                            (sym ? sizeof(int) * nrow : 0);
        const unsigned grid = (unsigned)std::min<int64_t>((nt + kRT - 1) / kRT, (int64_t)dev_sms * 8);
        if (f32) {
            ANI_CUDA(h, cudaFuncSetAttribute(fem3dtet_reftensor_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            fem3dtet_reftensor_kernel<float><<<grid, kRT, smem, h->stream>>>(nt, XY, kind, D, dA, dB, gradA, gradB, nfA,
                                                                              nfB, face, sym, T, (float*)A);
        } else {
            ANI_CUDA(h, cudaFuncSetAttribute(fem3dtet_reftensor_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            fem3dtet_reftensor_kernel<double><<<grid, kRT, smem, h->stream>>>(nt, XY, kind, D, dA, dB, gradA, gradB, nfA,
                                                                               nfB, face, sym, T, (double*)A);
        }
    }
    ANI_LAUNCHED(h);
    return ANIGPU_OK;
}

static int run_quadrature(anigpu_ctx* h, const ElemParams& p, int precision, int64_t nt, const double* XY,
                          const double* D, void* A);

int launch_fem3dtet(anigpu_ctx* h, int opA, int opB, int kind, int order, int precision, int64_t nt,
                    const double* XY, const double* D, void* A, int face, int normal) {
    int nfA, dA, bsA, ncA, oA, nfB, dB, bsB, ncB, oB;
    if (!op_info(opA, &nfA, &dA, &bsA, &ncA, &oA) || !op_info(opB, &nfB, &dB, &bsB, &ncB, &oB))
        return set_err(h, ANIGPU_ERR_UNSUPPORTED, "unknown operator code");
    if (nt < 0) return set_err(h, ANIGPU_ERR_ARG, "nt < 0");
    if (nt == 0) return ANIGPU_OK;
    if (kind < ANIGPU_TENSOR_NULL || kind > ANIGPU_TENSOR_POINT)
        return set_err(h, ANIGPU_ERR_UNSUPPORTED, "tensor kind");
    const int dBt = normal ? 3 * dB : dB;  // rows of the tensor the caller supplies
    if (normal && face < 0) return set_err(h, ANIGPU_ERR_ARG, "the normal needs a face");
    if (kind == ANIGPU_TENSOR_TET_SYM && (dA != 3 || dBt != 3))
        return set_err(h, ANIGPU_ERR_ARG, "TET_SYM needs 3x3 operators");
    if ((kind == ANIGPU_TENSOR_NULL || kind == ANIGPU_TENSOR_CONST_SCALAR || kind == ANIGPU_TENSOR_TET_SCALAR) &&
        dA != dBt && !(nfA == 1 && dA == 1))
        // diff_tensor.h:314-317: identity defined only for operators of the same dimension
        return set_err(h, ANIGPU_ERR_ARG, "Identity tensor defined only for compatible operators A and B");
    if (kind != ANIGPU_TENSOR_NULL && D == nullptr) return set_err(h, ANIGPU_ERR_ARG, "tensor data is NULL");
    if (!XY || !A) return set_err(h, ANIGPU_ERR_ARG, "NULL coordinates or output");
    const double *tA, *tB;
    ScalarBasisTable hA;
    const bool vecA = bsA == ANIGPU_ND0 || bsA == ANIGPU_RT0, vecB = bsB == ANIGPU_ND0 || bsB == ANIGPU_RT0;
    if (face > 3) return set_err(h, ANIGPU_ERR_ARG, "face number must be 0..3");
    int rc = get_basis_dev(h, vecA ? ANIGPU_P1 : bsA, order, &tA, &hA, face);
    if (rc) return rc;
    ScalarBasisTable hB;
    rc = get_basis_dev(h, vecB ? ANIGPU_P1 : bsB, order, &tB, &hB, face);
    if (rc) return rc;
    if (precision != ANIGPU_F32 && precision != ANIGPU_F64) return set_err(h, ANIGPU_ERR_ARG, "precision");
    if (!vecA && !vecB && ncA == 1 && ncB == 1 && !normal && kind != ANIGPU_TENSOR_POINT)
        return launch_reftensor(h, opA, opB, order, face, hA, hB, kind, precision, nt, XY, D, A);
    ElemParams p{};
    p.A = {nfA, dA, nfA / ncA, dA / ncA, ncA, oA, bsA, vecA ? 4 : nfA / ncA, tA, nullptr};
    p.B = {nfB, dB, nfB / ncB, dB / ncB, ncB, oB, bsB, vecB ? 4 : nfB / ncB, tB, nullptr};
    p.q = hA.q;
    p.kind = kind;
    p.face = face;
    p.normal = normal ? 1 : 0;
    p.w = tA + (size_t)hA.q * hA.nf * 4;
    p.same = opA == opB ? 1 : 0;
    return run_quadrature(h, p, precision, nt, XY, D, A);
}

// the warp-per-tet quadrature kernel on prepared parameters
static int run_quadrature(anigpu_ctx* h, const ElemParams& p, int precision, int64_t nt, const double* XY,
                          const double* D, void* A) {
    const int nfA = p.A.nf, dA = p.A.dim, nfB = p.B.nf, dB = p.B.dim;
    const size_t tabs = (size_t)p.q * (p.A.tnf + p.B.tnf) * 4;
    const size_t rsz = precision == ANIGPU_F32 ? sizeof(float) : sizeof(double);
    // per-warp region in doubles: geometry 26, tensor MAX_DIM^2, then U, V, DU and the entries
    const size_t wreal = (size_t)dA * nfA + (p.same ? 0 : (size_t)dB * nfB) + (size_t)dB * nfA + (size_t)nfA * nfB;
    const int wstride = (int)((26 + ANIGPU_MAX_DIM * ANIGPU_MAX_DIM) + (wreal * rsz + 7) / 8 + 1) & ~1;
    ElemParams pk = p;
    size_t smem = sizeof(double) * (tabs + p.q + (size_t)(kThreads / 32) * wstride);
    pk.tab_shared = smem <= 96 * 1024 ? 1 : 0;
    if (!pk.tab_shared) smem = sizeof(double) * (p.q + (size_t)(kThreads / 32) * wstride);
    if (smem > 227 * 1024) return set_err(h, ANIGPU_ERR_UNSUPPORTED, "element matrices too large for one warp's shared memory");
    int dev_sms = 148;
    cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, h->device);
    const unsigned grid = (unsigned)std::min<int64_t>((nt + kThreads / 32 - 1) / (kThreads / 32), (int64_t)dev_sms * 16);
    if (precision == ANIGPU_F32) {
        ANI_CUDA(h, cudaFuncSetAttribute(fem3dtet_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        fem3dtet_kernel<float><<<grid, kThreads, smem, h->stream>>>(pk, nt, XY, D, (float*)A, wstride);
    } else if (precision == ANIGPU_F64) {
        ANI_CUDA(h, cudaFuncSetAttribute(fem3dtet_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        fem3dtet_kernel<double><<<grid, kThreads, smem, h->stream>>>(pk, nt, XY, D, (double*)A, wstride);
    } else {
        return set_err(h, ANIGPU_ERR_ARG, "precision");
    }
    ANI_LAUNCHED(h);
    return ANIGPU_OK;
}

// fem3Dtet with user-defined operators (ApplyOpCustom, anifem++/fem/operators.h:450-471): the
// operators' values at the points of the rule of `order` come from the caller, per tet and point a
// dim x nf column-major matrix (UA[((t*q + n)*nf + i)*dim + k]); VB NULL: the B operator is A's
int launch_fem3dtet_custom(anigpu_ctx* h, int dimA, int nfA, const double* UA, int dimB, int nfB, const double* VB,
                           int kind, int order, int precision, int64_t nt, const double* XY, const double* D, void* A) {
    if (nt < 0) return set_err(h, ANIGPU_ERR_ARG, "nt < 0");
    if (dimA < 1 || dimA > ANIGPU_MAX_DIM || nfA < 1 || (VB && (dimB < 1 || dimB > ANIGPU_MAX_DIM || nfB < 1)))
        return set_err(h, ANIGPU_ERR_ARG, "operator dimensions: 1 <= dim <= 9, nf >= 1");
    if (!VB) {
        dimB = dimA;
        nfB = nfA;
    }
    if (nt == 0) return ANIGPU_OK;
    if (kind < ANIGPU_TENSOR_NULL || kind > ANIGPU_TENSOR_POINT) return set_err(h, ANIGPU_ERR_UNSUPPORTED, "tensor kind");
    if (kind == ANIGPU_TENSOR_TET_SYM && (dimA != 3 || dimB != 3)) return set_err(h, ANIGPU_ERR_ARG, "TET_SYM needs 3x3 operators");
    if ((kind == ANIGPU_TENSOR_NULL || kind == ANIGPU_TENSOR_CONST_SCALAR || kind == ANIGPU_TENSOR_TET_SCALAR) &&
        dimA != dimB && !(nfA == 1 && dimA == 1))
        return set_err(h, ANIGPU_ERR_ARG, "Identity tensor defined only for compatible operators A and B");
    if (kind != ANIGPU_TENSOR_NULL && D == nullptr) return set_err(h, ANIGPU_ERR_ARG, "tensor data is NULL");
    if (!XY || !A || !UA) return set_err(h, ANIGPU_ERR_ARG, "NULL coordinates, operator values or output");
    if (precision != ANIGPU_F32 && precision != ANIGPU_F64) return set_err(h, ANIGPU_ERR_ARG, "precision");
    const double* t1;
    ScalarBasisTable h1;
    int rc = get_basis_dev(h, ANIGPU_P1, order, &t1, &h1, -1);  // the rule's weights
    if (rc) return rc;
    ElemParams p{};
    p.A = {nfA, dimA, nfA, dimA, 1, 0, -1, 0, t1, UA};
    p.B = {nfB, dimB, nfB, dimB, 1, 0, -1, 0, t1, VB ? VB : UA};
    p.q = h1.q;
    p.kind = kind;
    p.face = -1;
    p.normal = 0;
    p.w = t1 + (size_t)h1.q * h1.nf * 4;
    p.same = VB ? 0 : 1;
    return run_quadrature(h, p, precision, nt, XY, D, A);
}

int launch_quad_points(anigpu_ctx* h, int order, int64_t nt, const double* XY, double* XYG, int face) {
    const double* tab;
    ScalarBasisTable host;
    if (face > 3) return set_err(h, ANIGPU_ERR_ARG, "face number must be 0..3");
    int rc = get_basis_dev(h, ANIGPU_P1, order, &tab, &host, face);
    if (rc) return rc;
    if (nt <= 0) return nt < 0 ? set_err(h, ANIGPU_ERR_ARG, "nt < 0") : ANIGPU_OK;
    const double* pts = tab + (size_t)host.q * host.nf * 4 + host.q;
    quad_points_kernel<<<grid_for(nt * host.q, 256), 256, 0, h->stream>>>(nt, host.q, pts, XY, XYG);
    ANI_LAUNCHED(h);
    return ANIGPU_OK;
}

int launch_apply_dir(anigpu_ctx* h, int64_t nt, int n, double* A, double* F, const uint32_t* mask, const double* bc) {
    if (n <= 0 || n > 32 || nt < 0 || !A || !F || !mask) return set_err(h, ANIGPU_ERR_ARG, "apply_dir arguments");
    if (nt == 0) return ANIGPU_OK;
    apply_dir_kernel<<<grid_for(nt, 128), 128, 0, h->stream>>>(nt, n, A, F, mask, bc);
    ANI_LAUNCHED(h);
    return ANIGPU_OK;
}

// Op(u) at points: per-tet coordinates and DOFs (XY, dofs non-null) or the handle's mesh and a
// global vector x (XY = dofs = null).
int launch_fem3d_apply(anigpu_ctx* h, int op, int64_t nt, const double* XY, int npts, const double* pts, int phys,
                       const double* dofs, const double* x, double* out) {
    int nf, dim, base, nc, o;
    if (!op_info(op, &nf, &dim, &base, &nc, &o)) return set_err(h, ANIGPU_ERR_UNSUPPORTED, "unknown operator code");
    if (nt < 0 || npts < 1) return set_err(h, ANIGPU_ERR_ARG, "nt < 0 or no points");
    if (!pts || !out) return set_err(h, ANIGPU_ERR_ARG, "NULL points or output");
    if (nt == 0) return ANIGPU_OK;
    ApplyParams p{};
    p.nf = nf;
    p.dim = dim;
    p.nfs = nf / nc;
    p.ncomp = nc;
    p.op = o;
    p.base = base;
    p.npts = npts;
    p.phys = phys;
    p.pts = pts;
    p.out = out;
    if (XY) {
        if (!dofs) return set_err(h, ANIGPU_ERR_ARG, "NULL element DOF values");
        p.XY = XY;
        p.dofs = dofs;
    } else {
        if (!h->tets || !h->edofs) return set_err(h, ANIGPU_ERR_STATE, "anigpu_problem_setup not called");
        if (!x) return set_err(h, ANIGPU_ERR_ARG, "NULL solution vector");
        p.xyz = h->xyz;
        p.tets = h->tets;
        p.x = x;
        p.edofs = h->edofs;
        p.sign = general_signs(h);  // null on the fast-path spaces
        p.nloc = h->nloc_s;
        p.nds = h->nds;
    }
    const unsigned g = grid_for(nt, 128);
    cudaStream_t st = h->stream;
    if (base == ANIGPU_ND0 || base == ANIGPU_RT0) {
        fem3d_apply_kernel<<<g, 128, 0, st>>>(p, nt);
        ANI_LAUNCHED(h);
        return ANIGPU_OK;
    }
    // shared barycentric points: the basis table once (when it fits in shared memory)
    const int nfs = p.nfs;
    const size_t tab_bytes = sizeof(double) * 4 * nfs * (size_t)npts;
    const bool use_table = !phys && tab_bytes <= 48 * 1024;
    double* table = nullptr;
    if (use_table) ANI_CUDA(h, cudaMallocAsync((void**)&table, tab_bytes, st));
    const size_t smem = use_table ? tab_bytes : 0;
#define APPLY_CASE(B)                                                                                   \
    case B:                                                                                             \
        if (use_table) {                                                                                \
            basis_table_kernel<B><<<grid_for(npts, 64), 64, 0, st>>>(npts, pts, table);                 \
            ANI_LAUNCHED(h);                                                                            \
        }                                                                                               \
        fem3d_apply_lagrange_kernel<B><<<g, 128, smem, st>>>(p, nt, table);                             \
        break;
    switch (base) {
        APPLY_CASE(ANIGPU_P0)
        APPLY_CASE(ANIGPU_P1)
        APPLY_CASE(ANIGPU_P2)
        APPLY_CASE(ANIGPU_P3)
        APPLY_CASE(ANIGPU_CR1)
        APPLY_CASE(ANIGPU_B2)
        APPLY_CASE(ANIGPU_B4)
    }
#undef APPLY_CASE
    ANI_LAUNCHED(h);
    if (table) ANI_CUDA(h, cudaFreeAsync(table, st));
    return ANIGPU_OK;
}
