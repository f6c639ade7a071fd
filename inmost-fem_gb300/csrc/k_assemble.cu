// Global assembly: GRAD.GRAD stiffness + P0 x IDEN right-hand side of a scalar
// Lagrange space, with element-level Dirichlet elimination, written straight into the
// CSR template.  Replaces the per-cell loop of AssemblerT::Assemble
// (anifem++/inmost_interface/assembler.inl:314-487) that calls fem3Dtet per cell and
// scatters into INMOST row lists.
//
// Formulation.  For a tensor that is constant on a tet (NULL, SCALAR, SYMMETRIC kinds)
// the quadrature sum of fem3Dtet factorises:
//     A_ij = sum_n w_n |T| (PSI^T g_i(n))^T D (PSI^T g_j(n)) = sum_{a<=b} K_ab Tsym^{ab}_ij
//     K = |T| PSI D PSI^T (3x3 symmetric, 6 numbers per tet)
//     Tsym^{aa} = S^{aa}, Tsym^{ab} = S^{ab} + S^{ba},  S^{ab}_ij = sum_n w_n g_i^a(n) g_j^b(n)
// where g are the reference gradients and S is computed once on the host with the same
// quadrature rule the caller asked for.  Phase 1 computes K (and f|T|) once per tet;
// phase 2 is a row gather: every CSR row is owned by one group of NLOC lanes, which walks
// the row's incident tets in ascending tet order, computes that tet's row of A (lane j
// computes A(i, j)) and adds it into a shared-memory copy of the row at the offsets held
// by the scatter record.  Each value is therefore summed in the same order as the
// reference's serial cell loop, without atomics, and written to HBM once, coalesced.
#include "anigpu_internal.h"

namespace {

constexpr int kChunk = 16;  // incidences staged per group per step

// ---------------------------------------------------------------- phase 1
// K = |T| PSI D PSI^T (k00 k11 k22 k01 k02 k12), then f*|T| and 0: 8 values per tet.
template <typename Real>
__global__ void tet_prepare_kernel(int64_t nt, const double* __restrict__ xyz, const int32_t* __restrict__ tets,
                                   int kind, const double* __restrict__ D, const double* __restrict__ f,
                                   double f_const, Real* __restrict__ out, int* __restrict__ status) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= nt) return;
    const int4 v = reinterpret_cast<const int4*>(tets)[t];
    double X0[3], e[9];
#pragma unroll
    for (int k = 0; k < 3; ++k) X0[k] = xyz[3 * (int64_t)v.x + k];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        e[k + 0] = xyz[3 * (int64_t)v.y + k] - X0[k];  // column 0: X1 - X0 (core.inl:230-236)
        e[k + 3] = xyz[3 * (int64_t)v.z + k] - X0[k];
        e[k + 6] = xyz[3 * (int64_t)v.w + k] - X0[k];
    }
    // symmetric tensor d00 d01 d02 d11 d12 d22
    double d[6];
    switch (kind) {
        case ANIGPU_TENSOR_NULL: d[0] = d[3] = d[5] = 1; d[1] = d[2] = d[4] = 0; break;
        case ANIGPU_TENSOR_CONST_SCALAR: d[0] = d[3] = d[5] = D[0]; d[1] = d[2] = d[4] = 0; break;
        case ANIGPU_TENSOR_TET_SCALAR: d[0] = d[3] = d[5] = D[t]; d[1] = d[2] = d[4] = 0; break;
        default:
#pragma unroll
            for (int k = 0; k < 6; ++k) d[k] = D[6 * t + k];
    }
    const double fv = f ? f[t] : f_const;
    Real K[8];
    bool bad = false;
    // cofactor inverse (inverse3x3, geometry.h:26-44).  The FP32 path inverts in FP32 unless
    // the tet is badly shaped (|det| small against the edge lengths), then in FP64.
    bool use64 = sizeof(Real) == 8;
    float ef[9], PSIf[9];
    float detf = 0.f;
    if (!use64) {
#pragma unroll
        for (int k = 0; k < 9; ++k) ef[k] = (float)e[k];
#define M(I, J) ef[(I) + 3 * (J)]
        const float da = M(1, 1) * M(2, 2) - M(1, 2) * M(2, 1);
        const float db = M(1, 2) * M(2, 0) - M(1, 0) * M(2, 2);
        const float dc = M(1, 0) * M(2, 1) - M(1, 1) * M(2, 0);
        detf = M(0, 0) * da + M(0, 1) * db + M(0, 2) * dc;
        const float l0 = sqrtf(M(0, 0) * M(0, 0) + M(1, 0) * M(1, 0) + M(2, 0) * M(2, 0));
        const float l1 = sqrtf(M(0, 1) * M(0, 1) + M(1, 1) * M(1, 1) + M(2, 1) * M(2, 1));
        const float l2 = sqrtf(M(0, 2) * M(0, 2) + M(1, 2) * M(1, 2) + M(2, 2) * M(2, 2));
        if (!(fabsf(detf) > 0.05f * l0 * l1 * l2)) {
            use64 = true;
        } else {
            const float inv = 1.0f / detf;
            PSIf[0] = da * inv;
            PSIf[1] = db * inv;
            PSIf[2] = dc * inv;
#pragma unroll
            for (int i = 1; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j)
                    PSIf[j + 3 * i] = (M((i + 1) % 3, (j + 1) % 3) * M((i + 2) % 3, (j + 2) % 3) -
                                       M((i + 1) % 3, (j + 2) % 3) * M((i + 2) % 3, (j + 1) % 3)) * inv;
        }
#undef M
    }
    if (use64) {
        double PSI[9];
#define M(I, J) e[(I) + 3 * (J)]
        const double da = M(1, 1) * M(2, 2) - M(1, 2) * M(2, 1);
        const double db = M(1, 2) * M(2, 0) - M(1, 0) * M(2, 2);
        const double dc = M(1, 0) * M(2, 1) - M(1, 1) * M(2, 0);
        const double det = M(0, 0) * da + M(0, 1) * db + M(0, 2) * dc;
        PSI[0] = da / det;
        PSI[1] = db / det;
        PSI[2] = dc / det;
#pragma unroll
        for (int i = 1; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j)
                PSI[j + 3 * i] = (M((i + 1) % 3, (j + 1) % 3) * M((i + 2) % 3, (j + 2) % 3) -
                                  M((i + 1) % 3, (j + 2) % 3) * M((i + 2) % 3, (j + 1) % 3)) / det;
#undef M
        const double mes = fabs(det) / 6.0;
        // M = PSI * D, K = mes * M * PSI^T ; PSI(a,a') = PSI[a + 3a']
        double Dm[9] = {d[0], d[1], d[2], d[1], d[3], d[4], d[2], d[4], d[5]};
        double Mm[9];
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b) {
                double s = 0;
#pragma unroll
                for (int c = 0; c < 3; ++c) s += PSI[a + 3 * c] * Dm[c + 3 * b];
                Mm[a + 3 * b] = s;
            }
        auto kab = [&](int a, int b) {
            double s = 0;
#pragma unroll
            for (int c = 0; c < 3; ++c) s += Mm[a + 3 * c] * PSI[b + 3 * c];
            return mes * s;
        };
        K[0] = (Real)kab(0, 0);
        K[1] = (Real)kab(1, 1);
        K[2] = (Real)kab(2, 2);
        K[3] = (Real)kab(0, 1);
        K[4] = (Real)kab(0, 2);
        K[5] = (Real)kab(1, 2);
        K[6] = (Real)(fv * mes);
        K[7] = (Real)0;
        bad = !isfinite(det) || det == 0.0;
    } else {
        const float mes = fabsf(detf) / 6.0f;
        const float Dm[9] = {(float)d[0], (float)d[1], (float)d[2], (float)d[1], (float)d[3],
                             (float)d[4], (float)d[2], (float)d[4], (float)d[5]};
        float Mm[9];
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b) {
                float s = 0;
#pragma unroll
                for (int c = 0; c < 3; ++c) s += PSIf[a + 3 * c] * Dm[c + 3 * b];
                Mm[a + 3 * b] = s;
            }
        auto kab = [&](int a, int b) {
            float s = 0;
#pragma unroll
            for (int c = 0; c < 3; ++c) s += Mm[a + 3 * c] * PSIf[b + 3 * c];
            return mes * s;
        };
        K[0] = (Real)kab(0, 0);
        K[1] = (Real)kab(1, 1);
        K[2] = (Real)kab(2, 2);
        K[3] = (Real)kab(0, 1);
        K[4] = (Real)kab(0, 2);
        K[5] = (Real)kab(1, 2);
        K[6] = (Real)((float)fv * mes);
        K[7] = (Real)0;
    }
#pragma unroll
    for (int k = 0; k < 7; ++k) bad |= !isfinite((double)K[k]);
    if (bad) atomicExch(status, ANIGPU_ERR_NONFINITE);
    if (sizeof(Real) == 4) {
        float4* o = reinterpret_cast<float4*>(out + 8 * t);
        o[0] = make_float4((float)K[0], (float)K[1], (float)K[2], (float)K[3]);
        o[1] = make_float4((float)K[4], (float)K[5], (float)K[6], (float)K[7]);
    } else {
        double2* o = reinterpret_cast<double2*>(out + 8 * t);
        o[0] = make_double2((double)K[0], (double)K[1]);
        o[1] = make_double2((double)K[2], (double)K[3]);
        o[2] = make_double2((double)K[4], (double)K[5]);
        o[3] = make_double2((double)K[6], (double)K[7]);
    }
}

// ---------------------------------------------------------------- phase 2
struct RowParams {
    int64_t nrows;
    const int64_t* inc_ptr;
    const ScatterRec* recs;
    const int64_t* rowptr;
    const uint8_t* dir_mask;
    const double* dir_bc;
    const int32_t* edofs;
    int bc_nonzero;
    int cap;  // row buffer capacity (>= longest row)
    double drop;
};

__device__ inline uint32_t rec_off(const ScatterRec& r, int j) {
    const uint32_t w = j < 4 ? r.off03 : (j < 8 ? r.off47 : (r.meta >> 16));
    return (w >> (8 * (j & 3))) & 0xffu;
}

template <typename Real, int NLOC>
__global__ void __launch_bounds__(128) row_gather_kernel(RowParams p, const Real* __restrict__ tables,
                                                         const Real* __restrict__ tetK, Real* __restrict__ vals,
                                                         double* __restrict__ rhs, uint8_t* __restrict__ touched_out,
                                                         int* __restrict__ status) {
    constexpr int G = 32 / NLOC;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane / NLOC, lj = lane - g * NLOC;
    const bool in_group = g < G;
    // tables: Tsym[6][NLOC][NLOC], m[NLOC]
    Real* sT = reinterpret_cast<Real*>(smem_raw);
    constexpr int ntab = 6 * NLOC * NLOC + NLOC;
    for (int k = threadIdx.x; k < ntab; k += blockDim.x) sT[k] = tables[k];
    const Real* sM = sT + 6 * NLOC * NLOC;
    // per-group regions
    const size_t tab_bytes = ((sizeof(Real) * ntab + 15) / 16) * 16;
    const size_t grp_bytes = ((kChunk * sizeof(ScatterRec) + kChunk * 8 * sizeof(Real) +
                               p.cap * sizeof(Real) + NLOC * sizeof(Real) + p.cap + 15) / 16) * 16;
    unsigned char* gbase = smem_raw + tab_bytes + grp_bytes * (size_t)(warp * G + (in_group ? g : 0));
    ScatterRec* sRec = reinterpret_cast<ScatterRec*>(gbase);
    Real* sK = reinterpret_cast<Real*>(gbase + kChunk * sizeof(ScatterRec));
    Real* sRow = sK + kChunk * 8;
    Real* sA = sRow + p.cap;
    uint8_t* sTouch = reinterpret_cast<uint8_t*>(sA + NLOC);
    __syncthreads();

    const int64_t row = ((int64_t)blockIdx.x * (blockDim.x >> 5) + warp) * G + g;
    const bool valid = in_group && row < p.nrows;
    int64_t ib = 0, ie = 0, rb = 0;
    int len = 0;
    bool isdir = false;
    double bcr = 0;
    if (valid) {
        ib = p.inc_ptr[row];
        ie = p.inc_ptr[row + 1];
        rb = p.rowptr[row];
        len = (int)(p.rowptr[row + 1] - rb);
        isdir = p.dir_mask[row] != 0;
        bcr = p.dir_bc[row];
        for (int s = lj; s < len; s += NLOC) {
            sRow[s] = Real(0);
            sTouch[s] = 0;
        }
    }
    Real racc = 0;  // right-hand side (lane lj == 0)
    double racc64 = 0;
    __syncwarp();
    const int ninc = valid ? (int)(ie - ib) : 0;
    int maxinc = ninc;
#pragma unroll
    for (int o = 16; o; o >>= 1) maxinc = max(maxinc, __shfl_xor_sync(0xffffffffu, maxinc, o));
    for (int c0 = 0; c0 < maxinc; c0 += kChunk) {
        // stage records and per-tet K of this chunk
        const int nch = min(kChunk, ninc - c0);
        for (int s = lj; s < nch; s += NLOC) {
            const ScatterRec r = p.recs[ib + c0 + s];
            sRec[s] = r;
            const Real* kp = tetK + 8 * (int64_t)r.tet;
            if (sizeof(Real) == 4) {
                const float4* k4 = reinterpret_cast<const float4*>(kp);
                reinterpret_cast<float4*>(sK + 8 * s)[0] = k4[0];
                reinterpret_cast<float4*>(sK + 8 * s)[1] = k4[1];
            } else {
                const double2* k2 = reinterpret_cast<const double2*>(kp);
#pragma unroll
                for (int q = 0; q < 4; ++q) reinterpret_cast<double2*>(sK + 8 * s)[q] = k2[q];
            }
        }
        __syncwarp();
        for (int s = 0; s < kChunk; ++s) {
            const bool act = s < nch;
            ScatterRec r = {0u, 0u, 0u, 0u};
            Real a = Real(0);
            if (act) {
                r = sRec[s];
                const int i = r.meta & 15;
                const Real* Kt = sK + 8 * s;
                if (isdir) {
                    // applyDir on the row DOF: the element row becomes e_i, F(i) = bc
                    if (lj == i) {
                        const uint32_t off = rec_off(r, i);
                        sRow[off] += Real(1);
                        sTouch[off] = 1;
                    }
                    if (lj == 0) racc64 += bcr;
                } else {
                    const Real* T = sT + i * NLOC + lj;
                    a = Kt[0] * T[0 * NLOC * NLOC];
                    a = fma(Kt[1], T[1 * NLOC * NLOC], a);
                    a = fma(Kt[2], T[2 * NLOC * NLOC], a);
                    a = fma(Kt[3], T[3 * NLOC * NLOC], a);
                    a = fma(Kt[4], T[4 * NLOC * NLOC], a);
                    a = fma(Kt[5], T[5 * NLOC * NLOC], a);
                    if (!isfinite((double)a)) atomicExch(status, ANIGPU_ERR_NONFINITE);
                    const uint32_t dm = (r.meta >> 4) & 0x3ffu;
                    const bool colDir = (dm >> lj) & 1u;
                    if (!colDir && fabs((double)a) > p.drop) {
                        const uint32_t off = rec_off(r, lj);
                        sRow[off] += a;
                        sTouch[off] = 1;
                    }
                }
            }
            if (p.bc_nonzero) {
                if (act && !isdir) sA[lj] = a;
                __syncwarp();
            }
            if (act && !isdir && lj == 0) {
                // right-hand side: fem3Dtet<IDEN P0, IDEN space> then applyDir on Dirichlet
                // columns in ascending local order (dc_on_dof.h:39-45)
                const int i = r.meta & 15;
                const uint32_t dm = (r.meta >> 4) & 0x3ffu;
                Real F = sK[8 * s + 6] * sM[i];
                if (p.bc_nonzero && dm) {
                    for (int j = 0; j < NLOC; ++j)
                        if ((dm >> j) & 1u) F -= sA[j] * Real(p.dir_bc[p.edofs[(int64_t)r.tet * NLOC + j]]);
                }
                racc += F;
            }
            __syncwarp();
        }
        __syncwarp();
    }
    if (valid) {
        for (int s = lj; s < len; s += NLOC) {
            vals[rb + s] = sRow[s];
            if (touched_out) touched_out[rb + s] = sTouch[s];
        }
        if (lj == 0) {
            const double F = isdir ? racc64 : (double)racc;
            if (!isfinite(F)) atomicExch(status, ANIGPU_ERR_NONFINITE);
            rhs[row] = F;
        }
    }
}

// ---------------------------------------------------------------- CSR compaction
__global__ void compact_count_kernel(int64_t n, const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                                     const uint8_t* __restrict__ touched, unsigned long long* __restrict__ cnt) {
    const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (r >= n) return;
    unsigned long long c = 0;
    for (int64_t k = rowptr[r]; k < rowptr[r + 1]; ++k) c += (touched[k] || col[k] == r) ? 1 : 0;
    cnt[r] = c;
}
template <typename Real>
__global__ void compact_fill_kernel(int64_t n, const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                                    const Real* __restrict__ vals, const uint8_t* __restrict__ touched,
                                    const int64_t* __restrict__ nptr, int32_t* __restrict__ ncol,
                                    Real* __restrict__ nvals) {
    const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (r >= n) return;
    int64_t w = nptr[r];
    for (int64_t k = rowptr[r]; k < rowptr[r + 1]; ++k)
        if (touched[k] || col[k] == r) {
            ncol[w] = col[k];
            if (vals) nvals[w] = vals[k];
            ++w;
        }
}

}  // namespace

// host: Tsym tables and m for (space, order) in precision
static int get_row_tables(anigpu_ctx* h, int space, int order, int precision, const void** dev) {
    const int key = 1000 * precision + 100 * space + order + 100000;
    for (auto& kv : h->basis_dev)
        if (kv.first == key) {
            *dev = kv.second;
            return ANIGPU_OK;
        }
    ScalarBasisTable tb;
    if (!make_scalar_basis(space, order, &tb)) return set_err(h, ANIGPU_ERR_UNSUPPORTED, "unsupported space/order");
    const int nf = tb.nf, q = tb.q;
    std::vector<double> T(6 * nf * nf + nf, 0.0);
    const int A[6] = {0, 1, 2, 0, 0, 1}, B[6] = {0, 1, 2, 1, 2, 2};
    for (int k = 0; k < 6; ++k)
        for (int i = 0; i < nf; ++i)
            for (int j = 0; j < nf; ++j) {
                double s = 0;
                for (int n = 0; n < q; ++n) {
                    const double* gi = &tb.grad[((size_t)n * nf + i) * 3];
                    const double* gj = &tb.grad[((size_t)n * nf + j) * 3];
                    double v = gi[A[k]] * gj[B[k]];
                    if (A[k] != B[k]) v += gi[B[k]] * gj[A[k]];
                    s += tb.wts[n] * v;
                }
                T[(size_t)k * nf * nf + i * nf + j] = s;
            }
    for (int i = 0; i < nf; ++i) {
        double s = 0;
        for (int n = 0; n < q; ++n) s += tb.wts[n] * tb.val[(size_t)n * nf + i];
        T[6 * nf * nf + i] = s;
    }
    void* d = nullptr;
    if (precision == ANIGPU_F32) {
        std::vector<float> Tf(T.begin(), T.end());
        ANI_CUDA(h, cudaMalloc(&d, Tf.size() * sizeof(float)));
        ANI_CUDA(h, cudaMemcpy(d, Tf.data(), Tf.size() * sizeof(float), cudaMemcpyHostToDevice));
    } else {
        ANI_CUDA(h, cudaMalloc(&d, T.size() * sizeof(double)));
        ANI_CUDA(h, cudaMemcpy(d, T.data(), T.size() * sizeof(double), cudaMemcpyHostToDevice));
    }
    h->basis_dev.push_back({key, (double*)d});
    *dev = d;
    return ANIGPU_OK;
}

template <typename Real, int NLOC>
static int launch_rows(anigpu_ctx* h, const RowParams& p, const void* tables, void* vals, double* rhs,
                       uint8_t* touched) {
    constexpr int G = 32 / NLOC;
    const int warps = 4;
    const size_t tab_bytes = ((sizeof(Real) * (6 * NLOC * NLOC + NLOC) + 15) / 16) * 16;
    const size_t grp_bytes = ((kChunk * sizeof(ScatterRec) + kChunk * 8 * sizeof(Real) + p.cap * sizeof(Real) +
                               NLOC * sizeof(Real) + p.cap + 15) / 16) * 16;
    const size_t smem = tab_bytes + grp_bytes * warps * G;
    auto kern = row_gather_kernel<Real, NLOC>;
    ANI_CUDA(h, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int64_t rows_per_block = (int64_t)warps * G;
    kern<<<grid_for(p.nrows, (int)rows_per_block), 32 * warps, smem, h->stream>>>(
        p, (const Real*)tables, (const Real*)h->tetdata, (Real*)vals, rhs, touched, h->d_status);
    ANI_LAUNCHED(h);
    return ANIGPU_OK;
}

int run_assemble(anigpu_ctx* h, int kind, const double* D, const double* f, double f_const, int order,
                 int precision, void* vals, double* rhs, uint8_t* touched, double drop_val) {
    if (h->space < 0) return set_err(h, ANIGPU_ERR_STATE, "anigpu_problem_setup not called");
    if (h->space == ANIGPU_VEC3_P2) return set_err(h, ANIGPU_ERR_UNSUPPORTED, "vector assembly not built yet");
    if (kind != ANIGPU_TENSOR_NULL && kind != ANIGPU_TENSOR_CONST_SCALAR && kind != ANIGPU_TENSOR_TET_SCALAR &&
        kind != ANIGPU_TENSOR_TET_SYM)
        return set_err(h, ANIGPU_ERR_UNSUPPORTED, "assembly tensor kind must be NULL, CONST_SCALAR, TET_SCALAR or TET_SYM");
    if (kind != ANIGPU_TENSOR_NULL && !D) return set_err(h, ANIGPU_ERR_ARG, "tensor data is NULL");
    if (!vals || !rhs) return set_err(h, ANIGPU_ERR_ARG, "NULL output");
    if (precision != ANIGPU_F32 && precision != ANIGPU_F64) return set_err(h, ANIGPU_ERR_ARG, "precision");
    const void* tables = nullptr;
    int rc = get_row_tables(h, h->space, order, precision, &tables);
    if (rc) return rc;
    const size_t rsz = precision == ANIGPU_F32 ? 4 : 8;
    const size_t need = (size_t)h->nt * 8 * rsz;
    if (h->tetdata_bytes < need) {
        if (h->tetdata) cudaFree(h->tetdata);
        h->tetdata = nullptr;
        ANI_CUDA(h, cudaMalloc(&h->tetdata, need));
        h->tetdata_bytes = need;
    }
    time_mark(h, 0);
    if (precision == ANIGPU_F32)
        tet_prepare_kernel<float><<<grid_for(h->nt, 256), 256, 0, h->stream>>>(h->nt, h->xyz, h->tets, kind, D, f,
                                                                              f_const, (float*)h->tetdata, h->d_status);
    else
        tet_prepare_kernel<double><<<grid_for(h->nt, 256), 256, 0, h->stream>>>(
            h->nt, h->xyz, h->tets, kind, D, f, f_const, (double*)h->tetdata, h->d_status);
    ANI_LAUNCHED(h);
    time_mark(h, 1);
    RowParams p;
    p.nrows = h->nds;
    p.inc_ptr = h->inc_ptr;
    p.recs = h->recs;
    p.rowptr = h->rowptr_s;
    p.dir_mask = h->dir_mask;
    p.dir_bc = h->dir_bc;
    p.edofs = h->edofs;
    p.bc_nonzero = h->bc_nonzero ? 1 : 0;
    p.cap = ((h->max_row_len_s + 15) / 16) * 16;
    p.drop = drop_val;
    if (h->nloc_s == 10) {
        rc = precision == ANIGPU_F32 ? launch_rows<float, 10>(h, p, tables, vals, rhs, touched)
                                     : launch_rows<double, 10>(h, p, tables, vals, rhs, touched);
    } else {
        rc = precision == ANIGPU_F32 ? launch_rows<float, 4>(h, p, tables, vals, rhs, touched)
                                     : launch_rows<double, 4>(h, p, tables, vals, rhs, touched);
    }
    time_mark(h, 2);
    return rc;
}

int run_compact(anigpu_ctx* h, int64_t* rowptr, int32_t* col, void* vals, int precision, const uint8_t* touched,
                int64_t* nnz_out) {
    if (h->space < 0) return set_err(h, ANIGPU_ERR_STATE, "anigpu_problem_setup not called");
    const int64_t n = h->ndof;
    cudaStream_t s = h->stream;
    int64_t nnz_old = 0;
    ANI_CUDA(h, cudaMemcpyAsync(&nnz_old, rowptr + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    ANI_CUDA(h, cudaStreamSynchronize(s));
    unsigned long long* cnt = nullptr;
    int64_t* nptr = nullptr;
    int32_t* ncol = nullptr;
    void* nvals = nullptr;
    const size_t rsz = precision == ANIGPU_F32 ? 4 : 8;
    ANI_CUDA(h, cudaMallocAsync((void**)&cnt, sizeof(unsigned long long) * (n + 1), s));
    ANI_CUDA(h, cudaMallocAsync((void**)&nptr, sizeof(int64_t) * (n + 1), s));
    ANI_CUDA(h, cudaMemsetAsync(cnt, 0, sizeof(unsigned long long) * (n + 1), s));
    compact_count_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, rowptr, col, touched, cnt);
    ANI_LAUNCHED(h);
    {
        int rc = scan_counts(h, cnt, n, nptr);
        if (rc) return rc;
        ANI_CUDA(h, cudaMemcpyAsync(nnz_out, nptr + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
        ANI_CUDA(h, cudaStreamSynchronize(s));
    }
    ANI_CUDA(h, cudaMallocAsync((void**)&ncol, sizeof(int32_t) * std::max<int64_t>(*nnz_out, 1), s));
    ANI_CUDA(h, cudaMallocAsync(&nvals, rsz * std::max<int64_t>(*nnz_out, 1), s));
    if (precision == ANIGPU_F32)
        compact_fill_kernel<float><<<grid_for(n, 256), 256, 0, s>>>(n, rowptr, col, (const float*)vals, touched, nptr,
                                                                   ncol, (float*)nvals);
    else
        compact_fill_kernel<double><<<grid_for(n, 256), 256, 0, s>>>(n, rowptr, col, (const double*)vals, touched,
                                                                    nptr, ncol, (double*)nvals);
    ANI_LAUNCHED(h);
    ANI_CUDA(h, cudaMemcpyAsync(rowptr, nptr, sizeof(int64_t) * (n + 1), cudaMemcpyDeviceToDevice, s));
    ANI_CUDA(h, cudaMemcpyAsync(col, ncol, sizeof(int32_t) * *nnz_out, cudaMemcpyDeviceToDevice, s));
    if (vals) ANI_CUDA(h, cudaMemcpyAsync(vals, nvals, rsz * *nnz_out, cudaMemcpyDeviceToDevice, s));
    ANI_CUDA(h, cudaFreeAsync(cnt, s));
    ANI_CUDA(h, cudaFreeAsync(nptr, s));
    ANI_CUDA(h, cudaFreeAsync(ncol, s));
    ANI_CUDA(h, cudaFreeAsync(nvals, s));
    ANI_CUDA(h, cudaStreamSynchronize(s));
    (void)nnz_old;
    return ANIGPU_OK;
}
