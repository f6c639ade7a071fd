// SpMV rows of the vector (3-component) CSR template.
//
// The template of an ANIGPU_VEC3_P2 problem is built from the scalar one (k_setup.cu): row
// (c, r) is DOF c*nds + r and holds, for c' = 0, 1, 2 in turn, the columns of scalar row r
// shifted by c'*nds.  Its values start at c*3*nnz_s + 3*rowptr_s[r]; block c' of the row is at
// offset c'*len (len = the scalar row's length).  A group of W lanes computes the three rows
// (0..2, r) together from one read of the scalar column list: 4 bytes of index per 9 values
// instead of 4 per value, and the three x components of a column read once.
#pragma once
#include <cstdint>

// lanes per scalar row of the vector kernels, unroll of their column loop, resident blocks
#ifndef SPMV3_W
#define SPMV3_W 4
#endif
#ifndef SPMV3_UNROLL
#define SPMV3_UNROLL 2
#endif
#ifndef SPMV3_MINB
#define SPMV3_MINB 1
#endif
#ifndef SPMV3_MINB_F32
#define SPMV3_MINB_F32 4  // FP32-only kernels: 64 registers, four 256-thread blocks per SM
#endif
constexpr int kSpmv3Unroll = SPMV3_UNROLL;

template <int W, typename VR, typename T>
__device__ __forceinline__ void vec3_rows(int64_t r, int lane, int64_t nds, int64_t nnz_s,
                                          const int64_t* __restrict__ rowptr_s, const int32_t* __restrict__ col_s,
                                          const VR* __restrict__ vals, const T* __restrict__ x, T& s0, T& s1,
                                          T& s2) {
    T a0 = 0, a1 = 0, a2 = 0;
    if (r < nds) {
        const int64_t b = rowptr_s[r];
        const int len = (int)(rowptr_s[r + 1] - b);
        const int64_t cs = 3 * nnz_s;
        const VR* v0 = vals + 3 * b;
        const VR* v1 = v0 + cs;
        const VR* v2 = v1 + cs;
#pragma unroll kSpmv3Unroll
        for (int k = lane; k < len; k += W) {
            const int64_t t = col_s[b + k];
            const T x0 = x[t], x1 = x[nds + t], x2 = x[2 * nds + t];
            // one fused multiply-add per value (FP64 issue rate is the bound of the FP64 solve)
            a0 = T(v0[k]) * x0 + a0;
            a1 = T(v1[k]) * x0 + a1;
            a2 = T(v2[k]) * x0 + a2;
            a0 = T(v0[len + k]) * x1 + a0;
            a1 = T(v1[len + k]) * x1 + a1;
            a2 = T(v2[len + k]) * x1 + a2;
            a0 = T(v0[2 * len + k]) * x2 + a0;
            a1 = T(v1[2 * len + k]) * x2 + a1;
            a2 = T(v2[2 * len + k]) * x2 + a2;
        }
    }
#pragma unroll
    for (int o = W / 2; o; o >>= 1) {
        a0 += __shfl_xor_sync(0xffffffffu, a0, o, W);
        a1 += __shfl_xor_sync(0xffffffffu, a1, o, W);
        a2 += __shfl_xor_sync(0xffffffffu, a2, o, W);
    }
    s0 = a0;
    s1 = a1;
    s2 = a2;
}
