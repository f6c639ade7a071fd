// The coarse part of the learned preconditioner as grid-barrier stages, and its prolongation (the
// device code of the preconditioner's fused kernels in k_learned.cu).
//
// M r = D^-1 r + P Dc^-1/2 B B^T Dc^-1/2 P^T r,  B = sum_{k<4} diag(a_k) A_hat^k:
//   restriction  u = Dc^-1/2 P^T r, t = a_3 u
//   Horner       t <- A_hat t + a_k u (k = 2, 1, 0; the last into P_0)
//   powers       P_k = A_hat P_{k-1} (k = 1, 2)
//   combination  c = Dc^-1/2 sum_k a_k P_k with P_3 = A_hat P_2
//   prolongation z = D^-1 r + P c
// One thread per coarse row; the coarse graph is read in 32-row slices (coalesced column and value
// loads).  Stages are separated by grid barriers whose waits are bounded: a wait that expires
// records ANIGPU_ERR_TIMEOUT in the status word, marks the barrier unusable (bar[2]) and poisons
// the correction with NaN, which the flexible CG treats as a breakdown; no wait can hang.
#pragma once
#include <cstdint>

#include "anigpu_internal.h"

// coarse nodes are the vertex DOFs of every component: coarse id c*nv + v <-> fine DOF c*nds + v
// (scalar P2: nds = ndof and the two numberings agree); fine DOF c*nds + nv + e is edge e of
// component c.  At most 3 components, so the component is found by two compares.
struct CMap {
    int64_t nv, nds;
    __device__ __forceinline__ int comp_fine(int64_t d) const { return d >= nds ? (d >= 2 * nds ? 2 : 1) : 0; }
    __device__ __forceinline__ int comp_coarse(int64_t cid) const { return cid >= nv ? (cid >= 2 * nv ? 2 : 1) : 0; }
    __device__ __forceinline__ int64_t fine_of(int64_t cid) const {
        const int c = comp_coarse(cid);
        return c * nds + (cid - c * nv);
    }
    __device__ __forceinline__ int64_t coarse_of(int64_t d) const {
        const int c = comp_fine(d);
        const int64_t s = d - c * nds;
        return s < nv ? c * nv + s : -1;
    }
};

constexpr int kChainK = 4;  // polynomial terms of B (A_hat^0 .. A_hat^3)

struct ChainArgs {
    int64_t nc;
    CMap map;
    const float* r;
    const int64_t* vrow;
    const int32_t* vedge;
    const float* isd;
    const float* coef;
    const int64_t* sbase;
    const int32_t* scol;
    const float* sval;
    float *u, *t0, *t1, *pw, *cc;
    unsigned int* bar;  // arrivals, generation, expired
    int* status;
    const int* stop;
};

struct ProlongArgs {
    int64_t nf;
    CMap map;
    const float* diag_f;
    const float* cc;
    const int32_t* ends;  // [ne][2] end vertices of the edge DOFs
};

constexpr unsigned kBarrierSpins = 1u << 22;  // ~0.3 s of 64-ns sleeps

// all blocks of the (co-resident) grid: returns false when the wait expired
__device__ __forceinline__ bool grid_barrier(unsigned int* bar, int* status) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        ok = 1;
        volatile unsigned int* gen = bar + 1;
        const unsigned int g0 = *gen;
        __threadfence();
        if (atomicAdd(bar, 1u) + 1u == gridDim.x) {
            bar[0] = 0u;
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            unsigned int spins = 0;
            volatile unsigned int* expired = bar + 2;
            while (*gen == g0) {
                if (*expired) {  // another block's wait expired: this barrier will not complete
                    ok = 0;
                    break;
                }
                if (++spins > kBarrierSpins) {
                    atomicExch(status, ANIGPU_ERR_TIMEOUT);
                    atomicExch(bar + 2, 1u);
                    ok = 0;
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return ok != 0;
}

__device__ __forceinline__ bool barrier_expired(const unsigned int* bar) {
    return ((volatile const unsigned int*)bar)[2] != 0u;
}

// row v of A_hat x from the slices (padding entries: column v, value 0)
__device__ __forceinline__ float chain_spmv(const ChainArgs& a, int64_t v, const float* __restrict__ x) {
    const int64_t s = v >> 5;
    const int64_t b = a.sbase[s], e = a.sbase[s + 1];
    const int lane = (int)(v & 31);
    float acc = 0.f;
#pragma unroll 4
    for (int64_t q = b + lane; q < e; q += 32) acc = fmaf(a.sval[q], x[a.scol[q]], acc);
    return acc;
}

// restriction .. combination: seven stages, six barriers inside (the caller separates the stages
// from what comes before and after); thread t0 of nthr takes rows t0, t0 + nthr, ...
__device__ inline bool chain_stages(const ChainArgs& a, int64_t t0, int64_t nthr) {
    constexpr int K = kChainK;
    bool ok = true;
    for (int64_t v = t0; v < a.nc; v += nthr) {
        const int c = a.map.comp_coarse(v);
        const int64_t vs = v - c * a.map.nv;
        const float* rc = a.r + c * a.map.nds;
        float sum = 0.f;
        for (int64_t k = a.vrow[vs]; k < a.vrow[vs + 1]; ++k) sum += rc[a.vedge[k]];
        const float uu = a.isd[v] * fmaf(0.5f, sum, rc[vs]);
        a.u[v] = uu;
        a.t0[v] = a.coef[K * v + K - 1] * uu;
    }
    const float* src = a.t0;
    for (int k = K - 2; k >= 0; --k) {
        ok &= grid_barrier(a.bar, a.status);
        float* dst = k == 0 ? a.pw : (src == a.t0 ? a.t1 : a.t0);
        for (int64_t v = t0; v < a.nc; v += nthr) dst[v] = fmaf(a.coef[K * v + k], a.u[v], chain_spmv(a, v, src));
        src = dst;
    }
    for (int k = 1; k <= K - 2; ++k) {
        ok &= grid_barrier(a.bar, a.status);
        const float* x = a.pw + (int64_t)(k - 1) * a.nc;
        float* y = a.pw + (int64_t)k * a.nc;
        for (int64_t v = t0; v < a.nc; v += nthr) y[v] = chain_spmv(a, v, x);
    }
    ok &= grid_barrier(a.bar, a.status);
    for (int64_t v = t0; v < a.nc; v += nthr) {
        float sum = a.coef[K * v + K - 1] * chain_spmv(a, v, a.pw + (int64_t)(K - 2) * a.nc);
#pragma unroll
        for (int k = K - 2; k >= 0; --k) sum = fmaf(a.coef[K * v + k], a.pw[(int64_t)k * a.nc + v], sum);
        a.cc[v] = ok ? a.isd[v] * sum : __int_as_float(0x7fc00000);
    }
    return ok;
}

#ifndef PROLONG_U
#define PROLONG_U 4
#endif

// z = D^-1 r + P c over the fine DOFs i0, i0 + S, ...; adds r.z and z.qold (FP32) of those DOFs.
// PROLONG_U DOFs per pass with their loads issued together (the edge DOFs' coarse values are a
// two-level gather: end vertices, then their corrections).
__device__ inline void prolong_rows(const ProlongArgs& pa, const float* __restrict__ r, float* __restrict__ z,
                                    const float* __restrict__ qold, int64_t i0, int64_t S, float& arz, float& azq) {
    constexpr int U = PROLONG_U;
    for (; i0 < pa.nf; i0 += U * S) {
        float ri[U], zi[U], ca[U], cb[U];
        int64_t ia[U], ib[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int64_t i = i0 + u * S;
            ia[u] = -1;
            ib[u] = -1;
            ri[u] = 0.f;
            zi[u] = 0.f;
            if (i < pa.nf) {
                const float d = pa.diag_f[i];
                ri[u] = r[i];
                zi[u] = d != 0.f ? ri[u] / d : ri[u];
                const int comp = pa.map.comp_fine(i);
                const int64_t s = i - comp * pa.map.nds;
                if (s < pa.map.nv) ia[u] = comp * pa.map.nv + s;
                else {
                    const int2 e = reinterpret_cast<const int2*>(pa.ends)[s - pa.map.nv];
                    ia[u] = comp * pa.map.nv + e.x;
                    ib[u] = comp * pa.map.nv + e.y;
                }
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            ca[u] = ia[u] >= 0 ? pa.cc[ia[u]] : 0.f;
            cb[u] = ib[u] >= 0 ? pa.cc[ib[u]] : 0.f;
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int64_t i = i0 + u * S;
            if (i < pa.nf) {
                const float zz = ib[u] < 0 ? zi[u] + ca[u] : fmaf(0.5f, ca[u] + cb[u], zi[u]);
                z[i] = zz;
                arz = fmaf(ri[u], zz, arz);
                if (qold) azq = fmaf(zz, qold[i], azq);
            }
        }
    }
}
