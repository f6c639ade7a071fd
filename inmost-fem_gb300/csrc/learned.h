// Learned preconditioner (k_learned.cu) and flexible CG (k_fcg.cu).
#pragma once
#include "anigpu_internal.h"

int run_fcg_learned(anigpu_ctx* h, const void* vals, int precision, const double* b, double* x, double rtol,
                    int64_t maxit, anigpu_solve_stats* st,
                    const double* vals64 = nullptr);
void free_learned(anigpu_ctx* h);
// a new mesh or problem: the binding is dropped (bind again) and captured solver graphs freed
void learned_invalidate(anigpu_ctx* h);

int gnn_init(anigpu_ctx* h, int layers, int act, uint64_t seed);
int64_t gnn_num_params(anigpu_ctx* h);
// which: 0 parameters, 1 gradients; set: 1 host -> device
int gnn_params(anigpu_ctx* h, float* host, int64_t n, int set, int which);
int gnn_bind(anigpu_ctx* h, const void* vals, int precision, int kind, const double* D);
int gnn_apply(anigpu_ctx* h, const double* r, double* z);
int gnn_apply_f32(anigpu_ctx* h, const float* r, float* z);
int gnn_coefficients(anigpu_ctx* h, float* coef);
int gnn_loss_grad(anigpu_ctx* h, const double* r, const double* e, double* loss);
int gnn_adam(anigpu_ctx* h, float lr, float b1, float b2, float eps, int step, float gscale);
int gnn_zero_grads(anigpu_ctx* h);
bool gnn_bound_to(anigpu_ctx* h, const void* vals);
const float* gnn_fine_diag(anigpu_ctx* h);
// z = M r (FP32, fused, capturable); partials of r.z and z.qold over nb blocks; kernels return
// at once while *stop is non-zero
int gnn_precond_f32(anigpu_ctx* h, const float* r, float* z, const float* qold, double* part_rz, double* part_zq,
                    int nb, const int* stop);
int64_t gnn_bind_generation(anigpu_ctx* h);
int gnn_chain_active(anigpu_ctx* h);
void free_fcg(anigpu_ctx* h);
