// Learned preconditioner + flexible CG (k_learned.cu).
#pragma once
#include "anigpu_internal.h"

int run_fcg_learned(anigpu_ctx* h, const void* vals, int precision, const double* b, double* x, double rtol,
                    int64_t maxit, anigpu_solve_stats* st);
void free_learned(anigpu_ctx* h);
