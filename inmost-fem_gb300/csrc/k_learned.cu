// Learned preconditioner for flexible CG: placeholder until the network kernels land.
#include "learned.h"

int run_fcg_learned(anigpu_ctx* h, const void*, int, const double*, double*, double, int64_t, anigpu_solve_stats*) {
    return set_err(h, ANIGPU_ERR_UNSUPPORTED, "learned preconditioner not loaded");
}
void free_learned(anigpu_ctx*) {}
