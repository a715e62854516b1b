// tlr_solve.cu -- placeholder until the sparse factorisation lands.
#include "tlr_internal.h"

namespace tlr {
int run_solve(tlr_ctx *ctx, const tlr_solve_opts *, double *, double *, double *,
              tlr_eig_diag *) {
  return fail(ctx, TLR_ERR_ARG, "eigensolver not available in this build");
}
void free_factor(tlr_ctx *) {}
}  // namespace tlr
