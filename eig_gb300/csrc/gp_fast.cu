/* fastmode (randomized block Krylov PCA): placeholder until the kernels land */
#include "gp_internal.h"
extern "C" int gp_fastpca(gp_ctx *ctx, int32_t K, int32_t L, int32_t I, uint64_t seed,
                          const double *omega, int32_t precision, double *evals, double *evecs)
{
  (void)K; (void)L; (void)I; (void)seed; (void)omega; (void)precision; (void)evals; (void)evecs;
  return gp_fail(ctx, GP_ERR_NOTBUILT, "fastmode not built yet");
}
