/* placeholder until the tcgen05 split-BF16 Gram lands */
#include "gp_internal.h"
int gp_gram_split_bf16(gp_ctx *ctx)
{
  return gp_fail(ctx, GP_ERR_NOTBUILT, "split-BF16 Gram not built yet");
}
extern "C" int gp_fastpca(gp_ctx *ctx, int32_t K, int32_t L, int32_t I, uint64_t seed,
                          const double *omega, int32_t precision, double *evals, double *evecs)
{
  (void)K; (void)L; (void)I; (void)seed; (void)omega; (void)precision; (void)evals; (void)evecs;
  return gp_fail(ctx, GP_ERR_NOTBUILT, "fastmode not built yet");
}
