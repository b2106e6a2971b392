/* Test infrastructure only (oracle/_ref build): the reference's fastmode
 * (src/ksrc/kjg_fpca.c:24) needs GSL, which is not installed, so the oracle build links
 * this stub in its place.  A parfile with `fastmode: YES` makes the reference binary exit. */
#include <stdio.h>
#include <stdlib.h>

void kjg_fpca(size_t K, size_t L, size_t I, double *eval, double *evec)
{
  (void)K; (void)L; (void)I; (void)eval; (void)evec;
  fprintf(stderr, "oracle/_ref: fastmode is not built (GSL absent)\n");
  exit(2);
}
