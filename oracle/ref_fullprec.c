/* Test infrastructure only (oracle/_ref build): the reference binary is linked with
 * -Wl,--wrap=fprintf so every fprintf lands here.  By default the call is passed through
 * unchanged.  With EIG_REF_FULLPREC=1 the number formats of the .eval file
 * (src/eigensrc/smartpca.c:1428 "%12.6f\n"), the .evec header (:1435 "%9.3f ") and the
 * .evec coordinates (:1584-1585 "%10.4f  " / "%12.6f  ") and the GRM text values
 * (:3803 "%0.6f\n"), the fstdetails values (:1897 "F_st ... %12.6f %12.6f %12.6f") and the
 * hiprecision SNP weights (:3096 " %12.6f") are printed as %.17g, so that the reference's
 * own results can be compared at 1e-10 instead of at 6 printed decimals.  The smartrel binary is also linked
 * with -Wl,--wrap=printf: its relatedness score (src/eigensrc/smartrel.c:614 " %9.3f")
 * prints as %.17g in the same mode. */
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static int fullprec_mode(void)
{
  static int mode = -1;
  if (mode < 0) {
    const char *e = getenv("EIG_REF_FULLPREC");
    mode = (e != NULL && e[0] == '1') ? 1 : 0;
  }
  return mode;
}

int __wrap_fprintf(FILE *f, const char *fmt, ...)
{
  const char *use = fmt;
  va_list ap;
  int r;
  if (fullprec_mode()) {
    if (strcmp(fmt, "%12.6f\n") == 0 || strcmp(fmt, "%0.6f\n") == 0)
      use = "%.17g\n";
    else if (strcmp(fmt, "%10.4f  ") == 0 || strcmp(fmt, "%12.6f  ") == 0)
      use = "%.17g  ";
    else if (strcmp(fmt, "%9.3f ") == 0)
      use = "%.17g ";
    else if (strcmp(fmt, "F_st %20s %20s %12.6f %12.6f %12.6f") == 0)
      use = "F_st %20s %20s %.17g %.17g %.17g";
    else if (strcmp(fmt, " %12.6f") == 0)
      use = " %.17g";
  }
  va_start(ap, fmt);
  r = vfprintf(f, use, ap);
  va_end(ap);
  return r;
}

int __wrap_printf(const char *fmt, ...)
{
  const char *use = fmt;
  va_list ap;
  int r;
  if (fullprec_mode() && strcmp(fmt, " %9.3f") == 0) use = " %.17g";
  va_start(ap, fmt);
  r = vprintf(use, ap);
  va_end(ap);
  return r;
}
