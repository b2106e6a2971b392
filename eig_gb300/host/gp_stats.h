/* Tail probabilities for the ANOVA statistics of smartpca's log (host functions). */
#ifndef GP_STATS_H
#define GP_STATS_H

/* regularised incomplete beta I_x(a, b) and upper incomplete gamma Q(a, x) */
double gp_betai(double a, double b, double x);
double gp_gammq(double a, double x);
/* upper tail of F(df1, df2) at F as the reference reports it (rtlf, src/nicksrc/statsubs.c:1400) */
double gp_ftail(int df1, int df2, double F);
/* upper tail of chi-square(df) at z (rtlchsq, src/nicksrc/statsubs.c:1268-1287) */
double gp_chitail(int df, double z);

#endif
