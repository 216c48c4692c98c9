/*
 * Oracle test infrastructure: stand-in for GSL's gsl_sf_pow_int, which
 * suzerain/diffwave.c calls for (2 pi k / L)^d.  Integer power by repeated
 * squaring (x^0 == 1, including 0^0); negative powers invert first.
 */
#ifndef ORACLE_GSL_SF_POW_INT_H
#define ORACLE_GSL_SF_POW_INT_H
static inline double gsl_sf_pow_int(double x, int n)
{
    double v = 1.0;
    if (n < 0) { x = 1.0 / x; n = -n; }
    while (n) {
        if (n & 1) v *= x;
        n >>= 1;
        x *= x;
    }
    return v;
}
#endif
