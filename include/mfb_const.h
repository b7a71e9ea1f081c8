/*
 * mfb_const.h -- the composite trapezoidal rule over the azimuth of the
 * focused-beam families (reference mfb_src/mfb_const.h): at most TRAP_MNUM
 * halvings, at least TRAP_LNUM + 1 before the convergence test counts, and
 * the relative tolerance of that test.
 */
#if !defined MFB_CONST_H
#define MFB_CONST_H

#define TRAP_MNUM 12
#define TRAP_LNUM 1
#define TRAP_EPS 1.0e-15

#endif
