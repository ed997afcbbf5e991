/*
 * Constant table for the argon build of the reference oracle.
 *
 * Test infrastructure only.  oracle/build_ref.sh pre-includes this file when
 * it compiles the reference engine a second time.  Because it defines the
 * include guard CONSTANTS_H first, the reference's own common/Constants.h is
 * skipped and this table is used instead.  Every macro has the same name and
 * the same float-literal form as common/Constants.h:13-79, and every value is
 * the reference's, except the NG (noble gas) slot: the reference's neon
 * (sigma 2.72 A, eps 0.391e-4, m 20.1797; Constants.h:36,41,57) becomes argon:
 *   sigma = 3.405 A, eps = 119.8 K * kB = 119.8 * 8.314e-7 = 9.960172e-5
 *   (energy unit 1e7 J/mol, kB as in common/DebugCalculations.cpp:122),
 *   m = 39.948 g/mol.
 * Cross terms NG-N and NG-O keep the reference's values.
 */
#ifndef CONSTANTS_H
#define CONSTANTS_H

#define N 0
#define O 1
#define NG 2

#define radN 0.71f
#define radO 0.63f
#define radNG 0.58f

#define reN    1.097f
#define reO    1.2075f
#define reNO   1.15f

#define sigNvdw   3.31f
#define sigOvdw   2.95f
#define reNvdw   3.72f
#define reOvdw   3.31f
#define reNOvdw  3.51f

#define sigNG    3.405f
#define sigNGN   3.015f
#define sigNGO   2.835f

#define epsNG   9.960172e-5f
#define epsNGN  0.328e-4f
#define epsNGO  0.447e-4f

#define deN   941.4e-4f
#define deO   493.55309e-4f
#define deNO  626.734e-4f

#define betaN  2.71009f
#define betaO  2.2478f
#define betaNO 2.24068f

#define mN 14.00674f
#define mO 15.9994f
#define mNG 39.948f

#define CUTOFF_RIJ 15*sigNvdw
#define CUTOFF_RIJSQ 225*sigNvdw*sigNvdw

#define GEAR1 0.15833333333333333333333333333333f
#define GEAR2 0.75f
#define GEAR3 0.5f
#define GEAR4 0.08333333333333333333333333333333f

#define S      2.0f
#define GM     0.3f
#define GMSQ   0.09f
#define ALFAV  3.0f
#define ALFAVSQ 9.0f
#define ALFA   2.0f
#define R0     1.3f
#define LAMDA3 1.33f
#define C      25.f
#define D      4.0417f
#define H      0.0f

#endif
