/*
 * intT.h -- reconstruction of the reference's missing configuration header.
 *
 * Every reference source includes "intT.h" (EffAct.c:5, intEV.cu:7,
 * intEVff.cu:7, Tint.c:11, Integrand.c:7, testT.c:5, periodic.c:11) but the file
 * is absent from the reference tree.  Its contents are restated from use:
 *
 *  - profile names are preprocessor macros with integer values, because
 *    intEV.cu:12 tests "#if profile == fixflux" and EffAct.c:239-260 /
 *    Integrand.c:104-136 switch on them as case labels;
 *  - "profile" selects one of them at compile time (-Dprofile=gaussian ...);
 *  - constants tubedist (lattice spacing a), lmin (EffAct.c:321, lmin = 0.1 a as
 *    in analysis-scripts/EAscffvsconst.sage:12), q1, q2
 *    (analysis-scripts/EAscffvsconst.sage:6-7), pi, Nspline and verbosity;
 *  - struct Wparams and the host prototypes (wl_legacy.h).
 *
 * Only legacy host code (a port of EffAct.c / Tint.c / Integrand.c) includes
 * this header.  The GPU library reads its profile at run time instead: the
 * legacy EV() evaluates the profile set with wl_legacy_configure() (wlgpu.h).
 */
#ifndef INTT_H
#define INTT_H

#include "wl_legacy.h"

#define step 0
#define smooth 1
#define quadratic 2
#define gaussian 3
#define periodic 4
#define spline 5
#define fixflux 6

#ifndef profile
#define profile smooth
#endif

#ifndef pi
#define pi 3.14159265358979323846
#endif

/* lattice spacing a of the periodic / fixflux profiles */
#ifndef tubedist
#define tubedist 1.0f
#endif

#ifndef lmin
#define lmin (0.1f * tubedist)
#endif

/* fixflux normalisation constants of the bump profile */
#ifndef q1
#define q1 0.443991f
#endif
#ifndef q2
#define q2 0.0742478f
#endif

/* knots of the spline profile table */
#ifndef Nspline
#define Nspline 1000
#endif

#ifndef verbosity
#define verbosity 1
#endif

#endif /* INTT_H */
