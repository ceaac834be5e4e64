/*
 * Compatibility header with the reference's name (src/define.h): its
 * constants and flags, same names and values, so that callers written
 * against libfmftsaxs compile unchanged against fmftsaxs-gb300.
 */
#ifndef FMFTSAXS_GB300_COMPAT_DEFINE_H
#define FMFTSAXS_GB300_COMPAT_DEFINE_H

#define SQRTPI 1.77245385091
/* the value every formula of the reference uses when <math.h> gives none */
#ifndef M_PI
#define M_PI 3.14159265358
#endif
#define QMAX 0.5            /* correlate's q range and point count */
#define QNUM 50
#define REL_ERR 0.05        /* default relative intensity error */
#define MINIMIZER_ITERMAX 1000
#define VERBOSE_LBFGS -1
#define C1_LOWER 0.96       /* L-BFGS-B bounds and start of (c1, c2) */
#define C1_UPPER 1.04
#define C2_LOWER -2.00
#define C2_UPPER 4.00
#define C1_DEFAULT 1.0
#define C2_DEFAULT 0.0

#endif
