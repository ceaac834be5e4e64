/* L-BFGS-B over (c1, c2) on the device: placeholder until the batched
 * solver lands; the launcher reports that the fit is unavailable. */
#include "kernels.h"

extern "C" int sxs_fit_lbfgsb_launch(const double *, int, int, const double *, const double *, double, double *,
                                     double *, double *, double *, int *, cudaStream_t)
{
	return (int)cudaErrorNotSupported;
}
