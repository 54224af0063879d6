/* MEX gateway NLSE1D_TAKE_STEPS_2SHOC_CUDA_F: 1D, 2SHOC, single precision (nlse_mex_gateway.h). */
#include <string.h>
#define NLSE_MEX_NDIM 1
#define NLSE_MEX_METHOD 2
#define NLSE_MEX_PRECISION 1
#include "nlse_mex_gateway.h"
