/* MEX gateway NLSE3D_TAKE_STEPS_2SHOC_CUDA_D: 3D, 2SHOC, double precision (nlse_mex_gateway.h). */
#include <string.h>
#define NLSE_MEX_NDIM 3
#define NLSE_MEX_METHOD 2
#define NLSE_MEX_PRECISION 2
#include "nlse_mex_gateway.h"
