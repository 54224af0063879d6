/* MEX gateway NLSE2D_TAKE_STEPS_CD_CUDA_F: 2D, CD, single precision (nlse_mex_gateway.h). */
#include <string.h>
#define NLSE_MEX_NDIM 2
#define NLSE_MEX_METHOD 1
#define NLSE_MEX_PRECISION 1
#include "nlse_mex_gateway.h"
