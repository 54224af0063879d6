/* MEX gateway NLSE3D_TAKE_STEPS_CD_CUDA_M: 3D, CD, mixed precision (nlse_mex_gateway.h). */
#include <string.h>
#define NLSE_MEX_NDIM 3
#define NLSE_MEX_METHOD 1
#define NLSE_MEX_PRECISION 3
#include "nlse_mex_gateway.h"
