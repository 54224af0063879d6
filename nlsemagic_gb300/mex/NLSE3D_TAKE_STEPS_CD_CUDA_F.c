/* MEX gateway NLSE3D_TAKE_STEPS_CD_CUDA_F: 3D, CD, single precision (nlse_mex_gateway.h). */
#include <string.h>
#define NLSE_MEX_NDIM 3
#define NLSE_MEX_METHOD 1
#define NLSE_MEX_PRECISION 1
#include "nlse_mex_gateway.h"
