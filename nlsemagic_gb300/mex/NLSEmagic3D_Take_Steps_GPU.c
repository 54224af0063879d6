/* v2 MEX gateway NLSEmagic3D_Take_Steps_GPU(U,V,s,a,h2,BC,chunk,k,precision,method) (nlse_mex_gateway.h). */
#include <string.h>
#define NLSE_MEX_NDIM 3
#define NLSE_MEX_V2 1
#include "nlse_mex_gateway.h"
