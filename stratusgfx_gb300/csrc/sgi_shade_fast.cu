// sgi_shade_fast.cu - the tolerance-mode build of the shading kernels: the
// same source as sgi_shade.cu, compiled with SGI_FAST_MATH = 1 and the
// compiler's fast arithmetic (see sgi_shade.cu and sgi_math.cuh).
#define SGI_FAST_MATH 1
#include "sgi_shade.cu"
