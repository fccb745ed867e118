// af_real64.cu -- the Complex Double (FP64) build of af_real.cu, in namespace af64.
#define AF_F64 1
#include "af_real.cu"
