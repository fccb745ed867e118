// af_api_typed64.cu -- the Complex Double (_f64) entry points: af_api_typed.cu
// compiled with double2 elements, in namespace af64.
#define AF_F64 1
#include "af_api_typed.cu"
