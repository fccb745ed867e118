// af_check64.cu -- the address checker over the Complex Double (FP64) engine:
// afx_*_f64 entry points, namespace af64.
#define AF_F64 1
#include "af_check.cu"
