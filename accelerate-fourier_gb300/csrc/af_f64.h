// af_f64.h -- the Complex Double engine (namespace af64) as the C ABI sees
// it: plans over the same plan trees, lowering and kernels as the Complex
// Float engine, compiled with double2 elements.
#pragma once
#include <cuda_runtime.h>

namespace af64 {

struct Plan;

// Plan of the reference tree for size n and algorithm `algo` (an af_algo);
// throws af::AfError.
Plan* plan_create(long long n, int sign, int algo);
void plan_destroy(Plan* p);
long long plan_n(const Plan* p);
// One transform of sign `sign` over `batch` rows: interleaved (double2) data
// when the im pointers are null, else planar re/im arrays.
void plan_exec(Plan* p, int sign, const double* in_re, const double* in_im, double* out_re, double* out_im,
               long long batch, cudaStream_t st);
long long plan_launches(Plan* p, long long batch);
// The plan's transform along the middle axis of an (outer, n, inner) array.
void plan_exec_axis(Plan* p, const double* in_re, const double* in_im, double* out_re, double* out_im,
                    long long outer, long long inner, cudaStream_t st);

}  // namespace af64
