// af_api.h -- error handling shared by the translation units of libaf's C ABI
// (af_api.cu and both precisions of af_api_typed.cu).
#pragma once
#include <string>

#include "af_host.h"

namespace af {
// records the message for af_last_error() and returns the code
af_status api_fail(af_status code, const std::string& msg);
}  // namespace af

// Every entry point converts exceptions to status codes; each translation
// unit defines its own `fail`.
#define AF_TRY try {
#define AF_CATCH                                                                          \
  }                                                                                       \
  catch (const af::AfError& e) { return fail(e.code, e.what()); }                        \
  catch (const std::bad_alloc&) { return fail(AF_ERR_ALLOC, "host allocation failed"); } \
  catch (const std::exception& e) { return fail(AF_ERR_INVALID, e.what()); }

static inline void check_cuda(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw af::AfError(AF_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
