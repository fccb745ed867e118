// af_api.cu -- the C ABI of libaf (declared in include/af.h).
#include <cstring>
#include <string>

#include "af_api.h"

using namespace af;

namespace af {
cudaError_t batch_run(BatchPlan* B, bool inverse, const float2* in, float2* out, const float* w, double* loss,
                      cudaStream_t st);
i64 batch_launches(BatchPlan* B);
// the persistent executor (af_fast_plan.cu)
struct FastBatch;
FastBatch* fast_create(const i64* ns, i64 count, bool emu, const int* tune, int ntune);
void fast_destroy(FastBatch* B);
cudaError_t fast_exec(FastBatch* B, int sign, const float2* in, float2* out, const float* w, double* loss,
                      cudaStream_t st);
int fast_status(FastBatch* B, cudaStream_t st);
bool fast_supports(const i64* ns, i64 count);
FastBatch* fast_create_tuned(const i64* ns, i64 count, const char* cache_path, cudaStream_t st, std::string* report);
std::string fast_tuning(FastBatch* B);
std::string fast_describe(FastBatch* B);
bool fast_poison_wait(FastBatch* B, long long spin_limit);
}  // namespace af

// A batch runs on the persistent executor (one launch per call) when every
// length fits its tables; otherwise on the multi-launch batch plan.
struct af_batch_s {
  af::FastBatch* f = nullptr;
  af::BatchPlan* b = nullptr;
  int sign = -1;
  std::string autotune;  // the autotuner's report (af_batch_create_tuned)
  ~af_batch_s() {
    af::fast_destroy(f);
    af::batch_destroy(b);
  }
};

static thread_local std::string g_err;

static af_status fail(af_status code, const std::string& msg) {
  g_err = msg;
  return code;
}

void af::set_last_error(const std::string& m) { g_err = m; }

af_status af::api_fail(af_status code, const std::string& msg) { return fail(code, msg); }

af_plan_s::~af_plan_s() {
  af::state_destroy(s32);
  af64::state_destroy(s64);
}

namespace af {
const Node* plan_root(Planner& pl, i64 n, int algo) {
  auto need = [&](bool ok, const char* what) {
    if (!ok) throw AfError(AF_ERR_INVALID, std::string("size ") + std::to_string(n) + " is not " + what);
  };
  switch (algo) {
    case AF_ALGO_AUTO: return pl.automatic(n);
    case AF_ALGO_DECOMPOSE: return pl.decompose(n);
    case AF_ALGO_CHIRP2: return n < 2 ? pl.decompose(n) : pl.chirp(n, ceiling_power_of_two(2 * n - 1));
    case AF_ALGO_CHIRP235: return n < 2 ? pl.decompose(n) : pl.chirp(n, ceiling_5smooth(2 * n - 1));
    case AF_ALGO_PREP_DIT2:
    case AF_ALGO_PREP_DIF2:
    case AF_ALGO_PREP_SPLITRADIX:
    case AF_ALGO_ADHOC_DIT2:
    case AF_ALGO_ADHOC_SPLITRADIX:
      need(n <= 1 || is_pow2(n), "a power of two");
      return pl.decompose(n);
    case AF_ALGO_ADHOC_DIT235:
      need(n <= 1 || is_5smooth(n), "5-smooth");
      return pl.decompose(n);
    case AF_ALGO_ADHOC_AUTO:  // Adhoc.hs:74-84
      if (n <= 1 || is_5smooth(n)) return pl.decompose(n);
      return pl.chirp(n, adhoc_ceiling_5smooth(2 * n));
    case AF_ALGO_ADHOC_CHIRP2:
      return n <= 1 ? pl.decompose(n) : pl.chirp(n, adhoc_pow2_pad(n));
    case AF_ALGO_ADHOC_CHIRP235:
      return n <= 1 ? pl.decompose(n) : pl.chirp(n, adhoc_ceiling_5smooth(2 * n));
  }
  throw AfError(AF_ERR_INVALID, "unknown algorithm");
}
}  // namespace af

extern "C" {

const char* af_version(void) { return "libaf 0.2 (sm_103a)"; }
const char* af_last_error(void) { return g_err.c_str(); }

af_status af_plan_destroy(af_plan plan) {
  AF_TRY
  delete plan;
  return AF_OK;
  AF_CATCH
}

af_status af_plan_describe(af_plan plan, char* buf, size_t len) {
  AF_TRY
  if (!plan || !buf) return fail(AF_ERR_INVALID, "null argument");
  const std::string s = Planner::describe(plan->root);
  if (s.size() + 1 > len) return fail(AF_ERR_INVALID, "buffer too small");
  memcpy(buf, s.c_str(), s.size() + 1);
  return AF_OK;
  AF_CATCH
}

af_status af_plan_tree(int64_t n, af_algo algo, char* buf, size_t len) {
  AF_TRY
  if (!buf || n < 0) return fail(AF_ERR_INVALID, "bad argument");
  Planner pl;
  const std::string s = Planner::describe(plan_root(pl, n, algo));
  if (s.size() + 1 > len) return fail(AF_ERR_INVALID, "buffer too small");
  memcpy(buf, s.c_str(), s.size() + 1);
  return AF_OK;
  AF_CATCH
}

af_status af_plan_launches(af_plan plan, int64_t batch, int64_t* launches) {
  AF_TRY
  if (!plan || !launches || batch < 0) return fail(AF_ERR_INVALID, "bad argument");
  if (batch == 0 || plan->n == 0) *launches = 0;
  else if (plan->s64) *launches = af64::state_launches(plan, batch);
  else *launches = af::state_launches(plan, batch);
  return AF_OK;
  AF_CATCH
}

// ----------------------------------------------------------------- batches
af_status af_batch_create(af_batch* batch, const int64_t* lengths, int64_t count, int sign) {
  AF_TRY
  if (!batch || (!lengths && count)) return fail(AF_ERR_INVALID, "null argument");
  *batch = nullptr;
  if (count < 0) return fail(AF_ERR_INVALID, "negative count");
  if (sign != 1 && sign != -1) return fail(AF_ERR_INVALID, "sign must be -1 or +1");
  af_batch_s* B = new af_batch_s();
  B->sign = sign;
  try {
    if (fast_supports((const i64*)lengths, count)) B->f = fast_create((const i64*)lengths, count, false, nullptr, 0);
    else B->b = batch_create((const i64*)lengths, count, sign);
  } catch (...) {
    delete B;
    throw;
  }
  *batch = B;
  return AF_OK;
  AF_CATCH
}

af_status af_batch_create_tuned(af_batch* batch, const int64_t* lengths, int64_t count, int sign,
                                const char* cache_path, af_stream stream) {
  AF_TRY
  if (!batch || (!lengths && count)) return fail(AF_ERR_INVALID, "null argument");
  *batch = nullptr;
  if (count < 0) return fail(AF_ERR_INVALID, "negative count");
  if (sign != 1 && sign != -1) return fail(AF_ERR_INVALID, "sign must be -1 or +1");
  af_batch_s* B = new af_batch_s();
  B->sign = sign;
  try {
    if (fast_supports((const i64*)lengths, count))
      B->f = fast_create_tuned((const i64*)lengths, count, cache_path, (cudaStream_t)stream, &B->autotune);
    else
      B->b = batch_create((const i64*)lengths, count, sign);
  } catch (...) {
    delete B;
    throw;
  }
  *batch = B;
  return AF_OK;
  AF_CATCH
}

af_status af_batch_describe(af_batch batch, char* buf, size_t len) {
  AF_TRY
  if (!batch || !buf) return fail(AF_ERR_INVALID, "null argument");
  std::string s;
  if (batch->f)
    s = "{\"executor\": \"persistent\", \"plan\": " + fast_describe(batch->f) + ", \"tuning\": " +
        fast_tuning(batch->f) + (batch->autotune.empty() ? std::string() : ", \"autotune\": " +
                                 (batch->autotune == "cached" ? std::string("\"cached\"") : batch->autotune)) +
        "}";
  else
    s = "{\"executor\": \"multi-launch\", \"launches\": " + std::to_string(batch_launches(batch->b)) + "}";
  if (s.size() + 1 > len) return fail(AF_ERR_INVALID, "buffer too small");
  memcpy(buf, s.c_str(), s.size() + 1);
  return AF_OK;
  AF_CATCH
}

af_status af_batch_destroy(af_batch batch) {
  AF_TRY
  delete batch;
  return AF_OK;
  AF_CATCH
}

af_status af_batch_launches(af_batch batch, int64_t* launches) {
  AF_TRY
  if (!batch || !launches) return fail(AF_ERR_INVALID, "null argument");
  *launches = batch->f ? 1 : batch_launches(batch->b);
  return AF_OK;
  AF_CATCH
}

static af_status batch_exec_impl(af_batch batch, bool inverse, const float* in, float* out, const float* w,
                                 double* loss, af_stream stream) {
  AF_TRY
  if (!batch || !in || !out) return fail(AF_ERR_INVALID, "null argument");
  if (((uintptr_t)in | (uintptr_t)out) & 7) return fail(AF_ERR_INVALID, "data must be 8-byte aligned");
  if (w && !loss) return fail(AF_ERR_INVALID, "the cotangent epilogue needs a loss accumulator");
  if (loss) check_cuda(cudaMemsetAsync(loss, 0, sizeof(double), (cudaStream_t)stream), "loss reset");
  if (batch->f)
    check_cuda(fast_exec(batch->f, inverse ? -batch->sign : batch->sign, (const float2*)in, (float2*)out, w, loss,
                         (cudaStream_t)stream),
               "batch launch");
  else
    check_cuda(batch_run(batch->b, inverse, (const float2*)in, (float2*)out, w, loss, (cudaStream_t)stream),
               "batch launch");
  return AF_OK;
  AF_CATCH
}

af_status af_batch_status(af_batch batch, af_stream stream) {
  AF_TRY
  if (!batch) return fail(AF_ERR_INVALID, "null argument");
  if (!batch->f) {
    check_cuda(cudaStreamSynchronize((cudaStream_t)stream), "batch status");
    return AF_OK;
  }
  if (fast_status(batch->f, (cudaStream_t)stream) != 0)
    return fail(AF_ERR_TIMEOUT, "a work item of the last batch call waited too long for its previous stage");
  return AF_OK;
  AF_CATCH
}

af_status af_batch_exec(af_batch batch, const float* in, float* out, af_stream stream) {
  return batch_exec_impl(batch, false, in, out, nullptr, nullptr, stream);
}

af_status af_batch_vjp(af_batch batch, const float* cot, float* grad, af_stream stream) {
  return batch_exec_impl(batch, true, cot, grad, nullptr, nullptr, stream);
}

af_status af_batch_forward_cotangent(af_batch batch, const float* x, const float* w, float* cot, double* loss,
                                     af_stream stream) {
  if (!w) return fail(AF_ERR_INVALID, "null weights");
  return batch_exec_impl(batch, false, x, cot, w, loss, stream);
}

}  // extern "C"

// Test hook of the timeout path (internal, used by the GPU tests): see
// fast_poison_wait.  Returns 0 when the batch's next call will time out.
extern "C" __attribute__((visibility("default"))) int afx_batch_poison_wait(af_batch batch, long long spin_limit) {
  try {
    if (!batch || !batch->f) return 1;
    return af::fast_poison_wait(batch->f, spin_limit) ? 0 : 1;
  } catch (const std::exception& e) {
    g_err = e.what();
    return -1;
  }
}
