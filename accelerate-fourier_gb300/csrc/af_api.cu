// af_api.cu -- the C ABI of libaf (declared in include/af.h).
#include <cstring>
#include <string>

#include "af_host.h"

using namespace af;

namespace af {
cudaError_t batch_run(BatchPlan* B, bool inverse, const float2* in, float2* out, const float* w, double* loss,
                      cudaStream_t st);
i64 batch_launches(BatchPlan* B);
}  // namespace af

struct af_batch_s {
  af::BatchPlan* b = nullptr;
  ~af_batch_s() { af::batch_destroy(b); }
};

static thread_local std::string g_err;

static af_status fail(af_status code, const std::string& msg) {
  g_err = msg;
  return code;
}

void af::set_last_error(const std::string& m) { g_err = m; }

#define AF_TRY try {
#define AF_CATCH                                                                          \
  }                                                                                       \
  catch (const AfError& e) { return fail(e.code, e.what()); }                            \
  catch (const std::bad_alloc&) { return fail(AF_ERR_ALLOC, "host allocation failed"); } \
  catch (const std::exception& e) { return fail(AF_ERR_INVALID, e.what()); }

af_plan_s::~af_plan_s() {
  if (ws) cudaFree(ws);
  res.release();
}

static void check_cuda(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw AfError(AF_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
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

static Program& program_for(af_plan_s* P, i64 batch, int sign) {
  auto key = std::make_pair((long long)batch, sign);
  auto it = P->progs.find(key);
  if (it != P->progs.end()) return it->second;
  Program& prog = P->progs[key];
  build_program(P->res, P->root, (float)sign, batch, &prog);
  return prog;
}

static void ensure_ws(af_plan_s* P, i64 elems) {
  if ((size_t)elems <= P->ws_elems) return;
  if (P->ws) { cudaFree(P->ws); P->ws = nullptr; P->ws_elems = 0; }
  if (cudaMalloc(&P->ws, sizeof(float2) * (size_t)elems) != cudaSuccess)
    throw AfError(AF_ERR_ALLOC, "workspace allocation failed");
  P->ws_elems = (size_t)elems;
}

static void check_io(af_layout layout, const float* a_re, const float* a_im, const float* b_re, const float* b_im) {
  if (layout != AF_LAYOUT_INTERLEAVED && layout != AF_LAYOUT_PLANAR) throw AfError(AF_ERR_INVALID, "bad layout");
  if (!a_re || !b_re) throw AfError(AF_ERR_INVALID, "null data pointer");
  if (layout == AF_LAYOUT_PLANAR && (!a_im || !b_im)) throw AfError(AF_ERR_INVALID, "planar layout needs im pointers");
  if (layout == AF_LAYOUT_INTERLEAVED && (((uintptr_t)a_re | (uintptr_t)b_re) & 7))
    throw AfError(AF_ERR_INVALID, "interleaved data must be 8-byte aligned");
}

static af_status exec_sign(af_plan plan, int sign, af_layout layout, const float* in_re, const float* in_im,
                           float* out_re, float* out_im, int64_t batch, af_stream stream) {
  AF_TRY
  if (!plan) return fail(AF_ERR_INVALID, "null plan");
  if (batch < 0) return fail(AF_ERR_INVALID, "negative batch");
  if (batch == 0 || plan->n == 0) return AF_OK;
  check_io(layout, in_re, in_im, out_re, out_im);
  if (plan->n * batch >= ((i64)1 << 31)) return fail(AF_ERR_UNSUPPORTED, "n * batch must be below 2^31");
  Program& prog = program_for(plan, batch, sign);
  ensure_ws(plan, prog.ws_elems);
  const bool planar = layout == AF_LAYOUT_PLANAR;
  TileBases b = make_bases(in_re, planar ? in_im : nullptr, out_re, planar ? out_im : nullptr, plan->ws,
                           nullptr, nullptr);
  check_cuda(run_program(prog, b, nullptr, (cudaStream_t)stream), "launch");
  return AF_OK;
  AF_CATCH
}

static MapDesc rows_map(int mode, i64 n, i64 batch) {
  MapDesc md;
  memset(&md, 0, sizeof md);
  md.mode = mode;
  md.nlines = batch;
  md.nout = n;
  md.n = n;
  md.scale = 1.f;
  md.dc_ws = md.x0_ws = -1;
  for (IoDesc* io : {&md.in, &md.out}) {
    io->s_e = 1;
    io->s_lo = n;
    io->lo_div = make_fastdiv((unsigned)std::min<i64>(batch, (i64)1 << 30));
  }
  md.in.buf = BUF_IN;
  md.out.buf = BUF_OUT;
  return md;
}

extern "C" {

const char* af_version(void) { return "libaf 0.2 (sm_103a)"; }
const char* af_last_error(void) { return g_err.c_str(); }

af_status af_plan_create(af_plan* plan, int64_t n, int sign, af_algo algo) {
  AF_TRY
  if (!plan) return fail(AF_ERR_INVALID, "null plan pointer");
  *plan = nullptr;
  if (n < 0) return fail(AF_ERR_INVALID, "negative size");
  if (sign != 1 && sign != -1) return fail(AF_ERR_INVALID, "sign must be -1 (forward) or +1 (inverse)");
  if (n >= ((i64)1 << 31)) return fail(AF_ERR_UNSUPPORTED, "size must be below 2^31");
  af_plan_s* P = new af_plan_s();
  try {
    P->n = n;
    P->sign = sign;
    P->algo = algo;
    P->root = plan_root(P->planner, n, algo);
    // build the batch-1 program now so that tables are generated at plan time
    if (n > 0) program_for(P, 1, sign);
    check_cuda(cudaDeviceSynchronize(), "plan tables");
  } catch (...) {
    delete P;
    throw;
  }
  *plan = P;
  return AF_OK;
  AF_CATCH
}

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
  *launches = (batch == 0 || plan->n == 0) ? 0 : (int64_t)program_for(plan, batch, plan->sign).launches.size();
  return AF_OK;
  AF_CATCH
}

af_status af_exec_c2c(af_plan plan, af_layout layout, const float* in_re, const float* in_im, float* out_re,
                      float* out_im, int64_t batch, af_stream stream) {
  if (!plan) return fail(AF_ERR_INVALID, "null plan");
  return exec_sign(plan, plan->sign, layout, in_re, in_im, out_re, out_im, batch, stream);
}

af_status af_vjp_c2c(af_plan plan, af_layout layout, const float* cot_re, const float* cot_im, float* grad_re,
                     float* grad_im, int64_t batch, af_stream stream) {
  if (!plan) return fail(AF_ERR_INVALID, "null plan");
  return exec_sign(plan, -plan->sign, layout, cot_re, cot_im, grad_re, grad_im, batch, stream);
}

af_status af_scale_down(af_layout layout, float* re, float* im, int64_t n, int64_t batch, af_stream stream) {
  AF_TRY
  if (n < 0 || batch < 0) return fail(AF_ERR_INVALID, "negative size");
  if (n == 0 || batch == 0) return AF_OK;
  check_io(layout, re, im, re, im);
  MapDesc md = rows_map(MAP_SCALE, n, batch);
  md.scale = 1.0f / (float)n;
  const bool planar = layout == AF_LAYOUT_PLANAR;
  TileBases b = make_bases(re, planar ? im : nullptr, re, planar ? im : nullptr, nullptr, nullptr, nullptr);
  check_cuda(launch_map(md, b, (cudaStream_t)stream), "scale_down");
  return AF_OK;
  AF_CATCH
}

af_status af_cyclic_reverse(af_layout layout, const float* in_re, const float* in_im, float* out_re, float* out_im,
                            int64_t n, int64_t batch, af_stream stream) {
  AF_TRY
  if (n < 0 || batch < 0) return fail(AF_ERR_INVALID, "negative size");
  if (n == 0 || batch == 0) return AF_OK;
  check_io(layout, in_re, in_im, out_re, out_im);
  if (in_re == out_re) return fail(AF_ERR_INVALID, "cyclic reverse cannot run in place");
  MapDesc md = rows_map(MAP_REVERSE, n, batch);
  const bool planar = layout == AF_LAYOUT_PLANAR;
  TileBases b = make_bases(in_re, planar ? in_im : nullptr, out_re, planar ? out_im : nullptr, nullptr, nullptr,
                           nullptr);
  check_cuda(launch_map(md, b, (cudaStream_t)stream), "cyclic_reverse");
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
  try {
    B->b = batch_create((const i64*)lengths, count, sign);
  } catch (...) {
    delete B;
    throw;
  }
  *batch = B;
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
  *launches = batch_launches(batch->b);
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
  check_cuda(batch_run(batch->b, inverse, (const float2*)in, (float2*)out, w, loss, (cudaStream_t)stream),
             "batch launch");
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
