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
  if (p64) af64::plan_destroy(p64);
  if (ws) cudaFree(ws);
  if (stage) cudaFree(stage);
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

static void need_f32(const af_plan_s* P) {
  if (P->p64) throw AfError(AF_ERR_INVALID, "the plan is Complex Double: use the _f64 entry points");
}

static Program& program_for(af_plan_s* P, i64 batch, int sign) {
  need_f32(P);
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

// Program of the plan's tree along the middle axis of an (outer, n, inner)
// array (inner = 1: contiguous rows).
static Program& axis_program(af_plan_s* P, i64 outer, i64 inner, int sign) {
  need_f32(P);
  if (inner == 1) return program_for(P, outer, sign);
  auto key = std::make_tuple((long long)outer, (long long)inner, sign);
  auto it = P->axis_progs.find(key);
  if (it != P->axis_progs.end()) return it->second;
  Program& prog = P->axis_progs[key];
  View in;
  in.buf = BUF_IN;
  in.off = 0;
  in.s_e = inner;
  in.s_lo = 1;
  in.lo_cnt = inner;
  in.s_hi = P->n * inner;
  View out = in;
  out.buf = BUF_OUT;
  build_program_view(P->res, P->root, (float)sign, outer * inner, in, out, &prog);
  return prog;
}

static float2* ensure_stage(af_plan_s* P, i64 elems) {
  if ((size_t)elems <= P->stage_elems) return P->stage;
  if (P->stage) { cudaFree(P->stage); P->stage = nullptr; P->stage_elems = 0; }
  if (cudaMalloc(&P->stage, sizeof(float2) * (size_t)elems) != cudaSuccess)
    throw AfError(AF_ERR_ALLOC, "staging allocation failed");
  P->stage_elems = (size_t)elems;
  return P->stage;
}

// Runs a program of plan P with the given input/output bases.
static void run_with(af_plan_s* P, Program& prog, const float* in_re, const float* in_im, float* out_re,
                     float* out_im, cudaStream_t st) {
  ensure_ws(P, prog.ws_elems);
  TileBases b = make_bases(in_re, in_im, out_re, out_im, P->ws, nullptr, nullptr);
  check_cuda(run_program(prog, b, nullptr, st), "launch");
}

static CPtr cptr(af_layout layout, const float* re, const float* im) {
  CPtr p;
  if (layout == AF_LAYOUT_PLANAR) {
    p.c = nullptr;
    p.re = (float*)re;
    p.im = (float*)im;
  } else {
    p.c = (float2*)re;
    p.re = p.im = nullptr;
  }
  return p;
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

af_status af_plan_create_f64(af_plan* plan, int64_t n, int sign, af_algo algo) {
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
    P->p64 = af64::plan_create(n, sign, algo);
    // build the batch-1 program now so that tables are generated at plan time
    if (n > 0) af64::plan_launches(P->p64, 1);
    check_cuda(cudaDeviceSynchronize(), "plan tables");
  } catch (...) {
    delete P;
    throw;
  }
  *plan = P;
  return AF_OK;
  AF_CATCH
}

static af_status exec_sign_f64(af_plan plan, int sign, af_layout layout, const double* in_re, const double* in_im,
                               double* out_re, double* out_im, int64_t batch, af_stream stream) {
  AF_TRY
  if (!plan) return fail(AF_ERR_INVALID, "null plan");
  if (!plan->p64) return fail(AF_ERR_INVALID, "the plan is Complex Float: use the entry points without _f64");
  if (batch < 0) return fail(AF_ERR_INVALID, "negative batch");
  if (batch == 0 || plan->n == 0) return AF_OK;
  if (layout != AF_LAYOUT_INTERLEAVED && layout != AF_LAYOUT_PLANAR) return fail(AF_ERR_INVALID, "bad layout");
  if (!in_re || !out_re) return fail(AF_ERR_INVALID, "null data pointer");
  const bool planar = layout == AF_LAYOUT_PLANAR;
  if (planar && (!in_im || !out_im)) return fail(AF_ERR_INVALID, "planar layout needs im pointers");
  if (!planar && (((uintptr_t)in_re | (uintptr_t)out_re) & 15))
    return fail(AF_ERR_INVALID, "interleaved Complex Double data must be 16-byte aligned");
  if (plan->n * batch >= ((i64)1 << 31)) return fail(AF_ERR_UNSUPPORTED, "n * batch must be below 2^31");
  af64::plan_exec(plan->p64, sign, in_re, planar ? in_im : nullptr, out_re, planar ? out_im : nullptr, batch,
                  (cudaStream_t)stream);
  return AF_OK;
  AF_CATCH
}

af_status af_exec_c2c_f64(af_plan plan, af_layout layout, const double* in_re, const double* in_im,
                          double* out_re, double* out_im, int64_t batch, af_stream stream) {
  if (!plan) return fail(AF_ERR_INVALID, "null plan");
  return exec_sign_f64(plan, plan->sign, layout, in_re, in_im, out_re, out_im, batch, stream);
}

af_status af_vjp_c2c_f64(af_plan plan, af_layout layout, const double* cot_re, const double* cot_im,
                         double* grad_re, double* grad_im, int64_t batch, af_stream stream) {
  if (!plan) return fail(AF_ERR_INVALID, "null plan");
  return exec_sign_f64(plan, -plan->sign, layout, cot_re, cot_im, grad_re, grad_im, batch, stream);
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
  if (batch == 0 || plan->n == 0) *launches = 0;
  else if (plan->p64) *launches = af64::plan_launches(plan->p64, batch);
  else *launches = (int64_t)program_for(plan, batch, plan->sign).launches.size();
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

// ================================================================ axes, real transforms, convolution
static void check_plan_size(af_plan_s* P, i64 rows) {
  if (P->n * rows >= ((i64)1 << 31)) throw AfError(AF_ERR_UNSUPPORTED, "n * rows must be below 2^31");
}

// in (outer, n, inner) -> out along the middle axis with plan P's sign; an
// im pointer of nullptr means interleaved data
static void run_axis(af_plan_s* P, const float* in_re, const float* in_im, float* out_re, float* out_im, i64 outer,
                     i64 inner, cudaStream_t st) {
  if (outer == 0 || inner == 0 || P->n == 0) return;
  check_plan_size(P, outer * inner);
  Program& prog = axis_program(P, outer, inner, P->sign);
  run_with(P, prog, in_re, in_im, out_re, out_im, st);
}

// the multi-axis transforms: plans[0] runs along the last axis
static void run_nd(af_plan_s* const* plans, int dims, const float* in_re, const float* in_im, float* out_re,
                   float* out_im, i64 batch, cudaStream_t st) {
  i64 total = batch;
  for (int d = 0; d < dims; ++d) {
    if (!plans[d]) throw AfError(AF_ERR_INVALID, "null plan");
    total *= plans[d]->n;
  }
  if (total == 0) return;
  if (total >= ((i64)1 << 31)) throw AfError(AF_ERR_UNSUPPORTED, "array must hold fewer than 2^31 values");
  i64 inner = 1;
  for (int d = 0; d < dims; ++d) {
    const i64 outer = total / (inner * plans[d]->n);
    if (d == 0) run_axis(plans[d], in_re, in_im, out_re, out_im, outer, inner, st);
    else run_axis(plans[d], out_re, out_im, out_re, out_im, outer, inner, st);
    inner *= plans[d]->n;
  }
}

// the multi-axis Complex Double transforms (same axis order as run_nd)
static void run_nd_f64(af_plan_s* const* plans, int dims, const double* in_re, const double* in_im,
                       double* out_re, double* out_im, i64 batch, cudaStream_t st) {
  i64 total = batch;
  for (int d = 0; d < dims; ++d) {
    if (!plans[d]) throw AfError(AF_ERR_INVALID, "null plan");
    if (!plans[d]->p64) throw AfError(AF_ERR_INVALID, "the plan is Complex Float: use the entry points without _f64");
    total *= plans[d]->n;
  }
  if (total == 0) return;
  if (total >= ((i64)1 << 31)) throw AfError(AF_ERR_UNSUPPORTED, "array must hold fewer than 2^31 values");
  i64 inner = 1;
  for (int d = 0; d < dims; ++d) {
    const i64 outer = total / (inner * plans[d]->n);
    if (d == 0) af64::plan_exec_axis(plans[d]->p64, in_re, in_im, out_re, out_im, outer, inner, st);
    else af64::plan_exec_axis(plans[d]->p64, out_re, out_im, out_re, out_im, outer, inner, st);
    inner *= plans[d]->n;
  }
}

static void check_io_f64(af_layout layout, const double* a_re, const double* a_im, const double* b_re,
                         const double* b_im) {
  if (layout != AF_LAYOUT_INTERLEAVED && layout != AF_LAYOUT_PLANAR) throw AfError(AF_ERR_INVALID, "bad layout");
  if (!a_re || !b_re) throw AfError(AF_ERR_INVALID, "null data pointer");
  if (layout == AF_LAYOUT_PLANAR && (!a_im || !b_im)) throw AfError(AF_ERR_INVALID, "planar layout needs im pointers");
  if (layout == AF_LAYOUT_INTERLEAVED && (((uintptr_t)a_re | (uintptr_t)b_re) & 15))
    throw AfError(AF_ERR_INVALID, "interleaved Complex Double data must be 16-byte aligned");
}

extern "C" {

af_status af_exec_c2c_2d_f64(af_plan plan0, af_plan plan1, af_layout layout, const double* in_re,
                             const double* in_im, double* out_re, double* out_im, int64_t batch, af_stream stream) {
  AF_TRY
  if (batch < 0) return fail(AF_ERR_INVALID, "negative batch");
  if (!plan0 || !plan1) return fail(AF_ERR_INVALID, "null plan");
  af_plan_s* plans[2] = {plan0, plan1};
  if (batch == 0 || plan0->n == 0 || plan1->n == 0) return AF_OK;
  check_io_f64(layout, in_re, in_im, out_re, out_im);
  const bool planar = layout == AF_LAYOUT_PLANAR;
  run_nd_f64(plans, 2, in_re, planar ? in_im : nullptr, out_re, planar ? out_im : nullptr, batch,
             (cudaStream_t)stream);
  return AF_OK;
  AF_CATCH
}

af_status af_exec_c2c_3d_f64(af_plan plan0, af_plan plan1, af_plan plan2, af_layout layout, const double* in_re,
                             const double* in_im, double* out_re, double* out_im, int64_t batch, af_stream stream) {
  AF_TRY
  if (batch < 0) return fail(AF_ERR_INVALID, "negative batch");
  if (!plan0 || !plan1 || !plan2) return fail(AF_ERR_INVALID, "null plan");
  af_plan_s* plans[3] = {plan0, plan1, plan2};
  if (batch == 0 || plan0->n == 0 || plan1->n == 0 || plan2->n == 0) return AF_OK;
  check_io_f64(layout, in_re, in_im, out_re, out_im);
  const bool planar = layout == AF_LAYOUT_PLANAR;
  run_nd_f64(plans, 3, in_re, planar ? in_im : nullptr, out_re, planar ? out_im : nullptr, batch,
             (cudaStream_t)stream);
  return AF_OK;
  AF_CATCH
}

af_status af_exec_c2c_axis(af_plan plan, af_layout layout, const float* in_re, const float* in_im, float* out_re,
                           float* out_im, int64_t outer, int64_t inner, af_stream stream) {
  AF_TRY
  if (!plan) return fail(AF_ERR_INVALID, "null plan");
  if (outer < 0 || inner < 0) return fail(AF_ERR_INVALID, "negative size");
  if (outer == 0 || inner == 0 || plan->n == 0) return AF_OK;
  check_io(layout, in_re, in_im, out_re, out_im);
  const bool planar = layout == AF_LAYOUT_PLANAR;
  run_axis(plan, in_re, planar ? in_im : nullptr, out_re, planar ? out_im : nullptr, outer, inner,
           (cudaStream_t)stream);
  return AF_OK;
  AF_CATCH
}

af_status af_exec_c2c_2d(af_plan plan0, af_plan plan1, af_layout layout, const float* in_re, const float* in_im,
                         float* out_re, float* out_im, int64_t batch, af_stream stream) {
  AF_TRY
  if (batch < 0) return fail(AF_ERR_INVALID, "negative batch");
  af_plan_s* plans[2] = {plan0, plan1};
  if (!plan0 || !plan1) return fail(AF_ERR_INVALID, "null plan");
  if (batch == 0 || plan0->n == 0 || plan1->n == 0) return AF_OK;
  check_io(layout, in_re, in_im, out_re, out_im);
  const bool planar = layout == AF_LAYOUT_PLANAR;
  run_nd(plans, 2, in_re, planar ? in_im : nullptr, out_re, planar ? out_im : nullptr, batch, (cudaStream_t)stream);
  return AF_OK;
  AF_CATCH
}

af_status af_exec_c2c_3d(af_plan plan0, af_plan plan1, af_plan plan2, af_layout layout, const float* in_re,
                         const float* in_im, float* out_re, float* out_im, int64_t batch, af_stream stream) {
  AF_TRY
  if (batch < 0) return fail(AF_ERR_INVALID, "negative batch");
  af_plan_s* plans[3] = {plan0, plan1, plan2};
  if (!plan0 || !plan1 || !plan2) return fail(AF_ERR_INVALID, "null plan");
  if (batch == 0 || plan0->n == 0 || plan1->n == 0 || plan2->n == 0) return AF_OK;
  check_io(layout, in_re, in_im, out_re, out_im);
  const bool planar = layout == AF_LAYOUT_PLANAR;
  run_nd(plans, 3, in_re, planar ? in_im : nullptr, out_re, planar ? out_im : nullptr, batch, (cudaStream_t)stream);
  return AF_OK;
  AF_CATCH
}

af_status af_to_spectrum(af_plan half, const float* x, af_spectrum spectrum, af_layout layout, float* out_re,
                         float* out_im, int64_t batch, af_stream stream) {
  AF_TRY
  if (!half) return fail(AF_ERR_INVALID, "null plan");
  if (batch < 0) return fail(AF_ERR_INVALID, "negative batch");
  if (spectrum != AF_SPECTRUM_FULL && spectrum != AF_SPECTRUM_HALF) return fail(AF_ERR_INVALID, "bad spectrum");
  const i64 n2 = half->n;
  if (batch == 0 || n2 == 0) return AF_OK;
  if (!x) return fail(AF_ERR_INVALID, "null data pointer");
  if ((uintptr_t)x & 7) return fail(AF_ERR_INVALID, "real input must be 8-byte aligned");
  check_io(layout, out_re, out_im, out_re, out_im);
  check_plan_size(half, 2 * batch);
  cudaStream_t st = (cudaStream_t)stream;
  float2* Z = ensure_stage(half, n2 * batch);
  run_with(half, program_for(half, batch, half->sign), x, nullptr, (float*)Z, nullptr, st);
  TwTable t = half->res.table(2 * n2);
  const i64 nout = spectrum == AF_SPECTRUM_FULL ? 2 * n2 : n2 + 1;
  check_cuda(launch_real_untangle(Z, cptr(layout, out_re, out_im), n2, nout, batch, t.p, t.S_log2, st),
             "toSpectrum untangle");
  return AF_OK;
  AF_CATCH
}

static af_status from_spectrum_impl(af_plan half, af_layout layout, const float* s_re, const float* s_im, float* x,
                                    int64_t batch, af_stream stream, bool vjp) {
  AF_TRY
  if (!half) return fail(AF_ERR_INVALID, "null plan");
  if (batch < 0) return fail(AF_ERR_INVALID, "negative batch");
  const i64 n2 = half->n;
  if (batch == 0 || n2 == 0) return AF_OK;
  if (!x) return fail(AF_ERR_INVALID, "null data pointer");
  if ((uintptr_t)x & 7) return fail(AF_ERR_INVALID, "real output must be 8-byte aligned");
  check_io(layout, s_re, s_im, s_re, s_im);
  if (vjp && half->sign != -1) return fail(AF_ERR_INVALID, "the toSpectrum VJP needs a forward half-length plan");
  check_plan_size(half, 2 * batch);
  cudaStream_t st = (cudaStream_t)stream;
  float2* f = ensure_stage(half, n2 * batch);
  TwTable t = half->res.table(2 * n2);
  check_cuda(launch_real_entangle(cptr(layout, s_re, s_im), f, n2, batch, t.p, t.S_log2, vjp ? 1 : 0, st),
             "fromSpectrum entangle");
  const int sign = vjp ? -half->sign : half->sign;
  run_with(half, program_for(half, batch, sign), (const float*)f, nullptr, x, nullptr, st);
  return AF_OK;
  AF_CATCH
}

af_status af_from_spectrum(af_plan half, af_layout layout, const float* spec_re, const float* spec_im, float* x,
                           int64_t batch, af_stream stream) {
  return from_spectrum_impl(half, layout, spec_re, spec_im, x, batch, stream, false);
}

af_status af_vjp_to_spectrum(af_plan half, af_layout layout, const float* cot_re, const float* cot_im, float* grad,
                             int64_t batch, af_stream stream) {
  return from_spectrum_impl(half, layout, cot_re, cot_im, grad, batch, stream, true);
}

af_status af_untangle_spectra_2d(af_layout layout, const float* s_re, const float* s_im, float* a_re, float* a_im,
                                 float* b_re, float* b_im, int64_t height, int64_t width, int64_t batch,
                                 af_stream stream) {
  AF_TRY
  if (height < 0 || width < 0 || batch < 0) return fail(AF_ERR_INVALID, "negative size");
  const i64 total = height * width * batch;
  if (total == 0) return AF_OK;
  check_io(layout, s_re, s_im, a_re, a_im);
  check_io(layout, s_re, s_im, b_re, b_im);
  if (s_re == a_re || s_re == b_re) return fail(AF_ERR_INVALID, "untangle cannot run in place");
  check_cuda(launch_untangle(cptr(layout, s_re, s_im), cptr(layout, a_re, a_im), cptr(layout, b_re, b_im), height,
                             width, total, (cudaStream_t)stream),
             "untangle");
  return AF_OK;
  AF_CATCH
}

af_status af_untangle_spectra(af_layout layout, const float* s_re, const float* s_im, float* a_re, float* a_im,
                              float* b_re, float* b_im, int64_t n, int64_t batch, af_stream stream) {
  return af_untangle_spectra_2d(layout, s_re, s_im, a_re, a_im, b_re, b_im, 1, n, batch, stream);
}

af_status af_cyclic_reverse_2d(af_layout layout, const float* in_re, const float* in_im, float* out_re,
                               float* out_im, int64_t height, int64_t width, int64_t batch, af_stream stream) {
  AF_TRY
  if (height < 0 || width < 0 || batch < 0) return fail(AF_ERR_INVALID, "negative size");
  const i64 total = height * width * batch;
  if (total == 0) return AF_OK;
  check_io(layout, in_re, in_im, out_re, out_im);
  if (in_re == out_re) return fail(AF_ERR_INVALID, "cyclic reverse cannot run in place");
  check_cuda(launch_reverse2d(cptr(layout, in_re, in_im), cptr(layout, out_re, out_im), height, width, total,
                              (cudaStream_t)stream),
             "reverse2d");
  return AF_OK;
  AF_CATCH
}

af_status af_entangle_spectra(af_layout layout, const float* c_re, const float* c_im, const float* d_re,
                              const float* d_im, float* out_re, float* out_im, int64_t n, int64_t batch,
                              af_stream stream) {
  AF_TRY
  if (n < 0 || batch < 0) return fail(AF_ERR_INVALID, "negative size");
  if (n == 0 || batch == 0) return AF_OK;
  check_io(layout, c_re, c_im, out_re, out_im);
  check_io(layout, d_re, d_im, out_re, out_im);
  check_cuda(launch_entangle(cptr(layout, c_re, c_im), cptr(layout, d_re, d_im), cptr(layout, out_re, out_im),
                             n * batch, (cudaStream_t)stream),
             "entangle");
  return AF_OK;
  AF_CATCH
}

static af_status two_to_impl(af_plan_s* const* plans, int dims, const float* f, const float* g, af_layout layout,
                             float* a_re, float* a_im, float* b_re, float* b_im, int64_t batch, af_stream stream) {
  AF_TRY
  for (int d = 0; d < dims; ++d)
    if (!plans[d]) return fail(AF_ERR_INVALID, "null plan");
  if (batch < 0) return fail(AF_ERR_INVALID, "negative batch");
  i64 img = 1;
  for (int d = 0; d < dims; ++d) img *= plans[d]->n;
  if (batch == 0 || img == 0) return AF_OK;
  if (!f || !g) return fail(AF_ERR_INVALID, "null data pointer");
  check_io(layout, a_re, a_im, b_re, b_im);
  if (img * batch >= ((i64)1 << 31)) return fail(AF_ERR_UNSUPPORTED, "array must hold fewer than 2^31 values");
  cudaStream_t st = (cudaStream_t)stream;
  float2* S = ensure_stage(plans[0], img * batch);
  run_nd(plans, dims, f, g, (float*)S, nullptr, batch, st);
  const i64 h = dims == 2 ? plans[1]->n : 1, w = plans[0]->n;
  CPtr sp{S, nullptr, nullptr};
  check_cuda(launch_untangle(sp, cptr(layout, a_re, a_im), cptr(layout, b_re, b_im), h, w, img * batch, st),
             "untangle");
  return AF_OK;
  AF_CATCH
}

af_status af_two_to_spectrum(af_plan plan, const float* f, const float* g, af_layout layout, float* a_re,
                             float* a_im, float* b_re, float* b_im, int64_t batch, af_stream stream) {
  af_plan_s* plans[1] = {plan};
  return two_to_impl(plans, 1, f, g, layout, a_re, a_im, b_re, b_im, batch, stream);
}

af_status af_two_to_spectrum_2d(af_plan plan0, af_plan plan1, const float* f, const float* g, af_layout layout,
                                float* a_re, float* a_im, float* b_re, float* b_im, int64_t batch,
                                af_stream stream) {
  af_plan_s* plans[2] = {plan0, plan1};
  return two_to_impl(plans, 2, f, g, layout, a_re, a_im, b_re, b_im, batch, stream);
}

static af_status two_from_impl(af_plan_s* const* plans, int dims, af_layout layout, const float* a_re,
                               const float* a_im, const float* b_re, const float* b_im, float* f, float* g,
                               int64_t batch, af_stream stream) {
  AF_TRY
  for (int d = 0; d < dims; ++d)
    if (!plans[d]) return fail(AF_ERR_INVALID, "null plan");
  if (batch < 0) return fail(AF_ERR_INVALID, "negative batch");
  i64 img = 1;
  for (int d = 0; d < dims; ++d) img *= plans[d]->n;
  if (batch == 0 || img == 0) return AF_OK;
  if (!f || !g) return fail(AF_ERR_INVALID, "null data pointer");
  check_io(layout, a_re, a_im, b_re, b_im);
  if (img * batch >= ((i64)1 << 31)) return fail(AF_ERR_UNSUPPORTED, "array must hold fewer than 2^31 values");
  cudaStream_t st = (cudaStream_t)stream;
  float2* S = ensure_stage(plans[0], img * batch);
  CPtr sp{S, nullptr, nullptr};
  check_cuda(launch_entangle(cptr(layout, a_re, a_im), cptr(layout, b_re, b_im), sp, img * batch, st), "entangle");
  run_nd(plans, dims, (const float*)S, nullptr, f, g, batch, st);
  return AF_OK;
  AF_CATCH
}

af_status af_two_from_spectrum(af_plan plan, af_layout layout, const float* a_re, const float* a_im,
                               const float* b_re, const float* b_im, float* f, float* g, int64_t batch,
                               af_stream stream) {
  af_plan_s* plans[1] = {plan};
  return two_from_impl(plans, 1, layout, a_re, a_im, b_re, b_im, f, g, batch, stream);
}

af_status af_two_from_spectrum_2d(af_plan plan0, af_plan plan1, af_layout layout, const float* a_re,
                                  const float* a_im, const float* b_re, const float* b_im, float* f, float* g,
                                  int64_t batch, af_stream stream) {
  af_plan_s* plans[2] = {plan0, plan1};
  return two_from_impl(plans, 2, layout, a_re, a_im, b_re, b_im, f, g, batch, stream);
}

af_status af_convolve_cyclic(af_plan plan, af_layout layout, const float* x_re, const float* x_im, const float* y_re,
                             const float* y_im, float* out_re, float* out_im, int64_t batch, af_stream stream) {
  AF_TRY
  if (!plan) return fail(AF_ERR_INVALID, "null plan");
  if (batch < 0) return fail(AF_ERR_INVALID, "negative batch");
  const i64 n = plan->n;
  if (batch == 0) return AF_OK;
  if (n == 0) return fail(AF_ERR_INVALID, "convolveCyclic needs non-empty signals");
  check_io(layout, x_re, x_im, out_re, out_im);
  check_io(layout, y_re, y_im, out_re, out_im);
  check_plan_size(plan, 2 * batch);
  cudaStream_t st = (cudaStream_t)stream;
  const bool planar = layout == AF_LAYOUT_PLANAR;
  float2* S = ensure_stage(plan, 2 * n * batch);
  float2* S2 = S + n * batch;
  Program& G = program_for(plan, batch, +1);
  run_with(plan, G, x_re, planar ? x_im : nullptr, (float*)S, nullptr, st);
  run_with(plan, G, y_re, planar ? y_im : nullptr, (float*)S2, nullptr, st);
  check_cuda(launch_conv_mul(S, S2, 1.0f / (float)n, n * batch, st), "convolution product");
  run_with(plan, program_for(plan, batch, -1), (const float*)S, nullptr, out_re, planar ? out_im : nullptr, st);
  return AF_OK;
  AF_CATCH
}

}  // extern "C"
