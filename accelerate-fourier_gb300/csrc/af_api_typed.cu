// af_api_typed.cu -- the entry points of libaf's C ABI that carry complex
// data: plans, complex transforms, multi-axis transforms, real and two-real
// transforms, cyclic convolution, reverse and scaleDown.  This file compiles
// twice: for Complex Float with the names of include/af.h, and with AF_F64
// defined (af_api_typed64.cu) for Complex Double with the same names and an
// _f64 suffix.  A plan holds the state of the precision it was created for.
#include <cstring>

#include "af_api.h"

#ifdef AF_F64
#define AFN(name) name##_f64
#define AF_STATE s64
static const char* const kAlignMsg = "interleaved Complex Double data must be 16-byte aligned";
static const char* const kOtherKind = "the plan is Complex Float: use the entry points without _f64";
#else
#define AFN(name) name
#define AF_STATE s32
static const char* const kAlignMsg = "interleaved data must be 8-byte aligned";
static const char* const kOtherKind = "the plan is Complex Double: use the _f64 entry points";
#endif

using namespace AF_NS;

static af_status fail(af_status code, const std::string& msg) { return af::api_fail(code, msg); }

namespace AF_NS {
PlanState::~PlanState() {
  if (ws) cudaFree(ws);
  if (stage) cudaFree(stage);
  res.release();
}
void state_destroy(PlanState* s) { delete s; }
}  // namespace AF_NS

// The plan's state of this precision; a plan of the other precision is refused.
static AF_NS::PlanState* state(const af_plan_s* P) {
  if (!P->AF_STATE) throw AfError(AF_ERR_INVALID, kOtherKind);
  return P->AF_STATE;
}

static Program& program_for(af_plan_s* P, i64 batch, int sign) {
  AF_NS::PlanState* S = state(P);
  auto key = std::make_pair((long long)batch, sign);
  auto it = S->progs.find(key);
  if (it != S->progs.end()) return it->second;
  Program& prog = S->progs[key];
  build_program(S->res, P->root, (rl)sign, batch, &prog);
  return prog;
}


static void ensure_ws(af_plan_s* P, i64 elems) {
  AF_NS::PlanState* S = state(P);
  if ((size_t)elems <= S->ws_elems) return;
  if (S->ws) { cudaFree(S->ws); S->ws = nullptr; S->ws_elems = 0; }
  if (cudaMalloc(&S->ws, sizeof(cx) * (size_t)elems) != cudaSuccess)
    throw AfError(AF_ERR_ALLOC, "workspace allocation failed");
  S->ws_elems = (size_t)elems;
}


// Program of the plan's tree along the middle axis of an (outer, n, inner)
// array (inner = 1: contiguous rows).
static Program& axis_program(af_plan_s* P, i64 outer, i64 inner, int sign) {
  if (inner == 1) return program_for(P, outer, sign);
  AF_NS::PlanState* S = state(P);
  auto key = std::make_tuple((long long)outer, (long long)inner, sign);
  auto it = S->axis_progs.find(key);
  if (it != S->axis_progs.end()) return it->second;
  Program& prog = S->axis_progs[key];
  View in;
  in.buf = BUF_IN;
  in.off = 0;
  in.s_e = inner;
  in.s_lo = 1;
  in.lo_cnt = inner;
  in.s_hi = P->n * inner;
  View out = in;
  out.buf = BUF_OUT;
  build_program_view(S->res, P->root, (rl)sign, outer * inner, in, out, &prog);
  return prog;
}


static cx* ensure_stage(af_plan_s* P, i64 elems) {
  AF_NS::PlanState* S = state(P);
  if ((size_t)elems <= S->stage_elems) return S->stage;
  if (S->stage) { cudaFree(S->stage); S->stage = nullptr; S->stage_elems = 0; }
  if (cudaMalloc(&S->stage, sizeof(cx) * (size_t)elems) != cudaSuccess)
    throw AfError(AF_ERR_ALLOC, "staging allocation failed");
  S->stage_elems = (size_t)elems;
  return S->stage;
}


// Runs a program of plan P with the given input/output bases.
static void run_with(af_plan_s* P, Program& prog, const rl* in_re, const rl* in_im, rl* out_re,
                     rl* out_im, cudaStream_t st) {
  ensure_ws(P, prog.ws_elems);
  TileBases b = make_bases(in_re, in_im, out_re, out_im, state(P)->ws, nullptr, nullptr);
  check_cuda(run_program(prog, b, nullptr, st), "launch");
}


static CPtr cptr(af_layout layout, const rl* re, const rl* im) {
  CPtr p;
  if (layout == AF_LAYOUT_PLANAR) {
    p.c = nullptr;
    p.re = (rl*)re;
    p.im = (rl*)im;
  } else {
    p.c = (cx*)re;
    p.re = p.im = nullptr;
  }
  return p;
}


static void check_io(af_layout layout, const rl* a_re, const rl* a_im, const rl* b_re, const rl* b_im) {
  if (layout != AF_LAYOUT_INTERLEAVED && layout != AF_LAYOUT_PLANAR) throw AfError(AF_ERR_INVALID, "bad layout");
  if (!a_re || !b_re) throw AfError(AF_ERR_INVALID, "null data pointer");
  if (layout == AF_LAYOUT_PLANAR && (!a_im || !b_im)) throw AfError(AF_ERR_INVALID, "planar layout needs im pointers");
  if (layout == AF_LAYOUT_INTERLEAVED && (((uintptr_t)a_re | (uintptr_t)b_re) & (sizeof(cx) - 1)))
    throw AfError(AF_ERR_INVALID, kAlignMsg);
}


static af_status exec_sign(af_plan plan, int sign, af_layout layout, const rl* in_re, const rl* in_im,
                           rl* out_re, rl* out_im, int64_t batch, af_stream stream) {
  AF_TRY
  if (!plan) return fail(AF_ERR_INVALID, "null plan");
  if (batch < 0) return fail(AF_ERR_INVALID, "negative batch");
  if (batch == 0 || plan->n == 0) return AF_OK;
  check_io(layout, in_re, in_im, out_re, out_im);
  if (batch >= ((i64)1 << 31) / plan->n) return fail(AF_ERR_UNSUPPORTED, "n * batch must be below 2^31");
  Program& prog = program_for(plan, batch, sign);
  ensure_ws(plan, prog.ws_elems);
  const bool planar = layout == AF_LAYOUT_PLANAR;
  TileBases b = make_bases(in_re, planar ? in_im : nullptr, out_re, planar ? out_im : nullptr, state(plan)->ws,
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


static void check_plan_size(af_plan_s* P, i64 rows) {
  if (P->n * rows >= ((i64)1 << 31)) throw AfError(AF_ERR_UNSUPPORTED, "n * rows must be below 2^31");
}

// in (outer, n, inner) -> out along the middle axis with plan P's sign; an
// im pointer of nullptr means interleaved data
static void run_axis(af_plan_s* P, const rl* in_re, const rl* in_im, rl* out_re, rl* out_im, i64 outer,
                     i64 inner, cudaStream_t st) {
  if (outer == 0 || inner == 0 || P->n == 0) return;
  check_plan_size(P, outer * inner);
  Program& prog = axis_program(P, outer, inner, P->sign);
  run_with(P, prog, in_re, in_im, out_re, out_im, st);
}

// the multi-axis transforms: plans[0] runs along the last axis
static void run_nd(af_plan_s* const* plans, int dims, const rl* in_re, const rl* in_im, rl* out_re,
                   rl* out_im, i64 batch, cudaStream_t st) {
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



namespace AF_NS {
long long state_launches(af_plan_s* P, long long batch) {
  return (long long)program_for(P, batch, P->sign).launches.size();
}
}  // namespace AF_NS

extern "C" {

af_status AFN(af_plan_create)(af_plan* plan, int64_t n, int sign, af_algo algo) {
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
    P->AF_STATE = new AF_NS::PlanState();
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

af_status AFN(af_exec_c2c)(af_plan plan, af_layout layout, const rl* in_re, const rl* in_im, rl* out_re, rl* out_im,
                           int64_t batch, af_stream stream) {
  if (!plan) return fail(AF_ERR_INVALID, "null plan");
  return exec_sign(plan, plan->sign, layout, in_re, in_im, out_re, out_im, batch, stream);
}

af_status AFN(af_vjp_c2c)(af_plan plan, af_layout layout, const rl* cot_re, const rl* cot_im, rl* grad_re,
                          rl* grad_im, int64_t batch, af_stream stream) {
  if (!plan) return fail(AF_ERR_INVALID, "null plan");
  return exec_sign(plan, -plan->sign, layout, cot_re, cot_im, grad_re, grad_im, batch, stream);
}

af_status AFN(af_scale_down)(af_layout layout, rl* re, rl* im, int64_t n, int64_t batch, af_stream stream) {
  AF_TRY
  if (n < 0 || batch < 0) return fail(AF_ERR_INVALID, "negative size");
  if (n == 0 || batch == 0) return AF_OK;
  check_io(layout, re, im, re, im);
  MapDesc md = rows_map(MAP_SCALE, n, batch);
  md.scale = 1.0f / (rl)n;
  const bool planar = layout == AF_LAYOUT_PLANAR;
  TileBases b = make_bases(re, planar ? im : nullptr, re, planar ? im : nullptr, nullptr, nullptr, nullptr);
  check_cuda(launch_map(md, b, (cudaStream_t)stream), "scale_down");
  return AF_OK;
  AF_CATCH
}

af_status AFN(af_cyclic_reverse)(af_layout layout, const rl* in_re, const rl* in_im, rl* out_re, rl* out_im,
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


af_status AFN(af_exec_c2c_axis)(af_plan plan, af_layout layout, const rl* in_re, const rl* in_im, rl* out_re,
                                rl* out_im, int64_t outer, int64_t inner, af_stream stream) {
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

af_status AFN(af_exec_c2c_2d)(af_plan plan0, af_plan plan1, af_layout layout, const rl* in_re, const rl* in_im,
                              rl* out_re, rl* out_im, int64_t batch, af_stream stream) {
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

af_status AFN(af_exec_c2c_3d)(af_plan plan0, af_plan plan1, af_plan plan2, af_layout layout, const rl* in_re,
                              const rl* in_im, rl* out_re, rl* out_im, int64_t batch, af_stream stream) {
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

af_status AFN(af_to_spectrum)(af_plan half, const rl* x, af_spectrum spectrum, af_layout layout, rl* out_re,
                              rl* out_im, int64_t batch, af_stream stream) {
  AF_TRY
  if (!half) return fail(AF_ERR_INVALID, "null plan");
  if (batch < 0) return fail(AF_ERR_INVALID, "negative batch");
  if (spectrum != AF_SPECTRUM_FULL && spectrum != AF_SPECTRUM_HALF) return fail(AF_ERR_INVALID, "bad spectrum");
  const i64 n2 = half->n;
  if (batch == 0 || n2 == 0) return AF_OK;
  if (!x) return fail(AF_ERR_INVALID, "null data pointer");
  if ((uintptr_t)x & (sizeof(cx) - 1)) return fail(AF_ERR_INVALID, "real input must be aligned like a complex element");
  check_io(layout, out_re, out_im, out_re, out_im);
  check_plan_size(half, 2 * batch);
  cudaStream_t st = (cudaStream_t)stream;
  cx* Z = ensure_stage(half, n2 * batch);
  run_with(half, program_for(half, batch, half->sign), x, nullptr, (rl*)Z, nullptr, st);
  TwTable t = state(half)->res.table(2 * n2);
  const i64 nout = spectrum == AF_SPECTRUM_FULL ? 2 * n2 : n2 + 1;
  check_cuda(launch_real_untangle(Z, cptr(layout, out_re, out_im), n2, nout, batch, t.p, t.S_log2, st),
             "toSpectrum untangle");
  return AF_OK;
  AF_CATCH
}

static af_status from_spectrum_impl(af_plan half, af_layout layout, const rl* s_re, const rl* s_im, rl* x,
                                    int64_t batch, af_stream stream, bool vjp) {
  AF_TRY
  if (!half) return fail(AF_ERR_INVALID, "null plan");
  if (batch < 0) return fail(AF_ERR_INVALID, "negative batch");
  const i64 n2 = half->n;
  if (batch == 0 || n2 == 0) return AF_OK;
  if (!x) return fail(AF_ERR_INVALID, "null data pointer");
  if ((uintptr_t)x & (sizeof(cx) - 1)) return fail(AF_ERR_INVALID, "real output must be aligned like a complex element");
  check_io(layout, s_re, s_im, s_re, s_im);
  if (vjp && half->sign != -1) return fail(AF_ERR_INVALID, "the toSpectrum VJP needs a forward half-length plan");
  check_plan_size(half, 2 * batch);
  cudaStream_t st = (cudaStream_t)stream;
  cx* f = ensure_stage(half, n2 * batch);
  TwTable t = state(half)->res.table(2 * n2);
  check_cuda(launch_real_entangle(cptr(layout, s_re, s_im), f, n2, batch, t.p, t.S_log2, vjp ? 1 : 0, st),
             "fromSpectrum entangle");
  const int sign = vjp ? -half->sign : half->sign;
  run_with(half, program_for(half, batch, sign), (const rl*)f, nullptr, x, nullptr, st);
  return AF_OK;
  AF_CATCH
}

af_status AFN(af_from_spectrum)(af_plan half, af_layout layout, const rl* spec_re, const rl* spec_im, rl* x,
                                int64_t batch, af_stream stream) {
  return from_spectrum_impl(half, layout, spec_re, spec_im, x, batch, stream, false);
}

af_status AFN(af_vjp_to_spectrum)(af_plan half, af_layout layout, const rl* cot_re, const rl* cot_im, rl* grad,
                                  int64_t batch, af_stream stream) {
  return from_spectrum_impl(half, layout, cot_re, cot_im, grad, batch, stream, true);
}

af_status AFN(af_untangle_spectra_2d)(af_layout layout, const rl* s_re, const rl* s_im, rl* a_re, rl* a_im, rl* b_re,
                                      rl* b_im, int64_t height, int64_t width, int64_t batch, af_stream stream) {
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

af_status AFN(af_untangle_spectra)(af_layout layout, const rl* s_re, const rl* s_im, rl* a_re, rl* a_im, rl* b_re,
                                   rl* b_im, int64_t n, int64_t batch, af_stream stream) {
  return AFN(af_untangle_spectra_2d)(layout, s_re, s_im, a_re, a_im, b_re, b_im, 1, n, batch, stream);
}

af_status AFN(af_cyclic_reverse_2d)(af_layout layout, const rl* in_re, const rl* in_im, rl* out_re, rl* out_im,
                                    int64_t height, int64_t width, int64_t batch, af_stream stream) {
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

af_status AFN(af_entangle_spectra)(af_layout layout, const rl* c_re, const rl* c_im, const rl* d_re, const rl* d_im,
                                   rl* out_re, rl* out_im, int64_t n, int64_t batch, af_stream stream) {
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

static af_status two_to_impl(af_plan_s* const* plans, int dims, const rl* f, const rl* g, af_layout layout,
                             rl* a_re, rl* a_im, rl* b_re, rl* b_im, int64_t batch, af_stream stream) {
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
  cx* S = ensure_stage(plans[0], img * batch);
  run_nd(plans, dims, f, g, (rl*)S, nullptr, batch, st);
  const i64 h = dims == 2 ? plans[1]->n : 1, w = plans[0]->n;
  CPtr sp{S, nullptr, nullptr};
  check_cuda(launch_untangle(sp, cptr(layout, a_re, a_im), cptr(layout, b_re, b_im), h, w, img * batch, st),
             "untangle");
  return AF_OK;
  AF_CATCH
}

af_status AFN(af_two_to_spectrum)(af_plan plan, const rl* f, const rl* g, af_layout layout, rl* a_re, rl* a_im,
                                  rl* b_re, rl* b_im, int64_t batch, af_stream stream) {
  af_plan_s* plans[1] = {plan};
  return two_to_impl(plans, 1, f, g, layout, a_re, a_im, b_re, b_im, batch, stream);
}

af_status AFN(af_two_to_spectrum_2d)(af_plan plan0, af_plan plan1, const rl* f, const rl* g, af_layout layout,
                                     rl* a_re, rl* a_im, rl* b_re, rl* b_im, int64_t batch, af_stream stream) {
  af_plan_s* plans[2] = {plan0, plan1};
  return two_to_impl(plans, 2, f, g, layout, a_re, a_im, b_re, b_im, batch, stream);
}

static af_status two_from_impl(af_plan_s* const* plans, int dims, af_layout layout, const rl* a_re,
                               const rl* a_im, const rl* b_re, const rl* b_im, rl* f, rl* g,
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
  cx* S = ensure_stage(plans[0], img * batch);
  CPtr sp{S, nullptr, nullptr};
  check_cuda(launch_entangle(cptr(layout, a_re, a_im), cptr(layout, b_re, b_im), sp, img * batch, st), "entangle");
  run_nd(plans, dims, (const rl*)S, nullptr, f, g, batch, st);
  return AF_OK;
  AF_CATCH
}

af_status AFN(af_two_from_spectrum)(af_plan plan, af_layout layout, const rl* a_re, const rl* a_im, const rl* b_re,
                                    const rl* b_im, rl* f, rl* g, int64_t batch, af_stream stream) {
  af_plan_s* plans[1] = {plan};
  return two_from_impl(plans, 1, layout, a_re, a_im, b_re, b_im, f, g, batch, stream);
}

af_status AFN(af_two_from_spectrum_2d)(af_plan plan0, af_plan plan1, af_layout layout, const rl* a_re, const rl* a_im,
                                       const rl* b_re, const rl* b_im, rl* f, rl* g, int64_t batch,
                                       af_stream stream) {
  af_plan_s* plans[2] = {plan0, plan1};
  return two_from_impl(plans, 2, layout, a_re, a_im, b_re, b_im, f, g, batch, stream);
}

af_status AFN(af_convolve_cyclic)(af_plan plan, af_layout layout, const rl* x_re, const rl* x_im, const rl* y_re,
                                  const rl* y_im, rl* out_re, rl* out_im, int64_t batch, af_stream stream) {
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
  cx* S = ensure_stage(plan, 2 * n * batch);
  cx* S2 = S + n * batch;
  Program& G = program_for(plan, batch, +1);
  run_with(plan, G, x_re, planar ? x_im : nullptr, (rl*)S, nullptr, st);
  run_with(plan, G, y_re, planar ? y_im : nullptr, (rl*)S2, nullptr, st);
  check_cuda(launch_conv_mul(S, S2, 1.0f / (rl)n, n * batch, st), "convolution product");
  run_with(plan, program_for(plan, batch, -1), (const rl*)S, nullptr, out_re, planar ? out_im : nullptr, st);
  return AF_OK;
  AF_CATCH
}

}  // extern "C"
