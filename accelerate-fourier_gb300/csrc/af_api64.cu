// af_api64.cu -- Complex Double plans behind the C ABI's *_f64 entry points:
// the reference plan tree (shared planner), lowered by the FP64 build of the
// engine and run by its executor.
#define AF_F64 1
#include "af_host.h"

namespace af64 {

struct Plan {
  long long n = 0;
  int sign = -1;
  af::Planner planner;
  const af::Node* root = nullptr;
  PlanRes res;
  std::map<std::pair<long long, int>, Program> progs;  // (batch, sign)
  std::map<std::tuple<long long, long long, int>, Program> axis_progs;  // (outer, inner, sign)
  cx* ws = nullptr;
  size_t ws_elems = 0;
  ~Plan() {
    if (ws) cudaFree(ws);
    res.release();
  }
};

Plan* plan_create(long long n, int sign, int algo) {
  std::unique_ptr<Plan> p(new Plan);
  p->n = n;
  p->sign = sign;
  p->root = af::plan_root(p->planner, n, algo);
  return p.release();
}

void plan_destroy(Plan* p) { delete p; }

long long plan_n(const Plan* p) { return p->n; }

static Program& program_for(Plan* P, long long batch, int sign) {
  auto key = std::make_pair(batch, sign);
  auto it = P->progs.find(key);
  if (it != P->progs.end()) return it->second;
  Program& prog = P->progs[key];
  build_program(P->res, P->root, (rl)sign, batch, &prog);
  return prog;
}

// Program along the middle axis of an (outer, n, inner) array.
static Program& axis_program(Plan* P, long long outer, long long inner, int sign) {
  if (inner == 1) return program_for(P, outer, sign);
  auto key = std::make_tuple(outer, inner, sign);
  auto it = P->axis_progs.find(key);
  if (it != P->axis_progs.end()) return it->second;
  Program& prog = P->axis_progs[key];
  View in;
  in.buf = BUF_IN;
  in.s_e = inner;
  in.s_lo = 1;
  in.lo_cnt = inner;
  in.s_hi = P->n * inner;
  View out = in;
  out.buf = BUF_OUT;
  build_program_view(P->res, P->root, (rl)sign, outer * inner, in, out, &prog);
  return prog;
}

static void run(Plan* P, Program& prog, const double* in_re, const double* in_im, double* out_re, double* out_im,
                cudaStream_t st) {
  if ((size_t)prog.ws_elems > P->ws_elems) {
    if (P->ws) { cudaFree(P->ws); P->ws = nullptr; P->ws_elems = 0; }
    if (cudaMalloc(&P->ws, sizeof(cx) * (size_t)prog.ws_elems) != cudaSuccess)
      throw af::AfError(AF_ERR_ALLOC, "workspace allocation failed");
    P->ws_elems = (size_t)prog.ws_elems;
  }
  TileBases b = make_bases(in_re, in_im, out_re, out_im, P->ws, nullptr, nullptr);
  const cudaError_t e = run_program(prog, b, nullptr, st);
  if (e != cudaSuccess) throw af::AfError(AF_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
}

void plan_exec(Plan* P, int sign, const double* in_re, const double* in_im, double* out_re, double* out_im,
               long long batch, cudaStream_t st) {
  run(P, program_for(P, batch, sign), in_re, in_im, out_re, out_im, st);
}

void plan_exec_axis(Plan* P, const double* in_re, const double* in_im, double* out_re, double* out_im,
                    long long outer, long long inner, cudaStream_t st) {
  run(P, axis_program(P, outer, inner, P->sign), in_re, in_im, out_re, out_im, st);
}

long long plan_launches(Plan* P, long long batch) { return program_for(P, batch, P->sign).tile_launches(); }

}  // namespace af64
