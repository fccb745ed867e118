// af_host.h -- host-side structures of libaf: plan resources, launch
// programs, tile builders, and the objects behind the C ABI's handles.
#pragma once
#include <map>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

#include "af.h"
#include "af_internal.h"
#include "af_plan.h"

// Shared by both precisions of the engine.
namespace af {

struct AfError : std::runtime_error {
  af_status code;
  AfError(af_status c, const std::string& m) : std::runtime_error(m), code(c) {}
};
void set_last_error(const std::string& m);
const Node* plan_root(Planner& pl, i64 n, int algo);

}  // namespace af

namespace AF_NS {

// A batch of lines: line l = hi * lo_cnt + lo, element e at
// off + hi*s_hi + lo*s_lo + e*s_e in buffer `buf` (complex units).
struct View {
  int buf = BUF_WS;
  i64 off = 0;
  i64 s_e = 1, s_lo = 0, s_hi = 0, lo_cnt = 1;
  static View rows(int buf, i64 off, i64 n, i64 lines) {
    View v;
    v.buf = buf;
    v.off = off;
    v.s_e = 1;
    v.s_lo = n;
    v.s_hi = 0;
    v.lo_cnt = lines < 1 ? 1 : lines;
    return v;
  }
};

enum LaunchType { L_TILE = 0, L_MAP = 1 };

struct Launch {
  int type = L_TILE;
  std::vector<TileDesc> descs;
  std::vector<WorkItem> items;
  int threads = 128;
  int smem_data = 0;
  int tw_max = 0;
  int g_max = 0;
  MapDesc md;
  size_t desc_off = 0, item_off = 0;  // byte offsets in the program's device blob
  // Concurrent execution (batched programs): the launch runs on side stream
  // `stream` (0 = the caller's) after the launches listed in `deps`
  // (indices into the program); launches on one stream run in program order.
  int stream = 0;
  int generic = 1;  // tile launch needs the general kernel (not only PLAIN tiles with AFFINE views)
  std::vector<int> deps;
  bool signal = false;  // a launch on another stream depends on this one
};

struct Program {
  std::vector<Launch> launches;
  i64 ws_elems = 0;
  int nstreams = 1;                // streams the launches use (1: sequential)
  std::vector<cudaStream_t> side;  // streams 1 .. nstreams-1
  std::vector<cudaEvent_t> ev;     // per launch (signalling launches), then fork and joins
  char* dblob = nullptr;  // device copy of every launch's descriptors and items
  int tile_launches() const;
};

struct TwTable {
  cx* p = nullptr;
  int S_log2 = 0, H = 0, len = 0;
};

struct RaderRes {
  i64 p = 0, g = 0;
  int* dlog = nullptr;   // dlog[r-1] = log_g r
  int* src = nullptr;    // src[q] = 1 + perm[(-q) mod (p-1)] = g^-q mod p
  int* inv = nullptr;    // inverse permutation
  int* gpow = nullptr;   // gpow[q] = g^q mod p (scatter target of conv index q)
  cx* zs = nullptr;  // kernel spectrum / M (M entries)
  i64 M = 0;             // conv transform length (rader_conv_len)
};
i64 rader_conv_len(i64 p);

struct ChirpRes {
  i64 len = 0, pad = 0;
  cx* chirp = nullptr;  // len entries
  cx* spec = nullptr;   // pad entries
};

struct PlanRes {
  bool dry = false;                       // address-checking mode (no device)
  bool no_alloc = false;                  // any device allocation is an error
  cx* arena = nullptr;                // when set, twiddle tables come from this
  size_t arena_cap = 0, arena_used = 0;   // preallocated device area (no allocation)
  char* blob = nullptr;                   // when set, programs upload here
  size_t blob_cap = 0;
  cudaStream_t stream = 0;                // stream for table generation and uploads
  unsigned long long fake_next = 1ull << 40;
  std::map<const void*, std::vector<int>> host_tabs;  // host copies of index tables
  std::map<const void*, std::vector<i64>> host_loffs; // host copies of gathered-line tables
  std::vector<void*> allocs;
  std::map<i64, TwTable> tables;
  std::map<std::pair<i64, i64>, const cx*> pair_tables;
  std::map<std::pair<i64, int>, RaderRes> rader;
  std::map<std::tuple<i64, i64, int>, ChirpRes> chirps;
  std::vector<cudaStream_t> streams;  // owned side streams of programs
  std::vector<cudaEvent_t> events;
  void* dalloc(size_t bytes);
  TwTable table(i64 n);
  const cx* pair_table(i64 a, i64 b, int* off_b);
  const RaderRes& rader_res(i64 p, int sign);
  const ChirpRes& chirp_res(i64 len, i64 pad, int sign);
  const i64* line_table(const std::vector<i64>& offs);  // device copy of line offsets
  void release();
};

bool tile_ok(i64 n);
void finalize_program(PlanRes& res, Program& prog);
cudaError_t run_program(const Program& prog, const TileBases& bases, double* loss, cudaStream_t st);
TileBases make_bases(const rl* in_re, const rl* in_im, rl* out_re, rl* out_im, cx* ws,
                     const rl* aux_re, const rl* aux_im);

// Builds the launch program of one plan tree over `batch` contiguous rows.
void build_program(PlanRes& res, const Node* root, rl sign, i64 batch, Program* prog);
// The same over `lines` lines addressed through two-level views (strided axes).
void build_program_view(PlanRes& res, const Node* root, rl sign, i64 lines, const View& in, const View& out,
                        Program* prog);

// Batched executor: many transforms of mixed lengths, concatenated.
struct BatchPlan;
BatchPlan* batch_create(const i64* ns, i64 count, int sign);
BatchPlan* batch_create_mode(const i64* ns, i64 count, int sign, bool dry);
void batch_destroy(BatchPlan* b);
const void* batch_res(BatchPlan* B);

}  // namespace af

// Per-precision state of a plan (defined below for this build's precision;
// both precisions' functions are visible to the shared C ABI code).
struct af_plan_s;
namespace af {
struct PlanState;
void state_destroy(PlanState* s);
long long state_launches(af_plan_s* P, long long batch);
}  // namespace af
namespace af64 {
struct PlanState;
void state_destroy(PlanState* s);
long long state_launches(af_plan_s* P, long long batch);
}  // namespace af64

namespace AF_NS {
// Tables, programs and buffers of a plan in one precision.
struct PlanState {
  PlanRes res;
  std::map<std::pair<long long, int>, Program> progs;                        // (batch, sign)
  std::map<std::tuple<long long, long long, int>, Program> axis_progs;  // (outer, inner, sign)
  cx* ws = nullptr;
  size_t ws_elems = 0;
  cx* stage = nullptr;  // staging for the real transforms and convolutions
  size_t stage_elems = 0;
  ~PlanState();
};
}  // namespace AF_NS

// The object behind an af_plan: the reference plan tree, and the state of the
// precision it was created for (af_plan_create: s32, af_plan_create_f64: s64).
struct af_plan_s {
  long long n = 0;
  int sign = -1;
  int algo = 0;
  af::Planner planner;
  const af::Node* root = nullptr;
  af::PlanState* s32 = nullptr;
  af64::PlanState* s64 = nullptr;
  ~af_plan_s();
};
