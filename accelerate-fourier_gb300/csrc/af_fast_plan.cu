// af_fast_plan.cu -- planner of the batched executor: shapes, work items,
// root tables and launches for a list of transform lengths, and the internal
// afx_fast_* entry points the tests use (device runs and host emulation).
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <cstring>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "af_fast_host.h"
#include "af.h"
#include "af_plan.h"

namespace af {

static int trailing_zeros(i64 n) {
  int z = 0;
  while (n > 0 && (n & 1) == 0) {
    n >>= 1;
    ++z;
  }
  return z;
}
static i64 even_up(i64 v) { return (v + 1) & ~(i64)1; }

// Planner choices the autotuner varies.
struct FastTune {
  int radix16 = 1;          // radix-16 passes where the length allows (else radix 8)
  int gl_max = 32;          // most lines in one multi-pass item
  int balance_v = 0;        // per-pass choice of lines per unit (else two whenever possible)
  int target = 4096;        // elements one item aims at
  int slack = 2736;         // items queued between dependent stages (six times the resident CTAs)
  int l2_mb = 48;           // workspace in flight, MB (kept well inside the 126 MB L2)
  int fixed = 1;            // compile-time line FFTs for the listed (L, GL) pairs
};

// The compile-time line lengths, and their pairwise products a b (a >= b)
// in increasing order.
static const std::vector<int>& fixed_lengths() {
  static const std::vector<int> v = [] {
    std::vector<int> r;
#define AFF_FIXED_LEN(l, g, r1, r2) r.push_back(l);
    AFF_FIXED_LINES(AFF_FIXED_LEN)
#undef AFF_FIXED_LEN
    return r;
  }();
  return v;
}
struct FixedProduct {
  i64 M;
  int a, b;
};
static const std::vector<FixedProduct>& fixed_products() {
  static const std::vector<FixedProduct> v = [] {
    std::vector<FixedProduct> r;
    const std::vector<int>& L = fixed_lengths();
    for (int a : L)
      for (int b : L)
        if (a >= b) r.push_back(FixedProduct{(i64)a * b, a, b});
    std::sort(r.begin(), r.end(), [](const FixedProduct& x, const FixedProduct& y) {
      return x.M != y.M ? x.M < y.M : (x.a - x.b) < (y.a - y.b);
    });
    return r;
  }();
  return v;
}
// the least product of two compiled lengths >= need (M = 0 when none)
static FixedProduct least_fixed_product(i64 need) {
  for (const FixedProduct& f : fixed_products())
    if (f.M >= need) return f;
  return FixedProduct{0, 0, 0};
}
// a split n = a b into compiled lengths, a >= b, the most balanced (M = 0 when none)
static FixedProduct fixed_split(i64 n) {
  FixedProduct best{0, 0, 0};
  for (int b : fixed_lengths())
    if (n % b == 0) {
      const i64 a = n / b;
      if (a < b) continue;
      for (int l : fixed_lengths())
        if (l == a && (!best.M || a - b < best.a - best.b)) best = FixedProduct{n, (int)a, b};
    }
  return best;
}

static bool is_fixed_line(int L, int GL) {
#define AFF_FIXED_TEST(l, g, r1, r2) if (L == l && GL == g) return true;
  AFF_FIXED_LINES(AFF_FIXED_TEST)
#undef AFF_FIXED_TEST
  return false;
}

// Radices of a 5-smooth line length: the two listed radices of a compile-time
// line (fixed), else 16s or 8s first (the first pass has no twiddles), then
// 5, 4, 3, 2.
static std::vector<int> line_radices(int L, bool r16, bool fixed = false) {
  std::vector<int> r;
  if (fixed) {
    const CRadices c = c_radices(L, true);
    return std::vector<int>(c.r, c.r + c.n);
  }
  int m = L;
  if (r16)
    while (m % 16 == 0) { r.push_back(16); m /= 16; }
  while (m % 8 == 0) { r.push_back(8); m /= 8; }
  while (m % 5 == 0) { r.push_back(5); m /= 5; }
  if (m % 4 == 0) { r.push_back(4); m /= 4; }
  while (m % 3 == 0) { r.push_back(3); m /= 3; }
  while (m % 2 == 0) { r.push_back(2); m /= 2; }
  if (m != 1) throw FastError("line length " + std::to_string(L) + " is not 5-smooth");
  return r;
}

// Fills the line FFT of length L; returns the twiddle entries it needs and
// appends their table segments (offsets relative to the shape's table).
static void make_line(FLine& ln, int L, std::vector<RootSeg>* segs, i64 base, bool r16, bool fixed = false) {
  memset(&ln, 0, sizeof ln);
  ln.L = L;
  const std::vector<int> rs = line_radices(L, r16, fixed);
  if ((int)rs.size() > AFF_MAXPASS) throw FastError("too many passes");
  int p = 1, tw = 0;
  ln.npass = (int)rs.size();
  for (size_t j = 0; j < rs.size(); ++j) {
    FPass& ps = ln.pass[j];
    ps.R = rs[j];
    ps.p = p;
    ps.nb = L / rs[j];
    ps.pdiv = make_fastdiv((unsigned)p);
    ps.plog = (p & (p - 1)) == 0 ? __builtin_ctz((unsigned)p) : -1;
    ps.tw = tw;
    if (p > 1) {
      RootSeg s;
      s.off = base + tw;
      s.count = (i64)p * (ps.R - 1);
      s.kind = RS_STOCK;
      s.a = p;
      s.b = ps.R;
      segs->push_back(s);
      tw += (int)even_up((i64)p * (ps.R - 1));
    }
    p *= rs[j];
  }
  ln.twn = tw;
}


// A Bluestein spectrum to generate: transform length n, convolution length M.
struct SpecJob {
  i64 n, M, off;
};

struct FastBatch {
  bool emu = false;
  std::vector<i64> ns, offs;
  i64 total = 0;
  i64 ws_elems = 0;
  std::vector<FShape> shapes;
  std::vector<i64> shape_tw, shape_ftw;  // table offsets of each shape
  std::vector<FXform> xf;
  // table offsets of each transform's ct / wt / spec (-1: none)
  std::vector<i64> xf_ct, xf_wt, xf_spec;
  std::vector<RootSeg> segs;
  std::vector<SpecJob> specs;
  i64 tab_elems = 0;
  std::map<i64, i64> tl3_of;         // N -> offset of the three-level table of W_N
  std::map<i64, i64> spec_of;        // n -> offset of its Bluestein spectrum
  std::map<std::pair<int, int>, int> line_shapes;  // (L, GL) -> shape
  std::vector<FItem> queue;  // the persistent launch's items, in order
  int nctrs = FC_FIRST;
  size_t smem = 0;
  unsigned* dctrs = nullptr;
  int grid = 0;
  long long spin_limit = 1ll << 20; // polls before a wait gives up (under a second)
  int last_status = 0;
  // device (or host, emulation) copies
  std::vector<cx> htab;
  cx* dtab = nullptr;
  cx* dws = nullptr;
  FShape* dshapes = nullptr;
  FXform* dxf = nullptr;
  FItem* ditems = nullptr;
  std::vector<FShape> hshapes;
  std::vector<FXform> hxf;
  std::vector<FItem> hitems;
  std::vector<cx> hws;
  FastTune tune;
  ~FastBatch() {
    if (dtab) cudaFree(dtab);
    if (dws) cudaFree(dws);
    if (dshapes) cudaFree(dshapes);
    if (dxf) cudaFree(dxf);
    if (ditems) cudaFree(ditems);
    if (dctrs) cudaFree(dctrs);
  }
};

// Every CTA of the persistent launch has 256 threads and the same shared
// memory: three fit one SM (228 KB, less 1 KB reserved and the kernel's
// 2.5 KB of staged descriptors and mbarrier per CTA).  The listed line counts
// of the compile-time lines (AFF_FIXED_LINES) are those that fit this size.
static const int kThreads = 256;
static const int kCtaSmem = 74240;
static const int kMaxSmem = kCtaSmem;

static size_t shape_smem(const FShape& s) {
  return sizeof(cx) * (size_t)(2 * s.cap + s.line.twn + s.ftwn + (s.aux ? 2 * AFF_TL3 : 0) + 16);
}

// The three-level root table of W_N (t < 2^18): W_N^j, W_N^(64 j), W_N^(4096 j), j < 64.
static i64 table_tl3(FastBatch* B, i64 N) {
  if (N > ((i64)1 << 18)) throw FastError("three-level root tables cover lengths up to 2^18");
  auto it = B->tl3_of.find(N);
  if (it != B->tl3_of.end()) return it->second;
  const i64 off = B->tab_elems;
  B->segs.push_back(RootSeg{off, 64, RS_LINEAR, N, 1});
  B->segs.push_back(RootSeg{off + 64, 64, RS_LINEAR, N, 64});
  B->segs.push_back(RootSeg{off + 128, 64, RS_LINEAR, N, 4096});
  B->tab_elems += AFF_TL3;
  B->tl3_of[N] = off;
  return off;
}

// Lines per unit of each pass: two lines share the twiddle loads and move as
// 16-byte vectors, but one line per unit wins when it spreads the units
// over the threads in fewer rounds.
static void choose_vectors(FShape& s, bool balance) {
  for (int j = 0; j < s.line.npass; ++j) {
    FPass& ps = s.line.pass[j];
    const i64 u1 = (i64)ps.nb * s.GL;
    const i64 r1 = (u1 + kThreads - 1) / kThreads;
    const i64 r2 = (u1 / 2 + kThreads - 1) / kThreads;
    // a two-line unit costs about 1.7 one-line units
    ps.V = (s.GL % 2 == 0 && ps.R <= 8 && (!balance || 2 * r2 * 17 <= r1 * 20)) ? 2 : 1;
  }
}

static void finish_shape(FShape& s, const FastTune& t) {
  choose_vectors(s, t.balance_v != 0);
  // the compile-time passes are those of radix-16 lines with paired units
  s.fixed = t.fixed && t.radix16 && !t.balance_v && s.kind < 0 && is_fixed_line(s.line.L, s.GL);
  s.LS = line_stride(s.line.L);
  s.cap = (int)even_up(std::max<i64>((i64)s.GL * s.line.L, (i64)s.GL * s.LS));
  s.aux = s.kind < 0 ? 1 : 0;
  s.ndiv = make_fastdiv((unsigned)s.n);
  s.L1div = make_fastdiv((unsigned)s.line.L);
  s.GLr = (int)((1u << 19) + (unsigned)s.GL - 1) / s.GL;
  s.smem = (int)shape_smem(s);
  if (s.smem > kMaxSmem) throw FastError("shape of length " + std::to_string(s.n) + " needs too much shared memory");
}

// Full-FFT shape (FK_DIRECT or FK_BLUE) of length n, Q transforms per CTA.
static int full_shape(FastBatch* B, int kind, i64 n, int Q) {
  FShape s;
  memset(&s, 0, sizeof s);
  s.kind = kind;
  s.n = (int)n;
  s.G = 1 << std::min(trailing_zeros(n), 3);
  const int L1 = (int)(n / s.G);
  const i64 tw_base = B->tab_elems;
  make_line(s.line, L1, &B->segs, tw_base, B->tune.radix16 != 0);
  B->tab_elems += s.line.twn;
  // the final radix-G pass needs W_n^k1 (none when G = 1)
  s.ftwn = s.G > 1 ? (int)even_up(L1) : 0;
  const i64 ftw_base = B->tab_elems;
  if (s.ftwn) {
    RootSeg f{ftw_base, L1, RS_LINEAR, n, 1};
    B->segs.push_back(f);
  }
  B->tab_elems += s.ftwn;
  s.Q = Q;
  s.GL = Q * s.G;
  finish_shape(s, B->tune);
  B->shapes.push_back(s);
  B->shape_tw.push_back(tw_base);
  B->shape_ftw.push_back(ftw_base);
  return (int)B->shapes.size() - 1;
}

// Line shape of the multi-pass schemes: FFT of length L over GL lines.
static int line_shape(FastBatch* B, int L) {
  auto fits = [&](int GL) {
    return (i64)sizeof(cx) * (2 * even_up((i64)GL * (L | 1)) + 2 * L + 2 * AFF_TL3 + 16) <= kMaxSmem;
  };
  // As many lines as fill the item target within the shared memory of a CTA
  // (two buffers of GL line-major rows): at most 64 on a compile-time line
  // (the listed pairs are these counts under the default tuning), at most
  // gl_max and 64 on the others (the item code divides by the line count
  // with a reciprocal that is exact up to 64).
  // (a tile of L GL elements moves as one bulk copy, whose size must be a
  // multiple of 16 bytes: an odd L takes an even count)
  auto fill = [&](int cap) {
    int g = (int)std::min<i64>(cap, std::max<i64>(2, B->tune.target / L));
    while (g > 2 && (!fits(g) || (L & g & 1))) --g;
    return g;
  };
  const int GLf = fill(64);
  const bool fixed_ok = B->tune.fixed && B->tune.radix16 && !B->tune.balance_v && is_fixed_line(L, GLf);
  const int GL = fixed_ok ? GLf : fill(std::min(B->tune.gl_max, 64));
  if (((i64)L * GL) % 2 != 0) throw FastError("a tile of an odd number of elements cannot move as one bulk copy");
  auto key = std::make_pair(L, GL);
  auto it = B->line_shapes.find(key);
  if (it != B->line_shapes.end()) return it->second;
  FShape s;
  memset(&s, 0, sizeof s);
  s.kind = -1;
  s.n = L;
  s.G = 1;
  s.Q = 1;
  s.GL = GL;
  const i64 tw_base = B->tab_elems;
  // a compile-time line takes its two listed radices (finish_shape marks it)
  const bool fixed = B->tune.fixed && B->tune.radix16 && !B->tune.balance_v && is_fixed_line(L, GL);
  make_line(s.line, L, &B->segs, tw_base, B->tune.radix16 != 0, fixed);
  B->tab_elems += s.line.twn;
  finish_shape(s, B->tune);
  B->shapes.push_back(s);
  B->shape_tw.push_back(tw_base);
  B->shape_ftw.push_back(tw_base);
  const int si = (int)B->shapes.size() - 1;
  B->line_shapes[key] = si;
  return si;
}

// The 5-smooth divisor of n nearest sqrt(n) from below (the column length
// of a four-step split); 0 when n has no split with both factors <= 1024.
static i64 four_step_n1(i64 n) {
  i64 best = 0;
  for (i64 d = 2; d * d <= n; ++d)
    if (n % d == 0 && is_5smooth(d) && n / d <= 1024) best = d;
  return best;
}

// shared memory a full-FFT shape of length n with Q transforms per CTA needs
static i64 full_smem(i64 n, int Q, bool r16) {
  const int G = 1 << std::min(trailing_zeros(n), 3);
  const i64 L1 = n / G;
  i64 twn = 0, p = 1;
  for (int r : line_radices((int)L1, r16)) {
    if (p > 1) twn += even_up(p * (r - 1));
    p *= r;
  }
  const i64 cap = even_up(std::max<i64>((i64)Q * n, (i64)Q * G * line_stride((int)L1)));
  return (i64)sizeof(cx) * (2 * cap + twn + (G > 1 ? even_up(L1) : 0) + 16);
}

// Bluestein convolution length: the least 5-smooth multiple of 8 >= 2n - 1.
static i64 blue_len(i64 n) { return 8 * ceiling_5smooth((2 * n - 1 + 7) / 8); }

static FXform blank_xf(i64 off, i64 n) {
  FXform x;
  memset(&x, 0, sizeof x);
  x.off = off;
  x.n = (int)n;
  x.M = (int)n;
  return x;
}

static void push_xf(FastBatch* B, const FXform& x, i64 ct, i64 wt, i64 spec) {
  B->xf.push_back(x);
  B->xf_ct.push_back(ct);
  B->xf_wt.push_back(wt);
  B->xf_spec.push_back(spec);
}

static i64 spectrum(FastBatch* B, i64 n, i64 M) {
  auto it = B->spec_of.find(n);
  if (it != B->spec_of.end()) return it->second;
  const i64 off = B->tab_elems;
  B->specs.push_back(SpecJob{n, M, off});
  B->tab_elems += even_up(M / 2 + 1);  // the spectrum is even: entries 0..M/2
  B->spec_of[n] = off;
  return off;
}

// A multi-pass transform's stages (items of stage s wait for every item of
// stage s-1) and the workspace it keeps in flight.
struct MultiT {
  std::vector<std::vector<FItem>> stages;
  i64 ws = 0;
};

// The queue: later stages of a started transform once `slack` items have
// been queued since its previous stage (by then that stage has most likely
// finished), new transforms while their workspace in flight stays within the
// L2 budget, single-CTA items to fill the gaps.  Every wait is on items
// earlier in the queue.
static void order_queue(FastBatch* B, std::vector<MultiT>& multi, std::vector<FItem>& singles, int slack,
                        i64 budget) {
  std::stable_sort(multi.begin(), multi.end(), [](const MultiT& a, const MultiT& b) { return a.ws > b.ws; });
  std::stable_sort(singles.begin(), singles.end(), [&](const FItem& a, const FItem& b) {
    return (i64)B->shapes[a.shape].cap > (i64)B->shapes[b.shape].cap;
  });
  struct Pend {
    size_t eligible;
    size_t t;
    size_t stage;
  };
  std::vector<Pend> pend;  // FIFO by eligibility (positions only grow)
  size_t ph = 0;
  std::vector<FItem>& q = B->queue;
  size_t next_t = 0, next_s = 0;
  i64 inflight = 0;
  int nctr = FC_FIRST;
  std::vector<int> stage_ctr;  // counter of the stage being emitted
  auto emit_stage = [&](size_t t, size_t st) {
    MultiT& m = multi[t];
    const bool last = st + 1 == m.stages.size();
    const int done = last ? -1 : nctr++;
    const int wait = st == 0 ? -1 : m.stages[st - 1].front().done_ctr;
    const int wcnt = st == 0 ? 0 : (int)m.stages[st - 1].size();
    for (FItem& it : m.stages[st]) {
      it.done_ctr = done;
      it.wait_ctr = wait;
      it.wait_cnt = wcnt;
      q.push_back(it);
    }
    if (last) inflight -= m.ws;
    else pend.push_back(Pend{q.size() + (size_t)slack, t, st + 1});
  };
  for (;;) {
    if (ph < pend.size() && pend[ph].eligible <= q.size()) {
      const Pend p = pend[ph++];
      emit_stage(p.t, p.stage);
    } else if (next_t < multi.size() && inflight + multi[next_t].ws <= budget) {
      inflight += multi[next_t].ws;
      emit_stage(next_t++, 0);
    } else if (next_s < singles.size()) {
      q.push_back(singles[next_s++]);
    } else if (ph < pend.size()) {
      const Pend p = pend[ph++];
      emit_stage(p.t, p.stage);
    } else if (next_t < multi.size()) {
      inflight += multi[next_t].ws;
      emit_stage(next_t++, 0);
    } else {
      break;
    }
  }
  B->nctrs = nctr;
}

static void plan_batch(FastBatch* B) {
  const bool r16 = B->tune.radix16 != 0;
  std::map<i64, std::vector<int>> direct_by_n, blue_by_M;
  struct Split {
    int t;
    i64 N, n1, n2;
  };
  std::vector<Split> four, blue3;
  for (size_t i = 0; i < B->ns.size(); ++i) {
    const i64 n = B->ns[i];
    if (n == 0) continue;
    if (is_5smooth(n)) {
      if (full_smem(n, 1, r16) <= kMaxSmem) {
        direct_by_n[n].push_back((int)i);
      } else {  // four-step: a split into compiled line lengths when there is one
        const FixedProduct f = B->tune.fixed ? fixed_split(n) : FixedProduct{0, 0, 0};
        const i64 d = f.M ? f.b : four_step_n1(n);
        if (!d) throw FastError("length " + std::to_string(n) + " is too long for the batched executor");
        four.push_back(Split{(int)i, n, d, n / d});
      }
    } else {
      const i64 M = blue_len(n);
      if (full_smem(M, 1, r16) <= kMaxSmem) {
        blue_by_M[M].push_back((int)i);
        continue;
      }
      // multi-pass Bluestein: the least product of two compiled line lengths
      // >= 2n - 1, the longer on the column passes (one FFT each), the
      // shorter on the row pass (two FFTs)
      const FixedProduct f = B->tune.fixed ? least_fixed_product(2 * n - 1) : FixedProduct{0, 0, 0};
      if (f.M) {
        blue3.push_back(Split{(int)i, f.M, f.a, f.b});
      } else {
        const i64 d = four_step_n1(M);
        if (!d) throw FastError("length " + std::to_string(n) + " is too long for the batched executor");
        blue3.push_back(Split{(int)i, M, d, M / d});
      }
    }
  }
  std::vector<FItem> singles;
  auto group_items = [&](int kind, i64 len, const std::vector<int>& idx) {
    int Q = 1;
    while ((i64)Q * 2 * len <= B->tune.target && Q * 2 <= (int)idx.size() && Q * 2 <= AFF_MAXQ &&
           full_smem(len, Q * 2, r16) <= kMaxSmem)
      Q *= 2;
    const int si = full_shape(B, kind, len, Q);
    for (size_t j = 0; j < idx.size(); j += Q) {
      FItem it{};
      memset(&it, 0, sizeof it);
      it.kind = kind;
      it.shape = si;
      it.first = (int)B->xf.size();
      it.count = (int)std::min<size_t>(Q, idx.size() - j);
      it.wait_ctr = it.done_ctr = -1;
      for (int q = 0; q < it.count; ++q) {
        const int t = idx[j + q];
        const i64 n = B->ns[t];
        FXform x = blank_xf(B->offs[t], n);
        i64 ct = -1, spec = -1;
        if (kind == FK_BLUE) {
          x.M = (int)len;
          x.n2x = (unsigned)(2 * n);
          x.r2n = 1.0f / (float)(2 * n);
          ct = table_tl3(B, 2 * n);
          spec = spectrum(B, n, len);
        }
        push_xf(B, x, ct, -1, spec);
      }
      singles.push_back(it);
    }
  };
  for (auto& kv : direct_by_n) group_items(FK_DIRECT, kv.first, kv.second);
  for (auto& kv : blue_by_M) group_items(FK_BLUE, kv.first, kv.second);
  // multi-pass transforms: each owns a workspace region
  std::vector<MultiT> multi;
  auto passes = [&](const Split& sp, bool blue) {
    const int t = sp.t;
    const i64 n = B->ns[t];
    const i64 N = sp.N, n1 = sp.n1, n2 = sp.n2;  // length of the FFTs and its split
    const int s1 = line_shape(B, (int)n1), s2 = line_shape(B, (int)n2);
    const int C1 = B->shapes[s1].GL, C2 = B->shapes[s2].GL;
    FXform x = blank_xf(B->offs[t], n);
    x.n1 = (int)n1;
    x.n2 = (int)n2;
    x.M = (int)N;
    // Workspace regions in blocks, one per consumer item, each laid out as
    // that item's shared-memory tile and starting on a 128-byte line:
    // region 1 (stage A -> stage B): block k1 / C2 holds (j2, k1) at
    // j2 C2 + k1 mod C2; region 2 (Bluestein stage B -> A'): block j2 / C1
    // holds (k1, j2) at k1 C1 + j2 mod C1.
    auto up16 = [](i64 v) { return (v + 15) & ~(i64)15; };
    x.gb = C2;
    x.gbr = (int)((1u << 19) + (unsigned)C2 - 1) / C2;
    x.s1 = (int)up16(n2 * C2);
    x.ga = C1;
    x.gar = (int)((1u << 19) + (unsigned)C1 - 1) / C1;
    x.s2 = blue ? (int)up16(n1 * C1) : 0;
    const i64 r1 = (n1 + C2 - 1) / C2 * x.s1;
    const i64 r2 = blue ? (n2 + C1 - 1) / C1 * x.s2 : 0;
    x.ws = B->ws_elems;
    x.ws2 = x.ws + r1;
    const i64 wsn = r1 + r2;
    B->ws_elems += wsn;
    i64 ct = -1, spec = -1;
    const i64 wt = table_tl3(B, N);
    if (blue) {
      x.n2x = (unsigned)(2 * n);
      x.r2n = 1.0f / (float)(2 * n);
      ct = table_tl3(B, 2 * n);
      spec = spectrum(B, n, N);
    }
    const int xi = (int)B->xf.size();
    push_xf(B, x, ct, wt, spec);
    MultiT mt;
    mt.ws = wsn;
    auto items = [&](int kind, int si, int C, i64 count) {
      std::vector<FItem> v;
      for (i64 c0 = 0; c0 < count; c0 += C) {
        FItem it{};
        memset(&it, 0, sizeof it);
        it.kind = kind;
        it.shape = si;
        it.first = xi;
        it.count = 1;
        it.c0 = (int)c0;
        it.cn = (int)std::min<i64>(C, count - c0);
        it.wait_ctr = it.done_ctr = -1;
        v.push_back(it);
      }
      mt.stages.push_back(v);
    };
    if (!blue) {
      items(FK_COLS, s1, C1, n2);  // columns j2 < n2, FFT over n1
      items(FK_ROWS, s2, C2, n1);  // lines k1 < n1, FFT over n2
    } else {
      items(FK_BCOLS, s1, C1, n2);
      items(FK_BROWS, s2, C2, n1);
      items(FK_BCOLS2, s1, C1, n2);
    }
    multi.push_back(std::move(mt));
  };
  for (const Split& sp : four) passes(sp, false);
  for (const Split& sp : blue3) passes(sp, true);
  B->smem = kCtaSmem;
  order_queue(B, multi, singles, B->tune.slack, (i64)B->tune.l2_mb << 17);
}

// ------------------------------------------------------------ spectra
// v[m] = conj(a_m) = W_{2n}^(-m^2) at m and M - m for 0 <= m < n, 0 elsewhere;
// spec = FFT(v) / M (forward sign), rounded to float.
AF_HD double2 conj_chirp64(i64 n, i64 m) {
  const i64 r = (m * m) % (2 * n);
  double s, c;
#ifdef __CUDA_ARCH__
  sincospi((double)r / (double)n, &s, &c);
#else
  const double a = M_PI * ((double)r / (double)n);
  s = std::sin(a);
  c = std::cos(a);
#endif
  return make_double2(c, s);
}

__global__ void chirp_vec_kernel(double2* v, i64 n, i64 M, i64 count) {
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < count * M; i += (i64)gridDim.x * blockDim.x) {
    const i64 m = i % M;
    double2 z = make_double2(0.0, 0.0);
    if (m < n) z = conj_chirp64(n, m);
    else if (M - m < n) z = conj_chirp64(n, M - m);
    v[i] = z;
  }
}

// entries 0..M/2 of the spectrum (the rest mirror them), scaled by 1/M and rounded
__global__ void spec_round_kernel(const double2* V, cx* out, i64 M) {
  const double s = 1.0 / (double)M;
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i <= M / 2; i += (i64)gridDim.x * blockDim.x)
    out[i] = make_cx((float)(V[i].x * s), (float)(V[i].y * s));
}

// host FP64 DFT of a 5-smooth length (emulation only: the device path uses
// the FP64 engine)
static void host_fft64(std::vector<double2>& a, int sign) {
  const size_t n = a.size();
  if (n <= 1) return;
  size_t r = n % 2 == 0 ? 2 : (n % 3 == 0 ? 3 : 5);
  const size_t m = n / r;
  std::vector<std::vector<double2>> sub(r, std::vector<double2>(m));
  for (size_t j = 0; j < m; ++j)
    for (size_t q = 0; q < r; ++q) sub[q][j] = a[j * r + q];
  for (size_t q = 0; q < r; ++q) host_fft64(sub[q], sign);
  for (size_t k = 0; k < n; ++k) {
    double re = 0, im = 0;
    for (size_t q = 0; q < r; ++q) {
      const double ang = sign * 2.0 * M_PI * (double)((q * k) % n) / (double)n;
      const double2 v = sub[q][k % m];
      re += v.x * std::cos(ang) - v.y * std::sin(ang);
      im += v.x * std::sin(ang) + v.y * std::cos(ang);
    }
    a[k] = make_double2(re, im);
  }
}

static void gen_spectra(FastBatch* B, cudaStream_t st) {
  if (B->specs.empty()) return;
  if (B->emu) {
    for (const SpecJob& j : B->specs) {
      std::vector<double2> v(j.M, make_double2(0, 0));
      for (i64 m = 0; m < j.n; ++m) {
        v[m] = conj_chirp64(j.n, m);
        if (m) v[j.M - m] = v[m];
      }
      host_fft64(v, -1);
      for (i64 k = 0; k <= j.M / 2; ++k)
        B->htab[j.off + k] = make_cx((float)(v[k].x / (double)j.M), (float)(v[k].y / (double)j.M));
    }
    return;
  }
  // group by M: one FP64 plan per length, the chirp vectors of a group as its batch
  std::map<i64, std::vector<const SpecJob*>> byM;
  for (const SpecJob& j : B->specs) byM[j.M].push_back(&j);
  for (auto& kv : byM) {
    const i64 M = kv.first;
    af_plan p = nullptr;
    if (af_plan_create_f64(&p, M, -1, AF_ALGO_AUTO) != AF_OK) throw FastError(std::string("FP64 plan: ") + af_last_error());
    const i64 cnt = (i64)kv.second.size();
    double2 *v = nullptr, *V = nullptr;
    try {
      fcheck(cudaMalloc(&v, sizeof(double2) * M * cnt), "spectrum buffers");
      fcheck(cudaMalloc(&V, sizeof(double2) * M * cnt), "spectrum buffers");
      for (i64 i = 0; i < cnt; ++i)
        chirp_vec_kernel<<<(int)std::min<i64>((M + 255) / 256, 4096), 256, 0, st>>>(v + i * M, kv.second[i]->n, M, 1);
      fcheck(cudaGetLastError(), "chirp vectors");
      if (af_exec_c2c_f64(p, AF_LAYOUT_INTERLEAVED, (const double*)v, nullptr, (double*)V, nullptr, cnt, st) != AF_OK)
        throw FastError(std::string("FP64 transform: ") + af_last_error());
      for (i64 i = 0; i < cnt; ++i)
        spec_round_kernel<<<(int)std::min<i64>((M + 255) / 256, 4096), 256, 0, st>>>(V + i * M,
                                                                                       B->dtab + kv.second[i]->off, M);
      fcheck(cudaGetLastError(), "spectrum rounding");
      fcheck(cudaStreamSynchronize(st), "spectra");
    } catch (...) {
      if (v) cudaFree(v);
      if (V) cudaFree(V);
      af_plan_destroy(p);
      throw;
    }
    cudaFree(v);
    cudaFree(V);
    af_plan_destroy(p);
  }
}

static void bind_batch(FastBatch* B, cudaStream_t st) {
  const i64 tabn = std::max<i64>(B->tab_elems, 2);
  B->hshapes = B->shapes;
  B->hxf = B->xf;
  B->hitems = B->queue;
  cx* base;
  if (B->emu) {
    B->htab.assign(tabn, make_cx(0.f, 0.f));
    gen_root_tables(B->segs, nullptr, B->htab.data(), st);
    gen_spectra(B, st);
    B->hws.assign(std::max<i64>(B->ws_elems, 2), make_cx(0.f, 0.f));
    base = B->htab.data();
  } else {
    fcheck(cudaMalloc(&B->dtab, sizeof(cx) * tabn), "root tables");
    gen_root_tables(B->segs, B->dtab, nullptr, st);
    gen_spectra(B, st);
    if (B->ws_elems) fcheck(cudaMalloc(&B->dws, sizeof(cx) * B->ws_elems), "workspace");
    base = B->dtab;
  }
  for (size_t i = 0; i < B->hshapes.size(); ++i) {
    B->hshapes[i].tw = base + B->shape_tw[i];
    B->hshapes[i].ftw = base + B->shape_ftw[i];
  }
  for (size_t i = 0; i < B->hxf.size(); ++i) {
    B->hxf[i].ct = B->xf_ct[i] >= 0 ? base + B->xf_ct[i] : nullptr;
    B->hxf[i].wt = B->xf_wt[i] >= 0 ? base + B->xf_wt[i] : nullptr;
    B->hxf[i].spec = B->xf_spec[i] >= 0 ? base + B->xf_spec[i] : nullptr;
  }
  if (B->emu) return;
  fcheck(cudaMalloc(&B->dshapes, sizeof(FShape) * std::max<size_t>(1, B->hshapes.size())), "shapes");
  fcheck(cudaMalloc(&B->dxf, sizeof(FXform) * std::max<size_t>(1, B->hxf.size())), "transforms");
  fcheck(cudaMalloc(&B->ditems, sizeof(FItem) * std::max<size_t>(1, B->hitems.size())), "items");
  fcheck(cudaMemcpyAsync(B->dshapes, B->hshapes.data(), sizeof(FShape) * B->hshapes.size(),
                         cudaMemcpyHostToDevice, st), "shapes");
  fcheck(cudaMemcpyAsync(B->dxf, B->hxf.data(), sizeof(FXform) * B->hxf.size(), cudaMemcpyHostToDevice, st),
         "transforms");
  fcheck(cudaMemcpyAsync(B->ditems, B->hitems.data(), sizeof(FItem) * B->hitems.size(), cudaMemcpyHostToDevice,
                         st), "items");
  fcheck(cudaMalloc(&B->dctrs, sizeof(unsigned) * B->nctrs), "counters");
  const int per_sm = fast_ctas_per_sm(kThreads, -1, B->smem);
  int dev = 0, sms = 0;
  fcheck(cudaGetDevice(&dev), "device");
  fcheck(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "device");
  if (per_sm < 1) throw FastError("the executor's CTA does not fit an SM");
  B->grid = (int)std::min<i64>((i64)per_sm * sms, (i64)std::max<size_t>(1, B->hitems.size()));
  fcheck(cudaStreamSynchronize(st), "batch upload");
}

// Whether the executor plans every length: 5-smooth lengths that fit one CTA
// or split into two factors of at most 1024; other lengths whose Bluestein
// convolution length does the same, with 2n within the three-level tables.
bool fast_supports(const i64* ns, i64 count) {
  i64 total = 0;
  for (i64 i = 0; i < count; ++i) {
    const i64 n = ns[i];
    if (n < 0) return false;
    total += n;
    if (n == 0) continue;
    if (is_5smooth(n)) {
      if (full_smem(n, 1, true) > kMaxSmem && (n > ((i64)1 << 18) || !four_step_n1(n))) return false;
    } else {
      if (2 * n > ((i64)1 << 18)) return false;  // the chirp's three-level table
      const i64 M = blue_len(n);
      if (full_smem(M, 1, true) > kMaxSmem && !least_fixed_product(2 * n - 1).M &&
          (M > ((i64)1 << 18) || !four_step_n1(M)))
        return false;
    }
  }
  return total < ((i64)1 << 31);
}

FastBatch* fast_create(const i64* ns, i64 count, bool emu, const int* tune, int ntune) {
  FastBatch* B = new FastBatch();
  try {
    B->emu = emu;
    // tuning overrides in FastTune field order; a negative entry keeps the default
    int* fields[] = {&B->tune.radix16, &B->tune.gl_max, &B->tune.balance_v, &B->tune.target, &B->tune.slack,
                     &B->tune.l2_mb, &B->tune.fixed};
    for (int i = 0; i < ntune && i < 7; ++i)
      if (tune[i] >= 0) *fields[i] = tune[i];
    if (B->tune.gl_max < 2 || B->tune.gl_max > 128 || (B->tune.gl_max & (B->tune.gl_max - 1)))
      throw FastError("lines per item must be a power of two in [2, 128]");
    if (B->tune.target < 256 || B->tune.target > 8192) throw FastError("item target must be in [256, 8192]");
    if (B->tune.l2_mb < 1 || B->tune.l2_mb > 4096) throw FastError("workspace budget must be in [1, 4096] MB");
    B->ns.assign(ns, ns + count);
    B->offs.resize(count);
    i64 o = 0;
    for (i64 i = 0; i < count; ++i) {
      if (ns[i] < 0) throw FastError("negative transform length");
      B->offs[i] = o;
      o += ns[i];
    }
    if (o >= ((i64)1 << 31)) throw FastError("total length must be below 2^31");
    B->total = o;
    plan_batch(B);
    bind_batch(B, 0);
  } catch (...) {
    delete B;
    throw;
  }
  return B;
}

void fast_destroy(FastBatch* B) { delete B; }

cudaError_t fast_exec(FastBatch* B, int sign, const cx* in, cx* out, const float* w, double* loss,
                      cudaStream_t st) {
  FArgs A;
  A.in = in;
  A.out = out;
  A.w = w;
  A.loss = loss;
  if (B->emu) {
    A.shapes = B->hshapes.data();
    A.xf = B->hxf.data();
    A.ws = B->hws.data();
    A.items = B->hitems.data();
    B->last_status = emulate_fast(kThreads, sign, A, A.items, (int)B->hitems.size(), B->smem, B->nctrs);
    return cudaSuccess;
  }
  A.shapes = B->dshapes;
  A.xf = B->dxf;
  A.ws = B->dws;
  A.items = B->ditems;
  cudaError_t e = cudaMemsetAsync(B->dctrs, 0, sizeof(unsigned) * B->nctrs, st);
  if (e != cudaSuccess) return e;
  return launch_fast(kThreads, sign, A, (int)B->hitems.size(), B->smem, B->dctrs, B->grid, B->spin_limit, st);
}

// Test hook: the first item of the queue that waits for a previous stage now
// waits for one completion more than that stage makes, and every wait polls
// at most `spin_limit` times, so the next launch ends with FE_TIMEOUT after a
// bounded wait.  Returns false when no item waits.
bool fast_poison_wait(FastBatch* B, long long spin_limit) {
  for (size_t i = 0; i < B->hitems.size(); ++i) {
    if (B->hitems[i].wait_ctr < 0) continue;
    B->hitems[i].wait_cnt += 1;
    B->queue[i].wait_cnt += 1;
    B->spin_limit = spin_limit;
    if (!B->emu)
      fcheck(cudaMemcpy(B->ditems + i, &B->hitems[i], sizeof(FItem), cudaMemcpyHostToDevice), "items");
    return true;
  }
  return false;
}

int fast_status(FastBatch* B, cudaStream_t st);

// ------------------------------------------------------------ autotuner
// The planner's choices are timed on the device for the batch at hand: from
// the defaults, each choice in turn (stage slack, workspace in flight, lines
// per multi-pass item, radix-16 passes with the compile-time lines, item
// size) takes the value
// with the shortest forward launch, the others held.  Operation counts do
// not predict the time (the reference's planner says as much of its own
// algorithm choice, Planned.hs:206-214); the launch is timed with CUDA events,
// three warm-up launches then five timed ones, on zero data.  The winner is
// kept as one JSON line per (GPU name, batch) in `cache_path` (when given):
//   {"gpu": "...", "key": "<count>:<hash of the lengths>", "tune": [...], "ms": t, "default_ms": t0}
static std::string tune_key(const i64* ns, i64 count) {
  unsigned long long h = 1469598103934665603ull;  // FNV-1a over the lengths
  for (i64 i = 0; i < count; ++i) {
    unsigned long long v = (unsigned long long)ns[i];
    for (int b = 0; b < 8; ++b) {
      h ^= (v >> (8 * b)) & 0xffu;
      h *= 1099511628211ull;
    }
  }
  std::ostringstream o;
  o << count << ":" << std::hex << h;
  return o.str();
}

static std::string gpu_name() {
  int dev = 0;
  cudaDeviceProp p;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&p, dev) != cudaSuccess) return "unknown";
  std::string n(p.name);
  for (char& c : n)
    if (c == '"' || c == '\\') c = ' ';
  return n;
}

static const int kTuneFields = 7;
static void tune_to(const FastTune& t, int* v) {
  v[0] = t.radix16;
  v[1] = t.gl_max;
  v[2] = t.balance_v;
  v[3] = t.target;
  v[4] = t.slack;
  v[5] = t.l2_mb;
  v[6] = t.fixed;
}

// the cached choice for (gpu, key), if any
static bool tune_lookup(const char* path, const std::string& gpu, const std::string& key, int* v, double* ms) {
  if (!path) return false;
  FILE* f = fopen(path, "r");
  if (!f) return false;
  char line[1024];
  bool found = false;
  const std::string g = "\"gpu\": \"" + gpu + "\"", k = "\"key\": \"" + key + "\"";
  while (fgets(line, sizeof line, f)) {
    const std::string ln(line);
    if (ln.find(g) == std::string::npos || ln.find(k) == std::string::npos) continue;
    const size_t p = ln.find("\"tune\": [");
    const size_t q = ln.find("\"ms\": ");
    if (p == std::string::npos || q == std::string::npos) continue;
    int t[kTuneFields];
    if (sscanf(ln.c_str() + p, "\"tune\": [%d, %d, %d, %d, %d, %d, %d]", &t[0], &t[1], &t[2], &t[3], &t[4], &t[5],
               &t[6]) != kTuneFields)
      continue;
    memcpy(v, t, sizeof t);
    *ms = atof(ln.c_str() + q + 6);
    found = true;  // the last matching line wins
  }
  fclose(f);
  return found;
}

static void tune_store(const char* path, const std::string& gpu, const std::string& key, const int* v, double ms,
                       double ms0) {
  if (!path) return;
  FILE* f = fopen(path, "a");
  if (!f) return;
  fprintf(f, "{\"gpu\": \"%s\", \"key\": \"%s\", \"tune\": [%d, %d, %d, %d, %d, %d, %d], \"ms\": %.4f, \"default_ms\": %.4f}\n",
          gpu.c_str(), key.c_str(), v[0], v[1], v[2], v[3], v[4], v[5], v[6], ms, ms0);
  fclose(f);
}

// mean time of one forward launch of B over zero data
static double time_batch(FastBatch* B, cx* in, cx* out, cudaStream_t st) {
  cudaEvent_t e0, e1;
  fcheck(cudaEventCreate(&e0), "tuning events");
  fcheck(cudaEventCreate(&e1), "tuning events");
  float ms = 0.f;
  try {
    for (int i = 0; i < 3; ++i) fcheck(fast_exec(B, -1, in, out, nullptr, nullptr, st), "tuning launch");
    fcheck(cudaEventRecord(e0, st), "tuning events");
    for (int i = 0; i < 5; ++i) fcheck(fast_exec(B, -1, in, out, nullptr, nullptr, st), "tuning launch");
    fcheck(cudaEventRecord(e1, st), "tuning events");
    fcheck(cudaEventSynchronize(e1), "tuning events");
    fcheck(cudaEventElapsedTime(&ms, e0, e1), "tuning events");
    if (fast_status(B, st) != FE_OK) throw FastError("a tuning launch timed out");
  } catch (...) {
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    throw;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return ms / 5.0;
}

FastBatch* fast_create_tuned(const i64* ns, i64 count, const char* cache_path, cudaStream_t st, std::string* report) {
  const std::string key = tune_key(ns, count), gpu = gpu_name();
  int best[kTuneFields];
  double best_ms = 0;
  if (tune_lookup(cache_path, gpu, key, best, &best_ms)) {
    if (report) *report = "cached";
    return fast_create(ns, count, false, best, kTuneFields);
  }
  i64 total = 0;
  for (i64 i = 0; i < count; ++i) total += ns[i];
  cx *in = nullptr, *out = nullptr;
  fcheck(cudaMalloc(&in, sizeof(cx) * std::max<i64>(total, 1)), "tuning buffers");
  if (cudaMalloc(&out, sizeof(cx) * std::max<i64>(total, 1)) != cudaSuccess) {
    cudaFree(in);
    throw FastError("tuning buffers: out of device memory");
  }
  std::ostringstream rep;
  double ms0 = 0;
  try {
    fcheck(cudaMemsetAsync(in, 0, sizeof(cx) * std::max<i64>(total, 1), st), "tuning buffers");
    auto measure = [&](const int* v) {
      FastBatch* B = fast_create(ns, count, false, v, kTuneFields);
      double t;
      try {
        t = time_batch(B, in, out, st);
      } catch (...) {
        fast_destroy(B);
        throw;
      }
      fast_destroy(B);
      rep << (rep.tellp() > 0 ? ", " : "") << "[" << v[0] << "," << v[1] << "," << v[2] << "," << v[3] << "," << v[4]
          << "," << v[5] << "," << v[6] << "]: " << t;
      return t;
    };
    const double kTuneMargin = 0.01;
    FastTune d;
    tune_to(d, best);
    best_ms = ms0 = measure(best);
    // coordinate descent over the choices, each value tried with the others held
    const struct {
      int field;
      std::vector<int> values;
    } axes[] = {{4, {1368, 5472}}, {5, {24, 96}}, {1, {16, 64}}, {0, {0}}, {3, {3072}}};
    for (const auto& ax : axes)
      for (int val : ax.values) {
        int cand[kTuneFields];
        memcpy(cand, best, sizeof cand);
        if (cand[ax.field] == val) continue;
        cand[ax.field] = val;
        double t;
        try {
          t = measure(cand);
        } catch (const FastError&) {
          continue;  // a choice the planner refuses for this batch
        }
        // a candidate replaces the incumbent only when it is faster by more
        // than the timing's run-to-run spread (about half a percent): a
        // smaller difference is noise, and the default choices keep the
        // workspace of the stages in flight within L2
        if (t < best_ms * (1.0 - kTuneMargin)) {
          best_ms = t;
          memcpy(best, cand, sizeof best);
        }
      }
  } catch (...) {
    cudaFree(in);
    cudaFree(out);
    throw;
  }
  cudaFree(in);
  cudaFree(out);
  tune_store(cache_path, gpu, key, best, best_ms, ms0);
  if (report) {
    std::ostringstream o;
    o << "{\"tune\": [" << best[0] << ", " << best[1] << ", " << best[2] << ", " << best[3] << ", " << best[4] << ", "
      << best[5] << ", " << best[6] << "], \"ms\": " << best_ms << ", \"default_ms\": " << ms0
      << ", \"candidates\": \"" << rep.str() << "\"}";
    *report = o.str();
  }
  return fast_create(ns, count, false, best, kTuneFields);
}

// the planner choices the batch was made with, as a JSON list (FastTune order)
std::string fast_tuning(FastBatch* B) {
  int v[kTuneFields];
  tune_to(B->tune, v);
  std::ostringstream o;
  o << "[" << v[0] << ", " << v[1] << ", " << v[2] << ", " << v[3] << ", " << v[4] << ", " << v[5] << ", " << v[6]
    << "]";
  return o.str();
}

// FE_OK or FE_TIMEOUT of the last launch (waits for it to finish)
int fast_status(FastBatch* B, cudaStream_t st) {
  if (B->emu) return B->last_status;
  unsigned v = 0;
  fcheck(cudaMemcpyAsync(&v, B->dctrs + FC_ERROR, sizeof v, cudaMemcpyDeviceToHost, st), "status");
  fcheck(cudaStreamSynchronize(st), "status");
  return (int)v;
}

std::string fast_describe(FastBatch* B) {
  std::ostringstream o;
  int kinds[8] = {0};
  i64 fixed = 0;
  for (const FItem& it : B->queue) {
    kinds[it.kind & 7]++;
    fixed += B->shapes[it.shape].fixed;
  }
  o << "{\"items\": " << B->queue.size() << ", \"grid\": " << B->grid << ", \"smem\": " << B->smem
    << ", \"counters\": " << B->nctrs << ", \"shapes\": " << B->shapes.size() << ", \"table_entries\": "
    << B->tab_elems << ", \"ws_elems\": " << B->ws_elems << ", \"fixed_items\": " << fixed << ", \"by_kind\": [";
  for (int k = 0; k < 7; ++k) o << (k ? ", " : "") << kinds[k];
  o << "]}";
  return o.str();
}

}  // namespace af

// ------------------------------------------------------------- internal C ABI
static thread_local std::string g_fast_err;

extern "C" {

__attribute__((visibility("default"))) const char* afx_fast_error(void) { return g_fast_err.c_str(); }

__attribute__((visibility("default"))) int afx_fast_create(const int64_t* ns, int64_t count, int emulate,
                                                           void** out) {
  try {
    *out = af::fast_create((const af::i64*)ns, count, emulate != 0, nullptr, 0);
    return 0;
  } catch (const std::exception& e) {
    g_fast_err = e.what();
    *out = nullptr;
    return 1;
  }
}

__attribute__((visibility("default"))) int afx_fast_create_tuned(const int64_t* ns, int64_t count, int emulate,
                                                                 const int* tune, int ntune, void** out) {
  try {
    *out = af::fast_create((const af::i64*)ns, count, emulate != 0, tune, ntune);
    return 0;
  } catch (const std::exception& e) {
    g_fast_err = e.what();
    *out = nullptr;
    return 1;
  }
}

__attribute__((visibility("default"))) int afx_fast_destroy(void* b) {
  af::fast_destroy((af::FastBatch*)b);
  return 0;
}

__attribute__((visibility("default"))) int afx_fast_exec(void* b, int sign, const float* in, float* out,
                                                         const float* w, double* loss, void* stream) {
  try {
    cudaError_t e = af::fast_exec((af::FastBatch*)b, sign, (const float2*)in, (float2*)out, w, loss,
                                  (cudaStream_t)stream);
    if (e != cudaSuccess) {
      g_fast_err = cudaGetErrorString(e);
      return 2;
    }
    return 0;
  } catch (const std::exception& e) {
    g_fast_err = e.what();
    return 1;
  }
}

__attribute__((visibility("default"))) int afx_fast_describe(void* b, char* buf, size_t len) {
  const std::string s = af::fast_describe((af::FastBatch*)b);
  if (s.size() + 1 > len) return 1;
  memcpy(buf, s.c_str(), s.size() + 1);
  return 0;
}

}  // extern "C"

extern "C" __attribute__((visibility("default"))) int afx_fast_ws(void* b, float* out, int64_t count) {
  af::FastBatch* B = (af::FastBatch*)b;
  if (!B->emu || count > (int64_t)B->hws.size()) return 1;
  memcpy(out, B->hws.data(), sizeof(float2) * count);
  return 0;
}

extern "C" __attribute__((visibility("default"))) int afx_fast_poison_wait(void* b, long long spin_limit) {
  try {
    return af::fast_poison_wait((af::FastBatch*)b, spin_limit) ? 0 : 1;
  } catch (const std::exception& e) {
    g_fast_err = e.what();
    return -1;
  }
}

extern "C" __attribute__((visibility("default"))) int afx_fast_status(void* b, void* stream) {
  try {
    return af::fast_status((af::FastBatch*)b, (cudaStream_t)stream);
  } catch (const std::exception& e) {
    g_fast_err = e.what();
    return -1;
  }
}
