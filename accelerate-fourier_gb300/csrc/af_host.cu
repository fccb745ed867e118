// af_host.cu -- libaf's plan objects: resources (FP64-generated tables),
// lowering of a reference plan tree to a program of tile / map launches, and
// execution.  The C ABI lives in af_api.cu.
#include "af_host.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <functional>
#include <map>
#include <mutex>

namespace AF_NS {

// ============================================================ FP64 spectra on the device
// The Rader kernel spectrum and the Bluestein chirp spectrum of a plan are
// FP64 transforms of tables generated on the device in FP64; they run on the
// device with the library's own Complex Double engine (an FP64 plan of the
// spectrum's length; its own Rader and Bluestein spectra come the same way,
// over shorter lengths), then are scaled and rounded to the element type.
struct DevBufs {
  std::vector<void*> p;
  double2* get(i64 n) {
    void* q = nullptr;
    if (cudaMalloc(&q, sizeof(double2) * (size_t)std::max<i64>(n, 1)) != cudaSuccess) {
      cudaGetLastError();
      throw AfError(AF_ERR_ALLOC, "cudaMalloc of a spectrum buffer failed");
    }
    p.push_back(q);
    return (double2*)q;
  }
  ~DevBufs() {
    for (void* q : p) cudaFree(q);
  }
};

// y = DFT of x (n points, sign as given, unscaled) in FP64 on the device
static void dev_fft64(const double2* x, double2* y, i64 n, int sign) {
  af_plan p = nullptr;
  if (af_plan_create_f64(&p, n, sign, AF_ALGO_AUTO) != AF_OK)
    throw AfError(AF_ERR_CUDA, std::string("FP64 spectrum plan: ") + af_last_error());
  const af_status st = af_exec_c2c_f64(p, AF_LAYOUT_INTERLEAVED, (const double*)x, nullptr, (double*)y, nullptr, 1, 0);
  af_plan_destroy(p);
  if (st != AF_OK) throw AfError(AF_ERR_CUDA, std::string("FP64 spectrum transform: ") + af_last_error());
}

// ============================================================ resources
void PlanRes::release() {
  for (void* p : allocs) cudaFree(p);
  allocs.clear();
  for (cudaStream_t t : streams) cudaStreamDestroy(t);
  streams.clear();
  for (cudaEvent_t e : events) cudaEventDestroy(e);
  events.clear();
  tables.clear();
  pair_tables.clear();
  rader.clear();
  chirps.clear();
}

void* PlanRes::dalloc(size_t bytes) {
  if (dry) {  // address-checking mode: distinct fake device addresses, no device work
    char* p = (char*)(uintptr_t)fake_next;
    fake_next += (bytes + 511) / 256 * 256;
    return p;
  }
  if (no_alloc) throw AfError(AF_ERR_UNSUPPORTED, "this transform needs device tables beyond the static arrays");
  void* p = nullptr;
  if (cudaMalloc(&p, bytes ? bytes : 16) != cudaSuccess) throw AfError(AF_ERR_ALLOC, "cudaMalloc of plan table failed");
  allocs.push_back(p);
  return p;
}

static int ceil_log2(i64 n) {
  int s = 0;
  while (((i64)1 << s) < n) ++s;
  return s;
}

static void cuda_check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw AfError(AF_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

TwTable PlanRes::table(i64 n) {
  auto it = tables.find(n);
  if (it != tables.end()) return it->second;
  TwTable t;
  t.S_log2 = (ceil_log2(n) + 1) / 2;
  const i64 S = (i64)1 << t.S_log2;
  t.H = (int)((n + S - 1) / S);
  t.len = (int)S + t.H;
  if (arena) {
    if (arena_used + (size_t)t.len > arena_cap) throw AfError(AF_ERR_UNSUPPORTED, "twiddle tables exceed the arena");
    t.p = arena + arena_used;
    arena_used += (size_t)t.len;
  } else {
    t.p = (cx*)dalloc(sizeof(cx) * t.len);
  }
  if (!dry) {
    cuda_check(launch_twiddle_table(t.p, n, (int)S, t.H, stream), "twiddle table");
    // tables made on first use (a new length inside a call) must be complete
    // before work on any other stream reads them
    if (!arena) cuda_check(cudaStreamSynchronize(stream), "twiddle table");
  }
  tables[n] = t;
  return t;
}

const i64* PlanRes::line_table(const std::vector<i64>& offs) {
  i64* p = (i64*)dalloc(sizeof(i64) * std::max<size_t>(offs.size(), 1));
  if (dry) host_loffs[p] = offs;
  else cuda_check(cudaMemcpy(p, offs.data(), sizeof(i64) * offs.size(), cudaMemcpyHostToDevice), "line table");
  return p;
}

const cx* PlanRes::pair_table(i64 a, i64 b, int* off_b) {
  auto key = std::make_pair(a, b);
  TwTable ta = table(a), tb = table(b);
  *off_b = ta.len;
  auto it = pair_tables.find(key);
  if (it != pair_tables.end()) return it->second;
  cx* p = (cx*)dalloc(sizeof(cx) * (ta.len + tb.len));
  if (!dry) {
    cuda_check(cudaMemcpy(p, ta.p, sizeof(cx) * ta.len, cudaMemcpyDeviceToDevice), "table copy");
    cuda_check(cudaMemcpy(p + ta.len, tb.p, sizeof(cx) * tb.len, cudaMemcpyDeviceToDevice), "table copy");
  }
  pair_tables[key] = p;
  return p;
}

// Length of the transforms carrying a Rader convolution of length p-1:
// p-1 itself when it is 13-smooth (the reference's Rader), otherwise the
// least 13-smooth M >= 2(p-1)-1, so that the cyclic convolution of length p-1
// runs as one zero-padded convolution instead of nested Rader transforms.
// Length of the transforms that carry Rader's cyclic convolution of p-1:
// p-1 itself when it is 13-smooth, else the least 5-smooth M >= 2(p-1)-1
// (zero padding; 5-smooth lengths avoid the costlier radix-7/11/13 passes
// for a few percent more elements).
i64 rader_conv_len(i64 p) {
  const i64 m = p - 1;
  if (is_13smooth(m)) return m;
  i64 M = 2 * m - 1;
  while (!is_5smooth(M)) ++M;
  return M;
}

// Planned.hs:650-664 levelCachePrime: permutations and the kernel spectrum
// zs = scaleDown (inverse-direction transform of kernel), kernel[i] = W^(g^i).
const RaderRes& PlanRes::rader_res(i64 p, int sign) {
  auto key = std::make_pair(p, sign);
  const i64 M = rader_conv_len(p);
  auto it = rader.find(key);
  if (it != rader.end()) return it->second;
  RaderRes r;
  r.p = p;
  r.g = multiplicative_generator(p);
  const i64 m = p - 1;
  std::vector<int> dlog(m), src(m), inv(m);
  std::vector<i64> perm(m);
  i64 x = 1;
  for (i64 i = 0; i < m; ++i) {  // Permutation.hs:48-54 multiplicative
    perm[i] = x - 1;
    dlog[x - 1] = (int)i;
    x = (i64)((__int128)x * r.g % p);
  }
  std::vector<int> gpow(m);
  for (i64 q = 0; q < m; ++q) src[q] = (int)(1 + perm[(m - q) % m]);  // 1 + reverse perm (75-80)
  for (i64 k = 0; k < m; ++k) inv[k] = dlog[k];                       // inverse perm (68-73)
  for (i64 q = 0; q < m; ++q) gpow[q] = (int)(1 + perm[q]);
  r.dlog = (int*)dalloc(sizeof(int) * m);
  r.src = (int*)dalloc(sizeof(int) * m);
  r.inv = (int*)dalloc(sizeof(int) * m);
  r.gpow = (int*)dalloc(sizeof(int) * m);
  host_tabs[r.dlog] = dlog;
  host_tabs[r.src] = src;
  host_tabs[r.inv] = inv;
  host_tabs[r.gpow] = gpow;
  if (dry) {
    r.M = M;
    r.zs = (cx*)dalloc(sizeof(cx) * M);
    rader[key] = r;
    return rader[key];
  }
  cuda_check(cudaMemcpy(r.dlog, dlog.data(), sizeof(int) * m, cudaMemcpyHostToDevice), "rader tables");
  cuda_check(cudaMemcpy(r.src, src.data(), sizeof(int) * m, cudaMemcpyHostToDevice), "rader tables");
  cuda_check(cudaMemcpy(r.inv, inv.data(), sizeof(int) * m, cudaMemcpyHostToDevice), "rader tables");
  cuda_check(cudaMemcpy(r.gpow, gpow.data(), sizeof(int) * m, cudaMemcpyHostToDevice), "rader tables");
  // kernel and spectrum in FP64 on the device.  The cyclic convolution of
  // length m is computed with transforms of length M >= m: the kernel is
  // placed periodically, kk[i] = k[i], kk[M-i] = k[m-i] (0 < i < m); for
  // M = m this is the reference's kernel spectrum
  {
    DevBufs tmp;
    double2* dk = tmp.get(m);
    double2* kk = tmp.get(M);
    double2* S = tmp.get(M);
    cuda_check(launch_rader_kernel(dk, p, r.g, sign, 0), "rader kernel");
    cuda_check(launch_spectrum_input(dk, m, kk, M, 0, 0), "rader kernel");
    dev_fft64(kk, S, M, +1);
    r.zs = (cx*)dalloc(sizeof(cx) * M);
    r.M = M;
    cuda_check(launch_scale_round(S, r.zs, M, 1.0 / (double)M, 0), "rader spectrum");
    cuda_check(cudaStreamSynchronize(0), "rader spectrum");
  }
  rader[key] = r;
  return rader[key];
}

// Planned.hs:744-754 levelCacheChirp: chirp (first len entries) and the
// spectrum scaleDown (inverse-direction transform of conj chirp) over pad.
const ChirpRes& PlanRes::chirp_res(i64 len, i64 pad, int sign) {
  auto key = std::make_tuple(len, pad, sign);
  auto it = chirps.find(key);
  if (it != chirps.end()) return it->second;
  ChirpRes c;
  c.len = len;
  c.pad = pad;
  if (dry) {
    c.chirp = (cx*)dalloc(sizeof(cx) * len);
    c.spec = (cx*)dalloc(sizeof(cx) * pad);
    chirps[key] = c;
    return chirps[key];
  }
  // chirp and spectrum in FP64 on the device
  {
    DevBufs tmp;
    double2* dc = tmp.get(pad);
    double2* cj = tmp.get(pad);
    double2* S = tmp.get(pad);
    cuda_check(launch_chirp(dc, pad, len, sign, pad, 0), "chirp");
    cuda_check(launch_spectrum_input(dc, pad, cj, pad, 1, 0), "chirp");
    dev_fft64(cj, S, pad, +1);
    c.chirp = (cx*)dalloc(sizeof(cx) * len);
    c.spec = (cx*)dalloc(sizeof(cx) * pad);
    cuda_check(launch_scale_round(dc, c.chirp, len, 1.0, 0), "chirp");
    cuda_check(launch_scale_round(S, c.spec, pad, 1.0 / (double)pad, 0), "chirp");
    cuda_check(cudaStreamSynchronize(0), "chirp");
  }
  chirps[key] = c;
  return chirps[key];
}


// ============================================================ tile building
// longest line one tile holds (two ping-pong buffers in 227 KB of shared memory)
static const i64 kTileCap = sizeof(cx) == 8 ? 13000 : 6200;

// Radix sequence of a tile phase: the fewest Stockham passes over the
// supported butterflies (prime radices 2..13 and the composites built from
// them), ties going to the smaller largest radix; largest radix first, so
// the pass without twiddles carries the most elements per butterfly.
static const int kRadices[] = {2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 15, 16, 20, 25, 27};
static std::vector<int> radices(i64 n) {
  static std::map<i64, std::vector<int>> memo;
  auto it = memo.find(n);
  if (it != memo.end()) return it->second;
  // best[d] over the divisors d of n: (passes, sum of radices) and the radix used
  std::vector<i64> divs;
  for (i64 d = 1; d * d <= n; ++d)
    if (n % d == 0) { divs.push_back(d); if (d != n / d) divs.push_back(n / d); }
  std::sort(divs.begin(), divs.end());
  std::map<i64, std::pair<std::pair<int, int>, int>> best;
  best[1] = {{0, 0}, 0};
  for (i64 d : divs) {
    if (d == 1) continue;
    std::pair<std::pair<int, int>, int> b{{1 << 30, 0}, 0};
    for (int R : kRadices) {
      if (d % R) continue;
      auto sub = best.find(d / R);
      if (sub == best.end() || sub->second.first.first >= (1 << 30)) continue;
      std::pair<int, int> c{sub->second.first.first + 1, sub->second.first.second + R};
      if (c < b.first) b = {c, R};
    }
    best[d] = b;
  }
  std::vector<int> r;
  i64 m = n;
  while (m > 1) {
    const auto& b = best[m];
    if (b.first.first >= (1 << 30)) throw AfError(AF_ERR_UNSUPPORTED, "length is not 13-smooth");
    r.push_back(b.second);
    m /= b.second;
  }
  std::sort(r.begin(), r.end(), std::greater<int>());
  memo[n] = r;
  return r;
}

bool tile_ok(i64 n) { return n >= 1 && n <= kTileCap && is_13smooth(n); }

// (n1, n2) with n = n1 n2, both tile lengths, n1 (the strided column
// transform) near sqrt(n) and at most 1024; false if no such split exists
static bool four_step_split(i64 n, i64* n1, i64* n2) {
  if (!is_13smooth(n)) return false;
  i64 best = 0;
  double bestd = 1e30;
  for (i64 a = 2; a <= 512 && a * a <= n * 4; ++a) {
    if (n % a) continue;
    const i64 b = n / a;
    if (!tile_ok(a) || !tile_ok(b)) continue;
    const double d = std::fabs(std::log((double)a) - 0.5 * std::log((double)n));
    if (d < bestd) { bestd = d; best = a; }
  }
  if (!best) return false;
  *n1 = best;
  *n2 = n / best;
  return true;
}

static void fill_phase(FftPhase& ph, i64 n, rl sign, int ls, int es, int lcnt, int tw_off, int S_log2) {
  memset(&ph, 0, sizeof ph);
  ph.n = (int)n;
  ph.ls = ls;
  ph.es = es;
  ph.lcnt = lcnt;
  ph.lcnt_div = make_fastdiv((unsigned)lcnt);
  ph.sign = sign;
  ph.tw_off = tw_off;
  ph.twS_log2 = S_log2;
  const std::vector<int> rs = radices(n);
  if ((int)rs.size() > AF_MAXP) throw AfError(AF_ERR_UNSUPPORTED, "too many passes");
  int p = 1;
  for (size_t i = 0; i < rs.size(); ++i) {
    PassDesc& pd = ph.pass[i];
    pd.R = rs[i];
    pd.p = p;
    pd.tw_stride = (int)(n / ((i64)p * rs[i]));
    pd.nb_div = make_fastdiv((unsigned)(n / rs[i]));
    pd.p_div = make_fastdiv((unsigned)p);
    p *= rs[i];
  }
  ph.npass = (int)rs.size();
}

static IoDesc io_of(const View& v) {
  IoDesc io;
  memset(&io, 0, sizeof io);
  io.buf = v.buf;
  io.map = IO_AFFINE;
  io.off = v.off;
  io.s_e = v.s_e;
  io.s_lo = v.s_lo;
  io.s_hi = v.s_hi;
  io.s_t = 1;
  io.lo_div = make_fastdiv((unsigned)std::min<i64>(v.lo_cnt, (i64)1 << 30));
  io.line_fast = v.s_e != 1 && v.s_lo == 1;
  io.dc_off = -1;
  return io;
}

// threads per CTA and lines per CTA (G) for a tile with `slen` shared
// elements per line; want_wide asks for >= 16 lines so that strided
// (line-fast) global access moves whole 32-byte sectors
// Every tile reserves the same allowance for twiddle tables (kMaxTw
// entries) and per-line scratch (kMaxG lines), so that any mix of tiles in
// one launch fits the shared memory the largest of them asked for.
static const int kMaxTw = 512;
static const int kMaxG = 128;
static void choose_geometry(i64 slen, i64 lines, int tw_total, bool want_wide, int* threads, int* G) {
  if (tw_total > kMaxTw) throw AfError(AF_ERR_UNSUPPORTED, "twiddle tables exceed the tile allowance");
  const i64 es = (i64)sizeof(cx);
  const i64 budget = 227 * 1024 - (i64)((sizeof(TileDesc) + 15) / 16 * 16) - es * kMaxTw - 4 * es * kMaxG - 256;
  auto fits = [&](i64 g) { return 2 * es * (spad_host((int)(g * slen)) + 2) <= budget; };
  // about 4096 elements per CTA keeps three CTAs resident per SM; strided
  // (line-fast) tiles take at least 4 lines, one 32-byte sector per row
  i64 g = std::max<i64>(1, 4096 / std::max<i64>(slen, 1));
  if (want_wide) g = std::max<i64>(g, 4);
  g = std::min(g, std::max<i64>(lines, 1));
  g = std::min<i64>(g, kMaxG);
  while (g > 1 && !fits(g)) --g;
  if (!fits(g)) throw AfError(AF_ERR_UNSUPPORTED, "transform does not fit a tile");
  *G = (int)g;
  const i64 elems = g * slen;
  // CTAs of up to 4096 elements (two buffers, 83 KB) fit two per SM; larger
  // tiles take 512 threads and a whole SM
  *threads = elems > 4096 ? 512 : (elems >= 1024 ? 256 : 128);
}

struct TileStep {
  TileDesc d;
  int threads = 128;
  i64 lines = 0;
};

// Wavefronts of one half-warp's 64-bit shared accesses: the busiest of the
// 16 eight-byte bank pairs serves one wavefront per distinct address (the
// model of FP32 elements; FP64 tiles use the same choice).
static int half_warp_wavefronts(int* a, int cnt) {
  std::sort(a, a + cnt);
  int per_bank[16] = {0}, worst = 0;
  for (int x = 0; x < cnt; ++x)
    if (x == 0 || a[x] != a[x - 1]) worst = std::max(worst, ++per_bank[a[x] & 15]);
  return worst;
}

// Shared-memory wavefronts of a tile for padding shift sh, from a sample of
// warps: the tile load and store (element- or line-fast) and every Stockham
// pass's reads and writes.
static i64 pad_cost(const TileDesc& d, int sh) {
  const int G = d.G;
  i64 cost = 0;
  int a[16];
  auto warp = [&](auto&& addr, int first, int total) {
    for (int h = first; h < std::min(total, first + 32); h += 16) {
      int cnt = 0;
      for (int g = h; g < std::min(total, h + 16); ++g) a[cnt++] = spad_host(addr(g), sh);
      cost += half_warp_wavefronts(a, cnt);
    }
  };
  auto sampled = [&](int total, auto&& body) {
    const int warps = (total + 31) / 32, step = std::max(1, warps / 4);
    for (int w = 0; w < warps; w += step) body(32 * w);
  };
  const int N = d.nlen, tot = G * N;
  for (int lf : {d.in.line_fast, d.out.line_fast})
    sampled(tot, [&](int first) {
      warp([&](int q) { return lf ? (q % G) * d.LS + q / G : (q / N) * d.LS + q % N; }, first, tot);
    });
  for (int ph = 0; ph < d.nph; ++ph) {
    const FftPhase& f = d.ph[ph];
    for (int ps = 0; ps < f.npass; ++ps) {
      const int R = f.pass[ps].R, p = f.pass[ps].p, nb = f.n / R;
      const int total = G * f.lcnt * nb;
      sampled(total, [&](int first) {
        for (int j = 0; j < R; ++j)
          for (int rw = 0; rw < 2; ++rw)
            warp([&](int g) {
              const int l = g / nb, i = g - l * nb, t = l / f.lcnt;
              const int base = t * d.LS + (l - t * f.lcnt) * f.ls;
              const int q = i / p, k = i - q * p;
              return base + (rw == 0 ? i + j * nb : q * p * R + k + j * p) * f.es;
            }, first, total);
      });
    }
  }
  return cost;
}

// The padding shift (one slot per 2^sh elements; 31 = none) with the fewest
// sampled shared-memory wavefronts.  Never more padding than one slot per 16:
// the geometry was sized for that.  Tiles of the same shape share the answer.
static int choose_pad(const TileDesc& d) {
  std::vector<int> key = {d.G, d.LS, d.nlen, d.in.line_fast, d.out.line_fast, d.nph};
  for (int ph = 0; ph < d.nph; ++ph) {
    const FftPhase& f = d.ph[ph];
    key.insert(key.end(), {f.n, f.lcnt, f.ls, f.es, f.npass});
    for (int ps = 0; ps < f.npass; ++ps) key.insert(key.end(), {f.pass[ps].R, f.pass[ps].p});
  }
  static std::mutex mu;
  static std::map<std::vector<int>, int> memo;
  {
    std::lock_guard<std::mutex> g(mu);
    auto it = memo.find(key);
    if (it != memo.end()) return it->second;
  }
  int best = 4;
  i64 bc = pad_cost(d, 4);
  for (int sh : {5, 6, 7, 8, 9, 10, 31}) {
    const i64 c = pad_cost(d, sh);
    if (c < bc) { bc = c; best = sh; }
  }
  std::lock_guard<std::mutex> g(mu);
  memo[key] = best;
  return best;
}

static void finish_geometry(TileStep& s, i64 slen, bool want_wide) {
  int threads, G;
  choose_geometry(slen, s.lines, s.d.tw_total, want_wide, &threads, &G);
  s.threads = threads;
  s.d.G = G;
  s.d.nlines = (int)s.lines;
  s.d.G_div = make_fastdiv((unsigned)G);
  s.d.N_div = make_fastdiv((unsigned)s.d.nlen);
  s.d.S_div = make_fastdiv((unsigned)s.d.slen);
  s.d.pad_sh = choose_pad(s.d);
}

static TileDesc blank_desc() {
  TileDesc d;
  memset(&d, 0, sizeof d);
  d.pad_sh = 4;
  d.scale = 1.f;
  d.dc_off = -1;
  d.x0_cap = -1;
  return d;
}

// plain tile: FFT of length n (sign) over `lines` lines, optional store twiddle W_ptwN^(lo e)
static TileStep plain_step(PlanRes& res, i64 n, rl sign, i64 lines, const View& in, const View& out,
                           i64 ptwN = 0) {
  TileStep s;
  s.d = blank_desc();
  TileDesc& d = s.d;
  d.kind = TILE_PLAIN;
  d.nlen = (int)n;
  d.slen = (int)n;
  d.LS = (int)n;
  TwTable t = res.table(n);
  d.tw_src = t.p;
  d.tw_total = t.len;
  fill_phase(d.ph[0], n, sign, (int)n, 1, 1, 0, t.S_log2);
  d.nph = 1;
  d.in = io_of(in);
  d.out = io_of(out);
  if (ptwN) {
    TwTable pt = res.table(ptwN);
    d.ptw = pt.p;
    d.ptwS_log2 = pt.S_log2;
    d.ptwN = ptwN;
    d.ptw_mod = make_modn((unsigned long long)ptwN);
    d.ptw_sign = sign;
  }
  s.lines = lines;
  finish_geometry(s, n, d.in.line_fast || d.out.line_fast);
  return s;
}

static i64 mod_inverse(i64 a, i64 m) {
  if (m == 1) return 0;
  i64 t = 0, nt = 1, r = m, nr = ((a % m) + m) % m;
  while (nr) {
    const i64 q = r / nr;
    i64 tmp = t - q * nt; t = nt; nt = tmp;
    tmp = r - q * nr; r = nr; nr = tmp;
  }
  return t < 0 ? t + m : t;
}

static bool gt_tile_ok(const Node* nd) {
  return nd->kind == N_COPRIME && nd->n <= kTileCap && tile_ok(nd->a->n) && tile_ok(nd->b->n);
}
static bool rader_tile_ok(const Node* nd) {
  return nd->kind == N_PRIME && nd->n > 13 && tile_ok(rader_conv_len(nd->n));
}
static bool chirp_tile_ok(const Node* nd) { return nd->kind == N_CHIRP && tile_ok(nd->a->n); }
static bool plain_ok(const Node* nd) {
  return tile_ok(nd->n) && nd->kind != N_CHIRP && !(nd->kind == N_PRIME && nd->n > 13);
}
static bool single_tile_ok(const Node* nd) {
  return nd->n <= 1 || gt_tile_ok(nd) || rader_tile_ok(nd) || chirp_tile_ok(nd) || plain_ok(nd);
}

// Good-Thomas tile (Planned.hs:584-617): grid m x n, n = first factor
static TileStep gt_step(PlanRes& res, const Node* nd, rl sign, i64 lines, const View& in, const View& out) {
  const i64 n = nd->a->n, m = nd->b->n, N = nd->n;
  TileStep s;
  s.d = blank_desc();
  TileDesc& d = s.d;
  d.kind = TILE_GT;
  d.nlen = (int)N;
  d.slen = (int)N;
  d.LS = (int)N;
  int offb = 0;
  d.tw_src = res.pair_table(n, m, &offb);
  d.tw_total = res.table(n).len + res.table(m).len;
  fill_phase(d.ph[0], n, sign, (int)n, 1, (int)m, 0, res.table(n).S_log2);     // rows (j)
  fill_phase(d.ph[1], m, sign, 1, (int)n, (int)n, offb, res.table(m).S_log2);  // cols (k)
  d.nph = 2;
  d.gt_n = (int)n;
  d.gt_m = (int)m;
  d.gt_cm = mod_inverse(n, m);  // i = (n k + m j) mod N  =>  k = i n^-1 mod m
  d.gt_cn = mod_inverse(m, n);  //                           j = i m^-1 mod n
  d.gt_m_mod = make_modn((unsigned long long)m);
  d.gt_n_mod = make_modn((unsigned long long)n);
  d.in = io_of(in);
  d.out = io_of(out);
  d.in.line_fast = d.out.line_fast = 0;
  s.lines = lines;
  finish_geometry(s, N, false);
  return s;
}

// Rader tile (Planned.hs:646-692), convolution length M = rader_conv_len(p)
static TileStep rader_step(PlanRes& res, const Node* nd, rl sign, i64 lines, const View& in, const View& out) {
  const i64 p = nd->n;
  const RaderRes& rr = res.rader_res(p, sign > 0 ? 1 : -1);
  const i64 M = rr.M;
  TileStep s;
  s.d = blank_desc();
  TileDesc& d = s.d;
  d.kind = TILE_RADER;
  d.nlen = (int)p;
  d.slen = (int)M;
  d.LS = (int)M;
  TwTable t = res.table(M);
  d.tw_src = t.p;
  d.tw_total = t.len;
  fill_phase(d.ph[0], M, +1.f, (int)M, 1, 1, 0, t.S_log2);
  fill_phase(d.ph[1], M, -1.f, (int)M, 1, 1, 0, t.S_log2);
  d.nph = 2;
  d.dlog = rr.dlog;
  d.vec_b = rr.zs;
  d.in = io_of(in);
  d.out = io_of(out);
  d.in.line_fast = d.out.line_fast = 0;
  s.lines = lines;
  finish_geometry(s, M, false);
  return s;
}

// Bluestein tile (Planned.hs:760-773)
static TileStep chirp_step(PlanRes& res, const Node* nd, rl sign, i64 lines, const View& in, const View& out) {
  const i64 N = nd->n, M = nd->a->n;
  const ChirpRes& cr = res.chirp_res(N, M, sign > 0 ? 1 : -1);
  TileStep s;
  s.d = blank_desc();
  TileDesc& d = s.d;
  d.kind = TILE_BLUESTEIN;
  d.nlen = (int)N;
  d.slen = (int)M;
  d.LS = (int)M;
  TwTable t = res.table(M);
  d.tw_src = t.p;
  d.tw_total = t.len;
  fill_phase(d.ph[0], M, +1.f, (int)M, 1, 1, 0, t.S_log2);
  fill_phase(d.ph[1], M, -1.f, (int)M, 1, 1, 0, t.S_log2);
  d.nph = 2;
  d.vec_a = cr.chirp;
  d.vec_b = cr.spec;
  d.in = io_of(in);
  d.out = io_of(out);
  d.in.line_fast = d.out.line_fast = 0;
  s.lines = lines;
  finish_geometry(s, M, false);
  return s;
}

static TileStep single_step(PlanRes& res, const Node* nd, rl sign, i64 lines, const View& in, const View& out) {
  if (gt_tile_ok(nd)) return gt_step(res, nd, sign, lines, in, out);
  if (rader_tile_ok(nd)) return rader_step(res, nd, sign, lines, in, out);
  if (chirp_tile_ok(nd)) return chirp_step(res, nd, sign, lines, in, out);
  return plain_step(res, nd->n, sign, lines, in, out);
}

// ------------------------------------------------------- multi-pass schemes
// A transform of length n too large for one tile runs as 2 or 3 passes over
// a workspace region of `ws_len` elements per transform.  Views are built
// for `T` transforms whose input/output rows are `xs` apart and whose
// workspace regions are `wst` apart (the batch path places each transform
// with per-item offsets and uses T = 1).
struct MultiPass {
  std::vector<TileStep> steps;
  i64 ws_len = 0;    // workspace stride per transform
  i64 ws_total = 0;  // workspace elements the scheme touches from ws_base (all T transforms)
};

// Cooley-Tukey four-step (Planned.hs:525-557 for composite nodes; the
// split-radix chain of Planned.hs:490-522 for even sizes): pass A FFT_n1 over
// columns x[n2 j1 + j2] with twiddle W_n^(j2 k1), pass B FFT_n2 over rows,
// X[k1 + n1 k2].
static bool four_step_plan(PlanRes& res, i64 n, rl sign, i64 T, i64 wst, const View& inb,
                           const View& outb, i64 ws_base, MultiPass* mp) {
  i64 n1, n2;
  if (!four_step_split(n, &n1, &n2)) return false;
  View a_in = inb;
  a_in.s_e = n2 * inb.s_e; a_in.s_lo = inb.s_e; a_in.lo_cnt = n2;
  View w;
  w.buf = BUF_WS; w.off = ws_base; w.s_e = n2; w.s_lo = 1; w.s_hi = wst; w.lo_cnt = n2;
  mp->steps.push_back(plain_step(res, n1, sign, T * n2, a_in, w, n));
  View b_in;
  b_in.buf = BUF_WS; b_in.off = ws_base; b_in.s_e = 1; b_in.s_lo = n2; b_in.s_hi = wst; b_in.lo_cnt = n1;
  View b_out = outb;
  b_out.s_e = n1 * outb.s_e; b_out.s_lo = outb.s_e; b_out.lo_cnt = n1;
  mp->steps.push_back(plain_step(res, n2, sign, T * n1, b_in, b_out));
  mp->ws_len = n;
  mp->ws_total = T * wst;
  return true;
}

// Good-Thomas in two passes (Planned.hs:584-617): pass 1 transforms the
// first factor n over the CRT gather x[(n k + m j) mod N] (line k, element j)
// and stores transposed; pass 2 transforms the second factor m over rows and
// scatters by the CRT map r = CRT(q, p).  Either factor may be any
// single-tile transform (split-radix, Rader, Bluestein, Good-Thomas tile).
static bool gt_two_pass_plan(PlanRes& res, const Node* nd, rl sign, i64 T, i64 wst, const View& inb,
                             const View& outb, i64 ws_base, MultiPass* mp) {
  const Node* na = nd->a;
  const Node* nb = nd->b;
  const i64 n = na->n, m = nb->n, N = nd->n;
  if (!single_tile_ok(na) || !single_tile_ok(nb)) return false;
  View in1 = inb;
  in1.s_lo = 0;
  in1.lo_cnt = m;
  View w1;
  w1.buf = BUF_WS; w1.off = ws_base; w1.s_e = m; w1.s_lo = 1; w1.s_hi = wst; w1.lo_cnt = m;
  TileStep s1 = single_step(res, na, sign, T * m, in1, w1);
  s1.d.in.map = IO_GT;
  s1.d.in.mA = n; s1.d.in.mB = m; s1.d.in.mN = N; s1.d.in.s_t = inb.s_e;
  s1.d.in.m_mod = make_modn((unsigned long long)N);
  s1.d.in.line_fast = 0;
  mp->steps.push_back(s1);
  View w2;
  w2.buf = BUF_WS; w2.off = ws_base; w2.s_e = 1; w2.s_lo = m; w2.s_hi = wst; w2.lo_cnt = n;
  View out2 = outb;
  out2.s_lo = 0;
  out2.lo_cnt = n;
  TileStep s2 = single_step(res, nb, sign, T * n, w2, out2);
  s2.d.out.map = IO_GT;
  s2.d.out.mA = (m * mod_inverse(m, n)) % N; s2.d.out.mB = (n * mod_inverse(n, m)) % N; s2.d.out.mN = N;
  s2.d.out.m_mod = make_modn((unsigned long long)N);
  s2.d.out.s_t = outb.s_e;
  s2.d.out.line_fast = 0;
  mp->steps.push_back(s2);
  mp->ws_len = N;
  mp->ws_total = T * wst;
  return true;
}

// Cyclic convolution of length M = n1 n2 in three passes (Planned.hs:803-821,
// directions as in the reference: G = sign +1 first, F = sign -1 after the
// spectrum product):
//   A   columns: FFT_n1(+1) over j1 of a[n2 j1 + j2], twiddle W_M^(+j2 k1)
//   R   rows:    FFT_n2(+1), * S[k1 + n1 k2], FFT_n2(-1), twiddle W_M^(-j2 k1)
//   A'  columns: FFT_n1(-1) over k1 -> c[n2 j1 + j2]
// The load of A and the store of A' carry the Rader or Bluestein maps.
static bool conv_plan(PlanRes& res, i64 M, const cx* S, i64 T, i64 wst, const View& inb,
                      const View& outb, i64 ws_base, MultiPass* mp, TileStep** a_step, TileStep** o_step,
                      i64 dc_off) {
  i64 n1, n2;
  if (!four_step_split(M, &n1, &n2)) return false;
  View a_in = inb;
  a_in.s_e = n2 * inb.s_e; a_in.s_lo = inb.s_e; a_in.lo_cnt = n2;
  View w;
  w.buf = BUF_WS; w.off = ws_base; w.s_e = n2; w.s_lo = 1; w.s_hi = wst; w.lo_cnt = n2;
  mp->steps.push_back(plain_step(res, n1, +1.f, T * n2, a_in, w, M));
  // rows
  View r;
  r.buf = BUF_WS; r.off = ws_base; r.s_e = 1; r.s_lo = n2; r.s_hi = wst; r.lo_cnt = n1;
  TileStep rs = plain_step(res, n2, +1.f, T * n1, r, r, M);
  rs.d.kind = TILE_CONVROW;
  fill_phase(rs.d.ph[1], n2, -1.f, (int)n2, 1, 1, 0, rs.d.ph[0].twS_log2);
  rs.d.nph = 2;
  rs.d.vec_b = S;
  rs.d.sq_lo = 1;
  rs.d.sq_e = n1;
  rs.d.ptw_sign = -1.f;
  rs.d.dc_off = dc_off;
  rs.d.in.line_fast = rs.d.out.line_fast = 0;
  mp->steps.push_back(rs);
  // columns back
  View c_in;
  c_in.buf = BUF_WS; c_in.off = ws_base; c_in.s_e = n2; c_in.s_lo = 1; c_in.s_hi = wst; c_in.lo_cnt = n2;
  View c_out = outb;
  c_out.s_e = n2 * outb.s_e; c_out.s_lo = outb.s_e; c_out.lo_cnt = n2;
  mp->steps.push_back(plain_step(res, n1, -1.f, T * n2, c_in, c_out));
  *a_step = &mp->steps[0];
  *o_step = &mp->steps[2];
  mp->ws_len = M;
  mp->ws_total = T * wst + 2 * T;  // regions, then T DC slots, then T x0 slots
  return true;
}

// Rader in three passes: the conv of length M with the dlog gather/scatter
// fused into the first load and the last store (x0 and DC fix-up included).
static bool rader_conv_plan(PlanRes& res, const Node* nd, rl sign, i64 T, i64 wst, const View& inb,
                            const View& outb, i64 ws_base, MultiPass* mp) {
  const i64 p = nd->n;
  const RaderRes& rr = res.rader_res(p, sign > 0 ? 1 : -1);
  const i64 M = rr.M, m = p - 1;
  TileStep *a, *o;
  // DC slots of the T transforms follow their T workspace regions
  const i64 dc = ws_base + T * wst;
  if (!conv_plan(res, M, rr.zs, T, wst, inb, outb, ws_base, mp, &a, &o, dc)) return false;
  i64 n1, n2;
  four_step_split(M, &n1, &n2);
  // A: a[q] = x[g^-q] for q < p-1, zero beyond; q = n2 j1 + j2 = lo + n2 e
  a->d.in.map = IO_TABLE;
  a->d.in.tab = rr.src;
  a->d.in.q_lo = 1; a->d.in.q_e = n2;
  a->d.in.mN = m;
  a->d.in.s_t = inb.s_e;
  a->d.in.line_fast = 0;
  // A': out[g^q] = x0 + c[q] for q < p-1; q == 0 also out[0] = x0 + DC
  o->d.out.map = IO_RADER;
  o->d.out.tab = rr.gpow;
  o->d.out.q_lo = 1; o->d.out.q_e = n2;
  o->d.out.mN = m;
  o->d.out.s_t = outb.s_e;
  // x0 = x[0] is captured by the first pass (before an in-place last pass
  // overwrites the input) into the T slots after the DC slots
  a->d.x0_cap = dc + T;
  o->d.out.x0_buf = BUF_WS;
  o->d.out.x0_off = dc + T;
  o->d.out.x0_shi = 1;
  o->d.out.dc_off = dc;
  o->d.out.line_fast = 0;
  return true;
}

// Bluestein in three passes: chirp * x (zero padded) fused into the first
// load, chirp * take N into the last store.
static bool chirp_conv_plan(PlanRes& res, const Node* nd, rl sign, i64 T, i64 wst, const View& inb,
                            const View& outb, i64 ws_base, MultiPass* mp) {
  const i64 N = nd->n, M = nd->a->n;
  const ChirpRes& cr = res.chirp_res(N, M, sign > 0 ? 1 : -1);
  TileStep *a, *o;
  if (!conv_plan(res, M, cr.spec, T, wst, inb, outb, ws_base, mp, &a, &o, -1)) return false;
  i64 n1, n2;
  four_step_split(M, &n1, &n2);
  a->d.in.map = IO_CHIRP;
  a->d.in.vec = cr.chirp;
  a->d.in.q_lo = 1; a->d.in.q_e = n2;
  a->d.in.mN = N;
  a->d.in.s_t = inb.s_e;
  a->d.in.line_fast = 0;
  o->d.out.map = IO_CHIRP;
  o->d.out.vec = cr.chirp;
  o->d.out.q_lo = 1; o->d.out.q_e = n2;
  o->d.out.mN = N;
  o->d.out.s_t = outb.s_e;
  o->d.out.line_fast = 0;
  return true;
}

static bool multi_pass(PlanRes& res, const Node* nd, rl sign, i64 T, i64 wst, const View& inb,
                       const View& outb, i64 ws_base, MultiPass* mp);

// workspace stride of a transform's multi-pass scheme
static i64 multi_pass_len(const Node* nd) {
  if (nd->kind == N_PRIME) return rader_conv_len(nd->n);
  if (nd->kind == N_CHIRP) return nd->a->n;
  return nd->n;
}

// Split-radix chains and composites over a factor with no smooth four-step
// split (one transform, T = 1): the power-of-two part of the chain (or the
// composite's first factor) runs as strided columns with the twiddle, and the
// remaining node (Good-Thomas, Rader, Bluestein, ...) runs over the rows
// with its own single-tile or multi-pass scheme, storing X[k1 + n1 k2].
static bool peel_plan(PlanRes& res, const Node* nd, rl sign, i64 T, const View& inb, const View& outb,
                      i64 ws_base, MultiPass* mp) {
  if (T != 1) return false;
  const i64 n = nd->n;
  std::vector<std::pair<i64, const Node*>> cands;
  if (nd->kind == N_SR) {
    const Node* c = nd;
    i64 n1 = 1;
    for (int k = 1; k <= 10 && c->kind == N_SR; ++k) {
      c = c->a;
      n1 *= 2;
      cands.emplace_back(n1, c);
    }
    std::reverse(cands.begin(), cands.end());
  } else if (nd->kind == N_COMPOSITE && tile_ok(nd->a->n)) {
    cands.emplace_back(nd->a->n, nd->b);
  }
  for (auto& cd : cands) {
    const i64 n1 = cd.first, n2 = n / n1;
    const Node* sub = cd.second;
    MultiPass trial;
    View a_in = inb;
    a_in.s_e = n2 * inb.s_e; a_in.s_lo = inb.s_e; a_in.lo_cnt = n2;
    View w;
    w.buf = BUF_WS; w.off = ws_base; w.s_e = n2; w.s_lo = 1; w.s_hi = n; w.lo_cnt = n2;
    trial.steps.push_back(plain_step(res, n1, sign, n2, a_in, w, n));
    // rows k1 of W -> out[k1 + n1 k2]
    if (single_tile_ok(sub)) {
      View r_in;
      r_in.buf = BUF_WS; r_in.off = ws_base; r_in.s_e = 1; r_in.s_lo = n2; r_in.s_hi = 0; r_in.lo_cnt = n1;
      View r_out = outb;
      r_out.s_e = n1 * outb.s_e; r_out.s_lo = outb.s_e; r_out.s_hi = 0; r_out.lo_cnt = n1;
      trial.steps.push_back(single_step(res, sub, sign, n1, r_in, r_out));
      trial.ws_len = n;
      trial.ws_total = n;
    } else {
      View r_in;
      r_in.buf = BUF_WS; r_in.off = ws_base; r_in.s_e = 1; r_in.s_hi = n2; r_in.s_lo = 0; r_in.lo_cnt = 1;
      View r_out = outb;
      r_out.s_e = n1 * outb.s_e; r_out.s_hi = outb.s_e; r_out.s_lo = 0; r_out.lo_cnt = 1;
      MultiPass sm;
      const i64 wst = multi_pass_len(sub);
      if (!multi_pass(res, sub, sign, n1, wst, r_in, r_out, ws_base + n, &sm)) continue;
      for (auto& st : sm.steps) trial.steps.push_back(st);
      trial.ws_len = n + sm.ws_total;
      trial.ws_total = n + sm.ws_total;
    }
    *mp = trial;
    return true;
  }
  return false;
}

// Multi-pass scheme of a node: smooth sizes as four-step, coprime nodes as
// two-pass Good-Thomas, primes as three-pass Rader, chirp nodes as
// three-pass Bluestein, other split-radix/composite nodes by peeling.
// inb/outb: single-level views whose s_hi is the stride between transforms.
static bool multi_pass(PlanRes& res, const Node* nd, rl sign, i64 T, i64 wst, const View& inb,
                       const View& outb, i64 ws_base, MultiPass* mp) {
  mp->steps.clear();
  switch (nd->kind) {
    case N_COPRIME:
      if (gt_two_pass_plan(res, nd, sign, T, wst, inb, outb, ws_base, mp)) return true;
      mp->steps.clear();
      return four_step_plan(res, nd->n, sign, T, wst, inb, outb, ws_base, mp);
    case N_PRIME: return rader_conv_plan(res, nd, sign, T, wst, inb, outb, ws_base, mp);
    case N_CHIRP: return chirp_conv_plan(res, nd, sign, T, wst, inb, outb, ws_base, mp);
    default:
      if (four_step_plan(res, nd->n, sign, T, wst, inb, outb, ws_base, mp)) return true;
      mp->steps.clear();
      return peel_plan(res, nd, sign, T, inb, outb, ws_base, mp);
  }
}

// ============================================================ programs
static Launch launch_of(const TileStep& s) {
  Launch L;
  L.type = L_TILE;
  L.descs.push_back(s.d);
  L.threads = s.threads;
  for (i64 l0 = 0; l0 < s.lines; l0 += s.d.G) {
    WorkItem w;
    memset(&w, 0, sizeof w);
    w.desc = 0;
    w.line0 = (int)l0;
    w.G = (int)std::min<i64>(s.d.G, s.lines - l0);
    L.items.push_back(w);
  }
  L.smem_data = spad_host(s.d.G * s.d.LS, s.d.pad_sh) + 2;
  L.tw_max = s.d.tw_total;
  L.g_max = s.d.G;
  return L;
}

static void append_tile(Launch& L, const TileStep& s, int desc_index, i64 in_add, i64 out_add) {
  for (i64 l0 = 0; l0 < s.lines; l0 += s.d.G) {
    WorkItem w;
    memset(&w, 0, sizeof w);
    w.desc = desc_index;
    w.line0 = (int)l0;
    w.G = (int)std::min<i64>(s.d.G, s.lines - l0);
    w.in_add = in_add;
    w.out_add = out_add;
    L.items.push_back(w);
  }
  L.smem_data = std::max(L.smem_data, spad_host(s.d.G * s.d.LS, s.d.pad_sh) + 2);
  L.tw_max = std::max(L.tw_max, s.d.tw_total);
  L.g_max = std::max(L.g_max, s.d.G);
  L.threads = std::max(L.threads, s.threads);
}

int Program::tile_launches() const { return (int)launches.size(); }

// Side streams and events of a concurrent program (fork-join on the
// caller's stream; under stream capture the branches become parallel graph
// nodes).
static void make_program_streams(PlanRes& res, Program& prog) {
  if (prog.nstreams <= 1 || res.dry || res.no_alloc) {
    prog.nstreams = 1;
    return;
  }
  for (int i = 1; i < prog.nstreams; ++i) {
    cudaStream_t t;
    cuda_check(cudaStreamCreateWithFlags(&t, cudaStreamNonBlocking), "side stream");
    res.streams.push_back(t);
    prog.side.push_back(t);
  }
  // one event per launch, then the fork event and one join event per side stream
  const size_t nev = prog.launches.size() + (size_t)prog.nstreams;
  for (size_t i = 0; i < nev; ++i) {
    cudaEvent_t e;
    cuda_check(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "program event");
    res.events.push_back(e);
    prog.ev.push_back(e);
  }
}

// A one-phase PLAIN tile with AFFINE views and no Rader capture: the
// specialised (smaller) kernel runs it.
static bool simple_desc(const TileDesc& d) {
  return d.kind == TILE_PLAIN && d.in.map == IO_AFFINE && d.out.map == IO_AFFINE && d.nph == 1 && d.x0_cap < 0;
}

void finalize_program(PlanRes& res, Program& prog) {
  for (Launch& L : prog.launches) {
    if (L.type != L_TILE) continue;
    L.generic = 0;
    for (const TileDesc& d : L.descs)
      if (!simple_desc(d)) L.generic = 1;
  }
  make_program_streams(res, prog);
  size_t bytes = 0;
  for (Launch& L : prog.launches) {
    if (L.type != L_TILE) continue;
    bytes = (bytes + 255) / 256 * 256;
    L.desc_off = bytes;
    bytes += sizeof(TileDesc) * L.descs.size();
    bytes = (bytes + 255) / 256 * 256;
    L.item_off = bytes;
    bytes += sizeof(WorkItem) * L.items.size();
  }
  if (!bytes) return;
  if (res.dry) {
    prog.dblob = (char*)res.dalloc(bytes);
    return;
  }
  std::vector<char> host(bytes, 0);
  for (Launch& L : prog.launches) {
    if (L.type != L_TILE) continue;
    memcpy(host.data() + L.desc_off, L.descs.data(), sizeof(TileDesc) * L.descs.size());
    memcpy(host.data() + L.item_off, L.items.data(), sizeof(WorkItem) * L.items.size());
  }
  if (res.blob) {
    // preallocated device area: an ordered copy on the caller's stream (a
    // copy from pageable memory returns once the source has been consumed)
    if (bytes > res.blob_cap) throw AfError(AF_ERR_UNSUPPORTED, "program exceeds the descriptor area");
    prog.dblob = res.blob;
    cuda_check(cudaMemcpyAsync(prog.dblob, host.data(), bytes, cudaMemcpyHostToDevice, res.stream),
               "program upload");
    return;
  }
  prog.dblob = (char*)res.dalloc(bytes);
  cuda_check(cudaMemcpy(prog.dblob, host.data(), bytes, cudaMemcpyHostToDevice), "program upload");
}

TileBases make_bases(const rl* in_re, const rl* in_im, rl* out_re, rl* out_im, cx* ws,
                     const rl* aux_re, const rl* aux_im) {
  TileBases b;
  memset(&b, 0, sizeof b);
  if (in_im) { b.re[BUF_IN] = (rl*)in_re; b.im[BUF_IN] = (rl*)in_im; }
  else b.c[BUF_IN] = (cx*)in_re;
  if (out_im) { b.re[BUF_OUT] = out_re; b.im[BUF_OUT] = out_im; }
  else b.c[BUF_OUT] = (cx*)out_re;
  b.c[BUF_WS] = ws;
  if (aux_im) { b.re[BUF_AUX] = (rl*)aux_re; b.im[BUF_AUX] = (rl*)aux_im; }
  else b.c[BUF_AUX] = (cx*)aux_re;
  return b;
}

static cudaError_t run_launch(const Program& prog, const Launch& L, const TileBases& bases, double* loss,
                              cudaStream_t st) {
  if (L.type == L_TILE) {
    LaunchSpec spec;
    spec.descs = reinterpret_cast<const TileDesc*>(prog.dblob + L.desc_off);
    spec.items = reinterpret_cast<const WorkItem*>(prog.dblob + L.item_off);
    spec.nitems = (int)L.items.size();
    spec.threads = L.threads;
    spec.smem_data = L.smem_data;
    // shared memory for this launch's largest buffers, tables and line count:
    // every tile fits the fixed allowances (choose_geometry), so the launch's
    // maxima fit too, and small tiles keep more CTAs per SM
    spec.smem_bytes = tile_smem_bytes(L.smem_data, L.tw_max, L.g_max);
    spec.generic = L.generic;
    return launch_tiles(spec, bases, loss, st);
  }
  return launch_map(L.md, bases, st);
}

cudaError_t run_program(const Program& prog, const TileBases& bases, double* loss, cudaStream_t st) {
  const size_t nl = prog.launches.size();
  cudaError_t err;
  if (prog.nstreams <= 1) {
    for (const Launch& L : prog.launches)
      if ((err = run_launch(prog, L, bases, loss, st)) != cudaSuccess) return err;
    return cudaSuccess;
  }
  auto strm = [&](int i) { return i == 0 ? st : prog.side[i - 1]; };
  // fork: every side stream waits for the caller's work before the program
  cudaEvent_t fork = prog.ev[nl];
  if ((err = cudaEventRecord(fork, st)) != cudaSuccess) return err;
  for (int i = 1; i < prog.nstreams; ++i)
    if ((err = cudaStreamWaitEvent(strm(i), fork, 0)) != cudaSuccess) return err;
  for (size_t k = 0; k < nl; ++k) {
    const Launch& L = prog.launches[k];
    cudaStream_t s = strm(L.stream);
    for (int d : L.deps)
      if (prog.launches[d].stream != L.stream)
        if ((err = cudaStreamWaitEvent(s, prog.ev[d], 0)) != cudaSuccess) return err;
    if ((err = run_launch(prog, L, bases, loss, s)) != cudaSuccess) return err;
    if (L.signal && (err = cudaEventRecord(prog.ev[k], s)) != cudaSuccess) return err;
  }
  // join: the caller's stream waits for every side stream
  for (int i = 1; i < prog.nstreams; ++i) {
    cudaEvent_t j = prog.ev[nl + i];
    if ((err = cudaEventRecord(j, strm(i))) != cudaSuccess) return err;
    if ((err = cudaStreamWaitEvent(st, j, 0)) != cudaSuccess) return err;
  }
  return cudaSuccess;
}

// ============================================================ single-plan lowering
struct Lowering {
  PlanRes& res;
  Program* prog;
  i64 top = 0;
  i64 peak = 0;

  i64 alloc(i64 elems) {
    const i64 o = top;
    top += (elems + 63) / 64 * 64;
    peak = std::max(peak, top);
    return o;
  }
  static bool simple(const View& v, i64 lines) { return v.lo_cnt >= lines; }

  void emit_step(const TileStep& s) { prog->launches.push_back(launch_of(s)); }

  void emit_map(MapDesc md, const View& in, const View& out) {
    Launch L;
    L.type = L_MAP;
    md.in = io_of(in);
    md.out = io_of(out);
    L.md = md;
    prog->launches.push_back(L);
  }

  static MapDesc map0(int mode, i64 lines, i64 nout) {
    MapDesc m;
    memset(&m, 0, sizeof m);
    m.mode = mode;
    m.nlines = lines;
    m.nout = nout;
    m.scale = 1.f;
    m.dc_ws = -1;
    m.x0_ws = -1;
    return m;
  }

  // Transform `lines` rows through any 2-level views.
  void node(const Node* nd, rl sign, i64 lines, const View& in, const View& out) {
    const i64 n = nd->n;
    if (n == 0 || lines == 0) return;
    if (n == 1) {
      emit_map(map0(MAP_COPY, lines, 1), in, out);
      return;
    }
    if (single_tile_ok(nd)) {
      emit_step(single_step(res, nd, sign, lines, in, out));
      return;
    }
    // multi-pass schemes need single-level views; route others via temps
    if (!simple(in, lines) || !simple(out, lines)) {
      const i64 mark = top;
      View tin = in, tout = out;
      if (!simple(in, lines)) {
        tin = View::rows(BUF_WS, alloc(lines * n), n, lines);
        emit_map(map0(MAP_COPY, lines, n), in, tin);
      }
      if (!simple(out, lines)) tout = View::rows(BUF_WS, alloc(lines * n), n, lines);
      node(nd, sign, lines, tin, tout);
      if (!simple(out, lines)) emit_map(map0(MAP_COPY, lines, n), tout, out);
      top = mark;
      return;
    }
    // fused multi-pass scheme over all rows
    {
      MultiPass mp;
      const i64 mark = top;
      const i64 wsr = multi_pass_len(nd);
      const i64 W = top;  // the scheme's workspace starts here; sized after planning
      View inb = in, outb = out;
      inb.s_hi = in.s_lo; inb.s_lo = 0; inb.lo_cnt = 1;
      outb.s_hi = out.s_lo; outb.s_lo = 0; outb.lo_cnt = 1;
      if (multi_pass(res, nd, sign, lines, wsr, inb, outb, W, &mp)) {
        alloc(mp.ws_total + 64);
        for (auto& s : mp.steps) emit_step(s);
        top = mark;
        return;
      }
      top = mark;
    }
    switch (nd->kind) {
      case N_COPRIME: good_thomas(nd, sign, lines, in, out); return;
      case N_PRIME: rader_multi(nd, sign, lines, in, out); return;
      case N_CHIRP: bluestein_multi(nd, sign, lines, in, out); return;
      default: recursive_four_step(nd, sign, lines, in, out); return;
    }
  }

  // Cooley-Tukey four-step with a recursive row transform (sizes whose rows
  // do not fit one tile): columns n1 = power of two from the SR chain or the
  // composite's first factor.
  void recursive_four_step(const Node* nd, rl sign, i64 lines, const View& in, const View& out) {
    const i64 n = nd->n;
    i64 n1;
    const Node* sub2;
    if (nd->kind == N_SR) {
      int a = 0;
      const Node* c = nd;
      while (c->kind == N_SR) { c = c->a; ++a; }
      int k = std::min(a, 10);
      n1 = (i64)1 << k;
      sub2 = nd;
      for (int i = 0; i < k; ++i) sub2 = sub2->a;
    } else if (nd->kind == N_COMPOSITE) {
      n1 = nd->a->n;
      sub2 = nd->b;
    } else {
      throw AfError(AF_ERR_UNSUPPORTED, "no lowering for node " + Planner::describe(nd));
    }
    const i64 n2 = n / n1;
    const i64 mark = top;
    const i64 W = alloc(lines * n);
    View a_in;
    a_in.buf = in.buf; a_in.off = in.off;
    a_in.s_e = n2 * in.s_e; a_in.s_lo = in.s_e; a_in.s_hi = in.s_lo; a_in.lo_cnt = n2;
    View a_out;
    a_out.buf = BUF_WS; a_out.off = W;
    a_out.s_e = n2; a_out.s_lo = 1; a_out.s_hi = n; a_out.lo_cnt = n2;
    if (tile_ok(n1)) {
      emit_step(plain_step(res, n1, sign, lines * n2, a_in, a_out, n));
    } else {
      const i64 T1 = alloc(lines * n), T2 = alloc(lines * n);
      View trows = View::rows(BUF_WS, T1, n1, lines * n2);
      emit_map(map0(MAP_COPY, lines * n2, n1), a_in, trows);
      View t2rows = View::rows(BUF_WS, T2, n1, lines * n2);
      node(nd->a, sign, lines * n2, trows, t2rows);
      MapDesc tw = map0(MAP_TWIDDLE, lines * n2, n1);
      tw.n = n;
      tw.m = n2;
      TwTable pt = res.table(n);
      tw.tab_tw = pt.p;
      tw.tw_log2 = pt.S_log2;
      tw.tw_sign = sign;
      emit_map(tw, t2rows, a_out);
    }
    View b_in = View::rows(BUF_WS, W, n2, lines * n1);
    View b_out;
    b_out.buf = out.buf; b_out.off = out.off;
    b_out.s_e = n1 * out.s_e; b_out.s_lo = out.s_e; b_out.s_hi = out.s_lo; b_out.lo_cnt = n1;
    node(sub2, sign, lines * n1, b_in, b_out);
    top = mark;
  }

  // Good-Thomas through explicit CRT maps (Planned.hs:584-617)
  void good_thomas(const Node* nd, rl sign, i64 lines, const View& in, const View& out) {
    const i64 n = nd->a->n, m = nd->b->n, N = nd->n;
    const i64 mark = top;
    const i64 W1 = alloc(lines * N), W2 = alloc(lines * N);
    MapDesc g = map0(MAP_GT_IN, lines, N);
    g.n = n; g.m = m; g.nm = N;
    emit_map(g, in, View::rows(BUF_WS, W1, N, lines));
    View r_in = View::rows(BUF_WS, W1, n, lines * m);
    View r_out;
    r_out.buf = BUF_WS; r_out.off = W2;
    r_out.s_e = m; r_out.s_lo = 1; r_out.s_hi = N; r_out.lo_cnt = m;
    node(nd->a, sign, lines * m, r_in, r_out);
    View c_in = View::rows(BUF_WS, W2, m, lines * n);
    View c_out = View::rows(BUF_WS, W1, m, lines * n);
    node(nd->b, sign, lines * n, c_in, c_out);
    MapDesc s = map0(MAP_GT_OUT, lines, N);
    s.n = n; s.m = m; s.nm = N;
    emit_map(s, View::rows(BUF_WS, W1, N, lines), out);
    top = mark;
  }

  // Rader through explicit permutation maps and the sub-plan of p-1
  // (Planned.hs:646-692); used only when p-1 has no fused scheme
  void rader_multi(const Node* nd, rl sign, i64 lines, const View& in, const View& out) {
    const i64 p = nd->n, m = p - 1;
    const RaderRes& rr = res.rader_res(p, sign > 0 ? 1 : -1);
    if (rr.M != m) throw AfError(AF_ERR_UNSUPPORTED, "Rader length without a fused scheme");
    const i64 mark = top;
    const i64 W1 = alloc(lines * m), W2 = alloc(lines * m), X0 = alloc(lines), DC = alloc(lines);
    View w1 = View::rows(BUF_WS, W1, m, lines), w2 = View::rows(BUF_WS, W2, m, lines);
    MapDesc g = map0(MAP_TABLE, lines, m);
    g.tab = rr.src;
    g.x0_ws = X0;
    emit_map(g, in, w1);
    node(nd->a, +1.f, lines, w1, w2);
    MapDesc mul = map0(MAP_MUL, lines, m);
    mul.vec = rr.zs;
    mul.dc_ws = DC;
    emit_map(mul, w2, w2);
    node(nd->a, -1.f, lines, w2, w1);
    MapDesc o = map0(MAP_RADER_OUT, lines, p);
    o.tab = rr.inv;
    o.x0_ws = X0;
    o.dc_ws = DC;
    emit_map(o, w1, out);
    top = mark;
  }

  // Bluestein through explicit chirp maps (Planned.hs:760-773)
  void bluestein_multi(const Node* nd, rl sign, i64 lines, const View& in, const View& out) {
    const i64 N = nd->n, M = nd->a->n;
    const ChirpRes& cr = res.chirp_res(N, M, sign > 0 ? 1 : -1);
    const i64 mark = top;
    const i64 W1 = alloc(lines * M), W2 = alloc(lines * M);
    View w1 = View::rows(BUF_WS, W1, M, lines), w2 = View::rows(BUF_WS, W2, M, lines);
    MapDesc ci = map0(MAP_CHIRP_IN, lines, M);
    ci.vec = cr.chirp;
    ci.n = N;
    emit_map(ci, in, w1);
    node(nd->a, +1.f, lines, w1, w2);
    MapDesc mul = map0(MAP_MUL, lines, M);
    mul.vec = cr.spec;
    emit_map(mul, w2, w2);
    node(nd->a, -1.f, lines, w2, w1);
    MapDesc co = map0(MAP_MUL, lines, N);
    co.vec = cr.chirp;
    emit_map(co, View::rows(BUF_WS, W1, M, lines), out);
    top = mark;
  }
};

void build_program(PlanRes& res, const Node* root, rl sign, i64 batch, Program* prog) {
  Lowering L{res, prog};
  prog->launches.clear();
  View in = View::rows(BUF_IN, 0, root->n, batch);
  View out = View::rows(BUF_OUT, 0, root->n, batch);
  L.node(root, sign, batch, in, out);
  prog->ws_elems = L.peak;
  finalize_program(res, *prog);
}

void build_program_view(PlanRes& res, const Node* root, rl sign, i64 lines, const View& in, const View& out,
                        Program* prog) {
  Lowering L{res, prog};
  prog->launches.clear();
  L.node(root, sign, lines, in, out);
  prog->ws_elems = L.peak;
  finalize_program(res, *prog);
}

// ============================================================ batched executor
// Many transforms of mixed lengths stored back to back.  Every transform is
// planned with the reference planner; transforms that fit one tile run in
// a handful of launches (split by CTA size), larger ones run their fused
// multi-pass scheme, with the transforms grouped into chunks whose
// workspace stays resident in L2 between passes.
struct BatchPlan {
  i64 count = 0;
  int sign = -1;
  std::vector<i64> ns, offs;
  Planner planner;
  PlanRes res;
  Program fwd, inv, cot;  // sign, -sign, sign with the cotangent epilogue
  i64 ws_elems = 0;
  cx* ws = nullptr;
  i64 fallback = 0;      // transforms executed through their own programs
  bool cot_ok = true;    // every transform has a fused program for the cotangent epilogue
  i64 bluestein_fallbacks = 0;  // transforms whose tree has no fused scheme (run as chirp-z)
  std::vector<std::pair<i64, Program>> fb_fwd, fb_inv;  // (index, program)
};

static const i64 kChunkElems = (i64)3 << 20;  // 24 MB of workspace per L2 chunk
static const int kLanes = 3;                   // chunks in flight (72 MB of workspace in L2)

static void build_batch_program(BatchPlan* B, rl sign, Program& prog,
                                std::vector<std::pair<i64, Program>>& fallback, bool cot) {
  prog.launches.clear();
  fallback.clear();
  std::map<i64, const Node*> roots;
  // stage 0: single-tile transforms, one launch per thread class
  // single-tile launches are split by CTA size and shared-memory class, so
  // that small transforms are not held to the occupancy of large ones
  std::map<std::pair<int, int>, Launch> single;  // (threads * 2 + simple, smem class)
  auto single_key = [](const TileStep& s) {
    int c = 0;
    while ((1 << c) < spad_host(s.d.G * s.d.LS, s.d.pad_sh) + 2) ++c;
    return std::make_pair(s.threads * 2 + (simple_desc(s.d) ? 1 : 0), c);
  };
  struct Big {
    i64 i;
    MultiPass mp;
  };
  std::vector<Big> bigs;
  std::map<i64, std::vector<i64>> singles_by_n;  // single-tile transforms by length
  for (i64 i = 0; i < B->count; ++i) {
    const i64 n = B->ns[i];
    if (n == 0) continue;
    const Node* nd = B->planner.automatic(n);
    View in = View::rows(BUF_IN, 0, n, 1), out = View::rows(BUF_OUT, 0, n, 1);
    if (single_tile_ok(nd)) {
      singles_by_n[n].push_back(i);
      continue;
    }
    Big b;
    b.i = i;
    View inb = in, outb = out;
    inb.s_hi = n; inb.s_lo = 0; inb.lo_cnt = 1;
    outb.s_hi = n; outb.s_lo = 0; outb.lo_cnt = 1;
    if (multi_pass(B->res, nd, sign, 1, multi_pass_len(nd), inb, outb, 0, &b.mp)) {
      b.mp.steps.back().d.cot = cot;
      bigs.push_back(std::move(b));
      continue;
    }
    // no fused scheme for this plan tree: the DFT of length n runs as one
    // zero-padded Bluestein convolution (chirp-z) of 13-smooth length
    i64 pad = 2 * n - 1;
    while (!is_5smooth(pad)) ++pad;
    const Node* ch = B->planner.chirp(n, pad);
    if (single_tile_ok(ch)) {
      TileStep s = single_step(B->res, ch, sign, 1, in, out);
      s.d.cot = cot;
      Launch& L = single[single_key(s)];
      L.type = L_TILE;
      const int di = (int)L.descs.size();
      L.descs.push_back(s.d);
      append_tile(L, s, di, B->offs[i], B->offs[i]);
      B->bluestein_fallbacks++;
    } else if (multi_pass(B->res, ch, sign, 1, multi_pass_len(ch), inb, outb, 0, &b.mp)) {
      b.mp.steps.back().d.cot = cot;
      bigs.push_back(std::move(b));
      B->bluestein_fallbacks++;
    } else {
      Program p;
      build_program(B->res, nd, sign, 1, &p);
      fallback.emplace_back(i, std::move(p));
    }
  }
  // Single-tile transforms of one length are the lines of one step: a
  // gathered-line view (each line's offset from a table) lets a CTA take
  // several small transforms at once.
  for (auto& kv : singles_by_n) {
    const i64 n = kv.first;
    const std::vector<i64>& idx = kv.second;
    const Node* nd = B->planner.automatic(n);
    const i64 cnt = (i64)idx.size();
    std::vector<i64> offs(idx.size());
    for (size_t j = 0; j < idx.size(); ++j) offs[j] = B->offs[idx[j]];
    const i64* lt = B->res.line_table(offs);
    View in = View::rows(BUF_IN, 0, n, cnt), out = View::rows(BUF_OUT, 0, n, cnt);
    TileStep s = n == 1 ? plain_step(B->res, 1, sign, cnt, in, out) : single_step(B->res, nd, sign, cnt, in, out);
    s.d.in.loff = lt;
    s.d.out.loff = lt;
    s.d.cot = cot;
    Launch& L = single[single_key(s)];
    L.type = L_TILE;
    const int di = (int)L.descs.size();
    L.descs.push_back(s.d);
    append_tile(L, s, di, 0, 0);
  }
  // Streams: (lane, CTA size class).  Lanes kLanes are the chunk pipelines,
  // lane kLanes holds the single-tile launches; classes are the CTA sizes
  // 128, 256, 512.
  // classes: CTA size x (specialised or general kernel)
  auto cls_of = [](int threads, bool simple) { return (threads >= 512 ? 2 : (threads >= 256 ? 1 : 0)) * 2 + simple; };
  const int NC = 6;
  i64 peak = 0;
  auto stream_of = [&](int lane, int threads, bool simple) { return lane * NC + cls_of(threads, simple); };
  int max_stream = 0;
  // the single-tile launches depend on nothing
  for (auto it = single.rbegin(); it != single.rend(); ++it) {
    Launch& L = it->second;
    // heavy items first
    std::stable_sort(L.items.begin(), L.items.end(), [&](const WorkItem& a, const WorkItem& b) {
      return L.descs[a.desc].slen > L.descs[b.desc].slen;
    });
    bool simple = true;
    for (const TileDesc& d : L.descs) simple = simple && simple_desc(d);
    L.stream = stream_of(kLanes, L.threads, simple);
    max_stream = std::max(max_stream, L.stream);
    prog.launches.push_back(L);
  }
  // multi-pass transforms: chunks of at most kChunkElems of workspace; chunk
  // c runs on lane c mod kLanes in that lane's workspace region, so kLanes
  // chunks are in flight and each chunk's passes stay in L2.  Within a chunk,
  // pass st of every transform waits for pass st-1 of the chunk; the first
  // pass of a chunk waits for the last pass of the lane's previous chunk
  // (workspace reuse).
  std::sort(bigs.begin(), bigs.end(), [](const Big& a, const Big& b) { return a.mp.ws_total > b.mp.ws_total; });
  std::vector<std::pair<size_t, size_t>> chunks;
  i64 lane_ws = 0;
  for (size_t k = 0; k < bigs.size();) {
    i64 used = 0;
    size_t e = k;
    while (e < bigs.size() && (e == k || used + bigs[e].mp.ws_total + 128 <= kChunkElems)) {
      used += (bigs[e].mp.ws_total + 63) / 64 * 64 + 64;
      ++e;
    }
    chunks.emplace_back(k, e);
    lane_ws = std::max(lane_ws, used);
    k = e;
  }
  lane_ws = (lane_ws + 63) / 64 * 64;
  std::vector<std::vector<int>> lane_last(kLanes);  // launches of the lane's previous chunk's last pass
  // chunks go to the least-loaded lane (element-phases as the cost), largest
  // chunks first, so that the lanes finish together
  std::vector<double> lane_load(kLanes, 0.0);
  for (size_t c = 0; c < chunks.size(); ++c) {
    const size_t k = chunks[c].first, e = chunks[c].second;
    int lane = 0;
    for (int l = 1; l < kLanes; ++l)
      if (lane_load[l] < lane_load[lane]) lane = l;
    for (size_t j = k; j < e; ++j)
      for (const TileStep& st : bigs[j].mp.steps) lane_load[lane] += (double)st.lines * st.d.slen * std::max(1, st.d.nph);
    const i64 ws0 = lane * lane_ws;
    size_t maxsteps = 0;
    for (size_t j = k; j < e; ++j) maxsteps = std::max(maxsteps, bigs[j].mp.steps.size());
    std::vector<int> prev = lane_last[lane];
    for (size_t st = 0; st < maxsteps; ++st) {
      // one launch per CTA size: a few large tiles do not hold the many
      // small ones to their shared-memory footprint
      std::map<int, Launch> cls;  // threads * 2 + simple
      std::map<int, std::map<std::pair<i64, int>, int>> dmaps;
      i64 wpos = ws0;
      for (size_t j = k; j < e; ++j) {
        const Big& b = bigs[j];
        const i64 woff = wpos;
        wpos += (b.mp.ws_total + 63) / 64 * 64 + 64;
        if (st >= b.mp.steps.size()) continue;
        const TileStep& s = b.mp.steps[st];
        const i64 n = B->ns[b.i];
        const int ck = s.threads * 2 + (simple_desc(s.d) ? 1 : 0);
        Launch& L = cls[ck];
        L.type = L_TILE;
        auto& dmap = dmaps[ck];
        auto key = std::make_pair(n, s.threads);
        int di;
        auto it = dmap.find(key);
        if (it == dmap.end()) {
          di = (int)L.descs.size();
          L.descs.push_back(s.d);
          dmap[key] = di;
        } else {
          di = it->second;
        }
        // in: user input (pass 0) or workspace; out: workspace or user output
        const i64 in_add = s.d.in.buf == BUF_WS ? woff : B->offs[b.i];
        const i64 out_add = s.d.out.buf == BUF_WS ? woff : B->offs[b.i];
        append_tile(L, s, di, in_add, out_add);
      }
      std::vector<int> cur;
      // largest CTAs first: their few long CTAs start before the many short ones
      for (auto it = cls.rbegin(); it != cls.rend(); ++it) {
        Launch& L = it->second;
        if (L.items.empty()) continue;
        L.stream = stream_of(lane, L.threads, (it->first & 1) != 0);
        max_stream = std::max(max_stream, L.stream);
        L.deps = prev;
        for (int d : prev)
          if (prog.launches[d].stream != L.stream) prog.launches[d].signal = true;
        cur.push_back((int)prog.launches.size());
        prog.launches.push_back(L);
      }
      prev = cur;
      peak = std::max(peak, wpos);
    }
    lane_last[lane] = prev;
  }
  prog.ws_elems = peak;
  prog.nstreams = max_stream + 1;
  finalize_program(B->res, prog);
}

BatchPlan* batch_create(const i64* ns, i64 count, int sign) { return batch_create_mode(ns, count, sign, false); }

BatchPlan* batch_create_mode(const i64* ns, i64 count, int sign, bool dry) {
  BatchPlan* B = new BatchPlan();
  B->res.dry = dry;
  try {
    B->count = count;
    B->sign = sign;
    B->ns.assign(ns, ns + count);
    B->offs.resize(count);
    i64 o = 0;
    for (i64 i = 0; i < count; ++i) {
      if (ns[i] < 0) throw AfError(AF_ERR_INVALID, "negative transform length");
      B->offs[i] = o;
      o += ns[i];
    }
    if (o >= ((i64)1 << 31)) throw AfError(AF_ERR_UNSUPPORTED, "total length must be below 2^31");
    build_batch_program(B, (rl)sign, B->fwd, B->fb_fwd, false);
    build_batch_program(B, (rl)-sign, B->inv, B->fb_inv, false);
    std::vector<std::pair<i64, Program>> fb_cot;
    build_batch_program(B, (rl)sign, B->cot, fb_cot, true);
    B->cot_ok = fb_cot.empty();
    i64 ws = std::max(std::max(B->fwd.ws_elems, B->inv.ws_elems), B->cot.ws_elems);
    for (auto& f : B->fb_fwd) ws = std::max(ws, f.second.ws_elems);
    for (auto& f : B->fb_inv) ws = std::max(ws, f.second.ws_elems);
    B->fallback = (i64)B->fb_fwd.size();
    B->ws_elems = ws;
    if (!dry) {
      if (ws) cuda_check(cudaMalloc(&B->ws, sizeof(cx) * ws), "batch workspace");
      cuda_check(cudaDeviceSynchronize(), "batch tables");
    }
  } catch (...) {
    batch_destroy(B);
    throw;
  }
  return B;
}

void batch_destroy(BatchPlan* B) {
  if (!B) return;
  if (B->ws) cudaFree(B->ws);
  B->res.release();
  delete B;
}

cudaError_t batch_run(BatchPlan* B, bool inverse, const cx* in, cx* out, const rl* w, double* loss,
                      cudaStream_t st) {
  if (w && !B->cot_ok) throw AfError(AF_ERR_UNSUPPORTED, "cotangent epilogue needs fused programs for every length");
  const Program& prog = w ? B->cot : (inverse ? B->inv : B->fwd);
  TileBases bases = make_bases((const rl*)in, nullptr, (rl*)out, nullptr, B->ws, w, nullptr);
  if (w) {
    // weights are real: BUF_AUX is read as a real plane indexed like the output
    bases.c[BUF_AUX] = nullptr;
    bases.re[BUF_AUX] = (rl*)w;
  }
  cudaError_t e = run_program(prog, bases, loss, st);
  if (e != cudaSuccess) return e;
  if (w) return cudaSuccess;
  for (auto& f : (inverse ? B->fb_inv : B->fb_fwd)) {
    const i64 o = B->offs[f.first];
    TileBases b2 = make_bases((const rl*)(in + o), nullptr, (rl*)(out + o), nullptr, B->ws,
                              w ? w + o : nullptr, nullptr);
    if (w) { b2.c[BUF_AUX] = nullptr; b2.re[BUF_AUX] = (rl*)(w + o); }
    e = run_program(f.second, b2, loss, st);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

const Program& batch_program(BatchPlan* B, int which) { return which == 0 ? B->fwd : (which == 1 ? B->inv : B->cot); }
i64 batch_ws(BatchPlan* B) { return B->ws_elems; }
i64 batch_total(BatchPlan* B) {
  i64 t = 0;
  for (i64 v : B->ns) t += v;
  return t;
}
const void* batch_res(BatchPlan* B) { return &B->res; }

i64 batch_launches(BatchPlan* B) {
  i64 n = (i64)B->fwd.launches.size();
  for (auto& f : B->fb_fwd) n += (i64)f.second.launches.size();
  return n;
}

}  // namespace af
