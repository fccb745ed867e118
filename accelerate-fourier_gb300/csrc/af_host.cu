// af_host.cu -- libaf's plan objects: resources (FP64-generated tables),
// lowering of a reference plan tree to a program of tile / map launches, and
// execution.  The C ABI lives in af_api.cu.
#include "af_host.h"

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>

namespace af {

typedef std::complex<double> cd;

// ============================================================ host FP64 FFT
// Used once per plan for the Rader kernel spectrum and the Bluestein chirp
// spectrum, whose inputs are generated on the device in FP64.
static int smallest_factor(i64 n) {
  for (i64 p = 2; p * p <= n && p <= 64; ++p)
    if (n % p == 0) return (int)p;
  return n <= 64 ? (int)n : 0;
}

static void fft64(const cd* x, i64 xs, cd* y, i64 n, int sign);

static void bluestein64(const cd* x, i64 xs, cd* y, i64 n, int sign) {
  const i64 M = ceiling_power_of_two(2 * n - 1);
  std::vector<cd> ch(n), a(M, 0.0), b(M, 0.0), A(M), B(M), C(M);
  for (i64 k = 0; k < n; ++k) {
    const unsigned long long r = (unsigned long long)((__int128)k * k % (2 * n));
    const double ang = M_PI * (double)r / (double)n;
    ch[k] = cd(std::cos(ang), sign * std::sin(ang));
  }
  for (i64 k = 0; k < n; ++k) a[k] = ch[k] * x[k * xs];
  for (i64 k = 0; k < n; ++k) {
    b[k] = std::conj(ch[k]);
    if (k) b[M - k] = std::conj(ch[k]);
  }
  fft64(a.data(), 1, A.data(), M, -1);
  fft64(b.data(), 1, B.data(), M, -1);
  for (i64 i = 0; i < M; ++i) A[i] *= B[i];
  fft64(A.data(), 1, C.data(), M, 1);
  for (i64 k = 0; k < n; ++k) y[k] = ch[k] * C[k] / (double)M;
}

static void fft64(const cd* x, i64 xs, cd* y, i64 n, int sign) {
  if (n == 1) { y[0] = x[0]; return; }
  const int r = smallest_factor(n);
  if (r == 0) { bluestein64(x, xs, y, n, sign); return; }
  const i64 m = n / r;
  std::vector<cd> sub(n);
  for (int s = 0; s < r; ++s) fft64(x + s * xs, xs * r, sub.data() + s * m, m, sign);
  std::vector<cd> w(n);
  for (i64 t = 0; t < n; ++t) {
    const double ang = 2.0 * M_PI * (double)t / (double)n;
    w[t] = cd(std::cos(ang), sign * std::sin(ang));
  }
  for (i64 k = 0; k < m; ++k)
    for (int q = 0; q < r; ++q) {
      cd acc = 0;
      const i64 kk = k + q * m;
      for (int s = 0; s < r; ++s) acc += sub[s * m + k] * w[(i64)((__int128)s * kk % n)];
      y[kk] = acc;
    }
}

// ============================================================ resources
void PlanRes::release() {
  for (void* p : allocs) cudaFree(p);
  allocs.clear();
  tables.clear();
  pair_tables.clear();
  rader.clear();
  chirps.clear();
}

void* PlanRes::dalloc(size_t bytes) {
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
  t.p = (float2*)dalloc(sizeof(float2) * t.len);
  cuda_check(launch_twiddle_table(t.p, n, (int)S, t.H, 0), "twiddle table");
  tables[n] = t;
  return t;
}

const float2* PlanRes::pair_table(i64 a, i64 b, int* off_b) {
  auto key = std::make_pair(a, b);
  TwTable ta = table(a), tb = table(b);
  *off_b = ta.len;
  auto it = pair_tables.find(key);
  if (it != pair_tables.end()) return it->second;
  float2* p = (float2*)dalloc(sizeof(float2) * (ta.len + tb.len));
  cuda_check(cudaMemcpy(p, ta.p, sizeof(float2) * ta.len, cudaMemcpyDeviceToDevice), "table copy");
  cuda_check(cudaMemcpy(p + ta.len, tb.p, sizeof(float2) * tb.len, cudaMemcpyDeviceToDevice), "table copy");
  pair_tables[key] = p;
  return p;
}

static std::vector<float2> to_f32(const std::vector<cd>& v) {
  std::vector<float2> o(v.size());
  for (size_t i = 0; i < v.size(); ++i) o[i] = make_float2((float)v[i].real(), (float)v[i].imag());
  return o;
}

// Planned.hs:650-664 levelCachePrime: permutations and the kernel spectrum
// zs = scaleDown (inverse-direction transform of kernel), kernel[i] = W^(g^i).
const RaderRes& PlanRes::rader_res(i64 p, int sign) {
  auto key = std::make_pair(p, sign);
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
  for (i64 q = 0; q < m; ++q) src[q] = (int)(1 + perm[(m - q) % m]);  // 1 + reverse perm (75-80)
  for (i64 k = 0; k < m; ++k) inv[k] = dlog[k];                       // inverse perm (68-73)
  r.dlog = (int*)dalloc(sizeof(int) * m);
  r.src = (int*)dalloc(sizeof(int) * m);
  r.inv = (int*)dalloc(sizeof(int) * m);
  cuda_check(cudaMemcpy(r.dlog, dlog.data(), sizeof(int) * m, cudaMemcpyHostToDevice), "rader tables");
  cuda_check(cudaMemcpy(r.src, src.data(), sizeof(int) * m, cudaMemcpyHostToDevice), "rader tables");
  cuda_check(cudaMemcpy(r.inv, inv.data(), sizeof(int) * m, cudaMemcpyHostToDevice), "rader tables");
  // kernel in FP64 on the device, spectrum in FP64 on the host
  double2* dk = nullptr;
  cuda_check(cudaMalloc(&dk, sizeof(double2) * m), "rader kernel");
  cudaError_t e = launch_rader_kernel(dk, p, r.g, sign, 0);
  std::vector<cd> kern(m), spec(m);
  if (e == cudaSuccess) e = cudaMemcpy(kern.data(), dk, sizeof(double2) * m, cudaMemcpyDeviceToHost);
  cudaFree(dk);
  cuda_check(e, "rader kernel");
  fft64(kern.data(), 1, spec.data(), m, +1);
  for (auto& v : spec) v /= (double)m;
  std::vector<float2> zs = to_f32(spec);
  r.zs = (float2*)dalloc(sizeof(float2) * m);
  cuda_check(cudaMemcpy(r.zs, zs.data(), sizeof(float2) * m, cudaMemcpyHostToDevice), "rader spectrum");
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
  double2* dc = nullptr;
  cuda_check(cudaMalloc(&dc, sizeof(double2) * pad), "chirp");
  cudaError_t e = launch_chirp(dc, pad, len, sign, pad, 0);
  std::vector<cd> ch(pad), cj(pad), spec(pad);
  if (e == cudaSuccess) e = cudaMemcpy(ch.data(), dc, sizeof(double2) * pad, cudaMemcpyDeviceToHost);
  cudaFree(dc);
  cuda_check(e, "chirp");
  for (i64 i = 0; i < pad; ++i) cj[i] = std::conj(ch[i]);
  fft64(cj.data(), 1, spec.data(), pad, +1);
  for (auto& v : spec) v /= (double)pad;
  std::vector<cd> head(ch.begin(), ch.begin() + len);
  std::vector<float2> hf = to_f32(head), sf = to_f32(spec);
  c.chirp = (float2*)dalloc(sizeof(float2) * len);
  c.spec = (float2*)dalloc(sizeof(float2) * pad);
  cuda_check(cudaMemcpy(c.chirp, hf.data(), sizeof(float2) * len, cudaMemcpyHostToDevice), "chirp");
  cuda_check(cudaMemcpy(c.spec, sf.data(), sizeof(float2) * pad, cudaMemcpyHostToDevice), "chirp");
  chirps[key] = c;
  return chirps[key];
}

// ============================================================ tile building
// elements per CTA the ping-pong tile can hold (two padded buffers + tables)
static const i64 kTileCap = 13000;

static std::vector<int> radices(i64 n) {
  std::vector<int> r;
  int a = 0;
  while (n % 2 == 0) { n /= 2; ++a; }
  while (a >= 4) { r.push_back(16); a -= 4; }
  if (a == 3) r.push_back(8);
  else if (a == 2) r.push_back(4);
  else if (a == 1) r.push_back(2);
  for (int p : {3, 5, 7, 11, 13})
    while (n % p == 0) { r.push_back(p); n /= p; }
  return r;
}

bool tile_ok(i64 n) { return n >= 1 && n <= kTileCap && is_13smooth(n); }

static void fill_phase(FftPhase& ph, i64 n, float sign, int ls, int es, int lcnt, int tw_off, int S_log2) {
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
  io.s_e = v.s_e;
  io.s_lo = v.s_lo;
  io.s_hi = v.s_hi;
  io.lo_div = make_fastdiv((unsigned)std::min<i64>(v.lo_cnt, (i64)1 << 30));
  io.line_fast = v.s_e != 1 && v.s_lo == 1;
  return io;
}

// choose threads per CTA and lines per CTA (G) for a tile whose shared
// footprint per line is `slen` elements; want_wide asks for >= 16 lines so
// that strided (line-fast) global access moves whole sectors
static void choose_geometry(i64 slen, i64 lines, int tw_total, bool want_wide, int* threads, int* G) {
  const i64 budget = 227 * 1024 - (i64)sizeof(FftPhase) * AF_MAXPH - 8 * (i64)tw_total - 256;
  auto fits = [&](i64 g) { return 2 * 8 * (g * slen + ((g * slen) >> 4)) + 16 * g <= budget; };
  i64 g = std::max<i64>(1, 4096 / std::max<i64>(slen, 1));
  if (want_wide) g = std::max<i64>(g, 16);
  g = std::min(g, std::max<i64>(lines, 1));
  while (g > 1 && !fits(g)) --g;
  if (!fits(g)) throw AfError(AF_ERR_UNSUPPORTED, "transform does not fit a tile");
  *G = (int)g;
  const i64 elems = g * slen;
  *threads = elems >= 6144 ? 512 : (elems >= 1024 ? 256 : 128);
}

// ============================================================ lowering
struct Lowering {
  af_plan_s* P;
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

  void emit_tile(const TileDesc& td, int threads, const View& in, const View& out) {
    Step s;
    s.type = STEP_TILE;
    s.td = td;
    s.threads = threads;
    s.vin = in;
    s.vout = out;
    prog->steps.push_back(s);
  }

  void emit_map(const MapDesc& md, const View& in, const View& out) {
    Step s;
    s.type = STEP_MAP;
    s.md = md;
    s.vin = in;
    s.vout = out;
    prog->steps.push_back(s);
  }

  MapDesc map0(int mode, i64 lines, i64 nout) {
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

  // plain tile: FFT of length n over `lines` lines with optional four-step twiddle
  void plain_tile(i64 n, float sign, i64 lines, const View& in, const View& out, i64 ptwN = 0,
                  float scale = 1.f) {
    TileDesc td;
    memset(&td, 0, sizeof td);
    td.kind = TILE_PLAIN;
    td.nlen = (int)n;
    td.nlines = (int)lines;
    td.slen = (int)n;
    td.LS = (int)n;
    TwTable t = P->res.table(n);
    td.tw_src = t.p;
    td.tw_total = t.len;
    fill_phase(td.ph[0], n, sign, (int)n, 1, 1, 0, t.S_log2);
    td.nph = 1;
    td.in = io_of(in);
    td.out = io_of(out);
    td.scale = scale;
    if (ptwN) {
      TwTable pt = P->res.table(ptwN);
      td.ptw = pt.p;
      td.ptwS_log2 = pt.S_log2;
      td.ptwN = ptwN;
      td.ptw_col_mul = 1;
      td.ptw_sign = sign;
    }
    int threads, G;
    choose_geometry(n, lines, td.tw_total, td.in.line_fast || td.out.line_fast, &threads, &G);
    td.G = G;
    td.N_div = make_fastdiv((unsigned)n);
    td.S_div = td.N_div;
    td.G_div = make_fastdiv((unsigned)G);
    emit_tile(td, threads, in, out);
  }

  bool gt_tile_ok(const Node* nd) {
    return nd->kind == N_COPRIME && nd->n <= kTileCap && tile_ok(nd->a->n) && tile_ok(nd->b->n);
  }
  bool rader_tile_ok(const Node* nd) { return nd->kind == N_PRIME && nd->n > 13 && tile_ok(nd->n - 1); }
  bool chirp_tile_ok(const Node* nd) { return nd->kind == N_CHIRP && tile_ok(nd->a->n); }

  // Good-Thomas tile (Planned.hs:584-617): grid m x n, n = first factor
  void gt_tile(const Node* nd, float sign, i64 lines, const View& in, const View& out) {
    const i64 n = nd->a->n, m = nd->b->n, N = nd->n;
    TileDesc td;
    memset(&td, 0, sizeof td);
    td.kind = TILE_GT;
    td.nlen = (int)N;
    td.nlines = (int)lines;
    td.slen = (int)N;
    td.LS = (int)N;
    int offb = 0;
    td.tw_src = P->res.pair_table(n, m, &offb);
    td.tw_total = P->res.table(n).len + P->res.table(m).len;
    fill_phase(td.ph[0], n, sign, (int)n, 1, (int)m, 0, P->res.table(n).S_log2);       // rows (j)
    fill_phase(td.ph[1], m, sign, 1, (int)n, (int)n, offb, P->res.table(m).S_log2);    // cols (k)
    td.nph = 2;
    td.gt_n = (int)n;
    td.gt_m = (int)m;
    // i = (n k + m j) mod N  =>  k = i * n^-1 mod m,  j = i * m^-1 mod n
    td.gt_cm = mod_inverse(n % m, m);
    td.gt_cn = mod_inverse(m % n, n);
    td.in = io_of(in);
    td.out = io_of(out);
    td.in.line_fast = 0;
    td.out.line_fast = 0;
    td.scale = 1.f;
    int threads, G;
    choose_geometry(N, lines, td.tw_total, false, &threads, &G);
    td.G = G;
    td.N_div = make_fastdiv((unsigned)N);
    td.S_div = td.N_div;
    td.G_div = make_fastdiv((unsigned)G);
    emit_tile(td, threads, in, out);
  }

  static i64 mod_inverse(i64 a, i64 m) {
    if (m == 1) return 0;
    // extended Euclid
    i64 t = 0, nt = 1, r = m, nr = a % m;
    while (nr) {
      i64 q = r / nr;
      i64 tmp = t - q * nt; t = nt; nt = tmp;
      tmp = r - q * nr; r = nr; nr = tmp;
    }
    return t < 0 ? t + m : t;
  }

  // Rader tile (Planned.hs:646-692)
  void rader_tile(const Node* nd, float sign, i64 lines, const View& in, const View& out) {
    const i64 p = nd->n, m = p - 1;
    const RaderRes& rr = P->res.rader_res(p, sign > 0 ? 1 : -1);
    TileDesc td;
    memset(&td, 0, sizeof td);
    td.kind = TILE_RADER;
    td.nlen = (int)p;
    td.nlines = (int)lines;
    td.slen = (int)m;
    td.LS = (int)m;
    TwTable t = P->res.table(m);
    td.tw_src = t.p;
    td.tw_total = t.len;
    fill_phase(td.ph[0], m, +1.f, (int)m, 1, 1, 0, t.S_log2);
    fill_phase(td.ph[1], m, -1.f, (int)m, 1, 1, 0, t.S_log2);
    td.nph = 2;
    td.dlog = rr.dlog;
    td.vec_b = rr.zs;
    td.in = io_of(in);
    td.out = io_of(out);
    td.in.line_fast = 0;
    td.out.line_fast = 0;
    td.scale = 1.f;
    int threads, G;
    choose_geometry(m, lines, td.tw_total, false, &threads, &G);
    td.G = G;
    td.N_div = make_fastdiv((unsigned)p);
    td.S_div = make_fastdiv((unsigned)m);
    td.G_div = make_fastdiv((unsigned)G);
    emit_tile(td, threads, in, out);
  }

  // Bluestein tile (Planned.hs:760-773)
  void chirp_tile(const Node* nd, float sign, i64 lines, const View& in, const View& out) {
    const i64 N = nd->n, M = nd->a->n;
    const ChirpRes& cr = P->res.chirp_res(N, M, sign > 0 ? 1 : -1);
    TileDesc td;
    memset(&td, 0, sizeof td);
    td.kind = TILE_BLUESTEIN;
    td.nlen = (int)N;
    td.nlines = (int)lines;
    td.slen = (int)M;
    td.LS = (int)M;
    TwTable t = P->res.table(M);
    td.tw_src = t.p;
    td.tw_total = t.len;
    fill_phase(td.ph[0], M, +1.f, (int)M, 1, 1, 0, t.S_log2);
    fill_phase(td.ph[1], M, -1.f, (int)M, 1, 1, 0, t.S_log2);
    td.nph = 2;
    td.vec_a = cr.chirp;
    td.vec_b = cr.spec;
    td.in = io_of(in);
    td.out = io_of(out);
    td.in.line_fast = 0;
    td.out.line_fast = 0;
    td.scale = 1.f;
    int threads, G;
    choose_geometry(M, lines, td.tw_total, false, &threads, &G);
    td.G = G;
    td.N_div = make_fastdiv((unsigned)N);
    td.S_div = make_fastdiv((unsigned)M);
    td.G_div = make_fastdiv((unsigned)G);
    emit_tile(td, threads, in, out);
  }

  bool tileable(const Node* nd) {
    if (nd->n <= 1) return true;
    if (gt_tile_ok(nd) || rader_tile_ok(nd) || chirp_tile_ok(nd)) return true;
    return tile_ok(nd->n) && nd->kind != N_CHIRP && !(nd->kind == N_PRIME && nd->n > 13);
  }

  // ---------------------------------------------------------------- node
  // Transform `lines` rows through any 2-level views.
  void node(const Node* nd, float sign, i64 lines, const View& in, const View& out) {
    const i64 n = nd->n;
    if (n == 0 || lines == 0) return;
    if (n == 1) {
      MapDesc md = map0(MAP_COPY, lines, 1);
      emit_map(md, in, out);
      return;
    }
    if (gt_tile_ok(nd)) { gt_tile(nd, sign, lines, in, out); return; }
    if (rader_tile_ok(nd)) { rader_tile(nd, sign, lines, in, out); return; }
    if (chirp_tile_ok(nd)) { chirp_tile(nd, sign, lines, in, out); return; }
    if (tile_ok(n) && nd->kind != N_CHIRP && !(nd->kind == N_PRIME && n > 13)) {
      plain_tile(n, sign, lines, in, out);
      return;
    }
    // multi-launch structures need single-level views; route others via temps
    if (!simple(in, lines) || !simple(out, lines)) {
      const i64 mark = top;
      View tin = in, tout = out;
      if (!simple(in, lines)) {
        tin = View::rows(BUF_WS, alloc(lines * n), n, lines);
        MapDesc md = map0(MAP_COPY, lines, n);
        emit_map(md, in, tin);
      }
      if (!simple(out, lines)) tout = View::rows(BUF_WS, alloc(lines * n), n, lines);
      node(nd, sign, lines, tin, tout);
      if (!simple(out, lines)) {
        MapDesc md = map0(MAP_COPY, lines, n);
        emit_map(md, tout, out);
      }
      top = mark;
      return;
    }
    switch (nd->kind) {
      case N_COPRIME: good_thomas(nd, sign, lines, in, out); return;
      case N_PRIME: rader_multi(nd, sign, lines, in, out); return;
      case N_CHIRP: bluestein_multi(nd, sign, lines, in, out); return;
      default: four_step(nd, sign, lines, in, out); return;
    }
  }

  // Cooley-Tukey four-step for SR chains and composite nodes:
  // n = n1 * n2, x[n2 j1 + j2]; pass A: FFT_n1 over j1 (+ twiddle W_n^(j2 k1));
  // pass B: FFT_n2 over j2; X[k1 + n1 k2].  (Planned.hs:490-557)
  void four_step(const Node* nd, float sign, i64 lines, const View& in, const View& out) {
    const i64 n = nd->n;
    i64 n1;
    const Node* sub2;
    if (nd->kind == N_SR) {
      int a = 0;
      const Node* c = nd;
      std::vector<const Node*> chain;
      while (c->kind == N_SR) { chain.push_back(c); c = c->a; ++a; }
      const int lg = ceil_log2(n);
      int k = (lg + 1) / 2;
      k = std::max(k, ceil_log2((n + kTileCap - 1) / kTileCap));
      k = std::min(k, std::min(a, 10));
      k = std::max(k, 1);
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
    // pass A
    View a_in;
    a_in.buf = in.buf; a_in.off = in.off;
    a_in.s_e = n2 * in.s_e; a_in.s_lo = in.s_e; a_in.s_hi = in.s_lo; a_in.lo_cnt = n2;
    View a_out;
    a_out.buf = BUF_WS; a_out.off = W;
    a_out.s_e = n2; a_out.s_lo = 1; a_out.s_hi = n; a_out.lo_cnt = n2;
    if (tile_ok(n1)) {
      plain_tile(n1, sign, lines * n2, a_in, a_out, n);
    } else {
      // columns that need a multi-launch transform: transpose, transform, twiddle
      const i64 T1 = alloc(lines * n), T2 = alloc(lines * n);
      View trows = View::rows(BUF_WS, T1, n1, lines * n2);
      MapDesc cp = map0(MAP_COPY, lines * n2, n1);
      emit_map(cp, a_in, trows);
      View t2rows = View::rows(BUF_WS, T2, n1, lines * n2);
      node(nd->a, sign, lines * n2, trows, t2rows);
      MapDesc tw = map0(MAP_MUL, lines * n2, n1);
      tw.vec = nullptr;
      tw.n = n;
      tw.m = n2;  // column = line % n2
      tw.mode = MAP_TWIDDLE;
      TwTable pt = P->res.table(n);
      tw.tab_tw = pt.p;
      tw.tw_log2 = pt.S_log2;
      tw.tw_sign = sign;
      emit_map(tw, t2rows, a_out);
    }
    // pass B: rows of W -> out[k1 + n1 k2]
    View b_in = View::rows(BUF_WS, W, n2, lines * n1);
    View b_out;
    b_out.buf = out.buf; b_out.off = out.off;
    b_out.s_e = n1 * out.s_e; b_out.s_lo = out.s_e; b_out.s_hi = out.s_lo; b_out.lo_cnt = n1;
    node(sub2, sign, lines * n1, b_in, b_out);
    top = mark;
  }

  // Good-Thomas through explicit CRT maps (Planned.hs:584-617)
  void good_thomas(const Node* nd, float sign, i64 lines, const View& in, const View& out) {
    const i64 n = nd->a->n, m = nd->b->n, N = nd->n;
    const i64 mark = top;
    const i64 W1 = alloc(lines * N), W2 = alloc(lines * N);
    View w1 = View::rows(BUF_WS, W1, N, lines);
    MapDesc g = map0(MAP_GT_IN, lines, N);
    g.n = n; g.m = m; g.nm = N;
    emit_map(g, in, w1);
    // FFT_n along rows of the m x n grid, stored transposed (n x m)
    View r_in = View::rows(BUF_WS, W1, n, lines * m);
    View r_out;
    r_out.buf = BUF_WS; r_out.off = W2;
    r_out.s_e = m; r_out.s_lo = 1; r_out.s_hi = N; r_out.lo_cnt = m;
    node(nd->a, sign, lines * m, r_in, r_out);
    // FFT_m along rows of the transposed grid
    View c_in = View::rows(BUF_WS, W2, m, lines * n);
    View c_out = View::rows(BUF_WS, W1, m, lines * n);
    node(nd->b, sign, lines * n, c_in, c_out);
    MapDesc s = map0(MAP_GT_OUT, lines, N);
    s.n = n; s.m = m; s.nm = N;
    emit_map(s, View::rows(BUF_WS, W1, N, lines), out);
    top = mark;
  }

  // Rader through explicit permutation maps (Planned.hs:646-692)
  void rader_multi(const Node* nd, float sign, i64 lines, const View& in, const View& out) {
    const i64 p = nd->n, m = p - 1;
    const RaderRes& rr = P->res.rader_res(p, sign > 0 ? 1 : -1);
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
  void bluestein_multi(const Node* nd, float sign, i64 lines, const View& in, const View& out) {
    const i64 N = nd->n, M = nd->a->n;
    const ChirpRes& cr = P->res.chirp_res(N, M, sign > 0 ? 1 : -1);
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

// ============================================================ plan object
void build_program(af_plan_s* P, const Node* root, float sign, i64 batch, Program* prog) {
  Lowering L{P, prog};
  prog->steps.clear();
  View in = View::rows(BUF_IN, 0, root->n, batch);
  View out = View::rows(BUF_OUT, 0, root->n, batch);
  L.node(root, sign, batch, in, out);
  prog->ws_elems = L.peak;
}

static IoDesc resolve(const View& v, const ExecBufs& b) {
  IoDesc io = io_of(v);
  switch (v.buf) {
    case BUF_IN:
      if (b.in_im) { io.re = (float*)b.in_re + v.off; io.im = (float*)b.in_im + v.off; }
      else io.c = (float2*)b.in_re + v.off;
      break;
    case BUF_OUT:
      if (b.out_im) { io.re = b.out_re + v.off; io.im = b.out_im + v.off; }
      else io.c = (float2*)b.out_re + v.off;
      break;
    default:
      io.c = b.ws + v.off;
      break;
  }
  return io;
}

cudaError_t run_program(const Program& prog, const ExecBufs& b, cudaStream_t st) {
  for (const Step& s : prog.steps) {
    cudaError_t e;
    if (s.type == STEP_TILE) {
      TileDesc td = s.td;
      const int lf_in = td.in.line_fast, lf_out = td.out.line_fast;
      td.in = resolve(s.vin, b);
      td.out = resolve(s.vout, b);
      td.in.line_fast = lf_in;
      td.out.line_fast = lf_out;
      e = launch_tile(td, s.threads, st);
    } else {
      MapDesc md = s.md;
      md.in = resolve(s.vin, b);
      md.out = resolve(s.vout, b);
      if (md.x0_ws >= 0) md.x0 = b.ws + md.x0_ws;
      if (md.dc_ws >= 0) md.dc = b.ws + md.dc_ws;
      e = launch_map(md, st);
    }
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace af
