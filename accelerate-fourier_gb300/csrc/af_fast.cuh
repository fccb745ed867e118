// af_fast.cuh -- the line-FFT engine of the batched executor (Complex Float).
//
// The building block is an FFT of length L over GL interleaved lines held in
// shared memory: element e of line l sits at e*GL + l.  A transform of
// length n = L*G is G such lines of its own natural order (x[e*G + l]), so a
// contiguous copy of x already has this layout; a CTA may hold Q transforms
// of one length (GL = Q*G lines).  Each Stockham pass (compile-time radix R)
// reads R elements of a pair of adjacent lines as 16-byte vectors, applies
// the pass twiddles W_{pR}^{k m} from a table in shared memory (one table
// serves both lines) and the radix-R DFT of each line, and writes the pair
// back.  The last pass writes line-major (line l at l*LS, LS odd), which both
// epilogues read without bank conflicts: along a line (consecutive elements)
// or across lines (stride LS).  A full transform ends with the radix-G pass
// across the G lines (twiddle W_n^(l k1), DFT_G), whose outputs are the
// natural-order spectrum X[k1 + L*l'].
//
// Everything below is __host__ __device__: the kernels run each phase once
// per thread with a barrier after it, and the host emulator (used by the CPU
// tests, with address sanitizer) runs the same phase for every thread index
// in turn.  The algorithm is the mixed-radix Cooley-Tukey FFT that the
// reference's split-radix and composite transforms compute
// (src/Data/Array/Accelerate/Fourier/Planned.hs:473-557); the Bluestein
// convolution follows Planned.hs:744-773.
#pragma once
#include "af_device.cuh"

namespace af {

#define AFF_MAXPASS 12

// One Stockham pass of a line FFT: butterfly b reads elements b + m*nb and
// writes q*p*R + k + m*p (k = b mod p, q = b div p) after the twiddles
// W_{pR}^(k m), read from tw + (m-1)*p + k.
// V: lines per unit of the pass (1 or 2, chosen so that the units spread
// evenly over the CTA's threads; 2 only when the line count is even).
struct FPass {
  int R, p, nb, tw;
  int plog;  // log2 p when p is a power of two, else -1
  int V;
  FastDiv pdiv;
};

// x / d for 0 <= x < 8192 from r = ceil(2^19 / d), 2 <= d: exact when
// d <= 64, since then x (r d - 2^19) < 8192 d <= 2^19, and for every power
// of two (r d = 2^19); x r < 2^31.  One multiply and one shift.
AF_HD int sdiv(int x, int r) { return (int)(((unsigned)x * (unsigned)r) >> 19); }
struct FLine {
  int L, npass, twn;  // length, passes, table entries
  FPass pass[AFF_MAXPASS];
};

// shared-memory element positions of the two layouts
AF_HD int ipos(int e, int line, int GL) { return e * GL + line; }
AF_HD int lpos(int e, int line, int LS) { return line * LS + e; }
// line-major stride: odd, so that a warp reading across lines hits distinct banks
AF_HD int line_stride(int L) { return L | 1; }

AF_HD cx ldcx(const cx* p) {
#ifdef __CUDA_ARCH__
  return __ldg(p);
#else
  return *p;
#endif
}
AF_HD float ldf(const float* p) {
#ifdef __CUDA_ARCH__
  return __ldg(p);
#else
  return *p;
#endif
}

// a * w (SIGN = -1) or a * conj(w) (SIGN = +1): tables hold forward roots
template <int SIGN>
AF_HD cx cmul_s(cx a, cx w) {
  if (SIGN < 0) return cmul(a, w);
  return make_cx(rfma(a.x, w.x, a.y * w.y), rfma(a.y, w.x, -a.x * w.y));
}

AF_HD cx conjc(cx a) { return make_cx(a.x, -a.y); }
// Bluestein spectrum entry k of M: the spectrum of the even chirp is even,
// so only entries 0..M/2 are stored
AF_HD cx spec_at(const cx* spec, int M, int k) { return ldcx(spec + (2 * k <= M ? k : M - k)); }

// What the last pass of a compile-time line does with its outputs.
// EPI_PLAIN: writes them line-major (stride L | 1).  EPI_SPEC (the first row
// FFT of a Bluestein row item): output e of line l becomes
// conj(y * spec[c0 + l + M1 e]) for l < cn, zero for the lines past cn, and
// is written interleaved (e GL + l), the layout the second row FFT reads, so
// that the spectrum product needs no pass of its own.
enum { EPI_PLAIN = 0, EPI_SPEC = 1 };
struct LineEpi {
  int mode;
  int c0, cn, M1, M;
  const cx* spec;
};

template <int V> struct FVec;
template <> struct FVec<1> {
  typedef float2 T;
  static AF_HD void get(const cx* p, cx* a) { a[0] = *p; }
  static AF_HD void put(cx* p, const cx* a) { *p = a[0]; }
};
template <> struct FVec<2> {
  typedef float4 T;
  static AF_HD void get(const cx* p, cx* a) {
    const float4 v = *reinterpret_cast<const float4*>(p);
    a[0] = make_cx(v.x, v.y);
    a[1] = make_cx(v.z, v.w);
  }
  static AF_HD void put(cx* p, const cx* a) {
    *reinterpret_cast<float4*>(p) = make_float4(a[0].x, a[0].y, a[1].x, a[1].y);
  }
};

// Pass twiddles of butterfly k: w[m] = W_{pR}^(k m), m = 1..R-1, stored
// m-major (entry (m-1) p + k) so that the lanes of a warp, which hold
// consecutive k, read consecutive entries
template <int R>
AF_HD void pass_twiddles(const cx* t, int k, int p, cx* w) {
#pragma unroll
  for (int m = 1; m < R; ++m) w[m] = t[(m - 1) * p + k];
}

// One unit of a Stockham pass: butterfly b of the V lines starting at `line`.
// LS == 0: interleaved output (GL lines); else line-major output with stride LS.
template <int R, int V, int SIGN>
AF_HD void fpass_unit(const cx* __restrict__ src, cx* __restrict__ dst, const FPass& ps, int b, int line, int GL,
                      int LS, const cx* __restrict__ tw) {
  cx a[V][R];
  const int ib = ipos(b, line, GL);
  const int istep = ps.nb * GL;
#pragma unroll
  for (int m = 0; m < R; ++m) {
    cx t[V];
    FVec<V>::get(src + ib + m * istep, t);
#pragma unroll
    for (int v = 0; v < V; ++v) a[v][m] = t[v];
  }
  const int q = ps.plog >= 0 ? b >> ps.plog : (int)fdiv((unsigned)b, ps.pdiv);
  const int k = b - q * ps.p;
  if (k > 0) {
    cx w[R];
    pass_twiddles<R>(tw + ps.tw, k, ps.p, w);
#pragma unroll
    for (int m = 1; m < R; ++m)
#pragma unroll
      for (int v = 0; v < V; ++v) a[v][m] = cmul_s<SIGN>(a[v][m], w[m]);
  }
#pragma unroll
  for (int v = 0; v < V; ++v) Dft<R>::run(a[v], (rl)SIGN, nullptr, 0, 0);
  const int oe = q * ps.p * R + k;
  if (LS == 0) {
    const int ob = ipos(oe, line, GL);
    const int ostep = ps.p * GL;
#pragma unroll
    for (int m = 0; m < R; ++m) {
      cx t[V];
#pragma unroll
      for (int v = 0; v < V; ++v) t[v] = a[v][m];
      FVec<V>::put(dst + ob + m * ostep, t);
    }
  } else {
#pragma unroll
    for (int v = 0; v < V; ++v)
#pragma unroll
      for (int m = 0; m < R; ++m) dst[lpos(oe + m * ps.p, line + v, LS)] = a[v][m];
  }
}

// All units of one pass for thread `tid` of T (GL lines, V lines per unit).
template <int R, int V, int SIGN>
AF_HD void fpass_thread(int tid, int T, const cx* src, cx* dst, const FPass& ps, int GL, int gr, int LS,
                        const cx* tw) {
  const int units = ps.nb * (GL / V);
  for (int u = tid; u < units; u += T) {
    const int b = sdiv(u * V, gr);  // unit u: butterfly b of lines (u mod GL/V) V ..
    const int line = u * V - b * GL;
    fpass_unit<R, V, SIGN>(src, dst, ps, b, line, GL, LS, tw);
  }
}

template <int V, int SIGN>
AF_HD void fpass_any(int tid, int T, const cx* src, cx* dst, const FPass& ps, int GL, int gr, int LS,
                     const cx* tw) {
  switch (ps.R) {
    case 2: fpass_thread<2, V, SIGN>(tid, T, src, dst, ps, GL, gr, LS, tw); break;
    case 3: fpass_thread<3, V, SIGN>(tid, T, src, dst, ps, GL, gr, LS, tw); break;
    case 4: fpass_thread<4, V, SIGN>(tid, T, src, dst, ps, GL, gr, LS, tw); break;
    case 5: fpass_thread<5, V, SIGN>(tid, T, src, dst, ps, GL, gr, LS, tw); break;
    case 8: fpass_thread<8, V, SIGN>(tid, T, src, dst, ps, GL, gr, LS, tw); break;
    default:  // 16: one line per unit (the planner never pairs lines at radix 16)
      if (V == 1) fpass_thread<16, 1, SIGN>(tid, T, src, dst, ps, GL, gr, LS, tw);
      break;
  }
}

// ------------------------------------------------------------ compile-time lines
// A line FFT whose length L and line count GL are template constants runs in
// two passes of radices R1 then R2 (L = R1 R2; radices above 8 are done in
// registers as composite butterflies, Cooley-Tukey inside the butterfly with
// constant roots), one line per unit above radix 8 and two lines per unit at
// 8 and below, the pass-2 twiddles W_L^(k m) m-major in shared memory, with
// every stride, loop bound and divisor known to the compiler.
// AFF_FIXED_LINES lists (L, GL, R1, R2): the lengths whose pairwise products
// serve as the Bluestein convolution lengths of the multi-pass scheme, GL the
// planner's line count for each under the default tuning (as many lines as
// fill a 4096-element item within the CTA's shared memory, at most 64; not
// only powers of two: two lines share a unit only when GL is even).
#define AFF_FIXED_LINES(X)                                                                                    \
  X(64, 64, 16, 4) X(80, 51, 16, 5) X(96, 42, 16, 6) X(100, 40, 10, 10) X(120, 34, 15, 8) X(128, 32, 16, 8) \
  X(144, 28, 16, 9) X(160, 25, 16, 10) X(180, 22, 15, 12) X(192, 21, 16, 12) X(200, 20, 20, 10)             \
  X(216, 18, 24, 9) X(240, 17, 16, 15) X(250, 16, 25, 10) X(256, 16, 16, 16) X(270, 15, 27, 10)              \
  X(288, 14, 32, 9) X(300, 13, 20, 15) X(320, 12, 16, 20) X(360, 11, 24, 15) X(384, 10, 32, 12) X(400, 10, 20, 20) \
  X(432, 9, 27, 16) X(480, 8, 32, 15) X(500, 7, 25, 20) X(512, 7, 32, 16)

struct CRadices {
  int n;
  int r[AFF_MAXPASS];
};
// the radices of a line: the listed pair for a compile-time line, else 16s,
// 8s, 5s, one 4, 3s, 2s
constexpr CRadices c_radices(int L, bool fixed = true) {
  if (fixed) {
#define AFF_FIXED_SPLIT(l, g, r1, r2) \
  if (L == l) return CRadices{2, {r1, r2}};
    AFF_FIXED_LINES(AFF_FIXED_SPLIT)
#undef AFF_FIXED_SPLIT
  }
  CRadices x{0, {}};
  int m = L;
  while (m % 16 == 0) { x.r[x.n++] = 16; m /= 16; }
  while (m % 8 == 0) { x.r[x.n++] = 8; m /= 8; }
  while (m % 5 == 0) { x.r[x.n++] = 5; m /= 5; }
  if (m % 4 == 0) { x.r[x.n++] = 4; m /= 4; }
  while (m % 3 == 0) { x.r[x.n++] = 3; m /= 3; }
  while (m % 2 == 0) { x.r[x.n++] = 2; m /= 2; }
  return x;
}
// span of the butterflies before pass j
constexpr int c_span(int L, int j) {
  int p = 1;
  for (int i = 0; i < j; ++i) p *= c_radices(L).r[i];
  return p;
}
// twiddle-table offset of pass j (each pass after the first: p (R-1) entries, even)
constexpr int c_twoff(int L, int j) {
  int t = 0;
  for (int i = 0; i < j; ++i) {
    const int p = c_span(L, i);
    if (p > 1) t += (p * (c_radices(L).r[i] - 1) + 1) & ~1;
  }
  return t;
}

// One unit of a compile-time pass (fpass_unit with constant P, NB, GL, LS).
template <int R, int V, int SIGN, int P, int NB, int GL, int LS>
AF_HD void cpass_unit(const cx* __restrict__ src, cx* __restrict__ dst, int b, int line, const cx* __restrict__ tw) {
  cx a[V][R];
  const int ib = b * GL + line;
#pragma unroll
  for (int m = 0; m < R; ++m) {
    cx t[V];
    FVec<V>::get(src + ib + m * (NB * GL), t);
#pragma unroll
    for (int v = 0; v < V; ++v) a[v][m] = t[v];
  }
  const int q = b / P;
  const int k = b - q * P;
  if (P > 1 && k > 0) {  // each twiddle applied as it is read (few live registers)
#pragma unroll
    for (int m = 1; m < R; ++m) {
      const cx w = tw[(m - 1) * P + k];
#pragma unroll
      for (int v = 0; v < V; ++v) a[v][m] = cmul_s<SIGN>(a[v][m], w);
    }
  }
#pragma unroll
  for (int v = 0; v < V; ++v) Dft<R>::run(a[v], (rl)SIGN, nullptr, 0, 0);
  const int oe = q * P * R + k;
  if (LS == 0) {
    const int ob = oe * GL + line;
#pragma unroll
    for (int m = 0; m < R; ++m) {
      cx t[V];
#pragma unroll
      for (int v = 0; v < V; ++v) t[v] = a[v][m];
      FVec<V>::put(dst + ob + m * (P * GL), t);
    }
  } else {
#pragma unroll
    for (int v = 0; v < V; ++v)
#pragma unroll
      for (int m = 0; m < R; ++m) dst[(line + v) * LS + oe + m * P] = a[v][m];
  }
}

// The last pass of a compile-time line with the EPI_SPEC epilogue (the last
// pass has P = NB, so butterfly b is k = b and its outputs are e = k + m P).
template <int R, int V, int SIGN, int P, int NB, int GL>
AF_HD void cpass_unit_spec(const cx* __restrict__ src, cx* __restrict__ dst, int b, int line,
                           const cx* __restrict__ tw, const LineEpi& ep) {
  static_assert(P == NB, "the spectrum epilogue belongs to the last pass");
  cx a[V][R];
  const int ib = b * GL + line;
#pragma unroll
  for (int m = 0; m < R; ++m) {
    cx t[V];
    FVec<V>::get(src + ib + m * (NB * GL), t);
#pragma unroll
    for (int v = 0; v < V; ++v) a[v][m] = t[v];
  }
  if (P > 1 && b > 0) {
#pragma unroll
    for (int m = 1; m < R; ++m) {
      const cx w = tw[(m - 1) * P + b];
#pragma unroll
      for (int v = 0; v < V; ++v) a[v][m] = cmul_s<SIGN>(a[v][m], w);
    }
  }
#pragma unroll
  for (int v = 0; v < V; ++v) Dft<R>::run(a[v], (rl)SIGN, nullptr, 0, 0);
#pragma unroll
  for (int m = 0; m < R; ++m) {
    const int e = b + m * P;
    cx t[V];
#pragma unroll
    for (int v = 0; v < V; ++v) {
      const int l = line + v;
      t[v] = l < ep.cn ? conjc(cmul_s<SIGN>(a[v][m], spec_at(ep.spec, ep.M, ep.c0 + l + ep.M1 * e)))
                       : make_cx(0.f, 0.f);
    }
    FVec<V>::put(dst + e * GL + line, t);
  }
}

template <int T, int R, int V, int SIGN, int P, int NB, int GL, int LS>
AF_HD void cpass_thread(int tid, const cx* src, cx* dst, const cx* tw) {
  constexpr int per = GL / V, units = NB * per;
  for (int u = tid; u < units; u += T) cpass_unit<R, V, SIGN, P, NB, GL, LS>(src, dst, u / per, (u % per) * V, tw);
}

// Passes J.. of the compile-time line (L, GL); src and dst swap after each;
// the last pass ends with the epilogue `ep`.
#pragma nv_exec_check_disable
template <int T, int SIGN, int L, int GL, int J, class E>
AF_HD void cline_passes(E& ex, cx*& src, cx*& dst, const cx* tw, const LineEpi& ep) {
  constexpr CRadices rs = c_radices(L);
  if constexpr (J < rs.n) {
    constexpr int R = rs.r[J], P = c_span(L, J), NB = L / R;
    constexpr int V = (GL % 2 == 0 && R <= 8) ? 2 : 1;
    constexpr bool LAST = J == rs.n - 1;
    constexpr int LSo = LAST ? (L | 1) : 0;
    constexpr int TW = c_twoff(L, J);
    cx* s = src;
    cx* d = dst;
    if constexpr (LAST) {
      if (ep.mode == EPI_SPEC) {
        ex.phase([&](int tid) {
          constexpr int per = GL / V, units = NB * per;
          for (int u = tid; u < units; u += T)
            cpass_unit_spec<R, V, SIGN, P, NB, GL>(s, d, u / per, (u % per) * V, tw + TW, ep);
        });
      } else {
        ex.phase([&](int tid) { cpass_thread<T, R, V, SIGN, P, NB, GL, LSo>(tid, s, d, tw + TW); });
      }
    } else {
      ex.phase([&](int tid) { cpass_thread<T, R, V, SIGN, P, NB, GL, LSo>(tid, s, d, tw + TW); });
    }
    src = d;
    dst = s;
    cline_passes<T, SIGN, L, GL, J + 1>(ex, src, dst, tw, ep);
  }
}

// w^l for l < G from w (at most three products deep for G <= 16)
template <int G>
AF_HD void powers(cx w, cx* p) {
  p[0] = make_cx(1.f, 0.f);
  if (G > 1) p[1] = w;
#pragma unroll
  for (int l = 2; l < G; ++l) {
    const int h = l / 2;
    p[l] = cmul(p[h], p[l - h]);
  }
}

// The radix-G pass across the G lines of one transform: inputs a[l] =
// element k1 of line l; outputs natural-order bins k1 + L1*l'.
template <int G, int SIGN>
AF_HD void final_radix(cx* a, cx w) {
  if constexpr (G > 1) {
    cx p[G];
    powers<G>(w, p);
#pragma unroll
    for (int l = 1; l < G; ++l) a[l] = cmul_s<SIGN>(a[l], p[l]);
    Dft<G>::run(a, (rl)SIGN, nullptr, 0, 0);
  }
}

}  // namespace af
