// af_device.cuh -- device-side building blocks of libaf: descriptors shared by
// host and device, complex arithmetic, fast integer division, twiddle lookup
// and the radix-R butterflies used by the shared-memory Stockham engine.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define AF_MAXP 14      // max Stockham passes per FFT phase
#define AF_MAXPH 2      // max FFT phases in one tile program
#define AF_HD __host__ __device__ __forceinline__

// Element precision of the engine.  The engine (descriptors, kernels,
// lowering, executor) compiles twice: Complex Float in namespace af, and with
// AF_F64 defined, Complex Double in namespace af64.  The reference transforms
// are polymorphic over the element type (A.RealFloat a,
// src/Data/Array/Accelerate/Fourier/Planned.hs:103-106).
#ifdef AF_F64
#define AF_NS af64
#else
#define AF_NS af
#endif

namespace af {}
namespace AF_NS {
#ifdef AF_F64
using namespace af;  // the planner and error types are shared by both precisions
#endif

#ifdef AF_F64
typedef double2 cx;
typedef double rl;
AF_HD cx make_cx(rl x, rl y) { return make_double2(x, y); }
AF_HD rl rfma(rl a, rl b, rl c) { return fma(a, b, c); }
#else
typedef float2 cx;
typedef float rl;
AF_HD cx make_cx(rl x, rl y) { return make_float2(x, y); }
AF_HD rl rfma(rl a, rl b, rl c) { return fmaf(a, b, c); }
#endif

typedef long long i64;

// ---------------------------------------------------------------- fast divide
// q = floor(x / d) for 0 <= x < 2^31 via a 32-bit magic multiply.
struct FastDiv {
  unsigned d, m, s;
};
static inline FastDiv make_fastdiv(unsigned d) {
  FastDiv f;
  f.d = d;
  if (d <= 1) { f.m = 0; f.s = 0; return f; }
  unsigned s = 0;
  while ((1ull << s) < d) ++s;
  f.s = s;
  f.m = (unsigned)(((1ull << 32) * ((1ull << s) - d)) / d + 1);
  return f;
}
__device__ __forceinline__ FastDiv make_fastdiv_dev(unsigned d) {
  FastDiv f;
  f.d = d;
  if (d <= 1) { f.m = 0; f.s = 0; return f; }
  const unsigned s = 32 - __clz(d - 1);  // ceil(log2 d)
  f.s = s;
  f.m = (unsigned)(((1ull << 32) * ((1ull << s) - d)) / d + 1);
  return f;
}
AF_HD unsigned umulhi32(unsigned a, unsigned b) {
#ifdef __CUDA_ARCH__
  return __umulhi(a, b);
#else
  return (unsigned)(((unsigned long long)a * b) >> 32);
#endif
}
AF_HD unsigned fdiv(unsigned x, const FastDiv& f) {
  return f.d <= 1 ? x : ((umulhi32(x, f.m) + x) >> f.s);
}

// (a * b) mod n for a, b < n < 2^31 without 64-bit division: rcp =
// floor((2^64-1)/n) gives a quotient estimate at most 2 below the true one.
struct ModN {
  unsigned long long rcp;
  unsigned n;
};
static inline ModN make_modn(unsigned long long n) {
  ModN m;
  m.n = (unsigned)n;
  m.rcp = n ? (~0ull) / n : 0;
  return m;
}
AF_HD unsigned long long umulhi64(unsigned long long a, unsigned long long b) {
#ifdef __CUDA_ARCH__
  return __umul64hi(a, b);
#else
  return (unsigned long long)(((unsigned __int128)a * b) >> 64);
#endif
}
AF_HD unsigned mod_of(unsigned long long x, const ModN& M) {
  const unsigned long long q = umulhi64(x, M.rcp);
  unsigned long long r = x - q * M.n;
#pragma unroll
  for (int k = 0; k < 2; ++k)
    if (r >= M.n) r -= M.n;
  return (unsigned)r;
}
AF_HD unsigned mulmod(unsigned a, unsigned b, const ModN& M) {
  return mod_of((unsigned long long)a * b, M);
}

// ---------------------------------------------------------------- complex ops
// Complex add and subtract use the packed two-lane FP32 add of sm_100+
// (one instruction for both parts) in FP32 device code.
AF_HD cx cadd(cx a, cx b) {
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000 && !defined(AF_F64)
  return __fadd2_rn(a, b);
#else
  return make_cx(a.x + b.x, a.y + b.y);
#endif
}
AF_HD cx csub(cx a, cx b) {
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000 && !defined(AF_F64)
  return __fadd2_rn(a, make_cx(-b.x, -b.y));
#else
  return make_cx(a.x - b.x, a.y - b.y);
#endif
}
AF_HD cx cmul(cx a, cx b) {
  return make_cx(rfma(a.x, b.x, -a.y * b.y), rfma(a.x, b.y, a.y * b.x));
}
AF_HD cx cscale(cx a, rl s) { return make_cx(a.x * s, a.y * s); }
AF_HD cx conjf2(cx a) { return make_cx(a.x, -a.y); }
// multiply by sign*i  (sign = +-1):  (sign*i)(x+iy) = sign*(-y + ix)
AF_HD cx mul_si(cx a, rl sign) { return make_cx(-sign * a.y, sign * a.x); }

// ---------------------------------------------------------------- descriptors
// One Stockham pass of radix R over a phase of length n: the pass reads
// element i + j*(n/R) and writes (i-k)*R + k + j*p with k = i mod p.
struct PassDesc {
  int R;
  int p;
  int tw_stride;   // n / (p*R): exponent step of the twiddle table for this pass
  FastDiv nb_div;  // n / R  (butterflies per line)
  FastDiv p_div;   // p
};

// One FFT phase: G transforms per CTA, each holding `lcnt` lines of length n.
// Line r of transform t starts at shared position t*LS + r*ls and its
// elements are es apart (positions before bank padding).
struct FftPhase {
  int n, npass, ls, es, lcnt;
  rl sign;
  int tw_off;      // offset of this phase's tables in the shared table area
  int twS_log2;    // two-level table split S = 1<<twS_log2 (lo table S, hi table H)
  FastDiv lcnt_div;
  PassDesc pass[AF_MAXP];
};

// Buffers a launch addresses: every IoDesc names one of them and the launch
// passes their base pointers (interleaved `c`, or planar `re`/`im` planes).
enum BufId { BUF_IN = 0, BUF_OUT = 1, BUF_WS = 2, BUF_AUX = 3, BUF_COUNT = 4 };
struct TileBases {
  cx* c[BUF_COUNT];
  rl* re[BUF_COUNT];
  rl* im[BUF_COUNT];
};

// Index maps of one side of a tile (element e of a line with lo index `lo`).
enum IoMap {
  IO_AFFINE = 0,  // hi*s_hi + lo*s_lo + e*s_e
  IO_GT = 1,      // hi*s_hi + ((mA*lo + mB*e) mod mN)*s_t   Good-Thomas CRT map
  IO_TABLE = 2,   // hi*s_hi + tab[q]*s_t, q = lo*q_lo + e*q_e (Rader gather)
  IO_CHIRP = 3,   // q < mN ? vec[q] * x[hi*s_hi + q*s_t] : 0 (load); vec[q]*v (store, q < mN)
  IO_RADER = 4    // store: out[tab[q]] = x0 + v; q == 0 also writes out[0] = x0 + dc
};

// Global-memory view of one side (input or output) of a tile program.
// A tile "line" l of a launch is split as hi = l / lo_count, lo = l % lo_count.
struct IoDesc {
  int buf;
  int map;
  int line_fast;    // 1: consecutive threads walk lines (strided element access)
  int x0_buf;       // IO_RADER: buffer holding the transform inputs (x0 = x[hi][0])
  i64 off;          // complex-unit offset into the buffer
  i64 s_e, s_lo, s_hi;
  FastDiv lo_div;
  i64 q_lo, q_e;    // logical index q = lo*q_lo + e*q_e
  i64 mA, mB, mN;   // GT map constants / logical length for IO_CHIRP
  ModN m_mod;       // IO_GT: reduction mod mN (constants mA, mB reduced mod mN)
  i64 s_t;          // element stride of a mapped transform
  const int* tab;
  const cx* vec;
  i64 x0_off, x0_shi;  // IO_RADER: x0 at x0_off + hi*x0_shi in buffer x0_buf
  i64 dc_off;          // IO_RADER: DC of transform hi at ws[dc_off + hi]
  const i64* loff;     // AFFINE views: when set, line l starts at loff[l] (gathered lines)
};

enum TileKind {
  TILE_PLAIN = 0,     // load -> FFT -> store (with the IoDesc maps)
  TILE_GT = 1,        // Good-Thomas: CRT load -> FFT_n rows -> FFT_m cols -> CRT store
  TILE_RADER = 2,     // Rader: dlog gather -> FFT(+1) -> *zs -> FFT(-1) -> dlog scatter + x0
  TILE_BLUESTEIN = 3, // Bluestein: chirp*x, pad -> FFT(+1) -> *spec -> FFT(-1) -> chirp*, take N
  TILE_CONVROW = 4    // four-step conv middle: row FFT(+1) -> *S[q] -> row FFT(-1) -> twiddle
};

struct TileDesc {
  int kind;
  int nlen;          // logical transform length N seen through in/out
  int G;             // lines per full CTA
  int nlines;        // total lines of the step (all CTAs)
  int LS;            // shared-memory stride between lines (unpadded units)
  int slen;          // elements per line held in shared memory (M for conv tiles)
  int tw_total;      // table entries staged in shared memory
  int nph;
  const cx* tw_src;  // table source (device)
  FftPhase ph[AF_MAXPH];
  FastDiv N_div, S_div, G_div;  // nlen, slen, G
  IoDesc in, out;
  rl scale;       // multiplies every stored element
  rl ptw_sign;
  // four-step twiddle on store: element e of a line with lo index c is
  // multiplied by W_N^(c*e) (two-level table: S lo entries then hi entries)
  const cx* ptw;
  int ptwS_log2;
  int cot;           // 1: store g = 2 w v (w read from BUF_AUX at the output
                     // address) and add w |v|^2 to the loss
  i64 ptwN;
  ModN ptw_mod;      // reduction mod ptwN
  // Good-Thomas tile grid m x n: logical input i sits at ((i*cm) mod m)*n + (i*cn) mod n
  int gt_n, gt_m;
  i64 gt_cm, gt_cn;
  ModN gt_m_mod, gt_n_mod;
  // Rader: dlog[r-1] = log_g(r) for r = 1..p-1
  const int* dlog;
  // Bluestein chirp (N entries); conv spectrum (Rader zs / chirp spectrum / S)
  const cx* vec_a;
  const cx* vec_b;
  // TILE_CONVROW: spectrum index q = lo*sq_lo + e*sq_e; DC of line lo == 0,
  // element 0 after the first FFT goes to ws[dc_off + hi] (dc_off < 0: none)
  i64 sq_lo, sq_e, dc_off;
  // x0 capture (first pass of a multi-pass Rader): x[hi][0] of the step's
  // input goes to ws[x0_cap + out_add + hi] (x0_cap < 0: none)
  i64 x0_cap;
  int pad_sh;        // shared-memory padding: one slot every 2^pad_sh elements
};

// One CTA's work in a launch: lines [line0, line0 + G) of descriptor `desc`;
// the *_add offsets shift the in/out/aux views (per-transform placement).
struct WorkItem {
  int desc;
  int line0;
  int G;
  int pad;
  i64 in_add, out_add, aux_add;
};

// ---------------------------------------------------------------- smem layout
// One padding slot every 2^sh elements keeps strided Stockham accesses off bank
// conflicts; each tile picks sh (sh = 31: no padding).
__device__ __forceinline__ int spd_(int i, int sh) { return i + (i >> sh); }

// ---------------------------------------------------------------- twiddles
// Tables hold the forward root: tab[t] = exp(-2*pi*i*t/n), as two levels
// lo[t & (S-1)] * hi[t >> log2 S].  sign > 0 conjugates.
__device__ __forceinline__ cx tw_lookup(const cx* tab, int S_log2, int t, rl sign) {
  cx lo = tab[t & ((1 << S_log2) - 1)];
  cx hi = tab[(1 << S_log2) + (t >> S_log2)];
  cx w = cmul(hi, lo);
  w.y *= -sign;  // forward (sign=-1) keeps the stored root
  return w;
}

// ---------------------------------------------------------------- butterflies
// In-register DFT of R points, y_k = sum_j u_j exp(sign*2*pi*i*j*k/R).
template <int R> struct Dft;

template <> struct Dft<2> {
  static AF_HD void run(cx* u, rl, const cx*, int, int) {
    cx a = u[0], b = u[1];
    u[0] = cadd(a, b);
    u[1] = csub(a, b);
  }
};

AF_HD void dft4(cx& u0, cx& u1, cx& u2, cx& u3, rl sign) {
  cx t0 = cadd(u0, u2), t1 = csub(u0, u2);
  cx t2 = cadd(u1, u3), t3 = mul_si(csub(u1, u3), sign);
  u0 = cadd(t0, t2);
  u2 = csub(t0, t2);
  u1 = cadd(t1, t3);
  u3 = csub(t1, t3);
}

template <> struct Dft<4> {
  static AF_HD void run(cx* u, rl sign, const cx*, int, int) {
    dft4(u[0], u[1], u[2], u[3], sign);
  }
};

#define AF_R2 ((rl)0.70710678118654752440)
#define AF_C8 ((rl)0.92387953251128675613)
#define AF_S8 ((rl)0.38268343236508977173)

// multiply by w8^m = exp(sign*2*pi*i*m/8)
AF_HD cx mul_w8(cx a, int m, rl sign) {
  switch (m & 7) {
    case 0: return a;
    case 1: return cmul(a, make_cx(AF_R2, sign * AF_R2));
    case 2: return mul_si(a, sign);
    case 3: return cmul(a, make_cx(-AF_R2, sign * AF_R2));
    case 4: return make_cx(-a.x, -a.y);
    case 5: return cmul(a, make_cx(-AF_R2, -sign * AF_R2));
    case 6: return mul_si(a, -sign);
    default: return cmul(a, make_cx(AF_R2, -sign * AF_R2));
  }
}

template <> struct Dft<8> {
  static AF_HD void run(cx* u, rl sign, const cx*, int, int) {
    cx a[4], b[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      a[j] = cadd(u[j], u[j + 4]);
      b[j] = mul_w8(csub(u[j], u[j + 4]), j, sign);
    }
    dft4(a[0], a[1], a[2], a[3], sign);
    dft4(b[0], b[1], b[2], b[3], sign);
#pragma unroll
    for (int k = 0; k < 4; ++k) { u[2 * k] = a[k]; u[2 * k + 1] = b[k]; }
  }
};

// multiply by w16^m, m in 0..9
AF_HD cx mul_w16(cx a, int m, rl sign) {
  switch (m) {
    case 0: return a;
    case 1: return cmul(a, make_cx(AF_C8, sign * AF_S8));
    case 2: return mul_w8(a, 1, sign);
    case 3: return cmul(a, make_cx(AF_S8, sign * AF_C8));
    case 4: return mul_w8(a, 2, sign);
    case 6: return mul_w8(a, 3, sign);
    case 9: return cmul(a, make_cx(-AF_C8, -sign * AF_S8));
    default: return a;  // unused
  }
}

template <> struct Dft<16> {
  static AF_HD void run(cx* u, rl sign, const cx*, int, int) {
    // 4 x 4: v_a = DFT4(u[a + 4m]); v_a[b] *= w16^(a b); y[b + 4c] = DFT4_a(v_a[b])
#pragma unroll
    for (int a = 0; a < 4; ++a) dft4(u[a], u[a + 4], u[a + 8], u[a + 12], sign);
#pragma unroll
    for (int a = 1; a < 4; ++a)
#pragma unroll
      for (int b = 1; b < 4; ++b) u[a + 4 * b] = mul_w16(u[a + 4 * b], a * b, sign);
    cx t[16];
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      cx x0 = u[0 + 4 * b], x1 = u[1 + 4 * b], x2 = u[2 + 4 * b], x3 = u[3 + 4 * b];
      dft4(x0, x1, x2, x3, sign);
      t[b] = x0; t[b + 4] = x1; t[b + 8] = x2; t[b + 12] = x3;
    }
#pragma unroll
    for (int i = 0; i < 16; ++i) u[i] = t[i];
  }
};

template <> struct Dft<3> {
  static AF_HD void run(cx* u, rl sign, const cx*, int, int) {
    const rl c = (rl)-0.5, s = (rl)0.86602540378443864676 * sign;
    cx t = cadd(u[1], u[2]);
    cx d = csub(u[1], u[2]);
    cx m = make_cx(rfma(c, t.x, u[0].x), rfma(c, t.y, u[0].y));
    cx r = make_cx(-s * d.y, s * d.x);
    u[0] = cadd(u[0], t);
    u[1] = cadd(m, r);
    u[2] = csub(m, r);
  }
};

template <> struct Dft<5> {
  static AF_HD void run(cx* u, rl sign, const cx*, int, int) {
    const rl c1 = (rl)0.30901699437494742410, c2 = (rl)-0.80901699437494742410;
    const rl s1 = (rl)0.95105651629515357212 * sign, s2 = (rl)0.58778525229247312917 * sign;
    cx p1 = cadd(u[1], u[4]), m1 = csub(u[1], u[4]);
    cx p2 = cadd(u[2], u[3]), m2 = csub(u[2], u[3]);
    cx a1 = make_cx(u[0].x + c1 * p1.x + c2 * p2.x, u[0].y + c1 * p1.y + c2 * p2.y);
    cx a2 = make_cx(u[0].x + c2 * p1.x + c1 * p2.x, u[0].y + c2 * p1.y + c1 * p2.y);
    // b = i*(s1 m1 + s2 m2), c = i*(s2 m1 - s1 m2)
    cx b1 = make_cx(-(s1 * m1.y + s2 * m2.y), s1 * m1.x + s2 * m2.x);
    cx b2 = make_cx(-(s2 * m1.y - s1 * m2.y), s2 * m1.x - s1 * m2.x);
    u[0] = cadd(u[0], cadd(p1, p2));
    u[1] = cadd(a1, b1);
    u[4] = csub(a1, b1);
    u[2] = cadd(a2, b2);
    u[3] = csub(a2, b2);
  }
};

// Odd prime radix (7, 11, 13): symmetric direct DFT with the constants
// cos(2 pi m/R), sin(2 pi m/R), m <= (R-1)/2 (computed in double precision
// and rounded to the element type).
template <int R> struct OddRoots;
template <> struct OddRoots<7> {
  static AF_HD rl c(int m) {
    constexpr rl v[4] = {1.0f, 0.62348980185873359439, -0.22252093395631433737, -0.90096886790241903498};
    return v[m];
  }
  static AF_HD rl s(int m) {
    constexpr rl v[4] = {0.0f, 0.78183148246802980363, 0.97492791218182361934, 0.43388373911755823142};
    return v[m];
  }
};
template <> struct OddRoots<11> {
  static AF_HD rl c(int m) {
    constexpr rl v[6] = {1.0f, 0.84125353283118120551, 0.41541501300188643508, -0.14231483827328500480,
                            -0.65486073394528498959, -0.95949297361449736865};
    return v[m];
  }
  static AF_HD rl s(int m) {
    constexpr rl v[6] = {0.0f, 0.54064081745559755543, 0.90963199535451833011, 0.98982144188093279524,
                            0.75574957435425826890, 0.28173255684142967104};
    return v[m];
  }
};
template <> struct OddRoots<13> {
  static AF_HD rl c(int m) {
    constexpr rl v[7] = {1.0f, 0.88545602565320991051, 0.56806474673115592289, 0.12053668025532300601,
                            -0.35460488704253545489, -0.74851074817110119231, -0.97094181742605201180};
    return v[m];
  }
  static AF_HD rl s(int m) {
    constexpr rl v[7] = {0.0f, 0.46472317204376850652, 0.82298386589365635224, 0.99270887409805397272,
                            0.93501624268541483342, 0.66312265824079519305, 0.23931566428755768339};
    return v[m];
  }
};

template <int R> struct DftOdd {
  static __device__ __forceinline__ void run(cx* u, rl sign, const cx*, int, int) {
    constexpr int h = (R - 1) / 2;
    cx P[h + 1], M[h + 1];
    cx y0 = u[0];
#pragma unroll
    for (int j = 1; j <= h; ++j) {
      P[j] = cadd(u[j], u[R - j]);
      M[j] = csub(u[j], u[R - j]);
      y0 = cadd(y0, P[j]);
    }
    cx out[R];
    out[0] = y0;
#pragma unroll
    for (int k = 1; k <= h; ++k) {
      cx a = u[0], b = make_cx(0.f, 0.f);
#pragma unroll
      for (int j = 1; j <= h; ++j) {
        // cos/sin of 2 pi (j k mod R)/R from the first half (symmetry)
        const int m = (j * k) % R;
        const rl cm = OddRoots<R>::c(m <= h ? m : R - m);
        const rl sm = m <= h ? OddRoots<R>::s(m) : -OddRoots<R>::s(R - m);
        a.x = rfma(cm, P[j].x, a.x);
        a.y = rfma(cm, P[j].y, a.y);
        b.x = rfma(sm, M[j].x, b.x);
        b.y = rfma(sm, M[j].y, b.y);
      }
      cx ib = mul_si(b, sign);
      out[k] = cadd(a, ib);
      out[R - k] = csub(a, ib);
    }
#pragma unroll
    for (int k = 0; k < R; ++k) u[k] = out[k];
  }
};
template <> struct Dft<7> : DftOdd<7> {};
template <> struct Dft<11> : DftOdd<11> {};
template <> struct Dft<13> : DftOdd<13> {};

// Roots of unity for the composite radices: Roots<R>::c(m) = cos(2 pi m/R),
// Roots<R>::s(m) = sin(2 pi m/R), m < R (computed in double precision and
// rounded to the element type).
template <int R> struct Roots;
template <> struct Roots<6> {
  static AF_HD rl c(int m) {
    constexpr rl v[6] = {1.00000000000000000000e+00, 5.00000000000000111022e-01, -4.99999999999999777955e-01, -1.00000000000000000000e+00, -5.00000000000000444089e-01, 5.00000000000000111022e-01};
    return v[m];
  }
  static AF_HD rl s(int m) {
    constexpr rl v[6] = {0.00000000000000000000e+00, 8.66025403784438596588e-01, 8.66025403784438707611e-01, 0.00000000000000000000e+00, -8.66025403784438374544e-01, -8.66025403784438596588e-01};
    return v[m];
  }
};
template <> struct Roots<9> {
  static AF_HD rl c(int m) {
    constexpr rl v[9] = {1.00000000000000000000e+00, 7.66044443118978013452e-01, 1.73648177666930414453e-01, -4.99999999999999777955e-01, -9.39692620785908316883e-01, -9.39692620785908427905e-01, -5.00000000000000444089e-01, 1.73648177666929970364e-01, 7.66044443118977791407e-01};
    return v[m];
  }
  static AF_HD rl s(int m) {
    constexpr rl v[9] = {0.00000000000000000000e+00, 6.42787609686539251896e-01, 9.84807753012208020316e-01, 8.66025403784438707611e-01, 3.42020143325668879442e-01, -3.42020143325668657397e-01, -8.66025403784438374544e-01, -9.84807753012208131338e-01, -6.42787609686539584963e-01};
    return v[m];
  }
};
template <> struct Roots<10> {
  static AF_HD rl c(int m) {
    constexpr rl v[10] = {1.00000000000000000000e+00, 8.09016994374947451263e-01, 3.09016994374947451263e-01, -3.09016994374947340241e-01, -8.09016994374947340241e-01, -1.00000000000000000000e+00, -8.09016994374947562285e-01, -3.09016994374947562285e-01, 3.09016994374947229218e-01, 8.09016994374947340241e-01};
    return v[m];
  }
  static AF_HD rl s(int m) {
    constexpr rl v[10] = {0.00000000000000000000e+00, 5.87785252292473137103e-01, 9.51056516295153531182e-01, 9.51056516295153642204e-01, 5.87785252292473248126e-01, 0.00000000000000000000e+00, -5.87785252292473026081e-01, -9.51056516295153531182e-01, -9.51056516295153642204e-01, -5.87785252292473359148e-01};
    return v[m];
  }
};
template <> struct Roots<12> {
  static AF_HD rl c(int m) {
    constexpr rl v[12] = {1.00000000000000000000e+00, 8.66025403784438707611e-01, 5.00000000000000111022e-01, 0.00000000000000000000e+00, -4.99999999999999777955e-01, -8.66025403784438707611e-01, -1.00000000000000000000e+00, -8.66025403784438818633e-01, -5.00000000000000444089e-01, 0.00000000000000000000e+00, 5.00000000000000111022e-01, 8.66025403784438374544e-01};
    return v[m];
  }
  static AF_HD rl s(int m) {
    constexpr rl v[12] = {0.00000000000000000000e+00, 4.99999999999999944489e-01, 8.66025403784438596588e-01, 1.00000000000000000000e+00, 8.66025403784438707611e-01, 4.99999999999999944489e-01, 0.00000000000000000000e+00, -4.99999999999999722444e-01, -8.66025403784438374544e-01, -1.00000000000000000000e+00, -8.66025403784438596588e-01, -5.00000000000000444089e-01};
    return v[m];
  }
};
template <> struct Roots<15> {
  static AF_HD rl c(int m) {
    constexpr rl v[15] = {1.00000000000000000000e+00, 9.13545457642600866599e-01, 6.69130606358858237570e-01, 3.09016994374947451263e-01, -1.04528463267653332069e-01, -4.99999999999999777955e-01, -8.09016994374947340241e-01, -9.78147600733805688833e-01, -9.78147600733805688833e-01, -8.09016994374947562285e-01, -5.00000000000000444089e-01, -1.04528463267654234126e-01, 3.09016994374947229218e-01, 6.69130606358858459615e-01, 9.13545457642600977621e-01};
    return v[m];
  }
  static AF_HD rl s(int m) {
    constexpr rl v[15] = {0.00000000000000000000e+00, 4.06736643075800152758e-01, 7.43144825477394133095e-01, 9.51056516295153531182e-01, 9.94521895368273400884e-01, 8.66025403784438707611e-01, 5.87785252292473248126e-01, 2.07911690817759314820e-01, -2.07911690817759065020e-01, -5.87785252292473026081e-01, -8.66025403784438374544e-01, -9.94521895368273289861e-01, -9.51056516295153642204e-01, -7.43144825477394022073e-01, -4.06736643075800152758e-01};
    return v[m];
  }
};
template <> struct Roots<20> {
  static AF_HD rl c(int m) {
    constexpr rl v[20] = {1.00000000000000000000e+00, 9.51056516295153531182e-01, 8.09016994374947451263e-01, 5.87785252292473137103e-01, 3.09016994374947451263e-01, 0.00000000000000000000e+00, -3.09016994374947340241e-01, -5.87785252292473026081e-01, -8.09016994374947340241e-01, -9.51056516295153531182e-01, -1.00000000000000000000e+00, -9.51056516295153753227e-01, -8.09016994374947562285e-01, -5.87785252292473248126e-01, -3.09016994374947562285e-01, 0.00000000000000000000e+00, 3.09016994374947229218e-01, 5.87785252292472915059e-01, 8.09016994374947340241e-01, 9.51056516295153531182e-01};
    return v[m];
  }
  static AF_HD rl s(int m) {
    constexpr rl v[20] = {0.00000000000000000000e+00, 3.09016994374947395752e-01, 5.87785252292473137103e-01, 8.09016994374947451263e-01, 9.51056516295153531182e-01, 1.00000000000000000000e+00, 9.51056516295153642204e-01, 8.09016994374947451263e-01, 5.87785252292473248126e-01, 3.09016994374947506774e-01, 0.00000000000000000000e+00, -3.09016994374946896151e-01, -5.87785252292473026081e-01, -8.09016994374947340241e-01, -9.51056516295153531182e-01, -1.00000000000000000000e+00, -9.51056516295153642204e-01, -8.09016994374947562285e-01, -5.87785252292473359148e-01, -3.09016994374947617796e-01};
    return v[m];
  }
};
template <> struct Roots<24> {
  static AF_HD rl c(int m) {
    constexpr rl v[24] = {1.00000000000000000000e+00, 9.65925826289068312214e-01, 8.66025403784438707611e-01, 7.07106781186547572737e-01, 5.00000000000000111022e-01, 2.58819045102520739476e-01, 6.12323399573676603587e-17, -2.58819045102520628454e-01, -4.99999999999999777955e-01, -7.07106781186547461715e-01, -8.66025403784438707611e-01, -9.65925826289068201191e-01, -1.00000000000000000000e+00, -9.65925826289068312214e-01, -8.66025403784438818633e-01, -7.07106781186547905804e-01, -5.00000000000000444089e-01, -2.58819045102520628454e-01, -1.83697019872102968750e-16, 2.58819045102520295387e-01, 5.00000000000000111022e-01, 7.07106781186547350693e-01, 8.66025403784438374544e-01, 9.65925826289068090169e-01};
    return v[m];
  }
  static AF_HD rl s(int m) {
    constexpr rl v[24] = {0.00000000000000000000e+00, 2.58819045102520739476e-01, 4.99999999999999944489e-01, 7.07106781186547461715e-01, 8.66025403784438596588e-01, 9.65925826289068312214e-01, 1.00000000000000000000e+00, 9.65925826289068312214e-01, 8.66025403784438707611e-01, 7.07106781186547572737e-01, 4.99999999999999944489e-01, 2.58819045102521017032e-01, 1.22464679914735320717e-16, -2.58819045102520794988e-01, -4.99999999999999722444e-01, -7.07106781186547128648e-01, -8.66025403784438374544e-01, -9.65925826289068312214e-01, -1.00000000000000000000e+00, -9.65925826289068423236e-01, -8.66025403784438596588e-01, -7.07106781186547683760e-01, -5.00000000000000444089e-01, -2.58819045102521572144e-01};
    return v[m];
  }
};
template <> struct Roots<25> {
  static AF_HD rl c(int m) {
    constexpr rl v[25] = {1.00000000000000000000e+00, 9.68583161128631076053e-01, 8.76306680043863583940e-01, 7.28968627421411552447e-01, 5.35826794978996545638e-01, 3.09016994374947451263e-01, 6.27905195293135265366e-02, -1.87381314585724600974e-01, -4.25779291565072715020e-01, -6.37423989748689745483e-01, -8.09016994374947340241e-01, -9.29776485888251347234e-01, -9.92114701314477764882e-01, -9.92114701314477875904e-01, -9.29776485888251458256e-01, -8.09016994374947784330e-01, -6.37423989748689523438e-01, -4.25779291565072159909e-01, -1.87381314585724628730e-01, 6.27905195293128326472e-02, 3.09016994374947229218e-01, 5.35826794978996767682e-01, 7.28968627421411219380e-01, 8.76306680043863139851e-01, 9.68583161128630965031e-01};
    return v[m];
  }
  static AF_HD rl s(int m) {
    constexpr rl v[25] = {0.00000000000000000000e+00, 2.48689887164854794843e-01, 4.81753674101715323452e-01, 6.84547105928688615073e-01, 8.44327925502015075310e-01, 9.51056516295153531182e-01, 9.98026728428271558968e-01, 9.82287250728688721146e-01, 9.04827052466019465804e-01, 7.70513242775789253258e-01, 5.87785252292473248126e-01, 3.68124552684678141290e-01, 1.25333233564304535879e-01, -1.25333233564304286078e-01, -3.68124552684677919245e-01, -5.87785252292472693014e-01, -7.70513242775789364281e-01, -9.04827052466019798871e-01, -9.82287250728688721146e-01, -9.98026728428271558968e-01, -9.51056516295153642204e-01, -8.44327925502014964287e-01, -6.84547105928688948140e-01, -4.81753674101716100608e-01, -2.48689887164855349955e-01};
    return v[m];
  }
};
template <> struct Roots<27> {
  static AF_HD rl c(int m) {
    constexpr rl v[27] = {1.00000000000000000000e+00, 9.73044870579823806267e-01, 8.93632640323412275052e-01, 7.66044443118978013452e-01, 5.97158591702786178956e-01, 3.96079766039156899726e-01, 1.73648177666930414453e-01, -5.81448289104757737311e-02, -2.86803232711090205775e-01, -4.99999999999999777955e-01, -6.86241637868733489469e-01, -8.35487811412936265398e-01, -9.39692620785908316883e-01, -9.93238357741943023171e-01, -9.93238357741943023171e-01, -9.39692620785908538927e-01, -8.35487811412936487443e-01, -6.86241637868733600492e-01, -5.00000000000000444089e-01, -2.86803232711090649865e-01, -5.81448289104762386370e-02, 1.73648177666930830787e-01, 3.96079766039156511148e-01, 5.97158591702785845889e-01, 7.66044443118977791407e-01, 8.93632640323412164030e-01, 9.73044870579824028312e-01};
    return v[m];
  }
  static AF_HD rl s(int m) {
    constexpr rl v[27] = {0.00000000000000000000e+00, 2.30615870742440165486e-01, 4.48799180200462166646e-01, 6.42787609686539251896e-01, 8.02123192755043734614e-01, 9.18216106880273996715e-01, 9.84807753012208020316e-01, 9.98308158271268175632e-01, 9.57989512315488900285e-01, 8.66025403784438707611e-01, 7.27373641573048845821e-01, 5.49508978070806231031e-01, 3.42020143325668879442e-01, 1.16092914125229929034e-01, -1.16092914125230123323e-01, -3.42020143325668213308e-01, -5.49508978070806008986e-01, -7.27373641573048623776e-01, -8.66025403784438374544e-01, -9.57989512315488789262e-01, -9.98308158271268175632e-01, -9.84807753012208020316e-01, -9.18216106880274107738e-01, -8.02123192755043956659e-01, -6.42787609686539584963e-01, -4.48799180200462444201e-01, -2.30615870742439582619e-01};
    return v[m];
  }
};
template <> struct Roots<32> {
  static AF_HD rl c(int m) {
    constexpr rl v[32] = {1.00000000000000000000e+00, 9.80785280403230430579e-01, 9.23879532511286738483e-01, 8.31469612302545235671e-01, 7.07106781186547572737e-01, 5.55570233019602288671e-01, 3.82683432365089837290e-01, 1.95090322016128331351e-01, 0.00000000000000000000e+00, -1.95090322016128192573e-01, -3.82683432365089726268e-01, -5.55570233019601955604e-01, -7.07106781186547461715e-01, -8.31469612302545346694e-01, -9.23879532511286738483e-01, -9.80785280403230430579e-01, -1.00000000000000000000e+00, -9.80785280403230430579e-01, -9.23879532511286849505e-01, -8.31469612302545457716e-01, -7.07106781186547683760e-01, -5.55570233019602177649e-01, -3.82683432365090336891e-01, -1.95090322016128664417e-01, 0.00000000000000000000e+00, 1.95090322016128303595e-01, 3.82683432365090003824e-01, 5.55570233019601844582e-01, 7.07106781186547350693e-01, 8.31469612302545235671e-01, 9.23879532511286516439e-01, 9.80785280403230319557e-01};
    return v[m];
  }
  static AF_HD rl s(int m) {
    constexpr rl v[32] = {0.00000000000000000000e+00, 1.95090322016128248084e-01, 3.82683432365089781779e-01, 5.55570233019602177649e-01, 7.07106781186547461715e-01, 8.31469612302545235671e-01, 9.23879532511286738483e-01, 9.80785280403230430579e-01, 1.00000000000000000000e+00, 9.80785280403230430579e-01, 9.23879532511286738483e-01, 8.31469612302545457716e-01, 7.07106781186547572737e-01, 5.55570233019602177649e-01, 3.82683432365089892802e-01, 1.95090322016128608906e-01, 0.00000000000000000000e+00, -1.95090322016128359106e-01, -3.82683432365089670757e-01, -5.55570233019601955604e-01, -7.07106781186547461715e-01, -8.31469612302545235671e-01, -9.23879532511286516439e-01, -9.80785280403230319557e-01, -1.00000000000000000000e+00, -9.80785280403230430579e-01, -9.23879532511286627461e-01, -8.31469612302545457716e-01, -7.07106781186547683760e-01, -5.55570233019602177649e-01, -3.82683432365090392402e-01, -1.95090322016128719929e-01};
    return v[m];
  }
};

// multiply by exp(sign * 2 pi i m / R) for a compile-time m (after unrolling)
template <int R>
AF_HD cx mul_root(cx a, int m, rl sign) {
  m %= R;
  if (m == 0) return a;
  if (4 * m == R) return mul_si(a, sign);
  if (2 * m == R) return make_cx(-a.x, -a.y);
  if (4 * m == 3 * R) return mul_si(a, -sign);
  return cmul(a, make_cx(Roots<R>::c(m), sign * Roots<R>::s(m)));
}

// Composite radix R = A*B (Cooley-Tukey inside the butterfly): DFT_A over j1
// of u[B j1 + j2], twiddle W_R^(j2 k1), DFT_B over j2; output k1 + A k2.
template <int A, int B>
struct DftComposite {
  static AF_HD void run(cx* u, rl sign, const cx* tab, int S, int n) {
    constexpr int R = A * B;
    cx v[R];
#pragma unroll
    for (int j2 = 0; j2 < B; ++j2) {
      cx t[A];
#pragma unroll
      for (int j1 = 0; j1 < A; ++j1) t[j1] = u[B * j1 + j2];
      Dft<A>::run(t, sign, tab, S, n);
#pragma unroll
      for (int k1 = 0; k1 < A; ++k1) v[j2 * A + k1] = mul_root<R>(t[k1], j2 * k1, sign);
    }
#pragma unroll
    for (int k1 = 0; k1 < A; ++k1) {
      cx t[B];
#pragma unroll
      for (int j2 = 0; j2 < B; ++j2) t[j2] = v[j2 * A + k1];
      Dft<B>::run(t, sign, tab, S, n);
#pragma unroll
      for (int k2 = 0; k2 < B; ++k2) u[k1 + A * k2] = t[k2];
    }
  }
};
template <> struct Dft<6> : DftComposite<2, 3> {};
template <> struct Dft<9> : DftComposite<3, 3> {};
template <> struct Dft<10> : DftComposite<2, 5> {};
template <> struct Dft<12> : DftComposite<4, 3> {};
template <> struct Dft<15> : DftComposite<3, 5> {};
template <> struct Dft<20> : DftComposite<4, 5> {};
template <> struct Dft<24> : DftComposite<8, 3> {};
template <> struct Dft<25> : DftComposite<5, 5> {};
template <> struct Dft<27> : DftComposite<3, 9> {};
template <> struct Dft<32> : DftComposite<4, 8> {};

}  // namespace AF_NS
