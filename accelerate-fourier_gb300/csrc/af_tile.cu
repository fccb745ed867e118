// af_tile.cu -- the shared-memory tile FFT kernel of libaf.
//
// Every FFT launch of the library is this kernel: a list of work items, one
// per CTA, each naming a tile descriptor (device memory) and the lines it
// owns.  A CTA copies its descriptor to shared memory, loads its lines
// through the descriptor's index map, runs one or two Stockham FFT phases
// (passes of radix 2 to 27 alternating between two shared buffers), and
// stores through the inverse map with the four-step twiddle, scale and
// optional cotangent epilogue.
//
// Tile kinds restate the reference's algorithms (file:line relative to the
// accelerate-fourier project):
//   TILE_PLAIN      Cooley-Tukey / split-radix passes (Fourier/Planned.hs:473-557),
//                   with Good-Thomas (584-617), Rader (646-692) and Bluestein
//                   (760-773) index maps fused into loads and stores
//   TILE_GT         Good-Thomas in one tile with the reference's CRT maps
//   TILE_RADER      Rader's algorithm in one tile (Permutation.hs:24-80)
//   TILE_BLUESTEIN  Bluestein in one tile (Private.hs:428-436)
//   TILE_CONVROW    middle pass of a four-step cyclic convolution (Planned.hs:803-821)
#include <atomic>

#include "af_device.cuh"
#include "af_internal.h"

namespace AF_NS {

// Scalars of one phase, held in registers (the descriptor lives in shared
// memory; reading its fields inside the pass loops would re-read them).
struct PhaseRegs {
  int n, lines, LS, ls, es, lcnt, S_log2, psh;
  rl sign;
  FastDiv lcnt_div;
};


// u[j] *= w^j for j = 1..R-1 with w = W^t1 from the phase table.  The
// powers are w^(Q a + b) = W^(Q a t1) * w^b: the W^(Q a t1) come from the
// table, the small powers w^b (b < Q <= 4) from at most two products, so
// every twiddle is within three rounded products of table values.
template <int R>
__device__ __forceinline__ void apply_twiddles(cx* u, const cx* __restrict__ ptab, int S_log2, int t1,
                                               rl sign) {
  constexpr int Q = R <= 4 ? 2 : (R <= 9 ? 3 : 4);
  cx s[Q];
  s[0] = make_cx(1.f, 0.f);
  s[1] = tw_lookup(ptab, S_log2, t1, sign);
#pragma unroll
  for (int b = 2; b < Q; ++b) s[b] = b == 2 ? cmul(s[1], s[1]) : cmul(s[2], s[1]);
  cx big = s[0];
#pragma unroll
  for (int j = 1; j < R; ++j) {
    const int a = j / Q, b = j % Q;
    if (a >= 1 && b == 0) big = tw_lookup(ptab, S_log2, j * t1, sign);
    const cx w = a == 0 ? s[b] : (b == 0 ? big : cmul(big, s[b]));
    u[j] = cmul(u[j], w);
  }
}

// One Stockham pass, src -> dst (ping-pong shared buffers).  Butterfly g (of
// the phase's lines*n/R) reads elements i + j*(n/R) of its line, applies the
// twiddles W^(j k tw_stride) (k = i mod p) and the radix-R DFT, and writes
// (i-k)*R + k + j*p.
template <int R, int T>
__device__ __forceinline__ void stockham_pass(const cx* __restrict__ src, cx* __restrict__ dst,
                                              const PhaseRegs& ph, const PassDesc& pd,
                                              const cx* __restrict__ ptab) {
  const int nb = ph.n / R;
  const int total = ph.lines * nb;
  const int p = pd.p, tws = pd.tw_stride;
  const FastDiv nbd = pd.nb_div, pdv = pd.p_div;
  const int pe = p * ph.es, nbe = nb * ph.es;
  for (int g = threadIdx.x; g < total; g += T) {
    const int l = (int)fdiv((unsigned)g, nbd);
    const int i = g - l * nb;
    const int t = (int)fdiv((unsigned)l, ph.lcnt_div);
    const int base = t * ph.LS + (l - t * ph.lcnt) * ph.ls;
    cx u[R];
    const int ib = base + i * ph.es;
#pragma unroll
    for (int j = 0; j < R; ++j) u[j] = src[spd_(ib + j * nbe, ph.psh)];
    const int q = (int)fdiv((unsigned)i, pdv);
    const int k = i - q * p;
    if (k > 0) apply_twiddles<R>(u, ptab, ph.S_log2, k * tws, ph.sign);
    Dft<R>::run(u, ph.sign, ptab, ph.S_log2, ph.n);
    const int ob = base + (q * p * R + k) * ph.es;
#pragma unroll
    for (int j = 0; j < R; ++j) dst[spd_(ob + j * pe, ph.psh)] = u[j];
  }
  __syncthreads();
}

// Runs every pass of a phase; returns the buffer holding the result.
template <int T>
__device__ __forceinline__ cx* run_phase(cx* cur, cx* oth, const FftPhase* phs, int LS, int G,
                                             const cx* tab, int psh) {
  PhaseRegs r;
  r.psh = psh;
  r.n = phs->n;
  r.lines = G * phs->lcnt;
  r.LS = LS;
  r.ls = phs->ls;
  r.es = phs->es;
  r.lcnt = phs->lcnt;
  r.lcnt_div = phs->lcnt_div;
  r.S_log2 = phs->twS_log2;
  r.sign = phs->sign;
  const cx* ptab = tab + phs->tw_off;
  const int npass = phs->npass;
  for (int p = 0; p < npass; ++p) {
    const PassDesc pd = phs->pass[p];
    switch (pd.R) {
      case 2: stockham_pass<2, T>(cur, oth, r, pd, ptab); break;
      case 3: stockham_pass<3, T>(cur, oth, r, pd, ptab); break;
      case 4: stockham_pass<4, T>(cur, oth, r, pd, ptab); break;
      case 5: stockham_pass<5, T>(cur, oth, r, pd, ptab); break;
      case 6: stockham_pass<6, T>(cur, oth, r, pd, ptab); break;
      case 7: stockham_pass<7, T>(cur, oth, r, pd, ptab); break;
      case 8: stockham_pass<8, T>(cur, oth, r, pd, ptab); break;
      case 9: stockham_pass<9, T>(cur, oth, r, pd, ptab); break;
      case 10: stockham_pass<10, T>(cur, oth, r, pd, ptab); break;
      case 11: stockham_pass<11, T>(cur, oth, r, pd, ptab); break;
      case 12: stockham_pass<12, T>(cur, oth, r, pd, ptab); break;
      case 13: stockham_pass<13, T>(cur, oth, r, pd, ptab); break;
      case 15: stockham_pass<15, T>(cur, oth, r, pd, ptab); break;
      case 16: stockham_pass<16, T>(cur, oth, r, pd, ptab); break;
      case 20: stockham_pass<20, T>(cur, oth, r, pd, ptab); break;
      case 25: stockham_pass<25, T>(cur, oth, r, pd, ptab); break;
      case 27: stockham_pass<27, T>(cur, oth, r, pd, ptab); break;
    }
    cx* tmp = cur;
    cur = oth;
    oth = tmp;
  }
  return cur;
}

__device__ __forceinline__ cx gld(const TileBases& B, int buf, i64 a) {
  if (B.c[buf]) return B.c[buf][a];
  return make_cx(B.re[buf][a], B.im[buf][a]);
}
__device__ __forceinline__ void gst(const TileBases& B, int buf, i64 a, cx v) {
  if (B.c[buf]) B.c[buf][a] = v;
  else { B.re[buf][a] = v.x; B.im[buf][a] = v.y; }
}
__device__ __forceinline__ void split_line(const IoDesc& io, int line, int& hi, int& lo) {
  hi = (int)fdiv((unsigned)line, io.lo_div);
  lo = line - hi * (int)io.lo_div.d;
}
// (mA lo + mB e) mod mN with the constants reduced mod mN
__device__ __forceinline__ unsigned gt_index(const IoDesc& io, int lo, int e) {
  unsigned r = mulmod((unsigned)io.mA, (unsigned)lo, io.m_mod) + mulmod((unsigned)io.mB, (unsigned)e, io.m_mod);
  if (r >= io.m_mod.n) r -= io.m_mod.n;
  return r;
}
// address of element e of a line (hi, lo) for the AFFINE and GT maps
__device__ __forceinline__ i64 io_addr(const IoDesc& io, i64 base, int hi, int lo, int e) {
  if (io.map == IO_GT) return base + (i64)hi * io.s_hi + (i64)gt_index(io, lo, e) * io.s_t;
  return base + (i64)hi * io.s_hi + (i64)lo * io.s_lo + (i64)e * io.s_e;
}
// the same with the line's base offset lb already known (AFFINE views)
__device__ __forceinline__ i64 io_addr_l(const IoDesc& io, i64 base, i64 lb, int hi, int lo, int e) {
  if (io.map == IO_GT) return io_addr(io, base, hi, lo, e);
  return base + lb + (i64)e * io.s_e;
}
// offset of line `line` of an AFFINE view (relative to the view's offset):
// from the gathered-line table when the view has one
__device__ __forceinline__ i64 line_base(const IoDesc& io, int line) {
  if (io.loff) return __ldg(io.loff + line);
  int hi, lo;
  split_line(io, line, hi, lo);
  return (i64)hi * io.s_hi + (i64)lo * io.s_lo;
}

// Visit (line, element) pairs of G lines x N elements in the coalescing
// order asked for (element-fast or line-fast).
template <int T, class F>
__device__ __forceinline__ void for_tile(int G, int N, const FastDiv& Ndiv, const FastDiv& Gdiv,
                                         int line_fast, F f) {
  const int tot = G * N;
  if (!line_fast) {
    for (int q = threadIdx.x; q < tot; q += T) {
      const int l = (int)fdiv((unsigned)q, Ndiv);
      f(l, q - l * N);
    }
  } else {
    for (int q = threadIdx.x; q < tot; q += T) {
      const int e = (int)fdiv((unsigned)q, Gdiv);
      f(q - e * G, e);
    }
  }
}

// global read through the read-only data path (no launch writes an address
// that another CTA of the same launch reads)
__device__ __forceinline__ cx gldr(const TileBases& B, int buf, i64 a) {
  if (B.c[buf]) return __ldg(&B.c[buf][a]);
  return make_cx(__ldg(&B.re[buf][a]), __ldg(&B.im[buf][a]));
}

// Loads G lines x N elements into shared memory: `fetch(l, e, v)` issues the
// load of element e of line l into v and returns its shared position.  Each
// thread issues U fetches before writing any of them.
template <int T, class F>
__device__ __forceinline__ void load_tile(int G, int N, const FastDiv& Ndiv, const FastDiv& Gdiv, int line_fast,
                                          F fetch, cx* sm) {
  constexpr int U = 8;
  const int tot = G * N;
  for (int q0 = threadIdx.x; q0 < tot; q0 += T * U) {
    cx v[U];
    int pos[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int q = q0 + u * T;
      pos[u] = -1;
      if (q < tot) {
        int l, e;
        if (!line_fast) {
          l = (int)fdiv((unsigned)q, Ndiv);
          e = q - l * N;
        } else {
          e = (int)fdiv((unsigned)q, Gdiv);
          l = q - e * G;
        }
        pos[u] = fetch(l, e, v[u]);
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u)
      if (pos[u] >= 0) sm[pos[u]] = v[u];
  }
}

// Asynchronous copy of G lines x N interleaved elements into shared memory
// (cp.async, one complex element per copy: 8 bytes in FP32, 16 in FP64):
// `src(l, e)` gives the global address of element e of line l, or nullptr for
// a zero.  No register staging: every element of the tile is in flight at
// once.  The caller's barrier follows the wait.
__device__ __forceinline__ void cp_async8(cx* sdst, const cx* gsrc) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(sdst);
#ifdef AF_F64
  asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gsrc) : "memory");
#else
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gsrc) : "memory");
#endif
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
}
template <int T, class F>
__device__ __forceinline__ void load_tile_async(int G, int N, const FastDiv& Ndiv, const FastDiv& Gdiv,
                                                int line_fast, int LS, int psh, F src, cx* sm) {
  const int tot = G * N;
  for (int q = threadIdx.x; q < tot; q += T) {
    int l, e;
    if (!line_fast) {
      l = (int)fdiv((unsigned)q, Ndiv);
      e = q - l * N;
    } else {
      e = (int)fdiv((unsigned)q, Gdiv);
      l = q - e * G;
    }
    int pos = spd_(l * LS + e, psh);  // src may move the element (permuted tiles)
    const cx* g = src(l, e, pos);
    cx* d = sm + pos;
    if (g) cp_async8(d, g);
    else *d = make_cx(0.f, 0.f);  // zero padding
  }
  cp_async_wait_all();
}

// A global view (IoDesc) copied into registers with its base pointer resolved.
struct IoRegs {
  cx* c;
  rl* re;
  rl* im;
  i64 s_e, s_lo, s_hi, s_t;
  FastDiv lo_div;
  unsigned mA, mB;
  ModN m_mod;
  i64 q_lo, q_e, mN;
  const int* tab;
  const cx* vec;
};
__device__ __forceinline__ IoRegs io_regs(const IoDesc& io, const TileBases& B, i64 base) {
  IoRegs r;
  r.c = B.c[io.buf] ? B.c[io.buf] + base : nullptr;
  r.re = B.re[io.buf] ? B.re[io.buf] + base : nullptr;
  r.im = B.im[io.buf] ? B.im[io.buf] + base : nullptr;
  r.s_e = io.s_e;
  r.s_lo = io.s_lo;
  r.s_hi = io.s_hi;
  r.s_t = io.s_t;
  r.lo_div = io.lo_div;
  r.mA = (unsigned)io.mA;
  r.mB = (unsigned)io.mB;
  r.m_mod = io.m_mod;
  r.q_lo = io.q_lo;
  r.q_e = io.q_e;
  r.mN = io.mN;
  r.tab = io.tab;
  r.vec = io.vec;
  return r;
}
__device__ __forceinline__ cx rld(const IoRegs& r, i64 a) {
  if (r.c) return __ldg(&r.c[a]);
  return make_cx(__ldg(&r.re[a]), __ldg(&r.im[a]));
}
__device__ __forceinline__ void rsplit(const IoRegs& r, int line, int& hi, int& lo) {
  hi = (int)fdiv((unsigned)line, r.lo_div);
  lo = line - hi * (int)r.lo_div.d;
}
__device__ __forceinline__ unsigned rgt(const IoRegs& r, int lo, int e) {
  unsigned v = mulmod(r.mA, (unsigned)lo, r.m_mod) + mulmod(r.mB, (unsigned)e, r.m_mod);
  if (v >= r.m_mod.n) v -= r.m_mod.n;
  return v;
}

struct StoreCtx {
  const TileBases* B;
  rl loss;
  int cot;
};

// final store of one element; the cotangent epilogue stores g = 2 w v with
// w at the same address in BUF_AUX (real weights, interleaved as (w, 0)
// pairs or a planar re plane) and adds w |v|^2 to the loss
__device__ __forceinline__ void store_final(StoreCtx& sc, int buf, i64 a, cx v) {
  if (sc.cot) {
    const rl w = sc.B->c[BUF_AUX] ? reinterpret_cast<const rl*>(sc.B->c[BUF_AUX])[a] : sc.B->re[BUF_AUX][a];
    sc.loss += w * (v.x * v.x + v.y * v.y);
    v = cscale(v, 2.f * w);
  }
  gst(*sc.B, buf, a, v);
}

// GEN = false compiles only PLAIN tiles with AFFINE views, one phase and no
// Rader captures (most tiles): a much smaller kernel, kinder to the
// instruction cache.
template <int T, bool GEN>
__device__ __forceinline__ void tile_body(const TileDesc& d, const WorkItem& it, const TileBases& B,
                                          cx* A, cx* Bf, const cx* tab, cx* xs, double* loss) {
  const int line0 = it.line0;
  const int G = it.G;
  const int N = d.nlen;
  const int psh = d.pad_sh;
  FastDiv Gdiv = d.G_div;
  if (G != d.G) {
    Gdiv.d = G;
    unsigned s = 0;
    while ((1u << s) < (unsigned)G) ++s;
    Gdiv.s = s;
    Gdiv.m = G <= 1 ? 0u : (unsigned)(((1ull << 32) * ((1ull << s) - (unsigned)G)) / (unsigned)G + 1);
  }
  cx* sm = A;
  const IoDesc& in = d.in;
  const IoDesc& out = d.out;
  const i64 ibase = in.off + it.in_add;
  const i64 obase = out.off + it.out_add;

  // Per-line base offsets of AFFINE views (relative to the view's offset)
  // for the CTA's G lines, input then output, after the 2G slots of Rader
  // scratch.
  const bool rows_kind = !GEN || d.kind == TILE_PLAIN || d.kind == TILE_CONVROW;
  i64* lbi = reinterpret_cast<i64*>(xs + 2 * d.G);
  i64* lbo = lbi + d.G;
  for (int l = threadIdx.x; l < G; l += T) {
    lbi[l] = line_base(in, line0 + l);
    lbo[l] = line_base(out, line0 + l);
  }
  __syncthreads();
  rl lsum = 0.f;

  // ------------------------------------------------------------ load
  // Loads are issued in groups of U independent read-only-path loads per
  // thread before any shared-memory write, so that many are in flight.
  const int LS = d.LS;
  if (rows_kind) {
    const IoRegs r = io_regs(in, B, ibase);
    const int lf = in.line_fast;
    switch (GEN ? in.map : (int)IO_AFFINE) {
      case IO_AFFINE:
        if (r.c) {  // interleaved: asynchronous copies straight into shared memory
          const cx* c = r.c;
          const i64 se = r.s_e;
          if (se == 1)
            load_tile_async<T>(G, N, d.N_div, Gdiv, lf, LS, psh, [&](int l, int e, int&) { return c + lbi[l] + e; }, sm);
          else
            load_tile_async<T>(G, N, d.N_div, Gdiv, lf, LS, psh,
                               [&](int l, int e, int&) { return c + lbi[l] + (i64)e * se; }, sm);
        } else if (r.s_e == 1) {
          load_tile<T>(G, N, d.N_div, Gdiv, lf, [&](int l, int e, cx& v) -> int {
            v = rld(r, lbi[l] + e);
            return spd_(l * LS + e, psh);
          }, sm);
        } else {
          const i64 se = r.s_e;
          load_tile<T>(G, N, d.N_div, Gdiv, lf, [&](int l, int e, cx& v) -> int {
            v = rld(r, lbi[l] + (i64)e * se);
            return spd_(l * LS + e, psh);
          }, sm);
        }
        break;
      case IO_GT:
        if (r.c) {
          const cx* c = r.c;
          load_tile_async<T>(G, N, d.N_div, Gdiv, lf, LS, psh, [&](int l, int e, int&) {
            int hi, lo;
            rsplit(r, line0 + l, hi, lo);
            return c + (i64)hi * r.s_hi + (i64)rgt(r, lo, e) * r.s_t;
          }, sm);
          break;
        }
        load_tile<T>(G, N, d.N_div, Gdiv, lf, [&](int l, int e, cx& v) -> int {
          int hi, lo;
          rsplit(r, line0 + l, hi, lo);
          v = rld(r, (i64)hi * r.s_hi + (i64)rgt(r, lo, e) * r.s_t);
          return spd_(l * LS + e, psh);
        }, sm);
        break;
      case IO_TABLE:  // zero beyond the table length mN
        if (r.c) {
          const cx* c = r.c;
          const cx* zero = nullptr;
          load_tile_async<T>(G, N, d.N_div, Gdiv, lf, LS, psh, [&](int l, int e, int&) {
            int hi, lo;
            rsplit(r, line0 + l, hi, lo);
            const i64 q = lo * r.q_lo + e * r.q_e;
            return q < r.mN ? c + (i64)hi * r.s_hi + (i64)__ldg(&r.tab[q]) * r.s_t : zero;
          }, sm);
          break;
        }
        load_tile<T>(G, N, d.N_div, Gdiv, lf, [&](int l, int e, cx& v) -> int {
          int hi, lo;
          rsplit(r, line0 + l, hi, lo);
          const i64 q = lo * r.q_lo + e * r.q_e;
          v = make_cx(0.f, 0.f);
          if (q < r.mN) v = rld(r, (i64)hi * r.s_hi + (i64)__ldg(&r.tab[q]) * r.s_t);
          return spd_(l * LS + e, psh);
        }, sm);
        break;
      default:  // IO_CHIRP: zero pad beyond the logical length
        load_tile<T>(G, N, d.N_div, Gdiv, lf, [&](int l, int e, cx& v) -> int {
          int hi, lo;
          rsplit(r, line0 + l, hi, lo);
          const i64 q = lo * r.q_lo + e * r.q_e;
          v = make_cx(0.f, 0.f);
          if (q < r.mN) v = cmul(__ldg(&r.vec[q]), rld(r, (i64)hi * r.s_hi + q * r.s_t));
          return spd_(l * LS + e, psh);
        }, sm);
        break;
    }
    if (GEN && d.x0_cap >= 0 && threadIdx.x == 0) {
      for (int l = 0; l < G; ++l) {
        int hi, lo;
        split_line(in, line0 + l, hi, lo);
        if (lo == 0) B.c[BUF_WS][d.x0_cap + it.out_add + hi] = gld(B, in.buf, ibase + (i64)hi * in.s_hi);
      }
    }
  } else if (d.kind == TILE_GT) {
    // grid position (k, j) holds x[(n k + m j) mod N]  (Planned.hs:597-606);
    // inverting: k = i*cm mod m, j = i*cn mod n
    if (B.c[in.buf]) {
      const cx* c = B.c[in.buf];
      load_tile_async<T>(G, N, d.N_div, Gdiv, 0, d.LS, psh, [&](int l, int i, int& pos) {
        int hi, lo;
        split_line(in, line0 + l, hi, lo);
        const int k = (int)mulmod((unsigned)i, (unsigned)d.gt_cm, d.gt_m_mod);
        const int j = (int)mulmod((unsigned)i, (unsigned)d.gt_cn, d.gt_n_mod);
        pos = spd_(l * d.LS + k * d.gt_n + j, psh);
        return c + io_addr_l(in, ibase, lbi[l], hi, lo, i);
      }, sm);
    } else {
      load_tile<T>(G, N, d.N_div, Gdiv, 0, [&](int l, int i, cx& v) -> int {
        int hi, lo;
        split_line(in, line0 + l, hi, lo);
        const int k = (int)mulmod((unsigned)i, (unsigned)d.gt_cm, d.gt_m_mod);
        const int j = (int)mulmod((unsigned)i, (unsigned)d.gt_cn, d.gt_n_mod);
        v = gldr(B, in.buf, io_addr_l(in, ibase, lbi[l], hi, lo, i));
        return spd_(l * d.LS + k * d.gt_n + j, psh);
      }, sm);
    }
  } else if (d.kind == TILE_RADER) {
    // a[q] = x[g^-q]  (Permutation.apply rev res, Planned.hs:686-692): input
    // index r >= 1 with g^dlog(r) = r goes to q = (-dlog r) mod (p-1)
    const int m = N - 1;
    // a convolution carried by longer transforms (slen > p-1) is zero padded
    for (int q = threadIdx.x; q < G * (d.slen - m); q += T) {
      const int l = q / (d.slen - m);
      sm[spd_(l * d.LS + m + (q - l * (d.slen - m)), psh)] = make_cx(0.f, 0.f);
    }
    const int xs_pos = (int)(xs - sm);  // x0 of line l goes to xs[2 l]
    if (B.c[in.buf]) {
      const cx* c = B.c[in.buf];
      load_tile_async<T>(G, N, d.N_div, Gdiv, 0, d.LS, psh, [&](int l, int r, int& pos) {
        int hi, lo;
        split_line(in, line0 + l, hi, lo);
        if (r == 0) {
          pos = xs_pos + 2 * l;
        } else {
          const int lg = __ldg(&d.dlog[r - 1]);
          pos = spd_(l * d.LS + (lg == 0 ? 0 : m - lg), psh);
        }
        return c + io_addr_l(in, ibase, lbi[l], hi, lo, r);
      }, sm);
    } else {
      load_tile<T>(G, N, d.N_div, Gdiv, 0, [&](int l, int r, cx& v) -> int {
        int hi, lo;
        split_line(in, line0 + l, hi, lo);
        v = gldr(B, in.buf, io_addr_l(in, ibase, lbi[l], hi, lo, r));
        if (r == 0) return xs_pos + 2 * l;
        const int lg = __ldg(&d.dlog[r - 1]);
        return spd_(l * d.LS + (lg == 0 ? 0 : m - lg), psh);
      }, sm);
    }
  } else {  // TILE_BLUESTEIN: chirp * x zero padded to M (Planned.hs:765-773)
    const int M = d.slen;
    load_tile<T>(G, M, d.S_div, Gdiv, 0, [&](int l, int e, cx& v) -> int {
      int hi, lo;
      split_line(in, line0 + l, hi, lo);
      v = make_cx(0.f, 0.f);
      if (e < N) v = cmul(__ldg(&d.vec_a[e]), gldr(B, in.buf, io_addr_l(in, ibase, lbi[l], hi, lo, e)));
      return spd_(l * d.LS + e, psh);
    }, sm);
  }
  cp_async_wait_all();  // tables (and any tile copies not yet waited for)
  __syncthreads();

  // ------------------------------------------------------------ phases
  // One inlined copy of the passes serves both phases (half the code of two).
  const int nph = GEN ? d.nph : 1;
  for (int phi = 0; phi < nph; ++phi) {
    if (GEN && phi == 1 && (d.kind == TILE_RADER || d.kind == TILE_BLUESTEIN || d.kind == TILE_CONVROW)) {
      // FFT(+1) -> * spectrum -> FFT(-1): the direction order of the reference's
      // convolveSingleSpectrumCyclicCache (Planned.hs:803-821)
      if (d.kind == TILE_RADER) {
        for (int l = threadIdx.x; l < G; l += T) xs[2 * l + 1] = sm[spd_(l * d.LS, psh)];  // sum res
        __syncthreads();
      }
      const int M = d.slen;
      if (d.kind == TILE_CONVROW) {
        if (d.dc_off >= 0 && threadIdx.x == 0) {
          for (int l = 0; l < G; ++l) {
            int hi, lo;
            split_line(out, line0 + l, hi, lo);
            if (lo == 0) B.c[BUF_WS][d.dc_off + it.out_add + hi] = sm[spd_(l * d.LS, psh)];
          }
        }
        __syncthreads();
        for_tile<T>(G, M, d.S_div, Gdiv, 0, [&](int l, int e) {
          int hi, lo;
          split_line(out, line0 + l, hi, lo);
          const int a = spd_(l * d.LS + e, psh);
          sm[a] = cmul(__ldg(&d.vec_b[lo * d.sq_lo + e * d.sq_e]), sm[a]);
        });
      } else {
        for_tile<T>(G, M, d.S_div, Gdiv, 0, [&](int l, int e) {
          const int a = spd_(l * d.LS + e, psh);
          sm[a] = cmul(__ldg(&d.vec_b[e]), sm[a]);
        });
      }
      __syncthreads();
    }
    sm = run_phase<T>(sm, sm == A ? Bf : A, &d.ph[phi], d.LS, G, tab, psh);
  }

  // ------------------------------------------------------------ store
  StoreCtx sc{&B, 0.f, d.cot};
  if (rows_kind) {
    const IoRegs ro = io_regs(out, B, obase);
    const cx* __restrict__ ptw = d.ptw;
    const int ptwS = d.ptwS_log2;
    const ModN pmod = d.ptw_mod;
    const rl psign = d.ptw_sign;
    const rl scale = d.scale;
    const int cot = d.cot;
    const rl* __restrict__ wp = B.c[BUF_AUX] ? reinterpret_cast<const rl*>(B.c[BUF_AUX]) : B.re[BUF_AUX];
    const int omap = GEN ? out.map : (int)IO_AFFINE;
    // Rader scatter: x0 of transform hi and the DC slot
    const cx* x0p = B.c[out.x0_buf] + out.x0_off + (out.x0_buf == in.buf ? it.in_add : it.out_add);
    const i64 x0_shi = out.x0_shi;
    const cx* dcp = B.c[BUF_WS] + out.dc_off + it.in_add;
    auto put = [&](i64 rel, cx v) {
      if (cot) {
        const rl w = __ldg(&wp[obase + rel]);
        lsum += w * (v.x * v.x + v.y * v.y);
        v = cscale(v, 2.f * w);
      }
      if (ro.c) ro.c[rel] = v;
      else { ro.re[rel] = v.x; ro.im[rel] = v.y; }
    };
    const i64 ose = ro.s_e;
    for_tile<T>(G, N, d.N_div, Gdiv, out.line_fast, [&](int l, int e) {
      int hi, lo;
      if (omap == IO_AFFINE && !ptw) {
        hi = lo = 0;
      } else {
        rsplit(ro, line0 + l, hi, lo);
      }
      cx v = sm[spd_(l * LS + e, psh)];
      if (ptw) {
        const unsigned t = mulmod((unsigned)lo, (unsigned)e, pmod);
        const cx wl = __ldg(&ptw[t & ((1u << ptwS) - 1)]);
        const cx wh = __ldg(&ptw[(1u << ptwS) + (t >> ptwS)]);
        cx w = cmul(wh, wl);
        w.y *= -psign;
        v = cmul(v, w);
      }
      v = cscale(v, scale);
      if (omap == IO_AFFINE) {
        put(lbo[l] + (i64)e * ose, v);
        return;
      }
      const i64 hb = (i64)hi * ro.s_hi;
      if (omap == IO_GT) {
        put(hb + (i64)rgt(ro, lo, e) * ro.s_t, v);
      } else if (omap == IO_CHIRP) {
        const i64 q = lo * ro.q_lo + e * ro.q_e;
        if (q < ro.mN) put(hb + q * ro.s_t, cmul(__ldg(&ro.vec[q]), v));
      } else {  // IO_RADER: c[q] -> out[g^q] = x0 + c[q]; q == 0 also out[0] = x0 + dc
        const i64 q = lo * ro.q_lo + e * ro.q_e;
        if (q >= ro.mN) return;  // padding of a longer convolution
        const cx x0 = x0p[(i64)hi * x0_shi];
        put(hb + (i64)__ldg(&ro.tab[q]) * ro.s_t, cadd(x0, v));
        if (q == 0) put(hb, cadd(x0, cscale(dcp[hi], scale)));
      }
    });
    sc.loss = lsum;
  } else if (d.kind == TILE_GT) {
    // out[r] = C[r mod n][r mod m]  (Planned.hs:608-617); C[q][p] sits at p*n + q
    for_tile<T>(G, N, d.N_div, Gdiv, 0, [&](int l, int r) {
      int hi, lo;
      split_line(out, line0 + l, hi, lo);
      const cx v = sm[spd_(l * d.LS + (int)mod_of((unsigned)r, d.gt_m_mod) * d.gt_n +
                               (int)mod_of((unsigned)r, d.gt_n_mod), psh)];
      store_final(sc, out.buf, io_addr_l(out, obase, lbo[l], hi, lo, r), cscale(v, d.scale));
    });
  } else if (d.kind == TILE_RADER) {
    // out[0] = x0 + sum res; out[r] = x0 + c[dlog r]  (Planned.hs:686-692)
    for_tile<T>(G, N, d.N_div, Gdiv, 0, [&](int l, int r) {
      int hi, lo;
      split_line(out, line0 + l, hi, lo);
      const cx x0 = xs[2 * l];
      const cx v = r == 0 ? xs[2 * l + 1] : sm[spd_(l * d.LS + __ldg(&d.dlog[r - 1]), psh)];
      store_final(sc, out.buf, io_addr_l(out, obase, lbo[l], hi, lo, r), cscale(cadd(x0, v), d.scale));
    });
  } else {  // Bluestein: y = chirp * (take N c)
    for_tile<T>(G, N, d.N_div, Gdiv, 0, [&](int l, int e) {
      int hi, lo;
      split_line(out, line0 + l, hi, lo);
      const cx v = cmul(__ldg(&d.vec_a[e]), sm[spd_(l * d.LS + e, psh)]);
      store_final(sc, out.buf, io_addr_l(out, obase, lbo[l], hi, lo, e), cscale(v, d.scale));
    });
  }

  if (d.cot && loss) {
    rl v = sc.loss;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();  // the per-line scratch is free again: reuse it for the reduction
    rl* red = reinterpret_cast<rl*>(xs);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
      double s = 0;
      for (int w = 0; w < T / 32; ++w) s += red[w];
      atomicAdd(loss, s);
    }
  }
}

// FP32 tiles keep three 256-thread CTAs per SM; FP64 tiles (twice the
// registers and shared memory per element) one.
#ifdef AF_F64
#define AF_MIN_CTAS(T) 1
#else
#define AF_MIN_CTAS(T) (T <= 256 ? 768 / T : 1)
#endif
template <int T, bool GEN>
__global__ void __launch_bounds__(T, AF_MIN_CTAS(T)) tile_kernel(const TileDesc* __restrict__ descs,
                                                 const WorkItem* __restrict__ items, TileBases bases,
                                                 double* loss, int smem_data) {
  extern __shared__ float4 smem4[];
  cx* smem = reinterpret_cast<cx*>(smem4);
  const WorkItem it = items[blockIdx.x];
  // shared layout: [descriptor] [A: smem_data] [B: smem_data] [tables] [scratch 4G]
  TileDesc* d = reinterpret_cast<TileDesc*>(smem);
  {
    const int words = (int)(sizeof(TileDesc) / 4);
    const int* srcw = reinterpret_cast<const int*>(descs + it.desc);
    int* dstw = reinterpret_cast<int*>(d);
    for (int i = threadIdx.x; i < words; i += T) dstw[i] = srcw[i];
  }
  __syncthreads();
  const int desc_f2 = (int)((sizeof(TileDesc) + 15) / 16 * 16 / sizeof(cx));
  cx* A = smem + desc_f2;
  cx* Bf = A + smem_data;
  cx* tab = Bf + smem_data;
  cx* xs = tab + d->tw_total;
  // the twiddle tables travel with the tile's own asynchronous copies (one
  // wait for both, before the first pass)
  for (int i = threadIdx.x; i < d->tw_total; i += T) cp_async8(tab + i, d->tw_src + i);
  tile_body<T, GEN>(*d, it, bases, A, Bf, tab, xs, loss);
}

// descriptor, two buffers, tables, per-line scratch (4 elements per line; at
// least 8: the loss reduction keeps one real per warp there)
size_t tile_smem_bytes(int smem_data, int tw_total, int G) {
  const int scratch = 4 * G > 8 ? 4 * G : 8;  // Rader x0/sum pairs, then the line bases
  return (sizeof(TileDesc) + 15) / 16 * 16 + (size_t)(2 * smem_data + tw_total + scratch) * sizeof(cx);
}

// Raises the kernel's dynamic shared-memory limit to what the device allows
// (the opt-in limit less the kernel's static usage), once per device: the
// attribute is set per device, so a process using several GPUs sets it on
// each the first time it launches there.
template <int T, bool GEN>
static cudaError_t launch_t(const LaunchSpec& L, const TileBases& bases, double* loss, cudaStream_t st) {
  // per device ordinal (0: not set yet; static storage starts at zero);
  // threads that race here compute and store the same value
  static std::atomic<int> limits[64];
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  std::atomic<int>& limit = limits[dev];
  if (limit.load(std::memory_order_acquire) <= 0) {
    int optin = 0;
    cudaFuncAttributes fa;
    e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, tile_kernel<T, GEN>);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(tile_kernel<T, GEN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               optin - (int)fa.sharedSizeBytes);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return e;
    }
    limit.store(optin - (int)fa.sharedSizeBytes, std::memory_order_release);
  }
  if (L.smem_bytes > (size_t)limit.load(std::memory_order_relaxed)) return cudaErrorInvalidValue;
  tile_kernel<T, GEN><<<L.nitems, T, L.smem_bytes, st>>>(L.descs, L.items, bases, loss, L.smem_data);
  return cudaGetLastError();
}

cudaError_t launch_tiles(const LaunchSpec& L, const TileBases& bases, double* loss, cudaStream_t st) {
  if (L.nitems <= 0) return cudaSuccess;
  if (L.generic) {
    switch (L.threads) {
      case 512: return launch_t<512, true>(L, bases, loss, st);
      case 128: return launch_t<128, true>(L, bases, loss, st);
      default: return launch_t<256, true>(L, bases, loss, st);
    }
  }
  switch (L.threads) {
    case 512: return launch_t<512, false>(L, bases, loss, st);
    case 128: return launch_t<128, false>(L, bases, loss, st);
    default: return launch_t<256, false>(L, bases, loss, st);
  }
}

}  // namespace af
