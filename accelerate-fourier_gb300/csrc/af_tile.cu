// af_tile.cu -- the shared-memory tile FFT kernel of libaf.
//
// Every FFT launch of the library is this kernel: a list of work items, one
// per CTA, each naming a tile descriptor (device memory) and the lines it
// owns.  A CTA copies its descriptor to shared memory, loads its lines
// through the descriptor's index map, runs one or two Stockham FFT phases
// (passes of radix 2,3,4,5,7,8,11,13,16 alternating between two shared
// buffers), and stores through the inverse map with the four-step twiddle,
// scale and optional cotangent epilogue.
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
#include "af_device.cuh"
#include "af_internal.h"

namespace af {

// One Stockham pass, src -> dst (ping-pong shared buffers): each thread
// walks butterflies g = tid, tid + T, ... holding one radix-R butterfly.
template <int R, int T>
__device__ __forceinline__ void stockham_pass(const float2* __restrict__ src, float2* __restrict__ dst,
                                              const FftPhase& ph, int LS, int lines, const PassDesc& pd,
                                              const float2* __restrict__ ptab) {
  const int n = ph.n;
  const int nb = n / R;
  const int total = lines * nb;
  const float sign = ph.sign;
  for (int g = threadIdx.x; g < total; g += T) {
    const int l = (int)fdiv((unsigned)g, pd.nb_div);
    const int i = g - l * nb;
    const int t = (int)fdiv((unsigned)l, ph.lcnt_div);
    const int base = t * LS + (l - t * ph.lcnt) * ph.ls;
    float2 u[R];
#pragma unroll
    for (int j = 0; j < R; ++j) u[j] = src[spad(base + (i + j * nb) * ph.es)];
    const int q = (int)fdiv((unsigned)i, pd.p_div);
    const int k = i - q * pd.p;
    if (k > 0) {
      const int st = k * pd.tw_stride;
#pragma unroll
      for (int j = 1; j < R; ++j) u[j] = cmul(u[j], tw_lookup(ptab, ph.twS_log2, j * st, sign));
    }
    Dft<R>::run(u, sign, ptab, ph.twS_log2, n);
    const int ob = q * pd.p * R + k;
#pragma unroll
    for (int j = 0; j < R; ++j) dst[spad(base + (ob + j * pd.p) * ph.es)] = u[j];
  }
  __syncthreads();
}

// Runs every pass of a phase; returns the buffer holding the result.
template <int T>
__device__ __noinline__ float2* run_phase(float2* cur, float2* oth, const FftPhase* phs, int LS, int G,
                                          const float2* tab) {
  const FftPhase& ph = *phs;
  const int lines = G * ph.lcnt;
  const float2* ptab = tab + ph.tw_off;
  for (int p = 0; p < ph.npass; ++p) {
    const PassDesc& pd = ph.pass[p];
    switch (pd.R) {
      case 2: stockham_pass<2, T>(cur, oth, ph, LS, lines, pd, ptab); break;
      case 3: stockham_pass<3, T>(cur, oth, ph, LS, lines, pd, ptab); break;
      case 4: stockham_pass<4, T>(cur, oth, ph, LS, lines, pd, ptab); break;
      case 5: stockham_pass<5, T>(cur, oth, ph, LS, lines, pd, ptab); break;
      case 7: stockham_pass<7, T>(cur, oth, ph, LS, lines, pd, ptab); break;
      case 8: stockham_pass<8, T>(cur, oth, ph, LS, lines, pd, ptab); break;
      case 11: stockham_pass<11, T>(cur, oth, ph, LS, lines, pd, ptab); break;
      case 13: stockham_pass<13, T>(cur, oth, ph, LS, lines, pd, ptab); break;
      case 16: stockham_pass<16, T>(cur, oth, ph, LS, lines, pd, ptab); break;
    }
    float2* tmp = cur;
    cur = oth;
    oth = tmp;
  }
  return cur;
}

__device__ __forceinline__ float2 gld(const TileBases& B, int buf, i64 a) {
  if (B.c[buf]) return B.c[buf][a];
  return make_float2(B.re[buf][a], B.im[buf][a]);
}
__device__ __forceinline__ void gst(const TileBases& B, int buf, i64 a, float2 v) {
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
__device__ __forceinline__ float2 gldr(const TileBases& B, int buf, i64 a) {
  if (B.c[buf]) return __ldg(&B.c[buf][a]);
  return make_float2(__ldg(&B.re[buf][a]), __ldg(&B.im[buf][a]));
}

// Loads G lines x N elements into shared memory: `fetch(l, e, v)` issues the
// load of element e of line l into v and returns its shared position.  Each
// thread issues U fetches before writing any of them.
template <int T, class F>
__device__ __forceinline__ void load_tile(int G, int N, const FastDiv& Ndiv, const FastDiv& Gdiv, int line_fast,
                                          F fetch, float2* sm) {
  constexpr int U = 8;
  const int tot = G * N;
  for (int q0 = threadIdx.x; q0 < tot; q0 += T * U) {
    float2 v[U];
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

struct StoreCtx {
  const TileBases* B;
  float loss;
  int cot;
};

// final store of one element; the cotangent epilogue stores g = 2 w v with
// w at the same address in BUF_AUX (real weights, interleaved as (w, 0)
// pairs or a planar re plane) and adds w |v|^2 to the loss
__device__ __forceinline__ void store_final(StoreCtx& sc, int buf, i64 a, float2 v) {
  if (sc.cot) {
    const float w = sc.B->c[BUF_AUX] ? reinterpret_cast<const float*>(sc.B->c[BUF_AUX])[a] : sc.B->re[BUF_AUX][a];
    sc.loss += w * (v.x * v.x + v.y * v.y);
    v = cscale(v, 2.f * w);
  }
  gst(*sc.B, buf, a, v);
}

template <int T>
__device__ __forceinline__ void tile_body(const TileDesc& d, const WorkItem& it, const TileBases& B,
                                          float2* A, float2* Bf, float2* tab, float2* xs, double* loss) {
  const int line0 = it.line0;
  const int G = it.G;
  const int N = d.nlen;
  FastDiv Gdiv = d.G_div;
  if (G != d.G) {
    Gdiv.d = G;
    unsigned s = 0;
    while ((1u << s) < (unsigned)G) ++s;
    Gdiv.s = s;
    Gdiv.m = G <= 1 ? 0u : (unsigned)(((1ull << 32) * ((1ull << s) - (unsigned)G)) / (unsigned)G + 1);
  }
  float2* sm = A;
  const IoDesc& in = d.in;
  const IoDesc& out = d.out;
  const i64 ibase = in.off + it.in_add;
  const i64 obase = out.off + it.out_add;

  // ------------------------------------------------------------ load
  // Loads are issued in groups of U independent read-only-path loads per
  // thread before any shared-memory write, so that many are in flight.
  if (d.kind == TILE_PLAIN || d.kind == TILE_CONVROW) {
    load_tile<T>(G, N, d.N_div, Gdiv, in.line_fast, [&](int l, int e, float2& v) -> int {
      int hi, lo;
      split_line(in, line0 + l, hi, lo);
      v = make_float2(0.f, 0.f);
      if (in.map == IO_AFFINE) {
        v = gldr(B, in.buf, ibase + (i64)hi * in.s_hi + (i64)lo * in.s_lo + (i64)e * in.s_e);
      } else if (in.map == IO_GT) {
        v = gldr(B, in.buf, ibase + (i64)hi * in.s_hi + (i64)gt_index(in, lo, e) * in.s_t);
      } else if (in.map == IO_TABLE) {  // zero beyond the table length mN
        const i64 q = lo * in.q_lo + e * in.q_e;
        if (q < in.mN) v = gldr(B, in.buf, ibase + (i64)hi * in.s_hi + (i64)__ldg(&in.tab[q]) * in.s_t);
      } else {  // IO_CHIRP: zero pad beyond the logical length
        const i64 q = lo * in.q_lo + e * in.q_e;
        if (q < in.mN) v = cmul(__ldg(&in.vec[q]), gldr(B, in.buf, ibase + (i64)hi * in.s_hi + q * in.s_t));
      }
      return spad(l * d.LS + e);
    }, sm);
    if (d.x0_cap >= 0 && threadIdx.x == 0) {
      for (int l = 0; l < G; ++l) {
        int hi, lo;
        split_line(in, line0 + l, hi, lo);
        if (lo == 0) B.c[BUF_WS][d.x0_cap + it.out_add + hi] = gld(B, in.buf, ibase + (i64)hi * in.s_hi);
      }
    }
  } else if (d.kind == TILE_GT) {
    // grid position (k, j) holds x[(n k + m j) mod N]  (Planned.hs:597-606);
    // inverting: k = i*cm mod m, j = i*cn mod n
    load_tile<T>(G, N, d.N_div, Gdiv, 0, [&](int l, int i, float2& v) -> int {
      int hi, lo;
      split_line(in, line0 + l, hi, lo);
      const int k = (int)mulmod((unsigned)i, (unsigned)d.gt_cm, d.gt_m_mod);
      const int j = (int)mulmod((unsigned)i, (unsigned)d.gt_cn, d.gt_n_mod);
      v = gldr(B, in.buf, io_addr(in, ibase, hi, lo, i));
      return spad(l * d.LS + k * d.gt_n + j);
    }, sm);
  } else if (d.kind == TILE_RADER) {
    // a[q] = x[g^-q]  (Permutation.apply rev res, Planned.hs:686-692): input
    // index r >= 1 with g^dlog(r) = r goes to q = (-dlog r) mod (p-1)
    const int m = N - 1;
    // a convolution carried by longer transforms (slen > p-1) is zero padded
    for (int q = threadIdx.x; q < G * (d.slen - m); q += T) {
      const int l = q / (d.slen - m);
      sm[spad(l * d.LS + m + (q - l * (d.slen - m)))] = make_float2(0.f, 0.f);
    }
    const int xs_pos = (int)(xs - sm);  // x0 of line l goes to xs[2 l]
    load_tile<T>(G, N, d.N_div, Gdiv, 0, [&](int l, int r, float2& v) -> int {
      int hi, lo;
      split_line(in, line0 + l, hi, lo);
      v = gldr(B, in.buf, io_addr(in, ibase, hi, lo, r));
      if (r == 0) return xs_pos + 2 * l;
      const int lg = __ldg(&d.dlog[r - 1]);
      return spad(l * d.LS + (lg == 0 ? 0 : m - lg));
    }, sm);
  } else {  // TILE_BLUESTEIN: chirp * x zero padded to M (Planned.hs:765-773)
    const int M = d.slen;
    load_tile<T>(G, M, d.S_div, Gdiv, 0, [&](int l, int e, float2& v) -> int {
      int hi, lo;
      split_line(in, line0 + l, hi, lo);
      v = make_float2(0.f, 0.f);
      if (e < N) v = cmul(__ldg(&d.vec_a[e]), gldr(B, in.buf, io_addr(in, ibase, hi, lo, e)));
      return spad(l * d.LS + e);
    }, sm);
  }
  __syncthreads();

  // ------------------------------------------------------------ phases
  sm = run_phase<T>(A, Bf, &d.ph[0], d.LS, G, tab);
  if (d.kind == TILE_RADER || d.kind == TILE_BLUESTEIN || d.kind == TILE_CONVROW) {
    // FFT(+1) -> * spectrum -> FFT(-1): the direction order of the reference's
    // convolveSingleSpectrumCyclicCache (Planned.hs:803-821)
    if (d.kind == TILE_RADER) {
      for (int l = threadIdx.x; l < G; l += T) xs[2 * l + 1] = sm[spad(l * d.LS)];  // sum res
      __syncthreads();
    }
    const int M = d.slen;
    if (d.kind == TILE_CONVROW) {
      if (d.dc_off >= 0 && threadIdx.x == 0) {
        for (int l = 0; l < G; ++l) {
          int hi, lo;
          split_line(out, line0 + l, hi, lo);
          if (lo == 0) B.c[BUF_WS][d.dc_off + it.out_add + hi] = sm[spad(l * d.LS)];
        }
      }
      __syncthreads();
      for_tile<T>(G, M, d.S_div, Gdiv, 0, [&](int l, int e) {
        int hi, lo;
        split_line(out, line0 + l, hi, lo);
        const int a = spad(l * d.LS + e);
        sm[a] = cmul(__ldg(&d.vec_b[lo * d.sq_lo + e * d.sq_e]), sm[a]);
      });
    } else {
      for_tile<T>(G, M, d.S_div, Gdiv, 0, [&](int l, int e) {
        const int a = spad(l * d.LS + e);
        sm[a] = cmul(__ldg(&d.vec_b[e]), sm[a]);
      });
    }
    __syncthreads();
  }
  if (d.nph > 1) sm = run_phase<T>(sm, sm == A ? Bf : A, &d.ph[1], d.LS, G, tab);

  // ------------------------------------------------------------ store
  StoreCtx sc{&B, 0.f, d.cot};
  if (d.kind == TILE_PLAIN || d.kind == TILE_CONVROW) {
    for_tile<T>(G, N, d.N_div, Gdiv, out.line_fast, [&](int l, int e) {
      int hi, lo;
      split_line(out, line0 + l, hi, lo);
      float2 v = sm[spad(l * d.LS + e)];
      if (d.ptw) {
        const unsigned t = mulmod((unsigned)lo, (unsigned)e, d.ptw_mod);
        const float2 wl = __ldg(&d.ptw[t & ((1 << d.ptwS_log2) - 1)]);
        const float2 wh = __ldg(&d.ptw[(1 << d.ptwS_log2) + (t >> d.ptwS_log2)]);
        float2 w = cmul(wh, wl);
        w.y *= -d.ptw_sign;
        v = cmul(v, w);
      }
      v = cscale(v, d.scale);
      const i64 hb = obase + (i64)hi * out.s_hi;
      if (out.map == IO_AFFINE) {
        store_final(sc, out.buf, hb + (i64)lo * out.s_lo + (i64)e * out.s_e, v);
      } else if (out.map == IO_GT) {
        store_final(sc, out.buf, hb + (i64)gt_index(out, lo, e) * out.s_t, v);
      } else if (out.map == IO_CHIRP) {
        const i64 q = lo * out.q_lo + e * out.q_e;
        if (q < out.mN) store_final(sc, out.buf, hb + q * out.s_t, cmul(__ldg(&out.vec[q]), v));
      } else {  // IO_RADER: c[q] -> out[g^q] = x0 + c[q]; q == 0 also out[0] = x0 + dc
        const i64 q = lo * out.q_lo + e * out.q_e;
        if (q >= out.mN) return;  // padding of a longer convolution
        // x0 lives with the transform's input: user input (placed like the
        // output) or a workspace region (placed like this step's input)
        const i64 x0_add = out.x0_buf == in.buf ? it.in_add : it.out_add;
        const float2 x0 = gld(B, out.x0_buf, out.x0_off + x0_add + (i64)hi * out.x0_shi);
        store_final(sc, out.buf, hb + (i64)__ldg(&out.tab[q]) * out.s_t, cadd(x0, v));
        if (q == 0) {
          const float2 dc = B.c[BUF_WS][out.dc_off + it.in_add + hi];
          store_final(sc, out.buf, hb, cadd(x0, cscale(dc, d.scale)));
        }
      }
    });
  } else if (d.kind == TILE_GT) {
    // out[r] = C[r mod n][r mod m]  (Planned.hs:608-617); C[q][p] sits at p*n + q
    for_tile<T>(G, N, d.N_div, Gdiv, 0, [&](int l, int r) {
      int hi, lo;
      split_line(out, line0 + l, hi, lo);
      const float2 v = sm[spad(l * d.LS + (int)mod_of((unsigned)r, d.gt_m_mod) * d.gt_n +
                               (int)mod_of((unsigned)r, d.gt_n_mod))];
      store_final(sc, out.buf, io_addr(out, obase, hi, lo, r), cscale(v, d.scale));
    });
  } else if (d.kind == TILE_RADER) {
    // out[0] = x0 + sum res; out[r] = x0 + c[dlog r]  (Planned.hs:686-692)
    for_tile<T>(G, N, d.N_div, Gdiv, 0, [&](int l, int r) {
      int hi, lo;
      split_line(out, line0 + l, hi, lo);
      const float2 x0 = xs[2 * l];
      const float2 v = r == 0 ? xs[2 * l + 1] : sm[spad(l * d.LS + __ldg(&d.dlog[r - 1]))];
      store_final(sc, out.buf, io_addr(out, obase, hi, lo, r), cscale(cadd(x0, v), d.scale));
    });
  } else {  // Bluestein: y = chirp * (take N c)
    for_tile<T>(G, N, d.N_div, Gdiv, 0, [&](int l, int e) {
      int hi, lo;
      split_line(out, line0 + l, hi, lo);
      const float2 v = cmul(__ldg(&d.vec_a[e]), sm[spad(l * d.LS + e)]);
      store_final(sc, out.buf, io_addr(out, obase, hi, lo, e), cscale(v, d.scale));
    });
  }

  if (d.cot && loss) {
    float v = sc.loss;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();  // the per-line scratch is free again: reuse it for the reduction
    float* red = reinterpret_cast<float*>(xs);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
      double s = 0;
      for (int w = 0; w < T / 32; ++w) s += red[w];
      atomicAdd(loss, s);
    }
  }
}

template <int T>
__global__ void __launch_bounds__(T, (T <= 256 ? 768 / T : 1)) tile_kernel(const TileDesc* __restrict__ descs,
                                                 const WorkItem* __restrict__ items, TileBases bases,
                                                 double* loss, int smem_data) {
  extern __shared__ float4 smem4[];
  float2* smem = reinterpret_cast<float2*>(smem4);
  const WorkItem it = items[blockIdx.x];
  // shared layout: [descriptor] [A: smem_data] [B: smem_data] [tables] [scratch 2G]
  TileDesc* d = reinterpret_cast<TileDesc*>(smem);
  {
    const int words = (int)(sizeof(TileDesc) / 4);
    const int* srcw = reinterpret_cast<const int*>(descs + it.desc);
    int* dstw = reinterpret_cast<int*>(d);
    for (int i = threadIdx.x; i < words; i += T) dstw[i] = srcw[i];
  }
  __syncthreads();
  const int desc_f2 = (int)((sizeof(TileDesc) + 15) / 16 * 2);
  float2* A = smem + desc_f2;
  float2* Bf = A + smem_data;
  float2* tab = Bf + smem_data;
  float2* xs = tab + d->tw_total;
  for (int i = threadIdx.x; i < d->tw_total; i += T) tab[i] = d->tw_src[i];
  tile_body<T>(*d, it, bases, A, Bf, tab, xs, loss);
}

size_t tile_smem_bytes(int smem_data, int tw_total, int G) {
  return (sizeof(TileDesc) + 15) / 16 * 16 + (size_t)(2 * smem_data + tw_total + 2 * G) * sizeof(float2);
}

// Raises the kernel's dynamic shared-memory limit to what the device allows
// once per process (the opt-in limit less the kernel's static usage).
template <int T>
static cudaError_t launch_t(const LaunchSpec& L, const TileBases& bases, double* loss, cudaStream_t st) {
  static int limit = -1;
  if (limit < 0) {
    int dev = 0, optin = 0;
    cudaFuncAttributes fa;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, tile_kernel<T>);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(tile_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               optin - (int)fa.sharedSizeBytes);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return e;
    }
    limit = optin - (int)fa.sharedSizeBytes;
  }
  if (L.smem_bytes > (size_t)limit) return cudaErrorInvalidValue;
  tile_kernel<T><<<L.nitems, T, L.smem_bytes, st>>>(L.descs, L.items, bases, loss, L.smem_data);
  return cudaGetLastError();
}

cudaError_t launch_tiles(const LaunchSpec& L, const TileBases& bases, double* loss, cudaStream_t st) {
  if (L.nitems <= 0) return cudaSuccess;
  switch (L.threads) {
    case 512: return launch_t<512>(L, bases, loss, st);
    case 128: return launch_t<128>(L, bases, loss, st);
    default: return launch_t<256>(L, bases, loss, st);
  }
}

}  // namespace af
