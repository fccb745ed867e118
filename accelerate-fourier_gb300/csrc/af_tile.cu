// af_tile.cu -- the shared-memory tile FFT kernel of libaf.
//
// One CTA transforms G lines (independent transforms) held in shared memory:
// load (through the tile kind's index map) -> one or two Stockham FFT phases
// -> store (through the inverse map, with four-step twiddle and scale).  A
// phase is a sequence of Stockham passes of radix 2,3,4,5,7,8,11,13 or 16
// that alternate between two shared-memory buffers.
//
// Tile kinds restate the reference's algorithms (file:line relative to the
// accelerate-fourier project):
//   TILE_PLAIN      Cooley-Tukey / split-radix leaves (Fourier/Planned.hs:473-557)
//   TILE_GT         Good-Thomas with the reference's CRT maps (Planned.hs:584-617)
//   TILE_RADER      Rader's algorithm (Planned.hs:646-692, Permutation.hs:24-80)
//   TILE_BLUESTEIN  Bluestein / chirp-z (Planned.hs:744-773, Private.hs:428-436)
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

// Runs every pass of a phase staged in shared memory; returns the buffer that
// holds the result (the two buffers alternate pass by pass).
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

__device__ __forceinline__ i64 io_addr(const IoDesc& io, int line, int e) {
  const int hi = (int)fdiv((unsigned)line, io.lo_div);
  const int lo = line - hi * (int)io.lo_div.d;
  return (i64)hi * io.s_hi + (i64)lo * io.s_lo + (i64)e * io.s_e;
}
__device__ __forceinline__ float2 io_load(const IoDesc& io, i64 a) {
  if (io.c) return io.c[a];
  return make_float2(io.re[a], io.im[a]);
}
__device__ __forceinline__ void io_store(const IoDesc& io, i64 a, float2 v) {
  if (io.c) io.c[a] = v;
  else { io.re[a] = v.x; io.im[a] = v.y; }
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

template <int T>
__global__ void __launch_bounds__(T) tile_kernel(const TileDesc d) {
  extern __shared__ float2 smem[];
  const int line0 = blockIdx.x * d.G;
  const int G = min(d.G, d.nlines - line0);
  if (G <= 0) return;
  // shared layout: [A: spad(G*LS)] [B: spad(G*LS)] [tables] [scratch 2G] [phase descriptors]
  const int dlen = spad(d.G * d.LS);
  float2* A = smem;
  float2* B = smem + dlen;
  float2* tab = B + dlen;
  float2* xs = tab + d.tw_total;
  FftPhase* phs = reinterpret_cast<FftPhase*>(xs + 2 * d.G);
  for (int i = threadIdx.x; i < d.tw_total; i += T) tab[i] = d.tw_src[i];
  {
    const int words = (int)(sizeof(FftPhase) * AF_MAXPH / 4);
    const int* srcw = reinterpret_cast<const int*>(&d.ph[0]);
    int* dstw = reinterpret_cast<int*>(phs);
    for (int i = threadIdx.x; i < words; i += T) dstw[i] = srcw[i];
  }

  const int N = d.nlen;
  // a partial last CTA walks its G lines with a divider computed here
  FastDiv Gdiv = d.G_div;
  if (G != d.G) {
    Gdiv.d = G;
    unsigned s = 0;
    while ((1u << s) < (unsigned)G) ++s;
    Gdiv.s = s;
    Gdiv.m = G <= 1 ? 0u : (unsigned)(((1ull << 32) * ((1ull << s) - (unsigned)G)) / (unsigned)G + 1);
  }
  float2* sm = A;

  // ------------------------------------------------------------ load
  if (d.kind == TILE_PLAIN) {
    for_tile<T>(G, N, d.N_div, Gdiv, d.in.line_fast, [&](int l, int e) {
      sm[spad(l * d.LS + e)] = io_load(d.in, io_addr(d.in, line0 + l, e));
    });
  } else if (d.kind == TILE_GT) {
    // grid position (k, j) holds x[(n k + m j) mod N]  (Planned.hs:597-606);
    // inverting: k = i*cm mod m, j = i*cn mod n
    for_tile<T>(G, N, d.N_div, Gdiv, 0, [&](int l, int i) {
      const int k = (int)(((i64)i * d.gt_cm) % d.gt_m);
      const int j = (int)(((i64)i * d.gt_cn) % d.gt_n);
      sm[spad(l * d.LS + k * d.gt_n + j)] = io_load(d.in, io_addr(d.in, line0 + l, i));
    });
  } else if (d.kind == TILE_RADER) {
    // a[q] = x[g^-q]  (Permutation.apply rev res, Planned.hs:686-692): input
    // index r >= 1 with g^dlog(r) = r goes to q = (-dlog r) mod (p-1)
    const int m = N - 1;
    for_tile<T>(G, N, d.N_div, Gdiv, 0, [&](int l, int r) {
      const float2 v = io_load(d.in, io_addr(d.in, line0 + l, r));
      if (r == 0) {
        xs[2 * l] = v;
      } else {
        const int lg = __ldg(&d.dlog[r - 1]);
        sm[spad(l * d.LS + (lg == 0 ? 0 : m - lg))] = v;
      }
    });
  } else {  // TILE_BLUESTEIN: chirp * x zero padded to M (Planned.hs:765-773)
    const int M = d.slen;
    for_tile<T>(G, M, d.S_div, Gdiv, 0, [&](int l, int e) {
      float2 v = make_float2(0.f, 0.f);
      if (e < N) v = cmul(__ldg(&d.vec_a[e]), io_load(d.in, io_addr(d.in, line0 + l, e)));
      sm[spad(l * d.LS + e)] = v;
    });
  }
  __syncthreads();

  // ------------------------------------------------------------ phases
  sm = run_phase<T>(A, B, &phs[0], d.LS, G, tab);
  if (d.kind == TILE_RADER || d.kind == TILE_BLUESTEIN) {
    // conv tiles: FFT(+1) -> * spectrum -> FFT(-1), the direction order of the
    // reference's convolveSingleSpectrumCyclicCache (Planned.hs:803-821)
    if (d.kind == TILE_RADER) {
      for (int l = threadIdx.x; l < G; l += T) xs[2 * l + 1] = sm[spad(l * d.LS)];  // sum res
      __syncthreads();
    }
    const int M = d.slen;
    for_tile<T>(G, M, d.S_div, Gdiv, 0, [&](int l, int e) {
      const int a = spad(l * d.LS + e);
      sm[a] = cmul(__ldg(&d.vec_b[e]), sm[a]);
    });
    __syncthreads();
  }
  if (d.nph > 1) sm = run_phase<T>(sm, sm == A ? B : A, &phs[1], d.LS, G, tab);

  // ------------------------------------------------------------ store
  if (d.kind == TILE_PLAIN) {
    for_tile<T>(G, N, d.N_div, Gdiv, d.out.line_fast, [&](int l, int e) {
      float2 v = sm[spad(l * d.LS + e)];
      if (d.ptw) {
        const int line = line0 + l;
        const int hi = (int)fdiv((unsigned)line, d.out.lo_div);
        const i64 col = (i64)(line - hi * (int)d.out.lo_div.d) * d.ptw_col_mul;
        const i64 t = (col * e) % d.ptwN;
        const float2 lo = __ldg(&d.ptw[t & ((1 << d.ptwS_log2) - 1)]);
        const float2 hh = __ldg(&d.ptw[(1 << d.ptwS_log2) + (t >> d.ptwS_log2)]);
        float2 w = cmul(hh, lo);
        w.y *= -d.ptw_sign;
        v = cmul(v, w);
      }
      io_store(d.out, io_addr(d.out, line0 + l, e), cscale(v, d.scale));
    });
  } else if (d.kind == TILE_GT) {
    // out[r] = C[r mod n][r mod m]  (Planned.hs:608-617); C[q][p] sits at p*n + q
    for_tile<T>(G, N, d.N_div, Gdiv, 0, [&](int l, int r) {
      const float2 v = sm[spad(l * d.LS + (r % d.gt_m) * d.gt_n + (r % d.gt_n))];
      io_store(d.out, io_addr(d.out, line0 + l, r), cscale(v, d.scale));
    });
  } else if (d.kind == TILE_RADER) {
    // out[0] = x0 + sum res; out[r] = x0 + c[dlog r]  (Planned.hs:686-692)
    for_tile<T>(G, N, d.N_div, Gdiv, 0, [&](int l, int r) {
      const float2 x0 = xs[2 * l];
      const float2 v = r == 0 ? xs[2 * l + 1] : sm[spad(l * d.LS + __ldg(&d.dlog[r - 1]))];
      io_store(d.out, io_addr(d.out, line0 + l, r), cscale(cadd(x0, v), d.scale));
    });
  } else {  // Bluestein: y = chirp * (take N c)
    for_tile<T>(G, N, d.N_div, Gdiv, 0, [&](int l, int e) {
      const float2 v = cmul(__ldg(&d.vec_a[e]), sm[spad(l * d.LS + e)]);
      io_store(d.out, io_addr(d.out, line0 + l, e), cscale(v, d.scale));
    });
  }
}

size_t tile_smem_bytes(const TileDesc& d) {
  const int data = d.G * d.LS;
  return (size_t)(2 * (data + (data >> 4)) + d.tw_total + 2 * d.G) * sizeof(float2) +
         sizeof(FftPhase) * AF_MAXPH;
}

template <int T>
static cudaError_t launch_t(const TileDesc& d, cudaStream_t st) {
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(tile_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  const int grid = (d.nlines + d.G - 1) / d.G;
  tile_kernel<T><<<grid, T, tile_smem_bytes(d), st>>>(d);
  return cudaGetLastError();
}

cudaError_t launch_tile(const TileDesc& d, int threads, cudaStream_t st) {
  if (d.nlines <= 0) return cudaSuccess;
  if (threads == 512) return launch_t<512>(d, st);
  if (threads == 128) return launch_t<128>(d, st);
  return launch_t<256>(d, st);
}

}  // namespace af
