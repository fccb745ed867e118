// af_kernels.cu -- libaf's element-wise kernels: exact integer index maps
// (Good-Thomas CRT maps, Rader permutations, cyclic reverse), pointwise
// spectrum products, and the FP64 generators of twiddle, chirp and Rader
// kernel tables.
#include <algorithm>

#include "af_internal.h"

namespace AF_NS {

__device__ __forceinline__ i64 view_addr(const IoDesc& io, i64 line, i64 e) {
  const i64 lo_cnt = io.lo_div.d;
  const i64 hi = line / lo_cnt;
  const i64 lo = line - hi * lo_cnt;
  return io.off + hi * io.s_hi + lo * io.s_lo + e * io.s_e;
}
__device__ __forceinline__ cx vload(const TileBases& B, const IoDesc& io, i64 a) {
  if (B.c[io.buf]) return B.c[io.buf][a];
  return make_cx(B.re[io.buf][a], B.im[io.buf][a]);
}
__device__ __forceinline__ void vstore(const TileBases& B, const IoDesc& io, i64 a, cx v) {
  if (B.c[io.buf]) B.c[io.buf][a] = v;
  else { B.re[io.buf][a] = v.x; B.im[io.buf][a] = v.y; }
}

__global__ void map_kernel(const MapDesc d, const TileBases B) {
  const i64 total = d.nlines * d.nout;
  cx* ws = B.c[BUF_WS];
  for (i64 q = (i64)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (i64)gridDim.x * blockDim.x) {
    const i64 line = q / d.nout;
    const i64 e = q - line * d.nout;
    cx v;
    switch (d.mode) {
      case MAP_COPY: v = vload(B, d.in, view_addr(d.in, line, e)); break;
      case MAP_GT_IN: {
        const i64 k = e / d.n, j = e - k * d.n;
        v = vload(B, d.in, view_addr(d.in, line, (d.n * k + d.m * j) % d.nm));
        break;
      }
      case MAP_GT_OUT:
        v = vload(B, d.in, view_addr(d.in, line, (e % d.n) * d.m + (e % d.m)));
        break;
      case MAP_TABLE:
        v = vload(B, d.in, view_addr(d.in, line, d.tab[e]));
        if (d.x0_ws >= 0 && e == 0) ws[d.x0_ws + line] = vload(B, d.in, view_addr(d.in, line, 0));
        break;
      case MAP_RADER_OUT: {
        const cx x0 = ws[d.x0_ws + line];
        const cx c = e == 0 ? ws[d.dc_ws + line] : vload(B, d.in, view_addr(d.in, line, d.tab[e - 1]));
        v = cadd(x0, c);
        break;
      }
      case MAP_CHIRP_IN:
        v = e < d.n ? cmul(d.vec[e], vload(B, d.in, view_addr(d.in, line, e))) : make_cx(0.f, 0.f);
        break;
      case MAP_MUL: {
        const cx u = vload(B, d.in, view_addr(d.in, line, e));
        if (d.dc_ws >= 0 && e == 0) ws[d.dc_ws + line] = u;
        v = cmul(d.vec[e], u);
        break;
      }
      case MAP_SCALE: v = cscale(vload(B, d.in, view_addr(d.in, line, e)), d.scale); break;
      case MAP_TWIDDLE: {
        const i64 col = line % d.m;
        const i64 t = (col * e) % d.n;
        const cx lo = d.tab_tw[t & ((1 << d.tw_log2) - 1)];
        const cx hi = d.tab_tw[(1 << d.tw_log2) + (t >> d.tw_log2)];
        cx w = cmul(hi, lo);
        w.y *= -d.tw_sign;
        v = cmul(vload(B, d.in, view_addr(d.in, line, e)), w);
        break;
      }
      default: {  // MAP_REVERSE
        const i64 s = e == 0 ? 0 : d.n - e;
        v = vload(B, d.in, view_addr(d.in, line, s));
        break;
      }
    }
    vstore(B, d.out, view_addr(d.out, line, e), v);
  }
}

cudaError_t launch_map(const MapDesc& d, const TileBases& bases, cudaStream_t st) {
  const i64 total = d.nlines * d.nout;
  if (total <= 0) return cudaSuccess;
  i64 blocks = (total + 255) / 256;
  if (blocks > 152 * 32) blocks = 152 * 32;
  map_kernel<<<(unsigned)blocks, 256, 0, st>>>(d, bases);
  return cudaGetLastError();
}

// ------------------------------------------------------------- FP64 tables
__global__ void twiddle_table_kernel(cx* dst, i64 n, int S, int H) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= S + H) return;
  i64 t = i < S ? (i64)i : (i64)(i - S) * S;
  t %= n;
  double s, c;
  sincospi(2.0 * (double)t / (double)n, &s, &c);
  dst[i] = make_cx((rl)c, (rl)-s);
}
cudaError_t launch_twiddle_table(cx* dst, i64 n, int S, int H, cudaStream_t st) {
  const int tot = S + H;
  twiddle_table_kernel<<<(tot + 255) / 256, 256, 0, st>>>(dst, n, S, H);
  return cudaGetLastError();
}

__global__ void chirp_kernel(double2* dst, i64 pad, i64 len, int sign, i64 count) {
  const i64 k = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  const i64 sk = pad > 2 * k ? k : k - pad;
  const i64 two_len = 2 * len;
  // pi * sk^2 / len = pi * (sk^2 mod 2 len) / len, exact in integers
  const unsigned long long r = (unsigned long long)(((__int128)sk * sk) % two_len);
  double s, c;
  sincospi((double)r / (double)len, &s, &c);
  dst[k] = make_double2(c, sign * s);
}
cudaError_t launch_chirp(double2* dst, i64 pad, i64 len, int sign, i64 count, cudaStream_t st) {
  chirp_kernel<<<(unsigned)((count + 255) / 256), 256, 0, st>>>(dst, pad, len, sign, count);
  return cudaGetLastError();
}

__device__ __forceinline__ i64 mulmod(i64 a, i64 b, i64 m) { return (i64)(((__int128)a * b) % m); }

__global__ void rader_kernel_kernel(double2* dst, i64 p, i64 g, int sign) {
  const i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p - 1) return;
  // g^i mod p by square and multiply
  i64 r = 1, b = g % p, e = i;
  while (e > 0) {
    if (e & 1) r = mulmod(r, b, p);
    b = mulmod(b, b, p);
    e >>= 1;
  }
  double s, c;
  sincospi(2.0 * (double)r / (double)p, &s, &c);
  dst[i] = make_double2(c, sign * s);
}
cudaError_t launch_rader_kernel(double2* dst, i64 p, i64 g, int sign, cudaStream_t st) {
  const i64 cnt = p - 1;
  rader_kernel_kernel<<<(unsigned)((cnt + 255) / 256), 256, 0, st>>>(dst, p, g, sign);
  return cudaGetLastError();
}

// The input of a spectrum table: k (m entries) placed periodically over M >= m
// (kk[i] = k[i] for i < m, kk[M - j] = k[m - j] for 0 < j < m when M > m,
// zero elsewhere), conjugated when conj != 0.
__global__ void spectrum_input_kernel(const double2* k, i64 m, double2* kk, i64 M, int conj) {
  for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < M; i += (i64)gridDim.x * blockDim.x) {
    double2 v = make_double2(0.0, 0.0);
    if (i < m) v = k[i];
    else if (M > m && M - i < m) v = k[m - (M - i)];
    if (conj) v.y = -v.y;
    kk[i] = v;
  }
}
cudaError_t launch_spectrum_input(const double2* k, i64 m, double2* kk, i64 M, int conj, cudaStream_t st) {
  const i64 blocks = std::min<i64>((M + 255) / 256, 4096);
  spectrum_input_kernel<<<(unsigned)blocks, 256, 0, st>>>(k, m, kk, M, conj);
  return cudaGetLastError();
}

// out[i] = S[i] * s in the element type (FP64 values rounded for Complex Float)
__global__ void scale_round_kernel(const double2* S, cx* out, i64 n, double s) {
  for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x)
    out[i] = make_cx((rl)(S[i].x * s), (rl)(S[i].y * s));
}
cudaError_t launch_scale_round(const double2* S, cx* out, i64 n, double s, cudaStream_t st) {
  const i64 blocks = std::min<i64>((n + 255) / 256, 4096);
  scale_round_kernel<<<(unsigned)blocks, 256, 0, st>>>(S, out, n, s);
  return cudaGetLastError();
}

}  // namespace af
