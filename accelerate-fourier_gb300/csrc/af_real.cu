// af_real.cu -- element-wise kernels around the complex transforms: the real
// transforms through a half-length complex transform (Real.hs:49-121), the
// two-real-signal untangle/entangle maps (Real.hs:129-240) and the spectrum
// product of the cyclic convolution (Planned.hs:779-821).
#include "af_internal.h"

namespace AF_NS {

__device__ __forceinline__ cx cp_ld(const CPtr& p, i64 i) {
  if (p.c) return p.c[i];
  return make_cx(p.re[i], p.im[i]);
}
__device__ __forceinline__ void cp_st(const CPtr& p, i64 i, cx v) {
  if (p.c) p.c[i] = v;
  else { p.re[i] = v.x; p.im[i] = v.y; }
}
__device__ __forceinline__ cx i_times(cx a) { return make_cx(-a.y, a.x); }

static unsigned grid_of(i64 total) {
  i64 b = (total + 255) / 256;
  if (b > 152 * 32) b = 152 * 32;
  return (unsigned)(b < 1 ? 1 : b);
}

// toSpectrum (Real.hs:49-70).  Z: rows of n2 = N/2 complex values (the
// half-length transform of the real row read as complex pairs).
//   xp = (Z + rev Z)/2, xm = (Z - rev Z)/2
//   even = Re xp + i Im xm, odd = (i W_N^k) (Re xm + i Im xp)
//   out = (even - odd) ++ (even + odd)           (nout = N)
// With nout = n2 + 1 only the first half and the Nyquist bin are written.
__global__ void real_untangle_kernel(const cx* __restrict__ Z, CPtr out, i64 n2, i64 nout, i64 rows,
                                     const cx* __restrict__ tab, int S_log2) {
  const i64 total = rows * n2;
  for (i64 q = (i64)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (i64)gridDim.x * blockDim.x) {
    const i64 b = q / n2, k = q - b * n2;
    const cx* z = Z + b * n2;
    const cx zk = z[k], zr = z[k == 0 ? 0 : n2 - k];
    const cx xp = cscale(cadd(zk, zr), 0.5f), xm = cscale(csub(zk, zr), 0.5f);
    const cx ev = make_cx(xp.x, xm.y);
    const cx oi = make_cx(xm.x, xp.y);
    const cx od = cmul(i_times(tw_lookup(tab, S_log2, (int)k, -1.f)), oi);
    cp_st(out, b * nout + k, csub(ev, od));
    if (nout == 2 * n2) cp_st(out, b * nout + n2 + k, cadd(ev, od));
    else if (k == 0) cp_st(out, b * nout + n2, cadd(ev, od));
  }
}

// fromSpectrum's pre-map (Real.hs:92-108): f[k] = (s[k] + s[k+n2])
// + (i W_N^-k) (s[k] - s[k+n2]), k < n2; f then goes through the inverse
// transform of n2 and is read back as N reals.  With herm != 0 the spectrum
// is first made self-adjoint, s = (g + conj(rev g))/2: that turns the map
// into the adjoint of toSpectrum (Re(DFT^H g) = fromSpectrum(s)).
__global__ void real_entangle_kernel(CPtr spec, cx* __restrict__ f, i64 n2, i64 rows,
                                     const cx* __restrict__ tab, int S_log2, int herm) {
  const i64 total = rows * n2, N = 2 * n2;
  for (i64 q = (i64)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (i64)gridDim.x * blockDim.x) {
    const i64 b = q / n2, k = q - b * n2;
    const i64 row = b * N;
    cx s0 = cp_ld(spec, row + k), s1 = cp_ld(spec, row + k + n2);
    if (herm) {
      const cx r0 = cp_ld(spec, row + (k == 0 ? 0 : N - k));
      const cx r1 = cp_ld(spec, row + (n2 - k));
      s0 = cscale(cadd(s0, conjf2(r0)), 0.5f);
      s1 = cscale(cadd(s1, conjf2(r1)), 0.5f);
    }
    const cx fe = cadd(s0, s1);
    const cx fo = cmul(i_times(tw_lookup(tab, S_log2, (int)k, 1.f)), csub(s0, s1));
    f[b * n2 + k] = cadd(fe, fo);
  }
}

// untangleSpectra / untangleSpectra2d (Real.hs:168-195): a = S[y,x],
// b = S[-y mod h, -x mod w]: A = (a + conj b)/2, B = (a - conj b)(-i/2).
// The 1-D form is h = 1.
__global__ void untangle_kernel(CPtr S, CPtr A, CPtr B, i64 h, i64 w, i64 total) {
  const i64 img = h * w;
  for (i64 q = (i64)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (i64)gridDim.x * blockDim.x) {
    const i64 bi = q / img, r = q - bi * img;
    const i64 y = r / w, x = r - y * w;
    const i64 ry = y == 0 ? 0 : h - y, rx = x == 0 ? 0 : w - x;
    const cx a = cp_ld(S, q);
    const cx bc = conjf2(cp_ld(S, bi * img + ry * w + rx));
    cp_st(A, q, cscale(cadd(a, bc), 0.5f));
    const cx d = csub(a, bc);
    cp_st(B, q, make_cx(0.5f * d.y, -0.5f * d.x));
  }
}

// Cyclic.reverse2d (Cyclic.hs:30-39): out[y, x] = in[-y mod h, -x mod w].
__global__ void reverse2d_kernel(CPtr in, CPtr out, i64 h, i64 w, i64 total) {
  const i64 img = h * w;
  for (i64 q = (i64)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (i64)gridDim.x * blockDim.x) {
    const i64 bi = q / img, r = q - bi * img;
    const i64 y = r / w, x = r - y * w;
    const i64 ry = y == 0 ? 0 : h - y, rx = x == 0 ? 0 : w - x;
    cp_st(out, q, cp_ld(in, bi * img + ry * w + rx));
  }
}

// entangleSpectra (Real.hs:207-236): out = c + d i (the first component of
// entangleCoefficient).
__global__ void entangle_kernel(CPtr C, CPtr D, CPtr out, i64 total) {
  for (i64 q = (i64)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (i64)gridDim.x * blockDim.x) {
    const cx c = cp_ld(C, q), d = cp_ld(D, q);
    cp_st(out, q, cadd(c, i_times(d)));
  }
}

// convolveCyclicCache (Planned.hs:793-821): gx = (gx * (1/n)) * gy.
__global__ void conv_mul_kernel(cx* __restrict__ gx, const cx* __restrict__ gy, rl s, i64 total) {
  for (i64 q = (i64)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (i64)gridDim.x * blockDim.x)
    gx[q] = cmul(cscale(gx[q], s), gy[q]);
}

cudaError_t launch_real_untangle(const cx* Z, CPtr out, i64 n2, i64 nout, i64 rows, const cx* tab,
                                 int S_log2, cudaStream_t st) {
  const i64 total = rows * n2;
  if (total <= 0) return cudaSuccess;
  real_untangle_kernel<<<grid_of(total), 256, 0, st>>>(Z, out, n2, nout, rows, tab, S_log2);
  return cudaGetLastError();
}
cudaError_t launch_real_entangle(CPtr spec, cx* f, i64 n2, i64 rows, const cx* tab, int S_log2, int herm,
                                 cudaStream_t st) {
  const i64 total = rows * n2;
  if (total <= 0) return cudaSuccess;
  real_entangle_kernel<<<grid_of(total), 256, 0, st>>>(spec, f, n2, rows, tab, S_log2, herm);
  return cudaGetLastError();
}
cudaError_t launch_untangle(CPtr S, CPtr A, CPtr B, i64 h, i64 w, i64 total, cudaStream_t st) {
  if (total <= 0) return cudaSuccess;
  untangle_kernel<<<grid_of(total), 256, 0, st>>>(S, A, B, h, w, total);
  return cudaGetLastError();
}
cudaError_t launch_reverse2d(CPtr in, CPtr out, i64 h, i64 w, i64 total, cudaStream_t st) {
  if (total <= 0) return cudaSuccess;
  reverse2d_kernel<<<grid_of(total), 256, 0, st>>>(in, out, h, w, total);
  return cudaGetLastError();
}
cudaError_t launch_entangle(CPtr C, CPtr D, CPtr out, i64 total, cudaStream_t st) {
  if (total <= 0) return cudaSuccess;
  entangle_kernel<<<grid_of(total), 256, 0, st>>>(C, D, out, total);
  return cudaGetLastError();
}
cudaError_t launch_conv_mul(cx* gx, const cx* gy, rl s, i64 total, cudaStream_t st) {
  if (total <= 0) return cudaSuccess;
  conv_mul_kernel<<<grid_of(total), 256, 0, st>>>(gx, gy, s, total);
  return cudaGetLastError();
}

}  // namespace af
