// af_karatsuba.cu -- Karatsuba linear convolution (Convolution/Adhoc.hs:36-98)
// and its cyclic and complex combinators (Convolution/Adhoc.hs:104-133).
//
// The reference's loop form, level by level on the GPU:
//   reorder  (karatsubaReorder, Adhoc.hs:66-79): rows of length len become
//            3 row blocks of length l2 = ceil(len/2): [xl | xl+xr | xr], xr
//            zero padded, the block index outermost among the rows;
//   leaves   (Adhoc.hs:51-52): z = x * y once every row has length 1;
//   combine  (karatsubaGo, Adhoc.hs:81-98): z[k] = zl[k] + zc[k-l2] +
//            zr[k-2 l2] with zc = zm - (zl + zr) and zero outside each row
//            (indexPad, Convolution/Private.hs:21-26).
// Every level is one launch over all rows of all batch items.  The arithmetic
// is the reference's in the same order (additions and one product per leaf),
// so integer results are exact and floating-point results are those of the
// same loop run on the CPU.
#include <cstring>
#include <string>
#include <vector>

#include "af_host.h"

namespace af {

static unsigned kgrid(i64 total) {
  i64 b = (total + 255) / 256;
  if (b > 152 * 64) b = 152 * 64;
  return (unsigned)(b < 1 ? 1 : b);
}

// level rows: [batch][cnt][len] -> [batch][3][cnt][l2]
template <class Tin, class T>
__global__ void kara_reorder(const Tin* __restrict__ xs, const Tin* __restrict__ ys, T* __restrict__ nx,
                             T* __restrict__ ny, i64 batch, i64 cnt, i64 len, i64 l2) {
  const i64 per = cnt * l2, total = batch * per;
  for (i64 q = (i64)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (i64)gridDim.x * blockDim.x) {
    const i64 b = q / per, rj = q - b * per;
    const i64 r = rj / l2, j = rj - r * l2;
    const i64 src = (b * cnt + r) * len + j;
    const bool has_r = l2 + j < len;
    const T xl = (T)xs[src], yl = (T)ys[src];
    const T xr = has_r ? (T)xs[src + l2] : T(0);
    const T yr = has_r ? (T)ys[src + l2] : T(0);
    const i64 d0 = (b * 3 * cnt + r) * l2 + j;
    nx[d0] = xl; nx[d0 + per] = xl + xr; nx[d0 + 2 * per] = xr;
    ny[d0] = yl; ny[d0 + per] = yl + yr; ny[d0 + 2 * per] = yr;
  }
}

template <class Tin, class T>
__global__ void kara_leaf(const Tin* __restrict__ x, const Tin* __restrict__ y, T* __restrict__ z, i64 total) {
  for (i64 q = (i64)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (i64)gridDim.x * blockDim.x)
    z[q] = (T)x[q] * (T)y[q];
}

// [batch][3 n3][zcur] -> [batch][n3][zlen]
template <class T>
__global__ void kara_combine(const T* __restrict__ zz, T* __restrict__ nz, i64 batch, i64 n3, i64 zcur, i64 zlen,
                             i64 xlen) {
  const i64 per = n3 * zlen, total = batch * per;
  for (i64 q = (i64)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (i64)gridDim.x * blockDim.x) {
    const i64 b = q / per, rk = q - b * per;
    const i64 r = rk / zlen, k = rk - r * zlen;
    const T* zl = zz + (b * 3 * n3 + r) * zcur;
    const T* zm = zl + n3 * zcur;
    const T* zr = zm + n3 * zcur;
    const T lv = k < zcur ? zl[k] : T(0);
    const i64 kc = k - xlen, kr = k - 2 * xlen;
    const T cv = (kc >= 0 && kc < zcur) ? zm[kc] - (zl[kc] + zr[kc]) : T(0);
    const T rv = (kr >= 0 && kr < zcur) ? zr[kr] : T(0);
    nz[q] = lv + cv + rv;
  }
}

// Convolution.Adhoc.cyclic (Adhoc.hs:104-111): out[k] = z[k] + z[k+L]
// (zero where k + L is past the 2L-1 values of z).
template <class T>
__global__ void kara_fold(const T* __restrict__ z, T* __restrict__ out, i64 batch, i64 L) {
  const i64 zl = 2 * L - 1, total = batch * L;
  for (i64 q = (i64)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (i64)gridDim.x * blockDim.x) {
    const i64 b = q / L, k = q - b * L;
    out[q] = z[b * zl + k] + (k + L < zl ? z[b * zl + k + L] : T(0));
  }
}

// Convolution.Adhoc.complex (Adhoc.hs:117-128): inputs of the three real
// convolutions and the combination of their results.
template <class T>
__global__ void kara_sum(const T* __restrict__ a, const T* __restrict__ b, T* __restrict__ s, i64 total) {
  for (i64 q = (i64)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (i64)gridDim.x * blockDim.x)
    s[q] = a[q] + b[q];
}
template <class T>
__global__ void kara_complex_combine(const T* __restrict__ rr, const T* __restrict__ ii, const T* __restrict__ mm,
                                     T* __restrict__ zre, T* __restrict__ zim, i64 total) {
  for (i64 q = (i64)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (i64)gridDim.x * blockDim.x) {
    const T a = rr[q], c = ii[q];
    zre[q] = a - c;
    zim[q] = mm[q] - (a + c);
  }
}

static void kcheck(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw AfError(AF_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// Stream-ordered scratch (cudaMallocAsync), released on the same stream.
struct Scratch {
  void* p = nullptr;
  cudaStream_t st;
  Scratch(size_t bytes, cudaStream_t s) : st(s) {
    if (bytes && cudaMallocAsync(&p, bytes, st) != cudaSuccess) {
      cudaGetLastError();
      throw AfError(AF_ERR_ALLOC, "Karatsuba scratch allocation failed");
    }
  }
  ~Scratch() {
    if (p) cudaFreeAsync(p, st);
  }
};

// Level sizes of the loop form for rows of length L: lens[0] = L, ...,
// lens[D] = 1; cnt_d = 3^d.
static std::vector<i64> kara_lens(i64 L) {
  std::vector<i64> lens{L};
  while (lens.back() > 1) lens.push_back((lens.back() + 1) / 2);
  return lens;
}

static const i64 kKaraMaxElems = (i64)1 << 31;

static i64 kara_scratch_elems(i64 L, i64 batch, i64* xmax, i64* zmax) {
  const std::vector<i64> lens = kara_lens(L);
  const int D = (int)lens.size() - 1;
  i64 cnt = 1;
  *xmax = 0;
  *zmax = 0;
  for (int d = 1; d <= D; ++d) {
    cnt *= 3;
    const i64 e = batch * cnt * lens[d];
    if (e > kKaraMaxElems) throw AfError(AF_ERR_UNSUPPORTED, "Karatsuba expansion exceeds 2^31 values");
    *xmax = std::max(*xmax, e);
  }
  // combine outputs: level d (from D-1 down to 1) holds batch * 3^d rows of 2 lens[d] - 1
  cnt = 1;
  for (int d = 0; d <= D; ++d) {
    if (d > 0) cnt *= 3;
    if (d == 0) continue;
    *zmax = std::max(*zmax, batch * cnt * (2 * lens[d] - 1));
  }
  return 4 * *xmax + 2 * *zmax;
}

// z (batch x (2L-1)) = Karatsuba(x, y); x, y: batch x L.
template <class Tin, class T>
static void karatsuba_run(const Tin* x, const Tin* y, T* z, i64 L, i64 batch, cudaStream_t st) {
  if (L <= 0 || batch <= 0) return;
  if (L == 1) {
    kara_leaf<Tin, T><<<kgrid(batch), 256, 0, st>>>(x, y, z, batch);
    kcheck(cudaGetLastError(), "karatsuba leaf");
    return;
  }
  const std::vector<i64> lens = kara_lens(L);
  const int D = (int)lens.size() - 1;
  i64 xmax, zmax;
  const i64 elems = kara_scratch_elems(L, batch, &xmax, &zmax);
  Scratch sc(sizeof(T) * (size_t)elems, st);
  T* base = (T*)sc.p;
  T* xb[2] = {base, base + xmax};
  T* yb[2] = {base + 2 * xmax, base + 3 * xmax};
  T* zb[2] = {base + 4 * xmax, base + 4 * xmax + zmax};
  // reorder levels (the first reads the caller's arrays, converting the type)
  i64 cnt = 1;
  int cur = 0;
  {
    const i64 l2 = lens[1];
    kara_reorder<Tin, T><<<kgrid(batch * cnt * l2), 256, 0, st>>>(x, y, xb[0], yb[0], batch, cnt, L, l2);
    kcheck(cudaGetLastError(), "karatsuba reorder");
    cnt = 3;
  }
  for (int d = 1; d < D; ++d) {
    const i64 len = lens[d], l2 = lens[d + 1];
    kara_reorder<T, T><<<kgrid(batch * cnt * l2), 256, 0, st>>>(xb[cur], yb[cur], xb[cur ^ 1], yb[cur ^ 1], batch,
                                                                 cnt, len, l2);
    kcheck(cudaGetLastError(), "karatsuba reorder");
    cur ^= 1;
    cnt *= 3;
  }
  // leaves: rows of length 1
  int zc = 0;
  kara_leaf<T, T><<<kgrid(batch * cnt), 256, 0, st>>>(xb[cur], yb[cur], zb[0], batch * cnt);
  kcheck(cudaGetLastError(), "karatsuba leaf");
  // combine levels: at level d rows have length 2 lens[d] - 1
  i64 zcur = 1;
  for (int d = D - 1; d >= 0; --d) {
    const i64 n3 = cnt / 3;
    const i64 zlen = 2 * lens[d] - 1;
    T* dst = d == 0 ? z : zb[zc ^ 1];
    kara_combine<T><<<kgrid(batch * n3 * zlen), 256, 0, st>>>(zb[zc], dst, batch, n3, zcur, zlen, lens[d + 1]);
    kcheck(cudaGetLastError(), "karatsuba combine");
    zc ^= 1;
    cnt = n3;
    zcur = zlen;
  }
}

template <class T>
static void fold_run(const T* z, T* out, i64 L, i64 batch, cudaStream_t st) {
  if (L <= 0 || batch <= 0) return;
  kara_fold<T><<<kgrid(batch * L), 256, 0, st>>>(z, out, batch, L);
  kcheck(cudaGetLastError(), "cyclic fold");
}

// complex (conv) with conv = karatsuba (cyclic = 0) or cyclic karatsuba (1)
template <class T>
static void complex_run(int cyclic, const T* xr, const T* xi, const T* yr, const T* yi, T* zr, T* zi, i64 L,
                        i64 batch, cudaStream_t st) {
  if (L <= 0 || batch <= 0) return;
  const i64 zl = 2 * L - 1;
  const i64 ol = cyclic ? L : zl;
  const i64 n_in = batch * L, n_z = batch * zl, n_o = batch * ol;
  Scratch sc(sizeof(T) * (size_t)(2 * n_in + 3 * n_z + (cyclic ? 3 * n_o : 0)), st);
  T* xm = (T*)sc.p;
  T* ym = xm + n_in;
  T* prod[3] = {ym + n_in, ym + n_in + n_z, ym + n_in + 2 * n_z};
  kara_sum<T><<<kgrid(n_in), 256, 0, st>>>(xr, xi, xm, n_in);
  kara_sum<T><<<kgrid(n_in), 256, 0, st>>>(yr, yi, ym, n_in);
  kcheck(cudaGetLastError(), "complex convolution inputs");
  karatsuba_run<T, T>(xr, yr, prod[0], L, batch, st);
  karatsuba_run<T, T>(xi, yi, prod[1], L, batch, st);
  karatsuba_run<T, T>(xm, ym, prod[2], L, batch, st);
  if (cyclic) {
    T* f = prod[2] + n_z;
    for (int i = 0; i < 3; ++i) {
      fold_run<T>(prod[i], f + i * n_o, L, batch, st);
      prod[i] = f + i * n_o;
    }
  }
  kara_complex_combine<T><<<kgrid(n_o), 256, 0, st>>>(prod[0], prod[1], prod[2], zr, zi, n_o);
  kcheck(cudaGetLastError(), "complex convolution combine");
}

static af_status kfail(af_status code, const std::string& m) {
  set_last_error(m);
  return code;
}

template <class F>
static af_status kguard(F&& f) {
  try {
    f();
    return AF_OK;
  } catch (const AfError& e) {
    return kfail(e.code, e.what());
  } catch (const std::bad_alloc&) {
    return kfail(AF_ERR_ALLOC, "host allocation failed");
  } catch (const std::exception& e) {
    return kfail(AF_ERR_INVALID, e.what());
  }
}

static void kargs(const void* a, const void* b, const void* c, int64_t L, int64_t batch) {
  if (L < 0 || batch < 0) throw AfError(AF_ERR_INVALID, "negative size");
  if (L > 0 && batch > 0 && (!a || !b || !c)) throw AfError(AF_ERR_INVALID, "null data pointer");
}

}  // namespace af

using namespace af;

// Integer rows run in unsigned 64-bit arithmetic: sums and products modulo
// 2^64 are the two's-complement wrap-around of the reference's Int, with no
// signed overflow in the kernels.  int32 inputs convert by sign extension.
typedef unsigned long long U64;

extern "C" {

af_status af_karatsuba_i64(const int64_t* x, const int64_t* y, int64_t* z, int64_t L, int64_t batch,
                           af_stream stream) {
  return kguard([&] {
    kargs(x, y, z, L, batch);
    karatsuba_run<U64, U64>((const U64*)x, (const U64*)y, (U64*)z, L, batch, (cudaStream_t)stream);
  });
}
af_status af_karatsuba_i32_i64(const int32_t* x, const int32_t* y, int64_t* z, int64_t L, int64_t batch,
                               af_stream stream) {
  return kguard([&] {
    kargs(x, y, z, L, batch);
    karatsuba_run<int, U64>((const int*)x, (const int*)y, (U64*)z, L, batch, (cudaStream_t)stream);
  });
}
af_status af_karatsuba_f32(const float* x, const float* y, float* z, int64_t L, int64_t batch, af_stream stream) {
  return kguard([&] {
    kargs(x, y, z, L, batch);
    karatsuba_run<float, float>(x, y, z, L, batch, (cudaStream_t)stream);
  });
}
af_status af_karatsuba_f64(const double* x, const double* y, double* z, int64_t L, int64_t batch,
                           af_stream stream) {
  return kguard([&] {
    kargs(x, y, z, L, batch);
    karatsuba_run<double, double>(x, y, z, L, batch, (cudaStream_t)stream);
  });
}

af_status af_conv_cyclic_fold_i64(const int64_t* z, int64_t* out, int64_t L, int64_t batch, af_stream stream) {
  return kguard([&] {
    kargs(z, out, z, L, batch);
    fold_run<U64>((const U64*)z, (U64*)out, L, batch, (cudaStream_t)stream);
  });
}
af_status af_conv_cyclic_fold_f32(const float* z, float* out, int64_t L, int64_t batch, af_stream stream) {
  return kguard([&] {
    kargs(z, out, z, L, batch);
    fold_run<float>(z, out, L, batch, (cudaStream_t)stream);
  });
}
af_status af_conv_cyclic_fold_f64(const double* z, double* out, int64_t L, int64_t batch, af_stream stream) {
  return kguard([&] {
    kargs(z, out, z, L, batch);
    fold_run<double>(z, out, L, batch, (cudaStream_t)stream);
  });
}

af_status af_conv_complex_i64(int cyclic, const int64_t* x_re, const int64_t* x_im, const int64_t* y_re,
                              const int64_t* y_im, int64_t* z_re, int64_t* z_im, int64_t L, int64_t batch,
                              af_stream stream) {
  return kguard([&] {
    kargs(x_re, y_re, z_re, L, batch);
    kargs(x_im, y_im, z_im, L, batch);
    complex_run<U64>(cyclic, (const U64*)x_re, (const U64*)x_im, (const U64*)y_re, (const U64*)y_im, (U64*)z_re,
                     (U64*)z_im, L, batch, (cudaStream_t)stream);
  });
}
af_status af_conv_complex_f32(int cyclic, const float* x_re, const float* x_im, const float* y_re,
                              const float* y_im, float* z_re, float* z_im, int64_t L, int64_t batch,
                              af_stream stream) {
  return kguard([&] {
    kargs(x_re, y_re, z_re, L, batch);
    kargs(x_im, y_im, z_im, L, batch);
    complex_run<float>(cyclic, x_re, x_im, y_re, y_im, z_re, z_im, L, batch, (cudaStream_t)stream);
  });
}
af_status af_conv_complex_f64(int cyclic, const double* x_re, const double* x_im, const double* y_re,
                              const double* y_im, double* z_re, double* z_im, int64_t L, int64_t batch,
                              af_stream stream) {
  return kguard([&] {
    kargs(x_re, y_re, z_re, L, batch);
    kargs(x_im, y_im, z_im, L, batch);
    complex_run<double>(cyclic, x_re, x_im, y_re, y_im, z_re, z_im, L, batch, (cudaStream_t)stream);
  });
}

}  // extern "C"
