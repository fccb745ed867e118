// af_internal.h -- declarations shared by libaf's translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "af_device.cuh"

namespace AF_NS {

__host__ __device__ __forceinline__ int spad_host(int i, int sh = 4) { return i + (i >> sh); }

// ------------------------------------------------------------- tile kernel
// One launch of the tile kernel: `nitems` CTAs, item i runs descs[items[i].desc].
struct LaunchSpec {
  const TileDesc* descs;
  const WorkItem* items;
  int nitems;
  int threads;
  int smem_data;      // elements per ping-pong buffer (max over the launch's descriptors)
  int generic;        // 0: every descriptor is a one-phase PLAIN tile with AFFINE views
  size_t smem_bytes;  // dynamic shared memory of the launch
};
size_t tile_smem_bytes(int smem_data, int tw_total, int G);
cudaError_t launch_tiles(const LaunchSpec& L, const TileBases& bases, double* loss, cudaStream_t st);

// ------------------------------------------------------------- map kernel
// Element-wise index maps and pointwise products between two views, one
// launch over nlines x nout elements.  Integer maps are exact.
enum MapMode {
  MAP_COPY = 0,       // out[e] = in[e]
  MAP_GT_IN = 1,      // out[k*n + j] = in[(n k + m j) mod nm]            (Planned.hs:597-606)
  MAP_GT_OUT = 2,     // out[r] = in[(r mod n)*m + (r mod m)]            (Planned.hs:608-617)
  MAP_TABLE = 3,      // out[e] = in[tab[e]]; x0[line] = in[0]           (Permutation.hs:24-33)
  MAP_RADER_OUT = 4,  // out[0] = x0 + dc; out[r] = x0 + in[tab[r-1]]   (Planned.hs:686-692)
  MAP_CHIRP_IN = 5,   // out[e] = e < n ? vec[e]*in[e] : 0               (Planned.hs:765-773)
  MAP_MUL = 6,        // out[e] = vec[e]*in[e]; dc[line] = in[0] if dc
  MAP_SCALE = 7,      // out[e] = scale*in[e]
  MAP_REVERSE = 8,    // out[e] = in[(-e) mod n]                         (Cyclic.hs:20-28)
  MAP_TWIDDLE = 9     // out[e] = in[e] * W_n^((line mod m) * e)         (Planned.hs:555)
};

struct MapDesc {
  int mode;
  i64 nlines, nout;
  IoDesc in, out;
  i64 n, m, nm;        // map parameters
  const int* tab;
  const cx* vec;
  i64 dc_ws, x0_ws;    // workspace offsets of the per-line DC / x0 (-1 = none)
  const cx* tab_tw;  // two-level twiddle table of n (MAP_TWIDDLE)
  int tw_log2;
  rl tw_sign;
  rl scale;
};
cudaError_t launch_map(const MapDesc& d, const TileBases& bases, cudaStream_t st);

// ------------------------------------------------------------- tables (FP64)
// tab[i] = exp(-2 pi i t_i / n) for the two-level layout: t_i = i (i < S),
// t_i = (i - S) * S (S <= i < S + H); computed in double, rounded to the
// element type.
cudaError_t launch_twiddle_table(cx* dst, i64 n, int S, int H, cudaStream_t st);
// chirp[k] = exp(sign * i * pi * sk^2 / len), sk = k for 2k < pad else k - pad,
// with sk^2 reduced mod 2*len in exact integers (Private.hs:428-436).
cudaError_t launch_chirp(double2* dst, i64 pad, i64 len, int sign, i64 count, cudaStream_t st);
// Rader kernel[i] = exp(sign * 2 pi i * (g^i mod p) / p) (Planned.hs:655-659)
cudaError_t launch_rader_kernel(double2* dst, i64 p, i64 g, int sign, cudaStream_t st);
cudaError_t launch_spectrum_input(const double2* k, i64 m, double2* kk, i64 M, int conj, cudaStream_t st);
cudaError_t launch_scale_round(const double2* S, cx* out, i64 n, double s, cudaStream_t st);

// ------------------------------------------------------------- real / two-real / convolution maps
// A complex array: interleaved when c is set, else planar re/im.
struct CPtr {
  cx* c;
  rl* re;
  rl* im;
};
cudaError_t launch_real_untangle(const cx* Z, CPtr out, i64 n2, i64 nout, i64 rows, const cx* tab,
                                 int S_log2, cudaStream_t st);
cudaError_t launch_real_entangle(CPtr spec, cx* f, i64 n2, i64 rows, const cx* tab, int S_log2, int herm,
                                 cudaStream_t st);
cudaError_t launch_untangle(CPtr S, CPtr A, CPtr B, i64 h, i64 w, i64 total, cudaStream_t st);
cudaError_t launch_reverse2d(CPtr in, CPtr out, i64 h, i64 w, i64 total, cudaStream_t st);
cudaError_t launch_entangle(CPtr C, CPtr D, CPtr out, i64 total, cudaStream_t st);
cudaError_t launch_conv_mul(cx* gx, const cx* gy, rl s, i64 total, cudaStream_t st);

}  // namespace af
