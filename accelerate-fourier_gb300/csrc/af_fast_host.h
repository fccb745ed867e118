// af_fast_host.h -- work items, shapes and tables of the batched executor
// (af_fast.cu), shared by the kernels, the planner and the host emulator.
#pragma once
#include <cuda_runtime.h>

#include <stdexcept>
#include <string>
#include <vector>

#include "af_fast.cuh"

namespace af {

// kinds of work item
enum FKind {
  FK_DIRECT = 0,  // whole transforms of one 5-smooth length in one CTA
  FK_BLUE = 1,    // whole Bluestein transforms sharing one convolution length in one CTA
  FK_COLS = 2,    // four-step pass A: column FFTs, twiddle, to the workspace
  FK_ROWS = 3,    // four-step pass B: row FFTs from the workspace to the output
  FK_BCOLS = 4,   // Bluestein pass A: chirp, column FFTs, twiddle, to the workspace
  FK_BROWS = 5,   // Bluestein pass R: row FFT, spectrum product, row FFT, twiddle
  FK_BCOLS2 = 6,  // Bluestein pass A': column FFTs, chirp, to the output
};

// A shape: what every transform of an item shares.  The line FFT has length
// L over GL interleaved lines (any GL for the compile-time lines, a power of
// two for the others and for full-FFT shapes);
// buffers hold `cap` elements each; LS is the line-major stride of the last
// pass.  Full-FFT shapes (FK_DIRECT, FK_BLUE) have n = L*G with GL = Q*G
// (Q transforms per CTA) and the final radix-G pass; multi-pass shapes have
// G = Q = 1 and GL lines (columns or rows) of one transform.
// Multi-pass shapes (aux = 1) also stage two three-level root tables of
// AFF_TL3 entries each.
#define AFF_TL3 192
// most transforms an item holds
#define AFF_MAXQ 16
struct FShape {
  FLine line;
  int kind;
  int n, G, Q, GL, LS, cap, ftwn, aux;
  int fixed;  // the line FFT is one of the compile-time lines (AFF_FIXED_LINES)
  int smem;  // shared-memory bytes an item of this shape uses
  FastDiv ndiv, L1div;
  int GLr;        // ceil(2^19 / GL): x / GL = (x GLr) >> 19 for x < 8192 (sdiv)
  const cx* tw;   // pass twiddles (line.twn entries)
  const cx* ftw;  // final twiddles W_n^k1, k1 < L (ftwn entries)
};

struct FItem {
  int kind, shape, first, count;  // transforms xf[first .. first + count)
  int c0, cn;                     // multi-pass items: columns or lines [c0, c0 + cn)
  int wait_ctr, wait_cnt;         // start once counter wait_ctr reaches wait_cnt (-1: no wait)
  int done_ctr;                   // counter this item increments when done (-1: none)
  int pad[3];                     // 48 bytes: the kernel prefetches an item with 16-byte copies
};

// Counters of a persistent launch: the queue head, the error word, then the
// per-pass completion counters of the multi-pass transforms.
enum { FC_HEAD = 0, FC_ERROR = 1, FC_FIRST = 2 };
// error word values
enum { FE_OK = 0, FE_TIMEOUT = 1 };

// One transform of the batch.
struct FXform {
  i64 off;         // offset in the batch (complex units)
  i64 ws, ws2;     // workspace regions 1 and 2 (multi-pass schemes; region 2: Bluestein)
  int gb, s1;      // region 1: lines per block (the stage-B items' GL), block stride
  int ga, s2;      // region 2: lines per block (the stage-A' items' GL), block stride
  int n;           // transform length
  int n1, n2;      // four-step split: n = n1 n2 (direct) or M = n1 n2 (Bluestein)
  int M;           // Bluestein convolution length
  const cx* ct;    // Bluestein: three-level table of W_{2n} (chirp a_m = W_{2n}^(m^2))
  const cx* wt;    // multi-pass: three-level table of W_n (direct) or W_M (Bluestein)
  const cx* spec;  // Bluestein: spectrum FFT(b)/M of the conjugate chirp, entries 0..M/2
  unsigned n2x;    // Bluestein: 2n, the chirp's modulus
  float r2n;       // Bluestein: 1 / (2n) rounded to float
  int gbr, gar;    // ceil(2^19 / gb), ceil(2^19 / ga) (sdiv)
};

struct FArgs {
  const FShape* shapes;
  const FItem* items;
  const FXform* xf;
  const cx* in;
  cx* out;
  const float* w;  // cotangent weights (null: plain transform)
  double* loss;
  cx* ws;
};

// Root table segments: forward roots computed in FP64 on the device.
enum { RS_STOCK = 0, RS_LINEAR = 1 };
struct RootSeg {
  i64 off, count;  // destination offset and entry count
  int kind;
  i64 a, b;  // RS_STOCK: p, R (entry (m-1) p + k = W_{pR}^(k m));  RS_LINEAR: entry i = W_a^(i b)
};

struct FastError : std::runtime_error {
  explicit FastError(const std::string& m) : std::runtime_error(m) {}
};
inline void fcheck(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw FastError(std::string(what) + ": " + cudaGetErrorString(e));
}

void gen_root_tables(const std::vector<RootSeg>& segs, cx* dbase, cx* hbase, cudaStream_t st);
// The persistent launch: `grid` CTAs of T threads take the items in queue
// order; a wait gives up after `spin_limit` polls (error word FE_TIMEOUT).
cudaError_t launch_fast(int T, int sign, const FArgs& A, int nitems, size_t smem, unsigned* ctrs, int grid,
                        long long spin_limit, cudaStream_t st);
int fast_ctas_per_sm(int T, int sign, size_t smem);
// Host emulation in queue order; returns FE_OK, or FE_TIMEOUT when an item
// would wait for an item later in the queue.
int emulate_fast(int T, int sign, const FArgs& A, const FItem* items, int nitems, size_t smem, int nctrs);

}  // namespace af
