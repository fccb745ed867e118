// af_fast.cu -- the batched executor of libaf: many Complex Float transforms
// of mixed lengths run as work items of one kernel (af_fast.cuh).
//
// Each transform of the batch is either
//   * direct: a 5-smooth length n, its mixed-radix FFT in one CTA
//     (several transforms of one length may share a CTA), or for long n a
//     four-step transform in two passes through an L2-resident workspace
//     (Planned.hs:525-557: columns, twiddle, rows);
//   * Bluestein: any other length, the chirp-z convolution of a 5-smooth
//     length M >= 2n-1 (Planned.hs:744-773, transformChirp235), in one CTA or
//     in three passes (columns, rows with the spectrum product, columns).
// The same code runs on the host, one thread index at a time, in the
// emulator that the CPU tests use.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "af_fast.cuh"
#include "af_fast_host.h"

namespace af {

// ============================================================ table generation
// Root tables hold forward roots W_den^num = exp(-2 pi i num / den), computed
// in double precision from the exactly reduced exponent and rounded to float.
AF_HD void root_segment_entry(const RootSeg& s, i64 i, i64* num, i64* den) {
  if (s.kind == RS_STOCK) {  // Stockham pass: entry (m-1)*p + k = W_{pR}^(k m)
    const i64 k = i % s.a, m = i / s.a + 1;
    *num = k * m;
    *den = s.a * s.b;
  } else {  // RS_LINEAR: entry i = W_a^(i * b)
    *num = i * s.b;
    *den = s.a;
  }
}

AF_HD cx root_value(i64 num, i64 den) {
  i64 r = num % den;
  if (r < 0) r += den;
  double c, s;
#ifdef __CUDA_ARCH__
  sincospi(-2.0 * (double)r / (double)den, &s, &c);
#else
  const double a = -2.0 * M_PI * ((double)r / (double)den);
  s = std::sin(a);
  c = std::cos(a);
#endif
  return make_cx((float)c, (float)s);
}

__global__ void root_tables_kernel(const RootSeg* segs, int nseg, cx* base) {
  for (int si = blockIdx.x; si < nseg; si += gridDim.x) {
    const RootSeg s = segs[si];
    for (i64 i = threadIdx.x; i < s.count; i += blockDim.x) {
      i64 num, den;
      root_segment_entry(s, i, &num, &den);
      base[s.off + i] = root_value(num, den);
    }
  }
}

void gen_root_tables(const std::vector<RootSeg>& segs, cx* dbase, cx* hbase, cudaStream_t st) {
  if (segs.empty()) return;
  if (hbase) {
    for (const RootSeg& s : segs)
      for (i64 i = 0; i < s.count; ++i) {
        i64 num, den;
        root_segment_entry(s, i, &num, &den);
        hbase[s.off + i] = root_value(num, den);
      }
    return;
  }
  RootSeg* d = nullptr;
  fcheck(cudaMallocAsync((void**)&d, sizeof(RootSeg) * segs.size(), st), "table segments");
  fcheck(cudaMemcpyAsync(d, segs.data(), sizeof(RootSeg) * segs.size(), cudaMemcpyHostToDevice, st),
         "table segments");
  root_tables_kernel<<<(int)std::min<size_t>(segs.size(), 4096), 256, 0, st>>>(d, (int)segs.size(), dbase);
  fcheck(cudaGetLastError(), "table kernel");
  fcheck(cudaFreeAsync(d, st), "table segments");
}

// ============================================================ execution policies
#ifdef __CUDACC__
// the CTA's mbarrier of its bulk copies (namespace scope: shared memory)
__shared__ unsigned long long s_mbar;
__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
#endif
// polls of a bulk copy's mbarrier before the CTA reports FE_TIMEOUT (a copy
// completes within microseconds; 2^20 polls take tens of milliseconds at least)
#define AFF_BULK_POLLS (1ll << 20)

// Device: each phase is one call per thread followed by a barrier.
struct DevExec {
  double loc = 0.0;  // the thread's running sum over every item it ran
  unsigned par = 0;  // parity of the mbarrier phase the next bulk copy completes
  unsigned* err = nullptr;  // the launch's error word
  bool failed = false;      // a bulk copy of this CTA timed out (uniform after the phase's barrier)
  unsigned* head = nullptr;  // the queue head (null: no claims)
  int nxt = 0;               // thread 0: the item claimed for the CTA's next round
  int ahead = 0;             // thread 0, during a load phase: the item claimed for the round after
  const FItem* items = nullptr;
  int nitems = 0;
#ifdef __CUDACC__
  // The CTA claims its items two rounds ahead.  At the start of an item's
  // load phase thread 0 takes the next item (claimed one round earlier),
  // copies its record into s_itn with the phase's asynchronous copies, and
  // claims the item after it; publish() hands both to the CTA at the end of
  // the phase.  Neither round trip delays the phase: the record's address is
  // known at once, and the claim's result is needed only at the phase's end.
  __device__ __forceinline__ void claim();
  __device__ __forceinline__ void publish();
  __device__ __forceinline__ void prefetch_next();
  template <class F>
  __device__ __forceinline__ void phase(F&& f) {
    f((int)threadIdx.x);
    __syncthreads();
  }
  // A load phase whose main transfer is one bulk copy of `bytes` (a multiple
  // of 16, both addresses 16-byte aligned) from global to shared memory,
  // issued by thread 0 on the CTA's mbarrier; f issues the phase's other
  // (cp.async) copies.  Each thread polls the mbarrier a bounded number of
  // times; a copy that does not complete sets FE_TIMEOUT and marks the CTA
  // failed.  After the wait the source lines `drop` .. `drop + drop_elems`
  // (whole 128-byte lines, read by no other item) are discarded from L2, so
  // that they are never written back.
  template <class F>
  __device__ __forceinline__ void phase_load(F&& f, cx* dst, const cx* src, unsigned bytes, const cx* drop,
                                             i64 drop_elems) {
    const unsigned mb = smem_u32(&s_mbar);
    claim();
    if (threadIdx.x == 0) {
      asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(mb), "r"(bytes) : "memory");
      asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                       smem_u32(dst)),
                   "l"(src), "r"(bytes), "r"(mb)
                   : "memory");
    }
    f((int)threadIdx.x);
    prefetch_next();
    asm volatile("cp.async.commit_group;\n" ::: "memory");
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    unsigned done = 0;
    for (long long k = 0; k < AFF_BULK_POLLS && !done; ++k)
      asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
                   : "=r"(done)
                   : "r"(mb), "r"(par)
                   : "memory");
    par ^= 1u;
    publish();
    if (!done) atomicExch(err + FC_ERROR, (unsigned)FE_TIMEOUT);
    for (i64 i = 16 * (i64)threadIdx.x; i < drop_elems; i += 16 * (i64)blockDim.x)
      asm volatile("discard.global.L2 [%0], 128;\n" ::"l"(drop + i) : "memory");
    failed = __syncthreads_or(!done) != 0;
  }
  template <class F>
  __device__ __forceinline__ void phase_async(F&& f) {
    claim();
    f((int)threadIdx.x);
    prefetch_next();
    asm volatile("cp.async.commit_group;\n" ::: "memory");
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    publish();
    __syncthreads();
  }
  // a phase whose threads accumulate into their own running sum
  template <class F>
  __device__ __forceinline__ void phase_sum(F&& f) {
    float l = 0.f;
    f((int)threadIdx.x, l);
    loc += l;
    __syncthreads();
  }
  // block sum of every thread's local value, added to *acc (one atomic per CTA)
  __device__ __forceinline__ void finish_sum(double* acc, double* red, int T) {
    double v = loc;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
      double s = 0;
      for (int w = 0; w < T / 32; ++w) s += red[w];
      atomicAdd(acc, s);
    }
  }
#endif
};

// Host: each phase runs for every thread index in turn.
struct HostExec {
  int T;
  bool failed = false;  // (host copies always complete)
  std::vector<double> locs;
  explicit HostExec(int t) : T(t), locs(t, 0.0) {}
  template <class F>
  void phase(F&& f) {
    for (int t = 0; t < T; ++t) f(t);
  }
  template <class F>
  void phase_async(F&& f) {
    phase(f);
  }
  template <class F>
  void phase_load(F&& f, cx* dst, const cx* src, unsigned bytes, const cx*, i64) {
    memcpy(dst, src, bytes);
    phase(f);
  }
  template <class F>
  void phase_sum(F&& f) {
    for (int t = 0; t < T; ++t) {
      float l = 0.f;
      f(t, l);
      locs[t] += l;
    }
  }
  void finish_sum(double* acc, double*, int) {
    double s = 0;
    for (double v : locs) s += v;
    *acc += s;
  }
};

AF_HD void cp_async8(cx* sdst, const cx* gsrc) {
#ifdef __CUDA_ARCH__
  const unsigned sa = (unsigned)__cvta_generic_to_shared(sdst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gsrc) : "memory");
#else
  *sdst = *gsrc;
#endif
}
// two elements; both addresses 16-byte aligned
AF_HD void cp_async16(cx* sdst, const cx* gsrc) {
#ifdef __CUDA_ARCH__
  const unsigned sa = (unsigned)__cvta_generic_to_shared(sdst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gsrc) : "memory");
#else
  sdst[0] = gsrc[0];
  sdst[1] = gsrc[1];
#endif
}

AF_HD int ilog2i(int v) {
  int l = 0;
  while ((1 << l) < v) ++l;
  return l;
}

// ============================================================ items
// Output of a transform: plain store, or the cotangent epilogue g = 2 w X
// with loss += w |X|^2 (w at the output's index).
struct Sink {
  cx* out;
  const float* w;
  AF_HD void put(i64 o, cx v, float& loss) const {
    if (w) {
      const float wt = ldf(w + o);
      loss += wt * (v.x * v.x + v.y * v.y);
      v = cscale(v, 2.f * wt);
    }
    out[o] = v;
  }
};

// A store phase over the u = tid, tid + T, ... < total elements of a tile:
// idx(u) gives element u's output offset from `base` (< 0: none), val(u) its
// value; the weights of the cotangent epilogue are loaded four elements at a
// time before the values are formed, so that their latency is paid once per
// four.
template <int T, class Idx, class Val>
AF_HD void store_phase(int tid, int total, const Sink& sk, i64 base, Idx idx, Val val, float& loss) {
  const float* w = sk.w ? sk.w + base : nullptr;
  cx* out = sk.out + base;
  for (int u0 = tid; u0 < total; u0 += 4 * T) {
    int o[4];
    float wt[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int u = u0 + r * T;
      o[r] = u < total ? idx(u) : -1;
      wt[r] = (w && o[r] >= 0) ? ldf(w + o[r]) : 0.f;
    }
#pragma unroll
    for (int r = 0; r < 4; ++r)
      if (o[r] >= 0) {
        cx t = val(u0 + r * T);
        if (w) {
          loss += wt[r] * (t.x * t.x + t.y * t.y);
          t = cscale(t, 2.f * wt[r]);
        }
        out[o[r]] = t;
      }
  }
}

// workspace element written by another CTA of this launch: read at L2 (no
// stale L1 line)
AF_HD cx ldws(const cx* p) {
#ifdef __CUDA_ARCH__
  return __ldcg(p);
#else
  return *p;
#endif
}

// W_N^t, t < 2^18, from a three-level table of 3 x 64 entries: W_N^j,
// W_N^(64 j), W_N^(4096 j).  GLOBAL: the table is in global memory (read
// through the read-only path), else in shared memory.
template <bool GLOBAL>
AF_HD cx tl3(const cx* tab, unsigned t) {
  cx a, b, c;
  if (GLOBAL) {
    a = ldcx(tab + (t & 63u));
    b = ldcx(tab + 64 + ((t >> 6) & 63u));
    c = ldcx(tab + 128 + (t >> 12));
  } else {
    a = tab[t & 63u];
    b = tab[64 + ((t >> 6) & 63u)];
    c = tab[128 + (t >> 12)];
  }
  return cmul(cmul(c, b), a);
}
// m^2 mod N for m^2 / N < 2^21 (the planner keeps N = 2n <= 2^18, m < n):
// the float estimate m m (1/N) of the quotient is within 3 * 2^-24 of it
// relatively, so off by at most one; the remainder, exact modulo 2^32, is
// then corrected once either way.
AF_HD unsigned sqmod(unsigned m, unsigned N, float rN) {
  const float fm = (float)m;
  const unsigned q = (unsigned)(fm * fm * rN);
  int r = (int)(m * m - q * N);
  if (r < 0) r += (int)N;
  if (r >= (int)N) r -= (int)N;
  return (unsigned)r;
}
// Bluestein chirp a_m = W_{2n}^(m^2 mod 2n) (forward root; the exact index
// keeps the phase of large m accurate); ct is the three-level table of W_{2n}
template <bool GLOBAL>
AF_HD cx chirp_at(const FXform& x, const cx* ct, int m) {
  return tl3<GLOBAL>(ct, sqmod((unsigned)m, x.n2x, x.r2n));
}

// The radix-G pass over `cnt` transforms of a full-FFT shape: element k1 of
// line l of transform q at src[(q G + l) LS + k1].  Per unit the sink gives
// a context c = f.at(q); f(c, q, m, v, loss) then receives natural bin
// m = k1 + L*l'.
template <int G, int SIGN, class F>
AF_HD void final_unit(int q, int k1, int L1, const cx* src, int LS, const cx* ftw, F& f, float& loss) {
  cx a[G];
#pragma unroll
  for (int l = 0; l < G; ++l) a[l] = src[lpos(k1, q * G + l, LS)];
  final_radix<G, SIGN>(a, G > 1 ? ftw[k1] : make_cx(1.f, 0.f));
  const auto c = f.at(q);
#pragma unroll
  for (int l = 0; l < G; ++l) f(c, q, k1 + l * L1, a[l], loss);
}
template <int G, int SIGN, class F>
AF_HD void final_thread(int tid, int T, int cnt, const FShape& S, const cx* src, int LS, const cx* ftw, F& f,
                        float& loss) {
  const int L1 = S.line.L;
  if (cnt == 1) {
    for (int k1 = tid; k1 < L1; k1 += T) final_unit<G, SIGN>(0, k1, L1, src, LS, ftw, f, loss);
    return;
  }
  for (int u = tid; u < cnt * L1; u += T) {
    const int q = (int)fdiv((unsigned)u, S.L1div);
    final_unit<G, SIGN>(q, u - q * L1, L1, src, LS, ftw, f, loss);
  }
}
template <int SIGN, class F>
AF_HD void final_any(int tid, int T, int cnt, const FShape& S, const cx* src, int LS, const cx* ftw, F& f,
                     float& loss) {
  switch (S.G) {
    case 1: final_thread<1, SIGN>(tid, T, cnt, S, src, LS, ftw, f, loss); break;
    case 2: final_thread<2, SIGN>(tid, T, cnt, S, src, LS, ftw, f, loss); break;
    case 4: final_thread<4, SIGN>(tid, T, cnt, S, src, LS, ftw, f, loss); break;
    default: final_thread<8, SIGN>(tid, T, cnt, S, src, LS, ftw, f, loss); break;
  }
}

// Every Stockham pass of the shape's line FFT, ping-ponging between the two
// buffers; returns the buffer holding the result (line-major, stride S.LS).
// Each pass moves V lines per unit (its own choice, see FPass).
// `ep` is the last pass's epilogue (compile-time lines only; the callers
// pass EPI_PLAIN for the others).
#pragma nv_exec_check_disable
template <int T, int SIGN, class E>
AF_HD cx* line_fft(E& ex, const FShape& S, cx* src, cx* dst, const cx* tw, const LineEpi& ep) {
  if (S.fixed) {  // a compile-time line (the planner sets `fixed` only for listed pairs)
    switch (S.line.L * 1024 + S.GL) {
#define AFF_FIXED_CASE(L, GL, R1, R2)                      \
  case L * 1024 + GL:                                      \
    cline_passes<T, SIGN, L, GL, 0>(ex, src, dst, tw, ep); \
    return src;
      AFF_FIXED_LINES(AFF_FIXED_CASE)
#undef AFF_FIXED_CASE
      default: break;
    }
  }
  const int np = S.line.npass;
  for (int j = 0; j < np; ++j) {
    const FPass ps = S.line.pass[j];
    const int LSo = j == np - 1 ? S.LS : 0;
    ex.phase([&](int tid) {
      if (ps.V == 2) fpass_any<2, SIGN>(tid, T, src, dst, ps, S.GL, S.GLr, LSo, tw);
      else fpass_any<1, SIGN>(tid, T, src, dst, ps, S.GL, S.GLr, LSo, tw);
    });
    cx* t = src;
    src = dst;
    dst = t;
  }
  return src;
}

// The kernel's shared memory: the dynamic area of the items, and the staged
// descriptors of the current item (namespace scope, so that the out-of-line
// line FFT addresses them as shared memory).
#ifdef __CUDACC__
extern __shared__ float4 fsm4[];
__shared__ FShape s_shape;
__shared__ FXform s_xf[AFF_MAXQ];
__shared__ FItem s_it;                 // the current item's record
__shared__ __align__(16) FItem s_itn;  // the record of the claimed next item
__shared__ int s_nxt, s_ok;            // the claimed next item's index; its wait succeeded
__shared__ int s_ahead;                // the item claimed for the round after the next
// thread 0 claims for the CTA; every thread reads s_nxt after the phase's
// closing barrier
__device__ __forceinline__ void DevExec::claim() {
  if (head && threadIdx.x == 0) {
    nxt = s_ahead;
    ahead = (int)atomicAdd(head, 1u);
  }
}
__device__ __forceinline__ void DevExec::publish() {
  if (head && threadIdx.x == 0) {
    s_nxt = nxt;
    s_ahead = ahead;
  }
}
__device__ __forceinline__ void DevExec::prefetch_next() {
  static_assert(sizeof(FItem) % 16 == 0, "item records move as 16-byte copies");
  if (head && threadIdx.x == 0 && nxt < nitems) {
    const cx* src = reinterpret_cast<const cx*>(items + nxt);
    cx* dst = reinterpret_cast<cx*>(&s_itn);
#pragma unroll
    for (int k = 0; k < (int)(sizeof(FItem) / 16); ++k) cp_async16(dst + 2 * k, src + 2 * k);
  }
}

// One out-of-line copy of the line FFT per sign, shared by every item kind
// (keeps the kernel's code, and its compile time, small); its buffers are
// element offsets into the dynamic shared area.
template <int T, int SIGN>
__device__ __noinline__ int line_fft_dev(int so, int doff, int toff, LineEpi ep) {
  DevExec ex;
  cx* base = reinterpret_cast<cx*>(fsm4);
  cx* r = line_fft<T, SIGN>(ex, s_shape, base + so, base + doff, base + toff, ep);
  return (int)(r - base);
}
template <int T, int SIGN>
__device__ __forceinline__ cx* run_line(DevExec&, const FShape&, cx* sm, cx* src, cx* dst, const cx* tw,
                                        const LineEpi& ep = LineEpi{EPI_PLAIN, 0, 0, 0, 0, nullptr}) {
  return sm + line_fft_dev<T, SIGN>((int)(src - sm), (int)(dst - sm), (int)(tw - sm), ep);
}
#endif
// the emulator runs the line FFT inline
template <int T, int SIGN>
cx* run_line(HostExec& ex, const FShape& S, cx*, cx* src, cx* dst, const cx* tw,
             const LineEpi& ep = LineEpi{EPI_PLAIN, 0, 0, 0, 0, nullptr}) {
  return line_fft<T, SIGN>(ex, S, src, dst, tw, ep);
}

// shared-memory areas of an item: the two data buffers, the pass twiddles,
// the final twiddles, the staged three-level tables (multi-pass shapes), and
// the reduction scratch
struct FSmem {
  cx *a, *b, *tw, *ftw, *wt3, *ct3;
  float* red;
};
AF_HD FSmem smem_of(const FShape& S, cx* sm) {
  FSmem m;
  m.a = sm;
  m.b = sm + S.cap;
  m.tw = m.b + S.cap;
  m.ftw = m.tw + S.line.twn;
  m.wt3 = m.ftw + S.ftwn;
  m.ct3 = m.wt3 + (S.aux ? AFF_TL3 : 0);
  m.red = reinterpret_cast<float*>(m.ct3 + (S.aux ? AFF_TL3 : 0));
  return m;
}

// copies the shape's tables (issued with the item's asynchronous loads);
// every table starts on an even entry, so 16-byte copies
AF_HD void copy_table(int tid, int T, cx* dst, const cx* src, int n) {
  for (int i = 2 * tid; i < n; i += 2 * T) cp_async16(dst + i, src + i);
}
AF_HD void copy_tables(int tid, int T, const FShape& S, const FSmem& m) {
  copy_table(tid, T, m.tw, S.tw, S.line.twn);
  copy_table(tid, T, m.ftw, S.ftw, S.ftwn);
}

// n contiguous elements into shared memory: 16-byte copies when the source
// is 16-byte aligned, else 8-byte copies
AF_HD void load_contiguous(int tid, int T, cx* dst, const cx* src, int n) {
  if ((reinterpret_cast<unsigned long long>(src) & 15) == 0) {
    for (int i = 2 * tid; i + 1 < n; i += 2 * T) cp_async16(dst + i, src + i);
    if ((n & 1) && tid == 0) cp_async8(dst + n - 1, src + n - 1);
  } else {
    for (int i = tid; i < n; i += T) cp_async8(dst + i, src + i);
  }
}

// Lines [0, cn) of a strided matrix, rows e < L, into the interleaved layout
// dst[e GL + c] = src[e stride + c]; lines cn..GL-1, and source positions
// e stride + c >= lim, read as zero.  Pairs of lines move as 16-byte copies
// at L2 when GL is even and every pair is 16-byte aligned; otherwise one
// element at a time,
// at L2 for workspace sources (WS: written by other CTAs of this launch, so
// never read through L1).
// no limit on the source positions
#define kAll ((i64)1 << 62)
template <bool WS>
AF_HD void load_lines(int tid, int T, cx* dst, int GL, int gr, const cx* src, i64 stride, int L, int cn,
                      i64 lim) {
  const cx z = make_cx(0.f, 0.f);
  const bool v16 = GL % 2 == 0 && ((reinterpret_cast<unsigned long long>(src) & 15) == 0) && (stride % 2 == 0) &&
                   (cn % 2 == 0);
  if (v16) {
    const int half = GL >> 1;
    for (int i = tid; i < L * half; i += T) {
      const int e = sdiv(2 * i, gr), c = 2 * i - e * GL;
      cx* d = dst + e * GL + c;
      const i64 s = e * stride + c;
      if (c < cn && s + 1 < lim) {
        cp_async16(d, src + s);
      } else if (c < cn && s < lim) {
        if (WS) d[0] = ldws(src + s);
        else cp_async8(d, src + s);
        d[1] = z;
      } else {
        d[0] = z;
        d[1] = z;
      }
    }
  } else {
    for (int i = tid; i < L * GL; i += T) {
      const int e = sdiv(i, gr), c = i - e * GL;
      const i64 s = e * stride + c;
      if (c >= cn || s >= lim) dst[i] = z;
      else if (WS) dst[i] = ldws(src + s);
      else cp_async8(dst + i, src + s);
    }
  }
}

// Lines cn..GL-1 of a loaded tile (the last block of a workspace region
// holds lines past the transform, which no item writes) set to zero.
#pragma nv_exec_check_disable
template <int T, class E>
AF_HD void zero_lines(E& ex, cx* a, int L, int GL, int gr, int cn) {
  ex.phase([&](int tid) {
    for (int i = tid; i < L * GL; i += T)
      if (i - sdiv(i, gr) * GL >= cn) a[i] = make_cx(0.f, 0.f);
  });
}

// sink of the direct items: bin m of transform q to the output
struct DirectOut {
  Sink sk;
  const FXform* xf;
  AF_HD i64 at(int q) const { return xf[q].off; }
  AF_HD void operator()(i64 base, int, int m, cx v, float& loss) const { sk.put(base + m, v, loss); }
};

// FK_DIRECT: Q transforms of one 5-smooth length, loaded in natural order
// (G interleaved lines each), line FFT, radix-G pass to the output.
#pragma nv_exec_check_disable
template <int T, int SIGN, class E>
AF_HD void direct_item(E& ex, const FArgs& A, const FItem& it, const FShape& S, const FXform* xf, cx* sm) {
  const FSmem m = smem_of(S, sm);
  const int n = S.n, G = S.G, GL = S.GL, Q = S.Q, glogG = ilog2i(G);
  const int cnt = it.count;
  ex.phase_async([&](int tid) {
    if (Q == 1) {  // one transform: its natural order is the layout
      load_contiguous(tid, T, m.a, A.in + xf[0].off, n);
    } else {
      for (int i = tid; i < Q * n; i += T) {
        const int q = (int)fdiv((unsigned)i, S.ndiv);
        const int e = i - q * n;
        const int pos = ipos(e >> glogG, q * G + (e & (G - 1)), GL);
        if (q < cnt) cp_async8(m.a + pos, A.in + xf[q].off + e);
        else m.a[pos] = make_cx(0.f, 0.f);
      }
    }
    copy_tables(tid, T, S, m);
  });
  const cx* res = run_line<T, SIGN>(ex, S, sm, m.a, m.b, m.tw);
  const int LS = S.line.npass ? S.LS : 1;  // no pass: the load layout read as line-major with LS 1
  DirectOut f{Sink{A.out, A.w}, xf};
  ex.phase_sum([&](int tid, float& loss) { final_any<SIGN>(tid, T, cnt, S, res, LS, m.ftw, f, loss); });
}

// sinks of the Bluestein item: the spectrum product (conjugated) into the
// other buffer, in the layout of the second FFT's input; and the chirp
// product of the first n bins to the output
struct BlueMid {
  const FXform* xf;
  int cnt, M;
  cx* nxt;
  int glogG, G, GL;
  AF_HD const cx* at(int q) const { return q < cnt ? xf[q].spec : nullptr; }
  template <int SIGN>
  AF_HD void put(const cx* spec, int q, int m, cx v) const {
    const cx p = spec ? conjc(cmul_s<SIGN>(v, spec_at(spec, M, m))) : make_cx(0.f, 0.f);
    nxt[ipos(m >> glogG, q * G + (m & (G - 1)), GL)] = p;
  }
};
template <int SIGN>
struct BlueMidS : BlueMid {
  AF_HD void operator()(const cx* spec, int q, int m, cx v, float&) const { put<SIGN>(spec, q, m, v); }
};
template <int SIGN>
struct BlueOut {
  Sink sk;
  const FXform* xf;
  AF_HD const FXform* at(int q) const { return xf + q; }
  AF_HD void operator()(const FXform* x, int, int m, cx v, float& loss) const {
    if (m < x->n) sk.put(x->off + m, cmul_s<SIGN>(conjc(v), chirp_at<true>(*x, x->ct, m)), loss);
  }
};

// FK_BLUE: Bluestein in one CTA (Planned.hs:760-773): u = a (.) x zero padded
// to M, FFT, times the spectrum, conjugate, FFT (= conj of the opposite-sign
// FFT), y = a (.) conj(.) for the first n bins.  Q transforms sharing M.
#pragma nv_exec_check_disable
template <int T, int SIGN, class E>
AF_HD void blue_item(E& ex, const FArgs& A, const FItem& it, const FShape& S, const FXform* xf, cx* sm) {
  const FSmem m = smem_of(S, sm);
  const int M = S.n, G = S.G, GL = S.GL, Q = S.Q, glogG = ilog2i(G);
  const int cnt = it.count;
  ex.phase_async([&](int tid) {
    for (int i = tid; i < Q * M; i += T) {
      const int q = (int)fdiv((unsigned)i, S.ndiv);
      const int e = i - q * M;
      cx v = make_cx(0.f, 0.f);
      if (q < cnt && e < xf[q].n) v = cmul_s<SIGN>(ldcx(A.in + xf[q].off + e), chirp_at<true>(xf[q], xf[q].ct, e));
      m.a[ipos(e >> glogG, q * G + (e & (G - 1)), GL)] = v;
    }
    copy_tables(tid, T, S, m);
  });
  const int LS = S.line.npass ? S.LS : 1;
  cx* res = run_line<T, SIGN>(ex, S, sm, m.a, m.b, m.tw);
  cx* nxt = res == m.a ? m.b : m.a;
  BlueMidS<SIGN> mid;
  mid.xf = xf;
  mid.cnt = cnt;
  mid.M = M;
  mid.nxt = nxt;
  mid.glogG = glogG;
  mid.G = G;
  mid.GL = GL;
  ex.phase_sum([&](int tid, float& loss) { final_any<SIGN>(tid, T, Q, S, res, LS, m.ftw, mid, loss); });
  res = run_line<T, SIGN>(ex, S, sm, nxt, res, m.tw);
  BlueOut<SIGN> out{Sink{A.out, A.w}, xf};
  ex.phase_sum([&](int tid, float& loss) { final_any<SIGN>(tid, T, cnt, S, res, LS, m.ftw, out, loss); });
}

// Multi-pass items work on one transform: columns [c0, c0 + cn) or lines
// [c0, c0 + cn) of its n1 x n2 matrix (element (j1, j2) at j1 n2 + j2); the
// shape's line FFT has GL lines (cn <= GL; any count on a compile-time line,
// else a power of two).  The item stages
// the transform's three-level tables of W_N (wt) and W_2n (ct) with its loads.
AF_HD void copy_multi_tables(int tid, int T, const FShape& S, const FSmem& m, const FXform& x) {
  copy_tables(tid, T, S, m);
  if (x.wt) copy_table(tid, T, m.wt3, x.wt, AFF_TL3);
  if (x.ct) copy_table(tid, T, m.ct3, x.ct, AFF_TL3);
}

// FK_COLS (four-step pass A, Planned.hs:525-557) and FK_BCOLS (Bluestein
// pass A): column FFT_n1 of x (FK_BCOLS: of a (.) x zero padded), twiddle
// W_N^(j2 k1), stored column-contiguous: ws[j2 n1 + k1].
#pragma nv_exec_check_disable
template <int T, int SIGN, class E>
AF_HD void cols_item(E& ex, const FArgs& A, const FItem& it, const FShape& S, const FXform* xf, cx* sm, bool blue) {
  const FSmem m = smem_of(S, sm);
  const FXform& x = xf[0];
  const int L = S.line.L, GL = S.GL;
  const int n2 = x.n2, c0 = it.c0, cn = it.cn;
  ex.phase_async([&](int tid) {
    // FK_BCOLS: x zero padded past n (natural index j = e n2 + c0 + c)
    load_lines<false>(tid, T, m.a, GL, S.GLr, A.in + x.off + c0, n2, L, cn, blue ? (i64)x.n - c0 : kAll);
    copy_multi_tables(tid, T, S, m, x);
  });
  if (blue) {  // the chirp a_j on the loaded x_j, from the staged table
    // rows e >= ceil((n - c0) / n2) hold only padding
    const i64 rr = ((i64)x.n - c0 + n2 - 1) / n2;
    const int rows = rr < L ? (int)rr : L;
    ex.phase([&](int tid) {
      for (int i = tid; i < rows * GL; i += T) {
        const int e = sdiv(i, S.GLr), c = i - e * GL;
        const int j = e * n2 + c0 + c;
        if (c < cn && j < x.n) m.a[i] = cmul_s<SIGN>(m.a[i], chirp_at<false>(x, m.ct3, j));
      }
    });
  }
  const cx* res = run_line<T, SIGN>(ex, S, sm, m.a, m.b, m.tw);
  ex.phase([&](int tid) {
    for (int u = tid; u < cn * L; u += T) {
      const int c = (int)fdiv((unsigned)u, S.L1div);
      const int k1 = u - c * L;
      const int j2 = c0 + c;
      const cx v = cmul_s<SIGN>(res[lpos(k1, c, S.LS)], tl3<false>(m.wt3, (unsigned)(j2 * k1)));
      const int kb = sdiv(k1, x.gbr);
      A.ws[x.ws + (i64)kb * x.s1 + j2 * x.gb + (k1 - kb * x.gb)] = v;  // block k1 / gb
    }
  });
}

// FK_ROWS (four-step pass B): lines k1 in [c0, c0 + cn), element j2 at
// ws[j2 n1 + k1]; FFT_n2; X[k1 + n1 k2] to the output.
#pragma nv_exec_check_disable
template <int T, int SIGN, class E>
AF_HD void rows_item(E& ex, const FArgs& A, const FItem& it, const FShape& S, const FXform* xf, cx* sm) {
  const FSmem m = smem_of(S, sm);
  const FXform& x = xf[0];
  const int L = S.line.L, GL = S.GL;
  const int n1 = x.n1, c0 = it.c0, cn = it.cn;
  // block c0 / GL of region 1, laid out as this item's tile
  const cx* blk = A.ws + x.ws + (i64)sdiv(c0, S.GLr) * x.s1;
  ex.phase_load([&](int tid) { copy_tables(tid, T, S, m); }, m.a, blk, (unsigned)(sizeof(cx) * L * GL), blk, x.s1);
  if (ex.failed) return;
  if (cn < GL) zero_lines<T>(ex, m.a, L, GL, S.GLr, cn);
  const cx* res = run_line<T, SIGN>(ex, S, sm, m.a, m.b, m.tw);
  const Sink sk{A.out, A.w};
  ex.phase_sum([&](int tid, float& loss) {
    store_phase<T>(
        tid, L * GL, sk, x.off,
        [&](int u) {
          const int k2 = sdiv(u, S.GLr), l = u - k2 * GL;
          return l < cn ? c0 + l + n1 * k2 : -1;
        },
        [&](int u) {
          const int k2 = sdiv(u, S.GLr);
          return res[lpos(k2, u - k2 * GL, S.LS)];
        },
        loss);
  });
}

// The two row FFTs of a Bluestein row item and the spectrum product between
// them as a pass of its own (lines that are not compile-time lines); returns
// the buffer holding the second FFT's result (line-major).
#pragma nv_exec_check_disable
template <int T, int SIGN, class E>
AF_HD cx* brows_spectrum(E& ex, const FShape& S, cx* sm, const FSmem& m, const FXform& x, int c0, int cn) {
  const int L = S.line.L, GL = S.GL;
  const int M1 = x.n1;
  cx* res = run_line<T, SIGN>(ex, S, sm, m.a, m.b, m.tw);
  cx* nxt = res == m.a ? m.b : m.a;
  ex.phase([&](int tid) {
    // four spectrum loads in flight per thread before their products
    const int tot = L * GL;
    for (int u0 = tid; u0 < tot; u0 += 4 * T) {
      cx sp[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const int u = u0 + r * T;
        const int k2 = sdiv(u, S.GLr), l = u - k2 * GL;
        sp[r] = (u < tot && l < cn) ? spec_at(x.spec, x.M, c0 + l + M1 * k2) : make_cx(0.f, 0.f);
      }
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const int u = u0 + r * T;
        if (u < tot) {
          const int k2 = sdiv(u, S.GLr), l = u - k2 * GL;
          nxt[ipos(k2, l, GL)] = conjc(cmul_s<SIGN>(res[lpos(k2, l, S.LS)], sp[r]));
        }
      }
    }
  });
  return run_line<T, SIGN>(ex, S, sm, nxt, res, m.tw);
}

// FK_BROWS (Bluestein pass R): lines k1 in [c0, c0 + cn), element j2 at
// ws[j2 M1 + k1]; FFT_M2; times the spectrum at k1 + M1 k2 and conjugated;
// FFT_M2 again; twiddle W_M^(j2 k1); stored line-contiguous in the
// transform's second workspace region: ws[M + k1 M2 + j2] (other items of
// this pass still read the first).
#pragma nv_exec_check_disable
template <int T, int SIGN, class E>
AF_HD void brows_item(E& ex, const FArgs& A, const FItem& it, const FShape& S, const FXform* xf, cx* sm) {
  const FSmem m = smem_of(S, sm);
  const FXform& x = xf[0];
  const int L = S.line.L, GL = S.GL;
  const int M1 = x.n1, c0 = it.c0, cn = it.cn;
  const cx* blk = A.ws + x.ws + (i64)sdiv(c0, S.GLr) * x.s1;
  ex.phase_load([&](int tid) { copy_multi_tables(tid, T, S, m, x); }, m.a, blk, (unsigned)(sizeof(cx) * L * GL), blk,
                x.s1);
  if (ex.failed) return;
  if (cn < GL) zero_lines<T>(ex, m.a, L, GL, S.GLr, cn);
  cx* res;
  if (S.fixed) {
    // the spectrum product in the first FFT's last pass, written in the
    // second FFT's input layout
    const LineEpi ep{EPI_SPEC, c0, cn, M1, x.M, x.spec};
    cx* nxt = run_line<T, SIGN>(ex, S, sm, m.a, m.b, m.tw, ep);
    res = run_line<T, SIGN>(ex, S, sm, nxt, nxt == m.a ? m.b : m.a, m.tw);
  } else {
    res = brows_spectrum<T, SIGN>(ex, S, sm, m, x, c0, cn);
  }
  ex.phase([&](int tid) {
    for (int u = tid; u < cn * L; u += T) {
      const int l = (int)fdiv((unsigned)u, S.L1div);
      const int j2 = u - l * L;
      const int k1 = c0 + l;
      const int jb = sdiv(j2, x.gar);
      A.ws[x.ws2 + (i64)jb * x.s2 + k1 * x.ga + (j2 - jb * x.ga)] =  // block j2 / ga
          cmul_s<SIGN>(res[lpos(j2, l, S.LS)], tl3<false>(m.wt3, (unsigned)(j2 * k1)));
    }
  });
}

// FK_BCOLS2 (Bluestein pass A'): columns j2 in [c0, c0 + cn), element k1 at
// ws[M + k1 M2 + j2]; FFT_M1; y_m = a_m (.) conj(.) at m = j1 M2 + j2 < n.
#pragma nv_exec_check_disable
template <int T, int SIGN, class E>
AF_HD void bcols2_item(E& ex, const FArgs& A, const FItem& it, const FShape& S, const FXform* xf, cx* sm) {
  const FSmem m = smem_of(S, sm);
  const FXform& x = xf[0];
  const int L = S.line.L, GL = S.GL;
  const int M2 = x.n2, c0 = it.c0, cn = it.cn;
  // block c0 / GL of region 2, laid out as this item's tile
  const cx* blk = A.ws + x.ws2 + (i64)sdiv(c0, S.GLr) * x.s2;
  ex.phase_load([&](int tid) { copy_multi_tables(tid, T, S, m, x); }, m.a, blk, (unsigned)(sizeof(cx) * L * GL), blk,
                x.s2);
  if (ex.failed) return;
  if (cn < GL) zero_lines<T>(ex, m.a, L, GL, S.GLr, cn);
  const cx* res = run_line<T, SIGN>(ex, S, sm, m.a, m.b, m.tw);
  const Sink sk{A.out, A.w};
  // rows j1 >= ceil((n - c0) / M2) fall past the transform's n outputs
  const i64 rr = ((i64)x.n - c0 + M2 - 1) / M2;
  const int rows = rr < L ? (int)rr : L;
  ex.phase_sum([&](int tid, float& loss) {
    store_phase<T>(
        tid, rows * GL, sk, x.off,
        [&](int u) {
          const int j1 = sdiv(u, S.GLr), c = u - j1 * GL, j = j1 * M2 + c0 + c;
          return c < cn && j < x.n ? j : -1;
        },
        [&](int u) {
          const int j1 = sdiv(u, S.GLr), c = u - j1 * GL;
          return cmul_s<SIGN>(conjc(res[lpos(j1, c, S.LS)]), chirp_at<false>(x, m.ct3, j1 * M2 + c0 + c));
        },
        loss);
  });
}

#pragma nv_exec_check_disable
template <int T, int SIGN, class E>
AF_HD void run_item(E& ex, const FArgs& A, const FItem& it, const FShape& S, const FXform* xf, cx* sm) {
  switch (it.kind) {
    case FK_BLUE: blue_item<T, SIGN>(ex, A, it, S, xf, sm); break;
    case FK_COLS: cols_item<T, SIGN>(ex, A, it, S, xf, sm, false); break;
    case FK_BCOLS: cols_item<T, SIGN>(ex, A, it, S, xf, sm, true); break;
    case FK_ROWS: rows_item<T, SIGN>(ex, A, it, S, xf, sm); break;
    case FK_BROWS: brows_item<T, SIGN>(ex, A, it, S, xf, sm); break;
    case FK_BCOLS2: bcols2_item<T, SIGN>(ex, A, it, S, xf, sm); break;
    default: direct_item<T, SIGN>(ex, A, it, S, xf, sm); break;
  }
}

// CTAs per SM the register budget allows for: 6 x 128, 3 x 256, 1 x 512 threads
#define AFF_MINB(T) ((T) <= 128 ? 6 : ((T) <= 256 ? 3 : 1))

#ifdef __CUDACC__
__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
  return v;
}
// n 4-byte words from global to shared memory, by the threads of warps 2..
__device__ __forceinline__ void copy_words64(void* dst, const void* src, int n) {
  const unsigned* s = reinterpret_cast<const unsigned*>(src);
  unsigned* d = reinterpret_cast<unsigned*>(dst);
  for (int i = threadIdx.x - 64; i < n; i += blockDim.x - 64) d[i] = __ldg(s + i);
}
#endif

// Persistent executor: every CTA takes the next item of the queue (items
// wait only for items earlier in the queue, and the smallest unfinished item
// is always held by a CTA that has started it or is about to, so the launch
// always completes, also with each CTA holding the items of its next two
// rounds: those follow its current one in the queue).  Thread 0 claims in the
// current item's load phase.  A wait (thread 32, in the item's prologue)
// polls its counter at most spin_limit times; then the CTA records
// FE_TIMEOUT and leaves, and the items that depend on it time out in turn.
// The item's shape and transforms are staged in shared memory (the shape only
// when it changes).
template <int T, int SIGN>
__global__ void __launch_bounds__(T, AFF_MINB(T)) fast_kernel(FArgs A, int nitems, unsigned* ctrs,
                                                              long long spin_limit) {
  DevExec ex;
  ex.err = ctrs;
  ex.head = ctrs + FC_HEAD;
  ex.items = A.items;
  ex.nitems = nitems;
  int loaded = -1;  // shape staged in s_shape (uniform across the CTA)
  if (threadIdx.x == 0) {
    ex.nxt = (int)atomicAdd(ctrs + FC_HEAD, 1u);
    s_nxt = ex.nxt;
    s_ahead = (int)atomicAdd(ctrs + FC_HEAD, 1u);
    if (ex.nxt < nitems) s_itn = A.items[ex.nxt];
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&s_mbar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  __syncthreads();
  for (;;) {
    // The claimed item (index and record staged in shared memory by thread 0
    // during the previous item's load phase, visible after its barriers).
    // Thread 32 waits for the item's stage counter while warps 2.. stage its
    // shape and transforms (the descriptors never change during the launch,
    // only the workspace the wait guards) and thread 0 finishes the previous
    // item's completion count: the three round trips overlap.
    if (s_nxt >= nitems) break;
    if (threadIdx.x == 0) {
      s_it = s_itn;
    } else if (threadIdx.x == 32) {
      const FItem it = s_itn;
      int ok = 1;
      if (it.wait_ctr >= 0) {
        long long k = 0;
        while (ld_acquire(ctrs + it.wait_ctr) < (unsigned)it.wait_cnt) {
          if (++k > spin_limit) {
            atomicExch(ctrs + FC_ERROR, (unsigned)FE_TIMEOUT);
            ok = 0;
            break;
          }
          __nanosleep(64);
        }
      }
      s_ok = ok;
    } else if (threadIdx.x >= 64) {
      const int shape = s_itn.shape;
      if (shape != loaded) copy_words64(&s_shape, A.shapes + shape, (int)(sizeof(FShape) / 4));
      copy_words64(s_xf, A.xf + s_itn.first, s_itn.count * (int)(sizeof(FXform) / 4));
    }
    __syncthreads();
    if (!s_ok) break;
    const FItem it = s_it;
    loaded = it.shape;
    run_item<T, SIGN>(ex, A, it, s_shape, s_xf, reinterpret_cast<cx*>(fsm4));
    // a bulk copy that never completed: this CTA takes no further items (the
    // items that wait for this one time out in turn)
    if (ex.failed) break;
    // every thread's stores of this item precede the barrier that closed its
    // last phase; thread 0's release increment publishes them with the count
    if (it.done_ctr >= 0 && threadIdx.x == 0)
      asm volatile("red.release.gpu.global.add.u32 [%0], 1;\n" ::"l"(ctrs + it.done_ctr) : "memory");
  }
  if (A.w && A.loss) {
    __syncthreads();
    ex.finish_sum(A.loss, reinterpret_cast<double*>(fsm4), T);
  }
}
template <int T, int SIGN>
static cudaError_t launch_fast_t(const FArgs& A, int nitems, size_t smem, unsigned* ctrs, int grid,
                                 long long spin_limit, cudaStream_t st) {
  static std::mutex mu;
  static int set_dev[64];
  static bool init = false;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  {
    std::lock_guard<std::mutex> g(mu);
    if (!init) {
      for (int& v : set_dev) v = -1;
      init = true;
    }
    if (dev >= 64 || set_dev[dev] < (int)smem) {
      e = cudaFuncSetAttribute(fast_kernel<T, SIGN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e == cudaSuccess)
        e = cudaFuncSetAttribute(fast_kernel<T, SIGN>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 cudaSharedmemCarveoutMaxShared);
      if (e != cudaSuccess) return e;
      if (dev < 64) set_dev[dev] = (int)smem;
    }
  }
  fast_kernel<T, SIGN><<<grid, T, smem, st>>>(A, nitems, ctrs, spin_limit);
  return cudaGetLastError();
}

cudaError_t launch_fast(int T, int sign, const FArgs& A, int nitems, size_t smem, unsigned* ctrs, int grid,
                        long long spin_limit, cudaStream_t st) {
  if (nitems <= 0) return cudaSuccess;
  if (T != 256) return cudaErrorInvalidValue;
  return sign < 0 ? launch_fast_t<256, -1>(A, nitems, smem, ctrs, grid, spin_limit, st)
                  : launch_fast_t<256, 1>(A, nitems, smem, ctrs, grid, spin_limit, st);
}

int fast_ctas_per_sm(int T, int sign, size_t smem) {
  int nb = 0;
  if (T != 256) return 0;
  cudaError_t e;
  if (sign < 0) {
    e = cudaFuncSetAttribute(fast_kernel<256, -1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(fast_kernel<256, -1>, cudaFuncAttributePreferredSharedMemoryCarveout,
                               cudaSharedmemCarveoutMaxShared);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fast_kernel<256, -1>, 256, smem);
  } else {
    e = cudaFuncSetAttribute(fast_kernel<256, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(fast_kernel<256, 1>, cudaFuncAttributePreferredSharedMemoryCarveout,
                               cudaSharedmemCarveoutMaxShared);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fast_kernel<256, 1>, 256, smem);
  }
  if (e != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return nb;
}

template <int T, int SIGN>
static int emulate_t(const FArgs& A, const FItem* items, int nitems, size_t smem, int nctrs) {
  std::vector<unsigned> ctr(std::max(nctrs, (int)FC_FIRST), 0u);
  HostExec ex(T);
  for (int i = 0; i < nitems; ++i) {
    const FItem& it = items[i];
    if (it.wait_ctr >= 0 && ctr.at(it.wait_ctr) < (unsigned)it.wait_cnt) return FE_TIMEOUT;
    // exactly the shape's shared memory, so that the sanitizer sees overruns
    const size_t bytes = (size_t)A.shapes[it.shape].smem;
    if (bytes > smem) throw FastError("item needs more shared memory than its launch");
    std::vector<cx> sm((bytes + sizeof(cx) - 1) / sizeof(cx));
    if (it.count < 1 || it.count > AFF_MAXQ) throw FastError("item transform count out of range");
    run_item<T, SIGN>(ex, A, it, A.shapes[it.shape], A.xf + it.first, sm.data());
    if (it.done_ctr >= 0) ctr.at(it.done_ctr)++;
  }
  if (A.w && A.loss) ex.finish_sum(A.loss, nullptr, T);
  return FE_OK;
}

int emulate_fast(int T, int sign, const FArgs& A, const FItem* items, int nitems, size_t smem, int nctrs) {
  if (T != 256) throw FastError("the executor runs 256-thread CTAs");
  return sign < 0 ? emulate_t<256, -1>(A, items, nitems, smem, nctrs)
                  : emulate_t<256, 1>(A, items, nitems, smem, nctrs);
}

}  // namespace af
