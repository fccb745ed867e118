// af_check.cpp -- host-side address checker for libaf launch programs.
//
// Programs are built in a dry-run mode (no device: fake table addresses,
// host copies of the index tables) and every global load and store address
// the tile and map kernels would compute is replayed here with the kernels'
// formulas and checked against the buffer sizes.  Every element of the
// output must be written exactly once (the index maps are bijections).  The
// entry points are internal (afx_*) and used by the CPU test suite.
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "af_host.h"

namespace AF_NS {

const Program& batch_program(BatchPlan* B, int which);
i64 batch_ws(BatchPlan* B);
i64 batch_total(BatchPlan* B);

struct Checker {
  const PlanRes& res;
  i64 sz[BUF_COUNT];
  std::vector<unsigned char> outw;  // writes per output element (final program only)
  std::string err;
  const char* where = "";

  Checker(const PlanRes& r) : res(r) {}

  bool ok() const { return err.empty(); }
  void fail(const std::string& m) {
    if (err.empty()) err = std::string(where) + ": " + m;
  }
  void rd(int buf, i64 a) {
    if (a < 0 || a >= sz[buf]) fail("read out of bounds: buffer " + std::to_string(buf) + " index " +
                                    std::to_string(a) + " size " + std::to_string(sz[buf]));
  }
  void wr(int buf, i64 a) {
    if (a < 0 || a >= sz[buf]) {
      fail("write out of bounds: buffer " + std::to_string(buf) + " index " + std::to_string(a) + " size " +
           std::to_string(sz[buf]));
      return;
    }
    if (buf == BUF_OUT && !outw.empty() && outw[a] < 255) outw[a]++;
  }
  int tab(const int* p, i64 q) {
    auto it = res.host_tabs.find(p);
    if (it == res.host_tabs.end()) { fail("unknown index table"); return 0; }
    if (q < 0 || q >= (i64)it->second.size()) { fail("index table read out of bounds"); return 0; }
    return it->second[q];
  }
  static void split(const IoDesc& io, i64 line, i64& hi, i64& lo) {
    const i64 d = io.lo_div.d ? io.lo_div.d : 1;
    hi = line / d;
    lo = line - hi * d;
  }
  i64 loff(const IoDesc& io, i64 line) {
    auto it = res.host_loffs.find(io.loff);
    if (it == res.host_loffs.end()) { fail("unknown line table"); return 0; }
    if (line < 0 || line >= (i64)it->second.size()) { fail("line table read out of bounds"); return 0; }
    return it->second[line];
  }
  // element e of line `line` (split into hi, lo) of an AFFINE or GT view
  i64 addr(const IoDesc& io, i64 base, i64 line, i64 hi, i64 lo, i64 e) {
    if (io.map == IO_GT) return base + hi * io.s_hi + ((io.mA * lo + io.mB * e) % io.mN) * io.s_t;
    if (io.loff) return base + loff(io, line) + e * io.s_e;
    return base + hi * io.s_hi + lo * io.s_lo + e * io.s_e;
  }

  void check_phase(const TileDesc& d, const FftPhase& ph) {
    if (ph.n <= 1) return;
    if ((i64)(ph.lcnt - 1) * ph.ls + (i64)(ph.n - 1) * ph.es >= d.LS) fail("phase exceeds the line stride");
    i64 prod = 1;
    for (int p = 0; p < ph.npass; ++p) {
      if (ph.pass[p].p != prod) fail("pass product mismatch");
      prod *= ph.pass[p].R;
    }
    if (prod != ph.n) fail("radices do not multiply to the phase length");
  }

  void tile(const Launch& L, const TileDesc& d, const WorkItem& it) {
    const i64 G = it.G, N = d.nlen;
    if (G < 1 || G > d.G || it.line0 + G > d.nlines) fail("work item lines out of range");
    if (spad_host(d.G * d.LS, d.pad_sh) + 2 > L.smem_data) fail("shared buffer too small");
    if (d.pad_sh < 4 || d.pad_sh > 31) fail("bad padding shift");
    if (d.slen > d.LS) fail("shared line shorter than the transform");
    for (int p = 0; p < d.nph; ++p) check_phase(d, d.ph[p]);
    const IoDesc& in = d.in;
    const IoDesc& out = d.out;
    const i64 ib = in.off + it.in_add, ob = out.off + it.out_add;
    for (i64 l = 0; l < G && ok(); ++l) {
      i64 hi, lo;
      split(in, it.line0 + l, hi, lo);
      // ---- loads
      if (d.kind == TILE_PLAIN || d.kind == TILE_CONVROW) {
        for (i64 e = 0; e < N; ++e) {
          if (in.map == IO_AFFINE || in.map == IO_GT) rd(in.buf, addr(in, ib, it.line0 + l, hi, lo, e));
          else if (in.map == IO_TABLE) {
            const i64 q = lo * in.q_lo + e * in.q_e;
            if (q < in.mN) rd(in.buf, ib + hi * in.s_hi + (i64)tab(in.tab, q) * in.s_t);
          } else {
            const i64 q = lo * in.q_lo + e * in.q_e;
            if (q < in.mN) rd(in.buf, ib + hi * in.s_hi + q * in.s_t);
          }
        }
        if (d.x0_cap >= 0 && lo == 0) {
          rd(in.buf, ib + hi * in.s_hi);
          wr(BUF_WS, d.x0_cap + it.out_add + hi);
        }
      } else {
        for (i64 e = 0; e < N; ++e) rd(in.buf, addr(in, ib, it.line0 + l, hi, lo, e));
      }
      // ---- middle
      i64 ohi, olo;
      split(out, it.line0 + l, ohi, olo);
      if (d.kind == TILE_CONVROW && d.dc_off >= 0 && olo == 0) wr(BUF_WS, d.dc_off + it.out_add + ohi);
      // ---- stores
      if (d.kind == TILE_PLAIN || d.kind == TILE_CONVROW) {
        for (i64 e = 0; e < N; ++e) {
          const i64 hb = ob + ohi * out.s_hi;
          if (out.map == IO_AFFINE || out.map == IO_GT) {
            wr(out.buf, addr(out, ob, it.line0 + l, ohi, olo, e));
          } else if (out.map == IO_CHIRP) {
            const i64 q = olo * out.q_lo + e * out.q_e;
            if (q < out.mN) wr(out.buf, hb + q * out.s_t);
          } else {
            const i64 q = olo * out.q_lo + e * out.q_e;
            if (q >= out.mN) continue;
            const i64 x0_add = out.x0_buf == in.buf ? it.in_add : it.out_add;
            rd(out.x0_buf, out.x0_off + x0_add + ohi * out.x0_shi);
            wr(out.buf, hb + (i64)tab(out.tab, q) * out.s_t);
            if (q == 0) {
              rd(BUF_WS, out.dc_off + it.in_add + ohi);
              wr(out.buf, hb);
            }
          }
        }
      } else {
        for (i64 e = 0; e < N; ++e) wr(out.buf, addr(out, ob, it.line0 + l, ohi, olo, e));
      }
    }
    if (d.kind == TILE_RADER && d.dlog) {
      for (i64 r = 1; r < N && ok(); ++r) {
        const int lg = tab(d.dlog, r - 1);
        if (lg < 0 || lg >= d.slen) fail("Rader position out of range");
      }
    }
  }

  static i64 vaddr(const IoDesc& io, i64 line, i64 e) {
    const i64 d = io.lo_div.d ? io.lo_div.d : 1;
    const i64 hi = line / d, lo = line - hi * d;
    return io.off + hi * io.s_hi + lo * io.s_lo + e * io.s_e;
  }

  void map(const MapDesc& d) {
    for (i64 line = 0; line < d.nlines && ok(); ++line)
      for (i64 e = 0; e < d.nout; ++e) {
        switch (d.mode) {
          case MAP_COPY: case MAP_SCALE: case MAP_CHIRP_IN: case MAP_MUL: case MAP_TWIDDLE:
            if (!(d.mode == MAP_CHIRP_IN && e >= d.n)) rd(d.in.buf, vaddr(d.in, line, e));
            if (d.mode == MAP_MUL && d.dc_ws >= 0 && e == 0) wr(BUF_WS, d.dc_ws + line);
            break;
          case MAP_GT_IN: {
            const i64 k = e / d.n, j = e - k * d.n;
            rd(d.in.buf, vaddr(d.in, line, (d.n * k + d.m * j) % d.nm));
            break;
          }
          case MAP_GT_OUT: rd(d.in.buf, vaddr(d.in, line, (e % d.n) * d.m + (e % d.m))); break;
          case MAP_TABLE:
            rd(d.in.buf, vaddr(d.in, line, tab(d.tab, e)));
            if (d.x0_ws >= 0 && e == 0) wr(BUF_WS, d.x0_ws + line);
            break;
          case MAP_RADER_OUT:
            rd(BUF_WS, d.x0_ws + line);
            if (e == 0) rd(BUF_WS, d.dc_ws + line);
            else rd(d.in.buf, vaddr(d.in, line, tab(d.tab, e - 1)));
            break;
          default: rd(d.in.buf, vaddr(d.in, line, e == 0 ? 0 : d.n - e)); break;
        }
        wr(d.out.buf, vaddr(d.out, line, e));
      }
  }

  void program(const Program& prog) {
    for (size_t k = 0; k < prog.launches.size() && ok(); ++k) {
      const Launch& L = prog.launches[k];
      if (L.type == L_TILE) {
        for (const WorkItem& it : L.items) {
          if (it.desc < 0 || it.desc >= (int)L.descs.size()) { fail("bad descriptor index"); break; }
          tile(L, L.descs[it.desc], it);
          if (!ok()) break;
        }
      } else {
        map(L.md);
      }
    }
  }

  void expect_out_once(i64 n_out) {
    for (i64 i = 0; i < n_out && ok(); ++i)
      if (outw[i] != 1) fail("output element " + std::to_string(i) + " written " + std::to_string(outw[i]) + " times");
  }
};

static int report(const std::string& err, char* msg, size_t len) {
  if (msg && len) {
    const size_t k = std::min(len - 1, err.size());
    memcpy(msg, err.data(), k);
    msg[k] = 0;
  }
  return err.empty() ? 0 : 1;
}

}  // namespace af

using namespace AF_NS;

// the checker of the Complex Double engine exports the same entry points
// with an _f64 suffix
#ifdef AF_F64
#define AFX(name) name##_f64
#else
#define AFX(name) name
#endif

// a plan without a device: reference tree and resources in dry mode
struct DryPlan {
  af::Planner planner;
  PlanRes res;
  const af::Node* root = nullptr;
  i64 n = 0;
  int sign = -1;
};

extern "C" {

// Builds the programs of a plan (both signs) for `batch` rows without a
// device and checks every address.  0: all in bounds and every output
// element written once; 1: violation (msg); -1: the plan could not be built.
int AFX(afx_check_plan)(int64_t n, int sign, int algo, int64_t batch, char* msg, size_t len) {
  try {
    DryPlan P;
    P.res.dry = true;
    P.n = n;
    P.sign = sign;
    P.root = plan_root(P.planner, n, algo);
    for (int s : {sign, -sign}) {
      Program prog;
      build_program(P.res, P.root, (rl)s, batch, &prog);
      Checker c(P.res);
      c.where = s == sign ? "forward program" : "vjp program";
      c.sz[BUF_IN] = c.sz[BUF_OUT] = c.sz[BUF_AUX] = n * batch;
      c.sz[BUF_WS] = prog.ws_elems;
      c.outw.assign((size_t)(n * batch), 0);
      c.program(prog);
      c.expect_out_once(n * batch);
      if (!c.ok()) return report(c.err, msg, len);
    }
    return 0;
  } catch (const std::exception& e) {
    report(e.what(), msg, len);
    return -1;
  }
}

// The same for a transform along the middle axis of (outer, n, inner) arrays
// (the programs behind af_exec_c2c_axis and the 2-D/3-D transforms).
int AFX(afx_check_axis)(int64_t n, int sign, int algo, int64_t outer, int64_t inner, char* msg, size_t len) {
  try {
    DryPlan P;
    P.res.dry = true;
    P.n = n;
    P.sign = sign;
    P.root = plan_root(P.planner, n, algo);
    View in;
    in.buf = BUF_IN;
    in.s_e = inner;
    in.s_lo = 1;
    in.lo_cnt = inner;
    in.s_hi = n * inner;
    View out = in;
    out.buf = BUF_OUT;
    Program prog;
    build_program_view(P.res, P.root, (rl)sign, outer * inner, in, out, &prog);
    Checker c(P.res);
    c.where = "axis program";
    const i64 total = outer * n * inner;
    c.sz[BUF_IN] = c.sz[BUF_OUT] = c.sz[BUF_AUX] = total;
    c.sz[BUF_WS] = prog.ws_elems;
    c.outw.assign((size_t)total, 0);
    c.program(prog);
    c.expect_out_once(total);
    if (!c.ok()) return report(c.err, msg, len);
    return 0;
  } catch (const std::exception& e) {
    report(e.what(), msg, len);
    return -1;
  }
}

// The same for a batch of mixed lengths (forward, VJP and cotangent programs).
int AFX(afx_check_batch)(const int64_t* ns, int64_t count, int sign, char* msg, size_t len) {
  BatchPlan* B = nullptr;
  try {
    B = batch_create_mode((const i64*)ns, count, sign, true);
    const i64 total = batch_total(B);
    for (int which = 0; which < 3; ++which) {
      Checker c(*(const PlanRes*)batch_res(B));
      c.where = which == 0 ? "batch forward" : which == 1 ? "batch vjp" : "batch cotangent";
      c.sz[BUF_IN] = c.sz[BUF_OUT] = c.sz[BUF_AUX] = total;
      c.sz[BUF_WS] = batch_ws(B);
      c.outw.assign((size_t)total, 0);
      c.program(batch_program(B, which));
      c.expect_out_once(total);
      if (!c.ok()) {
        batch_destroy(B);
        return report(c.err, msg, len);
      }
    }
    batch_destroy(B);
    return 0;
  } catch (const std::exception& e) {
    if (B) batch_destroy(B);
    report(e.what(), msg, len);
    return -1;
  }
}

}  // extern "C"

extern "C" {

// Text summary of a batch program (which: 0 forward, 1 VJP, 2 cotangent),
// built without a device: one line per launch with its type, threads, CTAs,
// shared buffer size and the tile descriptors' kinds, lengths and maps.
int AFX(afx_describe_batch)(const int64_t* ns, int64_t count, int sign, int which, char* buf, size_t len) {
  BatchPlan* B = nullptr;
  try {
    B = batch_create_mode((const i64*)ns, count, sign, true);
    const Program& prog = batch_program(B, which);
    std::string s;
    for (size_t k = 0; k < prog.launches.size(); ++k) {
      const Launch& L = prog.launches[k];
      char line[512];
      if (L.type == L_MAP) {
        snprintf(line, sizeof line, "%zu map mode=%d lines=%lld nout=%lld\n", k, L.md.mode, (long long)L.md.nlines,
                 (long long)L.md.nout);
        s += line;
        continue;
      }
      i64 elems = 0;
      std::map<std::string, i64> kinds;
      for (const WorkItem& it : L.items) {
        const TileDesc& d = L.descs[it.desc];
        elems += (i64)it.G * d.slen;
        char key[96];
        snprintf(key, sizeof key, "k%d n%d s%d in%d out%d ph%d p%d%s%s", d.kind, d.nlen, d.slen, d.in.map, d.out.map,
                 d.nph, d.pad_sh, d.ptw ? " tw" : "", d.in.line_fast || d.out.line_fast ? " lf" : "");
        kinds[key] += 1;
      }
      snprintf(line, sizeof line, "%zu tile T=%d ctas=%zu smem=%d elems=%lld descs=%zu :", k, L.threads,
               L.items.size(), L.smem_data, (long long)elems, L.descs.size());
      s += line;
      int shown = 0;
      for (auto& kv : kinds) {
        if (shown++ == 400) { s += " ..."; break; }
        s += " [" + kv.first + " x" + std::to_string(kv.second) + "]";
      }
      s += "\n";
    }
    batch_destroy(B);
    return report(s, buf, len) ? 0 : 0;
  } catch (const std::exception& e) {
    if (B) batch_destroy(B);
    report(e.what(), buf, len);
    return -1;
  }
}

}  // extern "C"
