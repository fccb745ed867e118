// af_oracle.cpp -- TEST INFRASTRUCTURE ONLY (the oracle).
//
// A CPU restatement of accelerate-fourier 1.0.0.5's transform algorithms, used
// as the checker for the CUDA library.  Only tests/, __graft_entry__.smoke()
// and bench.py's CPU-baseline leg may load it; the product never does.
//
// Parity status: the reference is Haskell/Accelerate and no Haskell toolchain
// exists here, so bit-level FP parity with a Haskell build is UNPINNED.  The
// oracle is pinned by (a) the reference's known-answer test (inverse transform
// of a unit impulse is a basis vector, test/Test/Data/Array/Accelerate/Fourier.hs:
// 219-223,367-376), (b) the permutation tables written in the reference's own
// source comments (src/Data/Array/Accelerate/Fourier/Planned.hs:621-643,
// src/Data/Array/Accelerate/Fourier/Private.hs:185-203,
// Planned.hs:563-572), (c) all 38 reference properties, and (d) an independent
// long-double naive DFT.  Integer paths (plans, index maps, Karatsuba) are exact.
//
// Every function cites the reference file:line it restates (paths relative to
// the accelerate-fourier project root).

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef long long i64;
template <class T> using cx = std::complex<T>;

// ---------------------------------------------------------------------------
// Complex helpers with the operation order of Data.Complex / Accelerate:
// (a+bi)(c+di) = (ac-bd) + (ad+bc)i.
template <class T> static inline cx<T> cmul(cx<T> a, cx<T> b) {
  return cx<T>(a.real() * b.real() - a.imag() * b.imag(),
               a.real() * b.imag() + a.imag() * b.real());
}
template <class T> static inline cx<T> cadd(cx<T> a, cx<T> b) {
  return cx<T>(a.real() + b.real(), a.imag() + b.imag());
}
template <class T> static inline cx<T> csub(cx<T> a, cx<T> b) {
  return cx<T>(a.real() - b.real(), a.imag() - b.imag());
}
template <class T> static inline T pi_t() { return (T)3.141592653589793238462643383279502884L; }

// Sign.hs:63-66  cis sign w = cos w :+ sign * sin w
template <class T> static inline cx<T> cis(T sign, T w) {
  return cx<T>(std::cos(w), sign * std::sin(w));
}
// Sign.hs:68-72  cisRat sign denom numer = cis sign (2*pi*numer/denom)
template <class T> static inline cx<T> cis_rat(T sign, i64 denom, i64 numer) {
  return cis<T>(sign, (T)2 * pi_t<T>() * (T)numer / (T)denom);
}

// ---------------------------------------------------------------------------
// NumberTheory.hs

// NumberTheory.hs:15-29 fermatFactors.  The merge of n + a^2 (a ascending)
// with b^2 emits (b-a, b+a) for b^2 - a^2 = n.  For odd n every divisor pair
// (d, n/d) with d <= sqrt n arises exactly once (a = (n/d - d)/2), and a
// ascending is d descending, so the list equals the divisor pairs ordered by
// the smaller factor descending.
static std::vector<std::pair<i64, i64>> fermat_factors(i64 n) {
  std::vector<std::pair<i64, i64>> out;
  i64 r = (i64)std::floor(std::sqrt((double)n));
  while (r * r > n) --r;
  while ((r + 1) * (r + 1) <= n) ++r;
  for (i64 d = r; d >= 1; --d)
    if (n % d == 0) out.push_back({d, n / d});
  return out;
}

static i64 gcd64(i64 a, i64 b) {
  while (b) { i64 t = a % b; a = b; b = t; }
  return a < 0 ? -a : a;
}

// NumberTheory.hs:53-63 modularPower (square-and-multiply, exact)
static i64 modular_power(i64 modu, i64 expo, i64 n) {
  if (expo == 0) return 1;  // go 0 _ = 1
  i64 half = expo / 2, r = expo % 2;
  i64 n2 = (i64)(((__int128)n * n) % modu);
  i64 g = modular_power(modu, half, n2);
  return r == 0 ? g : (i64)(((__int128)g * n) % modu);
}

// NumberTheory.hs:65-91 uniquePrimeFactors (trial division)
static std::vector<i64> unique_prime_factors(i64 n) {
  std::vector<i64> out;
  if (n <= 0) return out;
  i64 m = n;
  if ((m & 1) == 0) {
    out.push_back(2);
    while ((m & 1) == 0) m >>= 1;
  }
  for (i64 p = 3; m > 1; p += 2) {
    if (m % p == 0) {
      out.push_back(p);
      while (m % p == 0) m /= p;
    } else if (m / p < p) {
      out.push_back(m);
      break;
    }
  }
  return out;
}

// NumberTheory.hs:32-47 multiplicativeGenerator: smallest primitive root
static i64 multiplicative_generator(i64 p) {
  i64 order = p - 1;
  std::vector<i64> great;
  for (i64 q : unique_prime_factors(order)) great.push_back(order / q);
  for (i64 c = 1; c <= p - 1; ++c) {
    if (gcd64(c, p) != 1) continue;
    if (modular_power(p, order, c) != 1) continue;
    bool ok = true;
    for (i64 y : great)
      if (modular_power(p, y, c) == 1) { ok = false; break; }
    if (ok) return c;
  }
  return 0;
}

// NumberTheory.hs:94-101 ceilingPowerOfTwo
static i64 ceiling_power_of_two(i64 n) {
  if (n == 0) return 1;
  i64 m = n - 1;
  for (int d = 1; d < 64; d *= 2) m |= (m >> d);
  return m + 1;
}

// NumberTheory.hs:118-124 ceilingSmooths a b n m
static std::vector<i64> ceiling_smooths(i64 a, i64 b, i64 n, i64 m) {
  std::vector<i64> out;
  for (;;) {
    out.push_back(m);
    if (m % a != 0) break;
    i64 k = m * b;
    for (;;) {
      i64 q = k / a, r = k % a;
      if (r == 0 && q >= n) k = q; else break;
    }
    m = k;
  }
  return out;
}

// NumberTheory.hs:108-111 ceiling5Smooth
static i64 ceiling_5smooth(i64 n) {
  i64 best = -1;
  for (i64 c : ceiling_smooths(2, 3, n, ceiling_power_of_two(n))) {
    std::vector<i64> v = ceiling_smooths(2, 5, n, c);
    i64 mn = *std::min_element(v.begin(), v.end());
    if (best < 0 || mn < best) best = mn;
  }
  return best;
}

// Adhoc.hs:287-291 ceilingLogBase base x = ceiling (logBase base x) in Double
static i64 ceiling_log_base(i64 base, double x) {
  return (i64)std::ceil(std::log(x) / std::log((double)base));
}

// Adhoc.hs:229-248 ceiling5Smooth (device-side Double argmin over a grid)
static i64 adhoc_ceiling_5smooth(i64 ni) {
  double n = (double)ni;
  i64 d3 = ceiling_log_base(3, n), d5 = ceiling_log_base(5, n);
  double bestv = 0;
  i64 b2 = 0, b3 = 0, b5 = 0;
  bool have = false;
  for (i64 e5 = 0; e5 < d5; ++e5)
    for (i64 e3 = 0; e3 < d3; ++e3) {
      double p53 = std::pow(5.0, (double)e5) * std::pow(3.0, (double)e3);
      i64 e2 = std::max<i64>(0, ceiling_log_base(2, n / p53));
      double v = p53 * std::pow(2.0, (double)e2);
      if (!have || v < bestv) { have = true; bestv = v; b2 = e2; b3 = e3; b5 = e5; }
    }
  if (!have) return -1;
  i64 r = 1;
  for (i64 i = 0; i < b2; ++i) r *= 2;
  for (i64 i = 0; i < b3; ++i) r *= 3;
  for (i64 i = 0; i < b5; ++i) r *= 5;
  return r;
}

// ---------------------------------------------------------------------------
// Planned.hs:183-293 planner

enum Kind { K_ID = 0, K_SMALL, K_SR, K_PRIME, K_COPRIME, K_COMPOSITE, K_CHIRP };

struct Plan {
  i64 n;
  Kind kind;
  int small;        // 2..5 for K_SMALL
  const Plan* a;    // SR sub / prime sub / chirp sub / first of pair
  const Plan* b;    // second of pair
};

struct PlanSet {
  std::vector<std::unique_ptr<Plan>> arena;
  std::map<i64, const Plan*> memo;  // PlanMap (Planned.hs:234)
  const Plan* mk(i64 n, Kind k, int s, const Plan* a, const Plan* b) {
    arena.emplace_back(new Plan{n, k, s, a, b});
    return arena.back().get();
  }
  PlanSet() {  // Planned.hs:241-250 smallPlanMap
    memo[0] = mk(0, K_ID, 0, 0, 0);
    memo[1] = mk(1, K_ID, 0, 0, 0);
    for (int s = 2; s <= 5; ++s) memo[s] = mk(s, K_SMALL, s, 0, 0);
  }
  // Planned.hs:279-287 planDecomposeWithMapUpdate
  const Plan* decompose(i64 n) {
    auto it = memo.find(n);
    if (it != memo.end()) return it->second;
    const Plan* p = decompose_new(n);
    memo[n] = p;
    return p;
  }
  // Planned.hs:255-277 planDecomposeWithMap
  const Plan* decompose_new(i64 n) {
    if (n % 2 == 0) {
      const Plan* s = decompose(n / 2);
      return mk(n, K_SR, 0, s, 0);
    }
    std::vector<std::pair<i64, i64>> facs = fermat_factors(n);
    for (auto& q : facs)
      if (q.first > 1 && gcd64(q.first, q.second) == 1) {
        const Plan* a = decompose(q.first);
        const Plan* b = decompose(q.second);
        return mk(n, K_COPRIME, 0, a, b);
      }
    auto q = facs[0];
    if (q.first == 1) {
      const Plan* s = decompose(n - 1);
      return mk(n, K_PRIME, 0, s, 0);
    }
    const Plan* a = decompose(q.first);
    const Plan* b = decompose(q.second);
    return mk(n, K_COMPOSITE, 0, a, b);
  }
  // Planned.hs:731-737 planChirpWithMapUpdate
  const Plan* chirp(i64 n, bool pow2) {
    if (n < 2) return mk(n, K_ID, 0, 0, 0);
    i64 pad = pow2 ? ceiling_power_of_two(2 * n - 1) : ceiling_5smooth(2 * n - 1);
    return mk(n, K_CHIRP, 0, decompose(pad), 0);
  }
  // Planned.hs:215-220 planWithMapUpdate
  const Plan* automatic(i64 n) {
    const Plan* p = decompose(n);
    if (count_primes(p) < 3) return p;
    return chirp(n, false);
  }
  // Planned.hs:222-232 planCountPrimes
  static int count_primes(const Plan* p) {
    switch (p->kind) {
      case K_ID: case K_SMALL: return 0;
      case K_SR: return count_primes(p->a);
      case K_PRIME: return 1 + count_primes(p->a);
      case K_COPRIME: case K_COMPOSITE:
        return std::max(count_primes(p->a), count_primes(p->b));
      case K_CHIRP: return count_primes(p->a);
    }
    return 0;
  }
};

static void plan_string(const Plan* p, std::string& s) {
  char buf[64];
  switch (p->kind) {
    case K_ID: snprintf(buf, sizeof buf, "I%lld", p->n); s += buf; return;
    case K_SMALL: snprintf(buf, sizeof buf, "S%lld", p->n); s += buf; return;
    case K_SR: snprintf(buf, sizeof buf, "SR%lld(", p->n); break;
    case K_PRIME: snprintf(buf, sizeof buf, "P%lld(", p->n); break;
    case K_COPRIME: snprintf(buf, sizeof buf, "GT%lld(", p->n); break;
    case K_COMPOSITE: snprintf(buf, sizeof buf, "CT%lld(", p->n); break;
    case K_CHIRP: snprintf(buf, sizeof buf, "BL%lld(", p->n); break;
  }
  s += buf;
  plan_string(p->a, s);
  if (p->b) { s += ","; plan_string(p->b, s); }
  s += ")";
}

// mode: 0 = transform (auto), 1 = transformDecompose, 2 = transformChirp2,
//       3 = transformChirp235   (Planned.hs:103-130,704-729)
static const Plan* plan_for_mode(PlanSet& ps, int mode, i64 n) {
  switch (mode) {
    case 0: return ps.automatic(n);
    case 1: return ps.decompose(n);
    case 2: return ps.chirp(n, true);
    case 3: return ps.chirp(n, false);
  }
  return nullptr;
}

// ---------------------------------------------------------------------------
// Permutation.hs

// Permutation.hs:48-54 multiplicative: perm[i] = g^i mod p - 1, i < p-1
static std::vector<i64> perm_multiplicative(i64 p) {
  i64 g = multiplicative_generator(p);
  std::vector<i64> out(p - 1);
  i64 x = 1;
  for (i64 i = 0; i < p - 1; ++i) { out[i] = x - 1; x = (i64)(((__int128)g * x) % p); }
  return out;
}
// Permutation.hs:68-73 inverse
static std::vector<i64> perm_inverse(const std::vector<i64>& p) {
  std::vector<i64> out(p.size(), 0);
  for (size_t i = 0; i < p.size(); ++i) out[p[i]] += (i64)i;
  return out;
}
// Permutation.hs:75-80 reverse: out[i] = p[(-i) mod n]
static std::vector<i64> perm_reverse(const std::vector<i64>& p) {
  i64 n = (i64)p.size();
  std::vector<i64> out(n);
  for (i64 i = 0; i < n; ++i) out[i] = p[((-i) % n + n) % n];
  return out;
}

// ---------------------------------------------------------------------------
// Caches and the executor (Planned.hs:300-441 cache, 137-167 transformWithCache)

template <class T> struct Cache {
  const Plan* p = nullptr;
  T sign = 0;
  bool split = false;                 // SR node executed as split-radix step
  std::vector<cx<T>> tw, tw1, tw3;     // radix-2 / split-radix twiddles
  cx<T> imag;                          // Private.hs:347-350 imagSplitRadixPlain
  cx<T> z[4];                          // small caches
  const Cache* sub = nullptr;
  const Cache* sub2 = nullptr;
  std::vector<i64> rev, inv;          // Rader permutations
  std::vector<cx<T>> zs;              // Rader kernel spectrum / chirp spectrum
  std::vector<cx<T>> chirp;           // Bluestein chirp (first len entries)
  std::vector<cx<T>> tw2d;            // Cooley-Tukey twiddles
  const Cache* subInv = nullptr;      // inverse-direction sub cache
  const Cache* subFwd = nullptr;      // forward-direction sub cache
};

template <class T> struct CacheSet {
  std::vector<std::unique_ptr<Cache<T>>> arena;
  std::map<std::pair<i64, int>, const Cache<T>*> memo;  // CacheMap (Planned.hs:348)
  const Cache<T>* get(const Plan* p, T sign);
  const Cache<T>* build(const Plan* p, T sign);
};

template <class T> static void exec(const Cache<T>* c, const cx<T>* x, i64 xs, cx<T>* y);

// Private.hs:56-82 cache2..cache5
template <class T> static void small_cache(int s, T sign, cx<T>* z) {
  if (s == 2) { z[0] = cx<T>(-1, 0); return; }
  if (s == 3) {
    T sq = std::sqrt((T)3) / (T)2, mh = (T)-1 / (T)2;
    z[0] = cx<T>(mh, sign * sq);
    z[1] = cx<T>(mh, (-sign) * sq);
    return;
  }
  if (s == 4) { z[0] = cx<T>(0, sign); z[1] = cx<T>(-1, 0); z[2] = cx<T>(0, -sign); return; }
  for (int k = 1; k <= 4; ++k) z[k - 1] = cis_rat<T>(sign, 5, k);
}

// Private.hs:264-276 twiddleFactors2: cis sign (pi*k/n2)
template <class T> static std::vector<cx<T>> twiddle_factors2(T sign, i64 n2) {
  std::vector<cx<T>> t(n2);
  for (i64 k = 0; k < n2; ++k) t[k] = cis<T>(sign, pi_t<T>() * (T)k / (T)n2);
  return t;
}
// Private.hs:390-411 twiddleFactorsSR: cis sign (pi*(k*j)/(2*n4))
template <class T> static std::vector<cx<T>> twiddle_factors_sr(T sign, i64 n4, i64 k) {
  std::vector<cx<T>> t(n4);
  for (i64 j = 0; j < n4; ++j) t[j] = cis<T>(sign, pi_t<T>() * ((T)k * (T)j) / ((T)2 * (T)n4));
  return t;
}
// Private.hs:428-436 chirp
template <class T> static std::vector<cx<T>> chirp_vec(T sign, i64 pad, i64 len) {
  std::vector<cx<T>> c(pad);
  for (i64 k = 0; k < pad; ++k) {
    T sk = (T)(pad > 2 * k ? k : k - pad);
    c[k] = cis<T>(sign, pi_t<T>() * sk * sk / (T)len);
  }
  return c;
}

template <class T> const Cache<T>* CacheSet<T>::get(const Plan* p, T sign) {
  // Planned.hs:420-432 key (len, Direction)
  auto key = std::make_pair(p->n, sign > 0 ? 1 : 0);
  auto it = memo.find(key);
  if (it != memo.end() && it->second->p == p) return it->second;
  const Cache<T>* c = build(p, sign);
  memo[key] = c;
  return c;
}

template <class T> const Cache<T>* CacheSet<T>::build(const Plan* p, T sign) {
  arena.emplace_back(new Cache<T>());
  Cache<T>* c = arena.back().get();
  c->p = p;
  c->sign = sign;
  switch (p->kind) {
    case K_ID: break;
    case K_SMALL: small_cache<T>(p->small, sign, c->z); break;
    case K_SR: {  // Planned.hs:376-391
      const Plan* sub = p->a;
      i64 n2 = sub->n;
      c->sub = get(sub, sign);
      if (sub->kind == K_SR) {
        c->split = true;
        c->sub2 = get(sub->a, sign);
        c->imag = cx<T>(0, sign);  // Private.hs:347-350
        c->tw1 = twiddle_factors_sr<T>(sign, n2 / 2, 1);  // Planned.hs:494-499
        c->tw3 = twiddle_factors_sr<T>(sign, n2 / 2, 3);
      } else {
        c->tw = twiddle_factors2<T>(sign, n2);  // Planned.hs:473-478
      }
      break;
    }
    case K_PRIME: {  // Planned.hs:392-402, 650-664
      i64 len = p->n;
      c->subInv = get(p->a, (T)1);
      c->subFwd = get(p->a, (T)-1);
      std::vector<i64> perm = perm_multiplicative(len);
      c->rev = perm_reverse(perm);
      c->inv = perm_inverse(perm);
      std::vector<cx<T>> kernel(len - 1), spec(len - 1);
      for (i64 i = 0; i < len - 1; ++i) kernel[i] = cis_rat<T>(sign, len, 1 + perm[i]);
      exec(c->subInv, kernel.data(), 1, spec.data());
      T s = (T)1 / (T)(len - 1);  // Utility.hs:17-26 scaleDown
      for (auto& v : spec) v = cx<T>(s * v.real(), s * v.imag());
      c->zs = spec;
      break;
    }
    case K_COPRIME:  // Planned.hs:403-405
      c->sub = get(p->a, sign);
      c->sub2 = get(p->b, sign);
      break;
    case K_COMPOSITE: {  // Planned.hs:406-409, 529-534; Private.hs:279-291
      c->sub = get(p->a, sign);
      c->sub2 = get(p->b, sign);
      i64 n = p->a->n, m = p->b->n;
      c->tw2d.resize(n * m);
      for (i64 k = 0; k < n; ++k)
        for (i64 j = 0; j < m; ++j) c->tw2d[k * m + j] = cis_rat<T>(sign, n * m, (k * j) % (n * m));
      break;
    }
    case K_CHIRP: {  // Planned.hs:410-418, 744-754
      i64 pad = p->a->n, len = p->n;
      c->subInv = get(p->a, (T)1);
      c->subFwd = get(p->a, (T)-1);
      std::vector<cx<T>> ch = chirp_vec<T>(sign, pad, len);
      c->chirp.assign(ch.begin(), ch.begin() + len);
      std::vector<cx<T>> cj(pad), spec(pad);
      for (i64 i = 0; i < pad; ++i) cj[i] = std::conj(ch[i]);
      exec(c->subInv, cj.data(), 1, spec.data());
      T s = (T)1 / (T)pad;
      for (auto& v : spec) v = cx<T>(s * v.real(), s * v.imag());
      c->zs = spec;
      break;
    }
  }
  return c;
}

// Private.hs:95-103 transform2
template <class T> static inline void small2(cx<T> z, const cx<T>* x, i64 xs, cx<T>* y) {
  cx<T> x0 = x[0], x1 = x[xs];
  y[0] = cadd(x0, x1);
  y[1] = cadd(x0, cmul(z, x1));
}
// Private.hs:120-131 transform3 with Convolution/Small.hs:160-167 sumAndConvolvePair
template <class T> static inline void small3(const cx<T>* z, const cx<T>* x, i64 xs, cx<T>* y) {
  cx<T> x0 = x[0], a0 = x[xs], a1 = x[2 * xs], b0 = z[0], b1 = z[1];
  cx<T> sa01 = cadd(a0, a1), sb01 = cadd(b0, b1);
  cx<T> ab = cadd(cmul(a0, b0), cmul(a1, b1));
  cx<T> zx2 = csub(cmul(sa01, sb01), ab);
  y[0] = cadd(x0, sa01);
  y[1] = cadd(x0, ab);
  y[2] = cadd(x0, zx2);
}
// Private.hs:150-164 transform4
template <class T> static inline void small4(const cx<T>* zz, const cx<T>* x, i64 xs, cx<T>* y) {
  cx<T> z = zz[0], z2 = zz[1], z3 = zz[2];
  cx<T> x0 = x[0], x1 = x[xs], x2 = x[2 * xs], x3 = x[3 * xs];
  cx<T> x02a = cadd(x0, x2), x02b = cadd(x0, cmul(z2, x2));
  cx<T> x13a = cadd(x1, x3), x13b = cadd(x1, cmul(z2, x3));
  y[0] = cadd(x02a, x13a);
  y[1] = cadd(x02b, cmul(z, x13b));
  y[2] = cadd(x02a, cmul(z2, x13a));
  y[3] = cadd(x02b, cmul(z3, x13b));
}
// Convolution/Small.hs:203-226 sumAndConvolveQuadruple
template <class T>
static inline void sum_conv_quad(const cx<T>* a, const cx<T>* b, cx<T>& sa, cx<T>* d) {
  cx<T> ab0 = cmul(a[0], b[0]), ab1 = cmul(a[1], b[1]);
  cx<T> sa01 = cadd(a[0], a[1]), sb01 = cadd(b[0], b[1]);
  cx<T> ab01 = csub(cmul(sa01, sb01), cadd(ab0, ab1));
  cx<T> ab2 = cmul(a[2], b[2]), ab3 = cmul(a[3], b[3]);
  cx<T> sa23 = cadd(a[2], a[3]), sb23 = cadd(b[2], b[3]);
  cx<T> ab23 = csub(cmul(sa23, sb23), cadd(ab2, ab3));
  cx<T> c0 = csub(cadd(ab0, ab2), cadd(ab1, ab3));
  cx<T> c1 = cadd(ab01, ab23);
  cx<T> ab02 = cmul(cadd(a[0], a[2]), cadd(b[0], b[2]));
  cx<T> ab13 = cmul(cadd(a[1], a[3]), cadd(b[1], b[3]));
  cx<T> sa0123 = cadd(sa01, sa23), sb0123 = cadd(sb01, sb23);
  cx<T> ab0123 = csub(cmul(sa0123, sb0123), cadd(ab02, ab13));
  d[0] = cadd(ab13, c0);
  d[1] = c1;
  d[2] = csub(ab02, c0);
  d[3] = csub(ab0123, c1);
  sa = sa0123;
}
// Private.hs:204-218 transform5
template <class T> static inline void small5(const cx<T>* z, const cx<T>* x, i64 xs, cx<T>* y) {
  cx<T> x0 = x[0];
  cx<T> a[4] = {x[xs], x[3 * xs], x[4 * xs], x[2 * xs]};
  cx<T> b[4] = {z[0], z[1], z[3], z[2]};
  cx<T> s, d[4];
  sum_conv_quad(a, b, s, d);  // (d1,d2,d4,d3)
  y[0] = cadd(x0, s);
  y[1] = cadd(x0, d[0]);
  y[2] = cadd(x0, d[1]);
  y[3] = cadd(x0, d[3]);
  y[4] = cadd(x0, d[2]);
}

template <class T> static void exec(const Cache<T>* c, const cx<T>* x, i64 xs, cx<T>* y) {
  const Plan* p = c->p;
  i64 n = p->n;
  switch (p->kind) {
    case K_ID:
      for (i64 i = 0; i < n; ++i) y[i] = x[i * xs];
      return;
    case K_SMALL:
      switch (p->small) {
        case 2: small2(c->z[0], x, xs, y); return;
        case 3: small3(c->z, x, xs, y); return;
        case 4: small4(c->z, x, xs, y); return;
        case 5: small5(c->z, x, xs, y); return;
      }
      return;
    case K_SR: {
      i64 n2 = n / 2;
      if (c->split) {
        // Private.hs:358-364 ditSplitRadixReorder, 371-387 ditSplitRadixStep
        i64 n4 = n2 / 2;
        std::vector<cx<T>> E(n2), Z1(n4), Z3(n4);
        exec(c->sub, x, 2 * xs, E.data());
        exec(c->sub2, x + xs, 4 * xs, Z1.data());
        exec(c->sub2, x + 3 * xs, 4 * xs, Z3.data());
        for (i64 k = 0; k < n4; ++k) {
          cx<T> a = cmul(c->tw1[k], Z1[k]), b = cmul(c->tw3[k], Z3[k]);
          cx<T> zsum = cadd(a, b), zdiff = cmul(c->imag, csub(a, b));
          y[k] = cadd(E[k], zsum);
          y[k + n4] = cadd(E[k + n4], zdiff);
          y[k + n2] = csub(E[k], zsum);
          y[k + n2 + n4] = csub(E[k + n4], zdiff);
        }
      } else {
        // Private.hs:294-313 transformRadix2InterleavedTime
        std::vector<cx<T>> E(n2), O(n2);
        exec(c->sub, x, 2 * xs, E.data());
        exec(c->sub, x + xs, 2 * xs, O.data());
        for (i64 k = 0; k < n2; ++k) {
          cx<T> o = cmul(c->tw[k], O[k]);
          y[k] = cadd(E[k], o);
          y[k + n2] = csub(E[k], o);
        }
      }
      return;
    }
    case K_PRIME: {
      // Planned.hs:669-692 transformPrime
      i64 m = n - 1;
      cx<T> x0 = x[0];
      std::vector<cx<T>> a(m), u(m), c2(m);
      for (i64 i = 0; i < m; ++i) a[i] = x[(1 + c->rev[i]) * xs];  // Permutation.apply rev res
      exec(c->subInv, a.data(), 1, u.data());                     // trans (inverse dir)
      for (i64 i = 0; i < m; ++i) u[i] = cmul(c->zs[i], u[i]);      // zipWith (*) zs
      exec(c->subFwd, u.data(), 1, c2.data());                    // transInv (forward dir)
      cx<T> sum = x[xs];
      for (i64 i = 1; i < m; ++i) sum = cadd(sum, x[(1 + i) * xs]);   // fold1 (+) res
      y[0] = cadd(x0, sum);
      for (i64 k = 0; k < m; ++k) y[1 + k] = cadd(x0, c2[c->inv[k]]);  // apply inv
      return;
    }
    case K_COPRIME: {
      // Planned.hs:584-617 transformCoprime / permuteSkewGrid(Inv)
      i64 nn = p->a->n, mm = p->b->n;
      std::vector<cx<T>> M(nn), A(mm * nn), B(mm), C(nn * mm);
      for (i64 k = 0; k < mm; ++k) {
        for (i64 j = 0; j < nn; ++j) M[j] = x[((nn * k + mm * j) % n) * xs];
        exec(c->sub, M.data(), 1, A.data() + k * nn);
      }
      for (i64 q = 0; q < nn; ++q) {
        for (i64 k = 0; k < mm; ++k) B[k] = A[k * nn + q];  // transpose
        exec(c->sub2, B.data(), 1, C.data() + q * mm);
      }
      for (i64 r = 0; r < n; ++r) y[r] = C[(r % nn) * mm + (r % mm)];
      return;
    }
    case K_COMPOSITE: {
      // Planned.hs:543-557 transformComposite; Private.hs:233-243 merge
      i64 nn = p->a->n, mm = p->b->n;
      std::vector<cx<T>> Y(nn * mm), Z(nn), W(mm * nn);
      for (i64 k = 0; k < nn; ++k) {
        exec(c->sub2, x + k * xs, nn * xs, Y.data() + k * mm);  // sliceHorizontal; subTransM
        for (i64 l = 0; l < mm; ++l) Y[k * mm + l] = cmul(c->tw2d[k * mm + l], Y[k * mm + l]);
      }
      for (i64 l = 0; l < mm; ++l) {
        for (i64 k = 0; k < nn; ++k) Z[k] = Y[k * mm + l];  // transpose
        exec(c->sub, Z.data(), 1, W.data() + l * nn);       // subTransN
      }
      for (i64 r = 0; r < n; ++r) y[r] = W[(r % mm) * nn + (r / mm)];
      return;
    }
    case K_CHIRP: {
      // Planned.hs:760-773 transformChirp
      i64 pad = p->a->n;
      std::vector<cx<T>> t(pad, cx<T>(0, 0)), u(pad), v(pad);
      for (i64 i = 0; i < n; ++i) t[i] = cmul(c->chirp[i], x[i * xs]);
      exec(c->subInv, t.data(), 1, u.data());
      for (i64 i = 0; i < pad; ++i) u[i] = cmul(c->zs[i], u[i]);
      exec(c->subFwd, u.data(), 1, v.data());
      for (i64 i = 0; i < n; ++i) y[i] = cmul(c->chirp[i], v[i]);
      return;
    }
  }
}

// ---------------------------------------------------------------------------
// Preprocessed.hs / Adhoc.hs algorithm variants (all restated per row)

// Preprocessed.hs:479-491 dit2 (recursive radix-2 DIT, base len<=1)
template <class T> static void prep_dit2(T sign, i64 n, const cx<T>* x, i64 xs, cx<T>* y) {
  if (n <= 1) { for (i64 i = 0; i < n; ++i) y[i] = x[i * xs]; return; }
  i64 n2 = n / 2;
  std::vector<cx<T>> E(n2), O(n2);
  prep_dit2(sign, n2, x, 2 * xs, E.data());
  prep_dit2(sign, n2, x + xs, 2 * xs, O.data());
  std::vector<cx<T>> tw = twiddle_factors2<T>(sign, n2);
  for (i64 k = 0; k < n2; ++k) {
    cx<T> o = cmul(tw[k], O[k]);
    y[k] = cadd(E[k], o);
    y[k + n2] = csub(E[k], o);
  }
}

// Preprocessed.hs:497-515 dif2
template <class T> static void prep_dif2(T sign, i64 n, const cx<T>* x, i64 xs, cx<T>* y) {
  if (n <= 1) { for (i64 i = 0; i < n; ++i) y[i] = x[i * xs]; return; }
  i64 n2 = n / 2;
  std::vector<cx<T>> tw = twiddle_factors2<T>(sign, n2);
  std::vector<cx<T>> ev(n2), od(n2), E(n2), O(n2);
  for (i64 k = 0; k < n2; ++k) {
    ev[k] = cadd(x[k * xs], x[(k + n2) * xs]);
    od[k] = cmul(tw[k], csub(x[k * xs], x[(k + n2) * xs]));
  }
  prep_dif2(sign, n2, ev.data(), 1, E.data());
  prep_dif2(sign, n2, od.data(), 1, O.data());
  for (i64 q = 0; q < n2; ++q) { y[2 * q] = E[q]; y[2 * q + 1] = O[q]; }  // merge
}

// Preprocessed.hs:433-473 ditSplitRadix / Adhoc.hs:101-132 ditSplitRadix(Loop):
// split-radix down to the transform2 (-1) base (Private.hs:366-369).
template <class T> static void split_radix_pure(T sign, i64 n, const cx<T>* x, i64 xs, cx<T>* y) {
  if (n <= 1) { for (i64 i = 0; i < n; ++i) y[i] = x[i * xs]; return; }
  if (n == 2) { small2(cx<T>(-1, 0), x, xs, y); return; }
  i64 n2 = n / 2, n4 = n2 / 2;
  std::vector<cx<T>> E(n2), Z1(n4), Z3(n4);
  split_radix_pure(sign, n2, x, 2 * xs, E.data());
  split_radix_pure(sign, n4, x + xs, 4 * xs, Z1.data());
  split_radix_pure(sign, n4, x + 3 * xs, 4 * xs, Z3.data());
  std::vector<cx<T>> tw1 = twiddle_factors_sr<T>(sign, n4, 1), tw3 = twiddle_factors_sr<T>(sign, n4, 3);
  cx<T> imag(0, sign);
  for (i64 k = 0; k < n4; ++k) {
    cx<T> a = cmul(tw1[k], Z1[k]), b = cmul(tw3[k], Z3[k]);
    cx<T> zsum = cadd(a, b), zdiff = cmul(imag, csub(a, b));
    y[k] = cadd(E[k], zsum);
    y[k + n4] = cadd(E[k + n4], zdiff);
    y[k + n2] = csub(E[k], zsum);
    y[k + n2 + n4] = csub(E[k + n4], zdiff);
  }
}

// Adhoc.hs:138-163 dit2 (iterative twist then ditStep, same arithmetic as the
// recursive DIT with twiddleFactors2 over the current row length)
template <class T> static void adhoc_dit2(T sign, i64 n, const cx<T>* x, i64 xs, cx<T>* y) {
  prep_dit2(sign, n, x, xs, y);
}

// Adhoc.hs:171-223 dit235 / dit235Step
template <class T> static void adhoc_dit235(T sign, i64 n, const cx<T>* x, i64 xs, cx<T>* y) {
  if (n <= 1) { for (i64 i = 0; i < n; ++i) y[i] = x[i * xs]; return; }
  int fac = (n % 3 == 0) ? 3 : (n % 4 == 0) ? 4 : (n % 5 == 0) ? 5 : 2;  // Adhoc.hs:191-199
  i64 len = n / fac;
  std::vector<cx<T>> Y(n);
  for (int s = 0; s < fac; ++s) adhoc_dit235(sign, len, x + s * xs, fac * xs, Y.data() + s * len);
  cx<T> z[4];
  small_cache<T>(fac, sign, z);
  std::vector<cx<T>> v(fac), o(fac);
  for (i64 k = 0; k < len; ++k) {
    for (int s = 0; s < fac; ++s)  // Private.hs:287-291 twiddle sign (fac*len) s k
      v[s] = cmul(cis_rat<T>(sign, fac * len, (s * k) % (fac * len)), Y[s * len + k]);
    switch (fac) {
      case 2: small2(z[0], v.data(), 1, o.data()); break;
      case 3: small3(z, v.data(), 1, o.data()); break;
      case 4: small4(z, v.data(), 1, o.data()); break;
      case 5: small5(z, v.data(), 1, o.data()); break;
    }
    for (int q = 0; q < fac; ++q) y[k + len * q] = o[q];  // merge
  }
}

// Adhoc.hs:316-337 transformChirp with analysis/synthesis sub transforms
template <class T, class F>
static void adhoc_chirp(T sign, i64 n, i64 pad, F sub, const cx<T>* x, i64 xs, cx<T>* y) {
  if (n <= 1) { for (i64 i = 0; i < n; ++i) y[i] = x[i * xs]; return; }
  std::vector<cx<T>> ch = chirp_vec<T>(sign, pad, n);
  std::vector<cx<T>> cj(pad), A(pad), t(pad, cx<T>(0, 0)), B(pad), C(pad);
  for (i64 i = 0; i < pad; ++i) cj[i] = std::conj(ch[i]);
  sub((T)-1, pad, cj.data(), A.data());
  for (i64 i = 0; i < n; ++i) t[i] = cmul(ch[i], x[i * xs]);
  sub((T)-1, pad, t.data(), B.data());
  for (i64 i = 0; i < pad; ++i) B[i] = cmul(A[i], B[i]);
  sub((T)1, pad, B.data(), C.data());
  T s = (T)1 / (T)pad;
  for (i64 i = 0; i < n; ++i) {
    cx<T> v = cmul(ch[i], C[i]);
    y[i] = cx<T>(s * v.real(), s * v.imag());
  }
}

// Adhoc.hs:86-95 is2or5smooth
static void is2or5smooth(i64 len, bool& pow2, bool& smooth5) {
  i64 mp = len & (-len);
  i64 odd = len / mp;
  pow2 = odd == 1;
  while (odd % 3 == 0) odd /= 3;
  while (odd % 5 == 0) odd /= 5;
  smooth5 = odd == 1;
}

// algo: 0 prep dit2, 1 prep dif2, 2 prep ditSplitRadix, 3 adhoc dit2,
//       4 adhoc ditSplitRadix, 5 adhoc dit235, 6 adhoc chirp2, 7 adhoc chirp235,
//       8 adhoc transform (auto)
template <class T> static void variant(int algo, T sign, i64 n, const cx<T>* x, cx<T>* y) {
  auto sr = [](T s, i64 m, const cx<T>* a, cx<T>* b) { split_radix_pure<T>(s, m, a, 1, b); };
  auto d235 = [](T s, i64 m, const cx<T>* a, cx<T>* b) { adhoc_dit235<T>(s, m, a, 1, b); };
  switch (algo) {
    case 0: prep_dit2(sign, n, x, 1, y); return;
    case 1: prep_dif2(sign, n, x, 1, y); return;
    case 2: case 4: split_radix_pure(sign, n, x, 1, y); return;
    case 3: adhoc_dit2(sign, n, x, 1, y); return;
    case 5: adhoc_dit235(sign, n, x, 1, y); return;
    case 6: {  // Adhoc.hs:342-350
      i64 pad = n <= 1 ? 1 : ((i64)1 << ceiling_log_base(2, (double)(2 * n - 1)));
      adhoc_chirp<T>(sign, n, pad, sr, x, 1, y);
      return;
    }
    case 7: {  // Adhoc.hs:355-362
      i64 pad = n <= 1 ? 1 : adhoc_ceiling_5smooth(2 * n);
      adhoc_chirp<T>(sign, n, pad, d235, x, 1, y);
      return;
    }
    case 8: {  // Adhoc.hs:74-84
      if (n <= 1) { for (i64 i = 0; i < n; ++i) y[i] = x[i]; return; }
      bool p2, s5;
      is2or5smooth(n, p2, s5);
      if (p2) split_radix_pure(sign, n, x, 1, y);
      else if (s5) adhoc_dit235(sign, n, x, 1, y);
      else variant<T>(7, sign, n, x, y);
      return;
    }
  }
}

// ---------------------------------------------------------------------------
// Plan handles (plan + cache built once, executed many times: mirrors
// Planned.transform = transformWithCache (cache sign len), Planned.hs:103-106)

struct Handle {
  PlanSet ps;
  const Plan* p = nullptr;
  CacheSet<double> cs64;
  CacheSet<float> cs32;
  const Cache<double>* c64 = nullptr;
  const Cache<float>* c32 = nullptr;
};

template <class T> static int nthreads_of(int t) {
#ifdef _OPENMP
  return t > 0 ? t : omp_get_max_threads();
#else
  (void)t; return 1;
#endif
}

extern "C" {

int or_version() { return 3; }

int or_max_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

i64 or_ceiling_pow2(i64 n) { return ceiling_power_of_two(n); }
i64 or_ceiling_5smooth(i64 n) { return ceiling_5smooth(n); }
i64 or_adhoc_ceiling_5smooth(i64 n) { return adhoc_ceiling_5smooth(n); }
i64 or_multiplicative_generator(i64 p) { return multiplicative_generator(p); }
i64 or_modular_power(i64 m, i64 e, i64 n) { return modular_power(m, e, n); }

int or_fermat_factors(i64 n, i64* out, int maxpairs) {
  auto f = fermat_factors(n);
  int k = 0;
  for (auto& q : f) {
    if (k >= maxpairs) break;
    out[2 * k] = q.first;
    out[2 * k + 1] = q.second;
    ++k;
  }
  return (int)f.size();
}

int or_plan_string(int mode, i64 n, char* buf, int buflen) {
  PlanSet ps;
  const Plan* p = plan_for_mode(ps, mode, n);
  std::string s;
  plan_string(p, s);
  if ((int)s.size() + 1 > buflen) return -(int)s.size() - 1;
  memcpy(buf, s.c_str(), s.size() + 1);
  return (int)s.size();
}

int or_plan_count_primes(i64 n) {
  PlanSet ps;
  return PlanSet::count_primes(ps.decompose(n));
}

// Rader permutation tables (Permutation.hs:48-80)
void or_rader_perms(i64 p, i64* perm, i64* rev, i64* inv) {
  auto pm = perm_multiplicative(p);
  auto r = perm_reverse(pm);
  auto iv = perm_inverse(pm);
  for (i64 i = 0; i < p - 1; ++i) { perm[i] = pm[i]; rev[i] = r[i]; inv[i] = iv[i]; }
}

// Good-Thomas index maps (Planned.hs:597-617): fwd[k*n + j] = (n*k + m*j) mod nm
// for the m x n grid; inv_q[r] = r mod n, inv_p[r] = r mod m.
void or_skew_grid(i64 n, i64 m, i64* fwd, i64* inv_q, i64* inv_p) {
  i64 nm = n * m;
  for (i64 k = 0; k < m; ++k)
    for (i64 j = 0; j < n; ++j) fwd[k * n + j] = (n * k + m * j) % nm;
  for (i64 r = 0; r < nm; ++r) { inv_q[r] = r % n; inv_p[r] = r % m; }
}

void* or_handle_create(int mode, int sign, i64 n) {
  Handle* h = new Handle();
  h->p = plan_for_mode(h->ps, mode, n);
  h->c64 = h->cs64.get(h->p, (double)sign);
  h->c32 = h->cs32.get(h->p, (float)sign);
  return h;
}
void or_handle_destroy(void* h) { delete (Handle*)h; }
i64 or_handle_n(void* h) { return ((Handle*)h)->p->n; }

void or_handle_exec_f64(void* hv, i64 batch, const double* in, double* out, int threads) {
  Handle* h = (Handle*)hv;
  i64 n = h->p->n;
  const cx<double>* x = (const cx<double>*)in;
  cx<double>* y = (cx<double>*)out;
  int nt = nthreads_of<double>(threads);
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt) if (batch > 1)
  for (i64 b = 0; b < batch; ++b) exec(h->c64, x + b * n, 1, y + b * n);
}
void or_handle_exec_f32(void* hv, i64 batch, const float* in, float* out, int threads) {
  Handle* h = (Handle*)hv;
  i64 n = h->p->n;
  const cx<float>* x = (const cx<float>*)in;
  cx<float>* y = (cx<float>*)out;
  int nt = nthreads_of<float>(threads);
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt) if (batch > 1)
  for (i64 b = 0; b < batch; ++b) exec(h->c32, x + b * n, 1, y + b * n);
}

// One-shot planned transform (mode as in plan_for_mode) on batch rows.
void or_planned(int mode, int sign, i64 n, i64 batch, const double* in, double* out) {
  void* h = or_handle_create(mode, sign, n);
  or_handle_exec_f64(h, batch, in, out, 0);
  or_handle_destroy(h);
}

// Preprocessed/Adhoc variants (see `variant`)
void or_variant(int algo, int sign, i64 n, i64 batch, const double* in, double* out) {
  const cx<double>* x = (const cx<double>*)in;
  cx<double>* y = (cx<double>*)out;
#pragma omp parallel for schedule(dynamic, 1) if (batch > 1)
  for (i64 b = 0; b < batch; ++b) variant<double>(algo, (double)sign, n, x + b * n, y + b * n);
}

// Independent check: naive DFT in long double with exact phase reduction.
void or_naive_dft(int sign, i64 n, i64 batch, const double* in, double* out) {
#pragma omp parallel for schedule(dynamic, 1) if (batch > 1)
  for (i64 b = 0; b < batch; ++b) {
    const double* x = in + 2 * b * n;
    double* y = out + 2 * b * n;
    for (i64 k = 0; k < n; ++k) {
      long double sr = 0, si = 0;
      for (i64 j = 0; j < n; ++j) {
        i64 e = (i64)(((__int128)j * k) % n);
        long double w = 2.0L * 3.141592653589793238462643383279502884L * (long double)e / (long double)n;
        long double c = cosl(w), s = sign * sinl(w);
        sr += (long double)x[2 * j] * c - (long double)x[2 * j + 1] * s;
        si += (long double)x[2 * j] * s + (long double)x[2 * j + 1] * c;
      }
      y[2 * k] = (double)sr;
      y[2 * k + 1] = (double)si;
    }
  }
}

// Utility.hs:17-26 scaleDown
void or_scale_down(i64 n, i64 batch, double* io) {
  double s = 1.0 / (double)n;
  for (i64 i = 0; i < 2 * n * batch; ++i) io[i] = s * io[i];
}

// Cyclic.hs:20-28 reverse: out[k] = in[(-k) mod n]
void or_cyclic_reverse(i64 n, i64 batch, const double* in, double* out) {
  for (i64 b = 0; b < batch; ++b)
    for (i64 k = 0; k < n; ++k) {
      i64 s = ((-k) % n + n) % n;
      out[2 * (b * n + k)] = in[2 * (b * n + s)];
      out[2 * (b * n + k) + 1] = in[2 * (b * n + s) + 1];
    }
}

// Real.hs:49-70 toSpectrum with subTrans = Planned.transform forward (n/2).
// x: batch x n reals; out: batch x n complex (full spectrum).
void or_to_spectrum(i64 n, i64 batch, const double* x, double* out) {
  i64 n2 = n / 2;
  Handle* h = (Handle*)or_handle_create(0, -1, n2);
  std::vector<cx<double>> tw = twiddle_factors2<double>(-1.0, n2);
  for (auto& t : tw) t = cmul(cx<double>(0, 1), t);  // imagUnit *
  for (i64 b = 0; b < batch; ++b) {
    std::vector<cx<double>> z(n2), Z(n2);
    for (i64 j = 0; j < n2; ++j) z[j] = cx<double>(x[b * n + 2 * j], x[b * n + 2 * j + 1]);
    exec(h->c64, z.data(), 1, Z.data());
    cx<double>* y = (cx<double>*)out + b * n;
    for (i64 k = 0; k < n2; ++k) {
      cx<double> r = Z[n2 ? ((-k) % n2 + n2) % n2 : 0];
      cx<double> sp = cadd(Z[k], r), sm = csub(Z[k], r);
      cx<double> xp(sp.real() / 2, sp.imag() / 2), xm(sm.real() / 2, sm.imag() / 2);
      cx<double> ev(xp.real(), xm.imag());
      cx<double> od = cmul(tw[k], cx<double>(xm.real(), xp.imag()));
      y[k] = csub(ev, od);
      y[k + n2] = cadd(ev, od);
    }
  }
  or_handle_destroy(h);
}

// Real.hs:92-121 fromSpectrum with subTrans = Planned.transform inverse (n/2).
void or_from_spectrum(i64 n, i64 batch, const double* spec, double* out) {
  i64 n2 = n / 2;
  Handle* h = (Handle*)or_handle_create(0, 1, n2);
  std::vector<cx<double>> tw = twiddle_factors2<double>(1.0, n2);
  for (auto& t : tw) t = cmul(cx<double>(0, 1), t);
  for (i64 b = 0; b < batch; ++b) {
    const cx<double>* s = (const cx<double>*)spec + b * n;
    std::vector<cx<double>> f(n2), F(n2);
    for (i64 k = 0; k < n2; ++k) {
      cx<double> fe = cadd(s[k], s[k + n2]);
      cx<double> fo = cmul(tw[k], csub(s[k], s[k + n2]));
      f[k] = cadd(fe, fo);
    }
    exec(h->c64, f.data(), 1, F.data());
    for (i64 j = 0; j < n2; ++j) { out[b * n + 2 * j] = F[j].real(); out[b * n + 2 * j + 1] = F[j].imag(); }
  }
  or_handle_destroy(h);
}

// Real.hs:168-187 untangleSpectra: (a + conj b)/2, (a - conj b)*(-i/2), b = reverse a
void or_untangle(i64 n, i64 batch, const double* spec, double* outa, double* outb) {
  for (i64 b = 0; b < batch; ++b) {
    const cx<double>* s = (const cx<double>*)spec + b * n;
    cx<double>* A = (cx<double>*)outa + b * n;
    cx<double>* B = (cx<double>*)outb + b * n;
    for (i64 k = 0; k < n; ++k) {
      cx<double> a = s[k], bb = s[((-k) % n + n) % n];
      cx<double> bc = std::conj(bb);
      cx<double> sp = cadd(a, bc), sm = csub(a, bc);
      A[k] = cx<double>(sp.real() / 2, sp.imag() / 2);
      B[k] = cmul(sm, cx<double>(-0.0 / 2, -1.0 / 2));
    }
  }
}
// Real.hs:231-236 entangleCoefficient (first component): c + d*i
void or_entangle(i64 n, i64 batch, const double* c, double* d, double* out) {
  for (i64 i = 0; i < n * batch; ++i) {
    cx<double> cc(c[2 * i], c[2 * i + 1]), dd(d[2 * i], d[2 * i + 1]);
    cx<double> di = cmul(dd, cx<double>(0, 1));
    cx<double> r = cadd(cc, di);
    out[2 * i] = r.real();
    out[2 * i + 1] = r.imag();
  }
}

// Planned.hs:779-821 convolveCyclic: F(scaleDown(G x) * G y)
void or_convolve_cyclic(i64 n, i64 batch, const double* x, const double* yv, double* out) {
  Handle* g = (Handle*)or_handle_create(0, 1, n);
  Handle* f = (Handle*)or_handle_create(0, -1, n);
  for (i64 b = 0; b < batch; ++b) {
    std::vector<cx<double>> gx(n), gy(n), pr(n);
    exec(g->c64, (const cx<double>*)x + b * n, 1, gx.data());
    exec(g->c64, (const cx<double>*)yv + b * n, 1, gy.data());
    double s = 1.0 / (double)n;
    for (i64 i = 0; i < n; ++i) pr[i] = cmul(cx<double>(s * gx[i].real(), s * gx[i].imag()), gy[i]);
    exec(f->c64, pr.data(), 1, (cx<double>*)out + b * n);
  }
  or_handle_destroy(g);
  or_handle_destroy(f);
}

// Convolution/Adhoc.hs:36-98 karatsuba (loop form) over rows of length L;
// output rows of length max 0 (2L-1).  Generic over the ring (int64, double).
}  // extern "C"
template <class R>
static void karatsuba_loop(i64 L, i64 batch, const R* x, const R* y, R* z) {
  i64 zl = L > 0 ? 2 * L - 1 : 0;
  for (i64 b = 0; b < batch; ++b) {
    std::vector<R> xs(x + b * L, x + (b + 1) * L), ys(y + b * L, y + (b + 1) * L);
    i64 cnt = 1, len = L;
    std::vector<i64> lens = {L};
    while (len > 1) {  // karatsubaReorder (Adhoc.hs:66-79)
      i64 l2 = (len + 1) / 2;
      std::vector<R> nx(3 * cnt * l2), ny(3 * cnt * l2);
      for (i64 r = 0; r < cnt; ++r)
        for (i64 j = 0; j < l2; ++j) {
          R xl = xs[r * len + j], yl = ys[r * len + j];
          R xr = (l2 + j < len) ? xs[r * len + l2 + j] : R(0);
          R yr = (l2 + j < len) ? ys[r * len + l2 + j] : R(0);
          nx[r * l2 + j] = xl; nx[(cnt + r) * l2 + j] = xl + xr; nx[(2 * cnt + r) * l2 + j] = xr;
          ny[r * l2 + j] = yl; ny[(cnt + r) * l2 + j] = yl + yr; ny[(2 * cnt + r) * l2 + j] = yr;
        }
      xs.swap(nx); ys.swap(ny);
      cnt *= 3; len = l2;
      lens.insert(lens.begin(), len);
    }
    std::vector<R> zz(cnt * len);
    for (i64 i = 0; i < cnt * len; ++i) zz[i] = xs[i] * ys[i];
    i64 zlen_cur = len;
    while (lens.size() > 1) {  // karatsubaGo (Adhoc.hs:81-98), indexPad (Convolution/Private.hs:21-26)
      i64 xlen = lens[0], zlen = 2 * lens[1] - 1;
      i64 n3 = cnt / 3;
      std::vector<R> nz(n3 * zlen, R(0));
      auto at = [&](i64 row, i64 k) -> R { return (k >= 0 && k < zlen_cur) ? zz[row * zlen_cur + k] : R(0); };
      for (i64 r = 0; r < n3; ++r)
        for (i64 k = 0; k < zlen; ++k) {
          R lv = at(r, k);
          i64 kc = k - xlen, kr = k - 2 * xlen;
          R cv = (kc >= 0 && kc < zlen_cur) ? at(n3 + r, kc) - (at(r, kc) + at(2 * n3 + r, kc)) : R(0);
          R rv = at(2 * n3 + r, kr);
          nz[r * zlen + k] = lv + cv + rv;
        }
      zz.swap(nz);
      cnt = n3; zlen_cur = zlen;
      lens.erase(lens.begin());
    }
    for (i64 k = 0; k < zl; ++k) z[b * zl + k] = (k < zlen_cur) ? zz[k] : R(0);
  }
}
extern "C" {
void or_karatsuba_loop_i64(i64 L, i64 batch, const i64* x, const i64* y, i64* z) {
  karatsuba_loop<i64>(L, batch, x, y, z);
}
void or_karatsuba_loop_f64(i64 L, i64 batch, const double* x, const double* y, double* z) {
  karatsuba_loop<double>(L, batch, x, y, z);
}
void or_karatsuba_loop_f32(i64 L, i64 batch, const float* x, const float* y, float* z) {
  karatsuba_loop<float>(L, batch, x, y, z);
}

// Convolution/Preprocessed.hs:29-56 karatsuba (recursive form), int64
static void kara_rec(i64 len, const i64* x, const i64* y, i64* z) {
  if (len <= 1) { if (len == 1) z[0] = x[0] * y[0]; return; }
  i64 l2 = (len + 1) / 2;
  std::vector<i64> xl(l2), yl(l2), xm(l2), ym(l2), xr(l2, 0), yr(l2, 0);
  for (i64 j = 0; j < l2; ++j) {
    xl[j] = x[j]; yl[j] = y[j];
    if (l2 + j < len) { xr[j] = x[l2 + j]; yr[j] = y[l2 + j]; }
    xm[j] = xl[j] + xr[j]; ym[j] = yl[j] + yr[j];
  }
  i64 sl = 2 * l2 - 1;
  std::vector<i64> zl(sl), zm(sl), zr(sl);
  kara_rec(l2, xl.data(), yl.data(), zl.data());
  kara_rec(l2, xm.data(), ym.data(), zm.data());
  kara_rec(l2, xr.data(), yr.data(), zr.data());
  for (i64 k = 0; k < 2 * len - 1; ++k) {
    i64 v = (k < sl) ? zl[k] : 0;
    i64 kc = k - l2, kr = k - 2 * l2;
    if (kc >= 0 && kc < sl) v += zm[kc] - (zl[kc] + zr[kc]);
    if (kr >= 0 && kr < sl) v += zr[kr];
    z[k] = v;
  }
}
void or_karatsuba_rec_i64(i64 L, i64 batch, const i64* x, const i64* y, i64* z) {
  i64 zl = L > 0 ? 2 * L - 1 : 0;
  for (i64 b = 0; b < batch; ++b) kara_rec(L, x + b * L, y + b * L, z + b * zl);
}

// Convolution/Adhoc.hs:104-111 cyclic: z[k] + z[k+L]
void or_cyclic_fold_i64(i64 L, i64 batch, const i64* z, i64* out) {
  i64 zl = L > 0 ? 2 * L - 1 : 0;
  for (i64 b = 0; b < batch; ++b)
    for (i64 k = 0; k < L; ++k) out[b * L + k] = z[b * zl + k] + ((k + L < zl) ? z[b * zl + k + L] : 0);
}

// Mixed-size batch (the CPU baseline for the batched workload): count
// transforms of lengths ns[i] stored back to back.  handles built once.
void* or_mixed_create(int mode, int sign, i64 count, const i64* ns) {
  std::vector<void*>* hs = new std::vector<void*>();
  std::map<i64, void*> byn;
  for (i64 i = 0; i < count; ++i) {
    auto it = byn.find(ns[i]);
    if (it == byn.end()) { void* h = or_handle_create(mode, sign, ns[i]); byn[ns[i]] = h; hs->push_back(h); }
    else hs->push_back(it->second);
  }
  // store unique set for destruction after the per-transform list
  std::vector<void*>* uniq = new std::vector<void*>();
  for (auto& kv : byn) uniq->push_back(kv.second);
  hs->push_back((void*)uniq);
  hs->push_back((void*)(intptr_t)count);
  return hs;
}
void or_mixed_destroy(void* hv) {
  auto* hs = (std::vector<void*>*)hv;
  auto* uniq = (std::vector<void*>*)(*hs)[hs->size() - 2];
  for (void* h : *uniq) or_handle_destroy(h);
  delete uniq;
  delete hs;
}
// Executes transforms [first, first+cnt) of the mixed list (f32), threads over transforms.
void or_mixed_exec_f32(void* hv, i64 first, i64 cnt, const i64* offsets, const float* in, float* out, int threads) {
  auto* hs = (std::vector<void*>*)hv;
  int nt = nthreads_of<float>(threads);
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
  for (i64 i = first; i < first + cnt; ++i) {
    Handle* h = (Handle*)(*hs)[i];
    exec(h->c32, (const cx<float>*)in + offsets[i], 1, (cx<float>*)out + offsets[i]);
  }
}
void or_mixed_exec_f64(void* hv, i64 first, i64 cnt, const i64* offsets, const double* in, double* out, int threads) {
  auto* hs = (std::vector<void*>*)hv;
  int nt = nthreads_of<double>(threads);
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
  for (i64 i = first; i < first + cnt; ++i) {
    Handle* h = (Handle*)(*hs)[i];
    exec(h->c64, (const cx<double>*)in + offsets[i], 1, (cx<double>*)out + offsets[i]);
  }
}

}  // extern "C"
