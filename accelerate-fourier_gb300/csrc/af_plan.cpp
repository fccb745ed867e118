// af_plan.cpp -- libaf's planner: the reference's number theory and plan
// selection (file:line relative to the accelerate-fourier project root).
#include "af_plan.h"

#include <algorithm>
#include <cmath>
#include <cstdio>

namespace af {

i64 gcd64(i64 a, i64 b) {
  a = a < 0 ? -a : a;
  b = b < 0 ? -b : b;
  while (b) { i64 t = a % b; a = b; b = t; }
  return a;
}

i64 mod_pow(i64 b, i64 e, i64 m) {
  i64 r = 1 % m;
  b %= m;
  while (e > 0) {
    if (e & 1) r = (i64)((__int128)r * b % m);
    b = (i64)((__int128)b * b % m);
    e >>= 1;
  }
  return r;
}

bool is_pow2(i64 n) { return n > 0 && (n & (n - 1)) == 0; }

static i64 strip(i64 n, i64 p) {
  while (n % p == 0) n /= p;
  return n;
}
bool is_5smooth(i64 n) { return n > 0 && strip(strip(strip(n, 2), 3), 5) == 1; }
bool is_13smooth(i64 n) {
  if (n <= 0) return false;
  for (i64 p : {2, 3, 5, 7, 11, 13}) n = strip(n, p);
  return n == 1;
}

// NumberTheory.hs:15-29 fermatFactors.  Pairs (b-a, b+a) with b^2 - a^2 = n in
// order of a ascending; for odd n these are the divisor pairs (d, n/d),
// d <= sqrt n, ordered by d descending.
std::vector<std::pair<i64, i64>> fermat_factors(i64 n) {
  std::vector<std::pair<i64, i64>> out;
  i64 r = (i64)std::sqrt((double)n);
  while (r > 0 && r * r > n) --r;
  while ((r + 1) * (r + 1) <= n) ++r;
  for (i64 d = r; d >= 1; --d)
    if (n % d == 0) out.emplace_back(d, n / d);
  return out;
}

// NumberTheory.hs:65-91 uniquePrimeFactors
static std::vector<i64> unique_prime_factors(i64 n) {
  std::vector<i64> f;
  if (n % 2 == 0) { f.push_back(2); while (n % 2 == 0) n /= 2; }
  for (i64 p = 3; n > 1; p += 2) {
    if (n % p == 0) { f.push_back(p); while (n % p == 0) n /= p; }
    else if (n / p < p) { f.push_back(n); break; }
  }
  return f;
}

// NumberTheory.hs:32-47 multiplicativeGenerator: the smallest primitive root
i64 multiplicative_generator(i64 p) {
  const i64 order = p - 1;
  std::vector<i64> great;
  for (i64 q : unique_prime_factors(order)) great.push_back(order / q);
  for (i64 c = 1; c < p; ++c) {
    if (gcd64(c, p) != 1 || mod_pow(c, order, p) != 1) continue;
    bool prim = true;
    for (i64 y : great) if (mod_pow(c, y, p) == 1) { prim = false; break; }
    if (prim) return c;
  }
  return 0;
}

// NumberTheory.hs:94-101 ceilingPowerOfTwo
i64 ceiling_power_of_two(i64 n) {
  if (n <= 1) return 1;
  i64 m = n - 1;
  for (int s = 1; s < 64; s <<= 1) m |= m >> s;
  return m + 1;
}

// NumberTheory.hs:118-124 ceilingSmooths a b n m
static std::vector<i64> ceiling_smooths(i64 a, i64 b, i64 n, i64 m) {
  std::vector<i64> out;
  for (;;) {
    out.push_back(m);
    if (m % a) break;
    i64 k = m * b;
    while (k % a == 0 && k / a >= n) k /= a;
    m = k;
  }
  return out;
}

// NumberTheory.hs:108-111 ceiling5Smooth
i64 ceiling_5smooth(i64 n) {
  i64 best = -1;
  for (i64 c : ceiling_smooths(2, 3, n, ceiling_power_of_two(n)))
    for (i64 v : ceiling_smooths(2, 5, n, c))
      if (best < 0 || v < best) best = v;
  return best;
}

static i64 ceil_log_base(i64 base, double x) {
  return (i64)std::ceil(std::log(x) / std::log((double)base));
}

// Adhoc.hs:229-248 ceiling5Smooth: argmin over the (e5, e3) grid in Double
i64 adhoc_ceiling_5smooth(i64 ni) {
  const double n = (double)ni;
  const i64 d3 = ceil_log_base(3, n), d5 = ceil_log_base(5, n);
  bool have = false;
  double best = 0;
  i64 b2 = 0, b3 = 0, b5 = 0;
  for (i64 e5 = 0; e5 < d5; ++e5)
    for (i64 e3 = 0; e3 < d3; ++e3) {
      const double p53 = std::pow(5.0, (double)e5) * std::pow(3.0, (double)e3);
      const i64 e2 = std::max<i64>(0, ceil_log_base(2, n / p53));
      const double v = p53 * std::pow(2.0, (double)e2);
      if (!have || v < best) { have = true; best = v; b2 = e2; b3 = e3; b5 = e5; }
    }
  if (!have) return -1;
  i64 r = 1;
  while (b2--) r *= 2;
  while (b3--) r *= 3;
  while (b5--) r *= 5;
  return r;
}

// Adhoc.hs:342-350: 2 ^ ceilingLogBase 2 (2n-1) in Double
i64 adhoc_pow2_pad(i64 n) { return (i64)1 << ceil_log_base(2, (double)(2 * n - 1)); }

// ----------------------------------------------------------------- planner
Planner::Planner() {
  // Planned.hs:241-250 smallPlanMap: 0,1 identity; 2..5 small kernels
  memo_[0] = mk(0, N_ID, nullptr, nullptr);
  memo_[1] = mk(1, N_ID, nullptr, nullptr);
  for (i64 s = 2; s <= 5; ++s) memo_[s] = mk(s, N_SMALL, nullptr, nullptr);
}

const Node* Planner::mk(i64 n, NodeKind k, const Node* a, const Node* b) {
  arena_.emplace_back(new Node{n, k, a, b});
  return arena_.back().get();
}

const Node* Planner::decompose(i64 n) {
  auto it = memo_.find(n);
  if (it != memo_.end()) return it->second;
  const Node* p = decompose_new(n);
  memo_[n] = p;
  return p;
}

const Node* Planner::decompose_new(i64 n) {
  if (n % 2 == 0) return mk(n, N_SR, decompose(n / 2), nullptr);  // Planned.hs:258-263
  const auto facs = fermat_factors(n);
  for (const auto& q : facs)  // unitary divisors first (Planned.hs:266-268)
    if (q.first > 1 && gcd64(q.first, q.second) == 1) {
      const Node* a = decompose(q.first);
      const Node* b = decompose(q.second);
      return mk(n, N_COPRIME, a, b);
    }
  const auto q = facs.front();
  if (q.first == 1) return mk(n, N_PRIME, decompose(n - 1), nullptr);  // Rader (270-276)
  const Node* a = decompose(q.first);
  const Node* b = decompose(q.second);
  return mk(n, N_COMPOSITE, a, b);  // Cooley-Tukey (277)
}

int Planner::count_primes(const Node* p) {
  switch (p->kind) {
    case N_ID: case N_SMALL: return 0;
    case N_SR: case N_CHIRP: return count_primes(p->a);
    case N_PRIME: return 1 + count_primes(p->a);
    default: return std::max(count_primes(p->a), count_primes(p->b));
  }
}

const Node* Planner::automatic(i64 n) {
  const Node* p = decompose(n);
  if (count_primes(p) < 3) return p;
  return chirp(n, ceiling_5smooth(2 * n - 1));
}

const Node* Planner::chirp(i64 n, i64 pad) {
  if (n < 2) return mk(n, N_ID, nullptr, nullptr);
  return mk(n, N_CHIRP, decompose(pad), nullptr);
}

std::string Planner::describe(const Node* p) {
  char buf[48];
  const char* tag = "";
  switch (p->kind) {
    case N_ID: snprintf(buf, sizeof buf, "I%lld", p->n); return buf;
    case N_SMALL: snprintf(buf, sizeof buf, "S%lld", p->n); return buf;
    case N_SR: tag = "SR"; break;
    case N_PRIME: tag = "P"; break;
    case N_COPRIME: tag = "GT"; break;
    case N_COMPOSITE: tag = "CT"; break;
    case N_CHIRP: tag = "BL"; break;
  }
  snprintf(buf, sizeof buf, "%s%lld(", tag, p->n);
  std::string s = buf + describe(p->a);
  if (p->b) s += "," + describe(p->b);
  return s + ")";
}

}  // namespace af
