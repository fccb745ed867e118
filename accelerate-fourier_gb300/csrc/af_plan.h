// af_plan.h -- host planner of libaf: a restatement of accelerate-fourier's
// planner (src/Data/Array/Accelerate/Fourier/Planned.hs:183-293,731-737 and
// src/Data/Array/Accelerate/NumberTheory.hs), producing the same plan tree
// as the reference for every size, plus the pad rules of the Adhoc module.
#pragma once
#include <map>
#include <memory>
#include <string>
#include <vector>
#include <stdint.h>

namespace af {
typedef long long i64;

enum NodeKind { N_ID = 0, N_SMALL, N_SR, N_PRIME, N_COPRIME, N_COMPOSITE, N_CHIRP };

// Plan / PlanStructure (Planned.hs:183-195)
struct Node {
  i64 n;
  NodeKind kind;
  const Node* a;  // SplitRadix sub, Prime sub, Chirp sub, or first of a pair
  const Node* b;  // second of a pair (Coprime, Composite)
};

class Planner {
 public:
  Planner();
  const Node* decompose(i64 n);          // planDecomposeWithMapUpdate (Planned.hs:279-287)
  const Node* automatic(i64 n);          // planWithMapUpdate (Planned.hs:215-220)
  const Node* chirp(i64 n, i64 pad);     // planChirpWithMapUpdate (Planned.hs:731-737)
  static int count_primes(const Node* p);  // planCountPrimes (Planned.hs:222-232)
  static std::string describe(const Node* p);

 private:
  const Node* mk(i64 n, NodeKind k, const Node* a, const Node* b);
  const Node* decompose_new(i64 n);      // planDecomposeWithMap (Planned.hs:255-277)
  std::vector<std::unique_ptr<Node>> arena_;
  std::map<i64, const Node*> memo_;      // PlanMap (Planned.hs:234)
};

// NumberTheory.hs
std::vector<std::pair<i64, i64>> fermat_factors(i64 n);
i64 multiplicative_generator(i64 p);
i64 ceiling_power_of_two(i64 n);
i64 ceiling_5smooth(i64 n);
i64 adhoc_ceiling_5smooth(i64 n);      // Adhoc.hs:229-248 (Double argmin)
i64 adhoc_pow2_pad(i64 n);             // Adhoc.hs:342-350
i64 gcd64(i64 a, i64 b);
i64 mod_pow(i64 b, i64 e, i64 m);
bool is_pow2(i64 n);
bool is_5smooth(i64 n);
bool is_13smooth(i64 n);

}  // namespace af
