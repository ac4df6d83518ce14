// Exercises the C++ facade (include/fideslib_gb300.hpp) the way a reference-side caller would: context from
// generated primes, keys and a ciphertext from raw residues, then identities that must hold residue-for-residue:
// hoisted == individual rotations, Mult commutes, (a + b) - b == a, Rescale drops one tower, and a missing key
// is reported by an exception carrying FIDES_ENOKEY.  Prints "facade ok" and exits 0 on success.
#include <cstdio>
#include <random>

#include "fideslib_gb300.hpp"

using namespace fideslib_gb300;

int main() {
  const uint32_t log_n = 13, N = 1u << log_n;
  Params prm;
  prm.log_n = log_n;
  prm.q = FindPrimes(60, 1, log_n);
  auto q40 = FindPrimes(40, 5, log_n);
  prm.q.insert(prm.q.end(), q40.begin(), q40.end());
  prm.p = FindPrimes(60, 3, log_n, prm.q);
  prm.dnum = 2;
  CryptoContext cc(prm);
  const uint32_t nq = (uint32_t)prm.q.size(), np = (uint32_t)prm.p.size();
  std::vector<uint64_t> mods(prm.q);
  mods.insert(mods.end(), prm.p.begin(), prm.p.end());
  std::mt19937_64 rng(42);
  auto key = [&]() {
    std::vector<uint64_t> k((size_t)2 * prm.dnum * (nq + np) * N);
    for (uint32_t ab = 0; ab < 2; ab++)
      for (uint32_t d = 0; d < prm.dnum; d++)
        for (uint32_t t = 0; t < nq + np; t++)
          for (uint32_t i = 0; i < N; i++) k[(((size_t)ab * prm.dnum + d) * (nq + np) + t) * N + i] = rng() % mods[t];
    return k;
  };
  auto relin = key(), r1 = key(), r2 = key();
  cc.LoadEvalMultKey(relin.data());
  cc.LoadRotationKey(1, r1.data());
  cc.LoadRotationKey(2, r2.data());
  auto ct = [&](uint32_t t) {
    std::vector<uint64_t> c((size_t)2 * t * N);
    for (uint32_t p = 0; p < 2; p++)
      for (uint32_t j = 0; j < t; j++)
        for (uint32_t i = 0; i < N; i++) c[((size_t)p * t + j) * N + i] = rng() % mods[j];
    return c;
  };
  auto ha = ct(nq), hb = ct(nq);
  Ciphertext a = cc.LoadCiphertext(ha.data(), nq, 1099511627776.0), b = cc.LoadCiphertext(hb.data(), nq, 1099511627776.0);
  int fails = 0;
  auto same = [&](const Ciphertext& x, const Ciphertext& y, const char* what) {
    if (cc.StoreCiphertext(x) != cc.StoreCiphertext(y)) {
      std::printf("mismatch: %s\n", what);
      fails++;
    }
  };
  auto hoisted = cc.EvalFastRotation(a, {1, 2});
  same(hoisted[0], cc.EvalRotate(a, 1), "hoisted rotation by 1");
  same(hoisted[1], cc.EvalRotate(a, 2), "hoisted rotation by 2");
  same(cc.EvalMult(a, b), cc.EvalMult(b, a), "mult commutes");
  {  // EvalFastRotationPrecompute + EvalFastRotation(ct, index, m, precomp) == EvalRotate
    auto pre = cc.EvalFastRotationPrecompute(a);
    same(cc.EvalFastRotation(a, 2, cc.GetCyclotomicOrder(), pre), cc.EvalRotate(a, 2), "precomputed rotation");
    Ciphertext c = a;
    cc.EvalRotateInPlace(c, 1);
    same(c, hoisted[0], "in-place rotation");
    // index 0 of EvalFastRotationExt is (P c0, P c1); KeySwitchDown divides P out exactly
    auto ext = cc.EvalFastRotationExt(a, {0, 1}, pre, true);
    same(cc.KeySwitchDown(ext[0]), a, "KeySwitchDown(EvalFastRotationExt(a, 0))");
    same(cc.KeySwitchDown(cc.EvalAdd(ext[0], ext[0])), cc.EvalAdd(a, a), "KeySwitchDown of a sum");
  }
  if (cc.StoreCiphertext(cc.EvalSub(cc.EvalAdd(a, b), b)) != ha) {
    std::printf("mismatch: (a + b) - b\n");
    fails++;
  }
  if (cc.Rescale(cc.EvalMult(a, b)).GetTowers() != nq - 1) {
    std::printf("rescale did not drop a tower\n");
    fails++;
  }
  try {
    cc.EvalRotate(a, 3);
    std::printf("missing key not reported\n");
    fails++;
  } catch (const Error& e) {
    if (e.code() != FIDES_ENOKEY) {
      std::printf("wrong error code %d\n", e.code());
      fails++;
    }
  }
  cc.Synchronize();
  if (fails) return 1;
  std::printf("facade ok\n");
  return 0;
}
