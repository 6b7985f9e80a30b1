// Host check of the x passes' exchange maps (xpass_warp.cuh): for every x plan
// size, each stage boundary's map must send the N points of a line to N
// distinct words below the group pitch, and its bank cost (XPad::cost) must
// equal the conflict-free cost of that boundary.  Prints one line per boundary
// and exits 1 if any check fails.  Built and run by tests/test_exchange_maps.py.
#include <cstdio>

#include "xpass_staged.cuh"

using namespace wdm;

static int failures = 0;

template <int N, int T, int NP, int NS, int R, int... Rest>
void walk() {
  if constexpr (sizeof...(Rest) > 0) {
    constexpr int RN = First<Rest...>::value;
    constexpr int code = XMap<N, T, NP, R, NS, RN>::code;
    const int cost = XPad<N, T, NP>::cost(R, NS, RN, code);
    const int ideal = 2 * (N / (R * T)) * R + 2 * (N / (RN * T)) * RN;
    static bool seen[1 << 12];
    for (int w = 0; w < NP; ++w) seen[w] = false;
    bool bijective = true;
    for (int p = 0; p < N; ++p) {
      const int w = xaddr(p, code);
      if (w < 0 || w >= NP || seen[w]) bijective = false;
      else seen[w] = true;
    }
    const bool ok = bijective && cost == ideal;
    if (!ok) ++failures;
    std::printf("N=%d T=%d NP=%d R=%d NS=%d RN=%d code=%d cost=%d ideal=%d %s\n", N, T, NP, R, NS, RN, code, cost,
                ideal, ok ? "ok" : "FAIL");
    walk<N, T, NP, NS * R, Rest...>();
  }
}

template <int N, int T, int NP, int... Rs>
void plan(Radices<Rs...>) {
  walk<N, T, NP, 1, Rs...>();
}

template <int N>
void check() {
  using C = XCfg<N>;
  plan<N, C::T, C::NP>(typename XPlan<N>::Fwd{});
}

int main() {
  check<12>();
  check<16>();
  check<24>();
  check<32>();
  check<48>();
  check<64>();
  check<96>();
  check<128>();
  check<192>();
  check<256>();
  check<384>();
  check<512>();
  std::printf("%s\n", failures ? "FAILED" : "ALL OK");
  return failures ? 1 : 0;
}
