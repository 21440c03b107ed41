"""The library's binary64 -> binary32 round-to-nearest-even conversion on bit
patterns (lapack_gb300/csrc/fp_convert.h, used by the fused DLANGE + DLAG2S
pass in place of the FP64-unit conversion; SRC/dlag2s.f:143 converts with
REAL()) checked bit for bit against the host's IEEE conversion: random bit
patterns, exact ties at every exponent around the binary32 range, subnormal
results at every shift, the overflow boundary and special values.  Compiled
with g++ from the same header the CUDA code includes."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
HDR = os.path.join(HERE, "..", "lapack_gb300", "csrc", "fp_convert.h")

HARNESS = r"""
#include <cstdio>
#include <cstring>
#include <cstdint>
#include <random>
#include <cmath>
#include <cfloat>
#include "fp_convert.h"
static unsigned ref(double x) { float f = (float)x; unsigned u; std::memcpy(&u, &f, 4); return u; }
int main() {
  std::mt19937_64 g(7);
  long bad = 0, n = 0;
  auto check = [&](uint64_t b) {
    double x; std::memcpy(&x, &b, 8);
    unsigned a = gb::f64_bits_to_f32_bits_rn(b);
    ++n;
    if (std::isnan(x)) { if ((a & 0x7F800000u) != 0x7F800000u || !(a & 0x7FFFFFu)) ++bad; return; }
    if (a != ref(x)) ++bad;
  };
  for (long i = 0; i < 2000000; ++i) check(g());
  for (int be = 1023 - 160; be <= 1023 + 130; ++be)
    for (int i = 0; i < 4000; ++i) {
      uint64_t m = g() & 0x000FFFFFFFFFFFFFull;
      if (i % 4 == 1) m = (m & ~0x1FFFFFFFull) | 0x10000000ull;
      if (i % 4 == 2) m &= ~((1ull << 40) - 1);
      check(((uint64_t)be << 52) | m);
      check((1ull << 63) | ((uint64_t)be << 52) | m);
    }
  for (int be = 1023 - 150; be <= 1023 - 126; ++be)
    for (int sh = 0; sh < 52; ++sh) check(((uint64_t)be << 52) | (1ull << sh));
  double sp[] = {0.0, -0.0, FLT_MAX, -FLT_MAX, 3.4028235677973366e38, 3.4028235677973362e38, 1e39, FLT_MIN,
                 FLT_MIN / 2, 1.401298464324817e-45, 7.006492321624085e-46, 7.0064923216240862e-46, 1e-46,
                 INFINITY, -INFINITY, NAN, 1.0, 0.1};
  for (double x : sp) { uint64_t b; std::memcpy(&b, &x, 8); check(b); }
  std::printf("%ld %ld\n", n, bad);
  return bad != 0;
}
"""


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_f64_to_f32_rn_matches_host_conversion(tmp_path):
    src = tmp_path / "cvt.cpp"
    src.write_text(HARNESS)
    exe = tmp_path / "cvt"
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.dirname(HDR), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    n, bad = (int(v) for v in out.stdout.split())
    assert out.returncode == 0 and bad == 0 and n > 2000000, out.stdout
