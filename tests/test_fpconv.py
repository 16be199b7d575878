"""The integer double -> float rounding of emdee_gb300/csrc/fpconv.h (used by the
position packing kernels) against the C conversion (IEEE round to nearest even)
on the host: random doubles over many binades, exact ties, values next to ties,
carries into the exponent and both signs."""
import os
import subprocess
import tempfile

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SRC = r'''
#include <cstdio>
#include <cstring>
#include <cmath>
#include <random>
#include "fpconv.h"
static unsigned long long bits(double x) { unsigned long long b; std::memcpy(&b, &x, 8); return b; }
static unsigned int fbits(float x) { unsigned int b; std::memcpy(&b, &x, 4); return b; }
int main() {
  std::mt19937_64 rng(12345);
  long checked = 0, bad = 0;
  auto check = [&](double x) {
    unsigned long long b = bits(x);
    if (!emdee::d2f_normal(b)) return;
    checked++;
    if (emdee::d2f_bits(b) != fbits((float)x)) {
      if (bad < 5) std::printf("mismatch %.17g\n", x);
      bad++;
    }
  };
  std::uniform_real_distribution<double> u(-1.0, 1.0);
  std::uniform_int_distribution<int> ex(-140, 140);
  for (int k = 0; k < 4000000; k++) check(std::ldexp(u(rng), ex(rng)));
  for (int k = 0; k < 1000000; k++) {   // exact ties and their neighbours
    float f = (float)std::ldexp(u(rng), ex(rng));
    double a = f, n = std::nextafter(f, 2.0f * f + 1.0f), t = 0.5 * (a + (double)n);
    check(t); check(std::nextafter(t, 0.0)); check(std::nextafter(t, 1e300)); check(-t);
  }
  for (double x : {1.0, 0.9999999999999999, 1.9999999999999998, 3.4028234663852886e38, 1.1754943508222875e-38})
    check(x);
  std::printf("%ld %ld\n", checked, bad);
  return bad != 0;
}
'''


def test_integer_rounding_matches_ieee():
    with tempfile.TemporaryDirectory() as d:
        src, exe = os.path.join(d, "t.cpp"), os.path.join(d, "t")
        open(src, "w").write(SRC)
        subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", os.path.join(ROOT, "emdee_gb300", "csrc"),
                        src, "-o", exe], check=True)
        r = subprocess.run([exe], capture_output=True, text=True)
        checked, bad = map(int, r.stdout.split()[-2:])
        assert r.returncode == 0 and bad == 0 and checked > 4_000_000, r.stdout
