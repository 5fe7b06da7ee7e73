"""The FP64 helpers of ds_bits.cuh (integer-pipe replacements for FP64
instructions on the FP32 path) give the IEEE results, checked on the host
against the compiler's own conversion and comparisons (no GPU needed)."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "dustyshock3d_gb300", "csrc")

PROGRAM = r"""
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include "ds_bits.cuh"

static uint32_t fbits(float f) { uint32_t b; memcpy(&b, &f, 4); return b; }
static double dof(uint64_t b) { double d; memcpy(&d, &b, 8); return d; }

static long bad = 0, checked = 0;
static void check_d2f(double v) {
  const float a = ds_d2f(v), b = (float)v;
  checked++;
  if (std::isnan(b) ? !std::isnan(a) : fbits(a) != fbits(b)) {
    if (bad++ < 5) printf("d2f %.17g: %08x vs %08x\n", v, fbits(a), fbits(b));
  }
}

int main() {
  std::mt19937_64 rng(20261203);
  // every bit pattern class: uniform bits (NaNs, infinities, subnormals, huge)
  for (int i = 0; i < 4000000; i++) check_d2f(dof(rng()));
  // the FP32 range and its edges, with exact ties of both mantissa parities
  for (int e = -160; e <= 130; e++)
    for (int i = 0; i < 20000; i++) {
      uint64_t m = rng() & 0xfffffffffffffull;
      if (i % 4 == 0) m = (m & ~0x1fffffffull) | 0x10000000ull;  // a tie
      if (i % 4 == 1) m = (m & ~0x1fffffffull);                  // exact
      if (i % 8 == 2) m |= 0xfffffe0000000ull | 0x10000000ull;   // ties next to a binade carry
      const uint64_t sign = (rng() & 1) ? 0x8000000000000000ull : 0;
      check_d2f(dof(sign | ((uint64_t)(e + 1023) << 52) | m));
    }
  const double special[] = {0.0, -0.0, 1.0, -1.0, 3.4028234663852886e38, 3.4028235677973366e38, 1e39, -1e39,
                            1.1754943508222875e-38, 1.1754942106924411e-38, 1.401298464324817e-45,
                            7.006492321624085e-46, 7.0064923216240862e-46, 1e-46, 5e-324, INFINITY, -INFINITY, NAN};
  for (double v : special) check_d2f(v);
  // order keys: a < b exactly when key(a) < key(b); -0.0 == +0.0
  long badk = 0;
  for (int i = 0; i < 4000000; i++) {
    double a = dof(rng()), b = (i & 1) ? dof(rng()) : -a;
    if (i % 16 == 3) b = a;
    if (std::isnan(a) || std::isnan(b)) continue;
    if ((a < b) != (ds_order_key(a) < ds_order_key(b)) || (a == b) != (ds_order_key(a) == ds_order_key(b)))
      if (badk++ < 5) printf("key %.17g %.17g\n", a, b);
  }
  if (ds_order_key(-0.0) != ds_order_key(0.0)) badk++;
  printf("checked %ld bad %ld badkey %ld\n", checked, bad, badk);
  return (bad || badk) ? 1 : 0;
}
"""


def test_d2f_and_order_key_match_ieee(tmp_path):
    src = tmp_path / "bits.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "bits"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", CSRC, str(src), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "bad 0 badkey 0" in out.stdout
