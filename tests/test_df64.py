"""Double-float arithmetic of the split-precision block kernel
(pyscaledvecchia_gb300/csrc/sv_df64.cuh), compiled as host C++ and checked
against long double: the error-free transformations are exact, every
operation stays within a few 2^-46 of its operands' scale, and results are
normalised.  The device uses the same source with round-to-nearest
intrinsics, so these bounds carry over; the GPU tests check the kernel's
outputs against the float64 form."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "pyscaledvecchia_gb300", "csrc", "sv_df64.cuh")

DRIVER = r"""
#include "HEADER"
#include <cstdio>
#include <cstdint>
#include <cmath>
using namespace sv;
typedef long double LD;
static LD val(dfv v) { return (LD)v.hi + (LD)v.lo; }
static uint64_t st = 88172645463325252ULL;
static double uni() {  // xorshift64, uniform in [-1, 1)
  st ^= st << 13; st ^= st >> 7; st ^= st << 17;
  return (double)(st >> 11) * (2.0 / 9007199254740992.0) - 1.0;
}
static bool normalised(dfv v) { return v.hi == (float)((double)v.hi + (double)v.lo); }
int main() {
  double e_fms = 0, e_mul = 0, e_add = 0, e_rcp = 0, e_sqrt = 0, e_sd = 0, e_acc = 0;
  long bad_exact = 0, bad_norm = 0;
  for (int it = 0; it < 200000; ++it) {
    const double x = uni() * std::exp(3 * uni()), y = uni() * std::exp(3 * uni()),
                 z = uni() * std::exp(3 * uni());
    // error-free transformations
    {
      const float a = (float)x, b = (float)y;
      float s, e;
      two_sum(a, b, s, e);
      if ((LD)s + (LD)e != (LD)a + (LD)b) ++bad_exact;
      const float big = std::fabs(a) >= std::fabs(b) ? a : b, sm = std::fabs(a) >= std::fabs(b) ? b : a;
      fast_two_sum(big, sm, s, e);
      if ((LD)s + (LD)e != (LD)a + (LD)b) ++bad_exact;
      const float p = df_mulf(a, b), q = df_fmaf(a, b, -p);
      if ((LD)p + (LD)q != (LD)a * (LD)b) ++bad_exact;
    }
    const dfv a = df_from_double(x), b = df_from_double(y), c = df_from_double(z);
    const LD A = val(a), B = val(b), C = val(c);
    dfv o = df_fms(c, a, b);
    e_fms = std::fmax(e_fms, (double)(fabsl(val(o) - (C - A * B)) / (fabsl(C) + fabsl(A * B))));
    bad_norm += !normalised(o);
    o = df_mul(a, b);
    e_mul = std::fmax(e_mul, (double)(fabsl(val(o) - A * B) / fabsl(A * B)));
    bad_norm += !normalised(o);
    o = df_add(a, b);
    e_add = std::fmax(e_add, (double)(fabsl(val(o) - (A + B)) / (fabsl(A) + fabsl(B))));
    bad_norm += !normalised(o);
    o = df_rcp(a);
    e_rcp = std::fmax(e_rcp, (double)(fabsl(val(o) - 1 / A) * fabsl(A)));
    const dfv pa = df_from_double(std::fabs(x));
    o = df_sqrt(pa);
    e_sqrt = std::fmax(e_sqrt, (double)(fabsl(val(o) - sqrtl(val(pa))) / sqrtl(val(pa))));
    float D = (float)std::fabs(uni());
    if (it % 3 == 0) D = (float)(std::fabs(uni()) * 1e-6);
    o = df_scaled_deficit(pa, D);
    e_sd = std::fmax(e_sd, (double)(fabsl(val(o) - val(pa) * (1 - (LD)D)) / val(pa)));
    bad_norm += !normalised(o);
    // a 32-step unnormalised accumulation (one column of a forward solve)
    if (it % 100 == 0) {
      float s = (float)z, t = 0.0f;
      LD ref = (LD)s, scale = fabsl(ref);
      for (int k = 0; k < 32; ++k) {
        const dfv l = df_from_double(uni()), m = df_from_double(uni() * 4.0);
        df_fms_acc(s, t, l, m);
        ref -= val(l) * val(m);
        scale += fabsl(val(l) * val(m));
      }
      e_acc = std::fmax(e_acc, (double)(fabsl((LD)s + (LD)t - ref) / scale));
    }
  }
  std::printf("%ld %ld %.6g %.6g %.6g %.6g %.6g %.6g %.6g\n", bad_exact, bad_norm, e_fms, e_mul,
              e_add, e_rcp, e_sqrt, e_sd, e_acc);
  return 0;
}
"""


def test_df64_operations_on_host(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not available")
    src = tmp_path / "df64_check.cpp"
    src.write_text(DRIVER.replace("HEADER", HEADER))
    exe = tmp_path / "df64_check"
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", str(src), "-o", str(exe)],
                   check=True, capture_output=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    bad_exact, bad_norm = int(out[0]), int(out[1])
    e_fms, e_mul, e_add, e_rcp, e_sqrt, e_sd, e_acc = map(float, out[2:])
    u46 = 2.0 ** -46
    assert bad_exact == 0          # TwoSum, Fast2Sum and the FMA residual are exact
    assert bad_norm == 0           # results are normalised pairs
    assert e_fms < 4 * u46         # relative to |c| + |a b|
    assert e_mul < 2 * u46
    assert e_add < 2 * u46
    assert e_rcp < 2 * u46
    assert e_sqrt < 2 * u46
    assert e_sd < 2 * u46
    assert e_acc < 16 * u46        # 32 steps, relative to the sum of magnitudes
