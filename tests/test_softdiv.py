"""Integer-pipe FP64 division (csrc/softdiv.cuh) against IEEE division.

The FP64 kernels divide on the integer units (Moller & Granlund's division
by a precomputed reciprocal) to relieve the FP64 pipe; every quotient must
equal the `/` operator's bit for bit.  The CPU test compiles the same
header with the host compiler (whose division is IEEE) and checks 60 M
quotients; the GPU test checks the device build against the device's own
division."""
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "hamstr_oop_gb300", "csrc")

PROGRAM = r"""
#include "softdiv.cuh"
#include <cstdio>
#include <random>
using namespace hamstr::sd;
int main() {
   std::mt19937_64 rng(1);
   long bad = 0, n = 0;
   for (long i = 0; i < 4000000; i++) {
      uint64_t d = rng() | 0x8000000000000000ull;
      if (i < 1000) d = 0x8000000000000000ull + i;
      if (i >= 1000 && i < 2000) d = 0xFFFFFFFFFFFFFFFFull - (i - 1000);
      unsigned __int128 q = (~(unsigned __int128)0) / d;
      if ((q >> 64) != 1 || (uint64_t)q != reciprocal_word(d)) bad++;
   }
   auto rnd = [&](int emin, int emax) {
      uint64_t m = rng() & 0xFFFFFFFFFFFFFull;
      int e = emin + (int)(rng() % (uint64_t)(emax - emin + 1));
      uint64_t s = rng() & 0x8000000000000000ull, k = rng() % 16;
      if (k == 0) m = 0;
      if (k == 1) m = 0xFFFFFFFFFFFFFull;
      if (k == 2) m = rng() & 0xFFull;
      if (k == 3) m = 0xFFFFFFFFFFFFFull - (rng() & 0xFF);
      return from_bits(s | ((uint64_t)e << 52) | m);
   };
   for (long i = 0; i < 20000000; i++) {
      double a, b;
      if (i % 3 == 0) { a = rnd(1000, 1046); b = rnd(1000, 1046); }
      else if (i % 3 == 1) { a = rnd(1, 2046); b = rnd(1, 2046); }
      else { a = rnd(1020, 1026); b = a * (1.0 + 1e-15 * (double)(int)(rng() % 2001 - 1000)); }
      if (i % 97 == 0) a = 0.0;
      if (i % 101 == 0) b = rnd(0, 0);
      double w = a / b, g = div(a, b);
      n++;
      if (bits(w) != bits(g) && !(w != w && g != g)) bad++;
   }
   printf("%ld %ld\n", bad, n);
   return bad != 0;
}
"""


def test_softdiv_matches_ieee_division_on_the_host(tmp_path):
    src = tmp_path / "t.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "t"
    subprocess.run(["g++", "-O2", "-ffp-contract=off", "-std=c++17", "-I", CSRC, str(src), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    bad, n = (int(x) for x in out.stdout.split())
    assert out.returncode == 0 and bad == 0 and n == 20000000


@pytest.mark.gpu
def test_softdiv_matches_the_device_division(native_lib):
    import ctypes
    import torch
    rng = np.random.default_rng(3)
    n = 4_000_000
    m = rng.integers(0, 1 << 52, n, dtype=np.uint64)
    e = rng.integers(1, 2047, n, dtype=np.uint64)
    s = rng.integers(0, 2, n, dtype=np.uint64) << np.uint64(63)
    a = (s | (e << np.uint64(52)) | m).view(np.float64)
    m2 = rng.integers(0, 1 << 52, n, dtype=np.uint64)
    e2 = rng.integers(960, 1090, n, dtype=np.uint64)
    b = ((e2 << np.uint64(52)) | m2).view(np.float64)
    a[::7] = b[::7] * (1.0 + 1e-16 * rng.integers(-50, 50, a[::7].shape))   # near-unit quotients
    a[::11] = 0.0
    A, B = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    soft, hard = torch.empty_like(A), torch.empty_like(A)
    fn = native_lib.hamstr_check_softdiv
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p] * 4 + [ctypes.c_int, ctypes.c_void_p]
    assert fn(A.data_ptr(), B.data_ptr(), soft.data_ptr(), hard.data_ptr(), n, None) == 0
    torch.cuda.synchronize()
    sb = soft.cpu().numpy().view(np.uint64)
    hb = hard.cpu().numpy().view(np.uint64)
    nan = np.isnan(hard.cpu().numpy()) & np.isnan(soft.cpu().numpy())
    assert np.sum((sb != hb) & ~nan) == 0
    # and the host's IEEE division agrees too
    assert np.array_equal(hb, (a / b).view(np.uint64)) or np.sum(hb != (a / b).view(np.uint64)) == 0


SCALE_PROGRAM = r"""
#include "softdiv.cuh"
#include <cstdio>
#include <random>
using namespace hamstr::sd;
template <int K> long check(double x, double s) {
   const double w = x * s, g = scale2<K>(x);
   return (bits(w) != bits(g) && !(w != w && g != g)) ? 1 : 0;
}
int main() {
   std::mt19937_64 rng(2);
   long bad = 0, n = 0;
   for (long i = 0; i < 4000000; i++) {
      uint64_t u = rng();
      const int mode = (int)(i % 8);
      if (mode == 0) u &= 0x800FFFFFFFFFFFFFull;                 // zeros and subnormals
      if (mode == 1) u = (u & 0x800FFFFFFFFFFFFFull) | (1ull << 52) * (1 + rng() % 3);   // near the bottom
      if (mode == 2) u = (u & 0x800FFFFFFFFFFFFFull) | (0x7FEull - rng() % 3) << 52;   // near the top
      if (mode == 3) u = (u & 0x800FFFFFFFFFFFFFull) | 0x7FF0000000000000ull;          // inf, NaN
      if (mode == 4) u &= 0x8000000000000000ull;                 // +-0
      const double x = from_bits(u);
      bad += check<1>(x, 2.0) + check<2>(x, 4.0) + check<-1>(x, 0.5) + check<-2>(x, 0.25);
      n += 4;
   }
   printf("%ld %ld\n", bad, n);
   return bad != 0;
}
"""


def test_scale2_matches_the_multiply_on_the_host(tmp_path):
    """x * 2^K on the integer pipes equals the FP64 multiply for every
    class of x (normal, near the exponent limits, subnormal, zero, inf, NaN)."""
    src = tmp_path / "s.cpp"
    src.write_text(SCALE_PROGRAM)
    exe = tmp_path / "s"
    subprocess.run(["g++", "-O2", "-ffp-contract=off", "-std=c++17", "-I", CSRC, str(src), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    bad, n = (int(x) for x in out.stdout.split())
    assert out.returncode == 0 and bad == 0 and n == 16000000


MUL_PROGRAM = r"""
#include "softdiv.cuh"
#include <cstdio>
#include <random>
using namespace hamstr::sd;
int main() {
   std::mt19937_64 rng(3);
   long bad = 0, n = 0;
   auto rnd = [&](int emin, int emax) {
      uint64_t m = rng() & 0xFFFFFFFFFFFFFull;
      const int e = emin + (int)(rng() % (uint64_t)(emax - emin + 1));
      const uint64_t s = rng() & 0x8000000000000000ull, k = rng() % 16;
      if (k == 0) m = 0;
      if (k == 1) m = 0xFFFFFFFFFFFFFull;
      if (k == 2) m = rng() & 0xFFull;
      if (k == 3) m = 0xFFFFFFFFFFFFFull - (rng() & 0xFF);
      if (k == 4) m = (rng() & 0xFFFFFFFull) << 24;
      return from_bits(s | ((uint64_t)e << 52) | m);
   };
   for (long i = 0; i < 30000000; i++) {
      double a, b;
      const int mode = (int)(i % 6);
      if (mode == 0) { a = rnd(1000, 1046); b = rnd(1000, 1046); }
      else if (mode == 1) { a = rnd(1, 2046); b = rnd(1, 2046); }
      else if (mode == 2) { a = rnd(1, 60); b = rnd(960, 1023); }              // products near the subnormal edge
      else if (mode == 3) { a = rnd(1500, 2046); b = rnd(1023, 1100); }        // near overflow
      else if (mode == 4) { a = rnd(0, 0); b = rnd(900, 1100); }              // zeros and subnormals
      else { a = rnd(1020, 1026); b = from_bits(bits(1.0) + (rng() & 0xFF)); }
      if (i % 89 == 0) a = (i % 2) ? 0.0 : -0.0;
      if (i % 97 == 0) b = from_bits(0x7FF0000000000000ull | (rng() & 1));   // inf or NaN
      const double w = a * b, g = mul(a, b);
      n++;
      if (bits(w) != bits(g) && !(w != w && g != g)) bad++;
   }
   printf("%ld %ld\n", bad, n);
   return bad != 0;
}
"""


def test_soft_multiply_matches_the_multiply_on_the_host(tmp_path):
    """The integer-pipe FP64 multiply equals IEEE multiplication (round to
    nearest even) for normal, boundary, zero, subnormal, infinite and NaN
    operands."""
    src = tmp_path / "m.cpp"
    src.write_text(MUL_PROGRAM)
    exe = tmp_path / "m"
    subprocess.run(["g++", "-O2", "-ffp-contract=off", "-std=c++17", "-I", CSRC, str(src), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    bad, n = (int(x) for x in out.stdout.split())
    assert out.returncode == 0 and bad == 0 and n == 30000000


ZERO_PLUS_PROGRAM = r"""
#include "softdiv.cuh"
#include <cstdio>
#include <random>
using namespace hamstr::sd;
int main() {
   std::mt19937_64 rng(5);
   long bad = 0, n = 0;
   const double special[] = {0.0, -0.0, 1.0, -1.0, 4.9e-324, -4.9e-324, 2.2250738585072014e-308, -2.2e-308,
                             1.7976931348623157e308, -1.7976931348623157e308, from_bits(0x7FF0000000000000ull),
                             from_bits(0xFFF0000000000000ull)};
   volatile double zero = 0.0;
   for (long i = 0; i < 20000000; i++) {
      const double v = (i < 24) ? special[i / 2] : from_bits(rng());
      if (v != v) continue;
      const bool sub = (i & 1) != 0;
      const double w = sub ? zero - v : zero + v;
      n++;
      if (bits(w) != bits(zero_plus(v, sub))) bad++;
   }
   printf("%ld %ld\n", bad, n);
   return bad != 0;
}
"""


def test_zero_plus_matches_the_add_on_the_host(tmp_path):
    """The ADI assembly's first term on the integer pipes (sd::zero_plus)
    equals 0.0 + v and 0.0 - v bit for bit: random doubles over all
    exponents, zeros of both signs, subnormals, the largest finite values
    and infinities (NaN has no defined sign and is left out)."""
    src = tmp_path / "z.cpp"
    src.write_text(ZERO_PLUS_PROGRAM)
    exe = tmp_path / "z"
    subprocess.run(["g++", "-O2", "-ffp-contract=off", "-std=c++17", "-I", CSRC, str(src), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    bad, n = (int(x) for x in out.stdout.split())
    assert out.returncode == 0 and bad == 0 and n > 19900000
