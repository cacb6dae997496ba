"""Host checks of the numerical facts the GPU kernels' FP64 shortcuts rest
on (the kernels themselves are checked bit for bit on the GPU in
test_gpu_ns.py and test_gpu_poisson.py):

* Markstein's correction with the correctly rounded reciprocal of a fixed
  divisor, q = RN(x y), r = fma(-d, q, x), RN(q + r y), equals RN(x / d)
  (the predictor's division by rho), over random and near-midpoint
  quotients, by a small C program (gcc, fma from libm);
* the orientation of a face from the sign of uf[a] + uf[a - 1] (the
  halving by 0.5 changes the sign test only through -2^-1074 -> -0);
* van Leer's r + |r| as +0 or an exponent increment;
* the double-float split of a double (hi: the leading 24 bits truncated,
  lo: the next 29 bits rounded) within 2^-48 relative.
"""
import os
import shutil
import struct
import subprocess
import tempfile

import numpy as np
import pytest

MARKSTEIN_C = r"""
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>
static uint64_t s = 88172645463325252ull;
static uint64_t rnd(void) { s ^= s << 13; s ^= s >> 7; s ^= s << 17; return s; }
static double bits(uint64_t b) { double d; memcpy(&d, &b, 8); return d; }
static uint64_t ubits(double d) { uint64_t b; memcpy(&b, &d, 8); return b; }
int main(void) {
	const double ds[] = {1000.0, 3.0, 7.0, 0.7, 1e-3, 1.0 / 3.0, 997.0, 1234.5678, 6.02e23};
	long bad = 0, n = 0;
	for (int di = 0; di < (int)(sizeof ds / sizeof ds[0]); ++di) {
		const double d = ds[di], y = 1.0 / d;
		for (long k = 0; k < 400000; ++k) {
			double x;
			if (k & 1) {
				/* near a midpoint of two neighbouring quotients */
				const double q = bits((rnd() & 0x000fffffffffffffull)
						| ((uint64_t)(1023 + (int)(rnd() % 200) - 100) << 52));
				const long double mid = ((long double)q + (long double)nextafter(q, INFINITY)) / 2;
				x = bits(ubits((double)(mid * (long double)d)) + (int)(rnd() % 5) - 2);
			} else {
				x = bits((rnd() & 0x000fffffffffffffull)
						| ((uint64_t)(1023 + (int)(rnd() % 400) - 200) << 52));
			}
			if (rnd() & 1) x = -x;
			const double q = x * y, r = fma(-d, q, x), f = fma(r, y, q);
			++n;
			if (ubits(f) != ubits(x / d)) ++bad;
		}
	}
	printf("%ld %ld\n", n, bad);
	return 0;
}
"""


def test_markstein_fixed_divisor_is_correctly_rounded():
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    with tempfile.TemporaryDirectory() as d:
        src, exe = os.path.join(d, "m.c"), os.path.join(d, "m")
        open(src, "w").write(MARKSTEIN_C)
        subprocess.run([cc, "-O2", "-ffp-contract=off", "-o", exe, src, "-lm"], check=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split()
    n, bad = int(out[0]), int(out[1])
    assert n == 9 * 400000 and bad == 0, out


def orient(veo):
    return 1 if veo >= 0.0 else (-1 if veo < 0.0 else 0)


def orient_sum(s):
    """the kernels' integer form (bits.cuh split halves) of orient((x + y) * 0.5)"""
    b = struct.unpack("<Q", struct.pack("<d", s))[0]
    hi, lo = b >> 32, b & 0xFFFFFFFF
    mag = hi & 0x7FFFFFFF
    if mag > 0x7FF00000 or (mag == 0x7FF00000 and lo != 0):
        return 0
    if hi >> 31 == 0:
        return 1
    return 1 if (mag == 0 and lo <= 1) else -1


def test_orientation_from_the_sum():
    rng = np.random.default_rng(3)
    tiny = 5e-324
    vals = [0.0, -0.0, tiny, -tiny, 2 * tiny, -2 * tiny, -3 * tiny, 1.0, -1.0,
            float("inf"), float("-inf"), float("nan")]
    vals += list(rng.standard_normal(2000) * 10.0 ** rng.integers(-310, 300, 2000))
    for x in vals:
        for y in (0.0, -0.0, tiny, -tiny, -x, 1e-300, -1e-300):
            s = x + y
            assert orient_sum(s) == orient(s * 0.5), (x, y)


def r_plus_abs(r):
    """van Leer's r + |r| by the bits (the kernels' r_plus_abs)"""
    b = struct.unpack("<Q", struct.pack("<d", r))[0]
    hi, lo = b >> 32, b & 0xFFFFFFFF
    e = (hi >> 20) & 0x7FF
    if e < 2047 and (hi >> 31 != 0 or (hi | lo) == 0):
        return 0.0
    if hi >> 31 == 0 and 1 <= e <= 2045:
        return struct.unpack("<d", struct.pack("<Q", b + (1 << 52)))[0]
    return r + abs(r)


def test_r_plus_abs_bits():
    rng = np.random.default_rng(4)
    vals = [0.0, -0.0, 5e-324, -5e-324, 1e308, -1e308, 1.7e308, float("inf"),
            float("-inf")]
    vals += list(rng.standard_normal(5000) * 10.0 ** rng.integers(-320, 308, 5000))
    for r in vals:
        a, b = r_plus_abs(r), r + abs(r)
        assert struct.pack("<d", a) == struct.pack("<d", b), r
    assert np.isnan(r_plus_abs(float("nan")))


def df_split(d):
    """the kernels' df_from_double (dfloat.cuh) on the host"""
    b = struct.unpack("<Q", struct.pack("<d", d))[0]
    hi, lo = b >> 32, b & 0xFFFFFFFF
    e = ((hi >> 20) & 0x7FF) - 1023
    if e < -70 or e > 90:
        h = np.float32(d)
        return h, np.float32(d - float(h))
    sign = hi & 0x80000000
    m23 = ((hi & 0xFFFFF) << 3) | (lo >> 29)
    fh = np.frombuffer(struct.pack("<I", sign | ((e + 127) << 23) | m23), np.float32)[0]
    m29 = lo & 0x1FFFFFFF
    fl = np.float32(m29)
    if m29:
        fb = struct.unpack("<I", struct.pack("<f", fl))[0]
        nb = (sign | (fb + (((e - 52) & 0xFFFFFFFF) << 23))) & 0xFFFFFFFF
        assert 1 <= (nb >> 23) & 0xFF <= 254   # stays a normal float
        fl = np.frombuffer(struct.pack("<I", nb), np.float32)[0]
    return fh, fl


def test_double_float_split_within_2_pow_minus_48():
    rng = np.random.default_rng(5)
    worst = 0.0
    for k in range(20000):
        d = float(rng.standard_normal() * 2.0 ** rng.integers(-75, 95))
        if d == 0.0:
            continue
        h, lo = df_split(d)
        worst = max(worst, abs((float(h) + float(lo)) - d) / abs(d))
    assert worst <= 2.0 ** -48, worst
