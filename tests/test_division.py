"""The FP64 quotients the kernels take on the integer pipes, without a GPU.

* The host's divisor preparation (make_qrecip in ark_state.h, compiled here with g++) gives the
  exact ceiling of 2^116 / M for the divisor's significand M (2^64 - 1 for M = 2^52), the
  exponent offset and the sign, and marks zero, subnormal and non-finite divisors.
* A bit-exact model of the device's quotient (qdiv_try), its doubled form (qdiv2) and the
  per-cell reciprocal by Newton steps (qrecip_var) agrees with IEEE division wherever the
  integer path takes the quotient, including ties of short significands and the power-of-two
  divisors.  The FP32 seed of the Newton steps is modelled as RN32(1/f) moved by up to two
  units in the last place, the approximation's error bound.
* A model of the integer fixed-point image of the bulk-flow sum (fixed32) equals the FP64 form's
  round(v * 2^32), ties to even, clamping and NaN included.
The GPU's own check of the same code is ark_selftest_division (tests/test_gpu_parity.py).
"""
import os
import random
import shutil
import struct
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "ark-cpp-mpi_gb300", "csrc")
CUDA_INC = "/usr/local/cuda/include"

PROGRAM = r"""
#include "ark_state.h"
#include <cstdio>
#include <cstring>
int main() {
    unsigned long long bits;
    while (std::scanf("%llx", &bits) == 1) {
        double b;
        std::memcpy(&b, &bits, sizeof b);
        const ark::QRecip q = ark::make_qrecip(b);
        std::printf("%08x%08x %d %08x\n", q.r1, q.r0, q.k, q.sgn);
    }
    return 0;
}
"""


def bits(x):
    return struct.unpack("<Q", struct.pack("<d", x))[0]


def from_bits(b):
    return struct.unpack("<d", struct.pack("<Q", b))[0]


def exact_recip(b):
    """(r, k, sgn) as make_qrecip defines them, by exact integer arithmetic."""
    B = bits(b)
    eb = (B >> 52) & 0x7FF
    sgn = (B >> 32) & 0x80000000
    if eb in (0, 0x7FF):
        return None, -100000, sgn
    M = (B & ((1 << 52) - 1)) | (1 << 52)
    r = (1 << 64) - 1 if M == 1 << 52 else -(-(1 << 116) // M)
    return r, 1022 - eb, sgn


def divisors(n, seed):
    rng = random.Random(seed)
    out = [1.0, 0.5, 2.0, -4.0, 2.0 ** -1000, 2.0 ** 1000, 10.0, 100.0, 1.0 / 3.0, -7.0,
           1.0 + 2.0 ** -52, 2.0 - 2.0 ** -52, 2 * np.pi / 256, 2.0 / 128, np.pi / 128, 10.3 ** 2,
           0.0, -0.0, 5e-324, 2.0 ** -1030, float("inf"), float("nan")]
    while len(out) < n:
        out.append(from_bits(rng.getrandbits(64)))
    return out


@pytest.mark.skipif(shutil.which("g++") is None or not os.path.isfile(os.path.join(CUDA_INC, "cuda_runtime.h")),
                    reason="needs g++ and the CUDA headers")
def test_host_divisor_reciprocal_is_the_exact_ceiling(tmp_path):
    src = tmp_path / "qrecip.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "qrecip"
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I", CSRC, "-I", CUDA_INC, str(src), "-o", str(exe)],
                   check=True)
    bs = divisors(4000, 7)
    inp = "\n".join(f"{bits(b):016x}" for b in bs) + "\n"
    out = subprocess.run([str(exe)], input=inp, capture_output=True, text=True, check=True).stdout.split("\n")
    for b, line in zip(bs, out):
        r_s, k_s, sgn_s = line.split()
        r, k, sgn = exact_recip(b)
        assert int(k_s) == k, (b, line)
        assert int(sgn_s, 16) == sgn, (b, line)
        if r is not None:
            assert int(r_s, 16) == r, (b, line)


def qdiv_model(a, rk, twice=False):
    """The device's qdiv_try: the quotient's bits, or None where another path takes it."""
    r, k, sgn = rk
    A = bits(a)
    ea = (A >> 52) & 0x7FF
    Ma = (A & ((1 << 52) - 1)) | (1 << 52)
    T = (Ma * r) >> 53
    s = T >> 63
    sh = 10 + s
    below = (T << (32 - sh)) & 0xFFFFFFFF
    E = ea + s + k + (1 if twice else 0)
    if not (1 <= ea <= (2045 if twice else 2046)) or not (1 <= E <= 2046) or below == 0x80000000:
        return None
    sig = (T >> sh) + (1 if below > 0x80000000 else 0)
    out = sig + ((E - 1) << 52)
    return from_bits(out | ((((A >> 32) & 0x80000000) ^ sgn) << 32))


def newton_model(b, seed_ulps):
    """qrecip_var's r for divisor b, with its FP32 seed moved by seed_ulps units."""
    B = bits(b)
    m1 = ((B >> 32) & 0xFFFFF) | 0x100000
    m0 = B & 0xFFFFFFFF
    M = (m1 << 32) | m0
    fbits = 0x3F800000 | (((B >> 32) & 0xFFFFF) << 3) | (m0 >> 29)
    f = np.frombuffer(struct.pack("<I", fbits), dtype=np.float32)[0]
    rf = np.float32(np.float32(1.0) / f)
    rf = np.nextafter(rf, np.float32(2.0 if seed_ulps > 0 else 0.0), dtype=np.float32) if seed_ulps else rf
    for _ in range(abs(seed_ulps) - 1 if seed_ulps else 0):
        rf = np.nextafter(rf, np.float32(2.0 if seed_ulps > 0 else 0.0), dtype=np.float32)
    R = min(int(float(rf) * 2.0 ** 32), 2 ** 32 - 1) << 32
    mask = (1 << 64) - 1
    for _ in range(2):
        W = ((M * R) >> 32) & mask
        D = (-W) & mask
        if D >= 1 << 63:
            D -= 1 << 64
        R = (R + (((R * D) >> 64) >> 20)) & mask
    rem = (-(M * R)) & mask
    if rem >= 1 << 63:
        rem -= 1 << 64
    for _ in range(3):
        if rem > 0:
            R = (R + 1) & mask
            rem -= M
    return (1 << 64) - 1 if M == 1 << 52 else R


def test_integer_quotient_model_matches_ieee_division():
    rng = random.Random(11)
    checked = fallbacks = 0
    for b in divisors(600, 3):
        rk = exact_recip(b)
        if rk[0] is None:
            continue
        for t in range(60):
            if t % 5 == 0:  # quotients near ties: short significands
                a = float(rng.randint(1, 2 ** 27)) * b * rng.choice([1.0, 0.75, 1.5])
            else:
                a = rng.uniform(1.0, 2.0) * 2.0 ** rng.randint(-900, 900) * rng.choice([1.0, -1.0])
            if not np.isfinite(a) or a == 0.0:
                continue
            for twice in (False, True):
                got = qdiv_model(a, rk, twice)
                want = (2.0 * a) / b if twice else a / b
                if got is None:
                    # outside the normal range the other path is expected; inside it only the
                    # rounding-midpoint pattern (about 1 in 2048) should send a quotient there
                    if abs(want) >= 2.0 ** -1021 and np.isfinite(want) and abs(a) < 2.0 ** 1022:
                        fallbacks += 1
                    continue
                assert bits(got) == bits(want), (a, b, twice)
                checked += 1
    assert checked > 40000
    assert fallbacks < checked // 200


def test_newton_reciprocal_reaches_the_ceiling():
    rng = random.Random(5)
    ms = [2 ** 52, 2 ** 52 + 1, 2 ** 53 - 1, 2 ** 52 + 2 ** 29, 2 ** 53 - 2 ** 29] + [rng.randrange(2 ** 52, 2 ** 53)
                                                                                     for _ in range(3000)]
    for M in ms:
        b = from_bits((1023 << 52) | (M - (1 << 52)))
        want = exact_recip(b)[0]
        for u in (-2, -1, 0, 1, 2):
            assert newton_model(b, u) == want, (M, u)


def fixed32_model(v):
    """The device's integer fixed32: round(v * 2^32) to nearest even, v clamped to +-2^30, NaN -> 0."""
    b = bits(v)
    e = (b >> 52) & 0x7FF
    M = (b & ((1 << 52) - 1)) | (1 << 52)
    if e >= 1053:
        if e == 0x7FF and (b & ((1 << 52) - 1)):
            return 0
        m = 1 << 62
    elif e >= 1043:
        m = M << (e - 1043)
    elif e >= 1043 - 54:
        k = 1043 - e
        q, r, half = M >> k, M & ((1 << k) - 1), 1 << (k - 1)
        m = q + (1 if (r > half or (r == half and (q & 1))) else 0)
    else:
        m = 0
    return -m if b >> 63 else m


def test_fixed_point_image_model_matches_the_fp64_form():
    """round(v * 2^32) as the FP64 form computes it: clamp to +-2^30, scale (exact), round to
    nearest even; over the whole exponent range, ties, zeros, infinities and NaN."""
    rng = random.Random(17)
    vals = [0.0, -0.0, float("inf"), -float("inf"), float("nan"), 2.0 ** 30, -2.0 ** 30, 2.0 ** 31, 5e-324,
            2.0 ** -33, 3 * 2.0 ** -33, -2.0 ** -33, 2.0 ** -34, 2.0 ** 29 + 0.5]
    vals += [from_bits(rng.getrandbits(64)) for _ in range(20000)]
    vals += [rng.randint(-2 ** 44, 2 ** 44) * 2.0 ** -33 for _ in range(20000)]  # ties
    for v in vals:
        if v != v:
            want = 0
        else:
            c = min(max(v, -2.0 ** 30), 2.0 ** 30)
            want = int(np.rint(np.float64(c) * np.float64(2.0 ** 32)))  # exact scaling, ties to even
        assert fixed32_model(v) == want, v


def fixed32f_model(f_bits):
    """The device's fixed32 of an FP32 value, from its 32 bits: v = M 2^(e-150), so
    v * 2^32 = M 2^(e-118), shifted left or rounded right to nearest even; clamp at 2^30."""
    e = (f_bits >> 23) & 0xFF
    M = (f_bits & 0x7FFFFF) | 0x800000
    if e >= 157:
        if e == 0xFF and (f_bits & 0x7FFFFF):
            return 0
        m = 1 << 62
    elif e >= 118:
        m = M << (e - 118)
    elif e >= 118 - 25:
        k = 118 - e
        q, r, half = M >> k, M & ((1 << k) - 1), 1 << (k - 1)
        m = q + (1 if (r > half or (r == half and (q & 1))) else 0)
    else:
        m = 0
    return -m if f_bits >> 31 else m


def test_fp32_fixed_point_image_equals_the_image_of_the_widened_value():
    """The FP32 path's bulk-flow term taken from the FP32 bits is the FP64 path's image of the
    same value widened to FP64: every exponent, ties, subnormals, infinities and NaN."""
    rng = random.Random(23)
    pats = [0, 0x80000000, 0x7F800000, 0xFF800000, 0x7FC00000, 0x00000001, 0x807FFFFF, 0x4E800000, 0x4E7FFFFF,
            0x2F000000, 0x2F400000, 0x2E800000, 0x2EC00000]
    pats += [rng.getrandbits(32) for _ in range(40000)]
    pats += [e << 23 | rng.getrandbits(23) | (rng.getrandbits(1) << 31) for e in range(85, 130) for _ in range(200)]
    for fb in pats:
        v = float(np.frombuffer(struct.pack("<I", fb), dtype=np.float32)[0])
        assert fixed32f_model(fb) == fixed32_model(v), hex(fb)
