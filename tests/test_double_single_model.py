"""The double-single arithmetic of csrc/tp_dsf.cuh, restated operation for
operation on the CPU (FP32 rounding emulated exactly), against the error
bounds its comments state: two-sum exact; a + b within 2^-45 (|a| + |b|) and
a * b within 2^-45 |a| |b| however the high parts cancel (the split truncates h,
so l reaches 2^-23 |h|); the double -> pair
split within 2^-47 |v| down to |v| ~ 2^-102 (then within FP32's smallest
subnormal step); one Newton step from an FP32 estimate leaving 1/sqrt and
1/x within 2^-42. The device functions themselves are checked on the GPU
by the parity tests (test_fine_ec.py, test_coarse_solve.py)."""
from fractions import Fraction as Fr
import struct

import numpy as np
import pytest

f32 = np.float32


def fr(x):
    return Fr(float(x))  # float32 -> float64 is exact


def round32(x):
    """Round an exact rational to the nearest float32, ties to even."""
    if x == 0:
        return f32(0.0)
    c = f32(float(x))  # double rounding: the answer is c or a neighbour
    best = None
    for y in (np.nextafter(c, f32(-np.inf)), c, np.nextafter(c, f32(np.inf))):
        if not np.isfinite(y):
            continue
        d = abs(fr(y) - x)
        if best is None or d < best[0] or (d == best[0] and (struct.unpack("<I", struct.pack("<f", y))[0] & 1) == 0):
            best = (d, y)
    return best[1]


def add(a, b):
    return round32(fr(a) + fr(b))


def sub(a, b):
    return round32(fr(a) - fr(b))


def mul(a, b):
    return round32(fr(a) * fr(b))


def fma(a, b, c):
    return round32(fr(a) * fr(b) + fr(c))


# the device operations (tp_dsf.cuh), a value being the pair (h, l)
def ds_add(a, b):
    s = add(a[0], b[0])
    bb = sub(s, a[0])
    e = add(sub(a[0], sub(s, bb)), sub(b[0], bb))
    return (s, add(e, add(a[1], b[1])))


def ds_mul(a, b):
    p = mul(a[0], b[0])
    e = fma(a[0], b[0], -p)
    e = fma(a[0], b[1], e)
    e = fma(a[1], b[0], e)
    return (p, e)


def ds_from(v):
    b = struct.unpack("<Q", struct.pack("<d", v))[0]
    hw, lw = b >> 32, b & 0xFFFFFFFF
    sg = hw & 0x80000000
    e = (hw >> 20) & 0x7FF
    if e < 897:
        return (f32(0.0), f32(0.0))
    if e > 1150:
        nan = e == 2047 and ((hw & 0xFFFFF) | lw) != 0
        return (np.frombuffer(struct.pack("<I", 0x7FC00000 if nan else (sg | 0x7F800000)), f32)[0], f32(0.0))
    hb = sg | ((e - 896) << 23) | ((hw & 0xFFFFF) << 3) | (lw >> 29)
    h = np.frombuffer(struct.pack("<I", hb), f32)[0]
    low = round32(Fr(lw & 0x1FFFFFFF))  # the int -> float conversion rounds to nearest
    l = mul(mul(low, f32(2.0 ** -52)), np.frombuffer(struct.pack("<I", (e - 896) << 23), f32)[0])
    return (h, -l if sg else l)


def ds_rsqrt(d, est):
    x = add(d[0], d[1])
    h = est(x)
    th = mul(h, h)
    tl = fma(h, h, -th)
    p = mul(d[0], th)
    pe = fma(d[0], th, -p)
    pe = fma(d[0], tl, pe)
    pe = fma(d[1], th, pe)
    e = sub(sub(f32(1.0), p), pe)
    return (h, mul(mul(f32(0.5), h), e))


def ds_rcp(d):
    x = add(d[0], d[1])
    h = round32(1 / fr(x))  # __frcp_rn: correctly rounded
    p = mul(d[0], h)
    pe = fma(d[0], h, -p)
    pe = fma(d[1], h, pe)
    e = sub(sub(f32(1.0), p), pe)
    return (h, mul(h, e))


def val(a):
    return fr(a[0]) + fr(a[1])


def rand_ds(rng, scale):
    v = float(rng.uniform(-1, 1)) * scale
    return ds_from(v)


N = 400


def test_two_sum_is_exact():
    rng = np.random.default_rng(0)
    for _ in range(N):
        a, b = f32(rng.standard_normal() * 10.0 ** rng.integers(-3, 4)), f32(rng.standard_normal())
        s = add(a, b)
        bb = sub(s, a)
        e = add(sub(a, sub(s, bb)), sub(b, bb))
        assert fr(s) + fr(e) == fr(a) + fr(b)


def test_sum_and_product_bounds():
    rng = np.random.default_rng(1)
    for i in range(N):
        a = rand_ds(rng, 10.0 ** rng.integers(-6, 6))
        if i % 3 == 0:  # the high parts cancel
            v = float(val(a)) * (1 + float(rng.uniform(-1e-6, 1e-6)))
            b = ds_from(-v)
        else:
            b = rand_ds(rng, 10.0 ** rng.integers(-6, 6))
        s = ds_add(a, b)
        assert abs(val(s) - (val(a) + val(b))) <= Fr(2) ** -45 * (abs(val(a)) + abs(val(b)))
        p = ds_mul(a, b)
        assert abs(val(p) - val(a) * val(b)) <= Fr(2) ** -45 * abs(val(a)) * abs(val(b))


def test_chained_unnormalised_sums_stay_bounded():
    """Many additions without renormalisation (the element kernel's butterflies
    and accumulations): the error stays below 2^-45 times the sum of the
    magnitudes that went in."""
    rng = np.random.default_rng(2)
    for _ in range(20):
        acc = (f32(0.0), f32(0.0))
        exact, mag = Fr(0), Fr(0)
        for _ in range(40):
            t = rand_ds(rng, 10.0 ** rng.integers(-2, 3))
            if rng.uniform() < 0.5:
                t = (-t[0], -t[1])
            acc = ds_add(acc, t)
            exact += val(t)
            mag += abs(val(t))
        assert abs(val(acc) - exact) <= Fr(2) ** -45 * mag


@pytest.mark.parametrize("v", [1.0, -3.25, 1e-30, 7e30, 0.1, -2.0 / 3.0, 1.2e-38 * 1.5, 3.0e38])
def test_split_of_a_double(v):
    h, l = ds_from(v)
    assert abs(val((h, l)) - Fr(v)) <= Fr(2) ** -47 * abs(Fr(v)) + Fr(2) ** -149


def test_split_edges():
    assert ds_from(1e-39) == (0.0, 0.0)  # below FP32's normal range
    assert np.isinf(ds_from(1e39)[0]) and ds_from(-1e39)[0] < 0
    assert np.isnan(ds_from(float("nan"))[0])
    rng = np.random.default_rng(3)
    for _ in range(N):
        v = float(rng.standard_normal()) * 10.0 ** int(rng.integers(-37, 37))
        assert abs(val(ds_from(v)) - Fr(v)) <= Fr(2) ** -47 * abs(Fr(v)) + Fr(2) ** -150


def test_reciprocal_square_root_and_reciprocal():
    """rsqrtf is modelled at its documented worst (2 ulp either way); one
    Newton step must still leave 2^-42."""
    rng = np.random.default_rng(4)
    ulp = lambda x: np.spacing(x)
    ests = [lambda x: round32(Fr(1) / Fr(float(np.sqrt(np.float64(x))))),
            lambda x: f32(round32(Fr(1) / Fr(float(np.sqrt(np.float64(x))))) + 2 * ulp(f32(1 / np.sqrt(x)))),
            lambda x: f32(round32(Fr(1) / Fr(float(np.sqrt(np.float64(x))))) - 2 * ulp(f32(1 / np.sqrt(x))))]
    for _ in range(N // 4):
        d = ds_from(float(rng.uniform(1e-6, 1e6)))
        exact_rs = 1 / np.sqrt(np.longdouble(float(val(d))))
        for est in ests:
            r = ds_rsqrt(d, est)
            assert abs(float(val(r)) - float(exact_rs)) <= 2.0 ** -42 * float(exact_rs)
        q = ds_rcp(d)
        assert abs(val(q) * val(d) - 1) <= Fr(2) ** -42


def test_float_to_double_bits_on_the_host(tmp_path):
    """f32_to_f64_bits (the integer float -> double conversion that ds_to
    uses instead of FP64 conversions) compiled for the host with nvcc, against
    the exact conversion, on every exponent class: zeros, subnormals, normals,
    infinities and NaN."""
    import os
    import shutil
    import subprocess

    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    csrc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                        "topopt-in-openmp-gpu_gb300", "csrc")
    src = tmp_path / "cvt.cu"
    src.write_text(
        '#include <cstdio>\n#include "tp_dsf.cuh"\n'
        "int main(int argc, char** argv) {\n"
        '  FILE* fi = fopen(argv[1], "rb"); FILE* fo = fopen(argv[2], "wb");\n'
        "  unsigned u;\n"
        "  while (fread(&u, 4, 1, fi) == 1) { unsigned long long b = tp::f32_to_f64_bits(u); fwrite(&b, 8, 1, fo); }\n"
        "  fclose(fi); fclose(fo); return 0;\n}\n")
    exe = tmp_path / "cvt"
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17", "-I", csrc, str(src),
                    "-o", str(exe)], check=True,
                   capture_output=True)
    rng = np.random.default_rng(7)
    edge = np.array([0, 0x80000000, 1, 0x80000001, 0x007fffff, 0x00400000, 0x00000100, 0x00800000,
                     0x7f7fffff, 0xff7fffff, 0x3f800000, 0x7f800000, 0xff800000, 0x7fc00000, 0x7f800001],
                    dtype=np.uint32)
    subn = rng.integers(0, 1 << 23, 20000, dtype=np.uint32) | (rng.integers(0, 2, 20000, dtype=np.uint32) << 31)
    bits = np.concatenate([edge, subn, rng.integers(0, 1 << 32, 200000, dtype=np.uint64).astype(np.uint32)])
    (tmp_path / "in.bin").write_bytes(bits.tobytes())
    subprocess.run([str(exe), str(tmp_path / "in.bin"), str(tmp_path / "out.bin")], check=True)
    got = np.frombuffer((tmp_path / "out.bin").read_bytes(), dtype=np.uint64)
    assert got.size == bits.size
    want = bits.view(np.float32).astype(np.float64)
    nan = np.isnan(want)
    assert np.array_equal(got[~nan], want[~nan].view(np.uint64))
    assert np.all(np.isnan(got[nan].view(np.float64)))
