"""The integer float <-> double conversions of the mixed form (neofiz_gb300/csrc/nf_fpconv.h)
against the C conversions, compiled from the same header for the host.

The device kernels use these forms in place of the conversion instructions (the node geometry
split into float pairs, v dt, and the force gather's widening), and the mixed form's bits
depend on them giving exactly what the instructions give: IEEE round to nearest even, no
flushing. The check covers every float for the widening, and for the split and the narrowing
every exponent of their range with random significands, exact ties, values around the ties
and the 29-bit carries, plus the range ends and the special values.
"""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
HEADER = os.path.join(HERE, "..", "neofiz_gb300", "csrc", "nf_fpconv.h")

CHECK = r"""
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include "nf_fpconv.h"

static uint32_t fbits(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static float fval(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
static uint64_t dbits(double d) { uint64_t u; memcpy(&u, &d, 8); return u; }
static double dval(uint64_t u) { double d; memcpy(&d, &u, 8); return d; }

static long bad = 0, split = 0, narrow = 0;
static void one(double x) {
    const uint64_t b = dbits(x);
    uint32_t h, l, o;
    if (nf_split_bits((uint32_t)(b >> 32), (uint32_t)b, h, l)) {
        split++;
        const float hi = (float)x, lo = (float)(x - (double)hi);
        if (h != fbits(hi) || l != fbits(lo)) {
            if (bad < 5) printf("split %a\n", x);
            bad++;
        }
    }
    if (nf_narrow_bits((uint32_t)(b >> 32), (uint32_t)b, o)) {
        narrow++;
        if (o != fbits((float)x)) {
            if (bad < 5) printf("narrow %a\n", x);
            bad++;
        }
    }
}

int main() {
    for (uint64_t u = 0; u <= 0xffffffffull; u++) {
        const float f = fval((uint32_t)u);
        uint32_t hw, lw;
        nf_widen_words((uint32_t)u, hw, lw);
        const double got = dval(((uint64_t)hw << 32) | lw);
        if (std::isnan(f) ? !std::isnan(got) : dbits(got) != dbits((double)f)) {
            if (bad < 5) printf("widen %08x\n", (unsigned)u);
            bad++;
        }
    }
    std::mt19937_64 rng(20251204);
    for (long i = 0; i < 24000000; i++) {
        const uint64_t ed = 890 + rng() % 270, sign = rng() & 1;
        uint64_t b = (sign << 63) | (ed << 52) | (rng() & ((1ull << 52) - 1));
        switch (i % 4) {
        case 1: b = (b & ~0x1fffffffull) | 0x10000000ull; break;                    // a tie
        case 2: b = (b & ~0x1fffffffull) | (0x10000000ull + rng() % 9 - 4); break;  // near it
        case 3: b |= 0x1fffffc0ull; break;                                          // carries
        }
        one(dval(b));
    }
    const double special[] = {0.0, -0.0, 1.0, -1.0, INFINITY, -INFINITY, NAN, 0.1, -0.0123,
                              3.4028234663852886e38, 5e-324, 1e-300, 1e300};
    for (double x : special) one(x);
    for (int e = -80; e <= 128; e++)
        for (int k = 0; k < 512; k++) {
            const double x = std::ldexp(1.0 + k / 512.0, e);
            one(x);
            one(-x);
            one(std::nextafter(x, 0.0));
            one(std::nextafter(x, 1e300));
        }
    printf("bad %ld split %ld narrow %ld\n", bad, split, narrow);
    return bad ? 1 : 0;
}
"""


def test_integer_conversions_match_the_c_conversions(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    src = tmp_path / "check.cpp"
    src.write_text(CHECK)
    exe = tmp_path / "check"
    subprocess.run([cxx, "-O2", "-ffp-contract=off", "-I", os.path.dirname(HEADER), str(src),
                    "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stdout
    fields = dict(zip(out.stdout.split()[0::2], map(int, out.stdout.split()[1::2])))
    assert fields["bad"] == 0
    # most of the random cases fall inside the fast ranges, which is what is being checked
    assert fields["split"] > 15_000_000 and fields["narrow"] > 18_000_000
