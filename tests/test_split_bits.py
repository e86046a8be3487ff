r"""The integer high/low split (pyci_gb300/csrc/split_bits.h, used by the device
split kernel) against its FP64 definition hi = fl32(v), lo = fl32(v - hi),
bit for bit, on random values over the whole exponent range, exact rounding
ties, carries into the exponent and special values.  Compiled for the host
with g++ (the header is plain C++ outside nvcc)."""

import os
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

HARNESS = r"""
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <random>
#include "split_bits.h"

static unsigned fbits(float f) { unsigned u; std::memcpy(&u, &f, 4); return u; }
static double dfrom(unsigned long long u) { double d; std::memcpy(&d, &u, 8); return d; }

static long bad = 0, checked = 0;
static void check(double v) {
    float h, l;
    pyci_gpu::split_hi_lo(v, h, l);
    const float h_ref = static_cast<float>(v);
    const float l_ref = static_cast<float>(v - static_cast<double>(h_ref));
    ++checked;
    if (std::isnan(v)) {
        if (!std::isnan(h)) ++bad;
        return;
    }
    if (fbits(h) != fbits(h_ref) || fbits(l) != fbits(l_ref)) {
        if (bad < 10) std::printf("mismatch v=%.17g\n", v);
        ++bad;
    }
}

int main() {
    std::mt19937_64 g(12345);
    // random bit patterns (all exponents), random CI-like magnitudes
    for (int i = 0; i < 2000000; ++i) check(dfrom(g()));
    std::normal_distribution<double> nd;
    std::uniform_real_distribution<double> ue(-40.0, 10.0);
    for (int i = 0; i < 2000000; ++i) check(nd(g) * std::pow(2.0, ue(g)));
    // exact ties and carries: mantissa low 29 bits = 2^28, and all-ones high bits
    for (int e = 1023 - 80; e <= 1023 + 130; ++e)
        for (unsigned long long hi23 : {0ULL, 1ULL, 2ULL, 0x3FFFFEULL, 0x3FFFFFULL, 0x7FFFFFULL})
            for (unsigned long long lo29 : {0ULL, 1ULL, (1ULL << 28) - 1, 1ULL << 28, (1ULL << 28) + 1, (1ULL << 29) - 1})
                for (unsigned long long s : {0ULL, 1ULL}) {
                    const unsigned long long m = (hi23 << 29) | lo29;
                    check(dfrom((s << 63) | (static_cast<unsigned long long>(e) << 52) | (m & ((1ULL << 52) - 1))));
                }
    // special values
    const double sp[] = {0.0, -0.0, 1.0, -1.0, 1e-300, -1e-300, 4.9e-324, 1e300, -1e300,
                         std::numeric_limits<double>::infinity(), -std::numeric_limits<double>::infinity(),
                         std::numeric_limits<double>::quiet_NaN(), 3.4028234663852886e38, 3.4028235677973366e38,
                         1.1754943508222875e-38, 1.1754942106924411e-38};
    for (double v : sp) check(v);
    std::printf("checked %ld bad %ld\n", checked, bad);
    return bad ? 1 : 0;
}
"""


def test_integer_split_matches_fp64_definition():
    if subprocess.run(["which", "g++"], capture_output=True).returncode != 0:
        pytest.skip("g++ not available")
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "h.cpp")
        exe = os.path.join(d, "h")
        with open(src, "w") as f:
            f.write(HARNESS)
        subprocess.run(["g++", "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "pyci_gb300", "csrc"), src, "-o", exe],
                       check=True)
        out = subprocess.run([exe], capture_output=True, text=True)
        assert out.returncode == 0, out.stdout
        assert "bad 0" in out.stdout
