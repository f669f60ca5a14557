"""Exactness of the multiply-high division constants of the 2-D and 3-D
Life-like kernels.

``xk_div_magic(d, N)`` (``xentica_gb300/csrc/xk_internal.cuh``) returns a
32-bit m with floor(n * m / 2^32) == floor(n / d) for every n <= N, or 0 when
it cannot guarantee that (the kernels then divide); the kernels divide word
indices by the words per row and, in 3-D, by the height.  The host routine is
compiled with nvcc (host code only, no GPU needed) and checked against
integer division at the points where a rounded-up reciprocal errs first -- just
below multiples of d, and the top of the range -- plus random indices, for
divisors and ranges of the shapes the kernels see; every 2-D lattice up to
4096 x 65535 cells and every 3-D case listed must get a constant.
"""
import os
import shutil
import subprocess
import tempfile

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "xentica_gb300", "csrc")
INCLUDE = os.path.join(HERE, "..", "include")

PROGRAM = r"""
#include "xk_internal.cuh"
#include <cstdio>
#include <random>

int main()
{
    std::mt19937_64 rng(20261203);
    long long used = 0, declined = 0, checked = 0, bad = 0;
    auto run = [&](uint64_t d, uint64_t N) {
        const uint32_t m = xk_div_magic(d, N);
        if (!m) { ++declined; return; }
        ++used;
        auto test = [&](uint64_t n) {
            if (n > N) return;
            const uint64_t q = ((uint64_t)(uint32_t)n * m) >> 32;
            ++checked;
            if (q != n / d) ++bad;
        };
        for (uint64_t k = 0; k < 40; ++k) {
            test(k);
            test(N - k);
            test(k * d);
            if (k) test(k * d - 1);
            const uint64_t top = (N / d - k) * d;    // multiples near the top
            test(top);
            if (top) test(top - 1);
        }
        for (int r = 0; r < 2000; ++r) test(rng() % (N + 1));
    };
    // 2-D: words per row 2..128 (rows up to 4096 cells), up to 65535 rows
    for (uint64_t wpr = 2; wpr <= 128; ++wpr)
        for (uint64_t H : {1ull, 7ull, 640ull, 4096ull, 65535ull})
            run(wpr, H * wpr);
    // 3-D: N = H * D * wpr indices divided by wpr, then H * D by H
    for (uint64_t wpr : {2ull, 3ull, 5ull, 8ull, 9ull})
        for (uint64_t H : {2ull, 63ull, 64ull, 100ull, 255ull, 256ull, 1000ull})
            for (uint64_t D : {1ull, 17ull, 256ull, 4096ull}) {
                run(wpr, H * D * wpr);
                run(H, H * D);
            }
    const long long shape_declined = declined;
    // larger ranges (declining is allowed: the kernel then divides), among
    // them lattices of a million rows, and ranges near the 32-bit limit
    for (uint64_t wpr = 2; wpr <= 128; ++wpr) run(wpr, 1000003ull * wpr);
    for (int r = 0; r < 3000; ++r) {
        const uint64_t d = 2 + rng() % 1000000;
        const uint64_t N = rng() % 0xFFFFFFFFull;
        run(d, N);
    }
    run(3, 0xFFFFFFFFull);
    run(641, 0xFFFFFFFFull);
    run(65535, 0xFFFFFFFFull);
    std::printf("%lld %lld %lld %lld\n", used, shape_declined, checked, bad);
    return 0;
}
"""


def _nvcc():
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    path = os.path.join(cuda, "bin", "nvcc")
    return path if os.path.exists(path) else shutil.which("nvcc")


def test_div_magic_exact():
    nvcc = _nvcc()
    if not nvcc:
        pytest.skip("nvcc not found")
    with tempfile.TemporaryDirectory(prefix="xk_divmagic_") as tmp:
        src = os.path.join(tmp, "divmagic.cu")
        exe = os.path.join(tmp, "divmagic")
        with open(src, "w") as fh:
            fh.write(PROGRAM)
        subprocess.run([nvcc, "-std=c++17", "-O2", "-I", CSRC, "-I", INCLUDE, src, "-o", exe],
                       check=True, capture_output=True, text=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split()
    used, shape_declined, checked, bad = map(int, out)
    assert bad == 0, "%d of %d quotients wrong" % (bad, checked)
    # every lattice shape of the 2-D and 3-D cases gets a constant (else its
    # kernel would fall back to division)
    assert shape_declined == 0
    assert used > 1000 and checked > 1000000
