"""The device RNG stream equals the C library's rand() stream."""
import shutil
import subprocess

import pytest

from conftest import ROOT

PROG = r"""
#include <cstdio>
#include <cstdlib>
#include "rng.hpp"
int main() {
    const unsigned seeds[] = {0u, 1u, 7u, 1000u, 1511u, 123456789u, 2147483647u};
    for (unsigned s : seeds) {
        std::srand(s);
        mcacg::RandStream r;
        r.seed(s);
        for (int i = 0; i < 20000; ++i) {
            int a = std::rand(), b = r.next_int();
            if (a != b) { std::printf("seed %u draw %d: %d != %d\n", s, i, a, b); return 1; }
        }
        std::srand(s);
        r.seed(s);
        for (int i = 0; i < 100; ++i) {
            double x = std::rand(); x = x / RAND_MAX;
            if (x != r.uniform()) { std::printf("uniform differs\n"); return 1; }
        }
    }
    std::printf("ok\n");
    return 0;
}
"""


def test_rand_stream_matches_c_library(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    (tmp_path / "t.cpp").write_text(PROG)
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", str(ROOT / "mcac_gb300" / "csrc"), "-o", str(tmp_path / "t"),
                    str(tmp_path / "t.cpp")], check=True)
    out = subprocess.run([str(tmp_path / "t")], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout
