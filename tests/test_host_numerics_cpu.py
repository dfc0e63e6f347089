"""The library's host numerics of the Chebyshev / PPCG switch
(csrc/tl_host_numerics.cpp: tqli, the Lanczos eigenvalue estimate, the
Chebyshev coefficients; tea_leaf_cheby.f90:46-174) against the oracle's
restatement of the same routines, bit for bit, on the CPU.  Both are
compiled without implicit contraction (-ffp-contract=off), so every result
must be identical."""
import os
import shutil
import subprocess

import pytest

from tests.oracle_run import build_oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

DRIVER = r"""
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>
#include "tl_host_numerics.h"
extern "C" {
int ora_calc_eigenvalues(const double *cg_alphas, const double *cg_betas, int n, double *eigmin, double *eigmax);
void ora_calc_ch_coefs(double *alphas, double *betas, double eigmin, double eigmax, double *theta, int n);
}
static uint64_t state = 0x9E3779B97F4A7C15ull;
static double uniform(double lo, double hi) {  // splitmix64
    uint64_t z = (state += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return lo + (hi - lo) * (double)(z >> 11) * (1.0 / 9007199254740992.0);
}
static bool same(double a, double b) { return std::memcmp(&a, &b, sizeof a) == 0; }
int main() {
    int cases = 0, diff = 0;
    for (int n = 1; n <= 160; n += 3) {
        for (int rep = 0; rep < 4; ++rep) {
            std::vector<double> al(n), be(n);
            for (int k = 0; k < n; ++k) {
                al[k] = uniform(1e-3, 2.0);
                be[k] = uniform(1e-4, 0.999);
            }
            double a0 = 0, a1 = 0, b0 = 0, b1 = 0;
            const int i0 = tl::tl_calc_eigenvalues(al.data(), be.data(), n, &a0, &a1);
            const int i1 = ora_calc_eigenvalues(al.data(), be.data(), n, &b0, &b1);
            ++cases;
            if (i0 != i1 || (i0 == 0 && (!same(a0, b0) || !same(a1, b1)))) ++diff;
        }
    }
    for (int rep = 0; rep < 50; ++rep) {
        const double emin = uniform(1e-3, 10.0), emax = emin * uniform(1.5, 1e5);
        const int n = 1 + (int)uniform(0.0, 600.0);
        std::vector<double> a0(n), b0(n), a1(n), b1(n);
        double t0 = 0, t1 = 0;
        tl::tl_calc_ch_coefs(a0.data(), b0.data(), emin, emax, &t0, n);
        ora_calc_ch_coefs(a1.data(), b1.data(), emin, emax, &t1, n);
        ++cases;
        bool ok = same(t0, t1);
        for (int k = 0; k < n; ++k) ok = ok && same(a0[k], a1[k]) && same(b0[k], b1[k]);
        if (!ok) ++diff;
    }
    std::printf("%d %d\n", cases, diff);
    return 0;
}
"""


def test_library_host_numerics_equal_the_oracle_bit_for_bit(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no C++ compiler")
    build_oracle()
    src = tmp_path / "numerics.cpp"
    src.write_text(DRIVER)
    exe = tmp_path / "numerics"
    csrc = os.path.join(ROOT, "tealeaf_cuda_gb300", "csrc")
    oracle_build = os.path.join(ROOT, "oracle", "_build")
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", csrc, str(src),
                    os.path.join(csrc, "tl_host_numerics.cpp"), "-L", oracle_build, "-ltea_oracle",
                    "-Wl,-rpath," + oracle_build, "-o", str(exe)], check=True, capture_output=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    cases, diff = int(out[0]), int(out[1])
    assert cases > 200
    assert diff == 0
