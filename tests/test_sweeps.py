"""The checkpointed radial sweep of the FP32 path (lu_column_ckpt in
csrc/tc_bodies.cuh) against the plain LU sweep (lu_column), compiled for the
host from the same source text: same solution to 1e-12 (FP64 instantiation)
for every column length from 2 to 399 levels and both first levels (0 for
the theta and z components, 1 for the radial faces), which covers empty and
partial tails and whole batches (of 8 and 16 levels).  Both sweeps take
factors with the row scales folded in (l'_k = l_k sc_k-1 / sc_k,
u'_k = u_k / sc_k, di'_k = di_k sc_k, as the factors kernel stores them); the
harness also solves the row-scaled system with the unfolded factors and
checks that the folded sweep gives the same solution."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
BODIES = os.path.join(HERE, "..", "taylor-couette-afid_gb300", "csrc", "tc_bodies.cuh")

HARNESS = r'''
#include <cmath>
#include <cstdio>
#include <cstddef>
#define __device__
#define __forceinline__ inline
#define __restrict__
template <typename T> T ld(const T* p) { return *p; }
constexpr int kRB = 8;
constexpr int kRBr = 16;
constexpr int kCkpt = CKPT;
%s
int main() {
    int bad = 0;
    for (int nr = 2; nr < 400; ++nr)
        for (int k0 = 0; k0 < 2; ++k0) {
            if (k0 >= nr) continue;
            static double r1[512], r2[512], q1[512], q2[512], q0[512], l[512], di[512], u[512], sc[512];
            static double lf[512], uf[512], dif[512], y[512];
            for (int k = 0; k < 512; ++k) {
                r1[k] = r2[k] = std::sin(k + 1.0);
                q0[k] = q1[k] = q2[k] = std::cos(0.3 * k);
                l[k] = 0.1 * k / 512.0;
                di[k] = 1.0 / (2.0 + 0.01 * k);
                u[k] = 0.3;
                sc[k] = 1.0 + 0.001 * k + 0.2 * std::sin(0.7 * k);
            }
            // row-scaled solve with the unfolded factors
            y[k0] = (r1[k0] + 0.5) * sc[k0];
            for (int k = k0 + 1; k < nr; ++k) y[k] = r1[k] * sc[k] - l[k] * y[k - 1];
            double x = 0.0;
            for (int k = nr - 1; k >= k0; --k) {
                x = (y[k] - (k < nr - 1 ? u[k] * x : 0.0)) * di[k];
                q0[k] += x;
            }
            for (int k = 0; k < 512; ++k) {
                lf[k] = (k > k0 && k < nr) ? l[k] * sc[k - 1] / sc[k] : l[k];
                uf[k] = u[k] / sc[k];
                dif[k] = di[k] * sc[k];
            }
            lu_column<true>(r1, q1, 1, k0, nr, lf, dif, uf, 0.5);
            lu_column_ckpt<true>(r2, q2, 1, k0, nr, lf, dif, uf, 0.5);
            for (int k = 0; k < 512; ++k)
                if (std::fabs(q1[k] - q2[k]) > 1e-12 || std::fabs(q1[k] - q0[k]) > 1e-12) {
                    std::printf("nr %%d k0 %%d level %%d\n", nr, k0, k); ++bad; break;
                }
        }
    std::printf("bad %%d\n", bad);
    return bad != 0;
}
'''


def _extract(src, start, end):
    a = src.index(start)
    return src[a:src.index(end, a)]


@pytest.mark.parametrize("batch", [8, 16])
def test_checkpointed_sweep_matches_plain_sweep(tmp_path, batch):
    if shutil.which("g++") is None:
        pytest.skip("no host C++ compiler")
    src = open(BODIES).read()
    plain = _extract(src, "template <bool EXTRA, typename T>\n__device__ __forceinline__ void lu_column(",
                     "// lu_column without the round trip")
    ckpt = _extract(src, "// Lane operations of the checkpointed sweep",
                    "// Two neighbouring columns in packed FP32")
    cpp = tmp_path / "sweeps.cpp"
    cpp.write_text(HARNESS % (plain + ckpt))
    exe = tmp_path / "sweeps"
    subprocess.run(["g++", "-O1", "-std=c++17", f"-DCKPT={batch}", str(cpp), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
