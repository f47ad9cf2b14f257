"""The Bethe-Moliere inverse CDF of the CUDA sources (pt_moliere.cuh, its
float64 form compiled for the host) against the oracle, with and without
contraction into fused multiply-adds (the device contracts), on the CPU."""
import os
import platform
import shutil
import subprocess

import numpy as np
import pytest

from oracle import physics as P

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "petite_gb300", "csrc")
SRC = r'''
#include <cstdio>
#include "pt_moliere.cuh"
int main() {
  double u, B;
  while (scanf("%lf %lf", &u, &B) == 2) printf("%.17g\n", pt::moliere_x<double>(u, B));
  return 0;
}
'''


def nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    pytest.skip("nvcc not available")


def cases(seed=9):
    rng = np.random.default_rng(seed)
    U, Bs = [], []
    for B in (3.15, 3.7, 5.0, 7.5, 10.0, 14.0, 19.0):
        f00 = 0.5 * (2.0 + P.moliere_f1_at_zero() / B)
        u = np.concatenate([rng.uniform(0, 1, 300), 1 - 10 ** rng.uniform(-7, -0.5, 80),
                            rng.uniform(0.0095, 0.0105 * f00, 60)])
        U.append(u)
        Bs.append(np.full(len(u), B))
    return np.concatenate(U), np.concatenate(Bs)


FLAGS = [[]]
if platform.machine() == "x86_64":
    FLAGS.append(["-Xcompiler", "-mfma,-ffp-contract=fast"])
else:
    FLAGS.append(["-Xcompiler", "-ffp-contract=fast"])


@pytest.mark.parametrize("flags", FLAGS, ids=["plain", "contracted"])
def test_host_inverse_cdf_matches_oracle(tmp_path, flags):
    src = tmp_path / "m.cu"
    src.write_text(SRC)
    exe = tmp_path / "m"
    subprocess.run([nvcc(), "-std=c++17", "-O2", "-I" + CSRC, *flags, str(src), "-o", str(exe)], check=True,
                   capture_output=True)
    u, B = cases()
    inp = "\n".join(f"{float(a)!r} {float(b)!r}" for a, b in zip(u, B))
    out = subprocess.run([str(exe)], input=inp, capture_output=True, text=True, check=True).stdout.split()
    got = np.array([float(v) for v in out])
    want = np.array([P.moliere_x(a, b) for a, b in zip(u, B)])
    np.testing.assert_allclose(got, want, rtol=2e-13, atol=0)
