"""The FFT plans' host-side arithmetic, compiled from the library's own header on the CPU:
fft_radices and stage_twiddle_exponent (common.cuh) build the stage-major twiddle tables
of the lane-sweep FFT (forward radix order) and of the FFT-pair pass (reversed radix order
for its second transform).  A numpy model of both kernels' data movement with those exact
tables (Stockham stages, butterfly b = t + j T, the register hand-off between the two
transforms) must reproduce numpy's FFT.  No GPU needed."""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SIZES = [16, 32, 64, 128, 256, 512, 1024, 2048, 4096, 8192]

SRC = r"""
#include <cstdio>
#include "common.cuh"
int main() {
  const long sizes[] = {16, 32, 64, 128, 256, 512, 1024, 2048, 4096, 8192};
  for (int rmax : {8, 16})
    for (long n : sizes)
      for (int rev = 0; rev < 2; ++rev) {
        int rs[16];
        const int c = so::fft_radices(n, rmax, rev != 0, rs);
        std::printf("plan %d %ld %d %d", rmax, n, rev, c);
        for (int s = 0; s < c; ++s) std::printf(" %d", rs[s]);
        std::printf("\n");
        for (long e = 0; e < n; ++e)
          std::printf("%lld%c", (long long)so::stage_twiddle_exponent(e, n, rmax, rev != 0), e + 1 == n ? '\n' : ' ');
      }
  return 0;
}
"""


@pytest.fixture(scope="module")
def tables(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    cuda_inc = "/usr/local/cuda/include"
    if not cxx or not os.path.isdir(cuda_inc):
        pytest.skip("needs a host C++ compiler and the CUDA headers")
    d = tmp_path_factory.mktemp("fftplan")
    src, exe = d / "plan.cpp", d / "plan"
    src.write_text(SRC)
    subprocess.run([cxx, "-std=c++17", "-O1", "-I", cuda_inc, "-I", os.path.join(ROOT, "split_operator_gb300", "csrc"),
                    str(src), "-o", str(exe)], check=True, capture_output=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines()
    res = {}
    for i in range(0, len(out), 2):
        head = out[i].split()
        rmax, n, rev, c = int(head[1]), int(head[2]), int(head[3]), int(head[4])
        radices = [int(x) for x in head[5:5 + c]]
        exps = np.array([int(x) for x in out[i + 1].split()], dtype=np.int64)
        res[(rmax, n, rev)] = (radices, exps)
    return res


def stockham(x, n, radices, table, dirn):
    """The kernels' stage: butterfly (l, i), k = i mod p, inputs i + r nb twiddled by table
    entry (r - 1) p + k of the stage's section, outputs at (i - k) RS + k + q p."""
    w = np.exp(-2j * np.pi * table / n)
    if dirn > 0:
        w = np.conj(w)
    src, p, off = x.astype(np.complex128), 1, 0
    for rs in radices:
        nb = n // rs
        dst = np.empty_like(src)
        for i in range(nb):
            k = i & (p - 1)
            reg = np.array([src[i + r * nb] * (w[off + (r - 1) * p + k] if (r > 0 and k > 0) else 1.0)
                            for r in range(rs)])
            out = np.fft.fft(reg) if dirn < 0 else np.fft.ifft(reg) * rs
            base = (i - k) * rs + k
            dst[base + np.arange(rs) * p] = out
        if p > 1:
            off += (rs - 1) * p
        p *= rs
        src = dst
    return src


@pytest.mark.parametrize("rmax", [8, 16])
def test_radix_plans(tables, rmax):
    for n in SIZES:
        fwd, _ = tables[(rmax, n, 0)]
        rev, _ = tables[(rmax, n, 1)]
        assert int(np.prod(fwd)) == n and rev == fwd[::-1]
        assert all(r == rmax for r in fwd[:-1]) and fwd[-1] <= rmax
        # the FFT-pair kernel's closed form (rmax 16): S - 1 stages of 16, closing radix rl
        if rmax == 16:
            lg = n.bit_length() - 1
            s = (lg + 3) // 4
            assert fwd == [16] * (s - 1) + [1 << (lg - 4 * (s - 1))]


@pytest.mark.parametrize("rmax", [8, 16])
@pytest.mark.parametrize("n", SIZES)
def test_stage_tables_give_the_dft(tables, rmax, n):
    rng = np.random.default_rng(n + rmax)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    for rev in (0, 1):
        radices, exps = tables[(rmax, n, rev)]
        assert exps.min() >= 0 and exps.max() < n
        f = stockham(x, n, radices, exps, -1)
        assert np.allclose(f, np.fft.fft(x), atol=1e-9 * n)
        g = stockham(x, n, radices, exps, +1)
        assert np.allclose(g, np.fft.ifft(x) * n, atol=1e-9 * n)


@pytest.mark.parametrize("n", SIZES)
def test_fft_pair_register_handoff(tables, n):
    """The FFT-pair pass: forward transform in forward radix order, then the point-wise
    product, then the inverse in reversed order.  The forward's last stage leaves butterfly
    k's outputs at k + q p_last; the inverse's first stage reads i + r n / RS with the same
    butterfly index i = k and RS = the forward's closing radix, i.e. the same values."""
    fwd, ef = tables[(16, n, 0)]
    rev, er = tables[(16, n, 1)]
    rl = fwd[-1]
    p_last = n // rl
    for k in range(min(p_last, 64)):
        outs = {k + q * p_last for q in range(rl)}
        ins = {k + r * (n // rev[0]) for r in range(rev[0])}
        assert outs == ins
    rng = np.random.default_rng(7)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    kin = np.exp(-1j * rng.standard_normal(n))
    y = stockham(stockham(x, n, fwd, ef, -1) / np.sqrt(n) * kin, n, rev, er, +1) / np.sqrt(n)
    ref = np.fft.ifft(np.fft.fft(x, norm="ortho") * kin, norm="ortho")
    assert np.allclose(y, ref, atol=1e-12 * np.sqrt(n))
