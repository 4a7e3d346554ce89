"""The tensor-core pass's A operands as the library builds them on the host
(angular_tc_images, angular_tc_parity, angular_tc_parity_images in angular_tc.cu), decoded
on the CPU with a numpy model of the K-major core-matrix layout the kernel's descriptors
read: per K chunk 8 KB of high parts then 8 KB of remainders, row group r / 8 at stride
sbo_a = (chunk_k / kc) 128 B, K core matrix kk / kc at 128 B, row r % 8 at 16 B, element
kk % kc.  A small driver linked with the library's own object files does the packing, so
what is checked is the product code.  No GPU needed.

The Legendre matrices are those of the crate's legendre_diagonalization.rs:13-80
(T[l][j] = sqrt(l + 1/2) P_l(x_j) w_j and its inverse), taken from the oracle."""
import os
import subprocess

import numpy as np
import pytest

from oracle import split_operator_oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

DRIVER = r"""
#include <cstdio>
#include <vector>
#include "common.cuh"
// in: int32 n, n*n doubles (row-major).  out: int32 kind, then for bf = 0, 1: int64 count,
// count floats of the full images, int64 count, count floats of the parity images (0 if none)
int main(int argc, char** argv) {
  if (argc != 3) return 2;
  FILE* f = std::fopen(argv[1], "rb");
  if (!f) return 3;
  int n = 0;
  if (std::fread(&n, 4, 1, f) != 1) return 4;
  std::vector<double> m((size_t)n * n);
  if (std::fread(m.data(), 8, m.size(), f) != m.size()) return 5;
  std::fclose(f);
  FILE* o = std::fopen(argv[2], "wb");
  if (!o) return 6;
  const int kind = so::angular_tc_parity(m.data(), n);
  std::fwrite(&kind, 4, 1, o);
  for (int bf = 0; bf < 3; ++bf) {  // operand modes: 3xTF32, split-BF16x3, split-BF16x6
    std::vector<float> img, par;
    so::angular_tc_images(m.data(), n, bf, img);
    if (kind) so::angular_tc_parity_images(m.data(), n, kind, bf, par);
    for (auto* v : {&img, &par}) {
      const long long c = (long long)v->size();
      std::fwrite(&c, 8, 1, o);
      std::fwrite(v->data(), 4, v->size(), o);
    }
  }
  std::fclose(o);
  return 0;
}
"""


@pytest.fixture(scope="module")
def pack(tmp_path_factory):
    from split_operator_gb300 import build
    nvcc = build.NVCC
    if not os.path.exists(nvcc):
        pytest.skip("needs nvcc")
    objs = [os.path.join(build.OUT, s + ".o") for s in build.sources()]
    if not all(os.path.exists(p) for p in objs):
        build.build()
    d = tmp_path_factory.mktemp("tcimg")
    src, exe = d / "driver.cpp", d / "driver"
    src.write_text(DRIVER)
    r = subprocess.run([nvcc, "-std=c++17", *build.ARCH, "-I", build.CSRC, str(src), *objs, "-o", str(exe),
                        "-lpthread", "-ldl", "-lrt"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    count = [0]

    def run(m):
        m = np.ascontiguousarray(m, dtype=np.float64)
        n = m.shape[0]
        count[0] += 1
        fin, fout = d / f"in{count[0]}.bin", d / f"out{count[0]}.bin"
        fin.write_bytes(np.int32(n).tobytes() + m.tobytes())
        subprocess.run([str(exe), str(fin), str(fout)], check=True)
        raw = fout.read_bytes()
        kind = int(np.frombuffer(raw, np.int32, 1, 0)[0])
        pos, res = 4, {}
        for bf in (0, 1, 2):
            for key in ("full", "par"):
                c = int(np.frombuffer(raw, np.int64, 1, pos)[0])
                pos += 8
                res[(bf, key)] = np.frombuffer(raw, np.uint8, 4 * c, pos).copy()
                pos += 4 * c
        return kind, res

    return run


def shape(n, par, bf):
    """The kernel's operand shape for lane extent n: rows, K, K per chunk, K per core row."""
    mh = 2 if n == 256 else 1
    kc = 8 if bf else 4
    chunk_k = (32 if bf else 16) // mh
    kdim = n // 2 if (par and n == 256) else n
    return 128 * mh, kdim, chunk_k, kc


def chunk_bytes(n, bf):
    """Bytes of one slice of an A chunk (every row of M, chunk_k K values): 8 KB."""
    rows, _, chunk_k, _ = shape(n, False, bf)
    return rows * chunk_k * (2 if bf else 4)


def decode(img, n, par, bf):
    """hi, lo: rows x K float64 matrices read back from the chunk images."""
    rows, kdim, chunk_k, kc = shape(n, par, bf)
    nk = kdim // chunk_k
    es = 2 if bf else 4
    CHUNK = chunk_bytes(n, bf)
    assert img.size == nk * 2 * CHUNK
    sbo = (chunk_k // kc) * 128
    r = np.arange(rows)[:, None]
    kk = np.arange(chunk_k)[None, :]
    off = (r >> 3) * sbo + (kk // kc) * 128 + (r & 7) * 16 + (kk % kc) * es
    # every byte of a chunk half is covered exactly once
    assert np.array_equal(np.sort((off[..., None] + np.arange(es)).ravel()), np.arange(CHUNK))
    hi = np.zeros((rows, kdim))
    lo = np.zeros((rows, kdim))
    for q in range(nk):
        base = q * 2 * CHUNK
        for part, dst in ((0, hi), (1, lo)):
            buf = img[base + part * CHUNK: base + (part + 1) * CHUNK]
            if bf:
                h = buf.view(np.uint16)[off // 2].astype(np.uint32) << 16
            else:
                h = buf.view(np.uint32)[off // 4]
                assert not np.any(h & 0x1FFF), "tf32 parts keep 10 mantissa bits"
            dst[:, q * chunk_k:(q + 1) * chunk_k] = h.astype(np.uint32).view(np.float32)
    return hi, lo


def legendre(n, omega=None):
    x, w = O.gauss_legendre(n)
    polar = O.Grid.new_custom("polar", np.arccos(x), w, 1)
    t, tinv = O.legendre_matrices(polar) if omega is None else O.associated_legendre_matrices(polar, omega)
    return t.real.copy(), tinv.real.copy()


@pytest.mark.parametrize("n", [32, 64, 128, 256])
@pytest.mark.parametrize("bf", [0, 1])
def test_full_images_split_the_matrix(pack, n, bf):
    rng = np.random.default_rng(n + 7 * bf)
    m = rng.standard_normal((n, n)) * np.exp(rng.uniform(-6, 6, (n, n)))
    kind, res = pack(m)
    assert kind == 0 and res[(bf, "par")].size == 0
    hi, lo = decode(res[(bf, "full")], n, False, bf)
    rows = hi.shape[0]
    assert not hi[n:].any() and not lo[n:].any(), "rows beyond n are zero padding"
    ref = np.zeros((rows, n))
    ref[:n] = m
    # the high part is the operand-format rounding of the value, the remainder that of the rest
    bits = 8 if bf else 11
    assert np.all(np.abs(hi - ref) <= np.abs(ref) * 2.0 ** -bits)
    assert np.all(np.abs(hi + lo - ref) <= np.abs(ref) * 2.0 ** (-2 * bits + 1))
    x = rng.standard_normal(n)
    y = (hi + lo)[:n] @ x
    tol = 2e-6 if bf else 1e-7
    assert np.linalg.norm(y - m @ x) <= tol * np.linalg.norm(np.abs(m) @ np.abs(x))


@pytest.mark.parametrize("n", [32, 128, 256])
def test_parity_kinds(pack, n):
    t, tinv = legendre(n)
    assert pack(t)[0] == (1 if n == 256 else 0)
    assert pack(tinv)[0] == (2 if n == 256 else 0)
    if n == 256:
        # associated Legendre: the sign of P_l^m(-x) is (-1)^(l+m), so even m keeps the structure
        ta, tai = legendre(n, 2)
        assert pack(ta)[0] == 1 and pack(tai)[0] == 2
        to, toi = legendre(n, 1)
        assert pack(to)[0] == 0 and pack(toi)[0] == 0
        # a perturbation above the detection tolerance (1e-12 of the largest entry) breaks it
        tp = t.copy()
        tp[3, 5] += 1e-9 * np.abs(t).max()
        assert pack(tp)[0] == 0


@pytest.mark.parametrize("bf", [0, 1])
@pytest.mark.parametrize("which", ["forward", "inverse", "forward_m2"])
def test_parity_images_reproduce_the_product(pack, bf, which):
    n, hn = 256, 128
    t, tinv = legendre(n, 2 if which == "forward_m2" else None)
    m = tinv if which == "inverse" else t
    kind, res = pack(m)
    assert kind == (2 if which == "inverse" else 1)
    hi, lo = decode(res[(bf, "par")], n, True, bf)
    a = hi + lo
    assert a.shape == (n, hn)
    rng = np.random.default_rng(11 + bf)
    x = rng.standard_normal(n)
    y = np.empty(n)
    if kind == 1:
        # rows 0..127: even l, rows 128..255: odd l; K runs over the first half of the nodes
        s, dlt = x[:hn] + x[::-1][:hn], x[:hn] - x[::-1][:hn]
        y[0::2] = a[:hn] @ s
        y[1::2] = a[hn:] @ dlt
    else:
        # rows 0..127: E (even l), rows 128..255: O (odd l); K runs over l of one parity
        e, o = a[:hn] @ x[0::2], a[hn:] @ x[1::2]
        y[:hn] = e + o
        y[::-1][:hn] = e - o
    ref = m @ x
    tol = 2e-6 if bf else 1e-7
    assert np.linalg.norm(y - ref) <= tol * np.linalg.norm(np.abs(m) @ np.abs(x))
    # the split operands are the structured halves of the matrix itself, exactly
    h_full = decode(res[(bf, "full")], n, False, bf)[0]
    if kind == 1:
        assert np.array_equal(hi[:hn], h_full[0::2, :hn]) and np.array_equal(hi[hn:], h_full[1::2, :hn])
    else:
        assert np.array_equal(hi[:hn], h_full[:hn, 0::2]) and np.array_equal(hi[hn:], h_full[:hn, 1::2])


def decode_oz(img, n, par):
    """Split-BF16x6 images: per K chunk three bf16 slice images, same core-matrix order."""
    rows, kdim, chunk_k, kc = shape(n, par, True)
    nk = kdim // chunk_k
    CHUNK = chunk_bytes(n, True)
    assert img.size == nk * 3 * CHUNK
    sbo = (chunk_k // kc) * 128
    r = np.arange(rows)[:, None]
    kk = np.arange(chunk_k)[None, :]
    off = (r >> 3) * sbo + (kk // kc) * 128 + (r & 7) * 16 + (kk % kc) * 2
    sl = np.zeros((3, rows, kdim))
    for q in range(nk):
        for part in range(3):
            buf = img[(q * 3 + part) * CHUNK:(q * 3 + part + 1) * CHUNK]
            h = buf.view(np.uint16)[off // 2].astype(np.uint32) << 16
            sl[part, :, q * chunk_k:(q + 1) * chunk_k] = h.view(np.float32)
    return sl


@pytest.mark.parametrize("n", [32, 64, 128, 256])
def test_split_bf16x6_images_are_fixed_point_slices(pack, n):
    """Each row of the A operand as three bf16 slices on the fixed-point grid of that row:
    slice i a multiple of q_i = 2^(e - 8 - 8 i) (2^e just above the row's largest magnitude)
    with |s_i / q_i| <= 256, and s0 + s1 + s2 within 2^-24 2^e of the value -- the form whose
    products the tensor core sums exactly."""
    rng = np.random.default_rng(3 * n)
    m = rng.standard_normal((n, n)) * np.exp(rng.uniform(-6, 6, (n, 1))) * np.exp(rng.uniform(-2, 2, (n, n)))
    _, res = pack(m)
    sl = decode_oz(res[(2, "full")], n, False)
    rows = sl.shape[1]
    assert not sl[:, n:].any(), "rows beyond n are zero padding"
    e = np.ceil(np.log2(np.abs(m).max(axis=1)))
    e = np.where(np.abs(m).max(axis=1) >= 2.0 ** e, e + 1, e)  # 2^e strictly above the maximum
    for i in range(3):
        q = 2.0 ** (e - 8 - 8 * i)
        k = sl[i, :n] / q[:, None]
        assert np.array_equal(k, np.round(k)), i
        assert np.abs(k).max() <= 256
    assert np.all(np.abs(sl[:, :n].sum(axis=0) - m) <= 2.0 ** (e - 24)[:, None])


def test_split_bf16x6_block_diagonal_images(pack):
    """Packed tiles of lane extent 32: four copies of the 32 x 32 matrix on the diagonal of a
    128 x 128 one, each row with its own quanta, zero off the diagonal blocks."""
    t, _ = legendre(32)
    bd = np.zeros((128, 128))
    for b in range(4):
        bd[32 * b:32 * b + 32, 32 * b:32 * b + 32] = t
    _, res = pack(bd)
    sl = decode_oz(res[(2, "full")], 128, False)
    a = sl.sum(axis=0)
    mask = np.kron(np.eye(4), np.ones((32, 32))).astype(bool)
    assert not a[~mask].any()
    assert np.abs(a - bd).max() <= 2.0 ** -23 * np.abs(t).max()
    for b in range(4):
        np.testing.assert_array_equal(sl[:, 32 * b:32 * b + 32, 32 * b:32 * b + 32], sl[:, :32, :32])
