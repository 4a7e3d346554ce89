"""The allocation-free FFT + norm entry point (so_fft_norm_noalloc) against the
library's regular path (FFTTransformation on a WaveFunction + WaveFunction::norm).

Callers such as code inside a strict memory pool, or frameworks that only hand
over pre-sized device buffers, cannot let the library cudaMalloc its scratch;
this entry point uses fixed-size file-scope device arrays instead.  The test
owns all device buffers (allocated here through PyTorch, as such a caller
would) and calls the entry point twice in a row.
"""
import ctypes as C

import numpy as np
import pytest

from tests.gpu_common import ensure_built

pytestmark = pytest.mark.gpu


def _regular_path(so, psi, direction_sequence):
    lanes, n = psi.shape
    g_l = so.Grid.new_linear_countable("lane", 0.0, float(lanes - 1), lanes, 0)
    g_x = so.Grid.new_linear_continuos("x", -5.0, 5.0, n, 1)
    wf = so.WaveFunction(psi, [g_l, g_x])
    fft = so.FFTTransformation(g_x, "k")
    out = []
    for d in direction_sequence:
        (fft.transform if d < 0 else fft.inverse_transform)(wf)
        out.append((wf.array, wf.norm(), wf.grid(1).weights, wf.grid(0).weights))
    return out


@pytest.mark.parametrize("lanes,n", [(64, 1024), (300, 256), (7, 4096)])
def test_fft_norm_noalloc_matches_regular_path(lanes, n):
    ensure_built()
    import torch

    import split_operator_gb300 as so
    from split_operator_gb300 import _lib

    h = _lib.lib()
    f = h.so_fft_norm_noalloc
    f.argtypes = [C.c_void_p, C.c_size_t, C.c_size_t, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    f.restype = C.c_int

    rng = np.random.default_rng(lanes * n)
    psi = rng.standard_normal((lanes, n)) + 1j * rng.standard_normal((lanes, n))
    ref = _regular_path(so, psi, [-1, +1])

    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    buf = torch.from_numpy(psi.view(np.float64).copy()).to(dev)
    norm = torch.zeros(1, dtype=torch.float64, device=dev)
    for call, d in enumerate([-1, +1]):
        arr, nrm, wx, wl = ref[call]
        w_x = torch.from_numpy(np.ascontiguousarray(wx)).to(dev)
        w_l = torch.from_numpy(np.ascontiguousarray(wl)).to(dev)
        st = f(buf.data_ptr(), lanes, n, d, w_l.data_ptr(), w_x.data_ptr(), norm.data_ptr(), stream.cuda_stream)
        assert st == 0, h.so_last_error().decode()
        torch.cuda.synchronize()
        got = buf.cpu().numpy().view(np.complex128).reshape(lanes, n)
        err = np.linalg.norm(got - arr) / np.linalg.norm(arr)
        assert err < 1e-13, (call, err)
        assert abs(norm.item() - nrm) <= 1e-13 * abs(nrm), (call, norm.item(), nrm)


def test_fft_norm_noalloc_rejects_oversize():
    ensure_built()
    from split_operator_gb300 import _lib

    h = _lib.lib()
    f = h.so_fft_norm_noalloc
    f.argtypes = [C.c_void_p, C.c_size_t, C.c_size_t, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    # a lane of 8192 points is beyond the fixed twiddle table: rejected before any GPU work
    st = f(C.c_void_p(16), 1, 8192, -1, None, None, None, None)
    assert st == 4
    assert b"4096" in h.so_last_error()
