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


def _entry():
    from split_operator_gb300 import _lib

    h = _lib.lib()
    f = h.so_fft_norm_noalloc
    f.argtypes = [C.c_void_p, C.c_size_t, C.c_size_t, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    return h, f


# power-of-two lanes (Stockham stages), a non-power-of-two lane (direct DFT), lanes shorter
# than 16 points, a ragged last tile (300 lanes), and one lane of the 4096-point maximum
@pytest.mark.parametrize("lanes,n", [(64, 1024), (300, 256), (7, 4096), (96, 300), (50, 8)])
def test_fft_norm_noalloc_matches_regular_path(lanes, n):
    ensure_built()
    import torch

    import split_operator_gb300 as so

    h, f = _entry()
    rng = np.random.default_rng(lanes * n)
    psi = rng.standard_normal((lanes, n)) + 1j * rng.standard_normal((lanes, n))
    ref = _regular_path(so, psi, [-1, +1])

    # every device buffer is the caller's, allocated up front (as such a caller would)
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    buf = torch.from_numpy(psi.view(np.float64).copy()).to(dev)
    norm = torch.zeros(1, dtype=torch.float64, device=dev)
    w = [(torch.from_numpy(np.ascontiguousarray(r[3])).to(dev), torch.from_numpy(np.ascontiguousarray(r[2])).to(dev))
         for r in ref]
    torch.cuda.synchronize()
    for call, d in enumerate([-1, +1]):
        arr, nrm = ref[call][0], ref[call][1]
        w_l, w_x = w[call]
        st = f(buf.data_ptr(), lanes, n, d, w_l.data_ptr(), w_x.data_ptr(), norm.data_ptr(), stream.cuda_stream)
        assert st == 0, h.so_last_error().decode()
        torch.cuda.synchronize()
        got = buf.cpu().numpy().view(np.complex128).reshape(lanes, n)
        err = np.linalg.norm(got - arr) / np.linalg.norm(arr)
        assert err < 1e-13, (call, err)
        assert abs(norm.item() - nrm) <= 1e-13 * abs(nrm), (call, norm.item(), nrm)

    # the same two calls again: the device's free memory does not move (nothing is allocated;
    # the first pair above has loaded the kernels)
    buf.copy_(torch.from_numpy(psi.view(np.float64).copy()).to(dev))
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info(dev)[0]
    for call, d in enumerate([-1, +1]):
        w_l, w_x = w[call]
        assert f(buf.data_ptr(), lanes, n, d, w_l.data_ptr(), w_x.data_ptr(), norm.data_ptr(),
                 stream.cuda_stream) == 0
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info(dev)[0] == free0
    got = buf.cpu().numpy().view(np.complex128).reshape(lanes, n)
    assert np.linalg.norm(got - ref[1][0]) / np.linalg.norm(ref[1][0]) < 1e-13


def test_fft_norm_noalloc_without_norm():
    """FFT only (weights, lane_weights and norm_out all NULL), forward then inverse."""
    ensure_built()
    import torch

    import split_operator_gb300 as so

    h, f = _entry()
    lanes, n = 33, 512
    rng = np.random.default_rng(5)
    psi = rng.standard_normal((lanes, n)) + 1j * rng.standard_normal((lanes, n))
    ref = _regular_path(so, psi, [-1, +1])
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    buf = torch.from_numpy(psi.view(np.float64).copy()).to(dev)
    for call, d in enumerate([-1, +1]):
        st = f(buf.data_ptr(), lanes, n, d, None, None, None, stream.cuda_stream)
        assert st == 0, h.so_last_error().decode()
        torch.cuda.synchronize()
        got = buf.cpu().numpy().view(np.complex128).reshape(lanes, n)
        arr = ref[call][0]
        assert np.linalg.norm(got - arr) / np.linalg.norm(arr) < 1e-13, call


def test_fft_norm_noalloc_rejects_oversize():
    ensure_built()
    h, f = _entry()
    # a lane of 8192 points is beyond the fixed twiddle table: rejected before any GPU work
    st = f(C.c_void_p(16), 1, 8192, -1, None, None, None, None)
    assert st == 4
    assert b"4096" in h.so_last_error()
