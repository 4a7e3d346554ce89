"""Tensor-core (tcgen05) lane-matrix pass against FP64 references: 3xTF32, split-BF16x3 and
split-BF16x6 (three fixed-point bf16 slices per operand, exact FP32 sums)."""
import numpy as np
import pytest

from oracle import scenarios as S
from tests.gpu_common import ensure_built, rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def so():
    ensure_built()
    import split_operator_gb300 as so
    return so


@pytest.mark.parametrize("n,nr", [(128, 256), (64, 128), (32, 64), (128, 4096), (256, 256), (256, 1024)])
def test_real_lane_matrix_3xtf32_matches_fp64(so, n, nr):
    rng = np.random.default_rng(n + nr)
    psi = rng.standard_normal((nr, n)) + 1j * rng.standard_normal((nr, n))
    t = rng.standard_normal((n, n)) / np.sqrt(n)
    g0 = so.Grid.new_linear_continuos("r", 0.0, 1.0, nr, 0)
    g1 = so.Grid.new_linear_countable("th", 0.0, 1.0, n, 1)
    wf = so.WaveFunction(psi, [g0, g1])
    mt = so.MatrixTransformation(g1, so.Grid.new_linear_countable("l", 0.0, 1.0, n, 1))
    mt.set_diagonalization_matrix(t.astype(np.complex128), np.eye(n, dtype=np.complex128))
    st = so.OperationStack()
    st.add_transformation(mt, so.NORMAL)
    prop = so.Propagation(wf, so.TimeGrid(1.0, 3), st, "fp32_tf32x3")
    prop.steps(1)
    ref = psi @ t.T  # lane <- T lane along axis 1
    err = rel_l2(prop.get_array(), ref)
    # FP32 state in and out plus FP32 accumulation over K terms: ~sqrt(K) * 6e-8
    assert err < 2e-6, err
    prop.steps(1)
    err2 = rel_l2(prop.get_array(), ref @ t.T)
    assert err2 < 4e-6, err2


@pytest.mark.parametrize("precision", ["fp32_tf32x3", "fp32_simt", "fp32_bf16x6"])
@pytest.mark.parametrize("n", [128, 64, 256])
def test_two_lane_matrices_in_one_pass(so, precision, n):
    """Stack [T-transformation, diagonal D]: a step is T, D, T2 (the inverse slot holds T2),
    so the pass carries two matrix products with a table multiply between them."""
    nr = 256
    rng = np.random.default_rng(n)
    t1 = rng.standard_normal((n, n)) / np.sqrt(n)
    t2 = rng.standard_normal((n, n)) / np.sqrt(n)
    d = np.exp(1j * rng.uniform(0, 6.28, (nr, n)))
    psi = rng.standard_normal((nr, n)) + 1j * rng.standard_normal((nr, n))
    g0 = so.Grid.new_linear_countable("r", 0.0, float(nr - 1), nr, 0)
    g1 = so.Grid.new_linear_countable("th", 0.0, float(n - 1), n, 1)
    wf = so.WaveFunction(psi, [g0, g1])
    mt = so.MatrixTransformation(g1, so.Grid.new_linear_countable("l", 0.0, float(n - 1), n, 1))
    mt.set_diagonalization_matrix(t1.astype(np.complex128), t2.astype(np.complex128))
    dp = so.NDimPropagator()
    dp.set_operator(d)
    st = so.OperationStack()
    st.add_transformation(mt, so.NORMAL)
    st.add_propagator(dp)
    prop = so.Propagation(wf, so.TimeGrid(1.0, 10), st, precision)
    ref = psi.copy()
    for k in range(3):
        prop.steps(1)
        ref = ((d * (ref @ t1.T)) @ t2.T)
        err = rel_l2(prop.get_array(), ref)
        assert err < 5e-6, (k, err)
    prop.steps(3)  # passes merge across step boundaries: T2 then T in one pass
    for _ in range(3):
        ref = ((d * (ref @ t1.T)) @ t2.T)
    err = rel_l2(prop.get_array(), ref)
    assert err < 1e-5, err


@pytest.mark.parametrize("precision", ["fp32_tf32x3", "fp32_simt", "fp32_bf16x6"])
def test_orthogonal_lane_matrix_keeps_the_norm(so, precision):
    """200 applications of an orthogonal matrix: the norm may random-walk at the FP32
    level but must not drift systematically (a biased split would shrink it).  The
    split-BF16x6 sums are exact on the tensor core, so it keeps the norm like the FP32
    CUDA-core product does."""
    n, nr = 128, 512
    rng = np.random.default_rng(7)
    q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    psi = rng.standard_normal((nr, n)) + 1j * rng.standard_normal((nr, n))
    psi /= np.linalg.norm(psi)
    g0 = so.Grid.new_linear_countable("r", 0.0, float(nr - 1), nr, 0)
    g1 = so.Grid.new_linear_countable("th", 0.0, float(n - 1), n, 1)
    wf = so.WaveFunction(psi, [g0, g1])
    mt = so.MatrixTransformation(g1, so.Grid.new_linear_countable("l", 0.0, float(n - 1), n, 1))
    mt.set_diagonalization_matrix(q.astype(np.complex128), q.T.astype(np.complex128))
    st = so.OperationStack()
    st.add_transformation(mt, so.NORMAL)
    prop = so.Propagation(wf, so.TimeGrid(1.0, 200), st, precision)
    prop.steps(200)
    a = prop.get_array()
    drift = abs(np.linalg.norm(a) ** 2 - 1.0)
    # measured on GB300: SIMT ~1e-7, 3xTF32 ~2.4e-5 (tensor-core accumulation truncates;
    # the pass spreads the products over several accumulators, one accumulator gave 3.3e-4)
    assert drift < (4e-5 if precision == "fp32_tf32x3" else 2e-6), drift
    if precision == "fp32_bf16x6":
        # and the matrix products themselves: 200 applications of q against FP64
        ref = psi.copy()
        for _ in range(200):
            ref = ref @ q.T
        assert rel_l2(a, ref) < 2e-5


def test_tensor_core_pass_is_used(so):
    from split_operator_gb300 import workloads as W
    prop, _ = W.radial_angular_2d(nr=256, nth=32, step_no=4, r0=25.0, precision="fp32_tf32x3")
    prop.set_timing(True)
    prop.steps(3)
    names = [k for k, *_ in prop.kernel_times()]
    assert any("tc3xtf32" in k for k in names), names


@pytest.mark.parametrize("precision", ["fp32_tf32x3", "fp32_bf16x6"])
@pytest.mark.parametrize("nr,nth", [(256, 32), (512, 64), (1024, 128), (512, 256)])
def test_radial_angular_tf32x3_close_to_oracle(so, nr, nth, precision):
    from split_operator_gb300 import workloads as W
    steps = 20
    prop, h = W.radial_angular_2d(nr=nr, nth=nth, step_no=steps, r0=25.0, precision=precision)
    oprop, odamp = S.radial_angular_2d(nr=nr, nth=nth, step_no=steps, r0=25.0)
    prop.steps(1)
    oprop.step()
    e1 = rel_l2(prop.get_array(), oprop.wave_function.array)
    assert e1 < 3e-6, e1
    prop.steps(steps - 1)
    oprop.propagate(steps - 1)
    e = rel_l2(prop.get_array(), oprop.wave_function.array)
    assert e < 6e-5, e
    # FP32 state: ~2.7e-7 norm drift per step from FP32-rounded phase tables, plus the
    # tensor-core accumulation bias (larger at n = 256, where 3 accumulators share 32 K steps)
    assert abs(prop.norm() - oprop.wave_function.norm()) < (6e-5 if nth == 256 else 2.5e-5)


@pytest.mark.parametrize("precision,tol", [("fp32_bf16x6", 1e-6), ("fp32_tf32x3", 1e-6), ("fp32_bf16x3", 2e-5)])
def test_full_step_at_4096x128_matches_oracle(so, precision, tol):
    """The whole 2-D step at 4096 x 128 (Morse + P2, Legendre pair on the tensor cores, the
    fixed-shape radial FFT pair, border damping with a loss checker) in each tensor-core
    mode, step by step against the FP64 oracle (propagation.rs:134-190)."""
    from split_operator_gb300 import workloads as W
    steps = 3
    prop, _ = W.radial_angular_2d(nr=4096, nth=128, step_no=steps, seed=2026, precision=precision)
    oprop, _ = S.radial_angular_2d(nr=4096, nth=128, step_no=steps, seed=2026)
    prop.set_timing(True)
    for k in range(steps):
        prop.steps(1)
        oprop.step()
        assert rel_l2(prop.get_array(), oprop.wave_function.array) < tol * (k + 1), k
    assert abs(prop.all_losses()[0] - oprop.all_losses()[0][1]) < tol
    names = " ".join(t[0] for t in prop.kernel_times())
    tag = {"fp32_bf16x6": "tcbf16x6", "fp32_tf32x3": "tc3xtf32", "fp32_bf16x3": "tcbf16x3"}[precision]
    assert tag in names and "fftpair" in names, names


@pytest.mark.parametrize("precision", ["fp32_tf32x3", "fp32_bf16x6"])
def test_parity_split_legendre_pair_matches_plain_form(so, monkeypatch, precision):
    """n = 256 Legendre pair: the parity-split GEMMs (two K = 128 halves) give the same
    propagation as the plain 256 x 256 form, both within FP32 accuracy of FP64."""
    from split_operator_gb300 import workloads as W
    out = {}
    for flag in ("1", "0"):
        monkeypatch.setenv("SO_TC_PARITY", flag)
        prop, _ = W.radial_angular_2d(nr=512, nth=256, step_no=10 ** 6, precision=precision)
        prop.set_timing(True)
        prop.steps(6)
        names = [t[0] for t in prop.kernel_times()]
        assert any("parity" in nm for nm in names) == (flag == "1"), names
        out[flag] = prop.get_array()
    ref, _ = W.radial_angular_2d(nr=512, nth=256, step_no=10 ** 6, precision="fp64")
    ref.steps(6)
    r = ref.get_array()
    e_split, e_plain = rel_l2(out["1"], r), rel_l2(out["0"], r)
    # FP32 state: about 3e-7 per step against FP64
    assert e_split < 1e-5 and e_plain < 1e-5, (e_split, e_plain)
    assert rel_l2(out["1"], out["0"]) < 1e-5


@pytest.mark.parametrize("n,nr", [(128, 256), (32, 64), (256, 256)])
def test_real_lane_matrix_split_bf16x3(so, n, nr):
    """Split-BF16x3 tensor-core form (x = bf16(x) + bf16(remainder), three products, FP32
    accumulation): about 16 significant bits, so a few 1e-6 per product."""
    rng = np.random.default_rng(7 * n + nr)
    psi = rng.standard_normal((nr, n)) + 1j * rng.standard_normal((nr, n))
    t = rng.standard_normal((n, n)) / np.sqrt(n)
    g0 = so.Grid.new_linear_continuos("r", 0.0, 1.0, nr, 0)
    g1 = so.Grid.new_linear_countable("th", 0.0, 1.0, n, 1)
    wf = so.WaveFunction(psi, [g0, g1])
    mt = so.MatrixTransformation(g1, so.Grid.new_linear_countable("l", 0.0, 1.0, n, 1))
    mt.set_diagonalization_matrix(t.astype(np.complex128), np.eye(n, dtype=np.complex128))
    st = so.OperationStack()
    st.add_transformation(mt, so.NORMAL)
    prop = so.Propagation(wf, so.TimeGrid(1.0, 3), st, "fp32_bf16x3")
    prop.set_timing(True)
    prop.steps(1)
    assert any("tcbf16x3" in k[0] for k in prop.kernel_times())
    err = rel_l2(prop.get_array(), psi @ t.T)
    assert err < 3e-5, err


@pytest.mark.parametrize("n,nr", [(128, 256), (64, 128), (32, 64), (128, 4096), (256, 256), (256, 1024)])
def test_real_lane_matrix_split_bf16x6(so, n, nr):
    """Split-BF16x6: each operand as three fixed-point bf16 slices (8 significant bits each,
    one quantum per matrix row and per state column), six slice products accumulated exactly
    by the tensor core.  What remains is the FP32 state in and out, the 2^-24 slicing
    remainder and the final round-to-nearest: about 1e-7, several times below 3xTF32."""
    rng = np.random.default_rng(11 * n + nr)
    psi = rng.standard_normal((nr, n)) + 1j * rng.standard_normal((nr, n))
    # rows and columns of very different magnitudes: every row and column gets its own quantum
    psi *= np.exp(rng.uniform(-8, 8, nr))[:, None]
    t = rng.standard_normal((n, n)) / np.sqrt(n) * np.exp(rng.uniform(-4, 4, n))[:, None]
    g0 = so.Grid.new_linear_continuos("r", 0.0, 1.0, nr, 0)
    g1 = so.Grid.new_linear_countable("th", 0.0, 1.0, n, 1)
    wf = so.WaveFunction(psi, [g0, g1])
    mt = so.MatrixTransformation(g1, so.Grid.new_linear_countable("l", 0.0, 1.0, n, 1))
    mt.set_diagonalization_matrix(t.astype(np.complex128), np.eye(n, dtype=np.complex128))
    st = so.OperationStack()
    st.add_transformation(mt, so.NORMAL)
    prop = so.Propagation(wf, so.TimeGrid(1.0, 3), st, "fp32_bf16x6")
    prop.set_timing(True)
    prop.steps(1)
    assert any("tcbf16x6" in k[0] for k in prop.kernel_times())
    ref = psi @ t.T
    got = prop.get_array()
    # per output element: within a few FP32 rounding units of its row of |T| |psi|
    bound = (np.abs(psi) @ np.abs(t).T)
    assert np.max(np.abs(got - ref) / bound) < 6e-7, np.max(np.abs(got - ref) / bound)
    assert rel_l2(got, ref) < 5e-7


@pytest.mark.parametrize("nr,nth", [(512, 32), (1024, 64)])
def test_packed_short_lanes_match_the_oracle(so, nr, nth):
    """Split-BF16x6 with lanes of 32 or 64 points runs packed tiles: 128 / n column groups
    share one 128-row tensor-core tile through a block-diagonal lane matrix.  Against the FP64
    oracle step by step, and the packed pass is the one that ran."""
    from split_operator_gb300 import workloads as W
    steps = 6
    prop, _ = W.radial_angular_2d(nr=nr, nth=nth, step_no=steps, seed=13, r0=25.0, precision="fp32_bf16x6")
    oprop, _ = S.radial_angular_2d(nr=nr, nth=nth, step_no=steps, seed=13, r0=25.0)
    prop.set_timing(True)
    for k in range(steps):
        prop.steps(1)
        oprop.step()
        assert rel_l2(prop.get_array(), oprop.wave_function.array) < 1e-6 * (k + 1), k
    names = " ".join(t[0] for t in prop.kernel_times())
    assert "tcbf16x6 packed" in names, names
    assert abs(prop.all_losses()[0] - oprop.all_losses()[0][1]) < 1e-7
