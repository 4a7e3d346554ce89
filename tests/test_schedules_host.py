"""The launch schedule table the autotuner fills (schedule.cpp), through the C ABI on the host:
save / load round trip of the JSON cache, reset, and refusal of a file in another format.
No GPU: the table is host state."""
import json

import pytest


@pytest.fixture(scope="module")
def so():
    from tests.gpu_common import ensure_built
    ensure_built()
    import split_operator_gb300 as so
    return so


def test_schedule_cache_round_trip(so, tmp_path):
    so.reset_schedules()
    empty = tmp_path / "empty.json"
    so.save_schedules(str(empty))
    assert json.loads(empty.read_text()) == {"fft_pair": [], "tensor_core": []}
    cache = {"fft_pair": [{"n": 4096, "fp64": 0, "threads": 512, "radix": 8},
                          {"n": 512, "fp64": 0, "threads": 128, "radix": 16}],
             "tensor_core": [{"n": 128, "mode": 2, "ctas_per_sm": 1, "blocked": 1}]}
    src = tmp_path / "in.json"
    src.write_text(json.dumps(cache))
    so.load_schedules(str(src))
    out = tmp_path / "out.json"
    so.save_schedules(str(out))
    got = json.loads(out.read_text())
    key = lambda d: sorted(json.dumps(x, sort_keys=True) for x in d)  # noqa: E731
    assert key(got["fft_pair"]) == key(cache["fft_pair"])
    assert key(got["tensor_core"]) == key(cache["tensor_core"])
    so.reset_schedules()
    so.save_schedules(str(out))
    assert json.loads(out.read_text()) == {"fft_pair": [], "tensor_core": []}


def test_schedule_cache_in_another_format_is_refused(so, tmp_path):
    bad = tmp_path / "bad.json"
    bad.write_text('{"fft_pair": [{"n": 4096, "threads": 512}]}')  # radix and fp64 missing
    with pytest.raises(so.SplitOperatorError):
        so.load_schedules(str(bad))
    with pytest.raises(so.SplitOperatorError):
        so.load_schedules(str(tmp_path / "missing.json"))
