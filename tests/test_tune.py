"""Autotuner host logic (no GPU): the knobs of the C ABI and the on-disk cache.

The knobs are process-wide launch shapes; the cache maps a GPU name (and the
library version it was measured with) to the fastest value of each.  GPU tests
of the tuned shapes are in tests/test_gpu_tune.py."""
import json

import pytest

from gpurir_gb300 import _lib, tune


@pytest.fixture
def lib(built_lib):
    yield built_lib
    tune.reset()


@pytest.fixture(scope="module")
def built_lib():
    from gpurir_gb300 import _build
    _build.build()
    return _lib.load()


def test_knobs_default_and_ranges(lib):
    tune.reset()
    assert tune.get_knobs() == {"conv_rows": 2, "ism_blocks_per_sm": 0, "adjoint_blocks_per_sm": 0,
                                "traj_adjoint_blocks_per_sm": 0}
    tune.set_knobs({"conv_rows": 1, "adjoint_blocks_per_sm": 2})
    assert tune.get_knobs()["conv_rows"] == 1 and tune.get_knobs()["adjoint_blocks_per_sm"] == 2
    assert lib.gpurir_set_tuning(b"conv_rows", 3) == -1
    assert b"range" in lib.gpurir_last_error()
    assert lib.gpurir_set_tuning(b"no_such_knob", 1) == -1
    with pytest.raises(_lib.GpuRirError):
        tune.set_knobs({"ism_blocks_per_sm": -1})


def test_cache_roundtrip_applies_matching_entry(lib, tmp_path):
    path = str(tmp_path / "tuning.json")
    tune.save_entry("FAKE GPU (sm_103, 152 SMs)", {"knobs": {"conv_rows": 1, "ism_blocks_per_sm": 1},
                                                  "library": tune.library_version()}, path)
    tune.save_entry("OTHER GPU", {"knobs": {"conv_rows": 2}, "library": tune.library_version()}, path)
    tune.reset()
    assert tune.apply_cached("FAKE GPU (sm_103, 152 SMs)", path) == {"conv_rows": 1, "ism_blocks_per_sm": 1}
    assert tune.get_knobs()["conv_rows"] == 1 and tune.get_knobs()["ism_blocks_per_sm"] == 1
    with open(path) as f:
        assert set(json.load(f)["devices"]) == {"FAKE GPU (sm_103, 152 SMs)", "OTHER GPU"}


def test_cache_ignores_other_gpus_versions_and_bad_values(lib, tmp_path):
    path = str(tmp_path / "tuning.json")
    tune.save_entry("A", {"knobs": {"conv_rows": 1}, "library": "some older build"}, path)
    tune.save_entry("B", {"knobs": {"conv_rows": 7, "adjoint_blocks_per_sm": 1},
                          "library": tune.library_version()}, path)
    tune.reset()
    assert tune.apply_cached("A", path) is None           # measured with another library build
    assert tune.apply_cached("missing", path) is None
    assert tune.apply_cached("B", path) == {"adjoint_blocks_per_sm": 1}   # out-of-range value dropped
    assert tune.get_knobs()["conv_rows"] == 2
    (tmp_path / "bad.json").write_text("{not json")
    assert tune.apply_cached("B", str(tmp_path / "bad.json")) is None
