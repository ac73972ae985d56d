"""Launch knobs (nfem_knob_set / nfem_knob_get, host-only calls) and the
autotuner's cache file, without a GPU."""
import json

import pytest

from nfempy_gb300 import _lib, autotune


@pytest.fixture()
def lib():
    try:
        return _lib.lib()
    except _lib.NfemError:
        pytest.skip("library not built")


def test_knobs_validate_and_round_trip(lib):
    v = _lib.C.c_int(-1)
    assert lib.nfem_knob_set(0, 6) == 0
    assert lib.nfem_knob_get(0, _lib.C.byref(v)) == 0 and v.value == 6
    assert lib.nfem_knob_set(1, 300) == 1  # not a supported block size
    assert lib.nfem_knob_set(2, 3) == 1    # 2, 4 or 8 warps
    assert lib.nfem_knob_set(99, 1) == 1
    assert lib.nfem_knob_get(99, _lib.C.byref(v)) == 1
    autotune.reset_knobs()
    for k in range(3):
        assert lib.nfem_knob_get(k, _lib.C.byref(v)) == 0 and v.value == 0


def test_cache_applies_stored_choice(lib, tmp_path, monkeypatch):
    path = tmp_path / "tuning.json"
    monkeypatch.setenv("NFEM_TUNING_CACHE", str(path))
    cfg = {"form": {"use_records": True}, "knobs": {"darcy_rows_blocks_per_sm": 8, "darcy_cells_block": 128}}
    path.write_text(json.dumps({autotune.gpu_name(): {"w": {"config": cfg, "ms": 1.0, "candidates": 3}}}))

    class Form:
        use_records = None

    f = Form()
    assert autotune.apply_cached("w", f)["ms"] == 1.0
    assert f.use_records is True
    v = _lib.C.c_int()
    lib.nfem_knob_get(0, _lib.C.byref(v))
    assert v.value == 8
    lib.nfem_knob_get(1, _lib.C.byref(v))
    assert v.value == 128
    assert autotune.apply_cached("missing", f) is None
    autotune.reset_knobs()
