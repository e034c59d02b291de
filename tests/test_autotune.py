"""The run-time launch tuner (cmtj_gb300.autotune) on the CPU: candidate
log tiles, table keys and the persisted table."""
import json

import pytest

from cmtj_gb300 import autotune


def test_tile_candidates_fit_shared_memory_and_chunks():
    assert autotune.tile_candidates(0, 10, None) == [0]
    c = autotune.tile_candidates(1, 10, None)
    assert c == [4, 8, 12, 16, 24, 32, 48, 64, 96]
    assert all(t * 6 <= 96 for t in autotune.tile_candidates(6, 1, None))
    # a chunk of 400 steps at one sample per 10 steps holds tiles of 4, 8
    assert autotune.tile_candidates(1, 10, 400) == [4, 8]


def test_keys_name_the_kind_of_launch():
    k = autotune.f32_key(2, 1, (5 << 24) | 64 | (1 << 16), 1, False, 262144)
    assert k == "f32|L2|s1|v10040|c1|w0|n18"  # the bound bits are not part of the key
    assert autotune.f64_key(2, 1, 64) == "f64|G2|s1|n6"
    assert autotune.size_class(1) == 0 and autotune.size_class(1023) == 9


def test_table_persists_per_device(tmp_path, monkeypatch):
    monkeypatch.setattr(autotune, "PATH", str(tmp_path / "autotune.json"))
    monkeypatch.setattr(autotune, "_table", None)
    monkeypatch.setattr(autotune, "_prefix", "GPU-X|1")
    autotune.store("f32|L1|s0|v50|c0|w0|n10", {"bound": 2, "tile": 0})
    data = json.load(open(tmp_path / "autotune.json"))
    assert data["GPU-X|1"]["f32|L1|s0|v50|c0|w0|n10"]["bound"] == 2
    monkeypatch.setattr(autotune, "_table", None)
    assert autotune.lookup("f32|L1|s0|v50|c0|w0|n10") == {"bound": 2, "tile": 0}
    monkeypatch.setattr(autotune, "_table", None)
    monkeypatch.setattr(autotune, "_prefix", "GPU-Y|1")
    assert autotune.lookup("f32|L1|s0|v50|c0|w0|n10") is None


def test_off_switch(monkeypatch):
    monkeypatch.setenv("CMTJ_AUTOTUNE", "0")
    assert not autotune.enabled()
    monkeypatch.setenv("CMTJ_AUTOTUNE", "1")
    assert autotune.enabled()
