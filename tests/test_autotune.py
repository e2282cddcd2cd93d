"""Team-width autotuner of the split kernel (pyscaledvecchia_gb300/autotune.py):
the choice rule, the on-disk cache and the switch, with a stand-in for the
GPU measurement (CPU); one real measurement on the GPU."""
import json

import pytest

from pyscaledvecchia_gb300 import autotune


@pytest.fixture()
def fresh(monkeypatch, tmp_path):
    path = tmp_path / "team_lanes.json"
    monkeypatch.setenv("SV_AUTOTUNE_CACHE", str(path))
    monkeypatch.delenv("SV_AUTOTUNE", raising=False)
    monkeypatch.setattr(autotune, "_mem", {})
    monkeypatch.setattr(autotune, "_file_loaded", False)
    return path


def test_choose_keeps_the_default_within_the_margin():
    assert autotune.choose({}) == autotune.DEFAULT
    assert autotune.choose({4: 2.0, 8: 1.0}) == 8
    assert autotune.choose({4: 2.0, 8: 1.0, 16: 1.02, 32: 1.5}) == 16
    assert autotune.choose({4: 2.0, 8: 1.0, 16: 1.2, 32: 1.5}) == 8
    assert autotune.choose({4: 2.0, 8: 1.3, 16: 1.2, 32: 1.1}) == 32


def test_measures_once_per_shape_and_caches_on_disk(fresh):
    calls = []

    def fake(K, d, q, g, precision="split"):
        calls.append((K, d, q, g, precision))
        return {4: 3.0, 8: 1.0, 16: 2.0, 32: 2.5} if d == 3 else {4: 3.0, 8: 2.0, 16: 1.0, 32: 2.5}

    assert autotune.team_lanes(11, 3, 1, True, measure_fn=fake, device="dev") == 8
    assert autotune.team_lanes(11, 3, 1, True, measure_fn=fake, device="dev") == 8
    assert autotune.team_lanes(31, 10, 1, True, measure_fn=fake, device="dev") == 16
    assert calls == [(11, 3, 1, True, "split"), (31, 10, 1, True, "split")]
    data = json.loads(fresh.read_text())
    assert data[autotune.shape_key("dev", 11, 3, 1, True)] == 8
    # a new process reads the file instead of measuring
    autotune._mem.clear()
    autotune._file_loaded = False
    assert autotune.team_lanes(11, 3, 1, True, measure_fn=None, device="dev") == 8
    # another device is another key
    assert autotune.team_lanes(11, 3, 1, True, measure_fn=fake, device="other") == 8
    assert len(calls) == 3
    # another precision form is another key
    assert autotune.team_lanes(11, 3, 1, True, precision="split_df", measure_fn=fake, device="dev") == 8
    assert calls[-1] == (11, 3, 1, True, "split_df")
    assert autotune.shape_key("dev", 11, 3, 1, True, "split_df") in json.loads(fresh.read_text())


def test_switch_off_and_trivial_blocks(fresh, monkeypatch):
    def boom(*a, **kw):
        raise AssertionError("no measurement expected")

    assert autotune.team_lanes(1, 3, 1, True, measure_fn=boom, device="dev") == autotune.DEFAULT
    monkeypatch.setenv("SV_AUTOTUNE", "0")
    assert autotune.team_lanes(21, 3, 1, True, measure_fn=boom, device="dev") == autotune.DEFAULT


def test_unreadable_cache_is_ignored(fresh):
    fresh.write_text("not json")
    assert autotune.team_lanes(21, 4, 0, False, measure_fn=lambda *a, **kw: {4: 1.0, 8: 2.0, 16: 3.0, 32: 4.0},
                               device="dev") == 4


@pytest.mark.gpu
def test_measurement_on_the_device(fresh):
    times = autotune.measure(21, 3, 1, True, nblocks=6000)
    assert set(times) == set(autotune.WIDTHS)
    assert all(t > 0 for t in times.values())
    w = autotune.team_lanes(21, 3, 1, True)
    assert w in autotune.WIDTHS
    assert autotune.team_lanes(21, 3, 1, True, measure_fn=lambda *a, **kw: pytest.fail("measured twice")) == w
