"""Host logic of the autotuner (no GPU): the fastest candidate is picked and
stored, a stored choice is reused without timing, a candidate the library
refuses is skipped, a stored choice that is no longer a candidate is tuned
again, and the on-disk cache is read back by a fresh process state.  The
timer is replaced by a table of fake times; everything else is the
tuner's own code."""
import json
import os

import pytest

from pyspectrum_gb300 import _lib, tune


@pytest.fixture()
def fresh(tmp_path, monkeypatch):
    monkeypatch.setenv("PYSPEC_GB300_CACHE", str(tmp_path))
    monkeypatch.setattr(tune, "_mem", {})
    monkeypatch.setattr(tune, "_loaded", False)
    timed = []

    def fake_time(fn, reps=tune.REPS):
        return fn()          # the run callback below returns its fake duration

    monkeypatch.setattr(tune, "_time", fake_time)
    return tmp_path, timed


def _runner(times, timed, refuse=()):
    def run(c):
        timed.append(c)
        if c in refuse:
            raise _lib.PyspecError("refused for this size")
        return times[c]
    return run


def test_fastest_is_picked_and_stored(fresh):
    tmp, timed = fresh
    times = {"a": 2.0, "b": 0.5, "c": 1.0}
    assert tune._pick("k1", list(times), _runner(times, timed)) == "b"
    assert sorted(timed) == ["a", "b", "c"]
    on_disk = json.load(open(os.path.join(tmp, "tune.json")))
    assert on_disk["k1"]["choice"] == "b"
    assert on_disk["k1"]["ms"] == {"a": 2.0, "b": 0.5, "c": 1.0}


def test_stored_choice_is_reused_without_timing(fresh):
    _, timed = fresh
    times = {0: 3.0, 1: 1.0}
    assert tune._pick("k2", [0, 1], _runner(times, timed)) == 1
    timed.clear()
    assert tune._pick("k2", [0, 1], _runner({0: 0.1, 1: 9.0}, timed)) == 1
    assert timed == []


def test_refused_candidate_is_skipped(fresh):
    _, timed = fresh
    times = {"x": 0.1, "y": 0.7}
    assert tune._pick("k3", ["x", "y"], _runner(times, timed, refuse=("x",))) == "y"
    assert tune.choices()["k3"]["ms"] == {"y": 0.7}


def test_stale_choice_is_tuned_again(fresh):
    _, timed = fresh
    tune._store("k4", {"choice": "gone", "ms": {"gone": 0.1}})
    assert tune._cached("k4", ["p", "q"]) is None
    assert tune._pick("k4", ["p", "q"], _runner({"p": 0.4, "q": 0.2}, timed)) == "q"
    assert sorted(timed) == ["p", "q"]


def test_cache_file_is_read_by_a_fresh_state(fresh, monkeypatch):
    _, timed = fresh
    tune._pick("k5", [1, 2], _runner({1: 0.3, 2: 0.9}, timed))
    # a new process: nothing in memory, the file on disk
    monkeypatch.setattr(tune, "_mem", {})
    monkeypatch.setattr(tune, "_loaded", False)
    timed.clear()
    assert tune._pick("k5", [1, 2], _runner({1: 5.0, 2: 0.1}, timed)) == 1
    assert timed == []


def test_disabled_by_environment(monkeypatch):
    monkeypatch.setenv("PYSPEC_GB300_TUNE", "0")
    assert not tune.enabled()
    monkeypatch.setenv("PYSPEC_GB300_TUNE", "1")
    assert tune.enabled()
