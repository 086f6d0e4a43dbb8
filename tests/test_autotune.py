"""The autotuner's search, persistence and lookup on the CPU, with a fake library (it records the
tunables it is given) and a fake timer (a cost that depends on them)."""
import json

import pytest

from wavebit_gb300 import autotune as AT


class FakeLib:
    def __init__(self):
        self.values = {}
        self.calls = 0

    def wb_set_tuning(self, key, value):
        if key < 0 or value < 0:
            return 1
        self.values[key] = value
        return 0

    def wb_get_tuning(self, key):
        return self.values.get(key, 0)


def cost_timer(lib):
    """Seconds of a run: fastest with 512 QR threads and 1024 reduction threads."""
    def timer(run):
        run()
        qr, hrd = lib.values.get(0, 0), lib.values.get(1, 0)
        return 1.0 + (0.0 if qr == 512 else 0.3 + 0.001 * abs(qr - 512)) + (0.0 if hrd == 1024 else 0.2)
    return timer


def test_coordinate_descent_finds_the_fastest_shapes_and_persists_them(tmp_path):
    lib = FakeLib()
    runs = []
    path = str(tmp_path / 'tuning.json')
    tuner = AT.Autotuner(lib=lib, timer=cost_timer(lib), path=path)
    key = AT.bucket_key((12, 12), 4, 38, 'mixed')
    assert key == '12x12/L4/B38/mixed'
    best = tuner.tune(key, lambda: runs.append(1))
    assert best == {'qr_threads': 512, 'hrd_threads': 1024}
    assert tuner.current() == best                    # applied
    assert runs                                       # the run was executed by the trials
    saved = json.load(open(path))
    assert saved[key]['settings'] == best
    assert saved[key]['seconds'] == pytest.approx(1.0)
    # a new tuner loads the choice and applies it by lookup at a nearby batch size
    lib2 = FakeLib()
    t2 = AT.Autotuner(lib=lib2, timer=cost_timer(lib2), path=path)
    got = t2.lookup((12, 12), 4, 30, 'mixed')
    assert got == best
    t2.apply(got)
    assert lib2.values == {0: 512, 1: 1024}
    assert t2.lookup((12, 12), 4, 30, 'double') is None
    assert t2.lookup((11, 11), 4, 38, 'mixed') is None
    t2.reset()
    assert t2.current() == {'qr_threads': 0, 'hrd_threads': 0}


def test_a_candidate_must_beat_the_current_choice_by_the_margin():
    lib = FakeLib()

    def flat(run):
        run()
        return 1.0 - (0.01 if lib.values.get(0, 0) == 256 else 0.0)    # 1% better: under the 2% margin
    tuner = AT.Autotuner(lib=lib, timer=flat)
    assert tuner.tune('k', lambda: None) == {'qr_threads': 0, 'hrd_threads': 0}


def test_batch_limit_maximises_solves_per_second(tmp_path):
    lib = FakeLib()
    last = {}

    def timer(run):
        run()
        b = last['b']
        return 0.5 + 0.1 * b + (0.05 * (b - 16) ** 2 if b > 16 else 0.0)   # knee at 16
    tuner = AT.Autotuner(lib=lib, timer=timer, path=str(tmp_path / 't.json'))
    best = tuner.tune_batch_limit('5x5/L2/B*/double', lambda b: last.__setitem__('b', b), [1, 2, 4, 8, 16, 32])
    assert best == 16
    assert tuner.batch_limit('5x5/L2/B*/double') == 16


def test_refused_settings_raise():
    class Refusing(FakeLib):
        def wb_set_tuning(self, key, value):
            return 1
    with pytest.raises(ValueError):
        AT.Autotuner(lib=Refusing(), timer=lambda r: 1.0).apply({'qr_threads': 99})
