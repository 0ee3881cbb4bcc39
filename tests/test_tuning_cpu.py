"""The autotuner's cache: one timing per workload shape, atomic updates (CPU, fake tuner)."""
from elanfmt_gb300 import fields as F
from elanfmt_gb300 import inputs as I
from elanfmt_gb300 import tuning


def test_kchunk_cached_per_shape(tmp_path):
    path = str(tmp_path / "k.json")
    calls = []

    def fake(m, prec, fused, n):
        calls.append((m.nx, prec, fused))
        return 12 if m.nx == 20 else 6

    a = I.random_small(F.MODEL_ORTHO, 20, 18, 16, nt=5, seed=1)
    b = I.random_small(F.MODEL_ORTHO, 24, 18, 16, nt=5, seed=1)
    assert tuning.kchunk_for(a, path=path, device_name="gpuX", tune=fake) == 12
    assert tuning.kchunk_for(a, path=path, device_name="gpuX", tune=fake) == 12
    assert tuning.kchunk_for(b, path=path, device_name="gpuX", tune=fake) == 6
    assert tuning.kchunk_for(a, precision=F.PREC_F64, path=path, device_name="gpuX", tune=fake) == 12
    assert tuning.kchunk_for(a, path=path, device_name="gpuY", tune=fake) == 12
    assert len(calls) == 4                       # the repeated query was served from the file
    for form in (F.STEP_FUSED, F.STEP_WAVE):     # every step form has its own entry
        assert tuning.kchunk_for(a, fused=form, path=path, device_name="gpuX", tune=fake) == 12
    assert len(calls) == 6
    data = tuning.load(path)
    assert len(data) == 6 and all(isinstance(v, int) for v in data.values())


def test_unreadable_cache_is_empty(tmp_path):
    p = tmp_path / "bad.json"
    p.write_text("{not json")
    assert tuning.load(str(p)) == {}
    tuning.store("k", 8, str(p))
    assert tuning.load(str(p)) == {"k": 8}


def test_split_setting_cached_with_tile_height(tmp_path):
    path = str(tmp_path / "k.json")
    calls = []

    def fake(m, prec, n):
        calls.append((m.nx, prec))
        return (8, 16, 3) if m.nx == 20 else (24, 4, 0)

    a = I.random_small(F.MODEL_ORTHO, 20, 18, 16, nt=5, seed=1)
    b = I.random_small(F.MODEL_ISO, 24, 18, 16, nt=5, seed=1)
    assert tuning.split_setting_for(a, path=path, device_name="gpuX", tune=fake) == (8, 16, 3)
    assert tuning.split_setting_for(a, path=path, device_name="gpuX", tune=fake) == (8, 16, 3)
    assert tuning.split_setting_for(b, path=path, device_name="gpuX", tune=fake) == (24, 4, 0)
    assert len(calls) == 2
    # the z-chunk-only entries of the same shape stay separate
    assert tuning.kchunk_for(a, path=path, device_name="gpuX", tune=lambda *x: 12) == 12
    assert tuning.split_setting_for(a, path=path, device_name="gpuX", tune=fake) == (8, 16, 3)
    assert sorted(len(v) if isinstance(v, list) else 1 for v in tuning.load(path).values()) == [1, 3, 3]
