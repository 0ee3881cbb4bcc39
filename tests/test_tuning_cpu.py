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
