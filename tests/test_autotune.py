"""The autotuner: its JSON cache on the host (no GPU), and on the GPU a tuned
batch of uneven scenes that renders with the chosen sizes, answered from the
cache the second time."""
import json

import numpy as np
import pytest

import lisa_gb300 as L
from lisa_gb300 import _native as N
from lisa_gb300 import scenes


def _tuning(key, w=1 << 21, t=96, f=8, m=1234.5):
    x = N.Tuning()
    x.struct_size = C_SIZE
    x.paths_in_flight, x.threads_per_block, x.blocks_per_sm, x.refill_idle = w, t, 0, f
    x.probe_spp, x.mrays_per_s = 4, m
    x.key = key.encode()
    return x


C_SIZE = __import__("ctypes").sizeof(N.Tuning)


def test_cache_round_trip(tmp_path):
    path = str(tmp_path / "tune.json")
    assert L.tuning_cache_lookup(path, "absent") is None  # no file yet: a miss, not an error
    L.tuning_cache_store(path, _tuning("devA|px2^20", w=1 << 22))
    L.tuning_cache_store(path, _tuning("devB|px2^16", t=64, f=16))
    L.tuning_cache_store(path, _tuning("devA|px2^20", w=1 << 23, m=99.0))  # replaces
    doc = json.load(open(path))
    assert set(doc) == {"devA|px2^20", "devB|px2^16"}
    a = L.tuning_cache_lookup(path, "devA|px2^20")
    assert (a.paths_in_flight, a.threads_per_block, a.refill_idle) == (1 << 23, 96, 8)
    assert a.mrays_per_s == pytest.approx(99.0) and a.key == b"devA|px2^20"
    b = L.tuning_cache_lookup(path, "devB|px2^16")
    assert (b.threads_per_block, b.refill_idle, b.probe_spp) == (64, 16, 4)
    assert L.tuning_cache_lookup(path, "devC") is None
    o = L.apply_tuning(a)
    assert (o.paths_in_flight, o.threads_per_block, o.blocks_per_sm, o.refill_idle) == (1 << 23, 96, 0, 8)


def test_cache_rejects_bad_files_and_keys(tmp_path):
    path = tmp_path / "bad.json"
    path.write_text('{"k": {"paths_in_flight": 12,}')  # truncated
    with pytest.raises(L.LisaError):
        L.tuning_cache_lookup(str(path), "k")
    with pytest.raises(L.LisaError):  # a malformed file is not overwritten
        L.tuning_cache_store(str(path), _tuning("k"))
    assert path.read_text() == '{"k": {"paths_in_flight": 12,}'
    good = str(tmp_path / "good.json")
    for key in ("", 'has"quote', "back\\slash", "new\nline"):
        with pytest.raises(L.LisaError):
            L.tuning_cache_store(good, _tuning(key))
    # unknown numeric fields written by a later version are ignored
    (tmp_path / "extra.json").write_text('{"k": {"paths_in_flight": 65536, "future_field": 3}}')
    t = L.tuning_cache_lookup(str(tmp_path / "extra.json"), "k")
    assert t.paths_in_flight == 65536


@pytest.mark.gpu
def test_autotune_batch_and_cache(gpu, tmp_path):
    batch = scenes.batch_scenes(n=4, seed=9, max_res=160)
    params = [L.params_from_scene(s) for s in batch]
    cache = str(tmp_path / "tune.json")
    t = L.autotune(params, cache=cache)
    assert t.candidates >= 3 and t.mrays_per_s > 0
    assert t.threads_per_block in (64, 96, 128) and t.refill_idle in (8, 12, 16)
    assert t.key.decode() in json.load(open(cache))
    again = L.autotune(params, cache=cache)
    assert again.candidates == 0 and again.paths_in_flight == t.paths_in_flight
    # the tuned sizes render the same image as the defaults up to summation
    # order (the sizes change the schedule, not the per-sample streams)
    tuned = L.Renderer(params, L.apply_tuning(t))
    tuned.render_progressive(4)
    ref = L.Renderer(params)
    ref.render_progressive(4)
    for k in range(len(params)):
        np.testing.assert_allclose(tuned.image(k), ref.image(k), rtol=1e-5, atol=1e-6)
