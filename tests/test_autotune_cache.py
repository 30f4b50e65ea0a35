"""Host logic of the autotuner's JSON cache (no GPU): keys, validation,
atomic store, and a cache hit applying the stored launch choice."""
import json

from ucfd_sparse_gb300 import autotune as at


class FakeSys:
    kind = "blusgs"
    nlocal, nfaces, nvars, precision = 2097152, 6340608, 5, 2

    def __init__(self):
        self.cfg = dict(threads_per_block=0, sweep_variant=0, run_mode=0, ms=0.0)

    def set_launch_config(self, threads_per_block=0, sweep_variant=0, run_mode=0, **_):
        self.cfg.update(threads_per_block=threads_per_block, sweep_variant=sweep_variant, run_mode=run_mode)

    def launch_config(self):
        return dict(self.cfg)


def test_key_and_validation(monkeypatch):
    monkeypatch.setattr(at, "device_key", lambda: "GPU|152 SMs")
    assert at.cache_key(FakeSys()) == "GPU|152 SMs|blusgs|N=2097152|nface=6340608|nvars=5|prec=fp32"
    assert at.valid_entry(dict(threads_per_block=128, sweep_variant=1, run_mode=0))
    assert not at.valid_entry(dict(threads_per_block=100, sweep_variant=1, run_mode=0))
    assert at.valid_entry(dict(threads_per_block=0, sweep_variant=3, run_mode=1))
    assert not at.valid_entry(dict(threads_per_block=128, sweep_variant=5, run_mode=0))
    assert not at.valid_entry(dict(threads_per_block=128, sweep_variant=1, run_mode=2))
    assert not at.valid_entry(None)


def test_store_load_and_hit(tmp_path, monkeypatch):
    monkeypatch.setattr(at, "device_key", lambda: "GPU|152 SMs")
    path = str(tmp_path / "sub" / "tune.json")
    assert at.load_cache(path) == {}
    s = FakeSys()
    key = at.cache_key(s)
    at.store_cache(path, {key: dict(threads_per_block=192, sweep_variant=1, run_mode=0, ms=0.5)})
    assert json.load(open(path))[key]["threads_per_block"] == 192
    out = at.tune(s, cache=path)
    assert out["source"] == "cache" and out["ms"] == 0.5
    assert s.cfg["threads_per_block"] == 192 and s.cfg["sweep_variant"] == 1
    # only the cache file is left in the folder (no temporaries)
    assert sorted(p.name for p in (tmp_path / "sub").iterdir()) == ["tune.json"]


def test_corrupt_cache_is_empty(tmp_path):
    p = tmp_path / "bad.json"
    p.write_text("{not json")
    assert at.load_cache(str(p)) == {}
    p.write_text("[1, 2]")
    assert at.load_cache(str(p)) == {}
