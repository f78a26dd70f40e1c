"""CPU tests of the batched form's schedule cache: the key separates what changes the best
schedule (device, scheme, kernel variant, the multiset of instance sizes) and nothing else, and
the cache file round-trips. No GPU is touched."""
import importlib
import json

import pytest


@pytest.fixture(scope="module")
def autotune(dense):
    return importlib.import_module("2dense_gb300.autotune")


def cfgs(dense, sizes, recon=255, strict=0):
    return [dense.config_default(ni=n, nj=m, benchmark=11, splitting=101, recon=recon, strict=strict)
            for n, m in sizes]


def test_key_ignores_instance_order(dense, autotune):
    a = autotune.batch_key(cfgs(dense, [(64, 64), (96, 128), (32, 48)]))
    b = autotune.batch_key(cfgs(dense, [(32, 48), (64, 64), (96, 128)]))
    assert a == b


def test_key_separates_sizes_scheme_and_variant(dense, autotune):
    base = autotune.batch_key(cfgs(dense, [(64, 64), (96, 128)]))
    assert autotune.batch_key(cfgs(dense, [(64, 64), (128, 96)])) != base
    assert autotune.batch_key(cfgs(dense, [(64, 64), (96, 128)], recon=253)) != base
    assert autotune.batch_key(cfgs(dense, [(64, 64), (96, 128)], strict=1)) != base
    assert autotune.batch_key(cfgs(dense, [(64, 64), (96, 128), (64, 64)])) != base


def test_cache_round_trip(autotune, tmp_path, monkeypatch):
    path = tmp_path / "sub" / "autotune.json"
    monkeypatch.setattr(autotune, "CACHE", str(path))
    assert autotune._load_cache() == {}
    autotune._store_cache({"k": [1, 2, 0]})
    assert json.loads(path.read_text()) == {"k": [1, 2, 0]}
    assert autotune._load_cache() == {"k": [1, 2, 0]}
    path.write_text("not json")
    assert autotune._load_cache() == {}


def test_schedule_space_from_the_library(autotune):
    n_xi, n_eta, n_order = autotune.schedule_space()
    assert (n_xi, n_eta, n_order) == (4, 5, 3)
