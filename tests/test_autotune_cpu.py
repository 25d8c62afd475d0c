"""CPU: the engine tuner's search, cache and struct mapping, with a modelled trace time in place of a GPU."""
from __future__ import annotations

import random

from tardiis_and_claritas_gb300 import abi, autotune as AT, scene as S


def _model(opt: dict, noise: float, seed: int):
    """Trace time in seconds: 1.0 at the defaults, 3 % less for each setting of `opt` that is met."""
    rng = random.Random(seed)

    def t(cfg: dict) -> float:
        v = 1.0
        for k, want in opt.items():
            if k == "stage_blocks":
                for s, b in want.items():
                    if cfg.get("stage_blocks", {}).get(s) == b:
                        v *= 0.97
            elif cfg.get(k) == want:
                v *= 0.97
        return v * (1.0 + rng.uniform(-noise, noise))
    return t


def test_search_finds_the_modelled_optimum():
    opt = {"flight_steps": 6, "tail_photons": 131072, "stage_blocks": {"GEN": 1, "SIDE": 2}}
    res = AT.search(_model(opt, 0.002, 1), reps=3)
    assert res["config"] == opt
    assert 0.10 < res["gain"] < 0.15


def test_search_keeps_defaults_on_a_flat_cost():
    res = AT.search(_model({}, 0.005, 2), reps=2)
    assert res["config"] == {}
    assert res["gain"] == 0.0


def test_confirmation_rejects_a_lucky_draw():
    calls = {"n": 0}

    def t(cfg):
        calls["n"] += 1
        # one early draw of flight_steps=2 is fast by luck; later draws are not
        if cfg == {"flight_steps": 2} and calls["n"] < 5:
            return 0.5
        return 1.0
    res = AT.search(t, reps=1)
    assert res["config"] == {}


def test_engine_config_struct_mapping():
    c = abi.EngineConfig.from_dict({"flight_steps": 6, "pass_batch": 16, "stage_blocks": {"FLIGHT": 1, "FIN": 2}})
    assert c.flight_steps == 6 and c.pass_batch == 16 and c.tail_photons == 0
    sb = list(c.stage_blocks)
    assert sb[abi.STAGE_NAMES.index("FLIGHT")] == 1 and sb[abi.STAGE_NAMES.index("FIN")] == 2
    assert sum(sb) == 3
    assert abi.C.sizeof(abi.EngineConfig) == 4 * (4 + len(abi.STAGE_NAMES) + 3)


class _FakeCtx:
    def __init__(self, model):
        self.model, self.cfg, self.last = model, None, 0.0
        self.set_calls = []

    def set_engine_config(self, cfg):
        self.cfg = cfg
        self.set_calls.append(cfg)

    def trace(self, run):
        self.last = self.model(self.cfg or {})
        return {}, None

    def last_kernel_ms(self):
        return self.last * 1e3


def test_tune_caches_by_device_and_scene(tmp_path):
    cfg, parts, grid, zmax = S.full_scene_workload()
    sp, ps, ss = cfg.to_scene_params(), parts.spec(cfg), cfg.sediment_spec(grid, zmax)
    key = AT.scene_key(sp, ps, ss)
    cache = str(tmp_path / "t.json")
    ctx = _FakeCtx(_model({"flight_steps": 8}, 0.0, 3))
    mk = lambda i: S.run_params(10, seed=i)  # noqa: E731
    res = AT.tune(ctx, mk, key=key, photons=10_000, device="sm103x152", cache_file=cache)
    assert res["config"] == {"flight_steps": 8} and not res["cached"]
    assert ctx.set_calls[-1] == {"flight_steps": 8}
    n_trials = len(ctx.set_calls)
    res2 = AT.tune(ctx, mk, key=key, photons=12_000, device="sm103x152", cache_file=cache)
    assert res2["cached"] == "user" and len(ctx.set_calls) == n_trials + 1
    # another GPU or another scene is tuned afresh
    res3 = AT.tune(ctx, mk, key=key, photons=10_000, device="sm100x148", cache_file=cache)
    assert not res3["cached"]
    cfg2 = S.small_cell_config()
    assert AT.scene_key(cfg2.to_scene_params(), ps, ss) != key
    # the key follows the bins' values, not where the host buffers live
    import numpy as np
    d = np.array(parts.diameter_m, copy=True)
    ps2 = abi.ParticleSpec.from_buffer_copy(ps)
    ps2.diameter_m = d.ctypes.data_as(abi.PD)
    assert AT.scene_key(sp, ps2, ss) == key
    d[0] *= 1.01
    assert AT.scene_key(sp, ps2, ss) != key


def test_shipped_table_is_valid_and_used(tmp_path, monkeypatch):
    entries = AT.load_shipped()
    assert entries, "the package ships tuned settings"
    for k, e in entries.items():
        dev, work, bits = k.split("|")
        assert dev.startswith("sm") and int(bits) > 0 and work
        c = abi.EngineConfig.from_dict(e["config"])
        assert 0 <= c.flight_steps <= 64 and 0 <= c.pass_batch <= 64 and all(0 <= b <= 32 for b in c.stage_blocks)
        assert e["trace_s"] <= e["default_trace_s"]
    key = next(iter(entries))
    dev, work, bits = key.split("|")
    ctx = _FakeCtx(_model({}, 0.0, 5))
    res = AT.tune(ctx, lambda i: S.run_params(10, seed=i), key=work, photons=(1 << (int(bits) - 1)), device=dev,
                  cache_file=str(tmp_path / "empty.json"))
    assert res["cached"] == "shipped" and ctx.set_calls == [entries[key]["config"] or None]
    # without the shipped table the same call searches
    monkeypatch.setattr(AT, "SHIPPED_TABLE", str(tmp_path / "none.json"))
    res = AT.tune(ctx, lambda i: S.run_params(10, seed=i), key=work, photons=(1 << (int(bits) - 1)), device=dev,
                  cache_file=str(tmp_path / "empty2.json"))
    assert res["cached"] is False and res["trials"] > 10
