"""Autotuner: tunes the launch knobs of a problem class into its JSON cache,
applies them, and leaves the results unchanged (the knobs change the launch
configuration, not the arithmetic)."""
import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_tune_cache_apply_and_same_results(gpu_lib, tmp_path, monkeypatch):
    import nlsemagic_gb300 as ng
    from nlsemagic_gb300 import autotune
    from nlsemagic_gb300 import workloads as W
    cache = tmp_path / "tune.json"
    monkeypatch.setenv("NLSE_TUNE_CACHE", str(cache))
    shape = (40, 40, 40)
    saved = {k: autotune.get_knob(k) for k in autotune.KNOBS}
    try:
        entry = autotune.tune(shape, method=2, precision=ng.PREC_MIXED, BC=2, steps=4)
        assert cache.exists()
        data = json.loads(cache.read_text())
        key = autotune.problem_key(shape, 2, ng.PREC_MIXED, 2)
        assert key in data and data[key]["wide.zc"] == entry["wide.zc"]
        assert entry["candidates"] >= 2 and entry["gpt_steps_per_s"] > 0
        # a second call hits the cache
        assert autotune.tune(shape, method=2, precision=ng.PREC_MIXED, BC=2, steps=4) == entry
        w = W.vortex_rings_3d(n=40, steps=7)

        def run():  # a fresh solver: its graphs are captured with the current knobs
            with ng.Solver(w.U.shape, method=2, precision=ng.PREC_MIXED, BC=w.BC, s=w.s, a=w.a,
                           h2=w.h2, k=w.k) as sv:
                sv.upload(w.U, w.V)
                sv.run(w.steps)
                return sv.download()

        autotune.set_knob("wide.zc", 0)
        autotune.set_knob("graph.steps", 8)
        base = run()
        applied = autotune.apply(shape, method=2, precision=ng.PREC_MIXED, BC=2)
        assert applied == entry
        assert autotune.get_knob("wide.zc") == entry["wide.zc"]
        tuned = run()
        assert np.array_equal(np.ascontiguousarray(base).view(np.float64),
                              np.ascontiguousarray(tuned).view(np.float64))
    finally:
        for k, v in saved.items():
            autotune.set_knob(k, v)
