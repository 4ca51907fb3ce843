"""The batch autotuner (msm_tune_uneven): it measures whole passes of the caller's own uneven
mix, keeps the fastest form per size class for shared passes, persists it, and never changes a
result (every MSM is checked against the oracle after tuning)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_tune_uneven_keeps_results_exact(engine, ocpu, tmp_path, monkeypatch):
    cache = tmp_path / "tune.txt"
    monkeypatch.setenv("MSM_TUNE_CACHE", str(cache))
    nbase = 1 << 16
    pts = ocpu.gen_bases(301, nbase)
    rng = np.random.default_rng(5)
    sizes = [int(2 ** u) for u in rng.uniform(8, 14, 12)]
    offs = [int(rng.integers(0, nbase - s + 1)) for s in sizes]
    sc = np.concatenate([ocpu.gen_scalars(302, s, kind=1, msm_index=j) for j, s in enumerate(sizes)])
    first = np.concatenate([[0], np.cumsum(sizes)])
    want = [ocpu.msm(pts[o:o + s], sc[first[j]:first[j + 1]]) for j, (s, o) in enumerate(zip(sizes, offs))]
    ctx = engine.multi_scalar_mult_init(pts)
    try:
        res = ctx.tune_uneven(sizes, offs, sc, budget_ms=4000)
        assert 0 < res["tuned_ms"] <= res["untuned_ms"]
        assert res["passes_measured"] >= 2
        for cls, form in res["forms"].items():
            assert 6 <= form["window_bits"] <= 22 and form["bases"] in (0, 1, 2)
        for opts in (res["opts"], {}):
            out = ctx.mult_uneven(sizes, offs, sc, mode=2, **{k: v for k, v in opts.items() if k != "mode"})
            for j in range(len(sizes)):
                assert np.array_equal(out[j], want[j]), f"MSM {j} (n={sizes[j]}) with {opts}"
        forms = res["forms"]
    finally:
        ctx.close()
    lines = cache.read_text().splitlines()
    assert any(ln.startswith("b ") for ln in lines)
    # a new context reads the persisted forms back
    ctx = engine.multi_scalar_mult_init(pts)
    try:
        for cls, form in forms.items():
            assert ctx.tuned_form(1 << cls, shared_pass=True) == form
        out = ctx.mult_uneven(sizes, offs, sc, mode=2, use_graph=1)
        assert all(np.array_equal(out[j], want[j]) for j in range(len(sizes)))
    finally:
        ctx.close()
