"""bench.py's host side on CPU: the reference arm's JSON line (its timed CPU leg stubbed), the clock
sampler's fallback without nvidia-smi, the launch count per tick, and the per-model diagnostics of
the uneven hierarchical workload."""
import importlib.util
import json
import os
import types

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_reference_arm_line_keys(monkeypatch, capsys):
    b = _bench()
    fake = {"value": 20.0, "unit": "ESS/s", "cores": 16, "kind": "port", "grad_evals_per_s": 500.0,
            "sampling_s": 40.0, "sample": "stub"}
    monkeypatch.setattr(b, "reference_leg", lambda *a, **k: dict(fake))
    monkeypatch.setenv("RANK", "0")
    args = types.SimpleNamespace(n=1000, steps=3, warmup=1, gpus=1)
    assert b.run_reference(args) == 0
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    for key in ["metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"]:
        assert key in line, key
    assert line["impl"] == "reference" and line["metric"] == b.METRIC and line["value"] == 20.0
    assert line["e2e"] == {"value": 20.0, "unit": "ESS/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert "workload" in line["config"]


def test_reference_arm_other_ranks_print_nothing(monkeypatch, capsys):
    b = _bench()
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setattr(b, "reference_leg", lambda *a, **k: (_ for _ in ()).throw(AssertionError("ran")))
    assert b.run_reference(types.SimpleNamespace(n=1000, steps=3, warmup=1, gpus=2)) == 0
    assert capsys.readouterr().out == ""


def test_clock_sampler_without_nvidia_smi(monkeypatch):
    b = _bench()
    monkeypatch.setenv("PATH", "/nonexistent")
    c = b.Clocks(0)
    c.start()
    out = c.stop()
    assert out["sm_mhz"] is None and out["reasons"]


def test_launches_per_tick():
    b = _bench()
    assert b._launches_per_tick("bf16x3") == 2  # advance (with split and finish fused), tensor-core potential
    assert b._launches_per_tick("fp32") == 3    # advance, CUDA-core potential, finish


def test_per_model_diagnostics_match_the_host_estimators():
    """bench.py's per-model ESS / R-hat over a batch of uneven models (model-major view of the
    draws, each model's padding excluded) against the host estimators model by model."""
    torch = pytest.importorskip("torch")
    from numpyro_gb300 import diagnostics as D

    rng = np.random.default_rng(2)
    M, cpm, S, Dmax = 5, 4, 80, 7
    dims = [7, 3, 5, 2, 6]
    z = rng.standard_normal((M * cpm, S, Dmax)).cumsum(axis=1) * 0.2 + rng.standard_normal((M * cpm, S, Dmax))
    for m, d in enumerate(dims):
        z[m * cpm:(m + 1) * cpm, :, d:] = 0.0  # padding
    ess_m, rhat_m = _bench().per_model_diagnostics(torch.as_tensor(z), M, cpm, dims, chunk=6)
    for m, d in enumerate(dims):
        zz = z[m * cpm:(m + 1) * cpm, :, :d]
        np.testing.assert_allclose(float(ess_m[m]), D.bulk_effective_sample_size(zz).min(), rtol=1e-10)
        np.testing.assert_allclose(float(rhat_m[m]), D.split_gelman_rubin(zz).max(), rtol=1e-10)
