"""bench.py's JSON line helpers (host logic, no GPU): the summary of every form comes right
after the contract's keys, the contract's keys are all there, and floats are shortened."""
import importlib.util
import json
import os

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _line():
    rf = {"bound": "hbm", "achieved": 3354.713, "peak": 6656.6, "unit": "GB/s", "frac": 0.503967947, "traffic": 60367104}
    return {"metric": "m", "value": 132.90678021, "unit": "Gcell-updates/s", "n_gpus": 1, "steps": 3, "warmup": 3,
            "ms_per_step": 316.0109659, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic", "config": {"workload": "w"},
            "e2e": {"value": 132.5638134, "unit": "Gcell-updates/s", "h2d_bytes_per_step": 1, "d2h_bytes_per_step": 2},
            "e2e_zfp": {"value": 132.23135}, "gpu_launches": 45012, "roofline": rf,
            "cpu_baseline": {"value": 7.387, "cores": 16}, "clocks": {"sm_mhz": 2070.0},
            "precision": {"variants": [{"image_rel_l2_vs_fp64": 2.0704680633821205e-06}]},
            "batched": {"value": 136.99, "speedup_vs_plain": 1.3665, "members": 64,
                        "stencil_kernel_roofline": {"frac": 0.7767}, "forward_step_roofline": {"frac": 0.5518},
                        "autotuned_tile_x_by_width_class": {"1024": {"tile_x": 32}}},
            "served": {"requests": 96, "value": 97.259, "p50_latency_s": 1.9783, "p99_latency_s": 4.5702,
                       "hbm_occupancy_mean": 0.0317, "speedup_vs_plain_same_requests": 3.6591,
                       "plain": {"requests": 48, "p50_latency_s": 1.6, "p99_latency_s": 4.05},
                       "served_same_requests": {"p50_latency_s": 1.3, "p99_latency_s": 4.39}},
            "parity": {"image_rel_l2_vs_oracle": 2.626140665567384e-06, "image_rel_l2_vs_fp64_engine": 2.39e-06}}


def test_summary_follows_the_contract_keys():
    b = _bench()
    out = b.compact_line(_line())
    keys = list(out)
    contract = ["metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "e2e", "gpu_launches", "roofline",
                "cpu_baseline", "clocks"]
    assert keys[:len(contract)] == contract
    assert keys[len(contract)] == "summary"
    s = out["summary"]
    assert s["plain"]["value"] == 132.91 and s["plain"]["roofline_frac"] == 0.504
    assert s["batched"]["k_mstep_frac"] == 0.7767 and s["batched"]["tile_x_by_width_class"] == {"1024": 32}
    assert s["served"]["plain_p50_p99_s"] == [1.6, 4.05] and s["served"]["served_p50_p99_s"] == [1.3, 4.39]
    assert s["parity"]["image_rel_l2_vs_oracle"] == 2.63e-06
    # every detail key is still there, after the summary
    assert set(_line()) <= set(out)


def test_floats_are_shortened_and_the_line_is_json():
    b = _bench()
    out = b.compact_line(_line())
    assert out["value"] == 132.91 and out["roofline"]["frac"] == 0.50397
    assert out["gpu_launches"] == 45012 and isinstance(out["gpu_launches"], int)
    assert json.loads(json.dumps(out)) == out
