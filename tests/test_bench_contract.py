"""Shape of bench.py's JSON line: the keys and types its consumers read (CPU only)."""

import copy

import pytest


def good_line():
    return {
        "metric": "particle-substeps/s", "value": 5.0e9, "unit": "particle-substeps/s", "n_gpus": 1, "steps": 200,
        "warmup": 5, "ms_per_step": 1.9, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic", "config": {"workload": "plain large"},
        "roofline": {"bound": "hbm", "achieved": 1100.0, "peak": 6781.1, "unit": "GB/s", "frac": 0.17,
                     "traffic": 1.4e8},
        "e2e": {"value": 4.2e9, "unit": "particle-substeps/s", "h2d_bytes_per_step": 100, "d2h_bytes_per_step": 12},
        "gpu_launches": 8000,
        "clocks": {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": []},
        "cpu_baseline": {"value": 1.3e7, "unit": "particle-substeps/s", "cores": 16, "kind": "port",
                         "sample": "50 substeps"},
    }


def test_good_line_passes():
    import bench

    bench.validate_line(good_line())


@pytest.mark.parametrize("path,value", [
    (("clocks",), 2.07e9),                 # the clock dict replaced by a number
    (("clocks", "reasons"), "none"),
    (("roofline", "frac"), None),
    (("roofline", "traffic"), "n/a"),
    (("e2e", "h2d_bytes_per_step"), 1.5),
    (("gpu_launches",), True),
    (("cpu_baseline", "kind"), "estimate"),
    (("config", "workload"), None),
])
def test_malformed_line_is_rejected(path, value):
    import bench

    d = copy.deepcopy(good_line())
    obj = d
    for k in path[:-1]:
        obj = obj[k]
    obj[path[-1]] = value
    with pytest.raises(ValueError):
        bench.validate_line(d)


def test_reference_lines():
    import bench

    bench.validate_line({"impl": "reference", "unavailable": "why"})
    ref = {k: good_line()[k] for k in ("metric", "value", "unit", "cpu_baseline", "e2e")}
    ref["impl"] = "reference"
    bench.validate_line(ref)
    del ref["cpu_baseline"]
    with pytest.raises(ValueError):
        bench.validate_line(ref)
