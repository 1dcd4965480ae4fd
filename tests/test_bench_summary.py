"""bench.py's closing summary: the headline figures in a short object, the
line's last key (CPU only)."""
import json

import bench


def _line():
    return {
        "metric": "slid points/s", "value": 27149195.3, "ms_per_step": 0.36833,
        "e2e": {"value": 26201935.1, "synchronous": {"value": 23538273.2}},
        "exact_vs_fp64_oracle": True, "roofline": {"frac": 0.018988},
        "cfg0": {"value": 9487262.8, "e2e": {"value": 7394996.9}, "e2e_pipelined": {"value": 8927347.1},
                 "slides_exact_vs_reference_cpu": 100, "cpu_reference": {"slid_points_per_s": 113579.1}},
        "cfg2": {"value": 27702181.5, "rechecked_pairs_per_slide": 73.9,
                 "mismatches_vs_fp64_oracle": {"counts": 0, "labels": 0, "ids": 0}},
        "batched": {"value": 126222086.1, "round_ms_p50": 3.90195, "speedup_vs_plain": 9.2193,
                    "plain_one_at_a_time_default": {"value": 12368226.6},
                    "streams_exact_vs_fp64_oracle": "256/256", "phase_ms": {"union_ms": 2.17}},
        "serving": {"capacity_requests_per_s": 57712.1,
                    "sweep": [{"offered_fraction": f, "latency_ms_p50": p50, "latency_ms_p99": p99}
                              for f, p50, p99 in ((0.3, 0.75, 1.23), (0.6, 1.22, 2.23), (0.9, 3.34, 6.64))]},
    }


def test_summary_holds_the_headline_figures():
    s = bench.headline_summary(_line())
    assert s["walker"]["ms_per_slide"] == 0.3683 and s["walker"]["exact_vs_fp64_oracle"] is True
    assert s["batched"]["speedup_vs_tuned_plain"] == 9.22
    assert s["batched"]["speedup_vs_fixed_plain"] == 10.2
    assert s["cfg0"]["slides_exact_vs_reference_cpu"] == 100
    assert s["cfg2"]["mismatches_vs_fp64_oracle"] == {"counts": 0, "labels": 0, "ids": 0}
    assert s["serving"]["p50_p99_ms_by_load"]["0.9"] == [3.34, 6.64]


def test_summary_fits_the_end_of_the_line():
    line = _line()
    line["summary"] = bench.headline_summary(line)
    text = json.dumps(line)
    assert len(json.dumps(line["summary"])) < 1000
    assert text.endswith(json.dumps(line["summary"]) + "}")


def test_summary_without_optional_legs():
    line = {k: v for k, v in _line().items() if k not in ("cfg0", "cfg2", "batched", "serving")}
    line["e2e"] = {"value": None}
    s = bench.headline_summary(line)
    assert set(s) == {"walker"} and s["walker"]["e2e_pipelined"] is None
