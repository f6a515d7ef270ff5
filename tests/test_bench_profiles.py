"""The bench line's `roofline.traffic` and `roofline.issue` come from the
committed ncu summaries under profiles/: both lines must be present and
parse, and the issue roof they give must be a fraction below one for the
kernel durations those captures recorded.  CPU only."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
pytest.importorskip("torch")
sys.path.insert(0, ROOT)
import bench  # noqa: E402


@pytest.mark.parametrize("kernel", ["siddon_pj_f32", "siddon_bpj_f32"])
def test_profile_summaries_parse(kernel):
    traffic = bench.ncu_traffic(kernel)
    assert traffic is not None and 1e8 < traffic < 1e11
    prof = bench.ncu_issue(kernel)
    assert prof is not None
    assert set(prof) >= {"issue_active_pct", "warp_inst", "segments", "lanes_per_inst", "duration_ms"}
    assert 0 < prof["issue_active_pct"] <= 100 and 1 <= prof["lanes_per_inst"] <= 32
    # the capture's own launch against its issue roof at 2070 MHz
    roof = bench.issue_roofline(kernel, prof["segments"], prof["duration_ms"], 2070.0)
    assert 0.3 < roof["frac"] < 1.0
    assert roof["warp_inst_per_launch"] == pytest.approx(prof["warp_inst"])
