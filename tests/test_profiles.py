"""The committed ncu summaries feed the bench line: the field kernel's mean
DRAM traffic per launch and its instruction-issue utilisation must stay
readable from them, and every summary must give the command that made it."""
import os

import bench

PROFILES = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "profiles")


def test_field_profile_figures_parse():
    traffic = bench.field_traffic()
    issue = bench.field_issue()
    assert traffic is not None and 1e6 < traffic < 1e9
    assert issue is not None and 0.0 < issue <= 1.0


def test_profiles_name_their_commands():
    names = [f for f in os.listdir(PROFILES) if f.endswith((".md", ".txt"))]
    assert names
    for f in names:
        with open(os.path.join(PROFILES, f)) as fh:
            text = fh.read()
        assert "ncu " in text and "--clock-control none" in text, f
        assert "python bench.py" in text, f
