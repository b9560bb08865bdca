"""The autotuner's tables: the C table compiled into the library (csrc/tuned_launch.inc)
holds the JSON table's choices, entry for entry, and the tuner's candidate lists stay within
what a launch may ask for."""
import json
import re
from pathlib import Path

from sprout_gb300 import tune

PKG = Path(__file__).resolve().parents[1] / "sprout_gb300"


def test_compiled_table_matches_the_json():
    js = json.loads((PKG / "tuned_launch.json").read_text())
    inc = (PKG / "csrc" / "tuned_launch.inc").read_text()
    rows = [tuple(int(v) for v in m) for m in re.findall(r"\{(\d+), (\d+), (\d+), (\d+), (\d+)\}", inc)]
    want = [(s["grid"][0], s["grid"][1], s["best"]["pressure_blocks"], s["best"]["pressure_blocks_mixed"],
             s["best"]["viscosity_blocks"]) for s in js["sizes"]]
    assert rows == want
    for s in js["sizes"]:
        assert s["best"]["viscosity_mg_sweeps"] in (1, 2)
        assert any(t["effective"]["pressure_blocks"] == s["best"]["pressure_blocks"] for t in s["trials"] if t["precision"] == "plain")


def test_candidates_are_valid_counts():
    for nwg in (40, 144, 336, 2304):
        c = tune.candidates(nwg)
        assert c[0] == 0 and all(1 <= b < nwg for b in c[1:]) and c == sorted(set(c))
