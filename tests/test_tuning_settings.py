"""The plan-setting strings bench.py prints and replays (``tuning.setting_string``
/ ``parse_setting``): a round trip, and unknown knobs refused."""

import pytest

from ibamr_gb300 import tuning


def test_setting_round_trip():
    s = {"tile_shape": 1, "item_units": 128, "dense_min": 64, "dense_blocks_per_sm": 4, "visit_kernel": 2,
         "interp_kernel": 0, "step_mode": 1, "unit_cap": 16}
    text = tuning.setting_string(s)
    assert text.startswith("tile_shape=1,item_units=128,")
    assert tuning.parse_setting(text) == s
    assert tuning.parse_setting("") == {}


def test_unknown_knob_refused():
    with pytest.raises(ValueError):
        tuning.parse_setting("tile_shape=0,warp_size=64")


def test_default_candidates_cover_every_knob():
    for k in tuning.KNOBS:
        if k in ("item_units", "dense_min", "dense_blocks_per_sm"):
            continue
        assert k in tuning.DEFAULT_CANDIDATES
