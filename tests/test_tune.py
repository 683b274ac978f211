"""Tuning tables (pytorchsph_gb300.tune): size buckets, nearest-bucket lookup, spec
configuration and the JSON round trip (no GPU)."""
import numpy as np

from pytorchsph_gb300.tune import Tuning, bucket


def test_buckets_and_nearest_lookup():
    assert bucket(2048) == 11 and bucket(4095) == 11 and bucket(4096) == 12
    t = Tuning(serving={11: {"cell_ratio": 2, "tpp": 4}, 15: {"cell_ratio": 1, "tpp": 1}},
               search={20: {"sort": "radix", "digit_bits": 6}})
    assert t.scene_config(3000) == {"cell_ratio": 2, "tpp": 4}
    assert t.scene_config(10000) == {"cell_ratio": 2, "tpp": 4}     # bucket 13: 11 and 15 tie, lower wins
    assert t.scene_config(20000) == {"cell_ratio": 1, "tpp": 1}
    assert t.scene_config(10 ** 7) == {"cell_ratio": 1, "tpp": 1}
    assert t.search_config(1 << 16) == {"sort": "radix", "digit_bits": 6, "cell_ratio": 1}
    assert Tuning().scene_config(5000) == {"cell_ratio": 1, "tpp": 1}
    assert Tuning().search_config(5000) == {"sort": "counting", "digit_bits": 8, "cell_ratio": 1}


def test_configure_sets_spec_fields_and_json_round_trip(tmp_path):
    from pytorchsph_gb300.serve import SceneSpec
    from pytorchsph_gb300.sim import SimConfig
    t = Tuning(serving={12: {"cell_ratio": 2, "tpp": 2, "measured": {"2,2": {"ms_per_step": 0.1}}}},
               device="GB300")
    sp = SceneSpec({"pos": np.zeros((5000, 2), np.float32)}, SimConfig())
    t.configure(sp)
    assert (sp.cell_ratio, sp.tpp) == (2, 2)
    p = tmp_path / "tuning.json"
    t.save(str(p))
    u = Tuning.load(str(p))
    assert u.serving == t.serving and u.device == "GB300"


def test_search_cell_ratio_round_trip(tmp_path):
    """A search bucket tuned to cells of h/2 keeps its ratio through JSON; a table written
    before the ratio was a knob reads as cells of h."""
    t = Tuning(search={20: {"sort": "counting", "digit_bits": 8, "cell_ratio": 2,
                            "measured": {"counting,0,2": {"ms": 0.49}}},
                       16: {"sort": "radix", "digit_bits": 8}})
    p = tmp_path / "tuning.json"
    t.save(str(p))
    u = Tuning.load(str(p))
    assert u.search_config(1 << 20) == {"sort": "counting", "digit_bits": 8, "cell_ratio": 2}
    assert u.search_config(1 << 16) == {"sort": "radix", "digit_bits": 8, "cell_ratio": 1}
