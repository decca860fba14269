"""The shipped autotuning table (fk_mc_gb300/tuning_gb300.json) and how it is
applied, without a GPU: every entry names a compiled variant (a panel width or
the two-stage reduction) and keeps the fastest time per solve, every size class
of the uneven workload has a reduction entry per precision and a
back-transformation entry for the mixed path, and `apply` routes each entry to
the matching setter (fkg_set_tuning / fkg_set_tuning_back)."""
import json

from fk_mc_gb300 import autotune


def test_table_entries_name_compiled_variants():
    t = json.load(open(autotune.DEFAULT_TABLE))
    sizes = set()
    for e in t["entries"]:
        assert 1 <= e["n_max"] <= 1024
        sizes.add(e["n_max"])
        if e.get("stage") == "back":
            assert e["variant"] in autotune.BACK_VARIANTS
            assert e["kernel"] == autotune.BACK_VARIANTS[e["variant"]]
            assert len(e["ms_per_solve"]) == len(autotune.BACK_VARIANTS)
        else:
            widths = autotune.VARIANTS[e["precision"]]
            assert 0 <= e["variant"] < len(widths)
            assert e["panel_width"] == widths[e["variant"]]
            assert len(e["ms_per_solve"]) == len(widths)
        assert min(e["ms_per_solve"]) == e["ms_per_solve"][e["variant"]]  # the fastest was kept
    for n in sizes:
        kinds = {(e.get("stage", "reduce"), e.get("precision", "mixed")) for e in t["entries"] if e["n_max"] == n}
        assert kinds == {("reduce", "mixed"), ("reduce", "f64"), ("back", "mixed")}


class _Recorder:
    def __init__(self):
        self.calls = []

    def set_tuning(self, precision, n_max, variant):
        self.calls.append(("reduce", precision, n_max, variant))

    def set_tuning_back(self, n_max, variant):
        self.calls.append(("back", n_max, variant))


def test_apply_routes_entries(tmp_path):
    table = {"entries": [{"precision": "mixed", "n_max": 576, "variant": 1},
                         {"stage": "back", "n_max": 1024, "variant": 1},
                         {"precision": "f64", "n_max": 256, "variant": 0}]}
    path = tmp_path / "t.json"
    path.write_text(json.dumps(table))
    r = _Recorder()
    assert autotune.apply(r, str(path))
    assert r.calls == [("reduce", "mixed", 576, 1), ("back", 1024, 1), ("reduce", "f64", 256, 0)]
    assert not autotune.apply(_Recorder(), str(tmp_path / "missing.json"))
