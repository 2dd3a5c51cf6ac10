"""F3: .ORS solution files equal the reference serializer's output (golden
files it wrote for the two reference runs), read back the same way, and
.ORP board files are validated as the reference validates them (CPU)."""
import gzip
import json
import os

import pytest

from orthoroute_gb300 import ors
from tests.golden.make_ors_golden import STAMP, Payload, headless_inputs

G = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def golden():
    with gzip.open(os.path.join(G, "ors.json.gz"), "rt", encoding="utf-8") as f:
        return json.load(f)


@pytest.mark.parametrize("tag", ["r0", "r1"])
def test_ors_text_matches_reference_serializer(golden, tag, tmp_path):
    geo = json.load(open(os.path.join(G, "geometry.json")))[tag]
    meta = json.load(open(os.path.join(G, "golden.json")))[tag]
    metrics, metadata = headless_inputs(tag, meta)
    p1 = tmp_path / f"{tag}.ORS"
    ors.export_solution_to_ors(Payload(geo["tracks"], geo["vias"]), metrics, metadata, str(p1), compress=False,
                               timestamp=STAMP)
    assert p1.read_text(encoding="utf-8") == golden[tag]["first"]
    # read back, convert to the in-memory layout, write again (compressed)
    gdata, md = ors.import_solution_from_ors(str(p1))
    assert md["statistics"]["total_tracks"] == len(geo["tracks"])
    p2 = tmp_path / f"{tag}_again.ORS"
    ors.export_solution_to_ors(ors.convert_ors_to_geometry_payload(gdata), metrics, metadata, str(p2),
                               compress=True, timestamp=STAMP)
    with gzip.open(p2, "rt", encoding="utf-8") as f:
        assert f.read() == golden[tag]["second"]
    summary = ors.get_solution_summary(json.loads(golden[tag]["first"]))
    assert f"Total Tracks: {len(geo['tracks'])}" in summary


def test_ors_reader_rejects_bad_files(tmp_path):
    p = tmp_path / "bad.ORS"
    with pytest.raises(FileNotFoundError):
        ors.import_solution_from_ors(str(p))
    for doc, msg in [({}, "Missing format_version"), ({"format_version": "2.0"}, "Unsupported ORS"),
                     ({"format_version": "1.0", "metadata": {}}, "Missing required sections")]:
        p.write_text(json.dumps(doc))
        with pytest.raises(ValueError, match=msg):
            ors.import_solution_from_ors(str(p))
    assert ors.derive_ors_filename("boards/Main.ORP") == "boards/Main.ORS"


def _orp_doc():
    term = lambda x, y: {"pad_id": f"U1-{x}", "position": {"x": x, "y": y}, "layer": "F.Cu"}
    return {"format_version": "1.0", "metadata": {}, "board": {"bounds": {"x_min": 10.1, "y_min": 20.0,
                                                                          "x_max": 30.0, "y_max": 40.0}},
            "pads": [], "layers": [], "drc_rules": {}, "grid_parameters": {"pitch": 0.4},
            "nets": [{"name": "A", "is_routable": True, "terminals": [term(10.4, 20.0), term(12.0, 21.2)]},
                     {"name": "B", "is_routable": True, "terminals": [term(11.0, 20.4)]},
                     {"name": "C", "is_routable": False, "terminals": [term(11.0, 20.4), term(12.0, 20.4)]}]}


def test_orp_reader_and_two_pin_requests(tmp_path):
    p = tmp_path / "b.ORP"
    with gzip.open(p, "wt", encoding="utf-8") as f:
        json.dump(_orp_doc(), f)
    doc = ors.import_board_from_orp(str(p))
    # grid origin: round(10.1 / 0.4) * 0.4 = 10.0, round(20.0 / 0.4) * 0.4 = 20.0
    assert ors.orp_two_pin_requests(doc, nx=60, ny=60) == [("A", 1, 3 * 60 + 5)]
    bad = dict(_orp_doc())
    del bad["layers"]
    p.write_text(json.dumps(bad))
    with pytest.raises(ValueError, match="layers"):
        ors.import_board_from_orp(str(p))
