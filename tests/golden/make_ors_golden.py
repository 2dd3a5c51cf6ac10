"""Golden .ORS files written by the reference's own serializer.

Run in a container that holds the reference checkout (read only):

    python tests/golden/make_ors_golden.py /path/to/OrthoRoute

For the two reference routing runs (r0, r1) it takes the reference's emitted
tracks and vias (``tests/golden/geometry.json``), headless-style iteration
metrics and metadata (the dict layout of ``main.py``'s headless mode), and
calls ``export_solution_to_ors`` (uncompressed), then reads the file back
with ``import_solution_from_ors`` / ``convert_ors_to_geometry_payload`` and
exports that payload again (the start/end and position/size layouts).  The
export timestamps are replaced by a fixed string.  Output:
``tests/golden/ors.json.gz`` = {run: {"first": text, "second": text}}.
"""
from __future__ import annotations

import gzip
import json
import os
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
STAMP = "2026-01-01T00:00:00.000000Z"


class Payload:
    def __init__(self, tracks, vias):
        self.tracks = tracks
        self.vias = vias


def headless_inputs(tag, meta):
    metrics = [{"iteration": m["it"], "timestamp": "2026-01-01 00:00:00", "duration_s": 0.0,
                "overuse": m["node_over"], "barrel_conflicts": m["barrel"], "routed_nets": meta.get("n_nets", 0),
                "time": 0.5 * m["it"]}
               for m in meta["per_iter"]]
    metadata = {"orthoroute_version": "0.1.0", "total_time": 1.25, "iterations": len(metrics),
                "converged": False, "barrel_conflicts": 3, "nets_routed": meta.get("n_nets", 0),
                "wirelength": 0.0, "via_count": 7, "track_count": 11, "overflow": 0, "board_name": tag}
    return metrics, metadata


def stamp(text):
    doc = json.loads(text)
    old = doc["metadata"]["export_timestamp"]
    return text.replace(json.dumps(old), json.dumps(STAMP), 1)


def main(ref_root):
    sys.path.insert(0, ref_root)
    from orthoroute.infrastructure.serialization.ors_exporter import (
        convert_ors_to_geometry_payload, export_solution_to_ors, import_solution_from_ors)
    geo = json.load(open(os.path.join(HERE, "geometry.json")))
    meta = json.load(open(os.path.join(HERE, "golden.json")))
    out = {}
    with tempfile.TemporaryDirectory() as tmp:
        for tag in ("r0", "r1"):
            metrics, metadata = headless_inputs(tag, meta[tag])
            p1 = os.path.join(tmp, f"{tag}.ORS")
            export_solution_to_ors(Payload(geo[tag]["tracks"], geo[tag]["vias"]), metrics, metadata, p1,
                                   compress=False)
            gdata, _ = import_solution_from_ors(p1)
            p2 = os.path.join(tmp, f"{tag}_again.ORS")
            export_solution_to_ors(convert_ors_to_geometry_payload(gdata), metrics, metadata, p2, compress=True)
            with gzip.open(p2, "rt", encoding="utf-8") as f:
                second = f.read()
            out[tag] = {"first": stamp(open(p1, encoding="utf-8").read()), "second": stamp(second)}
    with gzip.open(os.path.join(HERE, "ors.json.gz"), "wt", encoding="utf-8") as f:
        json.dump(out, f)
    print({k: (len(v["first"]), len(v["second"])) for k, v in out.items()})


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
