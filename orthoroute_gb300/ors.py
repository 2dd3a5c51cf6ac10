"""F3: the .ORS solution file (and reading .ORP board files).

Restates the reference's ORS writer and reader
(``orthoroute/infrastructure/serialization/ors_exporter.py``:
``export_solution_to_ors`` :18-96, ``_build_solution_metadata`` :99-109,
``_build_geometry_data`` :112-255, ``_build_iteration_metrics`` :258-278,
``_build_statistics`` :281-339, ``import_solution_from_ors`` :342-401,
``convert_ors_to_geometry_payload`` :404-453) and the helpers of
``serialization/__init__.py`` (``derive_ors_filename`` :48-55,
``get_solution_summary`` :58-124, new-format branch).  The document has the
reference's keys, key order, defaults and fallbacks (for instance a via's
``diameter`` is read from its ``size`` key, default 0.4, and the wirelength
sums only tracks given by start/end), and it is written with the same JSON
settings, so for the same geometry, metrics and metadata the text equals the
reference's apart from ``export_timestamp``.

``import_board_from_orp`` reads and validates a .ORP board file
(``orp_exporter.py:543-589``).  Routing a board from its pads needs the
reference's pad escape (portal) planning, which this package does not do;
``orp_two_pin_requests`` gives the lattice-node tuple requests of an ORP
file's nets (first two terminals, layer 0) for the tuple-request router.
"""
from __future__ import annotations

import gzip
import json
from datetime import datetime, timezone
from pathlib import Path
from typing import Any, Dict, List, Optional, Tuple


class GeometryPayload:
    """Tracks and vias with attribute access."""

    def __init__(self, tracks: List[Dict], vias: List[Dict]):
        self.tracks = tracks
        self.vias = vias


# ---------------------------------------------------------------- writing
def export_solution_to_ors(geometry, iteration_metrics: List[Dict[str, Any]], metadata: Dict[str, Any],
                           filepath: str, compress: bool = True, timestamp: Optional[str] = None) -> None:
    """Write a routing solution (geometry with ``.tracks`` / ``.vias``) as
    .ORS; ``timestamp`` overrides the export time (ISO text, for
    reproducible files)."""
    if geometry is None:
        raise ValueError("Geometry cannot be None")
    if not hasattr(geometry, "tracks") or not hasattr(geometry, "vias"):
        raise ValueError("Geometry must have 'tracks' and 'vias' attributes")
    doc = solution_document(geometry, iteration_metrics, metadata, timestamp)
    out = Path(filepath)
    out.parent.mkdir(parents=True, exist_ok=True)
    opener = (lambda: gzip.open(out, "wt", encoding="utf-8")) if compress else \
        (lambda: open(out, "w", encoding="utf-8"))
    with opener() as f:
        json.dump(doc, f, indent=2, ensure_ascii=False)


def solution_document(geometry, iteration_metrics, metadata, timestamp: Optional[str] = None) -> Dict[str, Any]:
    """The .ORS document as a dict (sections in the reference's order)."""
    return {
        "format_version": "1.0",
        "metadata": _metadata(metadata, timestamp),
        "geometry": _geometry(geometry),
        "iteration_metrics": _iteration_metrics(iteration_metrics),
        "statistics": _statistics(geometry, iteration_metrics, metadata),
    }


def _metadata(metadata: Dict[str, Any], timestamp: Optional[str]) -> Dict[str, Any]:
    if timestamp is None:
        timestamp = datetime.now(timezone.utc).replace(tzinfo=None).isoformat() + "Z"
    return {
        "export_timestamp": timestamp,
        "orthoroute_version": metadata.get("orthoroute_version", "0.1.0"),
        "board_name": metadata.get("board_name", "unknown"),
        "total_iterations": metadata.get("total_iterations", 0),
        "converged": metadata.get("converged", False),
        "total_time_seconds": metadata.get("total_time", 0.0),
        "notes": metadata.get("notes", ""),
    }


def _net_key(item: Dict[str, Any]) -> str:
    return str(item.get("net_id") or item.get("net", "unknown"))


def _track_ends(track: Dict[str, Any]) -> Tuple[Any, Any, Any, Any]:
    """A track's end points from any of the three layouts the reader accepts."""
    if "start" in track and "end" in track:
        (x0, y0), (x1, y1) = track["start"], track["end"]
        return x0, y0, x1, y1
    if "x1" in track and "y1" in track:
        return track.get("x1", 0.0), track.get("y1", 0.0), track.get("x2", 0.0), track.get("y2", 0.0)
    return track.get("start_x", 0.0), track.get("start_y", 0.0), track.get("end_x", 0.0), track.get("end_y", 0.0)


def _via_position(via: Dict[str, Any]) -> Tuple[Any, Any]:
    if "position" in via:
        p = via["position"]
        if isinstance(p, (list, tuple)):
            return p[0], p[1]
        return p.get("x", 0.0), p.get("y", 0.0)
    if "x" in via and "y" in via:
        return via.get("x", 0.0), via.get("y", 0.0)
    return 0.0, 0.0


def _geometry(geometry) -> Dict[str, Any]:
    by_net: Dict[str, Dict[str, Any]] = {}
    layer_usage: Dict[Any, int] = {}

    def entry(net: str) -> Dict[str, Any]:
        if net not in by_net:
            by_net[net] = {"net_id": net, "tracks": [], "vias": []}
        return by_net[net]

    for track in geometry.tracks:
        x0, y0, x1, y1 = _track_ends(track)
        layer = track.get("layer", 0)
        entry(_net_key(track))["tracks"].append({
            "layer": layer,
            "start": {"x": float(x0), "y": float(y0)},
            "end": {"x": float(x1), "y": float(y1)},
            "width": float(track.get("width", 0.15)),
        })
        layer_usage[layer] = layer_usage.get(layer, 0) + 1
    for via in geometry.vias:
        px, py = _via_position(via)
        entry(_net_key(via))["vias"].append({
            "position": {"x": float(px), "y": float(py)},
            "from_layer": via.get("from_layer", 0),
            "to_layer": via.get("to_layer", 1),
            "diameter": float(via.get("size", 0.4)),
            "drill": float(via.get("drill", 0.2)),
        })
    all_tracks, all_vias = [], []
    for net in by_net.values():
        all_tracks.extend({**t, "net_id": net["net_id"]} for t in net["tracks"])
        all_vias.extend({**v, "net_id": net["net_id"]} for v in net["vias"])
    return {"by_net": by_net, "all_tracks": all_tracks, "all_vias": all_vias, "layer_usage": layer_usage}


def _iteration_metrics(iteration_metrics: List[Dict[str, Any]]) -> List[Dict[str, Any]]:
    return [{
        "iteration": m.get("iteration", 0),
        "overuse_count": m.get("overuse_count", m.get("overuse", 0)),
        "nets_routed": m.get("nets_routed", m.get("routed", 0)),
        "overflow_cost": m.get("overflow_cost", m.get("overflow", 0.0)),
        "wirelength": m.get("wirelength", 0.0),
        "via_count": m.get("via_count", m.get("vias", 0)),
        "iteration_time_seconds": m.get("iteration_time", m.get("time", 0.0)),
    } for m in iteration_metrics]


def _statistics(geometry, iteration_metrics: List[Dict[str, Any]], metadata: Dict[str, Any]) -> Dict[str, Any]:
    tracks = geometry.tracks if hasattr(geometry, "tracks") else []
    vias = geometry.vias if hasattr(geometry, "vias") else []
    wirelength = 0.0
    for t in tracks:
        # only start/end and start_x.. layouts count (the x1/y1 layout reads as zero length)
        if "start" in t and "end" in t:
            (x0, y0), (x1, y1) = t["start"], t["end"]
        else:
            x0, y0 = t.get("start_x", 0.0), t.get("start_y", 0.0)
            x1, y1 = t.get("end_x", 0.0), t.get("end_y", 0.0)
        dx, dy = x1 - x0, y1 - y0
        wirelength += (dx * dx + dy * dy) ** 0.5
    nets_routed = metadata.get("nets_routed", 0)
    if nets_routed == 0 and hasattr(geometry, "tracks"):
        nets_routed = len({str(t.get("net_id")) for t in tracks if t.get("net_id")})
    final_overuse, final_overflow = 0, 0.0
    if iteration_metrics:
        last = iteration_metrics[-1]
        final_overuse = last.get("overuse_count", last.get("overuse", 0))
        final_overflow = last.get("overflow_cost", last.get("overflow", 0.0))
    return {
        "total_tracks": len(tracks),
        "total_vias": len(vias),
        "total_wirelength_mm": wirelength,
        "nets_routed": nets_routed,
        "final_overuse_count": final_overuse,
        "final_overflow_cost": final_overflow,
        "converged": metadata.get("converged", final_overuse == 0),
        "iterations_completed": len(iteration_metrics),
    }


# ---------------------------------------------------------------- reading
def _read_json(path: Path) -> Dict[str, Any]:
    """gzip-compressed or plain JSON, detected by trying gzip first."""
    try:
        with gzip.open(path, "rt", encoding="utf-8") as f:
            return json.load(f)
    except (gzip.BadGzipFile, OSError):
        with open(path, "r", encoding="utf-8") as f:
            return json.load(f)


def _check(doc: Dict[str, Any], kind: str, sections: List[str]) -> None:
    version = doc.get("format_version")
    if not version:
        raise ValueError(f"Missing format_version in {kind} file")
    if version != "1.0":
        raise ValueError(f"Unsupported {kind} format version: {version}")
    missing = [s for s in sections if s not in doc]
    if missing:
        raise ValueError(f"Missing required sections: {', '.join(missing)}")


def import_solution_from_ors(filepath: str) -> Tuple[Dict[str, Any], Dict[str, Any]]:
    """(geometry section, {metadata, statistics, iteration_metrics}) of a .ORS file."""
    path = Path(filepath)
    if not path.exists():
        raise FileNotFoundError(f"ORS file not found: {path}")
    doc = _read_json(path)
    _check(doc, "ORS", ["metadata", "geometry", "iteration_metrics", "statistics"])
    return doc["geometry"], {"metadata": doc["metadata"], "statistics": doc["statistics"],
                             "iteration_metrics": doc["iteration_metrics"]}


def convert_ors_to_geometry_payload(geometry_data: Dict[str, Any]) -> GeometryPayload:
    """The flat track / via lists of an ORS geometry section in the in-memory
    layout (positions as tuples, via ``size`` = ORS ``diameter``)."""
    tracks = [{"net_id": t.get("net_id"), "layer": t.get("layer"),
               "start": (t["start"]["x"], t["start"]["y"]), "end": (t["end"]["x"], t["end"]["y"]),
               "width": t.get("width")} for t in geometry_data.get("all_tracks", [])]
    vias = [{"net_id": v.get("net_id"), "position": (v["position"]["x"], v["position"]["y"]),
             "from_layer": v.get("from_layer"), "to_layer": v.get("to_layer"), "size": v.get("diameter"),
             "drill": v.get("drill")} for v in geometry_data.get("all_vias", [])]
    return GeometryPayload(tracks, vias)


def derive_ors_filename(orp_filename: str) -> str:
    return str(Path(orp_filename).with_suffix(".ORS"))


def get_solution_summary(ors_data: Dict[str, Any]) -> str:
    """Human-readable summary of a solution document (metadata + statistics)."""
    md, st = ors_data.get("metadata", {}), ors_data.get("statistics", {})
    nets = ors_data.get("geometry", {}).get("by_net", {})
    return "\n".join([
        f"Solution Timestamp: {md.get('export_timestamp', 'Unknown')}",
        f"OrthoRoute Version: {md.get('orthoroute_version', 'Unknown')}",
        "",
        "=== Routing Quality ===",
        f"Convergence: {md.get('converged', False)}",
        f"Total Iterations: {md.get('total_iterations', 0)}",
        f"Total Runtime: {md.get('total_time_seconds', 0):.1f} seconds",
        "",
        f"Nets Routed: {st.get('nets_routed', 0)}",
        f"Total Wirelength: {st.get('total_wirelength_mm', 0):.1f} mm",
        f"Total Via Count: {st.get('total_vias', 0)}",
        f"Final Overflow: {st.get('final_overflow_cost', 0)}",
        "",
        "=== Geometry Details ===",
        f"Total Nets: {len(nets)}",
        f"Total Tracks: {st.get('total_tracks', 0)}",
        f"Total Vias: {st.get('total_vias', 0)}",
    ])


# ---------------------------------------------------------------- ORP boards
ORP_SECTIONS = ["metadata", "board", "pads", "nets", "layers", "drc_rules", "grid_parameters"]


def import_board_from_orp(filepath: str) -> Dict[str, Any]:
    """A .ORP board document, validated (format 1.0, every section present)."""
    path = Path(filepath)
    if not path.exists():
        raise FileNotFoundError(f"ORP file not found: {path}")
    doc = _read_json(path)
    _check(doc, "ORP", ORP_SECTIONS)
    return doc


def orp_two_pin_requests(doc: Dict[str, Any], nx: int, ny: int, pitch: Optional[float] = None
                         ) -> List[Tuple[str, int, int]]:
    """Tuple requests of an ORP document's routable nets: the first two
    terminals, snapped to the pitch grid of the board bounds (the lattice
    origin is the bounds' minimum rounded to the pitch, as the router's grid
    geometry places it), on layer 0.  The reference instead starts nets at
    the pads' escape portals."""
    b = doc["board"]["bounds"]
    p = float(pitch if pitch is not None else doc["grid_parameters"].get("pitch", 0.4))
    gx = round(float(b["x_min"]) / p) * p
    gy = round(float(b["y_min"]) / p) * p
    out = []
    for net in doc["nets"]:
        terms = net.get("terminals", [])
        if len(terms) < 2 or not net.get("is_routable", True):
            continue
        ends = []
        for t in terms[:2]:
            x = min(max(int(round((float(t["position"]["x"]) - gx) / p)), 0), nx - 1)
            y = min(max(int(round((float(t["position"]["y"]) - gy) / p)), 0), ny - 1)
            ends.append(y * nx + x)
        out.append((str(net.get("name", net.get("id"))), ends[0], ends[1]))
    return out
