"""Per-iteration fingerprints of a routing run.

A routing job's trajectory is the sequence of its path sets, one per
negotiation iteration (and per detail-pass round), as both the oracle loop
(``OracleRouter.trace``) and the GPU router (``PathFinderRouter.trace``)
append them.  Keeping every path of a 2,000-net job for 40 iterations costs
gigabytes of Python lists, so ``TrajectoryRecorder`` stands in for the
``trace`` list and keeps only fingerprints:

* ``sha256`` of the flat int64 array ``[len(p0), *p0, len(p1), *p1, ...]``
  over the nets in name order (the same flattening the parity tests use);
* an 8-byte BLAKE2b digest of every net whose path changed since the
  previous record (all nets in the first record), so the first differing
  net of a mismatching iteration can be named.

Two runs of the same job (this router on different GPUs, engines or
tunings, or this router against a recorded CPU run) are identical exactly
when their fingerprints are; a mismatch names its first iteration and nets.
"""
from __future__ import annotations

import gzip
import hashlib
import json
import re
from typing import Dict, List, Sequence

import numpy as np


def _name_key(name: str):
    m = re.fullmatch(r"([^\d]*)(\d+)(.*)", name)
    return (m.group(1), int(m.group(2)), m.group(3)) if m else (name, -1, "")


def _as_i64(path) -> np.ndarray:
    if isinstance(path, np.ndarray):
        return path.astype(np.int64, copy=False)
    return np.fromiter((int(v) for v in (path or ())), dtype=np.int64)


def flat_paths(paths: Dict[str, Sequence[int]]) -> np.ndarray:
    parts = []
    for name in sorted(paths, key=_name_key):
        p = _as_i64(paths[name])
        parts.append(np.asarray([len(p)], dtype=np.int64))
        parts.append(p)
    return np.concatenate(parts) if parts else np.zeros(0, dtype=np.int64)


def path_digest(path: Sequence[int]) -> str:
    return hashlib.blake2b(_as_i64(path).tobytes(), digest_size=8).hexdigest()


class TrajectoryRecorder:
    """A drop-in for a router's ``trace`` list: ``append(paths)`` records the
    fingerprints of one iteration's path set."""

    def __init__(self):
        self.records: List[dict] = []
        self._last: Dict[str, str] = {}

    def append(self, paths: Dict[str, Sequence[int]]) -> None:
        digests = {n: path_digest(p) for n, p in paths.items()}
        changed = {n: d for n, d in digests.items() if self._last.get(n) != d}
        gone = sorted(set(self._last) - set(digests))
        self._last = digests
        rec = {"sha256": hashlib.sha256(flat_paths(paths).tobytes()).hexdigest(),
               "nets": len(paths), "changed": changed}
        if gone:
            rec["removed"] = gone
        self.records.append(rec)

    def __len__(self):
        return len(self.records)


def first_difference(got: List[dict], want: List[dict]):
    """(record index, net names whose digests differ) of the first record
    where two trajectories part, or None when they agree."""
    for j, (a, b) in enumerate(zip(got, want)):
        if a["sha256"] != b["sha256"]:
            names = sorted(set(a["changed"]) | set(b["changed"]), key=_name_key)
            diff = [n for n in names if a["changed"].get(n) != b["changed"].get(n)]
            return j, diff[:20]
    if len(got) != len(want):
        return min(len(got), len(want)), []
    return None


def save(path: str, doc: dict) -> None:
    """gzip-compressed JSON with a zero header timestamp, so the same run
    writes the same bytes."""
    data = json.dumps(doc, sort_keys=True, separators=(",", ":")).encode("utf-8")
    with open(path, "wb") as raw, gzip.GzipFile(fileobj=raw, mode="wb", mtime=0, filename="") as f:
        f.write(data)


def load(path: str) -> dict:
    with gzip.open(path, "rt", encoding="utf-8") as f:
        return json.load(f)
