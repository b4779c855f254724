"""Structured per-step log: one JSON object per line (no counterpart in the
reference, which prints progress lines: gravlist.cpp:150-191, run.c:112).

A box's record: the step index, the scale factor after it, the device time of
each phase (ms) and the step's particle-updates/s.  A serving loop's records:
one per tick (running and queued jobs, particle updates so far) and one per
finished job (its latency and steps)."""
from __future__ import annotations

import json
import time


class StepLog:
    def __init__(self, target):
        """`target`: a path (opened for appending) or a writable text file."""
        self._own = isinstance(target, str)
        self._f = open(target, "a") if self._own else target

    def write(self, kind: str, **fields) -> None:
        rec = {"kind": kind, "wall": time.time()}
        rec.update(fields)
        self._f.write(json.dumps(rec) + "\n")
        self._f.flush()

    def close(self) -> None:
        if self._own:
            self._f.close()


def read(path: str) -> list[dict]:
    with open(path) as fh:
        return [json.loads(line) for line in fh if line.strip()]
