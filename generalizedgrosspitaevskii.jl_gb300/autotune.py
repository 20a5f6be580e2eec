"""A small autotuner for ensemble groups.

For a group (grid size, components, precision, trajectories) it times the candidate
configurations on the actual problem for a few chunks of steps and keeps the fastest:

* path: the resident plane kernel (whole trajectory in shared memory, when the grid fits)
  or the two-pass HBM path;
* line tiling of the two-pass path (``gpe_set_variant``): for FP32 one-component fields
  16 points a thread along x and 8 along y (variant 0) or 8 and 16 (variant 1), i.e. the
  radix of the register stages and the tile shape of each pass;
* steps_per_graph: the chunk length captured in the CUDA graph (launch amortisation vs
  graph size).

Results are cached in a JSON file keyed by the group shape and the GPU name
(``$GPE_AUTOTUNE_CACHE`` or ``~/.cache/gpe_gb300/autotune.json``).
"""
from __future__ import annotations

import json
import os
from pathlib import Path
from typing import Callable, Dict, Iterable, Optional, Tuple

CANDIDATE_CHUNKS = (10, 50, 200)


def cache_path() -> Path:
    p = os.environ.get("GPE_AUTOTUNE_CACHE")
    return Path(p) if p else Path.home() / ".cache" / "gpe_gb300" / "autotune.json"


def _load() -> Dict[str, dict]:
    p = cache_path()
    try:
        return json.loads(p.read_text())
    except (OSError, ValueError):
        return {}


def _store(db: Dict[str, dict]):
    p = cache_path()
    try:
        p.parent.mkdir(parents=True, exist_ok=True)
        p.write_text(json.dumps(db, indent=1, sort_keys=True))
    except OSError:
        pass  # a read-only home only loses the cache


def gpu_name() -> str:
    try:
        import subprocess
        out = subprocess.run(["nvidia-smi", "--query-gpu=name", "--format=csv,noheader", "-i", "0"],
                             capture_output=True, text=True, timeout=10).stdout.strip()
        return out or "unknown"
    except Exception:
        return "unknown"


def key(N: int, M: int, dtype: str, ntraj: int, gpu: str) -> str:
    return f"{gpu}|N{N}|M{M}|{dtype}|B{ntraj}"


def resident_fits(N: int, M: int, complex_bytes: int) -> bool:
    """Whether an N x N field of M components (complex_bytes per value) runs in the
    resident plane kernel: its whole trajectory must fit in 200 KiB of shared memory
    (the library's rule for square 2D grids of 16..128 points a side)."""
    return 16 <= N <= 128 and M * N * N * complex_bytes <= 200 * 1024


def tune(make_iterator: Callable[[bool, int], object], k: str, chunks: Iterable[int] = CANDIDATE_CHUNKS,
         trial_steps: int = 200, force: bool = False, variants: Iterable[int] = (0,),
         resident_ok: bool = True) -> Tuple[bool, int, int, dict]:
    """Pick (resident, variant, steps_per_graph) for one group.  make_iterator(resident,
    variant) builds a fresh iterator for the group; ``variants`` are the line tilings to
    try on the two-pass path; ``resident_ok`` False leaves the resident kernel out (the
    grid does not fit it).  Returns (resident, variant, steps_per_graph, timings)."""
    db = _load()
    if not force and k in db and "variant" in db[k]:
        r = db[k]
        return bool(r["resident"]) and resident_ok, int(r["variant"]), int(r["steps_per_graph"]), r.get("timings", {})
    from .twa import Ensemble
    timings = {}
    best = None
    candidates = ([(True, 0)] if resident_ok else []) + [(False, v) for v in variants]
    for resident, variant in candidates:
        for chunk in chunks:
            if trial_steps % chunk:
                continue
            it = make_iterator(resident, variant)
            ens = Ensemble([it])
            try:
                ens.run(chunk, chunk)  # capture + warm-up
                ens.run(trial_steps, chunk)
                ms = ens.last_run_ms()
            finally:
                ens.close()
                it.close()
            timings[f"resident={resident},variant={variant},chunk={chunk}"] = ms
            if best is None or ms < best[0]:
                best = (ms, resident, variant, chunk)
    db[k] = {"resident": best[1], "variant": best[2], "steps_per_graph": best[3], "timings": timings}
    _store(db)
    return best[1], best[2], best[3], timings
