"""Error measures shared by the parity tests at the benchmark sizes.

Two normalisations of |gpu - oracle| for H entries:
- term scale: divided by the sum of the magnitudes of the terms the oracle
  adds into the entry (its H['scale']), the measure of rounding in a sum
  whose terms may cancel;
- per entry: divided by |oracle entry| itself, over the entries at or above
  an absolute floor of FLOOR Hartree.  An H entry below 1e-15 Eh is below the
  FP64 resolution of the O(1) Eh diagonal entries of the same matrix and
  cannot change an eigenvalue at FP64 precision; such entries (often
  cancellations of much larger terms) are judged by the term-scale measure,
  and their largest absolute error is reported.
  Entries above the floor whose terms cancel to less than CANCEL of their
  sum of magnitudes are reported apart (cancel_entry_max): any FP64
  summation order, the oracle's included, leaves an error of ~1e-16 of the
  terms there, i.e. 1e-13 or more of such an entry, so their bar is the
  term-scale one too.
"""
import json
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np

FLOOR = 1e-15  # Hartree
CANCEL = 1e-3  # |entry| / (sum of |terms|) below which an entry counts as a cancellation


def errors(got, ref, scale=None):
    """Error statistics of complex arrays got vs ref (same pattern)."""
    got = np.asarray(got)
    ref = np.asarray(ref)
    d = np.abs(got - ref)
    a = np.abs(ref)
    out = {"n": int(ref.size)}
    if ref.size == 0:
        out.update(term_max=0.0, term_rms=0.0, entry_max=0.0, entry_rms=0.0, n_below_floor=0,
                   below_floor_abs_max=0.0, worst_entry=None, cancel_entry_max=0.0, n_cancel=0)
        return out
    above = a >= FLOOR
    if scale is not None:
        t = d / np.maximum(scale, 1e-300)
        out["term_max"] = float(t.max())
        out["term_rms"] = float(np.sqrt(np.mean(t ** 2)))
        canc = above & (a < CANCEL * scale)
        out["n_cancel"] = int(canc.sum())
        out["cancel_entry_max"] = float((d[canc] / a[canc]).max()) if canc.any() else 0.0
        above = above & ~canc
    if above.any():
        e = d[above] / a[above]
        out["entry_max"] = float(e.max())
        out["entry_rms"] = float(np.sqrt(np.mean(e ** 2)))
        i = int(np.flatnonzero(above)[np.argmax(e)])
        out["worst_entry"] = {"value": float(a[i]), "abs_err": float(d[i]),
                              "term_scale": float(scale[i]) if scale is not None else None}
    else:
        out["entry_max"] = out["entry_rms"] = 0.0
        out["worst_entry"] = None
    out["n_below_floor"] = int((~above).sum())
    out["below_floor_abs_max"] = float(d[~above].max()) if (~above).any() else 0.0
    return out


def merge(stats):
    """Worst case over several errors() results."""
    out = {"n": sum(s["n"] for s in stats),
           "n_cancel": sum(s.get("n_cancel", 0) for s in stats)}
    for key in ("term_max", "entry_max", "below_floor_abs_max", "cancel_entry_max"):
        vals = [s[key] for s in stats if key in s]
        if vals:
            out[key] = max(vals)
    for key in ("term_rms", "entry_rms"):
        vals = [(s[key], s["n"]) for s in stats if key in s and s["n"]]
        if vals:
            out[key] = float(np.sqrt(sum(v * v * n for v, n in vals) / sum(n for _, n in vals)))
    worst = [s for s in stats if s.get("worst_entry")]
    if worst:
        out["worst_entry"] = max(worst, key=lambda s: s["entry_max"])["worst_entry"]
    out["n_below_floor"] = sum(s.get("n_below_floor", 0) for s in stats)
    return out


def row_starts(n, places, per):
    """`places` starts spread over [0, n - per], each the first of `per` rows."""
    per = min(per, n)
    return sorted(set(np.linspace(0, n - per, places).astype(np.int64).tolist())), per


def oracle_rows(O, jobs, threads=None):
    """Runs O.construct_block for each (args, kwargs) job on host threads
    (ctypes releases the interpreter lock during the call)."""
    threads = threads or os.cpu_count() or 1
    with ThreadPoolExecutor(max_workers=threads) as ex:
        return list(ex.map(lambda j: O.construct_block(*j[0], **j[1]), jobs))


def report(name, data):
    """Writes data as JSON to $BS2E_REPORT_DIR/<name>.json when that is set."""
    d = os.environ.get("BS2E_REPORT_DIR")
    if d:
        os.makedirs(d, exist_ok=True)
        with open(os.path.join(d, name + ".json"), "w") as f:
            json.dump(data, f, indent=1)


def band_keys(tiles, k, n_b):
    """Every key (a, b, c, d) of the given tiles with c, d inside 1..n_b, and
    for each key its (tile, dc, dd) position in a rk_tiles array."""
    keys, pos = [], []
    for t, (a, b) in enumerate(np.asarray(tiles).reshape(-1, 2)):
        for dc in range(2 * k - 1):
            c = a + dc - (k - 1)
            if c < 1 or c > n_b:
                continue
            for dd in range(2 * k - 1):
                d = b + dd - (k - 1)
                if 1 <= d <= n_b:
                    keys.append((a, b, c, d))
                    pos.append((t, dc, dd))
    return np.array(keys, dtype=np.int64), np.array(pos, dtype=np.int64)
