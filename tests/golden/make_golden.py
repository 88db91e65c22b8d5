"""Generate the committed golden fixtures in this folder.

Run where the reference tree exists (REFERENCE, default: beside this repository); the GPU tests
only read the committed outputs:

* ``corr3d_golden.npz`` — make_corr_rand_3d (sim/corr_rand_3d.f90:191-386) evaluated by the
  C restatement linked against the reference's own vendored Ooura FFT (oracle/_ref), for a set of
  lattice shapes / seeds.  Pins the numpy oracle and the engine's host generator.
* ``philox_kat.json`` — Philox4x32-10 known-answer vectors published with Random123 (SC'11).
* ``ref_runs.json`` — excerpts of the reference's own production outputs under data/raw
  (cfen, cfpt, per-configuration cfxy / cfnd rows, run_meta parameters) used as statistical pins.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import glob
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
REFERENCE = os.environ.get("REFERENCE", os.path.join(os.path.dirname(ROOT), "reference"))

from oracle import oracle as O  # noqa: E402

CORR_CASES = [  # (n1, n2, n3, xi, seed, do_uniform, max_value, stride)
    (4, 4, 2, 3.0, 1, True, 2.0, 1),
    (8, 8, 8, 3.0, 7, False, 2.0, 1),
    (10, 10, 10, 3.0, 101, True, 2.0, 1),
    (12, 12, 6, 1.5, 5, True, 1.0, 1),
    (16, 16, 16, 3.0, 1, True, 2.0, 1),
    (24, 24, 24, 3.0, 2, True, 2.0, 3),
    (32, 32, 32, 3.0, 1, True, 2.0, 5),
]


def make_corr3d():
    out = {}
    for n1, n2, n3, xi, seed, uni, mx, stride in CORR_CASES:
        x = O.ref_corr_rand_3d(n1, n2, n3, xi, seed, uni, mx).reshape(-1)
        key = f"L{n1}x{n2}x{n3}_xi{xi}_s{seed}_u{int(uni)}_m{mx}"
        out[key + "__stride"] = np.array([stride])
        out[key + "__values"] = x[::stride].copy()
        out[key + "__sum"] = np.array([x.sum(), (x * x).sum()])
    np.savez_compressed(os.path.join(HERE, "corr3d_golden.npz"), **out)


def make_philox():
    kat = [
        {"ctr": [0, 0, 0, 0], "key": [0, 0],
         "out": [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]},
        {"ctr": [0xffffffff] * 4, "key": [0xffffffff] * 2,
         "out": [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]},
        {"ctr": [0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], "key": [0xa4093822, 0x299f31d0],
         "out": [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]},
    ]
    with open(os.path.join(HERE, "philox_kat.json"), "w") as f:
        json.dump(kat, f, indent=1)


def _meta(path):
    d = {}
    for line in open(path):
        if ":" in line and line.startswith("  "):
            k, v = line.strip().split(":", 1)
            d[k.strip()] = v.strip()
        elif line.startswith("duration_s:"):
            d["duration_s"] = line.split(":", 1)[1].strip()
    return d


def _table(path, skip_header_until=None, ncols=None):
    rows = []
    started = skip_header_until is None
    for line in open(path):
        if not started:
            if skip_header_until in line:
                started = True
            continue
        parts = line.split()
        try:
            vals = [float(v) for v in parts]
        except ValueError:
            continue
        if ncols is None or len(vals) == ncols:
            rows.append(vals)
    return rows


def make_ref_runs():
    base = os.path.join(REFERENCE, "data/raw/corr_random_field/p2/c3")
    runs = {}
    for d in sorted(glob.glob(os.path.join(base, "J2-1_P0.00_RAN_*_s100_scanpt_prod_main*/L10"))):
        meta = _meta(os.path.join(d, "run_meta.txt"))
        if meta.get("IRINIT") not in ("1", "101"):
            continue
        name = os.path.relpath(d, os.path.join(REFERENCE, "data/raw"))
        tag = f"L10_{meta['START']}{meta.get('STRAXIS', '')}_IRINIT{meta['IRINIT']}"
        cfen = _table(glob.glob(os.path.join(d, "cfen*.dat"))[0], "[<energy>]", 5)
        cfpt = _table(glob.glob(os.path.join(d, "cfpt*.dat"))[0], "pair,", 6)
        cfxy = _table(glob.glob(os.path.join(d, "cfxy*.dat"))[0], "iconf,", 10)
        cfnd = _table(glob.glob(os.path.join(d, "cfnd*.dat"))[0], "iconf,", None)
        runs[tag] = {"source": name, "params": meta, "cfen": cfen, "cfpt": cfpt,
                     "cfxy_first10": [r for r in cfxy if r[0] <= 10],
                     "cfnd_first10": [r for r in cfnd if r and r[0] <= 10]}
    d = os.path.join(base, "J2-1_P0.00_RAN_STRX_s100_scanpt_prod_main/L24")
    if os.path.isdir(d):
        meta = _meta(os.path.join(d, "run_meta.txt"))
        runs["L24_STRX_main"] = {
            "source": os.path.relpath(d, os.path.join(REFERENCE, "data/raw")), "params": meta,
            "cfen": _table(glob.glob(os.path.join(d, "cfen*.dat"))[0], "[<energy>]", 5),
            "cfpt": _table(glob.glob(os.path.join(d, "cfpt*.dat"))[0], "pair,", 6)}
    with open(os.path.join(HERE, "ref_runs.json"), "w") as f:
        json.dump(runs, f, separators=(",", ":"))


if __name__ == "__main__":
    if not os.path.isdir(REFERENCE):
        sys.exit("reference tree not found; the committed fixtures stay as they are")
    O.build(ref=True)
    make_corr3d()
    make_philox()
    make_ref_runs()
    for f in sorted(os.listdir(HERE)):
        print(f, os.path.getsize(os.path.join(HERE, f)))
