"""Measure the tensor-core tile table on this GPU: ``python -m helios_gb300.tune``.

The exact-slice GEMM of every precision mode has a few candidate output tile
widths (``api.tile_variants``) that form the same sums and differ in speed.
Which one is fastest depends on the contraction shapes: narrow tiles waste
less on the thin operands of small molecules, wide ones reuse each operand
tile over more columns. This script creates mixed-precision handles for the
workloads the engine is run on (the 160-site polyene, the 64-site ladder and
its five-point field batch, single polyenes and ladders of 20-80 sites, and
seeded ensembles of 8-64-site molecules) with ``tile_tuning="tune"``: at
creation every (precision mode, contraction group, size class) without a
table entry times each candidate on that handle's own contractions and keeps
the fastest. The table is written to ``helios_gb300/data/tile_table.json``,
which ``api.library()`` loads, so later handles of the same size classes take
the measured choice without timing anything.
"""
from __future__ import annotations

import argparse
import time

from . import api, learned, molecules


def workloads(ensemble: int):
    yield "polyene-160", [molecules.polyene(160)]
    yield "ladder-64 x5 (field batch)", [molecules.ladder(64)] * 5
    yield "ladder-64", [molecules.ladder(64)]
    for n in (20, 24, 40, 80):
        yield f"polyene-{n}", [molecules.polyene(n)]
    yield "ladder-24", [molecules.ladder(24)]
    if ensemble:
        yield f"ensemble-{ensemble}", molecules.ensemble(learned.HELD_OUT_SEED, ensemble)
    yield "ensemble-48", molecules.ensemble(learned.HELD_OUT_SEED, 48)


def tune(ensemble: int = 512, verbose: bool = True):
    """Fill the process-wide tile table by timing the candidates; returns its entries."""
    for name, mols in workloads(ensemble):
        t0 = time.perf_counter()
        cc = api.CoupledCluster(mols, api.Keywords(bond_alternation=0.1, precision="mixed", tile_tuning="tune"))
        choices, ms = cc.tile_choices()
        cc.finalizeCC()
        if verbose:
            print(f"{name}: {ms / 1e3:.2f} s timing candidates ({time.perf_counter() - t0:.1f} s in all); "
                  f"non-default choices per mode {[int((row != 0).sum()) for row in choices]}")
    return api.tile_table()


def main():
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--ensemble", type=int, default=512, help="molecules of the largest ensemble workload")
    ap.add_argument("--out", default=api.TILE_TABLE_PATH)
    args = ap.parse_args()
    return run(args)


def run(args):
    # measure afresh: a loaded table would answer every lookup (the library is
    # loaded lazily, by the first handle below)
    api.TILE_TABLE_PATH = ""
    entries = tune(args.ensemble)
    api.write_tile_table(args.out, entries, note="measured by python -m helios_gb300.tune on one GB300")
    print(f"{len(entries)} entries -> {args.out}")


if __name__ == "__main__":
    main()
