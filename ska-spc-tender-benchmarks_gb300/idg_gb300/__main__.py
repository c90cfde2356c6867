"""``python -m idg_gb300 <configuration file> <output file>``

The gridding benchmark driver (gridding/src/main.cpp:15-163): prints the
configuration table, runs a warm-up of the first configuration, runs every
configuration, prints the 12-column result table and writes the CSV.
"""
from __future__ import annotations

import sys
import time

from . import config as _config
from .launcher import launch_degridding, launch_gridding, operation_type


def run(configurations, output: str) -> list:
    print("##################################################")
    print("#### Gridding/degridding benchmarking utility ####")
    print("##################################################\n")
    print("##################################################")
    print("## Benchmarking configurations\n")
    table = [["Configuration ID", "  Operation", "  Grid size", "  Subgrid size", "  Number of channels",
              "  Number of stations", "  Hardware"]]
    for i, c in enumerate(configurations):
        table.append([str(i), c.operation.value, str(c.grid_size), str(c.subgrid_size), str(c.nchannels),
                      str(c.nstations), c.htype.value])
    _config.print_columns(table)
    print()
    print("##############")
    print("## Warmup step\n")
    t0 = time.time()
    launch_gridding(configurations[0])
    warm = int(time.time() - t0)
    print(f"Warming up… Done in {warm} seconds.")
    print(f"==> Total benchmark should take a bit more than {round(len(configurations) * warm)} seconds.\n")
    print("###############")
    print("## Benchmarking\n")
    results = []
    t_all = time.time()
    for i, c in enumerate(configurations):
        print(f"Running configuration {i}… ", end="", flush=True)
        t1 = time.time()
        r = launch_gridding(c) if c.operation == operation_type.gridding else launch_degridding(c)
        results.append(r)
        print(f"Done in {int(time.time() - t1)} seconds.")
    print(f"==> Total benchmarking time: {int(time.time() - t_all)} seconds.\n")
    rows = _config.result_rows(configurations, results)
    _config.print_columns(rows)
    _config.write_csv(output, rows)
    return results


def main(argv=None) -> int:
    argv = sys.argv[1:] if argv is None else argv
    if len(argv) < 2:
        print("gridding-benchmarks <configuration file> <output file>", file=sys.stderr)
        return 255
    try:
        cfgs = _config.read_configuration(argv[0])
    except _config.ConfigError as e:
        print("Error while reading configurations file:", file=sys.stderr)
        print(f"Error: {e}", file=sys.stderr)
        return 255
    run(cfgs, argv[1])
    return 0


if __name__ == "__main__":
    sys.exit(main())
