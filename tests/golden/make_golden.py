"""Generates the golden fixtures in this directory from the reference's own code.

Run where the reference sources are available (they are compiled by
``oracle/Makefile`` target ``ref`` into ``oracle/_ref/libidgref.so``):

    python tests/golden/make_golden.py

For each case it stores the reference's synthetic inputs (``srand(0)``
sequence of gridding/src/gridding_benchmark.cpp:203-213), the output of
``gridding_benchmark_launcher<cpu>::launch`` on them, and the output of
``degridding_benchmark_launcher<cpu>::launch`` on the reference's
``initialize_subgrids`` pattern.  The fixtures pin the float oracle bit for
bit and the product's reference-compatible generator value for value.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "oracle"))

import oracle as O  # noqa: E402

# (grid_size, subgrid_size, nstations, nchannels, ntimeslots, ntimesteps_per_subgrid)
CASES = {
    "ref_g1024_s32_ns3_c8_ts2_t32": (1024, 32, 3, 8, 2, 32),
    "ref_g512_s16_ns4_c5_ts1_t20": (512, 16, 4, 5, 1, 20),
    "ref_g256_s24_ns2_c3_ts3_t7": (256, 24, 2, 3, 3, 7),
}


def main() -> None:
    O.build(with_ref=True)
    for name, cfg in CASES.items():
        d = O.ref_dataset(*cfg)
        sub, _ = O.ref_cpu_gridding(cfg, d)
        nsg = d["metadata"].shape[0]
        sg_in = O.ref_subgrids(nsg, cfg[1])
        vis_out, _ = O.ref_cpu_degridding(cfg, d, sg_in)
        np.savez_compressed(
            os.path.join(HERE, name + ".npz"),
            cfg=np.array(cfg, np.int64),
            uvw=d["uvw"], frequencies=d["frequencies"], wavenumbers=d["wavenumbers"], vis=d["vis"],
            baselines=d["baselines"], spheroidal=d["spheroidal"], aterms=d["aterms"],
            metadata=d["metadata"].view(np.int32).reshape(-1, 9),
            gridder_out=sub, degridder_in=sg_in, degridder_out=vis_out,
        )
        print(f"wrote {name}.npz")


if __name__ == "__main__":
    main()
