"""YAML configuration and CSV/table output of the gridding benchmark.

Keys, validation messages and the hardware x operation cross product follow
gridding/src/gridding_configuration.cpp:10-144; the table and the
';'-separated CSV follow gridding/src/main.cpp:91-136 and
benchmarks-common/inc/benchmarks_common.h:48-87.  yaml-cpp is not available,
so the reader accepts the YAML subset the benchmark's files use: ``key: value``
scalars, flow sequences ``[a, b]``, block sequences (``- a``) and ``#``
comments.  Extra keys beyond the reference's (``image_size``, ``w_step``,
``variant``) are optional and default to the reference's hard-coded values.
"""
from __future__ import annotations

import os
import sys

from .launcher import configuration, hardware_type, operation_type
from . import _lib


class ConfigError(RuntimeError):
    pass


def _scalar(tok: str):
    tok = tok.strip()
    if len(tok) >= 2 and tok[0] == tok[-1] and tok[0] in "'\"":
        return tok[1:-1]
    for conv in (int, float):
        try:
            return conv(tok)
        except ValueError:
            pass
    return tok


def parse_yaml_subset(text: str) -> dict:
    out: dict = {}
    current_list_key = None
    for raw in text.splitlines():
        line = raw.split("#", 1)[0].rstrip()
        if not line.strip():
            continue
        stripped = line.strip()
        if stripped.startswith("- ") or stripped == "-":
            if current_list_key is None:
                raise ConfigError(f"sequence item outside a key: {raw!r}")
            out[current_list_key].append(_scalar(stripped[1:]))
            continue
        if ":" not in stripped:
            raise ConfigError(f"cannot parse line: {raw!r}")
        key, val = stripped.split(":", 1)
        key, val = key.strip(), val.strip()
        if val == "":
            out[key] = []
            current_list_key = key
            continue
        current_list_key = None
        if val.startswith("["):
            if not val.endswith("]"):
                raise ConfigError(f"unterminated flow sequence for {key}")
            inner = val[1:-1].strip()
            out[key] = [_scalar(t) for t in inner.split(",")] if inner else []
        else:
            out[key] = _scalar(val)
    return out


def _abort(message: str):
    """benchmarks_common::log_and_abort: 'Error: <message>' on stderr, exit(-1)."""
    raise ConfigError(message)


def read_configuration(path: str) -> list[configuration]:
    if not os.path.exists(path):
        raise ConfigError(f"File {path} not found.")
    with open(path) as f:
        y = parse_yaml_subset(f.read())

    htypes_cfg = y.get("hardware_types") or []
    if not isinstance(htypes_cfg, list):
        htypes_cfg = [htypes_cfg]
    if len(htypes_cfg) == 0:
        _abort("hardware_types section empty.")
    htypes = []
    for h in htypes_cfg:
        if h == "gpu":
            htypes.append(hardware_type.gpu)
        elif h == "cpu":
            _abort("CPU support is disabled")
        else:
            _abort(f"Invalid hardware_type token {h} was found. Must be either cpu or gpu.")

    ops_cfg = y.get("operation_types") or []
    if not isinstance(ops_cfg, list):
        ops_cfg = [ops_cfg]
    if len(ops_cfg) == 0:
        _abort("operation_types section empty.")
    ops = []
    for o in ops_cfg:
        if o == "gridding":
            ops.append(operation_type.gridding)
        elif o == "degridding":
            ops.append(operation_type.degridding)
        else:
            _abort(f"Invalid operation type token {o} was found. Must be either gridding or degridding.")

    def need(key: str, what: str) -> int:
        if key not in y:
            _abort(f"Invalid {key} section. Should look like this:\n  nbatches: <{what}>")
        v = y[key]
        if not isinstance(v, int) or v < 0:
            _abort(f"Invalid {key} value {v!r}")
        return v

    grid_size = need("grid_size", "grid size")
    subgrid_size = need("subgrid_size", "subgrid size")
    niterations = need("niterations", "niterations")
    nstations = need("nstations", "number of stations")
    nchannels = need("nchannels", "number of channels")
    ntimeslots = need("ntimeslots", "number of time slots")
    ntimesteps = need("ntimesteps_per_subgrid", "number of time steps per subgrid")
    image_size = float(y.get("image_size", 0.1))
    w_step = float(y.get("w_step", 0.0))
    variant = {"plain": _lib.VARIANT_PLAIN, "batched": _lib.VARIANT_BATCHED}.get(str(y.get("variant", "plain")))
    if variant is None:
        _abort(f"Invalid variant {y.get('variant')!r}: must be plain or batched")

    cfgs = []
    for h in htypes:
        for o in ops:
            cfgs.append(configuration(htype=h, operation=o, niterations=niterations, grid_size=grid_size,
                                      subgrid_size=subgrid_size, nstations=nstations, nchannels=nchannels,
                                      ntimeslots=ntimeslots, ntimesteps_per_subgrid=ntimesteps,
                                      image_size=image_size, w_step=w_step, variant=variant))
    return cfgs


RESULT_LABELS = [
    "  Configuration ID",
    "  Operation",
    "  Iterations",
    "  Grid size",
    "  Subgrid size",
    "  Number of channels",
    "  Number of stations",
    "  Mean input transfer time (us)",
    "  Achieved input bandwidth (MiB/s)",
    "  Mean compute time (us)",
    "  Mean output transfer time (us)",
    "  Achieved output bandwidth (MiB/s)",
]


def to_result_string(x: float) -> str:
    """main.cpp:108: N/A for negatives, else std::to_string (6 decimals)."""
    return "N/A" if x < 0.0 else f"{x:.6f}"


def result_rows(cfgs, results) -> list[list[str]]:
    rows = [list(RESULT_LABELS)]
    for i, (c, r) in enumerate(zip(cfgs, results)):
        rows.append([str(i), c.operation.value, str(c.niterations), str(c.grid_size), str(c.subgrid_size),
                     str(c.nchannels), str(c.nstations), to_result_string(r.in_transfer_time),
                     to_result_string(r.in_bandwidth), to_result_string(r.compute_time),
                     to_result_string(r.out_transfer_time), to_result_string(r.out_bandwidth)])
    return rows


def print_columns(rows, out=sys.stdout) -> None:
    """benchmarks_common.h:48-71: right-aligned columns, one space after each."""
    n = len(rows[0])
    width = [max(len(r[i]) for r in rows) for i in range(n)]
    for r in rows:
        out.write("".join(r[i].rjust(width[i]) + " " for i in range(n)) + "\n")
    out.flush()


def write_csv(path: str, rows) -> str:
    """benchmarks_common.h:73-87: ';' after every field, rows end with '\\n',
    written to the path's file name in the current directory.  Returns the path written."""
    target = os.path.basename(path)
    with open(target, "w") as f:
        for r in rows:
            f.write("".join(field + ";" for field in r) + "\n")
    return target
