"""Host logic: YAML configuration, result table / CSV format, synthetic
observations and the uvw-driven plan.  CPU only."""
import os

import numpy as np
import pytest

from conftest import ROOT


def _load_bench(name: str):
    """bench.py imported as a module (it is a script at the repo root)."""
    import importlib.util

    spec = importlib.util.spec_from_file_location(name, os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_yaml_subset_parses_reference_examples(idg, tmp_path):
    from idg_gb300 import config as C

    text = """grid_size: 1024
operation_types: [gridding, degridding]
niterations: 100
nstations: 2
ntimeslots: 2
ntimesteps_per_subgrid: 128
nchannels: 16
subgrid_size: 32
hardware_types: [gpu]
"""
    p = tmp_path / "example.yaml"
    p.write_text(text)
    cfgs = C.read_configuration(str(p))
    assert [c.operation.value for c in cfgs] == ["gridding", "degridding"]
    c = cfgs[0]
    assert (c.grid_size, c.niterations, c.nstations, c.ntimeslots, c.ntimesteps_per_subgrid, c.nchannels,
            c.subgrid_size) == (1024, 100, 2, 2, 128, 16, 32)
    assert c.image_size == pytest.approx(0.1) and c.w_step == 0.0


def test_yaml_block_lists_and_comments(idg, tmp_path):
    from idg_gb300 import config as C

    y = C.parse_yaml_subset("a: 3  # comment\nhardware_types:\n  - gpu\n  - gpu\nb: [x, 'y']\n")
    assert y == {"a": 3, "hardware_types": ["gpu", "gpu"], "b": ["x", "y"]}


@pytest.mark.parametrize(
    "body, message",
    [
        ("operation_types: [gridding]\n", "hardware_types section empty."),
        ("hardware_types: [tpu]\noperation_types: [gridding]\n", "Invalid hardware_type token tpu"),
        ("hardware_types: [cpu]\noperation_types: [gridding]\n", "CPU support is disabled"),
        ("hardware_types: [gpu]\n", "operation_types section empty."),
        ("hardware_types: [gpu]\noperation_types: [fft]\n", "Invalid operation type token fft"),
        ("hardware_types: [gpu]\noperation_types: [gridding]\n", "Invalid grid_size section"),
    ],
)
def test_config_errors(idg, tmp_path, body, message):
    from idg_gb300 import config as C

    p = tmp_path / "bad.yaml"
    p.write_text(body)
    with pytest.raises(C.ConfigError) as e:
        C.read_configuration(str(p))
    assert message in str(e.value)


def test_missing_file(idg):
    from idg_gb300 import config as C

    with pytest.raises(C.ConfigError, match="not found"):
        C.read_configuration("/nonexistent/x.yaml")


def test_csv_and_table_format(idg, tmp_path, monkeypatch):
    from idg_gb300 import config as C
    from idg_gb300 import launcher as L

    cfg = L.configuration(niterations=3)
    r = L.benchmark_result(in_transfer_time=12.5, compute_time=100.0)
    rows = C.result_rows([cfg], [r])
    assert rows[0] == C.RESULT_LABELS and len(rows[0]) == 12
    assert rows[1][:3] == ["0", "gridding", "3"]
    assert rows[1][7] == "12.500000" and rows[1][8] == "N/A" and rows[1][9] == "100.000000"
    monkeypatch.chdir(tmp_path)
    written = C.write_csv(os.path.join("some", "dir", "out.csv"), rows)
    assert written == "out.csv"
    lines = (tmp_path / "out.csv").read_text().split("\n")
    assert lines[0].endswith(";") and lines[0].count(";") == 12
    assert lines[1].startswith("0;gridding;3;")
    assert lines[-1] == ""


def test_observation_geometry_and_plan(idg):
    from idg_gb300 import datasets as D

    spec = D.config1()
    obs = D.make_observation(spec)
    assert obs.uvw.shape == (spec.n_rows, 3) and obs.uvw.dtype == np.float32
    assert spec.n_baselines == 28 and spec.n_subgrids == 28 and spec.n_visibilities == 28672
    # baseline lengths within the disk diameter; w non-zero (earth rotation at dec -30)
    assert np.linalg.norm(obs.uvw, axis=1).max() <= 2 * spec.disk_radius_m + 1e-3
    assert np.abs(obs.uvw[:, 2]).max() > 1.0
    # plan: every subgrid inside the grid and its uv extent fits with room for the taper
    md = obs.metadata
    S, G = spec.subgrid_size, spec.grid_size
    assert (md["x"] >= 0).all() and (md["x"] + S <= G).all() and (md["y"] >= 0).all() and (md["y"] + S <= G).all()
    assert D.uv_extent_pixels(spec, obs.uvw, obs.frequencies).max() < S - 8
    # the subgrid centre sits on the visibilities' uv centre (within half a cell)
    u = obs.uvw[:, 0].reshape(spec.n_baselines, -1).astype(np.float64)
    f = obs.frequencies
    u_lam = np.concatenate([u * f[0], u * f[-1]], axis=1) / D.SPEED_OF_LIGHT
    mid = 0.5 * (u_lam.min(1) + u_lam.max(1))
    centre = (md["x"] + S / 2 - G / 2) / spec.image_size
    assert np.all(np.abs(centre - mid) <= 0.5 / spec.image_size + 1e-6)
    # taper: separable, peak 1, small at the edges
    t = obs.taper
    assert t.shape == (S, S) and abs(t.max() - 1) < 1e-6 and t[0, 0] < 1e-3
    assert np.allclose(t, np.outer(t[S // 2], t[S // 2]) / t[S // 2, S // 2], atol=1e-6)


def test_config2_sizes(idg):
    from idg_gb300 import datasets as D

    spec = D.config2()
    assert spec.n_baselines == 4950
    assert spec.n_subgrids == 316800
    assert spec.n_visibilities == 648806400
    assert spec.n_aterm_slots == 32


def test_plan_is_deterministic(idg):
    from idg_gb300 import datasets as D

    a = D.make_observation(D.config1())
    b = D.make_observation(D.config1())
    assert np.array_equal(a.metadata.view(np.uint8), b.metadata.view(np.uint8))
    assert np.array_equal(a.uvw, b.uvw)


@pytest.mark.parametrize("S", [32, 64])
def test_split_plan_covers_every_sample_once_and_fits(idg, S):
    """The channel/time-splitting planner (long baselines, wide bands): every
    (baseline, timestep, channel) sample in exactly one subgrid, every subgrid's
    uv extent within S - S/4 cells, subgrids inside the grid, no subgrid across
    an A-term slot boundary, and the same plan from the same seed."""
    from idg_gb300 import datasets as D

    spec = D.config3(S, nstations=8, ntimesteps=512)
    obs = D.make_observation(spec, split=True)
    md, ext = obs.metadata, obs.ext
    assert md.shape == ext.shape and md.shape[0] > spec.n_baselines * (spec.ntimesteps // spec.timesteps_per_subgrid)
    count = np.zeros((obs.uvw.shape[0], spec.nchannels), np.int32)
    for m, e in zip(md, ext):
        count[m["time_offset"]:m["time_offset"] + m["nr_timesteps"], e["channel_begin"]:e["channel_end"]] += 1
    assert np.all(count == 1)
    assert D.subgrid_uv_extent(spec, obs.uvw, obs.frequencies, md, ext).max() <= S - S // 4
    G = spec.grid_size
    assert (md["x"] >= 0).all() and (md["x"] + S <= G).all() and (md["y"] >= 0).all() and (md["y"] + S <= G).all()
    t_in_bl = md["time_offset"] % spec.ntimesteps
    assert np.all(t_in_bl // spec.aterm_interval == (t_in_bl + md["nr_timesteps"] - 1) // spec.aterm_interval)
    assert np.all(md["aterm_index"] == t_in_bl // spec.aterm_interval)
    assert np.all(md["nr_timesteps"] <= spec.timesteps_per_subgrid)
    again = D.make_observation(spec, split=True)
    assert np.array_equal(again.metadata, md) and np.array_equal(again.ext, ext)


def test_split_plan_w_planes(idg):
    """w-stacking in the split planner: each subgrid's z is floor(w_mid / w_step),
    w_mid the centre of the w extent (wavelengths) of all its samples, clipped
    to [-W, W-1]; both signs occur; w_step = 0 leaves every z at 0 and the rest
    of the plan unchanged."""
    import dataclasses

    from idg_gb300 import datasets as D

    spec = D.ObservationSpec(nstations=8, disk_radius_m=2500.0, ntimesteps=256, timesteps_per_subgrid=64,
                             nchannels=16, f_start=140e6, f_end=170e6, subgrid_size=32, grid_size=512,
                             image_size=0.04, w_step=300.0, nr_w_planes=4, aterm_interval=128, dec_deg=20.0, seed=5)
    obs = D.make_observation(spec, split=True)
    md, ext = obs.metadata, obs.ext
    W, w_step = spec.nr_w_planes, float(np.float32(spec.w_step))
    f = obs.frequencies.astype(np.float64)
    want = np.empty(md.shape[0], np.int64)
    for i, (m, e) in enumerate(zip(md, ext)):
        r = slice(int(m["time_offset"]), int(m["time_offset"]) + int(m["nr_timesteps"]))
        wl = obs.uvw[r, 2].astype(np.float64)[:, None] * f[None, e["channel_begin"]:e["channel_end"]] / D.SPEED_OF_LIGHT
        want[i] = min(max(np.floor(0.5 * (wl.min() + wl.max()) / w_step), -W), W - 1)
    assert np.array_equal(md["z"], want)
    assert (md["z"] < 0).any() and (md["z"] >= 0).any()
    flat = D.make_observation(dataclasses.replace(spec, w_step=0.0), split=True)
    assert np.all(flat.metadata["z"] == 0)
    rest = [n for n in md.dtype.names if n != "z"]
    assert np.array_equal(flat.metadata[rest], md[rest]) and np.array_equal(flat.ext, ext)


def test_cpu_baseline_sample_stays_within_the_given_rows(idg):
    """The bench's CPU baseline sizes its sample from the measured time per
    subgrid; however fast the host, the sample only uses subgrids whose rows
    are all in the visibilities it was given (a faster host once read past
    them)."""
    bench = _load_bench("bench_under_test")
    from idg_gb300 import datasets as D

    spec = D.config1()
    obs = D.make_observation(spec)
    T = spec.timesteps_per_subgrid
    vis = np.zeros((5 * T + T // 2, spec.nchannels, 4), np.complex64)  # 5 whole subgrids and part of a sixth
    out = bench.cpu_baseline(obs, vis, 1000.0)
    assert out["sample"].startswith("first 5 of ")


def test_e2e_leg_fits_the_host_memory(idg):
    """bench.py's e2e leg pins the visibilities in and out per rank; with too
    little host memory for all ranks of a node it takes the leading subgrids
    whose rows fit (whole plan otherwise)."""
    bench = _load_bench("bench_under_test2")
    from idg_gb300 import datasets as D

    spec = D.config1()
    obs = D.make_observation(spec)
    row = 2 * spec.nchannels * 32
    assert bench.e2e_prefix(obs.metadata, spec.n_rows, row, 1e18) == (spec.n_subgrids, spec.n_rows)
    T = spec.timesteps_per_subgrid
    n, rows = bench.e2e_prefix(obs.metadata, spec.n_rows, row, (3 * T + T // 2) * row)
    assert (n, rows) == (3, 3 * T)
    assert bench.e2e_prefix(obs.metadata, spec.n_rows, row, 1.0)[0] == 1


def test_hostmem_arrays_without_registration():
    """idg_gb300.hostmem on a host without a GPU: the huge-page-advised mapping
    gives zeroed C-contiguous arrays of any dtype and shape; release() of an
    array that was never registered is a no-op."""
    from idg_gb300 import hostmem
    import idg_gb300._lib as L

    a = hostmem.pinned_empty((3, 5, 4), np.complex64, register=False)
    assert a.shape == (3, 5, 4) and a.dtype == np.complex64 and a.flags["C_CONTIGUOUS"] and a.flags["WRITEABLE"]
    assert not a.any()
    a[...] = 1 + 2j
    assert (a == 1 + 2j).all()
    md = np.zeros(7, L.METADATA_DTYPE)
    md["nr_timesteps"] = np.arange(7)
    b = hostmem.pinned_copy(md, register=False)
    assert b.dtype == L.METADATA_DTYPE and (b["nr_timesteps"] == np.arange(7)).all()
    assert np.ascontiguousarray(b, dtype=L.METADATA_DTYPE) is b  # passed to the C ABI without a copy
    e = hostmem.pinned_empty(0, np.float32, register=False)
    assert e.shape == (0,)
    for x in (a, b, e, a[1:]):
        hostmem.release(x)


def test_reference_arm_line(idg, monkeypatch):
    """bench.py --impl reference: rank 0 returns one line with the contract's
    keys (impl, value, zero copy bytes in its e2e block, a cpu_baseline that
    describes the run); the other ranks return nothing.  The CPU sample is cut
    to 0.2 s per half here."""
    import argparse
    import json

    bench = _load_bench("bench_under_test3")
    real = bench.cpu_baseline
    monkeypatch.setattr(bench, "cpu_baseline", lambda obs, vis, target_s, build="-O2": real(obs, vis, 0.2, build))
    args = argparse.Namespace(workload="config1", steps=2, warmup=1, no_ref_gpu=False)
    out = bench.run_reference(args, 0, 1)
    json.dumps(out)
    assert out["impl"] == "reference" and out["unit"] == "Mvis/s" and out["value"] > 0
    assert out["higher_is_better"] is True and out["steps"] == 2 and out["warmup"] == 1
    assert out["e2e"] == {"value": out["value"], "unit": "Mvis/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    cb = out["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == out["value"] and cb["sample"]
    assert out["config"]["workload"].startswith("config1")
    # the port as the reference's CMake builds it (-g, no optimisation) and at -O3, beside -O2
    assert set(out["cpu_builds_mvis_per_s"]) == {"-O2", "-O3", "-O0 -g"}
    assert all(v > 0 for v in out["cpu_builds_mvis_per_s"].values())
    # without a GPU (or cubins, or within the kernels' limits) the reference kernels' leg says why
    assert "unavailable" in out["reference_gpu"]
    assert bench.run_reference(args, 1, 2) is None
