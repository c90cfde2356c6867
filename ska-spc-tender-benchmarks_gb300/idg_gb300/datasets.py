"""Seeded synthetic observations and the uvw-driven subgrid plan.

No public data set is involved: every input is generated from a seed.

Observation model (all lengths in metres, angles in radians):

* ``nstations`` stations uniform in a disk of radius ``disk_radius_m``
  (east, north, up=0), all ``nstations*(nstations-1)/2`` baselines.
* Earth-rotation synthesis for a source at declination ``dec`` seen from
  latitude ``lat``: local (E, N, U) -> equatorial (X, Y, Z) with
  X = -sin(lat) N + cos(lat) U, Y = E, Z = cos(lat) N + sin(lat) U, then for
  hour angle H
      u =  sin H X + cos H Y
      v = -sin dec cos H X + sin dec sin H Y + cos dec Z
      w =  cos dec cos H X - cos dec sin H Y + sin dec Z
  with H advancing 7.2921159e-5 rad per second over ``ntimesteps`` integrations
  of ``integration_s`` seconds, centred on transit.
* ``nchannels`` channels linearly spaced from ``f_start`` to ``f_end``;
  wavenumbers k = 2 pi f / c in float32.
* A-terms: identity, or identity + ``aterm_sigma`` * complex N(0, 1), a new
  draw every ``aterm_interval`` timesteps (one A-term slot per interval).
* Taper: prolate spheroidal wave function psi_0(c, x) with c = 3 pi, separable
  in x and y, peak 1.
* Visibilities: real and imaginary parts N(0, 1) (generated on the device by
  ``visibilities()`` for the large configurations).

Plan: each baseline's time axis is cut into subgrids of
``timesteps_per_subgrid`` consecutive integrations covering all channels; a
subgrid's corner is placed so that its centre cell holds the centre of the
uv extent of its visibilities (in wavelengths, over all its channels):
``x = floor(u_mid * image_size + G/2 - S/2 + 1/2)``, the same for ``y``.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from ._lib import METADATA_DTYPE

SPEED_OF_LIGHT = 299792458.0
EARTH_ROTATION_RATE = 7.2921159e-5  # rad / s


@dataclass
class ObservationSpec:
    nstations: int
    disk_radius_m: float
    ntimesteps: int            # integrations per baseline
    timesteps_per_subgrid: int
    nchannels: int
    f_start: float
    f_end: float
    subgrid_size: int
    grid_size: int
    image_size: float
    w_step: float = 0.0
    integration_s: float = 1.0
    dec_deg: float = -30.0
    lat_deg: float = -30.0
    aterm_sigma: float = 0.0   # 0 -> identity A-terms
    aterm_interval: int = 0    # timesteps per A-term slot (0 -> one slot)
    seed: int = 1234
    taper_c: float = 3.0 * np.pi
    subgrid_limit: int = 0     # > 0: only the plan's first subgrid_limit subgrids (and their rows) are used
    nr_w_planes: int = 1       # w-stacking (split plans, w_step > 0): planes 0..W-1, negative w mirrored

    @property
    def n_baselines(self) -> int:
        return self.nstations * (self.nstations - 1) // 2

    @property
    def subgrids_per_baseline(self) -> int:
        return self.ntimesteps // self.timesteps_per_subgrid

    @property
    def n_subgrids(self) -> int:
        n = self.n_baselines * self.subgrids_per_baseline
        return min(n, self.subgrid_limit) if self.subgrid_limit > 0 else n

    @property
    def n_rows(self) -> int:
        if self.subgrid_limit > 0:
            last = self.n_subgrids - 1
            bl, ts = divmod(last, self.subgrids_per_baseline)
            return bl * self.ntimesteps + (ts + 1) * self.timesteps_per_subgrid
        return self.n_baselines * self.ntimesteps

    @property
    def n_aterm_slots(self) -> int:
        if self.aterm_interval <= 0:
            return 1
        return (self.ntimesteps + self.aterm_interval - 1) // self.aterm_interval

    @property
    def n_visibilities(self) -> int:
        return self.n_subgrids * self.timesteps_per_subgrid * self.nchannels


# The BASELINE configurations of this benchmark (sizes as specified there).
def config1(seed: int = 1) -> ObservationSpec:
    """8 stations in a 3 km disk, 64 x 1 s, 16 ch 150-160 MHz, identity A-terms, S=32, G=512, 0.05 rad.

    "An N km disk" is read as a disk N km across, so the longest baseline is N km."""
    return ObservationSpec(nstations=8, disk_radius_m=1500.0, ntimesteps=64, timesteps_per_subgrid=64,
                           nchannels=16, f_start=150e6, f_end=160e6, subgrid_size=32, grid_size=512,
                           image_size=0.05, seed=seed)


def config2(seed: int = 2) -> ObservationSpec:
    """100 stations in a 10 km disk, 8192 x 1 s in 128-step subgrids, 16 ch, near-identity A-terms
    renewed every 256 steps, S=32, G=4096, 0.05 rad: 4950 baselines, 316,800 subgrids, 6.49e8 visibilities."""
    return ObservationSpec(nstations=100, disk_radius_m=5000.0, ntimesteps=8192, timesteps_per_subgrid=128,
                           nchannels=16, f_start=150e6, f_end=160e6, subgrid_size=32, grid_size=4096,
                           image_size=0.05, aterm_sigma=0.05, aterm_interval=256, seed=seed)


@dataclass
class Observation:
    spec: ObservationSpec
    stations: np.ndarray     # [ns, 3] ENU metres
    baselines: np.ndarray    # [nb, 2] uint32
    uvw: np.ndarray          # [nb*nt, 3] float32
    frequencies: np.ndarray  # [C] float64
    wavenumbers: np.ndarray  # [C] float32
    aterms: np.ndarray       # [slots, ns, S, S, 4] complex64
    taper: np.ndarray        # [S, S] float32
    metadata: np.ndarray     # [N] METADATA_DTYPE
    ext: np.ndarray | None = None  # [N] SUBGRID_EXT_DTYPE channel ranges (split plans only)


def stations_in_disk(n: int, radius: float, rng: np.random.Generator) -> np.ndarray:
    r = radius * np.sqrt(rng.random(n))
    th = 2 * np.pi * rng.random(n)
    return np.stack([r * np.cos(th), r * np.sin(th), np.zeros(n)], axis=1)


def baseline_pairs(n: int) -> np.ndarray:
    i, j = np.triu_indices(n, k=1)
    return np.stack([i, j], axis=1).astype(np.uint32)


def earth_rotation_uvw(enu: np.ndarray, hour_angles: np.ndarray, dec: float, lat: float) -> np.ndarray:
    """uvw [nb, nt, 3] (float64) for baseline vectors enu [nb, 3]."""
    E, N, U = enu[:, 0], enu[:, 1], enu[:, 2]
    X = -np.sin(lat) * N + np.cos(lat) * U
    Y = E
    Z = np.cos(lat) * N + np.sin(lat) * U
    sH, cH = np.sin(hour_angles)[None, :], np.cos(hour_angles)[None, :]
    sd, cd = np.sin(dec), np.cos(dec)
    X, Y, Z = X[:, None], Y[:, None], Z[:, None]
    u = sH * X + cH * Y
    v = -sd * cH * X + sd * sH * Y + cd * Z
    w = cd * cH * X - cd * sH * Y + sd * Z
    return np.stack([u, v, w], axis=-1)


def pswf_taper(S: int, c: float = 3.0 * np.pi) -> np.ndarray:
    """Separable prolate spheroidal taper psi_0(c, x) psi_0(c, y), peak 1."""
    from scipy.special import pro_ang1

    x = (np.arange(S) + 0.5 - S / 2) / (S / 2)
    psi = np.array([pro_ang1(0, 0, c, xi)[0] for xi in x])
    psi = psi / np.max(np.abs(psi))
    return np.outer(psi, psi).astype(np.float32)


def plan_subgrids(spec: ObservationSpec, uvw: np.ndarray, frequencies: np.ndarray, baselines: np.ndarray) -> np.ndarray:
    """uvw-driven plan (see the module docstring); returns METADATA_DTYPE[N]."""
    nb, nt, T = spec.n_baselines, spec.ntimesteps, spec.timesteps_per_subgrid
    nsub = spec.subgrids_per_baseline
    S, G = spec.subgrid_size, spec.grid_size
    u = uvw[:, 0].astype(np.float64).reshape(nb, nt)[:, : nsub * T].reshape(nb, nsub, T)
    v = uvw[:, 1].astype(np.float64).reshape(nb, nt)[:, : nsub * T].reshape(nb, nsub, T)
    f0, f1 = float(frequencies[0]), float(frequencies[-1])

    def mid(a):
        lo = np.minimum(a.min(axis=2) * f0, a.min(axis=2) * f1) / SPEED_OF_LIGHT
        hi = np.maximum(a.max(axis=2) * f0, a.max(axis=2) * f1) / SPEED_OF_LIGHT
        return 0.5 * (lo + hi)

    x = np.floor(mid(u) * spec.image_size + G / 2 - S / 2 + 0.5).astype(np.int32)
    y = np.floor(mid(v) * spec.image_size + G / 2 - S / 2 + 0.5).astype(np.int32)
    md = np.zeros(nb * nsub, METADATA_DTYPE)
    bl = np.repeat(np.arange(nb), nsub)
    ts = np.tile(np.arange(nsub), nb)
    md["baseline_offset"] = 0
    md["time_offset"] = bl * nt + ts * T
    md["nr_timesteps"] = T
    md["aterm_index"] = (ts * T) // spec.aterm_interval if spec.aterm_interval > 0 else 0
    md["station1"] = baselines[bl, 0]
    md["station2"] = baselines[bl, 1]
    md["x"] = x.reshape(-1)
    md["y"] = y.reshape(-1)
    md["z"] = 0
    return md


def plan_subgrids_split(spec: ObservationSpec, uvw: np.ndarray, frequencies: np.ndarray, baselines: np.ndarray,
                        margin: int | None = None) -> tuple[np.ndarray, np.ndarray]:
    """uvw-driven plan with channel and time splitting, for baselines whose
    uv track over all channels and ``timesteps_per_subgrid`` steps does not
    fit one subgrid.

    Per baseline, the channels are cut into contiguous groups whose spread in
    frequency alone covers at most half the usable width (S - margin cells) at
    the baseline's longest |u| or |v|; per channel group the time axis is then
    walked and a subgrid closed when the uv extent of its visibilities (all its
    channels, all its timesteps) would exceed S - margin cells, when it holds
    ``timesteps_per_subgrid`` steps, or at an A-term slot boundary.  The corner
    is placed as in ``plan_subgrids`` (centre cell on the centre of the extent).
    Returns (metadata METADATA_DTYPE[N], ext SUBGRID_EXT_DTYPE[N] with the
    channel range [channel_begin, channel_end) of each subgrid).  Every
    (baseline, timestep, channel) sample belongs to exactly one subgrid.

    w-stacking (spec.w_step > 0): a subgrid's w-plane index is
    z = floor(w_mid / w_step), w_mid the centre of its samples' w extent in
    wavelengths, clipped to [-W, W-1] (W = spec.nr_w_planes); negative z are the
    mirrored planes of the adder.  w_step is taken at float32 precision, as
    the kernels see it."""
    from ._lib import SUBGRID_EXT_DTYPE

    nb, nt = spec.n_baselines, spec.ntimesteps
    S, G, img = spec.subgrid_size, spec.grid_size, spec.image_size
    width = S - (S // 4 if margin is None else margin)
    tmax = spec.timesteps_per_subgrid
    f = np.asarray(frequencies, np.float64)
    scale = img / SPEED_OF_LIGHT  # cells per (metre * Hz)
    w_step = float(np.float32(spec.w_step))
    W = spec.nr_w_planes
    rows_md, rows_ext = [], []
    for b in range(nb):
        u = uvw[b * nt:(b + 1) * nt, 0].astype(np.float64)
        v = uvw[b * nt:(b + 1) * nt, 1].astype(np.float64)
        w = uvw[b * nt:(b + 1) * nt, 2].astype(np.float64)
        reach = max(np.abs(u).max(), np.abs(v).max()) * scale
        # channel groups
        groups, c0 = [], 0
        for c in range(1, len(f) + 1):
            if c == len(f) or reach * (f[c] - f[c0]) > 0.5 * width:
                groups.append((c0, c))
                c0 = c
        for c0, c1 in groups:
            fa, fb = f[c0], f[c1 - 1]
            ua, ub, va, vb = u * fa * scale, u * fb * scale, v * fa * scale, v * fb * scale
            lo_u, hi_u = np.minimum(ua, ub), np.maximum(ua, ub)
            lo_v, hi_v = np.minimum(va, vb), np.maximum(va, vb)
            wa, wb = w * fa / SPEED_OF_LIGHT, w * fb / SPEED_OF_LIGHT
            lo_w, hi_w = np.minimum(wa, wb), np.maximum(wa, wb)
            t0 = 0
            while t0 < nt:
                t1 = min(nt, t0 + tmax)
                if spec.aterm_interval > 0:
                    t1 = min(t1, (t0 // spec.aterm_interval + 1) * spec.aterm_interval)
                seg = slice(t0, t1)
                ext_u = np.maximum.accumulate(hi_u[seg]) - np.minimum.accumulate(lo_u[seg])
                ext_v = np.maximum.accumulate(hi_v[seg]) - np.minimum.accumulate(lo_v[seg])
                fits = np.nonzero(np.maximum(ext_u, ext_v) > width)[0]
                n = int(fits[0]) if fits.size else t1 - t0
                n = max(n, 1)
                s = slice(t0, t0 + n)
                mid_u = 0.5 * (lo_u[s].min() + hi_u[s].max())
                mid_v = 0.5 * (lo_v[s].min() + hi_v[s].max())
                z = 0
                if w_step > 0:
                    mid_w = 0.5 * (lo_w[s].min() + hi_w[s].max())
                    z = int(min(max(np.floor(mid_w / w_step), -W), W - 1))
                rows_md.append((0, b * nt + t0, n, t0 // spec.aterm_interval if spec.aterm_interval > 0 else 0,
                                baselines[b, 0], baselines[b, 1],
                                int(np.floor(mid_u + G / 2 - S / 2 + 0.5)), int(np.floor(mid_v + G / 2 - S / 2 + 0.5)),
                                z))
                rows_ext.append((c0, c1))
                t0 += n
    md = np.array(rows_md, dtype=METADATA_DTYPE)
    ext = np.array(rows_ext, dtype=SUBGRID_EXT_DTYPE)
    return md, ext


def subgrid_uv_extent(spec: ObservationSpec, uvw: np.ndarray, frequencies: np.ndarray, md: np.ndarray,
                      ext: np.ndarray) -> np.ndarray:
    """Per subgrid of a split plan, the larger of its u and v extents in grid cells."""
    f = np.asarray(frequencies, np.float64)
    scale = spec.image_size / SPEED_OF_LIGHT
    out = np.empty(md.shape[0])
    for i, (m, e) in enumerate(zip(md, ext)):
        r = slice(int(m["time_offset"]), int(m["time_offset"]) + int(m["nr_timesteps"]))
        fr = f[int(e["channel_begin"]):int(e["channel_end"])]
        w = []
        for k in (0, 1):
            a = uvw[r, k].astype(np.float64)[:, None] * fr[None, :] * scale
            w.append(a.max() - a.min())
        out[i] = max(w)
    return out


def config3(subgrid_size: int = 32, nstations: int = 100, ntimesteps: int = 8192, seed: int = 3) -> ObservationSpec:
    """The precision-sweep generator: config 2's with baselines to 100 km, 64 channels
    100-200 MHz, subgrids of 32^2 or 64^2, an 8192^2 grid (long baselines reach
    +-3,300 cells at 200 MHz) and at most 128 timesteps per subgrid; planned with
    ``plan_subgrids_split``.  ``nstations`` / ``ntimesteps`` shrink it for tests."""
    return ObservationSpec(nstations=nstations, disk_radius_m=50000.0, ntimesteps=ntimesteps,
                           timesteps_per_subgrid=128, nchannels=64, f_start=100e6, f_end=200e6,
                           subgrid_size=subgrid_size, grid_size=8192, image_size=0.05, aterm_sigma=0.05,
                           aterm_interval=256, seed=seed)


def config3_sample(subgrid_size: int = 32, baselines_per_decile: int = 2, ntimesteps: int = 512,
                   seed: int = 3, pick_seed: int = 17):
    """A sample of the full config-3 geometry -- 100 stations in a disk 100 km
    across, 8192 x 1 s, 64 channels over 100-200 MHz -- small enough for the
    FP64 oracle: ``baselines_per_decile`` baselines drawn (seeded) from every
    decile of baseline length over all 4950 baselines, plus the longest
    baseline, each over the same window of ``ntimesteps`` steps of the 8192 (a
    seeded offset on the 256-step A-term slot grid).  The stations are those
    of ``make_observation(config3(...))`` (same seed); uvw is computed for the
    picked baselines only, and the plan is split in channel and time
    (``plan_subgrids_split``), rows numbered picked-baseline by picked-baseline.

    Returns (obs, decile, edges, lengths): ``decile`` and ``lengths`` (metres)
    per picked baseline, ``edges`` the nine decile boundaries (metres) of all
    4950 baseline lengths.  obs.spec is the full config-3 spec with
    ``ntimesteps`` = the window; its A-term table has the window's slots for all
    100 stations."""
    import dataclasses
    import types

    full = config3(subgrid_size, seed=seed)
    rng = np.random.default_rng(full.seed)
    st = stations_in_disk(full.nstations, full.disk_radius_m, rng)
    bl_all = baseline_pairs(full.nstations)
    enu_all = st[bl_all[:, 1]] - st[bl_all[:, 0]]
    length = np.linalg.norm(enu_all, axis=1)
    edges = np.quantile(length, np.linspace(0, 1, 11)[1:-1])
    dec_all = np.searchsorted(edges, length, side="right")
    prng = np.random.default_rng(pick_seed + subgrid_size)
    picks = [int(np.argmax(length))]
    for d in range(10):
        cand = np.setdiff1d(np.where(dec_all == d)[0], picks)
        picks += [int(x) for x in prng.choice(cand, min(baselines_per_decile, cand.size), replace=False)]
    picks = np.array(sorted(picks))
    interval = full.aterm_interval
    t0 = int(prng.integers(0, (full.ntimesteps - ntimesteps) // interval + 1)) * interval
    H = (np.arange(full.ntimesteps) - (full.ntimesteps - 1) / 2.0) * full.integration_s * EARTH_ROTATION_RATE
    uvw = earth_rotation_uvw(enu_all[picks], H[t0:t0 + ntimesteps], np.deg2rad(full.dec_deg), np.deg2rad(full.lat_deg))
    uvw = uvw.reshape(-1, 3).astype(np.float32)
    freqs = np.linspace(full.f_start, full.f_end, full.nchannels)
    k = (2 * np.pi * freqs / SPEED_OF_LIGHT).astype(np.float32)
    spec = dataclasses.replace(full, ntimesteps=ntimesteps)
    S = subgrid_size
    at = np.zeros((spec.n_aterm_slots, spec.nstations, S, S, 4), np.complex64)
    at[..., 0] = 1
    at[..., 3] = 1
    noise = prng.standard_normal((*at.shape, 2), dtype=np.float32)
    at += (spec.aterm_sigma * (noise[..., 0] + 1j * noise[..., 1])).astype(np.complex64)
    taper = pswf_taper(S, spec.taper_c)
    bl = bl_all[picks]
    # the planner walks len(picks) baselines of `ntimesteps` rows each
    view = types.SimpleNamespace(n_baselines=len(picks), ntimesteps=ntimesteps, subgrid_size=S,
                                 grid_size=spec.grid_size, image_size=spec.image_size,
                                 timesteps_per_subgrid=spec.timesteps_per_subgrid, w_step=spec.w_step,
                                 nr_w_planes=spec.nr_w_planes, aterm_interval=spec.aterm_interval)
    md, ext = plan_subgrids_split(view, uvw, freqs, bl)
    obs = Observation(spec, st, bl, uvw, freqs, k, at, taper, md, ext)
    return obs, dec_all[picks], edges, length[picks]


def config4(n_subgrids: int = 50000, nstations: int = 2000, sizes=(24, 32, 48), groups=(8, 16, 32, 64),
            seed: int = 4) -> list[Observation]:
    """The batched-uneven generator: `n_subgrids` subgrids sampled from the
    baselines of `nstations` stations in a 10 km disk (config-2 geometry), each
    with its own time window of T timesteps, T log-uniform in [16, 256], starting
    at a random hour angle within +-4 h; a channel group of 8, 16, 32 or 64 of 64
    channels over 150-160 MHz (at a random group-aligned offset); a subgrid size
    drawn from `sizes`; an 8192^2 grid.  A-terms are identity + 0.05 N(0,1), one
    slot.  Returns one Observation per subgrid size, each with its own uvw rows
    (a subgrid's rows are contiguous), metadata and channel sidecar; the
    ObservationSpec of each has ntimesteps = its row count, one "baseline" per
    row block, and must not be used to re-plan."""
    from ._lib import SUBGRID_EXT_DTYPE

    rng = np.random.default_rng(seed)
    st = stations_in_disk(nstations, 5000.0, rng)
    C, f0, f1, G, img = 64, 150e6, 160e6, 8192, 0.05
    freqs = np.linspace(f0, f1, C)
    k = (2 * np.pi * freqs / SPEED_OF_LIGHT).astype(np.float32)
    s1 = rng.integers(0, nstations - 1, n_subgrids)
    s2 = s1 + 1 + (rng.random(n_subgrids) * (nstations - 1 - s1)).astype(np.int64)
    T = np.clip(np.floor(np.exp(rng.uniform(np.log(16), np.log(257), n_subgrids))), 16, 256).astype(np.int64)
    H0 = rng.uniform(-4, 4, n_subgrids) * 3600 * EARTH_ROTATION_RATE
    glen = rng.choice(np.asarray(groups), n_subgrids)
    gofs = np.array([rng.integers(0, C // g) * g for g in glen])
    size = rng.choice(np.asarray(sizes), n_subgrids)
    out = []
    for S in sizes:
        idx = np.where(size == S)[0]
        n = idx.size
        rows = int(T[idx].sum())
        start = np.concatenate([[0], np.cumsum(T[idx])[:-1]]).astype(np.int64)
        sub_of_row = np.repeat(np.arange(n), T[idx])
        t_in = np.arange(rows) - start[sub_of_row]
        H = H0[idx][sub_of_row] + t_in * EARTH_ROTATION_RATE
        enu = (st[s2[idx]] - st[s1[idx]])[sub_of_row]
        lat = dec = np.deg2rad(-30.0)
        E, N_, U = enu[:, 0], enu[:, 1], enu[:, 2]
        X = -np.sin(lat) * N_ + np.cos(lat) * U
        Y, Z = E, np.cos(lat) * N_ + np.sin(lat) * U
        u = np.sin(H) * X + np.cos(H) * Y
        v = -np.sin(dec) * np.cos(H) * X + np.sin(dec) * np.sin(H) * Y + np.cos(dec) * Z
        w = np.cos(dec) * np.cos(H) * X - np.cos(dec) * np.sin(H) * Y + np.sin(dec) * Z
        uvw = np.stack([u, v, w], axis=1).astype(np.float32)
        md = np.zeros(n, METADATA_DTYPE)
        ext = np.zeros(n, SUBGRID_EXT_DTYPE)
        md["time_offset"] = start
        md["nr_timesteps"] = T[idx]
        md["station1"] = s1[idx]
        md["station2"] = s2[idx]
        ext["channel_begin"] = gofs[idx]
        ext["channel_end"] = gofs[idx] + glen[idx]
        scale = img / SPEED_OF_LIGHT
        for i in range(n):
            r = slice(int(start[i]), int(start[i] + T[idx][i]))
            fa, fb = freqs[gofs[idx][i]], freqs[gofs[idx][i] + glen[idx][i] - 1]
            uu = np.concatenate([uvw[r, 0] * fa, uvw[r, 0] * fb]) * scale
            vv = np.concatenate([uvw[r, 1] * fa, uvw[r, 1] * fb]) * scale
            md["x"][i] = int(np.floor(0.5 * (uu.min() + uu.max()) + G / 2 - S / 2 + 0.5))
            md["y"][i] = int(np.floor(0.5 * (vv.min() + vv.max()) + G / 2 - S / 2 + 0.5))
        at = np.zeros((1, nstations, S, S, 4), np.complex64)
        at[..., 0] = 1
        at[..., 3] = 1
        noise = rng.standard_normal((*at.shape, 2), dtype=np.float32)
        at += (0.05 * (noise[..., 0] + 1j * noise[..., 1])).astype(np.complex64)
        spec = ObservationSpec(nstations=nstations, disk_radius_m=5000.0, ntimesteps=rows, timesteps_per_subgrid=rows,
                               nchannels=C, f_start=f0, f_end=f1, subgrid_size=S, grid_size=G, image_size=img,
                               seed=seed)
        out.append(Observation(spec, st, np.stack([s1[idx], s2[idx]], 1).astype(np.uint32), uvw, freqs, k, at,
                               pswf_taper(S, spec.taper_c), md, ext))
    return out


def uv_extent_pixels(spec: ObservationSpec, uvw: np.ndarray, frequencies: np.ndarray) -> np.ndarray:
    """Per subgrid, the larger of its u and v extents in grid cells (must stay below S minus the taper support)."""
    nb, nt, T = spec.n_baselines, spec.ntimesteps, spec.timesteps_per_subgrid
    nsub = spec.subgrids_per_baseline
    f0, f1 = float(frequencies[0]), float(frequencies[-1])
    ext = []
    for k in (0, 1):
        a = uvw[:, k].astype(np.float64).reshape(nb, nt)[:, : nsub * T].reshape(nb, nsub, T)
        lo = np.minimum(a.min(axis=2) * f0, a.min(axis=2) * f1)
        hi = np.maximum(a.max(axis=2) * f0, a.max(axis=2) * f1)
        ext.append((hi - lo) / SPEED_OF_LIGHT * spec.image_size)
    return np.maximum(ext[0], ext[1]).reshape(-1)


def make_observation(spec: ObservationSpec, split: bool = False) -> Observation:
    """Stations, uvw, wavenumbers, A-terms, taper and the plan of `spec`;
    split=True plans with channel and time splitting (``plan_subgrids_split``)."""
    rng = np.random.default_rng(spec.seed)
    st = stations_in_disk(spec.nstations, spec.disk_radius_m, rng)
    bl = baseline_pairs(spec.nstations)
    enu = st[bl[:, 1]] - st[bl[:, 0]]
    H = (np.arange(spec.ntimesteps) - (spec.ntimesteps - 1) / 2.0) * spec.integration_s * EARTH_ROTATION_RATE
    uvw = earth_rotation_uvw(enu, H, np.deg2rad(spec.dec_deg), np.deg2rad(spec.lat_deg))
    uvw = uvw.reshape(-1, 3).astype(np.float32)
    freqs = np.linspace(spec.f_start, spec.f_end, spec.nchannels) if spec.nchannels > 1 else np.array([spec.f_start])
    k = (2 * np.pi * freqs / SPEED_OF_LIGHT).astype(np.float32)
    S = spec.subgrid_size
    at = np.zeros((spec.n_aterm_slots, spec.nstations, S, S, 4), np.complex64)
    at[..., 0] = 1
    at[..., 3] = 1
    if spec.aterm_sigma > 0:
        noise = rng.standard_normal((*at.shape, 2), dtype=np.float32)
        at += (spec.aterm_sigma * (noise[..., 0] + 1j * noise[..., 1])).astype(np.complex64)
    taper = pswf_taper(S, spec.taper_c)
    if split:
        md, ext = plan_subgrids_split(spec, uvw, freqs, bl)
        return Observation(spec, st, bl, uvw, freqs, k, at, taper, md, ext)
    md = plan_subgrids(spec, uvw, freqs, bl)
    return Observation(spec, st, bl, uvw, freqs, k, at, taper, md)


def truncate_observation(obs: Observation, max_subgrids: int) -> Observation:
    """The first `max_subgrids` subgrids of the plan and the rows they use
    (whole baselines first, so the rows stay contiguous)."""
    import dataclasses

    keep = max(1, min(max_subgrids, obs.spec.n_subgrids))
    spec = dataclasses.replace(obs.spec, subgrid_limit=keep)
    md = obs.metadata[:keep].copy()
    rows = spec.n_rows
    return Observation(spec, obs.stations, obs.baselines, np.ascontiguousarray(obs.uvw[:rows]), obs.frequencies,
                       obs.wavenumbers, obs.aterms, obs.taper, md)


def visibilities(spec: ObservationSpec, device="cpu", seed: int | None = None):
    """[rows, C, 4] complex64 with N(0,1) real and imaginary parts (torch tensor on `device`)."""
    import torch

    g = torch.Generator(device=device)
    g.manual_seed(spec.seed if seed is None else seed)
    n = spec.n_rows * spec.nchannels * 4
    re_im = torch.randn(n * 2, generator=g, device=device, dtype=torch.float32)
    return torch.view_as_complex(re_im.view(-1, 2)).view(spec.n_rows, spec.nchannels, 4)
