"""Redshift maps from recorded trajectories, computed on the GPU.

The reference's map script reads a trajectory file and, one photon at a time, drops the rows
holding a NaN, runs RedshiftCalculator(...).compute_all_components(), projects the first row's
direction onto the sky and grids the values with scipy's griddata
(_postprocessing/compute_redshift_map.py:30-171; create_2d_map,
_postprocessing/compute_time_delay_map.py:313-357). Here the NaN-padded record stack the tracer
leaves on the device (TraceConfig.record_every; records.trajectories_from_result's layout) is
read in place by the kernels of csrc/exc_maps.cu:

    table = redshift_table(records)                       # [n, 23] on the device (RS_COLUMNS)
    data, (x, y) = compute_redshift_map(records)          # the reference function's outputs
    X, Y, zmap, count = bin_sky_map(x, y, data["z_total"], grid_resolution=256)
    delays, path, chord, (x, y) = compute_time_delays(records)   # compute_time_delay_map's

The same table carries the time delay of _postprocessing/compute_time_delay_map.py (path over
the recorded rows minus the chord, so it depends on record_every like the reference's).

Maps are pixel means (binning) where the reference interpolates with griddata(method="cubic").
Only trajectories that carry the recorded quantities (n_cols >= 14: a, Phi, grad Phi, Phi_dot)
are handled; the reference's alternative of callables a_of_eta / potential_func evaluated per
row stays with RedshiftCalculator on the host.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .. import _native as N
from ..core.constants import c

RS_COLUMNS = N.RS_COLUMNS
_COL = {k: i for i, k in enumerate(RS_COLUMNS)}
# the longest history exc_record_redshift reads in one pass, without scratch
ONE_PASS_ROWS = 257


def _as_stack(trajectories, device=None):
    """[n, n_rows, n_cols] float64 CUDA tensor from a tensor, a stacked array, or a list of
    per-photon [rows, n_cols] arrays (NaN-padded to the longest)."""
    import torch

    if isinstance(trajectories, torch.Tensor):
        t = trajectories
    elif isinstance(trajectories, np.ndarray) and trajectories.ndim == 3:
        t = torch.from_numpy(np.ascontiguousarray(trajectories, dtype=np.float64))
    else:
        trs = [np.asarray(tr, dtype=np.float64) for tr in trajectories]
        if not trs:
            return torch.empty((0, 0, 14), dtype=torch.float64, device=device or "cuda")
        n_cols = max(tr.shape[1] for tr in trs if tr.ndim == 2) if any(tr.ndim == 2 for tr in trs) else 14
        stack = np.full((len(trs), max(len(tr) for tr in trs), n_cols), np.nan)
        for i, tr in enumerate(trs):
            if tr.size:
                stack[i, : len(tr), : tr.shape[1]] = tr
        t = torch.from_numpy(stack)
    if t.dtype != torch.float64 or t.dim() != 3:
        raise ValueError("trajectories must be float64 [n_photons, n_rows, n_cols]")
    if not t.is_cuda:
        t = t.to(device or "cuda", non_blocking=False)
    return t.contiguous()


def redshift_table(trajectories, velocity_func=None):
    """Per-photon redshift components [n, len(RS_COLUMNS)] float64 on the device: the columns of
    RS_COLUMNS (z_H, z_SW, z_ISW, z_D, z_total, z_total_exact, the endpoint Phi, a, eta and x,
    the clean row count, the recorded path, chord and time delay, and whether the time-delay
    loader keeps the photon). Photons with fewer than two clean rows keep zero components and
    delays, as compute_redshift_map and compute_time_delays leave them.
    `velocity_func(x, y, z, eta) -> (vx, vy, vz)` (the reference's peculiar-velocity callable)
    adds the Doppler term: it is called on the host at each photon's two endpoints, then the
    table is recomputed with those velocities."""
    import torch

    rec = _as_stack(trajectories)
    n, n_rows, n_cols = rec.shape
    if n_cols < 14:
        raise ValueError("the device redshift map needs the recorded quantities (n_cols >= 14); "
                         "use RedshiftCalculator with a_of_eta and potential_func for bare states")
    lib = N.load()
    # up to 257 rows the kernel reads each history once and needs no scratch; longer ones list
    # their clean rows there for a second, recursive Simpson pass
    scratch = torch.empty((n, n_rows), dtype=torch.int32, device=rec.device) if n_rows > ONE_PASS_ROWS else None
    out = torch.empty((n, len(RS_COLUMNS)), dtype=torch.float64, device=rec.device)
    stream = N.stream_handle(rec.device)
    N.check(lib.exc_record_redshift(N.ptr(rec), n, n_rows, n_cols, float(c), None, None, N.ptr(scratch),
                                    N.ptr(out), stream), "exc_record_redshift")
    if velocity_func is None or n == 0:
        return out
    t = out.cpu().numpy()
    v = np.zeros((2, n, 3))
    for i in np.flatnonzero(t[:, _COL["n_rows"]] >= 2):
        x_obs, x_em = t[i, _COL["x_obs0"]:_COL["x_obs0"] + 3], t[i, _COL["x_em0"]:_COL["x_em0"] + 3]
        v[0, i] = velocity_func(*x_obs, t[i, _COL["eta_obs"]])
        v[1, i] = velocity_func(*x_em, t[i, _COL["eta_em"]])
    vd = torch.from_numpy(v).to(rec.device)
    N.check(lib.exc_record_redshift(N.ptr(rec), n, n_rows, n_cols, float(c), N.ptr(vd[0]), N.ptr(vd[1]),
                                    N.ptr(scratch), N.ptr(out), stream), "exc_record_redshift")
    return out


def sky_frame(mean_dir, normalize_y: bool = False):
    """The reference's tangent-plane frame about a mean direction (unnormalised input): the unit
    mean, basis_x from the z axis (or the x axis when the mean is within ~26 deg of z) with its
    mean component removed, basis_y = mean x basis_x (divided by its norm with `normalize_y`,
    as the time-delay script's extract_initial_directions does, compute_time_delay_map.py:208)."""
    m = np.asarray(mean_dir, dtype=np.float64)
    m = m / np.linalg.norm(m)
    up = np.array([0.0, 0.0, 1.0]) if abs(m[2]) < 0.9 else np.array([1.0, 0.0, 0.0])
    bx = up - np.dot(up, m) * m
    bx = bx / np.linalg.norm(bx)
    by = np.cross(m, bx)
    if normalize_y:
        by = by / np.linalg.norm(by)
    return m, bx, by


def sky_projection(trajectories, normalize_y: bool = False):
    """(x_proj, y_proj, used) on the device for every photon: `used` marks the photons with at
    least one clean row (the only ones the reference's arrays hold); the others read NaN."""
    import torch

    rec = _as_stack(trajectories)
    n, n_rows, n_cols = rec.shape
    if n_cols < 8:
        raise ValueError("trajectories need the 8 state columns")
    lib = N.load()
    stream = N.stream_handle(rec.device)
    dirs = torch.empty((n, 3), dtype=torch.float64, device=rec.device)
    N.check(lib.exc_sky_directions(N.ptr(rec), n, n_rows, n_cols, N.ptr(dirs), stream), "exc_sky_directions")
    used = ~torch.isnan(dirs[:, 0])
    xp = torch.full((n,), float("nan"), dtype=torch.float64, device=rec.device)
    yp = torch.full_like(xp, float("nan"))
    n_used = int(used.sum())
    if n_used == 0:
        return xp, yp, used
    # np.mean over axis 0 on the host, as the reference takes it (rows accumulated in order):
    # the frame is then the reference's to the bit (3 doubles per photon copied back)
    m, bx, by = sky_frame(np.mean(dirs[used].cpu().numpy(), axis=0), normalize_y)
    d3 = lambda v: (C.c_double * 3)(*[float(x) for x in v])
    N.check(lib.exc_sky_project(N.ptr(dirs), n, d3(m), d3(bx), d3(by), N.ptr(xp), N.ptr(yp), stream),
            "exc_sky_project")
    return xp, yp, used


def extract_sky_positions(trajectories):
    """compute_redshift_map.py:54-95: (x_proj, y_proj) numpy arrays over the photons with at
    least one clean row."""
    xp, yp, used = sky_projection(trajectories)
    return xp[used].cpu().numpy(), yp[used].cpu().numpy()


def compute_redshift_map(trajectories, a_of_eta=None, potential_func=None, velocity_func=None, verbose=False):
    """compute_redshift_map.py:98-171 on the device: ({z_H, z_SW, z_ISW, z_D, z_total} numpy
    arrays over all photons, (x_proj, y_proj) over the photons with a clean row)."""
    table = redshift_table(trajectories, velocity_func).cpu().numpy()
    data = {k: np.ascontiguousarray(table[:, _COL[k]]) for k in ("z_H", "z_SW", "z_ISW", "z_D", "z_total")}
    if verbose:
        print(f"redshift map: {len(table)} photons, {int((table[:, _COL['n_rows']] >= 2).sum())} with >= 2 rows")
    return data, extract_sky_positions(trajectories)


def load_trajectories(filename, clean=True):
    """Trajectories of a save_all_histories file (n_photons attribute, photon_{i}_states
    datasets, optional photon_info): (list of [rows, cols] arrays, metadata dict with n_photons
    and photon_info). clean=True drops every row that holds a NaN, as the redshift-map script's
    loader does (compute_redshift_map.py:30-51); clean=False keeps the rows as stored, for
    compute_time_delays, which applies the time-delay script's own row filter. Needs h5py."""
    try:
        import h5py
    except ImportError as e:
        raise RuntimeError("h5py is not available; cannot read trajectory files.") from e
    out, meta = [], {}
    with h5py.File(filename, "r") as f:
        n = int(f.attrs["n_photons"])
        meta["n_photons"] = n
        if "photon_info" in f:
            meta["photon_info"] = f["photon_info"][:]
        for i in range(n):
            name = f"photon_{i}_states"
            if name not in f:
                continue
            rows = np.asarray(f[name][:], dtype=float)
            if clean and rows.ndim == 2:
                rows = rows[~np.isnan(rows).any(axis=1)]
            out.append(rows)
    return out, meta


def compute_time_delays(trajectories, metadata=None):
    """compute_time_delay_map.py:244-310 on the device, over the photons its loader keeps
    (load_trajectories, :76-92: a clean row, |x| < 1e26 m, |eta| < 3e18 s): (time_delays,
    distances_deflected, distances_straight, (x_proj, y_proj)) numpy arrays. The delay is the
    path summed over consecutive recorded rows minus the chord, over c; the sky positions are
    extract_initial_directions' (:157-239) over the kept photons. `metadata` is accepted for the
    reference's signature and not used."""
    rec = _as_stack(trajectories)
    table = redshift_table(rec)
    kept = table[:, _COL["td_kept"]] == 1.0
    t = table[kept].cpu().numpy()
    delays = np.ascontiguousarray(t[:, _COL["time_delay"]])
    path = np.ascontiguousarray(t[:, _COL["path"]])
    chord = np.ascontiguousarray(t[:, _COL["chord"]])
    if not bool(kept.any()):
        return delays, path, chord, (np.array([]), np.array([]))
    sub = rec[kept] if not bool(kept.all()) else rec
    xp, yp, used = sky_projection(sub, normalize_y=True)
    return delays, path, chord, (xp[used].cpu().numpy(), yp[used].cpu().numpy())


def square_extent(x, y, pad: float = 1.2):
    """create_2d_map's square extent (compute_time_delay_map.py:330-345): the larger of the two
    ranges, padded by `pad`, about the centre of the samples."""
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    if x.size == 0 or y.size == 0:
        raise ValueError("square_extent: no finite sky positions to map")
    xc, yc = (x.min() + x.max()) / 2, (y.min() + y.max()) / 2
    half = max(x.max() - x.min(), y.max() - y.min()) * pad / 2
    if not half > 0.0:
        # one sample, or samples on one point: a small square about it, so that the binning's
        # extent has a width (the reference's griddata cannot interpolate such a set at all)
        half = 1e-6 * max(1.0, abs(xc), abs(yc))
    return (xc - half, xc + half, yc - half, yc + half)


def bin_sky_map(x, y, values, grid_resolution: int = 50, extent=None):
    """Pixel means of scattered sky samples on the device: (X, Y) pixel-centre meshgrids,
    mean [res, res] numpy (NaN where empty) and counts. `extent` (x0, x1, y0, y1) defaults to
    create_2d_map's square extent over the finite samples."""
    import torch

    def dev(a):
        t = a if isinstance(a, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64))
        return t.to("cuda", torch.float64).contiguous()

    xs, ys, vs = dev(x), dev(y), dev(values)
    if not (xs.shape == ys.shape == vs.shape) or xs.dim() != 1:
        raise ValueError("x, y and values must be 1-D of the same length")
    if extent is None:
        ok = torch.isfinite(xs) & torch.isfinite(ys) & torch.isfinite(vs)
        extent = square_extent(xs[ok].cpu().numpy(), ys[ok].cpu().numpy())
    nx = ny = int(grid_resolution)
    s = torch.empty((ny, nx), dtype=torch.float64, device=xs.device)
    cnt = torch.empty((ny, nx), dtype=torch.int64, device=xs.device)
    mean = torch.empty_like(s)
    ext = (C.c_double * 4)(*[float(v) for v in extent])
    N.check(N.load().exc_sky_bin(N.ptr(xs), N.ptr(ys), N.ptr(vs), xs.numel(), nx, ny, ext, N.ptr(s), N.ptr(cnt),
                                 N.ptr(mean), N.stream_handle(xs.device)), "exc_sky_bin")
    x0, x1, y0, y1 = extent
    xc = x0 + (np.arange(nx) + 0.5) * (x1 - x0) / nx
    yc = y0 + (np.arange(ny) + 0.5) * (y1 - y0) / ny
    X, Y = np.meshgrid(xc, yc)
    return X, Y, mean.cpu().numpy(), cnt.cpu().numpy()
