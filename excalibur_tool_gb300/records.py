"""Trajectory files in the runners' layout.

The reference's comparison runners stack every photon's history rows into one
NaN-padded array `trajectories[n_photons, n_records, n_cols]` and write it with
h5py (gzip level 4, metadata as file attributes), falling back to
`numpy.savez_compressed(path.replace(".h5", ".npz"), trajectories=..., **meta)`
when h5py is unavailable
(_excalibur_runs/excalibur_run_compare_schwarzschild_vs_flrw_impact_parameter.py:232-286, 562-596).
Here the rows come straight from the tracer's on-device records
(TraceConfig.record_every): the padding is applied on the device and one copy
brings the stacked array to the host.
"""
from __future__ import annotations

import os

import numpy as np


def trajectories_from_result(res, x_offset=None) -> np.ndarray:
    """[n_photons, max_records, n_cols] float64, rows past each photon's record count = NaN.

    x_offset (3,) shifts the position columns 1..3, as the runners do for lens-centred output."""
    import torch

    if res.records is None:
        raise ValueError("the trace kept no records (set TraceConfig.record_every)")
    rec, n = res.records, res.n_records
    t = torch.arange(rec.shape[1], device=rec.device)
    out = torch.where((t[None, :] < n[:, None].long())[..., None], rec, torch.full_like(rec, float("nan")))
    if x_offset is not None:
        out[..., 1:4] += torch.as_tensor(np.asarray(x_offset, dtype=np.float64), device=rec.device)
    return out.cpu().numpy()


def write_trajectories(path: str, trajectories: np.ndarray, meta: dict) -> str:
    """Write the stacked trajectories like the runners: HDF5 (gzip 4, attrs) when h5py is
    importable, else the same data as a compressed .npz. Returns the path written."""
    d = os.path.dirname(path)
    if d:
        os.makedirs(d, exist_ok=True)
    try:
        import h5py  # noqa: F401
    except ImportError:
        h5py = None
    if h5py is not None:
        with h5py.File(path, "w") as f:
            f.create_dataset("trajectories", data=trajectories, compression="gzip", compression_opts=4)
            for k, v in meta.items():
                f.attrs[str(k)] = v
        return path
    npz_path = path.replace(".h5", ".npz")
    np.savez_compressed(npz_path, trajectories=trajectories, **meta)
    return npz_path
