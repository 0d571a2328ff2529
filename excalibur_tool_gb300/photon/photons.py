"""Photon collections and generators (excalibur/photon/photons.py).

The generators keep the reference's direction sampling (cone grid with the
theta = 0 de-duplication, random cone, impact-parameter bins, Rodrigues
rotation `_rotate_to_direction`); the null-normalised u^0 is solved on the
GPU by `exc_null_init` (`_solve_u0_from_null_condition`, photons.py:540-568).
Photons are held as one [N, 8] float64 batch; `Photon` objects are made on
demand for code that iterates over `photons.photons`.

New generators for the batched workloads: `generate_polar_grid`
(theta_i = (i + 1/2) alpha / n_theta, no on-axis ray), `generate_patch_grid`
(pixel centres of a square tangent-plane patch) and `generate_full_sky`
(uniform random directions on the sphere).
"""
from __future__ import annotations

import numpy as np

from ..core.constants import c
from ..core.coordinates import cartesian_velocity_to_spherical
from .photon import Photon


def rotate_to_direction(vectors, target_direction):
    """Rodrigues rotation taking +z onto `target_direction` (photons.py:426-459), batched."""
    v = np.atleast_2d(np.asarray(vectors, dtype=float))
    t = np.asarray(target_direction, dtype=float)
    t = t / np.linalg.norm(t)
    z = np.array([0, 0, 1])
    if np.allclose(t, z):
        return v.copy()
    if np.allclose(t, -z):
        return v @ np.array([[1, 0, 0], [0, -1, 0], [0, 0, -1]]).T
    k = np.cross(z, t)
    k = k / np.linalg.norm(k)
    cos_a = np.dot(z, t)
    sin_a = np.linalg.norm(np.cross(z, t))
    return v * cos_a + np.cross(k, v) * sin_a + k[None, :] * (v @ k)[:, None] * (1 - cos_a)


class Photons:
    def __init__(self, metric, *, defer_checks: bool = False):
        """`defer_checks=True` keeps generated states on the device and postpones the check of
        the null-condition solve (the ValueError the generators raise for an origin where the
        metric cannot be evaluated) to `check_generated()` or the first host access, so that a
        generator call does not wait for the GPU."""
        self.metric = metric
        self._batch = []          # list of [n, 8] arrays (host) or tensors (device)
        self._photons = None
        self.field_index = None
        self.defer_checks = bool(defer_checks)
        self._pending = []        # device status tensors of deferred null-condition solves

    def check_generated(self):
        pending, self._pending = self._pending, []
        for status in pending:
            if int((status != 0).sum()) != 0:
                raise ValueError("metric evaluation failed at a photon origin (outside the grid?)")

    # ---- storage ---------------------------------------------------------
    @property
    def photons(self):
        self.check_generated()
        if self._photons is None:
            st = self.states_numpy()
            self._photons = [Photon(s[:4].copy(), s[4:].copy()) for s in st]
        return self._photons

    def states_numpy(self):
        import torch

        self.check_generated()
        if self._photons is not None:
            return np.array([np.concatenate([p.x, p.u]) for p in self._photons]).reshape(-1, 8)
        if not self._batch:
            return np.zeros((0, 8))
        parts = [b.cpu().numpy() if isinstance(b, torch.Tensor) else b for b in self._batch]
        return np.concatenate(parts, axis=0)

    def states(self, device="cuda"):
        """All photons as one [N, 8] float64 tensor on `device`."""
        import torch

        return torch.as_tensor(self.states_numpy(), dtype=torch.float64, device=device).contiguous()

    def _append_batch(self, arr):
        self._batch.append(arr)
        self._photons = None

    def add_photon(self, photon):
        self.photons.append(photon)

    def positions(self):
        return self.states_numpy()[:, :4]

    def directions(self):
        return self.states_numpy()[:, 4:]

    def __len__(self):
        return len(self.photons) if self._photons is not None else sum(len(b) for b in self._batch)

    @property
    def n_photons(self):
        return len(self)

    def __getitem__(self, i):
        return self.photons[i]

    def __iter__(self):
        return iter(self.photons)

    def record_all(self):
        for p in self.photons:
            p.record()

    def update_quantities_all(self, relevant_quantities_func):
        """photon.state_quantities for every photon (photons.py:708-711)."""
        for p in self.photons:
            p.state_quantities(relevant_quantities_func)

    # ---- files (photons.py:713-910) ------------------------------------------
    def _replace(self, photons):
        self._batch, self._pending, self._photons = [], [], list(photons)

    def save_to_binary(self, filename):
        """Every photon's weight, x, u and history rows in one compressed .npz (object arrays,
        read back with allow_pickle). The reference reads photon.position / photon.velocity,
        which its Photon never sets; the photon's x and u are what they name."""
        data = np.empty(len(self.photons), dtype=object)
        for i, p in enumerate(self.photons):
            data[i] = {"weight": p.weight, "initial_position": np.asarray(p.x, dtype=float),
                       "initial_velocity": np.asarray(p.u, dtype=float),
                       "history_states": [np.asarray(h) for h in p.history.states]}
        np.savez_compressed(filename, n_photons=len(data), photon_data=data)

    def load_from_binary(self, filename):
        """Replace the photons by those of a save_to_binary file (trusted files only: the rows
        are pickled objects)."""
        data = np.load(filename, allow_pickle=True)
        out = []
        for d in data["photon_data"][:int(data["n_photons"])]:
            p = Photon(np.asarray(d["initial_position"]), np.asarray(d["initial_velocity"]), float(d["weight"]))
            for h in d["history_states"]:
                p.history.append(np.asarray(h))
            out.append(p)
        self._replace(out)

    @staticmethod
    def _h5py():
        try:
            import h5py
        except ImportError:
            return None
        return h5py

    def save_all_histories(self, filename):
        """The runners' HDF5 layout: attribute n_photons, one dataset photon_{i}_states per photon
        (its history rows, NaN-padded to the longest row; an empty array without history) and
        the structured dataset photon_info (id, n_states, initial_position, initial_velocity from
        the first row, weight). Needs h5py, as in the reference."""
        h5py = self._h5py()
        if h5py is None:
            raise RuntimeError("h5py is not available; cannot save photon histories. Install h5py or skip saving.")
        plist = self.photons
        info = np.empty(len(plist), dtype=[("id", "i4"), ("n_states", "i4"), ("initial_position", "4f8"),
                                           ("initial_velocity", "4f8"), ("weight", "f8")])
        with h5py.File(filename, "w") as f:
            f.attrs["n_photons"] = len(plist)
            for i, p in enumerate(plist):
                rows = p.history.states
                if rows:
                    f.create_dataset(f"photon_{i}_states", data=p.history.as_array())
                    first = np.asarray(rows[0], dtype=float)
                    info[i] = (i, len(rows), first[:4], first[4:8] if len(first) >= 8 else np.nan, p.weight)
                else:
                    f.create_dataset(f"photon_{i}_states", data=np.array([]))
                    info[i] = (i, 0, np.nan, np.nan, p.weight)
            if len(plist):
                f.create_dataset("photon_info", data=info)

    def load_from_hdf5(self, filename):
        """Replace the photons by those of a save_all_histories file: x and u from photon_info
        (else from the first row), history rows with their NaN padding removed."""
        h5py = self._h5py()
        if h5py is None:
            raise RuntimeError("h5py is not available; cannot load photon histories. Install h5py or skip loading.")
        out = []
        with h5py.File(filename, "r") as f:
            n = int(f.attrs["n_photons"])
            meta = {int(r["id"]): r for r in f["photon_info"][:]} if "photon_info" in f else {}
            for i in range(n):
                name = f"photon_{i}_states"
                if name not in f:
                    continue
                rows = f[name][:]
                if i in meta:
                    x0, u0, w = meta[i]["initial_position"], meta[i]["initial_velocity"], float(meta[i]["weight"])
                elif len(rows):
                    first = rows[0][~np.isnan(rows[0])]
                    x0 = first[:4] if len(first) >= 4 else np.zeros(4)
                    u0 = first[4:8] if len(first) >= 8 else np.array([1.0, 1.0, 0.0, 0.0])
                    w = 1.0
                else:
                    x0, u0, w = np.zeros(4), np.array([1.0, 1.0, 0.0, 0.0]), 1.0
                p = Photon(np.array(x0, dtype=float), np.array(u0, dtype=float), w)
                for r in rows:
                    r = r[~np.isnan(r)]
                    if len(r):
                        p.history.append(r)
                out.append(p)
        self._replace(out)

    # ---- u^0 on the device ------------------------------------------------
    def _finish(self, origins, u_spatial, sign=-1.0):
        import torch
        from .._evaluate import null_init

        n = len(u_spatial)
        st = np.zeros((n, 8))
        st[:, :4] = origins
        st[:, 5:8] = u_spatial
        t = torch.as_tensor(st, dtype=torch.float64, device="cuda")
        status = null_init(self.metric, t, sign)
        if self.defer_checks:
            self._pending.append(status)
            self._append_batch(t)
            return t
        if int((status != 0).sum()) != 0:
            raise ValueError("metric evaluation failed at a photon origin (outside the grid?)")
        self._append_batch(t.cpu().numpy())
        return t

    @staticmethod
    def _origin_looks_spherical(origin) -> bool:
        """Spherical-like [t, r, theta, phi] vs cartesian [eta, x, y, z] (photons.py:461-487)."""
        origin = np.asarray(origin, dtype=float)
        if origin.shape[0] < 4:
            return False
        r0, t0, p0 = float(origin[1]), float(origin[2]), float(origin[3])
        if not (np.isfinite(r0) and np.isfinite(t0) and np.isfinite(p0)) or r0 <= 0:
            return False
        if not (-1e-12 <= t0 <= np.pi + 1e-12):
            return False
        return -2 * np.pi - 1e-12 <= p0 <= 2 * np.pi + 1e-12

    def _spatial_from_directions(self, origin, dirs, direction_basis):
        """c * n-hat in the coordinate basis the metric integrates in."""
        u_cart = dirs * c
        if direction_basis == "coordinates":
            return u_cart
        if direction_basis != "cartesian":
            raise ValueError("direction_basis must be 'coordinates' or 'cartesian'")
        if self._origin_looks_spherical(origin):
            r0, t0, p0 = float(origin[1]), float(origin[2]), float(origin[3])
            x0 = r0 * np.sin(t0) * np.cos(p0)
            y0 = r0 * np.sin(t0) * np.sin(p0)
            z0 = r0 * np.cos(t0)
            vr, vt, vp = cartesian_velocity_to_spherical(x0, y0, z0, u_cart[:, 0], u_cart[:, 1], u_cart[:, 2])
            return np.stack([vr, vt, vp], axis=1)
        return u_cart

    @staticmethod
    def _basis_alias(direction_basis, direction_coords):
        if direction_coords is None:
            return direction_basis
        if direction_coords == "metric":
            return "coordinates"
        if direction_coords == "cartesian":
            return "cartesian"
        raise ValueError("direction_coords must be 'metric' or 'cartesian'")

    def _rotate_to_direction(self, vector, target_direction):
        return rotate_to_direction(vector, target_direction)[0]

    # ---- reference generators ---------------------------------------------
    @staticmethod
    def _cone_grid_directions(n_photons, central_direction, cone_angle):
        """Unit directions of the regular (theta, phi) cone grid (photons.py:159-232, 295-390):
        n_photons an int (floor(sqrt(n)) thetas and phis) or (n_theta, n_phi); theta in
        linspace(0, cone_angle), phi in [0, 2 pi) without the end point; the theta = 0 row kept
        once; rotated from +z onto the central direction and normalised."""
        if type(n_photons) == int:
            n_phi = n_theta = int(np.floor(np.sqrt(n_photons)))
        else:
            n_theta, n_phi = n_photons[0], n_photons[1]
        central = np.asarray(central_direction, dtype=float)
        central = central / np.linalg.norm(central)
        thetas = np.linspace(0, cone_angle, n_theta)
        phis = np.linspace(0, 2 * np.pi, n_phi, endpoint=False)
        dirs = []
        for th in thetas:
            for ph in phis:
                if th == 0 and ph != phis[0]:
                    continue
                dirs.append([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)])
        d = rotate_to_direction(np.array(dirs), central)
        return d / np.linalg.norm(d, axis=1)[:, None]

    def generate_cone_grid(self, n_photons, origin, central_direction, cone_angle, direction_basis="coordinates",
                           *, direction_coords=None):
        """Regular (theta, phi) grid in a cone (photons.py:295-424), skipping duplicate theta = 0 points."""
        direction_basis = self._basis_alias(direction_basis, direction_coords)
        origin = np.asarray(origin, dtype=float)
        d = self._cone_grid_directions(n_photons, central_direction, cone_angle)
        u_sp = self._spatial_from_directions(origin, d, direction_basis)
        return self._finish(np.tile(origin, (len(d), 1)), u_sp, -1.0)

    def generate_cone_grid_metric_tensor(self, n_photons, origin, central_direction, cone_angle,
                                         direction_basis="coordinates", *, direction_coords=None):
        """The cone grid with u^0 from the diagonal metric at the origin (photons.py:159-293):
        u^0 = -sqrt(|-(g11 u1^2 + g22 u2^2 + g33 u3^2) / g00|), the metric evaluated once on the
        device; a photon whose relative null error exceeds 1e-5 is reported as the reference
        does. Returns the [n, 8] states (host)."""
        from .._evaluate import null_error

        direction_basis = self._basis_alias(direction_basis, direction_coords)
        origin = np.asarray(origin, dtype=float)
        d = self._cone_grid_directions(n_photons, central_direction, cone_angle)
        u_sp = self._spatial_from_directions(origin, d, direction_basis)
        g = np.asarray(self.metric.metric_tensor(origin), dtype=float)
        spatial = g[1, 1] * u_sp[:, 0] ** 2 + g[2, 2] * u_sp[:, 1] ** 2 + g[3, 3] * u_sp[:, 2] ** 2
        st = np.zeros((len(d), 8))
        st[:, :4] = origin
        st[:, 4] = -np.sqrt(np.abs(-spatial / g[0, 0]))
        st[:, 5:8] = u_sp
        self._append_batch(st)
        rel, _ = null_error(self.metric, st)
        rel = np.atleast_1d(rel.cpu().numpy() if hasattr(rel, "cpu") else np.asarray(rel))
        for i in np.flatnonzero(rel > 1e-5):
            uu = float(st[i, 4:] @ (g @ st[i, 4:]))
            print(f"Warning: Photon {i} null condition violated: u.u = {uu:.3e}, rel_error = {rel[i]:.3e}")
        return st

    def generate_cone_random(self, n_photons, origin, central_direction, cone_angle,
                             direction_basis="coordinates", *, direction_coords=None, seed=None):
        """Random directions in a cone (photons.py:33-156); u^0 > 0 as in the reference. Without
        `seed` the angles come from numpy's global stream as the reference draws them (theta
        uniform in [0, cone_angle], then phi uniform in [0, 2 pi), photon after photon), so a
        caller's np.random.seed gives the reference's photons; `seed` selects a private
        generator instead."""
        direction_basis = self._basis_alias(direction_basis, direction_coords)
        origin = np.asarray(origin, dtype=float)
        if seed is None:
            u = np.random.random_sample(2 * n_photons)
            th = 0.0 + (cone_angle - 0.0) * u[0::2]
            ph = 0.0 + (2 * np.pi - 0.0) * u[1::2]
        else:
            rng = np.random.default_rng(seed)
            th = rng.uniform(0, cone_angle, n_photons)
            ph = rng.uniform(0, 2 * np.pi, n_photons)
        d = np.stack([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)], axis=1)
        d = rotate_to_direction(d, central_direction)
        d = d / np.linalg.norm(d, axis=1)[:, None]
        u_sp = self._spatial_from_directions(origin, d, direction_basis)
        return self._finish(np.tile(origin, (n_photons, 1)), u_sp, +1.0)

    def generate_impact_parameter_bins(self, origin, central_direction, b_edges, n_per_bin, *,
                                       direction_basis="cartesian", direction_coords=None, random_phi=True,
                                       seed=None, u0_sign=-1.0):
        """Screen sampling in impact-parameter annuli (photons.py:570-701)."""
        direction_basis = self._basis_alias(direction_basis, direction_coords)
        origin = np.asarray(origin, dtype=float)
        b_edges = np.asarray(b_edges, dtype=float)
        if b_edges.ndim != 1 or b_edges.size < 2:
            raise ValueError("b_edges must be a 1D array of length >= 2")
        if np.any(b_edges[1:] <= b_edges[:-1]):
            raise ValueError("b_edges must be strictly increasing")
        if b_edges[0] < 0:
            raise ValueError("b_edges must be >= 0")
        nbins = b_edges.size - 1
        n_list = [int(n_per_bin)] * nbins if isinstance(n_per_bin, (int, np.integer)) else [int(x) for x in n_per_bin]
        spherical = self._origin_looks_spherical(origin)
        if spherical and direction_basis != "cartesian":
            raise ValueError("For spherical-like origins [t,r,theta,phi], use direction_basis='cartesian'.")
        rng = np.random.default_rng(seed)
        k = np.asarray(central_direction, dtype=float).reshape(3)
        k = k / np.linalg.norm(k)
        up = np.array([0.0, 0.0, 1.0]) if abs(np.dot(k, [0, 0, 1.0])) <= 0.95 else np.array([0.0, 1.0, 0.0])
        e1 = np.cross(up, k)
        e1 /= np.linalg.norm(e1)
        e2 = np.cross(k, e1)
        t0 = float(origin[0])
        if spherical:
            r0, th0, ph0 = float(origin[1]), float(origin[2]), float(origin[3])
            oxyz = np.array([r0 * np.sin(th0) * np.cos(ph0), r0 * np.sin(th0) * np.sin(ph0), r0 * np.cos(th0)])
        else:
            oxyz = origin[1:4].astype(float)
        u_cart = k * c
        origins, u_sp = [], []
        for ib in range(nbins):
            b1, b2, nph = float(b_edges[ib]), float(b_edges[ib + 1]), n_list[ib]
            if nph == 0:
                continue
            phis = rng.uniform(0.0, 2.0 * np.pi, size=nph) if random_phi else np.linspace(0, 2 * np.pi, nph,
                                                                                          endpoint=False)
            us = rng.uniform(0.0, 1.0, size=nph)
            bs = np.sqrt(us * (b2 * b2 - b1 * b1) + b1 * b1)
            for b, ph in zip(bs, phis):
                xyz = oxyz + float(b) * (np.cos(ph) * e1 + np.sin(ph) * e2)
                if spherical:
                    # the reference's scalar x*x + y*y + z*z (a BLAS dot may fuse or reorder it)
                    px, py, pz = float(xyz[0]), float(xyz[1]), float(xyz[2])
                    r = np.sqrt(px * px + py * py + pz * pz)
                    origins.append([t0, r, np.arccos(np.clip(pz / r, -1.0, 1.0)), np.arctan2(py, px)])
                    u_sp.append(cartesian_velocity_to_spherical(xyz[0], xyz[1], xyz[2], *u_cart))
                else:
                    origins.append([t0, *xyz])
                    u_sp.append(u_cart)
        return self._finish(np.array(origins), np.array(u_sp, dtype=float), u0_sign)

    # ---- batched-workload generators --------------------------------------
    def generate_polar_grid(self, n_theta, n_phi, origin, central_direction, cone_angle,
                            direction_basis="cartesian", sign=-1.0):
        """theta_i = (i + 1/2) alpha / n_theta, phi_j = 2 pi j / n_phi: no on-axis ray, no duplicates."""
        origin = np.asarray(origin, dtype=float)
        th = (np.arange(n_theta) + 0.5) * cone_angle / n_theta
        ph = 2 * np.pi * np.arange(n_phi) / n_phi
        T, P = np.meshgrid(th, ph, indexing="ij")
        d = np.stack([np.sin(T) * np.cos(P), np.sin(T) * np.sin(P), np.cos(T)], -1).reshape(-1, 3)
        d = rotate_to_direction(d, np.asarray(central_direction, dtype=float) / np.linalg.norm(central_direction))
        d = d / np.linalg.norm(d, axis=1)[:, None]
        u_sp = self._spatial_from_directions(origin, d, direction_basis)
        return self._finish(np.tile(origin, (len(d), 1)), u_sp, sign)

    @staticmethod
    def patch_basis(central_direction):
        """Unit axis k and tangent-plane basis (e1, e2) of a patch around `central_direction`."""
        k = np.asarray(central_direction, dtype=float)
        k = k / np.linalg.norm(k)
        up = np.array([0.0, 0.0, 1.0]) if abs(k[2]) < 0.9 else np.array([0.0, 1.0, 0.0])
        e1 = np.cross(up, k)
        e1 /= np.linalg.norm(e1)
        e2 = np.cross(k, e1)
        return k, e1, e2

    def generate_patch_points(self, uv, origin, central_direction, patch_deg, sign=-1.0):
        """Directions at tangent-plane coordinates uv [n, 2] in [-1, 1]^2 of a patch_deg x patch_deg patch."""
        k, e1, e2 = self.patch_basis(central_direction)
        half = np.tan(np.deg2rad(patch_deg / 2.0))
        uv = np.asarray(uv, dtype=float)
        d = k[None] + (uv[:, :1] * half) * e1[None] + (uv[:, 1:2] * half) * e2[None]
        d /= np.linalg.norm(d, axis=1)[:, None]
        return self._finish(np.tile(np.asarray(origin, dtype=float), (len(d), 1)), d * c, sign)

    def generate_patch_grid(self, n_side, origin, central_direction, patch_deg, sign=-1.0, device="cuda"):
        """n_side^2 pixel centres of a patch_deg x patch_deg tangent-plane patch around the axis."""
        t = (np.arange(n_side) + 0.5) / n_side * 2 - 1
        A, B = np.meshgrid(t, t, indexing="ij")
        return self.generate_patch_points(np.stack([A.reshape(-1), B.reshape(-1)], 1), origin, central_direction,
                                          patch_deg, sign)

    # ---- device-side generators (exc_generate_photons) --------------------
    def _device_generate(self, gen, n):
        import ctypes as C

        import torch

        from .. import _native as N

        dev = torch.device("cuda", torch.cuda.current_device())
        desc = self.metric.descriptor(dev)
        states = torch.empty((n, 8), dtype=torch.float64, device=dev)
        status = torch.empty(n, dtype=torch.int32, device=dev)
        lib = N.load()
        N.check(lib.exc_generate_photons(C.byref(desc.struct), C.byref(gen), N.ptr(states), N.ptr(status),
                                         N.stream_handle(dev)), "exc_generate_photons")
        if int((status != 0).sum()) != 0:
            raise ValueError("metric evaluation failed at a photon origin (outside the grid?)")
        self._batch.append(states)
        self._photons = None
        return states

    def _gen_base(self, mode, origin, sign):
        from .. import _native as N

        g = N.ExcPhotonGen()
        g.mode = mode
        for i in range(4):
            g.origin[i] = float(origin[i])
        g.speed = float(c)
        g.sign = float(sign)
        return g

    def device_patch_grid(self, n_side, origin, central_direction, patch_deg, sign=-1.0):
        """generate_patch_grid computed on the device (bit-identical states)."""
        from .. import _native as N

        k, e1, e2 = self.patch_basis(central_direction)
        g = self._gen_base(N.GEN_PATCH_GRID, origin, sign)
        g.n_side = int(n_side)
        for i in range(3):
            g.axis[i], g.e1[i], g.e2[i] = k[i], e1[i], e2[i]
        g.half = float(np.tan(np.deg2rad(patch_deg / 2.0)))
        return self._device_generate(g, int(n_side) ** 2)

    def device_patch_points(self, uv, origin, central_direction, patch_deg, sign=-1.0):
        """generate_patch_points computed on the device; uv is a [n, 2] float64 device tensor."""
        from .. import _native as N

        k, e1, e2 = self.patch_basis(central_direction)
        g = self._gen_base(N.GEN_PATCH_POINTS, origin, sign)
        g.n = int(uv.shape[0])
        for i in range(3):
            g.axis[i], g.e1[i], g.e2[i] = k[i], e1[i], e2[i]
        g.half = float(np.tan(np.deg2rad(patch_deg / 2.0)))
        self._uv_keep = uv.contiguous()
        g.uv = self._uv_keep.data_ptr()
        return self._device_generate(g, g.n)

    @staticmethod
    def _cone_rotation(g, central_direction):
        """Rodrigues rotation of +z onto the cone axis (the host's _rotate_to_direction)."""
        t = np.asarray(central_direction, dtype=float)
        t = t / np.linalg.norm(t)
        z = np.array([0.0, 0.0, 1.0])
        if np.allclose(t, z):
            kr, ca, sa = np.array([1.0, 0.0, 0.0]), 1.0, 0.0
        elif np.allclose(t, -z):
            kr, ca, sa = np.array([1.0, 0.0, 0.0]), -1.0, 0.0
        else:
            kr = np.cross(z, t)
            kr = kr / np.linalg.norm(kr)
            ca, sa = float(np.dot(z, t)), float(np.linalg.norm(np.cross(z, t)))
        for i in range(3):
            g.rot_axis[i] = kr[i]
        g.rot_cos, g.rot_sin = ca, sa

    def device_polar_grid(self, n_theta, n_phi, origin, central_direction, cone_angle, sign=-1.0):
        """generate_polar_grid (cartesian basis) computed on the device."""
        from .. import _native as N

        g = self._gen_base(N.GEN_CONE_GRID, origin, sign)
        g.n_theta, g.n_phi = int(n_theta), int(n_phi)
        g.half = float(cone_angle)
        self._cone_rotation(g, central_direction)
        return self._device_generate(g, int(n_theta) * int(n_phi))

    def device_cone_random(self, n_photons, origin, central_direction, cone_angle, seed=0, sign=-1.0):
        """generate_cone_random on the device: theta uniform in [0, cone_angle), azimuth uniform,
        from the counter-based generator (seeded; not numpy's stream)."""
        from .. import _native as N

        g = self._gen_base(N.GEN_CONE_RANDOM, origin, sign)
        g.n = int(n_photons)
        g.half = float(cone_angle)
        g.seed = int(seed) & ((1 << 64) - 1)
        self._cone_rotation(g, central_direction)
        return self._device_generate(g, g.n)

    def device_impact_parameter_bins(self, origin, central_direction, b_edges, n_per_bin, *, random_phi=True,
                                     seed=0, u0_sign=-1.0):
        """generate_impact_parameter_bins on the device (photons.py:570-701): parallel rays along
        the axis from screen points in impact-parameter annuli (b area-uniform per bin; azimuth
        random or evenly spaced), states in the metric's coordinates (spherical-like origins
        [t, r, theta, phi] are converted as the reference does). Random numbers come from the
        counter-based generator (seeded; not numpy's stream)."""
        import torch

        from .. import _native as N

        origin = np.asarray(origin, dtype=float)
        b_edges = np.asarray(b_edges, dtype=float)
        if b_edges.ndim != 1 or b_edges.size < 2:
            raise ValueError("b_edges must be a 1D array of length >= 2")
        if np.any(~np.isfinite(b_edges)) or np.any(b_edges[1:] <= b_edges[:-1]) or b_edges[0] < 0:
            raise ValueError("b_edges must be finite, strictly increasing and >= 0")
        nbins = b_edges.size - 1
        n_list = [int(n_per_bin)] * nbins if isinstance(n_per_bin, (int, np.integer)) else [int(x) for x in n_per_bin]
        if len(n_list) != nbins or any(n < 0 for n in n_list):
            raise ValueError("n_per_bin must be a non-negative int or a list with length len(b_edges)-1")
        k = np.asarray(central_direction, dtype=float).reshape(3)
        k = k / np.linalg.norm(k)
        up = np.array([0.0, 0.0, 1.0]) if abs(np.dot(k, [0, 0, 1.0])) <= 0.95 else np.array([0.0, 1.0, 0.0])
        e1 = np.cross(up, k)
        e1 /= np.linalg.norm(e1)
        e2 = np.cross(k, e1)
        spherical = self._origin_looks_spherical(origin)
        o = origin.copy()
        if spherical:
            r0, th0, ph0 = o[1], o[2], o[3]
            o[1:4] = [r0 * np.sin(th0) * np.cos(ph0), r0 * np.sin(th0) * np.sin(ph0), r0 * np.cos(th0)]
        g = self._gen_base(N.GEN_IMPACT_BINS, o, u0_sign)
        offsets = np.concatenate([[0], np.cumsum(n_list)]).astype(np.int64)
        g.n = int(offsets[-1])
        if g.n == 0:
            return torch.empty((0, 8), dtype=torch.float64, device=torch.device("cuda", torch.cuda.current_device()))
        dev = torch.device("cuda", torch.cuda.current_device())
        self._bins_keep = (torch.as_tensor(b_edges, device=dev), torch.as_tensor(offsets, device=dev))
        g.b_edges, g.bin_offsets = self._bins_keep[0].data_ptr(), self._bins_keep[1].data_ptr()
        g.n_bins, g.random_phi, g.spherical = nbins, int(bool(random_phi)), int(spherical)
        g.seed = int(seed) & ((1 << 64) - 1)
        for i in range(3):
            g.axis[i], g.e1[i], g.e2[i] = k[i], e1[i], e2[i]
        return self._device_generate(g, g.n)

    def device_full_sky(self, n_photons, origin, seed, sign=-1.0):
        """Uniform directions on the sphere from the device's counter-based generator (seeded;
        a different stream from generate_full_sky's numpy one)."""
        from .. import _native as N

        g = self._gen_base(N.GEN_FULL_SKY, origin, sign)
        g.n = int(n_photons)
        g.seed = int(seed) & ((1 << 64) - 1)
        return self._device_generate(g, g.n)

    def generate_full_sky(self, n_photons, origin, seed, sign=-1.0):
        """Uniform random directions on the sphere (numpy default_rng(seed))."""
        rng = np.random.default_rng(seed)
        v = rng.standard_normal((n_photons, 3))
        v /= np.linalg.norm(v, axis=1)[:, None]
        return self._finish(np.tile(np.asarray(origin, dtype=float), (n_photons, 1)), v * c, sign)
