"""Device-side photon generation against the host generators (photon/photons.py)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _metric(cuda):
    from excalibur_tool_gb300 import workloads

    return workloads.flrw_patch(32, 2, device=cuda).metric


def _origin():
    from excalibur_tool_gb300 import workloads

    return [workloads.lcdm()._eta_at_a1, *workloads.OBSERVER]


def test_patch_grid_and_points_bit_identical(cuda):
    import torch
    from excalibur_tool_gb300 import workloads
    from excalibur_tool_gb300.photon.photons import Photons

    m = _metric(cuda)
    ax = workloads.LENS - workloads.OBSERVER
    host = Photons(m).generate_patch_grid(64, _origin(), ax, 10.0)
    dev = Photons(m).device_patch_grid(64, _origin(), ax, 10.0)
    torch.cuda.synchronize()
    assert torch.equal(host, dev)
    uv = np.random.default_rng(3).uniform(-1, 1, (5000, 2))
    host = Photons(m).generate_patch_points(uv, _origin(), ax, 20.0)
    dev = Photons(m).device_patch_points(torch.as_tensor(uv).cuda(), _origin(), ax, 20.0)
    assert torch.equal(host, dev)


def test_polar_grid_matches_host(cuda):
    from excalibur_tool_gb300 import workloads
    from excalibur_tool_gb300.photon.photons import Photons

    m = _metric(cuda)
    for axis in (workloads.LENS - workloads.OBSERVER, np.array([0.0, 0.0, 1.0]), np.array([0.3, -0.2, 0.9])):
        host = Photons(m).generate_polar_grid(16, 24, _origin(), axis, np.deg2rad(5.0)).cpu().numpy()
        dev = Photons(m).device_polar_grid(16, 24, _origin(), axis, np.deg2rad(5.0)).cpu().numpy()
        assert np.abs(dev - host).max() <= 4e-16 * np.abs(host).max()


def test_full_sky_uniform_and_null(cuda):
    import torch
    from excalibur_tool_gb300._evaluate import null_error
    from excalibur_tool_gb300.photon.photons import Photons

    m = _metric(cuda)
    n = 1 << 18
    a = Photons(m).device_full_sky(n, _origin(), seed=3)
    b = Photons(m).device_full_sky(n, _origin(), seed=3)
    c = Photons(m).device_full_sky(n, _origin(), seed=4)
    assert torch.equal(a, b) and not torch.equal(a, c)
    d = a[:, 5:8] / a[:, 5:8].norm(dim=1, keepdim=True)
    assert float(d.mean(0).norm()) < 5 / np.sqrt(n)
    for k in range(3):                                   # each coordinate uniform in [-1, 1]
        frac = float((d[:, k] > 0.5).double().mean())
        assert abs(frac - 0.25) < 5 * np.sqrt(0.25 * 0.75 / n)
    rel, st = null_error(m, a)
    assert int((st != 0).sum()) == 0 and float(rel.max()) <= 1e-15


def test_cone_random_distribution(cuda):
    """theta uniform in [0, cone) about the axis (photons.py:84-88), azimuth uniform, null u^0."""
    import torch
    from excalibur_tool_gb300 import workloads
    from excalibur_tool_gb300._evaluate import null_error
    from excalibur_tool_gb300.photon.photons import Photons

    m = _metric(cuda)
    n, cone = 1 << 17, np.deg2rad(5.0)
    axis = np.array([0.3, -0.2, 0.9])
    axis = axis / np.linalg.norm(axis)
    s = Photons(m).device_cone_random(n, _origin(), axis, cone, seed=11)
    assert torch.equal(s, Photons(m).device_cone_random(n, _origin(), axis, cone, seed=11))
    d = (s[:, 5:8] / s[:, 5:8].norm(dim=1, keepdim=True)).cpu().numpy()
    th = np.arccos(np.clip(d @ axis, -1.0, 1.0))
    assert th.max() < cone and th.min() >= 0.0
    assert abs(th.mean() / cone - 0.5) < 5 / np.sqrt(12 * n)              # uniform in theta, not in area
    assert abs(np.median(th) / cone - 0.5) < 0.01
    # azimuth about the axis: mean resultant of the transverse unit vectors ~ 0
    tr = d - np.outer(d @ axis, axis)
    tr /= np.linalg.norm(tr, axis=1)[:, None]
    assert np.linalg.norm(tr.mean(0)) < 5 / np.sqrt(n)
    err, st = null_error(m, s)
    assert int((st != 0).sum()) == 0 and float(err.abs().max()) < 1e-12


@pytest.mark.parametrize("random_phi", [True, False])
def test_impact_parameter_bins_flrw(cuda, random_phi):
    """Screen points in annuli (photons.py:663-701): b inside the photon's bin and area-uniform,
    all rays parallel to the axis at speed c, u^0 from the null condition."""
    import torch
    from excalibur_tool_gb300 import workloads
    from excalibur_tool_gb300._evaluate import null_error
    from excalibur_tool_gb300.core.constants import c, one_Mpc
    from excalibur_tool_gb300.photon.photons import Photons

    m = _metric(cuda)
    axis = workloads.LENS - workloads.OBSERVER
    k = axis / np.linalg.norm(axis)
    edges = np.array([0.0, 1.0, 5.0, 20.0]) * one_Mpc
    counts = [4000, 0, 12000]
    s = Photons(m).device_impact_parameter_bins(_origin(), axis, edges, counts, random_phi=random_phi, seed=5)
    assert s.shape == (16000, 8)
    x = s[:, 1:4].cpu().numpy() - np.asarray(workloads.OBSERVER)[None]
    assert np.abs(x @ k).max() < 1e-9 * one_Mpc                          # on the screen through the observer
    b = np.linalg.norm(x, axis=1)
    assert (b[:4000] >= edges[0] * (1 - 1e-12)).all() and (b[:4000] <= edges[1] * (1 + 1e-12)).all()
    assert (b[4000:] >= edges[2] * (1 - 1e-12)).all() and (b[4000:] <= edges[3] * (1 + 1e-12)).all()
    q = (b[4000:] ** 2 - edges[2] ** 2) / (edges[3] ** 2 - edges[2] ** 2)   # area-uniform -> q uniform
    assert abs(q.mean() - 0.5) < 5 / np.sqrt(12 * 12000)
    v = s[:, 5:8].cpu().numpy()
    assert np.abs(v - k[None] * float(c)).max() <= 1e-15 * float(c) * 4
    if not random_phi:
        # evenly spaced azimuths j 2 pi / n_bin on the screen basis of the reference generator
        up = np.array([0.0, 0.0, 1.0]) if abs(k[2]) <= 0.95 else np.array([0.0, 1.0, 0.0])
        e1 = np.cross(up, k)
        e1 /= np.linalg.norm(e1)
        e2 = np.cross(k, e1)
        for lo, n_bin in ((0, 4000), (4000, 12000)):
            ph = np.mod(np.arctan2(x[lo:lo + n_bin] @ e2, x[lo:lo + n_bin] @ e1), 2 * np.pi)
            want = np.arange(n_bin) * (2 * np.pi / n_bin)
            dphi = np.abs(np.angle(np.exp(1j * (ph - want))))
            assert dphi[b[lo:lo + n_bin] > 1e-3 * one_Mpc].max() < 1e-9
    err, st = null_error(m, s)
    assert int((st != 0).sum()) == 0 and float(err.abs().max()) < 1e-12
    torch.cuda.synchronize()


def test_impact_parameter_bins_spherical(cuda):
    """Spherical-like origins (Schwarzschild): states in (t, r, theta, phi) that map back to the
    screen points and to velocities c k (core/coordinates.py:31-84)."""
    from excalibur_tool_gb300 import workloads
    from excalibur_tool_gb300.core.constants import c, one_Mpc
    from excalibur_tool_gb300.core.coordinates import cartesian_to_spherical
    from excalibur_tool_gb300.photon.photons import Photons

    m = workloads.lens_cone(4, 4, device=cuda).metric
    rel = np.asarray(workloads.OBSERVER) - np.asarray(workloads.LENS)
    origin = [0.0, *cartesian_to_spherical(*rel)]
    k = -rel / np.linalg.norm(rel)
    edges = np.array([10.0, 50.0]) * one_Mpc
    s = Photons(m).device_impact_parameter_bins(origin, k, edges, 2048, seed=1).cpu().numpy()
    r, th, ph = s[:, 1], s[:, 2], s[:, 3]
    xyz = np.stack([r * np.sin(th) * np.cos(ph), r * np.sin(th) * np.sin(ph), r * np.cos(th)], 1)
    d = xyz - rel[None]
    assert np.abs(d @ k).max() < 1e-6 * one_Mpc
    b = np.linalg.norm(d, axis=1)
    assert (b >= edges[0] * (1 - 1e-9)).all() and (b <= edges[1] * (1 + 1e-9)).all()
    # the spherical velocity maps back to c k
    vr, vth, vph = s[:, 5], s[:, 6], s[:, 7]
    st_, ct_, sp_, cp_ = np.sin(th), np.cos(th), np.sin(ph), np.cos(ph)
    vx = vr * st_ * cp_ + r * vth * ct_ * cp_ - r * vph * st_ * sp_
    vy = vr * st_ * sp_ + r * vth * ct_ * sp_ + r * vph * st_ * cp_
    vz = vr * ct_ - r * vth * st_
    v = np.stack([vx, vy, vz], 1)
    assert np.abs(v - k[None] * float(c)).max() < 1e-9 * float(c)
