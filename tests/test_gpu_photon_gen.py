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
