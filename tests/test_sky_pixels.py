"""The surrogate map's pixel centres built on the device equal the host grid bit for bit (the map's
fallback and audit rays are traced from the host grid)."""
import numpy as np
import pytest


@pytest.mark.parametrize("n_side,start,stop", [(1, 0, None), (7, 0, None), (64, 5, 1000), (4096, 0, 70000),
                                               (4096, 16_777_000, None)])
def test_device_pixel_centres_equal_the_host_grid(n_side, start, stop):
    from excalibur_tool_gb300.surrogate.sky import pixel_centres, pixel_centres_t

    want = pixel_centres(n_side)[start:stop]
    got = pixel_centres_t(n_side, "cpu", start, stop).numpy()
    assert got.dtype == np.float64 and np.array_equal(got, want)
