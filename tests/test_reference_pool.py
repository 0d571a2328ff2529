"""The timed CPU baseline's harness (oracle/reference_pool.py) runs the reference's own pools --
Integrator(mode="chunked") and PersistentPoolIntegrator -- on a few photons of the golden FLRW
patch and reports their rates (skipped when the reference is not installed under baseline/_ref)."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.skipif(not os.path.isdir(os.path.join(ROOT, "baseline", "_ref", "excalibur")),
                    reason="reference package not installed under baseline/_ref")
def test_reference_pools_run_and_report(tmp_path):
    d = np.load(os.path.join(ROOT, "tests", "golden", "flrw_patch_32.npz"))
    inp, out = tmp_path / "in.npz", tmp_path / "out.json"
    np.savez(inp, phi=d["field"], box=float(d["box"]), states=d["states"][:6], dt=float(d["dl"]), n_steps=5)
    r = subprocess.run([sys.executable, os.path.join(ROOT, "oracle", "reference_pool.py"), "--inputs", str(inp),
                        "--out", str(out), "--workers", "2", "--persistent"], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    res = json.loads(out.read_text())
    assert res["succeeded"] == 6 and res["photon_steps"] == 30 and res["photon_steps_per_s"] > 0
    pp = res["persistent_pool"]
    assert pp["succeeded"] == 6 and pp["photon_steps"] == 30 and pp["photon_steps_per_s"] > 0
