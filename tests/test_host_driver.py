"""The C++ host layer (hpc-mpm-code_gb300/host/) over the C ABI: it builds and
links against libmpm_gb300.so here; on a GPU its explicit driver, which runs
the reference's explicit time loop with the reference's call names, agrees
with the oracle on the same scene."""
import os
import subprocess

import numpy as np
import pytest

from mpm_gb300 import build, scenes


def test_host_layer_builds_and_links():
    exe = build.build_host()
    assert os.path.exists(exe) and os.access(exe, os.X_OK)


@pytest.mark.gpu
def test_explicit_driver_matches_oracle():
    from oracle import port

    exe = build.build_host()
    out = subprocess.run([exe, "50", "64"], capture_output=True, text=True, check=True).stdout.split()
    vals = dict(zip(out[0::2], out[1::2]))
    assert int(vals["particles"]) == 64000
    s = scenes.elastic_block(jitter=0.0)
    o = port.PortSolid(s)
    o.steps(50)
    q = o.particles()
    assert abs(float(vals["mean_vz"]) - q["v"][:, 2].mean()) <= 1e-9 * abs(q["v"][:, 2].mean())
    assert abs(float(vals["mean_z"]) - q["x"][:, 2].mean()) <= 1e-12 * abs(q["x"][:, 2].mean())
