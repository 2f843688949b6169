"""The command-line driver: option parsing (CPU) and a short run checked against the C-ABI
(GPU)."""
import os
import subprocess

import numpy as np
import pytest

from leachingsim_gb300 import build
from leachingsim_gb300.geometry import reference_case, write_raw

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def cli():
    build.build()
    return build.CLI


def test_help_lists_reference_options(cli):
    out = subprocess.run([cli, "--help"], capture_output=True, text=True, check=True).stdout
    for opt in ("raw-file", "xext", "yext", "zext", "dt", "tmax", "nout", "D", "kreac", "csat",
                "evap_flux", "theta", "implicit_sat", "restart_step", "chk_freq", "use_out_time",
                "alpha_transfer", "rock_D_fac", "time_scalar"):
        assert f"--{opt}" in out


def test_dry_run_parses_reference_flags_and_petsc_passthrough(cli):
    res = subprocess.run([cli, "--raw-file", "x.raw", "--xext", "10", "--yext", "12", "--zext", "14",
                          "--dt=0.5", "--theta", "0.0", "--D", "1.0", "--implicit_sat", "true",
                          "-press_ksp_rtol", "1e-9", "-conc_ksp_max_it", "77", "-press_pc_type", "hypre",
                          "--dry-run"], capture_output=True, text=True, check=True)
    out = res.stdout
    assert "press_rtol=1e-09" in out and "conc_max_it=77" in out
    assert "implicit_sat=true" in out
    # explicit scheme: dt above dx^2/(2D) = 0.5 is not clamped at 0.5 (src/main.cpp:126-147)
    assert "Using user-specified dt = 0.5s (stable)." in out
    res = subprocess.run([cli, "--raw-file", "x.raw", "--xext", "10", "--yext", "12", "--zext", "14",
                          "--dt", "2", "--theta", "0.2", "--dry-run"], capture_output=True, text=True,
                         check=True)
    assert "Using adjusted dt = 0.45s." in res.stdout


def test_missing_required_option_fails(cli):
    res = subprocess.run([cli, "--xext", "10"], capture_output=True, text=True)
    assert res.returncode != 0
    assert "required" in res.stderr


@pytest.mark.gpu
def test_cli_run_matches_c_abi(cli, tmp_path):
    from leachingsim_gb300._abi import default_params
    from leachingsim_gb300.runtime import Context
    from vtk_read import read_vti

    lab = reference_case(1, n=20)
    raw = tmp_path / "case1.raw"
    write_raw(str(raw), lab)
    out = tmp_path / "out"
    args = [cli, "--raw-file", str(raw), "--xext", "20", "--yext", "20", "--zext", "20",
            "--csat", "1.0", "--dt", "1.0", "--tmax", "3", "--nout", "2", "--out_dir", str(out),
            "-press_ksp_rtol", "1e-11", "-conc_ksp_rtol", "1e-12"]
    res = subprocess.run(args, capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stdout[-2000:] + res.stderr[-2000:]
    assert "*** Simulation Finished ***" in res.stdout
    assert "Sub-steps:" in res.stdout
    for f in ("output_000000.pvti", "output_0_000000.vti", "output_000002.pvti", "time_mapping.pvd"):
        assert (out / f).exists(), f
    pvd = (out / "time_mapping.pvd").read_text()
    assert 'file="output_000002.pvti"' in pvd
    shape, arrays = read_vti(str(out / "output_0_000002.vti"))
    assert shape == lab.shape
    # the same three steps through the C-ABI; output at n=2 follows step 2 and the property sync
    p = default_params(c_sat=1.0, press_rtol=1e-11, conc_rtol=1e-12)
    g = Context(lab.shape, params=p)
    g.upload("label", lab)
    g.init_all()
    for n in range(3):
        ok, _ = g.step(float(n), 1.0)
        assert ok
    g.props()
    np.testing.assert_array_equal(arrays["MaterialType"], g.download("label"))
    for name, field in (("Pressure", "pressure"), ("Concentration", "conc"), ("Saturation", "saturation"),
                        ("EffectivePermeability", "permeability")):
        a = arrays[name]
        b = g.download(field)
        assert np.allclose(a, b, rtol=1e-9, atol=1e-300), name
    g.close()
