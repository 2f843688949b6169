"""Checkpoints and the failure paths of the time step, all made on the host.

* The checkpoint byte layout (src/Simulation.cpp:2235-2307): the oracle's writer against the
  reference's own writeCheckpoint (the parity library oracle/_ref, where the reference's
  sources are present), and the CLI's checkpoint against the oracle's reader and writer.
* A restart (src/main.cpp:155-182) loads the checkpoint of step n and, like the reference,
  runs step n again on it (the checkpoint is written after step n, src/main.cpp:530-533, and
  the restart sets n = restart_step): the restarted CLI run must equal that step taken
  through the C-ABI from the loaded state.
* Failures: a pressure solve capped at one iteration fails the step; ls_rollback restores
  every field of the snapshot bit for bit; the CLI's retry manager (src/main.cpp:436-452)
  rolls back and halves dt until it aborts below 1 ms. A non-finite value written into a
  solved field makes the solve report LS_NONFINITE and the step fail. A truncated or missing
  checkpoint ends the CLI with a clean error.
Nothing here faults, traps or hangs a GPU: every failure is a status the host reads.
"""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from helpers import params, rel_l2
from leachingsim_gb300 import _abi, build
from leachingsim_gb300.geometry import grf_geometry, write_raw

STATE = ["label", "frac", "precipitate", "saturation", "pressure", "conc", "acid", "flux_x", "flux_y", "flux_z"]
DERIVED = ["permeability", "viscosity", "cap_pressure", "rel_perm"]


def geometry(shape=(16, 14, 12), seed=2):
    lab, _ = grf_geometry(shape, porosity=0.35, corr_len=2.0, mineral_fraction=0.2, seed=seed, air_inlet=True)
    return lab


def random_state(shape, seed):
    rng = np.random.default_rng(seed)
    I, J, K = shape
    return {"frac": rng.uniform(0, 1, (I + 1, J, K)).astype(np.float32),
            "precipitate": rng.uniform(0, 1, (I + 1, J, K)), "saturation": rng.uniform(0, 1, (I + 1, J, K)),
            "pressure": rng.normal(0, 1, (I + 1, J, K)), "conc": rng.uniform(0, 1, (I + 1, J, K)),
            "acid": rng.uniform(0, 1, (I + 1, J, K))}


def test_checkpoint_layout_matches_reference(oracle_mod, tmp_path):
    refsim = pytest.importorskip("oracle.refsim")
    if not refsim.available():
        pytest.skip("the reference's sources are not present")
    lab, _ = grf_geometry((10, 9, 8), porosity=0.35, corr_len=2.0, mineral_fraction=0.2, seed=3, air_inlet=False)
    for lb, dtype in ((1, np.uint8), (2, np.uint16)):
        lab_t = lab.astype(dtype)
        o = oracle_mod.Oracle(lab.shape, label_bytes=lb, params=params())
        r = refsim.RefSim(lab.shape, label_bytes=lb, params=params())
        st = random_state(lab.shape, 5)
        for a in (o, r):
            a.load_labels(lab_t)
            for f, v in st.items():
                a.set(f, v, padded=True)
        d_ref = tmp_path / f"ref{lb}"
        d_ref.mkdir()
        r.write_checkpoint(d_ref, 7)
        mine = tmp_path / f"oracle{lb}.bin"
        assert o.write_checkpoint(str(mine)) == 0
        theirs = (d_ref / "checkpoint_rank0_000007.bin").read_bytes()
        assert mine.read_bytes() == theirs
        # and the reference reads the oracle's file back to the same fields
        r2 = refsim.RefSim(lab.shape, label_bytes=lb, params=params())
        (d_ref / "checkpoint_rank0_000008.bin").write_bytes(mine.read_bytes())
        r2.load_checkpoint(d_ref, 8)
        for f, v in st.items():
            np.testing.assert_array_equal(r2.get(f, padded=True), v.astype(r2.get(f, padded=True).dtype))
        for a in (o, r, r2):
            a.close()


# ---------------------------------------------------------------------------- GPU


@pytest.fixture(scope="module")
def cli():
    build.build()
    return build.CLI


def _download_all(g, names):
    return {f: g.download(f, padded=True).copy() for f in names}


@pytest.mark.gpu
def test_failed_pressure_solve_and_rollback():
    from leachingsim_gb300.runtime import Context
    lab = geometry()
    g = Context(lab.shape, params=params(press_max_it=1, press_rtol=1e-12))
    g.upload("label", lab)
    g.init_all()
    before = _download_all(g, STATE + DERIVED)
    ok, info = g.step(0.0, 1.0)
    assert not ok and info["success"] == 0
    assert info["pressure"]["converged"] == 0 and info["pressure"]["reason"] < 0
    g.rollback()
    after = _download_all(g, STATE + DERIVED)
    for f in STATE + DERIVED:
        np.testing.assert_array_equal(after[f], before[f], err_msg=f)
    # with the cap lifted, the same step now succeeds from the restored state
    g.set_params(params(press_rtol=1e-12))
    ok, info = g.step(0.0, 1.0)
    assert ok and info["success"] == 1
    g.close()


@pytest.mark.gpu
@pytest.mark.parametrize("field", ["pressure", "conc"])
def test_nonfinite_value_fails_the_step(field):
    """A NaN written into a field a linear solve starts from (a solution slot of a Pore row:
    slot row + J*K with the reference's write-back offset) is seen by the FP64 residual of
    that solve: LS_NONFINITE, reason -4, and the step fails for the retry manager."""
    from leachingsim_gb300.runtime import Context, load
    lab = geometry()
    g = Context(lab.shape, params=params())
    g.upload("label", lab)
    g.init_all()
    v = g.download(field, padded=True).copy()
    i, j, k = [int(x[0]) for x in np.nonzero(lab == _abi.PORE)]
    v[i + 1, j, k] = np.nan
    g.upload(field, v, padded=True)
    if field == "pressure":
        info = _abi.LsSolveInfo()
        g.props()
        st = load().ls_pressure_step(g.h, C.c_double(0.0), C.byref(info))
        assert st == _abi.LS_NONFINITE and info.reason == -4
        g.upload(field, v, padded=True)
    ok, info = g.step(0.0, 1.0)
    assert not ok and info["success"] == 0
    assert info["pressure" if field == "pressure" else "conc"]["reason"] == -4
    g.close()


def _run_cli(cli, raw, shape, out, extra, timeout=600):
    I, J, K = shape
    args = [cli, "--raw-file", str(raw), "--xext", str(K), "--yext", str(J), "--zext", str(I), "--csat", "1.0",
            "--dt", "1.0", "--out_dir", str(out), "-press_ksp_rtol", "1e-11", "-conc_ksp_rtol", "1e-12", *extra]
    return subprocess.run(args, capture_output=True, text=True, timeout=timeout)


@pytest.mark.gpu
def test_cli_retry_manager_halves_dt_until_abort(cli, tmp_path):
    lab = geometry()
    raw = tmp_path / "g.raw"
    write_raw(str(raw), lab)
    res = _run_cli(cli, raw, lab.shape, tmp_path / "out", ["--tmax", "3", "--nout", "1", "-press_ksp_max_it", "1"])
    out = res.stdout
    assert res.returncode == 1
    assert "[Retry Manager] Physics diverged! Rolling back memory and halving dt..." in out
    dts = [float(line.split("dt: ")[1].rstrip("s")) for line in out.splitlines() if line.startswith("Iteration: 0 ")]
    # the log prints six significant digits
    assert dts[0] == 1.0 and all(abs(b - a * 0.5) <= 1e-5 * a for a, b in zip(dts, dts[1:]))
    assert dts[-1] < 2e-3
    assert "Time step shrank below 1ms" in out


@pytest.mark.gpu
def test_cli_checkpoint_layout_and_restart(cli, tmp_path, oracle_mod):
    from leachingsim_gb300.runtime import Context
    from vtk_read import read_vti
    lab = geometry()
    raw = tmp_path / "g.raw"
    write_raw(str(raw), lab)
    out = tmp_path / "run"
    res = _run_cli(cli, raw, lab.shape, out, ["--tmax", "3", "--nout", "2", "--chk_freq", "2"])
    assert res.returncode == 0, res.stdout[-2000:] + res.stderr[-2000:]
    chk = out / "checkpoint_rank0_000002.bin"
    data = chk.read_bytes()
    NP = (lab.shape[0] + 1) * lab.shape[1] * lab.shape[2]
    assert len(data) == NP * (1 + 4 + 5 * 8)
    # the oracle reads it and writes the same bytes back (the reference's np=1 layout)
    o = oracle_mod.Oracle(lab.shape, params=params())
    assert o.load_checkpoint(str(chk)) == 0
    again = tmp_path / "again.bin"
    assert o.write_checkpoint(str(again)) == 0
    assert again.read_bytes() == data
    # the checkpoint holds the state the step-2 output shows (the output comes first)
    _, arrays = read_vti(str(out / "output_0_000002.vti"))
    np.testing.assert_array_equal(o.get("label").astype(np.uint8), arrays["MaterialType"])
    np.testing.assert_array_equal(o.get("pressure"), arrays["Pressure"])
    np.testing.assert_array_equal(o.get("conc"), arrays["Concentration"])
    o.close()
    # restart from step 2: the CLI runs step 2 again on the loaded state ...
    res = _run_cli(cli, raw, lab.shape, out, ["--tmax", "3", "--nout", "1", "--restart_step", "2"])
    assert res.returncode == 0, res.stdout[-2000:] + res.stderr[-2000:]
    assert "Restarting simulation from step 2" in res.stdout
    _, restarted = read_vti(str(out / "output_0_000002.vti"))
    # ... which is that step through the C-ABI from the checkpoint's state
    p = params(press_rtol=1e-11, conc_rtol=1e-12)
    g = Context(lab.shape, params=p)
    names = ["label", "frac", "precipitate", "saturation", "pressure", "conc", "acid"]
    offs = 0
    sizes = {"label": 1, "frac": 4}
    for f in names:
        nb = NP * sizes.get(f, 8)
        dt = {1: np.uint8, 4: np.float32, 8: np.float64}[sizes.get(f, 8)]
        g.upload(f, np.frombuffer(data[offs:offs + nb], dtype=dt), padded=True)
        offs += nb
    g.props()
    ok, _ = g.step(2.0, 1.0)
    assert ok
    g.props()
    np.testing.assert_array_equal(restarted["MaterialType"], g.download("label"))
    for name, f in (("Pressure", "pressure"), ("Concentration", "conc"), ("Saturation", "saturation")):
        assert rel_l2(restarted[name], g.download(f)) < 1e-12, name
    g.close()


@pytest.mark.gpu
def test_cli_truncated_or_missing_checkpoint(cli, tmp_path):
    lab = geometry()
    raw = tmp_path / "g.raw"
    write_raw(str(raw), lab)
    out = tmp_path / "out"
    out.mkdir()
    res = _run_cli(cli, raw, lab.shape, out, ["--tmax", "3", "--restart_step", "2"])
    assert res.returncode == 1
    assert "failed to locate checkpoint file" in res.stderr
    (out / "checkpoint_rank0_000002.bin").write_bytes(b"\x02" * 1000)
    res = _run_cli(cli, raw, lab.shape, out, ["--tmax", "3", "--restart_step", "2"])
    assert res.returncode == 1
    assert "checkpoint file truncated" in res.stderr
