"""The driver's time loop (driver.py) on the CPU with the oracle's step: a
small periodic FTS suspension written as initial_config.dat, the example
control_file.dat switched to that case.  The loop exits once T exceeds
END_TIME (strictly, main.f90:211), so END_TIME = 3 DT gives four steps; its
files must hold one frame and one viscosity record per step, and its last
configuration must equal four oracle steps taken directly."""
import importlib.util
import os
import sys

import numpy as np
import pytest

from oracle import oracle as o
from tests.test_gmres_variant import configs

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
IO = os.path.join(ROOT, "tests", "golden", "io")
LUBDAT = os.path.join(ROOT, "tests", "golden", "lubdat")


@pytest.fixture(scope="module")
def drv():
    """driver.py and driver_files.py loaded as a package of their own: host
    code, no CUDA library needed."""
    import types
    pkg = os.path.join(ROOT, "regularized-stokesian-dynamics_gb300")
    host = types.ModuleType("rsd_host")
    host.__path__ = [pkg]
    sys.modules["rsd_host"] = host
    for name in ("driver_files", "driver"):
        spec = importlib.util.spec_from_file_location("rsd_host." + name, os.path.join(pkg, name + ".py"))
        mod = importlib.util.module_from_spec(spec)
        sys.modules["rsd_host." + name] = mod
        spec.loader.exec_module(mod)
    return sys.modules["rsd_host.driver"], sys.modules["rsd_host.driver_files"]


def control_for_periodic_fts(tmp_path):
    src = open(os.path.join(IO, "control_file.dat")).read().split("\n")
    set_line = {1: ".true.", 3: ".true.", 7: ".false.", 9: ".true.", 10: ".true.", 18: "1.0", 19: "1.0",
                27: "0.5", 37: "0.003", 38: "1e-3", 39: "1"}  # 0-based records
    for i, v in set_line.items():
        src[i] = v + "    ! set by the test"
    p = tmp_path / "control_file.dat"
    p.write_text("\n".join(src))
    return str(p)


def test_loop_matches_direct_oracle_steps(drv, tmp_path):
    driver, files = drv
    control = control_for_periodic_fts(tmp_path)
    c = files.read_control(control)
    assert c["FTS_method"] and c["uselub"] and c["IsPeriod"] and c["simplePeriod"]
    assert (c["radii_test"], c["radii_true"], c["Gamma_alpha"], c["END_TIME"], c["BASE_DT"], c["K_WRITE"]) == \
        (1.0, 1.0, 0.5, 0.003, 1e-3, 1)
    pos, radii, L = configs().packing(8, 0.2, 0.05, seed=20261100)
    init = str(tmp_path / "initial_config.dat")
    files.write_initial_config(init, pos, radii, [L, L, L])
    tab = o.LubTab(LUBDAT)
    mu = 1.0 / np.pi

    def step(conf, r, T, dt, LB, gamma, mu_f, ews):
        return o.stepper_stokesian(conf, r, LB, T, dt, gamma, mu_f, ews, tab)

    vtf, yeta = str(tmp_path / "output.VTF"), str(tmp_path / "yeta_mu.txt")
    res = driver.run(control, init, step, vtf, yeta)
    assert res["steps"] == 4  # T = 0, 1e-3, 2e-3, 3e-3 (T == END_TIME does not exit)
    rows = files.read_vtf(vtf)
    assert len(rows) == 4 * 8 and [r[0] for r in rows[::8]] == pytest.approx([0.0, 1e-3, 2e-3, 3e-3], abs=1e-15)
    yl = [line for line in open(yeta) if line.strip()]
    assert len(yl) == 4 and all(len(line.rstrip("\n")) == 10 * 24 for line in yl)
    d = files.read_initial_config(init)  # positions and box as the file holds them (15 digits)
    conf, radii, LB, T = np.array(d["conf"]), np.array(d["radii"]), d["LB"], 0.0
    for _ in range(4):
        out = o.stepper_stokesian(conf, radii, LB, T, 1e-3, 0.5, mu, c["LINERR"], tab)
        conf, T = out["conf"], T + 1e-3
    assert np.abs(res["conf"] - conf).max() == 0.0


def test_unsupported_settings_are_refused(drv, tmp_path):
    driver, files = drv
    c = files.read_control(os.path.join(IO, "control_file.dat"))  # the example: not periodic, no FTS
    d = files.read_initial_config(os.path.join(IO, "initial_config.dat"))  # a conglomerate
    with pytest.raises(ValueError) as e:
        driver.check_supported(c, d)
    assert "IsPeriod" in str(e.value) and "conglomerates" in str(e.value)


def test_resume_from_the_last_frame(drv, tmp_path):
    """Checkpoint / resume: the last output.VTF frame of a four-step run as a
    hot start; one more step from it lands exactly on the four-step run's
    final configuration (the frame is the state before the last step)."""
    driver, files = drv
    control = control_for_periodic_fts(tmp_path)
    pos, radii, L = configs().packing(8, 0.2, 0.05, seed=20261100)
    init = str(tmp_path / "initial_config.dat")
    files.write_initial_config(init, pos, radii, [L, L, L])
    tab = o.LubTab(LUBDAT)

    def step(conf, r, T, dt, LB, gamma, mu_f, ews):
        return o.stepper_stokesian(conf, r, LB, T, dt, gamma, mu_f, ews, tab)

    vtf = str(tmp_path / "output.VTF")
    first = driver.run(control, init, step, vtf, str(tmp_path / "yeta_mu.txt"))
    LB = files.read_initial_config(init)["LB"]
    hot = str(tmp_path / "initial_config_hot.dat")
    n, T = files.hot_start_from_vtf(vtf, LB, hot)
    assert n == 8 and T == pytest.approx(3e-3, abs=1e-15)
    d = files.read_initial_config(hot)
    assert d["hot_start"] and len(d["U_pos"]) == 24
    second = driver.run(control, hot, step, str(tmp_path / "o2.VTF"), str(tmp_path / "y2.txt"), max_steps=1)
    assert second["steps"] == 1
    # the frame's positions went through 15-digit records
    assert np.abs(second["conf"] - first["conf"]).max() <= 1e-13 * L


def test_resume_with_a_time_unit_other_than_one(drv, tmp_path):
    """radii_test / radii_true = 2, so lambda_time = 2 and output.VTF holds
    T / 2.  Read back unscaled, as the reference's INITIAL_CONF does, the
    resume starts at half the time (another shear strain, so another
    configuration); with hot_start_time_scaled it continues exactly."""
    driver, files = drv
    control = control_for_periodic_fts(tmp_path)
    lines = open(control).read().split("\n")
    lines[18] = "2.0    ! set by the test"  # radii_test
    open(control, "w").write("\n".join(lines))
    c = files.read_control(control)
    assert c["radii_test"] / c["radii_true"] == 2.0
    pos, radii, L = configs().packing(8, 0.2, 0.05, seed=20261101)
    init = str(tmp_path / "initial_config.dat")
    files.write_initial_config(init, pos, radii, [L, L, L])
    tab = o.LubTab(LUBDAT)

    def step(conf, r, T, dt, LB, gamma, mu_f, ews):
        return o.stepper_stokesian(conf, r, LB, T, dt, gamma, mu_f, ews, tab)

    first = driver.run(control, init, step, str(tmp_path / "output.VTF"), str(tmp_path / "yeta_mu.txt"))
    assert first["steps"] == 4
    hot = str(tmp_path / "initial_config_hot.dat")
    n, T = files.hot_start_from_vtf(str(tmp_path / "output.VTF"), files.read_initial_config(init)["LB"], hot)
    assert T == pytest.approx(3e-3, abs=1e-15)  # file unit: internal 6e-3 / 2
    exact = driver.run(control, hot, step, str(tmp_path / "o2.VTF"), str(tmp_path / "y2.txt"), max_steps=1,
                       hot_start_time_scaled=True)
    assert exact["T"] == pytest.approx(4e-3, abs=1e-15)
    assert np.abs(exact["conf"] - first["conf"]).max() <= 1e-13 * L
    as_ref = driver.run(control, hot, step, str(tmp_path / "o3.VTF"), str(tmp_path / "y3.txt"), max_steps=1)
    assert as_ref["T"] == pytest.approx(2.5e-3, abs=1e-15)
    assert np.abs(as_ref["conf"] - first["conf"]).max() > 1e-9 * L


@pytest.mark.parametrize("key,value", [("useDEM", True), ("useDEMstepper", True), ("Boundary", True),
                                       ("wall_method", True), ("BROWN", True), ("Oscillation_shear", True),
                                       ("IsPeriod", False), ("FTS_method", False), ("IsCaseLattice", 2)])
def test_each_unsupported_setting_is_named(drv, tmp_path, key, value):
    driver, files = drv
    c = files.read_control(control_for_periodic_fts(tmp_path))
    d = {"K_rb": 0, "F_rb": 0}
    driver.check_supported(c, d)  # the periodic FTS case passes
    c[key] = value
    with pytest.raises(ValueError) as e:
        driver.check_supported(c, d)
    assert key in str(e.value)


def test_a_failed_factorisation_stops_the_loop(drv, tmp_path):
    """A step that reports a positive INFO (the grand resistance not positive
    definite) stops the loop, as CHOLESKY's INFO stops the reference; the
    steps before it are on file."""
    driver, files = drv
    control = control_for_periodic_fts(tmp_path)
    pos, radii, L = configs().packing(8, 0.2, 0.05, seed=20261101)
    init = str(tmp_path / "initial_config.dat")
    files.write_initial_config(init, pos, radii, [L, L, L])
    tab = o.LubTab(LUBDAT)
    calls = []

    def step(conf, r, T, dt, LB, gamma, mu_f, ews):
        out = o.stepper_stokesian(conf, r, LB, T, dt, gamma, mu_f, ews, tab)
        calls.append(T)
        out = dict(out, U_pos=out["U_pos"], yeta_mu=out["yeta_mu"])
        if len(calls) == 3:  # the third step's factorisation fails
            out["rc"] = 37
        return out

    vtf, yeta = str(tmp_path / "output.VTF"), str(tmp_path / "yeta_mu.txt")
    with pytest.raises(RuntimeError, match="INFO 37"):
        driver.run(control, init, step, vtf, yeta)
    assert len(calls) == 3
    assert len([line for line in open(yeta) if line.strip()]) == 2


def test_external_forces_reach_the_step(drv, tmp_path):
    """forces(conf, T) is called before every step and its Fe reaches the
    step (the place of main.f90's DEM contact forces)."""
    driver, files = drv
    control = control_for_periodic_fts(tmp_path)
    pos, radii, L = configs().packing(8, 0.2, 0.05, seed=20261102)
    init = str(tmp_path / "initial_config.dat")
    files.write_initial_config(init, pos, radii, [L, L, L])
    tab = o.LubTab(LUBDAT)
    seen = []

    def forces(conf, T):
        Fe = np.zeros(6 * 8)
        Fe[0] = 1.0 + T
        return Fe

    def step(conf, r, T, dt, LB, gamma, mu_f, ews, Fe=None):
        seen.append((T, Fe[0]))
        return o.stepper_stokesian(conf, r, LB, T, dt, gamma, mu_f, ews, tab, Fe=Fe)

    driver.run(control, init, step, str(tmp_path / "o.VTF"), str(tmp_path / "y.txt"), forces=forces)
    assert [f for _, f in seen] == pytest.approx([1.0 + t for t, _ in seen]) and len(seen) == 4
