"""The time loop of the reference's driver (main.f90:135-213) for the case
the fused step covers: a periodic FTS suspension (IsPeriod, FTS_method,
IsCaseLattice = 0) without DEM, walls, rigid conglomerates, filaments,
Brownian motion or oscillatory shear.  It reads control_file.dat and
initial_config.dat and writes output.VTF and yeta_mu.txt as the Fortran
driver does (driver_files.py), so either program can continue the other's
run from its files.

Units (dimentionless_calc / _translate, mymodules.f90:808-881):
lambda_Length = radii_test / radii_true, lambda_time = lambda_Length, the
viscosity mu_f -> 1/pi, BASE_DT, T0 and END_TIME times lambda_time; the
shear rate GAMMA = Gamma_alpha / lambda_time (main.f90:147-151); times are
written divided by lambda_time.  The start time is the first column of
initial_config.dat's last particle record (INITIAL_CONF reads T from every
record).  Those times were written divided by lambda_time and INITIAL_CONF
reads them back unscaled, so with lambda_time != 1 the reference resumes a
hot start at T / lambda_time in internal units (the wrong time and shear
strain); run() does the same by default, and hot_start_time_scaled=True
multiplies the start time by lambda_time, which makes a resume exact.  The
step itself is a callable, so that the same loop runs the GPU step or, in
tests, the oracle's:

    step(conf (N x 3), radii, T, dt, LB, gamma, mu_f, ews_err)
        -> dict(conf=..., U_pos=... (6N), yeta_mu=... (5))
"""
import math

import numpy as np

from . import driver_files as files

UNSUPPORTED = [("useDEM", True), ("useDEMstepper", True), ("Boundary", True), ("wall_method", True),
               ("BROWN", True), ("Oscillation_shear", True), ("IsPeriod", False), ("FTS_method", False)]


def check_supported(control, init):
    """Raise ValueError for settings outside the loop above."""
    bad = [k for k, v in UNSUPPORTED if control[k] is v]
    if control["IsCaseLattice"] != 0:
        bad.append("IsCaseLattice=%d" % control["IsCaseLattice"])
    if init["K_rb"] or init["F_rb"]:
        bad.append("rigid conglomerates or filaments")
    if bad:
        raise ValueError("not covered by this driver: " + ", ".join(bad))


def run(control_path, init_path, step, vtf_path, yeta_path, max_steps=None, hot_start_time_scaled=False,
        forces=None):
    """Runs the loop; returns the last configuration, U_pos, T (in the
    file's time unit) and the number of steps.  hot_start_time_scaled: take
    initial_config.dat's time as written in the file's unit (T / lambda_time)
    and scale it back; the default reads it unscaled, as the reference does.
    forces: optional host callable forces(conf, T) -> Fe (6N) of external
    forces for each step (the place of main.f90's DEM contact forces), passed
    to step as the keyword Fe."""
    c = files.read_control(control_path)
    d = files.read_initial_config(init_path)
    check_supported(c, d)
    lam_time = c["radii_test"] / c["radii_true"]
    mu = 1.0 / math.pi
    dt = c["BASE_DT"] * lam_time
    end_time = c["END_TIME"] * lam_time
    frequency = 1.0 / lam_time
    gamma = c["Gamma_alpha"] * frequency
    LB = list(d["LB"])
    conf = np.array(d["conf"], dtype=np.float64)
    radii = np.array(d["radii"], dtype=np.float64)
    N = len(radii)
    U_pos = np.zeros(6 * N)
    if d["U_pos"] is not None:
        U_pos[:3 * N] = d["U_pos"]
    if d["T"]:
        T = d["T"][-1] * (lam_time if hot_start_time_scaled else 1.0)
    else:
        T = c["T0"] * lam_time
    k = 0
    with open(vtf_path, "w") as vtf, open(yeta_path, "w") as yeta:
        while True:
            if k % c["K_WRITE"] == 0:
                files.write_vtf_frame(vtf, T / lam_time, conf, radii, U_pos)
            if forces is None:
                out = step(conf, radii, T, dt, LB, gamma, mu, c["LINERR"])
            else:
                out = step(conf, radii, T, dt, LB, gamma, mu, c["LINERR"], Fe=forces(conf, T))
            if out.get("rc", 0) > 0:  # CHOLESKY's INFO > 0 stops the reference (stepper.f90:375-393)
                raise RuntimeError("step %d (T = %g): the grand resistance is not positive definite (INFO %d)"
                                   % (k, T / lam_time, out["rc"]))
            conf, U_pos = np.asarray(out["conf"], dtype=np.float64).reshape(N, 3), np.asarray(out["U_pos"])
            if k % c["K_WRITE"] == 0:
                yeta.write(files.yeta_record(T / lam_time, out["yeta_mu"], LB[0], frequency, gamma, 0.0) + "\n")
            k += 1
            T = T + dt
            if T > end_time or (max_steps is not None and k >= max_steps):
                break
    return dict(conf=conf, U_pos=U_pos, T=T / lam_time, steps=k)
