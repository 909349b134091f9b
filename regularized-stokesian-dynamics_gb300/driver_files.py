"""The reference driver's file formats, so that runs exchange files with the
Fortran driver (host-side Python, no GPU).

  control_file.dat    INIT_READ_CONTROL (src/initial_conf.f90:109-189): one
                      list-directed record per item, in the order of CONTROL
                      below; text after the values of a record is ignored
  initial_config.dat  INITIAL_SIZE / INITIAL_CONF (src/initial_conf.f90:
                      356-476) for IsCaseLattice = 0: eight header records
                      (NX NY NZ; Np; K_rb Nswimer; the K_rb counts or an empty
                      record; F_rb Nfilament; the F_rb counts or an empty
                      record; three rotation angles and a shift; LB), the
                      hot-start flag, then one record per particle,
                      "T x y z a" (cold) or "T x y z a ux uy uz" (hot)
  output.VTF          VMD_WRITE (src/initial_conf.f90:250-262): one record
                      per particle and frame, T x y z a ux uy uz, format
                      (13e24.15e3); a hot start reads the same records
  yeta_mu.txt         main.f90:197-201: T yeta_mu(1:5) LB(1) frequency GAMMA
                      GAMMAangle, format (12ES24.15)

A run resumes from the last output.VTF frame written as a hot start
(hot_start_from_vtf), the reference's own checkpoint.

List-directed input follows Fortran's rules for what these files hold:
values separated by blanks or commas, repeat counts r*c, logicals written
T/F/.true./.false./true/false (the first letter after an optional period),
and the D exponent letter.
"""
import math
import re

# INIT_READ_CONTROL, in order: (name, kind, count); kind i integer, r real,
# l logical.  kBT follows only when BROWN is true.
CONTROL = [
    ("correction_method", "i", 1), ("FTS_method", "l", 1), ("filament_solve_implicit", "l", 1),
    ("uselub", "l", 1), ("useDEM", "l", 1), ("usecollision", "l", 1), ("useDEMstepper", "l", 1),
    ("useGMRESmethod", "l", 1), ("Xshear", "l", 1), ("IsPeriod", "l", 1), ("simplePeriod", "l", 1),
    ("Oscillation_shear", "l", 1), ("fix", "l", 1), ("IsCaseLattice", "i", 1), ("beginstep", "i", 1),
    ("interval", "i", 1), ("NUM_THREADS", "i", 1), ("timestep", "i", 1), ("radii_test", "r", 1),
    ("radii_true", "r", 1), ("g_gravity", "r", 1), ("u_bg", "r", 3), ("omega_bg", "r", 3), ("EI_bg", "r", 6),
    ("mu_f", "r", 1), ("pho_f", "r", 1), ("Re_number", "r", 1), ("Gamma_alpha", "r", 1),
    ("Youngs_module", "r", 1), ("Poisson_ratio", "r", 1), ("ksp", "r", 1), ("erest", "r", 1),
    ("pho_par", "r", 1), ("LINERR", "r", 1), ("collision_condition", "i", 1), ("muCalculate", "l", 1),
    ("T0", "r", 1), ("END_TIME", "r", 1), ("BASE_DT", "r", 1), ("K_WRITE", "i", 1), ("LJ_EPS", "r", 1),
    ("LJ_SIGMA", "r", 1), ("LJ_CUT", "r", 1), ("Boundary", "l", 1), ("wall_method", "l", 1),
    ("useDLVO", "l", 1), ("DebyeLength", "r", 1), ("z0", "r", 1), ("Lambda_l", "r", 1),
    ("Permittivity", "r", 1), ("Potential", "r", 1), ("AH", "r", 1), ("Surfaceenergy", "r", 1),
    ("BROWN", "l", 1),
]


class FormatError(ValueError):
    """A record that does not hold the values its reader expects."""


def _tokens(record):
    out = []
    for tok in re.split(r"[\s,]+", record.strip()):
        if not tok:
            continue
        m = re.fullmatch(r"(\d+)\*(.*)", tok)
        if m and m.group(2):
            out.extend([m.group(2)] * int(m.group(1)))
        else:
            out.append(tok)
    return out


def _value(tok, kind, where):
    try:
        if kind == "l":
            t = tok.lstrip(".")
            if t[:1].upper() not in ("T", "F"):
                raise ValueError(tok)
            return t[:1].upper() == "T"
        if kind == "i":
            return int(tok)
        return float(tok.replace("d", "e").replace("D", "E"))
    except (ValueError, IndexError):
        raise FormatError("%s: cannot read %r as %s" % (where, tok, {"l": "logical", "i": "integer",
                                                                     "r": "real"}[kind]))


def read_values(record, kinds, where="record"):
    """The leading values of one list-directed record (the rest of the record
    is ignored, as a Fortran READ ignores what follows its list)."""
    toks = _tokens(record)
    if len(toks) < len(kinds):
        raise FormatError("%s: %d values expected, found %r" % (where, len(kinds), record.rstrip("\n")))
    return [_value(t, k, where) for t, k in zip(toks, kinds)]


def read_control(path):
    """control_file.dat as a dict keyed by the reference's variable names
    (arrays as lists)."""
    with open(path) as fp:
        records = fp.read().split("\n")
    out, line = {}, 0
    items = list(CONTROL)
    k = 0
    while k < len(items):
        name, kind, count = items[k]
        if line >= len(records):
            raise FormatError("%s: ends before %s" % (path, name))
        vals = read_values(records[line], [kind] * count, "%s:%d (%s)" % (path, line + 1, name))
        out[name] = vals[0] if count == 1 else vals
        line += 1
        k += 1
        if name == "BROWN" and out["BROWN"]:
            items.append(("kBT", "r", 1))
    return out


def read_initial_config(path):
    """initial_config.dat for IsCaseLattice = 0.  Returns NX, NY, NZ, Np,
    K_rb, Nswimer, rb_counts, F_rb, Nfilament, filament_counts, angles
    (degrees, as written), shift, LB, hot_start, and per particle T, conf
    (Np x 3), radii and, for a hot start, U_pos (3 Np)."""
    with open(path) as fp:
        rec = fp.read().split("\n")
    where = lambda i: "%s:%d" % (path, i + 1)  # noqa: E731
    d = {}
    d["NX"], d["NY"], d["NZ"] = read_values(rec[0], "iii", where(0))
    (d["Np"],) = read_values(rec[1], "i", where(1))
    d["K_rb"], d["Nswimer"] = read_values(rec[2], "ii", where(2))
    d["rb_counts"] = read_values(rec[3], "i" * d["K_rb"], where(3)) if d["K_rb"] else []
    d["F_rb"], d["Nfilament"] = read_values(rec[4], "ii", where(4))
    d["filament_counts"] = read_values(rec[5], "i" * d["F_rb"], where(5)) if d["F_rb"] else []
    v = read_values(rec[6], "rrrrrr", where(6))
    d["angles"], d["shift"] = v[:3], v[3:]
    d["LB"] = read_values(rec[7], "rrr", where(7))
    (d["hot_start"],) = read_values(rec[8], "l", where(8))
    n = 8 if d["hot_start"] else 5
    rows = [read_values(rec[9 + i], "r" * n, where(9 + i)) for i in range(d["Np"])]
    d["T"] = [r[0] for r in rows]
    d["conf"] = [r[1:4] for r in rows]
    d["radii"] = [r[4] for r in rows]
    d["U_pos"] = [u for r in rows for u in r[5:8]] if d["hot_start"] else None
    return d


def write_initial_config(path, conf, radii, LB, T=0.0, U_pos=None, NXYZ=(1, 1, 1)):
    """initial_config.dat (IsCaseLattice = 0, no conglomerates or filaments)
    that INITIAL_SIZE / INITIAL_CONF read back; with U_pos a hot start whose
    particle records are output.VTF records."""
    hot = U_pos is not None
    lines = ["%d %d %d" % tuple(NXYZ), "%d" % len(radii), "0 0", "", "0 0", "", "0 0 0 0 0 0",
             " ".join(fortran_e(x) for x in LB), "T" if hot else "F"]
    for i, (x, a) in enumerate(zip(conf, radii)):
        if hot:
            lines.append(vtf_record(T, x, a, U_pos[3 * i:3 * i + 3]))
        else:
            lines.append("".join(fortran_e(v) for v in (T, x[0], x[1], x[2], a)))
    with open(path, "w") as fp:
        fp.write("\n".join(lines) + "\n")


def fortran_e(x, d=15, e=3, w=24):
    """Fortran Ew.dEe output (0.ddd...E+eee, right-justified in w)."""
    if x == 0.0 or not math.isfinite(x):
        if not math.isfinite(x):
            s = ("-" if x < 0 else "") + ("NaN" if math.isnan(x) else "Infinity")
            return s.rjust(w)
        s = ("-" if math.copysign(1.0, x) < 0 else "") + "0." + "0" * d + "E+" + "0" * e
        return s.rjust(w)
    m, ex = ("%.*e" % (d - 1, abs(x))).split("e")
    digits = m.replace(".", "")
    ex = int(ex) + 1
    s = ("-" if x < 0 else "") + "0." + digits + "E" + ("+" if ex >= 0 else "-") + ("%0*d" % (e, abs(ex)))
    return s.rjust(w)


def fortran_es(x, d=15, w=24):
    """Fortran ESw.d output (d.ddd...E+ee; three exponent digits drop the
    letter E)."""
    if not math.isfinite(x):
        return ("NaN" if math.isnan(x) else ("-" if x < 0 else "") + "Infinity").rjust(w)
    m, ex = ("%.*e" % (d, x)).split("e")
    ex = int(ex)
    s = m + ("E%+03d" % ex if abs(ex) <= 99 else "%+04d" % ex)
    return s.rjust(w)


def vtf_record(T, x, a, u):
    """One VMD_WRITE record: T, x(3), a, u(3) in (13e24.15e3)."""
    return "".join(fortran_e(v) for v in (T, x[0], x[1], x[2], a, u[0], u[1], u[2]))


def write_vtf_frame(fp, T, conf, radii, U_pos, nb=0):
    """VMD_WRITE for the free particles (all but the trailing nb boundary
    particles) of one frame."""
    for i in range(len(radii) - nb):
        fp.write(vtf_record(T, conf[i], radii[i], U_pos[3 * i:3 * i + 3]) + "\n")


def read_vtf(path):
    """The records of an output.VTF file as rows of 8 floats."""
    rows = []
    with open(path) as fp:
        for i, line in enumerate(fp):
            if line.strip():
                rows.append(read_values(line, "r" * 8, "%s:%d" % (path, i + 1)))
    return rows


def hot_start_from_vtf(vtf_path, LB, init_path):
    """Checkpoint / resume as the reference does it: the last frame of an
    output.VTF (its trailing records with one time value) written as a
    hot-start initial_config.dat.  A frame holds the state at the start of
    its step, so the resumed run repeats that step."""
    rows = read_vtf(vtf_path)
    if not rows:
        raise FormatError("%s: no records" % vtf_path)
    T = rows[-1][0]
    k = len(rows)
    while k > 0 and rows[k - 1][0] == T:
        k -= 1
    frame = rows[k:]
    conf = [r[1:4] for r in frame]
    radii = [r[4] for r in frame]
    U = [u for r in frame for u in r[5:8]]
    write_initial_config(init_path, conf, radii, LB, T=T, U_pos=U)
    return len(frame), T


def yeta_record(T, yeta_mu, L, frequency, gamma, gamma_angle):
    """One yeta_mu.txt record (12ES24.15): T, yeta_mu(1:5), LB(1),
    frequency, GAMMA, GAMMAangle."""
    return "".join(fortran_es(v) for v in [T] + list(yeta_mu) + [L, frequency, gamma, gamma_angle])
