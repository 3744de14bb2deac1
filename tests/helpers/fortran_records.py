"""Expected output records of PFMDS, built from the Fortran WRITE statements.

This module is written from the Fortran 2008 edit-descriptor rules and
gfortran's list-directed output conventions, independently of the library's
C++ formatter (pfmds_gb300/csrc/fortio.h) and settings echo
(pfmds_gb300/csrc/settings.h), so that tests can compare the files the
library and the oracle write against records derived here.

Edit descriptors (output):
  Aw     a character value of length len: w >= len right-justifies it in w
         columns, w < len keeps its leftmost w characters; plain A writes the
         whole value.  A CHARACTER(len=n) variable is its text padded with
         blanks to n characters; trim(...) drops the trailing blanks.
  Iw     right-justified integer, w asterisks when it does not fit.
  Lw     T or F right-justified in w columns.
  Fw.d   the value rounded to d decimals (correct rounding, ties to even, as
         the C library's conversion gfortran uses); the zero before the decimal
         point is optional and dropped only when the field is otherwise too
         narrow; w asterisks on overflow; a negative value that rounds to zero
         keeps its minus sign.
  ESw.d  one nonzero digit before the point, d after, exponent E+dd, or
         +ddd without the letter when it needs three digits.
List-directed (gfortran): an integer of the default kind is written in 12
columns (one separating blank and I11), a character constant after one blank,
and an empty WRITE is an empty record.
"""
from decimal import Decimal


def A(value, w=None, length=None):
    """Aw of a character value; `length` pads it to a CHARACTER(len=length)
    variable first (None: the value is an expression such as trim(x))."""
    s = value if length is None else (value + " " * length)[:length]
    if w is None:
        return s
    return s.rjust(w) if w >= len(s) else s[:w]


def I(value, w):
    s = str(int(value))
    return "*" * w if len(s) > w else s.rjust(w)


def L(value, w):
    return ("T" if value else "F").rjust(w)


def F(x, w, d):
    x = float(x)
    s = "%.*f" % (d, x)
    if len(s) > w:
        if s.startswith("0."):
            s = s[1:]
        elif s.startswith("-0."):
            s = "-" + s[2:]
    return "*" * w if len(s) > w else s.rjust(w)


def ES(x, w, d):
    x = float(x)
    m, e = ("%.*E" % (d, x)).split("E")
    e = int(e)
    if abs(e) <= 99:
        s = "%sE%s%02d" % (m, "-" if e < 0 else "+", abs(e))
    elif abs(e) <= 999:
        s = "%s%s%03d" % (m, "-" if e < 0 else "+", abs(e))
    else:
        return "*" * w
    return "*" * w if len(s) > w else s.rjust(w)


def list_int(v):
    return I(v, 12)


def list_str(s):
    return " " + s


def exact(x):
    """The exact decimal value of a double (for messages)."""
    return str(Decimal(float(x)))


# ---- records of md() (md_simulation.f90) and its writers ------------------

def log_line(integrator, step, sim_time, conserved, nhc, total, pe, ke, temperature, inter_e, nhc_e):
    """One log record: '(A6,i9,7f24.6)' then '(<n>f20.9)' over the interaction
    energies and '(<m>f20.9)' over the chains' energies
    (md_simulation.f90:205-208)."""
    s = A(integrator, 6) + I(step, 9)
    s += "".join(F(v, 24, 6) for v in (sim_time, conserved, nhc, total, pe, ke, temperature))
    s += "".join(F(v, 20, 9) for v in inter_e)
    s += "".join(F(v, 20, 9) for v in nhc_e)
    return s


def closing_record(prefix, steps, sim_time, total, pe, ke, temperature, inter_e):
    """The all_out / log closing record '(A32,i9,5f20.9)' + '(<n>f20.9)'
    (md_simulation.f90:263-268); prefix is trim(output_prefix)."""
    s = A(prefix, 32) + I(steps, 9)
    s += "".join(F(v, 20, 9) for v in (sim_time, total, pe, ke, temperature))
    s += "".join(F(v, 20, 9) for v in inter_e)
    return s


def snapshot_file(n, box, pos, vel, mass, types):
    """write_particle_group (md_read_write.f90:65-83): list-directed N, the
    Lattice record '(A,9f16.6,A)', then '(7f27.16,A,A)' per atom with the
    CHARACTER(len=32) type written untrimmed."""
    out = [list_int(n),
           "Lattice=\"" + "".join(F(v, 16, 6) for v in (box[0], 0, 0, 0, box[1], 0, 0, 0, box[2]))
           + " \" Properties=pos:R:3:vel:R:3:mass:R:1:species:S:1"]
    for p, v, m, t in zip(pos, vel, mass, types):
        out.append("".join(F(x, 27, 16) for x in (*p, *v, m)) + "    " + A(t, length=32))
    return "\n".join(out) + "\n"


def trajectory_frame(n, step, box, pos, vel, mass, types):
    """write_particle_group_append (md_read_write.f90:86-107): list-directed
    N, '(A,i9,A,9f10.4,A)', then '(7f10.4,A,A)' per atom with trim(type)."""
    out = [list_int(n),
           "time_step: " + I(step, 9) + "    Lattice=\""
           + "".join(F(v, 10, 4) for v in (box[0], 0, 0, 0, box[1], 0, 0, 0, box[2]))
           + " \" Properties=pos:R:3:vel:R:3:mass:R:1:species:S:1"]
    for p, v, m, t in zip(pos, vel, mass, types):
        out.append("".join(F(x, 10, 4) for x in (*p, *v, m)) + "    " + t.rstrip())
    return "\n".join(out) + "\n"


def nlists_load_lines(entries):
    """nlists_load (md_interactions.f90:427-444): 'neib lists load:' then
    '(A8,i3,i6,A,i6)' per list: trim(name), list number, the longest row,
    ' /', neighb_num_max.  entries: (name, j, maxnum, nmax)."""
    return ["neib lists load:"] + [A(name, 8) + I(j, 3) + I(mx, 6) + " /" + I(nmax, 6)
                                  for name, j, mx, nmax in entries]


def out_block(step, integrator, conserved, fsum, mcv, mc, maxvel, loads, warnings=()):
    """The output-unit block of one out_period step (md_simulation.f90:215-228)
    without its first record (the wall-clock 'exe time')."""
    lines = ["step = " + I(step, 12) + " integrator = " + A(integrator, 6),
             "conserved energy (eV) = " + ES(conserved, 21, 9),
             "forces sum (eV/A) = " + ES(fsum, 16, 6),
             "c.o.m. velocity (A/fs) = " + ES(mcv, 16, 6),
             "c.o.m. position (A) = " + "".join(F(v, 12, 6) for v in mc),
             "maximum velocity (A/fs) = " + F(maxvel, 12, 6)]
    lines += nlists_load_lines(loads)
    lines += [list_str(w) for w in warnings]
    lines.append("")
    return lines


def settings_echo(settings_text, n_atoms, box, group_sizes, settings_name):
    """The output-unit echo of the settings file while md() reads it
    (md_simulation.f90:48-94, create_groups and create_interactions in
    md_interactions.f90:38-136), from the file's text.  The items are read as
    list-directed READs would; `str` is CHARACTER(len=128), so '(A32,...)'
    writes its leftmost 32 characters."""
    rec = settings_text.split("\n")
    k = 0

    def nxt():
        nonlocal k
        r = rec[k]
        k += 1
        return r.split()

    def s128(t):
        return A(t, 32, 128)

    out = ["settings_filename: " + settings_name]
    t = nxt()
    out.append(s128(t[0]) + I(int(t[1]), 12))
    for _ in range(2):
        t = nxt()
        out.append(s128(t[0]) + "\t" + t[1])
    out.append("box_size: " + "".join(F(v, 16, 6) for v in box))
    out.append("particles_num: " + I(n_atoms, 12))
    t = nxt()
    out.append(s128(t[0]) + L(t[1].upper().lstrip(".").startswith("T"), 8))
    t = nxt()
    out.append(s128(t[0]) + I(int(t[1]), 12))
    # create_groups
    t = nxt()
    ntypes = int(t[1])
    out.append(s128(t[0]) + I(ntypes, 12))
    t = nxt()
    ngroups = int(t[1])
    out.append(s128(t[0]) + I(ngroups, 12))
    for g in range(ngroups):
        t = nxt()
        names = t[1:1 + ntypes]
        out.append(I(g + 1, 6) + " " + "".join(A(nm, 12, 32) for nm in names) + I(group_sizes[g], 9))
    for _ in range(7):  # group numbers, period_traj, change_group_num
        t = nxt()
        out.append(s128(t[0]) + I(int(t[1]), 12))
    nchange = int(t[1])
    for _ in range(nchange):
        t = nxt()
        out.append(s128(t[0]) + I(int(t[1]), 12) + I(int(t[2]), 12))
        t = nxt()
        out.append(s128(t[0]) + "".join(I(int(x), 12) for x in t[1:4]))
    t = nxt()
    out.append(s128(t[0]) + L(t[1].upper().lstrip(".").startswith("T"), 8))
    t = nxt()
    ninteg = int(t[1])
    out.append(s128(t[0]) + I(ninteg, 12))
    hdr = rec[k]
    k += 1
    out.append(A(hdr, None, 128))
    for _ in range(ninteg):
        t = nxt()
        out.append("  " + A(t[0], 6, 32) + F(float(t[1]), 10, 5) + "".join(I(int(x), 9) for x in t[2:5]))
    t = nxt()
    out.append(s128(t[0]) + ES(float(t[1]), 16, 6))
    t = nxt()
    nnhc = int(t[1])
    out.append(s128(t[0]) + I(nnhc, 12))
    for _ in range(nnhc):
        t = nxt()
        out.append(I(int(t[0]), 6) + F(float(t[1]), 16, 6) + I(int(t[2]), 6) + F(float(t[3]), 16, 6))
    t = nxt()
    out.append(s128(t[0]) + F(float(t[1]), 16, 6))
    # create_interactions
    t = nxt()
    ninter = int(t[1])
    out.append(s128(t[0]) + I(ninter, 12))
    nl_n = {"lj": 2, "lj1g": 1, "ljc": 3, "morsec": 3, "tb": 1, "rebosc": 1, "rjl": 1}
    for _ in range(ninter):
        t = nxt()
        n = nl_n[t[0]]
        out.append(A(t[0], 32, 32) + A(t[1], 32, 32) + I(n, 6))
        for _ in range(n):
            t = nxt()
            out.append(I(int(t[0]), 6) + I(int(t[1]), 6) + I(int(t[2]), 6) + F(float(t[3]), 16, 6)
                       + I(int(t[4]), 9))
    return out
