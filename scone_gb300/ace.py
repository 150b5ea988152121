"""ACE type-1 (ASCII) continuous-energy tables: a reader of the data the CE kernels use, and a writer
of synthetic nuclides in the same format.

The layout is the public ACE specification as SCONE's aceCard reads it
(NuclearData/DataDecks/ACE/aceCard_class.f90:1454-1530): a header line (ZAID a10, AW f12.6,
TZ e12.0, date a10), a comment line (a70, material a10), four lines of (IZ, AW) pairs, NXS(16) and
JXS(32) as 8i9, then the XSS array read list-directed.  Blocks used here: ESZ (JXS(1): energy grid,
total, absorption, elastic, heating, NXS(3) points each), MTR / LQR / TYR / LSIG / SIG (JXS(3..7):
the NXS(4) reactions other than elastic), LAND (JXS(8)).

`nuclide()` builds what aceNeutronNuclide%init keeps for a non-fissile nuclide
(NuclearData/ceNeutronData/aceDatabase/aceNeutronNuclide_class.f90:737-900): total, elastic and
capture (absorption) from ESZ, and the inelastic total as the sum of every scattering reaction
(TY not 0 and not 19, MT 4 left out) from its first grid point on, as the entry of
problems.ce_data.  The kernels model elastic scattering and capture; a nuclide whose inelastic
total is not zero is transported, but an inelastic collision is reported as an error.
"""
import numpy as np


def read_table(path, first_line=1):
    """The table that starts at 1-based line `first_line` of `path` (the line a SCONE library file
    gives for it): header values, NXS, JXS and the XSS array."""
    with open(path) as f:
        lines = f.read().splitlines()[first_line - 1:]
    head = lines[0]
    zaid = head[0:10].strip()
    aw = float(head[10:22])
    tz = float(head[22:34])
    ints = " ".join(lines[6:12]).split()
    nxs = [int(x) for x in ints[:16]]
    jxs = [int(x) for x in ints[16:48]]
    need = nxs[0]
    xss = []
    for ln in lines[12:]:
        xss.extend(float(x.replace("D", "E")) for x in ln.split())
        if len(xss) >= need:
            break
    if len(xss) < need:
        raise ValueError(f"ACE table {zaid}: XSS has {len(xss)} of {need} entries")
    return dict(zaid=zaid, aw=aw, tz=tz, comment=lines[1][:70].rstrip(), nxs=nxs, jxs=jxs,
                xss=np.array(xss[:need]))


def esz(t):
    """ESZ block (aceCard%ESZ_XS): energy grid, total, absorption and elastic cross sections."""
    nes = t["nxs"][2]
    p = t["jxs"][0] - 1
    blk = lambda k: t["xss"][p + k * nes: p + (k + 1) * nes].copy()
    return dict(e=blk(0), total=blk(1), absorption=blk(2), elastic=blk(3))


def reactions(t):
    """The NXS(4) reactions other than elastic (aceCard%setMTdata, :1286-1387): MT, Q, TY, first grid
    index IE (1-based) and the cross section from IE on."""
    nmt = t["nxs"][3]
    x = t["xss"]
    j = t["jxs"]
    out = []
    for i in range(nmt):
        mt = int(x[j[2] - 1 + i])
        q = float(x[j[3] - 1 + i])
        ty = int(x[j[4] - 1 + i])
        loca = int(x[j[5] - 1 + i])
        p = j[6] - 1 + loca - 1                    # SIG block entry: IE, NE, NE values
        ie, ne = int(x[p]), int(x[p + 1])
        out.append(dict(mt=mt, q=q, ty=ty, ie=ie, xs=x[p + 2: p + 2 + ne].copy()))
    return out


def nuclide(path, first_line=1):
    """One non-fissile nuclide for problems.ce_data: e, xs [NES][4] (total, elastic, inelastic,
    capture), A (AW) and kT (TZ, MeV), with the ZAID."""
    t = read_table(path, first_line)
    if t["jxs"][1] != 0:
        raise ValueError(f"ACE table {t['zaid']} is fissile; the CE kernels model non-fissile nuclides")
    z = esz(t)
    nes = len(z["e"])
    inel = np.zeros(nes)
    for r in reactions(t):
        if r["ty"] == 0 or r["ty"] == 19 or r["mt"] == 4:
            continue
        inel[r["ie"] - 1: r["ie"] - 1 + len(r["xs"])] += r["xs"]
    xs = np.stack([z["total"], z["elastic"], inel, z["absorption"]], axis=1)
    return dict(e=z["e"], xs=xs, A=t["aw"], kT=t["tz"], zaid=t["zaid"])


def _ints(vals):
    rows = []
    for k in range(0, len(vals), 8):
        rows.append("".join(f"{v:9d}" for v in vals[k:k + 8]))
    return rows


def write_table(path, zaid, aw, tz, e, total, elastic, capture, date="01/01/26",
                comment="synthetic nuclide", mat="mat 0", ext_mode="w"):
    """Write a non-fissile nuclide with isotropic (centre-of-mass) elastic scattering and radiative
    capture (MT 102) as one ACE type-1 table.  total must be elastic + capture.  Returns the 1-based
    line on which the table starts in the file (it is appended with ext_mode="a")."""
    e = np.asarray(e, np.float64)
    nes = len(e)
    total, elastic, capture = (np.asarray(a, np.float64) for a in (total, elastic, capture))
    if not (len(total) == len(elastic) == len(capture) == nes) or nes < 2:
        raise ValueError("energy grid and cross sections must have the same length (>= 2)")
    if np.any(np.diff(e) <= 0.0):
        raise ValueError("energy grid must ascend")
    xss = []
    j = [0] * 32
    j[0] = len(xss) + 1                                  # ESZ
    xss += list(e) + list(total) + list(capture) + list(elastic) + [0.0] * nes   # heating: 0
    j[2] = len(xss) + 1                                  # MTR
    xss += [102.0]
    j[3] = len(xss) + 1                                  # LQR
    xss += [0.0]
    j[4] = len(xss) + 1                                  # TYR: capture, no secondary neutrons
    xss += [0.0]
    j[5] = len(xss) + 1                                  # LSIG
    xss += [1.0]
    j[6] = len(xss) + 1                                  # SIG: IE, NE, values
    xss += [1.0, float(nes)] + list(capture)
    j[7] = len(xss) + 1                                  # LAND: elastic isotropic (LOCB 0)
    xss += [0.0]
    j[8] = len(xss) + 1                                  # AND: empty
    j[9] = len(xss) + 1                                  # LDLW: no reactions with secondaries
    j[10] = len(xss) + 1                                 # DLW: empty
    za = int(float(zaid.split(".")[0]))
    nxs = [len(xss), za, nes, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0]
    lines = [f"{zaid:>10s}{aw:12.6f}{tz:12.4E} {date:>10s}", f"{comment:<70.70s}{mat:>10.10s}"]
    lines += ["      0         0.      0         0.      0         0.      0         0."] * 4
    lines += _ints(nxs) + _ints(j)
    for k in range(0, len(xss), 4):
        lines.append("".join(f"{v:20.11E}" for v in xss[k:k + 4]))
    start = 1
    if ext_mode == "a":
        try:
            with open(path) as f:
                start = sum(1 for _ in f) + 1
        except FileNotFoundError:
            start = 1
    with open(path, ext_mode) as f:
        f.write("\n".join(lines) + "\n")
    return start
