"""Python restatement of the reference's restart, counter and monitor files.

TEST INFRASTRUCTURE ONLY: the checker for the library's C++ readers and
writers (turbulentbl_gb300/csrc/tbl_restart.cpp, reached through
turbulentbl_gb300/tpfile.py); tests compare their files byte for byte.

Formats (theparvezahmad/turbulentBL):
  * `3D.tp` / `3D%03d.tp`, Tecplot ASCII POINT data with 15 columns per point
    x, y, z, U, V, W, P, Um, Vm, Wm, Uf, Vf, Wf, Wt, Nk written with
    FORMAT(3(1X,F10.6),11(1X,E22.15),(1X,I4)) (dnstbl2/dnstbl.f90:2357-2384,
    format 97), an empty record before every i and every j block, and the
    header records 03/04 (title with time and nstep, variables, zone sizes).
  * the merged `3D.tp` that dnstbl2 reads (:147-159, :350-358) has all j
    (ghost rows included, dnstbl/restart.f90:67-86); a per-rank file holds
    j = 2..ny-1 and k = istart..iend of that rank (:2387-2396).
  * originalTBL writes 8 columns x y z U V W T P with
    FORMAT(3(1X,F10.6),5(1X,E22.15)) (originalTBL/fnldnstbl.f90:1696-1717);
    dnssetbl 7 columns x y z U V W P with FORMAT(3(1X,F10.6),4(1X,E22.15)),
    its own partition and title (dnssetbl/dnssetbl.f90:78-92, :908-932), and
    its merger a shorter title and an unquoted DATAPACKING
    (dnssetbl/combineFile.f90:59-61).
  * `cnt` holds "nz cnt proc" (list-directed), `cnt2` holds "cnt2"; dnssetbl's
    statData.dat FORMAT(4(1X,F15.7),I5.3) (dnssetbl.f90:1203-1208).
  * the monitor files of dnstbl2's rank 0 (massflow.xy, numrcltauwall.xy,
    kineticenergy.dat, lamda.dat, W.dat, boundarylthickness.dat, k.dat,
    meanvalues.dat, Umeanvalues.dat, means, medians, taustress;
    dnstbl2/dnstbl.f90:1613-1721, :2021-2302, formats :2385-2392).
Format codes: 0 dnstbl2, 1 originalTBL, 2 dnssetbl.
"""
import os

import numpy as np

COLS = ["x", "y", "z", "u", "v", "w", "p", "usum2", "vsum2", "wsum2", "uf", "vf", "wf", "wt", "newk"]


def fortran_e(v, w=22, d=15):
    """Fortran Ew.d: [-]0.<d digits>E+xx, right-justified in w columns.  The
    digits are Python's correctly rounded %.{d-1}E conversion, the exponent
    one more (0.d... instead of d.d...)."""
    if v == 0.0:
        return ("0." + "0" * d + "E+00").rjust(w)
    if not np.isfinite(v):
        return ("NaN" if np.isnan(v) else ("Infinity" if v > 0 else "-Infinity")).rjust(w)
    m, e = f"{abs(v):.{d - 1}E}".split("E")
    ex = int(e) + 1
    body = ("-" if v < 0 else "") + "0." + m.replace(".", "")
    body += (f"E{'+' if ex >= 0 else '-'}{abs(ex):02d}" if abs(ex) <= 99 else f"{'+' if ex >= 0 else '-'}{abs(ex):03d}")
    return body.rjust(w)


NCOL = {0: 15, 1: 8, 2: 7}
VARS = {0: ' Variables = "x","y","z","U","V","W","P","Um","Vm","Wm","Uf","Vf","Wf","Wt","Nk"\n',
        1: ' Variables = "x","y","z","U","V","W","T","P"\n',
        2: 'Variables = "x","y","z","U","V","W","P"\n'}


def _row(c, fmt):
    s = "".join(" " + f"{float(x):10.6f}" for x in c[:3])
    ne = 11 if fmt == 0 else NCOL[fmt] - 3
    s += "".join(" " + fortran_e(float(x)) for x in c[3:3 + ne])
    if fmt == 0:
        s += " " + f"{int(c[14]):4d}"
    return s + "\n"


def _header(fmt, style, time, nstep, nproc, nx, nyz, nz):
    if fmt == 2 and style == 1:
        t = f'TITLE ="{time:20.10f}{nstep:9d}{nproc:3d}"\n'
    else:
        t = f'TITLE ="{time:20.10f}{nstep:9d}"\n'
    pack = ",DATAPACKING=POINT" if (fmt == 2 and style == 2) else ',DATAPACKING="POINT"'
    return t + VARS[fmt] + f"ZONE k={nx:4d},j={nyz:4d},i={nz:4d}{pack}\n"


def _cols(fmt, mesh, st, i, j, k):
    c = [mesh.x1[i], mesh.x2[j], mesh.x3[k], st["u"][i, j, k], st["v"][i, j, k], st["w"][i, j, k]]
    if fmt == 1:
        return c + [0.0, st["p"][i, j, k]]
    c.append(st["p"][i, j, k])
    if fmt == 0:
        fl = [st.get(q) for q in ("uf", "vf", "wf")]
        c += [st["usum2"][i, k], st["vsum2"][i, k], st["wsum2"][i, k]]
        c += [(a[i, j, k] if a is not None else 0.0) for a in fl]
        c += [st["wt"][i, k], st["newk"][k]]
    return c


def write_tp(path, mesh, st, time, nstep, j_range=None, k_range=None, header=1, fmt=0, nproc=0):
    """One file; j_range/k_range are 0-based inclusive (default: all j, all
    k).  header: 0 none, 1 the program's writer, 2 the merger's."""
    nx, ny, nz = mesh.nx, mesh.ny, mesh.nz
    j0, j1 = j_range if j_range is not None else (0, ny - 1)
    k0, k1 = k_range if k_range is not None else (0, nz - 1)
    with open(path, "w") as f:
        if header:
            f.write(_header(fmt, header, time, nstep, nproc, nx, j1 - j0 + 1, nz))
        for i in range(nx):
            f.write("\n")
            for j in range(j0, j1 + 1):
                f.write("\n")
                for k in range(k0, k1 + 1):
                    f.write(_row(_cols(fmt, mesh, st, i, j, k), fmt))


def read_tp(path, nx=None, ny=None, nz=None, fmt=0):
    """Read a merged file (all j).  Returns (state dict, time, nstep)."""
    with open(path) as f:
        title = f.readline()
        f.readline()
        zone = f.readline()
        body = f.read().split()
    t = title.split('"')[1]
    time = float(t[:20])
    nstep = int(t[20:29])
    z = zone.replace(",", " ").replace("=", " ").split()
    znx, zny, znz = int(z[z.index("k") + 1]), int(z[z.index("j") + 1]), int(z[z.index("i") + 1])
    nx, ny, nz = nx or znx, ny or zny, nz or znz
    num = np.array(body, dtype=np.float64).reshape(nx, ny, nz, NCOL[fmt])
    st = {"x1": num[:, 0, 0, 0], "x2": num[0, :, 0, 1], "x3": num[0, 0, :, 2]}
    ip = 7 if fmt == 1 else 6
    for q, c in ((3, "u"), (4, "v"), (5, "w"), (ip, "p")):
        st[c] = np.asfortranarray(num[..., q])
    if fmt == 0:
        for q, c in enumerate(("usum2", "vsum2", "wsum2")):
            st[c] = np.asfortranarray(num[:, -1, :, 7 + q])
        for q, c in enumerate(("uf", "vf", "wf")):
            st[c] = np.asfortranarray(num[..., 10 + q])
        st["wt"] = np.asfortranarray(num[:, -1, :, 13])
        st["newk"] = num[-1, -1, :, 14].astype(np.int32)
    return st, time, nstep


def rank_ranges(nz, nproc, fmt=0):
    """0-based k range of each rank's restart file: istart..iend of the
    dnstbl2 partition (:469-485), or b(id)..e(id) of dnssetbl's
    (dnssetbl.f90:78-92)."""
    out = []
    if fmt == 2:
        b = 0
        for r in range(nproc):
            size = nz // nproc + (1 if r >= nproc - nz % nproc else 0)
            out.append((b, b + size - 1))
            b += size
        return out
    loc = (nz - 1) // nproc
    for r in range(nproc):
        bn = 1 + r * loc
        en = bn + loc - 1 if r < nproc - 1 else nz - 2
        out.append((bn - 1 if r == 0 else bn, en + 1 if r == nproc - 1 else en))
    return out


def rank_name(r, fmt):
    return f"3D{r + 1:03d}." + ("dat" if fmt == 2 else "tp")


def write_rank_files(dirname, mesh, st, time, nstep, nproc, fmt=0):
    """The per-rank restart files (j = 2..ny-1, own k range)."""
    for r, (k0, k1) in enumerate(rank_ranges(mesh.nz, nproc, fmt)):
        write_tp(os.path.join(dirname, rank_name(r, fmt)), mesh, st, time, nstep,
                 j_range=(1, mesh.ny - 2), k_range=(k0, k1), header=1 if r == 0 else 0, fmt=fmt, nproc=nproc)


def merge_rank_files(dirname, nz, nproc, out_name="3D.tp", fmt=0):
    """The mergers (dnstbl/restart.f90:17-86, originalTBL/restart.f90,
    dnssetbl/combineFile.f90): concatenate the ranks' k ranges and add the
    periodic ghost rows j = 1, ny of the Ut columns (U, V, W; T for
    originalTBL; P for dnssetbl, whose merger holds it in Ut(:,:,:,4)).  The
    (i,k) columns repeat on the ghost rows, the columns the mergers leave
    unset are written as zero, and x2(ny) continues the uniform spacing."""
    nc = NCOL[fmt]
    with open(os.path.join(dirname, rank_name(0, fmt))) as f:
        title = f.readline()
        f.readline()
        zone = f.readline()
    t = title.split('"')[1]
    time, nstep = float(t[:20]), int(t[20:29])
    z = zone.replace(",", " ").replace("=", " ").split()
    nx, nyi = int(z[z.index("k") + 1]), int(z[z.index("j") + 1])
    ny = nyi + 2
    data = np.zeros((nx, ny, nz, nc))
    for r, (k0, k1) in enumerate(rank_ranges(nz, nproc, fmt)):
        with open(os.path.join(dirname, rank_name(r, fmt))) as f:
            if r == 0:
                for _ in range(3):
                    f.readline()
            vals = np.array(f.read().split(), dtype=np.float64)
        data[:, 1:ny - 1, k0:k1 + 1, :] = vals.reshape(nx, nyi, k1 - k0 + 1, nc)
    periodic = (3, 4, 5) + ((6,) if fmt in (1, 2) else ())
    for q in periodic:
        data[:, 0, :, q] = data[:, ny - 2, :, q]
        data[:, ny - 1, :, q] = data[:, 1, :, q]
    for q in ((0, 2, 7, 8, 9, 13, 14) if fmt == 0 else (0, 2)):
        data[:, 0, :, q] = data[:, 1, :, q]
        data[:, ny - 1, :, q] = data[:, 1, :, q]
    dy = data[0, 2, 0, 1] - data[0, 1, 0, 1]
    data[:, 0, :, 1] = 0.0
    data[:, ny - 1, :, 1] = data[0, 1, 0, 1] + (ny - 2) * dy
    with open(os.path.join(dirname, out_name), "w") as f:
        f.write(_header(fmt, 2, time, nstep, nproc, nx, ny, nz))
        for i in range(nx):
            f.write("\n")
            for j in range(ny):
                f.write("\n")
                for k in range(nz):
                    f.write(_row(data[i, j, k], fmt))


def write_counters(dirname, nz, cnt, nproc, cnt2):
    with open(os.path.join(dirname, "cnt"), "w") as f:
        f.write(f"{nz:12d}{cnt:12d}{nproc:12d}\n")
    with open(os.path.join(dirname, "cnt2"), "w") as f:
        f.write(f"{cnt2:12d}\n")


def read_counters(dirname):
    with open(os.path.join(dirname, "cnt")) as f:
        nz, cnt, nproc = (int(x) for x in f.read().split()[:3])
    with open(os.path.join(dirname, "cnt2")) as f:
        cnt2 = int(f.read().split()[0])
    return nz, cnt, nproc, cnt2


def write_statdata(path, st, irec):
    """dnssetbl's statData.dat, FORMAT(4(1X,F15.7),I5.3) (dnssetbl.f90:1203-1208)."""
    ir = irec - 1
    with open(path, "w") as f:
        for k in range(st["usum2"].shape[1]):
            nk = str(int(st["newk"][k])).zfill(3).rjust(5)
            f.write(f" {st['usum2'][ir, k]:15.7f} {st['vsum2'][ir, k]:15.7f} {st['wsum2'][ir, k]:15.7f}"
                    f" {st['wt'][0, k]:15.7f}{nk}\n")


INFLOW_RECORDS = 37


def fortran_read_e(field, d):
    """One Fortran Ew.d input field as a formatted READ with BLANK='NULL'
    reads it: blanks ignored (all blank = 0), exponent letter E, D or Q or a
    bare sign, d implied decimals when the mantissa has no point."""
    t = "".join(ch for ch in field if not ch.isspace())
    if not t:
        return 0.0
    p, mant = 0, ""
    if t[0] in "+-":
        mant, p = t[0], 1
    point = digits = False
    while p < len(t) and (t[p].isdigit() or (t[p] == "." and not point)):
        point |= t[p] == "."
        digits |= t[p].isdigit()
        mant += t[p]
        p += 1
    if not digits:
        raise ValueError(field)
    ex = 0
    if p < len(t):
        rest = t[p:]
        if rest[0].upper() in "EDQ":
            rest = rest[1:]
        if not rest or not (rest.lstrip("+-").isdigit() and rest[0] in "+-0123456789") or rest.count("+") + rest.count("-") > 1:
            raise ValueError(field)
        ex = int(rest)
    if not point:
        ex -= d
    return float(f"{mant}E{ex}")


def inflow_profile_text(x3, ume1):
    """U_innerdns.dat as the library writes it: (1X,I4,1X,E18.8,1X,E18.8)
    records k, x3(k), Ume1(k) for k = 1..37."""
    return "".join(f" {k + 1:4d}" + " " + fortran_e(float(x3[k]), 18, 8) + fortran_e(float(ume1[k]), 18, 8) + "\n"
                   for k in range(INFLOW_RECORDS))


def read_inflow_profile(text, nz):
    """FORMAT(24X,E18.8) on 37 records, record 37 repeated above plane 37
    (dnstbl2/dnstbl.f90:322-345)."""
    recs = text.split("\n")
    if len(recs) < INFLOW_RECORDS or (len(recs) == INFLOW_RECORDS and recs[-1] == ""):
        raise ValueError("fewer than 37 records")
    vals = [fortran_read_e(r.ljust(42)[24:42], 8) for r in recs[:INFLOW_RECORDS]]
    out = np.array([vals[min(k, INFLOW_RECORDS - 1)] for k in range(nz)])
    return out


# ------------------------------------------------------------ monitor files

def fortran_f(v, w, d):
    """Fortran Fw.d: d decimals right-justified in w columns, w asterisks when
    the value needs more (Python's correctly rounded fixed-point conversion)."""
    v = float(v)
    if np.isnan(v):
        body = "NaN"
    elif np.isinf(v):
        body = ("Infinity" if v > 0 else "-Infinity") if w >= 9 else ("Inf" if v > 0 else "-Inf")
    else:
        body = f"{v:.{d}f}"
    return "*" * w if len(body) > w else body.rjust(w)


def _f157(*vals):
    return "".join(" " + fortran_f(v, 15, 7) for v in vals)


def _f2010(*vals):
    return "".join("  " + fortran_f(v, 20, 10) for v in vals)


def massflow_text(time, ubulk):
    """massflow.xy record, FORMAT(6(1X,F15.7)) (dnstbl2/dnstbl.f90:1613-1615)."""
    return _f157(time, *ubulk[:5]) + "\n"


def tauwall_text(time, nx, ny, ue, x1, tauw_window):
    """numrcltauwall.xy records, i = 2..nx-1, FORMAT(4(1X,F15.7)) (:1674-1679)."""
    span = float(ny - 2)
    return "".join(_f157(time, x1[i], tauw_window[i] / span, 2.0 * (tauw_window[i] / (ue * ue * span))) + "\n"
                   for i in range(1, nx - 1))


def kinetic_energy_text(time, ke):
    """kineticenergy.dat record, FORMAT(2(2X,E20.10)) (:1718-1721)."""
    return "".join("  " + fortran_e(float(v), 20, 10) for v in (time, ke)) + "\n"


def lamda_text(time, lamda, lamda03):
    """lamda.dat record, FORMAT(3(2X,F20.10)) (:2170-2174)."""
    return _f2010(time, lamda, lamda03) + "\n"


def blend_text(x1, x3, wt):
    """W.dat, per i, per k: x1, x3, Wt, FORMAT(3(1X,F15.7)) (:2180-2188)."""
    return "".join(_f157(x1[i], x3[k], wt[i, k]) + "\n" for i in range(len(x1)) for k in range(len(x3)))


def bl_thickness_text(time, x1, bltkns, deltastar, theta, ht, reth):
    """boundarylthickness.dat, FORMAT(7(2X,F20.10)) (:2258-2267)."""
    return "".join(_f2010(time, x1[i], bltkns[i], deltastar[i], theta[i], ht[i], reth[i]) + "\n"
                   for i in range(len(x1)))


def knew_text(newk, eta):
    """k.dat records k, new(k), eta(k), FORMAT(I5,2(F20.10)) (:2286-2292)."""
    return "".join(f"{k + 1:5d}" + fortran_f(float(newk[k]), 20, 10) + fortran_f(eta[k], 20, 10) + "\n"
                   for k in range(len(newk)))


def meanvalues_text(x1, x3, u, v, w, re=None):
    """meanvalues.dat (FORMAT(5(1X,F15.7)), :2296-2302) or, with re,
    Umeanvalues.dat (x3*Re appended, FORMAT(6(1X,F15.7)), :2098-2104)."""
    out = []
    for i in range(len(x1)):
        for k in range(len(x3)):
            c = (x1[i], x3[k], u[i, k], v[i, k], w[i, k]) + (() if re is None else (x3[k] * re,))
            out.append(_f157(*c) + "\n")
    return "".join(out)


def averages_text(a, b, c):
    """means / medians / taustress: one record of a, b, c and a zero
    temperature column per (i,k), i outer, FORMAT(4(1X,F15.7)) each
    (:2021-2049)."""
    nx, nz = a.shape
    return "".join(_f157(a[i, k], b[i, k], c[i, k], 0.0) for i in range(nx) for k in range(nz)) + "\n"
