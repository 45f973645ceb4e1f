"""The reference's restart and counter files (host side).

Formats (theparvezahmad/turbulentBL):
  * `3D.tp` / `3D%03d.tp`, Tecplot ASCII POINT data with 15 columns per point
    x, y, z, U, V, W, P, Um, Vm, Wm, Uf, Vf, Wf, Wt, Nk written with
    FORMAT(3(1X,F10.6),11(1X,E22.15),(1X,I4)) (dnstbl2/dnstbl.f90:2380-2397,
    format 97), an empty record before every i and every j block, and the
    header records 03/04 (title with time and nstep, variables, zone sizes).
  * the merged `3D.tp` that dnstbl2 reads (:147-159, :350-358) has all j
    (ghost rows included, dnstbl/restart.f90:67-86); a per-rank file holds
    j = 2..ny-1 and k = istart..iend of that rank (:2387-2396).
  * `cnt` holds "nz cnt proc" (list-directed), `cnt2` holds "cnt2".

Values round-trip at 15 significant digits (E22.15), as in the reference, so a
restart is not bit-exact in FP64.
"""
import os

import numpy as np

COLS = ["x", "y", "z", "u", "v", "w", "p", "usum2", "vsum2", "wsum2", "uf", "vf", "wf", "wt", "newk"]


def fortran_e(v, w=22, d=15):
    """Fortran Ew.d: 0.ddd...E+xx with d digits after the point."""
    if v == 0.0 or not np.isfinite(v):
        if not np.isfinite(v):
            return ("NaN" if np.isnan(v) else ("Infinity" if v > 0 else "-Infinity")).rjust(w)
        m, e = 0.0, 0
    else:
        e = int(np.floor(np.log10(abs(v)))) + 1
        m = abs(v) / 10.0 ** e
        # rounding can carry into the next decade
        if round(m, d) >= 1.0:
            e += 1
            m = abs(v) / 10.0 ** e
    digits = f"{m:.{d}f}"
    if digits.startswith("1."):  # carry after rounding
        e += 1
        digits = f"{abs(v) / 10.0 ** e:.{d}f}"
    sign = "-" if v < 0 else ""
    es = f"E{'+' if e >= 0 else '-'}{abs(e):02d}"
    return (sign + digits + es).rjust(w)


def _row(x1, x2, x3, vals, nk):
    s = " " + f"{x1:10.6f}" + " " + f"{x2:10.6f}" + " " + f"{x3:10.6f}"
    for v in vals:
        s += " " + fortran_e(float(v))
    s += " " + f"{int(nk):4d}"
    return s + "\n"


def write_tp(path, mesh, st, time, nstep, j_range=None, k_range=None, header=True, ny_header=None):
    """Write a 3D.tp-format file.  j_range/k_range are 0-based inclusive
    ranges (default: all j, all k, the merged file)."""
    nx, ny, nz = mesh.nx, mesh.ny, mesh.nz
    j0, j1 = j_range if j_range is not None else (0, ny - 1)
    k0, k1 = k_range if k_range is not None else (0, nz - 1)
    arrs = [st[c] for c in ("u", "v", "w", "p")]
    two = [st[c] for c in ("usum2", "vsum2", "wsum2")]
    fl = [st.get(c) for c in ("uf", "vf", "wf")]
    wt, newk = st["wt"], st["newk"]
    with open(path, "w") as f:
        if header:
            f.write(f'TITLE ="{time:20.10f}{nstep:9d}"\n')
            f.write(' Variables = "x","y","z","U","V","W","P","Um","Vm","Wm","Uf","Vf","Wf","Wt","Nk"\n')
            f.write(f"ZONE k={nx:4d},j={(ny_header if ny_header is not None else j1 - j0 + 1):4d},"
                    f"i={nz:4d},DATAPACKING=\"POINT\"\n")
        for i in range(nx):
            f.write("\n")
            for j in range(j0, j1 + 1):
                f.write("\n")
                for k in range(k0, k1 + 1):
                    vals = [a[i, j, k] for a in arrs] + [a[i, k] for a in two] + \
                           [(a[i, j, k] if a is not None else 0.0) for a in fl] + [wt[i, k]]
                    f.write(_row(mesh.x1[i], mesh.x2[j], mesh.x3[k], vals, newk[k]))


def read_tp(path, nx=None, ny=None, nz=None):
    """Read a merged 3D.tp (all j).  Returns (state dict, time, nstep)."""
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
    a = np.array(body, dtype=object).reshape(nx, ny, nz, 15)
    num = a[..., :14].astype(np.float64)
    newk = a[0, 0, :, 14].astype(np.int64).astype(np.int32)
    st = {}
    for q, c in enumerate(("u", "v", "w", "p")):
        st[c] = np.asfortranarray(num[..., 3 + q])
    for q, c in enumerate(("usum2", "vsum2", "wsum2")):
        st[c] = np.asfortranarray(num[:, 0, :, 7 + q])
    for q, c in enumerate(("uf", "vf", "wf")):
        st[c] = np.asfortranarray(num[..., 10 + q])
    st["wt"] = np.asfortranarray(num[:, 0, :, 13])
    st["newk"] = newk
    st["x1"], st["x2"], st["x3"] = num[:, 0, 0, 0], num[0, :, 0, 1], num[0, 0, :, 2]
    return st, time, nstep


def rank_ranges(nz, nproc):
    """istart..iend (0-based inclusive) of each rank's restart file (:469-485)."""
    loc = (nz - 1) // nproc
    out = []
    for r in range(nproc):
        bn = 1 + r * loc
        en = bn + loc - 1 if r < nproc - 1 else nz - 2
        ist = bn - 1 if r == 0 else bn
        ien = en + 1 if r == nproc - 1 else en
        out.append((ist, ien))
    return out


def write_rank_files(dirname, mesh, st, time, nstep, nproc):
    """The per-rank restart files 3D%03d.tp (j = 2..ny-1, own k range)."""
    for r, (k0, k1) in enumerate(rank_ranges(mesh.nz, nproc)):
        write_tp(os.path.join(dirname, f"3D{r + 1:03d}.tp"), mesh, st, time, nstep,
                 j_range=(1, mesh.ny - 2), k_range=(k0, k1), header=(r == 0), ny_header=mesh.ny - 2)


def merge_rank_files(dirname, nz, nproc, out_name="3D.tp"):
    """The restart merger (dnstbl/restart.f90:17-86): concatenate the ranks'
    k ranges, add the periodic ghost rows j=1, ny for U, V, W (P and the
    fluctuation columns of the ghost rows are written as zero, as the merger
    leaves them unset), and write the merged file with x2(ny) rewritten."""
    with open(os.path.join(dirname, "3D001.tp")) as f:
        title = f.readline()
        f.readline()
        zone = f.readline()
    z = zone.replace(",", " ").replace("=", " ").split()
    nx, nyi = int(z[z.index("k") + 1]), int(z[z.index("j") + 1])
    ny = nyi + 2
    data = np.zeros((nx, ny, nz, 15))
    for r, (k0, k1) in enumerate(rank_ranges(nz, nproc)):
        with open(os.path.join(dirname, f"3D{r + 1:03d}.tp")) as f:
            if r == 0:
                for _ in range(3):
                    f.readline()
            vals = np.array(f.read().split(), dtype=np.float64)
        data[:, 1:ny - 1, k0:k1 + 1, :] = vals.reshape(nx, nyi, k1 - k0 + 1, 15)
    for q in (3, 4, 5):
        data[:, 0, :, q] = data[:, ny - 2, :, q]
        data[:, ny - 1, :, q] = data[:, 1, :, q]
    for q in (0, 2, 7, 8, 9, 13, 14):
        data[:, 0, :, q] = data[:, 1, :, q]
        data[:, ny - 1, :, q] = data[:, 1, :, q]
    dy = data[0, 2, 0, 1] - data[0, 1, 0, 1]
    data[:, 0, :, 1] = 0.0
    data[:, ny - 1, :, 1] = data[0, 1, 0, 1] + (ny - 2) * dy
    with open(os.path.join(dirname, out_name), "w") as f:
        f.write(title)
        f.write(' Variables = "x","y","z","U","V","W","P","Um","Vm","Wm","Uf","Vf","Wf","Wt","Nk"\n')
        f.write(f"ZONE k={nx:4d},j={ny:4d},i={nz:4d},DATAPACKING=\"POINT\"\n")
        for i in range(nx):
            f.write("\n")
            for j in range(ny):
                f.write("\n")
                for k in range(nz):
                    d = data[i, j, k]
                    f.write(_row(d[0], d[1], d[2], d[3:14], d[14]))


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
