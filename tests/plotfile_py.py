"""Independent reader and writer of the AMReX plotfile layout (test
infrastructure only; the library's own implementation is C++).

A plotfile directory holds a text Header (version "HyperCLaw-V1.1", component
names, dimension, time, finest level, problem extents, refinement ratios,
level domains, level steps, cell sizes, coordinate system, boundary width,
then per level "<lev> <nboxes> <time>", the level step, the physical extents
of every box, one line per direction, and the multifab path "Level_<l>/Cell"),
and per level a multifab header Cell_H (version, layout, ncomp, ghost count,
the box list "(n 0 ... )", "FabOnDisk: <file> <offset>" per box, per-box
minima and maxima) and data files of FABs: a text line
"FAB ((<bytes>, (<format>)),(<bytes>, (<byte order>)))<box> <ncomp>" followed
by the values, x fastest, component slowest.

This module writes that layout in the variants a reader has to accept (byte
order, 4- or 8-byte reals, FABs grown by ghost cells, several data files per
level) and reads it back, so that the library's writer and reader are each
checked against code that shares nothing with them.
"""
import os
import re

import numpy as np

FMT = {8: "64 11 52 0 1 12 0 1023", 4: "32 8 23 0 1 9 0 127"}


def box_text(lo, hi, D):
    t = lambda v: "(" + ",".join(str(int(x)) for x in v[:D]) + ")"
    return "(" + t(lo) + " " + t(hi) + " " + t([0] * D) + ")"


def write_plotfile(path, D, names, time, prob_lo, prob_hi, levels, byte_order="<", real_bytes=8, ngrow=0,
                   boxes_per_file=None, ghost_value=np.nan):
    """levels: list of dict(domain=(lo, hi), dx=[..], step=int, boxes=[(lo, hi)],
    data=[array (ncomp, nz, ny, nx) per box]); lo/hi are D-tuples."""
    ncomp = len(names)
    os.makedirs(path, exist_ok=True)
    h = ["HyperCLaw-V1.1", str(ncomp), *names, str(D), repr(float(time)), str(len(levels) - 1),
         " ".join(repr(float(x)) for x in prob_lo[:D]) + " ",
         " ".join(repr(float(x)) for x in prob_hi[:D]) + " ",
         " ".join("2" for _ in levels[1:]) + " ",
         " ".join(box_text(L["domain"][0], L["domain"][1], D) for L in levels) + " ",
         " ".join(str(L["step"]) for L in levels) + " "]
    for L in levels:
        h.append(" ".join(repr(float(x)) for x in L["dx"][:D]) + " ")
    h += ["0", "0"]
    dt = np.dtype(f"{byte_order}f{real_bytes}")
    order = " ".join(str(k) for k in (range(real_bytes, 0, -1) if byte_order == "<" else range(1, real_bytes + 1)))
    for l, L in enumerate(levels):
        nb = len(L["boxes"])
        h += [f"{l} {nb} {float(time)!r}", str(L["step"])]
        for lo, hi in L["boxes"]:
            for d in range(D):
                a = float(prob_lo[d] + L["dx"][d] * int(lo[d]))
                b_ = float(prob_lo[d] + L["dx"][d] * (int(hi[d]) + 1))
                h.append(f"{a!r} {b_!r}")
        h.append(f"Level_{l}/Cell")
        ldir = os.path.join(path, f"Level_{l}")
        os.makedirs(ldir, exist_ok=True)
        per = boxes_per_file or nb
        fod, files = [], {}
        for b, ((lo, hi), arr) in enumerate(zip(L["boxes"], L["data"])):
            fname = f"Cell_D_{b // per:05d}"
            f = files.get(fname)
            if f is None:
                f = files[fname] = open(os.path.join(ldir, fname), "wb")
            glo = [lo[d] - ngrow for d in range(D)]
            ghi = [hi[d] + ngrow for d in range(D)]
            shape = (ncomp,) + tuple(ghi[d] - glo[d] + 1 for d in reversed(range(D)))
            full = np.full(shape, ghost_value, dtype=np.float64)
            inner = (slice(None),) + tuple(slice(ngrow, ngrow + hi[d] - lo[d] + 1) for d in reversed(range(D)))
            full[inner] = arr
            fod.append((fname, f.tell()))
            f.write(f"FAB (({real_bytes}, ({FMT[real_bytes]})),({real_bytes}, ({order})))"
                    f"{box_text(glo, ghi, D)} {ncomp}\n".encode())
            f.write(full.astype(dt).tobytes())
        for f in files.values():
            f.close()
        c = ["1", "1", str(ncomp), str(ngrow), f"({nb} 0"]
        c += [box_text(lo, hi, D) for lo, hi in L["boxes"]]
        c += [")", str(nb)]
        c += [f"FabOnDisk: {n} {o}" for n, o in fod]
        c.append("")
        for red in (np.min, np.max):
            c.append(f"{nb},{ncomp}")
            for arr in L["data"]:
                c.append("".join(f"{float(red(arr[k]))!r}," for k in range(ncomp)))
            c.append("")
        with open(os.path.join(ldir, "Cell_H"), "w") as f:
            f.write("\n".join(c) + "\n")
    with open(os.path.join(path, "Header"), "w") as f:
        f.write("\n".join(h) + "\n")


_INT = re.compile(r"-?\d+")


def _box(s, D):
    v = [int(x) for x in _INT.findall(s)]
    assert len(v) == 3 * D, s
    return tuple(v[:D]), tuple(v[D:2 * D])


def read_plotfile(path):
    """Parse a plotfile directory; returns a dict with the header fields and
    per level: boxes, extents, data (list of (ncomp, nz, ny, nx) arrays),
    mins, maxs (from Cell_H)."""
    with open(os.path.join(path, "Header")) as f:
        lines = f.read().split("\n")
    it = iter(lines)
    out = {"version": next(it)}
    ncomp = int(next(it))
    out["names"] = [next(it) for _ in range(ncomp)]
    D = out["dim"] = int(next(it))
    out["time"] = float(next(it))
    finest = out["finest_level"] = int(next(it))
    out["prob_lo"] = [float(x) for x in next(it).split()]
    out["prob_hi"] = [float(x) for x in next(it).split()]
    out["ref_ratio"] = [int(x) for x in next(it).split()]
    doms = re.findall(r"\(\([^()]*\) \([^()]*\) \([^()]*\)\)", next(it))
    out["domains"] = [_box(s, D) for s in doms]
    out["level_steps"] = [int(x) for x in next(it).split()]
    out["dx"] = [[float(x) for x in next(it).split()] for _ in range(finest + 1)]
    out["coord"] = int(next(it))
    out["bwidth"] = int(next(it))
    levels = []
    for l in range(finest + 1):
        lev, nb, t = next(it).split()
        assert int(lev) == l
        step = int(next(it))
        ext = [[tuple(float(x) for x in next(it).split()) for _ in range(D)] for _ in range(int(nb))]
        mf = next(it)
        levels.append(dict(nbox=int(nb), time=float(t), step=step, extents=ext, mf=mf))
    for L in levels:
        with open(os.path.join(path, L["mf"] + "_H")) as f:
            text = f.read()
        toks = text.split("\n")
        L["cellh_head"] = toks[:4]
        boxes = [_box(s, D) for s in re.findall(r"\(\([^()]*\) \([^()]*\) \([^()]*\)\)", text)]
        fods = re.findall(r"FabOnDisk: (\S+) (\d+)", text)
        assert len(boxes) == len(fods) == L["nbox"]
        mm = re.findall(r"^(\d+),(\d+)$", text, flags=re.M)
        tail = text.split("\n")
        rows = [r for r in tail if r.endswith(",") and "," in r and not r.startswith("FabOnDisk")]
        nb = L["nbox"]
        vals = [[float(x) for x in r.rstrip(",").split(",")] for r in rows]
        L["mins"], L["maxs"] = vals[:nb], vals[nb:2 * nb]
        assert len(mm) == 2
        L["boxes"] = boxes
        base = os.path.dirname(os.path.join(path, L["mf"]))
        data = []
        for (lo, hi), (fname, off) in zip(boxes, fods):
            with open(os.path.join(base, fname), "rb") as f:
                f.seek(int(off))
                head = f.readline().decode()
                m = re.match(r"FAB \(\((\d+), \(([0-9 ]+)\)\),\((\d+), \(([0-9 ]+)\)\)\)(\(.*\)) (\d+)\n$", head)
                assert m, head
                nbytes = int(m.group(1))
                order = [int(x) for x in m.group(4).split()]
                bo = "<" if order == list(range(nbytes, 0, -1)) else ">"
                flo, fhi = _box(m.group(5), D)
                nc = int(m.group(6))
                shape = (nc,) + tuple(fhi[d] - flo[d] + 1 for d in reversed(range(D)))
                arr = np.frombuffer(f.read(int(np.prod(shape)) * nbytes), dtype=f"{bo}f{nbytes}").reshape(shape)
                sl = (slice(None),) + tuple(slice(lo[d] - flo[d], hi[d] - flo[d] + 1) for d in reversed(range(D)))
                data.append(np.array(arr[sl], dtype=np.float64))
        L["data"] = data
    out["levels"] = levels
    return out


def level_from_state(U, ijk, boxes, D):
    """Per-box (ncomp, nz, ny, nx) arrays of U (cells in state order, [n, ncomp],
    with cell indices ijk [n, 3]) for the given boxes."""
    hi = ijk.max(axis=0)
    dense = np.full((U.shape[1],) + tuple(int(hi[d]) + 1 for d in reversed(range(D))), np.nan)
    dense[(slice(None),) + tuple(ijk[:, d] for d in reversed(range(D)))] = U.T
    return [dense[(slice(None),) + tuple(slice(lo[d], hi_[d] + 1) for d in reversed(range(D)))].copy()
            for lo, hi_ in boxes]
