"""Plotfile header parsing of the library on the CPU (no context, no GPU):
adg_plotfile_info on plotfiles written by an independent writer, in every
variant a reader must accept, and on malformed ones, which must be rejected
with ADG_ERR_IO and a reason instead of being read."""
import os
import shutil

import numpy as np
import pytest

from parity import G
from plotfile_py import write_plotfile

ADG_ERR_IO = 7


def two_level(D=2, ncomp=10, step=8, time=0.1234567890123456789):
    rng = np.random.default_rng(7)
    n0 = 8
    lv0 = dict(domain=((0,) * D, (n0 - 1,) * D), dx=[1.0 / n0] * D, step=step,
               boxes=[((0,) * D, (n0 // 2 - 1,) + (n0 - 1,) * (D - 1)),
                      ((n0 // 2,) + (0,) * (D - 1), (n0 - 1,) * D)])
    lv1 = dict(domain=((0,) * D, (2 * n0 - 1,) * D), dx=[0.5 / n0] * D, step=step,
               boxes=[((4,) * D, (11,) * D)])
    for L in (lv0, lv1):
        L["data"] = [rng.standard_normal((ncomp,) + tuple(hi[d] - lo[d] + 1 for d in reversed(range(D))))
                     for lo, hi in L["boxes"]]
    names = [f"mass_density_{m}" for m in range(ncomp)]
    return dict(D=D, names=names, time=time, prob_lo=[0.0] * D, prob_hi=[1.0] * D, levels=[lv0, lv1])


@pytest.mark.parametrize("variant", [dict(), dict(byte_order=">"), dict(real_bytes=4), dict(ngrow=1),
                                     dict(boxes_per_file=1)])
@pytest.mark.parametrize("D", [2, 3])
def test_info_accepts_reader_variants(tmp_path, D, variant):
    pf = two_level(D=D)
    path = str(tmp_path / "tstep_8_q_0_plt")
    write_plotfile(path, pf["D"], pf["names"], pf["time"], pf["prob_lo"], pf["prob_hi"], pf["levels"], **variant)
    info = G.plotfile_info(path)
    assert info == dict(dim=D, ncomp=10, finest_level=1, time=pf["time"], step=8)


def _corrupt(path, rel, fn):
    p = os.path.join(path, rel)
    with open(p, "rb") as f:
        b = f.read()
    with open(p, "wb") as f:
        f.write(fn(b))


CORRUPTIONS = {
    "version": ("Header", lambda b: b.replace(b"HyperCLaw-V1.1", b"HyperCLaw-V9.9", 1), "HyperCLaw"),
    "dimension": ("Header", lambda b: b.replace(b"\n2\n", b"\n7\n", 1), "dimension"),
    "ratio_count": ("Header", lambda b: b.replace(b"\n2 \n", b"\n2 2 \n", 1), "refinement ratio"),
    "box_count": ("Header", lambda b: b.replace(b"\n0 2 ", b"\n0 3 ", 1), "box extents"),
    "path_escape": ("Header", lambda b: b.replace(b"Level_1/Cell", b"../Level_1/Cell", 1), "multifab path"),
    "truncated_data": ("Level_1/Cell_D_00000", lambda b: b[:-8], "too short"),
    "fab_format": ("Level_0/Cell_D_00000", lambda b: b.replace(b"64 11 52", b"64 15 48", 1), "number format"),
    "byte_order": ("Level_0/Cell_D_00000", lambda b: b.replace(b"8 7 6 5 4 3 2 1", b"8 7 6 5 1 2 3 4", 1),
                   "byte order"),
    "fab_entry": ("Level_0/Cell_H", lambda b: b.replace(b"FabOnDisk:", b"FabOnDisc:", 1), "FabOnDisk"),
    "fab_file_escape": ("Level_0/Cell_H", lambda b: b.replace(b"FabOnDisk: Cell_D", b"FabOnDisk: ../Cell_D", 1),
                        "outside the level directory"),
    "ncomp": ("Level_1/Cell_H", lambda b: b.replace(b"1\n1\n10\n", b"1\n1\n11\n", 1), "component count"),
    "offset": ("Level_0/Cell_H", lambda b: b.replace(b"FabOnDisk: Cell_D_00000 0", b"FabOnDisk: Cell_D_00000 5", 1),
               "FAB header"),
}


@pytest.mark.parametrize("case", list(CORRUPTIONS))
def test_info_rejects_malformed(tmp_path, case):
    pf = two_level(D=2)
    path = str(tmp_path / "p")
    write_plotfile(path, pf["D"], pf["names"], pf["time"], pf["prob_lo"], pf["prob_hi"], pf["levels"])
    rel, fn, why = CORRUPTIONS[case]
    _corrupt(path, rel, fn)
    with pytest.raises(G.AdgError) as e:
        G.plotfile_info(path)
    assert f"status {ADG_ERR_IO}" in str(e.value) and why in str(e.value), str(e.value)


def test_info_rejects_missing_level_file(tmp_path):
    pf = two_level(D=2)
    path = str(tmp_path / "p")
    write_plotfile(path, pf["D"], pf["names"], pf["time"], pf["prob_lo"], pf["prob_hi"], pf["levels"])
    shutil.rmtree(os.path.join(path, "Level_1"))
    with pytest.raises(G.AdgError, match="cannot open"):
        G.plotfile_info(path)
