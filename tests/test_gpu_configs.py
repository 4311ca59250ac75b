"""The plain FP64 GPU path against the oracle on the benchmark configurations
at their stated sizes and step counts, each side from its own projection of
the initial condition:

  1  isentropic vortex p=1, 32^2, 20 steps
  2  Kelvin-Helmholtz p=3, 256^2, 100 steps
  3  Kelvin-Helmholtz p=3, three levels 64^2 -> 256^2, regrid every 4 steps,
     200 steps: tags and boxes identical before and after every step
  5  3D blast p=2, two levels with outflow boundaries.  The oracle holds every
     level as a dense array (the 128^3 level alone would need tens of GB), so
     this runs at 32^3 -> 64^3: unlimited for 30 steps (the unlimited scheme
     survives 44 steps at this size, then a cell mean density turns
     negative), and with the TVB limiter stage by stage, the limiter of both
     sides fed the identical pre-limiter state at every step.

Every modal coefficient must agree within 1e-12 relative (to the variable's
largest cell mean).  The density L1 and L2 norms of the difference over the
leaf cells (the reference's Lp norm machinery applied to the two solutions)
are reported per configuration; with ADG_ACCURACY_JSON set they are merged
into that JSON file.
"""
import json
import os

import numpy as np
import pytest

import oracle_ffi as O
from parity import G, rel_err

pytestmark = pytest.mark.gpu

import bench  # noqa: E402  (the workload definitions of the benchmark)

TOL = 1e-12


def record(name, entry):
    path = os.environ.get("ADG_ACCURACY_JSON")
    print(name, json.dumps(entry))
    if not path:
        return
    try:
        db = json.load(open(path))
    except Exception:
        db = {}
    db[name] = entry
    with open(path, "w") as f:
        json.dump(db, f, indent=1, sort_keys=True)


def same_layout(g, o):
    return g.num_levels() == o.num_levels() and all(
        np.array_equal(g.boxes(l), o.boxes(l)) for l in range(o.num_levels()))


def compare(name, g, o, w, steps, extra=None):
    assert same_layout(g, o)
    levels = [g.get_U_w(l) for l in range(g.num_levels())]
    per_level = [rel_err(levels[l], o.get_uw(l)) for l in range(o.num_levels())]
    entry = {"workload": w, "steps": steps, "levels": o.num_levels(),
             "cells": [o.ncells_level(l) for l in range(o.num_levels())],
             "max_rel_modal": per_level,
             "density_L1_diff": o.norm_diff(levels, 1, 0), "density_L2_diff": o.norm_diff(levels, 2, 0),
             "density_L2_oracle_scale": o.norm_diff([np.zeros_like(a) for a in levels], 2, 0),
             "dt_rel": abs(g.Dt - o.dt) / o.dt}
    if extra:
        entry.update(extra)
    record(name, entry)
    assert max(per_level) < TOL, per_level
    assert g.status() == 0


def run_pair(name, w, steps, check_tags=False):
    O.set_threads(os.cpu_count())
    o = bench.oracle_sim(w)
    o.init()
    g = bench.make_sim(G, w)
    assert same_layout(g, o)
    for l in range(o.num_levels()):
        assert rel_err(g.get_U_w(l), o.get_uw(l)) < 1e-13
    assert abs(g.Dt - o.dt) <= 1e-13 * o.dt
    amr = w.get("amr")
    regrids = 0
    for s in range(steps):
        if check_tags and amr:
            due = s == 0 or s % amr["dtn_regrid"] == 0
            if due:
                for l in range(min(o.num_levels(), amr["max_level"])):
                    assert np.array_equal(g.tags(l), o.tags(l).astype(np.uint8)), f"tags of level {l}, step {s}"
                regrids += 1
        o.step()
        g.time_integration()
        if amr:
            assert same_layout(g, o), f"layout after step {s}"
    compare(name, g, o, name.split(":")[0], steps, {"regrids_checked": regrids} if check_tags else None)


def test_config1_vortex_p1_32_20_steps():
    run_pair("vortex_p1_32", bench.WORKLOADS["vortex_p1_32"], 20)


def test_config2_kh_p3_256_100_steps():
    run_pair("kh_p3_256", bench.WORKLOADS["kh_p3_256"], 100)


def test_config3_kh_p3_amr3_200_steps_same_tags_and_boxes():
    run_pair("kh_p3_amr3", bench.WORKLOADS["kh_p3_amr3"], 200, check_tags=True)


def blast32(limited):
    w = dict(bench.WORKLOADS["blast3d_p2_amr2"])
    w["n"] = (32, 32, 32)
    if not limited:
        w.pop("limiter")
    return w


def test_config5_blast3d_unlimited_32_to_64_30_steps():
    run_pair("blast3d_p2_amr2:32^3 unlimited", blast32(False), 30, check_tags=True)


def test_config5_blast3d_limiter_on_identical_pre_limiter_state():
    """Every step: both sides start from the GPU's state (the oracle's ghost
    cells filled from it), run ADER, then both limiters run on the GPU's
    pre-limiter state.  The limiter's troubled-cell test is discontinuous and
    the symmetric blast puts cells on exact ties, so the two sides' ADER
    results (which differ in the last bits: the GPU contracts to FMA) would
    decide some ties differently; on identical input the limiters must agree
    on every cell."""
    w = blast32(True)
    o = bench.oracle_sim(w)
    o.init()
    g = bench.make_sim(G, w)
    o.step()
    g.time_integration()  # the first step regrids from the full-domain start
    assert same_layout(g, o)
    total, worst = 0, 0.0
    F = g.num_levels() - 1
    for s in range(8):
        for l in range(g.num_levels()):
            o.set_uw(g.get_U_w(l), l)
        o.fill_patch()
        o.dt = g.Dt
        o.ader()
        g.ADER()
        for l in range(g.num_levels()):
            o.set_uw(g.get_U_w(l), l)
        no = o.limit()
        ng = g.Limiter_w()
        assert ng == no, f"limited cells at step {s}: GPU {ng}, oracle {no}"
        total += ng
        d = rel_err(g.get_U_w(F), o.get_uw(F))
        worst = max(worst, d)
        assert d < 1e-13, f"step {s}: {d}"
        g.average_down()
        g.fill_ghosts()
        g.set_Dt()
    assert total > 0
    record("blast3d_p2_amr2:32^3 limiter on identical input",
           {"steps": 8, "limited_cells": total, "max_rel_modal_finest": worst})
