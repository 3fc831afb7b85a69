"""Parity at the benchmark configurations' stated sizes, and the error of
the single-precision runs against a double-precision run of the same scheme.

* Flat configuration (100 x 100 x 60, CFS-PML 10, explosive source, 20 line
  receivers and 20 stations), 501 executed steps: the GPU against the
  reference's own CPU build (tests/golden/configs/c0_flat_explosion_501.npz,
  made by tests/golden/configs/make_config_golden.py): line and station
  seismograms, four planes of the final state through the source, and the
  same planes after 251 steps (a second reference run).
* Topography configuration at its full 400 x 400 x 200 size (CFS-PML 12, 400
  surface receivers), 50 steps, and the VTI and GMB visco-elastic media at
  their full 300 x 300 x 150 size, 100 steps each: the GPU against the
  oracle (bit-identical to the reference, tests/test_oracle_golden.py and
  tests/test_oracle_configs.py), whole final state, PML auxiliaries and
  seismograms.  These runs start from a smooth seeded state (white noise
  smoothed by two binomial passes per axis) so that every receiver and
  every boundary branch carries signal from the first step; the
  configuration's own source runs as well.

The runs are also made by the double-precision oracle (oracle/
cgfd_oracle_f64.c: the same scheme and inputs, 53-bit arithmetic) -- the
flat configuration always, the full-size ones with $CGFD_PARITY_FP64 set --
and the relative L2 and max-abs/peak of both single-precision runs (the GPU
and the reference, or its bit-identical oracle) against it are printed and,
with $CGFD_PARITY_REPORT set, appended as JSON lines to that file.
"""

import json
import os

import numpy as np
import pytest

import oracle
from helpers import MAX_ABS_OF_PEAK, REL_L2, max_abs_of_peak, rel_l2

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
C0_FIXTURE = os.path.join(HERE, "golden", "configs", "c0_flat_explosion_501.npz")
NCPU = os.cpu_count() or 4


def _planes(p, w):
    """The planes the flat-configuration fixture keeps (padded indices)."""
    import sys
    sys.path.insert(0, os.path.join(HERE, "golden", "configs"))
    from make_config_golden import planes_of
    return planes_of(w, p.ncmp, p.nx, p.ny, p.nz)


def _binomial(a, axis, passes=2):
    k = np.array([1.0, 4.0, 6.0, 4.0, 1.0], np.float32) / 16.0
    for _ in range(passes):
        pad = [(0, 0)] * a.ndim
        pad[axis] = (2, 2)
        b = np.pad(a, pad, mode="edge")
        n = a.shape[axis]
        out = np.zeros_like(a)
        for t in range(5):
            sl = [slice(None)] * a.ndim
            sl[axis] = slice(t, t + n)
            out += k[t] * b[tuple(sl)]
        a = out
    return a


def smooth_state(p, seed, amp_v=1e-2):
    """Level 0 of the nine wavefield components set to seeded smooth noise
    on the physical points (velocity amp_v, stress amp_v * rho vp of a
    typical crust)."""
    rng = np.random.default_rng(seed)
    core = (slice(p.nk1, p.nk2 + 1), slice(p.nj1, p.nj2 + 1), slice(p.ni1, p.ni2 + 1))
    lev0 = p.level(0).reshape(p.ncmp, p.nz, p.ny, p.nx)
    for c in range(9):
        a = rng.uniform(-1.0, 1.0, (p.nk, p.nj, p.ni)).astype(np.float32)
        for ax in range(3):
            a = _binomial(a, ax)
        a *= np.float32(1.0 / max(float(np.abs(a).max()), 1e-30))
        amp = amp_v if c < 3 else amp_v * 2700.0 * 6000.0
        lev0[c][core] = (amp * a).astype(np.float32)


def _errors(got, ref):
    return {"rel_l2": rel_l2(got, ref), "max_abs_of_peak": max_abs_of_peak(got, ref)}


def _report(config, rows):
    for what, e in rows.items():
        print("%-28s %-36s rel_l2=%.3e max_abs/peak=%.3e"
              % (config, what, e["rel_l2"], e["max_abs_of_peak"]))
    path = os.environ.get("CGFD_PARITY_REPORT")
    if path:
        with open(path, "a") as f:
            f.write(json.dumps({"config": config, "errors": rows}) + "\n")


def _check(rows, keys):
    bad = {k: rows[k] for k in keys
           if rows[k]["rel_l2"] > REL_L2 or rows[k]["max_abs_of_peak"] > MAX_ABS_OF_PEAK}
    assert not bad, bad


def _truncated(p, nt):
    """The problem run for its first nt steps only (same inputs; the
    seismogram buffers sized for nt samples)."""
    q = p.copy()
    q.nt_total = nt
    for rec in (q.recv, q.line):
        if rec is not None:
            rec["max_nt"] = nt
            rec["seismo"] = np.zeros(rec["seismo"].size // p.nt_total * nt, np.float32)
    return q


def test_c0_flat_501_against_reference():
    """Seismograms after 501 steps and a snapshot after 251 steps within the
    stated bar of the reference; the final state after 501 steps -- most of
    the wavefield has left through the PML by then, and what is left is
    small next to FP32 rounding noise -- as close to the reference as the
    reference itself is to the double-precision run (the GPU no less
    accurate than the reference against FP64)."""
    from cgfd3d_gb300 import problem, solver
    p, exp = problem.from_golden(C0_FIXTURE)
    assert p.nt_total == 501 and (p.ni, p.nj, p.nk) == (100, 100, 60)
    fix = np.load(C0_FIXTURE)
    mid_ref = {k[len("out.t251.plane."):]: fix[k] for k in fix.files
               if k.startswith("out.t251.plane.")}
    rows = {}
    for tag, prob, ref_planes in (("", p, exp["planes"]), ("t251 ", _truncated(p, 251), mid_ref)):
        w = oracle.allstep64(prob, oracle.TIMG_ZERO, NCPU)
        g = prob.copy()
        solver.drv_rk_curv_col_allstep(g)
        lev = g.final_level()
        pg, pw = _planes(g, g.level(lev)), _planes(w, w.level(lev))
        for k in sorted(ref_planes):
            rows["gpu vs reference %splane %s" % (tag, k)] = _errors(pg[k], ref_planes[k])
            rows["gpu vs fp64 %splane %s" % (tag, k)] = _errors(pg[k], pw[k])
            rows["reference vs fp64 %splane %s" % (tag, k)] = _errors(ref_planes[k], pw[k])
        if tag:
            continue
        for name, key in (("line", "line"), ("stations", "recv")):
            got = (g.line if key == "line" else g.recv)["seismo"]
            f64 = (w.line if key == "line" else w.recv)["seismo"]
            rows["gpu vs reference " + name] = _errors(got, exp[key])
            rows["gpu vs fp64 " + name] = _errors(got, f64)
            rows["reference vs fp64 " + name] = _errors(exp[key], f64)
    _report("flat 100x100x60 501 steps", rows)
    _check(rows, ["gpu vs reference line", "gpu vs reference stations"] +
           ["gpu vs reference t251 plane " + k for k in mid_ref])
    for k in exp["planes"]:
        g64, r64 = rows["gpu vs fp64 plane " + k], rows["reference vs fp64 plane " + k]
        gr = rows["gpu vs reference plane " + k]
        for m in ("rel_l2", "max_abs_of_peak"):
            assert g64[m] <= 1.25 * r64[m], (k, m, g64, r64)
            assert gr[m] <= max(2.0 * r64[m], REL_L2 if m == "rel_l2" else MAX_ABS_OF_PEAK), \
                (k, m, gr, r64)


def _model_run(p, config, pml_check=True):
    """GPU against the FP32 oracle (the parity bar) and, with
    $CGFD_PARITY_FP64 set, both against the FP64 oracle (minutes of host
    time per full-size model, so off by default)."""
    from cgfd3d_gb300 import solver
    w = oracle.allstep64(p, oracle.TIMG_ZERO, NCPU) if os.environ.get("CGFD_PARITY_FP64") \
        else None
    q = p.copy()
    oracle.allstep(q, oracle.TIMG_ZERO, NCPU)
    solver.drv_rk_curv_col_allstep(p)
    lev = p.final_level()
    rows = {
        "gpu vs oracle state": _errors(p.level(lev), q.level(lev)),
        "gpu vs oracle receivers": _errors(p.recv["seismo"], q.recv["seismo"]),
    }
    if w is not None:
        rows.update({
            "gpu vs fp64 state": _errors(p.level(lev), w.level(lev)),
            "oracle vs fp64 state": _errors(q.level(lev), w.level(lev)),
            "gpu vs fp64 receivers": _errors(p.recv["seismo"], w.recv["seismo"]),
            "oracle vs fp64 receivers": _errors(q.recv["seismo"], w.recv["seismo"]),
        })
    keys = ["gpu vs oracle state", "gpu vs oracle receivers"]
    if pml_check:
        for d in range(3):
            for s in range(2):
                if p.pml[d][s] is not None:
                    k = "gpu vs oracle pml %d %d" % (d, s)
                    rows[k] = _errors(p.pml_final(d, s), q.pml_final(d, s))
                    keys.append(k)
    _report(config, rows)
    _check(rows, keys)


def test_c1_topography_full_size():
    from cgfd3d_gb300 import models
    p = models.topo_model(ni=400, nj=400, nk=200, steps=50, nrecv=400)
    assert p.recv["n"] == 400 and p.nt_total == 51
    smooth_state(p, 101)
    _model_run(p, "topography 400x400x200 50 steps")


@pytest.mark.parametrize("kind", ["vti", "visco"])
def test_c2_media_full_size(kind):
    from cgfd3d_gb300 import models
    p = models.topo_media_model(kind, ni=300, nj=300, nk=150, steps=100, nrecv=400)
    assert p.nt_total == 101
    smooth_state(p, 202 if kind == "vti" else 303)
    _model_run(p, "%s 300x300x150 100 steps" % kind)
