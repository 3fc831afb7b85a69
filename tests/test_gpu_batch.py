"""Batched shots (cgfd_batch_*) against single-shot runs of the same problems.

A batch steps every shot with one stage launch per RK stage over all shots'
tiles and replays whole 8-step operator cycles from a CUDA graph; the
per-point arithmetic is the single-shot kernel's, so every shot's wavefield,
PML auxiliaries and seismograms must equal its single-shot run exactly.
"""

import numpy as np
import pytest

from helpers import assert_parity

pytestmark = pytest.mark.gpu


def _noise(p, seed):
    rng = np.random.default_rng(seed)
    lev0 = p.level(0).reshape(p.ncmp, p.nz, p.ny, p.nx)
    core = (slice(p.nk1, p.nk2 + 1), slice(p.nj1, p.nj2 + 1), slice(p.ni1, p.ni2 + 1))
    for c in range(p.ncmp):
        amp = 1e-2 if c < 3 else 1e-2 * 2700 * 6000
        lev0[c][core] = (amp * rng.uniform(-1, 1, lev0[c][core].shape)).astype(np.float32)


@pytest.fixture(scope="module")
def base():
    from cgfd3d_gb300 import models
    return models._topo_base(150, 140, 110, 11)


def _shots(base, n, steps, seed):
    from cgfd3d_gb300 import models
    shots = models.window_shots(n, base=(150, 140, 110), wmin=(56, 48, 40),
                                wmax=(110, 100, 80), steps=steps, base_model=base,
                                seed=seed, nrecv=16)
    for k, p in enumerate(shots):
        _noise(p, seed + k)
    return shots


def _same(a, b, what):
    np.testing.assert_array_equal(a, b, err_msg=what)


@pytest.mark.parametrize("graph,persistent", [("1", 0), ("0", 0), ("1", 1), ("0", 1)])
def test_batch_equals_single_shots(base, graph, persistent, monkeypatch):
    """Three windows of different sizes, 19 steps (two graph cycles and an
    eager tail, or all eager), one CTA per item or persistent CTAs taking
    the items largest first: each shot equals its single-shot run."""
    from cgfd3d_gb300 import solver
    monkeypatch.setenv("CGFD_BATCH_GRAPH", graph)
    shots = _shots(base, 3, 18, 21)
    singles = [p.copy() for p in shots]
    with solver.Batch(shots, kchunk=12) as b:
        b.set_schedule(persistent)
        assert b.schedule() == persistent
        b.run(3)
        b.run(16)
        b.fetch()
        ms, launches = b.times()
        assert ms > 0 and launches > 0
    for p, q in zip(shots, singles):
        solver.drv_rk_curv_col_allstep(q)
        lev = p.final_level()
        _same(p.level(lev), q.level(lev), "wavefield")
        for d in range(3):
            for s in range(2):
                if p.pml[d][s] is not None:
                    _same(p.pml_final(d, s), q.pml_final(d, s), "pml %d %d" % (d, s))
        _same(p.recv["seismo"], q.recv["seismo"], "receivers")


def test_batch_autotune_resets_state(base, tmp_path):
    """The autotuner times candidate k-chunks on the live shots, then resets
    them: the run afterwards equals single-shot runs from the inputs; the
    choice is cached."""
    from cgfd3d_gb300 import solver
    shots = _shots(base, 2, 9, 31)
    singles = [p.copy() for p in shots]
    cache = str(tmp_path / "tune.json")
    with solver.Batch(shots) as b:
        res = b.autotune(candidates=(8, 16, 24), steps=2, cache=cache, key="k")
        assert res["kchunk"] in (8, 16, 24) and len(res["ms"]) == 3
        assert res["persistent"] in (0, 1) and len(res["ms_persistent"]) == 3
        assert b.schedule() == res["persistent"]
        b.run(shots[0].nt_total)
        b.fetch()
    with solver.Batch([p.copy() for p in singles]) as b2:
        got = b2.autotune(cache=cache, key="k")
        assert got["kchunk"] == res["kchunk"] and b2.schedule() == res["persistent"]
    for p, q in zip(shots, singles):
        solver.drv_rk_curv_col_allstep(q)
        lev = p.final_level()
        assert_parity(p.level(lev), q.level(lev), "autotuned batch")
        _same(p.level(lev), q.level(lev), "autotuned batch (exact)")


def test_batch_vti(base):
    """VTI windows in a batch equal their single-shot runs."""
    from cgfd3d_gb300 import models, solver
    shots = _shots(base, 2, 9, 41)
    for p in shots:
        rho = 1.0 / p.media["slw"].astype(np.float64)
        mu = p.media["mu"].astype(np.float64)
        lam = p.media["lambda"].astype(np.float64)
        vp, vs = np.sqrt((lam + 2 * mu) / rho), np.sqrt(mu / rho)
        c11, c13, c33, c55, c66 = models.thomsen_to_vti(vp, vs, rho, 0.1, 0.05, 0.08)
        p.medium_type = 3
        p.media = {"slw": p.media["slw"], "c11": c11, "c13": c13, "c33": c33,
                   "c55": c55, "c66": c66}
    singles = [p.copy() for p in shots]
    with solver.Batch(shots) as b:
        b.run(shots[0].nt_total)
        b.fetch()
    for p, q in zip(shots, singles):
        solver.drv_rk_curv_col_allstep(q)
        lev = p.final_level()
        _same(p.level(lev), q.level(lev), "vti wavefield")


def test_batch_rejects_mixed_media(base):
    from cgfd3d_gb300 import _lib, solver
    shots = _shots(base, 2, 3, 51)
    shots[1].medium_type = 3
    shots[1].media = dict(shots[1].media, c11=shots[1].media["lambda"],
                          c13=shots[1].media["lambda"], c33=shots[1].media["lambda"],
                          c55=shots[1].media["mu"], c66=shots[1].media["mu"])
    with pytest.raises(_lib.CgfdError):
        solver.Batch(shots)


def test_batch_graves_q(base):
    """Graves Q attenuation (the last stage's factor) in a batch equals the
    single-shot runs; the exponential sponge is refused in batches."""
    from cgfd3d_gb300 import _lib, solver
    shots = _shots(base, 2, 9, 61)
    rng = np.random.default_rng(3)
    for p in shots:
        p.graves_qs = dict(Qs=rng.uniform(15, 25, p.vol).astype(np.float32), freq=2.0)
    singles = [p.copy() for p in shots]
    with solver.Batch(shots) as b:
        b.run(shots[0].nt_total)
        b.fetch()
    for p, q in zip(shots, singles):
        solver.drv_rk_curv_col_allstep(q)
        lev = p.final_level()
        _same(p.level(lev), q.level(lev), "graves wavefield")
    bad = _shots(base, 2, 3, 71)
    bad[1].ablexp = dict(Ex=np.ones(bad[1].nx, np.float32), Ey=np.ones(bad[1].ny, np.float32),
                         Ez=np.ones(bad[1].nz, np.float32), blk=np.zeros((6, 7), np.int32))
    with pytest.raises(_lib.CgfdError):
        solver.Batch(bad)
