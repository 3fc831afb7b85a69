"""GPU against the oracle for the isotropic, VTI and GMB visco-elastic media.

The oracle is pinned bit-for-bit to the reference for both media
(test_oracle_golden.py, fixtures vti_topo_noise and visco_topo_noise).  Here
the GPU library and the oracle run the same synthetic topography model with
a VTI or a visco-elastic (three Maxwell bodies) medium from a seeded noise
state -- wavefield, memory variables and PML auxiliaries -- so that every
operator tap, every boundary branch and the attenuation terms act from the
first step, with the CFS-PML terms inside the stage kernel and by the face
kernels.  Tolerance: relative L2 <= 1e-5 and max-abs <= 1e-4 of the peak
(tests/helpers.py).
"""

import os

import numpy as np
import pytest

import oracle
from helpers import assert_parity

pytestmark = pytest.mark.gpu


def _noise(p, seed, amp_v=1e-2):
    rng = np.random.default_rng(seed)
    lev0 = p.level(0).reshape(p.ncmp, p.nz, p.ny, p.nx)
    core = (slice(p.nk1, p.nk2 + 1), slice(p.nj1, p.nj2 + 1), slice(p.ni1, p.ni2 + 1))
    for c in range(p.ncmp):
        amp = amp_v if c < 3 else amp_v * 2700 * 6000
        if c >= 9:
            amp *= 1e-3      # memory variables
        lev0[c][core] = (amp * rng.uniform(-1, 1, lev0[c][core].shape)).astype(np.float32)
    for row in p.pml:
        for f in row:
            if f is not None:
                n = f["aux"].size // 4
                f["aux"][:n] = (amp_v * 0.1 * rng.uniform(-1, 1, n)).astype(np.float32)


def _compare(p_gpu, p_cpu, what):
    lev = p_gpu.final_level()
    g = p_gpu.level(lev).reshape(p_gpu.ncmp, -1)
    c = p_cpu.level(lev).reshape(p_cpu.ncmp, -1)
    assert_parity(g[:9], c[:9], what + " wavefield")
    if p_gpu.ncmp > 9:
        assert_parity(g[9:], c[9:], what + " memory variables")
    for d in range(3):
        for s in range(2):
            if p_gpu.pml[d][s] is not None:
                assert_parity(p_gpu.pml_final(d, s), p_cpu.pml_final(d, s),
                              "%s pml %d %d" % (what, d, s))
    if p_gpu.recv is not None and p_gpu.recv["n"] > 0:
        assert_parity(p_gpu.recv["seismo"], p_cpu.recv["seismo"], what + " receivers")


@pytest.fixture(params=["default", "fused", "split"])
def pml_mode(request, monkeypatch):
    """CFS-PML inside the stage kernel or by the face kernels (both forms
    must give the same result for every medium)."""
    if request.param == "fused":
        monkeypatch.setenv("CGFD_PML_SPLIT", "0")
    elif request.param == "split":
        monkeypatch.setenv("CGFD_PML_SPLIT", "1")
    return request.param


@pytest.mark.parametrize("kind", ["iso", "vti", "visco", "aniso"])
@pytest.mark.parametrize("shape", [(96, 80, 48), (70, 45, 37)])
def test_media_model_noise_state(kind, shape, pml_mode):
    from cgfd3d_gb300 import models, solver
    ni, nj, nk = shape
    if kind == "iso":
        p = models.topo_model(ni=ni, nj=nj, nk=nk, steps=9, dt=0.005, nrecv=16)
    else:
        p = models.topo_media_model(kind, ni=ni, nj=nj, nk=nk, steps=9,
                                    dt=0.005, nrecv=16)
    _noise(p, 5)
    q = p.copy()
    solver.drv_rk_curv_col_allstep(p)
    oracle.allstep(q, oracle.TIMG_ZERO, os.cpu_count() or 4)
    _compare(p, q, "%s %s" % (kind, shape))


@pytest.mark.parametrize("kind", ["vti", "visco", "aniso"])
def test_media_surface_matrices(kind):
    """Free-surface matrices computed on the device against the oracle's
    (and, for visco, the surface rotation matrices)."""
    from cgfd3d_gb300 import models, solver
    p = models.topo_media_model(kind, ni=64, nj=48, nk=30, steps=1, dt=0.005,
                                nrecv=0)
    want = oracle.surface_matrices(p)
    with solver.Solver(p) as s:
        mVx, mVy, _ = s.fetch_surface_matrices()
        got = {"matVx2Vz2": mVx, "matVy2Vz2": mVy}
        if kind == "visco":
            got["matD"] = s.fetch_surface_rotation()
    for k, v in got.items():
        w = want[k].reshape(p.ny, p.nx, 9)[p.nj1:p.nj2 + 1, p.ni1:p.ni2 + 1]
        g = v.reshape(p.ny, p.nx, 9)[p.nj1:p.nj2 + 1, p.ni1:p.ni2 + 1]
        assert_parity(g, w, "%s %s" % (kind, k))


def test_visco_attenuation_changes_result():
    """The memory variables act: zero relaxation rates give another state."""
    from cgfd3d_gb300 import models, solver
    p = models.topo_media_model("visco", ni=48, nj=40, nk=30, steps=5, dt=0.005,
                                nrecv=0)
    _noise(p, 9)
    q = p.copy()
    q.wl = np.zeros_like(q.wl)
    solver.drv_rk_curv_col_allstep(p)
    solver.drv_rk_curv_col_allstep(q)
    lev = p.final_level()
    a, b = p.level(lev), q.level(lev)
    assert np.abs(a - b).max() > 1e-4 * np.abs(a).max()
