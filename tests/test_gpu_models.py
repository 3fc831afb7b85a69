"""GPU against the oracle on the benchmark model generators.

The oracle is pinned bit-for-bit to the reference (test_oracle_golden.py);
here both run the same synthetic model: the flat configuration at its full
100 x 100 x 60 size and a reduced topography model, from a zero state and
from a seeded noise state (every operator tap, every boundary branch).
Both stage-kernel forms (TMA z-marching, direct loads) are checked.
"""

import os

import numpy as np
import pytest

import oracle
from helpers import assert_parity

pytestmark = pytest.mark.gpu


def _noise(p, seed, amp_v=1e-2):
    rng = np.random.default_rng(seed)
    V = p.vol
    lev0 = p.level(0).reshape(p.ncmp, p.nz, p.ny, p.nx)
    core = (slice(p.nk1, p.nk2 + 1), slice(p.nj1, p.nj2 + 1), slice(p.ni1, p.ni2 + 1))
    for c in range(p.ncmp):
        amp = amp_v if c < 3 else amp_v * 2700 * 6000
        lev0[c][core] = (amp * rng.uniform(-1, 1, lev0[c][core].shape)).astype(np.float32)
    for row in p.pml:
        for f in row:
            if f is not None:
                n = f["aux"].size // 4
                f["aux"][:n] = (amp_v * 0.1 * rng.uniform(-1, 1, n)).astype(np.float32)
    assert V > 0


def _compare(p_gpu, p_cpu, what):
    lev = p_gpu.final_level()
    assert_parity(p_gpu.level(lev), p_cpu.level(lev), what + " wavefield")
    for d in range(3):
        for s in range(2):
            if p_gpu.pml[d][s] is not None:
                assert_parity(p_gpu.pml_final(d, s), p_cpu.pml_final(d, s),
                              "%s pml %d %d" % (what, d, s))
    if p_gpu.recv is not None:
        assert_parity(p_gpu.recv["seismo"], p_cpu.recv["seismo"], what + " receivers")


@pytest.fixture(params=["2", "1"], ids=["tma", "direct"])
def kernel(request, monkeypatch):
    monkeypatch.setenv("CGFD_STAGE_KERNEL", request.param)
    return request.param


def test_flat_model_full_size(kernel):
    from cgfd3d_gb300 import models, solver
    p = models.flat_model(steps=8)
    q = p.copy()
    solver.drv_rk_curv_col_allstep(p)
    oracle.allstep(q, oracle.TIMG_ZERO, os.cpu_count() or 4)
    _compare(p, q, "flat")


@pytest.mark.parametrize("shape", [(96, 80, 48), (70, 45, 37)])
def test_topo_model_noise_state(kernel, shape):
    from cgfd3d_gb300 import models, solver
    ni, nj, nk = shape
    p = models.topo_model(ni=ni, nj=nj, nk=nk, steps=9, dt=0.005, nrecv=16)
    _noise(p, 7)
    q = p.copy()
    solver.drv_rk_curv_col_allstep(p)
    oracle.allstep(q, oracle.TIMG_ZERO, os.cpu_count() or 4)
    _compare(p, q, "topo %s" % (shape,))


def test_kernel_forms_agree():
    """TMA and direct-load stage kernels compute the same thing."""
    from cgfd3d_gb300 import models, solver
    p = models.topo_model(ni=64, nj=40, nk=30, steps=9, dt=0.005, nrecv=9)
    _noise(p, 11)
    q = p.copy()
    os.environ["CGFD_STAGE_KERNEL"] = "2"
    solver.drv_rk_curv_col_allstep(p)
    os.environ["CGFD_STAGE_KERNEL"] = "1"
    try:
        solver.drv_rk_curv_col_allstep(q)
    finally:
        del os.environ["CGFD_STAGE_KERNEL"]
    lev = p.final_level()
    assert_parity(p.level(lev), q.level(lev), "tma vs direct")
