"""Python mirror of the reference's time-loop entry point.

``drv_rk_curv_col_allstep(problem)`` does what CGFD3D's
``drv_rk_curv_col_allstep`` (forward/drv_rk_curv_col.c:27-556) does to the
arrays of a :class:`cgfd3d_gb300.problem.Problem`: it runs ``nt_total`` RK4
steps, leaves the final wavefield and PML state in level 0 (even nt_total)
or level 3 (odd), and fills the receiver and line seismograms.  All compute
runs in the CUDA library through the flat C ABI (include/cgfd3d_gpu.h).

:class:`Solver` keeps the state resident in HBM between calls for callers
that step, inspect and continue.
"""

import ctypes as C

from . import _lib


class Solver:
    def __init__(self, problem):
        self.problem = problem
        self._c = problem.to_c()
        self._h = C.c_void_p()
        _lib.check(_lib.lib().cgfd_solver_create(C.addressof(self._c),
                                                  C.byref(self._h)))

    @property
    def step(self):
        return _lib.lib().cgfd_solver_step(self._h)

    def run(self, nsteps):
        _lib.check(_lib.lib().cgfd_solver_run(self._h, int(nsteps)))

    def fetch(self):
        _lib.check(_lib.lib().cgfd_solver_fetch(self._h))

    def check_finite(self):
        _lib.check(_lib.lib().cgfd_solver_check_finite(self._h))

    def kernel_times(self):
        t = (C.c_float * 3)()
        n = (C.c_int * 3)()
        _lib.check(_lib.lib().cgfd_solver_kernel_times(self._h, t, n))
        return list(t), list(n)

    def fetch_pg(self):
        """Surface peak-motion maps (15 x ny x nx)."""
        import numpy as np
        p = self.problem
        out = np.zeros(15 * p.nx * p.ny, np.float32)
        _lib.check(_lib.lib().cgfd_solver_fetch_pg(self._h, out.ctypes.data))
        return out.reshape(15, p.ny, p.nx)

    def fetch_surface_matrices(self):
        import numpy as np
        p = self.problem
        mats = [np.zeros(p.nx * p.ny * 9, np.float32) for _ in range(3)]
        _lib.check(_lib.lib().cgfd_solver_fetch_surface_matrices(
            self._h, *[m.ctypes.data for m in mats]))
        return mats

    def fetch_surface_rotation(self):
        """Visco-elastic surface rotation matrices (nx*ny*9)."""
        import numpy as np
        p = self.problem
        out = np.zeros(p.nx * p.ny * 9, np.float32)
        _lib.check(_lib.lib().cgfd_solver_fetch_surface_rotation(
            self._h, out.ctypes.data))
        return out

    def set_timing(self, on=True):
        _lib.check(_lib.lib().cgfd_solver_set_timing(self._h, int(bool(on))))

    def transfer_bytes(self):
        h, d = C.c_size_t(), C.c_size_t()
        _lib.check(_lib.lib().cgfd_solver_transfer_bytes(self._h, C.byref(h), C.byref(d)))
        return h.value, d.value

    def close(self):
        if self._h:
            _lib.lib().cgfd_solver_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def drv_rk_curv_col_allstep(problem):
    """Run the whole time loop of `problem` on the GPU (one shot)."""
    c = problem.to_c()
    _lib.check(_lib.lib().cgfd_allstep(C.addressof(c)))
    return problem


def drv_rk_curv_col_allstep_structs(structs, dt, nt_total, t0=0.0,
                                    qc_check_nan_num_of_step=0, verbose=0):
    """Call the drop-in entry point with reference structs (refabi)."""
    order = ["fd", "gd", "metric", "md", "src", "bdry", "wav", "mympi",
             "iorecv", "ioline", "ioslice", "iosnap"]
    args = [C.addressof(structs[n]) for n in order]
    _lib.dropin().drv_rk_curv_col_allstep(*args, float(dt), int(nt_total), float(t0),
                                          b"", b"", int(qc_check_nan_num_of_step),
                                          0, int(verbose))


def device_bytes(problem):
    c = problem.to_c()
    return _lib.lib().cgfd_device_bytes(C.addressof(c))


class Batch:
    """Independent shots stepped together (cgfd_batch_* of the C ABI): one
    stage launch per RK stage over every shot's tiles, one CUDA graph per
    8-step operator cycle.  Results per shot equal a single-shot run."""

    def __init__(self, problems, kchunk=0):
        self.problems = list(problems)
        self._c = [p.to_c() for p in self.problems]
        arr = (C.c_void_p * len(self._c))(*[C.addressof(c) for c in self._c])
        self._arr = arr
        self._h = C.c_void_p()
        _lib.check(_lib.lib().cgfd_batch_create(arr, len(self._c), int(kchunk),
                                                 C.byref(self._h)))

    def run(self, nsteps):
        _lib.check(_lib.lib().cgfd_batch_run(self._h, int(nsteps)))

    def times(self):
        ms, n = C.c_float(), C.c_int()
        _lib.check(_lib.lib().cgfd_batch_times(self._h, C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def fetch(self):
        _lib.check(_lib.lib().cgfd_batch_fetch(self._h))

    def reset(self):
        _lib.check(_lib.lib().cgfd_batch_reset(self._h))

    def set_kchunk(self, kchunk):
        _lib.check(_lib.lib().cgfd_batch_set_kchunk(self._h, int(kchunk)))

    def autotune(self, candidates=(8, 12, 16, 24, 32), steps=2, cache=None, key=None):
        """Pick k planes per CTA by timing `steps` steps per candidate; with
        `cache` (a JSON file path) and `key`, reuse or record the choice."""
        import json
        import os
        if cache and key and os.path.exists(cache):
            try:
                with open(cache) as f:
                    got = json.load(f).get(key)
                if got:
                    self.set_kchunk(got["kchunk"])
                    return got
            except (OSError, ValueError):
                pass
        cand = (C.c_int * len(candidates))(*candidates)
        ms = (C.c_float * len(candidates))()
        best = C.c_int()
        _lib.check(_lib.lib().cgfd_batch_autotune(self._h, cand, len(candidates),
                                                   int(steps), ms, C.byref(best)))
        res = {"kchunk": best.value, "candidates": list(candidates),
               "ms": [float(v) for v in ms], "steps": int(steps)}
        if cache and key:
            data = {}
            try:
                with open(cache) as f:
                    data = json.load(f)
            except (OSError, ValueError):
                pass
            data[key] = res
            os.makedirs(os.path.dirname(os.path.abspath(cache)), exist_ok=True)
            with open(cache, "w") as f:
                json.dump(data, f, indent=1)
        return res

    def shot_pg(self, k):
        """Peak-motion maps of shot k (15 x ny x nx)."""
        import numpy as np
        p = self.problems[k]
        h = _lib.lib().cgfd_batch_shot(self._h, int(k))
        out = np.zeros(15 * p.nx * p.ny, np.float32)
        _lib.check(_lib.lib().cgfd_solver_fetch_pg(h, out.ctypes.data))
        return out.reshape(15, p.ny, p.nx)

    def close(self):
        if self._h:
            _lib.lib().cgfd_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def metric_calc(dims, x3d, y3d, z3d):
    """Grid metrics on the GPU from node coordinates (cgfd_metric_calc):
    dims = (ni, nj, nk, nx, ny, nz, ni1, ni2, nj1, nj2, nk1, nk2); returns a
    dict jac, xi_x, ..., zeta_z of flat float32 arrays (reference layout)."""
    import numpy as np
    from . import abi
    ni, nj, nk, nx, ny, nz, ni1, ni2, nj1, nj2, nk1, nk2 = [int(v) for v in dims]
    x, y, z = [np.ascontiguousarray(a, np.float32).ravel() for a in (x3d, y3d, z3d)]
    out = np.zeros(10 * nx * ny * nz, np.float32)
    _lib.check(_lib.lib().cgfd_metric_calc(nx, ny, nz, ni1, ni2, nj1, nj2, nk1, nk2,
                                            x.ctypes.data, y.ctypes.data,
                                            z.ctypes.data, out.ctypes.data))
    v = nx * ny * nz
    return {n: out[c * v:(c + 1) * v] for c, n in enumerate(abi.METRIC_NAMES)}
