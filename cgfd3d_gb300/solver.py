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
