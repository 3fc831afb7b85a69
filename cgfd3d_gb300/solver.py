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

from . import _lib, abi


def _box_array(boxes):
    """ctypes array of cgfd_box_t from Box structs, dicts or 11-tuples
    (c1, c2, i1, ni, di, j1, nj, dj, k1, nk, dk)."""
    out = (abi.Box * len(boxes))()
    for m, b in enumerate(boxes):
        if isinstance(b, abi.Box):
            out[m] = b
        elif isinstance(b, dict):
            out[m] = abi.Box(**b)
        else:
            out[m] = abi.Box(*[int(v) for v in b])
    return out


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

    def run_async(self, nsteps):
        """Queue nsteps steps and return; errors surface at the next
        collect or blocking call."""
        _lib.check(_lib.lib().cgfd_solver_run_async(self._h, int(nsteps)))

    def fetch(self):
        _lib.check(_lib.lib().cgfd_solver_fetch(self._h))

    def set_wait_test(self, wait_limit, skip_plane=-1):
        """Polls before a stage-kernel wait gives up (0: default) and, for
        tests, a wavefield plane whose copy the first CTA leaves out."""
        _lib.check(_lib.lib().cgfd_solver_set_wait_test(self._h, int(wait_limit),
                                                        int(skip_plane)))

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

    def fetch_state(self, out=None):
        """The current state as (ncmp, nz, ny, nx), reference layout (into
        ``out`` when given: C-contiguous float32 of that shape)."""
        import numpy as np
        p = self.problem
        shape = (p.ncmp, p.nz, p.ny, p.nx)
        if out is None:
            out = np.empty(shape, np.float32)
        elif out.shape != shape or out.dtype != np.float32 or not out.flags.c_contiguous:
            raise ValueError("out must be C-contiguous float32 %r" % (shape,))
        _lib.check(_lib.lib().cgfd_solver_fetch_state(self._h, out.ctypes.data))
        return out

    def pack_boxes(self, boxes):
        """Output boxes of the current state, packed on the device: one array
        (ncomp, nk, nj, ni) per box, the order of the reference's slice and
        snapshot writers."""
        import numpy as np
        arr = _box_array(boxes)
        n = _lib.lib().cgfd_box_floats(arr, len(arr))
        if n == 0:
            raise ValueError("empty or malformed output box")
        flat = np.empty(n, np.float32)
        _lib.check(_lib.lib().cgfd_solver_pack_boxes(self._h, arr, len(arr),
                                                      flat.ctypes.data))
        out, q = [], 0
        for b in arr:
            shape = (b.c2 - b.c1 + 1, b.nk, b.nj, b.ni)
            cnt = shape[0] * shape[1] * shape[2] * shape[3]
            out.append(flat[q:q + cnt].reshape(shape))
            q += cnt
        return out

    def pack_boxes_async(self, boxes, slot):
        """Queue the packing of boxes of the state after the queued steps into
        output slot 0 or 1; collect_boxes(slot) hands them out."""
        arr = _box_array(boxes)
        if _lib.lib().cgfd_box_floats(arr, len(arr)) == 0:
            raise ValueError("empty or malformed output box")
        self._slot_boxes = getattr(self, "_slot_boxes", {})
        self._slot_boxes[slot] = arr
        _lib.check(_lib.lib().cgfd_solver_pack_boxes_async(self._h, arr, len(arr),
                                                            int(slot)))

    def collect_boxes(self, slot, w=None):
        """Wait for output slot `slot`.  With w: scatter the boxes into it (as
        fetch_boxes) and return None; without: return them as arrays (as
        pack_boxes)."""
        import numpy as np
        arr = self._slot_boxes.get(slot) if hasattr(self, "_slot_boxes") else None
        if arr is None:
            raise ValueError("output slot %r holds no boxes" % (slot,))
        flat = None
        if w is None:
            flat = np.empty(_lib.lib().cgfd_box_floats(arr, len(arr)), np.float32)
        wp = None
        if w is not None:
            p = self.problem
            if (w.dtype != np.float32 or not w.flags.c_contiguous or
                    w.size != p.ncmp * p.nx * p.ny * p.nz):
                raise ValueError("w must be a C-contiguous float32 array of the state's size")
            wp = w.ctypes.data
        del self._slot_boxes[slot]
        _lib.check(_lib.lib().cgfd_solver_collect_boxes(
            self._h, int(slot), wp, None if flat is None else flat.ctypes.data))
        if flat is None:
            return None
        out, q = [], 0
        for b in arr:
            shape = (b.c2 - b.c1 + 1, b.nk, b.nj, b.ni)
            cnt = shape[0] * shape[1] * shape[2] * shape[3]
            out.append(flat[q:q + cnt].reshape(shape))
            q += cnt
        return out

    def fetch_boxes(self, boxes, w):
        """Write the boxes of the current state into w (ncmp x nz x ny x nx,
        float32, C order) at their own positions; other points untouched."""
        import numpy as np
        p = self.problem
        if (not isinstance(w, np.ndarray) or w.dtype != np.float32 or
                not w.flags.c_contiguous or w.size != p.ncmp * p.nx * p.ny * p.nz):
            raise ValueError("w must be a C-contiguous float32 array of the state's size")
        arr = _box_array(boxes)
        _lib.check(_lib.lib().cgfd_solver_fetch_boxes(self._h, arr, len(arr),
                                                       w.ctypes.data))
        return w

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

    def fetch_seismograms(self):
        """Receiver and line seismograms of every shot (no wavefield)."""
        _lib.check(_lib.lib().cgfd_batch_fetch_seismograms(self._h))

    def reset(self):
        _lib.check(_lib.lib().cgfd_batch_reset(self._h))

    def set_kchunk(self, kchunk):
        _lib.check(_lib.lib().cgfd_batch_set_kchunk(self._h, int(kchunk)))

    def set_schedule(self, persistent):
        """0: one CTA per (shot, tile, k chunk) item; 1: persistent CTAs."""
        _lib.check(_lib.lib().cgfd_batch_set_schedule(self._h, int(bool(persistent))))

    def schedule(self):
        return int(_lib.lib().cgfd_batch_schedule(self._h))

    def autotune(self, candidates=(8, 12, 16, 24, 32), steps=2, cache=None, key=None,
                 schedules=True):
        """Pick k planes per CTA (and, with `schedules`, the launch schedule)
        by timing `steps` steps per candidate; with `cache` (a JSON file
        path) and `key`, reuse or record the choice."""
        import json
        import os
        if cache and key and os.path.exists(cache):
            try:
                with open(cache) as f:
                    got = json.load(f).get(key)
                if got:
                    self.set_kchunk(got["kchunk"])
                    self.set_schedule(got.get("persistent", 0))
                    return got
            except (OSError, ValueError):
                pass
        cand = (C.c_int * len(candidates))(*candidates)
        best = C.c_int()
        if schedules:
            ms = (C.c_float * (2 * len(candidates)))()
            pbest = C.c_int()
            _lib.check(_lib.lib().cgfd_batch_autotune_schedule(
                self._h, cand, len(candidates), int(steps), ms, C.byref(best), C.byref(pbest)))
            n = len(candidates)
            res = {"kchunk": best.value, "persistent": pbest.value,
                   "candidates": list(candidates), "ms": [float(v) for v in ms[:n]],
                   "ms_persistent": [float(v) for v in ms[n:]], "steps": int(steps)}
        else:
            ms = (C.c_float * len(candidates))()
            _lib.check(_lib.lib().cgfd_batch_autotune(self._h, cand, len(candidates),
                                                       int(steps), ms, C.byref(best)))
            res = {"kchunk": best.value, "persistent": self.schedule(),
                   "candidates": list(candidates), "ms": [float(v) for v in ms],
                   "steps": int(steps)}
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
