"""Host-side mirror of WARP3D's two element-block entry points on top of
the C-ABI (include/w3g.h).

``Engine.tanstf``  <- tanstf (src/tanstf.f:17)
``Engine.recover`` <- drive_eps_sig_internal_forces
                      (src/drive_eps_sig_internal_forces.f:20)
``Engine.update``  <- update (src/update.f:73-94)

Same argument meaning as the Fortran: ``step``/``iter`` are the load step
and Newton iteration, ``c``, ``u``, ``du`` the global coordinate,
displacement and displacement-increment vectors, ``ifv`` the internal
force vector (overwritten). A step-cut request comes back as the status
``abi.STEP_CUT`` (WARP3D's material_cut_step); fatal errors raise
:class:`abi.W3GError`. There is no CPU fallback: without the CUDA library
or a device, construction raises.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from .model import HostState, Model, block_ptrs, dptr


def _read_cache(path: str) -> dict:
    import json
    import os
    if not os.path.exists(path):
        return {}
    with open(path) as f:
        return json.load(f)


def _write_cache(path: str, data: dict):
    import json
    import os
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


class Engine:
    def __init__(self, model: Model, device: int = 0, precision: int = abi.TANGENT_FP64):
        self.lib = abi.load()
        self.model = model
        self.desc = model.desc()
        self.ctx = C.c_void_p()
        self.device = device
        self.precision = abi.TANGENT_FP64
        abi.check(self.lib, self.lib.w3g_create(device, C.byref(self.desc), C.byref(self.ctx)))
        if precision != abi.TANGENT_FP64:
            self.set_precision(precision)

    # ---- lifecycle --------------------------------------------------------
    def close(self):
        if self.ctx:
            self.lib.w3g_destroy(self.ctx)
            self.ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_wait_limit(self, polls: int):
        """Bound on the polls of every wait in the tensor-core kernels
        (w3g_set_wait_limit; negative: the default). 0 makes them give up
        before any MMA: w3g_tanstf then reports W3G_EFATAL with NaN Ke."""
        abi.check(self.lib, self.lib.w3g_set_wait_limit(self.ctx, polls))

    def set_update_mode(self, mode: int):
        """abi.UPDATE_COPY (WARP3D's copies n+1 -> n) or abi.UPDATE_SWAP
        (the n and n+1 arrays exchanged; mm10 history copied back), see
        w3g_set_update_mode."""
        abi.check(self.lib, self.lib.w3g_set_update_mode(self.ctx, mode))

    def set_precision(self, precision: int):
        abi.check(self.lib, self.lib.w3g_set_tangent_precision(self.ctx, precision))
        self.precision = precision

    # ---- timing and output checks -----------------------------------------
    def timers(self) -> dict:
        """Host wall time and call counts per entry point (WARP3D's timing
        categories: tangent stiffness, sig-eps & internal force, update)."""
        t = abi.Timers()
        abi.check(self.lib, self.lib.w3g_timers_get(self.ctx, C.byref(t)))
        return {f: getattr(t, f) for f, _ in t._fields_}

    def reset_timers(self):
        abi.check(self.lib, self.lib.w3g_timers_reset(self.ctx))

    def check_finite(self) -> int:
        """Number of NaN/Inf values in the resident outputs."""
        n = C.c_longlong()
        abi.check(self.lib, self.lib.w3g_check_finite(self.ctx, C.byref(n)))
        return n.value

    # ---- state transfer ----------------------------------------------------
    def upload(self, state: HostState, names=None):
        s = state.struct(names)
        abi.check(self.lib, self.lib.w3g_state_upload(self.ctx, C.byref(s)))

    def download(self, state: HostState, names=None):
        s = state.struct(names)
        abi.check(self.lib, self.lib.w3g_state_download(self.ctx, C.byref(s)))

    # ---- restart records (store_blocks / reopen) ---------------------------
    def store_blocks(self, path: str, append: bool = False):
        """Writes the element-block section of a WARP3D restart file
        (w3g_store_blocks: store_blocks' records, src/store.f:915)."""
        abi.check(self.lib, self.lib.w3g_store_blocks(self.ctx, path.encode(), 1 if append else 0))

    def reopen_blocks(self, path: str, offset: int = 0) -> int:
        """Reads that section from byte `offset` (w3g_reopen_blocks); returns
        the offset after it."""
        end = C.c_longlong()
        abi.check(self.lib, self.lib.w3g_reopen_blocks(self.ctx, path.encode(), offset, C.byref(end)))
        return end.value

    # ---- hot path, host arrays --------------------------------------------
    def tanstf(self, step: int, it: int, c: np.ndarray, u: np.ndarray, du: np.ndarray, estiff_blocks=None):
        """estiff_blocks: a list of per-block (span, utsz) arrays, or one
        C-contiguous float64 array holding all blocks back to back (its
        per-block pointers are then computed without a Python loop)."""
        ptrs = None
        if isinstance(estiff_blocks, np.ndarray):
            ptrs = C.cast(self._contiguous_ptrs(estiff_blocks), C.POINTER(C.POINTER(C.c_double)))
        elif estiff_blocks is not None:
            ptrs = C.cast(block_ptrs(estiff_blocks), C.POINTER(C.POINTER(C.c_double)))
        return abi.check(self.lib, self.lib.w3g_tanstf(self.ctx, step, it, dptr(c), dptr(u), dptr(du), ptrs))

    def _contiguous_ptrs(self, buf: np.ndarray):
        m = self.model
        if not hasattr(self, "_estiff_off"):
            sizes = np.array(m.spans, dtype=np.uintp) * np.array(m.block_ek_rows, dtype=np.uintp)
            self._estiff_off = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.uintp) * np.uintp(8)
            self._estiff_total = int(sizes.sum())
        if buf.dtype != np.float64 or not buf.flags.c_contiguous or buf.size != self._estiff_total:
            raise ValueError("estiff buffer must be C-contiguous float64 with all blocks' values")
        addr = self._estiff_off + np.uintp(buf.ctypes.data)
        return (C.c_void_p * m.nelblk).from_buffer(addr)

    def recover(self, step: int, it: int, extrapolated: bool, c, u, du, ifv):
        info = abi.RecoverInfo()
        st = self.lib.w3g_recover(self.ctx, step, it, 1 if extrapolated else 0, dptr(c), dptr(u), dptr(du),
                                  dptr(ifv) if ifv is not None else None, C.byref(info))
        abi.check(self.lib, st, allow=(abi.OK, abi.STEP_CUT, abi.LOCAL_FAIL))
        return st, info

    def update(self):
        return abi.check(self.lib, self.lib.w3g_update(self.ctx))

    # ---- batching form ------------------------------------------------------
    def set_schedule(self, mode=abi.SCHED_PERSISTENT, recover_ctas_per_sm=0, tangent_ctas_per_sm=0,
                     recover_grain=1, tangent_grain=1, order=abi.ORDER_HEAVY_FIRST):
        sc = abi.Schedule(mode, recover_ctas_per_sm, tangent_ctas_per_sm, recover_grain, tangent_grain, order)
        abi.check(self.lib, self.lib.w3g_set_schedule(self.ctx, C.byref(sc)))

    def local_iterations(self) -> np.ndarray:
        """Local Newton iterations of the last recovery per mm10 Gauss point."""
        n = int(sum(s * g for s, g, cr in zip(self.model.spans, self.model.block_ngp, self.model.block_crystal) if cr))
        out = np.zeros(n, dtype=np.int32)
        abi.check(self.lib, self.lib.w3g_local_iterations(self.ctx, out.ctypes.data_as(C.POINTER(C.c_int)), n))
        return out

    def schedule(self) -> dict:
        sc = abi.Schedule()
        abi.check(self.lib, self.lib.w3g_get_schedule(self.ctx, C.byref(sc)))
        return sc.as_dict()

    def iteration_dev(self, step, it, extrapolated, what, d_c: int, d_u: int, d_du: int, d_ifv: int,
                      stream: int = 0):
        """One Newton iteration's element work (recovery and/or tangent),
        replayed as a CUDA graph."""
        return abi.check(self.lib, self.lib.w3g_iteration_dev(self.ctx, step, it, 1 if extrapolated else 0, what,
                                                              d_c, d_u, d_du, d_ifv or None, stream or None))

    def autotune(self, step, it, extrapolated, d_c: int, d_u: int, d_du: int, d_ifv: int, stream: int = 0,
                 reps: int = 3, cache: str | None = None):
        """Times the candidate schedules on this model and keeps the fastest
        (w3g_autotune). With ``cache`` (a JSON file), the choice is stored
        under a key of the device, the tangent precision and, per element
        type and material model, the element and Gauss-point counts, and
        reused without timing when the key is already there."""
        key = self.tuning_key() if cache else None
        if cache:
            entry = _read_cache(cache).get(key)
            if entry is not None:
                self.set_schedule(**entry["schedule"])
                return dict(entry["schedule"]), float(entry["ms"])
        sc = abi.Schedule()
        ms = C.c_double()
        abi.check(self.lib, self.lib.w3g_autotune(self.ctx, step, it, 1 if extrapolated else 0, d_c, d_u, d_du,
                                                  d_ifv, stream or None, reps, C.byref(sc), C.byref(ms)))
        if cache:
            data = _read_cache(cache)
            data[key] = {"schedule": sc.as_dict(), "ms": ms.value}
            _write_cache(cache, data)
        return sc.as_dict(), ms.value

    def tuning_key(self) -> str:
        """Autotuning cache key: device name, precision, and per (element
        type, Gauss points, material model) the elements and blocks."""
        m = self.model
        buf = C.create_string_buffer(256)
        abi.check(self.lib, self.lib.w3g_device_name(self.device, buf, 256))
        groups = {}
        for b in range(m.nelblk):
            k = (m.block_etype[b], m.block_ngp[b], "mm10" if m.block_crystal[b] else "mm01")
            e, n = groups.get(k, (0, 0))
            groups[k] = (e + m.spans[b], n + 1)
        parts = [f"{t}/{g}/{mat}:{e}e{n}b" for (t, g, mat), (e, n) in sorted(groups.items())]
        return f"{buf.value.decode()}|p{self.precision}|" + ",".join(parts)

    # ---- hot path, device pointers (ints) ----------------------------------
    def tanstf_dev(self, step, it, d_c: int, d_u: int, d_du: int, stream: int = 0):
        return abi.check(self.lib, self.lib.w3g_tanstf_dev(self.ctx, step, it, d_c, d_u, d_du, stream or None))

    def recover_dev(self, step, it, extrapolated, d_c: int, d_u: int, d_du: int, d_ifv: int, stream: int = 0):
        return abi.check(self.lib, self.lib.w3g_recover_dev(self.ctx, step, it, 1 if extrapolated else 0, d_c, d_u,
                                                            d_du, d_ifv, stream or None))

    def recover_info(self):
        info = abi.RecoverInfo()
        st = self.lib.w3g_recover_info_get(self.ctx, C.byref(info))
        abi.check(self.lib, st, allow=(abi.OK, abi.STEP_CUT, abi.LOCAL_FAIL))
        return st, info

    def estiff_device(self):
        p = C.c_void_p()
        n = C.c_longlong()
        abi.check(self.lib, self.lib.w3g_estiff_device(self.ctx, C.byref(p), C.byref(n)))
        return p.value, n.value

    def last_launch_count(self) -> int:
        return self.lib.w3g_last_launch_count(self.ctx)
