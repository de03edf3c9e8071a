"""Serving form: continuous batching of liquid-simulation requests (pxf_server_* in libpxlflip).

Requests queue on submit(); each tick retires finished requests, admits queued ones while their
device footprint fits the HBM budget, and advances all active requests by one batched substep.
"""
import ctypes as C
from typing import Optional

import numpy as np

from . import _lib as L
from .fluid import Fluid, FluidError


class Server:
    def __init__(self, hbm_budget_bytes: int = 150_000_000_000, max_active: int = 256, substeps_per_tick: int = 1,
                 wait_timeout_s: float = 600.0):
        self._lib = L.load()
        cfg = L.ServerConfig()
        self._lib.pxf_server_config_init(C.byref(cfg))
        cfg.hbm_budget_bytes = int(hbm_budget_bytes)
        cfg.max_active = int(max_active)
        cfg.substeps_per_tick = int(substeps_per_tick)
        cfg.wait_timeout_s = float(wait_timeout_s)
        out = C.c_void_p()
        rc = self._lib.pxf_server_create(C.byref(cfg), C.byref(out))
        if rc != 0:
            raise FluidError(rc, self._lib.pxf_last_error(None).decode())
        self.h = out

    def _chk(self, rc):
        if rc != 0:
            msg = self._lib.pxf_server_last_error(self.h)
            raise FluidError(rc, msg.decode() if msg else f"error {rc}")

    def submit(self, fluid: Fluid, substeps: int, fps: float = 24.0, seed: int = 0,
               options: Optional[L.Options] = None) -> int:
        d = fluid.to_desc()
        rid = C.c_uint64()
        rc = self._lib.pxf_server_submit(self.h, C.byref(d), seed, float(fps),
                                         C.byref(options) if options else None, int(substeps), C.byref(rid))
        if rc == L.PXF_ENOMEM:
            return rid.value    # rejected: status reports PXF_REQ_FAILED / PXF_ENOMEM
        self._chk(rc)
        return rid.value

    def cancel(self, rid: int) -> None:
        self._chk(self._lib.pxf_server_cancel(self.h, rid))

    def tick(self) -> int:
        a = C.c_uint32()
        self._chk(self._lib.pxf_server_tick(self.h, C.byref(a)))
        return a.value

    def status(self, rid: int) -> L.RequestStatus:
        st = L.RequestStatus()
        self._chk(self._lib.pxf_server_status(self.h, rid, C.byref(st)))
        return st

    def take_result(self, rid: int) -> np.ndarray:
        st = self.status(rid)
        out = np.empty((st.particles, 8), dtype=np.float32)
        self._chk(self._lib.pxf_server_take_result(self.h, rid, out.ctypes.data, st.particles))
        return out

    def stats(self) -> dict:
        s = L.ServerStats()
        self._chk(self._lib.pxf_server_stats_get(self.h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in L.ServerStats._fields_}

    def start(self) -> None:
        self._chk(self._lib.pxf_server_start(self.h))

    def stop(self) -> None:
        self._chk(self._lib.pxf_server_stop(self.h))

    def close(self):
        if self.h is not None:
            self._lib.pxf_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
