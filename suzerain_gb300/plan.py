"""Resident batched substep driver (Python face of sgb_plan_*).

A Plan holds one case's bands and coefficients, the wavenumber pairs of every
system, and the device workspace; each substep() runs the explicit operator,
the implicit band solve (complex128 LU, or complex64 LU with FP64
refinement) and the permutations back to natural order, for all systems, in
the stream it is given.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as nat
from .synth import SynthCase


def _ptr(x) -> int:
    """Device/host address of a torch tensor, numpy array or int."""
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        return x.data_ptr()
    return x.ctypes.data


class RefineSpec:
    """zcgbsvx refinement controls (aiter, siter, diter, tolsc)."""

    def __init__(self, aiter=5, siter=25, diter=5, tolsc=1.0):
        self.aiter, self.siter, self.diter, self.tolsc = aiter, siter, diter, tolsc

    def ctypes(self) -> nat.RefineSpec:
        return nat.RefineSpec(self.aiter, self.siter, self.diter, self.tolsc)

    @classmethod
    def from_string(cls, text: str) -> "RefineSpec":
        """From a reference solver specification string (its zcgbsvx fields;
        see SolverSpec)."""
        s = SolverSpec(text)
        return cls(s.aiter, s.siter, s.diter, s.tolsc)


class _SpecStruct(C.Structure):
    _fields_ = [("method", C.c_int), ("equil", C.c_int), ("reuse", C.c_int),
                ("aiter", C.c_int), ("siter", C.c_int), ("diter", C.c_int),
                ("tolsc", C.c_double)]


class SolverSpec:
    """suzerain::specification_zgbsv: parse a specification string with the
    reference's grammar and defaults; str() gives its canonical form."""
    METHODS = {1: "zgbsv", 2: "zgbsvx", 3: "zcgbsvx"}

    def __init__(self, text: str = ""):
        L = nat.load()
        self._s = _SpecStruct()
        err = C.create_string_buffer(512)
        if L.sgb_solver_spec_parse(text.encode(), C.byref(self._s), err, len(err)) != 0:
            raise ValueError(err.value.decode())

    def __getattr__(self, name):
        if name in ("equil", "reuse"):
            return bool(getattr(self._s, name))
        if name in ("aiter", "siter", "diter", "tolsc"):
            return getattr(self._s, name)
        if name == "method":
            return self.METHODS.get(self._s.method, "UNKNOWN")
        raise AttributeError(name)

    def __str__(self) -> str:
        buf = C.create_string_buffer(256)
        nat.check(nat.load().sgb_solver_spec_format(C.byref(self._s), buf, len(buf)),
                  "sgb_solver_spec_format")
        return buf.value.decode()

    def __eq__(self, other) -> bool:
        return isinstance(other, SolverSpec) and bytes(self._s) == bytes(other._s)

    def in_place(self) -> bool:
        """zgbsv factors in place (packf storage); the others do not."""
        return self.method == "zgbsv"


class Plan:
    def __init__(self, case: SynthCase, kx: np.ndarray, kz: np.ndarray,
                 max_double_slots: int = 0):
        self.L = nat.load()
        self.case = case
        self.nsys = int(len(kx))
        self.N = case.N
        self.KL, self.KU = case.KL, case.KU
        self._kx = np.ascontiguousarray(kx, dtype=np.float64)
        self._kz = np.ascontiguousarray(kz, dtype=np.float64)
        self._cs = case.ctypes_case()
        h = self.L.sgb_plan_create(C.byref(self._cs), self.nsys,
                                   self._kx.ctypes.data, self._kz.ctypes.data,
                                   int(max_double_slots))
        if not h:
            raise RuntimeError(f"sgb_plan_create failed: {nat.last_error()}")
        self.handle = h

    def close(self):
        if getattr(self, "handle", None):
            self.L.sgb_plan_destroy(self.handle)
            self.handle = None

    __del__ = close

    def device_bytes(self) -> int:
        return int(self.L.sgb_plan_device_bytes(self.handle))

    @staticmethod
    def estimate_bytes(case: SynthCase, nsys: int, max_double_slots: int = 0,
                       method: str = "M") -> int:
        """Device bytes a plan of this case holds after its first substep of
        `method` (without creating it)."""
        L = nat.load()
        cs = case.ctypes_case()
        return int(L.sgb_plan_estimate_bytes(C.byref(cs), int(nsys), int(max_double_slots),
                                             method.encode()))

    def substep(self, method: str, phi_exp: float, phi_imp: float, u_in, u_out,
                spec: RefineSpec | None = None, stream=0) -> None:
        sp = (spec or RefineSpec()).ctypes()
        rc = self.L.sgb_plan_substep(self.handle, method.encode(), phi_exp,
                                     phi_imp, _ptr(u_in), _ptr(u_out),
                                     C.byref(sp), _ptr(stream))
        nat.check(rc, "sgb_plan_substep")

    def substep_capturable(self, method: str, phi_exp: float, phi_imp: float, u_in, u_out,
                           spec: RefineSpec | None = None, stream=0) -> None:
        """substep without host synchronization or allocation, so that it can
        be recorded into a CUDA graph (run substep once with the same method
        first).  See sgb_plan_substep_capturable for the refinement caps."""
        sp = (spec or RefineSpec()).ctypes()
        rc = self.L.sgb_plan_substep_capturable(self.handle, method.encode(), phi_exp,
                                                phi_imp, _ptr(u_in), _ptr(u_out),
                                                C.byref(sp), _ptr(stream))
        nat.check(rc, "sgb_plan_substep_capturable")

    def substep_stage(self, stage: int, phi_exp: float, phi_imp: float, u_in, u_out,
                      spec: RefineSpec | None = None, stream=0) -> None:
        """One of the two stages of the capturable mixed substep around an
        external complex64 factor (a RaggedFactor over several plans):
        stage 1 the explicit operator and the refinement's initial state,
        stage 2 everything after the factor."""
        sp = (spec or RefineSpec()).ctypes()
        rc = self.L.sgb_plan_substep_stage(self.handle, int(stage), b"M", phi_exp, phi_imp,
                                           _ptr(u_in), _ptr(u_out), C.byref(sp), _ptr(stream))
        nat.check(rc, "sgb_plan_substep_stage")

    def prepare(self, method: str = "M") -> None:
        """Allocate what the first substep of `method` would (then every
        substep may take the capturable form)."""
        nat.check(self.L.sgb_plan_prepare(self.handle, method.encode()), "sgb_plan_prepare")

    def unserved(self) -> int:
        """Fallback systems of the last capturable 'M' substep that did not
        fit its complex128 chunk (0 when none; synchronizes)."""
        n = C.c_int()
        nat.check(self.L.sgb_plan_unserved(self.handle, C.byref(n)), "sgb_plan_unserved")
        return n.value

    def substep_host(self, method: str, phi_exp: float, phi_imp: float,
                     u_in: np.ndarray, u_out: np.ndarray,
                     spec: RefineSpec | None = None, stream=0) -> None:
        sp = (spec or RefineSpec()).ctypes()
        rc = self.L.sgb_plan_substep_host(self.handle, method.encode(),
                                          phi_exp, phi_imp, _ptr(u_in),
                                          _ptr(u_out), C.byref(sp),
                                          _ptr(stream))
        nat.check(rc, "sgb_plan_substep_host")

    def report(self) -> dict:
        n = self.nsys
        info = np.zeros(n, np.int32)
        siter = np.zeros(n, np.int32)
        diter = np.zeros(n, np.int32)
        res = np.zeros(n)
        tolsc = np.zeros(n)
        fact = np.zeros(n, np.uint8)
        rc = self.L.sgb_plan_report(self.handle, info.ctypes.data,
                                    siter.ctypes.data, diter.ctypes.data,
                                    res.ctypes.data, tolsc.ctypes.data,
                                    fact.ctypes.data)
        nat.check(rc, "sgb_plan_report")
        return dict(info=info, siter=siter, diter=diter, res=res, tolsc=tolsc,
                    fact=fact.tobytes().decode())

    def assemble_packed(self, phi: float, ab, ldab: int, off: int = 0, stream=0) -> None:
        """Write every system's operator M + phi L as a packed complex128 band
        into the device buffer ab (nsys x ldab x N, column-major per system):
        off = 0, ldab = LD is packc; off = KL, ldab = LD + KL is packf."""
        nat.check(self.L.sgb_plan_assemble_packed(self.handle, phi, _ptr(ab), int(ldab),
                                                  int(ldab) * self.N, int(off), _ptr(stream)),
                  "sgb_plan_assemble_packed")

    def set_timing(self, on: bool) -> None:
        nat.check(self.L.sgb_plan_set_timing(self.handle, int(on)), "sgb_plan_set_timing")

    def timings(self) -> dict:
        """{phase: (total_ms, calls)} recorded since set_timing(True)."""
        buf = C.create_string_buffer(1 << 16)
        nat.check(self.L.sgb_plan_timings(self.handle, buf, len(buf)), "sgb_plan_timings")
        out = {}
        for line in buf.value.decode().splitlines():
            name, ms, calls = line.split()
            out[name] = (float(ms), int(calls))
        return out

    def backward_error(self, stream=0) -> np.ndarray:
        out = np.zeros(self.nsys)
        nat.check(self.L.sgb_plan_backward_error(self.handle, out.ctypes.data,
                                                 _ptr(stream)),
                  "sgb_plan_backward_error")
        return out


class RaggedFactor:
    """The complex64 factors of several plans' mixed substeps, each plan at
    its own implicit coefficient, as one launch per row-tile class (the
    systems of the largest plans first).  Between stage 1 and
    stage 2 of every plan's substep_stage; the plans must outlive it and
    hold their mixed workspace (a substep with 'M', or prepare('M'))."""

    def __init__(self, plans: list, phi_imp: list, spec: RefineSpec | None = None):
        self.L = nat.load()
        self.plans = list(plans)
        n = len(self.plans)
        arr = (C.c_void_p * n)(*[p.handle for p in self.plans])
        phis = (C.c_double * n)(*[float(v) for v in phi_imp])
        sp = (spec or RefineSpec()).ctypes()
        h = self.L.sgb_ragged_create(arr, n, phis, C.byref(sp))
        if not h:
            raise RuntimeError(f"sgb_ragged_create failed: {nat.last_error()}")
        self.handle = h

    def factor(self, stream=0) -> None:
        nat.check(self.L.sgb_ragged_factor(self.handle, _ptr(stream)), "sgb_ragged_factor")

    def close(self):
        if getattr(self, "handle", None):
            self.L.sgb_ragged_destroy(self.handle)
            self.handle = None

    __del__ = close


class BatchPlan:
    """One batch of systems of a case split into `parts` resident plans over
    consecutive wavenumber ranges (sgb_batch_*), each substep issued on the
    part's own CUDA stream (forked from and joined into the caller's stream)
    in the capturable form, which keeps the host out of the refinement loop:
    the parts' kernels overlap on the device, the FP64 residual and
    explicit-operator kernels of one part alongside the complex64 factor of
    another.  Results are those of one Plan over the whole batch with the
    capturable substep (each system is solved by the same kernels on the
    same data).  substep_host runs the same from host buffers with each
    part's copies overlapping the other parts' computation."""

    def __init__(self, case: SynthCase, kx: np.ndarray, kz: np.ndarray,
                 parts: int = 4, max_double_slots: int = 0, method: str = "M"):
        self.L = nat.load()
        self.case = case
        self._kx = np.ascontiguousarray(kx, dtype=np.float64)
        self._kz = np.ascontiguousarray(kz, dtype=np.float64)
        self.nsys = int(len(self._kx))
        self.N = case.N
        self._cs = case.ctypes_case()
        h = self.L.sgb_batch_create(C.byref(self._cs), self.nsys, self._kx.ctypes.data,
                                    self._kz.ctypes.data, int(parts), int(max_double_slots),
                                    method.encode() if method else b"\0")
        if not h:
            raise RuntimeError(f"sgb_batch_create failed: {nat.last_error()}")
        self.handle = h
        self.bounds = bounds(self.nsys, parts)

    @property
    def parts(self) -> int:
        return len(self.bounds) - 1

    def substep(self, method: str, phi_exp: float, phi_imp: float, u_in, u_out,
                spec: RefineSpec | None = None, stream=None) -> None:
        """u_in, u_out: device tensors (nsys x N); stream: the caller's
        stream (default torch's current stream)."""
        if stream is None:
            import torch
            stream = torch.cuda.current_stream().cuda_stream
        sp = (spec or RefineSpec()).ctypes()
        nat.check(self.L.sgb_batch_substep(self.handle, method.encode(), phi_exp, phi_imp,
                                           _ptr(u_in), _ptr(u_out), C.byref(sp), _ptr(stream)),
                  "sgb_batch_substep")

    def substep_host(self, method: str, phi_exp: float, phi_imp: float,
                     u_in: np.ndarray, u_out: np.ndarray, spec: RefineSpec | None = None,
                     stream=0) -> None:
        """u_in, u_out: host arrays (nsys x N complex128, pinned for overlap);
        returns when u_out holds the result."""
        sp = (spec or RefineSpec()).ctypes()
        nat.check(self.L.sgb_batch_substep_host(self.handle, method.encode(), phi_exp, phi_imp,
                                                _ptr(u_in), _ptr(u_out), C.byref(sp),
                                                _ptr(stream)),
                  "sgb_batch_substep_host")

    def report(self) -> dict:
        n = self.nsys
        info = np.zeros(n, np.int32)
        siter = np.zeros(n, np.int32)
        diter = np.zeros(n, np.int32)
        res = np.zeros(n)
        tolsc = np.zeros(n)
        fact = np.zeros(n, np.uint8)
        nat.check(self.L.sgb_batch_report(self.handle, info.ctypes.data, siter.ctypes.data,
                                          diter.ctypes.data, res.ctypes.data,
                                          tolsc.ctypes.data, fact.ctypes.data),
                  "sgb_batch_report")
        return dict(info=info, siter=siter, diter=diter, res=res, tolsc=tolsc,
                    fact=fact.tobytes().decode())

    def backward_error(self, stream=0) -> np.ndarray:
        out = np.zeros(self.nsys)
        nat.check(self.L.sgb_batch_backward_error(self.handle, out.ctypes.data, _ptr(stream)),
                  "sgb_batch_backward_error")
        return out

    def unserved(self) -> int:
        n = C.c_int()
        nat.check(self.L.sgb_batch_unserved(self.handle, C.byref(n)), "sgb_batch_unserved")
        return n.value

    def device_bytes(self) -> int:
        return int(self.L.sgb_batch_device_bytes(self.handle))

    def close(self) -> None:
        if getattr(self, "handle", None):
            self.L.sgb_batch_destroy(self.handle)
            self.handle = None

    __del__ = close


def bounds(nsys: int, parts: int) -> list:
    """Row offsets of a batch's parts (sgb_batch_bounds): consecutive ranges,
    part i holding rows i nsys / parts .. (i + 1) nsys / parts - 1."""
    L = nat.load()
    out = (C.c_int * (max(1, min(parts, nsys)) + 1))()
    p = L.sgb_batch_bounds(int(nsys), int(parts), out)
    if p < 1:
        raise ValueError(f"sgb_batch_bounds({nsys}, {parts}): {nat.last_error()}")
    return [int(out[i]) for i in range(p + 1)]
