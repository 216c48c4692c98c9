"""ctypes binding of libsuzerain_gb300.so (the C-ABI in include/suzerain_gb300.h).

The library is built in-tree by suzerain_gb300.build.  Loading fails loudly
when it is missing: there is no CPU implementation behind this package.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

_i, _d, _p, _ll, _sz = C.c_int, C.c_double, C.c_void_p, C.c_longlong, C.c_size_t
_u64 = C.c_uint64


class ZC(C.Structure):
    """double _Complex / std::complex<double> by value."""
    _fields_ = [("re", C.c_double), ("im", C.c_double)]


class CC(C.Structure):
    """float _Complex / std::complex<float> by value."""
    _fields_ = [("re", C.c_float), ("im", C.c_float)]


class Bsmbsm(C.Structure):
    _fields_ = [(k, C.c_int) for k in ("S", "n", "kl", "ku", "ld", "N", "KL",
                                       "KU", "LD")]


class Permutation(C.Structure):
    """Layout of gsl_permutation."""
    _fields_ = [("size", C.c_size_t), ("data", C.POINTER(C.c_size_t))]


class Case(C.Structure):
    _fields_ = [("S", _i), ("n", _i), ("kl", _i), ("ku", _i), ("ld", _i),
                ("M", _p), ("D1", _p), ("D2", _p), ("a", _p), ("b", _p),
                ("c", _p), ("g", _p), ("dirichlet_mask", C.c_uint),
                ("pad_", _i)]


class RefineSpec(C.Structure):
    _fields_ = [("aiter", _i), ("siter", _i), ("diter", _i), ("tolsc", _d)]


class RefineReport(C.Structure):
    _fields_ = [("info", _p), ("siter", _p), ("diter", _p), ("res", _p),
                ("tolsc", _p), ("fact", _p)]


class BsplineopWorkspace(C.Structure):
    _fields_ = [("method", _i), ("k", _i), ("n", _i), ("nderiv", _i),
                ("kl", C.POINTER(_i)), ("ku", C.POINTER(_i)), ("max_kl", _i),
                ("max_ku", _i), ("ld", _i),
                ("D_T", C.POINTER(C.POINTER(_d)))]


class BsplineopLuWorkspace(C.Structure):
    _fields_ = [("n", _i), ("kl", _i), ("ku", _i), ("ld", _i),
                ("ipiv", C.POINTER(_i)), ("A_T", C.POINTER(_d))]


class BsplineopLuzWorkspace(C.Structure):
    _fields_ = [("n", _i), ("kl", _i), ("ku", _i), ("ld", _i),
                ("ipiv", C.POINTER(_i)), ("A_T", C.POINTER(_d))]   # interleaved re, im


_BW = C.POINTER(BsplineopWorkspace)
_LU = C.POINTER(BsplineopLuWorkspace)
_LUZ = C.POINTER(BsplineopLuzWorkspace)

_SIGS = {
    # drop-ins
    "suzerain_bsmbsm_construct": (Bsmbsm, [_i, _i, _i, _i]),
    "suzerain_bsmbsm_q": (_i, [_i, _i, _i]),
    "suzerain_bsmbsm_qinv": (_i, [_i, _i, _i]),
    "suzerain_bsmbsm_saPxpby": (_i, [C.c_char, _i, _i, C.c_float, _p, _i,
                                     C.c_float, _p, _i]),
    "suzerain_bsmbsm_daPxpby": (_i, [C.c_char, _i, _i, _d, _p, _i, _d, _p,
                                     _i]),
    "suzerain_bsmbsm_caPxpby": (_i, [C.c_char, _i, _i, CC, _p, _i, CC, _p,
                                     _i]),
    "suzerain_bsmbsm_zaPxpby": (_i, [C.c_char, _i, _i, ZC, _p, _i, ZC, _p,
                                     _i]),
    "suzerain_bsmbsm_dpack": (_i, [_i] * 6 + [_d, _p, _i, _i, _i, _p, _i]),
    "suzerain_bsmbsm_zpack": (_i, [_i] * 6 + [ZC, _p, _i, _i, _i, _p, _i]),
    "suzerain_bsmbsm_zdpack": (_i, [_i] * 6 + [ZC, _p, _i, _i, _i, _p, _i]),
    "suzerain_bsmbsm_spack": (_i, [_i] * 6 + [C.c_float, _p, _i, _i, _i, _p, _i]),
    "suzerain_bsmbsm_cpack": (_i, [_i] * 6 + [CC, _p, _i, _i, _i, _p, _i]),
    "suzerain_bsmbsm_cspack": (_i, [_i] * 6 + [CC, _p, _i, _i, _i, _p, _i]),
    "suzerain_bsmbsm_spackc": (_i, [_p, _i, _i, C.c_float, _p, _p]),
    "suzerain_bsmbsm_spackf": (_i, [_p, _i, _i, C.c_float, _p, _p]),
    "suzerain_bsmbsm_dpackc": (_i, [_p, _i, _i, _d, _p, _p]),
    "suzerain_bsmbsm_dpackf": (_i, [_p, _i, _i, _d, _p, _p]),
    "suzerain_bsmbsm_cpackc": (_i, [_p, _i, _i, CC, _p, _p]),
    "suzerain_bsmbsm_cpackf": (_i, [_p, _i, _i, CC, _p, _p]),
    "suzerain_bsmbsm_cspackc": (_i, [_p, _i, _i, CC, _p, _p]),
    "suzerain_bsmbsm_cspackf": (_i, [_p, _i, _i, CC, _p, _p]),
    "suzerain_bsmbsm_permutation": (C.POINTER(Permutation), [_i, _i]),
    "sgb_permutation_free": (None, [C.POINTER(Permutation)]),
    "suzerain_bsmbsm_zpackc": (_i, [_p, _i, _i, ZC, _p, _p]),
    "suzerain_bsmbsm_zpackf": (_i, [_p, _i, _i, ZC, _p, _p]),
    "suzerain_bsmbsm_zdpackc": (_i, [_p, _i, _i, ZC, _p, _p]),
    "suzerain_bsmbsm_zdpackf": (_i, [_p, _i, _i, ZC, _p, _p]),
    "suzerain_lapack_zgbtrf": (_i, [_i, _i, _i, _i, _p, _i, _p]),
    "suzerain_lapack_cgbtrf": (_i, [_i, _i, _i, _i, _p, _i, _p]),
    "suzerain_lapack_zgbtrs": (_i, [C.c_char, _i, _i, _i, _i, _p, _i, _p,
                                    _p, _i]),
    "suzerain_lapack_cgbtrs": (_i, [C.c_char, _i, _i, _i, _i, _p, _i, _p,
                                    _p, _i]),
    "suzerain_lapackext_zgbsv": (_i, [_p, C.c_char, _i, _i, _i, _i, _p, _i,
                                      _p, _p, _i]),
    "suzerain_lapackext_cgbsv": (_i, [_p, C.c_char, _i, _i, _i, _i, _p, _i,
                                      _p, _p, _i]),
    "suzerain_lapackext_dgbsv": (_i, [_p, C.c_char, _i, _i, _i, _i, _p, _i,
                                      _p, _p, _i]),
    "suzerain_lapackext_sgbsv": (_i, [_p, C.c_char, _i, _i, _i, _i, _p, _i,
                                      _p, _p, _i]),
    "suzerain_lapackext_dsgbsvx": (_i, [_p, _p, _i, C.c_char, _i, _i, _i, _p,
                                        _p, _p, _p, _p, _p, _p, _p, _p, _p,
                                        _p]),
    "suzerain_lapack_zgbsvx": (_i, [C.c_char, C.c_char, _i, _i, _i, _i, _p, _i,
                                    _p, _i, _p, _p, _p, _p, _p, _i, _p, _i,
                                    _p, _p, _p, _p, _p]),
    "sgb_zgbsvx_batched": (_i, [C.c_char, C.c_char, _i, _i, _i, _i, _p, _i,
                                _ll, _p, _i, _ll, _p, _p, _p, _p, _p, _p, _p,
                                _p, _p, _p, _p, _p]),
    "suzerain_lapackext_zcgbsvx": (_i, [_p, _p, _i, C.c_char, _i, _i, _i, _p,
                                        _p, _p, _p, _p, _p, _p, _p, _p, _p,
                                        _p]),
    "suzerain_blas_zgbmv": (_i, [C.c_char, _i, _i, _i, _i, ZC, _p, _i, _p, _i,
                                 ZC, _p, _i]),
    "sgb_bsplineop_alloc_breakpoints": (C.POINTER(BsplineopWorkspace),
                                        [_i, _i, _p, _i]),
    "suzerain_bsplineop_free": (None, [C.POINTER(BsplineopWorkspace)]),
    "suzerain_bsplineop_accumulate_complex": (
        _i, [_i, _i, ZC, _p, _i, _i, ZC, _p, _i, _i,
             C.POINTER(BsplineopWorkspace)]),
    "suzerain_bsplineop_apply": (_i, [_i, _i, _d, _p, _i, _i, _BW]),
    "suzerain_bsplineop_accumulate": (_i, [_i, _i, _d, _p, _i, _i, _d, _p, _i, _i, _BW]),
    "suzerain_bsplineop_apply_complex": (_i, [_i, _i, _d, _p, _i, _i, _BW]),
    "suzerain_bsplineop_lu_alloc": (_LU, [_BW]),
    "suzerain_bsplineop_lu_free": (None, [_LU]),
    "suzerain_bsplineop_lu_opaccumulate": (_i, [_i, _p, _BW, _d, _LU]),
    "suzerain_bsplineop_lu_opnorm": (_i, [_LU, _p]),
    "suzerain_bsplineop_lu_factor": (_i, [_LU]),
    "suzerain_bsplineop_lu_rcond": (_i, [_d, _p, _LU]),
    "suzerain_bsplineop_lu_solve": (_i, [_i, _p, _i, _i, _LU]),
    "suzerain_bsplineop_lu_opform": (_i, [_i, _p, _BW, _LU]),
    "suzerain_bsplineop_lu_opform_mass": (_i, [_BW, _LU]),
    "suzerain_bsplineop_lu_factor_mass": (_i, [_BW, _LU]),
    "suzerain_bsplineop_luz_alloc": (_LUZ, [_BW]),
    "suzerain_bsplineop_luz_free": (None, [_LUZ]),
    "suzerain_bsplineop_luz_opaccumulate": (_i, [_i, _p, _BW, ZC, _LUZ]),
    "suzerain_bsplineop_luz_opnorm": (_i, [_LUZ, _p]),
    "suzerain_bsplineop_luz_factor": (_i, [_LUZ]),
    "suzerain_bsplineop_luz_rcond": (_i, [_d, _p, _LUZ]),
    "suzerain_bsplineop_luz_solve": (_i, [_i, _p, _i, _i, _LUZ]),
    "suzerain_bsplineop_luz_opform": (_i, [_i, _p, _BW, _LUZ]),
    "suzerain_bsplineop_luz_opform_mass": (_i, [_BW, _LUZ]),
    "suzerain_bsplineop_luz_factor_mass": (_i, [_BW, _LUZ]),
    "suzerain_lapack_zgbcon": (_i, [C.c_char, _i, _i, _i, _p, _i, _p, _d, _p, _p, _p]),
    "sgb_bspline_collocation_bands": (_i, [_i, _i, _p, _i, _p, _p, _p, _p,
                                           _p]),
    "suzerain_htstretch2": (_d, [_d, _d, _d]),
    "suzerain_inorder_wavenumber": (_i, [_i, _i]),
    "suzerain_diffwave_apply": (_i, [_i, _i, ZC, _p, _d, _d, _i, _i, _i, _i,
                                     _i, _i, _i, _i, _i]),
    "suzerain_diffwave_accumulate": (_i, [_i, _i, ZC, _p, ZC, _p, _d, _d, _i, _i,
                                          _i, _i, _i, _i, _i, _i, _i]),
    **{f"suzerain_blasext_{nm}_{sfx}": (_i, [C.c_char, _i, _i, _i] + [ZC, _p, _i] * k
                                            + [_p, _i, _p, _i, ZC, _p, _i])
       for k, nm in enumerate(("zgbdmv", "zgbddmv", "zgbdddmv", "zgbddddmv", "zgbdddddmv"), 1)
       for sfx in ("d_z", "d_d")},
    # batched device API
    "sgb_last_error": (C.c_char_p, []),
    "sgb_device_ok": (_i, []),
    "sgb_factor_elems": (_ll, [_i, _i, _i]),
    "sgb_gbtrf_batched": (_i, [C.c_char, _i, _i, _i, _i, _p, _i, _ll, _p, _p,
                               _p, _p]),
    "sgb_gbtrf_batched_ex": (_i, [C.c_char, _i, _i, _i, _i, _p, _i, _ll, _p,
                                  _p, _p, _i, _i, _i, _p]),
    "sgb_gbtrf_phase_cycles": (_i, [C.c_char, _i, _i, _i, _i, _p, _i, _ll, _p,
                                    _p, _p, _i, _i, _p, _p]),
    "sgb_measure_peaks": (_i, [_p, _p]),
    "sgb_gbtrf_set_shape": (_i, [C.c_char, _i, _i, _i, _i, _i]),
    "sgb_gbtrf_get_shape": (_i, [C.c_char, _i, _i, _i, _p, _p]),
    "sgb_gbtrs_batched": (_i, [C.c_char, C.c_char, _i, _i, _i, _i, _p, _p, _p,
                               _p, _p]),
    "sgb_gbtrs_batched_ws": (_i, [C.c_char, C.c_char, _i, _i, _i, _i, _p, _p, _p,
                                  _p, _p, _p]),
    "sgb_gbtrs_shared": (_i, [C.c_char, C.c_char, _i, _i, _i, _i, _p, _p, _p, _ll,
                              _p, _ll, _p, _p]),
    "sgb_factor_to_lapack": (_i, [C.c_char, _i, _i, _i, _i, _p, _p, _p]),
    "sgb_zcgbsvx_batched": (_i, [_i, _i, _i, _i, C.c_char, _p, _i, _ll, _p,
                                 _p, C.POINTER(RefineSpec),
                                 C.POINTER(RefineReport), _p]),
    "sgb_zcgbsvx_batched_static": (_i, [_i, _i, _i, _i, C.c_char, _p, _i, _ll,
                                        _p, _p, C.POINTER(RefineSpec),
                                        C.POINTER(RefineReport), _p]),
    "sgb_plan_create": (_p, [C.POINTER(Case), _i, _p, _p, _i]),
    "sgb_plan_destroy": (_i, [_p]),
    "sgb_plan_device_bytes": (_sz, [_p]),
    "sgb_plan_pool_trim": (_i, [_sz]),
    "sgb_gbtrs_set_quad_depth": (_i, [_i, _i]),
    "sgb_gbtrs_set_quad_bulk": (_i, [_i]),
    "sgb_gbtrf_set_specialized": (_i, [_i]),
    "sgb_async_faults": (_i, []),
    "sgb_plan_substep": (_i, [_p, C.c_char, _d, _d, _p, _p,
                              C.POINTER(RefineSpec), _p]),
    "sgb_plan_substep_host": (_i, [_p, C.c_char, _d, _d, _p, _p,
                                   C.POINTER(RefineSpec), _p]),
    "sgb_plan_substep_capturable": (_i, [_p, C.c_char, _d, _d, _p, _p,
                                         C.POINTER(RefineSpec), _p]),
    "sgb_plan_unserved": (_i, [_p, _p]),
    "sgb_plan_prepare": (_i, [_p, C.c_char]),
    "sgb_plan_substep_stage": (_i, [_p, _i, C.c_char, _d, _d, _p, _p,
                                    C.POINTER(RefineSpec), _p]),
    "sgb_ragged_create": (_p, [_p, _i, _p, C.POINTER(RefineSpec)]),
    "sgb_ragged_factor": (_i, [_p, _p]),
    "sgb_ragged_destroy": (None, [_p]),
    "sgb_solver_spec_default": (None, [_p]),
    "sgb_solver_spec_parse": (_i, [C.c_char_p, _p, _p, C.c_size_t]),
    "sgb_solver_spec_format": (_i, [_p, _p, C.c_size_t]),
    "sgb_plan_estimate_bytes": (C.c_size_t, [_p, _i, _i, C.c_char]),
    "sgb_plan_report": (_i, [_p, _p, _p, _p, _p, _p, _p]),
    "sgb_plan_backward_error": (_i, [_p, _p, _p]),
    "sgb_plan_set_timing": (_i, [_p, _i]),
    "sgb_plan_timings": (_i, [_p, C.c_char_p, _i]),
    "sgb_launch_count": (_ll, []),
    "sgb_plan_assemble_packed": (_i, [_p, _d, _p, _i, _ll, _i, _p]),
    "suzerain_blasext_zgb_diag_scale_acc_d": (_i, [C.c_char, _i, _i, _i, _i] + [ZC, _p, _i]
                                              + [_p, _i, _i, ZC, _p, _i, _i]),
    "suzerain_blasext_zgb_ddiag_scale_acc_d": (_i, [C.c_char, _i, _i, _i, _i] + [ZC, _p, _i] * 2
                                               + [_p, _i, _i, ZC, _p, _i, _i]),
    "suzerain_blasext_zgb_dddiag_scale_acc_d": (_i, [C.c_char, _i, _i, _i, _i] + [ZC, _p, _i] * 3
                                                + [_p, _i, _i, ZC, _p, _i, _i]),
    "suzerain_blasext_zgb_ddddiag_scale_acc_d": (_i, [C.c_char, _i, _i, _i, _i]
                                                 + [ZC, _p, _i] * 4
                                                 + [_p, _i, _i, ZC, _p, _i, _i]),
    "suzerain_blasext_zgb_dddddiag_scale_acc_d": (_i, [C.c_char, _i, _i, _i, _i]
                                                  + [ZC, _p, _i] * 5
                                                  + [_p, _i, _i, ZC, _p, _i, _i]),
    "suzerain_blas_zgb_acc_d": (_i, [_i, _i, _i, _i, ZC, _p, _i, ZC, _p, _i]),
    "suzerain_blasext_zdemote": (_i, [_i, _p]),
    "suzerain_blasext_zpromote": (_i, [_i, _p]),
    "suzerain_blasext_ddemote": (_i, [_i, _p]),
    "suzerain_blasext_dpromote": (_i, [_i, _p]),
    "suzerain_blasext_zgbnorm1": (_i, [_i, _i, _i, _i, _p, _i, _p]),
    "suzerain_blasext_dgbnorm1": (_i, [_i, _i, _i, _i, _p, _i, _p]),
    "sgb_rholut_create": (_p, [_p, _p, _p, C.POINTER(BsplineopWorkspace), _p, _p, _p, _p]),
    "sgb_rholut_destroy": (_i, [_p]),
    "sgb_rholut_geometry": (_i, [_p, _p]),
    "sgb_rholut_pack_batched": (_i, [_p, _d, _d, _i, _p, _p, _p, _i, _ll, _i, _p]),
    "sgb_rholut_accumulate_batched": (_i, [_p, _d, _d, _i, _p, _p, _p, _ll, _d, _d, _p, _ll,
                                           _p]),
    "suzerain_rholut_imexop_accumulate": (None, [ZC, _d, _d, _p, _p, _p,
                                                 C.POINTER(BsplineopWorkspace)]
                                          + [_p] * 5 + [ZC] + [_p] * 5 + [_p] * 3),
    "suzerain_rholut_imexop_accumulate00": (None, [ZC, _p, _p, _p,
                                                   C.POINTER(BsplineopWorkspace)]
                                            + [_p] * 5 + [ZC] + [_p] * 5 + [_p]),
    "suzerain_rholut_imexop_packc": (None, [ZC, _d, _d, _p, _p, _p,
                                            C.POINTER(BsplineopWorkspace)] + [_i] * 5
                                     + [_p, _p, _p] + [_p] * 3),
    "suzerain_rholut_imexop_packf": (None, [ZC, _d, _d, _p, _p, _p,
                                            C.POINTER(BsplineopWorkspace)] + [_i] * 5
                                     + [_p, _p, _p] + [_p] * 3),
    "suzerain_rholut_imexop_packc00": (None, [ZC, _p, _p, _p, C.POINTER(BsplineopWorkspace)]
                                       + [_i] * 5 + [_p, _p, _p] + [_p]),
    "suzerain_rholut_imexop_packf00": (None, [ZC, _p, _p, _p, C.POINTER(BsplineopWorkspace)]
                                       + [_i] * 5 + [_p, _p, _p] + [_p]),
    "sgb_batch_bounds": (_i, [_i, _i, _p]),
    "sgb_batch_create": (_p, [C.POINTER(Case), _i, _p, _p, _i, _i, C.c_char]),
    "sgb_batch_destroy": (_i, [_p]),
    "sgb_batch_parts": (_i, [_p]),
    "sgb_batch_plan": (_p, [_p, _i]),
    "sgb_batch_device_bytes": (C.c_size_t, [_p]),
    "sgb_batch_substep": (_i, [_p, C.c_char, _d, _d, _p, _p, _p, _p]),
    "sgb_batch_substep_host": (_i, [_p, C.c_char, _d, _d, _p, _p, _p, _p]),
    "sgb_batch_report": (_i, [_p, _p, _p, _p, _p, _p, _p]),
    "sgb_batch_backward_error": (_i, [_p, _p, _p]),
    "sgb_batch_unserved": (_i, [_p, _p]),
    "sgb_synth_case": (_i, [_i, _i, _i, _d, _d, _d, _d, _i, _u64, C.c_uint,
                            _p, _p, _p, _p, _p, _p, _p, _p, _p]),
    "sgb_synth_wavenumbers": (_i, [_i, _i, _d, _d, _p, _p]),
    "sgb_synth_rhs": (_i, [_u64, _ll, _i, _p]),
}

_lib = None
_generator = None
_GEN_SIGS = ("sgb_synth_case", "sgb_synth_wavenumbers", "sgb_synth_rhs")


def bind_generator(path: str):
    """Use a host-only build of the seeded input generator (the same C++
    sources, without the CUDA code) for the sgb_synth_* calls, so that a
    process that only generates inputs never maps the GPU library."""
    global _generator
    G = C.CDLL(path)
    for name in _GEN_SIGS:
        f = getattr(G, name)
        f.restype, f.argtypes = _SIGS[name]
    _generator = G
    return G


def generator():
    """The library that serves sgb_synth_*: the bound host-only generator,
    else the full native library."""
    return _generator if _generator is not None else load()


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = False):
    """Load the native library; raise if it is absent (no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_build.LIB):
        if build_if_missing:
            _build.build()
        else:
            raise ImportError(
                "suzerain_gb300 native library is not built "
                f"({_build.LIB}); run suzerain_gb300.build.build()")
    L = C.CDLL(_build.LIB)
    for name, (res, args) in _SIGS.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def last_error() -> str:
    return load().sgb_last_error().decode()


def check(rc: int, what: str) -> None:
    if rc != 0:
        raise RuntimeError(f"{what} failed ({rc}): {last_error()}")


def zc(v) -> ZC:
    v = complex(v)
    return ZC(v.real, v.imag)


def cc(v) -> CC:
    v = complex(v)
    return CC(v.real, v.imag)
