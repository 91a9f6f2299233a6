"""born_gb300 — GB300-native Born modelling / RTM propagator (host side).

The compute path is ``_build/libborn_gb300.so`` (hand-written sm_103a CUDA
kernels behind the C ABI declared in ``include/born_gb300.h``).  This module
binds that ABI with ctypes and mirrors the reference's propagator interface
``baseProp`` (``base/base_prop.h:4-72``) as :class:`Gb300Prop`, with the same
method names, argument meaning and call order as ``cpuProp`` / ``gpuProp``, so
code written against the reference drives the GPU unchanged.  There is no CPU
fallback: if the library cannot be loaded, every entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libborn_gb300.so")

BORN_OK = 0
ERRORS = {-1: "EINVAL", -2: "ECUDA", -3: "ENOMEM", -4: "ESTATE",
          -5: "ETIMEOUT", -6: "ENODEV"}


class BornError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"born_gb300 {ERRORS.get(code, code)}: {msg}")
        self.code = code


_fp = C.POINTER(C.c_float)
_ip = C.POINTER(C.c_int)
_vp = C.c_void_p

# name -> (restype, argtypes); mirrors include/born_gb300.h
_SIGS = {
    # reference-compatible names (base/gpu/gpu_funcs_3d.h)
    "setup_cuda": (None, [C.c_int]),
    "create_gpu_space": (None, [C.c_float] * 6 + [C.c_int] * 3),
    "transfer_sinc_table_s": (None, [C.c_int, C.c_int, _fp]),
    "transfer_sinc_table_d": (None, [C.c_int, C.c_int, _fp]),
    "transfer_source_func": (None, [C.c_int, C.c_int, _ip, _fp]),
    "load_source": (None, [C.c_int]),
    "transfer_receiver_func": (None, [C.c_int, C.c_int, C.c_int, _ip, _fp]),
    "transfer_vel_func1": (None, [C.c_int, C.c_int, C.c_int, _fp]),
    "transfer_vel_func2": (None, [C.c_int, C.c_int, C.c_int, _fp]),
    "source_prop": (None, [C.c_int, C.c_int, C.c_int, C.c_bool, C.c_bool,
                           _fp, _fp, C.c_int, C.c_int, C.c_int]),
    "rtm_adjoint": (None, [C.c_int, C.c_int, C.c_int, C.c_int, _fp, _fp, _fp,
                           C.c_int, C.c_int]),
    "set_ntblock": (None, [C.c_int]),
    "rtm_forward": (None, [C.c_int, C.c_int, C.c_int, C.c_int, _fp, _fp,
                           C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]),
    "born_default_status": (C.c_int, []),
    "born_default_error": (C.c_char_p, []),
    "born_default_handle": (_vp, []),
    # handle API
    "born_create": (C.c_int, [C.c_int, C.POINTER(_vp)]),
    "born_destroy": (C.c_int, [_vp]),
    "born_error_string": (C.c_char_p, [_vp]),
    "born_create_space": (C.c_int, [_vp] + [C.c_float] * 6 + [C.c_int] * 3),
    "born_set_sinc_table": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, _fp]),
    "born_set_source_func": (C.c_int, [_vp, C.c_int, C.c_int, _ip, _fp]),
    "born_set_receiver_func": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, _ip,
                                         _fp]),
    "born_set_velocity": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, C.c_int,
                                    _fp]),
    "born_set_reflectivity": (C.c_int, [_vp, _fp]),
    "born_make_velocity": (C.c_int, [_vp, C.c_int, _fp, C.c_int, C.c_int,
                                     C.c_int] + [C.c_float] * 7 +
                           [C.c_ulonglong, C.c_int, C.c_int, C.c_int] +
                           [C.c_float] * 7),
    "born_get_velocity": (C.c_int, [_vp, C.c_int, _fp]),
    "born_source_prop": (C.c_int, [_vp, C.c_int, C.c_int, _fp, _fp]),
    "born_rtm_adjoint": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, _fp]),
    "born_set_host_levels": (C.c_int, [_vp, C.c_int]),
    "born_rtm_adjoint_host": (C.c_int, [_vp, C.c_int, C.c_int, _fp, _fp,
                                        _fp]),
    "born_rtm_forward": (C.c_int, [_vp, C.c_int, C.c_int, _fp]),
    "born_model": (C.c_int, [_vp, C.c_int, C.c_int, _fp]),
    "born_lin_forward": (C.c_int, [_vp, C.c_int, C.c_int, _fp]),
    "born_lin_adjoint": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, _fp]),
    "born_get_image": (C.c_int, [_vp, _fp]),
    "born_image_device": (_vp, [_vp]),
    "born_get_traces": (C.c_int, [_vp, _fp]),
    "born_get_source_levels": (C.c_int, [_vp, _fp, _fp]),
    "born_set_source_levels": (C.c_int, [_vp, _fp, _fp]),
    "born_zero_traces": (C.c_int, [_vp]),
    "born_synchronize": (C.c_int, [_vp]),
    "born_tile_config_count": (C.c_int, []),
    "born_set_tiling": (C.c_int, [_vp, C.c_int, C.c_int]),
    "born_set_storage": (C.c_int, [_vp, C.c_int]),
    "born_get_storage": (C.c_int, [_vp]),
    "born_autotune": (C.c_int, [_vp, C.c_int]),
    "born_tuned_config": (C.c_int, [_vp, C.c_int, _ip, _fp]),
    "born_loop_tile_ms": (C.c_int, [_vp, C.c_int, _fp, C.c_int]),
    "born_tuned_zseg": (C.c_int, [_vp, C.c_int]),
    "born_set_launch_overlap": (C.c_int, [_vp, C.c_int]),
    "born_set_host_prewarm": (C.c_int, [_vp, C.c_int]),
    "born_host_prewarm_count": (C.c_longlong, [_vp]),
    "born_couple_exact_device": (C.c_int, [_vp, _vp, _vp, _vp, C.c_longlong,
                                           _vp]),
    "born_op_checkpoint_shots": (C.c_int, [_vp]),
    "born_op_checkpoints_reused": (C.c_longlong, [_vp]),
    "born_set_checkpoint_interval": (C.c_int, [_vp, C.c_int]),
    "born_set_checkpoint_storage": (C.c_int, [_vp, C.c_int]),
    "born_checkpoints_reused": (C.c_int, [_vp]),
    "born_time_phases": (C.c_int, [_vp, C.c_int]),
    "born_phase_times": (C.c_int, [_vp, _fp, C.c_int]),
    "born_selftest_wait_timeout": (C.c_int, [_vp]),
    "born_stream_mix_gbs": (C.c_int, [C.c_int, C.c_int, C.c_longlong,
                                      C.c_int, _fp]),
    "born_kernel_launches": (C.c_longlong, [_vp]),
    "born_stream": (_vp, [_vp]),
    # batched shots (include/born_gb300.h section 4)
    "born_batch_create": (C.c_int, [C.POINTER(_vp), C.c_int,
                                    C.POINTER(_vp)]),
    "born_batch_destroy": (C.c_int, [_vp]),
    "born_batch_error": (C.c_char_p, [_vp]),
    "born_batch_set_graph": (C.c_int, [_vp, C.c_int]),
    "born_batch_stream": (_vp, [_vp]),
    "born_batch_launches": (C.c_longlong, [_vp]),
    "born_batch_graph_launches": (C.c_longlong, [_vp]),
    "born_batch_source_prop": (C.c_int, [_vp, C.c_int, C.c_int]),
    "born_batch_rtm_adjoint": (C.c_int, [_vp, C.c_int, C.c_int]),
    "born_batch_rtm_forward": (C.c_int, [_vp, C.c_int, C.c_int]),
    "born_batch_synchronize": (C.c_int, [_vp]),
    # operator and CG (include/born_gb300.h section 3)
    "born_op_create": (C.c_int, [_vp, _vp, _fp, _fp, _fp, C.POINTER(_vp)]),
    "born_op_destroy": (C.c_int, [_vp]),
    "born_op_sizes": (C.c_int, [_vp, C.POINTER(C.c_longlong),
                                C.POINTER(C.c_longlong), _ip, _fp]),
    "born_op_forward": (C.c_int, [_vp, C.c_int, _vp, _vp]),
    "born_op_adjoint": (C.c_int, [_vp, C.c_int, _vp, _vp]),
    "born_dot_f64": (C.c_int, [_vp, _vp, _vp, C.c_longlong,
                               C.POINTER(C.c_double)]),
    "born_cg_solve": (C.c_int, [_vp, _vp, _vp, C.c_int,
                                C.POINTER(C.c_double)]),
    "born_vec_create": (C.c_int, [_vp, C.c_longlong, C.POINTER(_vp)]),
    "born_vec_destroy": (C.c_int, [_vp, _vp]),
    "born_vec_fill": (C.c_int, [_vp, _vp, C.c_longlong, C.c_double]),
    "born_vec_scale": (C.c_int, [_vp, _vp, C.c_longlong, C.c_double]),
    "born_vec_scale_add": (C.c_int, [_vp, _vp, C.c_double, _vp, C.c_double,
                                     C.c_longlong]),
    "born_vec_lincomb": (C.c_int, [_vp, _vp, C.c_double, _vp, C.c_double,
                                   _vp, C.c_longlong]),
    "born_vec_add": (C.c_int, [_vp, _vp, _vp, C.c_longlong]),
    "born_vec_copy": (C.c_int, [_vp, _vp, _vp, C.c_longlong]),
    "born_vec_upload": (C.c_int, [_vp, _vp, _fp, C.c_longlong]),
    "born_vec_download": (C.c_int, [_vp, _fp, _vp, C.c_longlong]),
    "born_dot_f64_noalloc": (C.c_int, [_vp, _vp, C.c_longlong,
                                       C.POINTER(C.c_double), _vp]),
    # host geometry (csrc/born_host.h)
    "born_sinc_table": (C.c_int, [C.c_int, C.c_int, _fp]),
    "born_calc_stability": (C.c_float, [C.c_float, C.c_float, C.c_float,
                                        C.c_int, _ip]),
    "born_compute_size": (C.c_int, [C.c_int, C.c_int, C.c_int]),
    "born_source_geometry": (C.c_int, [C.c_float] * 9 + [
        C.c_int, C.c_int, _fp, C.c_int, C.c_int, _ip, _fp]),
    "born_wavelet_deriv": (C.c_int, [_fp, C.c_int, C.c_float, _fp]),
    "born_receiver_geometry": (C.c_int, [C.c_int, C.c_int] + [C.c_float] * 11
                               + [C.c_int, C.c_int, _ip]),
    "born_rand_subspace": (C.c_int, [_fp, C.c_int, C.c_int, C.c_int] +
                           [C.c_float] * 7 + [C.c_int] * 4 + [C.c_float] +
                           [C.c_int] * 3 + [C.c_float] * 6 + [_fp]),
    "born_laplac_forward": (C.c_int, [C.c_int, _fp, _fp, C.c_int, C.c_int,
                                      C.c_int]),
    "born_laplac_adjoint": (C.c_int, [C.c_int, _fp, _fp, C.c_int, C.c_int,
                                      C.c_int]),
    "born_deriv_forward": (C.c_int, [C.c_int, _fp, _fp, C.c_int, C.c_int,
                                     C.c_int, C.c_float]),
    "born_deriv_adjoint": (C.c_int, [C.c_int, _fp, _fp, C.c_int, C.c_int,
                                     C.c_int, C.c_float]),
    "born_map_data_forward": (C.c_int, [C.c_int, _fp, _fp, C.c_int, C.c_int,
                                        C.c_int, C.c_int]),
    "born_map_data_adjoint": (C.c_int, [C.c_int, _fp, _fp, C.c_int, C.c_int,
                                        C.c_int, C.c_int]),
    "born_extract_sub": (C.c_int, [_fp, C.c_int, C.c_int, C.c_int, _fp,
                                   C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                   C.c_int]),
    "born_add_image": (C.c_int, [_fp, C.c_int, C.c_int, C.c_int, _fp, C.c_int,
                                 C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]),
    "born_window_offset": (C.c_int, [C.c_float] * 3),
    "born_sep_read_info": (C.c_int, [C.c_char_p, _vp]),
    "born_sep_read": (C.c_int, [C.c_char_p, _fp, C.c_longlong]),
    "born_sep_write": (C.c_int, [C.c_char_p, _vp, _fp, C.c_int]),
    "born_json_read_info": (C.c_int, [C.c_char_p, _vp]),
    "born_regfile_read_info": (C.c_int, [C.c_char_p, _vp]),
    "born_regfile_read": (C.c_int, [C.c_char_p, _fp, C.c_longlong]),
    "born_regfile_write": (C.c_int, [C.c_char_p, _vp, _fp]),
    "born_add_regfiles": (C.c_int, [C.c_char_p, C.c_char_p, C.c_char_p]),
}

_lib = None


def build(force: bool = False) -> str:
    """Compile the CUDA library in-tree (nvcc, sm_103a)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "born_gb300_build", os.path.join(HERE, "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build(force=force)


def lib():
    """The loaded CUDA library; raises if it is missing (no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with "
                "`python sc17-born_gb300/build.py` (needs nvcc)")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def exported_symbols() -> list[str]:
    return list(_SIGS)


def fptr(a):
    if a is None:
        return None
    assert a.dtype == np.float32 and a.flags.c_contiguous, "need C float32"
    return a.ctypes.data_as(_fp)


def iptr(a):
    assert a.dtype == np.int32 and a.flags.c_contiguous, "need C int32"
    return a.ctypes.data_as(_ip)


def f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


class Handle:
    """Owns one ``born_handle`` (one device, one stream)."""

    def __init__(self, device: int = 0):
        self.lib = lib()
        h = _vp()
        rc = self.lib.born_create(device, C.byref(h))
        if rc != BORN_OK:
            raise BornError(rc, f"born_create(device={device}) failed")
        self.h = h
        self.device = device

    def check(self, rc: int) -> int:
        if rc != BORN_OK:
            msg = self.lib.born_error_string(self.h)
            raise BornError(rc, msg.decode() if msg else "")
        return rc

    def close(self):
        if getattr(self, "h", None):
            self.lib.born_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def launches(self) -> int:
        return int(self.lib.born_kernel_launches(self.h))

    @property
    def stream(self) -> int:
        return int(self.lib.born_stream(self.h) or 0)

    def set_tiling(self, cfg: int = -1, zseg: int = 0):
        self.check(self.lib.born_set_tiling(self.h, cfg, zseg))

    def set_launch_overlap(self, enable: bool = True):
        """Programmatic dependent launch of the time steps (default on)."""
        self.check(self.lib.born_set_launch_overlap(self.h, int(enable)))

    def set_host_prewarm(self, enable: bool = True):
        """Warm the closing host copies during the loops (default on)."""
        self.check(self.lib.born_set_host_prewarm(self.h, int(enable)))

    def autotune(self, enable: bool = True):
        self.check(self.lib.born_autotune(self.h, int(enable)))

    STORAGE = {"f32": 0, "bf16": 1, "f16": 2, "f32fma": 3, "f32exact": 4}

    def set_storage(self, storage: str = "f32"):
        """Storage of the wavefield levels: "f32" (reference operation
        order), "f32exact" (as "f32", with the rtm forward loop's Born
        coupling formed exactly as the reference's double expression),
        "f32fma" (FP32 levels, fused multiply-add stencil), "bf16" or "f16"
        (16-bit values with a power-of-two scale per level, FP32
        arithmetic)."""
        self.check(self.lib.born_set_storage(self.h, self.STORAGE[storage]))

    @property
    def storage(self) -> str:
        k = int(self.lib.born_get_storage(self.h))
        return {v: n for n, v in self.STORAGE.items()}[k]

    def tuned_config(self, mode: int):
        cfg, ms = C.c_int(), C.c_float()
        self.check(self.lib.born_tuned_config(self.h, mode, C.byref(cfg),
                                              C.byref(ms)))
        return cfg.value, ms.value

    def tuned_zseg(self, mode: int) -> int:
        """z-segment depth (planes per CTA) a step of `mode` uses now."""
        z = int(self.lib.born_tuned_zseg(self.h, mode))
        self.check(min(z, 0))
        return z

    def loop_tile_ms(self, mode: int):
        """ms per launch of every tile configuration (with its best z
        segmentation) as the last complete in-loop refinement of `mode`
        measured it (0.0: not measured)."""
        n = int(self.lib.born_tile_config_count())
        out = (C.c_float * n)()
        self.check(self.lib.born_loop_tile_ms(self.h, mode, out, n))
        return [float(v) for v in out]

    def synchronize(self):
        self.check(self.lib.born_synchronize(self.h))


class Gb300Prop(Handle):
    """GPU propagator with the baseProp interface (base/base_prop.h:4-72).

    Semantics follow the reference CPU propagator ``cpuProp``
    (``base/cpu_prop.cc``): the receiver array given to
    ``transferReceiverFunc`` is retained and ``rtmForward`` accumulates the
    modelled traces into it; ``sourceProp`` leaves the final two levels in
    ``p0``/``p1`` (and on the device); ``rtmAdjoint`` accumulates into
    ``img``.  Device state persists between calls, as in ``gpuProp``.
    """

    def __init__(self, device: int = 0):
        super().__init__(device)
        self._rec = None
        self._src_arrays = (None, None)
        self.shape = None

    def setNtblock(self, nb: int):  # base_prop.h:10-13
        pass

    def createSpace(self, d1, d2, d3, bc_a, bc_b, bc_y, nx, ny, nz):
        self.check(self.lib.born_create_space(self.h, d1, d2, d3, bc_a, bc_b,
                                              bc_y, nx, ny, nz))
        self.shape = (nz, ny, nx)

    def transferSincTableS(self, nsinc, jts, table):
        t = f32(np.asarray(table).reshape(-1))
        self.check(self.lib.born_set_sinc_table(self.h, 0, nsinc, jts,
                                                fptr(t)))

    def transferSincTableD(self, nsinc, jtd, table):
        t = f32(np.asarray(table).reshape(-1))
        self.check(self.lib.born_set_sinc_table(self.h, 1, nsinc, jtd,
                                                fptr(t)))

    def transferSourceFunc(self, npts, nt_big, locs, vals):
        l = np.ascontiguousarray(locs, np.int32)
        v = f32(vals)
        self.check(self.lib.born_set_source_func(self.h, npts, nt_big, iptr(l),
                                                 fptr(v)))

    def transferVelFunc1(self, nx, ny, nz, vloc):
        self.check(self.lib.born_set_velocity(self.h, 1, nx, ny, nz,
                                              fptr(f32(vloc))))

    def transferVelFunc2(self, nx, ny, nz, vloc):
        self.check(self.lib.born_set_velocity(self.h, 2, nx, ny, nz,
                                              fptr(f32(vloc))))

    def transferReceiverFunc(self, nx, ny, nt, locs, rec):
        l = np.ascontiguousarray(locs, np.int32)
        assert rec.dtype == np.float32 and rec.flags.c_contiguous
        self._rec = rec
        self._rec_nx, self._rec_ny, self._rec_nt = nx, ny, nt
        self._rec_locs = l
        self.check(self.lib.born_set_receiver_func(self.h, nx, ny, nt, iptr(l),
                                                   fptr(rec)))

    def sourceProp(self, nx, ny, nz, damp, getLast, p0, p1, jts, npts, nt):
        """The final levels are written into p0/p1 whatever getLast says, as
        cpuProp does (cpu_prop.cc:106-129), and kept on the device."""
        out0 = fptr(p0) if p0 is not None else None
        out1 = fptr(p1) if p1 is not None else None
        self.check(self.lib.born_source_prop(self.h, jts, nt, out0, out1))
        self._src_arrays = (p0, p1)

    HOST_LEVELS = {"resident": 0, "verify": 1, "upload": 2}

    def set_host_levels(self, policy: str = "resident"):
        """How rtmAdjoint reads its source-level arrays: "resident" (the
        arrays sourceProp filled select the device-resident levels, their
        contents unread), "verify" (the same, unless a checksum shows the
        arrays changed since sourceProp wrote them) or "upload" (always
        read, as cpuProp does)."""
        self.check(self.lib.born_set_host_levels(self.h,
                                                 self.HOST_LEVELS[policy]))

    def rtmAdjoint(self, n1, n2, n3, jtd, p0, p1, img, npts_s, nt):
        # the arrays must keep their addresses for the pointer comparison
        assert p0.dtype == np.float32 and p0.flags.c_contiguous
        assert p1.dtype == np.float32 and p1.flags.c_contiguous
        self.check(self.lib.born_rtm_adjoint_host(self.h, jtd, nt, fptr(p0),
                                                  fptr(p1), fptr(img)))
        self._src_arrays = (p0, p1)

    def rtmForward(self, n1, n2, n3, jt, img, rec, npts, nt, nt_big, rec_nx,
                   rec_ny):
        self.check(self.lib.born_set_reflectivity(self.h, fptr(f32(img))))
        target = self._rec if self._rec is not None else rec
        self.check(self.lib.born_rtm_forward(self.h, jt, nt, fptr(target)))
        if rec is not None and target is not rec:
            rec[...] = target

    def make_velocity(self, slot, vel, vo, vd, vmax, seed, nrand, dt, o, d):
        """vel_fd_3d::rand_subspace on the device (counter-based draws)."""
        vel = f32(vel)
        vn3, vn2, vn1 = vel.shape
        self.check(self.lib.born_make_velocity(
            self.h, slot, fptr(vel), vn1, vn2, vn3, vo[0], vo[1], vo[2],
            vd[0], vd[1], vd[2], vmax, seed, nrand[0], nrand[1], nrand[2], dt,
            o[0], o[1], o[2], d[0], d[1], d[2]))

    def get_velocity(self, slot):
        out = np.empty(self.shape, np.float32)
        self.check(self.lib.born_get_velocity(self.h, slot, fptr(out)))
        return out

    # ---- device-resident variants (no host round trips) ----
    def source_prop_device(self, jts, nt):
        self.check(self.lib.born_source_prop(self.h, jts, nt, None, None))

    def rtm_adjoint_device(self, jtd, nt, swap=1):
        self.check(self.lib.born_rtm_adjoint(self.h, jtd, nt, swap, None))

    def rtm_forward_device(self, jt, nt):
        self.check(self.lib.born_rtm_forward(self.h, jt, nt, None))

    # ---- nonlinear modelling and the exact linearised Born pair ----
    def set_traces(self, traces):
        """Replace the device traces (same receivers, same nt)."""
        self.transferReceiverFunc(self._rec_nx, self._rec_ny, self._rec_nt,
                                  self._rec_locs, f32(traces))

    def model(self, jt, nt):
        """Nonlinear modelling through vel2; returns the traces."""
        out = np.zeros_like(self._rec)
        self.zero_traces()
        self.check(self.lib.born_model(self.h, jt, nt, fptr(out)))
        return out

    def lin_forward(self, jt, nt, m):
        """Exact linearised Born forward along m (perturbation of vel2)."""
        self.check(self.lib.born_set_reflectivity(self.h, fptr(f32(m))))
        out = np.zeros_like(self._rec)
        self.zero_traces()
        self.check(self.lib.born_lin_forward(self.h, jt, nt, fptr(out)))
        return out

    def lin_adjoint(self, jt, nt, traces, interval=50):
        """Exact adjoint of lin_forward applied to traces."""
        self.set_traces(traces)
        out = np.zeros(self.shape, np.float32)
        self.check(self.lib.born_lin_adjoint(self.h, jt, nt, interval,
                                             fptr(out)))
        return out

    def lin_adjoint_device(self, jt, nt, interval=50):
        """born_lin_adjoint on the device traces, result left in the device
        image (no host copy)."""
        self.check(self.lib.born_lin_adjoint(self.h, jt, nt, interval, None))

    def lin_forward_device(self, jt, nt):
        """born_lin_forward along the device reflectivity, traces left on
        the device (accumulated onto the current device traces)."""
        self.check(self.lib.born_lin_forward(self.h, jt, nt, None))

    def set_checkpoint_storage(self, storage="f32"):
        """Storage of the exact adjoint's checkpoints: "f32" or "f16" (one
        power-of-two scale per level)."""
        self.check(self.lib.born_set_checkpoint_storage(
            self.h, {"f32": 0, "f16": 1}[storage]))

    def time_phases(self, enable=True):
        self.check(self.lib.born_time_phases(self.h, int(enable)))

    def phase_times(self):
        """ms of the last born_lin_adjoint's phases: forward sweep,
        recompute, reverse adjoint steps, division."""
        out = (C.c_float * 4)()
        self.check(self.lib.born_phase_times(self.h, out, 4))
        return [float(v) for v in out]

    def get_image(self):
        out = np.empty(self.shape, np.float32)
        self.check(self.lib.born_get_image(self.h, fptr(out)))
        return out

    def image_tensor(self):
        """The device image as a torch tensor without a copy (shape
        ``self.shape``, float32, on this handle's device).  It aliases the
        handle's buffer: synchronize the handle before reading it on another
        stream, and do not keep it past the next createSpace."""
        import torch
        ptr = self.lib.born_image_device(self.h)
        if not ptr:
            raise BornError(-4, "no grid (createSpace first)")

        class _View:  # __cuda_array_interface__ (version 3) of the buffer
            __cuda_array_interface__ = {
                "shape": tuple(self.shape), "typestr": "<f4",
                "data": (int(ptr), False), "version": 3, "strides": None,
                "stream": None}
        return torch.as_tensor(_View(), device=f"cuda:{self.device}")

    def get_traces(self, like):
        out = np.empty_like(like, dtype=np.float32)
        self.check(self.lib.born_get_traces(self.h, fptr(out)))
        return out

    def zero_traces(self):
        self.check(self.lib.born_zero_traces(self.h))


# ---------------------------------------------------------------------------
# Stacking images across ranks

def stream_mix_gbs(reads: int, writes: int, n: int, reps: int = 20) -> float:
    """GB/s that plain float4 streaming sustains over `reads` input and
    `writes` output arrays of n floats on the current device (the ceiling of
    a step kernel's mix of arrays)."""
    out = C.c_float()
    rc = lib().born_stream_mix_gbs(reads, writes, n, reps, C.byref(out))
    if rc != BORN_OK:
        raise BornError(rc, "born_stream_mix_gbs failed")
    return out.value


def stack_tensor(t, group=None):
    """Sums a tensor over the ranks of ``torch.distributed`` in place (NCCL
    for CUDA tensors, gloo for CPU ones); a no-op without a process group or
    with one rank.  Shots are independent, so this sum is the only exchange
    a multi-GPU RTM needs: each rank migrates its own shots and the image is
    the sum of theirs (the reference sums shot images on the host,
    util/Add)."""
    import torch
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized() and \
            dist.get_world_size(group) > 1:
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
        if t.is_cuda:  # the buffer may be reused on another stream next
            torch.cuda.current_stream(t.device).synchronize()
    return t


def stack_image(prop, group=None):
    """The RTM image of ``prop`` (a Gb300Prop after rtm_adjoint) summed over
    the ranks, on the device, without a host copy; returns the tensor view of
    the handle's image buffer, which then holds the stacked image."""
    prop.synchronize()
    return stack_tensor(prop.image_tensor(), group)


# ---------------------------------------------------------------------------
# Batched shots

class Batch:
    """Several set-up shots (Gb300Prop) advanced together: one launch per
    time step for all shots, each time loop recorded once into a CUDA graph
    (``graph=False`` launches step by step).  Results stay in the shots."""

    def __init__(self, shots, graph: bool = True):
        self.lib = lib()
        self.shots = list(shots)  # keeps the handles alive
        arr = (_vp * len(self.shots))(*[s.h for s in self.shots])
        b = _vp()
        rc = self.lib.born_batch_create(arr, len(self.shots), C.byref(b))
        if rc != BORN_OK:
            raise BornError(rc, "born_batch_create failed")
        self.b = b
        self.check(self.lib.born_batch_set_graph(b, int(graph)))

    def check(self, rc):
        if rc != BORN_OK:
            msg = self.lib.born_batch_error(self.b)
            raise BornError(rc, msg.decode() if msg else "")

    def close(self):
        if getattr(self, "b", None):
            self.lib.born_batch_destroy(self.b)
            self.b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self) -> int:
        return int(self.lib.born_batch_stream(self.b) or 0)

    @property
    def launches(self) -> int:
        return int(self.lib.born_batch_launches(self.b))

    @property
    def graph_launches(self) -> int:
        return int(self.lib.born_batch_graph_launches(self.b))

    def source_prop(self, jts, nt):
        self.check(self.lib.born_batch_source_prop(self.b, jts, nt))

    def rtm_adjoint(self, jtd, nt):
        self.check(self.lib.born_batch_rtm_adjoint(self.b, jtd, nt))

    def rtm_forward(self, jt, nt):
        self.check(self.lib.born_batch_rtm_forward(self.b, jt, nt))

    def synchronize(self):
        self.check(self.lib.born_batch_synchronize(self.b))


# ---------------------------------------------------------------------------
# Born operator (rtm_zero_op behind the my_operator contract) and CG

class OpParams(C.Structure):
    _fields_ = [("n1", C.c_int), ("n2", C.c_int), ("n3", C.c_int),
                ("o1", C.c_float), ("o2", C.c_float), ("o3", C.c_float),
                ("d1", C.c_float), ("d2", C.c_float), ("d3", C.c_float),
                ("nt_data", C.c_int), ("dt_data", C.c_float),
                ("rec_nx", C.c_int), ("rec_ny", C.c_int),
                ("rec_ox", C.c_float), ("rec_dx", C.c_float),
                ("rec_oy", C.c_float), ("rec_dy", C.c_float),
                ("rec_depth", C.c_float), ("nshots", C.c_int),
                ("nt_wavelet", C.c_int), ("dt_wavelet", C.c_float),
                ("nbound", C.c_int), ("exact", C.c_int),
                ("ckpt_interval", C.c_int)]


class BornOperator(Handle):
    """rtm_zero_op (base/rtm_zero_op_3d.cc) with the my_operator contract
    forward/adjoint(add, model, data) (base/my_operator.h:18-25).

    model / data are CUDA tensors (float32, contiguous) on this handle's
    device: model [n3, n2, n1], data [nshots, rec_ny, rec_nx, nt_data].
    ``exact=True`` selects the exact linearised pair (adjoint = transpose).
    """

    def __init__(self, velocity, o, d, shots, wavelet, dt_wavelet, nt_data,
                 dt_data, rec_n, rec_o, rec_d, rec_depth, nbound,
                 exact=False, ckpt_interval=50, device=0):
        super().__init__(device)
        vel = f32(velocity)
        n3, n2, n1 = vel.shape
        shots = f32(shots).reshape(-1, 3)
        wav = f32(wavelet)
        self.params = OpParams(n1, n2, n3, o[0], o[1], o[2], d[0], d[1], d[2],
                               nt_data, dt_data, rec_n[0], rec_n[1],
                               rec_o[0], rec_d[0], rec_o[1], rec_d[1],
                               rec_depth, shots.shape[0], wav.size,
                               dt_wavelet, nbound, int(exact), ckpt_interval)
        op = _vp()
        self.check(self.lib.born_op_create(self.h, C.byref(self.params),
                                           fptr(vel), fptr(shots), fptr(wav),
                                           C.byref(op)))
        self.op = op
        mn, dn = C.c_longlong(), C.c_longlong()
        nt, dt = C.c_int(), C.c_float()
        self.check(self.lib.born_op_sizes(op, C.byref(mn), C.byref(dn),
                                          C.byref(nt), C.byref(dt)))
        self.model_shape = (n3, n2, n1)
        self.data_shape = (shots.shape[0], rec_n[1], rec_n[0], nt_data)
        self.nt_fd, self.dt_fd = nt.value, dt.value

    def close(self):
        if getattr(self, "op", None):
            self.lib.born_op_destroy(self.op)
            self.op = None
        super().close()

    @staticmethod
    def _dev(t, shape):
        assert t.is_cuda and t.dtype.itemsize == 4 and t.is_contiguous()
        assert tuple(t.shape) == tuple(shape), (t.shape, shape)
        return C.c_void_p(t.data_ptr())

    def _ordered(self, fn):
        """Runs fn (which queues work on the handle's own stream) between
        two cross-stream waits: the handle's stream first waits for what
        torch's current stream has queued (the tensors passed in may still
        be being written there), and torch's current stream then waits for
        the handle's work (so a tensor written here is complete for whatever
        torch runs next).  Neither side blocks the host."""
        import torch
        cur = torch.cuda.current_stream(self.device)
        own = torch.cuda.ExternalStream(self.stream, device=self.device)
        own.wait_stream(cur)
        try:
            return fn()
        finally:
            cur.wait_stream(own)

    def forward(self, add, model, data):
        m = self._dev(model, self.model_shape)
        d = self._dev(data, self.data_shape)
        self._ordered(lambda: self.check(self.lib.born_op_forward(
            self.op, int(add), m, d)))
        return True

    def adjoint(self, add, model, data):
        m = self._dev(model, self.model_shape)
        d = self._dev(data, self.data_shape)
        self._ordered(lambda: self.check(self.lib.born_op_adjoint(
            self.op, int(add), m, d)))
        return True

    def dot(self, a, b):
        assert a.is_cuda and b.is_cuda and a.numel() == b.numel()
        out = C.c_double()
        self._ordered(lambda: self.check(self.lib.born_dot_f64(
            self.op, C.c_void_p(a.data_ptr()), C.c_void_p(b.data_ptr()),
            a.numel(), C.byref(out))))
        return out.value

    @property
    def checkpoint_shots(self) -> int:
        """Shots whose background checkpoints the operator keeps (exact)."""
        return int(self.lib.born_op_checkpoint_shots(self.op))

    @property
    def checkpoints_reused(self) -> int:
        """Shot adjoints that reused kept checkpoints instead of a sweep."""
        return int(self.lib.born_op_checkpoints_reused(self.op))

    def cg(self, data, model, niter):
        """Least squares by cgstep CG; model is updated in place."""
        res = (C.c_double * (niter + 1))()
        d = self._dev(data, self.data_shape)
        m = self._dev(model, self.model_shape)
        self._ordered(lambda: self.check(self.lib.born_cg_solve(
            self.op, d, m, niter, res)))
        return list(res)


# ---------------------------------------------------------------------------
# host geometry (csrc/born_host.h)

def _ck(rc):
    if rc != BORN_OK:
        raise BornError(rc, "host geometry call failed")


def sinc_table(ntab: int, nsinc: int = 8) -> np.ndarray:
    out = np.zeros((ntab, nsinc), np.float32)
    _ck(lib().born_sinc_table(ntab, nsinc, fptr(out)))
    return out


def calc_stability(vmax, dmin, dt_data, nt_data):
    nt = C.c_int(0)
    dt = lib().born_calc_stability(vmax, dmin, dt_data, nt_data, C.byref(nt))
    return float(dt), int(nt.value)


def compute_size(n_model, nbound, fat=4):
    return int(lib().born_compute_size(n_model, nbound, fat))


def source_geometry(sx, sy, sz, o, d, n1, n2, wavelet, nts):
    locs = np.zeros(9, np.int32)
    vals = np.zeros((9, nts), np.float32)
    w = f32(wavelet)
    _ck(lib().born_source_geometry(sx, sy, sz, o[0], o[1], o[2], d[0], d[1],
                                   d[2], n1, n2, fptr(w), w.size, nts,
                                   iptr(locs), fptr(vals)))
    return locs, vals


def wavelet_deriv(raw, dt):
    raw = f32(raw)
    out = np.zeros_like(raw)
    _ck(lib().born_wavelet_deriv(fptr(raw), raw.size, dt, fptr(out)))
    return out


def receiver_geometry(rec_nx, rec_ny, rx0, rdx, ry0, rdy, rz, o, d, n1, n2):
    locs = np.zeros(rec_nx * rec_ny, np.int32)
    _ck(lib().born_receiver_geometry(rec_nx, rec_ny, rx0, rdx, ry0, rdy, rz,
                                     o[0], o[1], o[2], d[0], d[1], d[2], n1,
                                     n2, iptr(locs)))
    return locs


def extract_sub(whole, shape, offsets):
    """Window of ``shape`` (n3, n2, n1) cut from the model-grid array
    ``whole`` starting at sample ``offsets`` (f1, f2, f3) of its axes 1..3
    (image_rtm_3d.cc:53-95); cells outside ``whole`` are zero."""
    whole = f32(whole)
    w3, w2, w1 = whole.shape
    s3, s2, s1 = shape
    out = np.zeros(shape, np.float32)
    _ck(lib().born_extract_sub(fptr(whole), w1, w2, w3, fptr(out), s1, s2, s3,
                               offsets[0], offsets[1], offsets[2]))
    return out


def laplac_forward(m):
    """The reference's laplac forward, a first difference along z
    (laplac_3d.cc:51-105)."""
    m = f32(m)
    n3, n2, n1 = m.shape
    out = np.zeros_like(m)
    _ck(lib().born_laplac_forward(0, fptr(m), fptr(out), n1, n2, n3))
    return out


def rand_subspace(vel, vo, vd, vmax, irand, nrand, dt, shape, o, d):
    """vel: model velocity [vn3][vn2][vn1]; shape (n3, n2, n1) compute grid."""
    vel = f32(vel)
    vn3, vn2, vn1 = vel.shape
    n3, n2, n1 = shape
    out = np.zeros(shape, np.float32)
    _ck(lib().born_rand_subspace(fptr(vel), vn1, vn2, vn3, vo[0], vo[1], vo[2],
                                 vd[0], vd[1], vd[2], vmax, irand, nrand[0],
                                 nrand[1], nrand[2], dt, n1, n2, n3, o[0],
                                 o[1], o[2], d[0], d[1], d[2], fptr(out)))
    return out


# ---------------------------------------------------------------------------
# SEP regular files (csrc/born_sepio.cc)

class SepInfo(C.Structure):
    _fields_ = [("ndim", C.c_int), ("n", C.c_longlong * 6),
                ("o", C.c_float * 6), ("d", C.c_float * 6),
                ("big_endian", C.c_int), ("in_", C.c_char * 1024)]


def read_sep(path: str):
    """Reads a SEP regular file; returns (array, o, d).  The array has the
    header's axes reversed (n1 fastest), e.g. [n3, n2, n1] for a cube."""
    info = SepInfo()
    _ck(lib().born_sep_read_info(path.encode(), C.byref(info)))
    shape = tuple(int(info.n[a]) for a in range(max(info.ndim, 1)))
    out = np.empty(int(np.prod(shape)), np.float32)
    _ck(lib().born_sep_read(path.encode(), fptr(out), out.size))
    k = max(info.ndim, 1)
    return (out.reshape(shape[::-1]), tuple(info.o[:k]), tuple(info.d[:k]))


def write_sep(path: str, array, o=None, d=None, big_endian: bool = True):
    """Writes a SEP regular file (path and path + '@'); axis 1 is the
    array's last (fastest) axis."""
    a = f32(array)
    shape = a.shape[::-1]
    info = SepInfo()
    info.ndim = len(shape)
    for i, n in enumerate(shape):
        info.n[i] = n
        info.o[i] = 0.0 if o is None else o[i]
        info.d[i] = 1.0 if d is None else d[i]
    _ck(lib().born_sep_write(path.encode(), C.byref(info), fptr(a),
                             int(big_endian)))


def read_regfile(path: str):
    """Reads a SEP or JSON regular file (by name: ".json" is JSON); returns
    (array, o, d) with the axes reversed (n1 fastest)."""
    info = SepInfo()
    _ck(lib().born_regfile_read_info(path.encode(), C.byref(info)))
    k = max(info.ndim, 1)
    shape = tuple(int(info.n[a]) for a in range(k))
    out = np.empty(int(np.prod(shape)), np.float32)
    _ck(lib().born_regfile_read(path.encode(), fptr(out), out.size))
    return out.reshape(shape[::-1]), tuple(info.o[:k]), tuple(info.d[:k])


def write_regfile(path: str, array, o=None, d=None):
    """Writes a SEP (big-endian data in path + '@') or, for names ending in
    '.json', a JSON regular file (host-order data in path + '.dat')."""
    a = f32(array)
    shape = a.shape[::-1]
    info = SepInfo()
    info.ndim = len(shape)
    for i, n in enumerate(shape):
        info.n[i] = n
        info.o[i] = 0.0 if o is None else o[i]
        info.d[i] = 1.0 if d is None else d[i]
    _ck(lib().born_regfile_write(path.encode(), C.byref(info), fptr(a)))


def add_regfiles(in1: str, in2: str, out: str):
    """util/Add: out = in1 + in2 (regular files of the same size)."""
    _ck(lib().born_add_regfiles(in1.encode(), in2.encode(), out.encode()))
