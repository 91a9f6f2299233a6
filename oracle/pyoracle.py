"""ctypes front end of the CPU oracle — TEST INFRASTRUCTURE ONLY.

Loads two checkers built by ``oracle/Makefile``:

* ``PortProp`` / ``PortProp64``: the C restatement of the reference's
  ``cpuProp`` (``base/cpu_prop.cc``) in float (parity) and double (accuracy).
* ``RefProp``: the reference's own ``cpuProp`` compiled from its sources into
  ``oracle/_ref`` (only where the reference sources are present).

Both mirror the ``baseProp`` call sequence (``base/base_prop.h:4-72``):
createSpace -> transferSincTableS/D -> transferSourceFunc -> transferVelFunc1/2
-> transferReceiverFunc -> sourceProp / rtmAdjoint / rtmForward.  Only tests,
``__graft_entry__.smoke`` and the CPU-baseline leg of ``bench.py`` use this
module; the product never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libref_cpuprop.so")
# The reference checkout (its base/ folder holds cpu_prop.cc and the
# geometry sources) comes from the environment; unset, only libraries built
# earlier into _ref/ are used.
REF_SRC = os.environ.get("SC17_BORN_REF") or None

_fp = C.POINTER(C.c_float)
_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


def build_port(force: bool = False) -> str:
    # make rebuilds only what is older than its sources
    subprocess.run(["make", "-s", "-C", HERE, "port"] + (["-B"] if force
                                                          else []),
                   check=True)
    return PORT_SO


def build_ref(force: bool = False) -> str | None:
    """Compile the reference CPU path when its sources are present here."""
    if not REF_SRC or not os.path.isdir(os.path.join(REF_SRC, "base")):
        return REF_SO if os.path.exists(REF_SO) else None
    # make rebuilds only what is older than its sources
    subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={REF_SRC}"] +
                   (["-B"] if force else []), check=True)
    return REF_SO


def ref_program(name: str) -> str | None:
    """A program of oracle/_ref built on the reference's own sources (see
    the Makefile), or None where it was never built."""
    build_ref()
    path = os.path.join(HERE, "_ref", name)
    return path if os.path.exists(path) else None


REF_GEOM_SO = os.path.join(HERE, "_ref", "libref_geom.so")
_ref_geom = None


def ref_geom_lib():
    """The reference's own geometry and glue code (vel_fd_3d::rand_subspace,
    set_compute_size, the wavelet reader and source points, map_data,
    laplac, deriv), compiled from its sources with oracle/ref_geom_shim.cc,
    or None where the sources are absent."""
    global _ref_geom
    if _ref_geom is None:
        if REF_SRC and os.path.isdir(os.path.join(REF_SRC, "base")):
            subprocess.run(["make", "-s", "-C", HERE, "_ref/libref_geom.so",
                            f"REF={REF_SRC}"], check=True)
        if not os.path.exists(REF_GEOM_SO):
            return None
        lib = C.CDLL(REF_GEOM_SO)
        i, f = C.c_int, C.c_float
        sig = {
            "ref_geom_compute_size": (i, [i, i, i]),
            "ref_geom_rand_subspace": (i, [_fp, i, i, i] + [f] * 6 +
                                       [i, i, i, i, f, i, i, i] + [f] * 6 +
                                       [_fp]),
            "ref_geom_source": (i, [_fp, i, f, f, f, f] + [f] * 6 +
                                [i, i, i, i, _ip, _fp]),
            "ref_geom_map_locs": (i, [i, _fp, _fp, _fp, i, i, _ip]),
            "ref_geom_receivers": (i, [i, i] + [f] * 11 + [i, i, i, i, _ip]),
            "ref_geom_calc_stability": (i, [_fp, i, i, i, f, f, f, f, i, _fp,
                                            _ip]),
            "ref_geom_map_data": (i, [i, i, _fp, _fp, i, i, i, i]),
            "ref_geom_laplac": (i, [i, i, _fp, _fp, i, i, i]),
            "ref_geom_deriv": (i, [i, i, _fp, _fp, i, i, i, f]),
            "ref_geom_image_window": (i, [i, _fp, i, i, i] + [f] * 6 +
                                      [_fp, i, i, i] + [f] * 6),
        }
        for name, (res, args) in sig.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _ref_geom = lib
    return _ref_geom


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def fptr(a: np.ndarray):
    assert a.dtype == np.float32 and a.flags.c_contiguous
    return a.ctypes.data_as(_fp)


def dptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def iptr(a: np.ndarray):
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(_ip)


class _PropF(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("n123", C.c_longlong),
        ("coeffs", C.c_float * 13), ("bound", C.c_float * 40),
        ("nsinc_s", C.c_int), ("jt_s", C.c_int), ("table_s", _fp),
        ("nsinc_d", C.c_int), ("jt_d", C.c_int), ("table_d", _fp),
        ("npts_s", C.c_int), ("nt_src", C.c_int), ("locs_s", _ip),
        ("source", _fp),
        ("nrec", C.c_int), ("nt_rec", C.c_int), ("locs_r", _ip), ("rec", _fp),
        ("vel1", _fp), ("vel2", _fp),
        ("dir", C.c_int), ("jt", C.c_int),
    ]


class _PropD(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("n123", C.c_longlong),
        ("coeffs", C.c_double * 13), ("bound", C.c_double * 40),
        ("nsinc_s", C.c_int), ("jt_s", C.c_int), ("table_s", _dp),
        ("nsinc_d", C.c_int), ("jt_d", C.c_int), ("table_d", _dp),
        ("npts_s", C.c_int), ("nt_src", C.c_int), ("locs_s", _ip),
        ("source", _dp),
        ("nrec", C.c_int), ("nt_rec", C.c_int), ("locs_r", _ip), ("rec", _dp),
        ("vel1", _dp), ("vel2", _dp),
        ("dir", C.c_int), ("jt", C.c_int),
    ]


_port_lib = None


def port_lib():
    global _port_lib
    if _port_lib is None:
        lib = C.CDLL(build_port())
        P, PD = C.POINTER(_PropF), C.POINTER(_PropD)
        sig = {
            "oracle_create_space": (None, [P, C.c_float, C.c_float, C.c_float,
                                           C.c_int, C.c_int, C.c_int]),
            "oracle_create_space_d": (None, [PD, C.c_float, C.c_float,
                                             C.c_float, C.c_int, C.c_int,
                                             C.c_int]),
            "oracle_num_threads": (C.c_int, []),
            "oracle_set_num_threads": (None, [C.c_int]),
            "oracle_prop_stepf": (None, [P, _fp, _fp, _fp]),
            "oracle_dampf": (None, [P, _fp, _fp]),
            "oracle_image_addf": (None, [P, _fp, _fp, _fp]),
            "oracle_image_conditionf": (None, [P, _fp, _fp, _fp]),
            "oracle_source_propf": (None, [P, _fp, _fp, C.c_int, C.c_int]),
            "oracle_rtm_adjointf": (None, [P, _fp, _fp, _fp, C.c_int,
                                           C.c_int]),
            "oracle_rtm_forwardf": (None, [P, C.c_int, _fp, _fp, C.c_int]),
            "oracle_source_propd": (None, [PD, _dp, _dp, C.c_int, C.c_int]),
            "oracle_rtm_adjointd": (None, [PD, _dp, _dp, _dp, C.c_int,
                                           C.c_int]),
            "oracle_rtm_forwardd": (None, [PD, C.c_int, _dp, _dp, C.c_int]),
            "oracle_modelf": (None, [P, C.c_int, _fp, C.c_int]),
            "oracle_lin_forwardf": (None, [P, C.c_int, _fp, _fp, C.c_int]),
            "oracle_modeld": (None, [PD, C.c_int, _dp, C.c_int]),
            "oracle_lin_forwardd": (None, [PD, C.c_int, _dp, _dp, C.c_int]),
            "oracle_lin_adjointf": (None, [P, C.c_int, _fp, _fp, C.c_int]),
            "oracle_lin_adjointd": (None, [PD, C.c_int, _dp, _dp, C.c_int]),
            "oracle_sinc_table": (None, [C.c_int, C.c_int, _fp]),
            "oracle_calc_stability": (C.c_float, [C.c_float, C.c_float,
                                                  C.c_float, C.c_int, _ip]),
            "oracle_compute_size": (C.c_int, [C.c_int, C.c_int, C.c_int]),
            "oracle_source_geometry": (None, [C.c_float] * 9 + [
                C.c_int, C.c_int, _fp, C.c_int, C.c_int, _ip, _fp]),
            "oracle_wavelet_deriv": (None, [_fp, C.c_int, C.c_float, _fp]),
            "oracle_receiver_geometry": (None, [C.c_int, C.c_int] +
                                         [C.c_float] * 11 +
                                         [C.c_int, C.c_int, _ip]),
            "oracle_rand_subspace": (None, [_fp, C.c_int, C.c_int, C.c_int] +
                                     [C.c_float] * 7 + [C.c_int] * 4 +
                                     [C.c_float] + [C.c_int] * 3 +
                                     [C.c_float] * 6 + [_fp]),
            "oracle_laplac_forward": (None, [C.c_int, _fp, _fp, C.c_int,
                                             C.c_int, C.c_int]),
            "oracle_laplac_adjoint": (None, [C.c_int, _fp, _fp, C.c_int,
                                             C.c_int, C.c_int]),
            "oracle_deriv_forward": (None, [C.c_int, _fp, _fp, C.c_int,
                                            C.c_int, C.c_int, C.c_float]),
            "oracle_deriv_adjoint": (None, [C.c_int, _fp, _fp, C.c_int,
                                            C.c_int, C.c_int, C.c_float]),
            "oracle_map_data_forward": (None, [C.c_int, _fp, _fp, C.c_int,
                                               C.c_int, C.c_int, C.c_int]),
            "oracle_map_data_adjoint": (None, [C.c_int, _fp, _fp, C.c_int,
                                               C.c_int, C.c_int, C.c_int]),
            "oracle_extract_sub": (None, [_fp, C.c_int, C.c_int, C.c_int, _fp,
                                          C.c_int, C.c_int, C.c_int, C.c_int,
                                          C.c_int, C.c_int]),
            "oracle_add_image": (None, [_fp, C.c_int, C.c_int, C.c_int, _fp,
                                        C.c_int, C.c_int, C.c_int, C.c_int,
                                        C.c_int, C.c_int]),
            "oracle_window_offset": (C.c_int, [C.c_float] * 3),
        }
        for name, (res, args) in sig.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _port_lib = lib
    return _port_lib


_ref_lib = None


def ref_lib():
    """The reference's own cpuProp, or None where it cannot be built."""
    global _ref_lib
    if _ref_lib is None:
        path = build_ref()
        if path is None or not os.path.exists(path):
            return None
        lib = C.CDLL(path)
        v = C.c_void_p
        sig = {
            "ref_quiet": (None, [C.c_int]),
            "ref_create": (v, [C.c_float, C.c_float, C.c_float, C.c_int,
                               C.c_int, C.c_int]),
            "ref_destroy": (None, [v]),
            "ref_set_sinc_s": (None, [v, C.c_int, C.c_int, _fp]),
            "ref_set_sinc_d": (None, [v, C.c_int, C.c_int, _fp]),
            "ref_set_source": (None, [v, C.c_int, C.c_int, _ip, _fp]),
            "ref_set_vel1": (None, [v, C.c_int, C.c_int, C.c_int, _fp]),
            "ref_set_vel2": (None, [v, C.c_int, C.c_int, C.c_int, _fp]),
            "ref_set_receivers": (None, [v, C.c_int, C.c_int, C.c_int, _ip,
                                         _fp]),
            "ref_source_prop": (None, [v, C.c_int, C.c_int, C.c_int, _fp, _fp,
                                       C.c_int, C.c_int, C.c_int]),
            "ref_rtm_adjoint": (None, [v, C.c_int, C.c_int, C.c_int, C.c_int,
                                       _fp, _fp, _fp, C.c_int, C.c_int]),
            "ref_rtm_forward": (None, [v, C.c_int, C.c_int, C.c_int, C.c_int,
                                       _fp, _fp, C.c_int, C.c_int, C.c_int,
                                       C.c_int, C.c_int]),
            "ref_prop": (None, [v, _fp, _fp, _fp]),
            "ref_damp": (None, [v, _fp, _fp]),
            "ref_image_add": (None, [v, _fp, _fp, _fp]),
            "ref_image_condition": (None, [v, _fp, _fp, _fp]),
            "ref_sinc_table": (None, [C.c_int, C.c_int, _fp]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        lib.ref_quiet(1)
        _ref_lib = lib
    return _ref_lib


def set_threads(n: int) -> None:
    port_lib().oracle_set_num_threads(int(n))


def num_threads() -> int:
    return int(port_lib().oracle_num_threads())


class PortProp:
    """Float oracle with the baseProp call sequence (base/base_prop.h)."""

    dtype = np.float32

    def __init__(self):
        self.lib = port_lib()
        self.s = _PropF()
        self._keep = {}

    def _arr(self, a):
        return _f32(a)

    def _ptr(self, a):
        return fptr(a)

    def createSpace(self, d1, d2, d3, bc_a, bc_b, bc_y, nx, ny, nz):
        self.lib.oracle_create_space(C.byref(self.s), d1, d2, d3, nx, ny, nz)
        self.shape = (nz, ny, nx)

    def transferSincTableS(self, nsinc, jts, table):
        t = self._keep["ts"] = self._arr(np.asarray(table).reshape(-1))
        self.s.nsinc_s, self.s.jt_s, self.s.table_s = nsinc, jts, self._ptr(t)

    def transferSincTableD(self, nsinc, jtd, table):
        t = self._keep["td"] = self._arr(np.asarray(table).reshape(-1))
        self.s.nsinc_d, self.s.jt_d, self.s.table_d = nsinc, jtd, self._ptr(t)

    def transferSourceFunc(self, npts, nt_big, locs, vals):
        l = self._keep["ls"] = np.ascontiguousarray(locs, dtype=np.int32)
        v = self._keep["vs"] = self._arr(vals)
        self.s.npts_s, self.s.nt_src = npts, nt_big
        self.s.locs_s, self.s.source = iptr(l), self._ptr(v)

    def transferVelFunc1(self, nx, ny, nz, v):
        v = self._keep["v1"] = self._arr(v)
        self.s.vel1 = self._ptr(v)

    def transferVelFunc2(self, nx, ny, nz, v):
        v = self._keep["v2"] = self._arr(v)
        self.s.vel2 = self._ptr(v)

    def transferReceiverFunc(self, rec_nx, rec_ny, nt_big, locs, rec):
        """``rec`` is retained and written by rtmForward, as in cpuProp."""
        l = self._keep["lr"] = np.ascontiguousarray(locs, dtype=np.int32)
        assert rec.dtype == self.dtype and rec.flags.c_contiguous
        self._keep["rec"] = rec
        self.s.nrec, self.s.nt_rec = rec_nx * rec_ny, nt_big
        self.s.locs_r, self.s.rec = iptr(l), self._ptr(rec)

    def sourceProp(self, nx, ny, nz, damp, get_last, p0, p1, jts, npts, nt):
        self.lib.oracle_source_propf(C.byref(self.s), fptr(p0), fptr(p1), jts,
                                     nt)

    def rtmAdjoint(self, n1, n2, n3, jtd, p0, p1, img, npts_s, nt):
        self.lib.oracle_rtm_adjointf(C.byref(self.s), fptr(p0), fptr(p1),
                                     fptr(img), jtd, nt)

    def rtmForward(self, n1, n2, n3, jt, img, rec, npts, nt, nt_big, rec_nx,
                   rec_ny):
        self.lib.oracle_rtm_forwardf(C.byref(self.s), jt, fptr(img),
                                     fptr(rec), nt)

    def model(self, jt, rec, nt):
        """Nonlinear modelling (background of rtmForward, traces from s)."""
        self._keep["rec"] = rec
        self.lib.oracle_modelf(C.byref(self.s), jt, fptr(rec), nt)

    def lin_forward(self, jt, m, rec, nt):
        """Exact linearised Born forward along m (= perturbation of vel2)."""
        m = self._keep["m"] = self._arr(m)
        self._keep["rec"] = rec
        self.lib.oracle_lin_forwardf(C.byref(self.s), jt, fptr(m), fptr(rec),
                                     nt)

    def lin_adjoint(self, jt, rec, nt):
        """Exact adjoint of lin_forward applied to the traces rec
        ([nrec][nt_rec]); returns the model-space result (n123)."""
        rec = self._arr(rec)
        out = np.zeros(self.shape, self.dtype)
        self.lib.oracle_lin_adjointf(C.byref(self.s), jt, fptr(rec),
                                     fptr(out), nt)
        return out

    # primitives, for unit tests
    def prop(self, p0, p1, vel):
        self.lib.oracle_prop_stepf(C.byref(self.s), fptr(p0), fptr(p1),
                                   fptr(vel))

    def damp(self, p0, p1):
        self.lib.oracle_dampf(C.byref(self.s), fptr(p0), fptr(p1))


class PortProp64(PortProp):
    """Double-precision accuracy oracle (same algorithm and order)."""

    dtype = np.float64

    def __init__(self):
        self.lib = port_lib()
        self.s = _PropD()
        self._keep = {}

    def _arr(self, a):
        return np.ascontiguousarray(a, dtype=np.float64)

    def _ptr(self, a):
        return dptr(a)

    def createSpace(self, d1, d2, d3, bc_a, bc_b, bc_y, nx, ny, nz):
        self.lib.oracle_create_space_d(C.byref(self.s), d1, d2, d3, nx, ny, nz)
        self.shape = (nz, ny, nx)

    def sourceProp(self, nx, ny, nz, damp, get_last, p0, p1, jts, npts, nt):
        self.lib.oracle_source_propd(C.byref(self.s), dptr(p0), dptr(p1), jts,
                                     nt)

    def rtmAdjoint(self, n1, n2, n3, jtd, p0, p1, img, npts_s, nt):
        self.lib.oracle_rtm_adjointd(C.byref(self.s), dptr(p0), dptr(p1),
                                     dptr(img), jtd, nt)

    def rtmForward(self, n1, n2, n3, jt, img, rec, npts, nt, nt_big, rec_nx,
                   rec_ny):
        self.lib.oracle_rtm_forwardd(C.byref(self.s), jt, dptr(img),
                                     dptr(rec), nt)

    def model(self, jt, rec, nt):
        self._keep["rec"] = rec
        self.lib.oracle_modeld(C.byref(self.s), jt, dptr(rec), nt)

    def lin_forward(self, jt, m, rec, nt):
        m = self._keep["m"] = self._arr(m)
        self._keep["rec"] = rec
        self.lib.oracle_lin_forwardd(C.byref(self.s), jt, dptr(m), dptr(rec),
                                     nt)

    def lin_adjoint(self, jt, rec, nt):
        rec = self._arr(rec)
        out = np.zeros(self.shape, self.dtype)
        self.lib.oracle_lin_adjointd(C.byref(self.s), jt, dptr(rec),
                                     dptr(out), nt)
        return out


class RefProp:
    """The reference's own cpuProp (oracle/_ref), same call sequence."""

    def __init__(self):
        self.lib = ref_lib()
        if self.lib is None:
            raise RuntimeError("reference CPU path not built")
        self.h = None
        self._keep = {}

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.ref_destroy(self.h)

    def createSpace(self, d1, d2, d3, bc_a, bc_b, bc_y, nx, ny, nz):
        self.h = self.lib.ref_create(d1, d2, d3, nx, ny, nz)

    def transferSincTableS(self, nsinc, jts, table):
        t = _f32(np.asarray(table).reshape(-1))
        self.lib.ref_set_sinc_s(self.h, nsinc, jts, fptr(t))

    def transferSincTableD(self, nsinc, jtd, table):
        t = _f32(np.asarray(table).reshape(-1))
        self.lib.ref_set_sinc_d(self.h, nsinc, jtd, fptr(t))

    def transferSourceFunc(self, npts, nt_big, locs, vals):
        l = np.ascontiguousarray(locs, dtype=np.int32)
        v = self._keep["vs"] = _f32(vals)
        self.lib.ref_set_source(self.h, npts, nt_big, iptr(l), fptr(v))

    def transferVelFunc1(self, nx, ny, nz, v):
        v = self._keep["v1"] = _f32(v)
        self.lib.ref_set_vel1(self.h, nx, ny, nz, fptr(v))

    def transferVelFunc2(self, nx, ny, nz, v):
        v = self._keep["v2"] = _f32(v)
        self.lib.ref_set_vel2(self.h, nx, ny, nz, fptr(v))

    def transferReceiverFunc(self, rec_nx, rec_ny, nt_big, locs, rec):
        l = np.ascontiguousarray(locs, dtype=np.int32)
        self._keep["rec"] = rec
        self.lib.ref_set_receivers(self.h, rec_nx, rec_ny, nt_big, iptr(l),
                                   fptr(rec))

    def sourceProp(self, nx, ny, nz, damp, get_last, p0, p1, jts, npts, nt):
        self.lib.ref_source_prop(self.h, nx, ny, nz, fptr(p0), fptr(p1), jts,
                                 npts, nt)

    def rtmAdjoint(self, n1, n2, n3, jtd, p0, p1, img, npts_s, nt):
        self.lib.ref_rtm_adjoint(self.h, n1, n2, n3, jtd, fptr(p0), fptr(p1),
                                 fptr(img), npts_s, nt)

    def rtmForward(self, n1, n2, n3, jt, img, rec, npts, nt, nt_big, rec_nx,
                   rec_ny):
        self.lib.ref_rtm_forward(self.h, n1, n2, n3, jt, fptr(img), fptr(rec),
                                 npts, nt, nt_big, rec_nx, rec_ny)

    def prop(self, p0, p1, vel):
        self.lib.ref_prop(self.h, fptr(p0), fptr(p1), fptr(vel))

    def damp(self, p0, p1):
        self.lib.ref_damp(self.h, fptr(p0), fptr(p1))


def sinc_table(ntab: int, nsinc: int = 8, ref: bool = False) -> np.ndarray:
    out = np.zeros((ntab, nsinc), np.float32)
    if ref:
        ref_lib().ref_sinc_table(ntab, nsinc, fptr(out))
    else:
        port_lib().oracle_sinc_table(ntab, nsinc, fptr(out))
    return out


class Geometry:
    """The host geometry and glue of the restatement (pinned bit for bit to
    the reference's own sources) under the function names of the product's
    host-geometry module, so that the shot builder can make a case's inputs
    without the product library: calc_stability (fd_prop_3d.cc:6-33),
    compute_size (source_func_3d.cc:4-61), sinc_table (sinc_bob.cc),
    wavelet_deriv and source_geometry (source_func_3d.cc:76-127),
    receiver_geometry (data_rtm_3d.cc:59-90, map_data_3d.cc:4-35),
    rand_subspace (vel_fd_3d.cc:29-134), extract_sub (image_rtm_3d.cc:53-95)
    and laplac_forward (laplac_3d.cc:51-105)."""

    @staticmethod
    def calc_stability(vmax, dmin, dt_data, nt_data):
        nt = C.c_int(0)
        dt = port_lib().oracle_calc_stability(vmax, dmin, dt_data, nt_data,
                                              C.byref(nt))
        return float(dt), int(nt.value)

    @staticmethod
    def compute_size(n_model, nbound, fat=4):
        return int(port_lib().oracle_compute_size(n_model, nbound, fat))

    @staticmethod
    def sinc_table(ntab, nsinc=8):
        return sinc_table(ntab, nsinc)

    @staticmethod
    def wavelet_deriv(raw, dt):
        raw = _f32(raw)
        out = np.zeros_like(raw)
        port_lib().oracle_wavelet_deriv(fptr(raw), raw.size, dt, fptr(out))
        return out

    @staticmethod
    def source_geometry(sx, sy, sz, o, d, n1, n2, wavelet, nts):
        locs = np.zeros(9, np.int32)
        vals = np.zeros((9, nts), np.float32)
        w = _f32(wavelet)
        port_lib().oracle_source_geometry(sx, sy, sz, o[0], o[1], o[2], d[0],
                                          d[1], d[2], n1, n2, fptr(w), w.size,
                                          nts, iptr(locs), fptr(vals))
        return locs, vals

    @staticmethod
    def receiver_geometry(rec_nx, rec_ny, rx0, rdx, ry0, rdy, rz, o, d, n1,
                          n2):
        locs = np.zeros(rec_nx * rec_ny, np.int32)
        port_lib().oracle_receiver_geometry(rec_nx, rec_ny, rx0, rdx, ry0, rdy,
                                            rz, o[0], o[1], o[2], d[0], d[1],
                                            d[2], n1, n2, iptr(locs))
        return locs

    @staticmethod
    def rand_subspace(vel, vo, vd, vmax, irand, nrand, dt, shape, o, d):
        vel = _f32(vel)
        vn3, vn2, vn1 = vel.shape
        n3, n2, n1 = shape
        out = np.zeros(shape, np.float32)
        port_lib().oracle_rand_subspace(
            fptr(vel), vn1, vn2, vn3, vo[0], vo[1], vo[2], vd[0], vd[1], vd[2],
            vmax, irand, nrand[0], nrand[1], nrand[2], dt, n1, n2, n3, o[0],
            o[1], o[2], d[0], d[1], d[2], fptr(out))
        return out

    @staticmethod
    def extract_sub(whole, shape, offsets):
        whole = _f32(whole)
        w3, w2, w1 = whole.shape
        s3, s2, s1 = shape
        out = np.zeros(shape, np.float32)
        port_lib().oracle_extract_sub(fptr(whole), w1, w2, w3, fptr(out), s1,
                                      s2, s3, offsets[0], offsets[1],
                                      offsets[2])
        return out

    @staticmethod
    def laplac_forward(m):
        m = _f32(m)
        n3, n2, n1 = m.shape
        out = np.zeros_like(m)
        port_lib().oracle_laplac_forward(0, fptr(m), fptr(out), n1, n2, n3)
        return out


# ---------------------------------------------------------------------------
# Whole-path drivers used by tests and the CPU baseline.  ``case`` is a dict
# of propagator inputs (see tests/cases.py): velocity arrays already in
# v^2 dt^2 form, sinc tables, point locations and traces.

def run_case(prop, case: dict, which: str = "all") -> dict:
    """Run the reference call sequence of rtm_zero_op (rtm_zero_op_3d.cc:
    101-197 forward, 199-299 adjoint) on one shot's propagator inputs."""
    nz, ny, nx = case["shape"]
    dt = prop.dtype if hasattr(prop, "dtype") else np.float32
    out = {}
    prop.createSpace(case["d"], case["d"], case["d"], 50.0, 0.0005, 0.0005,
                     nx, ny, nz)
    prop.transferSincTableS(8, case["jts"], case["table_s"])
    prop.transferSincTableD(8, case["jtd"], case["table_d"])
    prop.transferSourceFunc(case["locs_s"].size, case["nt_big"],
                            case["locs_s"], case["src"])
    prop.transferVelFunc1(nx, ny, nz, case["vel1"])
    prop.transferVelFunc2(nx, ny, nz, case["vel2"])
    nt = case["nt"]
    if which == "none":
        return out
    if which in ("all", "adjoint", "source"):
        rec = np.ascontiguousarray(case["rec_in"], dtype=dt)
        prop.transferReceiverFunc(case["rec_nx"], case["rec_ny"],
                                  case["nt_big"], case["locs_r"], rec)
        p0 = np.zeros(case["shape"], dt)
        p1 = np.zeros(case["shape"], dt)
        prop.sourceProp(nx, ny, nz, False, True, p0, p1, case["jts"], 9, nt)
        out["src_p0"], out["src_p1"] = p0.copy(), p1.copy()
        if which != "source":
            img = np.zeros(case["shape"], dt)
            prop.rtmAdjoint(nx, ny, nz, case["jtd"], p1, p0, img, 9, nt)
            out["image"] = img
    if which in ("all", "forward"):
        rec = np.zeros_like(case["rec_in"], dtype=dt)
        prop.transferReceiverFunc(case["rec_nx"], case["rec_ny"],
                                  case["nt_big"], case["locs_r"], rec)
        img = np.ascontiguousarray(case["refl"], dtype=dt)
        prop.rtmForward(nx, ny, nz, case["jtd"], img, rec, 9, nt,
                        case["nt_big"], case["rec_nx"], case["rec_ny"])
        out["traces"] = rec
    return out
