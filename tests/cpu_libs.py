"""ctypes access to the CPU checkers (test infrastructure only).

OracleLib  -> oracle/liboracle.so   the C restatement of the reference algorithms
RefLib     -> oracle/_ref/libref.so the reference's own CPU code compiled from its sources

Both return the same dict layout so tests can swap them:
  DMC: v (float64, 3/vertex), n, q (int32, 4/quad), t (int32, 3/tri), he (int32, 5/halfedge), hv, hf
  TMC: v, n, t
"""
import ctypes
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_SO = os.path.join(ORACLE_DIR, "liboracle.so")
REF_SO = os.path.join(ORACLE_DIR, "_ref", "libref.so")


def build_oracle():
    subprocess.run(["make", "-s", "-C", ORACLE_DIR, "liboracle.so"], check=True)


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _vol_args(vol):
    d = np.ascontiguousarray(vol.data, dtype=np.float32)
    nx, ny, nz = vol.dims
    return d, [nx, ny, nz, (ctypes.c_double * 3)(*vol.origin), (ctypes.c_double * 3)(*vol.spacing),
               _p(d), ctypes.c_double(vol.iso)]


class _Lib:
    prefix = ""

    def _dmc_fetch(self, h):
        lib, pre = self.lib, self.prefix
        h = ctypes.c_void_p(h)
        sz = (ctypes.c_int64 * 4)()
        getattr(lib, pre + "_dmc_sizes")(h, sz)
        nv, nq, nt, nhe = list(sz)
        out = dict(v=np.zeros(3 * nv), n=np.zeros(3 * nv), q=np.zeros(4 * nq, np.int32),
                   t=np.zeros(3 * nt, np.int32), he=np.zeros(5 * nhe, np.int32),
                   hv=np.zeros(nv if nhe else 0, np.int32), hf=np.zeros(nq if nhe else 0, np.int32))
        getattr(lib, pre + "_dmc_copy")(h, _p(out["v"]), _p(out["n"]), _p(out["q"]), _p(out["t"]),
                                        _p(out["he"]), _p(out["hv"]) if nhe else None,
                                        _p(out["hf"]) if nhe else None)
        return h, out

    def _tmc_fetch(self, h):
        lib, pre = self.lib, self.prefix
        h = ctypes.c_void_p(h)
        sz = (ctypes.c_int64 * 2)()
        getattr(lib, pre + "_tmc_sizes")(h, sz)
        nv, nt = list(sz)
        out = dict(v=np.zeros(3 * nv), n=np.zeros(3 * nv), t=np.zeros(3 * nt, np.int32))
        getattr(lib, pre + "_tmc_copy")(h, _p(out["v"]), _p(out["n"]), _p(out["t"]))
        return h, out


class OracleLib(_Lib):
    prefix = "oracle"

    def __init__(self):
        if not os.path.exists(ORACLE_SO):
            build_oracle()
        self.lib = ctypes.CDLL(ORACLE_SO)
        self.lib.oracle_dmc_run.restype = ctypes.c_void_p
        self.lib.oracle_tmc_run.restype = ctypes.c_void_p

    def dmc(self, vol, simplify=0, flip=0):
        d, a = _vol_args(vol)
        h, out = self._dmc_fetch(self.lib.oracle_dmc_run(*a, int(simplify), int(flip), 0))
        self.lib.oracle_dmc_free(h)
        return out

    def dmc_front(self, vol, flip=0):
        """Front end only: vertices with their generating cell and local coordinates, quads in
        key order with their inherited colours."""
        d, a = _vol_args(vol)
        h, out = self._dmc_fetch(self.lib.oracle_dmc_run(*a, 0, int(flip), 1))
        nv, nq = out["v"].size // 3, out["q"].size // 4
        out["colors"] = np.zeros(nq, np.int32)
        out["vcell"] = np.zeros(nv, np.int64)
        out["vuvw"] = np.zeros(3 * nv, np.float32)
        self.lib.oracle_dmc_copy_front(h, _p(out["colors"]), _p(out["vcell"]), _p(out["vuvw"]))
        pf = (ctypes.c_int64 * 2)()
        self.lib.oracle_dmc_proj_fail(h, pf)
        out["proj_fail"] = np.array(list(pf))
        self.lib.oracle_dmc_free(h)
        return out

    def tmc(self, vol, key_bits=32):
        d, a = _vol_args(vol)
        h, out = self._tmc_fetch(self.lib.oracle_tmc_run(*a, int(key_bits)))
        cs = (ctypes.c_int64 * 11)()
        self.lib.oracle_tmc_cases(h, cs)
        out["cases"] = np.array(list(cs))
        self.lib.oracle_tmc_free(h)
        return out

    def tmc_connectivity(self, vol):
        """The reference's connectivity() on its t_mc mesh: (components, orientation changes)."""
        d, a = _vol_args(vol)
        out = (ctypes.c_int64 * 2)()
        self.lib.ref_tmc_connectivity(*a, out)
        return int(out[0]), int(out[1])

    def tmc_files(self, iso, volume, obj, off):
        """The reference's MarchingCubes::operator(): ushort volume file in, OBJ and OFF files out."""
        self.lib.ref_tmc_files(ctypes.c_double(iso), volume.encode(), obj.encode(), off.encode())

    def color_valence(self, nv, quads, colors):
        q = np.ascontiguousarray(quads, dtype=np.int32)
        col = np.ascontiguousarray(colors, dtype=np.int32).copy()
        val = np.zeros(nv, np.int32)
        self.lib.oracle_dmc_color_valence(int(nv), int(q.size // 4), _p(q), _p(col), _p(val))
        return col, val

    def halfedges(self, faces, P, nv):
        """Halfedges of a P-gon mesh with the reference's halfedges() rules: he (5 per halfedge:
        origin, face, next, twin, flag), hv, hf."""
        f = np.ascontiguousarray(faces, dtype=np.int32)
        nf = f.size // P
        he = np.zeros(5 * P * nf, np.int32)
        hv = np.zeros(nv, np.int32)
        hf = np.zeros(nf, np.int32)
        self.lib.oracle_halfedges.restype = ctypes.c_int64
        self.lib.oracle_halfedges(_p(f), int(P), int(nf), int(nv), _p(he), _p(hv), _p(hf))
        return dict(he=he, hv=hv, hf=hf)


class RefLib(_Lib):
    prefix = "ref"

    def __init__(self):
        if not os.path.exists(REF_SO):
            raise FileNotFoundError(REF_SO)
        self.lib = ctypes.CDLL(REF_SO)
        self.lib.ref_dmc_run.restype = ctypes.c_void_p
        self.lib.ref_tmc_run.restype = ctypes.c_void_p

    def dmc(self, vol, simplify=0, flip=0):
        d, a = _vol_args(vol)
        h, out = self._dmc_fetch(self.lib.ref_dmc_run(*a, int(simplify), int(flip)))
        self.lib.ref_dmc_free(h)
        return out

    def tmc(self, vol):
        d, a = _vol_args(vol)
        h, out = self._tmc_fetch(self.lib.ref_tmc_run(*a))
        self.lib.ref_tmc_free(h)
        return out

    def tmc_connectivity(self, vol):
        """The reference's connectivity() on its t_mc mesh: (components, orientation changes)."""
        d, a = _vol_args(vol)
        out = (ctypes.c_int64 * 2)()
        self.lib.ref_tmc_connectivity(*a, out)
        return int(out[0]), int(out[1])

    def tmc_files(self, iso, volume, obj, off):
        """The reference's MarchingCubes::operator(): ushort volume file in, OBJ and OFF files out."""
        self.lib.ref_tmc_files(ctypes.c_double(iso), volume.encode(), obj.encode(), off.encode())

    def color_valence(self, nv, quads, colors):
        q = np.ascontiguousarray(quads, dtype=np.int32)
        col = np.ascontiguousarray(colors, dtype=np.int32).copy()
        val = np.zeros(nv, np.int32)
        self.lib.ref_dmc_color_valence(int(nv), int(q.size // 4), _p(q), _p(col), _p(val))
        return col, val


def ref_available():
    return os.path.exists(REF_SO)
