"""ctypes binding of the C ABI in include/tmc_gb300.h (libtmc_gb300.so, built in-tree).

The library is the product path: there is no CPU fallback.  Loading fails loudly when the
extension has not been built (run tmc_gb300.build.build()) or no CUDA device is present.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libtmc_gb300.so")

TMC_OK = 0
TMC_ERR_INVALID_ARG = 1
TMC_ERR_OOM = 2
TMC_ERR_CAPACITY = 3
TMC_ERR_CUDA = 4
TMC_ERR_TIMEOUT = 5
TMC_ERR_NUMERIC = 6
STATUS = {0: "TMC_OK", 1: "TMC_ERR_INVALID_ARG", 2: "TMC_ERR_OOM", 3: "TMC_ERR_CAPACITY", 4: "TMC_ERR_CUDA",
          5: "TMC_ERR_TIMEOUT", 6: "TMC_ERR_NUMERIC", 7: "TMC_ERR_INTERNAL"}

DMC_SIMPLIFY = 1 << 0
DMC_P3X3Y_COLOR = 1 << 1
DMC_P3X3Y_ISOLATED = 1 << 2
DMC_P3333 = 1 << 3
OUT_TRIANGLES = 1 << 4
OUT_HALFEDGES = 1 << 5
OUT_HOST = 1 << 6
OUT_POS_F64 = 1 << 7
OUT_LOCAL = 1 << 8
GRAD_FLIP = 1 << 9
TMC_KEY32 = 1 << 10
ALGO_DMC = 0
ALGO_TMC = 1

# every symbol include/tmc_gb300.h declares
EXPORTS = ["tmc_ctx_create", "tmc_ctx_destroy", "tmc_last_error", "tmc_ctx_stream", "tmc_ctx_synchronize",
           "tmc_ctx_launch_count", "tmc_ctx_set_profiling", "tmc_ctx_profile_read", "tmc_dmc_extract", "tmc_tmc_sharedvertex", "tmc_tmc_halfedge",
           "tmc_mesh_free", "tmc_batch_extract", "tmc_dmc_count_static", "tmc_server_create", "tmc_server_destroy",
           "tmc_server_submit", "tmc_server_poll", "tmc_server_wait", "tmc_server_release", "tmc_server_last_error",
           "tmc_server_stats", "tmc_ctx_set_tuning", "tmc_ctx_get_tuning", "tmc_ctx_autotune",
           "tmc_volume_file_info", "tmc_field_load", "tmc_field_free", "tmc_mesh_write_obj", "tmc_mesh_write_off",
           "tmc_mesh_quality", "tmc_mesh_valence", "tmc_mesh_check", "tmc_field_generate", "tmc_dmc_color_valence",
           "tmc_field_generate_ex", "tmc_dmc_extract_generated", "tmc_tmc_extract_generated"]

SURFACES = ("sphere", "torus", "two_holed_torus", "four_holed_torus", "genus_two", "iwp", "pw_hybrid", "neovius",
            "goursat", "steiner_roman")

FACES_QUADS = 0
FACES_TRIS = 1

FILE_DMC = 0
FILE_INT_F32 = 1
FILE_INT_U16 = 2
FILE_U16 = 3
OBJ_DMC_TRIS = 0
OBJ_DMC_QUADS = 1
OBJ_TMC = 2

TUNE_GROUP_LANES = 1
TUNE_WARP_LIST_MAX = 2
TUNE_VERTEX_BLOCKS_PER_SM = 3
TUNE_EMIT_BLOCKS_PER_SM = 4
TUNE_SLAB_MIB = 5
TUNE_MAX_SLABS = 6
TUNE_QUAD_BLOCKS_PER_SM = 7


class TmcError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class CtxOpts(ctypes.Structure):
    _fields_ = [("reserve_bytes", ctypes.c_size_t), ("check_numeric", ctypes.c_int32), ("priority", ctypes.c_int32)]


class Volume(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("nz", ctypes.c_int32),
                ("origin", ctypes.c_double * 3), ("spacing", ctypes.c_double * 3),
                ("data", ctypes.c_void_p), ("on_device", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class Mesh(ctypes.Structure):
    _fields_ = [("nr_v", ctypes.c_int64), ("nr_q", ctypes.c_int64), ("nr_t", ctypes.c_int64), ("nr_he", ctypes.c_int64),
                ("on_device", ctypes.c_int32), ("reserved", ctypes.c_int32),
                ("v", ctypes.c_void_p), ("n", ctypes.c_void_p), ("v64", ctypes.c_void_p),
                ("quads", ctypes.c_void_p), ("tris", ctypes.c_void_p), ("he", ctypes.c_void_p),
                ("he_v", ctypes.c_void_p), ("he_f", ctypes.c_void_p), ("vcell", ctypes.c_void_p),
                ("vuvw", ctypes.c_void_p), ("stats", ctypes.c_int64 * 8), ("priv", ctypes.c_void_p)]


class Field(ctypes.Structure):
    _fields_ = [("vol", Volume), ("priv", ctypes.c_void_p)]


SURF_PERIODIC = 10
SURF_BLOBS = 11


class Generator(ctypes.Structure):
    _fields_ = [("surface", ctypes.c_int32), ("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("nz", ctypes.c_int32),
                ("count", ctypes.c_int32), ("reserved", ctypes.c_int32), ("params", ctypes.c_double * 64)]


def make_generator(surface: int, dims, params=(), count: int = 0) -> Generator:
    """A tmc_generator: surface id (SURFACES index, SURF_PERIODIC or SURF_BLOBS), (nx, ny, nz),
    parameters (periodic: (k,); blobs: (cx, cy, cz, sigma) per blob)."""
    g = Generator()
    g.surface = int(surface)
    g.nx, g.ny, g.nz = (int(d) for d in dims)
    g.count = int(count)
    for i, x in enumerate(params):
        g.params[i] = float(x)
    return g


class Request(ctypes.Structure):
    _fields_ = [("vol", Volume), ("iso", ctypes.c_double), ("algo", ctypes.c_uint32), ("flags", ctypes.c_uint32)]


class ServerOpts(ctypes.Structure):
    _fields_ = [("hbm_budget", ctypes.c_size_t), ("workers", ctypes.c_int32), ("max_batch", ctypes.c_int32),
                ("reserved", ctypes.c_int32), ("max_batch_cells", ctypes.c_int64)]


_lib = None


def load(path: str = LIB_PATH):
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with tmc_gb300.build.build() (no CPU fallback exists)")
    lib = ctypes.CDLL(path)
    lib.tmc_ctx_create.argtypes = [ctypes.c_int, ctypes.POINTER(CtxOpts), ctypes.POINTER(ctypes.c_void_p)]
    lib.tmc_ctx_destroy.argtypes = [ctypes.c_void_p]
    lib.tmc_last_error.argtypes = [ctypes.c_void_p]
    lib.tmc_last_error.restype = ctypes.c_char_p
    lib.tmc_ctx_stream.argtypes = [ctypes.c_void_p]
    lib.tmc_ctx_stream.restype = ctypes.c_void_p
    lib.tmc_ctx_synchronize.argtypes = [ctypes.c_void_p]
    lib.tmc_ctx_launch_count.argtypes = [ctypes.c_void_p]
    lib.tmc_ctx_launch_count.restype = ctypes.c_int64
    for name in ("tmc_dmc_extract", "tmc_tmc_sharedvertex", "tmc_tmc_halfedge"):
        if hasattr(lib, name):
            f = getattr(lib, name)
            f.argtypes = [ctypes.c_void_p, ctypes.POINTER(Volume), ctypes.c_double, ctypes.c_uint32, ctypes.POINTER(Mesh)]
    lib.tmc_mesh_free.argtypes = [ctypes.c_void_p, ctypes.POINTER(Mesh)]
    lib.tmc_ctx_set_profiling.argtypes = [ctypes.c_void_p, ctypes.c_int]
    lib.tmc_ctx_profile_read.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_char_p,
                                         ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int64)]
    lib.tmc_ctx_profile_read.restype = ctypes.c_int32
    lib.tmc_dmc_count_static.argtypes = [ctypes.c_void_p, ctypes.POINTER(Volume), ctypes.c_double,
                                         ctypes.POINTER(ctypes.c_int64)]
    lib.tmc_dmc_count_static.restype = ctypes.c_int
    lib.tmc_dmc_color_valence.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p,
                                          ctypes.c_void_p, ctypes.c_void_p]
    lib.tmc_dmc_color_valence.restype = ctypes.c_int
    lib.tmc_field_generate_ex.argtypes = [ctypes.c_void_p, ctypes.POINTER(Generator), ctypes.POINTER(Field)]
    lib.tmc_dmc_extract_generated.argtypes = [ctypes.c_void_p, ctypes.POINTER(Generator), ctypes.c_double,
                                              ctypes.c_uint32, ctypes.POINTER(Mesh)]
    lib.tmc_tmc_extract_generated.argtypes = [ctypes.c_void_p, ctypes.POINTER(Generator), ctypes.c_double,
                                              ctypes.c_uint32, ctypes.c_int32, ctypes.POINTER(Mesh)]
    lib.tmc_server_create.argtypes = [ctypes.c_int, ctypes.POINTER(ServerOpts), ctypes.POINTER(ctypes.c_void_p)]
    lib.tmc_server_destroy.argtypes = [ctypes.c_void_p]
    lib.tmc_server_submit.argtypes = [ctypes.c_void_p, ctypes.POINTER(Request), ctypes.POINTER(ctypes.c_int64)]
    lib.tmc_server_poll.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.POINTER(ctypes.c_int32)]
    lib.tmc_server_wait.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_double, ctypes.POINTER(Mesh)]
    lib.tmc_server_release.argtypes = [ctypes.c_void_p, ctypes.POINTER(Mesh)]
    lib.tmc_server_last_error.argtypes = [ctypes.c_void_p]
    lib.tmc_server_last_error.restype = ctypes.c_char_p
    lib.tmc_server_stats.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64)]
    lib.tmc_volume_file_info.argtypes = [ctypes.c_char_p, ctypes.c_int32, ctypes.POINTER(ctypes.c_int32),
                                         ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int64)]
    lib.tmc_field_load.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int32, ctypes.POINTER(Field)]
    lib.tmc_field_free.argtypes = [ctypes.c_void_p, ctypes.POINTER(Field)]
    lib.tmc_mesh_write_obj.argtypes = [ctypes.c_void_p, ctypes.POINTER(Mesh), ctypes.c_char_p, ctypes.c_int32]
    lib.tmc_mesh_write_off.argtypes = [ctypes.c_void_p, ctypes.POINTER(Mesh), ctypes.c_char_p]
    lib.tmc_mesh_quality.argtypes = [ctypes.c_void_p, ctypes.POINTER(Mesh), ctypes.c_int32,
                                     ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_double)]
    lib.tmc_mesh_valence.argtypes = [ctypes.c_void_p, ctypes.POINTER(Mesh), ctypes.c_int32,
                                     ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_int32)]
    lib.tmc_field_generate.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                       ctypes.POINTER(Field)]
    lib.tmc_mesh_check.argtypes = [ctypes.c_void_p, ctypes.POINTER(Mesh), ctypes.c_int32, ctypes.POINTER(ctypes.c_int64)]
    lib.tmc_ctx_set_tuning.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64]
    lib.tmc_ctx_get_tuning.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.POINTER(ctypes.c_int64)]
    lib.tmc_ctx_autotune.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.POINTER(Request), ctypes.c_int32,
                                     ctypes.POINTER(ctypes.c_double)]
    if hasattr(lib, "tmc_batch_extract"):
        lib.tmc_batch_extract.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.POINTER(Request), ctypes.POINTER(Mesh)]
    _lib = lib
    return lib


def make_volume(vol, data_ptr: int | None = None, on_device: bool = False) -> Volume:
    """A tmc_volume for a tmc_gb300.volumes.Volume (host numpy data) or a device pointer."""
    nx, ny, nz = vol.dims
    v = Volume()
    v.nx, v.ny, v.nz = nx, ny, nz
    v.origin = (ctypes.c_double * 3)(*vol.origin)
    v.spacing = (ctypes.c_double * 3)(*vol.spacing)
    if data_ptr is None:
        arr = np.ascontiguousarray(vol.data, dtype=np.float32)
        vol._keep = arr  # keep alive
        v.data = arr.ctypes.data
        v.on_device = 0
    else:
        v.data = data_ptr
        v.on_device = 1 if on_device else 0
    return v


def volume_file_info(path: str, fmt: int):
    """tmc_volume_file_info: (dims, spacing, data offset) of a volume file; needs no GPU."""
    lib = load()
    dims = (ctypes.c_int32 * 3)()
    sp = (ctypes.c_double * 3)()
    off = ctypes.c_int64()
    st = lib.tmc_volume_file_info(path.encode(), int(fmt), dims, sp, ctypes.byref(off))
    if st != TMC_OK:
        raise TmcError(st, f"{path}: not a valid volume file of format {fmt}")
    return tuple(dims), tuple(sp), off.value


def host_mesh(v, n, quads=None, tris=None, v64=None) -> Mesh:
    """A tmc_mesh over numpy arrays in host memory (for the writers); keeps the arrays alive."""
    m = Mesh()
    keep = []

    def ptr(a, dtype):
        if a is None:
            return None
        a = np.ascontiguousarray(a, dtype=dtype)
        keep.append(a)
        return a.ctypes.data

    m.nr_v = len(v) // 3
    m.nr_q = 0 if quads is None else len(quads) // 4
    m.nr_t = 0 if tris is None else len(tris) // 3
    m.on_device = 0
    m.v, m.n, m.v64 = ptr(v, np.float32), ptr(n, np.float32), ptr(v64, np.float64)
    m.quads, m.tris = ptr(quads, np.int32), ptr(tris, np.int32)
    m._keep = keep
    return m


def write_obj(mesh: Mesh, path: str, style: int, ctx=None):
    st = load().tmc_mesh_write_obj(ctx.h if ctx else None, ctypes.byref(mesh), path.encode(), int(style))
    if st != TMC_OK:
        raise TmcError(st, ctx.lib.tmc_last_error(ctx.h).decode() if ctx else f"writing {path} failed")


def write_off(mesh: Mesh, path: str, ctx=None):
    st = load().tmc_mesh_write_off(ctx.h if ctx else None, ctypes.byref(mesh), path.encode())
    if st != TMC_OK:
        raise TmcError(st, ctx.lib.tmc_last_error(ctx.h).decode() if ctx else f"writing {path} failed")


def _host_array(ptr, count, dtype):
    if not ptr or count == 0:
        return np.zeros(0, dtype=dtype)
    ct = np.ctypeslib.as_ctypes_type(np.dtype(dtype))
    buf = (ct * count).from_address(ptr)
    return np.ctypeslib.as_array(buf).copy()


class Context:
    """One CUDA stream, pooled device memory; mirrors a reference extraction object."""

    def __init__(self, device: int = 0, reserve_bytes: int = 0, check_numeric: bool = False, priority: int = 0):
        self.lib = load()
        self.device = device
        self.h = ctypes.c_void_p()
        opts = CtxOpts(reserve_bytes, 1 if check_numeric else 0, priority)
        st = self.lib.tmc_ctx_create(device, ctypes.byref(opts), ctypes.byref(self.h))
        if st != TMC_OK:
            raise TmcError(st, "tmc_ctx_create failed (is a CUDA device visible?)")

    def close(self):
        if self.h:
            self.lib.tmc_ctx_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self) -> int:
        return self.lib.tmc_ctx_stream(self.h)

    def launches(self) -> int:
        return self.lib.tmc_ctx_launch_count(self.h)

    def set_profiling(self, on: bool):
        self._check(self.lib.tmc_ctx_set_profiling(self.h, 1 if on else 0))

    def profile(self) -> dict:
        """{stage: (total_ms, count)} accumulated since profiling was enabled."""
        n = 64
        names = ctypes.create_string_buffer(32 * n)
        ms = (ctypes.c_double * n)()
        cnt = (ctypes.c_int64 * n)()
        k = self.lib.tmc_ctx_profile_read(self.h, n, names, ms, cnt)
        out = {}
        for i in range(max(k, 0)):
            nm = names.raw[32 * i: 32 * i + 32].split(b"\0")[0].decode()
            out[nm] = (ms[i], cnt[i])
        return out

    def synchronize(self):
        self._check(self.lib.tmc_ctx_synchronize(self.h))

    def _check(self, st):
        if st != TMC_OK:
            raise TmcError(st, self.lib.tmc_last_error(self.h).decode())

    def _run(self, fn, volume: Volume, iso: float, flags: int) -> Mesh:
        m = Mesh()
        self._check(getattr(self.lib, fn)(self.h, ctypes.byref(volume), float(iso), int(flags), ctypes.byref(m)))
        return m

    def free(self, m: Mesh):
        self._check(self.lib.tmc_mesh_free(self.h, ctypes.byref(m)))

    # -- raw calls (mesh stays where flags put it; caller frees) -----------------------------
    def dmc_raw(self, volume: Volume, iso: float, flags: int) -> Mesh:
        return self._run("tmc_dmc_extract", volume, iso, flags)

    def tmc_raw(self, volume: Volume, iso: float, flags: int, halfedge: bool = False) -> Mesh:
        return self._run("tmc_tmc_halfedge" if halfedge else "tmc_tmc_sharedvertex", volume, iso, flags)

    def dmc_count_static(self, volume: Volume, iso: float) -> tuple:
        """tmc_dmc_count_static: (vertices, quads, active cells, ambiguous cells) of a DMC extraction
        of a device-resident field, computed in a static scratch array without allocating."""
        counts = (ctypes.c_int64 * 4)()
        self._check(self.lib.tmc_dmc_count_static(self.h, ctypes.byref(volume), float(iso), counts))
        return tuple(counts)

    def dmc_color_valence(self, nr_v: int, quads, inherited):
        """tmc_dmc_color_valence on host arrays (copied to the device and back): the reduced face
        colours and the vertex valences of a quad mesh with its inherited colours."""
        import numpy as np
        import torch
        q = torch.from_numpy(np.ascontiguousarray(quads, dtype=np.int32)).cuda(self.device)
        col = torch.from_numpy(np.ascontiguousarray(inherited).astype(np.uint8)).cuda(self.device)
        val = torch.zeros(max(int(nr_v), 1), dtype=torch.int32, device=f"cuda:{self.device}")
        torch.cuda.synchronize(self.device)
        self._check(self.lib.tmc_dmc_color_valence(self.h, int(nr_v), q.numel() // 4, q.data_ptr(), col.data_ptr(),
                                                   val.data_ptr()))
        return col.cpu().numpy().astype(np.int32), val[:int(nr_v)].cpu().numpy()

    def batch_raw(self, volumes: list, isos: list, algos: list, flags: list) -> list:
        """tmc_batch_extract over prepared tmc_volume structs; returns the meshes (caller frees)."""
        n = len(volumes)
        reqs = (Request * n)()
        for q in range(n):
            reqs[q].vol = volumes[q]
            reqs[q].iso = float(isos[q])
            reqs[q].algo = int(algos[q])
            reqs[q].flags = int(flags[q])
        outs = (Mesh * n)()
        self._check(self.lib.tmc_batch_extract(self.h, n, reqs, outs))
        return [outs[q] for q in range(n)]

    def quality(self, m: Mesh, faces: int):
        """tmc_mesh_quality: (per-face quality, (min, max, mean))."""
        nf = m.nr_q if faces == FACES_QUADS else m.nr_t
        q = np.zeros(max(nf, 1), np.float32)
        summ = (ctypes.c_double * 3)()
        self._check(self.lib.tmc_mesh_quality(self.h, ctypes.byref(m), int(faces),
                                              q.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), summ))
        return q[:nf], tuple(summ)

    def valence(self, m: Mesh, faces: int) -> np.ndarray:
        """tmc_mesh_valence: the valence distribution, trimmed after its last non-empty bin."""
        h = (ctypes.c_uint32 * 100)()
        n = ctypes.c_int32()
        self._check(self.lib.tmc_mesh_valence(self.h, ctypes.byref(m), int(faces), h, ctypes.byref(n)))
        return np.array(list(h)[:n.value], np.int64)

    def check(self, m: Mesh, faces: int) -> dict:
        """tmc_mesh_check: components, orientation defects, boundary / non-manifold / degenerate counts."""
        r = (ctypes.c_int64 * 6)()
        self._check(self.lib.tmc_mesh_check(self.h, ctypes.byref(m), int(faces), r))
        return dict(zip(("components", "orientation_defects", "boundary_edges", "nonmanifold_halfedges",
                         "degenerate_faces", "boundary_vertices"), list(r)))

    def field_load(self, path: str, fmt: int) -> Field:
        """tmc_field_load: a volume file read into device memory (float32)."""
        f = Field()
        self._check(self.lib.tmc_field_load(self.h, path.encode(), int(fmt), ctypes.byref(f)))
        return f

    def field_generate(self, surface: int, nx: int, ny: int, nz: int) -> Field:
        """tmc_field_generate: one of the reference's implicit surfaces sampled on [-1, 1]^3."""
        f = Field()
        self._check(self.lib.tmc_field_generate(self.h, int(surface), nx, ny, nz, ctypes.byref(f)))
        return f

    def field_generate_ex(self, gen: Generator) -> Field:
        """tmc_field_generate_ex: a parameterised generated field written to device memory."""
        f = Field()
        self._check(self.lib.tmc_field_generate_ex(self.h, ctypes.byref(gen), ctypes.byref(f)))
        return f

    def dmc_generated_raw(self, gen: Generator, iso: float, flags: int) -> Mesh:
        """tmc_dmc_extract_generated: DMC with the field generation fused into the classification."""
        m = Mesh()
        self._check(self.lib.tmc_dmc_extract_generated(self.h, ctypes.byref(gen), float(iso), int(flags),
                                                       ctypes.byref(m)))
        return m

    def tmc_generated_raw(self, gen: Generator, iso: float, flags: int, halfedge: bool = False) -> Mesh:
        """tmc_tmc_extract_generated: TMC with the field generation fused into the classification."""
        m = Mesh()
        self._check(self.lib.tmc_tmc_extract_generated(self.h, ctypes.byref(gen), float(iso), int(flags),
                                                       1 if halfedge else 0, ctypes.byref(m)))
        return m

    def field_free(self, f: Field):
        self._check(self.lib.tmc_field_free(self.h, ctypes.byref(f)))

    def set_tuning(self, key: int, value: int):
        self._check(self.lib.tmc_ctx_set_tuning(self.h, key, int(value)))

    def get_tuning(self, key: int) -> int:
        v = ctypes.c_int64()
        self._check(self.lib.tmc_ctx_get_tuning(self.h, key, ctypes.byref(v)))
        return v.value

    def autotune(self, volumes: list, isos: list, algos: list, flags: list, rounds: int = 3) -> float:
        """tmc_ctx_autotune over prepared tmc_volume structs; returns the best batch time (ms)."""
        n = len(volumes)
        reqs = (Request * n)()
        for q in range(n):
            reqs[q].vol = volumes[q]
            reqs[q].iso = float(isos[q])
            reqs[q].algo = int(algos[q])
            reqs[q].flags = int(flags[q])
        best = ctypes.c_double()
        self._check(self.lib.tmc_ctx_autotune(self.h, n, reqs, rounds, ctypes.byref(best)))
        return best.value

    def batch(self, vols: list, algos: list, flags: list) -> list:
        """Batched extraction of host volumes (tmc_gb300.volumes.Volume); numpy results."""
        tv = [make_volume(v) for v in vols]
        ms = self.batch_raw(tv, [v.iso for v in vols], algos, [f | OUT_HOST for f in flags])
        return [self.fetch(m) for m in ms]

    # -- numpy results --------------------------------------------------------------------
    def fetch(self, m: Mesh) -> dict:
        """Copy a host-resident mesh (OUT_HOST) into numpy arrays and free it."""
        assert not m.on_device, "fetch() needs a mesh extracted with OUT_HOST"
        nv, nq, nt, nh = m.nr_v, m.nr_q, m.nr_t, m.nr_he
        out = dict(v=_host_array(m.v, 3 * nv, np.float32), n=_host_array(m.n, 3 * nv, np.float32),
                   v64=_host_array(m.v64, 3 * nv, np.float64), q=_host_array(m.quads, 4 * nq, np.int32),
                   t=_host_array(m.tris, 3 * nt, np.int32), he=_host_array(m.he, 4 * nh, np.int32),
                   hv=_host_array(m.he_v, nv if m.he_v else 0, np.int32),
                   hf=_host_array(m.he_f, (nq if nq else nt) if m.he_f else 0, np.int32),
                   vcell=_host_array(m.vcell, nv if m.vcell else 0, np.int64),
                   vuvw=_host_array(m.vuvw, 3 * nv if m.vuvw else 0, np.float32),
                   stats=np.array(list(m.stats)))
        self.free(m)
        return out

    def dmc(self, vol, flags: int = 0, iso: float | None = None) -> dict:
        m = self.dmc_raw(make_volume(vol), vol.iso if iso is None else iso, flags | OUT_HOST)
        return self.fetch(m)

    def tmc(self, vol, flags: int = 0, halfedge: bool = False, iso: float | None = None) -> dict:
        m = self.tmc_raw(make_volume(vol), vol.iso if iso is None else iso, flags | OUT_HOST, halfedge)
        return self.fetch(m)


class Server:
    """tmc_server_*: continuous batching of requests on one GPU (thread-safe submit / wait)."""

    def __init__(self, device: int = 0, hbm_budget: int = 0, workers: int = 0, max_batch: int = 0,
                 max_batch_cells: int = 0):
        self.lib = load()
        self.h = ctypes.c_void_p()
        opts = ServerOpts(hbm_budget, workers, max_batch, 0, max_batch_cells)
        st = self.lib.tmc_server_create(device, ctypes.byref(opts), ctypes.byref(self.h))
        if st != TMC_OK:
            raise TmcError(st, "tmc_server_create failed")

    def close(self):
        if self.h:
            self.lib.tmc_server_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st):
        if st != TMC_OK:
            raise TmcError(st, self.lib.tmc_server_last_error(self.h).decode())

    def submit(self, volume: Volume, iso: float, algo: int, flags: int) -> int:
        r = Request()
        r.vol = volume
        r.iso = float(iso)
        r.algo = int(algo)
        r.flags = int(flags)
        t = ctypes.c_int64()
        self._check(self.lib.tmc_server_submit(self.h, ctypes.byref(r), ctypes.byref(t)))
        return t.value

    def poll(self, ticket: int) -> bool:
        d = ctypes.c_int32()
        self._check(self.lib.tmc_server_poll(self.h, ticket, ctypes.byref(d)))
        return bool(d.value)

    def wait_raw(self, ticket: int, timeout: float = -1.0) -> Mesh:
        m = Mesh()
        self._check(self.lib.tmc_server_wait(self.h, ticket, float(timeout), ctypes.byref(m)))
        return m

    def release(self, m: Mesh):
        self._check(self.lib.tmc_server_release(self.h, ctypes.byref(m)))

    def wait(self, ticket: int, timeout: float = -1.0) -> dict:
        """The ticket's mesh as numpy arrays (the request must have TMC_OUT_HOST); releases it."""
        m = self.wait_raw(ticket, timeout)
        assert not m.on_device, "wait() needs a request with OUT_HOST"
        nv, nq, nt, nh = m.nr_v, m.nr_q, m.nr_t, m.nr_he
        out = dict(v=_host_array(m.v, 3 * nv, np.float32), n=_host_array(m.n, 3 * nv, np.float32),
                   v64=_host_array(m.v64, 3 * nv, np.float64), q=_host_array(m.quads, 4 * nq, np.int32),
                   t=_host_array(m.tris, 3 * nt, np.int32), he=_host_array(m.he, 4 * nh, np.int32),
                   hv=_host_array(m.he_v, nv if m.he_v else 0, np.int32),
                   hf=_host_array(m.he_f, (nq if nq else nt) if m.he_f else 0, np.int32),
                   vcell=_host_array(m.vcell, nv if m.vcell else 0, np.int64),
                   vuvw=_host_array(m.vuvw, 3 * nv if m.vuvw else 0, np.float32),
                   stats=np.array(list(m.stats)))
        self.release(m)
        return out

    def stats(self) -> list:
        a = (ctypes.c_int64 * 8)()
        self._check(self.lib.tmc_server_stats(self.h, a))
        return list(a)
