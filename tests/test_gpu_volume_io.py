"""tmc_field_load on the GPU: each of the reference's volume file layouts read into device memory
(uint16 data widened to float32 there) gives the same meshes as the same values passed as a float32
host field; the writers give the same files from a device-resident mesh as from its host copy."""
import numpy as np
import pytest

from tmc_gb300 import native
from tmc_gb300 import volumes as V

from test_volume_io import _write_volume

pytestmark = pytest.mark.gpu

KEYS = ("v", "n", "v64", "q", "t")


@pytest.fixture(scope="module")
def ctx():
    c = native.Context(0)
    yield c
    c.close()


def _field(fmt):
    rng = np.random.Generator(np.random.PCG64(21 + fmt))
    d = V.gaussian_blobs(23, 19, 17, rng)  # 7429 values: not a multiple of 8
    if fmt in (native.FILE_INT_U16, native.FILE_U16):
        return np.round(d * 4000).astype(np.uint16), 1900.5
    return d.astype(np.float32), 0.45


@pytest.mark.parametrize("fmt", [native.FILE_DMC, native.FILE_INT_F32, native.FILE_INT_U16, native.FILE_U16])
def test_loaded_field_gives_the_same_meshes(ctx, tmp_path, fmt):
    data, iso = _field(fmt)
    spacing = (0.5, 0.375, 0.25)
    p = str(tmp_path / "v.raw")
    _write_volume(p, fmt, data, spacing)
    f = ctx.field_load(p, fmt)
    try:
        assert (f.vol.nx, f.vol.ny, f.vol.nz, f.vol.on_device) == (23, 19, 17, 1)
        host = V.Volume(data.astype(np.float32), spacing=tuple(f.vol.spacing), origin=(0.0, 0.0, 0.0), iso=iso)
        for algo in ("dmc", "tmc"):
            flags = native.OUT_POS_F64 | native.OUT_HOST
            if algo == "dmc":
                got = ctx.fetch(ctx.dmc_raw(f.vol, iso, flags))
                want = ctx.dmc(host, native.OUT_POS_F64)
            else:
                got = ctx.fetch(ctx.tmc_raw(f.vol, iso, flags))
                want = ctx.tmc(host, native.OUT_POS_F64)
            assert want["v"].size > 0
            for k in KEYS:
                np.testing.assert_array_equal(got[k], want[k], err_msg=f"format {fmt} {algo}: {k}")
    finally:
        ctx.field_free(f)


def test_writers_from_device_mesh(ctx, tmp_path):
    data, iso = _field(native.FILE_INT_F32)
    vol = V.Volume(data, spacing=(0.5, 0.5, 0.5), iso=iso)
    tv = native.make_volume(vol)
    md = ctx.dmc_raw(tv, iso, native.OUT_TRIANGLES)  # device-resident
    mh = ctx.dmc_raw(tv, iso, native.OUT_TRIANGLES | native.OUT_HOST)
    try:
        assert md.on_device == 1 and mh.on_device == 0
        for style in (native.OBJ_DMC_TRIS, native.OBJ_DMC_QUADS):
            native.write_obj(md, str(tmp_path / "d.obj"), style, ctx)
            native.write_obj(mh, str(tmp_path / "h.obj"), style, ctx)
            assert open(tmp_path / "d.obj").read() == open(tmp_path / "h.obj").read()
        native.write_off(md, str(tmp_path / "d.off"), ctx)
        native.write_off(mh, str(tmp_path / "h.off"), ctx)
        assert open(tmp_path / "d.off").read() == open(tmp_path / "h.off").read()
    finally:
        ctx.free(md)
        ctx.free(mh)


def test_field_load_errors(ctx, tmp_path):
    with pytest.raises(native.TmcError) as e:
        ctx.field_load(str(tmp_path / "missing.raw"), native.FILE_U16)
    assert e.value.status == native.TMC_ERR_INVALID_ARG
