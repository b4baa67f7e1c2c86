"""The C ABI library loads and exports every entry point include/jx.h declares.

Only calls that touch no GPU run here (validation, sizing, selectors).
"""

import ctypes
import re
from pathlib import Path

import pytest

from jathenax_gb300 import _lib

HEADER = Path(__file__).resolve().parents[1] / "include" / "jx.h"


def declared_functions():
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    return sorted(set(re.findall(r"\b(jx_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_expected_surface():
    names = declared_functions()
    for required in ("jx_stage", "jx_step", "jx_timestep", "jx_recover", "jx_begin_step",
                     "jx_force_render", "jx_force_kick", "jx_workspace_bytes", "jx_last_error"):
        assert required in names


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    missing = [name for name in declared_functions() if not hasattr(lib, name)]
    assert not missing, missing
    assert set(declared_functions()) <= set(_lib.PROTOTYPES), "binding lacks a prototype"


def test_version_and_stage_counts():
    lib = _lib.load()
    assert b"sm_103a" in lib.jx_version()
    assert [lib.jx_num_stages(i) for i in range(3)] == [2, 3, 4]
    assert lib.jx_num_stages(7) == 0


def _desc(**kw):
    base = dict(ny=48, nx=64, nvar=3, dtype=0, recon=2, rsolver=2, integrator=1,
                dx=1 / 64, dy=1 / 48, cs=1.0, dfloor=1e-10)
    base.update(kw)
    return _lib.Desc(**base)


@pytest.mark.parametrize(("field", "value", "status"), [
    ("recon", 5, _lib.JX_ERR_UNSUPPORTED), ("rsolver", -1, _lib.JX_ERR_UNSUPPORTED),
    ("integrator", 3, _lib.JX_ERR_UNSUPPORTED), ("dtype", 2, _lib.JX_ERR_UNSUPPORTED),
    ("nvar", 2, _lib.JX_ERR_INVALID), ("nx", 0, _lib.JX_ERR_INVALID),
    ("cs", 0.0, _lib.JX_ERR_INVALID), ("viscosity", -1.0, _lib.JX_ERR_INVALID),
    ("dx", float("nan"), _lib.JX_ERR_INVALID), ("smagorinsky_cs", float("inf"), _lib.JX_ERR_INVALID),
])
def test_descriptor_validation(field, value, status):
    lib = _lib.load()
    assert lib.jx_check_desc(ctypes.byref(_desc(**{field: value}))) == status
    assert lib.jx_last_error()  # a message is always set


def test_workspace_and_tiles():
    lib = _lib.load()
    size = ctypes.c_size_t()
    assert lib.jx_workspace_bytes(ctypes.byref(_desc()), ctypes.byref(size)) == 0
    assert size.value % 256 == 0 and size.value > 0
    tx, ty, smem = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int64()
    # float32 with 3/4 variables defaults to the register-marching kernel
    # (58-column tiles), float64 to the 32-column shared-memory tile.
    assert lib.jx_tile_info(ctypes.byref(_desc(nvar=4, dtype=_lib.JX_F32)), ctypes.byref(tx),
                            ctypes.byref(ty), ctypes.byref(smem)) == 0
    assert tx.value == 58 and 8 <= ty.value <= 64 and smem.value == 0
    assert lib.jx_tile_info(ctypes.byref(_desc(nvar=4)), ctypes.byref(tx), ctypes.byref(ty),
                            ctypes.byref(smem)) == 0
    assert (tx.value, ty.value) == (32, 16) and smem.value <= 112 * 1024
    assert lib.jx_tile_info(ctypes.byref(_desc(nvar=4, tile_x=32, tile_y=16)), ctypes.byref(tx),
                            ctypes.byref(ty), ctypes.byref(smem)) == 0
    assert (tx.value, ty.value) == (32, 16) and smem.value <= 112 * 1024
    assert lib.jx_tile_info(ctypes.byref(_desc(nvar=3, tile_x=58, tile_y=4)), ctypes.byref(tx),
                            ctypes.byref(ty), ctypes.byref(smem)) == _lib.JX_ERR_INVALID
    # 26- and 90-column tiles: the marching kernel with one and three columns
    # per lane (float32); float64 marches with two columns only.
    for width in (26, 90):
        assert lib.jx_tile_info(ctypes.byref(_desc(nvar=4, dtype=_lib.JX_F32, tile_x=width, tile_y=12)),
                                ctypes.byref(tx), ctypes.byref(ty), ctypes.byref(smem)) == 0
        assert (tx.value, ty.value, smem.value) == (width, 12, 0)
        assert lib.jx_tile_info(ctypes.byref(_desc(nvar=4, tile_x=width, tile_y=12)), ctypes.byref(tx),
                                ctypes.byref(ty), ctypes.byref(smem)) == _lib.JX_ERR_INVALID
    # Many scalars shrink the default tile to keep two CTAs per SM.
    assert lib.jx_tile_info(ctypes.byref(_desc(nvar=12)), ctypes.byref(tx), ctypes.byref(ty),
                            ctypes.byref(smem)) == 0
    assert smem.value <= 112 * 1024
    # An explicit tile beyond the shared-memory limit is refused.
    assert lib.jx_tile_info(ctypes.byref(_desc(nvar=8, tile_x=128, tile_y=64)), ctypes.byref(tx),
                            ctypes.byref(ty), ctypes.byref(smem)) == _lib.JX_ERR_INVALID


def test_stage_rejects_bad_arguments_before_touching_the_gpu():
    lib = _lib.load()
    d = _desc()
    ws = ctypes.c_void_p(256)  # never dereferenced: argument checks fail first
    assert lib.jx_stage(ctypes.byref(d), 0, None, None, None, None, None, 0, None, None, ws, 1 << 30,
                        None) == _lib.JX_ERR_INVALID
    assert lib.jx_stage(ctypes.byref(d), 1, ctypes.c_void_p(4096), ctypes.c_void_p(4096),
                        ctypes.c_void_p(4096), None, None, 0, ctypes.c_void_p(8192), None, ws, 16,
                        None) == _lib.JX_ERR_WORKSPACE


def test_python_selectors_raise_key_error():
    from jathenax_gb300.hydro import make_desc
    with pytest.raises(KeyError):
        make_desc((8, 8, 3), "float64", 1.0, 1.0, 1.0, 1e-10, reconstruct="ppm5")
    with pytest.raises(KeyError):
        make_desc((8, 8, 3), "float64", 1.0, 1.0, 1.0, 1e-10, rsolver="hllc")
    with pytest.raises(KeyError):
        make_desc((8, 8, 3), "float64", 1.0, 1.0, 1.0, 1e-10, integrator="rk5")
    with pytest.raises(ValueError):
        make_desc((8, 8, 3), "float64", 1.0, 1.0, -1.0, 1e-10)
