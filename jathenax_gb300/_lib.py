"""ctypes binding of libjx.so (include/jx.h) and CUDA buffer helpers.

The library is loaded from this package directory. There is no CPU fallback:
if libjx.so is missing or no CUDA device is visible, every operator raises.
Device buffers are torch CUDA tensors (PyTorch is used only as the device
memory/stream holder); the kernels are reached through the C ABI.
"""

import ctypes
from pathlib import Path

import numpy as np

_PACKAGE = Path(__file__).resolve().parent
LIBRARY_PATH = _PACKAGE / "libjx.so"

JX_OK, JX_ERR_INVALID, JX_ERR_UNSUPPORTED, JX_ERR_CUDA, JX_ERR_WORKSPACE = 0, -1, -2, -3, -4
JX_F64, JX_F32 = 0, 1
RECON_IDS = {"dc": 0, "plm": 1, "ppm4": 2, "ppmx": 3, "wenoz": 4}
RSOLVER_IDS = {"llf": 0, "hlle": 1, "roe": 2}
INTEGRATOR_IDS = {"rk2": 0, "rk3": 1, "rk4": 2}


class Desc(ctypes.Structure):
    _fields_ = [
        ("ny", ctypes.c_int32), ("nx", ctypes.c_int32), ("nvar", ctypes.c_int32),
        ("dtype", ctypes.c_int32), ("recon", ctypes.c_int32), ("rsolver", ctypes.c_int32),
        ("integrator", ctypes.c_int32), ("tile_x", ctypes.c_int32), ("tile_y", ctypes.c_int32),
        ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("cs", ctypes.c_double),
        ("dfloor", ctypes.c_double), ("viscosity", ctypes.c_double),
        ("smagorinsky_cs", ctypes.c_double), ("drag_rate", ctypes.c_double),
    ]


class Clock(ctypes.Structure):
    _fields_ = [
        ("time", ctypes.c_double), ("dt", ctypes.c_double), ("prev_dt", ctypes.c_double),
        ("tlim", ctypes.c_double), ("cfl", ctypes.c_double), ("power", ctypes.c_double),
        ("t_start", ctypes.c_double), ("dt_update", ctypes.c_double), ("dedt", ctypes.c_double),
        ("reserved0", ctypes.c_double), ("reserved1", ctypes.c_double),
        ("reserved2", ctypes.c_double),
        ("cycle", ctypes.c_int32), ("nlim", ctypes.c_int32), ("update", ctypes.c_int32),
        ("render", ctypes.c_int32), ("done", ctypes.c_int32), ("pending", ctypes.c_int32),
        ("n_updates", ctypes.c_int32), ("status", ctypes.c_int32),
    ]


class Forcing(ctypes.Structure):
    _fields_ = [
        ("table", ctypes.c_void_p), ("cos_x", ctypes.c_void_p), ("sin_x", ctypes.c_void_p),
        ("cos_y", ctypes.c_void_p), ("sin_y", ctypes.c_void_p), ("raw_force", ctypes.c_void_p),
        ("n_updates", ctypes.c_int32), ("n_modes", ctypes.c_int32),
    ]


class Trace(ctypes.Structure):
    _fields_ = [(name, ctypes.c_void_p) for name in (
        "primitives", "left_x", "right_x", "left_y", "right_y", "flux_x", "flux_y",
        "saved", "conserved", "before_kick", "acceleration")]


class SolveStruct(ctypes.Structure):
    _fields_ = [("desc", Desc), ("S", ctypes.c_void_p), ("A", ctypes.c_void_p), ("B", ctypes.c_void_p),
                ("clock", ctypes.c_void_p), ("forcing", Forcing), ("workspace", ctypes.c_void_p),
                ("workspace_bytes", ctypes.c_size_t)]


assert ctypes.sizeof(Clock) == 128

_P, _I32, _I64, _D, _SZ = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_double, ctypes.c_size_t
_DP = ctypes.POINTER(Desc)

# name -> argument types (all return int32 status unless listed in _RESTYPES)
PROTOTYPES = {
    "jx_last_error": [],
    "jx_version": [],
    "jx_workspace_bytes": [_DP, ctypes.POINTER(_SZ)],
    "jx_check_desc": [_DP],
    "jx_num_stages": [_I32],
    "jx_recover": [_DP, _P, _P, _P, _P],
    "jx_timestep": [_DP, _P, _D, _D, _D, _D, _P, _P, _SZ, _P],
    "jx_timestep_noalloc": [_DP, _P, _D, _D, _D, _D, _P, _P],
    "jx_stage": [_DP, _I32, _P, _P, _P, _P, _P, _I32, _P, ctypes.POINTER(Trace), _P, _SZ, _P],
    "jx_cfl_partials": [_DP, _P, _P, _SZ, _P],
    "jx_begin_step": [_DP, _P, _I32, _P, _SZ, _P],
    "jx_force_render": [_DP, ctypes.POINTER(Forcing), _P, _P],
    "jx_force_kick": [_DP, ctypes.POINTER(Forcing), _P, _P, ctypes.POINTER(Trace), _P, _SZ, _P],
    "jx_step": [_DP, _P, _P, _P, ctypes.POINTER(Forcing), _P, _P, _SZ, _P],
    "jx_rk_stage": [_I32, _I64, _P, _P, _P, _D, _D, _D, _D, _D, _I32, _P, _P, _P],
    "jx_flux_divergence": [_I32, _I32, _I32, _I32, _P, _P, _D, _D, _P, _P],
    "jx_stress_face_fluxes": [_I32, _I32, _I32, _P, _P, _P, _P],
    "jx_face_states": [_I32, _I32, _I32, _I32, _I32, _P, _I32, _D, _P, _P, _P],
    "jx_face_flux": [_I32, _I32, _I64, _I32, _I32, _P, _P, _D, _P, _P],
    "jx_viscous_flux": [_I32, _I32, _I32, _I32, _P, _D, _D, _D, _D, _I32, _P, _P],
    "jx_box_sums": [_DP, _P, _P, _P, _SZ, _P],
    "jx_face_velocity_gradients": [_I32, _I32, _I32, _I32, _P, _D, _D, _I32, _P, _P, _P],
    "jx_smagorinsky_viscosity": [_I32, _I64, _P, _P, _D, _D, _D, _P, _P],
    "jx_tile_info": [_DP, ctypes.POINTER(_I32), ctypes.POINTER(_I32), ctypes.POINTER(_I64)],
    "jx_probe_fma": [_I32, _I32, _I32, _I32, _P, _P],
    "jx_probe_math": [_I32, _I64, _P, _P, _P, _P, _P, _P],
    "jx_batch_plan_bytes": [ctypes.POINTER(SolveStruct), _I32, ctypes.POINTER(_SZ)],
    "jx_batch_plan": [ctypes.POINTER(SolveStruct), _I32, _P, _SZ],
    "jx_batch_step": [_P, _P, _I32, _P],
    "jx_batch_groups": [_P],
    "jx_ou_table": [_P, _I32, _D, _D, _I32, _I32, _D, _D, _I64, _D, _D, _I32, _P],
}
_RESTYPES = {"jx_last_error": ctypes.c_char_p, "jx_version": ctypes.c_char_p,
             "jx_num_stages": ctypes.c_int32, "jx_batch_groups": ctypes.c_int32}

_lib = None


def load():
    """Load libjx.so once; raise if it has not been built."""
    global _lib
    if _lib is None:
        if not LIBRARY_PATH.exists():
            raise RuntimeError(
                f"{LIBRARY_PATH} is missing: build it with `python -m jathenax_gb300.build` "
                "(there is no CPU fallback)")
        lib = ctypes.CDLL(str(LIBRARY_PATH))
        for name, args in PROTOTYPES.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = _RESTYPES.get(name, ctypes.c_int32)
        _lib = lib
    return _lib


def check(status, what=""):
    """Turn a jx_status into the reference's exception types."""
    if status == JX_OK:
        return
    message = load().jx_last_error().decode()
    text = f"{what}: {message}" if what else message
    if status == JX_ERR_INVALID:
        raise ValueError(text)
    if status == JX_ERR_UNSUPPORTED:
        raise KeyError(text)
    raise RuntimeError(text)


def call(name, *args):
    check(getattr(load(), name)(*args), name)


# ---------------------------------------------------------------------------
# Device buffers (torch CUDA tensors).
# ---------------------------------------------------------------------------

def torch():
    import torch as _torch
    if not _torch.cuda.is_available():
        raise RuntimeError("jathenax_gb300 needs a CUDA device; none is visible")
    return _torch


def device():
    return torch().device("cuda", torch().cuda.current_device())


def stream_handle():
    return ctypes.c_void_p(torch().cuda.current_stream().cuda_stream)


def dtype_id(dtype):
    name = str(dtype).replace("torch.", "")
    if name == "float64":
        return JX_F64
    if name == "float32":
        return JX_F32
    raise ValueError(f"state dtype must be float64 or float32, not {name}")


def ptr(tensor):
    return ctypes.c_void_p(tensor.data_ptr()) if tensor is not None else ctypes.c_void_p(0)


def is_device_array(x):
    try:
        import torch as _torch
    except ImportError:  # pragma: no cover
        return False
    return isinstance(x, _torch.Tensor)


def to_device(x, dtype=None):
    """Contiguous CUDA tensor view/copy of a NumPy array, scalar or tensor."""
    t = torch()
    if isinstance(x, t.Tensor):
        out = x.to(device=device(), dtype=dtype) if (x.device.type != "cuda" or dtype is not None) else x
        return out.contiguous()
    arr = np.asarray(x)
    if dtype is None and arr.dtype not in (np.float32, np.float64):
        arr = arr.astype(np.float64)
    out = _upload(np.ascontiguousarray(arr))
    return out.to(dtype) if dtype is not None else out


def _upload(arr):
    """Host array -> new device tensor, stream-ordered: staged in pinned memory
    (torch's host allocator keeps the staging block until the copy is done),
    so the caller does not wait for work already queued on the GPU."""
    t = torch()
    host = t.from_numpy(arr)
    if host.numel() == 0:
        return host.to(device())
    return host.pin_memory().to(device(), non_blocking=True)


def like_input(tensor, template):
    """Return `tensor` as the caller's array type (NumPy for host input)."""
    if is_device_array(template):
        return tensor
    return tensor.cpu().numpy()


def new_clock(**fields):
    """A device jx_clock filled from keyword fields (uint8 tensor of 128 bytes)."""
    c = Clock()
    c.prev_dt = float("inf")
    c.update = -1
    for key, value in fields.items():
        setattr(c, key, value)
    host = np.frombuffer(bytes(c), dtype=np.uint8).copy()
    return _upload(host)


def read_clock(tensor):
    raw = tensor.cpu().numpy().tobytes()
    return Clock.from_buffer_copy(raw)


def workspace(desc):
    size = ctypes.c_size_t()
    call("jx_workspace_bytes", ctypes.byref(desc), ctypes.byref(size))
    # torch's caching allocator returns 512-byte aligned blocks.
    ws = torch().empty(int(size.value), dtype=torch().uint8, device=device())
    return ws, size.value
