"""ctypes binding of the in-tree C ABI (include/pmgpu.h -> plainmp_gb300/libpmgpu.so).

The library is the product: there is no Python or CPU fallback.  Importing this module
fails loudly if the shared library is missing; batch calls fail loudly (CudaError) on a
host without a CUDA device.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "libpmgpu.so"

PMGPU_OK = 0
PMGPU_ERR_INVALID = 1
PMGPU_ERR_RUNTIME = 2
PMGPU_ERR_CUDA = 3
PMGPU_ERR_TIMEOUT = 4
MEM_HOST = 0
MEM_DEVICE = 1


class CudaError(RuntimeError):
    """A CUDA failure, or no CUDA device on this host."""


class DeviceTimeout(RuntimeError):
    """A bounded device-side wait gave up."""


def _load() -> C.CDLL:
    if not LIB_PATH.exists():
        raise ImportError(
            f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
            "(or `python plainmp_gb300/build.py`)"
        )
    return C.CDLL(str(LIB_PATH))


lib = _load()

_p = C.c_void_p
_i = C.c_int
_i64 = C.c_int64
_d = C.c_double
_dp = C.POINTER(C.c_double)
_i64p = C.POINTER(C.c_int64)
_i32p = C.POINTER(C.c_int32)
_u8p = C.POINTER(C.c_uint8)
_fp = C.POINTER(C.c_float)
_cpp = C.POINTER(C.c_char_p)

_SIGS = {
    "pmgpu_last_error": (C.c_char_p, []),
    "pmgpu_version": (_i, []),
    "pmgpu_device_count": (_i, []),
    "pmgpu_model_create": (_i, [C.c_char_p, C.POINTER(_p)]),
    "pmgpu_model_destroy": (None, [_p]),
    "pmgpu_model_counts": (_i, [_p, C.POINTER(_i), C.POINTER(_i), C.POINTER(_i)]),
    "pmgpu_model_get_joint_ids": (_i, [_p, _cpp, _i, _i64p]),
    "pmgpu_model_get_link_ids": (_i, [_p, _cpp, _i, _i64p]),
    "pmgpu_model_get_joint_position_limits": (_i, [_p, _i64p, _i, _dp, _dp]),
    "pmgpu_model_link_name": (_i, [_p, _i64, C.c_char_p, _i]),
    "pmgpu_model_joint_name": (_i, [_p, _i64, C.c_char_p, _i]),
    "pmgpu_model_structure": (_i, [_p, _i32p, _dp, _i32p, _i32p, _i32p, _dp, _i32p]),
    "pmgpu_model_set_joint_positions": (_i, [_p, _i64p, _i, _dp, _i]),
    "pmgpu_model_get_joint_positions": (_i, [_p, _i64p, _i, _dp]),
    "pmgpu_model_set_base_pose": (_i, [_p, _dp]),
    "pmgpu_model_get_base_pose": (_i, [_p, _dp]),
    "pmgpu_model_link_poses": (_i, [_p, _i64p, _i, _dp]),
    "pmgpu_model_add_new_link": (_i, [_p, C.c_char_p, C.c_char_p, _dp, _dp, _i, _i64p]),
    "pmgpu_pose_flags": (_i, [_dp, C.POINTER(_i), C.POINTER(_i), _dp]),
    "pmgpu_sdf_box_create": (_i, [_dp, _dp, _dp, C.POINTER(_p)]),
    "pmgpu_sdf_cylinder_create": (_i, [_d, _d, _dp, _dp, C.POINTER(_p)]),
    "pmgpu_sdf_sphere_create": (_i, [_d, _dp, _dp, C.POINTER(_p)]),
    "pmgpu_sdf_ground_create": (_i, [_d, C.POINTER(_p)]),
    "pmgpu_sdf_cloud_create": (_i, [_dp, _i64, _d, _d, C.POINTER(_p)]),
    "pmgpu_sdf_cloud_stats": (_i, [_p, _i64p]),
    "pmgpu_sdf_union_create": (_i, [C.POINTER(_p), _i, C.POINTER(_p)]),
    "pmgpu_sdf_union_add": (_i, [_p, _p, _i]),
    "pmgpu_sdf_clone": (_i, [_p, C.POINTER(_p)]),
    "pmgpu_sdf_destroy": (None, [_p]),
    "pmgpu_sdf_translate": (_i, [_p, _dp]),
    "pmgpu_sdf_rotate_z": (_i, [_p, _d]),
    "pmgpu_sdf_info": (_i, [_p, C.POINTER(_i), _dp, _dp, C.POINTER(_i), C.POINTER(_i), _dp, _dp]),
    "pmgpu_sdf_evaluate": (_i, [_p, _p, _i64, _p, _i, _p]),
    "pmgpu_sdf_is_outside": (_i, [_p, _p, _p, _i64, _p, _i, _p]),
    "pmgpu_cloud_nearest": (_i, [_p, _p, _i64, _p, _p, _i, _p]),
    "pmgpu_cst_create": (_i, [_p, _cpp, _i, _i, _i, _cpp, _i32p, _dp, _dp, _u8p, _i, _cpp, _cpp, _p, _i, C.POINTER(_p)]),
    "pmgpu_cst_destroy": (None, [_p]),
    "pmgpu_cst_set_sdf": (_i, [_p, _p]),
    "pmgpu_cst_dims": (_i, [_p, C.POINTER(_i), C.POINTER(_i), C.POINTER(_i), C.POINTER(_i)]),
    "pmgpu_cst_groups": (_i, [_p, _i32p, _dp, _dp, _i32p, _dp, _dp]),
    "pmgpu_cst_update_kintree": (_i, [_p, _dp, _i]),
    "pmgpu_cst_get_all_spheres": (_i, [_p, _dp]),
    "pmgpu_cst_get_group_spheres": (_i, [_p, _dp]),
    "pmgpu_cst_is_valid": (_i, [_p, _p, _i64, _p, _i, _p]),
    "pmgpu_cst_evaluate": (_i, [_p, _p, _i64, _p, _p, _i, _p]),
    "pmgpu_cst_sphere_distances": (_i, [_p, _p, _i64, _i, _p, _p, _i, _p]),
    "pmgpu_cst_is_valid_fast": (_i, [_p, _p, _i64, _p, _p, _p, _i, _p]),
    "pmgpu_check_motion": (_i, [_p, _p, _p, _i64, _i, _p, _d, _p, _i64p, _i, _p]),
    "pmgpu_check_motion_fast": (_i, [_p, _p, _p, _i64, _i, _p, _d, _p, _p, _i, _p]),
    "pmgpu_cst_set_fast_launch": (_i, [_p, _i, _i]),
    "pmgpu_cst_get_fast_launch": (_i, [_p, C.POINTER(_i), C.POINTER(_i)]),
    "pmgpu_cst_set_fast_tuning": (_i, [_p, _i, _i, _i, _i]),
    "pmgpu_cst_get_fast_tuning": (_i, [_p, C.POINTER(_i), C.POINTER(_i), C.POINTER(_i), C.POINTER(_i)]),
    "pmgpu_cst_link_poses": (_i, [_p, C.c_int32, _p, _i64, _p, _i, _p]),
    "pmgpu_linkpose_create": (_i, [_p, _cpp, _i, _i, _cpp, _i, _dp, _i32p, C.POINTER(_p)]),
    "pmgpu_linkbound_create": (_i, [_p, _cpp, _i, _i, C.c_char_p, _i, _i, _d, _i, _d, C.POINTER(_p)]),
    "pmgpu_posecst_destroy": (None, [_p]),
    "pmgpu_posecst_dims": (_i, [_p, C.POINTER(_i), C.POINTER(_i), C.POINTER(_i)]),
    "pmgpu_posecst_update_kintree": (_i, [_p, _dp, _i]),
    "pmgpu_posecst_evaluate": (_i, [_p, _p, _i64, _p, _p, _i, _p]),
    "pmgpu_posecst_is_valid": (_i, [_p, _p, _i64, _p, _i, _p]),
    "pmgpu_composite_is_valid_fast": (_i, [_p, _p, _i, _p, _i64, _p, _p, _i, _p]),
    "pmgpu_composite_check_motion_fast": (_i, [_p, _p, _i, _p, _p, _i64, _i, _p, _d, _p, _p, _i, _p]),
    "pmgpu_ik_cost": (_i, [_p, _p, _p, _p, _i64, _p, _p, _i, _p]),
    "pmgpu_ik_descend": (_i, [_p, _p, _p, _p, _i64, C.c_int32, C.c_float, C.c_int32, _p, _p, _i, _p]),
    "pmgpu_traj_cost": (_i, [_p, _p, _p, _p, _i64, _i64, _p, _p, _i, _p]),
    "pmgpu_profile_enable": (_i, [_i]),
    "pmgpu_profile_read": (_i, [C.c_char_p, _dp, _i64p]),
    "pmgpu_measure_fma_peak": (_i, [_i, _dp, _p]),
}

for _name, (_res, _args) in _SIGS.items():
    _f = getattr(lib, _name)
    _f.restype = _res
    _f.argtypes = _args


def check(rc: int) -> None:
    """Raise the Python exception matching a C ABI status."""
    if rc == PMGPU_OK:
        return
    msg = lib.pmgpu_last_error().decode(errors="replace")
    if rc == PMGPU_ERR_INVALID:
        raise ValueError(msg)
    if rc == PMGPU_ERR_CUDA:
        raise CudaError(msg)
    if rc == PMGPU_ERR_TIMEOUT:
        raise DeviceTimeout(msg)
    raise RuntimeError(msg)


def profile_enable(on: bool = True) -> None:
    """Record CUDA events around every library kernel launch (on its own stream)."""
    check(lib.pmgpu_profile_enable(int(bool(on))))


def profile_read(kernel: str = "*"):
    """(summed device ms, launches) of a library kernel since the last read; clears them."""
    ms = C.c_double(0.0)
    n = C.c_int64(0)
    check(lib.pmgpu_profile_read(kernel.encode(), C.byref(ms), C.byref(n)))
    return float(ms.value), int(n.value)


def measure_fma_peak(fp64: bool = False, stream=None) -> float:
    """Measured FMA throughput of the current GPU in TFLOP/s (FP32, or FP64 with fp64=True)."""
    t = C.c_double(0.0)
    check(lib.pmgpu_measure_fma_peak(int(bool(fp64)), C.byref(t), stream))
    return float(t.value)


def device_count() -> int:
    return int(lib.pmgpu_device_count())


def dptr(a: np.ndarray):
    return a.ctypes.data_as(_dp)


def cstrs(names) -> C.Array:
    arr = (C.c_char_p * max(len(names), 1))()
    for i, n in enumerate(names):
        arr[i] = n.encode()
    return arr


def f64(a, shape=None) -> np.ndarray:
    out = np.ascontiguousarray(np.asarray(a, dtype=np.float64))
    if shape is not None:
        out = out.reshape(shape)
    return out


class Batch:
    """Normalises a batch argument: a numpy array (host memory) or a torch CUDA tensor
    (device memory, enqueued on torch's current stream)."""

    def __init__(self, x, dtype=np.float64):
        self.torch = None
        self.keep = None
        try:  # torch is optional for host-memory callers
            import torch  # noqa: F401

            if isinstance(x, torch.Tensor):
                self.torch = torch
        except ImportError:  # pragma: no cover
            pass
        if self.torch is not None and x.is_cuda:
            cur = self.torch.cuda.current_device()
            if x.device.index != cur:  # the library's kernels run on the current device
                raise ValueError(f"the batch is on {x.device} but the current CUDA device is cuda:{cur}: "
                                 "select its device first (torch.cuda.set_device)")
            tdt = {np.float64: self.torch.float64, np.float32: self.torch.float32, np.uint8: self.torch.uint8,
                   np.int64: self.torch.int64}[dtype]
            self.keep = x.detach().to(tdt).contiguous()
            self.mem = MEM_DEVICE
            self.ptr = C.c_void_p(self.keep.data_ptr())
            self.stream = C.c_void_p(self.torch.cuda.current_stream(self.keep.device).cuda_stream)
            self.shape = tuple(self.keep.shape)
        else:
            if self.torch is not None and isinstance(x, self.torch.Tensor):
                x = x.detach().cpu().numpy()
            self.keep = np.ascontiguousarray(np.asarray(x, dtype=dtype))
            self.mem = MEM_HOST
            self.ptr = C.c_void_p(self.keep.ctypes.data)
            self.stream = C.c_void_p(0)
            self.shape = self.keep.shape

    def out(self, buf, shape, dtype):
        """Pointer to a caller's preallocated output, which the call writes in place: it must be
        a C-contiguous, writeable array of exactly this shape and dtype in this batch's memory
        space (a CUDA tensor on the same device, or a host array).  Anything else raises
        ValueError: a converted copy would receive the results instead, and a smaller buffer
        would be overrun."""
        shape = tuple(int(x) for x in shape)
        if self.mem == MEM_DEVICE:
            tdt = {np.float64: self.torch.float64, np.float32: self.torch.float32, np.uint8: self.torch.uint8,
                   np.int64: self.torch.int64}[dtype]
            ok = (isinstance(buf, self.torch.Tensor) and buf.is_cuda and buf.device == self.keep.device and buf.dtype == tdt
                  and buf.is_contiguous() and tuple(buf.shape) == shape)
            if not ok:
                raise ValueError(f"output buffer must be a contiguous {tdt} CUDA tensor of shape {shape} on {self.keep.device}")
            return C.c_void_p(buf.data_ptr())
        if type(buf).__module__.startswith("torch"):  # a torch tensor, whatever the input was
            if buf.is_cuda:
                raise ValueError("output buffer must be in host memory, like the input")
            buf = buf.detach().numpy()  # shares the tensor's memory
        ok = (isinstance(buf, np.ndarray) and buf.dtype == np.dtype(dtype) and buf.flags.c_contiguous and buf.flags.writeable
              and buf.shape == shape)
        if not ok:
            raise ValueError(f"output buffer must be a C-contiguous, writeable {np.dtype(dtype)} host array of shape {shape}")
        return C.c_void_p(buf.ctypes.data)

    def empty(self, shape, dtype):
        """An output buffer in the same memory space."""
        if self.mem == MEM_DEVICE:
            tdt = {np.float64: self.torch.float64, np.float32: self.torch.float32, np.uint8: self.torch.uint8,
                   np.int64: self.torch.int64}[dtype]
            t = self.torch.empty(shape, dtype=tdt, device=self.keep.device)
            return t, C.c_void_p(t.data_ptr())
        a = np.empty(shape, dtype=dtype)
        return a, C.c_void_p(a.ctypes.data)
