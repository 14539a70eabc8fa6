"""GPU test of pmgpu_cst_is_valid_fast_noalloc, the validity check for callers that must not
allocate device memory during the call (real-time loops, devices whose memory another allocator
owns, code that cannot afford cudaMalloc's implicit synchronisation).

It calls the entry point through the C ABI with device buffers, twice in a row (the fixed
scratch array keeps the previous call's contents, so the second call checks that it is cleared),
and compares both with pmgpu_cst_is_valid_fast: validity identical and FP32 distances bit for
bit (both paths take the same exact float minimum over the same searches).  After the first
call on the device (which looks up the array's address), the device's free memory is unchanged
across the calls.  The file is named to be collected last."""
import ctypes as C

import numpy as np
import pytest

from plainmp_gb300 import _lib, scenes
from plainmp_gb300 import workloads as W

pytestmark = pytest.mark.gpu

lib = _lib.lib
lib.pmgpu_cst_is_valid_fast_noalloc.restype = C.c_int
lib.pmgpu_cst_is_valid_fast_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p]


def noalloc(cst, Q, out, dist, stream):
    return lib.pmgpu_cst_is_valid_fast_noalloc(cst._h, C.c_void_p(Q.data_ptr()), Q.shape[0], C.c_void_p(out.data_ptr()),
                                               C.c_void_p(dist.data_ptr()) if dist is not None else None,
                                               C.c_void_p(stream.cuda_stream))


@pytest.mark.parametrize("which", ["chain7", "dualarm"])
def test_noalloc_matches_fast_path(which):
    import torch

    if which == "chain7":
        robot, scene, q = W.chain7_robot(), W.chain7_scene(), W.chain7_configs(4096, seed=77)
    else:
        robot, scene, q = W.dualarm_robot(), W.Scene(cloud=W.box_surface_cloud(), cloud_radius=0.0), W.dualarm_configs(2048, seed=78)
    _, cst, _ = scenes.make_constraint(robot, scene)
    Q = torch.tensor(q, device="cuda")
    ref_ok, ref_d = cst.is_valid_fast(Q, distances=True)  # allocating entry point; also puts the tables on the device
    ref_ok, ref_d = ref_ok.cpu().numpy(), ref_d.cpu().numpy()
    stream = torch.cuda.current_stream()
    # every buffer exists before the calls, so nothing else in the loop allocates
    out = torch.empty((Q.shape[0],), dtype=torch.uint8, device="cuda")
    dist = torch.empty((Q.shape[0], cst.n_spheres), dtype=torch.float32, device="cuda")
    out2 = torch.empty((Q.shape[0],), dtype=torch.uint8, device="cuda")
    assert noalloc(cst, Q, out, dist, stream) == _lib.PMGPU_OK, lib.pmgpu_last_error()  # per-device set-up
    torch.cuda.synchronize()
    free0 = None
    # the first pass also loads the kernels it launches for the first time in this process (torch's
    # fills among them: lazy module loading takes device memory for code), so the free memory is read
    # after it and must not move over the passes that follow
    for it in range(3):
        if it == 1:
            free0 = torch.cuda.mem_get_info()[0]
        out.fill_(7)
        dist.fill_(float("nan"))
        out2.fill_(7)
        assert noalloc(cst, Q, out, dist, stream) == _lib.PMGPU_OK, lib.pmgpu_last_error()
        torch.cuda.synchronize()
        assert np.array_equal(out.cpu().numpy(), ref_ok)
        got_d = dist.cpu().numpy()
        assert np.array_equal(got_d, ref_d), float(np.nanmax(np.abs(got_d.astype(np.float64) - ref_d)))
        assert noalloc(cst, Q, out2, None, stream) == _lib.PMGPU_OK
        torch.cuda.synchronize()
        assert np.array_equal(out2.cpu().numpy(), ref_ok)
    assert torch.cuda.mem_get_info()[0] == free0  # the calls allocated no device memory


def test_noalloc_limits():
    import torch

    _, cst, _ = scenes.make_constraint(W.chain7_robot(), W.chain7_scene())
    Q = torch.tensor(W.chain7_configs(8), device="cuda")
    out = torch.zeros(8, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()
    # tables not on the device yet: refused rather than allocated
    assert noalloc(cst, Q, out, None, stream) == _lib.PMGPU_ERR_RUNTIME
    cst.is_valid_fast(Q)
    assert noalloc(cst, Q, out, None, stream) == _lib.PMGPU_OK
    big = lib.pmgpu_cst_is_valid_fast_noalloc(cst._h, C.c_void_p(Q.data_ptr()), (1 << 20) + 1, C.c_void_p(out.data_ptr()), None,
                                              C.c_void_p(stream.cuda_stream))
    assert big == _lib.PMGPU_ERR_INVALID
    assert b"1048576" in lib.pmgpu_last_error()
