"""The no-allocation entry point.

Some callers of this library cannot allocate device memory: hosts that own
every byte of GPU memory through their own allocator or budget and forbid a
plug-in's cudaMalloc, and FFI callers that see only the C ABI.
tg_conic_full_backprojector_deterministic_noalloc serves them with a fixed
scratch array inside the library instead of a caller-provided workspace.
These tests call it through the C ABI and check it against the workspace
entry point (tg_conic_full_backprojector_deterministic) on two calls in a
row -- the second call must not see the first call's left-over scratch.
The file is named to be collected last.
"""
import ctypes

import numpy as np
import pytest

from tomograpy_gb300 import _lib, siddon, synthetic

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _args(mh, views, T, y, cube, mask=None, obstacle=_lib.TG_OBSTACLE_SUN):
    cshape = list(cube.shape) + ([1] if cube.dim() == 3 else [])
    cstr = list(cube.stride()) + ([0] if cube.dim() == 3 else [])
    if mask is None:
        m = (None, _lib.TG_U8, _lib.i64([0, 0, 0]))
    else:
        m = (ctypes.c_void_p(mask.data_ptr()), _lib.TG_U8, _lib.i64(mask.stride()))
    return (ctypes.byref(mh), ctypes.c_void_p(views.data_ptr()), T, ctypes.c_void_p(y.data_ptr()),
            int(y.shape[0]), int(y.shape[1]), _lib.i64(y.stride()), ctypes.c_void_p(cube.data_ptr()),
            _lib.i64(cshape), _lib.i64(cstr)) + m + (obstacle,)


def _with_workspace(L, args, shape, mode, stream):
    cube = torch.zeros(shape, dtype=torch.float32, device="cuda")
    need = L.tg_deterministic_workspace_bytes(_lib.i64(list(shape) + ([1] if len(shape) == 3 else [])))
    ws = torch.empty(need, dtype=torch.uint8, device="cuda")
    st = L.tg_conic_full_backprojector_deterministic(*args(cube), mode, ctypes.c_void_p(ws.data_ptr()), need,
                                                     stream)
    _lib.check(st)
    return cube


def _without_allocation(L, args, shape, mode, stream):
    cube = torch.zeros(shape, dtype=torch.float32, device="cuda")
    st = L.tg_conic_full_backprojector_deterministic_noalloc(*args(cube), mode, stream)
    _lib.check(st)
    return cube


# (4-D cube, obstacle, u8 mask): the sun-occulted 3-D and 4-D cases, and an
# unobstructed 3-D case whose rays are partly masked out
CASES = [(False, _lib.TG_OBSTACLE_SUN, False), (True, _lib.TG_OBSTACLE_SUN, False),
         (False, _lib.TG_OBSTACLE_NONE, True)]


@pytest.mark.parametrize("four_d,obstacle,use_mask", CASES)
def test_noalloc_matches_workspace_entry_point(built, four_d, obstacle, use_mask):
    L = _lib.load()
    n, T, N = 40, 10, 64
    ch, vh = synthetic.make_geometry({"n": n, "T": T, "N": N, "d": 215.0, "lon_range": (0.2, 2.9)})
    frames = np.arange(T) // 2 if four_d else None
    views = siddon.upload_views(vh, frames, torch.device("cuda"))
    mh = siddon.pack_map_header(ch)
    shape = (n, n, n, T // 2) if four_d else (n, n, n)
    mode = _lib.TG_BPJT if four_d else _lib.TG_BPJ
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rng = np.random.default_rng(21)
    mask = None
    if use_mask:
        mask = torch.from_numpy((rng.random((N, N, T)) < 0.3).astype(np.uint8)).cuda()
    for call in range(2):  # two calls in a row share the library's scratch
        y = torch.from_numpy(rng.random((N, N, T)).astype(np.float32) * (1 + 9 * call)).cuda()

        def args(cube):
            return _args(mh, views, T, y, cube, mask, obstacle)
        ref = _with_workspace(L, args, shape, mode, stream)
        out = _without_allocation(L, args, shape, mode, stream)
        torch.cuda.synchronize()
        # the same fixed-point kernels on the same inputs: bitwise equal, so
        # stale scratch or a wrong output scale cannot hide in a tolerance
        assert torch.equal(out, ref), call
        assert float(ref.abs().max()) > 0


def test_noalloc_rejects_a_cube_beyond_its_scratch(built):
    L = _lib.load()
    limit = (L.tg_noalloc_scratch_bytes() - 256) // 8
    ch, vh = synthetic.make_geometry({"n": 256, "T": 1, "N": 8, "d": 215.0, "lon_range": (0.2, 0.2)})
    assert 256 ** 3 > limit
    views = siddon.upload_views(vh, None, torch.device("cuda"))
    mh = siddon.pack_map_header(ch)
    y = torch.ones((8, 8, 1), dtype=torch.float32, device="cuda")
    cube = torch.zeros((256, 256, 256), dtype=torch.float32, device="cuda")
    st = L.tg_conic_full_backprojector_deterministic_noalloc(
        *_args(mh, views, 1, y, cube), _lib.TG_BPJ, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == _lib.TG_ENOMEM
    assert b"scratch" in L.tg_last_error()
    assert float(cube.abs().max()) == 0.0
