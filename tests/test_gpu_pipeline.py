"""Operator with pinned host buffers: the kernels read / write the stack in
host memory directly (overwrite-mode projection), or -- where that is off or
impossible -- the stack is traced and transferred in blocks of image rows
(views with CRPIX1 shifted by the block's first row) on two streams; results
must equal the device-resident path."""
import numpy as np
import pytest

from helpers import CUBE_SIG, CUBE_TOL, image_errors
from tomograpy_gb300 import lo_wrapper, synthetic

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def _build(built):
    return built


@pytest.mark.parametrize("use_mask", [False, True])
def test_pinned_host_blocks_match_device_path(use_mask):
    ch, vh = synthetic.make_geometry({"n": 40, "T": 9, "N": 112, "d": 215.0, "lon_range": (0.3, 5.0)})
    rng = np.random.default_rng(0)
    mask = rng.random((112, 112, 9)) < 0.2 if use_mask else None
    op = lo_wrapper.siddon_lo(vh, ch, obstacle="sun", dtype=np.float32, mask=mask)
    op.HOST_DIRECT = False
    op.PIPE_BLOCKS = 4                       # 112 rows -> blocks of 32, 32, 32, 16
    x = torch.from_numpy(synthetic.phantom(ch, seed=2) / np.float32(1e8))
    ref = op.project(x.cuda()).cpu()
    out = torch.empty(op.data_shape, dtype=torch.float32).pin_memory()
    op.project(x.pin_memory(), out=out)
    assert len(op._row_blocks()) == 4
    torch.testing.assert_close(out, ref, rtol=0, atol=0)    # same rays, same arithmetic
    y = torch.from_numpy(rng.random(op.data_shape).astype(np.float32))
    cref = op.backproject(y.cuda()).cpu().numpy()
    cout = torch.empty(op.cube_shape, dtype=torch.float32).pin_memory()
    op.backproject(y.pin_memory(), out=cout)
    rel, norm = image_errors(cout.numpy(), cref, sig=CUBE_SIG)
    assert rel <= CUBE_TOL and norm <= CUBE_TOL, (rel, norm)


def test_four_d_blocks_keep_frames():
    ch, vh = synthetic.make_geometry({"n": 16, "T": 6, "N": 64, "d": 215.0, "lon_range": (0.3, 5.0), "n_frames": 3})
    op = lo_wrapper.siddon4d_lo(vh, ch, ng=2, obstacle="sun", dtype=np.float32)
    op.HOST_DIRECT = False
    x = torch.from_numpy(synthetic.phantom4d(ch, 3, seed=1) / np.float32(1e8))
    ref = op.project(x.cuda()).cpu()
    out = torch.empty(op.data_shape, dtype=torch.float32).pin_memory()
    op.project(x, out=out)
    torch.testing.assert_close(out, ref, rtol=0, atol=0)


@pytest.mark.parametrize("layout", ["reference", "view_major"])
@pytest.mark.parametrize("use_mask", [False, True])
def test_pinned_host_stack_traced_in_place(layout, use_mask):
    """A view-major pinned host stack is written / read by the kernels
    directly: the projection overwrites every pixel (stale contents and
    masked pixels become the device path's values, bitwise), the
    backprojection reads it in place.  The reference's layout (T fastest)
    takes the row-block staging instead; both give the device results."""
    from tomograpy_gb300 import _lib
    ch, vh = synthetic.make_geometry({"n": 40, "T": 9, "N": 112, "d": 215.0, "lon_range": (0.3, 5.0)})
    rng = np.random.default_rng(1)
    mask = rng.random((112, 112, 9)) < 0.2 if use_mask else None
    op = lo_wrapper.siddon_lo(vh, ch, obstacle="sun", dtype=np.float32, mask=mask)
    x = torch.from_numpy(synthetic.phantom(ch, seed=3) / np.float32(1e8))
    ref = op.project(x.cuda()).cpu()
    if layout == "reference":
        out = torch.empty(op.data_shape, dtype=torch.float32).pin_memory()
    else:
        out = torch.empty((9, 112, 112), dtype=torch.float32).pin_memory().permute(1, 2, 0)
    assert _lib.host_alias(out) is not None
    assert (op._host_stack(out) is not None) == (layout == "view_major")
    out.fill_(7.0)                            # stale contents: overwritten
    op.project(x.pin_memory(), out=out)
    torch.testing.assert_close(out, ref, rtol=0, atol=0)
    y = torch.from_numpy(rng.random(op.data_shape).astype(np.float32))
    cref = op.backproject(y.cuda()).cpu().numpy()
    yh = out.copy_(y)
    rel, norm = image_errors(op.backproject(yh).cpu().numpy(), cref, sig=CUBE_SIG)
    assert rel <= CUBE_TOL and norm <= CUBE_TOL, (rel, norm)
    # pageable memory has no device alias
    assert _lib.host_alias(torch.empty(4)) is None


@pytest.mark.parametrize("layout", ["reference", "view_major"])
def test_host_buffers_reusable_when_the_call_returns(layout):
    """Once project / backproject return, the operator no longer reads the
    caller's pinned host cube or stack (in-place tracing, row-block staging
    and plain copies alike): overwriting them at once leaves the results
    equal to the device path's."""
    ch, vh = synthetic.make_geometry({"n": 40, "T": 9, "N": 112, "d": 215.0, "lon_range": (0.3, 5.0)})
    op = lo_wrapper.siddon_lo(vh, ch, obstacle="sun", dtype=np.float32)
    x = torch.from_numpy(synthetic.phantom(ch, seed=4) / np.float32(1e8))
    y = torch.from_numpy(np.random.default_rng(2).random(op.data_shape).astype(np.float32))
    ref = op.project(x.cuda()).cpu()
    cref = op.backproject(y.cuda()).cpu().numpy()
    xh = x.pin_memory()
    res = op.project(xh)                      # device result from a pinned host cube
    xh.fill_(float("nan"))
    torch.testing.assert_close(res.cpu(), ref, rtol=0, atol=0)
    if layout == "reference":
        yh = torch.empty(op.data_shape, dtype=torch.float32).pin_memory()
    else:
        yh = torch.empty((9, 112, 112), dtype=torch.float32).pin_memory().permute(1, 2, 0)
    for out in (None, torch.empty(op.cube_shape, device="cuda")):
        yh.copy_(y)
        c = op.backproject(yh, out=out)
        yh.fill_(float("nan"))
        rel, norm = image_errors(c.cpu().numpy(), cref, sig=CUBE_SIG)
        assert rel <= CUBE_TOL and norm <= CUBE_TOL, (layout, out is None, rel, norm)


def test_overwrite_projection_through_the_c_abi():
    """TG_OVERWRITE on a device stack: every pixel written, equal to
    zero-then-project; rejected for backprojections."""
    from tomograpy_gb300 import siddon
    ch, vh = synthetic.make_geometry({"n": 24, "T": 5, "N": 48, "d": 215.0, "lon_range": (0.3, 3.0)})
    x = torch.from_numpy(synthetic.phantom(ch, seed=4)).cuda()
    views = siddon.upload_views(vh, None, x.device)
    mh = siddon.pack_map_header(ch)
    mask = torch.from_numpy(np.random.default_rng(2).random((48, 48, 5)) < 0.3).cuda()
    ref = torch.zeros((48, 48, 5), device="cuda")
    siddon.run_device("pj", ref, x, views, mh, 5, mask=mask, obstacle="sun")
    y = torch.full((48, 48, 5), -3.0, device="cuda")
    siddon.run_device("pj", y, x, views, mh, 5, mask=mask, obstacle="sun", overwrite=True)
    torch.testing.assert_close(y, ref, rtol=0, atol=0)
    with pytest.raises(ValueError):
        siddon.run_device("bpj", y, torch.zeros_like(x), views, mh, 5, overwrite=True)
