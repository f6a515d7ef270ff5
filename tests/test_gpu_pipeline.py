"""Operator with pinned host buffers: the stack is traced and transferred in
blocks of image rows (views with CRPIX1 shifted by the block's first row) on
two streams; results must equal the device-resident path."""
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
    x = torch.from_numpy(synthetic.phantom4d(ch, 3, seed=1) / np.float32(1e8))
    ref = op.project(x.cuda()).cpu()
    out = torch.empty(op.data_shape, dtype=torch.float32).pin_memory()
    op.project(x, out=out)
    torch.testing.assert_close(out, ref, rtol=0, atol=0)
