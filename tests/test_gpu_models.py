"""Solar models on the GPU operator: the reference's integration test
(tests/test_models.py:14-37) re-expressed -- reconstruct a ones object with
srt / stsrt / thomson through CG and check the voxels the data see to one
decimal -- plus mask / weight semantics against the oracle."""
import numpy as np
import pytest

import oracle
import tomograpy_gb300 as tg
from helpers import IMG_TOL, degenerate_rays, image_errors
from tomograpy_gb300 import models
from tomograpy_gb300.infoarray import InfoArray

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def _build(built):
    return built


def _geometry(dtype=np.float32):
    obj_h = tg.centered_cubic_map_header(3.0, 16, dtype=dtype)
    obj = tg.InfoArray(data=np.ones((16, 16, 16), dtype), header=dict(obj_h))
    ih = tg.centered_image_header(tg.fov(obj_h, 200.0), 32, dtype=dtype)
    ih.update({"radius": 200.0, "max_lon": 3 * np.pi, "n_images": 100, "DATE_OBS": "2010-01-01T00:00:00Z",
               "dtype": dtype})
    data = tg.simu.circular_trajectory_data(**ih)
    return obj, data


@pytest.mark.parametrize("name", ["srt", "stsrt", "thomson"])
def test_models_reconstruct_ones(name):
    from tomograpy_gb300 import cg
    obj, data = _geometry()
    P, D, obj_mask, data_mask = getattr(models, name)(data, obj, obj_rmin=1.0)
    dev = P.device
    truth = np.ones(P.cube_shape, np.float32)
    if obj_mask is not None:
        keep = ~obj_mask
        truth = truth * (keep[..., None] if truth.ndim == 4 else keep)
    seen = (P.backproject(torch.ones(P.data_shape, device=dev)).cpu().numpy() != 0)
    y = P.project(torch.from_numpy(truth).to(dev))
    b = P.backproject(y)
    A = cg.NormalOperator(P, hypers=[1e-10] * len(D))
    sol = cg.cg(A, b, maxiter=300).x.cpu().numpy()
    err = np.abs(sol[seen] - truth[seen])
    assert seen.sum() > 100
    assert err.max() < 0.15, err.max()


def test_data_mask_radius_and_values():
    obj, data = _geometry()
    for h in data.header:
        h["D"] = 200.0
    d = np.asarray(data)
    d[0, 0, 0] = np.nan
    d[1, 0, 0] = -1.0
    m = models.define_data_mask(data, data_rmin=1.0, mask_negative=True)
    R = models.distance_to_sun_center(data)
    assert m[0, 0, 0] and m[1, 0, 0]
    np.testing.assert_array_equal(m[..., 1], (R[..., 1] < 1.0) | np.isnan(d[..., 1]) | (d[..., 1] < 0))


def test_srt_masks_match_oracle():
    obj, data = _geometry()
    P, D, obj_mask, data_mask = models.srt(data, obj, obj_rmin=1.2, data_rmin=0.5)
    x = np.random.default_rng(0).random((16, 16, 16)).astype(np.float32)
    y = P.project(torch.from_numpy(x).to(P.device)).cpu().numpy()
    xm = x.astype(np.float64) * (~obj_mask)
    ref = InfoArray(shape=data.shape, header=[dict(h) for h in data.header])
    oracle.projector(ref, InfoArray(data=xm, header=dict(obj.header)), mask=data_mask.astype(np.float64),
                     obstacle="sun")
    # rays within 1e-12 rad of a voxel plane (lon = k pi views) are compared in
    # test_gpu_parity.test_degenerate_rays_trace_their_chord
    degen = degenerate_rays(data.header, 32, 32)
    rel, norm = image_errors(y, ref, exclude=degen)
    assert rel <= IMG_TOL and norm <= IMG_TOL, (rel, norm)
