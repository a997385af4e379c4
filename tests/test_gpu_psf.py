"""GPU PSF-patch interpolation against its float64 oracle, and the pre-cut
windows feeding the response."""
import numpy as np
import pytest
import torch

import psf_oracle as PO
import jubik_gb300 as ju
from jubik_gb300 import psf as jpsf
from jubik_gb300 import synthetic

pytestmark = pytest.mark.gpu


def relmax(a, b):
    a = a.detach().double().cpu().numpy() if isinstance(a, torch.Tensor) else a
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.mark.parametrize("field,npatch,dist", [((64, 64), 4, (1.0, 1.0)),
                                               ((96, 96), 6, (0.7, 0.7)),
                                               ((128, 64), 8, (1.0, 1.3))])
def test_full_layout_matches_oracle(cuda, field, npatch, dist):
    infos = synthetic.erosita_like_psf_infos(n_energies=2, field=field, distances=dist, seed=3)
    dom = ju.Domain((2,) + field, (1.0,) + dist)
    got = jpsf.psf_interpolator(dom, npatch, infos, layout="full")
    ref = PO.psf_interpolator((2,) + field, (1.0,) + dist, npatch, infos)
    assert got.shape == ref.shape
    assert relmax(got, ref) < 1e-12
    # the pre-cut windows are the cut of the full array, evaluated directly
    win = jpsf.psf_interpolator(dom, npatch, infos, layout="precut")
    assert relmax(win, PO.precut_windows(ref, npatch)) < 1e-12
    w32 = jpsf.psf_interpolator(dom, npatch, infos, layout="precut", dtype=torch.float32)
    assert relmax(w32, PO.precut_windows(ref, npatch)) < 1e-7


def test_precut_windows_feed_the_response(cuda):
    field, npatch, m = (128, 128), 8, 8
    infos = synthetic.erosita_like_psf_infos(n_energies=2, field=field, seed=5)
    dom = ju.Domain((2,) + field, (1.0, 1.0, 1.0))
    full = jpsf.psf_interpolator(dom, npatch, infos, layout="full")
    win = jpsf.psf_interpolator(dom, npatch, infos, layout="precut")
    sky = np.exp(np.random.default_rng(0).normal(size=(2,) + field))
    p_full = ju.ResponsePlan(1, 2, field, npatch, m, dtype=torch.float64).set_psf(full[None])
    p_win = ju.ResponsePlan(1, 2, field, npatch, m, dtype=torch.float64).set_psf(win[None])
    a, b = p_full.psf_forward(sky), p_win.psf_forward(sky)
    assert float(torch.linalg.norm(a - b) / torch.linalg.norm(b)) < 1e-14
    # and the drop-in linpatch_convolve takes the reference's full array as is
    c = ju.linpatch_convolve(torch.as_tensor(sky, device=cuda), dom, full, npatch, m)
    assert float(torch.linalg.norm(c - b[0]) / torch.linalg.norm(b[0])) < 1e-13
    p_full.close()
    p_win.close()


def test_interpolator_errors(cuda):
    infos = synthetic.erosita_like_psf_infos(n_energies=1, field=(64, 64))
    dom = ju.Domain((1, 64, 64), (1.0, 1.0, 1.0))
    bad = dict(infos[0], patch_center_ids=np.full((5, 2), 100.0))
    with pytest.raises(ValueError):
        jpsf.psf_interpolator(dom, 4, [bad])
    with pytest.raises(ValueError):
        jpsf.psf_interpolator(ju.Domain((1, 62, 62), (1.0, 1.0, 1.0)), 4, infos)
    with pytest.raises(ValueError):
        jpsf.psf_interpolator(dom, 4, [dict(infos[0], rs=np.arange(3.0))])
