"""The limits of the target size: the widest and tallest targets the
library takes (RF_MAX_TARGET_DIM = 32768) and a 16384 x 16384 target, each
against the oracle bit-exactly; one more pixel is refused."""
import numpy as np
import pytest

import retrofire_gb300 as rf
from retrofire_gb300 import scenes
from rfhelp import DrawSpec, assert_parity, gpu_render, oracle_render

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    from retrofire_gb300 import build
    build.build()
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")


def fill(ntri, w, h, seed, amax):
    s = scenes.fill_stress(ntri=ntri, w=w, h=h, seed=seed, amax=amax)
    return [DrawSpec(s["verts"], s["faces"], rf.GOURAUD, None, pos_dim=4)], s["vp"]


@pytest.mark.parametrize("w,h,ntri,amax", [(32768, 48, 6000, 2000.0), (48, 32768, 6000, 2000.0),
                                           (16384, 16384, 20000, 40000.0)])
def test_largest_targets(w, h, ntri, amax):
    draws, vp = fill(ntri, w, h, 31, amax)
    g = gpu_render(draws, vp, w, h)
    o = oracle_render(draws, vp, w, h)
    assert o[2]["frags_i"] > 100000
    assert_parity(g, o, what="%dx%d" % (w, h))


def test_one_past_the_limit_is_refused():
    dev = rf.Device()
    try:
        for w, h in ((32769, 1), (1, 32769)):
            with pytest.raises(rf.RfError) as e:
                rf.Framebuf(w, h, device=dev)
            assert e.value.code == 2
    finally:
        dev.close()
