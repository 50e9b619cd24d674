"""Headless readout against the reference's own summary and colour-map
shaders (translated to C++, oracle/_ref): bit-exact per cell, and the frame's
pixel-to-cell lookup against the quad geometry of the reference's draw."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def run_pair(lbm, P, nx, ny, steps, seed):
    from lbm_gb300 import geometry
    mask = geometry.single_circle(nx, ny, nx // 4, ny / 2, max(3, ny // 8))
    mask[0] = 1
    mask[-1] = 1
    rng = np.random.default_rng(seed)
    lat = lbm.Lattice(nx, ny, 1.0 / 0.6, lbm.EDGE_REF, lbm.F32)
    lat.init_equilibrium(1.0, 0.1, 0.0, 1e-2, seed)
    lat.draw_mask(mask)
    ref = P.RefShaders(nx, ny, float(np.float32(1.0 / 0.6)))
    ref.put_state(lat.populations())
    ref.set_barrier(mask)
    lat.iterate(steps)
    ref.iterate(steps)
    del rng
    return lat, ref, mask


def frame_cells(nx, ny, w, h):
    """Cell shown at each pixel centre by the reference's quads (lbm.rs:108-114,
    render.wgsl:13-15): cell cx spans NDC x in [-1 + 2 cx / nx, -1 + 2 (cx+1) / nx]."""
    px = np.arange(w)
    py = np.arange(h)
    cx = ((2 * px + 1) * nx) // (2 * w)
    cy = ((2 * py + 1) * ny) // (2 * h)
    return cy[:, None], cx[None, :]


@pytest.mark.parametrize("nx,ny", [(96, 48), (61, 37)])
def test_gpu_summary_and_colours_match_reference_shaders(lbm, cuda_ok, oracle_mod, nx, ny):
    P = oracle_mod
    lat, ref, mask = run_pair(lbm, P, nx, ny, 40, 3)
    for stat in range(5):  # curl first: the reference's output buffer is still all zero
        want = ref.summary(stat)
        np.testing.assert_array_equal(lat.summary(stat), want, err_msg="stat %d" % stat)
        for cmap in range(3):
            cols = ref.color_map(cmap)
            got = lat.render(nx, ny, stat=stat, cmap=cmap)
            np.testing.assert_array_equal(got, cols, err_msg="stat %d cmap %d" % (stat, cmap))
    lat.close()


def test_gpu_frame_upsampling_and_rgba(lbm, cuda_ok, oracle_mod):
    P = oracle_mod
    nx, ny = 50, 30
    lat, ref, mask = run_pair(lbm, P, nx, ny, 25, 5)
    ref.summary(0)
    cols = ref.color_map(2)
    for w, h in [(175, 105), (50, 30), (37, 64), (400, 9)]:
        cy, cx = frame_cells(nx, ny, w, h)
        got = lat.render(w, h, stat=0, cmap=2)
        np.testing.assert_array_equal(got, cols[cy, cx])
    rgba = lat.render(175, 105, stat=0, cmap=2, rgba=True)
    f = lat.render(175, 105, stat=0, cmap=2)
    assert rgba.shape == (105, 175, 4) and (rgba[..., 3] == 255).all()
    assert np.abs(rgba[..., :3].astype(np.int32) - np.floor(np.clip(f, 0, 1) * 255 + 0.5)).max() <= 1
    s = lat.render(175, 105, stat=0, cmap=2, rgba=True, srgb=True)
    lin = np.clip(f, 0, 1)
    enc = np.where(lin <= 0.0031308, 12.92 * lin, 1.055 * lin ** (1 / 2.4) - 0.055)
    assert np.abs(s[..., :3].astype(np.int32) - np.floor(enc * 255 + 0.5)).max() <= 1
    lat.close()


def test_gpu_render_arguments(lbm, cuda_ok):
    with lbm.Lattice(20, 10, 1.0, lbm.EDGE_CHANNEL, lbm.F16) as lat:
        lat.iterate(3)
        assert lat.render(40, 20).shape == (20, 40, 3)
        with pytest.raises(lbm.LBMError):
            lat.render(0, 5)
        with pytest.raises(lbm.LBMError):
            lat.render(10, 10, cmap=3)
        with pytest.raises(lbm.LBMError):
            lat.summary(5)
