"""A rendered frame written as PNG holds the RGBA8 conversion of the frame,
top row first."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_write_png_of_a_frame(gpu_ctx, tmp_path):
    import livre_gb300 as lv
    from test_png import read_png
    vi = lv.VolumeInformation(64, 16, 1)
    vol = gpu_ctx.blob_volume(vi, 6, 2)
    tf = gpu_ctx.transfer_function(lv.linear_ramp_tf())
    mv, proj = lv.orbit_camera(1, 8, vi.world_size, 40, 30, radius_scale=1.2)
    img = gpu_ctx.render(vol, tf, gpu_ctx.render_desc(mv, proj, 40, 30))
    path = tmp_path / "frame.png"
    gpu_ctx.write_png(img, path)
    got = read_png(path.read_bytes())
    want = gpu_ctx.to_rgba8(img).cpu().numpy()[::-1]
    assert np.array_equal(got, want)
    vol.close()
    tf.close()
