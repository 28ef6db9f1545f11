"""Image output and input: the reference savers' 8-bit conversion, RGBE, and
Radiance .hdr files.

Pins: the golden fixture image_codec.npz holds what the reference's own code
produced (FileSaver::CopyColorArrayToImage + Utils::ToRgb, HDRImage::Color2RGBE
and RGBE2Color, HDRImage::WriteToRadianceFile / ReadFromRadianceFile) on seeded
inputs.  The bar is byte-exact for bytes and bit-exact for decoded floats.
"""
import numpy as np
import pytest

from conftest import golden


def test_oracle_conversions_match_reference(orc):
    g = golden("image_codec.npz")
    np.testing.assert_array_equal(orc.encode_rgb8(g["ldr"], True), g["rgb8_gamma"])
    np.testing.assert_array_equal(orc.encode_rgb8(g["ldr"], False), g["rgb8_linear"])
    np.testing.assert_array_equal(orc.encode_rgbe(g["hdr"]), g["rgbe"])
    np.testing.assert_array_equal(orc.decode_rgbe(g["rgbe_in"]), g["rgbe_decoded"])


@pytest.mark.parametrize("name", ["rle", "flat"])
def test_read_hdr_parses_the_reference_writers_files(pkg, orc, name):
    # host-only parser: no GPU needed
    g = golden("image_codec.npz")
    rgbe = pkg.read_hdr(g["hdr_%s_file" % name].tobytes())
    dec = g["hdr_%s_decoded" % name]
    assert rgbe.shape[:2] == dec.shape[:2]
    # the bytes are the reference encoder's output for the image it wrote
    np.testing.assert_array_equal(rgbe.reshape(-1, 4), orc.encode_rgbe(g["hdr_%s_image" % name].reshape(-1, 3)))
    if name == "rle":
        # and decode to what the reference's reader returns
        np.testing.assert_array_equal(orc.decode_rgbe(rgbe.reshape(-1, 4)).reshape(dec.shape), dec)
    else:
        # The reference cannot read back images narrower than 8 pixels: its
        # run-length reader hands (width, height) to the flat reader as
        # (pixel_count, start offset) (src/tools/HDRImage.cpp:114 vs :96), so
        # it returns `width` pixels of which only the one at index `height`
        # was read.  The fixture records exactly that.
        w, h = dec.shape[1], dec.shape[0]
        ref_px = dec.reshape(-1, 3)
        assert (ref_px[:h] == 0).all() and (ref_px[w:] == 0).all()
        np.testing.assert_array_equal(ref_px[h], orc.decode_rgbe(rgbe.reshape(-1, 4))[0])


def test_read_hdr_rejects_malformed_files(pkg):
    g = golden("image_codec.npz")
    good = g["hdr_rle_file"].tobytes()
    for bad in (b"", b"P6\n", good[:60], good.replace(b"-Y 23", b"+Y 23"), good[:-7]):
        with pytest.raises(pkg.Or3Error):
            pkg.read_hdr(bad)


# ---------------------------------------------------------------- GPU

@pytest.mark.gpu
def test_device_conversions_match_reference(pkg, ctx):
    g = golden("image_codec.npz")
    np.testing.assert_array_equal(ctx.encode_rgb8(g["ldr"], True), g["rgb8_gamma"])
    np.testing.assert_array_equal(ctx.encode_rgb8(g["ldr"], False), g["rgb8_linear"])
    np.testing.assert_array_equal(ctx.encode_rgbe(g["hdr"]), g["rgbe"])
    np.testing.assert_array_equal(ctx.decode_rgbe(g["rgbe_in"]).astype(np.float64), g["rgbe_decoded"])


@pytest.mark.gpu
@pytest.mark.parametrize("layout", [0, 1])
def test_frame_encoded_on_device_equals_encoded_frame(pkg, ctx, orc, layout):
    sd, cam, st = pkg.workloads.cornell_box(40, 24)
    sid = ctx.upload(sd)
    try:
        ctx.render(sid, cam, layout=layout, **dict(st, supersamples=2))
        f64, n = ctx.frame(cam.width, cam.height, layout)
        b8, n8 = ctx.frame_rgb8(cam.width, cam.height, layout)
        be, ne = ctx.frame_rgbe(cam.width, cam.height, layout)
    finally:
        ctx.release(sid)
    assert n == n8 == ne
    np.testing.assert_array_equal(b8.reshape(-1, 3), orc.encode_rgb8(f64.reshape(-1, 3), True))
    np.testing.assert_array_equal(be.reshape(-1, 4), orc.encode_rgbe(f64.reshape(-1, 3)))


@pytest.mark.gpu
def test_env_from_rgbe_renders_like_decoded_floats(pkg, ctx, orc):
    # the environment given as RGBE bytes (decoded on the device) renders the
    # same paths as the same map given as the floats RGBE2Color decodes
    sd, cam = pkg.workloads.sky_floor(32, 24, env=(128, 64))
    rgbe = orc.encode_rgbe(sd.env.reshape(-1, 3).astype(np.float64)).reshape(sd.env.shape[0], sd.env.shape[1], 4)
    sd_f = pkg.workloads.sky_floor(32, 24, env=(128, 64))[0]
    sd_f.set_env(orc.decode_rgbe(rgbe.reshape(-1, 4)).reshape(sd.env.shape).astype(np.float32))
    sd_b = pkg.workloads.sky_floor(32, 24, env=(128, 64))[0]
    sd_b.set_env_rgbe(rgbe)
    st = dict(supersamples=2, min_samples=2, max_samples=2, rr_min_depth=3, max_depth=6, seed=9,
              next_event_estimation=True)
    out = []
    for s in (sd_f, sd_b):
        sid = ctx.upload(s)
        try:
            ctx.render(sid, cam, flags=pkg.abi.OR3_FLAG_KEEP_PATHS, **st)
            out.append(ctx.path_radiance())
        finally:
            ctx.release(sid)
    np.testing.assert_array_equal(out[0], out[1])


@pytest.mark.gpu
def test_server_rgb8_frames_equal_encoded_f64_frames(pkg, ctx, orc):
    import threading
    sd, cam, _ = pkg.workloads.cornell_box(24, 16)
    sid = ctx.upload(sd)
    st = dict(supersamples=2, min_samples=3, max_samples=3, rr_min_depth=3, max_depth=8, seed=3)
    got = {}
    lock = threading.Lock()
    try:
        for rgb8 in (False, True):
            frames = []

            def cb(jid, samples, img, final, frames=frames):
                with lock:
                    frames.append((samples, final, img))
            ctx.server_start(frame_every_samples=1, on_frame=cb, rgb8=rgb8)
            try:
                ctx.server_submit(sid, cam, **st)
                ctx.server_drain(60.0)
            finally:
                ctx.server_stop()
            got[rgb8] = frames
    finally:
        ctx.release(sid)
    assert [f[0] for f in got[True]] == [f[0] for f in got[False]]
    for (s, fin, img8), (_, _, img64) in zip(got[True], got[False]):
        assert img8.dtype == np.uint8
        np.testing.assert_array_equal(img8.reshape(-1, 3), orc.encode_rgb8(img64.reshape(-1, 3), True))
